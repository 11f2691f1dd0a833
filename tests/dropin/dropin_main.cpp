// dropin_main.cpp -- a driver that uses the GPU library exactly the way the
// reference's drivers use its labeler classes (pado.cpp:188-291 label and
// store; query_distance.cpp:55-73 load and answer stdin pairs), through the
// drop-in header only.
//
//   dropin label <edge_list> <index_out> [-w 0|1]
//   dropin query <index> [-w 0|1]          (pairs "a b" on stdin)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "pado_gpu.hpp"

using namespace PADO;

int main(int argc, char **argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: dropin label <edges> <index> [-w 0|1] | dropin query <index> [-w 0|1]\n");
        return EXIT_FAILURE;
    }
    const std::string mode = argv[1];
    bool weighted = false;
    for (int i = 2; i + 1 < argc; ++i)
        if (!strcmp(argv[i], "-w")) weighted = strtoul(argv[i + 1], nullptr, 0) != 0;
    if (mode == "label") {
        if (argc < 4) return EXIT_FAILURE;
        if (!weighted) {
            Graph G(argv[2]);
            std::vector<idi> rank = G.make_rank();
            G.id_transfer(rank);
            ParaVertexCentricPLL<1024> *p = new ParaVertexCentricPLL<1024>(G);
            p->store_index_to_file(argv[3], rank);
            delete p;
        } else {
            WeightedGraph G(argv[2]);
            std::vector<idi> rank = G.make_rank();
            G.id_transfer(rank);
            WeightedParaVertexCentricPLL<512> *p = new WeightedParaVertexCentricPLL<512>(G);
            p->store_index_to_file(argv[3], rank);
            delete p;
        }
    } else if (mode == "query") {
        idi a, b;
        if (!weighted) {
            VertexCentricPLL<1024> *q = new VertexCentricPLL<1024>();
            q->load_index_from_file(argv[2]);
            while (std::cin >> a >> b) printf("%u\n", q->query_distance(a, b));
            delete q;
        } else {
            WeightedVertexCentricPLL<512> *q = new WeightedVertexCentricPLL<512>();
            q->load_index_from_file(argv[2]);
            while (std::cin >> a >> b) printf("%d\n", (int)q->query_distance(a, b));
            delete q;
        }
    } else {
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}
