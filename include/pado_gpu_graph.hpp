// pado_gpu_graph.hpp -- a Graph / WeightedGraph with the public layout the
// reference's labelers consume (includes/graph.h:31-92, :223-259 of the
// reference), for programs built without the reference tree.
//
// It shares the reference header's include guard, so a program that includes
// the reference's graph.h first gets the reference's classes and this file
// adds nothing.  Semantics kept from the reference:
//   * undirected CSR from an edge list, duplicates and self-loops kept
//     (graph.h:125-153); n = max id + 1;
//   * text loader skipping '#' / '%' lines; weights cast to uint8 (graph.h:300);
//   * id_transfer(rank) relabels so id == rank and sorts every neighbour list
//     in descending (id, weight) order (graph.h:176-206, :367-400).
// Differs on purpose: make_rank() breaks degree ties by ascending id instead
// of the reference's rand()/RAND_MAX jitter (graph.h:156-174), so orders are
// reproducible.
#ifndef INCLUDES_GRAPH_H_
#define INCLUDES_GRAPH_H_

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <numeric>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#ifndef INCLUDES_GLOBALS_H_
#define INCLUDES_GLOBALS_H_
namespace PADO {
typedef uint32_t idi;
typedef uint8_t weighti;
typedef int16_t weightiLarge;
typedef uint8_t smalli;
typedef uint32_t inti;
const uint8_t WEIGHTI_MAX = 255;
const int16_t WEIGHTILARGE_MAX = 32767;
const uint8_t SMALLI_MAX = 255;
}  // namespace PADO
#endif

namespace PADO {

namespace detail {
template <typename W>
inline void csr_from_edges(const std::vector<std::pair<idi, idi>> &edges, const std::vector<W> *weights,
                           idi &num_v, idi &num_e, idi *&vertices, idi *&out_edges, idi *&out_degrees,
                           W *&out_weights)
{
    num_v = 0;
    for (const auto &e : edges) num_v = std::max(num_v, std::max(e.first, e.second) + 1);
    num_e = (idi)(2 * edges.size());
    std::vector<idi> deg(num_v, 0);
    for (const auto &e : edges) {
        ++deg[e.first];
        ++deg[e.second];
    }
    vertices = (idi *)malloc(std::max<size_t>(num_v, 1) * sizeof(idi));
    out_degrees = (idi *)malloc(std::max<size_t>(num_v, 1) * sizeof(idi));
    out_edges = (idi *)malloc(std::max<size_t>(num_e, 1) * sizeof(idi));
    out_weights = weights ? (W *)malloc(std::max<size_t>(num_e, 1) * sizeof(W)) : nullptr;
    idi loc = 0;
    for (idi v = 0; v < num_v; ++v) {
        vertices[v] = loc;
        out_degrees[v] = 0;
        loc += deg[v];
    }
    for (size_t i = 0; i < edges.size(); ++i) {
        const idi u = edges[i].first, v = edges[i].second;
        const idi pu = vertices[u] + out_degrees[u]++;
        out_edges[pu] = v;
        if (weights) out_weights[pu] = (*weights)[i];
        const idi pv = vertices[v] + out_degrees[v]++;
        out_edges[pv] = u;
        if (weights) out_weights[pv] = (*weights)[i];
    }
}

inline std::vector<idi> degree_rank(idi n, const idi *deg)
{
    std::vector<idi> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](idi a, idi b) { return deg[a] > deg[b]; });
    std::vector<idi> rank(n);
    for (idi r = 0; r < n; ++r) rank[order[r]] = r;
    return rank;
}

template <typename W>
inline std::vector<idi> relabel(idi num_v, idi *vertices, idi *out_edges, idi *out_degrees, W *out_weights,
                                const std::vector<idi> &rank)
{
    std::vector<std::vector<std::pair<idi, W>>> lists(num_v);
    for (idi v = 0; v < num_v; ++v)
        for (idi e = vertices[v]; e < vertices[v] + out_degrees[v]; ++e)
            lists[rank[v]].emplace_back(rank[out_edges[e]], out_weights ? out_weights[e] : W());
    idi loc = 0;
    for (idi v = 0; v < num_v; ++v) {
        std::sort(lists[v].rbegin(), lists[v].rend());
        vertices[v] = loc;
        out_degrees[v] = (idi)lists[v].size();
        for (size_t i = 0; i < lists[v].size(); ++i) {
            out_edges[loc + i] = lists[v][i].first;
            if (out_weights) out_weights[loc + i] = lists[v][i].second;
        }
        loc += out_degrees[v];
    }
    std::vector<idi> rank2id(num_v);
    for (idi v = 0; v < num_v; ++v) rank2id[rank[v]] = v;
    return rank2id;
}

inline bool read_edges(const char *filename, bool weighted, std::vector<std::pair<idi, idi>> &edges,
                       std::vector<weighti> &weights)
{
    std::ifstream in(filename);
    if (!in.is_open()) return false;
    std::string line;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#' || line[0] == '%') continue;
        std::istringstream ls(line);
        idi a, b;
        inti w = 0;
        if (!(ls >> a >> b)) continue;
        edges.emplace_back(a, b);
        if (weighted) {
            ls >> w;
            weights.push_back(static_cast<weighti>(w));
        }
    }
    return true;
}
}  // namespace detail

class Graph final {
public:
    idi num_v = 0;
    idi num_e = 0;
    idi *vertices = nullptr;
    idi *out_edges = nullptr;
    idi *out_degrees = nullptr;

    Graph() = default;
    explicit Graph(const char *filename)
    {
        std::vector<std::pair<idi, idi>> edges;
        std::vector<weighti> w;
        if (!detail::read_edges(filename, false, edges, w)) {
            fprintf(stderr, "Error: cannot open file %s\n", filename);
            exit(EXIT_FAILURE);
        }
        construct(edges);
    }
    explicit Graph(std::vector<std::pair<idi, idi>> &edge_list) { construct(edge_list); }
    Graph(const Graph &) = delete;
    Graph &operator=(const Graph &) = delete;
    ~Graph()
    {
        free(vertices);
        free(out_edges);
        free(out_degrees);
    }
    void construct(const std::vector<std::pair<idi, idi>> &edge_list)
    {
        weighti *none = nullptr;
        detail::csr_from_edges<weighti>(edge_list, nullptr, num_v, num_e, vertices, out_edges, out_degrees, none);
    }
    idi get_num_v() const { return num_v; }
    idi get_num_e() const { return num_e; }
    std::vector<idi> make_rank() const { return detail::degree_rank(num_v, out_degrees); }
    std::vector<idi> id_transfer(const std::vector<idi> &rank)
    {
        return detail::relabel<weighti>(num_v, vertices, out_edges, out_degrees, nullptr, rank);
    }
};

class WeightedGraph final {
public:
    idi num_v = 0;
    idi num_e = 0;
    idi *vertices = nullptr;
    idi *out_edges = nullptr;
    idi *out_degrees = nullptr;
    weighti *out_weights = nullptr;

    WeightedGraph() = default;
    explicit WeightedGraph(const char *filename)
    {
        std::vector<std::pair<idi, idi>> edges;
        std::vector<weighti> w;
        if (!detail::read_edges(filename, true, edges, w)) {
            fprintf(stderr, "Error: cannot open file %s\n", filename);
            exit(EXIT_FAILURE);
        }
        construct(edges, w);
    }
    WeightedGraph(const std::vector<std::pair<idi, idi>> &edge_list, const std::vector<weighti> &weight_list)
    {
        construct(edge_list, weight_list);
    }
    WeightedGraph(const WeightedGraph &) = delete;
    WeightedGraph &operator=(const WeightedGraph &) = delete;
    ~WeightedGraph()
    {
        free(vertices);
        free(out_edges);
        free(out_degrees);
        free(out_weights);
    }
    void construct(const std::vector<std::pair<idi, idi>> &edge_list, const std::vector<weighti> &weight_list)
    {
        detail::csr_from_edges<weighti>(edge_list, &weight_list, num_v, num_e, vertices, out_edges, out_degrees,
                                        out_weights);
    }
    idi get_num_v() const { return num_v; }
    idi get_num_e() const { return num_e; }
    std::vector<idi> make_rank() const { return detail::degree_rank(num_v, out_degrees); }
    std::vector<idi> id_transfer(const std::vector<idi> &rank)
    {
        return detail::relabel<weighti>(num_v, vertices, out_edges, out_degrees, out_weights, rank);
    }
};

}  // namespace PADO

#endif  // INCLUDES_GRAPH_H_
