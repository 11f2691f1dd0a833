// ref_vec_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's AVX-512 labeler classes -- the `-v 1` modes of
// pado.cpp (pado.cpp:239-261 unweighted, :297-341 weighted) -- through their
// public API, so that a CPU test can check that they produce the same
// canonical labels as the scalar classes (which the GPU labelers are pinned
// to).  Compiled from the staged, patched copy of the reference headers
// (build_oracle.py) with AVX-512 enabled, on x86 hosts whose CPU has it only:
//   Graph -> id_transfer(rank) (graph.h:176-206)
//   -> VertexCentricPLLVec<B>(G)        (pado_unw_vec_unp.h:56-292)
//      ParaVertexCentricPLLVec<B>(G)    (pado_unw_vec_para.h)
//      WeightedVertexCentricPLLVec<B>(G)      (pado_weighted_vec_unp.h)
//      WeightedParaVertexCentricPLLVec<B>(G)  (pado_weighted_vec_para.h:50-313)
//   -> order_labels(rank2id, rank) -> Index.
// Build with -DPADO_REF_BP_SIZE=<K>.

#include <fcntl.h>
#include <omp.h>
#include <unistd.h>

#include <algorithm>
#include <bitset>
#include <cassert>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdint>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <unordered_map>

#include "ref_prelude.h"

#define private public
#include "globals.h"
#include "graph.h"
#include "pado_unw_vec_unp.h"
#include "pado_unw_vec_para.h"
#include "pado_weighted_vec_unp.h"
#include "pado_weighted_vec_para.h"
#undef private

using namespace PADO;

namespace {

struct QuietStdout {
    int saved = -1;
    QuietStdout()
    {
        fflush(stdout);
        saved = dup(1);
        int nul = open("/dev/null", O_WRONLY);
        if (nul >= 0) { dup2(nul, 1); close(nul); }
    }
    ~QuietStdout()
    {
        fflush(stdout);
        if (saved >= 0) { dup2(saved, 1); close(saved); }
    }
};

template <typename G>
void fill_graph(G &g, uint32_t n, const uint64_t *off, const uint32_t *adj)
{
    g.num_v = n;
    g.num_e = (idi)off[n];
    g.vertices = (idi *)malloc(std::max<size_t>(1, n) * sizeof(idi));
    g.out_degrees = (idi *)malloc(std::max<size_t>(1, n) * sizeof(idi));
    g.out_edges = (idi *)malloc(std::max<size_t>(1, off[n]) * sizeof(idi));
    for (uint32_t v = 0; v < n; ++v) {
        g.vertices[v] = (idi)off[v];
        g.out_degrees[v] = (idi)(off[v + 1] - off[v]);
    }
    for (uint64_t e = 0; e < off[n]; ++e) g.out_edges[e] = adj[e];
}

// Canonical labels of one run: per original vertex, (rank hub, dist) sorted,
// plus the BP rows (unweighted).
struct Result {
    uint32_t n = 0, K = 0;
    std::vector<uint64_t> off;
    std::vector<uint32_t> hub;
    std::vector<int16_t> dist;  // unweighted distances widened
    std::vector<uint8_t> bpd;
    std::vector<uint64_t> bps;
};

template <typename PLL>
void export_index(PLL &p, uint32_t n, uint32_t K, Result &r)
{
    r.n = n;
    r.K = K;
    r.off.assign(n + 1, 0);
    for (uint32_t v = 0; v < n; ++v) r.off[v + 1] = r.off[v] + (p.Index[v].label_id.size() - 1);
    r.hub.resize(r.off[n]);
    r.dist.resize(r.off[n]);
    for (uint32_t v = 0; v < n; ++v) {
        const auto &I = p.Index[v];
        for (uint64_t j = 0; j + 1 < I.label_id.size(); ++j) {
            r.hub[r.off[v] + j] = I.label_id[j];
            r.dist[r.off[v] + j] = (int16_t)I.label_dists[j];
        }
    }
}

template <typename PLL>
void export_bp(PLL &p, uint32_t n, Result &r)
{
    const uint32_t K = PADO_REF_BP_SIZE;
    r.bpd.resize((size_t)n * K);
    r.bps.resize((size_t)n * K * 2);
    for (uint32_t v = 0; v < n; ++v) {
        const auto &I = p.Index[v];
        for (uint32_t i = 0; i < K; ++i) {
            r.bpd[(size_t)v * K + i] = I.bp_dist[i];
            r.bps[((size_t)v * K + i) * 2] = I.bp_sets[i][0];
            r.bps[((size_t)v * K + i) * 2 + 1] = I.bp_sets[i][1];
        }
    }
}

template <inti B>
Result *unw_run(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, int mode)
{
    Result *r = new Result;
    Graph G;
    fill_graph(G, n, off, adj);
    std::vector<idi> rk(rank, rank + n);
    std::vector<idi> rank2id = G.id_transfer(rk);
    QuietStdout q;
    if (mode == 0) {
        VertexCentricPLLVec<B> p(G);
        p.order_labels(rank2id, rk);
        export_index(p, n, PADO_REF_BP_SIZE, *r);
        export_bp(p, n, *r);
    } else {
        ParaVertexCentricPLLVec<B> p(G);
        p.order_labels(rank2id, rk);
        export_index(p, n, PADO_REF_BP_SIZE, *r);
        export_bp(p, n, *r);
    }
    return r;
}

template <inti B>
Result *w_run(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
              int mode)
{
    Result *r = new Result;
    WeightedGraph G;
    fill_graph(G, n, off, adj);
    G.out_weights = (weighti *)malloc(std::max<size_t>(1, off[n]));
    for (uint64_t e = 0; e < off[n]; ++e) G.out_weights[e] = w[e];
    std::vector<idi> rk(rank, rank + n);
    std::vector<idi> rank2id = G.id_transfer(rk);
    QuietStdout q;
    if (mode == 0) {
        WeightedVertexCentricPLLVec<B> p(G);
        p.order_labels(rank2id, rk);
        export_index(p, n, 0, *r);
    } else {
        WeightedParaVertexCentricPLLVec<B> p(G);
        p.order_labels(rank2id, rk);
        export_index(p, n, 0, *r);
    }
    return r;
}

}  // namespace

#define PADO_REFVEC_BATCHES(X) X(64) X(128) X(256) X(512) X(1024)

extern "C" {

void refvec_set_threads(int t)
{
    if (t < 1) t = 1;
    NUM_THREADS = (inti)t;
    omp_set_num_threads(t);
}

// mode 0: the sequential Vec class, 1: the OpenMP Vec class.  NULL for an
// unsupported batch size.
void *refvec_unw_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, uint32_t B,
                       int mode)
{
    switch (B) {
#define X(b) case b: return unw_run<b>(n, off, adj, rank, mode);
        PADO_REFVEC_BATCHES(X)
#undef X
    default: return nullptr;
    }
}

void *refvec_w_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
                     uint32_t B, int mode)
{
    switch (B) {
#define X(b) case b: return w_run<b>(n, off, adj, w, rank, mode);
        PADO_REFVEC_BATCHES(X)
#undef X
    default: return nullptr;
    }
}

uint64_t refvec_num_labels(void *h) { Result *r = (Result *)h; return r->off[r->n]; }
uint32_t refvec_bp_size(void *h) { return ((Result *)h)->K; }
void refvec_export(void *h, uint64_t *off, uint32_t *hub, int16_t *dist, uint8_t *bpd, uint64_t *bps)
{
    Result *r = (Result *)h;
    memcpy(off, r->off.data(), (r->n + 1) * 8);
    memcpy(hub, r->hub.data(), r->hub.size() * 4);
    memcpy(dist, r->dist.data(), r->dist.size() * 2);
    if (bpd && !r->bpd.empty()) memcpy(bpd, r->bpd.data(), r->bpd.size());
    if (bps && !r->bps.empty()) memcpy(bps, r->bps.data(), r->bps.size() * 8);
}
void refvec_free(void *h) { delete (Result *)h; }

}  // extern "C"
