// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own labeler classes (compiled from a staged, patched
// copy of the reference headers; see build_oracle.py) through their public
// API, so that the tests and the bench can compare against, and time, the
// reference itself:
//   Graph (graph.h:31-92) -> id_transfer(rank) (graph.h:176-206)
//   -> X(G) (the constructor labels the whole graph, e.g.
//      pado_unw_unv_unp.h:260-264) -> order_labels(rank2id, rank)
//      (pado_unw_unv_unp.h:1227-1310) -> query_distance(a, b).
// The reference's Index member is read through the access macro below to
// export the canonical labels; nothing in the reference code is changed by it.
//
// Build with -DPADO_REF_BP_SIZE=<K> (the staged headers take their bit-parallel
// root count from that macro).

#include <fcntl.h>
#include <omp.h>
#include <unistd.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <map>
#include <memory>
#include <unordered_map>
#include <bitset>
#include <cmath>
#include <cassert>
#include <climits>
#include <string>
#include <sstream>

#include "ref_prelude.h"

#define private public
#include "globals.h"
#include "graph.h"
#include "pado_unw_unv_unp.h"
#include "pado_unw_unv_para.201912311607.parallel_bp_labeling.h"
#include "pado_weighted_unv_unp.h"
#include "pado_weighted_unv_para.h"
#undef private

using namespace PADO;

namespace {

// Silence the reference's progress printf()s while it runs.
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

// Fill a reference Graph with the caller's CSR (original ids), both
// directions present.  Graph::construct() would derive the same arrays from an
// edge list; filling them directly keeps isolated top-id vertices.
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

struct UnwResult {
    uint32_t n = 0, K = 0;
    std::vector<uint64_t> off;
    std::vector<uint32_t> hub;
    std::vector<uint8_t> dist, bpd;
    std::vector<uint64_t> bps;
    double seconds = 0;
};

struct WResult {
    uint32_t n = 0;
    std::vector<uint64_t> off;
    std::vector<uint32_t> hub;
    std::vector<int16_t> dist;
    double seconds = 0;
};

template <typename PLL>
void export_unw(PLL &p, uint32_t n, UnwResult &r)
{
    const uint32_t K = PADO_REF_BP_SIZE;
    r.n = n;
    r.K = K;
    r.off.assign(n + 1, 0);
    for (uint32_t v = 0; v < n; ++v) r.off[v + 1] = r.off[v] + (p.Index[v].label_id.size() - 1);
    r.hub.resize(r.off[n]);
    r.dist.resize(r.off[n]);
    r.bpd.resize((size_t)n * K);
    r.bps.resize((size_t)n * K * 2);
    for (uint32_t v = 0; v < n; ++v) {
        const auto &I = p.Index[v];
        for (uint64_t j = 0; j + 1 < I.label_id.size(); ++j) {
            r.hub[r.off[v] + j] = I.label_id[j];
            r.dist[r.off[v] + j] = I.label_dists[j];
        }
        for (uint32_t i = 0; i < K; ++i) {
            r.bpd[(size_t)v * K + i] = I.bp_dist[i];
            r.bps[((size_t)v * K + i) * 2] = I.bp_sets[i][0];
            r.bps[((size_t)v * K + i) * 2 + 1] = I.bp_sets[i][1];
        }
    }
}

template <typename PLL>
void export_w(PLL &p, uint32_t n, WResult &r)
{
    r.n = n;
    r.off.assign(n + 1, 0);
    for (uint32_t v = 0; v < n; ++v) r.off[v + 1] = r.off[v] + (p.Index[v].label_id.size() - 1);
    r.hub.resize(r.off[n]);
    r.dist.resize(r.off[n]);
    for (uint32_t v = 0; v < n; ++v) {
        const auto &I = p.Index[v];
        for (uint64_t j = 0; j + 1 < I.label_id.size(); ++j) {
            r.hub[r.off[v] + j] = I.label_id[j];
            r.dist[r.off[v] + j] = I.label_dists[j];
        }
    }
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <inti B>
UnwResult *unw_run(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, int mode)
{
    UnwResult *r = new UnwResult;
    Graph G;
    fill_graph(G, n, off, adj);
    std::vector<idi> rk(rank, rank + n);
    std::vector<idi> rank2id = G.id_transfer(rk);
    QuietStdout q;
    if (mode == 0) {
        double t0 = now_s();
        VertexCentricPLL<B> p(G);
        r->seconds = now_s() - t0;
        p.order_labels(rank2id, rk);
        export_unw(p, n, *r);
    } else {
        double t0 = now_s();
        ParaVertexCentricPLL<B> p(G);
        r->seconds = now_s() - t0;
        p.order_labels(rank2id, rk);
        export_unw(p, n, *r);
    }
    return r;
}

template <inti B>
WResult *w_run(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
               const uint32_t *rank, int mode)
{
    WResult *r = new WResult;
    WeightedGraph G;
    fill_graph(G, n, off, adj);
    G.out_weights = (weighti *)malloc(std::max<size_t>(1, off[n]));
    for (uint64_t e = 0; e < off[n]; ++e) G.out_weights[e] = w[e];
    std::vector<idi> rk(rank, rank + n);
    std::vector<idi> rank2id = G.id_transfer(rk);
    QuietStdout q;
    if (mode == 0) {
        double t0 = now_s();
        WeightedVertexCentricPLL<B> p(G);
        r->seconds = now_s() - t0;
        p.order_labels(rank2id, rk);
        export_w(p, n, *r);
    } else {
        double t0 = now_s();
        WeightedParaVertexCentricPLL<B> p(G);
        r->seconds = now_s() - t0;
        p.order_labels(rank2id, rk);
        export_w(p, n, *r);
    }
    return r;
}

// Labeling followed by the reference's own index writer, as pado.cpp:186-189
// (unweighted, VertexCentricPLL::store_index_to_file, pado_unw_unv_unp.h:1120-1180)
// and pado.cpp:270-275 (weighted, WeightedVertexCentricPLL::store_index_to_file,
// pado_weighted_unv_unp.h:1639-1676) call it: with the original-id -> rank map.
template <inti B>
void unw_store(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, const char *path)
{
    Graph G;
    fill_graph(G, n, off, adj);
    std::vector<idi> rk(rank, rank + n);
    G.id_transfer(rk);
    QuietStdout q;
    VertexCentricPLL<B> p(G);
    p.store_index_to_file(path, rk);
}

template <inti B>
void w_store(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
             const char *path)
{
    WeightedGraph G;
    fill_graph(G, n, off, adj);
    G.out_weights = (weighti *)malloc(std::max<size_t>(1, off[n]));
    for (uint64_t e = 0; e < off[n]; ++e) G.out_weights[e] = w[e];
    std::vector<idi> rk(rank, rank + n);
    G.id_transfer(rk);
    QuietStdout q;
    WeightedVertexCentricPLL<B> p(G);
    p.store_index_to_file(path, rk);
}

// Partial unweighted run for a bounded CPU-baseline sample: the reference's
// bit-parallel labeling plus its first `nbatches` root batches, called the way
// ParaVertexCentricPLL::construct() calls them
// (pado_unw_unv_para.201912311607.parallel_bp_labeling.h:1740-1895).
template <inti B>
double unw_para_prefix(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank,
                       uint32_t nbatches, uint64_t *labels_out, double *bp_seconds)
{
    Graph G;
    fill_graph(G, n, off, adj);
    std::vector<idi> rk(rank, rank + n);
    G.id_transfer(rk);
    QuietStdout q;
    ParaVertexCentricPLL<B> *p = new ParaVertexCentricPLL<B>();
    p->num_v_ = n;
    p->L.resize(n);
    std::vector<uint8_t> used_bp_roots(n, 0);
    double t0 = now_s();
    p->bit_parallel_labeling(G, p->L, used_bp_roots);
    double t1 = now_s();
    std::vector<idi> active_queue(n);
    idi end_active_queue = 0;
    std::vector<idi> candidate_queue(n);
    idi end_candidate_queue = 0;
    std::vector<typename ParaVertexCentricPLL<B>::ShortIndex> short_index(n);
    std::vector<std::vector<smalli>> dist_matrix(B, std::vector<smalli>(n, SMALLI_MAX));
    std::vector<uint8_t> got_candidates(n, 0);
    std::vector<uint8_t> is_active(n, 0);
    std::vector<idi> once_candidated_queue(n);
    idi end_once_candidated_queue = 0;
    std::vector<uint8_t> once_candidated(n, 0);
    uint32_t nb = std::min<uint32_t>(nbatches, (n + B - 1) / B);
    for (uint32_t b = 0; b < nb; ++b) {
        uint32_t size = std::min<uint32_t>(B, n - b * B);
        p->batch_process(G, b, b * B, size, p->L, used_bp_roots, active_queue, end_active_queue,
                         candidate_queue, end_candidate_queue, short_index, dist_matrix,
                         got_candidates, is_active, once_candidated_queue,
                         end_once_candidated_queue, once_candidated);
    }
    double t2 = now_s();
    uint64_t cnt = 0;
    for (uint32_t v = 0; v < n; ++v) cnt += p->L[v].vertices.size();
    *labels_out = cnt;
    *bp_seconds = t1 - t0;
    delete p;
    return t2 - t0;
}

}  // namespace

#define PADO_REF_BATCHES(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048)

extern "C" {

uint32_t ref_bp_size() { return PADO_REF_BP_SIZE; }

void ref_set_threads(int t)
{
    if (t < 1) t = 1;
    NUM_THREADS = (inti)t;
    omp_set_num_threads(t);
}

// mode 0 = VertexCentricPLL (sequential), 1 = ParaVertexCentricPLL (OpenMP,
// the variant pado.cpp compiles).  Returns NULL for an unsupported batch size.
void *ref_unw_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank,
                    uint32_t B, int mode)
{
    switch (B) {
#define X(b) case b: return unw_run<b>(n, off, adj, rank, mode);
        PADO_REF_BATCHES(X)
#undef X
    default: return nullptr;
    }
}

void *ref_w_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                  const uint32_t *rank, uint32_t B, int mode)
{
    switch (B) {
#define X(b) case b: return w_run<b>(n, off, adj, w, rank, mode);
        PADO_REF_BATCHES(X)
#undef X
    default: return nullptr;
    }
}

double ref_unw_prefix(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank,
                      uint32_t B, uint32_t nbatches, uint64_t *labels_out, double *bp_seconds)
{
    switch (B) {
#define X(b) case b: return unw_para_prefix<b>(n, off, adj, rank, nbatches, labels_out, bp_seconds);
        PADO_REF_BATCHES(X)
#undef X
    default: return -1.0;
    }
}

// The reference's index writers.  0 on success, -1 for an unsupported batch.
int ref_unw_store(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, uint32_t B,
                  const char *path)
{
    switch (B) {
#define X(b) case b: unw_store<b>(n, off, adj, rank, path); return 0;
        PADO_REF_BATCHES(X)
#undef X
    default: return -1;
    }
}

int ref_w_store(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
                uint32_t B, const char *path)
{
    switch (B) {
#define X(b) case b: w_store<b>(n, off, adj, w, rank, path); return 0;
        PADO_REF_BATCHES(X)
#undef X
    default: return -1;
    }
}

// query_distance.cpp:52-75: the reference's loader (load_index_from_file,
// pado_unw_unv_unp.h:1182-1224 with the root count read into a local;
// pado_weighted_unv_unp.h:1678-1711) followed by its query_distance per pair.
// The unweighted file's root count must equal this build's; returns -1 if it
// does not (or the file cannot be opened), else the loaded vertex count.
int64_t ref_unw_load_query(const char *path, uint64_t k, const uint32_t *a, const uint32_t *b, uint8_t *out)
{
    uint32_t hdr[2] = {0, 0};
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    const size_t got = fread(hdr, 4, 2, f);
    fclose(f);
    if (got != 2 || hdr[1] != (uint32_t)PADO_REF_BP_SIZE) return -1;
    QuietStdout q;
    VertexCentricPLL<1024> p;
    p.load_index_from_file(path);
    for (uint64_t i = 0; i < k; ++i) out[i] = p.query_distance(a[i], b[i]);
    return (int64_t)p.num_v_;
}

int64_t ref_w_load_query(const char *path, uint64_t k, const uint32_t *a, const uint32_t *b, int16_t *out)
{
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    fclose(f);
    QuietStdout q;
    WeightedVertexCentricPLL<512> p;
    p.load_index_from_file(path);
    for (uint64_t i = 0; i < k; ++i) out[i] = p.query_distance(a[i], b[i]);
    return (int64_t)p.num_v_;
}

uint64_t ref_unw_num_labels(void *h) { UnwResult *r = (UnwResult *)h; return r->off[r->n]; }
double ref_unw_seconds(void *h) { return ((UnwResult *)h)->seconds; }
void ref_unw_export(void *h, uint64_t *off, uint32_t *hub, uint8_t *dist, uint8_t *bpd, uint64_t *bps)
{
    UnwResult *r = (UnwResult *)h;
    memcpy(off, r->off.data(), (r->n + 1) * 8);
    memcpy(hub, r->hub.data(), r->hub.size() * 4);
    memcpy(dist, r->dist.data(), r->dist.size());
    memcpy(bpd, r->bpd.data(), r->bpd.size());
    memcpy(bps, r->bps.data(), r->bps.size() * 8);
}
void ref_unw_free(void *h) { delete (UnwResult *)h; }

uint64_t ref_w_num_labels(void *h) { WResult *r = (WResult *)h; return r->off[r->n]; }
double ref_w_seconds(void *h) { return ((WResult *)h)->seconds; }
void ref_w_export(void *h, uint64_t *off, uint32_t *hub, int16_t *dist)
{
    WResult *r = (WResult *)h;
    memcpy(off, r->off.data(), (r->n + 1) * 8);
    memcpy(hub, r->hub.data(), r->hub.size() * 4);
    memcpy(dist, r->dist.data(), r->dist.size() * 2);
}
void ref_w_free(void *h) { delete (WResult *)h; }

// The reference's graph preparation: Graph(const char *) / Graph(edge_list)
// (graph.h:95-153) or their weighted forms (graph.h:262-309), the degrees
// make_rank reads, and id_transfer(rank) (graph.h:176-206, :367-400).
struct RefGraph {
    std::unique_ptr<Graph> g;
    std::unique_ptr<WeightedGraph> wg;
    idi n() const { return g ? g->num_v : wg->num_v; }
    idi e() const { return g ? g->num_e : wg->num_e; }
    const idi *deg() const { return g ? g->out_degrees : wg->out_degrees; }
};

void *ref_graph_read(const char *path, int weighted)
{
    RefGraph *r = new RefGraph;
    if (weighted)
        r->wg.reset(new WeightedGraph(path));
    else
        r->g.reset(new Graph(path));
    return r;
}

void *ref_graph_make(uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w)
{
    std::vector<std::pair<idi, idi>> edges(m);
    for (uint64_t e = 0; e < m; ++e) edges[e] = std::make_pair(u[e], v[e]);
    RefGraph *r = new RefGraph;
    if (w) {
        std::vector<weighti> ws(w, w + m);
        r->wg.reset(new WeightedGraph(edges, ws));
    } else {
        r->g.reset(new Graph(edges));
    }
    return r;
}

uint32_t ref_graph_n(void *h) { return ((RefGraph *)h)->n(); }
uint64_t ref_graph_entries(void *h) { return ((RefGraph *)h)->e(); }
void ref_graph_degrees(void *h, uint32_t *deg)
{
    RefGraph *r = (RefGraph *)h;
    memcpy(deg, r->deg(), (size_t)r->n() * 4);
}

// id_transfer(rank), then the relabeled CSR: off[n+1], adj[entries], w[entries].
void ref_graph_transfer(void *h, const uint32_t *rank, uint64_t *off, uint32_t *adj, uint8_t *w)
{
    RefGraph *r = (RefGraph *)h;
    const idi n = r->n();
    std::vector<idi> rk(rank, rank + n);
    const idi *vert, *deg, *out;
    if (r->g) {
        r->g->id_transfer(rk);
        vert = r->g->vertices;
        deg = r->g->out_degrees;
        out = r->g->out_edges;
    } else {
        r->wg->id_transfer(rk);
        vert = r->wg->vertices;
        deg = r->wg->out_degrees;
        out = r->wg->out_edges;
    }
    off[0] = 0;
    for (idi x = 0; x < n; ++x) {
        off[x + 1] = off[x] + deg[x];
        for (idi k = 0; k < deg[x]; ++k) {
            adj[off[x] + k] = out[vert[x] + k];
            if (w && r->wg) w[off[x] + k] = r->wg->out_weights[vert[x] + k];
        }
    }
}

void ref_graph_free(void *h) { delete (RefGraph *)h; }

// The reference's query loop (pado.cpp:105-125 style) over a pair array, on
// a loaded label set: builds a VertexCentricPLL / WeightedVertexCentricPLL
// Index from canonical arrays and calls its query_distance for each pair.
// threads > 1 splits the pairs over OpenMP threads (query_distance only reads
// the Index).  Returns wall seconds of the query loop.
double ref_unw_query(uint32_t n, const uint64_t *off, const uint32_t *hub, const uint8_t *dist,
                     const uint8_t *bpd, const uint64_t *bps, uint64_t k, const uint32_t *a,
                     const uint32_t *b, uint8_t *out, int threads)
{
    const uint32_t K = PADO_REF_BP_SIZE;
    VertexCentricPLL<1024> p;
    p.num_v_ = n;
    p.Index.resize(n);
    for (uint32_t v = 0; v < n; ++v) {
        auto &I = p.Index[v];
        uint64_t c = off[v + 1] - off[v];
        I.label_id.resize(c + 1);
        I.label_dists.resize(c + 1);
        for (uint64_t j = 0; j < c; ++j) {
            I.label_id[j] = hub[off[v] + j];
            I.label_dists[j] = dist[off[v] + j];
        }
        I.label_id[c] = n;
        I.label_dists[c] = WEIGHTI_MAX;
        for (uint32_t i = 0; i < K; ++i) {
            I.bp_dist[i] = bpd[(size_t)v * K + i];
            I.bp_sets[i][0] = bps[((size_t)v * K + i) * 2];
            I.bp_sets[i][1] = bps[((size_t)v * K + i) * 2 + 1];
        }
    }
    double t0 = now_s();
    if (threads <= 1) {
        for (uint64_t i = 0; i < k; ++i) out[i] = p.query_distance(a[i], b[i]);
    } else {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (uint64_t i = 0; i < k; ++i) out[i] = p.query_distance(a[i], b[i]);
    }
    return now_s() - t0;
}

double ref_w_query(uint32_t n, const uint64_t *off, const uint32_t *hub, const int16_t *dist,
                   uint64_t k, const uint32_t *a, const uint32_t *b, int16_t *out, int threads)
{
    WeightedVertexCentricPLL<512> p;
    p.num_v_ = n;
    p.Index.resize(n);
    for (uint32_t v = 0; v < n; ++v) {
        auto &I = p.Index[v];
        uint64_t c = off[v + 1] - off[v];
        I.label_id.resize(c + 1);
        I.label_dists.resize(c + 1);
        for (uint64_t j = 0; j < c; ++j) {
            I.label_id[j] = hub[off[v] + j];
            I.label_dists[j] = dist[off[v] + j];
        }
        I.label_id[c] = n;
        I.label_dists[c] = WEIGHTILARGE_MAX;
    }
    double t0 = now_s();
    if (threads <= 1) {
        for (uint64_t i = 0; i < k; ++i) out[i] = p.query_distance(a[i], b[i]);
    } else {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (uint64_t i = 0; i < k; ++i) out[i] = p.query_distance(a[i], b[i]);
    }
    return now_s() - t0;
}

}  // extern "C"
