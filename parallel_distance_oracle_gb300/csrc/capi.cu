// capi.cu -- the C ABI (include/pado_gpu.h): index handles, host-side graph
// relabeling, export/import, queries and the reference's index file format.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <fstream>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>

#include "pado_internal.cuh"

struct pado_index {
    uint32_t kind = PADO_UNWEIGHTED;
    uint32_t n = 0, K = 0, B = 0;
    int device = 0;
    pado::DBuf<uint32_t> rank;   // original id -> rank (empty: identity)
    pado::LabelStore store;      // rank-indexed canonical labels
    pado::DBuf<uint8_t> bpd;     // n * K, rank-indexed
    pado::DBuf<uint64_t> bps;    // n * K * 2
    pado_info info{};
    // page-locked copies while the device arrays are offloaded
    bool offloaded = false;
    struct Host {
        pado::HBuf<uint32_t> rank, hub;
        pado::HBuf<uint64_t> off, bps;
        pado::HBuf<uint8_t> dist8, bpd;
        pado::HBuf<int16_t> dist16;
    } host;

    pado::IndexView view() const
    {
        pado::IndexView v;
        v.n = n;
        v.K = K;
        v.rank = rank.n ? rank.p : nullptr;
        v.off = store.off.p;
        v.hub = store.hub.p;
        v.dist8 = store.dist8.p;
        v.dist16 = store.dist16.p;
        v.bpd = bpd.p;
        v.bps = bps.p;
        return v;
    }
    uint64_t device_bytes() const
    {
        return rank.bytes() + store.off.bytes() + store.hub.bytes() + store.dist8.bytes() + store.dist16.bytes() +
               bpd.bytes() + bps.bytes();
    }
};

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

template <typename F>
int guarded(F &&f)
{
    try {
        f();
        return PADO_OK;
    } catch (const pado::Error &e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc &) {
        return fail(PADO_E_NOMEM, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(PADO_E_CUDA, e.what());
    }
}

// Set on threads that already run one of several parallel workers (the
// union builder's): their loops stay serial instead of spawning threads of
// their own.
thread_local bool t_serial = false;

// Run f(lo, hi) over [0, n) on the host's cores (plain threads, no OpenMP).
template <typename F>
void parallel_ranges(uint32_t n, F &&f)
{
    unsigned T = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096 || T == 1 || t_serial) {
        f(0u, n);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned i = 0; i < T; ++i) {
        uint32_t lo = (uint32_t)((uint64_t)n * i / T), hi = (uint32_t)((uint64_t)n * (i + 1) / T);
        th.emplace_back([&, lo, hi] { f(lo, hi); });
    }
    for (auto &t : th) t.join();
}

void check_graph(uint32_t n, const uint64_t *off, const uint32_t *adj)
{
    PADO_CHECK(off != nullptr, PADO_E_ARG, "null offsets");
    PADO_CHECK(off[0] == 0, PADO_E_ARG, "off[0] must be 0");
    for (uint32_t v = 0; v < n; ++v) PADO_CHECK(off[v + 1] >= off[v], PADO_E_ARG, "offsets must be non-decreasing");
    PADO_CHECK(off[n] < (1ull << 32), PADO_E_ARG, "more than 2^32-1 adjacency entries");
    PADO_CHECK(off[n] == 0 || adj != nullptr, PADO_E_ARG, "null adjacency");
    std::atomic<bool> bad{false};
    parallel_ranges(n, [&](uint32_t lo, uint32_t hi) {
        for (uint64_t e = off[lo]; e < off[hi]; ++e)
            if (adj[e] >= n) {
                bad = true;
                return;
            }
    });
    PADO_CHECK(!bad, PADO_E_ARG, "adjacency id out of range");
}

void check_rank(uint32_t n, const uint32_t *rank)
{
    PADO_CHECK(rank != nullptr || n == 0, PADO_E_ARG, "null rank");
    std::vector<uint8_t> seen(n, 0);
    for (uint32_t v = 0; v < n; ++v) {
        PADO_CHECK(rank[v] < n && !seen[rank[v]], PADO_E_ARG, "rank is not a permutation of 0..n-1");
        seen[rank[v]] = 1;
    }
}

void upload_graph(const pado::HostGraph &hg, pado::DevGraph &g, bool weighted, cudaStream_t s)
{
    g.n = hg.n;
    g.m = hg.m();
    g.off.alloc(hg.n + 1);
    g.off.upload(hg.off.data(), hg.n + 1, s);
    g.adj.alloc(std::max<uint64_t>(g.m, 1));
    g.adj.upload(hg.adjp(), g.m, s);
    if (weighted) {
        g.w.alloc(std::max<uint64_t>(g.m, 1));
        g.w.upload(hg.wp(), g.m, s);
    }
}

// Builds the labels of a rank-relabeled graph already on the device into h
// (kind, sizes and, where the input was not ranked, h->rank set by the
// caller).  `hg` holds the offsets and at least the adjacency of the ids the
// bit-parallel root selection reads.
template <typename Phase>
void label_into(pado_index *h, const pado::HostGraph &hg, const pado::DevGraph &g, uint32_t K, uint32_t B,
                cudaStream_t s, Phase &&phase)
{
    const uint32_t n = hg.n;
    pado::LabelRun run;
    if (h->kind == PADO_UNWEIGHTED) {
        std::vector<uint8_t> used(n, 0);
        h->bpd.alloc(std::max<uint64_t>((uint64_t)n * K, 1));
        h->bps.alloc(std::max<uint64_t>((uint64_t)n * K * 2, 1));
        pado::BpResult bp = pado::bp_label(hg, g, K, used, h->bpd.p, h->bps.p, s);
        phase("bit-parallel");
        run = pado::unw_label(g, K, B, used, h->bpd.p, h->bps.p, h->store, s);
        phase("labeling");
        h->info.bp_seconds = bp.ms * 1e-3;
        h->info.build_seconds = (bp.ms + run.ms) * 1e-3;
        h->info.levels = run.levels + bp.levels;
    } else {
        run = pado::w_label(g, B, h->store, s);
        phase("labeling");
        h->info.build_seconds = run.ms * 1e-3;
        h->info.levels = run.levels;
    }
    PADO_CUDA(cudaStreamSynchronize(s));
    h->info.n = n;
    h->info.kind = h->kind;
    h->info.bp_roots = h->K;
    h->info.batch = B;
    h->info.num_labels = h->store.total;
    h->info.batches = run.batches;
    h->info.device_bytes = h->device_bytes();
}

// PADO_TRACE=1: host phases of a build on stderr.
struct PhaseTrace {
    bool on = std::getenv("PADO_TRACE") != nullptr;
    std::chrono::steady_clock::time_point prev = std::chrono::steady_clock::now();
    void operator()(const char *what)
    {
        if (!on) return;
        const auto t = std::chrono::steady_clock::now();
        fprintf(stderr, "build %s %.3f ms\n", what, std::chrono::duration<double, std::milli>(t - prev).count());
        prev = t;
    }
};

struct StreamGuard {
    cudaStream_t s = nullptr;
    StreamGuard() { PADO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~StreamGuard() { cudaStreamDestroy(s); }
};

void check_build_args(uint32_t K, uint32_t B)
{
    PADO_CHECK(B >= 1 && B <= pado::MAX_BATCH, PADO_E_ARG, "batch size must be in [1, 2048]");
    PADO_CHECK(K <= pado::MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");
}

// Argument checks first: a bad call fails before touching the device.
std::unique_ptr<pado_index> new_index(bool weighted, uint32_t n, uint32_t K, uint32_t B)
{
    check_build_args(K, B);
    std::unique_ptr<pado_index> h(new pado_index);
    PADO_CUDA(cudaGetDevice(&h->device));
    h->kind = weighted ? PADO_WEIGHTED : PADO_UNWEIGHTED;
    h->n = n;
    h->K = weighted ? 0 : K;
    h->B = B;
    return h;
}

int build_common(bool weighted, uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w,
                 const uint32_t *rank, uint32_t K, uint32_t B, pado_index **out)
{
    if (!out) return fail(PADO_E_ARG, "null output handle");
    *out = nullptr;
    return guarded([&] {
        PhaseTrace phase;
        check_build_args(K, B);
        PADO_CHECK(off != nullptr, PADO_E_ARG, "null offsets");
        PADO_CHECK(off[0] == 0, PADO_E_ARG, "off[0] must be 0");
        PADO_CHECK(off[n] < (1ull << 32), PADO_E_ARG, "more than 2^32-1 adjacency entries");
        PADO_CHECK(off[n] == 0 || adj != nullptr, PADO_E_ARG, "null adjacency");
        PADO_CHECK(!weighted || w != nullptr || off[n] == 0, PADO_E_ARG, "null weights");
        std::unique_ptr<pado_index> h = new_index(weighted, n, K, B);
        StreamGuard sg;
        const cudaStream_t s = sg.s;
        // upload, check and (when needed) relabel and sort on the device
        pado::DevGraph g = pado::prepare_csr(n, off, adj, weighted ? w : nullptr, rank, s, &h->rank);
        phase("prepare");
        // root selection reads the offsets and a prefix of the adjacency
        // (see build_ingested); only those come back to the host
        pado::HostGraph hg;
        hg.n = n;
        hg.off.resize((uint64_t)n + 1);
        g.off.download(hg.off.data(), (uint64_t)n + 1, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        if (!weighted && h->K) {
            const uint32_t R = (uint32_t)std::min<uint64_t>(n, 65ull * h->K);
            hg.adj.resize(hg.off[R]);
            g.adj.download(hg.adj.data(), hg.off[R], s);
            PADO_CUDA(cudaStreamSynchronize(s));
        }
        phase("host view");
        label_into(h.get(), hg, g, h->K, B, s, phase);
        *out = h.release();
    });
}

// Labels the graph that ingest_edges made (ranked CSR on the device) and
// installs its order, so queries take original ids.
void build_ingested(pado_index *h, pado::IngestResult &r, uint32_t K, uint32_t B, cudaStream_t s, PhaseTrace &phase)
{
    const uint32_t n = r.n;
    h->n = n;
    PADO_CHECK(n < 0xffffffffu, PADO_E_ARG, "too many vertices");
    pado::DevGraph g;
    g.n = n;
    g.m = r.m;
    g.off = std::move(r.off);
    g.adj = std::move(r.adj);
    g.w = std::move(r.w);
    // Root selection reads the lists of the first roots and their neighbours
    // only: root i is the smallest id no earlier root or selected neighbour
    // took, so every root id is below 65 * K.  The offsets and only that
    // prefix of the adjacency come to the host.
    pado::HostGraph hg;
    hg.n = n;
    hg.off.resize((uint64_t)n + 1);
    g.off.download(hg.off.data(), (uint64_t)n + 1, s);
    PADO_CUDA(cudaStreamSynchronize(s));
    if (h->kind == PADO_UNWEIGHTED && h->K) {
        const uint32_t R = (uint32_t)std::min<uint64_t>(n, 65ull * h->K);
        hg.adj.resize(hg.off[R]);
        g.adj.download(hg.adj.data(), hg.off[R], s);
    }
    h->rank = std::move(r.rank);
    PADO_CUDA(cudaStreamSynchronize(s));
    phase("upload");
    label_into(h, hg, g, h->K, B, s, phase);
}

using pado::download_bytes;
using pado::mapped_host;

// Export in original-id order: vertex v takes the list (and BP row) of rank[v].
__global__ void __launch_bounds__(256) export_permute_kernel(uint32_t n, uint32_t K, int bp, const uint32_t *rank,
                                                             const uint64_t *roff, const uint64_t *noff,
                                                             const uint32_t *hub, const uint8_t *dist, uint32_t dsz,
                                                             const uint8_t *bpd, const uint64_t *bps, uint32_t *ohub,
                                                             uint8_t *odist, uint8_t *obpd, uint64_t *obps)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < n; v += nw) {
        const uint32_t r = rank[v];
        const uint64_t b = roff[r], len = roff[r + 1] - b, o = noff[v];
        for (uint64_t j = lane; j < len; j += 32) ohub[o + j] = hub[b + j];
        for (uint64_t j = lane; j < len * dsz; j += 32) odist[o * dsz + j] = dist[b * dsz + j];
        if (bp) {
            for (uint32_t i = lane; i < K; i += 32) obpd[(uint64_t)v * K + i] = bpd[(uint64_t)r * K + i];
            for (uint32_t i = lane; i < 2 * K; i += 32) obps[(uint64_t)v * K * 2 + i] = bps[(uint64_t)r * K * 2 + i];
        }
    }
}

// One graph's share of the union label store, BP rows and ranks, and the
// graph's own buffers they are copied into.
struct SplitDesc {
    uint64_t l0, tot;   // its labels: union entries [l0, l0 + tot)
    uint32_t base, ng;  // its vertices: union ids [base, base + ng)
    uint64_t *off;      // ng + 1 offsets, rebased to l0
    uint32_t *hub;
    uint8_t *dist8;
    uint8_t *bpd;       // ng * K
    uint64_t *bps;      // ng * K * 2
    uint32_t *rank;     // ng entries, or null
};

// The union's label offsets at the graph boundaries: bnd[i] = aoff[gbase[i]].
__global__ void split_bounds_kernel(const uint64_t *__restrict__ aoff, const uint32_t *__restrict__ gbase,
                                    uint32_t G, uint64_t *__restrict__ bnd)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= G) bnd[i] = aoff[gbase[i]];
}

// All graphs' copies in one launch: the blocks of grid row y copy graph y's
// slices, striding over its elements together.
__global__ void __launch_bounds__(256) split_many_kernel(const SplitDesc *__restrict__ ds, uint32_t K,
                                                         const uint64_t *__restrict__ aoff,
                                                         const uint32_t *__restrict__ ahub,
                                                         const uint8_t *__restrict__ adist,
                                                         const uint8_t *__restrict__ abpd,
                                                         const uint64_t *__restrict__ abps,
                                                         const uint32_t *__restrict__ arank)
{
    const SplitDesc d = ds[blockIdx.y];
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t st = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = t; i <= d.ng; i += st) d.off[i] = aoff[d.base + i] - d.l0;
    for (uint64_t i = t; i < d.tot; i += st) {
        d.hub[i] = ahub[d.l0 + i];
        d.dist8[i] = adist[d.l0 + i];
    }
    const uint64_t nb = (uint64_t)d.ng * K, b0 = (uint64_t)d.base * K;
    for (uint64_t i = t; i < nb; i += st) d.bpd[i] = abpd[b0 + i];
    for (uint64_t i = t; i < 2 * nb; i += st) d.bps[i] = abps[2 * b0 + i];
    if (d.rank)
        for (uint64_t i = t; i < d.ng; i += st) d.rank[i] = arank[d.base + i];
}

// Many graphs laid side by side: graph i relabeled by its rank and shifted to
// ids [gbase[i], gbase[i+1]).
struct UnionGraph {
    pado::HostGraph hg;
    std::vector<uint32_t> gbase;
};

UnionGraph union_graph(uint32_t G, const uint32_t *n, const uint64_t *const *off, const uint32_t *const *adj,
                       const uint32_t *const *rank, const std::vector<uint32_t> &pick)
{
    UnionGraph u;
    u.gbase.assign(pick.size() + 1, 0);
    uint64_t N = 0, M = 0;
    for (size_t i = 0; i < pick.size(); ++i) {
        const uint32_t gi = pick[i];
        PADO_CHECK(gi < G, PADO_E_ARG, "graph index out of range");
        PADO_CHECK(off[gi] != nullptr, PADO_E_ARG, "null offsets");
        N += n[gi];
        M += n[gi] ? off[gi][n[gi]] : 0;
        PADO_CHECK(N < (1ull << 32) - 1, PADO_E_ARG, "more than 2^32-2 vertices in all graphs together");
        PADO_CHECK(M < (1ull << 32), PADO_E_ARG, "more than 2^32-1 adjacency entries in all graphs together");
        u.gbase[i + 1] = (uint32_t)N;
    }
    pado::HostGraph &hg = u.hg;
    hg.n = (uint32_t)N;
    hg.off.assign(N + 1, 0);
    hg.adj.resize(M);
    std::vector<uint32_t> abase(pick.size() + 1, 0);
    for (size_t i = 0; i < pick.size(); ++i) abase[i + 1] = abase[i] + (n[pick[i]] ? (uint32_t)off[pick[i]][n[pick[i]]] : 0);
    // relabel the graphs on the host's cores, several graphs per thread
    const unsigned T = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    std::vector<std::string> errs(T);
    for (unsigned t = 0; t < T; ++t)
        th.emplace_back([&, t] {
            t_serial = true;
            try {
                for (size_t i = t; i < pick.size(); i += T) {
                    const uint32_t gi = pick[i], ng = n[gi], base = u.gbase[i];
                    check_graph(ng, off[gi], adj[gi]);
                    if (rank && rank[gi]) check_rank(ng, rank[gi]);
                    pado::HostGraph one = pado::relabel_host(ng, off[gi], adj[gi], nullptr, rank ? rank[gi] : nullptr);
                    for (uint32_t v = 0; v < ng; ++v) hg.off[base + v + 1] = abase[i] + one.off[v + 1];
                    const uint32_t *oa = one.adjp();
                    for (uint64_t k = 0; k < one.m(); ++k) hg.adj[abase[i] + k] = oa[k] + base;
                }
            } catch (const std::exception &e) {
                errs[t] = e.what();
            }
        });
    for (auto &x : th) x.join();
    for (auto &e : errs) PADO_CHECK(e.empty(), PADO_E_ARG, e);
    return u;
}

// BP rows and batched labels of a union, all on the device.
struct ManyRun {
    pado::DevGraph g;
    pado::DBuf<uint8_t> bpd;
    pado::DBuf<uint64_t> bps;
    std::vector<uint8_t> used;
    float bp_ms = 0.f;
    uint32_t bp_levels = 0;
};

void many_bp(const UnionGraph &u, uint32_t K, ManyRun &r, cudaStream_t s)
{
    const uint32_t N = u.hg.n;
    upload_graph(u.hg, r.g, false, s);
    r.used.assign(N, 0);
    r.bpd.alloc(std::max<uint64_t>((uint64_t)N * K, 1));
    r.bps.alloc(std::max<uint64_t>((uint64_t)N * K * 2, 1));
    std::vector<std::vector<pado::BpSeed>> seeds;
    if (K)
        for (size_t i = 0; i + 1 < u.gbase.size(); ++i) pado::bp_select(u.hg, u.gbase[i], u.gbase[i + 1], K, r.used, seeds);
    pado::BpResult bp = pado::bp_run(u.hg, r.g, K, seeds, r.bpd.p, r.bps.p, s);
    r.bp_ms = bp.ms;
    r.bp_levels = bp.levels;
}

}  // namespace

namespace pado {

int set_error(int code, const std::string &msg) { return fail(code, msg); }

bool index_resident(const pado_index *h) { return !h->offloaded; }
uint64_t index_device_bytes(const pado_index *h) { return h->info.device_bytes; }

namespace {
template <typename T>
void to_host(DBuf<T> &d, HBuf<T> &hb, cudaStream_t s)
{
    hb.alloc(d.n);
    d.download(hb.p, d.n, s);
}
}  // namespace

void index_offload(pado_index *h, cudaStream_t s)
{
    if (h->offloaded) return;
    auto &H = h->host;
    to_host(h->rank, H.rank, s);
    to_host(h->store.off, H.off, s);
    to_host(h->store.hub, H.hub, s);
    to_host(h->store.dist8, H.dist8, s);
    to_host(h->store.dist16, H.dist16, s);
    to_host(h->bpd, H.bpd, s);
    to_host(h->bps, H.bps, s);
    PADO_CUDA(cudaStreamSynchronize(s));
    h->rank.release();
    h->store.off.release();
    h->store.hub.release();
    h->store.dist8.release();
    h->store.dist16.release();
    h->bpd.release();
    h->bps.release();
    h->offloaded = true;
}

void index_reload(pado_index *h, cudaStream_t s)
{
    if (!h->offloaded) return;
    auto &H = h->host;
    auto back = [&](auto &hb, auto &d) {
        d.alloc(hb.n);
        d.upload(hb.p, hb.n, s);
    };
    back(H.rank, h->rank);
    back(H.off, h->store.off);
    back(H.hub, h->store.hub);
    back(H.dist8, h->store.dist8);
    back(H.dist16, h->store.dist16);
    back(H.bpd, h->bpd);
    back(H.bps, h->bps);
    PADO_CUDA(cudaStreamSynchronize(s));
    H.rank.release();
    H.off.release();
    H.hub.release();
    H.dist8.release();
    H.dist16.release();
    H.bpd.release();
    H.bps.release();
    h->offloaded = false;
}
IndexView index_view(const pado_index *h) { return h->view(); }
uint32_t index_kind(const pado_index *h) { return h->kind; }
int index_device(const pado_index *h) { return h->device; }

HostGraph relabel_host(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank)
{
    HostGraph g;
    g.n = n;
    g.off.assign(n + 1, 0);
    const uint64_t m = off[n];
    if (!rank) {
        // already ranked: used in place when every list is in descending
        // (id, weight) order
        std::atomic<bool> sorted{true};
        parallel_ranges(n, [&](uint32_t lo, uint32_t hi) {
            for (uint32_t v = lo; v < hi && sorted; ++v)
                for (uint64_t k = off[v] + 1; k < off[v + 1]; ++k)
                    if (adj[k - 1] < adj[k] || (adj[k - 1] == adj[k] && w && w[k - 1] < w[k])) {
                        sorted = false;
                        break;
                    }
        });
        if (sorted) {
            for (uint32_t v = 0; v <= n; ++v) g.off[v] = (uint32_t)off[v];
            g.adj_view = adj;
            g.w_view = w;
            return g;
        }
    }
    g.adj.resize(m);
    if (w) g.w.resize(m);
    if (rank) {
        for (uint32_t v = 0; v < n; ++v) g.off[rank[v] + 1] = (uint32_t)(off[v + 1] - off[v]);
        for (uint32_t v = 0; v < n; ++v) g.off[v + 1] += g.off[v];
    } else {
        for (uint32_t v = 0; v <= n; ++v) g.off[v] = (uint32_t)off[v];
    }
    parallel_ranges(n, [&](uint32_t lo, uint32_t hi) {
        std::vector<std::pair<uint32_t, uint8_t>> tmp;
        for (uint32_t v = lo; v < hi; ++v) {
            const uint32_t nv = rank ? rank[v] : v;
            const uint64_t b = off[v], e = off[v + 1];
            uint32_t *dst = g.adj.data() + g.off[nv];
            uint8_t *dw = w ? g.w.data() + g.off[nv] : nullptr;
            bool sorted = true;
            for (uint64_t k = b; k < e; ++k) {
                const uint32_t x = rank ? rank[adj[k]] : adj[k];
                dst[k - b] = x;
                if (dw) dw[k - b] = w[k];
                if (k > b) {
                    const uint32_t y = dst[k - b - 1];
                    if (y < x || (y == x && dw && dw[k - b - 1] < dw[k - b])) sorted = false;
                }
            }
            if (sorted) continue;
            // descending (id, weight), as Graph::id_transfer sorts (graph.h:192, :389)
            tmp.resize(e - b);
            for (uint64_t k = 0; k < e - b; ++k) tmp[k] = {dst[k], dw ? dw[k] : (uint8_t)0};
            std::sort(tmp.rbegin(), tmp.rend());
            for (uint64_t k = 0; k < e - b; ++k) {
                dst[k] = tmp[k].first;
                if (dw) dw[k] = tmp[k].second;
            }
        }
    });
    return g;
}

}  // namespace pado

extern "C" {

const char *pado_last_error(void) { return g_err.c_str(); }

const char *pado_status_string(int status)
{
    switch (status) {
    case PADO_OK: return "ok";
    case PADO_E_ARG: return "invalid argument";
    case PADO_E_NOMEM: return "out of memory";
    case PADO_E_CUDA: return "CUDA error";
    case PADO_E_OVERFLOW: return "distance overflow";
    case PADO_E_IO: return "I/O error";
    case PADO_E_TIMEOUT: return "device wait timed out";
    case PADO_E_STATE: return "invalid state";
    default: return "unknown status";
    }
}

const char *pado_version(void) { return "pado-gpu 0.1 sm_103a"; }

int pado_unw_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint32_t *rank, uint32_t bp_roots,
                   uint32_t batch, pado_index **out)
{
    if (!rank && n) return fail(PADO_E_ARG, "null rank");
    return build_common(false, n, off, adj, nullptr, rank, bp_roots, batch, out);
}

int pado_unw_build_ranked(uint32_t n, const uint64_t *off, const uint32_t *adj, uint32_t bp_roots, uint32_t batch,
                          pado_index **out)
{
    return build_common(false, n, off, adj, nullptr, nullptr, bp_roots, batch, out);
}

int pado_w_build(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, const uint32_t *rank,
                 uint32_t batch, pado_index **out)
{
    if (!rank && n) return fail(PADO_E_ARG, "null rank");
    return build_common(true, n, off, adj, w, rank, 0, batch, out);
}

int pado_w_build_ranked(uint32_t n, const uint64_t *off, const uint32_t *adj, const uint8_t *w, uint32_t batch,
                        pado_index **out)
{
    return build_common(true, n, off, adj, w, nullptr, 0, batch, out);
}

namespace {
// Bytes of ingest scratch kept reserved between calls (pado_set_scratch_cache).
std::atomic<uint64_t> g_scratch_keep{0};
uint64_t scratch_keep() { return g_scratch_keep.load(std::memory_order_relaxed); }
}  // namespace

int pado_set_scratch_cache(uint64_t bytes)
{
    return guarded([&] {
        g_scratch_keep.store(bytes, std::memory_order_relaxed);
        pado::release_scratch(bytes);
    });
}

int pado_graph_ingest(uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w, uint32_t n, uint32_t flags,
                      uint64_t *off, uint32_t *adj, uint8_t *w_out, uint32_t *rank, uint64_t *entries)
{
    return guarded([&] {
        PADO_CHECK((flags & ~(uint32_t)PADO_INGEST_DEDUPE) == 0, PADO_E_ARG, "unknown ingest flags");
        PADO_CHECK(m == 0 || (u && v), PADO_E_ARG, "null edge arrays");
        PADO_CHECK(n > 0 || m == 0, PADO_E_ARG, "n must be given (more than the largest id)");
        PADO_CHECK(off && rank && entries && (m == 0 || adj), PADO_E_ARG, "null output array");
        PADO_CHECK(!w || w_out || m == 0, PADO_E_ARG, "null weight output");
        StreamGuard sg;
        const cudaStream_t s = sg.s;
        pado::DBuf<uint32_t> du(std::max<uint64_t>(m, 1)), dv(std::max<uint64_t>(m, 1));
        pado::DBuf<uint8_t> dw(w ? std::max<uint64_t>(m, 1) : 0);
        du.upload(u, m, s);
        dv.upload(v, m, s);
        if (w) dw.upload(w, m, s);
        pado::IngestResult r = pado::ingest_edges(m, du.p, dv.p, w ? dw.p : nullptr, n, flags & PADO_INGEST_DEDUPE, s);
        pado::DBuf<uint64_t> off64((uint64_t)n + 1);
        pado::widen_u32(r.off.p, (uint64_t)n + 1, off64.p, s);
        r.adj.download(adj, r.m, s);
        if (w) r.w.download(w_out, r.m, s);
        off64.download(off, (uint64_t)n + 1, s);
        r.rank.download(rank, n, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        pado::release_scratch(scratch_keep());
        *entries = r.m;
    });
}

int pado_graph_ingest_device(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, const uint8_t *d_w, uint32_t n,
                             uint32_t flags, uint64_t *d_off, uint32_t *d_adj, uint8_t *d_w_out, uint32_t *d_rank,
                             uint64_t *entries, void *stream)
{
    return guarded([&] {
        PADO_CHECK((flags & ~(uint32_t)PADO_INGEST_DEDUPE) == 0, PADO_E_ARG, "unknown ingest flags");
        PADO_CHECK(m == 0 || (d_u && d_v), PADO_E_ARG, "null edge arrays");
        PADO_CHECK(n > 0 || m == 0, PADO_E_ARG, "n must be given (more than the largest id)");
        PADO_CHECK(d_off && d_rank && entries && (m == 0 || d_adj), PADO_E_ARG, "null output array");
        PADO_CHECK(!d_w || d_w_out || m == 0, PADO_E_ARG, "null weight output");
        const cudaStream_t s = (cudaStream_t)stream;
        pado::IngestResult r = pado::ingest_edges(m, d_u, d_v, d_w, n, flags & PADO_INGEST_DEDUPE, s, d_adj, d_w_out);
        pado::widen_u32(r.off.p, (uint64_t)n + 1, d_off, s);
        if (n) PADO_CUDA(cudaMemcpyAsync(d_rank, r.rank.p, (uint64_t)n * 4, cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaStreamSynchronize(s));
        pado::release_scratch(scratch_keep());
        *entries = r.m;
    });
}

int pado_reduce_degree1_device(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t n, uint8_t *d_deleted,
                               uint64_t *d_kept, uint64_t *m_kept, void *stream)
{
    return guarded([&] {
        PADO_CHECK(m == 0 || (d_u && d_v && d_kept), PADO_E_ARG, "null edge array");
        PADO_CHECK(m_kept && (n == 0 || d_deleted), PADO_E_ARG, "null output");
        const cudaStream_t s = (cudaStream_t)stream;
        const pado::ReduceResult r = pado::reduce_degree1(m, d_u, d_v, n, s, d_deleted, d_kept);
        pado::release_scratch(scratch_keep());
        *m_kept = r.kept;
    });
}

int pado_reduce_equivalent_device(uint64_t m, const uint32_t *d_u, const uint32_t *d_v, uint32_t n,
                                  uint8_t *d_redundant, uint32_t *d_new_id, uint64_t *d_kept, uint64_t *m_kept,
                                  uint32_t *n_out, void *stream)
{
    return guarded([&] {
        PADO_CHECK(m == 0 || (d_u && d_v && d_kept), PADO_E_ARG, "null edge array");
        PADO_CHECK(m_kept && n_out && (n == 0 || (d_redundant && d_new_id)), PADO_E_ARG, "null output");
        const cudaStream_t s = (cudaStream_t)stream;
        const pado::ReduceResult r = pado::reduce_equivalent(m, d_u, d_v, n, s, d_redundant, d_new_id, d_kept);
        pado::release_scratch(scratch_keep());
        *m_kept = r.kept;
        *n_out = r.n_out;
    });
}

namespace {

// Host arrays in and out around a device reduction: the edges go up, flags,
// new ids and kept indices come back.
using ReduceRun = std::function<pado::ReduceResult(const uint32_t *, const uint32_t *, uint8_t *, uint32_t *,
                                                     uint64_t *, cudaStream_t)>;

int reduce_host(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *flags, uint32_t *new_id,
                uint64_t *kept, uint64_t *m_kept, const ReduceRun &run)
{
    return guarded([&] {
        PADO_CHECK(m == 0 || (u && v && kept), PADO_E_ARG, "null edge array");
        PADO_CHECK(m_kept && (n == 0 || flags), PADO_E_ARG, "null output");
        PADO_CHECK(m < (1ull << 31), PADO_E_ARG, "at most 2^31 - 1 edges");
        StreamGuard sg;
        const cudaStream_t s = sg.s;
        pado::DBuf<uint32_t> du(std::max<uint64_t>(m, 1)), dv(std::max<uint64_t>(m, 1));
        pado::DBuf<uint8_t> dflag(std::max<uint32_t>(n, 1));
        pado::DBuf<uint32_t> dnid(new_id ? std::max<uint32_t>(n, 1) : 1);
        pado::DBuf<uint64_t> dkept(std::max<uint64_t>(m, 1));
        du.upload(u, m, s);
        dv.upload(v, m, s);
        const pado::ReduceResult r = run(du.p, dv.p, dflag.p, dnid.p, dkept.p, s);
        dflag.download(flags, n, s);
        if (new_id) dnid.download(new_id, n, s);
        dkept.download(kept, r.kept, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        pado::release_scratch(scratch_keep());
        *m_kept = r.kept;
    });
}

}  // namespace

int pado_reduce_degree1(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *deleted,
                        uint64_t *kept, uint64_t *m_kept)
{
    return reduce_host(m, u, v, n, deleted, nullptr, kept, m_kept,
                       [&](const uint32_t *du, const uint32_t *dv, uint8_t *dflag, uint32_t *, uint64_t *dkept,
                           cudaStream_t s) { return pado::reduce_degree1(m, du, dv, n, s, dflag, dkept); });
}

int pado_reduce_equivalent(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint8_t *redundant,
                           uint32_t *new_id, uint64_t *kept, uint64_t *m_kept, uint32_t *n_out)
{
    if (!n_out || (n && !new_id)) return fail(PADO_E_ARG, "null output");
    pado::ReduceResult res;
    const int st = reduce_host(m, u, v, n, redundant, new_id, kept, m_kept,
                               [&](const uint32_t *du, const uint32_t *dv, uint8_t *dflag, uint32_t *dnid,
                                   uint64_t *dkept, cudaStream_t s) {
                                   res = pado::reduce_equivalent(m, du, dv, n, s, dflag, dnid, dkept);
                                   return res;
                               });
    if (st == PADO_OK) *n_out = res.n_out;
    return st;
}

namespace {
int edges_build(bool weighted, uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w, uint32_t n,
                uint32_t flags, uint32_t K, uint32_t B, pado_index **out)
{
    if (!out) return fail(PADO_E_ARG, "null output handle");
    *out = nullptr;
    return guarded([&] {
        PhaseTrace phase;
        PADO_CHECK((flags & ~(uint32_t)PADO_INGEST_DEDUPE) == 0, PADO_E_ARG, "unknown ingest flags");
        PADO_CHECK(m == 0 || (u && v), PADO_E_ARG, "null edge arrays");
        PADO_CHECK(!weighted || w || m == 0, PADO_E_ARG, "null weights");
        std::unique_ptr<pado_index> h = new_index(weighted, n, K, B);
        StreamGuard sg;
        const cudaStream_t s = sg.s;
        pado::IngestResult r;
        {
            pado::DBuf<uint32_t> du(std::max<uint64_t>(m, 1)), dv(std::max<uint64_t>(m, 1));
            pado::DBuf<uint8_t> dw(weighted ? std::max<uint64_t>(m, 1) : 0);
            du.upload(u, m, s);
            dv.upload(v, m, s);
            if (weighted) dw.upload(w, m, s);
            r = pado::ingest_edges(m, du.p, dv.p, weighted ? dw.p : nullptr, n, flags & PADO_INGEST_DEDUPE, s);
        }
        pado::release_scratch(scratch_keep());
        phase("ingest");
        build_ingested(h.get(), r, h->K, B, s, phase);
        *out = h.release();
    });
}
}  // namespace

int pado_unw_build_edges(uint64_t m, const uint32_t *u, const uint32_t *v, uint32_t n, uint32_t flags,
                         uint32_t bp_roots, uint32_t batch, pado_index **out)
{
    return edges_build(false, m, u, v, nullptr, n, flags, bp_roots, batch, out);
}

int pado_w_build_edges(uint64_t m, const uint32_t *u, const uint32_t *v, const uint8_t *w, uint32_t n,
                       uint32_t flags, uint32_t batch, pado_index **out)
{
    return edges_build(true, m, u, v, w, n, flags, 0, batch, out);
}

int pado_build_edge_file(const char *path, uint32_t kind, uint32_t flags, uint32_t bp_roots, uint32_t batch,
                         pado_index **out)
{
    if (!out) return fail(PADO_E_ARG, "null output handle");
    *out = nullptr;
    return guarded([&] {
        PhaseTrace phase;
        PADO_CHECK(kind == PADO_UNWEIGHTED || kind == PADO_WEIGHTED, PADO_E_ARG, "unknown index kind");
        PADO_CHECK((flags & ~(uint32_t)PADO_INGEST_DEDUPE) == 0, PADO_E_ARG, "unknown ingest flags");
        const bool weighted = kind == PADO_WEIGHTED;
        std::unique_ptr<pado_index> h = new_index(weighted, 0, bp_roots, batch);
        StreamGuard sg;
        const cudaStream_t s = sg.s;
        pado::IngestResult r;
        {
            pado::EdgeTextParser p = pado::read_edge_file(path, weighted, s);
            phase("read+parse");
            r = pado::ingest_edges(p.m, p.u.p, p.v.p, weighted ? p.w.p : nullptr, 0, flags & PADO_INGEST_DEDUPE, s);
        }
        pado::release_scratch(scratch_keep());
        phase("ingest");
        build_ingested(h.get(), r, h->K, batch, s, phase);
        *out = h.release();
    });
}

int pado_edge_text_parse(const char *text, uint64_t bytes, uint32_t weighted, uint64_t capacity, uint32_t *u,
                         uint32_t *v, uint8_t *w, uint64_t *m)
{
    return guarded([&] {
        PADO_CHECK(m != nullptr, PADO_E_ARG, "null edge count");
        *m = 0;
        PADO_CHECK(bytes == 0 || text, PADO_E_ARG, "null text");
        PADO_CHECK(capacity == 0 || (u && v && (!weighted || w)), PADO_E_ARG, "null output array");
        StreamGuard sg;
        pado::EdgeTextParser p(weighted != 0, std::min<uint64_t>(pado::edge_bound_for_text(bytes), (1ull << 32) - 1),
                               sg.s);
        // pieces of at most 1 GiB, each ending at a line end
        const uint64_t piece = pado::text_piece_bytes(1ull << 30);
        uint64_t at = 0;
        while (at < bytes) {
            uint64_t end = std::min(bytes, at + piece);
            if (end < bytes) {
                while (end > at && text[end - 1] != '\n') --end;
                PADO_CHECK(end > at, PADO_E_ARG, "a line longer than the parse piece (1 GiB)");
            }
            p.feed(text + at, end - at);
            at = end;
        }
        *m = p.m;
        PADO_CHECK(p.m <= capacity, PADO_E_ARG, "more edges than the output capacity (*m holds the count)");
        p.u.download(u, p.m, sg.s);
        p.v.download(v, p.m, sg.s);
        if (weighted) p.w.download(w, p.m, sg.s);
        PADO_CUDA(cudaStreamSynchronize(sg.s));
    });
}

int pado_unw_build_many(uint32_t G, const uint32_t *n, const uint64_t *const *off, const uint32_t *const *adj,
                        const uint32_t *const *rank, uint32_t bp_roots, uint32_t batch, pado_index **out)
{
    if (!out || (G && (!n || !off || !adj))) return fail(PADO_E_ARG, "null argument");
    for (uint32_t i = 0; i < G; ++i) out[i] = nullptr;
    std::vector<std::unique_ptr<pado_index>> hs(G);
    const int st = guarded([&] {
        PADO_CHECK(G >= 1 && G <= 65535, PADO_E_ARG, "between 1 and 65535 graphs");
        PADO_CHECK(batch >= 1 && batch <= pado::MAX_BATCH, PADO_E_ARG, "batch size must be in [1, 2048]");
        PADO_CHECK(bp_roots <= pado::MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");
        PhaseTrace phase;
        std::vector<uint32_t> pick(G);
        std::iota(pick.begin(), pick.end(), 0u);
        UnionGraph u = union_graph(G, n, off, adj, rank, pick);
        phase("union");
        int dev = 0;
        PADO_CUDA(cudaGetDevice(&dev));
        cudaStream_t s;
        PADO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{s};
        ManyRun r;
        many_bp(u, bp_roots, r, s);
        phase("bit-parallel");
        pado::LabelStore all;
        pado::LabelRun run = pado::unw_label_many(r.g, u.gbase, bp_roots, batch, r.used, r.bpd.p, r.bps.p, all, s);
        phase("labeling");
        // split: label totals at the graph boundaries, one upload of every
        // graph's ranks, then per graph its buffers, and ONE kernel copies
        // every graph's slices (offsets rebased on the device)
        const uint32_t N = u.hg.n;
        const uint32_t K = bp_roots;
        std::vector<uint64_t> bnd(G + 1);
        {
            pado::DBuf<uint32_t> dgb(G + 1);
            pado::DBuf<uint64_t> dbnd(G + 1);
            dgb.upload(u.gbase.data(), G + 1, s);
            PADO_LAUNCH("split_bounds_kernel", s,
                        split_bounds_kernel<<<(G + 256) / 256, 256, 0, s>>>(all.off.p, dgb.p, G, dbnd.p));
            dbnd.download(bnd.data(), G + 1, s);
            PADO_CUDA(cudaStreamSynchronize(s));
        }
        std::vector<uint32_t> rank_all;
        pado::DBuf<uint32_t> drank;
        if (rank) {
            rank_all.assign(std::max<uint32_t>(N, 1), 0);
            for (uint32_t i = 0; i < G; ++i)
                if (rank[i] && n[i]) memcpy(rank_all.data() + u.gbase[i], rank[i], (size_t)n[i] * 4);
            drank.alloc_async(rank_all.size(), s);
            drank.upload(rank_all.data(), rank_all.size(), s);
        }
        std::vector<SplitDesc> desc(G);
        for (uint32_t i = 0; i < G; ++i) {
            const uint32_t base = u.gbase[i], ng = n[i];
            const uint64_t l0 = bnd[i], tot = bnd[i + 1] - l0;
            std::unique_ptr<pado_index> h(new pado_index);
            h->device = dev;
            h->kind = PADO_UNWEIGHTED;
            h->n = ng;
            h->K = K;
            h->B = batch;
            const bool ranked = rank && rank[i];
            if (ranked) h->rank.alloc_async(std::max<uint32_t>(ng, 1), s);
            h->store.total = tot;
            h->store.off.alloc_async(ng + 1, s);
            h->store.hub.alloc_async(std::max<uint64_t>(tot, 1), s);
            h->store.dist8.alloc_async(std::max<uint64_t>(tot, 1), s);
            h->bpd.alloc_async(std::max<uint64_t>((uint64_t)ng * K, 1), s);
            h->bps.alloc_async(std::max<uint64_t>((uint64_t)ng * K * 2, 1), s);
            desc[i] = SplitDesc{l0, tot, base, ng, h->store.off.p, h->store.hub.p, h->store.dist8.p, h->bpd.p,
                                h->bps.p, ranked ? h->rank.p : nullptr};
            h->info.n = ng;
            h->info.kind = PADO_UNWEIGHTED;
            h->info.bp_roots = K;
            h->info.batch = batch;
            h->info.num_labels = tot;
            h->info.batches = (uint32_t)(((uint64_t)ng + batch - 1) / batch);
            h->info.levels = run.levels + r.bp_levels;
            h->info.bp_seconds = r.bp_ms * 1e-3;
            h->info.build_seconds = (r.bp_ms + run.ms) * 1e-3;
            h->info.device_bytes = h->device_bytes();
            hs[i] = std::move(h);
        }
        pado::DBuf<SplitDesc> ddesc;
        ddesc.alloc_async(G, s);
        ddesc.upload(desc.data(), G, s);
        PADO_LAUNCH("split_many_kernel", s,
                    split_many_kernel<<<dim3(16, G), 256, 0, s>>>(ddesc.p, K, all.off.p, all.hub.p, all.dist8.p,
                                                                 r.bpd.p, r.bps.p, rank ? drank.p : nullptr));
        PADO_CUDA(cudaStreamSynchronize(s));  // rank_all, desc and the copies
        phase("split");
    });
    if (st == PADO_OK)
        for (uint32_t i = 0; i < G; ++i) out[i] = hs[i].release();
    return st;
}

int pado_unw_tune_batch(uint32_t G, const uint32_t *n, const uint64_t *const *off, const uint32_t *const *adj,
                        const uint32_t *const *rank, uint32_t bp_roots, const uint32_t *candidates,
                        uint32_t ncand, uint32_t sample, uint32_t *best, float *ms)
{
    if (!best || !candidates || !ncand || (G && (!n || !off || !adj))) return fail(PADO_E_ARG, "null argument");
    return guarded([&] {
        PADO_CHECK(G >= 1 && G <= 65535, PADO_E_ARG, "between 1 and 65535 graphs");
        PADO_CHECK(bp_roots <= pado::MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");
        for (uint32_t c = 0; c < ncand; ++c)
            PADO_CHECK(candidates[c] >= 1 && candidates[c] <= pado::MAX_BATCH, PADO_E_ARG,
                       "batch size must be in [1, 2048]");
        // sample: graphs evenly spaced in size order, both ends included
        std::vector<uint32_t> bysize(G);
        std::iota(bysize.begin(), bysize.end(), 0u);
        std::stable_sort(bysize.begin(), bysize.end(), [&](uint32_t a, uint32_t b) { return n[a] < n[b]; });
        const uint32_t k = sample == 0 || sample >= G ? G : sample;
        std::vector<uint32_t> pick;
        for (uint32_t i = 0; i < k; ++i) pick.push_back(bysize[k == 1 ? G - 1 : (uint64_t)i * (G - 1) / (k - 1)]);
        std::sort(pick.begin(), pick.end());
        pick.erase(std::unique(pick.begin(), pick.end()), pick.end());
        UnionGraph u = union_graph(G, n, off, adj, rank, pick);
        cudaStream_t s;
        PADO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{s};
        ManyRun r;
        many_bp(u, bp_roots, r, s);  // BP rows do not depend on the batch size
        float best_ms = 0.f;
        for (uint32_t c = 0; c < ncand; ++c) {
            pado::LabelStore st;
            pado::LabelRun run = pado::unw_label_many(r.g, u.gbase, bp_roots, candidates[c], r.used, r.bpd.p, r.bps.p,
                                                      st, s);
            if (ms) ms[c] = run.ms;
            if (c == 0 || run.ms < best_ms) {
                best_ms = run.ms;
                *best = candidates[c];
            }
        }
    });
}

int pado_set_order(pado_index *h, const uint32_t *rank)
{
    if (!h) return fail(PADO_E_ARG, "null index");
    if (h->offloaded) return fail(PADO_E_STATE, "index is offloaded to host memory by a serving loop");
    return guarded([&] {
        check_rank(h->n, rank);
        PADO_CUDA(cudaSetDevice(h->device));
        // the calling thread's stream: other streams of the device (a serving
        // loop's, say) keep running
        const cudaStream_t s = cudaStreamPerThread;
        h->rank.alloc(std::max<uint32_t>(h->n, 1));
        h->rank.upload(rank, h->n, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        h->info.device_bytes = h->device_bytes();
    });
}

void pado_free(pado_index *h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    delete h;
}

int pado_get_info(const pado_index *h, pado_info *info)
{
    if (!h || !info) return fail(PADO_E_ARG, "null argument");
    *info = h->info;
    return PADO_OK;
}

int pado_export(const pado_index *h, uint64_t *off, uint32_t *hub, void *dist, uint8_t *bp_dist, uint64_t *bp_sets)
{
    if (!h || !off || (h->store.total && (!hub || !dist))) return fail(PADO_E_ARG, "null argument");
    if (h->offloaded) return fail(PADO_E_STATE, "index is offloaded to host memory by a serving loop");
    return guarded([&] {
        pado::HostPhase ph("export");
        PADO_CUDA(cudaSetDevice(h->device));
        const uint32_t n = h->n, K = h->K;
        const uint64_t tot = h->store.total;
        const size_t dsz = h->kind == PADO_WEIGHTED ? 2 : 1;
        const void *ddist = dsz == 1 ? (const void *)h->store.dist8.p : (const void *)h->store.dist16.p;
        const bool bp = K && (bp_dist || bp_sets);
        cudaStream_t s = cudaStreamPerThread;
        if (!h->rank.n) {
            // ids are ranks: the store is already in export order
            download_bytes(off, h->store.off.p, (uint64_t)(n + 1) * 8, s);
            download_bytes(hub, h->store.hub.p, tot * 4, s);
            download_bytes(dist, ddist, tot * dsz, s);
            if (K && bp_dist) download_bytes(bp_dist, h->bpd.p, (uint64_t)n * K, s);
            if (K && bp_sets) download_bytes(bp_sets, h->bps.p, (uint64_t)n * K * 16, s);
            PADO_CUDA(cudaStreamSynchronize(s));
            return;
        }
        // original-id order: offsets on the host, lists and BP rows gathered on
        // the device, then one copy of each array
        std::vector<uint64_t> roff(n + 1);
        std::vector<uint32_t> rk(n);
        h->store.off.download(roff.data(), n + 1, s);
        h->rank.download(rk.data(), n, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        off[0] = 0;
        for (uint32_t v = 0; v < n; ++v) off[v + 1] = off[v] + (roff[rk[v] + 1] - roff[rk[v]]);
        // a page-locked destination is written by the gather kernel itself
        // (through its device alias); any other goes through a device buffer
        // and one copy
        uint32_t *ohub = tot ? static_cast<uint32_t *>(mapped_host(hub)) : nullptr;
        uint8_t *odist = tot ? static_cast<uint8_t *>(mapped_host(dist)) : nullptr;
        uint8_t *obpd = bp && bp_dist ? static_cast<uint8_t *>(mapped_host(bp_dist)) : nullptr;
        uint64_t *obps = bp && bp_sets ? static_cast<uint64_t *>(mapped_host(bp_sets)) : nullptr;
        pado::DBuf<uint64_t> noff(n + 1);
        pado::DBuf<uint32_t> thub(ohub ? 1 : std::max<uint64_t>(tot, 1));
        pado::DBuf<uint8_t> tdist(odist ? 1 : std::max<uint64_t>(tot * dsz, 1));
        pado::DBuf<uint8_t> tbpd(bp && !obpd ? (uint64_t)n * K : 1);
        pado::DBuf<uint64_t> tbps(bp && !obps ? (uint64_t)n * K * 2 : 1);
        noff.upload(off, n + 1, s);
        if (n)
            PADO_LAUNCH("export_permute_kernel", s,
                        export_permute_kernel<<<pado::grid_for((uint64_t)n * 32, 256), 256, 0, s>>>(
                            n, K, bp ? 1 : 0, h->rank.p, h->store.off.p, noff.p, h->store.hub.p,
                            static_cast<const uint8_t *>(ddist), (uint32_t)dsz, h->bpd.p, h->bps.p,
                            ohub ? ohub : thub.p, odist ? odist : tdist.p, obpd ? obpd : tbpd.p,
                            obps ? obps : tbps.p));
        if (!ohub) thub.download(hub, tot, s);
        if (!odist) tdist.download(static_cast<uint8_t *>(dist), tot * dsz, s);
        if (K && bp_dist && !obpd) tbpd.download(bp_dist, (uint64_t)n * K, s);
        if (K && bp_sets && !obps) tbps.download(bp_sets, (uint64_t)n * K * 2, s);
        PADO_CUDA(cudaStreamSynchronize(s));
    });
}

int pado_import(uint32_t kind, uint32_t n, uint32_t bp_roots, const uint64_t *off, const uint32_t *hub, const void *dist,
                const uint8_t *bp_dist, const uint64_t *bp_sets, pado_index **out)
{
    if (!out || !off) return fail(PADO_E_ARG, "null argument");
    *out = nullptr;
    return guarded([&] {
        PADO_CHECK(kind == PADO_UNWEIGHTED || kind == PADO_WEIGHTED, PADO_E_ARG, "unknown index kind");
        PADO_CHECK(bp_roots <= pado::MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");
        PADO_CHECK(kind == PADO_UNWEIGHTED || bp_roots == 0, PADO_E_ARG, "weighted indexes have no BP roots");
        PADO_CHECK(bp_roots == 0 || (bp_dist && bp_sets), PADO_E_ARG, "null bit-parallel rows");
        PADO_CHECK(off[0] == 0, PADO_E_ARG, "off[0] must be 0");
        for (uint32_t v = 0; v < n; ++v) PADO_CHECK(off[v + 1] >= off[v], PADO_E_ARG, "offsets must be non-decreasing");
        const uint64_t tot = off[n];
        PADO_CHECK(tot == 0 || (hub && dist), PADO_E_ARG, "null labels");
        for (uint32_t v = 0; v < n; ++v)
            for (uint64_t j = off[v]; j < off[v + 1]; ++j) {
                PADO_CHECK(hub[j] < n, PADO_E_ARG, "hub id out of range");
                PADO_CHECK(j == off[v] || hub[j - 1] < hub[j], PADO_E_ARG, "labels must be sorted by hub, unique");
            }
        std::unique_ptr<pado_index> h(new pado_index);
        PADO_CUDA(cudaGetDevice(&h->device));
        h->kind = kind;
        h->n = n;
        h->K = bp_roots;
        h->store.total = tot;
        h->store.off.alloc(n + 1);
        h->store.off.upload(off, n + 1, cudaStreamPerThread);
        h->store.hub.alloc(std::max<uint64_t>(tot, 1));
        h->store.hub.upload(hub, tot, cudaStreamPerThread);
        if (kind == PADO_UNWEIGHTED) {
            h->store.dist8.alloc(std::max<uint64_t>(tot, 1));
            h->store.dist8.upload(static_cast<const uint8_t *>(dist), tot, cudaStreamPerThread);
        } else {
            h->store.dist16.alloc(std::max<uint64_t>(tot, 1));
            h->store.dist16.upload(static_cast<const int16_t *>(dist), tot, cudaStreamPerThread);
        }
        if (bp_roots) {
            h->bpd.alloc((uint64_t)n * bp_roots);
            h->bpd.upload(bp_dist, (uint64_t)n * bp_roots, cudaStreamPerThread);
            h->bps.alloc((uint64_t)n * bp_roots * 2);
            h->bps.upload(bp_sets, (uint64_t)n * bp_roots * 2, cudaStreamPerThread);
        }
        PADO_CUDA(cudaStreamSynchronize(cudaStreamPerThread));  // this thread's stream only
        h->info.n = n;
        h->info.kind = kind;
        h->info.bp_roots = bp_roots;
        h->info.num_labels = tot;
        h->info.device_bytes = h->device_bytes();
        *out = h.release();
    });
}

int pado_query_device(pado_index *h, uint64_t k, const uint32_t *d_a, const uint32_t *d_b, void *d_out, void *stream)
{
    if (!h || (k && (!d_a || !d_b || !d_out))) return fail(PADO_E_ARG, "null argument");
    if (h->offloaded) return fail(PADO_E_STATE, "index is offloaded to host memory by a serving loop");
    return guarded([&] {
        PADO_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        if (h->kind == PADO_UNWEIGHTED)
            pado::launch_query_unw(h->view(), k, d_a, d_b, static_cast<uint8_t *>(d_out), s);
        else
            pado::launch_query_w(h->view(), k, d_a, d_b, static_cast<int16_t *>(d_out), s);
    });
}

namespace {

// Pairs per chunk of the host query path.
constexpr uint64_t QUERY_CHUNK = 1ull << 21;

// The second stream of the chunked host query path: one per device, created
// on first use and kept for the life of the process.
cudaStream_t query_aux_stream(int dev)
{
    static std::mutex mu;
    static std::vector<std::pair<int, cudaStream_t>> streams;
    std::lock_guard<std::mutex> lk(mu);
    for (const auto &e : streams)
        if (e.first == dev) return e.second;
    cudaStream_t s = nullptr;
    PADO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    streams.emplace_back(dev, s);
    return s;
}

void launch_query(const pado_index *h, uint64_t k, const uint32_t *da, const uint32_t *db, void *dout,
                  cudaStream_t s)
{
    if (h->kind == PADO_UNWEIGHTED)
        pado::launch_query_unw(h->view(), k, da, db, static_cast<uint8_t *>(dout), s);
    else
        pado::launch_query_w(h->view(), k, da, db, static_cast<int16_t *>(dout), s);
}

}  // namespace

// Host arrays in, host array out.  Up to QUERY_CHUNK pairs: copy in, one
// launch, copy out.  Beyond that the pairs go in chunks alternating between
// two streams, and chunk c's results are copied out only after chunk c + 1 is
// queued: a copy out to pageable memory returns when it has completed, and
// with the next chunk's kernel already queued on the other stream the GPU
// keeps working while the host copies (and stages the chunk after).
int pado_query(pado_index *h, uint64_t k, const uint32_t *a, const uint32_t *b, void *out)
{
    if (!h || (k && (!a || !b || !out))) return fail(PADO_E_ARG, "null argument");
    if (h->offloaded) return fail(PADO_E_STATE, "index is offloaded to host memory by a serving loop");
    if (!k) return PADO_OK;
    return guarded([&] {
        PADO_CUDA(cudaSetDevice(h->device));
        cudaStream_t s = cudaStreamPerThread;
        const size_t osz = h->kind == PADO_UNWEIGHTED ? 1 : 2;
        void *buf = nullptr;
        PADO_CUDA(cudaMallocAsync(&buf, k * (8 + osz), s));
        uint32_t *da = static_cast<uint32_t *>(buf), *db = da + k;
        unsigned char *dout = reinterpret_cast<unsigned char *>(db + k);
        if (k <= QUERY_CHUNK) {
            try {
                PADO_CUDA(cudaMemcpyAsync(da, a, k * 4, cudaMemcpyHostToDevice, s));
                PADO_CUDA(cudaMemcpyAsync(db, b, k * 4, cudaMemcpyHostToDevice, s));
                launch_query(h, k, da, db, dout, s);
                PADO_CUDA(cudaMemcpyAsync(out, dout, k * osz, cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaFreeAsync(buf, s));
                PADO_CUDA(cudaStreamSynchronize(s));
            } catch (...) {
                cudaFreeAsync(buf, s);
                cudaStreamSynchronize(s);
                throw;
            }
            return;
        }
        cudaStream_t s2 = nullptr;
        cudaEvent_t ev[2] = {nullptr, nullptr};
        try {
            s2 = query_aux_stream(h->device);
            PADO_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
            PADO_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
            PADO_CUDA(cudaEventRecord(ev[0], s));  // the buffer exists for s2 too
            PADO_CUDA(cudaStreamWaitEvent(s2, ev[0], 0));
            const cudaStream_t st[2] = {s, s2};
            const uint64_t nch = (k + QUERY_CHUNK - 1) / QUERY_CHUNK;
            auto back = [&](uint64_t c) {
                const uint64_t lo = c * QUERY_CHUNK, n = std::min(QUERY_CHUNK, k - lo);
                PADO_CUDA(cudaMemcpyAsync(static_cast<unsigned char *>(out) + lo * osz, dout + lo * osz, n * osz,
                                          cudaMemcpyDeviceToHost, st[c & 1]));
            };
            for (uint64_t c = 0; c < nch; ++c) {
                const uint64_t lo = c * QUERY_CHUNK, n = std::min(QUERY_CHUNK, k - lo);
                PADO_CUDA(cudaMemcpyAsync(da + lo, a + lo, n * 4, cudaMemcpyHostToDevice, st[c & 1]));
                PADO_CUDA(cudaMemcpyAsync(db + lo, b + lo, n * 4, cudaMemcpyHostToDevice, st[c & 1]));
                launch_query(h, n, da + lo, db + lo, dout + lo * osz, st[c & 1]);
                if (c) back(c - 1);
            }
            back(nch - 1);
            PADO_CUDA(cudaEventRecord(ev[1], s2));  // s2's chunks are done before the buffer is freed
            PADO_CUDA(cudaStreamWaitEvent(s, ev[1], 0));
            PADO_CUDA(cudaFreeAsync(buf, s));
            PADO_CUDA(cudaStreamSynchronize(s));
        } catch (...) {
            if (s2) cudaStreamSynchronize(s2);
            cudaStreamSynchronize(s);
            cudaFreeAsync(buf, s);
            cudaStreamSynchronize(s);
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            throw;
        }
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    });
}

int pado_store(const pado_index *h, const char *path)
{
    if (!h || !path) return fail(PADO_E_ARG, "null argument");
    if (h->offloaded) return fail(PADO_E_STATE, "index is offloaded to host memory by a serving loop");
    const uint32_t n = h->n, K = h->K;
    const uint64_t tot = h->store.total;
    std::vector<uint64_t> off(n + 1);
    std::vector<uint32_t> hub(std::max<uint64_t>(tot, 1));
    std::vector<uint8_t> dist(std::max<uint64_t>(tot, 1) * (h->kind == PADO_WEIGHTED ? 2 : 1));
    std::vector<uint8_t> bpd((size_t)n * K);
    std::vector<uint64_t> bps((size_t)n * K * 2);
    int st = pado_export(h, off.data(), hub.data(), dist.data(), K ? bpd.data() : nullptr, K ? bps.data() : nullptr);
    if (st != PADO_OK) return st;
    std::ofstream f(path, std::ios::binary);
    if (!f) return fail(PADO_E_IO, std::string("cannot open ") + path);
    f.write(reinterpret_cast<const char *>(&n), 4);
    if (h->kind == PADO_UNWEIGHTED) f.write(reinterpret_cast<const char *>(&K), 4);
    for (uint32_t v = 0; v < n; ++v) {
        for (uint32_t i = 0; i < K; ++i) {
            f.write(reinterpret_cast<const char *>(&bpd[(size_t)v * K + i]), 1);
            f.write(reinterpret_cast<const char *>(&bps[((size_t)v * K + i) * 2]), 16);
        }
        const uint32_t cnt = (uint32_t)(off[v + 1] - off[v]);
        f.write(reinterpret_cast<const char *>(&cnt), 4);
        for (uint64_t j = off[v]; j < off[v + 1]; ++j) {
            f.write(reinterpret_cast<const char *>(&hub[j]), 4);
            if (h->kind == PADO_UNWEIGHTED)
                f.write(reinterpret_cast<const char *>(&dist[j]), 1);
            else
                f.write(reinterpret_cast<const char *>(&dist[j * 2]), 2);
        }
    }
    f.close();
    if (!f) return fail(PADO_E_IO, std::string("write failed: ") + path);
    return PADO_OK;
}

int pado_load(const char *path, uint32_t kind, pado_index **out)
{
    if (!path || !out) return fail(PADO_E_ARG, "null argument");
    *out = nullptr;
    if (kind != PADO_UNWEIGHTED && kind != PADO_WEIGHTED) return fail(PADO_E_ARG, "unknown index kind");
    std::ifstream f(path, std::ios::binary);
    if (!f) return fail(PADO_E_IO, std::string("cannot open ") + path);
    uint32_t n = 0, K = 0;
    auto rd = [&](void *p, size_t sz) { f.read(static_cast<char *>(p), sz); return (bool)f; };
    if (!rd(&n, 4)) return fail(PADO_E_IO, "truncated index header");
    if (kind == PADO_UNWEIGHTED && !rd(&K, 4)) return fail(PADO_E_IO, "truncated index header");
    if (K > pado::MAX_BP) return fail(PADO_E_IO, "index has more than 64 bit-parallel roots");
    std::vector<uint64_t> off(n + 1, 0);
    std::vector<uint32_t> hub;
    std::vector<uint8_t> d8;
    std::vector<int16_t> d16;
    std::vector<uint8_t> bpd((size_t)n * K);
    std::vector<uint64_t> bps((size_t)n * K * 2);
    for (uint32_t v = 0; v < n; ++v) {
        for (uint32_t i = 0; i < K; ++i) {
            if (!rd(&bpd[(size_t)v * K + i], 1) || !rd(&bps[((size_t)v * K + i) * 2], 16))
                return fail(PADO_E_IO, "truncated bit-parallel rows");
        }
        uint32_t cnt = 0;
        if (!rd(&cnt, 4)) return fail(PADO_E_IO, "truncated label count");
        off[v + 1] = off[v] + cnt;
        for (uint32_t j = 0; j < cnt; ++j) {
            uint32_t x;
            if (!rd(&x, 4)) return fail(PADO_E_IO, "truncated labels");
            hub.push_back(x);
            if (kind == PADO_UNWEIGHTED) {
                uint8_t dd;
                if (!rd(&dd, 1)) return fail(PADO_E_IO, "truncated labels");
                d8.push_back(dd);
            } else {
                int16_t dd;
                if (!rd(&dd, 2)) return fail(PADO_E_IO, "truncated labels");
                d16.push_back(dd);
            }
        }
    }
    const void *dist = kind == PADO_UNWEIGHTED ? (const void *)d8.data() : (const void *)d16.data();
    int st = pado_import(kind, n, K, off.data(), hub.data(), dist, K ? bpd.data() : nullptr, K ? bps.data() : nullptr, out);
    if (st == PADO_E_ARG) return fail(PADO_E_IO, std::string("malformed index file: ") + g_err);
    return st;
}

}  // extern "C"
