// bp.cu -- bit-parallel (BP) labeling on the device.
//
// Restates bit_parallel_labeling (reference includes/pado_unw_unv_unp.h:268-384;
// the OpenMP variant pado_unw_unv_para.201912311607.parallel_bp_labeling.h:545-836
// computes the same rows).  For BP slot i:
//   * root r = smallest unused rank; up to 64 unused neighbours of r, scanned
//     from the end of its descending list (so in ascending id order), get
//     S^-1 = {bit j} in that order and distance 1 (:284-326).  This selection
//     only depends on the adjacency and the used flags, so the host does it for
//     all slots up front, sequentially, exactly as the reference.
//   * BFS by levels d = 0, 1, ...: first every sibling edge (both ends at d)
//     ORs S^-1 of each end into S^0 of the other (:362-366), then every child
//     edge (d -> d+1) ORs the parent's S^-1 / S^0 into the child's (:367-371).
//   * stored row: (d, S^-1, S^0 & ~S^-1) (:377-381); an unused slot (no root
//     left) stores d = 255 and empty sets (:288-292).
// Device mapping: the BFS of up to GROUP roots run together, level by level,
// over one combined frontier of (slot, vertex) entries, and every set update
// is a PULL (an OR reduction over a vertex's own adjacency, stored by the one
// thread that owns the vertex) instead of a per-edge atomic push:
//   bp_level_kernel(d):  each v at level d ORs S^-1 of its level-d neighbours
//       into S^0[v] (the sibling step) and claims its unreached neighbours for
//       level d+1 (CAS on the level array; warp-aggregated appends);
//   bp_parent_kernel(d): each u at level d+1 ORs S^-1 and S^0 of its level-d
//       neighbours (its parents, whose S^0 the previous kernel finished) into
//       its own sets (the child step).
// The child step of the reference pushes parent sets along every d -> d+1
// edge; pulling them over the same edges gives the same ORs.  Frontier
// vertices of degree >= HEAVY are spread over every warp of the grid (partial
// ORs combined with one atomicOr per warp); those of degree <= SMALL_DEG get
// SUB lanes each (8 per warp: most vertices of sparse graphs); the rest get one
// warp each.  OR is order-independent, so rows are bit-identical.  Per root
// the adjacency of every reached vertex is streamed twice with a 4 B level
// lookup per edge; per-vertex state is 20 B.

#include <algorithm>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr uint32_t LV_INF = 255u;
constexpr uint32_t GROUP = 16;       // BP roots labeled concurrently
constexpr uint32_t HEAVY = 4096;     // frontier vertices split over all warps
constexpr uint32_t SMALL_DEG = 16;   // frontier vertices up to this degree share a warp ...
constexpr uint32_t SUB = 4;          // ... SUB lanes each

enum FrontClass : int { FC_LIGHT = 0, FC_HEAVY = 1, FC_SMALL = 2 };

__host__ __device__ __forceinline__ int front_class(uint32_t deg)
{
    return deg >= HEAVY ? FC_HEAVY : (deg <= SMALL_DEG ? FC_SMALL : FC_LIGHT);
}

__device__ __forceinline__ uint64_t warp_or64(uint64_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct BpState {
    uint32_t n;
    uint32_t slots;
    const uint32_t *off;
    const uint32_t *adj;
    uint32_t *lvl;   // [slots][n], LV_INF = unreached
    uint64_t *sm1;   // [slots][n]
    uint64_t *s0;    // [slots][n]
    unsigned long long *work;
};

// Frontier entry: slot << 32 | vertex.
__device__ __forceinline__ uint32_t ent_slot(uint64_t e) { return (uint32_t)(e >> 32); }
__device__ __forceinline__ uint32_t ent_v(uint64_t e) { return (uint32_t)e; }

// A frontier: entry lists by class (FC_*), with their counts.
struct Front {
    const uint64_t *list[3];
    const uint32_t *cnt;  // cnt[FC_*]
};
struct NextFront {
    uint64_t *list[3];
    uint32_t *cnt;
};

__global__ void bp_reset_kernel(BpState st)
{
    const uint64_t tot = (uint64_t)st.slots * st.n;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < tot; i += (uint64_t)gridDim.x * blockDim.x) {
        st.lvl[i] = LV_INF;
        st.sm1[i] = 0;
        st.s0[i] = 0;
    }
}

// seeds: (slot, vertex, level, S^-1) for each root and its selected neighbours.
__global__ void bp_seed_kernel(BpState st, const uint32_t *sslot, const uint32_t *sv, const uint32_t *slv,
                               const uint64_t *sbits, uint32_t cnt)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < cnt) {
        const uint64_t k = (uint64_t)sslot[i] * st.n + sv[i];
        st.lvl[k] = slv[i];
        st.sm1[k] = sbits[i];
    }
}

// Per-entry accumulator of the two pull kernels.
struct BpAcc {
    uint64_t a = 0, b = 0;
    uint32_t hits = 0;
};

// Runs `edge(so, slot, v, tv, acc)` over the adjacency of every frontier entry
// and `fin(so, v, acc, atomic)` once per entry with the entry's OR-reduced
// accumulator (atomic: several warps share the entry, combine with atomicOr).
template <class Edge, class Fin>
__device__ __forceinline__ void bp_pull(const BpState &st, const Front &f, unsigned long long &bytes, Edge edge, Fin fin)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    // heavy vertices: every warp takes 32-edge chunks of each
    const uint32_t hc = f.cnt[FC_HEAVY];
    for (uint32_t q = 0; q < hc; ++q) {
        const uint64_t ent = f.list[FC_HEAVY][q];
        const uint32_t slot = ent_slot(ent), v = ent_v(ent);
        const uint64_t so = (uint64_t)slot * st.n;
        const uint32_t e_end = st.off[v + 1];
        BpAcc acc;
        for (uint32_t e = st.off[v] + gw * 32 + lane; e < e_end; e += nw * 32) edge(so, slot, v, st.adj[e], acc);
        acc.a = warp_or64(acc.a);
        acc.b = warp_or64(acc.b);
        if (lane == 0) fin(so, v, acc, true);
        if (lane == 0 && gw == 0) bytes += 20 + 8ull * (e_end - st.off[v]);
        bytes += 8ull * acc.hits;
    }
    // light vertices: a warp each
    const uint32_t lc = f.cnt[FC_LIGHT];
    for (uint32_t q = gw; q < lc; q += nw) {
        const uint64_t ent = f.list[FC_LIGHT][q];
        const uint32_t slot = ent_slot(ent), v = ent_v(ent);
        const uint64_t so = (uint64_t)slot * st.n;
        const uint32_t e_end = st.off[v + 1];
        BpAcc acc;
        for (uint32_t e = st.off[v] + lane; e < e_end; e += 32) edge(so, slot, v, st.adj[e], acc);
        acc.a = warp_or64(acc.a);
        acc.b = warp_or64(acc.b);
        if (lane == 0) {
            fin(so, v, acc, false);
            bytes += 20 + 8ull * (e_end - st.off[v]);
        }
        bytes += 8ull * acc.hits;
    }
    // small vertices: SUB lanes each, 32 / SUB per warp (warp-uniform loop)
    const uint32_t sc = f.cnt[FC_SMALL];
    const uint32_t per = 32 / SUB, sub = lane % SUB;
    for (uint64_t qb = (uint64_t)gw * per; qb < sc; qb += (uint64_t)nw * per) {
        const uint64_t q = qb + lane / SUB;
        BpAcc acc;
        uint64_t so = 0;
        uint32_t v = 0;
        if (q < sc) {
            const uint64_t ent = f.list[FC_SMALL][q];
            const uint32_t slot = ent_slot(ent);
            v = ent_v(ent);
            so = (uint64_t)slot * st.n;
            const uint32_t e_end = st.off[v + 1];
            for (uint32_t e = st.off[v] + sub; e < e_end; e += SUB) edge(so, slot, v, st.adj[e], acc);
            if (sub == 0) bytes += 20 + 8ull * (e_end - st.off[v]);
        }
#pragma unroll
        for (int o = 1; o < (int)SUB; o <<= 1) {
            acc.a |= __shfl_xor_sync(0xffffffffu, acc.a, o);
            acc.b |= __shfl_xor_sync(0xffffffffu, acc.b, o);
        }
        if (q < sc && sub == 0) fin(so, v, acc, false);
        bytes += 8ull * acc.hits;
    }
}

// Level d: the sibling step (S^0[v] |= S^-1[tv], tv at level d) and the
// discovery of level d+1 (pado_unw_unv_unp.h:362-371).
__global__ void __launch_bounds__(256, 4) bp_level_kernel(BpState st, Front f, uint32_t d, NextFront nx,
                                                          uint32_t *status)
{
    unsigned long long bytes = 0;
    bp_pull(
        st, f, bytes,
        [&](uint64_t so, uint32_t slot, uint32_t, uint32_t tv, BpAcc &acc) {
            const uint32_t l = st.lvl[so + tv];
            if (l == d) {
                acc.a |= st.sm1[so + tv];
                ++acc.hits;
            } else if (l == LV_INF) {
                if (d + 1 >= LV_INF) {
                    atomicOr(status, ST_LEVEL_OVERFLOW);
                } else if (atomicCAS(&st.lvl[so + tv], LV_INF, d + 1) == LV_INF) {
                    const int c = front_class(st.off[tv + 1] - st.off[tv]);
                    nx.list[c][agg_append_by(&nx.cnt[c], (unsigned)c)] = ((uint64_t)slot << 32) | tv;
                    acc.hits += 2;
                }
            }
        },
        [&](uint64_t so, uint32_t v, const BpAcc &acc, bool atomic) {
            if (!acc.a) return;
            if (atomic)
                atomicOr((unsigned long long *)&st.s0[so + v], (unsigned long long)acc.a);
            else
                st.s0[so + v] |= acc.a;
        });
    if (st.work && bytes) atomicAdd(&st.work[W_BP_SIB], bytes);
}

// The child step for the vertices first reached at level d+1: OR the sets of
// their level-d neighbours (pado_unw_unv_unp.h:367-371).
__global__ void __launch_bounds__(256, 4) bp_parent_kernel(BpState st, Front f, uint32_t d)
{
    unsigned long long bytes = 0;
    bp_pull(
        st, f, bytes,
        [&](uint64_t so, uint32_t, uint32_t, uint32_t p, BpAcc &acc) {
            if (st.lvl[so + p] == d) {
                acc.a |= st.sm1[so + p];
                acc.b |= st.s0[so + p];
                acc.hits += 2;
            }
        },
        [&](uint64_t so, uint32_t u, const BpAcc &acc, bool atomic) {
            if (atomic) {
                if (acc.a) atomicOr((unsigned long long *)&st.sm1[so + u], (unsigned long long)acc.a);
                if (acc.b) atomicOr((unsigned long long *)&st.s0[so + u], (unsigned long long)acc.b);
            } else {
                if (acc.a) st.sm1[so + u] |= acc.a;
                if (acc.b) st.s0[so + u] |= acc.b;
            }
        });
    if (st.work && bytes) atomicAdd(&st.work[W_BP_CHILD], bytes);
}

// Rows of slots [0, slots) into BP columns [i0, i0 + slots).
__global__ void bp_store_kernel(BpState st, uint32_t K, uint32_t i0, uint8_t *bpd, uint64_t *bps)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < st.n; v += gridDim.x * blockDim.x) {
        for (uint32_t j = 0; j < st.slots; ++j) {
            const uint64_t k = (uint64_t)j * st.n + v;
            const uint64_t a = st.sm1[k];
            bpd[(uint64_t)v * K + i0 + j] = (uint8_t)st.lvl[k];
            bps[((uint64_t)v * K + i0 + j) * 2] = a;
            bps[((uint64_t)v * K + i0 + j) * 2 + 1] = st.s0[k] & ~a;
        }
    }
}

__global__ void bp_empty_slots_kernel(uint32_t n, uint32_t K, uint32_t i0, uint8_t *bpd, uint64_t *bps)
{
    const uint32_t w = K - i0;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < (uint64_t)n * w;
         x += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t v = x / w, i = i0 + x % w;
        bpd[v * K + i] = U8_INF;
        bps[(v * K + i) * 2] = 0;
        bps[(v * K + i) * 2 + 1] = 0;
    }
}

}  // namespace

void bp_select(const HostGraph &hg, uint32_t lo, uint32_t hi, uint32_t K, std::vector<uint8_t> &used,
               std::vector<std::vector<BpSeed>> &seeds)
{
    // Root and neighbour selection for every slot, in the reference's order
    // (pado_unw_unv_unp.h:284-326), restricted to the ids [lo, hi).
    if (seeds.size() < K) seeds.resize(K);
    uint32_t r = lo;
    for (uint32_t i = 0; i < K; ++i) {
        while (r < hi && used[r]) ++r;
        if (r == hi) break;
        used[r] = 1;
        seeds[i].push_back({r, 0, 0});
        int ns = 0;
        for (uint32_t k = hg.off[r + 1]; k > hg.off[r]; --k) {
            const uint32_t v = hg.adj[k - 1];
            if (!used[v]) {
                used[v] = 1;
                seeds[i].push_back({v, 1, 1ULL << ns});
                if (++ns == 64) break;
            }
        }
    }
}

BpResult bp_label(const HostGraph &hg, const DevGraph &g, uint32_t K, std::vector<uint8_t> &used,
                  uint8_t *d_bpd, uint64_t *d_bps, cudaStream_t s)
{
    std::vector<std::vector<BpSeed>> seeds;
    if (K) bp_select(hg, 0, hg.n, K, used, seeds);
    return bp_run(hg, g, K, seeds, d_bpd, d_bps, s);
}

BpResult bp_run(const HostGraph &hg, const DevGraph &g, uint32_t K, const std::vector<std::vector<BpSeed>> &seeds,
                uint8_t *d_bpd, uint64_t *d_bps, cudaStream_t s)
{
    BpResult res;
    const uint32_t n = hg.n;
    if (K == 0 || n == 0) return res;
    // slots [0, nroots) have a root in at least one graph; a graph with fewer
    // roots gets unreached (255, empty) rows in its remaining slots, which is
    // what the reference stores for a slot without a root (:288-292).
    uint32_t nroots = 0;
    while (nroots < std::min<size_t>(K, seeds.size()) && !seeds[nroots].empty()) ++nroots;

    const uint32_t gsize = std::min<uint32_t>(GROUP, std::max<uint32_t>(nroots, 1));
    DBuf<uint32_t> lvl((uint64_t)gsize * n), cnts(8), status(1);
    DBuf<uint64_t> sm1((uint64_t)gsize * n), s0((uint64_t)gsize * n);
    // frontier lists by class, double-buffered: fr[buffer][class]
    DBuf<uint64_t> fr[2][3];
    for (auto &side : fr)
        for (auto &l : side) l.alloc((uint64_t)gsize * n);
    size_t max_seeds = 1;
    for (uint32_t i = 0; i < nroots; i += gsize) {
        size_t c = 0;
        for (uint32_t j = i; j < std::min(nroots, i + gsize); ++j) c += seeds[j].size();
        max_seeds = std::max(max_seeds, c);
    }
    DBuf<uint32_t> seed_slot(max_seeds), seed_v(max_seeds), seed_l(max_seeds);
    DBuf<uint64_t> seed_b(max_seeds);
    status.fill_bytes(0, s);
    uint32_t *h_cnt = nullptr;
    PADO_CUDA(cudaMallocHost((void **)&h_cnt, 8 * sizeof(uint32_t)));
    cudaEvent_t e0, e1;
    PADO_CUDA(cudaEventCreate(&e0));
    PADO_CUDA(cudaEventCreate(&e1));
    PADO_CUDA(cudaEventRecord(e0, s));
    const unsigned vb = 256;
    const unsigned level_grid = 152u * 8u;
    try {
        for (uint32_t g0 = 0; g0 < nroots; g0 += gsize) {
            const uint32_t slots = std::min(gsize, nroots - g0);
            BpState st{n, slots, g.off.p, g.adj.p, lvl.p, sm1.p, s0.p, work_counters()};
            PADO_LAUNCH("bp_reset_kernel", s, bp_reset_kernel<<<grid_for((uint64_t)slots * n, vb), vb, 0, s>>>(st));
            std::vector<uint32_t> ss, sv, sl;
            std::vector<uint64_t> sb, f0[3], f1[3];
            for (uint32_t j = 0; j < slots; ++j) {
                for (const BpSeed &x : seeds[g0 + j]) {
                    ss.push_back(j);
                    sv.push_back(x.v);
                    sl.push_back(x.lvl);
                    sb.push_back(x.bits);
                    const uint64_t ent = ((uint64_t)j << 32) | x.v;
                    const int c = front_class(hg.off[x.v + 1] - hg.off[x.v]);
                    (x.lvl == 0 ? f0 : f1)[c].push_back(ent);
                }
            }
            seed_slot.upload(ss.data(), ss.size(), s);
            seed_v.upload(sv.data(), sv.size(), s);
            seed_l.upload(sl.data(), sl.size(), s);
            seed_b.upload(sb.data(), sb.size(), s);
            PADO_LAUNCH("bp_seed_kernel", s,
                        bp_seed_kernel<<<grid_for(sv.size(), 128), 128, 0, s>>>(st, seed_slot.p, seed_v.p, seed_l.p,
                                                                              seed_b.p, (uint32_t)sv.size()));
            // frontier 0 = the roots; frontier 1 starts with the selected neighbours
            uint32_t init_cnt[8] = {};
            for (int c = 0; c < 3; ++c) {
                fr[0][c].upload(f0[c].data(), f0[c].size(), s);
                fr[1][c].upload(f1[c].data(), f1[c].size(), s);
                init_cnt[c] = (uint32_t)f0[c].size();
                init_cnt[4 + c] = (uint32_t)f1[c].size();
            }
            PADO_CUDA(cudaMemcpyAsync(cnts.p, init_cnt, sizeof(init_cnt), cudaMemcpyHostToDevice, s));
            int cur = 0;  // fr[cur] / counts cnts[4*cur ..] hold level d
            uint32_t fsize = (uint32_t)(f0[0].size() + f0[1].size() + f0[2].size());
            for (uint32_t d = 0; fsize > 0; ++d) {
                uint32_t *cc = cnts.p + 4 * cur, *nc = cnts.p + 4 * (cur ^ 1);
                Front f{{fr[cur][0].p, fr[cur][1].p, fr[cur][2].p}, cc};
                NextFront nx{{fr[cur ^ 1][0].p, fr[cur ^ 1][1].p, fr[cur ^ 1][2].p}, nc};
                PADO_LAUNCH("bp_level_kernel", s,
                            bp_level_kernel<<<level_grid, 256, 0, s>>>(st, f, d, nx, status.p));
                // the next frontier, complete now, pulls its parents' sets
                const Front fn{{nx.list[0], nx.list[1], nx.list[2]}, nc};
                PADO_LAUNCH("bp_parent_kernel", s, bp_parent_kernel<<<level_grid, 256, 0, s>>>(st, fn, d));
                ++res.levels;
                PADO_CUDA(cudaMemcpyAsync(h_cnt, nc, 3 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaMemcpyAsync(h_cnt + 3, status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaMemsetAsync(cc, 0, 3 * sizeof(uint32_t), s));
                PADO_CUDA(cudaStreamSynchronize(s));
                if (h_cnt[3] & ST_LEVEL_OVERFLOW)
                    throw Error(PADO_E_OVERFLOW, "bit-parallel BFS reached level 255 (uint8 distance overflow)");
                fsize = h_cnt[0] + h_cnt[1] + h_cnt[2];
                cur ^= 1;
            }
            PADO_LAUNCH("bp_store_kernel", s,
                        bp_store_kernel<<<grid_for(n, vb), vb, 0, s>>>(st, K, g0, d_bpd, d_bps));
        }
        if (nroots < K)
            PADO_LAUNCH("bp_empty_slots_kernel", s,
                        bp_empty_slots_kernel<<<grid_for((uint64_t)n * (K - nroots), vb), vb, 0, s>>>(n, K, nroots, d_bpd,
                                                                                                      d_bps));
        PADO_CUDA(cudaEventRecord(e1, s));
        PADO_CUDA(cudaEventSynchronize(e1));
        PADO_CUDA(cudaEventElapsedTime(&res.ms, e0, e1));
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFreeHost(h_cnt);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeHost(h_cnt);
    return res;
}

}  // namespace pado
