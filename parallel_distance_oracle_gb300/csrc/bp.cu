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
// over one combined frontier of (slot, vertex) entries.  Per level, kernel 1
// lets each frontier vertex pull S^0 from its same-level neighbours (64-bit OR
// reduction), kernel 2 pushes along child edges, claiming undiscovered vertices
// with a CAS on a 32-bit level array and ORing the sets with 64-bit atomicOr.
// Frontier vertices of degree >= HEAVY are spread over every warp of the grid
// (each warp takes 32-edge chunks and ORs its share atomically); lighter ones
// get one warp each.  OR is order-independent, so rows are bit-identical.
// Per root the adjacency of every reached vertex is streamed twice (sibling and
// child kernels) with a 4 B level lookup per edge; per-vertex state is 20 B.

#include <algorithm>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr uint32_t LV_INF = 255u;
constexpr uint32_t GROUP = 16;       // BP roots labeled concurrently
constexpr uint32_t HEAVY = 4096;     // frontier vertices split over all warps

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

struct Front {
    const uint64_t *light;
    const uint32_t *light_cnt;
    const uint64_t *heavy;
    const uint32_t *heavy_cnt;
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

// Sibling step of level d: S^0[v] |= S^-1[tv] for tv adjacent at the same level.
__global__ void __launch_bounds__(256, 4) bp_sibling_kernel(BpState st, Front f, uint32_t d)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned long long bytes = 0;
    // heavy vertices: every warp takes 32-edge chunks of each
    const uint32_t hc = *f.heavy_cnt;
    for (uint32_t q = 0; q < hc; ++q) {
        const uint64_t ent = f.heavy[q];
        const uint32_t slot = ent_slot(ent), v = ent_v(ent);
        const uint64_t so = (uint64_t)slot * st.n;
        const uint32_t e_end = st.off[v + 1];
        uint64_t acc = 0;
        uint32_t same = 0;
        for (uint32_t e = st.off[v] + gw * 32 + lane; e < e_end; e += nw * 32) {
            const uint32_t tv = st.adj[e];
            if (st.lvl[so + tv] == d) {
                acc |= st.sm1[so + tv];
                ++same;
            }
        }
        acc = warp_or64(acc);
        if (lane == 0 && acc) atomicOr((unsigned long long *)&st.s0[so + v], (unsigned long long)acc);
        if (lane == 0 && gw == 0) bytes += 20 + 8ull * (e_end - st.off[v]);
        bytes += 8ull * same;
    }
    const uint32_t lc = *f.light_cnt;
    for (uint32_t q = gw; q < lc; q += nw) {
        const uint64_t ent = f.light[q];
        const uint32_t slot = ent_slot(ent), v = ent_v(ent);
        const uint64_t so = (uint64_t)slot * st.n;
        uint64_t acc = 0;
        uint32_t same = 0;
        for (uint32_t e = st.off[v] + lane; e < st.off[v + 1]; e += 32) {
            const uint32_t tv = st.adj[e];
            if (st.lvl[so + tv] == d) {
                acc |= st.sm1[so + tv];
                ++same;
            }
        }
        acc = warp_or64(acc);
        if (lane == 0 && acc) st.s0[so + v] |= acc;
        if (lane == 0) bytes += 20 + 8ull * (st.off[v + 1] - st.off[v]);
        bytes += 8ull * same;
    }
    if (st.work && bytes) atomicAdd(&st.work[W_BP_SIB], bytes);
}

__device__ __forceinline__ void bp_child_edge(const BpState &st, uint64_t so, uint32_t slot, uint32_t tv, uint32_t d,
                                              uint64_t a, uint64_t b, uint64_t *next_l, uint32_t *next_l_cnt,
                                              uint64_t *next_h, uint32_t *next_h_cnt, uint32_t *status,
                                              unsigned long long &bytes)
{
    const uint32_t t = st.lvl[so + tv];
    if (t <= d) return;
    if (t == LV_INF) {
        if (d + 1 >= LV_INF) {
            atomicOr(status, ST_LEVEL_OVERFLOW);
            return;
        }
        if (atomicCAS(&st.lvl[so + tv], LV_INF, d + 1) == LV_INF) {
            const uint64_t ent = ((uint64_t)slot << 32) | tv;
            if (st.off[tv + 1] - st.off[tv] >= HEAVY)
                next_h[atomicAdd(next_h_cnt, 1u)] = ent;
            else
                next_l[atomicAdd(next_l_cnt, 1u)] = ent;
            bytes += 16;
        }
    }
    if (a) atomicOr((unsigned long long *)&st.sm1[so + tv], (unsigned long long)a);
    if (b) atomicOr((unsigned long long *)&st.s0[so + tv], (unsigned long long)b);
    bytes += 16;
}

// Child step of level d: claim unreached neighbours for level d+1 and OR the
// parent's sets into every level-(d+1) neighbour.
__global__ void __launch_bounds__(256, 4) bp_child_kernel(BpState st, Front f, uint32_t d, uint64_t *next_l,
                                                       uint32_t *next_l_cnt, uint64_t *next_h, uint32_t *next_h_cnt,
                                                       uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    unsigned long long bytes = 0;
    const uint32_t hc = *f.heavy_cnt;
    for (uint32_t q = 0; q < hc; ++q) {
        const uint64_t ent = f.heavy[q];
        const uint32_t slot = ent_slot(ent), v = ent_v(ent);
        const uint64_t so = (uint64_t)slot * st.n;
        const uint64_t a = st.sm1[so + v], b = st.s0[so + v];
        const uint32_t e_end = st.off[v + 1];
        if (lane == 0 && gw == 0) bytes += 28 + 8ull * (e_end - st.off[v]);
        for (uint32_t e = st.off[v] + gw * 32 + lane; e < e_end; e += nw * 32)
            bp_child_edge(st, so, slot, st.adj[e], d, a, b, next_l, next_l_cnt, next_h, next_h_cnt, status, bytes);
    }
    const uint32_t lc = *f.light_cnt;
    for (uint32_t q = gw; q < lc; q += nw) {
        const uint64_t ent = f.light[q];
        const uint32_t slot = ent_slot(ent), v = ent_v(ent);
        const uint64_t so = (uint64_t)slot * st.n;
        const uint64_t a = st.sm1[so + v], b = st.s0[so + v];
        if (lane == 0) bytes += 28 + 8ull * (st.off[v + 1] - st.off[v]);
        for (uint32_t e = st.off[v] + lane; e < st.off[v + 1]; e += 32)
            bp_child_edge(st, so, slot, st.adj[e], d, a, b, next_l, next_l_cnt, next_h, next_h_cnt, status, bytes);
    }
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
    DBuf<uint64_t> fl0((uint64_t)gsize * n), fl1((uint64_t)gsize * n), fh0((uint64_t)gsize * n),
        fh1((uint64_t)gsize * n);
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
            std::vector<uint64_t> sb, f0l, f0h, f1l, f1h;
            for (uint32_t j = 0; j < slots; ++j) {
                for (const BpSeed &x : seeds[g0 + j]) {
                    ss.push_back(j);
                    sv.push_back(x.v);
                    sl.push_back(x.lvl);
                    sb.push_back(x.bits);
                    const uint64_t ent = ((uint64_t)j << 32) | x.v;
                    const bool heavy = hg.off[x.v + 1] - hg.off[x.v] >= HEAVY;
                    if (x.lvl == 0)
                        (heavy ? f0h : f0l).push_back(ent);
                    else
                        (heavy ? f1h : f1l).push_back(ent);
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
            uint64_t *cur_l = fl0.p, *cur_h = fh0.p, *nxt_l = fl1.p, *nxt_h = fh1.p;
            fl0.upload(f0l.data(), f0l.size(), s);
            fh0.upload(f0h.data(), f0h.size(), s);
            fl1.upload(f1l.data(), f1l.size(), s);
            fh1.upload(f1h.data(), f1h.size(), s);
            uint32_t init_cnt[4] = {(uint32_t)f0l.size(), (uint32_t)f0h.size(), (uint32_t)f1l.size(),
                                    (uint32_t)f1h.size()};
            PADO_CUDA(cudaMemcpyAsync(cnts.p, init_cnt, sizeof(init_cnt), cudaMemcpyHostToDevice, s));
            uint32_t *cc = cnts.p, *nc = cnts.p + 2;  // [light, heavy] counts of current / next
            uint32_t fsize = (uint32_t)(f0l.size() + f0h.size());
            for (uint32_t d = 0; fsize > 0; ++d) {
                Front f{cur_l, cc, cur_h, cc + 1};
                PADO_LAUNCH("bp_sibling_kernel", s, bp_sibling_kernel<<<level_grid, 256, 0, s>>>(st, f, d));
                PADO_LAUNCH("bp_child_kernel", s,
                            bp_child_kernel<<<level_grid, 256, 0, s>>>(st, f, d, nxt_l, nc, nxt_h, nc + 1, status.p));
                ++res.levels;
                PADO_CUDA(cudaMemcpyAsync(h_cnt, nc, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaMemcpyAsync(h_cnt + 2, status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaMemsetAsync(cc, 0, 2 * sizeof(uint32_t), s));
                PADO_CUDA(cudaStreamSynchronize(s));
                if (h_cnt[2] & ST_LEVEL_OVERFLOW)
                    throw Error(PADO_E_OVERFLOW, "bit-parallel BFS reached level 255 (uint8 distance overflow)");
                fsize = h_cnt[0] + h_cnt[1];
                std::swap(cur_l, nxt_l);
                std::swap(cur_h, nxt_h);
                std::swap(cc, nc);
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
