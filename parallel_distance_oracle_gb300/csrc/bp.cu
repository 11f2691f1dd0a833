// bp.cu -- bit-parallel (BP) labeling on the device.
//
// Restates bit_parallel_labeling (reference includes/pado_unw_unv_unp.h:268-384;
// the OpenMP variant pado_unw_unv_para.201912311607.parallel_bp_labeling.h:545-836
// computes the same rows).  For BP slot i:
//   * root r = smallest unused rank; up to 64 unused neighbours of r, scanned
//     from the end of its descending list (so in ascending id order), get
//     S^-1 = {bit j} in that order and distance 1 (:284-326).  This selection
//     only depends on the adjacency and the used flags, so the host does it,
//     sequentially, exactly as the reference.
//   * BFS by levels d = 0, 1, ...: first every sibling edge (both ends at d)
//     ORs S^-1 of each end into S^0 of the other (:362-366), then every child
//     edge (d -> d+1) ORs the parent's S^-1 / S^0 into the child's (:367-371).
//   * stored row: (d, S^-1, S^0 & ~S^-1) (:377-381); an unused slot (no root
//     left) stores d = 255 and empty sets (:288-292).
// Device mapping: per level, kernel 1 lets each frontier vertex pull S^0 from
// its same-level neighbours (a warp per vertex, lanes over the adjacency,
// 64-bit OR reduction); kernel 2 pushes along child edges, claiming undiscovered
// vertices with a CAS on a 32-bit level array and ORing the sets with 64-bit
// atomicOr.  OR is order-independent, so the rows are bit-identical.
// HBM bound: per root the adjacency of every reached vertex is streamed twice
// (sibling + child kernels); the per-vertex state (level, S^-1, S^0) is 17 B.

#include <algorithm>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr uint32_t LV_INF = 255u;

__device__ __forceinline__ uint64_t warp_or64(uint64_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v |= __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

struct BpState {
    uint32_t n;
    const uint32_t *off;
    const uint32_t *adj;
    uint32_t *lvl;   // n, LV_INF = unreached
    uint64_t *sm1;   // n
    uint64_t *s0;    // n
    unsigned long long *work;
};

__global__ void bp_reset_kernel(BpState st)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < st.n; v += gridDim.x * blockDim.x) {
        st.lvl[v] = LV_INF;
        st.sm1[v] = 0;
        st.s0[v] = 0;
    }
}

// seeds: (vertex, level, S^-1) for the root and its selected neighbours.
__global__ void bp_seed_kernel(BpState st, const uint32_t *sv, const uint32_t *slv, const uint64_t *sbits,
                               uint32_t cnt)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < cnt) {
        st.lvl[sv[i]] = slv[i];
        st.sm1[sv[i]] = sbits[i];
    }
}

// Sibling step of level d: S^0[v] |= S^-1[tv] for tv adjacent at the same level.
__global__ void __launch_bounds__(256) bp_sibling_kernel(BpState st, const uint32_t *front, const uint32_t *front_cnt,
                                                         uint32_t d)
{
    const int lane = threadIdx.x & 31;
    const uint32_t cnt = *front_cnt;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long bytes = 0;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const uint32_t v = front[q];
        uint64_t acc = 0;
        uint32_t same = 0;
        for (uint32_t e = st.off[v] + lane; e < st.off[v + 1]; e += 32) {
            const uint32_t tv = st.adj[e];
            if (st.lvl[tv] == d) {
                acc |= st.sm1[tv];
                ++same;
            }
        }
        acc = warp_or64(acc);
        if (lane == 0 && acc) st.s0[v] |= acc;
        // front entry, offsets, S^0 update; 4 B adjacency + 4 B level per edge;
        // 8 B S^-1 per same-level neighbour
        if (lane == 0) bytes += 20 + 8ull * (st.off[v + 1] - st.off[v]);
        bytes += 8ull * same;
    }
    if (st.work && bytes) atomicAdd(&st.work[W_BP_SIB], bytes);
}

// Child step of level d: claim unreached neighbours for level d+1 and OR the
// parent's sets into every level-(d+1) neighbour.
__global__ void __launch_bounds__(256) bp_child_kernel(BpState st, const uint32_t *front, const uint32_t *front_cnt,
                                                       uint32_t d, uint32_t *next, uint32_t *next_cnt,
                                                       uint32_t *status)
{
    const int lane = threadIdx.x & 31;
    const uint32_t cnt = *front_cnt;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long bytes = 0;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const uint32_t v = front[q];
        const uint64_t a = st.sm1[v], b = st.s0[v];
        if (lane == 0) bytes += 28 + 8ull * (st.off[v + 1] - st.off[v]);  // entry, offsets, sets; adj + level
        for (uint32_t e = st.off[v] + lane; e < st.off[v + 1]; e += 32) {
            const uint32_t tv = st.adj[e];
            uint32_t t = st.lvl[tv];
            if (t <= d) continue;
            bytes += 16;  // S^-1 / S^0 of the child
            if (t == LV_INF) {
                if (d + 1 >= LV_INF) {
                    atomicOr(status, ST_LEVEL_OVERFLOW);
                    continue;
                }
                if (atomicCAS(&st.lvl[tv], LV_INF, d + 1) == LV_INF) next[atomicAdd(next_cnt, 1u)] = tv;
            }
            if (a) atomicOr((unsigned long long *)&st.sm1[tv], (unsigned long long)a);
            if (b) atomicOr((unsigned long long *)&st.s0[tv], (unsigned long long)b);
        }
    }
    if (st.work && bytes) atomicAdd(&st.work[W_BP_CHILD], bytes);
}

__global__ void bp_store_kernel(BpState st, uint32_t K, uint32_t i, uint8_t *bpd, uint64_t *bps)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < st.n; v += gridDim.x * blockDim.x) {
        const uint64_t a = st.sm1[v];
        bpd[(uint64_t)v * K + i] = (uint8_t)st.lvl[v];
        bps[((uint64_t)v * K + i) * 2] = a;
        bps[((uint64_t)v * K + i) * 2 + 1] = st.s0[v] & ~a;
    }
}

__global__ void bp_empty_slot_kernel(uint32_t n, uint32_t K, uint32_t i, uint8_t *bpd, uint64_t *bps)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        bpd[(uint64_t)v * K + i] = U8_INF;
        bps[((uint64_t)v * K + i) * 2] = 0;
        bps[((uint64_t)v * K + i) * 2 + 1] = 0;
    }
}

}  // namespace

BpResult bp_label(const HostGraph &hg, const DevGraph &g, uint32_t K, std::vector<uint8_t> &used,
                  uint8_t *d_bpd, uint64_t *d_bps, cudaStream_t s)
{
    BpResult res;
    const uint32_t n = hg.n;
    if (K == 0 || n == 0) return res;
    DBuf<uint32_t> lvl(n), f0(n), f1(n), cnts(4), status(1);
    DBuf<uint64_t> sm1(n), s0(n);
    DBuf<uint32_t> seed_v(65), seed_l(65);
    DBuf<uint64_t> seed_b(65);
    status.fill_bytes(0, s);
    BpState st{n, g.off.p, g.adj.p, lvl.p, sm1.p, s0.p, work_counters()};
    uint32_t *h_cnt = nullptr;
    PADO_CUDA(cudaMallocHost((void **)&h_cnt, 4 * sizeof(uint32_t)));
    cudaEvent_t e0, e1;
    PADO_CUDA(cudaEventCreate(&e0));
    PADO_CUDA(cudaEventCreate(&e1));
    PADO_CUDA(cudaEventRecord(e0, s));
    const unsigned vb = 256, vg = grid_for(n, vb);
    try {
        uint32_t r = 0;
        std::vector<uint32_t> sv, sl;
        std::vector<uint64_t> sb;
        for (uint32_t i = 0; i < K; ++i) {
            while (r < n && used[r]) ++r;
            if (r == n) {
                PADO_LAUNCH("bp_empty_slot_kernel", s,
                            bp_empty_slot_kernel<<<vg, vb, 0, s>>>(n, K, i, d_bpd, d_bps));
                continue;
            }
            used[r] = 1;
            sv.assign(1, r);
            sl.assign(1, 0);
            sb.assign(1, 0);
            int ns = 0;
            for (uint32_t k = hg.off[r + 1]; k > hg.off[r]; --k) {
                uint32_t v = hg.adj[k - 1];
                if (!used[v]) {
                    used[v] = 1;
                    sv.push_back(v);
                    sl.push_back(1);
                    sb.push_back(1ULL << ns);
                    if (++ns == 64) break;
                }
            }
            PADO_LAUNCH("bp_reset_kernel", s,
                        bp_reset_kernel<<<vg, vb, 0, s>>>(st));
            seed_v.upload(sv.data(), sv.size(), s);
            seed_l.upload(sl.data(), sl.size(), s);
            seed_b.upload(sb.data(), sb.size(), s);
            PADO_LAUNCH("bp_seed_kernel", s,
                        bp_seed_kernel<<<1, 128, 0, s>>>(st, seed_v.p, seed_l.p, seed_b.p, (uint32_t)sv.size()));
            // frontier 0 = {r}; frontier 1 starts with the selected neighbours
            uint32_t init_cnt[2] = {1u, (uint32_t)(sv.size() - 1)};
            PADO_CUDA(cudaMemcpyAsync(f0.p, &r, sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            if (sv.size() > 1)
                PADO_CUDA(cudaMemcpyAsync(f1.p, sv.data() + 1, (sv.size() - 1) * sizeof(uint32_t),
                                          cudaMemcpyHostToDevice, s));
            PADO_CUDA(cudaMemcpyAsync(cnts.p, init_cnt, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            uint32_t *cur = f0.p, *nxt = f1.p;
            uint32_t *ccur = cnts.p, *cnxt = cnts.p + 1;
            uint32_t fsize = 1;
            for (uint32_t d = 0; fsize > 0; ++d) {
                const unsigned g2 = grid_for((uint64_t)fsize * 32, 256);
                PADO_LAUNCH("bp_sibling_kernel", s,
                            bp_sibling_kernel<<<g2, 256, 0, s>>>(st, cur, ccur, d));
                PADO_LAUNCH("bp_child_kernel", s,
                            bp_child_kernel<<<g2, 256, 0, s>>>(st, cur, ccur, d, nxt, cnxt, status.p));
                ++res.levels;
                PADO_CUDA(cudaMemcpyAsync(h_cnt, cnxt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaMemcpyAsync(h_cnt + 1, status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaMemsetAsync(ccur, 0, sizeof(uint32_t), s));
                PADO_CUDA(cudaStreamSynchronize(s));
                if (h_cnt[1] & ST_LEVEL_OVERFLOW)
                    throw Error(PADO_E_OVERFLOW, "bit-parallel BFS reached level 255 (uint8 distance overflow)");
                fsize = h_cnt[0];
                std::swap(cur, nxt);
                std::swap(ccur, cnxt);
            }
            PADO_LAUNCH("bp_store_kernel", s,
                        bp_store_kernel<<<vg, vb, 0, s>>>(st, K, i, d_bpd, d_bps));
        }
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
