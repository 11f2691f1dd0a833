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
//
// Device mapping: all K <= 64 BFSes run together, level by level, over the
// final vertex-major rows (bpd[v][K], bps[v][K]) -- a multi-source BFS.  Per
// vertex a 64-bit mask says which slots have reached it, and a level-stamped
// mask which slots have it on the current level.  A warp works on one vertex
// with lane i owning slots i and i + 32, so a neighbour's row is read with
// one coalesced 16-byte load per lane and only for the slots where it matters;
// the adjacency of a vertex is scanned once per level for all slots together
// instead of once per slot.  Per level d:
//   bp_sibling_kernel: each vertex v on level d (in any slot) ORs S^-1 of its
//       neighbours that share a level-d slot into S^0[v] (the sibling step),
//       and lists the neighbours that still miss a slot v has on level d;
//   bp_child_kernel: each listed vertex w takes, per slot it has not reached,
//       the OR of S^-1 / S^0 over its neighbours on level d in that slot (the
//       child step); slots so reached get level d+1 and put w on level d+1.
// The child step pulls along the same edges the reference pushes along, and
// every update is an OR, so the rows are bit-identical.  Vertices of degree
// >= HEAVY are worked on by a whole block (8 warps over the neighbours, one
// shared-memory reduction).  For many graphs in one union id space, slot i
// holds every graph's i-th root: the graphs are disjoint, so their BFSes
// never meet.

#include <algorithm>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULL_MASK = 0xffffffffu;
constexpr uint32_t HEAVY = 2048;     // vertices worked on by a whole block
constexpr int BP_THREADS = 256;
constexpr int BP_WARPS = BP_THREADS / 32;
constexpr int NB = 4;                // neighbours whose rows are loaded together

// Slots where a vertex is on level `lvl`; valid only if `lvl` matches the level
// being read (the two parity buffers are never cleared).
struct LevelMask {
    unsigned long long bits;
    unsigned long long lvl;
};

struct MsState {
    uint32_t n, K;
    const uint32_t *off;
    const uint32_t *adj;
    uint8_t *bpd;          // [n][K]: level per slot, 255 = unreached (final rows)
    ulonglong2 *bps;       // [n][K]: (S^-1, S^0); S^0 is masked by ~S^-1 at the end
    unsigned long long *reach;  // [n]: slots that have reached v
    LevelMask *lm[2];      // [n]: slots with v on level d, in lm[d & 1]
    uint32_t *cstamp;      // [n]: candidate stamp (level + 1)
    uint32_t *fstamp;      // [n]: frontier stamp (level)
    unsigned long long *work;
};

// A list of vertices split by degree: light (a warp each) and heavy (a block each).
struct VList {
    uint32_t *light, *heavy;
    uint32_t *cnt;         // cnt[0] light, cnt[1] heavy
};

__device__ __forceinline__ unsigned long long level_bits(const MsState &st, uint32_t v, uint32_t d)
{
    const LevelMask m = st.lm[d & 1][v];
    return m.lvl == d ? m.bits : 0ull;
}

__device__ __forceinline__ void vlist_append(const MsState &st, const VList &l, uint32_t v)
{
    const bool heavy = st.off[v + 1] - st.off[v] >= HEAVY;
    if (heavy)
        l.heavy[agg_append_by(&l.cnt[1], 1u)] = v;
    else
        l.light[agg_append_by(&l.cnt[0], 0u)] = v;
}

// Sibling step for frontier vertex v over the neighbour range handled by this
// warp (chunks w, w + nw, ...); returns the per-lane ORs (slots lane, lane+32).
__device__ __forceinline__ void sibling_range(const MsState &st, uint32_t v, unsigned long long fv, uint32_t d,
                                              uint32_t w, uint32_t nw, const VList &cand, unsigned long long &acc0,
                                              unsigned long long &acc1, unsigned long long &bytes)
{
    const int lane = threadIdx.x & 31;
    const uint32_t e_end = st.off[v + 1];
    for (uint32_t e0 = st.off[v] + 32 * w; e0 < e_end; e0 += 32 * nw) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t u = in ? st.adj[e] : 0u;
        const unsigned long long fu = in ? level_bits(st, u, d) : 0ull;
        const unsigned long long ru = in ? st.reach[u] : ~0ull;
        // u misses a slot v has on level d: it may be reached at d+1
        if (in && (fv & ~ru) && st.cstamp[u] != d + 1 && atomicExch(&st.cstamp[u], d + 1) != d + 1)
            vlist_append(st, cand, u);
        unsigned long long common = fv & fu;
        uint32_t mask = __ballot_sync(FULL_MASK, common != 0);
        bytes += 20ull * __popc(__ballot_sync(FULL_MASK, in));
        // NB neighbours per round, their rows loaded before any is ORed in
        while (mask) {
            uint32_t uk[NB];
            unsigned long long ck[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                const int k = mask ? __ffs(mask) - 1 : 0;
                const bool has = mask != 0;
                if (has) mask &= mask - 1;
                uk[j] = __shfl_sync(FULL_MASK, u, k);
                const unsigned long long cc = __shfl_sync(FULL_MASK, common, k);
                ck[j] = has ? cc : 0ull;
            }
            unsigned long long x0[NB], x1[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                x0[j] = (ck[j] >> lane) & 1ull ? st.bps[(uint64_t)uk[j] * st.K + lane].x : 0ull;
                x1[j] = (ck[j] >> (lane + 32)) & 1ull ? st.bps[(uint64_t)uk[j] * st.K + lane + 32].x : 0ull;
            }
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                acc0 |= x0[j];
                acc1 |= x1[j];
                bytes += 8ull * __popcll(ck[j]);
            }
        }
    }
}

// Child step for candidate w over this warp's neighbour chunks: per lane, the
// ORs of S^-1 / S^0 of level-d neighbours in the slots w has not reached, and
// the mask of slots so reached.
__device__ __forceinline__ void child_range(const MsState &st, uint32_t w, unsigned long long rw, uint32_t d,
                                            uint32_t wi, uint32_t nw, unsigned long long &newm, ulonglong2 &a0,
                                            ulonglong2 &a1, unsigned long long &bytes)
{
    const int lane = threadIdx.x & 31;
    const uint32_t e_end = st.off[w + 1];
    for (uint32_t e0 = st.off[w] + 32 * wi; e0 < e_end; e0 += 32 * nw) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t u = in ? st.adj[e] : 0u;
        const unsigned long long m = in ? (level_bits(st, u, d) & ~rw) : 0ull;
        uint32_t mask = __ballot_sync(FULL_MASK, m != 0);
        bytes += 20ull * __popc(__ballot_sync(FULL_MASK, in));
        // NB neighbours per round, their rows loaded before any is ORed in
        while (mask) {
            uint32_t uk[NB];
            unsigned long long mk[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                const int k = mask ? __ffs(mask) - 1 : 0;
                const bool has = mask != 0;
                if (has) mask &= mask - 1;
                uk[j] = __shfl_sync(FULL_MASK, u, k);
                const unsigned long long mm = __shfl_sync(FULL_MASK, m, k);
                mk[j] = has ? mm : 0ull;
            }
            const ulonglong2 z = make_ulonglong2(0, 0);
            ulonglong2 x0[NB], x1[NB];
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                x0[j] = (mk[j] >> lane) & 1ull ? st.bps[(uint64_t)uk[j] * st.K + lane] : z;
                x1[j] = (mk[j] >> (lane + 32)) & 1ull ? st.bps[(uint64_t)uk[j] * st.K + lane + 32] : z;
            }
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                newm |= mk[j];
                a0.x |= x0[j].x;
                a0.y |= x0[j].y;
                a1.x |= x1[j].x;
                a1.y |= x1[j].y;
                bytes += 16ull * __popcll(mk[j]);
            }
        }
    }
}

// Commit of the child step for w by one warp: levels, sets, masks, frontier.
__device__ __forceinline__ void child_commit(const MsState &st, uint32_t w, unsigned long long rw,
                                             unsigned long long newm, ulonglong2 a0, ulonglong2 a1, uint32_t d,
                                             const VList &next)
{
    const int lane = threadIdx.x & 31;
    if (!newm) return;
    const uint64_t row = (uint64_t)w * st.K;
    if ((newm >> lane) & 1ull) {
        st.bpd[row + lane] = (uint8_t)(d + 1);
        ulonglong2 x = st.bps[row + lane];
        x.x |= a0.x;
        x.y |= a0.y;
        st.bps[row + lane] = x;
    }
    if ((newm >> (lane + 32)) & 1ull) {
        st.bpd[row + lane + 32] = (uint8_t)(d + 1);
        ulonglong2 x = st.bps[row + lane + 32];
        x.x |= a1.x;
        x.y |= a1.y;
        st.bps[row + lane + 32] = x;
    }
    if (lane == 0) {
        st.reach[w] = rw | newm;
        LevelMask &nm = st.lm[(d + 1) & 1][w];
        const unsigned long long prev = nm.lvl == d + 1 ? nm.bits : 0ull;  // level-1 seeds are there already
        nm.bits = prev | newm;
        nm.lvl = d + 1;
        if (atomicExch(&st.fstamp[w], d + 1) != d + 1) vlist_append(st, next, w);
    }
}

__device__ __forceinline__ void block_or(unsigned long long *sm, unsigned long long &v, int lane, int warp)
{
    sm[warp * 32 + lane] = v;
    __syncthreads();
    if (warp == 0) {
        for (int k = 1; k < BP_WARPS; ++k) v |= sm[k * 32 + lane];
    }
    __syncthreads();
}

// Level d, sibling step over the frontier (heavy vertices by blocks, then
// light ones by warps); also lists the child candidates of level d.
__global__ void __launch_bounds__(BP_THREADS) bp_sibling_kernel(MsState st, VList front, uint32_t d, VList cand)
{
    __shared__ unsigned long long sm[BP_WARPS * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long bytes = 0;
    const uint32_t hc = front.cnt[1];
    for (uint32_t q = blockIdx.x; q < hc; q += gridDim.x) {
        const uint32_t v = front.heavy[q];
        const unsigned long long fv = level_bits(st, v, d);
        unsigned long long a0 = 0, a1 = 0;
        sibling_range(st, v, fv, d, warp, BP_WARPS, cand, a0, a1, bytes);
        block_or(sm, a0, lane, warp);
        block_or(sm, a1, lane, warp);
        if (warp == 0) {
            const uint64_t row = (uint64_t)v * st.K;
            if (a0 && lane < (int)st.K) st.bps[row + lane].y |= a0;
            if (a1 && lane + 32 < (int)st.K) st.bps[row + lane + 32].y |= a1;
        }
    }
    const uint32_t lc = front.cnt[0];
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < lc; q += nw) {
        const uint32_t v = front.light[q];
        const unsigned long long fv = level_bits(st, v, d);
        unsigned long long a0 = 0, a1 = 0;
        sibling_range(st, v, fv, d, 0, 1, cand, a0, a1, bytes);
        const uint64_t row = (uint64_t)v * st.K;
        if (a0 && lane < (int)st.K) st.bps[row + lane].y |= a0;
        if (a1 && lane + 32 < (int)st.K) st.bps[row + lane + 32].y |= a1;
    }
    if (st.work && lane == 0 && bytes) atomicAdd(&st.work[W_BP_SIB], bytes);
}

// Level d, child step over the candidates; builds the frontier of level d+1.
__global__ void __launch_bounds__(BP_THREADS) bp_child_kernel(MsState st, VList cand, uint32_t d, VList next,
                                                              uint32_t *status)
{
    __shared__ unsigned long long sm[BP_WARPS * 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long bytes = 0;
    if (d + 1 >= U8_INF) {
        if ((cand.cnt[0] || cand.cnt[1]) && threadIdx.x == 0 && blockIdx.x == 0) atomicOr(status, ST_LEVEL_OVERFLOW);
        return;
    }
    const uint32_t hc = cand.cnt[1];
    for (uint32_t q = blockIdx.x; q < hc; q += gridDim.x) {
        const uint32_t w = cand.heavy[q];
        const unsigned long long rw = st.reach[w];
        unsigned long long newm = 0;
        ulonglong2 a0 = make_ulonglong2(0, 0), a1 = make_ulonglong2(0, 0);
        child_range(st, w, rw, d, warp, BP_WARPS, newm, a0, a1, bytes);
        block_or(sm, newm, lane, warp);
        block_or(sm, a0.x, lane, warp);
        block_or(sm, a0.y, lane, warp);
        block_or(sm, a1.x, lane, warp);
        block_or(sm, a1.y, lane, warp);
        if (warp == 0) child_commit(st, w, rw, newm, a0, a1, d, next);  // newm is the same in every lane
    }
    const uint32_t lc = cand.cnt[0];
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < lc; q += nw) {
        const uint32_t w = cand.light[q];
        const unsigned long long rw = st.reach[w];
        unsigned long long newm = 0;
        ulonglong2 a0 = make_ulonglong2(0, 0), a1 = make_ulonglong2(0, 0);
        child_range(st, w, rw, d, 0, 1, newm, a0, a1, bytes);
        child_commit(st, w, rw, newm, a0, a1, d, next);
    }
    if (st.work && lane == 0 && bytes) atomicAdd(&st.work[W_BP_CHILD], bytes);
}

__global__ void bp_init_kernel(LevelMask *a, LevelMask *b, uint32_t n)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        a[v] = LevelMask{0ull, ~0ull};
        b[v] = LevelMask{0ull, ~0ull};
    }
}

// Seeds: (slot, vertex, level, S^-1) for each root and its selected neighbours.
__global__ void bp_seed_kernel(MsState st, const uint32_t *sslot, const uint32_t *sv, const uint32_t *slv,
                               const uint64_t *sbits, uint32_t cnt)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cnt) return;
    const uint32_t v = sv[i], slot = sslot[i], l = slv[i];
    st.bpd[(uint64_t)v * st.K + slot] = (uint8_t)l;
    st.bps[(uint64_t)v * st.K + slot].x = sbits[i];
    atomicOr(&st.reach[v], 1ull << slot);
    atomicOr(&st.lm[l & 1][v].bits, 1ull << slot);
    st.lm[l & 1][v].lvl = l;
    if (l == 1) st.fstamp[v] = 1;
}

__global__ void bp_finish_kernel(MsState st)
{
    const uint64_t tot = (uint64_t)st.n * st.K;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < tot; x += (uint64_t)gridDim.x * blockDim.x)
        st.bps[x].y &= ~st.bps[x].x;
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
            const uint32_t v = hg.adjp()[k - 1];
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
    PADO_CHECK(K <= MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");
    cudaEvent_t e0, e1;
    PADO_CUDA(cudaEventCreate(&e0));
    PADO_CUDA(cudaEventCreate(&e1));
    uint32_t *h_cnt = nullptr;
    try {
        PADO_CUDA(cudaMallocHost((void **)&h_cnt, 8 * sizeof(uint32_t)));
        PADO_CUDA(cudaEventRecord(e0, s));
        // rows start unreached: level 255, empty sets (also the rows of slots no graph has a root for)
        PADO_CUDA(cudaMemsetAsync(d_bpd, 0xff, (uint64_t)n * K, s));
        PADO_CUDA(cudaMemsetAsync(d_bps, 0, (uint64_t)n * K * 16, s));
        DBuf<unsigned long long> reach(n);
        DBuf<LevelMask> lm0(n), lm1(n);
        DBuf<uint32_t> cstamp(n), fstamp(n), cnts(8), status(1);
        DBuf<uint32_t> fl[2], fh[2], cl, ch;
        for (int i = 0; i < 2; ++i) {
            fl[i].alloc(n);
            fh[i].alloc(n);
        }
        cl.alloc(n);
        ch.alloc(n);
        reach.fill_bytes(0, s);
        // empty masks stamped with a level no BFS reaches
        PADO_LAUNCH("bp_init_kernel", s, bp_init_kernel<<<grid_for(n, 256), 256, 0, s>>>(lm0.p, lm1.p, n));
        cstamp.fill_bytes(0, s);
        fstamp.fill_bytes(0xff, s);
        status.fill_bytes(0, s);
        cnts.fill_bytes(0, s);
        MsState st{n, K, g.off.p, g.adj.p, d_bpd, reinterpret_cast<ulonglong2 *>(d_bps), reach.p,
                   {lm0.p, lm1.p}, cstamp.p, fstamp.p, work_counters()};

        // seeds and the frontiers of levels 0 (roots) and 1 (selected neighbours), deduplicated
        std::vector<uint32_t> ss, sv, sl;
        std::vector<uint64_t> sb;
        std::vector<uint32_t> f0[2], f1[2];
        std::vector<uint8_t> in0(n, 0), in1(n, 0);
        for (uint32_t j = 0; j < std::min<size_t>(K, seeds.size()); ++j) {
            for (const BpSeed &x : seeds[j]) {
                ss.push_back(j);
                sv.push_back(x.v);
                sl.push_back(x.lvl);
                sb.push_back(x.bits);
                const bool heavy = hg.off[x.v + 1] - hg.off[x.v] >= HEAVY;
                if (x.lvl == 0 && !in0[x.v]) {
                    in0[x.v] = 1;
                    f0[heavy].push_back(x.v);
                } else if (x.lvl == 1 && !in1[x.v]) {
                    in1[x.v] = 1;
                    f1[heavy].push_back(x.v);
                }
            }
        }
        if (sv.empty()) {
            PADO_CUDA(cudaEventRecord(e1, s));
            PADO_CUDA(cudaEventSynchronize(e1));
            PADO_CUDA(cudaEventElapsedTime(&res.ms, e0, e1));
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            cudaFreeHost(h_cnt);
            return res;
        }
        DBuf<uint32_t> d_ss(ss.size()), d_sv(sv.size()), d_sl(sl.size());
        DBuf<uint64_t> d_sb(sb.size());
        d_ss.upload(ss.data(), ss.size(), s);
        d_sv.upload(sv.data(), sv.size(), s);
        d_sl.upload(sl.data(), sl.size(), s);
        d_sb.upload(sb.data(), sb.size(), s);
        PADO_LAUNCH("bp_seed_kernel", s,
                    bp_seed_kernel<<<grid_for(sv.size(), 128), 128, 0, s>>>(st, d_ss.p, d_sv.p, d_sl.p, d_sb.p,
                                                                          (uint32_t)sv.size()));
        fl[0].upload(f0[0].data(), f0[0].size(), s);
        fh[0].upload(f0[1].data(), f0[1].size(), s);
        fl[1].upload(f1[0].data(), f1[0].size(), s);
        fh[1].upload(f1[1].data(), f1[1].size(), s);
        // cnts: [0,1] frontier d (light, heavy), [2,3] frontier d+1, [4,5] candidates
        uint32_t init_cnt[8] = {(uint32_t)f0[0].size(), (uint32_t)f0[1].size(), (uint32_t)f1[0].size(),
                                (uint32_t)f1[1].size(), 0, 0, 0, 0};
        PADO_CUDA(cudaMemcpyAsync(cnts.p, init_cnt, sizeof(init_cnt), cudaMemcpyHostToDevice, s));
        const unsigned grid = 152u * 8u;
        int cur = 0;
        uint32_t *ccur = cnts.p, *cnxt = cnts.p + 2, *ccand = cnts.p + 4;
        uint32_t fsize = (uint32_t)(f0[0].size() + f0[1].size());
        for (uint32_t d = 0; fsize > 0; ++d) {
            const VList front{fl[cur].p, fh[cur].p, ccur};
            const VList next{fl[cur ^ 1].p, fh[cur ^ 1].p, cnxt};
            const VList cand{cl.p, ch.p, ccand};
            PADO_LAUNCH("bp_sibling_kernel", s, bp_sibling_kernel<<<grid, BP_THREADS, 0, s>>>(st, front, d, cand));
            PADO_LAUNCH("bp_child_kernel", s,
                        bp_child_kernel<<<grid, BP_THREADS, 0, s>>>(st, cand, d, next, status.p));
            ++res.levels;
            PADO_CUDA(cudaMemcpyAsync(h_cnt, cnxt, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            PADO_CUDA(cudaMemcpyAsync(h_cnt + 2, status.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            PADO_CUDA(cudaMemsetAsync(ccur, 0, 2 * sizeof(uint32_t), s));
            PADO_CUDA(cudaMemsetAsync(ccand, 0, 2 * sizeof(uint32_t), s));
            PADO_CUDA(cudaStreamSynchronize(s));
            if (h_cnt[2] & ST_LEVEL_OVERFLOW)
                throw Error(PADO_E_OVERFLOW, "bit-parallel BFS reached level 255 (uint8 distance overflow)");
            fsize = h_cnt[0] + h_cnt[1];
            cur ^= 1;
            std::swap(ccur, cnxt);
        }
        PADO_LAUNCH("bp_finish_kernel", s,
                    bp_finish_kernel<<<grid_for((uint64_t)n * K, 256), 256, 0, s>>>(st));
        PADO_CUDA(cudaEventRecord(e1, s));
        PADO_CUDA(cudaEventSynchronize(e1));
        PADO_CUDA(cudaEventElapsedTime(&res.ms, e0, e1));
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (h_cnt) cudaFreeHost(h_cnt);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeHost(h_cnt);
    return res;
}

}  // namespace pado
