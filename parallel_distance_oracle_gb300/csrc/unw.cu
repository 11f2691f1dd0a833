// unw.cu -- batched pruned-BFS labeling for unweighted graphs.
//
// Restates the batched vertex-centric labeling of the reference
// (includes/pado_unw_unv_unp.h:425-1118; OpenMP variant
// pado_unw_unv_para.201912311607.parallel_bp_labeling.h:848-1737):
//   for each batch of B consecutive ranks [s, e):
//     every non-BP root r gets the label (r, 0) and starts active (:425-528);
//     dist_matrix[r - s][h] = d for every label (h, d) of root r (:492-526);
//     level iter = 1, 2, ...:
//       push (:531-641): an active head h offers each label r it gained at the
//         previous level to every neighbour t with t > r (neighbour lists are
//         descending; t < s ends the scan), unless t is a BP vertex.  The first
//         offer of r to t in the batch sets indicator[t][r]; later offers are
//         ignored.  A first offer is dropped if the BP rows cover it:
//         exists i: td = bpd_r[i] + bpd_t[i] (unsigned), td - 2 <= iter and
//         td minus 2 / 1 / 0 (S^-1 & S^-1, S^-1 & S^0 mixes) <= iter.
//       add (:647-775): a surviving candidate r of t is dropped if some label
//         (h, d) of t has d < iter, h < r and d + dist_matrix[r - s][h] <= iter;
//         otherwise t gets label (r, iter) and is active at the next level.  If
//         t is itself a root, dist_matrix[t - s][r] = iter.
//     dist_matrix rows of the roots are reset to 255 (:780-816).
// The result is independent of the order candidates are processed in (each
// (t, r) pair is decided once per batch, and a dist_matrix entry written at
// level iter can only matter through a hub at distance 0, which the rank
// conditions exclude), so the level-synchronous device schedule below gives
// bit-identical labels.
//
// Device mapping (one GPU, HBM-resident state, ranks as ids):
//   * mark kernel: a warp per active head scans its neighbour prefix t > min(r)
//     and stamps each non-BP tail once per level (atomicExch), building the
//     tail list;
//   * pull kernel: a warp per tail owns everything about that tail for the
//     level -- it gathers the previous-level label groups of its active
//     neighbours, dedups roots against its indicator row (kept in shared
//     memory), runs the BP test lane-per-candidate against its own BP row in
//     shared memory, runs the distance test against its labels with d < iter,
//     and appends the survivors.  No per-pair global atomics.
//   * the label store is a bump-allocated pool of (u32 hub, u8 dist) entries;
//     a vertex's list grows by relocation to a doubled slot, and the previous
//     level's group of every vertex is addressed by absolute pool position in
//     parity-double-buffered arrays, so neighbours can read it while its owner
//     appends or relocates.  A warp that cannot reserve pool space commits
//     nothing and is queued for an exact re-run after the host grows the pool.
//   * finalize: each vertex's list is sorted per batch run (hubs of one batch
//     are contiguous), which yields the canonical hub-sorted order.

#include <algorithm>
#include <cstring>
#include <numeric>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SMALL_CAP = 256;                 // labels with d < iter staged in smem
constexpr uint32_t HEAVY_DEG = 2048;           // tails this large are processed by a block

struct UnwDev {
    uint32_t n, K, B, words;
    const uint32_t *off;
    const uint32_t *adj;
    const uint8_t *used;
    const uint8_t *bpd;
    const uint64_t *bps;
    uint32_t *pool_hub;
    uint8_t *pool_dist;
    unsigned long long pool_cap;
    unsigned long long *pool_top;
    uint64_t *lab_off;
    uint32_t *lab_len;
    uint32_t *lab_cap;
    uint64_t *last_pos[2];
    uint32_t *last_cnt[2];
    uint32_t *last_min[2];
    uint32_t *act_stamp[2];  // by level parity: level id at which the vertex gained labels
    uint32_t *tail_stamp;
    uint32_t *ind;        // n * words
    uint32_t *ind_stamp;  // batch + 1 when the row is valid
    uint8_t *dm;          // B * n
    uint32_t *status;
    unsigned long long *work;  // algorithmic-byte counters (profiling only)
};

__device__ __forceinline__ uint32_t warp_min_u32(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// Reserve room for `need` entries in v's list; relocates (warp-cooperative
// copy) when the slot is too small.  Returns false, with nothing changed
// except pool_top, when the pool is exhausted.
__device__ __forceinline__ bool warp_reserve(const UnwDev &d, uint32_t v, uint32_t need, uint64_t &base, int lane)
{
    const uint32_t len = d.lab_len[v], cap = d.lab_cap[v];
    base = d.lab_off[v];
    if (need <= cap) return true;
    uint32_t ncap = max(max(2u * cap, need), 8u);
    ncap = (ncap + 7u) & ~7u;
    unsigned long long pos = 0;
    if (lane == 0) pos = atomicAdd(d.pool_top, (unsigned long long)ncap);
    pos = __shfl_sync(FULL, pos, 0);
    if (pos + ncap > d.pool_cap) return false;
    for (uint32_t j = lane; j < len; j += 32) {
        d.pool_hub[pos + j] = d.pool_hub[base + j];
        d.pool_dist[pos + j] = d.pool_dist[base + j];
    }
    __syncwarp();
    if (lane == 0) {
        d.lab_off[v] = pos;
        d.lab_cap[v] = ncap;
    }
    base = pos;
    return true;
}

// Batch start: self label (r, 0) for every non-BP root, indicator row with
// the root's own bit, active at level stamp lid0 (pado_unw_unv_unp.h:425-491).
__device__ void root_init_phase(const UnwDev &d, const uint32_t *roots, uint32_t nroots, uint32_t s, uint32_t b,
                                uint32_t lid0, uint32_t *front, uint32_t *front_cnt, uint32_t *retry,
                                uint32_t *retry_cnt)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int p = lid0 & 1;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nroots; q += nw) {
        const uint32_t r = roots[q];
        uint64_t base;
        if (!warp_reserve(d, r, d.lab_len[r] + 1, base, lane)) {
            if (lane == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                retry[atomicAdd(retry_cnt, 1u)] = r;
            }
            continue;
        }
        const uint32_t len = d.lab_len[r];
        const uint32_t idx = r - s;
        for (uint32_t w = lane; w < d.words; w += 32)
            d.ind[(uint64_t)r * d.words + w] = (w == (idx >> 5)) ? (1u << (idx & 31)) : 0u;
        if (lane == 0) {
            d.pool_hub[base + len] = r;
            d.pool_dist[base + len] = 0;
            d.lab_len[r] = len + 1;
            d.last_pos[p][r] = base + len;
            d.last_cnt[p][r] = 1;
            d.last_min[p][r] = r;
            d.act_stamp[p][r] = lid0;
            d.ind_stamp[r] = b + 1;
            front[atomicAdd(front_cnt, 1u)] = r;
        }
    }
}

__global__ void __launch_bounds__(256) root_init_kernel(UnwDev d, const uint32_t *roots, uint32_t nroots,
                                                        uint32_t s, uint32_t b, uint32_t lid0,
                                                        uint32_t *front, uint32_t *front_cnt,
                                                        uint32_t *retry, uint32_t *retry_cnt)
{
    root_init_phase(d, roots, nroots, s, b, lid0, front, front_cnt, retry, retry_cnt);
}

// dist_matrix rows of the batch roots: fill from their labels (value = d) or
// reset to 255 (pado_unw_unv_unp.h:492-526 and :780-816).
__device__ void dm_rows_phase(const UnwDev &d, const uint32_t *roots, uint32_t nroots, uint32_t s, int fill)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nroots; q += nw) {
        const uint32_t r = roots[q];
        uint8_t *row = d.dm + (uint64_t)(r - s) * d.n;
        const uint64_t base = d.lab_off[r];
        const uint32_t len = d.lab_len[r];
        for (uint32_t j = lane; j < len; j += 32)
            row[d.pool_hub[base + j]] = fill ? d.pool_dist[base + j] : U8_INF;
    }
}

__global__ void __launch_bounds__(256) dm_rows_kernel(UnwDev d, const uint32_t *roots, uint32_t nroots, uint32_t s,
                                                      int fill)
{
    dm_rows_phase(d, roots, nroots, s, fill);
}

// Tail marking: for each active head, neighbours t (descending) with
// t > min(root of its last group) that are not BP vertices.
__device__ void mark_phase(const UnwDev &d, const uint32_t *front, uint32_t cnt, uint32_t lid_cur, uint32_t *tails,
                           uint32_t *tails_cnt, uint32_t *htails, uint32_t *htails_cnt)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int pp = (lid_cur - 1) & 1;
    unsigned long long bytes = 0;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const uint32_t h = front[q];
        const uint32_t mn = d.last_min[pp][h];
        const uint32_t e_end = d.off[h + 1];
        bytes += 16;  // front entry, last_min, offsets
        for (uint32_t e0 = d.off[h]; e0 < e_end; e0 += 32) {
            const uint32_t e = e0 + lane;
            const bool in = e < e_end;
            const uint32_t t = in ? d.adj[e] : 0u;
            const bool ok = in && t > mn;
            bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ok)) * 5ull;
            bool appended = false;
            if (ok && !d.used[t] && d.tail_stamp[t] != lid_cur) {
                if (atomicExch(&d.tail_stamp[t], lid_cur) != lid_cur) {
                    if (d.off[t + 1] - d.off[t] >= HEAVY_DEG)
                        htails[atomicAdd(htails_cnt, 1u)] = t;
                    else
                        tails[atomicAdd(tails_cnt, 1u)] = t;
                    appended = true;
                }
            }
            bytes += __popc(__ballot_sync(FULL, appended)) * 8ull;
            if (__ballot_sync(FULL, in && !ok)) break;  // descending: the rest are smaller
        }
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_MARK], bytes);
}

__global__ void __launch_bounds__(256) mark_kernel(UnwDev d, const uint32_t *front, const uint32_t *front_cnt,
                                                   uint32_t lid_cur, uint32_t *tails, uint32_t *tails_cnt,
                                                   uint32_t *htails, uint32_t *htails_cnt)
{
    mark_phase(d, front, *front_cnt, lid_cur, tails, tails_cnt, htails, htails_cnt);
}

// Shared-memory layout of the pull kernel, carved from dynamic shared memory
// by batch size: 8 per-warp regions for light tails, aliased by one
// block-wide region for heavy tails (the two phases do not overlap).
constexpr int PULL_THREADS = 256;
constexpr int PULL_NW = PULL_THREADS / 32;
constexpr int HSMALL_CAP = 1024;          // heavy tail: labels with d < iter staged

__host__ __device__ __forceinline__ uint32_t align16(uint32_t x) { return (x + 15u) & ~15u; }

struct WarpRegion {
    uint32_t *ind;        // words
    uint16_t *offered;    // B
    uint8_t *tbpd;        // 64
    ulonglong2 *tbps;     // 64
    uint32_t *sh;         // SMALL_CAP
    uint8_t *sd;          // SMALL_CAP
    uint32_t *ctr;        // [0] noff, [1] nsmall
};

__host__ __device__ __forceinline__ uint32_t warp_region_bytes(uint32_t words, uint32_t B)
{
    return align16(words * 4) + align16(B * 2) + 64 + 64 * 16 + SMALL_CAP * 4 + SMALL_CAP + 16;
}

__host__ __device__ __forceinline__ uint32_t heavy_region_bytes(uint32_t words, uint32_t B)
{
    return align16(words * 4) + 2 * align16(B * 2) + 64 + 64 * 16 + HSMALL_CAP * 4 + HSMALL_CAP + 64;
}

__host__ __device__ __forceinline__ uint32_t pull_smem_bytes(uint32_t words, uint32_t B)
{
    const uint32_t l = PULL_NW * warp_region_bytes(words, B), h = heavy_region_bytes(words, B);
    return l > h ? l : h;
}

__device__ __forceinline__ WarpRegion warp_region(unsigned char *base, uint32_t words, uint32_t B, int w)
{
    unsigned char *p = base + (size_t)w * warp_region_bytes(words, B);
    WarpRegion r;
    r.tbps = reinterpret_cast<ulonglong2 *>(p);
    p += 64 * 16;
    r.ind = reinterpret_cast<uint32_t *>(p);
    p += align16(words * 4);
    r.sh = reinterpret_cast<uint32_t *>(p);
    p += SMALL_CAP * 4;
    r.ctr = reinterpret_cast<uint32_t *>(p);
    p += 16;
    r.offered = reinterpret_cast<uint16_t *>(p);
    p += align16(B * 2);
    r.tbpd = p;
    p += 64;
    r.sd = p;
    return r;
}

struct HeavyRegion {
    ulonglong2 *tbps;
    uint32_t *ind;
    uint32_t *sh;
    uint16_t *offered;
    uint16_t *surv;
    uint8_t *tbpd;
    uint8_t *sd;
    uint32_t *ctr;                   // noff, nsurv, nsmall, nadd, mn, ok, reloc, ncap
    unsigned long long *base;
};

__device__ __forceinline__ HeavyRegion heavy_region(unsigned char *p, uint32_t words, uint32_t B)
{
    HeavyRegion r;
    r.tbps = reinterpret_cast<ulonglong2 *>(p);
    p += 64 * 16;
    r.base = reinterpret_cast<unsigned long long *>(p);
    p += 16;
    r.ctr = reinterpret_cast<uint32_t *>(p);
    p += 48;
    r.ind = reinterpret_cast<uint32_t *>(p);
    p += align16(words * 4);
    r.sh = reinterpret_cast<uint32_t *>(p);
    p += HSMALL_CAP * 4;
    r.offered = reinterpret_cast<uint16_t *>(p);
    p += align16(B * 2);
    r.surv = reinterpret_cast<uint16_t *>(p);
    p += align16(B * 2);
    r.tbpd = p;
    p += 64;
    r.sd = p;
    return r;
}

// BP test of one (root, tail) pair on BP root i only.
__device__ __forceinline__ bool bp_one(uint8_t rd, ulonglong2 rs, uint8_t td, ulonglong2 ts, uint32_t iter)
{
    uint32_t x = (uint32_t)rd + (uint32_t)td;
    if (x - 2u > iter) return false;
    if (rs.x & ts.x)
        x -= 2u;
    else if ((rs.x & ts.y) | (rs.y & ts.x))
        x -= 1u;
    return x <= iter;
}

// Warp-cooperative BP test of candidate root r against the tail's row held in
// registers (lane i holds BP roots i and i + 32); roots < skip were already
// tested.  Pruned iff any root covers the pair -- order-independent.
__device__ __forceinline__ bool bp_covered_warp(const UnwDev &d, uint32_t r, int lane, uint32_t skip, uint8_t td0,
                                                ulonglong2 ts0, uint8_t td1, ulonglong2 ts1, uint32_t iter)
{
    const uint8_t *rd = d.bpd + (uint64_t)r * d.K;
    const ulonglong2 *rs = reinterpret_cast<const ulonglong2 *>(d.bps + (uint64_t)r * d.K * 2);
    bool cov = false;
    const uint32_t i0 = lane, i1 = lane + 32;
    if (i0 >= skip && i0 < d.K) cov = bp_one(rd[i0], rs[i0], td0, ts0, iter);
    if (i1 >= skip && i1 < d.K) cov = cov || bp_one(rd[i1], rs[i1], td1, ts1, iter);
    return __ballot_sync(FULL, cov) != 0;
}

struct PullArgs {
    const uint32_t *tails;        // light tails
    const uint32_t *tails_cnt;
    const uint32_t *htails;       // heavy tails
    const uint32_t *htails_cnt;
    uint32_t s, e_roots, b, iter, lid_cur;
    uint32_t *front_next;
    uint32_t *front_next_cnt;
    uint32_t *retry;
    uint32_t *retry_cnt;
};

// One heavy tail, processed by the whole block.
__device__ void pull_heavy_tail(const UnwDev &d, const PullArgs &a, uint32_t t, HeavyRegion &hs,
                                unsigned long long &bytes)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t s = a.s, iter = a.iter;
    const int pp = (a.lid_cur - 1) & 1, cp = a.lid_cur & 1;
    const uint32_t lid_prev = a.lid_cur - 1;
    const bool valid = d.ind_stamp[t] == a.b + 1;
    for (uint32_t x = tid; x < d.words; x += blockDim.x) hs.ind[x] = valid ? d.ind[(uint64_t)t * d.words + x] : 0u;
    if (tid < 8) hs.ctr[tid] = (tid == 4) ? 0xffffffffu : 0u;
    if (tid == 0) bytes += 8 + 8ull * d.words;
    __syncthreads();
    // (a) first offers from active neighbours, warps striding over the list
    const uint32_t e_end = d.off[t + 1];
    for (uint32_t e0 = d.off[t] + 32 * warp; e0 < e_end; e0 += 32 * (blockDim.x >> 5)) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t h = in ? d.adj[e] : 0u;
        const bool ge = in && h >= s;
        const bool act = ge && d.act_stamp[pp][h] == lid_prev;
        uint32_t mask = __ballot_sync(FULL, act);
        if (lane == 0) bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ge)) * 4ull;
        else { __ballot_sync(FULL, in); __ballot_sync(FULL, ge); }
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const uint32_t hh = __shfl_sync(FULL, h, src);
            const uint64_t pos = d.last_pos[pp][hh];
            const uint32_t c = d.last_cnt[pp][hh];
            if (lane == 0) bytes += 12 + 4ull * c;
            for (uint32_t j = lane; j < c; j += 32) {
                const uint32_t r = d.pool_hub[pos + j];
                if (r < t) {
                    const uint32_t idx = r - s;
                    const uint32_t bit = 1u << (idx & 31);
                    const uint32_t old = atomicOr(&hs.ind[idx >> 5], bit);
                    if (!(old & bit)) hs.offered[atomicAdd(&hs.ctr[0], 1u)] = (uint16_t)idx;
                }
            }
        }
        if (__ballot_sync(FULL, in && !ge)) break;  // descending list: the rest are < s
    }
    __syncthreads();
    const uint32_t noff = hs.ctr[0];
    if (noff == 0) return;  // uniform: nothing changed
    // (b) BP test: thread per candidate on BP root 0, then warps take the
    // survivors one at a time over the remaining roots.
    if (tid == 0) bytes += 17ull * d.K;
    const ulonglong2 zero2 = make_ulonglong2(0, 0);
    const uint8_t td0 = lane < (int)d.K ? d.bpd[(uint64_t)t * d.K + lane] : (uint8_t)U8_INF;
    const uint8_t td1 = lane + 32 < (int)d.K ? d.bpd[(uint64_t)t * d.K + lane + 32] : (uint8_t)U8_INF;
    const ulonglong2 ts0 = lane < (int)d.K ? reinterpret_cast<const ulonglong2 *>(d.bps)[(uint64_t)t * d.K + lane] : zero2;
    const ulonglong2 ts1 =
        lane + 32 < (int)d.K ? reinterpret_cast<const ulonglong2 *>(d.bps)[(uint64_t)t * d.K + lane + 32] : zero2;
    const uint8_t tr0d = __shfl_sync(FULL, td0, 0);
    const ulonglong2 tr0s = make_ulonglong2(__shfl_sync(FULL, ts0.x, 0), __shfl_sync(FULL, ts0.y, 0));
    for (uint32_t c = tid; c < noff; c += blockDim.x) {
        const uint16_t idx = hs.offered[c];
        const uint64_t rr = s + idx;
        if (d.K == 0 ||
            !bp_one(d.bpd[rr * d.K], reinterpret_cast<const ulonglong2 *>(d.bps)[rr * d.K], tr0d, tr0s, iter))
            hs.surv[atomicAdd(&hs.ctr[1], 1u)] = idx;
    }
    __syncthreads();
    const uint32_t nsurv1 = hs.ctr[1];
    if (d.K > 1 && nsurv1) {
        if (tid == 0) hs.ctr[1] = 0;
        __syncthreads();
        for (uint32_t c = warp; c < nsurv1; c += blockDim.x >> 5) {
            const uint16_t idx = hs.surv[c];
            const bool cov = bp_covered_warp(d, s + idx, lane, 1, td0, ts0, td1, ts1, iter);
            if (!cov && lane == 0) hs.offered[atomicAdd(&hs.ctr[1], 1u)] = idx;
        }
        __syncthreads();
        // survivors now sit in `offered`; move them back for the distance test
        const uint32_t ns2 = hs.ctr[1];
        for (uint32_t c = tid; c < ns2; c += blockDim.x) hs.surv[c] = hs.offered[c];
        __syncthreads();
    }
    const uint32_t nsurv = hs.ctr[1];
    const uint32_t len = d.lab_len[t];
    const uint64_t base = d.lab_off[t];
    // (c) distance test
    if (nsurv) {
        for (uint32_t j = tid; j < len; j += blockDim.x) {
            const uint8_t dd = d.pool_dist[base + j];
            if (dd < iter) {
                const uint32_t slot = atomicAdd(&hs.ctr[2], 1u);
                if (slot < HSMALL_CAP) {
                    hs.sh[slot] = d.pool_hub[base + j];
                    hs.sd[slot] = dd;
                }
            }
        }
        __syncthreads();
        const uint32_t nsmall = hs.ctr[2];
        if (tid == 0) bytes += 12 + (uint64_t)len + 4ull * min(nsmall, (uint32_t)HSMALL_CAP) + (uint64_t)nsurv * nsmall;
        for (uint32_t c = tid; c < nsurv; c += blockDim.x) {
            const uint16_t idx = hs.surv[c];
            const uint32_t rr = s + idx;
            const uint8_t *row = d.dm + (uint64_t)idx * d.n;
            bool keep = true;
            if (nsmall <= HSMALL_CAP) {
                for (uint32_t k = 0; k < nsmall; ++k) {
                    const uint32_t hh = hs.sh[k];
                    if (hh < rr && (uint32_t)hs.sd[k] + (uint32_t)row[hh] <= iter) { keep = false; break; }
                }
            } else {
                for (uint32_t j = 0; j < len; ++j) {
                    const uint32_t dd = d.pool_dist[base + j];
                    if (dd >= iter) continue;
                    const uint32_t hh = d.pool_hub[base + j];
                    if (hh < rr && dd + (uint32_t)row[hh] <= iter) { keep = false; break; }
                }
            }
            if (keep) hs.offered[atomicAdd(&hs.ctr[3], 1u)] = idx;
        }
        __syncthreads();
    }
    const uint32_t nadd = hs.ctr[3];
    if (nadd) {
        // (d) reserve, relocating if the slot is too small
        if (tid == 0) {
            const uint32_t cap = d.lab_cap[t], need = len + nadd;
            hs.ctr[5] = 1;
            hs.ctr[6] = 0;
            *hs.base = base;
            if (need > cap) {
                uint32_t ncap = max(max(2u * cap, need), 8u);
                ncap = (ncap + 7u) & ~7u;
                const unsigned long long pos = atomicAdd(d.pool_top, (unsigned long long)ncap);
                if (pos + ncap > d.pool_cap) {
                    hs.ctr[5] = 0;
                } else {
                    hs.ctr[6] = 1;
                    hs.ctr[7] = ncap;
                    *hs.base = pos;
                }
            }
        }
        __syncthreads();
        if (!hs.ctr[5]) {
            if (tid == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                a.retry[atomicAdd(a.retry_cnt, 1u)] = t;
            }
            return;  // uniform; nothing committed
        }
        const uint64_t nbase = *hs.base;
        if (hs.ctr[6]) {
            for (uint32_t j = tid; j < len; j += blockDim.x) {
                d.pool_hub[nbase + j] = d.pool_hub[base + j];
                d.pool_dist[nbase + j] = d.pool_dist[base + j];
            }
        }
        const bool is_root = t >= s && t < a.e_roots;
        for (uint32_t j = tid; j < nadd; j += blockDim.x) {
            const uint32_t idx = hs.offered[j];
            d.pool_hub[nbase + len + j] = s + idx;
            d.pool_dist[nbase + len + j] = (uint8_t)iter;
            if (is_root) d.dm[(uint64_t)(t - s) * d.n + s + idx] = (uint8_t)iter;
            atomicMin(&hs.ctr[4], s + idx);
        }
        __syncthreads();
        if (tid == 0) {
            if (hs.ctr[6]) {
                d.lab_off[t] = nbase;
                d.lab_cap[t] = hs.ctr[7];
            }
            d.lab_len[t] = len + nadd;
            d.last_pos[cp][t] = nbase + len;
            d.last_cnt[cp][t] = nadd;
            d.last_min[cp][t] = hs.ctr[4];
            d.act_stamp[cp][t] = a.lid_cur;
            a.front_next[atomicAdd(a.front_next_cnt, 1u)] = t;
            bytes += 5ull * nadd + 28 + (is_root ? (uint64_t)nadd : 0) + (hs.ctr[6] ? 10ull * len : 0);
        }
    }
    for (uint32_t x = tid; x < d.words; x += blockDim.x) d.ind[(uint64_t)t * d.words + x] = hs.ind[x];
    if (tid == 0) d.ind_stamp[t] = a.b + 1;
}

// One light tail, processed by one warp.
__device__ void pull_light_tail(const UnwDev &d, const PullArgs &a, uint32_t t, WarpRegion &wr,
                                unsigned long long &bytes)
{
    const int lane = threadIdx.x & 31;
    long long c0 = d.work ? clock64() : 0, c1 = 0;
    // phase clock: adds the cycles since the last mark to slot `w` (profiling only)
    auto tick = [&](int w) {
        if (d.work) {
            c1 = clock64();
            if (lane == 0) atomicAdd(&d.work[w], (unsigned long long)(c1 - c0));
            c0 = c1;
        }
    };
    const uint32_t s = a.s, iter = a.iter;
    const int pp = (a.lid_cur - 1) & 1, cp = a.lid_cur & 1;
    const uint32_t lid_prev = a.lid_cur - 1;
    bytes += 8 + 4ull * d.words;  // tail entry, indicator stamp and row
    // (a) indicator row of t for this batch
    const bool valid = d.ind_stamp[t] == a.b + 1;
    for (uint32_t x = lane; x < d.words; x += 32) wr.ind[x] = valid ? d.ind[(uint64_t)t * d.words + x] : 0u;
    if (lane == 0) wr.ctr[0] = 0;
    __syncwarp();
    // (b) gather first offers from active neighbours (heads >= s)
    const uint32_t e_end = d.off[t + 1];
    for (uint32_t e0 = d.off[t]; e0 < e_end; e0 += 32) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t h = in ? d.adj[e] : 0u;
        const bool ge = in && h >= s;
        const bool act = ge && d.act_stamp[pp][h] == lid_prev;
        uint32_t mask = __ballot_sync(FULL, act);
        bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ge)) * 4ull;
        while (mask) {
            const int src = __ffs(mask) - 1;
            mask &= mask - 1;
            const uint32_t hh = __shfl_sync(FULL, h, src);
            const uint64_t pos = d.last_pos[pp][hh];
            const uint32_t c = d.last_cnt[pp][hh];
            bytes += 12 + 4ull * c;  // last-group position/count and its hubs
            for (uint32_t j = lane; j < c; j += 32) {
                const uint32_t r = d.pool_hub[pos + j];
                if (r < t) {
                    const uint32_t idx = r - s;
                    const uint32_t bit = 1u << (idx & 31);
                    const uint32_t old = atomicOr(&wr.ind[idx >> 5], bit);
                    if (!(old & bit)) wr.offered[atomicAdd(&wr.ctr[0], 1u)] = (uint16_t)idx;
                }
            }
        }
        if (__ballot_sync(FULL, in && !ge)) break;
    }
    __syncwarp();
    const uint32_t noff = wr.ctr[0];
    tick(W_CYC_SCAN);
    if (noff == 0) return;
    bytes += 17ull * d.K + 4ull * d.words + 4;  // tail BP row; indicator write-back
    // (c) BP test in two stages: lane per candidate on BP root 0 (which settles
    // most pairs), then warp-cooperative over the remaining roots for the rest.
    const ulonglong2 zero2 = make_ulonglong2(0, 0);
    const uint8_t td0 = lane < (int)d.K ? d.bpd[(uint64_t)t * d.K + lane] : (uint8_t)U8_INF;
    const uint8_t td1 = lane + 32 < (int)d.K ? d.bpd[(uint64_t)t * d.K + lane + 32] : (uint8_t)U8_INF;
    const ulonglong2 ts0 = lane < (int)d.K ? reinterpret_cast<const ulonglong2 *>(d.bps)[(uint64_t)t * d.K + lane] : zero2;
    const ulonglong2 ts1 =
        lane + 32 < (int)d.K ? reinterpret_cast<const ulonglong2 *>(d.bps)[(uint64_t)t * d.K + lane + 32] : zero2;
    const uint8_t tr0d = __shfl_sync(FULL, td0, 0);
    const ulonglong2 tr0s = make_ulonglong2(__shfl_sync(FULL, ts0.x, 0), __shfl_sync(FULL, ts0.y, 0));
    uint32_t nsurv = 0;
    for (uint32_t c0 = 0; c0 < noff; c0 += 32) {
        const uint32_t c = c0 + lane;
        bool keep = false;
        uint16_t idx = 0;
        if (c < noff) {
            idx = wr.offered[c];
            const uint64_t rr = s + idx;
            keep = d.K == 0 || !bp_one(d.bpd[rr * d.K], reinterpret_cast<const ulonglong2 *>(d.bps)[rr * d.K], tr0d,
                                       tr0s, iter);
        }
        const uint32_t km = __ballot_sync(FULL, keep);
        __syncwarp();
        if (keep) wr.offered[nsurv + __popc(km & ((1u << lane) - 1u))] = idx;
        nsurv += __popc(km);
        __syncwarp();
    }
    if (d.K > 1 && nsurv) {
        uint32_t n2 = 0;
        for (uint32_t c = 0; c < nsurv; c += 2) {
            const uint16_t ia = wr.offered[c];
            const bool two = c + 1 < nsurv;
            const uint16_t ib = two ? wr.offered[c + 1] : ia;
            const bool ca = bp_covered_warp(d, s + ia, lane, 1, td0, ts0, td1, ts1, iter);
            const bool cb = two && bp_covered_warp(d, s + ib, lane, 1, td0, ts0, td1, ts1, iter);
            __syncwarp();
            if (lane == 0) {
                if (!ca) wr.offered[n2] = ia;
                if (two && !cb) wr.offered[n2 + (ca ? 0 : 1)] = ib;
            }
            n2 += (ca ? 0 : 1) + (two && !cb ? 1 : 0);
            __syncwarp();
        }
        nsurv = n2;
    }
    tick(W_CYC_BP);
    // (d) distance test against t's labels with d < iter
    uint32_t nadd = 0;
    const uint32_t len = d.lab_len[t];
    uint64_t base = d.lab_off[t];
    if (nsurv) {
        if (lane == 0) wr.ctr[1] = 0;
        __syncwarp();
        for (uint32_t j = lane; j < len; j += 32) {
            const uint8_t dd = d.pool_dist[base + j];
            if (dd < iter) {
                const uint32_t slot = atomicAdd(&wr.ctr[1], 1u);
                if (slot < SMALL_CAP) {
                    wr.sh[slot] = d.pool_hub[base + j];
                    wr.sd[slot] = dd;
                }
            }
        }
        __syncwarp();
        const uint32_t nsmall = wr.ctr[1];
        bytes += 12 + (uint64_t)len + 4ull * min(nsmall, (uint32_t)SMALL_CAP) + (uint64_t)nsurv * nsmall;
        for (uint32_t c0 = 0; c0 < nsurv; c0 += 32) {
            const uint32_t c = c0 + lane;
            bool keep = false;
            uint16_t idx = 0;
            if (c < nsurv) {
                idx = wr.offered[c];
                const uint32_t rr = s + idx;
                const uint8_t *row = d.dm + (uint64_t)idx * d.n;
                keep = true;
                if (nsmall <= SMALL_CAP) {
                    for (uint32_t k = 0; k < nsmall; ++k) {
                        const uint32_t hh = wr.sh[k];
                        if (hh < rr && (uint32_t)wr.sd[k] + (uint32_t)row[hh] <= iter) { keep = false; break; }
                    }
                } else {
                    for (uint32_t j = 0; j < len; ++j) {
                        const uint32_t dd = d.pool_dist[base + j];
                        if (dd >= iter) continue;
                        const uint32_t hh = d.pool_hub[base + j];
                        if (hh < rr && dd + (uint32_t)row[hh] <= iter) { keep = false; break; }
                    }
                }
            }
            const uint32_t km = __ballot_sync(FULL, keep);
            __syncwarp();
            if (keep) wr.offered[nadd + __popc(km & ((1u << lane) - 1u))] = idx;
            nadd += __popc(km);
            __syncwarp();
        }
    }
    tick(W_CYC_DIST);
    // (e) reserve room and commit
    if (nadd) {
        if (!warp_reserve(d, t, len + nadd, base, lane)) {
            if (lane == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                a.retry[atomicAdd(a.retry_cnt, 1u)] = t;
            }
            return;  // nothing committed; re-run after the pool grows
        }
        const bool is_root = t >= s && t < a.e_roots;
        uint32_t mn = 0xffffffffu;
        for (uint32_t j = lane; j < nadd; j += 32) {
            const uint32_t idx = wr.offered[j];
            d.pool_hub[base + len + j] = s + idx;
            d.pool_dist[base + len + j] = (uint8_t)iter;
            if (is_root) d.dm[(uint64_t)(t - s) * d.n + s + idx] = (uint8_t)iter;
            mn = min(mn, s + idx);
        }
        mn = warp_min_u32(mn);
        bytes += 5ull * nadd + 28 + (is_root ? (uint64_t)nadd : 0);
        if (lane == 0) {
            d.lab_len[t] = len + nadd;
            d.last_pos[cp][t] = base + len;
            d.last_cnt[cp][t] = nadd;
            d.last_min[cp][t] = mn;
            d.act_stamp[cp][t] = a.lid_cur;
            a.front_next[atomicAdd(a.front_next_cnt, 1u)] = t;
        }
    }
    for (uint32_t x = lane; x < d.words; x += 32) d.ind[(uint64_t)t * d.words + x] = wr.ind[x];
    if (lane == 0) d.ind_stamp[t] = a.b + 1;
    __syncwarp();
    tick(W_CYC_COMMIT);
}

// Pull phase of a level: heavy tails block-by-block, then light tails
// warp-by-warp.  Ends with the block converged.
__device__ void pull_phase(const UnwDev &d, const PullArgs &a, unsigned char *pull_smem)
{
    const int lane = threadIdx.x & 31;
    unsigned long long bytes = 0;
    const uint32_t hcnt = a.htails_cnt ? *a.htails_cnt : 0u;
    if (hcnt) {
        const long long h0 = d.work ? clock64() : 0;
        HeavyRegion hs = heavy_region(pull_smem, d.words, d.B);
        for (uint32_t q = blockIdx.x; q < hcnt; q += gridDim.x) {
            pull_heavy_tail(d, a, a.htails[q], hs, bytes);
            __syncthreads();
        }
        if (d.work && threadIdx.x == 0) atomicAdd(&d.work[W_CYC_HEAVY], (unsigned long long)(clock64() - h0));
    }
    const uint32_t cnt = *a.tails_cnt;
    WarpRegion wr = warp_region(pull_smem, d.words, d.B, threadIdx.x >> 5);
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw)
        pull_light_tail(d, a, a.tails[q], wr, bytes);
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_PULL], bytes);
    __syncthreads();
}

__global__ void __launch_bounds__(PULL_THREADS, 4) pull_kernel(UnwDev d, PullArgs a)
{
    extern __shared__ __align__(16) unsigned char pull_smem[];
    pull_phase(d, a, pull_smem);
}

// ---------------------------------------------------------------------------
// Persistent labeling loop: one cooperative launch runs batch after batch,
// level after level, with a grid barrier between phases instead of a kernel
// boundary and a host round trip.  The kernel returns to the host only when
// every batch is done, when the label pool must grow (a warp could not
// reserve space; the failed tails or roots are re-run exactly after the
// growth), or on an error.  The barrier's spin is bounded: after
// BARRIER_TIMEOUT_NS a block records ST_BARRIER_TIMEOUT and returns, so a
// logic error can never leave the GPU spinning.
// ---------------------------------------------------------------------------
enum LoopPhase : uint32_t { PH_BATCH = 0, PH_ROOT_RETRY = 1, PH_LEVEL = 2, PH_PULL_RETRY = 3, PH_DONE = 4 };
enum LoopExit : uint32_t { EX_RUNNING = 0, EX_DONE = 1, EX_NEED_POOL = 2, EX_OVERFLOW = 3, EX_TIMEOUT = 4 };
constexpr unsigned long long BARRIER_TIMEOUT_NS = 4000000000ull;
constexpr uint32_t ST_BARRIER_TIMEOUT = 8u;

struct LoopCtl {
    uint32_t bar_arrive, bar_gen;
    uint32_t phase, b, iter, lid;
    uint32_t front_cnt[2], tails_cnt[2], htails_cnt[2];
    uint32_t nroots[2];  // roots of batch b in nroots[b & 1]
    uint32_t rr_cnt, retry_cnt, status, exit_code;
    uint32_t levels, pad;
};

struct LoopBufs {
    uint32_t *roots;      // roots of the current batch
    uint32_t *rr;         // roots to re-run after a pool growth
    uint32_t *front[2];
    uint32_t *tails, *htails, *retry;
    unsigned long long *batch_ns;  // optional per-batch end time (trace)
    uint32_t nbatches;
};

__device__ __forceinline__ uint32_t vload(const uint32_t *p) { return *(const volatile uint32_t *)p; }

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch.  Returns false (in every
// thread of the block) if the wait timed out.
__device__ bool grid_barrier(LoopCtl *c)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t *gen = &c->bar_gen;
        const uint32_t g = *gen;
        __threadfence();
        const uint32_t arrived = atomicAdd(&c->bar_arrive, 1u) + 1u;
        int good = 1;
        if (arrived == gridDim.x) {
            atomicExch(&c->bar_arrive, 0u);
            __threadfence();
            atomicAdd(&c->bar_gen, 1u);
        } else {
            const unsigned long long t0 = gtimer();
            while (*gen == g) {
                __nanosleep(32);
                if (gtimer() - t0 > BARRIER_TIMEOUT_NS) {
                    atomicOr(&c->status, ST_BARRIER_TIMEOUT);
                    good = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

__global__ void __launch_bounds__(PULL_THREADS, 4) label_loop_kernel(UnwDev d, LoopCtl *c, LoopBufs bf)
{
    extern __shared__ __align__(16) unsigned char pull_smem[];
    const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
    for (;;) {
        const uint32_t phase = vload(&c->phase);
        const uint32_t b = vload(&c->b);
        if (phase == PH_DONE) return;
        if (b >= bf.nbatches) {
            if (leader) {
                c->phase = PH_DONE;
                c->exit_code = EX_DONE;
            }
            return;
        }
        const uint32_t s = b * d.B;
        const uint32_t e = (uint32_t)min((uint64_t)s + d.B, (uint64_t)d.n);
        if (phase == PH_BATCH || phase == PH_ROOT_RETRY) {
            const uint32_t lid0 = vload(&c->lid) + 1;
            const int p0 = lid0 & 1;
            if (phase == PH_BATCH) {
                for (uint32_t r = s + blockIdx.x * blockDim.x + threadIdx.x; r < e; r += gridDim.x * blockDim.x)
                    if (!d.used[r]) bf.roots[atomicAdd(&c->nroots[b & 1], 1u)] = r;
                if (!grid_barrier(c)) return;
                const uint32_t nr = vload(&c->nroots[b & 1]);
                if (nr == 0) {  // every vertex of this batch is a BP vertex
                    if (!grid_barrier(c)) return;
                    if (leader) {
                        c->b = b + 1;
                        c->nroots[(b + 1) & 1] = 0;
                    }
                    if (!grid_barrier(c)) return;
                    continue;
                }
                root_init_phase(d, bf.roots, nr, s, b, lid0, bf.front[p0], &c->front_cnt[p0], bf.retry,
                                &c->retry_cnt);
            } else {
                root_init_phase(d, bf.rr, vload(&c->rr_cnt), s, b, lid0, bf.front[p0], &c->front_cnt[p0], bf.retry,
                                &c->retry_cnt);
            }
            if (!grid_barrier(c)) return;
            if (vload(&c->retry_cnt)) {
                if (leader) {
                    c->phase = PH_ROOT_RETRY;
                    c->exit_code = EX_NEED_POOL;
                }
                return;
            }
            dm_rows_phase(d, bf.roots, vload(&c->nroots[b & 1]), s, 1);
            if (leader) {
                const int p1 = (lid0 + 1) & 1;
                c->nroots[(b + 1) & 1] = 0;  // next batch's count; nobody reads it until then
                c->lid = lid0;
                c->iter = 0;
                c->tails_cnt[p1] = 0;
                c->htails_cnt[p1] = 0;
                c->front_cnt[p1] = 0;
                c->phase = PH_LEVEL;
            }
            if (!grid_barrier(c)) return;
            continue;
        }
        // PH_LEVEL / PH_PULL_RETRY
        const uint32_t lid_cur = vload(&c->lid) + 1;
        const uint32_t iter = vload(&c->iter) + 1;
        const int pp = (lid_cur - 1) & 1, cp = lid_cur & 1;
        if (iter >= U8_INF) {
            if (leader) {
                c->phase = PH_DONE;
                c->exit_code = EX_OVERFLOW;
            }
            return;
        }
        if (phase == PH_LEVEL) {
            mark_phase(d, bf.front[pp], vload(&c->front_cnt[pp]), lid_cur, bf.tails, &c->tails_cnt[cp], bf.htails,
                       &c->htails_cnt[cp]);
            if (!grid_barrier(c)) return;
        }
        PullArgs a{bf.tails, &c->tails_cnt[cp], bf.htails, &c->htails_cnt[cp], s, e, b, iter, lid_cur,
                   bf.front[cp], &c->front_cnt[cp], bf.retry, &c->retry_cnt};
        pull_phase(d, a, pull_smem);
        if (!grid_barrier(c)) return;
        if (vload(&c->retry_cnt)) {
            if (leader) {
                c->phase = PH_PULL_RETRY;
                c->exit_code = EX_NEED_POOL;
            }
            return;
        }
        const uint32_t fn = vload(&c->front_cnt[cp]);
        if (fn == 0) dm_rows_phase(d, bf.roots, vload(&c->nroots[b & 1]), s, 0);
        if (leader) {
            c->lid = lid_cur;
            c->iter = iter;
            c->levels += 1;
            c->tails_cnt[pp] = 0;
            c->htails_cnt[pp] = 0;
            c->front_cnt[pp] = 0;
            if (fn == 0) {
                c->b = b + 1;
                c->phase = PH_BATCH;
                if (bf.batch_ns) bf.batch_ns[b] = gtimer();
            } else {
                c->phase = PH_LEVEL;
            }
        }
        if (!grid_barrier(c)) return;
    }
}

// Final store: copy every list out of the pool, sorting each batch run by hub
// (runs are contiguous because batches append in order).  Entries are unique
// per vertex, so a rank-by-count sort is exact.
__global__ void __launch_bounds__(256) finalize_kernel(UnwDev d, const uint64_t *fin_off, uint32_t *fin_hub,
                                                       uint8_t *fin_dist)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < d.n; v += nw) {
        const uint64_t base = d.lab_off[v], fo = fin_off[v];
        const uint32_t len = d.lab_len[v];
        uint32_t rs = 0;
        while (rs < len) {
            const uint32_t batch = d.pool_hub[base + rs] / d.B;
            // run end: first entry of a later batch (monotone by batch)
            uint32_t re = rs;
            for (;;) {
                const uint32_t j = re + lane;
                const bool same = j < len && d.pool_hub[base + j] / d.B == batch;
                const uint32_t m = __ballot_sync(FULL, same);
                if (m == FULL) { re += 32; continue; }
                re += __ffs(~m) - 1;
                break;
            }
            for (uint32_t c0 = rs; c0 < re; c0 += 32) {
                const uint32_t j = c0 + lane;
                const bool mine = j < re;
                const uint32_t key = mine ? d.pool_hub[base + j] : 0xffffffffu;
                const uint8_t dist = mine ? d.pool_dist[base + j] : 0;
                uint32_t rank = 0;
                for (uint32_t o0 = rs; o0 < re; o0 += 32) {
                    const uint32_t oj = o0 + lane;
                    const uint32_t other = oj < re ? d.pool_hub[base + oj] : 0xffffffffu;
                    for (int k = 0; k < 32; ++k) rank += (__shfl_sync(FULL, other, k) < key) ? 1u : 0u;
                }
                if (mine) {
                    fin_hub[fo + rs + rank] = key;
                    fin_dist[fo + rs + rank] = dist;
                }
            }
            rs = re;
        }
    }
}

}  // namespace

LabelRun unw_label(const DevGraph &g, uint32_t K, uint32_t B, const std::vector<uint8_t> &used,
                   const uint8_t *d_bpd, const uint64_t *d_bps, LabelStore &out, cudaStream_t s)
{
    LabelRun run;
    const uint32_t n = g.n;
    const uint32_t words = (B + 31) / 32;
    PADO_CHECK(B >= 1 && B <= MAX_BATCH, PADO_E_ARG, "batch size must be in [1, 2048]");
    PADO_CHECK(K <= MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");

    DBuf<uint8_t> d_used(std::max<uint32_t>(n, 1));
    d_used.upload(used.data(), n, s);
    uint64_t cap = initial_pool_entries(n);
    DBuf<uint32_t> pool_hub(cap);
    DBuf<uint8_t> pool_dist(cap);
    DBuf<unsigned long long> pool_top(1);
    DBuf<uint64_t> lab_off(n), last_pos0(n), last_pos1(n);
    DBuf<uint32_t> lab_len(n), lab_cap(n), last_cnt0(n), last_cnt1(n), last_min0(n), last_min1(n);
    DBuf<uint32_t> act_stamp0(n), act_stamp1(n), tail_stamp(n), ind_stamp(n);
    DBuf<uint32_t> ind((uint64_t)n * words);
    DBuf<uint8_t> dm((uint64_t)B * n);
    DBuf<uint32_t> front0(n), front1(n), tails(n), htails(n), retry(n), counters(8), status(1);
    DBuf<uint32_t> roots(B);
    pool_top.fill_bytes(0, s);
    lab_off.fill_bytes(0, s);
    lab_len.fill_bytes(0, s);
    lab_cap.fill_bytes(0, s);
    act_stamp0.fill_bytes(0, s);
    act_stamp1.fill_bytes(0, s);
    tail_stamp.fill_bytes(0, s);
    ind_stamp.fill_bytes(0, s);
    dm.fill_bytes(0xff, s);
    status.fill_bytes(0, s);
    counters.fill_bytes(0, s);

    UnwDev d{};
    d.n = n;
    d.K = K;
    d.B = B;
    d.words = words;
    d.off = g.off.p;
    d.adj = g.adj.p;
    d.used = d_used.p;
    d.bpd = d_bpd;
    d.bps = d_bps;
    d.pool_hub = pool_hub.p;
    d.pool_dist = pool_dist.p;
    d.pool_cap = cap;
    d.pool_top = pool_top.p;
    d.lab_off = lab_off.p;
    d.lab_len = lab_len.p;
    d.lab_cap = lab_cap.p;
    d.last_pos[0] = last_pos0.p;
    d.last_pos[1] = last_pos1.p;
    d.last_cnt[0] = last_cnt0.p;
    d.last_cnt[1] = last_cnt1.p;
    d.last_min[0] = last_min0.p;
    d.last_min[1] = last_min1.p;
    d.act_stamp[0] = act_stamp0.p;
    d.act_stamp[1] = act_stamp1.p;
    d.tail_stamp = tail_stamp.p;
    d.ind = ind.p;
    d.ind_stamp = ind_stamp.p;
    d.dm = dm.p;
    d.status = status.p;
    d.work = work_counters();

    // host-pinned mirror of the per-level counters
    struct Ctr { uint32_t front_next, tails, retry, status; unsigned long long top; };
    Ctr *hc = nullptr;
    PADO_CUDA(cudaMallocHost((void **)&hc, sizeof(Ctr)));
    uint32_t *c_front[2] = {counters.p + 0, counters.p + 1};
    uint32_t *c_tails = counters.p + 2, *c_retry = counters.p + 3, *c_htails = counters.p + 4;
    const uint32_t smem = pull_smem_bytes(words, B);
    PADO_CUDA(cudaFuncSetAttribute(pull_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned pull_grid = 152u * 4u;
    uint32_t *fronts[2] = {front0.p, front1.p};

    auto read_ctrs = [&](uint32_t *c_fn) {
        PADO_CUDA(cudaMemcpyAsync(&hc->front_next, c_fn, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->tails, c_tails, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->retry, c_retry, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->status, status.p, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->top, pool_top.p, 8, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaStreamSynchronize(s));
    };
    // Grow the pool to hold at least `need` entries (plus slack), keeping content.
    auto grow_pool = [&](unsigned long long need) {
        uint64_t ncap = std::max<uint64_t>(cap * 2, need + need / 2 + (1u << 20));
        DBuf<uint32_t> nh(ncap);
        DBuf<uint8_t> nd(ncap);
        PADO_CUDA(cudaMemcpyAsync(nh.p, pool_hub.p, cap * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaMemcpyAsync(nd.p, pool_dist.p, cap, cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaStreamSynchronize(s));
        pool_hub = std::move(nh);
        pool_dist = std::move(nd);
        cap = ncap;
        d.pool_hub = pool_hub.p;
        d.pool_dist = pool_dist.p;
        d.pool_cap = cap;
    };

    cudaEvent_t e0, e1;
    PADO_CUDA(cudaEventCreate(&e0));
    PADO_CUDA(cudaEventCreate(&e1));
    PADO_CUDA(cudaEventRecord(e0, s));
    uint32_t lid = 0;
    std::vector<uint32_t> hroots;
    hroots.reserve(B);
    // PADO_TRACE=1: per-batch device time, levels and tails on stderr.
    const bool trace = std::getenv("PADO_TRACE") != nullptr;
    struct TraceRow { uint32_t b, levels; uint64_t tails, front; cudaEvent_t ev; };
    std::vector<TraceRow> trace_rows;
    const uint32_t nbatches = (uint32_t)(((uint64_t)n + B - 1) / B);
    const char *loop_env = std::getenv("PADO_LEVEL_LOOP");
    const bool host_loop = loop_env && !strcmp(loop_env, "host");
    try {
        if (!host_loop && n) {
            // ---- persistent cooperative loop ----
            DBuf<LoopCtl> ctl(1);
            DBuf<uint32_t> rr(B);
            DBuf<unsigned long long> bns(trace ? nbatches : 1);
            ctl.fill_bytes(0, s);
            if (trace) bns.fill_bytes(0, s);
            LoopBufs bf{roots.p, rr.p, {front0.p, front1.p}, tails.p, htails.p, retry.p, trace ? bns.p : nullptr,
                        nbatches};
            PADO_CUDA(cudaFuncSetAttribute(label_loop_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int dev = 0, sms = 0, per_sm = 0;
            PADO_CUDA(cudaGetDevice(&dev));
            PADO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            PADO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, label_loop_kernel, PULL_THREADS, smem));
            PADO_CHECK(per_sm >= 1, PADO_E_CUDA, "labeling loop kernel cannot be resident");
            const unsigned grid = (unsigned)(sms * std::min(per_sm, 4));
            LoopCtl h{};
            LoopCtl *cp_ = ctl.p;
            for (int launch = 0;; ++launch) {
                PADO_CHECK(launch < 256, PADO_E_NOMEM, "label pool could not be grown enough");
                void *args[] = {&d, &cp_, &bf};
                PADO_LAUNCH("label_loop_kernel", s,
                            PADO_CUDA(cudaLaunchCooperativeKernel((void *)label_loop_kernel, grid, PULL_THREADS, args,
                                                                  smem, s)));
                PADO_CUDA(cudaMemcpyAsync(&h, ctl.p, sizeof(LoopCtl), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaStreamSynchronize(s));
                if (h.status & ST_BARRIER_TIMEOUT)
                    throw Error(PADO_E_TIMEOUT, "labeling loop: a grid barrier timed out");
                if (h.exit_code == EX_DONE) break;
                if (h.exit_code == EX_OVERFLOW)
                    throw Error(PADO_E_OVERFLOW, "BFS level reached 255 (uint8 distance overflow)");
                PADO_CHECK(h.exit_code == EX_NEED_POOL, PADO_E_STATE, "labeling loop stopped unexpectedly");
                unsigned long long top = 0;
                PADO_CUDA(cudaMemcpy(&top, pool_top.p, 8, cudaMemcpyDeviceToHost));
                grow_pool(top);
                if (h.phase == PH_ROOT_RETRY) {
                    PADO_CUDA(cudaMemcpyAsync(rr.p, retry.p, h.retry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                    h.rr_cnt = h.retry_cnt;
                } else {
                    const int cpar = (h.lid + 1) & 1;
                    PADO_CUDA(cudaMemcpyAsync(tails.p, retry.p, h.retry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                    h.tails_cnt[cpar] = h.retry_cnt;
                    h.htails_cnt[cpar] = 0;
                }
                h.retry_cnt = 0;
                h.status = 0;
                h.exit_code = EX_RUNNING;
                PADO_CUDA(cudaMemcpyAsync(ctl.p, &h, sizeof(LoopCtl), cudaMemcpyHostToDevice, s));
            }
            run.levels = h.levels;
            run.batches = nbatches;
            if (trace) {
                std::vector<unsigned long long> t(nbatches);
                bns.download(t.data(), nbatches, s);
                PADO_CUDA(cudaStreamSynchronize(s));
                unsigned long long prev = 0;
                for (uint32_t i = 0; i < nbatches; ++i) {
                    if (!t[i]) continue;
                    if (prev) fprintf(stderr, "batch %u ms %.3f\n", i, (t[i] - prev) * 1e-6);
                    prev = t[i];
                }
            }
        }
        for (uint32_t bs = 0, b = 0; host_loop && bs < n; bs += B, ++b) {
            uint32_t b_levels = 0;
            uint64_t b_tails = 0, b_front = 0;
            const uint32_t be = std::min<uint64_t>((uint64_t)bs + B, n);
            hroots.clear();
            for (uint32_t r = bs; r < be; ++r)
                if (!used[r]) hroots.push_back(r);
            ++run.batches;
            if (hroots.empty()) continue;
            const uint32_t nr = (uint32_t)hroots.size();
            roots.upload(hroots.data(), nr, s);
            const uint32_t lid0 = ++lid;
            int cur = lid0 & 1;  // front index holding the vertices active at stamp lid
            PADO_CUDA(cudaMemsetAsync(counters.p, 0, 8 * sizeof(uint32_t), s));
            // roots: self labels (retry until the pool holds them)
            const uint32_t *init_list = roots.p;
            uint32_t init_n = nr;
            for (int attempt = 0;; ++attempt) {
                PADO_CHECK(attempt < 64, PADO_E_NOMEM, "label pool could not be grown enough");
                PADO_LAUNCH("root_init_kernel", s,
                            root_init_kernel<<<grid_for((uint64_t)init_n * 32, 256), 256, 0, s>>>(
                    d, init_list, init_n, bs, b, lid0, fronts[cur], c_front[cur], retry.p, c_retry));
                read_ctrs(c_front[cur]);
                if (!hc->retry) break;
                grow_pool(hc->top);
                PADO_CUDA(cudaMemcpyAsync(tails.p, retry.p, hc->retry * 4, cudaMemcpyDeviceToDevice, s));
                PADO_CUDA(cudaMemsetAsync(c_retry, 0, 4, s));
                PADO_CUDA(cudaMemsetAsync(status.p, 0, 4, s));
                init_list = tails.p;
                init_n = hc->retry;
            }
            PADO_LAUNCH("dm_rows_kernel(fill)", s,
                        dm_rows_kernel<<<grid_for((uint64_t)nr * 32, 256), 256, 0, s>>>(d, roots.p, nr, bs, 1));
            uint32_t fsize = nr;
            for (uint32_t iter = 1; fsize > 0; ++iter) {
                if (iter >= U8_INF)
                    throw Error(PADO_E_OVERFLOW, "BFS level reached 255 (uint8 distance overflow)");
                const uint32_t lid_cur = ++lid;
                const int nxt = cur ^ 1;
                PADO_CUDA(cudaMemsetAsync(c_tails, 0, 4, s));
                PADO_CUDA(cudaMemsetAsync(c_htails, 0, 4, s));
                PADO_CUDA(cudaMemsetAsync(c_front[nxt], 0, 4, s));
                PADO_LAUNCH("mark_kernel", s,
                            mark_kernel<<<grid_for((uint64_t)fsize * 32, 256), 256, 0, s>>>(d, fronts[cur], c_front[cur], lid_cur,
                                                                               tails.p, c_tails, htails.p, c_htails));
                // The tail count is only known on the device: launch for the
                // upper bound n with a grid-stride loop over the real count.
                PADO_LAUNCH("pull_kernel", s,
                            pull_kernel<<<pull_grid, PULL_THREADS, smem, s>>>(
                                d, PullArgs{tails.p, c_tails, htails.p, c_htails, bs, be, b, iter, lid_cur, fronts[nxt],
                                            c_front[nxt], retry.p, c_retry}));
                read_ctrs(c_front[nxt]);
                ++run.levels;
                ++b_levels;
                b_tails += hc->tails;
                b_front += hc->front_next;
                for (int attempt = 0; hc->retry; ++attempt) {
                    PADO_CHECK(attempt < 64, PADO_E_NOMEM, "label pool could not be grown enough");
                    grow_pool(hc->top);
                    PADO_CUDA(cudaMemcpyAsync(tails.p, retry.p, hc->retry * 4, cudaMemcpyDeviceToDevice, s));
                    PADO_CUDA(cudaMemcpyAsync(c_tails, c_retry, 4, cudaMemcpyDeviceToDevice, s));
                    PADO_CUDA(cudaMemsetAsync(c_retry, 0, 4, s));
                    PADO_CUDA(cudaMemsetAsync(status.p, 0, 4, s));
                    PADO_LAUNCH("pull_kernel(retry)", s,
                                pull_kernel<<<pull_grid, PULL_THREADS, smem, s>>>(
                                    d, PullArgs{tails.p, c_tails, nullptr, nullptr, bs, be, b, iter, lid_cur, fronts[nxt],
                                                c_front[nxt], retry.p, c_retry}));
                    read_ctrs(c_front[nxt]);
                }
                fsize = hc->front_next;
                cur = nxt;
            }
            PADO_LAUNCH("dm_rows_kernel(reset)", s,
                        dm_rows_kernel<<<grid_for((uint64_t)nr * 32, 256), 256, 0, s>>>(d, roots.p, nr, bs, 0));
            if (trace) {
                TraceRow tr{b, b_levels, b_tails, b_front, nullptr};
                PADO_CUDA(cudaEventCreate(&tr.ev));
                PADO_CUDA(cudaEventRecord(tr.ev, s));
                trace_rows.push_back(tr);
            }
        }
        if (trace) {
            PADO_CUDA(cudaStreamSynchronize(s));
            cudaEvent_t prev = e0;
            for (auto &tr : trace_rows) {
                float ms = 0;
                cudaEventElapsedTime(&ms, prev, tr.ev);
                fprintf(stderr, "batch %u levels %u tails %llu labeled_vertices %llu ms %.3f\n", tr.b, tr.levels,
                        (unsigned long long)tr.tails, (unsigned long long)tr.front, ms);
                if (prev != e0) cudaEventDestroy(prev);
                prev = tr.ev;
            }
            if (prev != e0) cudaEventDestroy(prev);
        }
        // finalize: exact-size canonical store
        std::vector<uint32_t> lens(n);
        lab_len.download(lens.data(), n, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        std::vector<uint64_t> fo(n + 1, 0);
        for (uint32_t v = 0; v < n; ++v) fo[v + 1] = fo[v] + lens[v];
        out.total = fo[n];
        out.off.alloc(n + 1);
        out.off.upload(fo.data(), n + 1, s);
        out.hub.alloc(std::max<uint64_t>(out.total, 1));
        out.dist8.alloc(std::max<uint64_t>(out.total, 1));
        if (n) {
            PADO_LAUNCH("finalize_kernel", s,
                        finalize_kernel<<<grid_for((uint64_t)n * 32, 256), 256, 0, s>>>(d, out.off.p, out.hub.p, out.dist8.p));
        }
        PADO_CUDA(cudaEventRecord(e1, s));
        PADO_CUDA(cudaEventSynchronize(e1));
        PADO_CUDA(cudaEventElapsedTime(&run.ms, e0, e1));
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFreeHost(hc);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeHost(hc);
    return run;
}

}  // namespace pado
