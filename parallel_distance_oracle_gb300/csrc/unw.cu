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
#include <numeric>

#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int PULL_WARPS = 4;                  // warps per block in the pull kernel
constexpr int SMALL_CAP = 256;                 // labels with d < iter staged in smem

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
__global__ void __launch_bounds__(256) root_init_kernel(UnwDev d, const uint32_t *roots, uint32_t nroots,
                                                        uint32_t s, uint32_t b, uint32_t lid0,
                                                        uint32_t *front, uint32_t *front_cnt,
                                                        uint32_t *retry, uint32_t *retry_cnt)
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

// dist_matrix rows of the batch roots: fill from their labels (value = d) or
// reset to 255 (pado_unw_unv_unp.h:492-526 and :780-816).
__global__ void __launch_bounds__(256) dm_rows_kernel(UnwDev d, const uint32_t *roots, uint32_t nroots, uint32_t s,
                                                      int fill)
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

// Tail marking: for each active head, neighbours t (descending) with
// t > min(root of its last group) that are not BP vertices.
__global__ void __launch_bounds__(256) mark_kernel(UnwDev d, const uint32_t *front, const uint32_t *front_cnt,
                                                   uint32_t lid_cur, uint32_t *tails, uint32_t *tails_cnt)
{
    const int lane = threadIdx.x & 31;
    const uint32_t cnt = *front_cnt;
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

struct PullSmem {
    uint32_t ind[PULL_WARPS][MAX_BATCH / 32];
    uint16_t offered[PULL_WARPS][MAX_BATCH];
    uint8_t tbpd[PULL_WARPS][MAX_BP];
    ulonglong2 tbps[PULL_WARPS][MAX_BP];
    uint32_t sh[PULL_WARPS][SMALL_CAP];
    uint8_t sd[PULL_WARPS][SMALL_CAP];
    uint32_t noff[PULL_WARPS];
    uint32_t nsmall[PULL_WARPS];
};

// BP coverage of (root r, tail t) at `iter`, t's row in shared memory
// (pado_unw_unv_unp.h:599-623, unsigned arithmetic).
__device__ __forceinline__ bool bp_covered(const UnwDev &d, uint32_t r, const uint8_t *tbpd, const ulonglong2 *tbps,
                                           uint32_t iter)
{
    const uint8_t *rd = d.bpd + (uint64_t)r * d.K;
    const ulonglong2 *rs = reinterpret_cast<const ulonglong2 *>(d.bps + (uint64_t)r * d.K * 2);
    for (uint32_t i = 0; i < d.K; ++i) {
        uint32_t td = (uint32_t)rd[i] + (uint32_t)tbpd[i];
        if (td - 2u <= iter) {
            const ulonglong2 a = rs[i], t = tbps[i];
            if (a.x & t.x)
                td -= 2u;
            else if ((a.x & t.y) | (a.y & t.x))
                td -= 1u;
            if (td <= iter) return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(PULL_WARPS * 32) pull_kernel(UnwDev d, const uint32_t *tails, const uint32_t *tails_cnt,
                                                               uint32_t s, uint32_t e_roots, uint32_t b, uint32_t iter,
                                                               uint32_t lid_cur, uint32_t *front_next,
                                                               uint32_t *front_next_cnt, uint32_t *retry,
                                                               uint32_t *retry_cnt)
{
    __shared__ PullSmem sm;
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const uint32_t cnt = *tails_cnt;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int pp = (lid_cur - 1) & 1, cp = lid_cur & 1;
    const uint32_t lid_prev = lid_cur - 1;
    uint32_t *s_ind = sm.ind[w];
    uint16_t *s_off = sm.offered[w];
    unsigned long long bytes = 0;  // lane 0's tally of algorithmic bytes
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const uint32_t t = tails[q];
        bytes += 8 + 4ull * d.words;  // tail entry, indicator stamp and row
        // (a) indicator row of t for this batch
        const bool valid = d.ind_stamp[t] == b + 1;
        for (uint32_t x = lane; x < d.words; x += 32) s_ind[x] = valid ? d.ind[(uint64_t)t * d.words + x] : 0u;
        if (lane == 0) sm.noff[w] = 0;
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
                        const uint32_t old = atomicOr(&s_ind[idx >> 5], bit);
                        if (!(old & bit)) s_off[atomicAdd(&sm.noff[w], 1u)] = (uint16_t)idx;
                    }
                }
            }
            if (__ballot_sync(FULL, in && !ge)) break;
        }
        __syncwarp();
        const uint32_t noff = sm.noff[w];
        if (noff == 0) continue;
        bytes += 17ull * d.K + 4ull * d.words + 4;  // tail BP row; indicator write-back
        // (c) BP test, lane per candidate, t's BP row in shared memory
        for (uint32_t i = lane; i < d.K; i += 32) {
            sm.tbpd[w][i] = d.bpd[(uint64_t)t * d.K + i];
            sm.tbps[w][i] = reinterpret_cast<const ulonglong2 *>(d.bps)[(uint64_t)t * d.K + i];
        }
        __syncwarp();
        uint32_t nsurv = 0;
        for (uint32_t c0 = 0; c0 < noff; c0 += 32) {
            const uint32_t c = c0 + lane;
            bool keep = false;
            uint16_t idx = 0;
            if (c < noff) {
                idx = s_off[c];
                keep = !bp_covered(d, s + idx, sm.tbpd[w], sm.tbps[w], iter);
            }
            const uint32_t km = __ballot_sync(FULL, keep);
            __syncwarp();
            if (keep) s_off[nsurv + __popc(km & ((1u << lane) - 1u))] = idx;
            nsurv += __popc(km);
            __syncwarp();
        }
        // (d) distance test against t's labels with d < iter
        uint32_t nadd = 0;
        const uint32_t len = d.lab_len[t];
        uint64_t base = d.lab_off[t];
        if (nsurv) {
            if (lane == 0) sm.nsmall[w] = 0;
            __syncwarp();
            for (uint32_t j = lane; j < len; j += 32) {
                const uint8_t dd = d.pool_dist[base + j];
                if (dd < iter) {
                    const uint32_t slot = atomicAdd(&sm.nsmall[w], 1u);
                    if (slot < SMALL_CAP) {
                        sm.sh[w][slot] = d.pool_hub[base + j];
                        sm.sd[w][slot] = dd;
                    }
                }
            }
            __syncwarp();
            const uint32_t nsmall = sm.nsmall[w];
            bytes += 12 + (uint64_t)len + 4ull * min(nsmall, (uint32_t)SMALL_CAP) + (uint64_t)nsurv * nsmall;
            for (uint32_t c0 = 0; c0 < nsurv; c0 += 32) {
                const uint32_t c = c0 + lane;
                bool keep = false;
                uint16_t idx = 0;
                if (c < nsurv) {
                    idx = s_off[c];
                    const uint32_t rr = s + idx;
                    const uint8_t *row = d.dm + (uint64_t)idx * d.n;
                    keep = true;
                    if (nsmall <= SMALL_CAP) {
                        for (uint32_t k = 0; k < nsmall; ++k) {
                            const uint32_t hh = sm.sh[w][k];
                            if (hh < rr && (uint32_t)sm.sd[w][k] + (uint32_t)row[hh] <= iter) { keep = false; break; }
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
                if (keep) s_off[nadd + __popc(km & ((1u << lane) - 1u))] = idx;
                nadd += __popc(km);
                __syncwarp();
            }
        }
        // (e) reserve room and commit
        if (nadd) {
            if (!warp_reserve(d, t, len + nadd, base, lane)) {
                if (lane == 0) {
                    atomicOr(d.status, ST_POOL_RETRY);
                    retry[atomicAdd(retry_cnt, 1u)] = t;
                }
                continue;  // nothing committed; re-run after the pool grows
            }
            const bool is_root = t >= s && t < e_roots;
            uint32_t mn = 0xffffffffu;
            for (uint32_t j = lane; j < nadd; j += 32) {
                const uint32_t idx = s_off[j];
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
                d.act_stamp[cp][t] = lid_cur;
                front_next[atomicAdd(front_next_cnt, 1u)] = t;
            }
        }
        for (uint32_t x = lane; x < d.words; x += 32) d.ind[(uint64_t)t * d.words + x] = s_ind[x];
        if (lane == 0) d.ind_stamp[t] = b + 1;
        __syncwarp();
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_PULL], bytes);
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
    DBuf<uint32_t> front0(n), front1(n), tails(n), retry(n), counters(8), status(1);
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
    uint32_t *c_tails = counters.p + 2, *c_retry = counters.p + 3;
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
    try {
        for (uint32_t bs = 0, b = 0; bs < n; bs += B, ++b) {
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
                PADO_CUDA(cudaMemsetAsync(c_front[nxt], 0, 4, s));
                PADO_LAUNCH("mark_kernel", s,
                            mark_kernel<<<grid_for((uint64_t)fsize * 32, 256), 256, 0, s>>>(d, fronts[cur], c_front[cur], lid_cur,
                                                                               tails.p, c_tails));
                // The tail count is only known on the device: launch for the
                // upper bound n with a grid-stride loop over the real count.
                PADO_LAUNCH("pull_kernel", s,
                            pull_kernel<<<grid_for((uint64_t)n * 32, PULL_WARPS * 32, 152u * 16u), PULL_WARPS * 32, 0, s>>>(
                    d, tails.p, c_tails, bs, be, b, iter, lid_cur, fronts[nxt], c_front[nxt], retry.p, c_retry));
                read_ctrs(c_front[nxt]);
                ++run.levels;
                for (int attempt = 0; hc->retry; ++attempt) {
                    PADO_CHECK(attempt < 64, PADO_E_NOMEM, "label pool could not be grown enough");
                    grow_pool(hc->top);
                    PADO_CUDA(cudaMemcpyAsync(tails.p, retry.p, hc->retry * 4, cudaMemcpyDeviceToDevice, s));
                    PADO_CUDA(cudaMemcpyAsync(c_tails, c_retry, 4, cudaMemcpyDeviceToDevice, s));
                    PADO_CUDA(cudaMemsetAsync(c_retry, 0, 4, s));
                    PADO_CUDA(cudaMemsetAsync(status.p, 0, 4, s));
                    PADO_LAUNCH("pull_kernel(retry)", s,
                                pull_kernel<<<grid_for((uint64_t)hc->retry * 32, PULL_WARPS * 32, 152u * 16u), PULL_WARPS * 32, 0,
                                  s>>>(d, tails.p, c_tails, bs, be, b, iter, lid_cur, fronts[nxt], c_front[nxt],
                                       retry.p, c_retry));
                    read_ctrs(c_front[nxt]);
                }
                fsize = hc->front_next;
                cur = nxt;
            }
            PADO_LAUNCH("dm_rows_kernel(reset)", s,
                        dm_rows_kernel<<<grid_for((uint64_t)nr * 32, 256), 256, 0, s>>>(d, roots.p, nr, bs, 0));
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
