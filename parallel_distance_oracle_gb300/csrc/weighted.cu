// weighted.cu -- batched pruned relaxation labeling for weighted graphs.
//
// Restates WeightedVertexCentricPLL (reference
// includes/pado_weighted_unv_unp.h:281-1526; OpenMP variant
// includes/pado_weighted_unv_para.h:305-1706).  Per batch of B consecutive
// ranks [s, e) (every vertex is a root; there are no BP labels):
//   initialize (:281-330): roots_labels_buffer[c][h] = d for each committed
//     label (h, d) of root c, buffer[c][c] = 0; each root holds the temporary
//     label (c, 0) and is active.
//   rounds until nothing is active:
//     send (:409-474): an active head h relaxes every root c it accepted in the
//       previous round to each neighbour t > c (lists are descending; t <= s
//       ends the scan): m = (int16)(d_h(c) + w(h, t)) is kept when
//       m < dists_table[t][c] and m < this round's best for (t, c);
//       dists_table[t][c] becomes the round minimum.
//     check (:476-870, :1300-1345): candidate (t, c, m) is pruned when
//       (1) some committed label (h, d) of t has buffer[c][h] finite and
//           d + buffer[c][h] <= m, or
//       (2) some temporary label r < c of t gives d_t(r) + T[c][r] <= m, where
//           T is the temporary table of the vertex whose id is c's batch-local
//           index (:585) -- a no-op after batch 0, since those vertices hold no
//           temporary labels then.
//       Pruned with a smaller covering value q lowers dists_table[t][c] to q.
//       Otherwise t's temporary label for c becomes m and t is active.
//   filter (:1052-1184): drop temporary (v, c) when a temporary r < c of v has
//     d_v(r) <= d_v(c), d_c(r) <= d_v(c) and d_v(r) + d_c(r) <= d_v(c).
//   update_index (:913-950): append the survivors (hub = c's rank, int16 d).
// Device schedule: the reference runs these phases in queue order on one
// thread; here each round is level-synchronous -- all candidates of a round
// are checked against the temporary labels as they stood when the round
// started, and the filter reads the pre-filter values.  The CPU restatement of
// exactly this schedule (the oracle's snapshot mode) produced byte-identical
// label sets to the reference on every graph it was compared on.
//
// Device mapping: as in the unweighted labeler -- the tails of the active
// heads are stamped and listed, and a pull runs a warp per tail that owns the
// tail's rows of dists_table / temporary labels for the round: it min-reduces
// the incoming relaxations per root in shared memory, walks checks (1) and (2)
// per candidate (list entries across the lanes, a ballot for the first
// covering entry), and commits.  The previous round's accepted (root,
// distance) pairs of each vertex are read from a parity-double-buffered log,
// so heads can be read while their owners accept new roots.  dists_table
// entries carry a batch stamp and never need resetting.
//
// Schedule: one persistent cooperative launch (w_loop_kernel) runs every
// batch with a bounded grid barrier between phases instead of a kernel launch
// and a host round trip each: start (the previous batch's roots' temporary
// rows cleared; root tables; the roots mark the first round's tails), one
// phase per round (the pull; a tail that accepts marks the next round's tails
// itself; batch 0 takes a snapshot phase first), end (later batches: filter
// and commit each vertex in one phase; batch 0: filter, then the long lists'
// remaining chunks over the grid, then commit).  It returns to the host only
// to grow the round logs or the label pool (the failed tails or vertices are
// re-run exactly afterwards) or on an error.  PADO_LEVEL_LOOP=host selects the
// host-driven loop of separate kernels (mark, pull, filter, commit) instead.

#include <algorithm>
#include <climits>
#include <cstring>

#include "grid_barrier.cuh"
#include "pado_internal.cuh"

namespace pado {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WPULL_WARPS = 4;
constexpr int32_t RMIN_EMPTY = INT_MAX;

struct WDev {
    uint32_t n, B;
    const uint32_t *off;
    const uint32_t *adj;
    const uint8_t *w;
    uint32_t *pool_hub;
    int16_t *pool_dist;
    unsigned long long pool_cap;
    unsigned long long *pool_top;
    uint64_t *lab_off;
    uint32_t *lab_len;
    uint32_t *lab_cap;
    int16_t *buf;        // [B][n]  roots' committed labels
    int16_t *vd;         // [n][B]  temporary label distances
    uint16_t *vq;        // [n][B]  temporary label roots, first-acceptance order
    uint32_t *vq_len;    // n
    uint32_t *dt;        // [n][B]  (batch+1) << 16 | uint16 distance
    uint32_t *log[2];    // accepted (c << 16 | uint16 d) of each round, by parity
    unsigned long long log_cap;
    unsigned long long *log_top;  // [2]
    uint64_t *last_pos[2];
    uint32_t *last_cnt[2];
    uint32_t *last_min[2];
    uint32_t *act_stamp[2];  // by round parity: round id at which the vertex accepted roots
    uint32_t *tail_stamp;
    int16_t *snap;       // [B][B] rows of vertices < B at round start (batch 0)
    uint64_t *rbase;     // [B] pool position of root c's labels when its buf row was filled
    uint32_t *rlen;      // [B] their count (the row's reset reads these, not the live list,
                         // which a commit in the same phase may extend or move)
    uint32_t *status;
    unsigned long long *work;
};

__device__ __forceinline__ int32_t dt_get(const WDev &d, uint32_t t, uint32_t c, uint32_t stamp)
{
    const uint32_t x = d.dt[(uint64_t)t * d.B + c];
    return (x >> 16) == stamp ? (int32_t)(int16_t)(x & 0xffffu) : (int32_t)I16_INF;
}

__device__ __forceinline__ void dt_put(const WDev &d, uint32_t t, uint32_t c, uint32_t stamp, int32_t v)
{
    d.dt[(uint64_t)t * d.B + c] = (stamp << 16) | (uint32_t)(uint16_t)(int16_t)v;
}

__device__ __forceinline__ uint32_t warp_min_u32(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

__device__ __forceinline__ bool warp_reserve_w(const WDev &d, uint32_t v, uint32_t need, uint64_t &base, int lane)
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

// A head h of round lid - 1 whose smallest accepted root is mn: its
// neighbours t > mn become tails of round lid (stamp lid), once each.  The
// adjacency is in descending order, so the walk stops at the first t <= mn.
// Called by one whole warp.
__device__ __forceinline__ void w_mark_head(const WDev &d, uint32_t h, uint32_t mn, uint32_t lid, uint32_t *tails,
                                            uint32_t *tails_cnt)
{
    const int lane = threadIdx.x & 31;
    const uint32_t e_end = d.off[h + 1];
    for (uint32_t e0 = d.off[h]; e0 < e_end; e0 += 32) {
        const uint32_t e = e0 + lane;
        const bool in = e < e_end;
        const uint32_t t = in ? d.adj[e] : 0u;
        const bool ok = in && t > mn;
        if (ok && d.tail_stamp[t] != lid) {
            if (atomicExch(&d.tail_stamp[t], lid) != lid) tails[agg_append(tails_cnt)] = t;
        }
        if (__ballot_sync(FULL, in && !ok)) break;
    }
}

// The temporary rows of the B vertices from s on (a batch's roots), back to
// INF (the rows are contiguous).
__device__ void w_rows_clear_phase(const WDev &d, uint32_t s)
{
    const uint32_t rows = min(d.B, d.n - s);
    const uint64_t tot = (uint64_t)rows * d.B;
    int16_t *p = d.vd + (uint64_t)s * d.B;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < tot; i += (uint64_t)gridDim.x * blockDim.x)
        p[i] = I16_INF;
}

// initialize_tables (pado_weighted_unv_unp.h:281-330).
// front: the batch roots as the heads of the first round (host-driven loop);
// with `tails` instead, the roots mark the first round's tails themselves.
__device__ void w_root_init_phase(const WDev &d, uint32_t s, uint32_t nroots, uint32_t lid0, uint32_t *front,
                                  uint32_t *front_cnt, uint32_t *news, uint32_t *news_cnt, uint32_t *tails = nullptr,
                                  uint32_t *tails_cnt = nullptr)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int p = lid0 & 1;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nroots; c += nw) {
        const uint32_t r = s + c;
        int16_t *row = d.buf + (uint64_t)c * d.n;
        const uint64_t base = d.lab_off[r];
        const uint32_t len = d.lab_len[r];
        for (uint32_t j = lane; j < len; j += 32) row[d.pool_hub[base + j]] = d.pool_dist[base + j];
        __syncwarp();
        if (lane == 0) {
            d.rbase[c] = base;
            d.rlen[c] = len;
            row[r] = 0;
            d.vq[(uint64_t)r * d.B] = (uint16_t)c;
            d.vq_len[r] = 1;
            d.vd[(uint64_t)r * d.B + c] = 0;
            const unsigned long long pos = atomicAdd(&d.log_top[p], 1ull);
            d.log[p][pos] = (uint32_t)c << 16;
            d.last_pos[p][r] = pos;
            d.last_cnt[p][r] = 1;
            d.last_min[p][r] = r;
            d.act_stamp[p][r] = lid0;
            if (front) front[atomicAdd(front_cnt, 1u)] = r;
            news[atomicAdd(news_cnt, 1u)] = r;
        }
        if (tails) w_mark_head(d, r, r, lid0 + 1, tails, tails_cnt);
    }
}

__global__ void __launch_bounds__(256) w_root_init_kernel(WDev d, uint32_t s, uint32_t nroots, uint32_t lid0,
                                                          uint32_t *front, uint32_t *front_cnt, uint32_t *news,
                                                          uint32_t *news_cnt)
{
    w_root_init_phase(d, s, nroots, lid0, front, front_cnt, news, news_cnt);
}

__device__ void w_mark_phase(const WDev &d, const uint32_t *front, uint32_t cnt, uint32_t lid_cur, uint32_t *tails,
                             uint32_t *tails_cnt)
{
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int pp = (lid_cur - 1) & 1;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) {
        const uint32_t h = front[q];
        w_mark_head(d, h, d.last_min[pp][h], lid_cur, tails, tails_cnt);
    }
}

__global__ void __launch_bounds__(256) w_mark_kernel(WDev d, const uint32_t *front, const uint32_t *front_cnt,
                                                     uint32_t lid_cur, uint32_t *tails, uint32_t *tails_cnt)
{
    w_mark_phase(d, front, *front_cnt, lid_cur, tails, tails_cnt);
}

__device__ void w_snap_phase(const WDev &d, uint32_t rows)
{
    const uint64_t tot = (uint64_t)rows * d.B;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < tot; i += (uint64_t)gridDim.x * blockDim.x)
        d.snap[i] = d.vd[i];
}

__global__ void w_snap_kernel(WDev d, uint32_t rows) { w_snap_phase(d, rows); }

// One chunk of an in-order covering walk (checks (1) and (2) of the pull):
// lane l holds list entry l of the chunk (`in`: the entry exists) with row
// index `key`, order key `kcmp` and distance `el`.  Each pending lane j (bit j
// of `pend`) has candidate root c_j, round minimum m_j and dists row
// base + c_j * stride; the first entry with kcmp < s + c_j whose row value is
// not INF and whose 16-bit sum with el is <= m_j covers it: lane j's r takes
// that sum and bit j leaves the returned mask.  Four candidates are gathered
// per step so that four loads are in flight.
__device__ __forceinline__ uint32_t cover_chunk(uint32_t pend, bool in, uint32_t key, uint32_t kcmp, int32_t el,
                                                const int16_t *base, uint64_t stride, uint32_t c, int32_t m,
                                                uint32_t s, int32_t &r)
{
    const int lane = threadIdx.x & 31;
    uint32_t todo = pend;
    while (todo) {
        int jj[4];
        int32_t mm[4], sk[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            jj[u] = todo ? __ffs(todo) - 1 : -1;
            todo &= todo - 1;  // (0 stays 0)
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t cu = __shfl_sync(FULL, c, jj[u] & 31);
            mm[u] = __shfl_sync(FULL, m, jj[u] & 31);
            sk[u] = (jj[u] >= 0 && in && kcmp < s + cu) ? (int32_t)base[(uint64_t)cu * stride + key] : (int32_t)I16_INF;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int32_t val = (int16_t)(el + sk[u]);
            const uint32_t cov = __ballot_sync(FULL, sk[u] != I16_INF && val <= mm[u]);
            if (cov) {
                const int32_t v = __shfl_sync(FULL, val, __ffs(cov) - 1);
                if (lane == jj[u]) r = v;
                pend &= ~(1u << jj[u]);
            }
        }
    }
    return pend;
}

// The pull of one round (send_messages, pado_weighted_unv_unp.h:409-870, as
// a pull).  Per-warp dynamic shared memory: rmin[B] int32, res[B] int32,
// touched[B] u16.  Run by blocks of WPULL_WARPS warps.
// tq: the round's work counter for dynamic tail claiming (null: static
// grid-stride assignment).  front_next (may be null) collects the next round's
// heads; next_tails (may be null) collects the next round's tails directly.
__device__ void w_pull_phase(const WDev &d, const uint32_t *tails, uint32_t cnt, uint32_t s, uint32_t b,
                             uint32_t lid_cur, uint32_t *front_next, uint32_t *front_next_cnt, uint32_t *news,
                             uint32_t *news_cnt, uint32_t *retry, uint32_t *retry_cnt, unsigned char *wsm,
                             uint32_t *tq = nullptr, uint32_t *next_tails = nullptr, uint32_t *next_tails_cnt = nullptr)
{
    const int lane = threadIdx.x & 31;
    const int w = threadIdx.x >> 5;
    const uint32_t B = d.B;
    int32_t *rmin = reinterpret_cast<int32_t *>(wsm) + (size_t)w * B;
    int32_t *res = reinterpret_cast<int32_t *>(wsm) + (size_t)WPULL_WARPS * B + (size_t)w * B;
    uint16_t *touched = reinterpret_cast<uint16_t *>(reinterpret_cast<int32_t *>(wsm) + (size_t)2 * WPULL_WARPS * B) +
                        (size_t)w * B;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int pp = (lid_cur - 1) & 1, cp = lid_cur & 1;
    const uint32_t lid_prev = lid_cur - 1;
    const uint32_t stamp = b + 1;
    for (uint32_t c = lane; c < B; c += 32) rmin[c] = RMIN_EMPTY;
    __syncwarp();
    unsigned long long bytes = 0;
    const uint32_t below = (1u << lane) - 1u;
    auto pull_tail = [&](const uint32_t t) {
        bytes += 8;
        // (a) round minimum of the relaxations arriving at t, per root.  The
        // active heads' logged roots are flattened into one item list over
        // the lanes (inclusive counts sa), so one round of loads covers 32
        // entries whichever heads they belong to.
        uint32_t ntouch = 0;  // roots touched so far, in `touched`
        const uint32_t e_end = d.off[t + 1];
        for (uint32_t e0 = d.off[t]; e0 < e_end; e0 += 32) {
            const uint32_t e = e0 + lane;
            const bool in = e < e_end;
            const uint32_t h = in ? d.adj[e] : 0u;
            const bool ge = in && h >= s;
            // stamp, log position and size of every head: independent loads
            const uint32_t st = ge ? d.act_stamp[pp][h] : 0u;
            const uint64_t hp = ge ? d.last_pos[pp][h] : 0ull;
            const uint32_t hc = ge ? d.last_cnt[pp][h] : 0u;
            const bool act = ge && st == lid_prev;
            const int32_t wt = act ? (int32_t)d.w[e] : 0;
            const uint32_t ca = act ? hc : 0u;
            const uint64_t pa = act ? hp : 0ull;
            uint32_t sa = ca;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL, sa, o);
                if (lane >= o) sa += y;
            }
            const uint32_t tot = __shfl_sync(FULL, sa, 31);
            if (d.work)
                bytes += __popc(__ballot_sync(FULL, in)) * 4ull + __popc(__ballot_sync(FULL, ge)) * 4ull +
                         __popc(__ballot_sync(FULL, act)) * 13ull + 4ull * tot;
            for (uint32_t i0 = 0; i0 < tot; i0 += 32) {
                const uint32_t i = i0 + lane;
                uint32_t L = 0;  // head lane: the lanes whose inclusive count is <= i
#pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1)
                    if (__shfl_sync(FULL, sa, L + step - 1) <= i) L += step;
                const uint64_t qp = __shfl_sync(FULL, pa, L);
                const uint32_t x0 = __shfl_sync(FULL, sa - ca, L);
                const int32_t ww = __shfl_sync(FULL, wt, L);
                bool fresh = false;
                uint32_t cr = 0;
                if (i < tot) {
                    const uint32_t x = d.log[pp][qp + (i - x0)];
                    cr = x >> 16;
                    if (s + cr < t) {
                        const int32_t m = (int32_t)(int16_t)((int32_t)(int16_t)(x & 0xffffu) + ww);
                        fresh = atomicMin(&rmin[cr], m) == RMIN_EMPTY;
                    }
                }
                // first touches of this round appended in lane order
                const uint32_t fm = __ballot_sync(FULL, fresh);
                if (fresh) touched[ntouch + __popc(fm & below)] = (uint16_t)cr;
                ntouch += __popc(fm);
            }
            if (__ballot_sync(FULL, in && !ge)) break;
        }
        __syncwarp();
        if (ntouch == 0) return;
        // (b) candidates: round minimum below dists_table; checks (1) and (2)
        const uint64_t cbase = d.lab_off[t];
        const uint32_t clen = d.lab_len[t];
        const uint32_t vql = d.vq_len[t];
        uint32_t nacc = 0, nnew = 0, mnacc = 0xffffffffu;
        for (uint32_t i0 = 0; i0 < ntouch; i0 += 32) {
            const uint32_t i = i0 + lane;
            bool acc = false, isnew = false;
            // checks (1) and (2) walk a list in order and stop at its first
            // covering entry, as the reference's loops do.  The lanes hold 32
            // consecutive entries of the list; the candidates still looking
            // (bits of `pend`, one per lane of this group) are taken 4 at a
            // time, each gathering its own row at the 32 entries' keys, and a
            // ballot gives the first covering entry of each.  A candidate
            // leaves the walk at the chunk that covers it.
            uint32_t c = 0, creal = 0;
            int32_t m = 0, r = INT_MAX;  // INT_MAX: not a candidate
            if (i < ntouch) {
                c = touched[i];
                m = rmin[c];
                creal = s + c;
                if (m < dt_get(d, t, c, stamp)) r = INT_MIN;  // accepted unless pruned below
            }
            uint32_t pend = __ballot_sync(FULL, r == INT_MIN);
            // check (1): t's committed labels (hub, distance) against the
            // candidate roots' dists_table rows (buf[c][hub])
            for (uint32_t j0 = 0; j0 < clen && pend; j0 += 32) {
                const bool in = j0 + lane < clen;
                const uint32_t hl = in ? d.pool_hub[cbase + j0 + lane] : 0xffffffffu;
                const int32_t dl = in ? (int32_t)d.pool_dist[cbase + j0 + lane] : 0;
                pend = cover_chunk(pend, in, hl, hl, dl, d.buf, d.n, c, m, s, r);
            }
            // check (2) (batch 0 only): t's temporary labels in acceptance
            // order (root, distance) against the snapshot rows of the
            // candidates' temporary tables, roots before the candidate only
            if (b == 0) {
                const uint16_t *tqp = d.vq + (uint64_t)t * B;
                const int16_t *trow = d.vd + (uint64_t)t * B;
                for (uint32_t k0 = 0; k0 < vql && pend; k0 += 32) {
                    const bool in = k0 + lane < vql;
                    const uint32_t rl = in ? (uint32_t)tqp[k0 + lane] : 0u;
                    const int32_t tl = in ? (int32_t)trow[rl] : 0;
                    pend = cover_chunk(pend, in, rl, s + rl, tl, d.snap, B, c, m, s, r);
                }
            }
            if (i < ntouch) {
                if (r != INT_MAX) {
                    if (r == INT_MIN) {
                        acc = true;
                        isnew = d.vd[(uint64_t)t * B + c] == I16_INF;
                        mnacc = min(mnacc, creal);
                    }
                }
                res[i] = r;
            }
            nacc += __popc(__ballot_sync(FULL, acc));
            nnew += __popc(__ballot_sync(FULL, isnew));
        }
        mnacc = warp_min_u32(mnacc);
        // dists_table reads, committed-label scans (6 B each), accepted entries
        bytes += 4ull * ntouch + 12 + 6ull * clen * ntouch + 8ull * nacc;
        // (c) reserve the log slots for the accepted roots, then commit
        unsigned long long lpos = 0;
        if (nacc) {
            if (lane == 0) lpos = atomicAdd(&d.log_top[cp], (unsigned long long)nacc);
            lpos = __shfl_sync(FULL, lpos, 0);
            if (lpos + nacc > d.log_cap) {
                if (lane == 0) {
                    atomicOr(d.status, ST_POOL_RETRY);
                    retry[atomicAdd(retry_cnt, 1u)] = t;
                }
                for (uint32_t i = lane; i < ntouch; i += 32) rmin[touched[i]] = RMIN_EMPTY;
                __syncwarp();
                return;
            }
        }
        uint32_t accb = 0, newb = 0;
        for (uint32_t i0 = 0; i0 < ntouch; i0 += 32) {
            const uint32_t i = i0 + lane;
            bool acc = false, isnew = false;
            uint32_t c = 0;
            int32_t m = 0;
            if (i < ntouch) {
                c = touched[i];
                m = rmin[c];
                const int32_t r = res[i];
                if (r != INT_MAX) {
                    dt_put(d, t, c, stamp, m);
                    if (r == INT_MIN) {
                        acc = true;
                        isnew = d.vd[(uint64_t)t * B + c] == I16_INF;
                    } else if (r < m) {
                        dt_put(d, t, c, stamp, r);
                    }
                }
            }
            const uint32_t am = __ballot_sync(FULL, acc), nm = __ballot_sync(FULL, isnew);
            const uint32_t below = (1u << lane) - 1u;
            if (acc) {
                d.log[cp][lpos + accb + __popc(am & below)] = (c << 16) | (uint32_t)(uint16_t)(int16_t)m;
                d.vd[(uint64_t)t * B + c] = (int16_t)m;
            }
            if (isnew) d.vq[(uint64_t)t * B + vql + newb + __popc(nm & below)] = (uint16_t)c;
            accb += __popc(am);
            newb += __popc(nm);
        }
        for (uint32_t i = lane; i < ntouch; i += 32) rmin[touched[i]] = RMIN_EMPTY;
        __syncwarp();
        bytes += 4ull * ntouch;  // dists_table writes
        if (lane == 0) {
            if (nnew) {
                d.vq_len[t] = vql + nnew;
                if (vql == 0) news[atomicAdd(news_cnt, 1u)] = t;
            }
            if (nacc) {
                d.last_pos[cp][t] = lpos;
                d.last_cnt[cp][t] = nacc;
                d.last_min[cp][t] = mnacc;
                d.act_stamp[cp][t] = lid_cur;
                if (front_next) front_next[atomicAdd(front_next_cnt, 1u)] = t;
            }
        }
        __syncwarp();
        // t is a head of the next round: with next_tails it marks that
        // round's tails itself (no separate mark phase)
        if (nacc && next_tails) w_mark_head(d, t, mnacc, lid_cur + 1, next_tails, next_tails_cnt);
    };
    if (tq) {
        // dynamic claiming: the next claim is issued before the current tail
        // is processed; each warp over-claims once at the end
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd(tq, 1u);
        q = __shfl_sync(FULL, q, 0);
        while (q < cnt) {
            uint32_t nq = 0;
            if (lane == 0) nq = atomicAdd(tq, 1u);
            pull_tail(tails[q]);
            q = __shfl_sync(FULL, nq, 0);
        }
    } else {
        for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < cnt; q += nw) pull_tail(tails[q]);
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_WPULL], bytes);
}

__global__ void __launch_bounds__(WPULL_WARPS * 32, 8) w_pull_kernel(WDev d, const uint32_t *tails, const uint32_t *tails_cnt,
                                                                  uint32_t s, uint32_t b, uint32_t lid_cur,
                                                                  uint32_t *front_next, uint32_t *front_next_cnt,
                                                                  uint32_t *news, uint32_t *news_cnt, uint32_t *retry,
                                                                  uint32_t *retry_cnt)
{
    extern __shared__ __align__(16) unsigned char wsm[];
    w_pull_phase(d, tails, *tails_cnt, s, b, lid_cur, front_next, front_next_cnt, news, news_cnt, retry, retry_cnt,
                 wsm);
}

// filter_out_labels (pado_weighted_unv_unp.h:1052-1184) on pre-filter values
// for the temporary labels i0 .. i0 + 31 of v (one per lane): label c is
// dropped, by setting bit 15 of its vq slot, when some root r < c of v's list
// has d(v, r) <= d(v, c), d(c, r) <= d(v, c) and d(v, r) + d(c, r) <= d(v, c),
// d(c, r) read from root c's temporary row.  v's list is taken 32 entries at
// a time into the lanes and broadcast; each lane still looking keeps four
// root-row gathers in flight.  Bit 15 is masked off wherever a slot is read,
// so chunks of one v may run in different warps at once.
__device__ __forceinline__ void w_filter_chunk(const WDev &d, uint32_t v, uint32_t L, uint32_t i0, uint32_t s)
{
    const int lane = threadIdx.x & 31;
    const uint32_t B = d.B;
    uint16_t *vq = d.vq + (uint64_t)v * B;
    const int16_t *row = d.vd + (uint64_t)v * B;
    const uint32_t i = i0 + lane;
    const bool valid = i < L;
    uint32_t c = 0;
    int32_t dvc = 0;
    if (valid) {
        c = vq[i] & 0x7fffu;
        dvc = row[c];
    }
    const int16_t *crow = d.vd + (uint64_t)(s + c) * B;
    bool filt = false;
    for (uint32_t k0 = 0; k0 < L && __any_sync(FULL, valid && !filt); k0 += 32) {
        const uint32_t kn = min(32u, L - k0);
        const uint32_t rl = (uint32_t)lane < kn ? (uint32_t)(vq[k0 + lane] & 0x7fffu) : 0u;
        const int32_t dl = (uint32_t)lane < kn ? (int32_t)row[rl] : 0;
        for (uint32_t k = 0; k < kn; k += 4) {
            uint32_t ru[4];
            int32_t du[4], gu[4];
            bool pu[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                ru[u] = __shfl_sync(FULL, rl, (int)(k + u) & 31);
                du[u] = __shfl_sync(FULL, dl, (int)(k + u) & 31);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                pu[u] = valid && !filt && k + u < kn && ru[u] < c && du[u] <= dvc;
                gu[u] = pu[u] ? (int32_t)crow[ru[u]] : 0;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (pu[u] && gu[u] <= dvc && du[u] + gu[u] <= dvc) filt = true;
        }
    }
    __syncwarp();
    if (valid && filt) vq[i] |= 0x8000u;
    __syncwarp();
}

// update_index (pado_weighted_unv_unp.h:913-950) for one vertex v: append the
// unfiltered temporary labels in ascending root order, then clear v's
// temporary row unless `keep_row` (a batch root's row, which other vertices'
// filters still read; it is cleared when the next batch starts).
__device__ __forceinline__ void w_commit_one(const WDev &d, uint32_t v, uint32_t s, uint32_t *retry,
                                             uint32_t *retry_cnt, bool keep_row)
{
    const int lane = threadIdx.x & 31;
    const uint32_t B = d.B;
    const uint32_t L = d.vq_len[v];
    uint16_t *vq = d.vq + (uint64_t)v * B;
    int16_t *row = d.vd + (uint64_t)v * B;
    uint32_t keep = 0;
    for (uint32_t i = lane; i < L; i += 32) keep += (vq[i] & 0x8000u) ? 0u : 1u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) keep += __shfl_xor_sync(FULL, keep, o);
    const uint32_t len = d.lab_len[v];
    uint64_t base;
    if (keep && !warp_reserve_w(d, v, len + keep, base, lane)) {
        if (lane == 0) {
            atomicOr(d.status, ST_POOL_RETRY);
            retry[atomicAdd(retry_cnt, 1u)] = v;
        }
        return;
    }
    if (keep) {
        for (uint32_t i0 = 0; i0 < L; i0 += 32) {
            const uint32_t i = i0 + lane;
            const bool mine = i < L && !(vq[i] & 0x8000u);
            const uint32_t key = mine ? vq[i] : 0xffffffffu;
            uint32_t rank = 0;
            for (uint32_t o0 = 0; o0 < L; o0 += 32) {
                const uint32_t oj = o0 + lane;
                const uint32_t other = (oj < L && !(vq[oj] & 0x8000u)) ? (uint32_t)vq[oj] : 0xffffffffu;
                for (int k = 0; k < 32; ++k) rank += (__shfl_sync(FULL, other, k) < key) ? 1u : 0u;
            }
            if (mine) {
                d.pool_hub[base + len + rank] = s + key;
                d.pool_dist[base + len + rank] = row[key];
            }
        }
    }
    __syncwarp();
    if (!keep_row)
        for (uint32_t i = lane; i < L; i += 32) row[vq[i] & 0x7fffu] = I16_INF;
    __syncwarp();
    if (lane == 0) {
        d.lab_len[v] = len + keep;
        d.vq_len[v] = 0;
    }
}

// Filter of a batch's new-label vertices, a warp per vertex.  With `heavy`,
// a warp filters only the first 32 labels of its vertex and lists the
// vertices with more, whose other chunks w_filter_heavy_phase spreads over the
// grid; with `commit`, each warp commits its vertex right after filtering it
// (roots' rows kept, see w_commit_one).
__device__ void w_filter_phase(const WDev &d, const uint32_t *news, uint32_t nnews, uint32_t s,
                               uint32_t *heavy = nullptr, uint32_t *heavy_cnt = nullptr, bool commit = false,
                               uint32_t nroots = 0, uint32_t *retry = nullptr, uint32_t *retry_cnt = nullptr)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nnews; q += nw) {
        const uint32_t v = news[q];
        const uint32_t L = d.vq_len[v];
        if (heavy) {
            w_filter_chunk(d, v, L, 0, s);
            if (L > 32 && lane == 0) heavy[atomicAdd(heavy_cnt, 1u)] = v;
        } else {
            for (uint32_t i0 = 0; i0 < L; i0 += 32) w_filter_chunk(d, v, L, i0, s);
        }
        if (commit) w_commit_one(d, v, s, retry, retry_cnt, v >= s && v - s < nroots);
    }
}

// The chunks after the first of the listed vertices, one (vertex, chunk) item
// per warp: item j is chunk 1 + j / nheavy of vertex heavy[j % nheavy].
__device__ void w_filter_heavy_phase(const WDev &d, const uint32_t *heavy, uint32_t nheavy, uint32_t s)
{
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint64_t items = (uint64_t)nheavy * ((d.B + 31) / 32 - 1);
    for (uint64_t j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; j < items; j += nw) {
        const uint32_t v = heavy[j % nheavy];
        const uint32_t i0 = 32u * (uint32_t)(1 + j / nheavy);
        const uint32_t L = d.vq_len[v];
        if (i0 < L) w_filter_chunk(d, v, L, i0, s);
    }
}

__global__ void __launch_bounds__(256) w_filter_kernel(WDev d, const uint32_t *news, uint32_t nnews, uint32_t s)
{
    w_filter_phase(d, news, nnews, s);
}

// reset_tables for the roots' buffer rows (pado_weighted_unv_unp.h:872-891):
// the entries the root init set, from the label list as it was then (a list
// slot keeps its first entries when the list grows or moves).
__device__ void w_buf_reset_phase(const WDev &d, uint32_t s, uint32_t nroots)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < nroots; c += nw) {
        const uint32_t r = s + c;
        int16_t *row = d.buf + (uint64_t)c * d.n;
        const uint64_t base = d.rbase[c];
        const uint32_t len = d.rlen[c];
        for (uint32_t j = lane; j < len; j += 32) row[d.pool_hub[base + j]] = I16_INF;
        if (lane == 0) row[r] = I16_INF;
    }
}

__global__ void __launch_bounds__(256) w_buf_reset_kernel(WDev d, uint32_t s, uint32_t nroots)
{
    w_buf_reset_phase(d, s, nroots);
}

// update_index (pado_weighted_unv_unp.h:913-950) for a list of vertices.
__device__ void w_commit_phase(const WDev &d, const uint32_t *news, uint32_t nnews, uint32_t s, uint32_t *retry,
                               uint32_t *retry_cnt, uint32_t nroots = 0)
{
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nnews; q += nw) {
        const uint32_t v = news[q];
        w_commit_one(d, v, s, retry, retry_cnt, v >= s && v - s < nroots);
    }
}

__global__ void __launch_bounds__(256) w_commit_kernel(WDev d, const uint32_t *news, uint32_t nnews, uint32_t s,
                                                       uint32_t *retry, uint32_t *retry_cnt)
{
    w_commit_phase(d, news, nnews, s, retry, retry_cnt);
}

__global__ void __launch_bounds__(256) w_compact_kernel(WDev d, const uint64_t *fin_off, uint32_t *fin_hub,
                                                        int16_t *fin_dist)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t v = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v < d.n; v += nw) {
        const uint64_t base = d.lab_off[v], fo = fin_off[v];
        const uint32_t len = d.lab_len[v];
        for (uint32_t j = lane; j < len; j += 32) {
            fin_hub[fo + j] = d.pool_hub[base + j];
            fin_dist[fo + j] = d.pool_dist[base + j];
        }
    }
}

// ---------------------------------------------------------------------------
// Persistent loop.  Every block keeps the loop state in registers and derives
// the same transitions from the same post-barrier counters; the leader saves
// the state to WLoopCtl only when the launch returns.  Counters are reused by
// parity and cleared one phase ahead of their next use (see each site).
// ---------------------------------------------------------------------------
enum WPhase : uint32_t { WP_START = 0, WP_ROUND = 1, WP_PULL_RETRY = 2, WP_END = 3, WP_COMMIT_RETRY = 4, WP_DONE = 5 };
enum WExit : uint32_t { WX_RUNNING = 0, WX_DONE = 1, WX_NEED_LOG = 2, WX_NEED_POOL = 3, WX_STALL = 4 };

// Round lid reads tails[lid % 3] and appends the next round's tails to
// tails[(lid + 1) % 3] as its heads accept; the leader clears the third slot
// for the round after.
struct WLoopCtl {
    GridBar bar;
    uint32_t phase, b, lid;           // resume point: phase, batch, last stamp
    uint32_t rounds, levels;
    uint32_t tails_cnt[3], news_cnt[2];
    uint32_t tq[3];                   // the pull's work counter, by the round's tails slot
    uint32_t heavy_cnt;               // batch 0's vertices with more than 32 temporary labels
    uint32_t rr_cnt, retry_cnt, status, exit_code;
};

struct WLoopBufs {
    uint32_t *tails[3], *news[2];  // news by batch parity
    uint32_t *rr, *retry, *heavy;
    uint32_t nbatches;
};

__global__ void __launch_bounds__(WPULL_WARPS * 32, 8) w_loop_kernel(WDev d, WLoopCtl *c, WLoopBufs bf)
{
    extern __shared__ __align__(16) unsigned char wsm[];
    const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
    uint32_t phase = vload(&c->phase), b = vload(&c->b), lid = vload(&c->lid);
    uint32_t rounds = vload(&c->rounds), levels = vload(&c->levels);
    auto save = [&](uint32_t ph, uint32_t ex) {
        if (leader) {
            c->phase = ph;
            c->b = b;
            c->lid = lid;
            c->rounds = rounds;
            c->levels = levels;
            c->exit_code = ex;
        }
    };
    for (;;) {
        if (phase == WP_START) {
            if (b >= bf.nbatches) {
                save(WP_DONE, WX_DONE);
                return;
            }
            const uint32_t s = b * d.B, nr = min(d.B, d.n - s);
            const uint32_t lid0 = lid + 1;
            // news[b & 1], log[lid0 & 1] and the first round's tails slot
            // were cleared at the end of the previous batch; the roots mark
            // the first round's tails
            if (b > 0) w_rows_clear_phase(d, s - d.B);  // the previous batch's roots' temporary rows
            w_root_init_phase(d, s, nr, lid0, nullptr, nullptr, bf.news[b & 1], &c->news_cnt[b & 1],
                              bf.tails[(lid0 + 1) % 3], &c->tails_cnt[(lid0 + 1) % 3]);
            if (leader) {
                c->tails_cnt[(lid0 + 2) % 3] = 0;  // filled by the first round
                c->tq[(lid0 + 2) % 3] = 0;
                d.log_top[(lid0 + 1) & 1] = 0;     // the first round's log
            }
            if (!grid_barrier(&c->bar, &c->status)) return;
            lid = lid0;
            rounds = 0;
            phase = WP_ROUND;
            continue;
        }
        if (phase == WP_ROUND || phase == WP_PULL_RETRY) {
            const uint32_t s = b * d.B, nr = min(d.B, d.n - s);
            const uint32_t lid_cur = lid + 1, tp = lid_cur % 3, tn = (lid_cur + 1) % 3;
            if (phase == WP_ROUND) {
                // Bellman-Ford rounds are bounded by the vertex count
                if (rounds > d.n + 2) {
                    save(WP_DONE, WX_STALL);
                    return;
                }
                if (b == 0) {
                    // check (2) reads the batch's temporary tables as of the round start
                    w_snap_phase(d, nr);
                    if (!grid_barrier(&c->bar, &c->status)) return;
                }
            }
            w_pull_phase(d, bf.tails[tp], vload(&c->tails_cnt[tp]), s, b, lid_cur, nullptr, nullptr, bf.news[b & 1],
                         &c->news_cnt[b & 1], bf.retry, &c->retry_cnt, wsm, &c->tq[tp], bf.tails[tn],
                         &c->tails_cnt[tn]);
            if (leader) {
                c->tails_cnt[(lid_cur + 2) % 3] = 0;  // read by the previous round's pull
                c->tq[(lid_cur + 2) % 3] = 0;
                d.log_top[(lid_cur + 1) & 1] = 0;     // the next round's log, last read by this pull
            }
            if (!grid_barrier(&c->bar, &c->status)) return;
            if (vload(&c->retry_cnt)) {
                save(WP_PULL_RETRY, WX_NEED_LOG);
                return;
            }
            ++levels;
            ++rounds;
            lid = lid_cur;
            phase = vload(&c->tails_cnt[tn]) ? WP_ROUND : WP_END;
            continue;
        }
        if (phase == WP_END || phase == WP_COMMIT_RETRY) {
            const uint32_t s = b * d.B, nr = min(d.B, d.n - s), nb = b & 1;
            if (phase == WP_END) {
                const uint32_t nn = vload(&c->news_cnt[nb]);
                if (leader) {
                    d.log_top[(lid + 1) & 1] = 0;  // the next batch's root log (read by the last pull)
                    c->news_cnt[nb ^ 1] = 0;       // the next batch's new-label list
                    c->tails_cnt[(lid + 2) % 3] = 0;  // the next batch's first tails
                    c->tq[(lid + 2) % 3] = 0;
                }
                if (b == 0) {
                    // batch 0 has vertices with hundreds of temporary labels:
                    // their chunks after the first are spread over the grid,
                    // and the commit follows once every filter is done
                    w_filter_phase(d, bf.news[nb], nn, s, bf.heavy, &c->heavy_cnt);
                    if (!grid_barrier(&c->bar, &c->status)) return;
                    w_filter_heavy_phase(d, bf.heavy, vload(&c->heavy_cnt), s);
                    w_buf_reset_phase(d, s, nr);
                    if (!grid_barrier(&c->bar, &c->status)) return;
                    w_commit_phase(d, bf.news[nb], nn, s, bf.retry, &c->retry_cnt);
                } else {
                    // filter and commit each vertex in one go; the roots'
                    // rows, read by other vertices' filters, are cleared when
                    // the next batch starts
                    w_filter_phase(d, bf.news[nb], nn, s, nullptr, nullptr, true, nr, bf.retry, &c->retry_cnt);
                    w_buf_reset_phase(d, s, nr);
                }
            } else {
                w_commit_phase(d, bf.rr, vload(&c->rr_cnt), s, bf.retry, &c->retry_cnt);
            }
            if (!grid_barrier(&c->bar, &c->status)) return;
            if (vload(&c->retry_cnt)) {
                save(WP_COMMIT_RETRY, WX_NEED_POOL);
                return;
            }
            ++b;
            phase = WP_START;
            continue;
        }
        save(WP_DONE, WX_STALL);  // unknown phase
        return;
    }
}

}  // namespace

LabelRun w_label(const DevGraph &g, uint32_t B, LabelStore &out, cudaStream_t s)
{
    LabelRun run;
    const uint32_t n = g.n;
    PADO_CHECK(B >= 1 && B <= MAX_BATCH, PADO_E_ARG, "batch size must be in [1, 2048]");
    PADO_CHECK(n < (1u << 31), PADO_E_ARG, "too many vertices");

    uint64_t cap = initial_pool_entries(n);
    uint64_t lcap = initial_log_entries(n, B);
    DBuf<uint32_t> pool_hub(cap);
    DBuf<int16_t> pool_dist(cap);
    DBuf<unsigned long long> pool_top(1), log_top(2);
    DBuf<uint64_t> lab_off(n), last_pos0(n), last_pos1(n);
    DBuf<uint32_t> lab_len(n), lab_cap(n), last_cnt0(n), last_cnt1(n), last_min0(n), last_min1(n);
    DBuf<uint32_t> act_stamp0(n), act_stamp1(n), tail_stamp(n), vq_len(n);
    DBuf<int16_t> buf((uint64_t)B * n), vd((uint64_t)n * B), snap((uint64_t)B * B);
    DBuf<uint64_t> rbase(B);
    DBuf<uint32_t> rlen(B);
    DBuf<uint16_t> vq((uint64_t)n * B);
    DBuf<uint32_t> dt((uint64_t)n * B);
    DBuf<uint32_t> log0(lcap), log1(lcap);
    DBuf<uint32_t> front0(n), front1(n), tails(n), retry(n), news(n), counters(8), status(1);
    pool_top.fill_bytes(0, s);
    log_top.fill_bytes(0, s);
    lab_off.fill_bytes(0, s);
    lab_len.fill_bytes(0, s);
    lab_cap.fill_bytes(0, s);
    act_stamp0.fill_bytes(0, s);
    act_stamp1.fill_bytes(0, s);
    tail_stamp.fill_bytes(0, s);
    vq_len.fill_bytes(0, s);
    dt.fill_bytes(0, s);       // stamp 0 never matches a batch (stamps start at 1)
    buf.fill_bytes(0xff, s);   // 0xffff is not INF: fixed just below
    vd.fill_bytes(0xff, s);
    status.fill_bytes(0, s);
    {
        // INF = 0x7fff for the int16 tables
        auto fill_inf = [&](int16_t *p, uint64_t cnt) {
            std::vector<int16_t> h(std::min<uint64_t>(cnt, 1u << 20), I16_INF);
            for (uint64_t o = 0; o < cnt; o += h.size()) {
                uint64_t k = std::min<uint64_t>(h.size(), cnt - o);
                PADO_CUDA(cudaMemcpyAsync(p + o, h.data(), k * 2, cudaMemcpyHostToDevice, s));
                PADO_CUDA(cudaStreamSynchronize(s));
            }
        };
        fill_inf(buf.p, buf.n);
        fill_inf(vd.p, vd.n);
    }

    WDev d{};
    d.n = n;
    d.B = B;
    d.off = g.off.p;
    d.adj = g.adj.p;
    d.w = g.w.p;
    d.pool_hub = pool_hub.p;
    d.pool_dist = pool_dist.p;
    d.pool_cap = cap;
    d.pool_top = pool_top.p;
    d.lab_off = lab_off.p;
    d.lab_len = lab_len.p;
    d.lab_cap = lab_cap.p;
    d.buf = buf.p;
    d.vd = vd.p;
    d.vq = vq.p;
    d.vq_len = vq_len.p;
    d.dt = dt.p;
    d.log[0] = log0.p;
    d.log[1] = log1.p;
    d.log_cap = lcap;
    d.log_top = log_top.p;
    d.last_pos[0] = last_pos0.p;
    d.last_pos[1] = last_pos1.p;
    d.last_cnt[0] = last_cnt0.p;
    d.last_cnt[1] = last_cnt1.p;
    d.last_min[0] = last_min0.p;
    d.last_min[1] = last_min1.p;
    d.act_stamp[0] = act_stamp0.p;
    d.act_stamp[1] = act_stamp1.p;
    d.tail_stamp = tail_stamp.p;
    d.rbase = rbase.p;
    d.rlen = rlen.p;
    d.snap = snap.p;
    d.status = status.p;
    d.work = work_counters();

    const size_t pull_smem = (size_t)WPULL_WARPS * B * (4 + 4 + 2);
    PADO_CUDA(cudaFuncSetAttribute(w_pull_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pull_smem));

    struct Ctr { uint32_t front_next, tails, retry, news; unsigned long long top; unsigned long long ltop[2]; };
    Ctr *hc = nullptr;
    PADO_CUDA(cudaMallocHost((void **)&hc, sizeof(Ctr)));
    uint32_t *c_front[2] = {counters.p + 0, counters.p + 1};
    uint32_t *c_tails = counters.p + 2, *c_retry = counters.p + 3, *c_news = counters.p + 4;
    uint32_t *fronts[2] = {front0.p, front1.p};
    auto read_ctrs = [&](uint32_t *c_fn) {
        PADO_CUDA(cudaMemcpyAsync(&hc->front_next, c_fn, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->tails, c_tails, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->retry, c_retry, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->news, c_news, 4, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->top, pool_top.p, 8, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaMemcpyAsync(&hc->ltop[0], log_top.p, 16, cudaMemcpyDeviceToHost, s));
        PADO_CUDA(cudaStreamSynchronize(s));
    };
    auto grow_pool = [&](unsigned long long need) {
        uint64_t ncap = std::max<uint64_t>(cap * 2, need + need / 2 + (1u << 20));
        DBuf<uint32_t> nh(ncap);
        DBuf<int16_t> nd(ncap);
        PADO_CUDA(cudaMemcpyAsync(nh.p, pool_hub.p, cap * 4, cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaMemcpyAsync(nd.p, pool_dist.p, cap * 2, cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaStreamSynchronize(s));
        pool_hub = std::move(nh);
        pool_dist = std::move(nd);
        cap = ncap;
        d.pool_hub = pool_hub.p;
        d.pool_dist = pool_dist.p;
        d.pool_cap = cap;
    };
    // Grow both round logs (the one being written and the one being read).
    auto grow_logs = [&](unsigned long long need) {
        uint64_t ncap = std::max<uint64_t>(lcap * 4, 2 * need);  // a growth costs a relaunch: grow far
        DBuf<uint32_t> n0(ncap), n1(ncap);
        PADO_CUDA(cudaMemcpyAsync(n0.p, log0.p, lcap * 4, cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaMemcpyAsync(n1.p, log1.p, lcap * 4, cudaMemcpyDeviceToDevice, s));
        PADO_CUDA(cudaStreamSynchronize(s));
        log0 = std::move(n0);
        log1 = std::move(n1);
        lcap = ncap;
        d.log[0] = log0.p;
        d.log[1] = log1.p;
        d.log_cap = lcap;
    };

    cudaEvent_t e0, e1;
    PADO_CUDA(cudaEventCreate(&e0));
    PADO_CUDA(cudaEventCreate(&e1));
    PADO_CUDA(cudaEventRecord(e0, s));
    uint32_t lid = 0;
    const uint32_t nbatches = (uint32_t)(((uint64_t)n + B - 1) / B);
    const char *loop_env = std::getenv("PADO_LEVEL_LOOP");
    const bool host_loop = loop_env && !strcmp(loop_env, "host");
    try {
        PADO_CHECK(nbatches < 65535u, PADO_E_ARG, "more than 65534 batches");
        if (!host_loop && n) {
            DBuf<WLoopCtl> ctl(1);
            DBuf<uint32_t> tails2(n), tails3(n), news2(n), rr(n), heavy(n);
            ctl.fill_bytes(0, s);
            WLoopBufs bf{{tails.p, tails2.p, tails3.p}, {news.p, news2.p}, rr.p, retry.p, heavy.p, nbatches};
            const void *kfn = (const void *)w_loop_kernel;
            PADO_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pull_smem));
            int dev = 0, sms = 0, per_sm = 0;
            PADO_CUDA(cudaGetDevice(&dev));
            PADO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            PADO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, WPULL_WARPS * 32, pull_smem));
            PADO_CHECK(per_sm >= 1, PADO_E_CUDA, "weighted labeling loop kernel cannot be resident");
            const unsigned grid = (unsigned)(sms * std::min(per_sm, 8));
            PADO_CHECK(grid <= BAR_GROUP * BAR_MAX_GROUPS, PADO_E_CUDA, "grid larger than the barrier supports");
            WLoopCtl h{};
            WLoopCtl *cptr = ctl.p;
            for (int launch = 0;; ++launch) {
                PADO_CHECK(launch < 512, PADO_E_NOMEM, "round log or label pool could not be grown enough");
                void *args[] = {&d, &cptr, &bf};
                PADO_LAUNCH("w_loop_kernel", s,
                            PADO_CUDA(cudaLaunchCooperativeKernel(kfn, grid, WPULL_WARPS * 32, args, pull_smem, s)));
                PADO_CUDA(cudaMemcpyAsync(&h, ctl.p, sizeof(WLoopCtl), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaStreamSynchronize(s));
                if (h.status & ST_BARRIER_TIMEOUT)
                    throw Error(PADO_E_TIMEOUT, "weighted labeling loop: a grid barrier timed out");
                if (std::getenv("PADO_TRACE"))
                    fprintf(stderr, "weighted loop launch %d: exit %u at batch %u (retry %u)\n", launch, h.exit_code,
                            h.b, h.retry_cnt);
                if (h.exit_code == WX_DONE) break;
                if (h.exit_code == WX_STALL) throw Error(PADO_E_STATE, "relaxation did not converge");
                if (h.exit_code == WX_NEED_LOG) {
                    unsigned long long lt[2];
                    PADO_CUDA(cudaMemcpy(lt, log_top.p, 16, cudaMemcpyDeviceToHost));
                    grow_logs(lt[(h.lid + 1) & 1]);
                    // the failed tails become the whole tail list of the round;
                    // the next round's tails marked so far stay
                    const uint32_t tp = (h.lid + 1) % 3;
                    PADO_CUDA(cudaMemcpyAsync(bf.tails[tp], retry.p, h.retry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                    h.tails_cnt[tp] = h.retry_cnt;
                    h.tq[tp] = 0;  // the re-run pull claims from zero
                } else {
                    PADO_CHECK(h.exit_code == WX_NEED_POOL, PADO_E_STATE, "weighted labeling loop stopped unexpectedly");
                    unsigned long long top = 0;
                    PADO_CUDA(cudaMemcpy(&top, pool_top.p, 8, cudaMemcpyDeviceToHost));
                    grow_pool(top);
                    PADO_CUDA(cudaMemcpyAsync(rr.p, retry.p, h.retry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                    h.rr_cnt = h.retry_cnt;
                }
                h.retry_cnt = 0;
                h.status = 0;
                h.exit_code = WX_RUNNING;
                PADO_CUDA(cudaMemsetAsync(status.p, 0, 4, s));
                PADO_CUDA(cudaMemcpyAsync(ctl.p, &h, sizeof(WLoopCtl), cudaMemcpyHostToDevice, s));
            }
            run.levels = h.levels;
            run.batches = nbatches;
        }
        for (uint32_t bs = 0, b = 0; host_loop && bs < n; bs += B, ++b) {
            PADO_CHECK(b + 1 < 65536u, PADO_E_ARG, "more than 65534 batches");
            const uint32_t nr = (uint32_t)std::min<uint64_t>(B, (uint64_t)n - bs);
            ++run.batches;
            const uint32_t lid0 = ++lid;
            int cur = lid0 & 1;
            PADO_CUDA(cudaMemsetAsync(counters.p, 0, 8 * sizeof(uint32_t), s));
            PADO_CUDA(cudaMemsetAsync(&log_top.p[lid0 & 1], 0, 8, s));
            PADO_LAUNCH("w_root_init_kernel", s,
                        w_root_init_kernel<<<grid_for((uint64_t)nr * 32, 256), 256, 0, s>>>(d, bs, nr, lid0, fronts[cur], c_front[cur],
                                                                                news.p, c_news));
            uint32_t fsize = nr;
            for (uint64_t round = 0; fsize > 0; ++round) {
                // Bellman-Ford rounds are bounded by the vertex count
                PADO_CHECK(round <= (uint64_t)n + 2, PADO_E_STATE, "relaxation did not converge");
                const uint32_t lid_cur = ++lid;
                const int nxt = cur ^ 1;
                PADO_CUDA(cudaMemsetAsync(c_tails, 0, 4, s));
                PADO_CUDA(cudaMemsetAsync(c_front[nxt], 0, 4, s));
                PADO_CUDA(cudaMemsetAsync(&log_top.p[lid_cur & 1], 0, 8, s));
                if (b == 0) {
                    PADO_LAUNCH("w_snap_kernel", s,
                                w_snap_kernel<<<grid_for((uint64_t)nr * B, 256), 256, 0, s>>>(d, nr));
                }
                PADO_LAUNCH("w_mark_kernel", s,
                            w_mark_kernel<<<grid_for((uint64_t)fsize * 32, 256), 256, 0, s>>>(d, fronts[cur], c_front[cur], lid_cur,
                                                                                 tails.p, c_tails));
                PADO_LAUNCH("w_pull_kernel", s,
                            w_pull_kernel<<<grid_for((uint64_t)n * 32, WPULL_WARPS * 32, 152u * 8u), WPULL_WARPS * 32, pull_smem, s>>>(
                    d, tails.p, c_tails, bs, b, lid_cur, fronts[nxt], c_front[nxt], news.p, c_news, retry.p, c_retry));
                read_ctrs(c_front[nxt]);
                ++run.levels;
                for (int attempt = 0; hc->retry; ++attempt) {
                    PADO_CHECK(attempt < 64, PADO_E_NOMEM, "round log could not be grown enough");
                    grow_logs(hc->ltop[lid_cur & 1]);
                    PADO_CUDA(cudaMemcpyAsync(tails.p, retry.p, hc->retry * 4, cudaMemcpyDeviceToDevice, s));
                    PADO_CUDA(cudaMemcpyAsync(c_tails, c_retry, 4, cudaMemcpyDeviceToDevice, s));
                    PADO_CUDA(cudaMemsetAsync(c_retry, 0, 4, s));
                    PADO_CUDA(cudaMemsetAsync(status.p, 0, 4, s));
                    PADO_LAUNCH("w_pull_kernel(retry)", s,
                                w_pull_kernel<<<grid_for((uint64_t)hc->retry * 32, WPULL_WARPS * 32, 152u * 8u), WPULL_WARPS * 32,
                                    pull_smem, s>>>(d, tails.p, c_tails, bs, b, lid_cur, fronts[nxt], c_front[nxt],
                                                    news.p, c_news, retry.p, c_retry));
                    read_ctrs(c_front[nxt]);
                }
                fsize = hc->front_next;
                cur = nxt;
            }
            read_ctrs(c_front[cur]);
            const uint32_t nn = hc->news;
            PADO_LAUNCH("w_filter_kernel", s,
                        w_filter_kernel<<<grid_for((uint64_t)nn * 32, 256), 256, 0, s>>>(d, news.p, nn, bs));
            PADO_LAUNCH("w_buf_reset_kernel", s,
                        w_buf_reset_kernel<<<grid_for((uint64_t)nr * 32, 256), 256, 0, s>>>(d, bs, nr));
            const uint32_t *clist = news.p;
            uint32_t cn = nn;
            for (int attempt = 0;; ++attempt) {
                PADO_CHECK(attempt < 64, PADO_E_NOMEM, "label pool could not be grown enough");
                PADO_LAUNCH("w_commit_kernel", s,
                            w_commit_kernel<<<grid_for((uint64_t)cn * 32, 256), 256, 0, s>>>(d, clist, cn, bs, retry.p, c_retry));
                read_ctrs(c_front[cur]);
                if (!hc->retry) break;
                grow_pool(hc->top);
                PADO_CUDA(cudaMemcpyAsync(tails.p, retry.p, hc->retry * 4, cudaMemcpyDeviceToDevice, s));
                PADO_CUDA(cudaMemsetAsync(c_retry, 0, 4, s));
                PADO_CUDA(cudaMemsetAsync(status.p, 0, 4, s));
                clist = tails.p;
                cn = hc->retry;
            }
        }
        std::vector<uint32_t> lens(n);
        lab_len.download(lens.data(), n, s);
        PADO_CUDA(cudaStreamSynchronize(s));
        std::vector<uint64_t> fo(n + 1, 0);
        for (uint32_t v = 0; v < n; ++v) fo[v + 1] = fo[v] + lens[v];
        out.total = fo[n];
        out.off.alloc(n + 1);
        out.off.upload(fo.data(), n + 1, s);
        out.hub.alloc(std::max<uint64_t>(out.total, 1));
        out.dist16.alloc(std::max<uint64_t>(out.total, 1));
        if (n) {
            PADO_LAUNCH("w_compact_kernel", s,
                        w_compact_kernel<<<grid_for((uint64_t)n * 32, 256), 256, 0, s>>>(d, out.off.p, out.hub.p, out.dist16.p));
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
