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
#include <optional>

#include "unw_device.cuh"

namespace pado {
namespace {

__global__ void __launch_bounds__(256) root_init_kernel(UnwDev d, const uint32_t *roots, uint32_t nroots,
                                                        uint32_t s, uint32_t b, uint32_t lid0,
                                                        uint32_t *front, uint32_t *front_cnt,
                                                        uint32_t *retry, uint32_t *retry_cnt)
{
    root_init_phase(d, roots, nroots, s, b, lid0, front, front_cnt, retry, retry_cnt);
}

__global__ void __launch_bounds__(256) dm_rows_kernel(UnwDev d, const uint32_t *roots, uint32_t nroots, uint32_t s,
                                                      int fill)
{
    dm_rows_phase(d, roots, nroots, s, fill);
}

__global__ void __launch_bounds__(256) mark_kernel(UnwDev d, const uint32_t *front, const uint32_t *front_cnt,
                                                   uint32_t lid_cur, uint32_t *tails, uint32_t *tails_cnt,
                                                   uint32_t *htails, uint32_t *htails_cnt)
{
    mark_phase(d, front, *front_cnt, lid_cur, tails, tails_cnt, htails, htails_cnt);
}

__global__ void __launch_bounds__(PULL_THREADS, 4) pull_kernel(UnwDev d, PullArgs a)
{
    extern __shared__ __align__(16) unsigned char pull_smem[];
    pull_phase(d, a, pull_smem);
}

// ---------------------------------------------------------------------------
// Persistent labeling loop: one cooperative launch runs batch after batch,
// level after level, with ONE grid barrier per step:
//   batch step (batch b at stamp L): each root r of b gets its self label
//       (stamp L), fills dist_matrix row r - s from its labels and marks its
//       own tails for L+1; the rows of batch b-1 are reset in the same step
//       (dist_matrix is double-buffered by batch parity, so the two never
//       share a row);
//   level step (stamp L, level iter): pull over the tails marked for L; a
//       tail that gains labels marks its tails for L+1 at once.
// After the barrier every block reads the same tail count for L+1 and takes
// the same decision (no tails: the batch is over -- its next level would add
// nothing -- and the next step starts batch b+1), so no leader round trip is
// needed.  Tail lists and their counters rotate over 3 slots by stamp: slot
// L % 3 is read, (L+1) % 3 is appended to, and (L+2) % 3 -- last read at L-1
// -- is cleared for the step after.  The kernel returns to the host only when
// every batch is done, when the label pool must grow (a warp could not
// reserve space; the failed tails or roots are re-run exactly after the
// growth), or on an error.  The barrier's spin is bounded: after
// BARRIER_TIMEOUT_NS a block records ST_BARRIER_TIMEOUT and returns, so a
// logic error can never leave the GPU spinning.
// ---------------------------------------------------------------------------
enum LoopPhase : uint32_t { PH_BATCH = 0, PH_ROOT_RETRY = 1, PH_LEVEL = 2, PH_PULL_RETRY = 3, PH_DONE = 4 };
enum LoopExit : uint32_t { EX_RUNNING = 0, EX_DONE = 1, EX_NEED_POOL = 2, EX_OVERFLOW = 3, EX_TIMEOUT = 4 };

struct LoopCtl {
    GridBar bar;
    uint32_t phase, b, iter, lid;       // the step to run next: phase, batch, level, last completed stamp
    uint32_t tcnt[3], hcnt[3];          // light / heavy tails marked for stamp x, in slot x % 3
    uint32_t tq[3], hq[3];              // work counters of the level at stamp x (dynamic assignment)
    uint32_t rr_cnt, retry_cnt, status, exit_code;
    uint32_t levels, pad;
};

struct LoopBufs {
    const uint32_t *broots;   // roots of every batch, batch by batch
    const uint32_t *boff;     // batch b's roots: broots[boff[b], boff[b+1])
    uint32_t *rr;             // roots to re-run after a pool growth
    uint32_t *tails[3], *htails[3], *retry;
    uint8_t *dm[2];           // dist_matrix by batch parity
    unsigned long long *batch_ns;  // optional per-batch end time (trace)
    unsigned long long *level_log; // optional per level: end time, tails << 32 | batch (trace)
    uint32_t level_cap;
    uint32_t nbatches;
};

// Batch step for roots[0, nr): self label at stamp L, dist_matrix row, tails for L+1.
__device__ void root_step_phase(const UnwDev &d, const uint32_t *roots, uint32_t nr, uint32_t s, uint32_t b,
                                uint32_t L, uint8_t *dm, const LoopBufs &bf, LoopCtl *c)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int p = L & 1, nx = (L + 1) % 3;
    unsigned long long bytes = 0;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nr; q += nw) {
        const uint32_t r = roots[q];
        uint64_t base;
        if (!warp_reserve(d, r, UD_AT(d.lab_len, r, d.n, 1) + 1, base, lane)) {
            if (lane == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                bf.retry[atomicAdd(&c->retry_cnt, 1u)] = r;
            }
            continue;
        }
        const uint32_t len = UD_AT(d.lab_len, r, d.n, 1);
        const uint32_t idx = r - s;
        for (uint32_t w = lane; w < d.words; w += 32)
            UD_AT(d.ind, (uint64_t)r * d.words + w, (uint64_t)d.n * d.words, 5) = (w == (idx >> 5)) ? (1u << (idx & 31)) : 0u;
        if (lane == 0) {
            if (d.work) atomicAdd(&d.work[W_EV_LABELS], 1ull);
            UD_AT(d.pool_hub, base + len, d.pool_cap, 2) = r;
            UD_AT(d.pool_dist, base + len, d.pool_cap, 2) = 0;
            UD_AT(d.lab_len, r, d.n, 1) = len + 1;
            UD_AT(d.last[p], r, d.n, 1) = LastGroup{base + len, 1u, L};
            UD_AT(d.last_min[p], r, d.n, 1) = r;
            UD_AT(d.ind_stamp, r, d.n, 1) = b + 1;
        }
        __syncwarp();
        // dist_matrix row of r from all its labels, the new (r, 0) included
        uint8_t *row = dm + (uint64_t)idx * d.n;
        for (uint32_t j = lane; j <= len; j += 32)
            UD_AT(row, UD_AT(d.pool_hub, base + j, d.pool_cap, 2), d.n, 4) = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
        mark_tails(d, r, r, L + 1, bf.tails[nx], &c->tcnt[nx], bf.htails[nx], &c->hcnt[nx], lane, 0, 1, bytes);
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_MARK], bytes);
}

__global__ void __launch_bounds__(PULL_THREADS, 4) label_loop_kernel(UnwDev d, LoopCtl *c, LoopBufs bf)
{
    extern __shared__ __align__(16) unsigned char pull_smem[];
    const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
    // the loop state lives in registers; every block derives the same
    // transitions from the same post-barrier counters
    uint32_t phase = vload(&c->phase), b = vload(&c->b), iter = vload(&c->iter), L = vload(&c->lid) + 1;
    uint32_t levels = vload(&c->levels);
    for (;;) {
        if (phase == PH_BATCH || phase == PH_ROOT_RETRY) {
            if (b >= bf.nbatches) break;
            const uint32_t s = b * d.B;
            uint8_t *dm = bf.dm[b & 1];
            if (phase == PH_BATCH) {
                // rows of the previous batch go back to 255 (other parity)
                if (b > 0)
                    dm_rows_phase(d, bf.broots + bf.boff[b - 1], bf.boff[b] - bf.boff[b - 1], s - d.B, 0,
                                  nullptr, nullptr, bf.dm[(b - 1) & 1]);
                root_step_phase(d, bf.broots + bf.boff[b], bf.boff[b + 1] - bf.boff[b], s, b, L, dm, bf, c);
            } else {
                root_step_phase(d, bf.rr, vload(&c->rr_cnt), s, b, L, dm, bf, c);
            }
            if (leader) {
                c->tcnt[(L + 2) % 3] = 0;
                c->hcnt[(L + 2) % 3] = 0;
                c->tq[(L + 2) % 3] = 0;
                c->hq[(L + 2) % 3] = 0;
            }
            if (!grid_barrier(&c->bar, &c->status)) return;
            if (vload(&c->retry_cnt)) {
                if (leader) {
                    c->phase = PH_ROOT_RETRY;
                    c->b = b;
                    c->iter = 0;
                    c->lid = L - 1;
                    c->levels = levels;
                    c->exit_code = EX_NEED_POOL;
                }
                return;
            }
            const uint32_t nt = vload(&c->tcnt[(L + 1) % 3]) + vload(&c->hcnt[(L + 1) % 3]);
            if (nt == 0) {  // no tails: nothing can change in this batch
                if (leader && bf.batch_ns) bf.batch_ns[b] = gtimer();
                ++b;
                phase = PH_BATCH;
            } else {
                iter = 1;
                phase = PH_LEVEL;
            }
            ++L;
            continue;
        }
        // PH_LEVEL / PH_PULL_RETRY: level iter of batch b at stamp L
        if (iter >= U8_INF) {
            if (leader) {
                c->phase = PH_DONE;
                c->exit_code = EX_OVERFLOW;
            }
            return;
        }
        const uint32_t s = b * d.B;
        const uint32_t e = (uint32_t)min((uint64_t)s + d.B, (uint64_t)d.n);
        const int cur = L % 3, nx = (L + 1) % 3;
        PullArgs a{bf.tails[cur], &c->tcnt[cur], bf.htails[cur], &c->hcnt[cur], s, e, b, iter, L,
                   nullptr, nullptr, bf.retry, &c->retry_cnt};
        a.next_tails = bf.tails[nx];
        a.next_tails_cnt = &c->tcnt[nx];
        a.next_htails = bf.htails[nx];
        a.next_htails_cnt = &c->hcnt[nx];
        a.next_stamp = L + 1;
        a.dm = bf.dm[b & 1];
        a.tail_q = &c->tq[cur];
        a.htail_q = &c->hq[cur];
        pull_phase(d, a, pull_smem);
        if (leader && phase == PH_LEVEL) {
            c->tcnt[(L + 2) % 3] = 0;
            c->hcnt[(L + 2) % 3] = 0;
            c->tq[(L + 2) % 3] = 0;
            c->hq[(L + 2) % 3] = 0;
        }
        if (!grid_barrier(&c->bar, &c->status)) return;
        if (vload(&c->retry_cnt)) {
            if (leader) {
                c->phase = PH_PULL_RETRY;
                c->b = b;
                c->iter = iter;
                c->lid = L - 1;
                c->levels = levels;
                c->exit_code = EX_NEED_POOL;
            }
            return;
        }
        const uint32_t nt = vload(&c->tcnt[nx]) + vload(&c->hcnt[nx]);
        if (leader && bf.level_log && levels < bf.level_cap) {
            const unsigned long long tl = vload(&c->tcnt[cur]) + vload(&c->hcnt[cur]);
            bf.level_log[2ull * levels] = gtimer();
            bf.level_log[2ull * levels + 1] = (tl << 32) | b;
        }
        ++levels;
        if (nt == 0) {
            if (leader && bf.batch_ns) bf.batch_ns[b] = gtimer();
            ++b;
            phase = PH_BATCH;
        } else {
            ++iter;
            phase = PH_LEVEL;
        }
        ++L;
    }
    if (leader) {
        c->phase = PH_DONE;
        c->b = b;
        c->lid = L - 1;
        c->levels = levels;
        c->exit_code = EX_DONE;
    }
}

__global__ void __launch_bounds__(256) finalize_kernel(UnwDev d, const uint64_t *fin_off, uint32_t *fin_hub,
                                                       uint8_t *fin_dist)
{
    finalize_phase(d, fin_off, fin_hub, fin_dist, nullptr, nullptr);
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
    // destroyed after every buffer below: times their release
    std::optional<HostPhase> release_phase;
    std::optional<HostPhase> alloc_phase(std::in_place, "label alloc");

    DBuf<uint8_t> d_used(std::max<uint32_t>(n, 1));
    d_used.upload(used.data(), n, s);
    if (n) PADO_LAUNCH("heavy_flag_kernel", s, heavy_flag_kernel<<<grid_for(n, 256), 256, 0, s>>>(g.off.p, n, d_used.p));
    uint64_t cap = initial_pool_entries(n);
    DBuf<uint32_t> pool_hub(cap);
    DBuf<uint8_t> pool_dist(cap);
    DBuf<unsigned long long> pool_top(1);
    DBuf<uint64_t> lab_off(n);
    DBuf<LastGroup> last0(n), last1(n);
    DBuf<uint32_t> lab_len(n), lab_cap(n), last_min0(n), last_min1(n);
    DBuf<uint32_t> tail_stamp(n), ind_stamp(n);
    DBuf<uint32_t> ind((uint64_t)n * words);
    DBuf<uint8_t> dm((uint64_t)B * n);
    DBuf<uint32_t> front0(n), front1(n), tails(n), htails(n), retry(n), counters(8), status(1);
    DBuf<uint32_t> roots(B);
    pool_top.fill_bytes(0, s);
    lab_off.fill_bytes(0, s);
    lab_len.fill_bytes(0, s);
    lab_cap.fill_bytes(0, s);
    last0.fill_bytes(0, s);  // stamp 0: no group yet
    last1.fill_bytes(0, s);
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
    d.m = g.m;
#ifdef PADO_DEBUG_BOUNDS
    DBuf<uint32_t> dbg_word(1);
    dbg_word.fill_bytes(0, s);
    d.dbg = dbg_word.p;
#endif
    d.off = g.off.p;
    d.adj = g.adj.p;
    d.used = d_used.p;
    d.bpd = d_bpd;
    d.bps = d_bps;
    DBuf<uint8_t> bpmin(std::max<uint32_t>(n, 1));
    if (K && n)
        PADO_LAUNCH("bpmin_kernel", s, bpmin_kernel<<<grid_for(n, 256), 256, 0, s>>>(d_bpd, n, K, bpmin.p));
    d.bpmin = bpmin.p;
    d.pool_hub = pool_hub.p;
    d.pool_dist = pool_dist.p;
    d.pool_cap = cap;
    d.pool_top = pool_top.p;
    d.lab_off = lab_off.p;
    d.lab_len = lab_len.p;
    d.lab_cap = lab_cap.p;
    d.last[0] = last0.p;
    d.last[1] = last1.p;
    d.last_min[0] = last_min0.p;
    d.last_min[1] = last_min1.p;
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
    alloc_phase.reset();
    std::optional<HostPhase> loop_phase(std::in_place, "label loop");
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
            // every batch's roots (non-BP vertices), fixed before labeling starts
            std::vector<uint32_t> hb_roots, hb_off(nbatches + 1, 0);
            hb_roots.reserve(n);
            for (uint32_t b = 0; b < nbatches; ++b) {
                const uint32_t lo = b * B, hi = (uint32_t)std::min<uint64_t>((uint64_t)lo + B, n);
                for (uint32_t r = lo; r < hi; ++r)
                    if (!used[r]) hb_roots.push_back(r);
                hb_off[b + 1] = (uint32_t)hb_roots.size();
            }
            DBuf<uint32_t> d_broots(std::max<size_t>(hb_roots.size(), 1)), d_boff(nbatches + 1);
            d_broots.upload(hb_roots.data(), hb_roots.size(), s);
            d_boff.upload(hb_off.data(), nbatches + 1, s);
            DBuf<uint8_t> dm2((uint64_t)B * n);  // second dist_matrix buffer (odd batches)
            dm2.fill_bytes(0xff, s);
            DBuf<uint32_t> tails2(n), htails3(n);
            DBuf<LoopCtl> ctl(1);
            DBuf<uint32_t> rr(B);
            DBuf<unsigned long long> bns(trace ? nbatches : 1);
            const uint32_t level_cap = trace ? (1u << 22) : 0u;
            DBuf<unsigned long long> llog(trace ? 2ull * level_cap : 1);
            ctl.fill_bytes(0, s);
            if (trace) bns.fill_bytes(0, s);
            // tail slots: the three light lists reuse the host loop's front and tail buffers
            LoopBufs bf{d_broots.p, d_boff.p, rr.p, {tails.p, front0.p, tails2.p}, {htails.p, front1.p, htails3.p},
                        retry.p, {dm.p, dm2.p}, trace ? bns.p : nullptr, trace ? llog.p : nullptr, level_cap,
                        nbatches};
            const void *kfn = (const void *)label_loop_kernel;
            PADO_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int dev = 0, sms = 0, per_sm = 0;
            PADO_CUDA(cudaGetDevice(&dev));
            PADO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            PADO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, PULL_THREADS, smem));
            PADO_CHECK(per_sm >= 1, PADO_E_CUDA, "labeling loop kernel cannot be resident");
            const unsigned grid = (unsigned)(sms * std::min(per_sm, 4));  // compiled for 4 blocks/SM
            PADO_CHECK(grid <= BAR_GROUP * BAR_MAX_GROUPS, PADO_E_CUDA, "grid larger than the barrier supports");
            LoopCtl h{};
            LoopCtl *cp_ = ctl.p;
            for (int launch = 0;; ++launch) {
                PADO_CHECK(launch < 256, PADO_E_NOMEM, "label pool could not be grown enough");
                void *args[] = {&d, &cp_, &bf};
                PADO_LAUNCH("label_loop_kernel", s,
                            PADO_CUDA(cudaLaunchCooperativeKernel(kfn, grid, PULL_THREADS, args,
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
                    // the failed tails become the whole light list of the step (any degree is fine there)
                    const int cur = (h.lid + 1) % 3;
                    uint32_t *lists[3] = {tails.p, front0.p, tails2.p};
                    PADO_CUDA(cudaMemcpyAsync(lists[cur], retry.p, h.retry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                    h.tcnt[cur] = h.retry_cnt;
                    h.hcnt[cur] = 0;
                }
                for (int x = 0; x < 3; ++x) h.tq[x] = h.hq[x] = 0;  // the re-run level claims from zero
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
                // time per level, bucketed by the level's tail count
                const uint32_t nl = std::min(h.levels, level_cap);
                std::vector<unsigned long long> lg(2ull * nl);
                llog.download(lg.data(), lg.size(), s);
                PADO_CUDA(cudaStreamSynchronize(s));
                const uint64_t edges[] = {0, 64, 512, 4096, 32768, 262144, ~0ull};
                double ms[6] = {}, tl[6] = {};
                uint64_t cnt[6] = {};
                for (uint32_t i = 1; i < nl; ++i) {
                    const uint64_t nt = lg[2 * i + 1] >> 32;
                    int k = 0;
                    while (nt >= edges[k + 1]) ++k;
                    ms[k] += (lg[2 * i] - lg[2 * i - 2]) * 1e-6;
                    tl[k] += (double)nt;
                    ++cnt[k];
                }
                for (int k = 0; k < 6; ++k)
                    fprintf(stderr, "levels with tails in [%llu, %llu): %llu levels, %.3f ms, %.0f tails\n",
                            (unsigned long long)edges[k], (unsigned long long)edges[k + 1], (unsigned long long)cnt[k],
                            ms[k], tl[k]);
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
            nvtxRangePushA("batch");
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
                nvtxRangePushA("level");
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
                nvtxRangePop();
            }
            PADO_LAUNCH("dm_rows_kernel(reset)", s,
                        dm_rows_kernel<<<grid_for((uint64_t)nr * 32, 256), 256, 0, s>>>(d, roots.p, nr, bs, 0));
            if (trace) {
                TraceRow tr{b, b_levels, b_tails, b_front, nullptr};
                PADO_CUDA(cudaEventCreate(&tr.ev));
                PADO_CUDA(cudaEventRecord(tr.ev, s));
                trace_rows.push_back(tr);
            }
            nvtxRangePop();
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
        loop_phase.reset();
        HostPhase fin_phase("label finalize");
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
#ifdef PADO_DEBUG_BOUNDS
        {
            uint32_t w = 0;
            dbg_word.download(&w, 1, s);
            PADO_CUDA(cudaStreamSynchronize(s));
            if (w) {
                char msg[96];
                snprintf(msg, sizeof(msg), "device bounds check failed (sites mask 0x%x)", w);
                throw Error(PADO_E_STATE, msg);
            }
        }
#endif
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
    release_phase.emplace("label release");
    return run;
}

}  // namespace pado
