// unw_many.cu -- batched pruned-BFS labeling of many independent graphs at once.
//
// Labeling a small graph alone leaves the GPU idle: a batch of a 5,000-vertex
// graph touches a few thousand vertices per level, and every level still pays
// a grid barrier (or a kernel launch and a host round trip).  Here the graphs
// are laid side by side in one union id space -- graph g owns the ids
// [base_g, base_g + n_g) of a disjoint-union CSR -- and ONE persistent
// cooperative launch advances every graph by one BFS level per step:
//
//   step L (stamp L), one pass then a grid barrier:
//     A. reset the dist_matrix rows of batches that ended at step L-1; give the
//        roots of graphs that start a batch their self labels (stamp L), fill
//        their dist_matrix rows and mark their tails for L+1; pull (the same
//        warp-per-tail / block-per-heavy-tail code as the one-graph labeler,
//        each tail reading its own graph's batch, level and rows), every tail
//        that gains labels marking its tails for L+1 at once.  Each graph has
//        two dist_matrix buffers used by alternate batches, so the reset of
//        the old batch and the fill of the new one never share a row.
//     C. (after the barrier) a warp per graph: a graph with no tails for L+1
//        ends its batch -- its next level would add nothing -- and queues the
//        next batch's roots; the others go one level deeper.  A second barrier
//        publishes the new per-graph state.
//
// Each graph runs exactly the reference's batch sequence (batches of B
// consecutive ranks of that graph, pado_unw_unv_unp.h:1080-1118) and, within
// a batch, exactly its levels, so every graph's labels are those of labeling it
// alone.  Graphs never share a vertex, so their work within a step is
// independent: label stamps and tail stamps use the global step number, while
// indicator stamps, batch starts and levels are per graph.  The number of
// steps is the largest per-graph sum of (levels + 1) over its batches, instead
// of the sum over all graphs.
//
// Pool growth works as in the one-graph loop: a warp that cannot reserve label
// space commits nothing, the launch returns, the host grows the pool and
// relaunches at the failed part of the step.

#include <algorithm>
#include <cstring>
#include <numeric>

#include "unw_device.cuh"

namespace pado {
namespace {

enum ManyPhase : uint32_t { MP_STEP = 0, MP_RETRY = 1, MP_DONE = 2 };
enum ManyExit : uint32_t { MX_RUNNING = 0, MX_DONE = 1, MX_NEED_POOL = 2, MX_OVERFLOW = 3 };

struct ManyCtl {
    GridBar bar;
    uint32_t phase, lid, active, steps;
    uint32_t tcnt[3], hcnt[3];  // light / heavy tails marked for stamp x, in slot x % 3
    uint32_t tq[3], hq[3];      // work counters of the step at stamp x (dynamic assignment)
    uint32_t rq_cnt[2];         // roots to start in step L: rq[L & 1]
    uint32_t zq_cnt[2];         // roots whose dist_matrix rows are reset in step L
    uint32_t rr_cnt, rretry_cnt, tretry_cnt, status, exit_code, pad;
};

struct ManyBufs {
    GDesc *gd;
    const uint16_t *gmap;      // union id -> graph
    const uint32_t *broots;    // every batch's roots, graph by graph, batch by batch
    const uint32_t *bcnt;      // roots per batch (graph g's batch b at gd[g].bfirst + b)
    uint32_t G;
    uint32_t *rq[2], *zq[2], *rr;
    uint32_t *tails[3], *htails[3];
    uint32_t *rretry, *tretry;
};

// Batch start for roots[0, nr) of graphs in GS_START: self label at stamp L,
// the dist_matrix row of the root in its graph's current buffer, tails for L+1.
__device__ void many_root_step(const UnwDev &d, const ManyBufs &bf, ManyCtl *c, const uint32_t *roots, uint32_t nr,
                               uint32_t L)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int p = L & 1, nx = (L + 1) % 3;
    unsigned long long bytes = 0;
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < nr; q += nw) {
        const uint32_t r = roots[q];
        const uint32_t g = bf.gmap[r];
        const GDesc &x = bf.gd[g];
        const uint32_t gs = gd_u32(x.s), gb = gd_u32(x.b), gbase = x.base, gn = x.n;
        uint8_t *dm = d.dm + x.dm_off + (uint64_t)gd_u32(x.dmp) * d.B * gn;
        uint64_t base;
        if (!warp_reserve(d, r, UD_AT(d.lab_len, r, d.n, 1) + 1, base, lane)) {
            if (lane == 0) {
                atomicOr(d.status, ST_POOL_RETRY);
                bf.rretry[atomicAdd(&c->rretry_cnt, 1u)] = r;
            }
            continue;
        }
        const uint32_t len = UD_AT(d.lab_len, r, d.n, 1);
        const uint32_t idx = r - gs;
        for (uint32_t w = lane; w < d.words; w += 32)
            UD_AT(d.ind, (uint64_t)r * d.words + w, (uint64_t)d.n * d.words, 5) = (w == (idx >> 5)) ? (1u << (idx & 31)) : 0u;
        if (lane == 0) {
            if (d.work) atomicAdd(&d.work[W_EV_LABELS], 1ull);
            UD_AT(d.pool_hub, base + len, d.pool_cap, 2) = r;
            UD_AT(d.pool_dist, base + len, d.pool_cap, 2) = 0;
            UD_AT(d.lab_len, r, d.n, 1) = len + 1;
            UD_AT(d.last[p], r, d.n, 1) = LastGroup{base + len, 1u, L};
            UD_AT(d.last_min[p], r, d.n, 1) = r;
            UD_AT(d.ind_stamp, r, d.n, 1) = gb + 1;
        }
        __syncwarp();
        uint8_t *row = dm + (uint64_t)idx * gn;
        for (uint32_t j = lane; j <= len; j += 32)
            UD_AT(row, UD_AT(d.pool_hub, base + j, d.pool_cap, 2) - gbase, gn, 4) = UD_AT(d.pool_dist, base + j, d.pool_cap, 2);
        mark_tails(d, r, r, L + 1, bf.tails[nx], &c->tcnt[nx], bf.htails[nx], &c->hcnt[nx], lane, 0, 1, bytes,
                   &bf.gd[g].tc[nx]);
    }
    if (d.work && lane == 0 && bytes) atomicAdd(&d.work[W_MARK], bytes);
}

// Step bookkeeping, a warp per graph (see the file comment, part C).
__device__ void many_bookkeep(const UnwDev &d, ManyCtl *c, const ManyBufs &bf, uint32_t L)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int nx = (L + 1) % 3, nn = (L + 2) % 3, np = (L + 1) & 1;
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < bf.G; g += nw) {
        GDesc &x = bf.gd[g];
        // every lane reads the descriptor before lane 0 rewrites it
        const uint32_t st = vload(&x.state);
        if (st == GS_DONE) continue;
        const uint32_t nt = vload(&x.tc[nx]);
        const uint32_t xb = vload(&x.b), xnr = vload(&x.nr), xroff = vload(&x.roff), xiter = vload(&x.iter);
        const uint32_t xdmp = vload(&x.dmp);
        const uint32_t xnb = x.nb, xbf = x.bfirst, xbase = x.base, xn = x.n;
        __syncwarp();
        if (nt != 0) {
            if (lane == 0) {
                const uint32_t it = st == GS_START ? 1u : xiter + 1;
                if (it >= U8_INF) atomicOr(&c->status, ST_LEVEL_OVERFLOW);
                x.iter = it;
                x.state = GS_LEVEL;
            }
        } else {
            // batch over: its rows are reset at the next step
            uint32_t pos = 0;
            if (lane == 0) pos = atomicAdd(&c->zq_cnt[np], xnr);
            pos = __shfl_sync(FULL, pos, 0);
            for (uint32_t j = lane; j < xnr; j += 32) bf.zq[np][pos + j] = bf.broots[xroff + j];
            uint32_t b = xb + 1;
            const uint32_t roff = xroff + xnr;
            while (b < xnb && bf.bcnt[xbf + b] == 0) ++b;
            if (b < xnb) {
                const uint32_t nr = bf.bcnt[xbf + b];
                if (lane == 0) pos = atomicAdd(&c->rq_cnt[np], nr);
                pos = __shfl_sync(FULL, pos, 0);
                for (uint32_t j = lane; j < nr; j += 32) bf.rq[np][pos + j] = bf.broots[roff + j];
                if (lane == 0) {
                    x.zqp = xdmp;
                    x.dmp = xdmp ^ 1u;
                    x.b = b;
                    x.s = xbase + b * d.B;
                    x.e = min(x.s + d.B, xbase + xn);
                    x.roff = roff;
                    x.nr = nr;
                    x.iter = 0;
                    x.state = GS_START;
                }
            } else if (lane == 0) {
                x.zqp = xdmp;
                x.state = GS_DONE;
                atomicSub(&c->active, 1u);
            }
        }
        if (lane == 0) x.tc[nn] = 0;  // counted during step L+1
        __syncwarp();
    }
}

__global__ void __launch_bounds__(PULL_THREADS, 4) many_loop_kernel(UnwDev d, ManyCtl *c, ManyBufs bf)
{
    extern __shared__ __align__(16) unsigned char pull_smem[];
    const bool leader = blockIdx.x == 0 && threadIdx.x == 0;
    for (;;) {
        const uint32_t phase = vload(&c->phase);
        if (phase == MP_DONE) return;
        if (vload(&c->active) == 0) {
            if (leader) {
                c->phase = MP_DONE;
                c->exit_code = MX_DONE;
            }
            return;
        }
        const uint32_t L = vload(&c->lid) + 1;
        const int cur = L % 3, nx = (L + 1) % 3, cp = L & 1;
        PullArgs a{bf.tails[cur], &c->tcnt[cur], bf.htails[cur], &c->hcnt[cur], 0u, 0u, 0u, 0u, L,
                   nullptr, nullptr, bf.tretry, &c->tretry_cnt, bf.gd, bf.gmap, bf.gd};
        a.next_tails = bf.tails[nx];
        a.next_tails_cnt = &c->tcnt[nx];
        a.next_htails = bf.htails[nx];
        a.next_htails_cnt = &c->hcnt[nx];
        a.next_stamp = L + 1;
        a.tail_q = &c->tq[cur];
        a.htail_q = &c->hq[cur];
        if (phase == MP_STEP) {
            dm_rows_phase(d, bf.zq[cp], vload(&c->zq_cnt[cp]), 0u, 0, bf.gd, bf.gmap);
            many_root_step(d, bf, c, bf.rq[cp], vload(&c->rq_cnt[cp]), L);
        } else {
            many_root_step(d, bf, c, bf.rr, vload(&c->rr_cnt), L);
        }
        pull_phase(d, a, pull_smem);
        if (leader) {
            c->tcnt[(L + 2) % 3] = 0;
            c->hcnt[(L + 2) % 3] = 0;
            c->tq[(L + 2) % 3] = 0;
            c->hq[(L + 2) % 3] = 0;
        }
        if (!grid_barrier(&c->bar, &c->status)) return;
        if (vload(&c->rretry_cnt) || vload(&c->tretry_cnt)) {
            if (leader) {
                c->phase = MP_RETRY;
                c->exit_code = MX_NEED_POOL;
            }
            return;
        }
        many_bookkeep(d, c, bf, L);
        if (leader) {
            c->lid = L;
            c->steps += 1;
            c->rq_cnt[cp] = 0;
            c->zq_cnt[cp] = 0;
            c->phase = MP_STEP;
        }
        if (!grid_barrier(&c->bar, &c->status)) return;
        if (vload(&c->status) & ST_LEVEL_OVERFLOW) {
            if (leader) {
                c->phase = MP_DONE;
                c->exit_code = MX_OVERFLOW;
            }
            return;
        }
    }
}

__global__ void __launch_bounds__(256) many_finalize_kernel(UnwDev d, const uint64_t *fin_off, uint32_t *fin_hub,
                                                            uint8_t *fin_dist, const uint16_t *gmap,
                                                            const uint32_t *gbase)
{
    finalize_phase(d, fin_off, fin_hub, fin_dist, gmap, gbase);
}

}  // namespace

LabelRun unw_label_many(const DevGraph &g, const std::vector<uint32_t> &gbase, uint32_t K, uint32_t B,
                        const std::vector<uint8_t> &used, const uint8_t *d_bpd, const uint64_t *d_bps,
                        LabelStore &out, cudaStream_t s)
{
    LabelRun run;
    const uint32_t n = g.n;
    const uint32_t G = (uint32_t)gbase.size() - 1;
    const uint32_t words = (B + 31) / 32;
    PADO_CHECK(B >= 1 && B <= MAX_BATCH, PADO_E_ARG, "batch size must be in [1, 2048]");
    PADO_CHECK(K <= MAX_BP, PADO_E_ARG, "at most 64 bit-parallel roots");
    PADO_CHECK(G >= 1 && G <= 65535, PADO_E_ARG, "between 1 and 65535 graphs");
    PADO_CHECK(gbase[0] == 0 && gbase[G] == n, PADO_E_ARG, "graph ranges must tile the union");

    // Per-graph batches and their roots (non-BP vertices of each batch).
    std::vector<GDesc> hgd(G);
    std::vector<uint16_t> hgmap(n);
    std::vector<uint32_t> broots, bcnt, rq0;
    broots.reserve(n);
    uint32_t active = 0;
    for (uint32_t gi = 0; gi < G; ++gi) {
        const uint32_t base = gbase[gi], ng = gbase[gi + 1] - gbase[gi];
        PADO_CHECK(gbase[gi + 1] >= gbase[gi], PADO_E_ARG, "graph ranges must be non-decreasing");
        GDesc &x = hgd[gi];
        x = GDesc{};
        x.base = base;
        x.n = ng;
        x.nb = (uint32_t)(((uint64_t)ng + B - 1) / B);
        x.bfirst = (uint32_t)bcnt.size();
        x.dm_off = 2ull * B * base;
        x.state = GS_DONE;
        const uint32_t first_root = (uint32_t)broots.size();
        for (uint32_t v = base; v < base + ng; ++v) hgmap[v] = (uint16_t)gi;
        for (uint32_t b = 0; b < x.nb; ++b) {
            const uint32_t lo = base + b * B, hi = std::min(base + ng, lo + B);
            uint32_t c = 0;
            for (uint32_t r = lo; r < hi; ++r)
                if (!used[r]) {
                    broots.push_back(r);
                    ++c;
                }
            bcnt.push_back(c);
        }
        // first batch that has roots
        uint32_t b = 0;
        while (b < x.nb && bcnt[x.bfirst + b] == 0) ++b;
        if (b < x.nb) {
            x.b = b;
            x.s = base + b * B;
            x.e = std::min(x.s + B, base + ng);
            x.roff = first_root;
            x.nr = bcnt[x.bfirst + b];
            x.state = GS_START;
            rq0.insert(rq0.end(), broots.begin() + x.roff, broots.begin() + x.roff + x.nr);
            ++active;
        }
        run.batches += x.nb;
    }

    DBuf<uint8_t> d_used(std::max<uint32_t>(n, 1));
    d_used.upload(used.data(), n, s);
    if (n) PADO_LAUNCH("heavy_flag_kernel", s, heavy_flag_kernel<<<grid_for(n, 256), 256, 0, s>>>(g.off.p, n, d_used.p));
    // Many small graphs carry more labels per vertex than one large sparse
    // one, and every growth stops the loop: start at 3x the one-graph pool.
    uint64_t cap = debug_pool_entries() ? initial_pool_entries(n)
                                        : std::min<uint64_t>(3 * initial_pool_entries(n), 1ull << 31);
    DBuf<uint32_t> pool_hub(cap);
    DBuf<uint8_t> pool_dist(cap);
    DBuf<unsigned long long> pool_top(1);
    DBuf<uint64_t> lab_off(n);
    DBuf<LastGroup> last0(n), last1(n);
    DBuf<uint32_t> lab_len(n), lab_cap(n), last_min0(n), last_min1(n);
    DBuf<uint32_t> tail_stamp(n), ind_stamp(n);
    DBuf<uint32_t> ind((uint64_t)n * words);
    DBuf<uint8_t> dm(2ull * B * n);  // two buffers per graph, by batch
    DBuf<uint32_t> tl0(n), tl1(n), tl2(n), th0(n), th1(n), th2(n), rretry(n), tretry(n), status(1);
    DBuf<uint32_t> rq0b(n), rq1b(n), zq0b(n), zq1b(n), rr(n);
    DBuf<GDesc> d_gd(G);
    DBuf<uint16_t> d_gmap(std::max<uint32_t>(n, 1));
    DBuf<uint32_t> d_broots(std::max<size_t>(broots.size(), 1)), d_bcnt(std::max<size_t>(bcnt.size(), 1));
    DBuf<uint32_t> d_gbase(G + 1);
    DBuf<ManyCtl> ctl(1);
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
    d_gd.upload(hgd.data(), G, s);
    d_gmap.upload(hgmap.data(), n, s);
    d_broots.upload(broots.data(), broots.size(), s);
    d_bcnt.upload(bcnt.data(), bcnt.size(), s);
    d_gbase.upload(gbase.data(), G + 1, s);
    // step 1 self-labels the first batches' roots: rq[1]
    rq1b.upload(rq0.data(), rq0.size(), s);
    ManyCtl h{};
    h.phase = MP_STEP;
    h.active = active;
    h.rq_cnt[1] = (uint32_t)rq0.size();
    ctl.upload(&h, 1, s);

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

    ManyBufs bf{d_gd.p,           d_gmap.p,           d_broots.p, d_bcnt.p, G, {rq0b.p, rq1b.p}, {zq0b.p, zq1b.p},
                rr.p,             {tl0.p, tl1.p, tl2.p}, {th0.p, th1.p, th2.p}, rretry.p, tretry.p};

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

    const uint32_t smem = pull_smem_bytes(words, B);
    cudaEvent_t e0, e1;
    PADO_CUDA(cudaEventCreate(&e0));
    PADO_CUDA(cudaEventCreate(&e1));
    PADO_CUDA(cudaEventRecord(e0, s));
    try {
        if (active) {
            const void *kfn = (const void *)many_loop_kernel;
            PADO_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            int dev = 0, sms = 0, per_sm = 0;
            PADO_CUDA(cudaGetDevice(&dev));
            PADO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            PADO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, PULL_THREADS, smem));
            PADO_CHECK(per_sm >= 1, PADO_E_CUDA, "many-graph labeling kernel cannot be resident");
            const unsigned grid = (unsigned)(sms * std::min(per_sm, 4));  // compiled for 4 blocks/SM
            ManyCtl *cptr = ctl.p;
            for (int launch = 0;; ++launch) {
                PADO_CHECK(launch < 256, PADO_E_NOMEM, "label pool could not be grown enough");
                void *args[] = {&d, &cptr, &bf};
                PADO_LAUNCH("many_loop_kernel", s,
                            PADO_CUDA(cudaLaunchCooperativeKernel(kfn, grid, PULL_THREADS, args,
                                                                  smem, s)));
                PADO_CUDA(cudaMemcpyAsync(&h, ctl.p, sizeof(ManyCtl), cudaMemcpyDeviceToHost, s));
                PADO_CUDA(cudaStreamSynchronize(s));
                if (h.status & ST_BARRIER_TIMEOUT)
                    throw Error(PADO_E_TIMEOUT, "many-graph labeling loop: a grid barrier timed out");
                if (h.exit_code == MX_DONE) break;
                if (h.exit_code == MX_OVERFLOW)
                    throw Error(PADO_E_OVERFLOW, "BFS level reached 255 (uint8 distance overflow)");
                PADO_CHECK(h.exit_code == MX_NEED_POOL, PADO_E_STATE, "many-graph labeling loop stopped unexpectedly");
                unsigned long long top = 0;
                PADO_CUDA(cudaMemcpy(&top, pool_top.p, 8, cudaMemcpyDeviceToHost));
                grow_pool(top);
                // failed roots run again from rr; failed tails become the whole light
                // list of the step (any degree is fine there)
                PADO_CUDA(cudaMemcpyAsync(rr.p, rretry.p, h.rretry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                h.rr_cnt = h.rretry_cnt;
                const int cur = (h.lid + 1) % 3;
                uint32_t *lists[3] = {tl0.p, tl1.p, tl2.p};
                PADO_CUDA(cudaMemcpyAsync(lists[cur], tretry.p, h.tretry_cnt * 4ull, cudaMemcpyDeviceToDevice, s));
                h.tcnt[cur] = h.tretry_cnt;
                h.hcnt[cur] = 0;
                for (int x = 0; x < 3; ++x) h.tq[x] = h.hq[x] = 0;  // the re-run step claims from zero
                h.rretry_cnt = 0;
                h.tretry_cnt = 0;
                h.status = 0;
                h.exit_code = MX_RUNNING;
                PADO_CUDA(cudaMemcpyAsync(ctl.p, &h, sizeof(ManyCtl), cudaMemcpyHostToDevice, s));
            }
            run.levels = h.steps;
        }
        // finalize: exact-size canonical store, graph-local hubs
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
            PADO_LAUNCH("many_finalize_kernel", s,
                        many_finalize_kernel<<<grid_for((uint64_t)n * 32, 256), 256, 0, s>>>(
                            d, out.off.p, out.hub.p, out.dist8.p, d_gmap.p, d_gbase.p));
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
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return run;
}

}  // namespace pado
