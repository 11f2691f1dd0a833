// unw_many.cu -- batched pruned-BFS labeling of many independent graphs at once.
//
// Labeling a small graph alone leaves the GPU idle: a batch of a 5,000-vertex
// graph touches a few thousand vertices per level, and every level still pays
// a grid barrier (or a kernel launch and a host round trip).  Here the graphs
// are laid side by side in one union id space -- graph g owns the ids
// [base_g, base_g + n_g) of a disjoint-union CSR -- and ONE persistent
// cooperative launch advances every graph by one BFS level per step:
//
//   step L (stamp L):
//     A. reset the dist_matrix rows of graphs that finished a batch at step
//        L-1; self-label the roots of graphs that start a batch (stamp L);
//        mark the tails of every vertex that gained labels at step L-1.
//     B. fill the dist_matrix rows of the new batches' roots; pull (the same
//        warp-per-tail / block-per-heavy-tail code as the one-graph labeler)
//        with each tail reading its own graph's batch, level and rows.
//     C. per graph: a graph whose level produced no labels ends its batch and
//        queues the next batch's roots; the others go one level deeper.
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

enum ManyPhase : uint32_t { MP_STEP = 0, MP_A_RETRY = 1, MP_B_RETRY = 2, MP_DONE = 3 };
enum ManyExit : uint32_t { MX_RUNNING = 0, MX_DONE = 1, MX_NEED_POOL = 2, MX_OVERFLOW = 3 };

struct ManyCtl {
    GridBar bar;
    uint32_t phase, lid, active, steps;
    uint32_t front_cnt[2], tails_cnt[2], htails_cnt[2];
    uint32_t rq_cnt[2];   // roots to self-label in step L: rq[L & 1]
    uint32_t zq_cnt[2];   // roots whose dist_matrix rows are reset in step L
    uint32_t rr_cnt, retry_cnt, status, exit_code;
};

struct ManyBufs {
    GDesc *gd;
    const uint16_t *gmap;      // union id -> graph
    const uint32_t *broots;    // every batch's roots, graph by graph, batch by batch
    const uint32_t *bcnt;      // roots per batch (graph g's batch b at gd[g].bfirst + b)
    uint32_t G;
    uint32_t *rq[2], *zq[2], *rr;
    uint32_t *front[2];
    uint32_t *tails, *htails, *retry;
};

// Step bookkeeping, a warp per graph (see the file comment, part C).
__device__ void many_bookkeep(const UnwDev &d, ManyCtl *c, const ManyBufs &bf, uint32_t L)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const int cp = L & 1, np = (L + 1) & 1;
    for (uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < bf.G; g += nw) {
        GDesc &x = bf.gd[g];
        // every lane reads the descriptor before lane 0 rewrites it
        const uint32_t st = vload(&x.state);
        if (st == GS_DONE) continue;
        const uint32_t fc = vload(&x.fcnt[cp]);
        const uint32_t xb = vload(&x.b), xnr = vload(&x.nr), xroff = vload(&x.roff), xiter = vload(&x.iter);
        const uint32_t xnb = x.nb, xbf = x.bfirst, xbase = x.base, xn = x.n;
        __syncwarp();
        if (st == GS_START) {
            if (lane == 0) {
                x.state = GS_LEVEL;
                x.iter = 1;
            }
        } else if (fc != 0) {
            if (lane == 0) {
                if (xiter + 1 >= U8_INF) atomicOr(&c->status, ST_LEVEL_OVERFLOW);
                x.iter = xiter + 1;
            }
        } else {
            // batch done: its rows are reset at the next step
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
                    x.b = b;
                    x.s = xbase + b * d.B;
                    x.e = min(x.s + d.B, xbase + xn);
                    x.roff = roff;
                    x.nr = nr;
                    x.iter = 0;
                    x.state = GS_START;
                }
            } else if (lane == 0) {
                x.state = GS_DONE;
                atomicSub(&c->active, 1u);
            }
        }
        if (lane == 0) x.fcnt[np] = 0;  // counted during step L+1
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
        const int cp = L & 1, pp = (L - 1) & 1;
        PullArgs a{bf.tails, &c->tails_cnt[cp], bf.htails, &c->htails_cnt[cp], 0u, 0u, 0u, 0u, L,
                   bf.front[cp], &c->front_cnt[cp], bf.retry, &c->retry_cnt, bf.gd, bf.gmap, bf.gd};
        if (phase == MP_STEP || phase == MP_A_RETRY) {
            if (phase == MP_STEP) {
                dm_rows_phase(d, bf.zq[cp], vload(&c->zq_cnt[cp]), 0u, 0, bf.gd, bf.gmap);
                root_init_phase(d, bf.rq[cp], vload(&c->rq_cnt[cp]), 0u, 0u, L, bf.front[cp], &c->front_cnt[cp],
                                bf.retry, &c->retry_cnt, bf.gd, bf.gmap);
                mark_phase(d, bf.front[pp], vload(&c->front_cnt[pp]), L, bf.tails, &c->tails_cnt[cp], bf.htails,
                           &c->htails_cnt[cp]);
            } else {
                root_init_phase(d, bf.rr, vload(&c->rr_cnt), 0u, 0u, L, bf.front[cp], &c->front_cnt[cp], bf.retry,
                                &c->retry_cnt, bf.gd, bf.gmap);
            }
            if (!grid_barrier(&c->bar, &c->status)) return;
            if (vload(&c->retry_cnt)) {
                if (leader) {
                    c->phase = MP_A_RETRY;
                    c->exit_code = MX_NEED_POOL;
                }
                return;
            }
            dm_rows_phase(d, bf.rq[cp], vload(&c->rq_cnt[cp]), 0u, 1, bf.gd, bf.gmap);
        }
        pull_phase(d, a, pull_smem);
        if (!grid_barrier(&c->bar, &c->status)) return;
        if (vload(&c->retry_cnt)) {
            if (leader) {
                c->phase = MP_B_RETRY;
                c->exit_code = MX_NEED_POOL;
            }
            return;
        }
        many_bookkeep(d, c, bf, L);
        if (leader) {
            const int np = (L + 1) & 1;
            c->lid = L;
            c->steps += 1;
            c->front_cnt[np] = 0;
            c->tails_cnt[np] = 0;
            c->htails_cnt[np] = 0;
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
        x.dm_off = (uint64_t)B * base;
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
    uint64_t cap = initial_pool_entries(n);
    DBuf<uint32_t> pool_hub(cap);
    DBuf<uint8_t> pool_dist(cap);
    DBuf<unsigned long long> pool_top(1);
    DBuf<uint64_t> lab_off(n), last_pos0(n), last_pos1(n);
    DBuf<uint32_t> lab_len(n), lab_cap(n), last_cnt0(n), last_cnt1(n), last_min0(n), last_min1(n);
    DBuf<uint32_t> act_stamp0(n), act_stamp1(n), tail_stamp(n), ind_stamp(n);
    DBuf<uint32_t> ind((uint64_t)n * words);
    DBuf<uint8_t> dm((uint64_t)B * n);
    DBuf<uint32_t> front0(n), front1(n), tails(n), htails(n), retry(n), status(1);
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
    act_stamp0.fill_bytes(0, s);
    act_stamp1.fill_bytes(0, s);
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

    ManyBufs bf{d_gd.p, d_gmap.p, d_broots.p, d_bcnt.p, G, {rq0b.p, rq1b.p}, {zq0b.p, zq1b.p}, rr.p,
                {front0.p, front1.p}, tails.p, htails.p, retry.p};

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
                if (h.phase == MP_A_RETRY) {
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
