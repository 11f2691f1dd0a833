// serve.cu -- the serving loop: label sets resident in HBM, query requests of
// any size coalesced into mixed batches, label sets admitted and evicted by an
// HBM budget.
//
// The reference answers one pair per call on the host (query_distance,
// pado_unw_unv_unp.h:1312-1445; query_distance.cpp:25-78 reads pairs from
// stdin).  A GPU answers millions of pairs per launch, but a request of a few
// pairs launched alone costs a host round trip and a launch that occupies a
// handful of warps.  The loop here is continuous batching:
//
//   * callers submit requests (index id, k pairs, result buffer) from any
//     thread; a request is queued and its pointers are used until it
//     completes;
//   * one dispatcher thread owns the GPU side.  It keeps up to `slots`
//     batches in flight, each on its own stream with its own page-locked
//     staging and device buffers.  Whenever a slot is free it drains the queue
//     into a batch -- whatever has arrived, up to max_pairs pairs, splitting a
//     request across batches when it does not fit -- copies the pairs,
//     launches ONE kernel for the whole batch (a warp per pair; each pair finds
//     its request's run of pairs, and through it its index, by a binary search
//     over the batch's run table) and queues the copy back.  Requests that
//     arrive while batches are on the GPU go into the next free slot, so
//     transfers and kernels of consecutive batches overlap;
//   * when an event says a batch is done, its results are copied into the
//     callers' buffers and requests whose last pairs were in it complete;
//   * a request for an index whose label set is not in HBM is admitted first:
//     least-recently-used label sets that no in-flight batch uses are
//     offloaded to page-locked host memory until the resident bytes fit the
//     budget (and free HBM holds the set), then the set is copied back.
//
// Each pair is answered by the same per-pair code as pado_query, against the
// same arrays, so a request's results are identical alone and in any mix.

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "query_device.cuh"

namespace pado {
namespace {

// A run of consecutive pairs of one batch that belong to one request chunk.
struct ServeRun {
    uint64_t start;     // first pair of the run within the batch
    uint64_t out_off;   // byte offset of its first result in the batch output
    IndexView v;
    uint32_t weighted;
    uint32_t pad;
};

__global__ void __launch_bounds__(256) serve_query_kernel(const ServeRun *__restrict__ runs, uint32_t nrun, uint64_t k,
                                                          const uint32_t *__restrict__ qa,
                                                          const uint32_t *__restrict__ qb,
                                                          unsigned char *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long bytes = 0;
    uint32_t r = 0;
    for (uint64_t p = warp; p < k; p += nwarps) {
        // run of pair p: last run with start <= p (runs are sorted by start)
        if (!(p >= runs[r].start && (r + 1 == nrun || p < runs[r + 1].start))) {
            uint32_t lo = 0, hi = nrun - 1;
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (runs[mid].start <= p) lo = mid; else hi = mid - 1;
            }
            r = lo;
        }
        const ServeRun &run = runs[r];
        const uint64_t i = p - run.start;
        if (run.weighted) {
            const int16_t d = query_w_pair(run.v, qa[p], qb[p], lane, bytes);
            if (lane == 0) reinterpret_cast<int16_t *>(out + run.out_off)[i] = d;
        } else {
            const uint8_t d = query_unw_pair(run.v, qa[p], qb[p], lane, bytes);
            if (lane == 0) out[run.out_off + i] = d;
        }
    }
    unsigned long long *w = runs[0].v.work;
    if (w && lane == 0 && bytes) atomicAdd(&w[W_Q_UNW], bytes);
}

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Req {
    uint32_t index = 0;
    uint64_t k = 0;
    const uint32_t *a = nullptr, *b = nullptr;
    void *out = nullptr;
    uint64_t next = 0;          // pairs placed in batches so far (dispatcher only)
    uint32_t chunks_out = 0;    // batches holding its pairs (dispatcher only)
    int status = PADO_OK;
    std::atomic<int> done{0};
    double t_arrival = 0, t_done = 0;
};

// One staging copy: caller memory <-> page-locked slot memory.
struct CopyJob {
    void *dst;
    const void *src;
    uint64_t bytes;
};

// Helper threads that split a batch's staging copies.  A full batch moves 8
// bytes per pair from callers' pageable arrays into page-locked staging (2 MiB
// at 2^18 pairs) and the results back; one host core copies about 10 GB/s,
// which would cap the loop below what the GPU answers.  Lists under MIN_SPLIT
// bytes are copied by the calling thread alone.
class CopyCrew {
public:
    explicit CopyCrew(unsigned helpers) : nhelp_(helpers)
    {
        for (unsigned i = 0; i < helpers; ++i) th_.emplace_back([this, i] { loop(i); });
    }
    ~CopyCrew()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (std::thread &t : th_) t.join();
    }
    // Performs every job; the calling thread copies the last share itself.
    void run(const std::vector<CopyJob> &jobs)
    {
        uint64_t total = 0;
        for (const CopyJob &j : jobs) total += j.bytes;
        if (!nhelp_ || total < MIN_SPLIT) {
            copy_range(jobs, 0, total);
            return;
        }
        const unsigned parts = nhelp_ + 1;
        {
            std::lock_guard<std::mutex> lk(mu_);
            jobs_ = &jobs;
            total_ = total;
            pending_ = nhelp_;
            ++gen_;
        }
        cv_.notify_all();
        copy_range(jobs, total * nhelp_ / parts, total);
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return pending_ == 0; });
        jobs_ = nullptr;
    }

private:
    static constexpr uint64_t MIN_SPLIT = 256ull << 10;

    // bytes [lo, hi) of the jobs laid end to end
    static void copy_range(const std::vector<CopyJob> &jobs, uint64_t lo, uint64_t hi)
    {
        uint64_t at = 0;
        for (const CopyJob &j : jobs) {
            if (at >= hi) break;
            const uint64_t a = std::max(lo, at), b = std::min(hi, at + j.bytes);
            if (a < b)
                memcpy(static_cast<unsigned char *>(j.dst) + (a - at),
                       static_cast<const unsigned char *>(j.src) + (a - at), b - a);
            at += j.bytes;
        }
    }

    void loop(unsigned i)
    {
        uint64_t seen = 0;
        for (;;) {
            const std::vector<CopyJob> *jobs;
            uint64_t total;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
                jobs = jobs_;
                total = total_;
            }
            const unsigned parts = nhelp_ + 1;
            copy_range(*jobs, total * i / parts, total * (i + 1) / parts);
            std::lock_guard<std::mutex> lk(mu_);
            if (--pending_ == 0) done_.notify_one();
        }
    }

    const unsigned nhelp_;
    std::vector<std::thread> th_;
    std::mutex mu_;
    std::condition_variable cv_, done_;
    const std::vector<CopyJob> *jobs_ = nullptr;
    uint64_t total_ = 0, gen_ = 0;
    unsigned pending_ = 0;
    bool stop_ = false;
};

struct Slot {
    HBuf<uint32_t> ha, hb;
    HBuf<unsigned char> hout;
    HBuf<ServeRun> hrun;
    DBuf<uint32_t> da, db;
    DBuf<unsigned char> dout;
    DBuf<ServeRun> drun;
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    struct Item {
        Req *r;
        uint64_t off, len, out_pos;  // request pairs [off, off+len) -> batch output bytes from out_pos
        uint32_t esz;
    };
    std::vector<Item> items;
    std::vector<uint32_t> used;   // indexes this batch reads (in-flight references)
    std::vector<CopyJob> copies;  // staging copies of the batch being filled or retired
};

struct Entry {
    pado_index *h = nullptr;
    uint64_t bytes = 0;
    uint64_t last_use = 0;
    uint32_t inflight = 0;
    bool weighted = false;
};

}  // namespace
}  // namespace pado

using pado::CopyCrew;
using pado::CopyJob;
using pado::Entry;
using pado::Req;
using pado::Slot;

struct pado_server {
    int device = 0;
    uint64_t budget = 0, resident_bytes = 0;
    uint32_t max_pairs = 0, max_runs = 0;
    std::deque<Entry> idx;         // a deque: entries keep their address as indexes are added
    std::vector<Slot> slots;
    std::mutex mu;                 // queue, tickets, completion
    std::condition_variable cv_work, cv_done;
    std::deque<Req *> q;
    std::mutex idx_mu;             // index table and residency
    std::thread worker;
    std::atomic<bool> stop{false};
    std::unordered_map<uint64_t, std::unique_ptr<Req>> tickets;
    uint64_t next_ticket = 1, use_clock = 0;
    cudaStream_t admin = nullptr;
    pado_server_stats st{};
    std::string fatal;             // a CUDA error that stopped the dispatcher
    std::unique_ptr<CopyCrew> crew;  // splits the dispatcher's staging copies

    void run();
    bool acquire(uint32_t i, Slot &sl, pado::IndexView *v, bool *weighted);
    void release(Slot &sl);
    void evict_to_fit(uint64_t need, uint32_t keep);
    void complete(Slot &sl);
    bool dispatch(Slot &sl);
    void fail_all(const std::string &why);
};

namespace {

constexpr uint64_t HBM_RESERVE = 512ull << 20;  // left free for the loop's own buffers and other users

void finish(pado_server *S, Req *r, int status)
{
    r->status = status;
    r->t_done = pado::now_s();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->done.store(1, std::memory_order_release);
    }
    S->cv_done.notify_all();
}

}  // namespace

// Offload least-recently-used idle label sets until `need` more bytes fit the
// budget and free HBM.  Caller holds idx_mu.
void pado_server::evict_to_fit(uint64_t need, uint32_t keep)
{
    for (;;) {
        size_t free_b = 0, total_b = 0;
        PADO_CUDA(cudaMemGetInfo(&free_b, &total_b));
        const bool budget_ok = resident_bytes + need <= budget;
        const bool hbm_ok = need == 0 || free_b >= need + HBM_RESERVE;
        if (budget_ok && hbm_ok) return;
        int victim = -1;
        for (size_t j = 0; j < idx.size(); ++j) {
            const Entry &e = idx[j];
            if (j == keep || e.inflight || !pado::index_resident(e.h)) continue;
            if (victim < 0 || e.last_use < idx[victim].last_use) victim = (int)j;
        }
        if (victim < 0) {
            if (budget_ok) return;  // HBM is short but nothing idle is left to offload: try anyway
            throw pado::Error(PADO_E_NOMEM, "label sets in use exceed the HBM budget");
        }
        pado::index_offload(idx[victim].h, admin);
        resident_bytes -= idx[victim].bytes;
        st.evictions++;
    }
}

// Makes label set i resident and, unless batch `sl` already holds it, takes an
// in-flight reference for the batch (so it cannot be evicted before the batch
// retires); returns its view.  Returns false if it cannot be admitted while
// other batches hold the memory.  One lock covers the check, the admission and
// the reference, so nothing can offload the set in between.
bool pado_server::acquire(uint32_t i, Slot &sl, pado::IndexView *v, bool *weighted)
{
    std::lock_guard<std::mutex> lk(idx_mu);
    Entry &e = idx[i];
    e.last_use = ++use_clock;
    if (!pado::index_resident(e.h)) {
        if (e.bytes > budget) throw pado::Error(PADO_E_NOMEM, "label set is larger than the HBM budget");
        try {
            evict_to_fit(e.bytes, i);
        } catch (const pado::Error &) {
            return false;  // everything else is in flight: retry once batches retire
        }
        pado::index_reload(e.h, admin);
        resident_bytes += e.bytes;
        st.admissions++;
    }
    if (std::find(sl.used.begin(), sl.used.end(), i) == sl.used.end()) {
        e.inflight++;
        sl.used.push_back(i);
    }
    *v = pado::index_view(e.h);
    *weighted = e.weighted;
    return true;
}

void pado_server::release(Slot &sl)
{
    std::lock_guard<std::mutex> lk(idx_mu);
    for (uint32_t i : sl.used) idx[i].inflight--;
    sl.used.clear();
}

void pado_server::complete(Slot &sl)
{
    sl.copies.clear();
    for (const Slot::Item &it : sl.items)
        sl.copies.push_back({static_cast<unsigned char *>(it.r->out) + it.off * it.esz, sl.hout.p + it.out_pos,
                             it.len * it.esz});
    crew->run(sl.copies);
    sl.copies.clear();
    for (const Slot::Item &it : sl.items)
        if (--it.r->chunks_out == 0 && it.r->next == it.r->k) finish(this, it.r, PADO_OK);
    release(sl);
    sl.items.clear();
}

// Fill `sl` from the queue and launch it.  Returns false if nothing was taken.
bool pado_server::dispatch(Slot &sl)
{
    uint64_t pairs = 0, out_bytes = 0;
    uint32_t nrun = 0;
    sl.copies.clear();
    for (;;) {
        Req *r = nullptr;
        {
            std::lock_guard<std::mutex> lk(mu);
            if (q.empty()) break;
            r = q.front();
        }
        if (pairs >= max_pairs || nrun >= max_runs) break;

        pado::IndexView view;
        bool weighted = false, resident;
        try {
            resident = acquire(r->index, sl, &view, &weighted);
        } catch (const pado::Error &e) {
            {
                std::lock_guard<std::mutex> lk(mu);
                q.pop_front();
            }
            finish(this, r, e.code);
            continue;
        }
        if (!resident) break;  // its label set waits for in-flight batches to retire
        const uint32_t esz = weighted ? 2u : 1u;
        const uint64_t take = std::min<uint64_t>(r->k - r->next, max_pairs - pairs);
        out_bytes = (out_bytes + 1) & ~1ull;  // int16 results start 2-byte aligned
        // the request's arrays stay valid until it completes, which is after this batch retires
        sl.copies.push_back({sl.ha.p + pairs, r->a + r->next, take * 4});
        sl.copies.push_back({sl.hb.p + pairs, r->b + r->next, take * 4});
        pado::ServeRun &run = sl.hrun.p[nrun++];
        run.start = pairs;
        run.out_off = out_bytes;
        run.v = view;
        run.v.work = nullptr;
        run.weighted = weighted ? 1u : 0u;
        sl.items.push_back({r, r->next, take, out_bytes, esz});
        r->next += take;
        r->chunks_out++;
        pairs += take;
        out_bytes += take * esz;
        if (r->next == r->k) {
            std::lock_guard<std::mutex> lk(mu);
            q.pop_front();
        }
    }
    if (!pairs) {
        release(sl);  // a set admitted for a request that did not fit
        return false;
    }
    crew->run(sl.copies);
    sl.copies.clear();
    sl.hrun.p[0].v.work = pado::work_counters();
    PADO_CUDA(cudaMemcpyAsync(sl.da.p, sl.ha.p, pairs * 4, cudaMemcpyHostToDevice, sl.s));
    PADO_CUDA(cudaMemcpyAsync(sl.db.p, sl.hb.p, pairs * 4, cudaMemcpyHostToDevice, sl.s));
    PADO_CUDA(cudaMemcpyAsync(sl.drun.p, sl.hrun.p, nrun * sizeof(pado::ServeRun), cudaMemcpyHostToDevice, sl.s));
    const unsigned grid = pado::grid_for(pairs * 32, 256, 152u * 64u);
    PADO_LAUNCH("serve_query_kernel", sl.s,
                pado::serve_query_kernel<<<grid, 256, 0, sl.s>>>(sl.drun.p, nrun, pairs, sl.da.p, sl.db.p,
                                                                 sl.dout.p));
    PADO_CUDA(cudaMemcpyAsync(sl.hout.p, sl.dout.p, out_bytes, cudaMemcpyDeviceToHost, sl.s));
    PADO_CUDA(cudaEventRecord(sl.ev, sl.s));
    st.batches++;
    st.pairs += pairs;
    st.max_batch_pairs = std::max<uint64_t>(st.max_batch_pairs, pairs);
    return true;
}

void pado_server::fail_all(const std::string &why)
{
    fatal = why;
    for (Slot &sl : slots)
        for (const Slot::Item &it : sl.items)
            if (!it.r->done.load()) finish(this, it.r, PADO_E_CUDA);
    std::deque<Req *> rest;
    {
        std::lock_guard<std::mutex> lk(mu);
        rest.swap(q);
    }
    for (Req *r : rest) finish(this, r, PADO_E_CUDA);
}

void pado_server::run()
{
    cudaSetDevice(device);
    std::deque<size_t> busy;      // slots in issue order
    std::vector<size_t> free_slots;
    for (size_t i = 0; i < slots.size(); ++i) free_slots.push_back(slots.size() - 1 - i);
    try {
        for (;;) {
            bool progress = false;
            while (!busy.empty()) {
                Slot &sl = slots[busy.front()];
                const cudaError_t e = cudaEventQuery(sl.ev);
                if (e == cudaErrorNotReady) break;
                PADO_CUDA(e);
                complete(sl);
                free_slots.push_back(busy.front());
                busy.pop_front();
                progress = true;
            }
            if (!free_slots.empty() && dispatch(slots[free_slots.back()])) {
                busy.push_back(free_slots.back());
                free_slots.pop_back();
                progress = true;
            }
            if (progress) continue;
            std::unique_lock<std::mutex> lk(mu);
            if (busy.empty()) {
                if (stop.load() && q.empty()) break;
                if (q.empty()) cv_work.wait(lk, [&] { return stop.load() || !q.empty(); });
            } else {
                lk.unlock();
                std::this_thread::yield();  // batches in flight: poll their events
            }
        }
    } catch (const std::exception &e) {
        fail_all(e.what());
    }
}

namespace {

int serr(int code, const std::string &m)
{
    pado::set_error(code, m);
    return code;
}

void submit(pado_server *S, Req *r)
{
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->q.push_back(r);
        S->st.requests++;
    }
    S->cv_work.notify_one();
}

}  // namespace

extern "C" {

int pado_server_create(uint64_t hbm_budget_bytes, uint32_t max_batch_pairs, uint32_t slots, pado_server **out)
{
    if (!out) return serr(PADO_E_ARG, "null output handle");
    *out = nullptr;
    if (!max_batch_pairs || max_batch_pairs > (1u << 26)) return serr(PADO_E_ARG, "max_batch_pairs must be in [1, 2^26]");
    if (!slots || slots > 16) return serr(PADO_E_ARG, "slots must be in [1, 16]");
    try {
        std::unique_ptr<pado_server> S(new pado_server);
        PADO_CUDA(cudaGetDevice(&S->device));
        S->budget = hbm_budget_bytes;
        S->max_pairs = max_batch_pairs;
        S->max_runs = std::min<uint32_t>(max_batch_pairs, 65536u);
        PADO_CUDA(cudaStreamCreateWithFlags(&S->admin, cudaStreamNonBlocking));
        S->slots.resize(slots);
        for (Slot &sl : S->slots) {
            sl.ha.alloc(max_batch_pairs);
            sl.hb.alloc(max_batch_pairs);
            sl.hout.alloc((uint64_t)max_batch_pairs * 2 + 2 * S->max_runs);
            sl.hrun.alloc(S->max_runs);
            sl.da.alloc(max_batch_pairs);
            sl.db.alloc(max_batch_pairs);
            sl.dout.alloc((uint64_t)max_batch_pairs * 2 + 2 * S->max_runs);
            sl.drun.alloc(S->max_runs);
            PADO_CUDA(cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking));
            PADO_CUDA(cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
        }
        // helpers for the staging copies: a quarter of the host threads, at most 4
        S->crew.reset(new CopyCrew(std::min(4u, std::thread::hardware_concurrency() / 4)));
        pado_server *raw = S.get();
        S->worker = std::thread([raw] { raw->run(); });
        *out = S.release();
        return PADO_OK;
    } catch (const pado::Error &e) {
        return serr(e.code, e.what());
    }
}

void pado_server_destroy(pado_server *S)
{
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop.store(true);
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    cudaSetDevice(S->device);
    // label sets go back to HBM, so the caller's handles work as before
    for (Entry &e : S->idx) {
        try {
            pado::index_reload(e.h, S->admin);
        } catch (...) {
        }
    }
    for (Slot &sl : S->slots) {
        if (sl.s) cudaStreamDestroy(sl.s);
        if (sl.ev) cudaEventDestroy(sl.ev);
    }
    if (S->admin) cudaStreamDestroy(S->admin);
    delete S;
}

int pado_server_add(pado_server *S, pado_index *h, uint32_t *index_id)
{
    if (!S || !h || !index_id) return serr(PADO_E_ARG, "null argument");
    if (!pado::index_resident(h)) return serr(PADO_E_STATE, "index is offloaded");
    if (pado::index_device(h) != S->device) return serr(PADO_E_ARG, "index lives on another device");
    try {
        std::lock_guard<std::mutex> lk(S->idx_mu);
        for (const Entry &e : S->idx)
            if (e.h == h) return serr(PADO_E_ARG, "index already added");
        Entry e;
        e.h = h;
        e.bytes = pado::index_device_bytes(h);
        e.weighted = pado::index_kind(h) == PADO_WEIGHTED;
        e.last_use = ++S->use_clock;
        S->idx.push_back(e);
        S->resident_bytes += e.bytes;
        *index_id = (uint32_t)(S->idx.size() - 1);
        // keep the resident set within the budget: older idle sets go first
        // (if all of them are in use the budget is exceeded until they retire)
        if (S->resident_bytes > S->budget) {
            cudaSetDevice(S->device);
            try {
                S->evict_to_fit(0, 0xffffffffu);
            } catch (const pado::Error &) {
            }
        }
        return PADO_OK;
    } catch (const pado::Error &e) {
        return serr(e.code, e.what());
    }
}

int pado_server_submit(pado_server *S, uint32_t index_id, uint64_t k, const uint32_t *a, const uint32_t *b, void *out,
                       uint64_t *ticket)
{
    if (!S || !ticket || (k && (!a || !b || !out))) return serr(PADO_E_ARG, "null argument");
    {
        std::lock_guard<std::mutex> lk(S->idx_mu);
        if (index_id >= S->idx.size()) return serr(PADO_E_ARG, "unknown index id");
    }
    if (!S->fatal.empty()) return serr(PADO_E_CUDA, "serving loop stopped: " + S->fatal);
    std::unique_ptr<Req> r(new Req);
    r->index = index_id;
    r->k = k;
    r->a = a;
    r->b = b;
    r->out = out;
    r->t_arrival = pado::now_s();
    Req *raw = r.get();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        *ticket = S->next_ticket++;
        S->tickets.emplace(*ticket, std::move(r));
    }
    if (k == 0) {
        finish(S, raw, PADO_OK);
        return PADO_OK;
    }
    submit(S, raw);
    return PADO_OK;
}

int pado_server_wait(pado_server *S, uint64_t ticket, double timeout_s, double *latency_s)
{
    if (!S) return serr(PADO_E_ARG, "null argument");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->tickets.find(ticket);
    if (it == S->tickets.end()) return serr(PADO_E_ARG, "unknown ticket");
    Req *r = it->second.get();
    const auto pred = [&] { return r->done.load(std::memory_order_acquire) != 0; };
    if (timeout_s < 0)
        S->cv_done.wait(lk, pred);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
        return serr(PADO_E_TIMEOUT, "request not finished within the timeout");
    const int st = r->status;
    if (latency_s) *latency_s = r->t_done - r->t_arrival;
    S->tickets.erase(it);
    if (st != PADO_OK) return serr(st, "request failed" + (S->fatal.empty() ? std::string() : ": " + S->fatal));
    return PADO_OK;
}

int pado_server_get_stats(pado_server *S, pado_server_stats *out)
{
    if (!S || !out) return serr(PADO_E_ARG, "null argument");
    std::lock_guard<std::mutex> lk(S->idx_mu);
    *out = S->st;
    out->resident_bytes = S->resident_bytes;
    uint32_t res = 0;
    for (const Entry &e : S->idx) res += pado::index_resident(e.h) ? 1u : 0u;
    out->resident_indexes = res;
    return PADO_OK;
}

int pado_server_replay(pado_server *S, uint64_t nreq, const double *arrival_s, const uint32_t *index_id,
                       const uint64_t *k, const uint64_t *pair_off, const uint32_t *a, const uint32_t *b, uint8_t *out8,
                       int16_t *out16, uint32_t mode, double *latency_s)
{
    if (!S || (nreq && (!arrival_s || !index_id || !k || !pair_off || !a || !b || !latency_s)))
        return serr(PADO_E_ARG, "null argument");
    if (mode > 1) return serr(PADO_E_ARG, "mode must be 0 (batched) or 1 (one launch per request)");
    std::vector<uint8_t> wt;
    {
        std::lock_guard<std::mutex> lk(S->idx_mu);
        for (uint64_t i = 0; i < nreq; ++i)
            if (index_id[i] >= S->idx.size()) return serr(PADO_E_ARG, "unknown index id");
        for (const Entry &e : S->idx) wt.push_back(e.weighted ? 1 : 0);
    }
    for (uint64_t i = 0; i < nreq; ++i)
        if ((wt[index_id[i]] ? out16 : (int16_t *)out8) == nullptr) return serr(PADO_E_ARG, "null output");
    std::vector<Req> reqs(nreq);
    for (uint64_t i = 0; i < nreq; ++i) {
        Req &r = reqs[i];
        r.index = index_id[i];
        r.k = k[i];
        r.a = a + pair_off[i];
        r.b = b + pair_off[i];
        r.out = wt[r.index] ? (void *)(out16 + pair_off[i]) : (void *)(out8 + pair_off[i]);
    }
    const double t0 = pado::now_s() + 1e-3;
    try {
        if (mode == 0) {
            for (uint64_t i = 0; i < nreq; ++i) {
                Req &r = reqs[i];
                r.t_arrival = t0 + arrival_s[i];
                while (pado::now_s() < r.t_arrival) {
                }
                if (r.k == 0) {
                    finish(S, &r, PADO_OK);
                    continue;
                }
                submit(S, &r);
            }
            std::unique_lock<std::mutex> lk(S->mu);
            for (uint64_t i = 0; i < nreq; ++i)
                S->cv_done.wait(lk, [&] { return reqs[i].done.load(std::memory_order_acquire) != 0; });
        } else {
            // unbatched: each request copied, launched and read back on its own,
            // in arrival order (a FIFO server doing one launch per request), with
            // buffers of its own so the dispatcher's slots are never shared
            PADO_CUDA(cudaSetDevice(S->device));
            Slot sl;
            sl.ha.alloc(S->max_pairs);
            sl.hb.alloc(S->max_pairs);
            sl.hout.alloc((uint64_t)S->max_pairs * 2);
            sl.da.alloc(S->max_pairs);
            sl.db.alloc(S->max_pairs);
            sl.dout.alloc((uint64_t)S->max_pairs * 2);
            PADO_CUDA(cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking));
            struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } sg{sl.s};
            struct RefGuard {  // drop in-flight references if a request fails midway
                pado_server *S;
                Slot &sl;
                ~RefGuard() { S->release(sl); }
            } rg{S, sl};
            for (uint64_t i = 0; i < nreq; ++i) {
                Req &r = reqs[i];
                r.t_arrival = t0 + arrival_s[i];
                while (pado::now_s() < r.t_arrival) {
                }
                for (uint64_t off = 0; off < r.k; off += S->max_pairs) {
                    const uint64_t take = std::min<uint64_t>(r.k - off, S->max_pairs);
                    pado::IndexView v;
                    bool weighted = false;
                    if (!S->acquire(r.index, sl, &v, &weighted))
                        throw pado::Error(PADO_E_NOMEM, "label set cannot be admitted");
                    memcpy(sl.ha.p, r.a + off, take * 4);
                    memcpy(sl.hb.p, r.b + off, take * 4);
                    PADO_CUDA(cudaMemcpyAsync(sl.da.p, sl.ha.p, take * 4, cudaMemcpyHostToDevice, sl.s));
                    PADO_CUDA(cudaMemcpyAsync(sl.db.p, sl.hb.p, take * 4, cudaMemcpyHostToDevice, sl.s));
                    const uint32_t esz = wt[r.index] ? 2 : 1;
                    if (wt[r.index])
                        pado::launch_query_w(v, take, sl.da.p, sl.db.p, reinterpret_cast<int16_t *>(sl.dout.p), sl.s);
                    else
                        pado::launch_query_unw(v, take, sl.da.p, sl.db.p, sl.dout.p, sl.s);
                    PADO_CUDA(cudaMemcpyAsync(sl.hout.p, sl.dout.p, take * esz, cudaMemcpyDeviceToHost, sl.s));
                    PADO_CUDA(cudaStreamSynchronize(sl.s));
                    S->release(sl);
                    memcpy(static_cast<unsigned char *>(r.out) + off * esz, sl.hout.p, take * esz);
                }
                r.t_done = pado::now_s();
                r.done.store(1);
                S->st.requests++;
                S->st.batches++;
                S->st.pairs += r.k;
            }
        }
    } catch (const pado::Error &e) {
        return serr(e.code, e.what());
    }
    int status = PADO_OK;
    for (uint64_t i = 0; i < nreq; ++i) {
        latency_s[i] = reqs[i].t_done - reqs[i].t_arrival;
        if (reqs[i].status != PADO_OK) status = reqs[i].status;
    }
    if (status != PADO_OK) return serr(status, "a request failed" + (S->fatal.empty() ? std::string() : ": " + S->fatal));
    return PADO_OK;
}

}  // extern "C"
