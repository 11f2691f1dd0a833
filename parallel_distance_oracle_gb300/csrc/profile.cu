// profile.cu -- launch accounting and optional per-kernel timing.
//
// Every kernel launch in the library goes through PADO_LAUNCH, which counts
// it (pado_kernel_launches) and, while profiling is enabled, brackets it with
// a CUDA event pair recorded on the launch's own stream.  Elapsed times are
// collected when the table is read (after the work has completed).  Kernels on
// the hot path also add their algorithmic bytes (the bytes their algorithm
// must move: adjacency, label entries, BP rows, appends -- not re-reads) to a
// device counter that the profile table reports per kernel.

#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "pado_internal.cuh"

namespace pado {
namespace {

std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_profile{0};
std::mutex g_mu;

struct Pending {
    const char *name;
    cudaEvent_t a, b;
};
std::vector<Pending> g_pending;
struct Row {
    uint64_t launches = 0;
    double ms = 0;
    uint64_t bytes = 0;
};
std::map<std::string, Row> g_table;
thread_local cudaEvent_t t_start = nullptr;

unsigned long long *g_work = nullptr;  // device counters, one per WorkSlot

void collect_locked()
{
    for (auto &p : g_pending) {
        float ms = 0;
        if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            Row &r = g_table[p.name];
            r.launches += 1;
            r.ms += ms;
        }
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    g_pending.clear();
    if (g_work) {
        unsigned long long h[WORK_SLOTS] = {};
        if (cudaMemcpy(h, g_work, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess) {
            for (int i = 0; i < WORK_SLOTS; ++i)
                if (h[i]) g_table[work_slot_name(i)].bytes += h[i];
            cudaMemset(g_work, 0, sizeof(h));
        }
    }
}

}  // namespace

const char *work_slot_name(int i)
{
    static const char *names[WORK_SLOTS] = {"pull_kernel",      "mark_kernel",      "bp_sibling_kernel",
                                            "bp_child_kernel",  "query_unw_kernel", "query_w_kernel",
                                            "w_pull_kernel",    "w_mark_kernel",    "finalize_kernel",
                                            "pull.cycles.scan", "pull.cycles.bp",   "pull.cycles.dist",
                                            "pull.cycles.commit", "pull.cycles.heavy", "events.first_offers",
                                            "events.labels_appended"};
    return names[i];
}

bool profiling() { return g_profile.load(std::memory_order_relaxed) != 0; }

unsigned long long *work_counters()
{
    return g_profile.load(std::memory_order_relaxed) == 1 ? g_work : nullptr;
}

void prof_begin(cudaStream_t s)
{
    if (!profiling()) return;
    cudaEventCreate(&t_start);
    cudaEventRecord(t_start, s);
}

void prof_end(const char *name, cudaStream_t s)
{
    if (!profiling() || !t_start) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, s);
    std::lock_guard<std::mutex> lk(g_mu);
    g_pending.push_back({name, t_start, e});
    t_start = nullptr;
}

void check_launch(const char *what)
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw Error(PADO_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// ---- allocation accounting (failure-injection tests) ------------------------
namespace {
std::atomic<int64_t> g_fail_countdown{0};  // > 0: the allocation that brings it to 0 fails
std::atomic<int64_t> g_live{0};            // device buffers of the library not yet released
}  // namespace

void alloc_point()
{
    if (g_fail_countdown.load(std::memory_order_relaxed) <= 0) return;
    if (g_fail_countdown.fetch_sub(1) == 1)
        throw Error(PADO_E_NOMEM, "device allocation failed (injected by pado_debug_fail_alloc)");
}

void alloc_live(int delta) { g_live.fetch_add(delta, std::memory_order_relaxed); }

}  // namespace pado

extern "C" {

int pado_debug_fail_alloc(uint64_t nth)
{
    pado::g_fail_countdown.store((int64_t)nth);
    return PADO_OK;
}

int64_t pado_debug_live_allocations(void) { return pado::g_live.load(); }


uint64_t pado_kernel_launches(void) { return pado::g_launches.load(); }

int pado_profile(int enable)
{
    std::lock_guard<std::mutex> lk(pado::g_mu);
    if (enable && !pado::g_work) {
        if (cudaMalloc((void **)&pado::g_work, pado::WORK_SLOTS * sizeof(unsigned long long)) != cudaSuccess)
            return PADO_E_CUDA;
        cudaMemset(pado::g_work, 0, pado::WORK_SLOTS * sizeof(unsigned long long));
    }
    if (!enable) pado::collect_locked();
    pado::g_profile.store(enable == 2 ? 2 : enable ? 1 : 0);
    return PADO_OK;
}

size_t pado_profile_read(char *buf, size_t len, int reset)
{
    std::lock_guard<std::mutex> lk(pado::g_mu);
    cudaDeviceSynchronize();
    pado::collect_locked();
    std::string out;
    char line[256];
    for (auto &kv : pado::g_table) {
        snprintf(line, sizeof(line), "%s %llu %.6f %llu\n", kv.first.c_str(), (unsigned long long)kv.second.launches,
                 kv.second.ms, (unsigned long long)kv.second.bytes);
        out += line;
    }
    if (reset) pado::g_table.clear();
    if (buf && len) {
        size_t k = std::min(len - 1, out.size());
        memcpy(buf, out.data(), k);
        buf[k] = 0;
    }
    return out.size() + 1;
}

}  // extern "C"
