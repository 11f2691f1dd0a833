// pado_common.cuh -- shared device/host helpers for the PADO GPU library.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "pado_gpu.h"

namespace pado {

constexpr uint8_t U8_INF = 255;      // includes/globals.h:37 (WEIGHTI_MAX)
constexpr int16_t I16_INF = 32767;   // includes/globals.h:39 (WEIGHTILARGE_MAX)
constexpr uint32_t MAX_BP = 64;      // bit-parallel roots the kernels support
constexpr uint32_t MAX_BATCH = 2048; // root batch sizes the kernels support

// Error carried from a failing CUDA call or argument check to the C ABI.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define PADO_CUDA(call)                                                                     \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            throw ::pado::Error(e_ == cudaErrorMemoryAllocation ? PADO_E_NOMEM : PADO_E_CUDA, \
                                std::string(#call) + ": " + cudaGetErrorString(e_));       \
    } while (0)

#define PADO_CHECK(cond, code, msg)                                  \
    do {                                                             \
        if (!(cond)) throw ::pado::Error((code), (msg));             \
    } while (0)

// A host-side phase of a library call: an NVTX range (shown by Nsight tools
// when one is attached; a no-op otherwise) and, with PADO_TRACE set in the
// environment, the phase's wall time on stderr when it ends.
struct HostPhase {
    const char *name;
    std::chrono::steady_clock::time_point t0;
    explicit HostPhase(const char *n) : name(n), t0(std::chrono::steady_clock::now()) { nvtxRangePushA(n); }
    HostPhase(const HostPhase &) = delete;
    HostPhase &operator=(const HostPhase &) = delete;
    ~HostPhase()
    {
        nvtxRangePop();
        static const bool trace = std::getenv("PADO_TRACE") != nullptr;
        if (trace)
            fprintf(stderr, "phase %s %.3f ms\n", name,
                    std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
};

#ifdef PADO_DEBUG_BOUNDS
// p[i] when i < lim; otherwise records `site` in *dbg and returns a reference
// to a scratch slot (a write there is harmless, a read returns its bytes).
__device__ __align__(16) static unsigned char g_dbg_sink[64];
template <typename T>
__device__ __forceinline__ T &dbg_ref(T *p, uint64_t i, uint64_t lim, uint32_t site, uint32_t *dbg)
{
    static_assert(sizeof(T) <= sizeof(g_dbg_sink), "scratch slot too small");
    if (i < lim) return p[i];
    if (dbg) atomicOr(dbg, 1u << site);
    return *reinterpret_cast<T *>(g_dbg_sink);
}
#endif

// Allocation accounting (profile.cu): every device buffer of the library
// passes alloc_point() before it allocates -- which fails the allocation
// with PADO_E_NOMEM when a test armed pado_debug_fail_alloc for it -- and
// counts itself live until released (pado_debug_live_allocations).
void alloc_point();
void alloc_live(int delta);

// Owning device buffer.
template <typename T>
struct DBuf {
    T *p = nullptr;
    size_t n = 0;
    DBuf() = default;
    explicit DBuf(size_t count) { alloc(count); }
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf &operator=(DBuf &&o) noexcept
    {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count)
    {
        release();
        if (count) {
            alloc_point();
            PADO_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
            alloc_live(1);
        }
        n = count;
    }
    // Stream-ordered allocation from the device's default memory pool (cheap
    // when many small buffers are made at once); cudaFree releases it like
    // any other.
    void alloc_async(size_t count, cudaStream_t s)
    {
        release();
        if (count) {
            alloc_point();
            PADO_CUDA(cudaMallocAsync((void **)&p, count * sizeof(T), s));
            alloc_live(1);
        }
        n = count;
    }
    void release()
    {
        if (p) {
            cudaFree(p);
            alloc_live(-1);
        }
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
    void upload(const T *h, size_t count, cudaStream_t s = 0)
    {
        if (count) PADO_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T *h, size_t count, cudaStream_t s = 0) const
    {
        if (count) PADO_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void fill_bytes(int v, cudaStream_t s = 0)
    {
        if (n) PADO_CUDA(cudaMemsetAsync(p, v, bytes(), s));
    }
};

// Owning page-locked host buffer (DMA-able without a driver-side staging copy).
template <typename T>
struct HBuf {
    T *p = nullptr;
    size_t n = 0;
    HBuf() = default;
    explicit HBuf(size_t count) { alloc(count); }
    HBuf(const HBuf &) = delete;
    HBuf &operator=(const HBuf &) = delete;
    HBuf(HBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    HBuf &operator=(HBuf &&o) noexcept
    {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~HBuf() { release(); }
    void alloc(size_t count)
    {
        release();
        if (count) PADO_CUDA(cudaMallocHost((void **)&p, count * sizeof(T)));
        n = count;
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
};

inline unsigned grid_for(uint64_t items, unsigned block, unsigned cap = 152u * 64u)
{
    uint64_t g = (items + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

#ifdef __CUDACC__
// Slot for one new entry of a list whose length is *cnt.  The threads that
// reach this call together share one atomicAdd (warp-aggregated), which keeps
// a global list counter from serialising every append of a wide frontier.
__device__ __forceinline__ uint32_t agg_append(uint32_t *cnt)
{
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(cnt, (uint32_t)g.size());
    return g.shfl(base, 0) + g.thread_rank();
}

// Same, for threads that may target different counters: they are grouped by
// the counter's class `c` first.
__device__ __forceinline__ uint32_t agg_append_by(uint32_t *cnt, unsigned c)
{
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::labeled_partition(cg::coalesced_threads(), c);
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(cnt, (uint32_t)g.size());
    return g.shfl(base, 0) + g.thread_rank();
}
#endif

// Device-side status word bits (written by kernels, read by the host).
enum : uint32_t {
    ST_LEVEL_OVERFLOW = 1u,   // a BFS level reached 255 (uint8 distance)
    ST_POOL_RETRY = 2u,       // a warp could not allocate label space
    ST_BAD_INPUT = 4u,
};

// Launch accounting (profile.cu).  PADO_LAUNCH(name, stream, kernel<<<...>>>(...))
// counts the launch, checks it, and times it while profiling is enabled.
void check_launch(const char *what);
bool profiling();
void prof_begin(cudaStream_t s);
void prof_end(const char *name, cudaStream_t s);
#define PADO_LAUNCH(name, stream, ...)         \
    do {                                       \
        ::pado::prof_begin(stream);            \
        __VA_ARGS__;                           \
        ::pado::check_launch(name);            \
        ::pado::prof_end(name, stream);        \
    } while (0)

// Device counters of algorithmic bytes, one slot per hot kernel (null unless
// profiling).
enum WorkSlot : int {
    W_PULL = 0, W_MARK, W_BP_SIB, W_BP_CHILD, W_Q_UNW, W_Q_W, W_WPULL, W_WMARK, W_FINAL,
    // pull_kernel phase cycles (light tails, summed over warps)
    W_CYC_SCAN, W_CYC_BP, W_CYC_DIST, W_CYC_COMMIT, W_CYC_HEAVY,
    // event counts of the unweighted labeling: first offers of a root to a
    // tail in a batch (each one BP test) and labels appended (self labels
    // included) -- the same events as the reference's push order counts
    W_EV_OFFERS, W_EV_LABELS, WORK_SLOTS
};
const char *work_slot_name(int i);
unsigned long long *work_counters();

// Initial label-pool / round-log capacities (entries).  Both grow on demand;
// PADO_DEBUG_POOL_ENTRIES (tests only) starts them tiny so that the exact
// re-run path after a failed reservation is exercised on small graphs.
inline uint64_t debug_pool_entries()
{
    const char *e = std::getenv("PADO_DEBUG_POOL_ENTRIES");
    return e ? std::strtoull(e, nullptr, 10) : 0;
}
// The label pool starts at 256 entries per vertex (1.3 KB/vertex unweighted,
// capped at 2^31 entries): enough for a social-graph labeling plus its list
// relocations in one persistent launch, so growth relaunches are rare.
inline uint64_t initial_pool_entries(uint32_t n)
{
    const uint64_t dbg = debug_pool_entries();
    return dbg ? dbg : std::min<uint64_t>(std::max<uint64_t>((uint64_t)n * 256, 1u << 22), 1ull << 31);
}
// The weighted round logs start at 128 entries per vertex (1 KB per vertex
// for both parities): the busiest rounds of the first batch of a social graph
// accept that many roots per vertex, and every growth stops the persistent
// loop once.
inline uint64_t initial_log_entries(uint32_t n, uint32_t B)
{
    const uint64_t dbg = debug_pool_entries();
    return dbg ? std::max<uint64_t>(dbg, B)
               : std::min<uint64_t>(std::max<uint64_t>((uint64_t)n * 128, (uint64_t)B + (1u << 16)), 1ull << 31);
}

}  // namespace pado
