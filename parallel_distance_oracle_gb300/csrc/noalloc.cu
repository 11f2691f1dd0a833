// noalloc.cu -- distance queries that allocate no device memory.
//
// pado_query() stages the caller's pairs and results in device memory it
// allocates per call.  Some callers cannot let a library allocate:
//   * serving threads with a latency budget, where cudaMalloc / cudaFree (and
//     even the stream-ordered allocator when its pool has to grow) can block
//     on device-wide synchronisation or a driver lock and stall every other
//     stream in the process;
//   * processes whose device memory is owned by another allocator (a
//     framework's caching allocator that reserved the GPU up front, or a
//     fixed budget handed out by a host application), where an allocation
//     from a library either fails or breaks the owner's accounting.
// For them pado_query_noalloc() stages through one fixed area that is part of
// the library image: a file-scope __device__ array of NOALLOC_MAX_PAIRS pairs
// (2.5 MiB), held on every GPU where the library's device code is loaded
// until the process exits.  Host code cannot use the array's name as a device
// address, so the first call on each device looks its address up with
// cudaGetSymbolAddress while that device is current and remembers it; that
// first call should happen before any stream capture, and it is the slow one:
// with lazy module loading (the default since CUDA 12.2) it is also what loads
// the library's device code and creates the area, which the driver may do
// with allocations and synchronisation of its own.  Callers make one warm-up
// call per device (k >= 1) before their latency-sensitive section.  A device
// reset (cudaDeviceReset) unloads the area; the remembered address is stale
// afterwards, so this entry point must not be used on a device after it was
// reset.  Nothing in the area needs to start at zero: every call writes the
// slots it reads.  All calls on a device share the area and keep the last
// call's contents, so calls that overlap on the GPU (for example from two host
// threads at once) race on it; callers must serialise them.  The caller's
// current device is left as it was.

#include <map>
#include <mutex>

#include "pado_internal.cuh"

namespace {

constexpr uint64_t NOALLOC_MAX_PAIRS = PADO_NOALLOC_MAX_PAIRS;

// [0, 4M): endpoints a; [4M, 8M): endpoints b; [8M, 10M): results
// (M = NOALLOC_MAX_PAIRS; uint8 results use the first half of the last part).
static __device__ __align__(256) unsigned char g_query_scratch[NOALLOC_MAX_PAIRS * 10];

std::mutex g_setup_mu;
std::map<int, unsigned char *> g_scratch_addr;  // device -> address of g_query_scratch

// Address of the scratch array on the current device (looked up once).
int scratch_on_device(int dev, unsigned char **out)
{
    std::lock_guard<std::mutex> lk(g_setup_mu);
    auto it = g_scratch_addr.find(dev);
    if (it != g_scratch_addr.end()) {
        *out = it->second;
        return PADO_OK;
    }
    unsigned char *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_query_scratch);
    if (e != cudaSuccess || !p)
        return pado::set_error(PADO_E_CUDA, std::string("cudaGetSymbolAddress(query scratch): ") +
                                                cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
    *out = p;
    return PADO_OK;
}

}  // namespace

extern "C" {

int pado_query_noalloc(pado_index *h, uint64_t k, const uint32_t *a, const uint32_t *b, void *out)
{
    if (!h || (k && (!a || !b || !out))) return pado::set_error(PADO_E_ARG, "null argument");
    if (k > NOALLOC_MAX_PAIRS)
        return pado::set_error(PADO_E_ARG, "pado_query_noalloc: " + std::to_string(k) +
                                               " pairs exceed its fixed staging area of " +
                                               std::to_string(NOALLOC_MAX_PAIRS) +
                                               " pairs; split the batch or use pado_query");
    if (!k) return PADO_OK;
    if (!pado::index_resident(h))
        return pado::set_error(PADO_E_STATE, "index is offloaded to host memory by a serving loop");
    int prev = -1;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return pado::set_error(PADO_E_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    const int dev = pado::index_device(h);
    if (dev != prev) {
        e = cudaSetDevice(dev);
        if (e != cudaSuccess)
            return pado::set_error(PADO_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    }
    cudaStream_t s = cudaStreamPerThread;
    int st = PADO_OK;
    try {
        unsigned char *base = nullptr;
        st = scratch_on_device(dev, &base);
        if (st == PADO_OK) {
            uint32_t *da = reinterpret_cast<uint32_t *>(base);
            uint32_t *db = reinterpret_cast<uint32_t *>(base + NOALLOC_MAX_PAIRS * 4);
            unsigned char *dout = base + NOALLOC_MAX_PAIRS * 8;
            const bool unw = pado::index_kind(h) == PADO_UNWEIGHTED;
            const size_t osz = unw ? 1 : 2;
            PADO_CUDA(cudaMemcpyAsync(da, a, k * 4, cudaMemcpyHostToDevice, s));
            PADO_CUDA(cudaMemcpyAsync(db, b, k * 4, cudaMemcpyHostToDevice, s));
            const pado::IndexView v = pado::index_view(h);
            if (unw)
                pado::launch_query_unw(v, k, da, db, dout, s);
            else
                pado::launch_query_w(v, k, da, db, reinterpret_cast<int16_t *>(dout), s);
            PADO_CUDA(cudaMemcpyAsync(out, dout, k * osz, cudaMemcpyDeviceToHost, s));
            PADO_CUDA(cudaStreamSynchronize(s));
        }
    } catch (const pado::Error &err) {
        cudaStreamSynchronize(s);
        st = pado::set_error(err.code, err.what());
    } catch (const std::bad_alloc &) {
        st = pado::set_error(PADO_E_NOMEM, "host allocation failed");
    } catch (const std::exception &err) {
        cudaStreamSynchronize(s);
        st = pado::set_error(PADO_E_CUDA, err.what());
    }
    if (dev != prev) cudaSetDevice(prev);
    return st;
}

}  // extern "C"
