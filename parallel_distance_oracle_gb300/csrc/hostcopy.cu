// hostcopy.cu -- host <-> device copies that the SMs carry out.
//
// Page-locked host memory (cudaHostAlloc / cudaHostRegister) has a device
// alias that kernels can read and write directly.  Copies to and from such
// memory are done here by a plain copy kernel rather than by the copy engines
// (cudaMemcpyAsync): on hosts where the copy engines are slowed by other work,
// half of the 1.5 GB exports of an R-MAT s20 index took 120 ms through them and
// 8-27 ms through the SMs.  Any other host memory goes through cudaMemcpyAsync.

#include "pado_internal.cuh"

namespace pado {
namespace {

// dst[0, bytes) = src[0, bytes), 16 bytes per thread step where the two
// pointers share their alignment; the unaligned head and the tail bytewise.
__global__ void __launch_bounds__(256) sm_copy_kernel(const unsigned char *src, unsigned char *dst, uint64_t bytes)
{
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t mis = (16 - ((uintptr_t)dst & 15)) & 15;
    const uint64_t head = ((uintptr_t)src & 15) == ((uintptr_t)dst & 15) ? (mis < bytes ? mis : bytes) : bytes;
    for (uint64_t i = tid; i < head; i += nth) dst[i] = src[i];
    if (head == bytes) return;
    const uint64_t body = (bytes - head) / 16;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src + head);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst + head);
    for (uint64_t i = tid; i < body; i += nth) d4[i] = s4[i];
    for (uint64_t i = head + body * 16 + tid; i < bytes; i += nth) dst[i] = src[i];
}

void sm_copy(const void *src, void *dst, uint64_t bytes, cudaStream_t s, const char *name)
{
    PADO_LAUNCH(name, s,
                sm_copy_kernel<<<grid_for(bytes / 16 + 1, 256, 152u * 16u), 256, 0, s>>>(
                    static_cast<const unsigned char *>(src), static_cast<unsigned char *>(dst), bytes));
}

}  // namespace

void *mapped_host(const void *p)
{
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // an unknown pointer is not an error here
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

void download_bytes(void *h, const void *d, uint64_t bytes, cudaStream_t s)
{
    if (!bytes) return;
    void *dh = mapped_host(h);
    if (dh)
        sm_copy(d, dh, bytes, s, "host_write_kernel");
    else
        PADO_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s));
}

void upload_bytes(void *d, const void *h, uint64_t bytes, cudaStream_t s)
{
    if (!bytes) return;
    const void *dh = mapped_host(h);
    if (dh)
        sm_copy(dh, d, bytes, s, "host_read_kernel");
    else
        PADO_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s));
}

}  // namespace pado
