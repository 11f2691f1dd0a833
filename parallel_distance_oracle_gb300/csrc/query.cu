// query.cu -- exact 2-hop distance queries on a device-resident label set: a
// warp per pair (the per-pair code and its derivation are in
// query_device.cuh), grid-stride over the batch.

#include "query_device.cuh"

namespace pado {
namespace {

__global__ void __launch_bounds__(256) query_unw_kernel(IndexView v, uint64_t k, const uint32_t *__restrict__ qa,
                                                        const uint32_t *__restrict__ qb, uint8_t *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long bytes = 0;
    for (uint64_t p = warp; p < k; p += nwarps) {
        bytes += 9;  // endpoints, result
        const uint8_t d = query_unw_pair(v, qa[p], qb[p], lane, bytes);
        if (lane == 0) out[p] = d;
    }
    if (v.work && lane == 0 && bytes) atomicAdd(&v.work[W_Q_UNW], bytes);
}

__global__ void __launch_bounds__(256) query_w_kernel(IndexView v, uint64_t k, const uint32_t *__restrict__ qa,
                                                      const uint32_t *__restrict__ qb, int16_t *__restrict__ out)
{
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long bytes = 0;
    for (uint64_t p = warp; p < k; p += nwarps) {
        bytes += 10;
        const int16_t d = query_w_pair(v, qa[p], qb[p], lane, bytes);
        if (lane == 0) out[p] = d;
    }
    if (v.work && lane == 0 && bytes) atomicAdd(&v.work[W_Q_W], bytes);
}

}  // namespace

void launch_query_unw(const IndexView &v0, uint64_t k, const uint32_t *a, const uint32_t *b, uint8_t *out,
                      cudaStream_t s)
{
    if (!k) return;
    IndexView v = v0;
    v.work = work_counters();
    const unsigned block = 256;
    const unsigned grid = grid_for(k * 32, block, 152u * 64u);
    PADO_LAUNCH("query_unw_kernel", s,
                query_unw_kernel<<<grid, block, 0, s>>>(v, k, a, b, out));
}

void launch_query_w(const IndexView &v0, uint64_t k, const uint32_t *a, const uint32_t *b, int16_t *out,
                    cudaStream_t s)
{
    if (!k) return;
    IndexView v = v0;
    v.work = work_counters();
    const unsigned block = 256;
    const unsigned grid = grid_for(k * 32, block, 152u * 64u);
    PADO_LAUNCH("query_w_kernel", s,
                query_w_kernel<<<grid, block, 0, s>>>(v, k, a, b, out));
}

}  // namespace pado
