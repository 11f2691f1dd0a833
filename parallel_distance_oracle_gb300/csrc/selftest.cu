// selftest.cu -- device-side failure detection, checked without a fault.
//
// The persistent labeling loops synchronise their blocks with a bounded grid
// barrier (grid_barrier.cuh): a block that waits longer than the limit records
// ST_BARRIER_TIMEOUT and returns, and the host turns the status into
// PADO_E_TIMEOUT.  pado_selftest_barrier runs that barrier in a small
// cooperative launch in which one chosen block never arrives, with a short
// limit, so a test can see the wait run out, every block return and the
// status reach the host -- the same path a stuck labeling loop would take.

#include "grid_barrier.cuh"

namespace pado {
namespace {

// Every block except `absent` waits at the barrier (at most timeout_ns);
// each block that returns counts itself.
__global__ void barrier_selftest_kernel(GridBar *bar, uint32_t *status, uint32_t absent,
                                        unsigned long long timeout_ns, uint32_t *returned)
{
    if (blockIdx.x != absent) grid_barrier(bar, status, timeout_ns);
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(returned, 1u);
}

}  // namespace
}  // namespace pado

extern "C" {

int pado_selftest_barrier(uint32_t blocks, uint32_t absent_block, uint64_t timeout_ns, uint32_t *blocks_returned)
{
    using namespace pado;
    if (blocks == 0 || blocks > 152 || !blocks_returned) return set_error(PADO_E_ARG, "blocks must be in [1, 152]");
    if (timeout_ns == 0 || timeout_ns > 1000000000ull) return set_error(PADO_E_ARG, "timeout must be in (0, 1 s]");
    try {
        DBuf<GridBar> bar(1);
        DBuf<uint32_t> word(2);  // status, blocks returned
        bar.fill_bytes(0, 0);
        word.fill_bytes(0, 0);
        uint32_t *status = word.p, *ret = word.p + 1;
        unsigned long long tns = timeout_ns;
        GridBar *bp = bar.p;
        void *args[] = {&bp, &status, &absent_block, &tns, &ret};
        PADO_LAUNCH("barrier_selftest_kernel", 0,
                    PADO_CUDA(cudaLaunchCooperativeKernel((const void *)barrier_selftest_kernel, blocks, 64, args, 0, 0)));
        uint32_t h[2] = {0, 0};
        PADO_CUDA(cudaMemcpy(h, word.p, sizeof(h), cudaMemcpyDeviceToHost));
        *blocks_returned = h[1];
        if (h[0] & ST_BARRIER_TIMEOUT) return set_error(PADO_E_TIMEOUT, "grid barrier timed out (self-test)");
    } catch (const Error &e) {
        return set_error(e.code, e.what());
    }
    return PADO_OK;
}

}  // extern "C"
