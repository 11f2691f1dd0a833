// grid_barrier.cuh -- bounded grid-wide barrier for the persistent
// cooperative loops (unweighted one-graph and many-graph labeling, weighted
// labeling).
#pragma once

#include "pado_internal.cuh"

namespace pado {
namespace {

// ---------------------------------------------------------------------------
// Grid-wide barrier for persistent cooperative launches.  The spin is bounded:
// after BARRIER_TIMEOUT_NS a block records ST_BARRIER_TIMEOUT and the barrier
// returns false, so a logic error can never leave the GPU spinning.
// ---------------------------------------------------------------------------
constexpr unsigned long long BARRIER_TIMEOUT_NS = 4000000000ull;
constexpr uint32_t ST_BARRIER_TIMEOUT = 8u;

// Arrivals are counted per group of BAR_GROUP blocks (each group counter on
// its own 128-byte line); the last arriver of a group bumps the top counter,
// and the last group releases everyone by advancing `gen`.  That keeps the
// serialised atomics on any one address to ~BAR_GROUP instead of the grid size.
constexpr uint32_t BAR_GROUP = 32;
constexpr uint32_t BAR_MAX_GROUPS = 64;   // grids up to 2048 blocks
struct GridBar {
    uint32_t gen, top, pad[30];
    uint32_t grp[BAR_MAX_GROUPS][32];
};

__device__ __forceinline__ uint32_t vload(const uint32_t *p) { return *(const volatile uint32_t *)p; }

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Returns false (in every thread of the block) if the wait timed out
// (after timeout_ns; the self-test passes a short limit).
__device__ bool grid_barrier(GridBar *bar, uint32_t *status, unsigned long long timeout_ns = BARRIER_TIMEOUT_NS)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t *gen = &bar->gen;
        const uint32_t g = *gen;
        __threadfence();
        const uint32_t grp = blockIdx.x / BAR_GROUP;
        const uint32_t ngrp = (gridDim.x + BAR_GROUP - 1) / BAR_GROUP;
        const uint32_t gsize = min(BAR_GROUP, gridDim.x - grp * BAR_GROUP);
        int good = 1;
        bool last = false;
        if (atomicAdd(&bar->grp[grp][0], 1u) + 1u == gsize) {
            atomicExch(&bar->grp[grp][0], 0u);
            if (atomicAdd(&bar->top, 1u) + 1u == ngrp) {
                atomicExch(&bar->top, 0u);
                last = true;
            }
        }
        if (last) {
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            const unsigned long long t0 = gtimer();
            while (*gen == g) {
                __nanosleep(20);
                if (gtimer() - t0 > timeout_ns) {
                    atomicOr(status, ST_BARRIER_TIMEOUT);
                    good = 0;
                    break;
                }
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

}  // namespace
}  // namespace pado
