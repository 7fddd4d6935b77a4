// grid_sync.cuh -- the bounded software grid barrier of the batched heat
// kernels' cooperative launches (every block co-resident).
#pragma once

#include "tam_device.cuh"
#include "tam_kernels.h"

namespace tam {
namespace {

constexpr long long BARRIER_CYCLES = 4000000000ll;  // ~2 s at 2 GHz

// Bounded grid-wide barrier for co-resident blocks.  Returns false (for the
// whole block) once any block has flagged a time-out.
__device__ bool grid_barrier(BatchSync *g, unsigned nblocks, unsigned *err)
{
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        volatile unsigned *gen = &g->gen;
        volatile unsigned *abort_flag = &g->abort;
        const unsigned my = *gen;
        __threadfence();
        if (atomicAdd(&g->count, 1u) == nblocks - 1) {
            g->count = 0;
            __threadfence();
            atomicAdd(&g->gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == my) {
                if (*abort_flag) {
                    ok = 0;
                    break;
                }
                if (clock64() - t0 > BARRIER_CYCLES) {
                    atomicOr(err, (unsigned)DEVERR_SYNC_TIMEOUT);
                    atomicExch(&g->abort, 1u);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        if (*abort_flag) ok = 0;
    }
    return __syncthreads_and(ok) != 0;
}

}  // namespace
}  // namespace tam
