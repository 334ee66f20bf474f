// Software grid barrier for persistent cooperative launches (internal).
//
// Counter + generation word.  The last block to arrive resets the counter and
// advances the generation; the others spin on the generation with a bounded
// number of 64 ns back-offs, after which they record an error and go on (no
// unbounded wait).  All blocks must be co-resident (cooperative launch).
#pragma once

#include <cuda_runtime.h>

namespace fts {

struct BarrierState {
    unsigned count;
    unsigned gen;
    int error;
    int active;
};

constexpr long long kSpinLimit = 1LL << 26;  // ~ seconds with the 64 ns back-off

// Returns false once any block has timed out at a barrier.
__device__ __forceinline__ bool grid_barrier(BarrierState* b) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &b->gen;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
            b->count = 0;
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (++spins > kSpinLimit) {
                    atomicOr(&b->error, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *((volatile int*)&b->error) == 0;
}

}  // namespace fts
