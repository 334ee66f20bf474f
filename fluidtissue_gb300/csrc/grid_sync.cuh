// Software grid barrier for persistent cooperative launches (internal).
//
// Counter + generation word.  The last block to arrive resets the counter and
// advances the generation; the others wait on the generation for at most
// `limit_ns` nanoseconds of the GPU's global timer (a runtime field, set by the
// host), after which they record an error and leave.  A waiting block also
// leaves as soon as another block has recorded one, so after a failure every
// block is out within one limit: no wait is unbounded.  All blocks must be
// co-resident (cooperative launch).
//
// Failure-detection tests: with `absent_block` >= 0 that block leaves at its
// first barrier without arriving (a block that dies between phases); the
// others' waits run out, the error is recorded and the launch returns.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace fts {

struct BarrierState {
    // reset to zero before every launch (the first kBarrierResetBytes bytes)
    unsigned count;
    unsigned gen;
    int active;
    int pad;
    // 1: a wait ran out; cleared by the host at the start of a solve, so a
    // failure in any launch of the solve stays visible (and makes the later
    // launches of the same solve return at once)
    int error;
    // configuration, kept across launches and written by the host
    int absent_block;             // -1, or the block that never arrives (tests)
    unsigned long long limit_ns;  // longest wait at one barrier
};

constexpr size_t kBarrierResetBytes = offsetof(BarrierState, error);
constexpr size_t kBarrierErrorOffset = offsetof(BarrierState, error);
constexpr unsigned long long kDefaultBarrierLimitNs = 2000000000ull;  // 2 s

inline BarrierState barrier_config(unsigned long long limit_ns, int absent_block) {
    BarrierState b = {};
    b.limit_ns = limit_ns;
    b.absent_block = absent_block;
    return b;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Returns false once any block has timed out at a barrier (and always for the
// absent block of a failure-detection test).
__device__ __forceinline__ bool grid_barrier(BarrierState* b) {
    __shared__ int s_leave;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_leave = 0;
        if ((int)blockIdx.x == b->absent_block) {
            s_leave = 1;  // leaves without arriving
        } else {
            volatile unsigned* vgen = &b->gen;
            volatile int* verr = &b->error;
            const unsigned g = *vgen;
            __threadfence();
            if (atomicAdd(&b->count, 1u) == gridDim.x - 1) {
                b->count = 0;
                __threadfence();
                atomicAdd(&b->gen, 1u);
            } else {
                const unsigned long long limit = b->limit_ns;
                const unsigned long long t0 = global_ns();
                while (*vgen == g) {
                    if (*verr) break;  // another block already gave up
                    if (global_ns() - t0 > limit) {
                        atomicOr(&b->error, 1);
                        break;
                    }
                    __nanosleep(64);
                }
            }
            __threadfence();
        }
    }
    __syncthreads();
    return s_leave == 0 && *((volatile int*)&b->error) == 0;
}

}  // namespace fts
