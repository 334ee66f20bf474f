// Deterministic grid-wide sums: warp shuffles, then shared memory across the
// warps of a block, then one partial per block; the last block to arrive (an
// atomic ticket) adds the partials in a fixed order and runs the caller's
// finaliser.  The result does not depend on block scheduling.
#pragma once

#include "fts_device.cuh"

namespace fts {

template <int NV>
__device__ __forceinline__ void warp_sum(double (&v)[NV]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// Block sum; the total is valid in thread 0.  Uses 32*NV doubles of shared.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double sh[NV][32];
    warp_sum<NV>(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k][wid] = v[k];
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = lane < nw ? sh[k][lane] : 0.0;
        warp_sum<NV>(v);
    }
}

// Contributes this block's v[] to a grid-wide sum.  Returns true in every
// thread of the last block, where tot[] (thread 0 only) holds the totals.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], const Reduction& red,
                                         double (&tot)[NV]) {
    __shared__ bool am_last;
    block_sum<NV>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) red.partials[k * kMaxPartials + blockIdx.x] = v[k];
        __threadfence();
        unsigned t = atomicAdd(red.ticket, 1u);
        am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&red.partials[k * kMaxPartials + i]);
    block_sum<NV>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) tot[k] = acc[k];
        *red.ticket = 0u;
    }
    return true;
}

// Ticket only (no sum): true in the last block to finish.
__device__ __forceinline__ bool last_block(const Reduction& red) {
    __shared__ bool am_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(red.ticket, 1u);
        am_last = (t == gridDim.x - 1);
        if (am_last) *red.ticket = 0u;
    }
    __syncthreads();
    return am_last;
}

}  // namespace fts
