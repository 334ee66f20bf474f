// The FP32 lattice half-stencil operator (internal), shared by the single-solve
// Krylov kernels (krylov.cu) and the batched persistent kernel (batch.cu).
#pragma once

#include "fts_device.cuh"
#include "mg_device.cuh"

namespace fts {

// Lattice half stencil: row r of node v's block towards direction d (0 = self,
// 1..7 positive Kuhn directions) is one float4 at lat_idx(d, r, v); tiles of 32
// nodes, so a warp's load of one (d, r) is 512 contiguous bytes.
__device__ __forceinline__ int64_t lat_idx(int d, int r, int64_t v) {
    return ((v >> 5) * 32 + d * 4 + r) * 32 + (v & 31);
}

// (S x)_v from the half stencil: own blocks towards v + d, and the blocks of
// the neighbours v - d towards v, transposed (S is symmetric).  `wadd` is added
// to the pressure component of every x read (the lazily applied rank-one term).
__device__ __forceinline__ float4 lat_row(int n, int64_t v64, const float4* __restrict__ L,
                                          const V4<float>* __restrict__ X, float wadd) {
    const int v = (int)v64;
    const int nn = n * n;
    const int k = v / nn;
    const int rem = v - k * nn;
    const int j = rem / n;
    const int i = rem - j * n;
    const bool inner = i > 0 && j > 0 && k > 0 && i < n - 1 && j < n - 1 && k < n - 1;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int d = 0; d < 8; ++d) {
        const int w = inner ? v + off_x(d) + n * off_y(d) + nn * off_z(d) : nbr(i, j, k, d, n);
        if (w < 0) continue;
        const V4<float> xv = X[w];
        const float x3 = xv.w + wadd;
        const float4 b0 = __ldg(L + lat_idx(d, 0, v64)), b1 = __ldg(L + lat_idx(d, 1, v64)),
                     b2 = __ldg(L + lat_idx(d, 2, v64)), b3 = __ldg(L + lat_idx(d, 3, v64));
        a0 = fmaf(b0.x, xv.x, fmaf(b0.y, xv.y, fmaf(b0.z, xv.z, fmaf(b0.w, x3, a0))));
        a1 = fmaf(b1.x, xv.x, fmaf(b1.y, xv.y, fmaf(b1.z, xv.z, fmaf(b1.w, x3, a1))));
        a2 = fmaf(b2.x, xv.x, fmaf(b2.y, xv.y, fmaf(b2.z, xv.z, fmaf(b2.w, x3, a2))));
        a3 = fmaf(b3.x, xv.x, fmaf(b3.y, xv.y, fmaf(b3.z, xv.z, fmaf(b3.w, x3, a3))));
    }
#pragma unroll
    for (int d = 1; d < 8; ++d) {
        const int w = inner ? v - off_x(d) - n * off_y(d) - nn * off_z(d) : nbr(i, j, k, d + 7, n);
        if (w < 0) continue;
        const V4<float> xv = X[w];
        const float x3 = xv.w + wadd;
        const int64_t w64 = w;
        const float4 b0 = __ldg(L + lat_idx(d, 0, w64)), b1 = __ldg(L + lat_idx(d, 1, w64)),
                     b2 = __ldg(L + lat_idx(d, 2, w64)), b3 = __ldg(L + lat_idx(d, 3, w64));
        a0 = fmaf(b0.x, xv.x, fmaf(b1.x, xv.y, fmaf(b2.x, xv.z, fmaf(b3.x, x3, a0))));
        a1 = fmaf(b0.y, xv.x, fmaf(b1.y, xv.y, fmaf(b2.y, xv.z, fmaf(b3.y, x3, a1))));
        a2 = fmaf(b0.z, xv.x, fmaf(b1.z, xv.y, fmaf(b2.z, xv.z, fmaf(b3.z, x3, a2))));
        a3 = fmaf(b0.w, xv.x, fmaf(b1.w, xv.y, fmaf(b2.w, xv.z, fmaf(b3.w, x3, a3))));
    }
    return make_float4(a0, a1, a2, a3);
}

}  // namespace fts
