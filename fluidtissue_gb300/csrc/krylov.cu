// Block-sparse operator application and preconditioned MINRES (Paige &
// Saunders 1975) on the symmetric form of the stabilised Stokes system, in FP64
// or FP32.  One MINRES iteration is three kernels:
//   A: q = S v (v = y / beta) fused with the dot products v.q and v.r1
//   B: Lanczos update r_new = q - (beta/oldb) r1 - (alpha/beta) r2, the
//      block-diagonal preconditioner y = P^-1 r_new and the dot r_new.y
//   C: w_new = (v - oldeps w_prev - delta w_cur) / gamma, x += phi w_new
// The scalar recurrences run in the last block of A and B (a grid ticket), so
// the iteration never waits on the host; the host polls the stop flag every few
// iterations.  Dot products accumulate in FP64 in both precisions.
//
// The reference solves the same system with Eigen's un-preconditioned BiCGSTAB
// (src/growth/Flow.hpp:62, Flow.cpp:266); the stopping quantity is the same
// relative residual ||b - A x|| / ||b||, checked in FP64 by the outer loop.
#include <cfloat>
#include <cmath>

#include "fts_device.cuh"
#include "lat_device.cuh"
#include "mg.cuh"
#include "mg_device.cuh"
#include "pmg_device.cuh"
#include "reduce.cuh"

namespace fts {

template <typename T>
__device__ __forceinline__ T bsr_row_dot(const T* __restrict__ A, const int32_t* __restrict__ cols,
                                         int32_t k0, int32_t k1, int r,
                                         const V4<T>* __restrict__ x) {
    T acc = T(0);
    for (int32_t k = k0; k < k1; ++k) {
        const int32_t j = __ldg(cols + k);
        const V4<T> a = *reinterpret_cast<const V4<T>*>(A + (int64_t)k * 16 + r * 4);
        const V4<T> xj = x[j];
        acc = fma(a.x, xj.x, acc);
        acc = fma(a.y, xj.y, acc);
        acc = fma(a.z, xj.z, acc);
        acc = fma(a.w, xj.w, acc);
    }
    return acc;
}

// ---------------------------------------------------------------------------
// Plain operator application (tests / inspection): out = S in.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_apply(int64_t np, const int32_t* __restrict__ rowptr,
                        const int32_t* __restrict__ cols, const T* __restrict__ A,
                        const V4<T>* __restrict__ in, T* __restrict__ out) {
    const int r = threadIdx.x & 3;
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 2; row < np;
         row += ((int64_t)gridDim.x * blockDim.x) >> 2) {
        out[row * 4 + r] = bsr_row_dot<T>(A, cols, rowptr[row], rowptr[row + 1], r, in);
    }
}

__global__ void k_cast_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void k_cast_f2d(int64_t n, const float* __restrict__ a, double* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

__global__ void k_apply_ell(int64_t np, int64_t nslices, const int32_t* __restrict__ ell_ptr,
                            const int32_t* __restrict__ ell_col, const float* __restrict__ ell_val,
                            const V4<float>* __restrict__ in, float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int r = lane & 3;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; sl < nslices;
         sl += warps) {
        const int32_t p0 = ell_ptr[sl];
        const int32_t kmax = (ell_ptr[sl + 1] - p0) >> 3;
        float ax = 0.f;
        for (int32_t k = 0; k < kmax; ++k) {
            const int64_t slot = (int64_t)p0 + (lane >> 2) + 8 * k;
            const int32_t j = ell_col[slot];
            const float4 a = reinterpret_cast<const float4*>(ell_val)[slot * 4 + r];
            const V4<float> xj = in[j];
            ax = fmaf(a.x, xj.x, ax);
            ax = fmaf(a.y, xj.y, ax);
            ax = fmaf(a.z, xj.z, ax);
            ax = fmaf(a.w, xj.w, ax);
        }
        const int64_t row = 8 * sl + (lane >> 2);
        if (row < np) out[row * 4 + r] = ax;
    }
}

__global__ void k_apply_lat(int n, int64_t np, const float4* __restrict__ L,
                            const V4<float>* __restrict__ in, float4* __restrict__ out) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x)
        out[v] = lat_row(n, v, L, in, 0.f);
}

void launch_apply(Ctx& c, int precision, const V4<double>* in, V4<double>* out) {
    int grid = grid_for(c, c.np * 4);
    if (precision == FTS_PREC_MIXED) {
        if ((c.use_lat && !c.lat_val) || (!c.use_lat && c.use_ell && !c.ell_val) ||
            (!c.use_lat && !c.use_ell && !c.A32))
            throw CudaError(cudaErrorInvalidValue, "FP32 operator copy not built", __FILE__,
                            __LINE__);
        k_cast_d2f<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(
            c.np * 4, reinterpret_cast<const double*>(in), reinterpret_cast<float*>(c.w32.q));
        if (c.use_lat)
            k_apply_lat<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
                c.topo.lattice_n, c.np, reinterpret_cast<const float4*>(c.lat_val), c.w32.q,
                reinterpret_cast<float4*>(c.w32.r0));
        else if (c.use_ell)
            k_apply_ell<<<grid_for(c, c.nslices * 32), kThreads, 0, c.stream>>>(
                c.np, c.nslices, c.ell_ptr, c.ell_col, c.ell_val, c.w32.q,
                reinterpret_cast<float*>(c.w32.r0));
        else
            k_apply<float><<<grid, kThreads, 0, c.stream>>>(c.np, c.rowptr, c.cols, c.A32,
                                                            c.w32.q,
                                                            reinterpret_cast<float*>(c.w32.r0));
        k_cast_f2d<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(
            c.np * 4, reinterpret_cast<const float*>(c.w32.r0), reinterpret_cast<double*>(out));
    } else {
        k_apply<double><<<grid, kThreads, 0, c.stream>>>(c.np, c.rowptr, c.cols, c.A64, in,
                                                         reinterpret_cast<double*>(out));
    }
    FTS_CUDA(cudaGetLastError());
    c.launches += precision == FTS_PREC_MIXED ? 3 : 1;
}

// ---------------------------------------------------------------------------
// Outer residual (FP64): r = b - S x, ||r||^2, ||b||^2.
// ---------------------------------------------------------------------------
__global__ void k_residual64(int64_t np, const int32_t* __restrict__ rowptr,
                             const int32_t* __restrict__ cols, const double* __restrict__ A,
                             const V4<double>* __restrict__ x, const V4<double>* __restrict__ b,
                             double* __restrict__ r, Reduction red, OuterScalars* os) {
    const int rr = threadIdx.x & 3;
    double acc[2] = {0.0, 0.0};
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 2; row < np;
         row += ((int64_t)gridDim.x * blockDim.x) >> 2) {
        double ax = bsr_row_dot<double>(A, cols, rowptr[row], rowptr[row + 1], rr, x);
        double bv = reinterpret_cast<const double*>(b)[row * 4 + rr];
        double v = bv - ax;
        r[row * 4 + rr] = v;
        acc[0] += v * v;
        acc[1] += bv * bv;
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        os->rr = tot[0];
        os->bb = tot[1];
        os->scale = tot[0] > 0.0 ? 1.0 / sqrt(tot[0]) : 0.0;
        os->nonfinite = isfinite(tot[0]) ? 0 : 1;
    }
}

// The same from the FP64 lattice half stencil, one thread per node.
__global__ void __launch_bounds__(kThreads)
k_residual64_lat(int n, int64_t np, const double2* __restrict__ L,
                 const V4<double>* __restrict__ x, const V4<double>* __restrict__ b,
                 V4<double>* __restrict__ r, Reduction red, OuterScalars* os) {
    double acc[2] = {0.0, 0.0};
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x) {
        const int vi = (int)v;
        const int k = vi / (n * n), j = (vi / n) % n, i = vi % n;
        double a[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < 8; ++d) {  // own blocks: row r . x_w
            const int w = nbr(i, j, k, d, n);
            if (w < 0) continue;
            const V4<double> xw = x[w];
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const double2 u = L[lat64_idx(d, rr, 0, v)], s2 = L[lat64_idx(d, rr, 1, v)];
                a[rr] += u.x * xw.x + u.y * xw.y + s2.x * xw.z + s2.y * xw.w;
            }
        }
#pragma unroll
        for (int d = 1; d < 8; ++d) {  // the neighbour's block towards v, transposed
            const int w = nbr(i, j, k, d + 7, n);
            if (w < 0) continue;
            const V4<double> xw = x[w];
            const double xr[4] = {xw.x, xw.y, xw.z, xw.w};
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const double2 u = L[lat64_idx(d, rr, 0, w)], s2 = L[lat64_idx(d, rr, 1, w)];
                a[0] += u.x * xr[rr];
                a[1] += u.y * xr[rr];
                a[2] += s2.x * xr[rr];
                a[3] += s2.y * xr[rr];
            }
        }
        const V4<double> bv = b[v];
        V4<double> o;
        o.x = bv.x - a[0];
        o.y = bv.y - a[1];
        o.z = bv.z - a[2];
        o.w = bv.w - a[3];
        r[v] = o;
        acc[0] += o.x * o.x + o.y * o.y + o.z * o.z + o.w * o.w;
        acc[1] += bv.x * bv.x + bv.y * bv.y + bv.z * bv.z + bv.w * bv.w;
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        os->rr = tot[0];
        os->bb = tot[1];
        os->scale = tot[0] > 0.0 ? 1.0 / sqrt(tot[0]) : 0.0;
        os->nonfinite = isfinite(tot[0]) ? 0 : 1;
    }
}

void launch_residual64(Ctx& c) {
    if (c.matfree) {
        launch_mf_residual64(c);
        return;
    }
    if (c.use_lat64) {
        k_residual64_lat<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
            c.topo.lattice_n, c.np, c.lat64, c.x, c.b, c.r, c.red, c.os);
        FTS_CUDA(cudaGetLastError());
        c.launches += 1;
        return;
    }
    k_residual64<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(
        c.np, c.rowptr, c.cols, c.A64, c.x, c.b, reinterpret_cast<double*>(c.r), c.red, c.os);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// ---------------------------------------------------------------------------
// MINRES kernels
//
// Preconditioner P (SPD, block diagonal): velocity block = node 3x3 block
// Jacobi or one multigrid V-cycle (mg.cu); pressure block = diag(alpha D +
// eps M + lumped mass/mu)^-1 plus the rank-one term crank * 1 1^T with
// crank = 1/(eps * volume), which lifts the constant pressure mode (eigenvalue
// ~eps of the Schur complement) to ~1.  The rank-one part of y = P^-1 r is kept
// as a scalar ycorr[buffer] added to the pressure component wherever y is
// read, so applying P needs no extra pass over memory.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void pc_jacobi(const T* __restrict__ pc, int64_t i, const V4<T>& v,
                                          V4<T>& z) {
    const V4<T> p0 = *reinterpret_cast<const V4<T>*>(pc + 8 * i);
    const V4<T> p1 = *reinterpret_cast<const V4<T>*>(pc + 8 * i + 4);
    z.x = p0.x * v.x + p0.y * v.y + p0.z * v.z;
    z.y = p0.y * v.x + p0.w * v.y + p1.x * v.z;
    z.z = p0.z * v.x + p1.x * v.y + p1.y * v.z;
    z.w = p1.z * v.w;
}

__global__ void k_minres_reset(MinresScalars* s, double rtol, long long maxit, double crank) {
    s->rtol = rtol;
    s->maxit = maxit;
    s->crank = crank;
    s->iters = 0;
    s->stop = 0;
    s->c_pending = 0;
    s->status = 0;
    s->ycorr[0] = s->ycorr[1] = 0.0;
}

// beta^2 of a new Lanczos vector is known: initialise (init) or run the
// Givens step of the QR factorisation and the convergence test.
__device__ void finalize_beta(MinresScalars* s, double beta2, bool init) {
    const bool finite = isfinite(beta2);
    const double beta = beta2 > 0.0 ? sqrt(beta2) : 0.0;
    if (init) {
        s->beta1 = beta;
        s->beta = beta;
        s->oldb = 0.0;
        s->alfa = 0.0;
        s->dbar = 0.0;
        s->epsln = 0.0;
        s->oldeps = 0.0;
        s->delta = 0.0;
        s->gamma = 1.0;
        s->phi = 0.0;
        s->phibar = beta;
        s->cs = -1.0;
        s->sn = 0.0;
        s->target = s->rtol * beta;
        s->status = finite ? 0 : 2;
        s->stop = (!(beta > 0.0) || !finite) ? 1 : 0;
        return;
    }
    const double alfa = s->alfa;
    s->oldb = s->beta;
    s->beta = beta;
    s->oldeps = s->epsln;
    const double delta = s->cs * s->dbar + s->sn * alfa;
    const double gbar = s->sn * s->dbar - s->cs * alfa;
    s->epsln = s->sn * beta;
    s->dbar = -s->cs * beta;
    double gamma = sqrt(gbar * gbar + beta * beta);
    if (gamma < DBL_MIN) gamma = DBL_MIN;
    s->delta = delta;
    s->gamma = gamma;
    s->cs = gbar / gamma;
    s->sn = beta / gamma;
    s->phi = s->cs * s->phibar;
    s->phibar = s->sn * s->phibar;
    s->iters += 1;
    s->c_pending = 1;
    if (!finite || !isfinite(s->phibar)) {
        s->status = 2;
        s->stop = 1;
    } else if (s->phibar <= s->target || !(beta > 0.0)) {
        s->stop = 1;
    } else if (s->iters >= s->maxit) {
        s->status = 1;
        s->stop = 1;
    }
}

// A: q = S v with v = (y + ycorr e_p) / beta; partial dots v.q and v.r1.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_minres_A(int64_t np, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
           const T* __restrict__ A, const V4<T>* __restrict__ Y, int ybuf,
           const V4<T>* __restrict__ R1, T* __restrict__ q, Reduction red, MinresScalars* s) {
    pdl_wait();
    if (s->stop) return;
    const double invb = 1.0 / s->beta;
    const T tinv = (T)invb;
    const T wadd = (T)s->ycorr[ybuf];
    const int r = threadIdx.x & 3;
    double acc[2] = {0.0, 0.0};
    const T* y = reinterpret_cast<const T*>(Y);
    const T* r1 = reinterpret_cast<const T*>(R1);
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 2; row < np;
         row += ((int64_t)gridDim.x * blockDim.x) >> 2) {
        T ax = T(0);
        const int32_t k1 = rowptr[row + 1];
        for (int32_t k = rowptr[row]; k < k1; ++k) {
            const int32_t j = __ldg(cols + k);
            const V4<T> a = *reinterpret_cast<const V4<T>*>(A + (int64_t)k * 16 + r * 4);
            const V4<T> xj = Y[j];
            ax = fma(a.x, xj.x, ax);
            ax = fma(a.y, xj.y, ax);
            ax = fma(a.z, xj.z, ax);
            ax = fma(a.w, xj.w + wadd, ax);
        }
        const T qv = ax * tinv;
        const int64_t e = row * 4 + r;
        q[e] = qv;
        const T ve = (y[e] + (r == 3 ? wadd : T(0))) * tinv;
        acc[0] += (double)(ve * qv);
        acc[1] += (double)(ve * r1[e]);
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
        s->alfa = tot[0] - c1 * tot[1];
    }
}

// A on the FP32 sliced-ELL copy: one warp per slice of 8 block rows, lane l =
// (row 8s + l/4, block row l%4); the k-th blocks of the slice are one
// contiguous 512-byte segment.
__global__ void __launch_bounds__(kThreads)
k_minres_A_ell(int64_t np, int64_t nslices, const int32_t* __restrict__ ell_ptr,
               const int32_t* __restrict__ ell_col, const float* __restrict__ ell_val,
               const V4<float>* __restrict__ Y, int ybuf, const V4<float>* __restrict__ R1,
               float* __restrict__ q, Reduction red, MinresScalars* s) {
    pdl_wait();
    if (s->stop) return;
    const float tinv = (float)(1.0 / s->beta);
    const float wadd = (float)s->ycorr[ybuf];
    const int lane = threadIdx.x & 31;
    const int r = lane & 3;
    const float* y = reinterpret_cast<const float*>(Y);
    const float* r1 = reinterpret_cast<const float*>(R1);
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double acc[2] = {0.0, 0.0};
    for (int64_t sl = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; sl < nslices;
         sl += warps) {
        const int32_t p0 = ell_ptr[sl];
        const int32_t kmax = (ell_ptr[sl + 1] - p0) >> 3;
        const int64_t slot0 = (int64_t)p0 + (lane >> 2);
        float ax = 0.f;
#pragma unroll 4
        for (int32_t k = 0; k < kmax; ++k) {
            const int64_t slot = slot0 + 8 * k;
            const int32_t j = __ldg(ell_col + slot);
            const float4 a = __ldg(reinterpret_cast<const float4*>(ell_val) + slot * 4 + r);
            const V4<float> xj = Y[j];
            ax = fmaf(a.x, xj.x, ax);
            ax = fmaf(a.y, xj.y, ax);
            ax = fmaf(a.z, xj.z, ax);
            ax = fmaf(a.w, xj.w + wadd, ax);
        }
        const int64_t row = 8 * sl + (lane >> 2);
        if (row < np) {
            const float qv = ax * tinv;
            const int64_t e = row * 4 + r;
            q[e] = qv;
            const float ve = (y[e] + (r == 3 ? wadd : 0.f)) * tinv;
            acc[0] += (double)(ve * qv);
            acc[1] += (double)(ve * r1[e]);
        }
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
        s->alfa = tot[0] - c1 * tot[1];
    }
}

// Kernel A on the lattice half stencil: thread per node.
__global__ void __launch_bounds__(kThreads)
k_minres_A_lat(int n, int64_t np, const float4* __restrict__ L, const V4<float>* __restrict__ Y,
               int ybuf, const V4<float>* __restrict__ R1, V4<float>* __restrict__ q,
               Reduction red, MinresScalars* s) {
    pdl_wait();
    if (s->stop) return;
    const float tinv = (float)(1.0 / s->beta);
    const float wadd = (float)s->ycorr[ybuf];
    double acc[2] = {0.0, 0.0};
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x) {
        const float4 a = lat_row(n, v, L, Y, wadd);
        V4<float> qv;
        qv.x = a.x * tinv;
        qv.y = a.y * tinv;
        qv.z = a.z * tinv;
        qv.w = a.w * tinv;
        q[v] = qv;
        const V4<float> yv = Y[v], r1 = R1[v];
        const float e0 = yv.x * tinv, e1 = yv.y * tinv, e2 = yv.z * tinv,
                    e3 = (yv.w + wadd) * tinv;
        // a node's four products summed in FP32, the node sums in FP64: one
        // conversion and one FP64 add per dot and node (GB300's FP64 pipe is
        // narrow; four of each per node kept it a third busy)
        acc[0] += (double)fmaf(e0, qv.x, fmaf(e1, qv.y, fmaf(e2, qv.z, e3 * qv.w)));
        acc[1] += (double)fmaf(e0, r1.x, fmaf(e1, r1.y, fmaf(e2, r1.z, e3 * r1.w)));
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
        s->alfa = tot[0] - c1 * tot[1];
    }
}

// Kernel A in FP64 on the FP64 lattice half stencil (lat64_idx), thread per
// node: the same half-stencil walk as the outer residual.
__global__ void __launch_bounds__(kThreads)
k_minres_A_lat64(int n, int64_t np, const double2* __restrict__ L,
                 const V4<double>* __restrict__ Y, int ybuf, const V4<double>* __restrict__ R1,
                 V4<double>* __restrict__ q, Reduction red, MinresScalars* s) {
    pdl_wait();
    if (s->stop) return;
    const double tinv = 1.0 / s->beta;
    const double wadd = s->ycorr[ybuf];
    double acc[2] = {0.0, 0.0};
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x) {
        const int vi = (int)v;
        const int k = vi / (n * n), j = (vi / n) % n, i = vi % n;
        double a[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < 8; ++d) {  // own blocks: row r . y_w
            const int w = nbr(i, j, k, d, n);
            if (w < 0) continue;
            const V4<double> yw = Y[w];
            const double y3 = yw.w + wadd;
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const double2 u = L[lat64_idx(d, rr, 0, v)], s2 = L[lat64_idx(d, rr, 1, v)];
                a[rr] = fma(u.x, yw.x, fma(u.y, yw.y, fma(s2.x, yw.z, fma(s2.y, y3, a[rr]))));
            }
        }
#pragma unroll
        for (int d = 1; d < 8; ++d) {  // the neighbour's block towards v, transposed
            const int w = nbr(i, j, k, d + 7, n);
            if (w < 0) continue;
            const V4<double> yw = Y[w];
            const double yr[4] = {yw.x, yw.y, yw.z, yw.w + wadd};
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const double2 u = L[lat64_idx(d, rr, 0, w)], s2 = L[lat64_idx(d, rr, 1, w)];
                a[0] = fma(u.x, yr[rr], a[0]);
                a[1] = fma(u.y, yr[rr], a[1]);
                a[2] = fma(s2.x, yr[rr], a[2]);
                a[3] = fma(s2.y, yr[rr], a[3]);
            }
        }
        V4<double> qv;
        qv.x = a[0] * tinv;
        qv.y = a[1] * tinv;
        qv.z = a[2] * tinv;
        qv.w = a[3] * tinv;
        q[v] = qv;
        const V4<double> yv = Y[v], r1 = R1[v];
        const double e0 = yv.x * tinv, e1 = yv.y * tinv, e2 = yv.z * tinv,
                     e3 = (yv.w + wadd) * tinv;
        acc[0] += e0 * qv.x + e1 * qv.y + e2 * qv.z + e3 * qv.w;
        acc[1] += e0 * r1.x + e1 * r1.y + e2 * r1.z + e3 * r1.w;
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
        s->alfa = tot[0] - c1 * tot[1];
    }
}

// Preconditioner stage 1.
//   init: n = r0 (written to Rn)      else: n = q - c1 R1 - c2 R2 (written to Rn = R1)
//   y.w = ip * n.w;  Jacobi: y.xyz = D3^-1 n.xyz;  multigrid: b0 = n.xyz (SoA)
//   pressure multigrid (pmg): y.w = 0 here, pressure b0 = n.w (stage 2 sets y.w)
// Jacobi finishes beta here; multigrid leaves sum(n.w) and n.w y.w for stage 2.
template <typename T, bool MGV>
__global__ void __launch_bounds__(kThreads)
k_minres_pc1(int64_t np, int init, const V4<T>* __restrict__ q, V4<T>* R1,
             const V4<T>* __restrict__ R2, V4<T>* Rn, const T* __restrict__ pc,
             V4<T>* __restrict__ Ynew, int ybuf, LevelView<T> L0, PView<T> P0, int pmg,
             Reduction red, MinresScalars* s) {
    pdl_wait();
    if (s->stop) return;
    T c1 = T(0), c2 = T(0);
    if (!init) {
        c1 = (T)(s->iters >= 1 ? s->beta / s->oldb : 0.0);
        c2 = (T)(s->alfa / s->beta);
    }
    double acc[3] = {0.0, 0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        V4<T> n;
        if (init) {
            n = R1[i];  // r0
        } else {
            const V4<T> qv = q[i], a = R1[i], b2 = R2[i];
            n.x = qv.x - c1 * a.x - c2 * b2.x;
            n.y = qv.y - c1 * a.y - c2 * b2.y;
            n.z = qv.z - c1 * a.z - c2 * b2.z;
            n.w = qv.w - c1 * a.w - c2 * b2.w;
        }
        Rn[i] = n;
        V4<T> z;
        if (MGV) {
            z.x = z.y = z.z = T(0);
            if (pmg) {
                z.w = T(0);
                P0.b[i] = n.w;
                pmg_first_dir<T>(P0, i, n.w);
            } else {
                z.w = pc[8 * i + 6] * n.w;
            }
            L0.b[i] = n.x;
            L0.b[np + i] = n.y;
            L0.b[2 * np + i] = n.z;
            const T bv[3] = {n.x, n.y, n.z};
            mg_first_dir<T>(L0, i, bv);
        } else {
            pc_jacobi<T>(pc, i, n, z);
            acc[2] += (double)(n.x * z.x + n.y * z.y + n.z * z.z);
        }
        // with both V-cycles stage 2 writes all of y: nothing to store here
        if (!(MGV && pmg)) {
            Ynew[i] = z;
            acc[1] += (double)(n.w * z.w);
        }
        acc[0] += (double)n.w;
    }
    double tot[3];
    if (grid_sum<3>(acc, red, tot) && threadIdx.x == 0) {
        if (MGV) {
            s->psum = tot[0];
            s->pdot = tot[1];
        } else {
            const double cr = s->crank;
            s->ycorr[ybuf] = cr * tot[0];
            finalize_beta(s, tot[2] + tot[1] + cr * tot[0] * tot[0], init != 0);
        }
    }
}

// Multigrid stage 2, fused with the V-cycle's last post-smoothing step on the
// finest level: y.xyz = the step's new x (not stored in the level), and with
// pmg y.w likewise from the pressure V-cycle; beta.  With degree-1 smoothing on
// a finest level (fine1 / pfine1) that step is the pointwise x + d_0.  (Running
// the pressure V-cycle's last step on its own stream instead, and reading its x
// here, made the solve slower: 224.7 -> 226.2 ms on ellipsoid129, the pressure
// stream then ends after the velocity one.)  FORM: how y.xyz is formed —
// kPc2Step the fused last Chebyshev step; kPc2Fine1 the pointwise x + d_0;
// kPc2Post the velocity V-cycle left out its degree-1 finest post-smoothing
// residual (kSkipPost), which runs here from the prolongated x:
// y.xyz = x + D^-1 (b - K x) / theta, nothing stored but y.  PFORM: y.w from
// stage 1's pressure diagonal (kPc2None), the pressure V-cycle's pointwise
// x + d_0 (kPc2Fine1) or its fused last step (kPc2Step).  Each form is its own
// kernel so that the pointwise ones keep few registers (one kernel for all
// held 168 registers and an eighth of the warps).
enum : int { kPc2Step = 0, kPc2Fine1 = 1, kPc2Post = 2, kPc2None = 3 };
template <typename T, int FORM, int PFORM>
__global__ void __launch_bounds__(kThreads, 4)
k_minres_pc2(LevelView<T> L0, int step, int mode, const T* __restrict__ din, PView<T> P0,
             int init, const V4<T>* __restrict__ Rn, V4<T>* __restrict__ Ynew, int ybuf,
             Reduction red, MinresScalars* s) {
    pdl_wait();
    if (s->stop) return;
    double acc[1] = {0.0};
    // the pressure V-cycle's last finest step (its own smoothing degree)
    constexpr int ps = kPSmooth - 1;
    constexpr int pmode = ps == 1 ? kStepAfterFirst : kStepRegular;
    const T* pdin = (ps & 1) ? P0.d0 : P0.d1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L0.N;
         i += (int64_t)gridDim.x * blockDim.x) {
        T xo[3];
        if (FORM == kPc2Post) {
            mg_post1_node<T>(L0, i, xo);
        } else if (FORM == kPc2Fine1) {  // degree-1 finest level: x + d_0
#pragma unroll
            for (int cc = 0; cc < 3; ++cc) xo[cc] = L0.x[cc * L0.N + i] + L0.d0[cc * L0.N + i];
        } else {
            mg_step_node<T>(L0, i, step, mode, din, nullptr, xo, false, false);
        }
        const V4<T> n = Rn[i];
        V4<T> z;
        z.x = xo[0];
        z.y = xo[1];
        z.z = xo[2];
        T dz = n.x * z.x + n.y * z.y + n.z * z.z;  // node sum in T, FP64 across nodes
        if (PFORM != kPc2None) {
            z.w = PFORM == kPc2Fine1 ? P0.x[i] + P0.d0[i]
                                     : pmg_step_node<T>(P0, i, ps, pmode, pdin, nullptr, false);
            dz += n.w * z.w;
        } else {
            z.w = Ynew[i].w;  // stage 1's pressure diagonal (its dot is in pdot)
        }
        Ynew[i] = z;
        acc[0] += (double)dz;
    }
    double tot[1];
    if (grid_sum<1>(acc, red, tot) && threadIdx.x == 0) {
        const double cr = s->crank;
        s->ycorr[ybuf] = cr * s->psum;
        finalize_beta(s, tot[0] + s->pdot + cr * s->psum * s->psum, init != 0);
    }
}

template <typename T>
using Pc2Kernel = void (*)(LevelView<T>, int, int, const T*, PView<T>, int, const V4<T>*,
                           V4<T>*, int, Reduction, MinresScalars*);

// The stage-2 kernel of a velocity form and a pressure form.
template <typename T>
static Pc2Kernel<T> pc2_kernel(int form, int pform) {
    static const Pc2Kernel<T> table[3][4] = {
        {k_minres_pc2<T, kPc2Step, kPc2Step>, k_minres_pc2<T, kPc2Step, kPc2Fine1>, nullptr,
         k_minres_pc2<T, kPc2Step, kPc2None>},
        {k_minres_pc2<T, kPc2Fine1, kPc2Step>, k_minres_pc2<T, kPc2Fine1, kPc2Fine1>, nullptr,
         k_minres_pc2<T, kPc2Fine1, kPc2None>},
        {k_minres_pc2<T, kPc2Post, kPc2Step>, k_minres_pc2<T, kPc2Post, kPc2Fine1>, nullptr,
         k_minres_pc2<T, kPc2Post, kPc2None>}};
    return table[form][pform];
}

// C: w_new = (v - oldeps w_prev - delta w_cur) / gamma (into w_prev), x += phi w_new.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_minres_C(int64_t np, const V4<T>* __restrict__ Yk, int ybuf, V4<T>* Wprev,
           const V4<T>* __restrict__ Wcur, V4<T>* __restrict__ X, Reduction red,
           MinresScalars* s) {
    pdl_wait();
    if (!s->c_pending) return;
    const T inv = (T)(1.0 / s->oldb);
    const T wadd = (T)s->ycorr[ybuf];
    const T oe = (T)s->oldeps, de = (T)s->delta, ig = (T)(1.0 / s->gamma), ph = (T)s->phi;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const V4<T> y = Yk[i], wp = Wprev[i], wc = Wcur[i];
        V4<T> w, xv = X[i];
        w.x = (y.x * inv - oe * wp.x - de * wc.x) * ig;
        w.y = (y.y * inv - oe * wp.y - de * wc.y) * ig;
        w.z = (y.z * inv - oe * wp.z - de * wc.z) * ig;
        w.w = ((y.w + wadd) * inv - oe * wp.w - de * wc.w) * ig;
        Wprev[i] = w;
        xv.x += ph * w.x;
        xv.y += ph * w.y;
        xv.z += ph * w.z;
        xv.w += ph * w.w;
        X[i] = xv;
    }
    if (last_block(red) && threadIdx.x == 0) s->c_pending = 0;
}

// The P2 velocity level as a LevelView (p2mg.cu).
template <typename T>
LevelView<T> p2_level_view(Ctx& c);

template <typename T>
static const T* op_of(const Ctx& c);
template <>
const double* op_of<double>(const Ctx& c) { return c.A64; }
template <>
const float* op_of<float>(const Ctx& c) { return c.A32; }
template <typename T>
static const T* pc_of(const Ctx& c);
template <>
const double* pc_of<double>(const Ctx& c) { return c.pc64; }
template <>
const float* pc_of<float>(const Ctx& c) { return c.pc32; }
template <typename T>
static KrylovWork<T>& work_of(Ctx& c);
template <>
KrylovWork<double>& work_of<double>(Ctx& c) { return c.w64; }
template <>
KrylovWork<float>& work_of<float>(Ctx& c) { return c.w32; }
template <typename T>
static MG<T>& mg_of(Ctx& c);
template <>
MG<double>& mg_of<double>(Ctx& c) { return c.mg64; }
template <>
MG<float>& mg_of<float>(Ctx& c) { return c.mg32; }
template <typename T>
static PMG<T>& pmg_of(Ctx& c);
template <>
PMG<double>& pmg_of<double>(Ctx& c) { return c.pmg64; }
template <>
PMG<float>& pmg_of<float>(Ctx& c) { return c.pmg32; }

// y = P^-1 n for the Lanczos vector in Rn (stage 1, V-cycle, stage 2).
template <typename T>
static void launch_pc(Ctx& c, bool use_mg, int init, const V4<T>* q, V4<T>* R1, const V4<T>* R2,
                      V4<T>* Rn, V4<T>* Ynew, int ybuf) {
    KrylovWork<T>& w = work_of<T>(c);
    const int gn = grid_for(c, c.np);
    const T* pc = pc_of<T>(c);
    if (use_mg) {
        MG<T>& mg = mg_of<T>(c);
        // P2-P1: the finest level is the P2 velocity level (degree-1 smoothing)
        const LevelView<T> L0 = c.p2 ? p2_level_view<T>(c) : level_view(mg, 0);
        const bool fine1 = c.p2 || mg_level_degree1(mg, 0);
        const bool pmg = c.use_pmg;
        const PView<T> P0 = pmg ? pview(pmg_of<T>(c), 0) : PView<T>{};
        pdl_launch(k_minres_pc1<T, true>, gn, kThreads, c.stream, c.np, init, q, R1, R2, Rn, pc, Ynew,
                                                             ybuf, L0, P0, pmg ? 1 : 0, c.red,
                                                             c.ms);
        if (pmg) {  // pressure V-cycle on the second stream, beside the velocity one
            FTS_CUDA(cudaEventRecord(c.ev_fork, c.stream));
            FTS_CUDA(cudaStreamWaitEvent(c.aux_stream, c.ev_fork, 0));
            pmg_vcycle<T>(c, pmg_of<T>(c), c.aux_stream, &c.ms->stop, true);
            FTS_CUDA(cudaEventRecord(c.ev_join, c.aux_stream));
        }
        // a degree-1 finest velocity level's post-smoothing residual runs in stage 2
        const bool post = !c.p2 && mg_level_degree1(mg, 0);
        if (c.p2) p2mg_vcycle<T>(c, &c.ms->stop);
        else mg_vcycle<T>(c, mg, &c.ms->stop, post ? kSkipPost : kSkipFinal);
        if (pmg) FTS_CUDA(cudaStreamWaitEvent(c.stream, c.ev_join, 0));
        // the last post-smoothing step: step kSmooth - 1 reads d0 when it is odd
        constexpr int s = kSmooth - 1;
        const int form = post ? kPc2Post : (fine1 ? kPc2Fine1 : kPc2Step);
        const int pform =
            !pmg ? kPc2None : (pmg_level_degree1(pmg_of<T>(c), 0) ? kPc2Fine1 : kPc2Step);
        pdl_launch(pc2_kernel<T>(form, pform), gn, kThreads, c.stream,
            L0, s, s == 1 ? kStepAfterFirst : kStepRegular, (s & 1) ? L0.d0 : L0.d1, P0,
            init, Rn, Ynew, ybuf, c.red, c.ms);
        c.launches += 2;
    } else {
        pdl_launch(k_minres_pc1<T, false>, gn, kThreads, c.stream, c.np, init, q, R1, R2, Rn, pc, Ynew,
                                                              ybuf, LevelView<T>{}, PView<T>{}, 0,
                                                              c.red, c.ms);
        c.launches += 1;
    }
    (void)w;
}

// Runs MINRES on S d = r0 (work.r0; for FP64 the outer residual c.r) from
// d = 0 until the preconditioned residual norm drops by rtol.  Returns the
// iteration count; *achieved = phibar / beta1, *status = scalar status.
template <typename T>
long long minres_inner(Ctx& c, double rtol, long long maxit, double* achieved, int* status) {
    KrylovWork<T>& w = work_of<T>(c);
    const T* A = op_of<T>(c);
    const int64_t np = c.np;
    const bool use_mg = c.use_mg;
    FTS_CUDA(cudaMemsetAsync(w.W[0], 0, np * sizeof(V4<T>), c.stream));
    FTS_CUDA(cudaMemsetAsync(w.W[1], 0, np * sizeof(V4<T>), c.stream));
    FTS_CUDA(cudaMemsetAsync(w.X, 0, np * sizeof(V4<T>), c.stream));
    FTS_CUDA(cudaMemsetAsync(w.R[1], 0, np * sizeof(V4<T>), c.stream));
    const int ge = grid_for(c, np * 4);
    const int gn = grid_for(c, np);
    k_minres_reset<<<1, 1, 0, c.stream>>>(c.ms, rtol, maxit, c.crank);
    c.launches += 1;
    // initial Lanczos vector r0 -> R[0], y = P^-1 r0 -> Y[0]
    launch_pc<T>(c, use_mg, 1, nullptr, const_cast<V4<T>*>(w.r0), nullptr, w.R[0], w.Y[0], 0);
    FTS_CUDA(cudaGetLastError());
    const bool timed = c.par.time_kernels != 0;
    if (timed && !c.tev_ready) {
        for (auto& e : c.tev) FTS_CUDA(cudaEventCreate(&e));
        c.tev_ready = true;
    }
    const int poll = use_mg ? (np > 200000 ? 4 : 16) : (np > 200000 ? 8 : 32);
    long long k = 0, done_before = 0;
    for (;;) {
        for (int u = 0; u < poll; ++u) {
            ++k;
            const int p = (int)(k & 1);       // r1 = R[p], r2 = R[1-p], new -> R[p]
            V4<T>* R1 = w.R[p];
            V4<T>* R2 = w.R[1 - p];
            const int yk = (int)((k - 1) & 1), yn = (int)(k & 1);
            V4<T>* Wprev = w.W[p];
            V4<T>* Wcur = w.W[1 - p];
            if (timed) FTS_CUDA(cudaEventRecord(c.tev[2 * u], c.stream));
            if (sizeof(T) == 4 && c.matfree)
                launch_mf_minres_A(c, reinterpret_cast<const V4<float>*>(w.Y[yk]), yk,
                                   reinterpret_cast<const V4<float>*>(R1),
                                   reinterpret_cast<V4<float>*>(w.q));
            else if (sizeof(T) == 4 && c.use_lat)
                pdl_launch(k_minres_A_lat, gn, kThreads, c.stream,
                    c.topo.lattice_n, np, reinterpret_cast<const float4*>(c.lat_val),
                    reinterpret_cast<const V4<float>*>(w.Y[yk]),
                    yk, reinterpret_cast<const V4<float>*>(R1), reinterpret_cast<V4<float>*>(w.q),
                    c.red, c.ms);
            else if (sizeof(T) == 8 && c.use_lat64)
                pdl_launch(k_minres_A_lat64, gn, kThreads, c.stream,
                    c.topo.lattice_n, np, c.lat64,
                    reinterpret_cast<const V4<double>*>(w.Y[yk]), yk,
                    reinterpret_cast<const V4<double>*>(R1), reinterpret_cast<V4<double>*>(w.q),
                    c.red, c.ms);
            else if (sizeof(T) == 4 && c.use_ell)
                pdl_launch(k_minres_A_ell, grid_for(c, c.nslices * 32), kThreads, c.stream,
                    np, c.nslices, c.ell_ptr, c.ell_col, c.ell_val,
                    reinterpret_cast<const V4<float>*>(w.Y[yk]), yk,
                    reinterpret_cast<const V4<float>*>(R1), reinterpret_cast<float*>(w.q),
                    c.red, c.ms);
            else
                pdl_launch(k_minres_A<T>, ge, kThreads, c.stream, np, c.rowptr, c.cols, A, w.Y[yk], yk,
                                                             R1, reinterpret_cast<T*>(w.q), c.red,
                                                             c.ms);
            if (timed) FTS_CUDA(cudaEventRecord(c.tev[2 * u + 1], c.stream));
            launch_pc<T>(c, use_mg, 0, w.q, R1, R2, R1, w.Y[yn], yn);
            pdl_launch(k_minres_C<T>, gn, kThreads, c.stream, np, w.Y[yk], yk, Wprev, Wcur, w.X, c.red,
                                                         c.ms);
            c.launches += 2;
        }
        FTS_CUDA(cudaGetLastError());
        FTS_CUDA(cudaMemcpyAsync(c.ms_host, c.ms, sizeof(MinresScalars), cudaMemcpyDeviceToHost,
                                 c.stream));
        FTS_CUDA(cudaStreamSynchronize(c.stream));
        // operator applications that did work in this chunk = completed iterations
        const long long ran = c.ms_host->iters - done_before;
        done_before = c.ms_host->iters;
        if (timed) {
            for (long long u = 0; u < ran && u < poll; ++u) {
                float ms = 0.f;
                FTS_CUDA(cudaEventElapsedTime(&ms, c.tev[2 * u], c.tev[2 * u + 1]));
                c.ms_spmv += ms;
            }
        }
        c.spmv_runs += ran;
        if (c.ms_host->stop) break;
    }
    const MinresScalars& S = *c.ms_host;
    *achieved = S.beta1 > 0.0 ? S.phibar / S.beta1 : 0.0;
    *status = S.status;
    return S.iters;
}

template long long minres_inner<double>(Ctx&, double, long long, double*, int*);
template long long minres_inner<float>(Ctx&, double, long long, double*, int*);

template <typename T>
void setup_preconditioner(Ctx& c) {
    if (c.use_mg && c.use_pmg && c.aux_stream) {
        // the pressure hierarchy's set-up on the second stream, under the
        // velocity hierarchy's (both read the assembled operator only)
        PMG<T>& pm = pmg_of<T>(c);
        pmg_build<T>(c, pm);
        FTS_CUDA(cudaEventRecord(c.ev_fork, c.stream));
        FTS_CUDA(cudaStreamWaitEvent(c.aux_stream, c.ev_fork, 0));
        pmg_setup_enqueue<T>(c, pm, c.aux_stream);
        mg_setup<T>(c, mg_of<T>(c));
        pmg_setup_finish<T>(c, pm, c.aux_stream);
        return;
    }
    if (c.use_mg && c.p2) p2mg_setup<T>(c);  // the P2 level first: its K2 feeds the P1 level
    if (c.use_mg) mg_setup<T>(c, mg_of<T>(c));
    if (c.use_pmg) pmg_setup<T>(c, pmg_of<T>(c));
}
template void setup_preconditioner<double>(Ctx&);
template void setup_preconditioner<float>(Ctx&);

// r0_32 = r * (1/||r||) (FP32 right-hand side of the inner solve).
__global__ void k_prepare_inner32(int64_t n, const double* __restrict__ r,
                                  const OuterScalars* __restrict__ os, float* __restrict__ r32) {
    const double sc = os->scale;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        r32[i] = (float)(r[i] * sc);
}

void launch_prepare_inner32(Ctx& c) {
    k_prepare_inner32<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(
        c.np * 4, reinterpret_cast<const double*>(c.r), c.os, reinterpret_cast<float*>(c.w32.r0));
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

__global__ void k_update_x64(int64_t n, const double* __restrict__ d, double* __restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] += d[i];
}

void launch_update_x64(Ctx& c) {
    k_update_x64<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(
        c.np * 4, reinterpret_cast<const double*>(c.w64.X), reinterpret_cast<double*>(c.x));
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

__global__ void k_update_x_from32(int64_t n, const float* __restrict__ d,
                                  const OuterScalars* __restrict__ os, double* __restrict__ x) {
    const double rn = os->scale > 0.0 ? 1.0 / os->scale : 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] += rn * (double)d[i];
}

void launch_update_x_from32(Ctx& c) {
    k_update_x_from32<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(
        c.np * 4, reinterpret_cast<const float*>(c.w32.X), c.os, reinterpret_cast<double*>(c.x));
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

}  // namespace fts
