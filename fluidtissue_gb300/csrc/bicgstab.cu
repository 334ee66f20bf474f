// The reference's solver on the GPU: un-preconditioned BiCGSTAB (van der
// Vorst 1992) on the reference's sign convention A = [K -B; B^T C] (the stored
// symmetric form with the pressure rows of every product negated), FP64,
// warm-started from x, stopping when the updated residual satisfies
// ||r|| <= tol ||b|| (Eigen's BiCGSTAB as configured by src/growth/Flow.hpp:62,
// Flow.cpp:77-82, :266-285).  When rho collapses relative to ||r0||^2 the
// shadow residual is reset to the true residual.
//
// Per iteration: p update, v = A p (+ r0.v), s = r - alpha v, t = A s (+ t.t,
// t.s), x/r update (+ r.r, r0.r); scalars advance in the last block.
#include <cfloat>
#include <cmath>

#include "fts_device.cuh"
#include "reduce.cuh"

namespace fts {

struct BicgScalars {
    double rho, rho_old, alpha, w, beta, rr, bb, r0n, tol2;
    long long iters, maxit;
    long long total;  // all iterations (iters restarts at 0 on the first restart, as Eigen)
    int stop, restart, status, nrestart;
};

__device__ __forceinline__ double bsr_row(const double* __restrict__ A,
                                          const int32_t* __restrict__ cols, int32_t k0,
                                          int32_t k1, int r, const V4<double>* __restrict__ x) {
    double acc = 0.0;
    for (int32_t k = k0; k < k1; ++k) {
        const int32_t j = __ldg(cols + k);
        const V4<double> a = *reinterpret_cast<const V4<double>*>(A + (int64_t)k * 16 + r * 4);
        const V4<double> xj = x[j];
        acc = fma(a.x, xj.x, acc);
        acc = fma(a.y, xj.y, acc);
        acc = fma(a.z, xj.z, acc);
        acc = fma(a.w, xj.w, acc);
    }
    return r == 3 ? -acc : acc;  // reference sign: pressure rows of S negated back
}

// r = b_ref - A x, r0 = r, ||r||^2, ||b||^2 (b_ref = b with pressure negated)
__global__ void k_bicg_init(int64_t np, const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ cols, const double* __restrict__ A,
                            const V4<double>* __restrict__ x, const double* __restrict__ b,
                            double* __restrict__ r, double* __restrict__ r0, int keep_rho,
                            double tol, long long maxit, Reduction red, BicgScalars* s) {
    const int rr = threadIdx.x & 3;
    double acc[2] = {0.0, 0.0};
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 2; row < np;
         row += ((int64_t)gridDim.x * blockDim.x) >> 2) {
        const int64_t e = row * 4 + rr;
        const double be = rr == 3 ? -b[e] : b[e];
        const double v = be - bsr_row(A, cols, rowptr[row], rowptr[row + 1], rr, x);
        r[e] = v;
        r0[e] = v;
        acc[0] += v * v;
        acc[1] += be * be;
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        s->rr = tot[0];
        s->bb = tot[1];
        s->r0n = tot[0];
        s->rho = tot[0];
        s->tol2 = tol * tol * tot[1];
        s->restart = 0;
        s->status = 0;
        if (!keep_rho) {
            s->rho_old = 1.0;
            s->alpha = 1.0;
            s->w = 1.0;
            s->iters = 0;
            s->total = 0;
            s->nrestart = 0;
            s->maxit = maxit;
        } else {
            s->nrestart += 1;
        }
        s->beta = (s->rho / s->rho_old) * (s->alpha / s->w);
        s->stop = (tot[1] == 0.0 || tot[0] <= s->tol2) ? 1 : 0;
    }
}

// p = r + beta (p - w v)
__global__ void k_bicg_p(int64_t n, const double* __restrict__ r, double* __restrict__ p,
                         const double* __restrict__ v, const BicgScalars* s) {
    if (s->stop || s->restart) return;
    const double be = s->beta, w = s->w;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        p[i] = r[i] + be * (p[i] - w * v[i]);
}

// y = A x (reference signs) and partial dots; mode 0: r0.y -> alpha;
// mode 1: y.y and y.s -> w
__global__ void k_bicg_spmv(int64_t np, const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ cols, const double* __restrict__ A,
                            const V4<double>* __restrict__ x, double* __restrict__ y,
                            const double* __restrict__ aux, int mode, Reduction red,
                            BicgScalars* s) {
    if (s->stop || s->restart) return;
    const int rr = threadIdx.x & 3;
    double acc[2] = {0.0, 0.0};
    const double* xs = reinterpret_cast<const double*>(x);
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 2; row < np;
         row += ((int64_t)gridDim.x * blockDim.x) >> 2) {
        const int64_t e = row * 4 + rr;
        const double v = bsr_row(A, cols, rowptr[row], rowptr[row + 1], rr, x);
        y[e] = v;
        if (mode == 0) {
            acc[0] += aux[e] * v;
        } else {
            acc[0] += v * v;
            acc[1] += v * xs[e];
        }
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        if (mode == 0) s->alpha = s->rho / tot[0];
        else s->w = tot[0] > 0.0 ? tot[1] / tot[0] : 0.0;
    }
}

// s = r - alpha v
__global__ void k_bicg_s(int64_t n, const double* __restrict__ r, const double* __restrict__ v,
                         double* __restrict__ sv, const BicgScalars* s) {
    if (s->stop || s->restart) return;
    const double al = s->alpha;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        sv[i] = r[i] - al * v[i];
}

// x += alpha p + w s; r = s - w t; r.r, r0.r
__global__ void k_bicg_xr(int64_t n, double* __restrict__ x, const double* __restrict__ p,
                          const double* __restrict__ sv, const double* __restrict__ t,
                          double* __restrict__ r, const double* __restrict__ r0, Reduction red,
                          BicgScalars* s) {
    if (s->stop || s->restart) return;
    const double al = s->alpha, w = s->w;
    double acc[2] = {0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += al * p[i] + w * sv[i];
        const double rn = sv[i] - w * t[i];
        r[i] = rn;
        acc[0] += rn * rn;
        acc[1] += r0[i] * rn;
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        s->rr = tot[0];
        s->iters += 1;
        s->total += 1;
        s->rho_old = s->rho;
        s->rho = tot[1];
        s->beta = (s->rho / s->rho_old) * (s->alpha / s->w);
        if (!isfinite(tot[0])) {
            s->status = 2;
            s->stop = 1;
        } else if (tot[0] <= s->tol2) {
            s->stop = 1;
        } else if (s->iters >= s->maxit) {
            s->status = 1;
            s->stop = 1;
        } else if (fabs(s->rho) < DBL_EPSILON * DBL_EPSILON * s->r0n) {
            s->restart = 1;
        }
    }
}

// Runs the reference algorithm on S (stored symmetric form) from the current
// c.x; returns iterations; *err = ||r|| / ||b|| of the updated residual.
long long bicgstab_solve(Ctx& c, double tol, long long maxit, double* err, int* status) {
    if (!c.bicg) c.bicg = dev_alloc<double>(c, 32);
    BicgScalars* s = reinterpret_cast<BicgScalars*>(c.bicg);
    static_assert(sizeof(BicgScalars) <= 32 * sizeof(double), "scalar slot");
    const int64_t np = c.np, n = 4 * np;
    double* x = reinterpret_cast<double*>(c.x);
    double* b = reinterpret_cast<double*>(c.b);
    double* r = reinterpret_cast<double*>(c.r);
    double* r0 = reinterpret_cast<double*>(c.w64.Y[0]);
    double* p = reinterpret_cast<double*>(c.w64.W[0]);
    double* v = reinterpret_cast<double*>(c.w64.W[1]);
    double* sv = reinterpret_cast<double*>(c.w64.R[0]);
    double* t = reinterpret_cast<double*>(c.w64.R[1]);
    BicgScalars* sh = reinterpret_cast<BicgScalars*>(c.ms_host);  // pinned, large enough
    static_assert(sizeof(BicgScalars) <= sizeof(MinresScalars), "host scalar slot");
    FTS_CUDA(cudaMemsetAsync(p, 0, n * sizeof(double), c.stream));
    FTS_CUDA(cudaMemsetAsync(v, 0, n * sizeof(double), c.stream));
    const int ge = grid_for(c, n);
    k_bicg_init<<<ge, kThreads, 0, c.stream>>>(np, c.rowptr, c.cols, c.A64, c.x, b, r, r0, 0,
                                               tol, maxit, c.red, s);
    c.launches += 1;
    int restarts = 0;
    const int poll = np > 200000 ? 8 : 32;
    for (;;) {
        for (int u = 0; u < poll; ++u) {
            k_bicg_p<<<ge, kThreads, 0, c.stream>>>(n, r, p, v, s);
            k_bicg_spmv<<<ge, kThreads, 0, c.stream>>>(np, c.rowptr, c.cols, c.A64,
                                                       reinterpret_cast<V4<double>*>(p), v, r0, 0,
                                                       c.red, s);
            k_bicg_s<<<ge, kThreads, 0, c.stream>>>(n, r, v, sv, s);
            k_bicg_spmv<<<ge, kThreads, 0, c.stream>>>(np, c.rowptr, c.cols, c.A64,
                                                       reinterpret_cast<V4<double>*>(sv), t, nullptr,
                                                       1, c.red, s);
            k_bicg_xr<<<ge, kThreads, 0, c.stream>>>(n, x, p, sv, t, r, r0, c.red, s);
        }
        c.launches += 5 * poll;
        FTS_CUDA(cudaGetLastError());
        FTS_CUDA(cudaMemcpyAsync(sh, s, sizeof(BicgScalars), cudaMemcpyDeviceToHost, c.stream));
        FTS_CUDA(cudaStreamSynchronize(c.stream));
        if (sh->stop) break;
        if (sh->restart) {
            // shadow residual reset from the true residual (keeps the iteration count
            // unless this is the first restart, as the restatement does)
            k_bicg_init<<<ge, kThreads, 0, c.stream>>>(np, c.rowptr, c.cols, c.A64, c.x, b, r, r0,
                                                       1, tol, maxit, c.red, s);
            c.launches += 1;
            if (restarts++ == 0) {
                static const long long zero = 0;
                FTS_CUDA(cudaMemcpyAsync(&s->iters, &zero, sizeof(zero), cudaMemcpyHostToDevice,
                                         c.stream));
                FTS_CUDA(cudaStreamSynchronize(c.stream));
            }
        }
    }
    *err = sh->bb > 0.0 ? std::sqrt(sh->rr / sh->bb) : 0.0;
    *status = sh->status;
    c.spmv_runs += 2 * sh->total;
    c.bicg_restarts = sh->nrestart;
    return sh->total;
}

}  // namespace fts
