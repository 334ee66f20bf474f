// Per-node bodies of the pressure V-cycle (internal), shared by its own
// kernels (pmg.cu) and the preconditioner stages of MINRES (krylov.cu), which
// write the finest right-hand side and run the last finest smoothing step.
// Same Chebyshev recurrences and step modes as the velocity V-cycle
// (mg_device.cuh), on one value per node.
#pragma once

#include "mg_device.cuh"
#include "pmg.cuh"

namespace fts {

// (Kp x)(v) from the half stencil: own entries towards self and the 7
// positive directions, the neighbours' entries for the 7 negative ones.
// INNER: all 14 neighbours exist; no range checks, so every load of the node
// can be issued before the first use.
template <typename T, bool INNER>
__device__ __forceinline__ T pmg_stencil_body(int n, int64_t N, int v, int i, int j, int k,
                                              const T* __restrict__ K,
                                              const T* __restrict__ x) {
    const int nn = n * n;
    T a = T(0);
#pragma unroll
    for (int d = 0; d < 8; ++d) {
        const int w = INNER ? v + off_x(d) + n * off_y(d) + nn * off_z(d) : nbr(i, j, k, d, n);
        if (!INNER && w < 0) continue;
        a = fma(__ldg(K + d * N + v), __ldg(x + w), a);
    }
#pragma unroll
    for (int d = 1; d < 8; ++d) {
        const int w = INNER ? v - off_x(d) - n * off_y(d) - nn * off_z(d) : nbr(i, j, k, d + 7, n);
        if (!INNER && w < 0) continue;
        a = fma(__ldg(K + d * N + w), __ldg(x + w), a);
    }
    return a;
}

template <typename T>
__device__ __forceinline__ T pmg_stencil(int n, int64_t N, int64_t v64, const T* __restrict__ K,
                                         const T* __restrict__ x) {
    const int v = (int)v64;
    const int nn = n * n;
    const int k = v / nn;
    const int rem = v - k * nn;
    const int j = rem / n;
    const int i = rem - j * n;
    if (i > 0 && j > 0 && k > 0 && i < n - 1 && j < n - 1 && k < n - 1)
        return pmg_stencil_body<T, true>(n, N, v, i, j, k, K, x);
    return pmg_stencil_body<T, false>(n, N, v, i, j, k, K, x);
}

// Degree-1 pre-smoothing from zero: r = b - Kp d_0 (the smoothed x is d_0,
// written by the prolongation as x = d_0 + P e).
template <typename T>
__device__ __forceinline__ void pmg_resid_d0_node(const PView<T>& L, int64_t v) {
    L.r[v] = L.b[v] - pmg_stencil<T>(L.n, L.N, v, L.K, L.d0);
}

// d_0 = D^-1 b / theta.
template <typename T>
__device__ __forceinline__ void pmg_first_dir(const PView<T>& L, int64_t v, T bv) {
    L.d0[v] = L.Di[v] * bv * (T)L.coef[0];
}

// Chebyshev step s >= 1 at node v; returns the new x.  write: store r, d_out
// and x (the fused caller of the last finest step stores nothing).
template <typename T>
__device__ __forceinline__ T pmg_step_node(const PView<T>& L, int64_t v, int step, int mode,
                                           const T* __restrict__ din, T* __restrict__ dout,
                                           bool write) {
    const T A = (T)L.coef[2 * step - 1], B = (T)L.coef[2 * step];
    const T y = pmg_stencil<T>(L.n, L.N, v, L.K, din);
    const T rr = (mode == kStepFromZero ? L.b[v] : L.r[v]) - y;
    const T di = din[v];
    const T dd = A * di + B * (L.Di[v] * rr);
    T xv;
    if (mode == kStepFromZero) xv = di + dd;
    else if (mode == kStepAfterFirst) xv = L.x[v] + di + dd;
    else xv = L.x[v] + dd;
    if (write) {
        L.r[v] = rr;
        dout[v] = dd;
        L.x[v] = xv;
    }
    return xv;
}

// r = b - Kp x.
template <typename T>
__device__ __forceinline__ void pmg_resid_node(const PView<T>& L, int64_t v) {
    L.r[v] = L.b[v] - pmg_stencil<T>(L.n, L.N, v, L.K, L.x);
}

// r = b - Kp x and d_0 = D^-1 r / theta (x is updated by the next step);
// WR = false: r is not stored (degree-1 levels).
template <typename T, bool WR = true>
__device__ __forceinline__ void pmg_resid_first_node(const PView<T>& L, int64_t v) {
    const T rr = L.b[v] - pmg_stencil<T>(L.n, L.N, v, L.K, L.x);
    if (WR) L.r[v] = rr;
    pmg_first_dir<T>(L, v, rr);
}

// b_c(I) = sum_d w_d r_f(2I + off[d]) over the fine nodes that exist (P^T r);
// then the coarse first direction.
template <typename T>
__device__ __forceinline__ void pmg_restrict_node(const PView<T>& F, const PView<T>& C,
                                                  int64_t I) {
    const int nf = F.n, nc = C.n;
    const int ci = (int)(I % nc), cj = (int)((I / nc) % nc), ck = (int)(I / ((int64_t)nc * nc));
    T a = T(0);
#pragma unroll
    for (int d = 0; d < 15; ++d) {
        const int f = nbr(2 * ci, 2 * cj, 2 * ck, d, nf);
        if (f < 0) continue;
        a += (d == 0 ? T(1) : T(0.5)) * F.r[f];
    }
    C.b[I] = a;
    pmg_first_dir<T>(C, I, a);
}

// x_f += (P x_c)(f): the coarse value at even positions, the mean of the two
// ends of the coarse Kuhn edge through f elsewhere; FROM_D0: x_f = d_0 + P x_c
// (a degree-1 level).
template <typename T, bool FROM_D0 = false>
__device__ __forceinline__ void pmg_prolong_node(const PView<T>& F, const PView<T>& C,
                                                 int64_t f) {
    const int nf = F.n, nc = C.n;
    const int fi = (int)(f % nf), fj = (int)((f / nf) % nf), fk = (int)(f / ((int64_t)nf * nf));
    const int Ai = fi >> 1, Aj = fj >> 1, Ak = fk >> 1;
    const int oi = fi & 1, oj = fj & 1, ok = fk & 1;
    const int64_t A = Ai + (int64_t)nc * (Aj + (int64_t)nc * Ak);
    T s;
    if ((oi | oj | ok) == 0) {
        s = C.x[A];
    } else {
        const int64_t Bn = (Ai + oi) + (int64_t)nc * ((Aj + oj) + (int64_t)nc * (Ak + ok));
        s = T(0.5) * (C.x[A] + C.x[Bn]);
    }
    F.x[f] = (FROM_D0 ? F.d0[f] : F.x[f]) + s;
}

}  // namespace fts
