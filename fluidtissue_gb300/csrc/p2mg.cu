// P2 -> P1 multigrid level of the Taylor-Hood solve (see p2mg.cuh).
#include <cmath>
#include <vector>

#include "fts_device.cuh"
#include "mg.cuh"
#include "mg_device.cuh"
#include "p2mg.cuh"
#include "reduce.cuh"

namespace fts {

// The P2 level's sparse velocity operator and its transfer to the vertices.
template <typename T>
struct P2View {
    int64_t nn, nv;
    const int32_t* rowptr;
    const int32_t* cols;
    const T* K;             // 9 values per block (row-major 3x3)
    const uint8_t* mask;    // Dirichlet nodes (vertices and edges)
    const int32_t* ends;    // [2 ne]
    const int32_t* vinc_ptr;
    const int32_t* vinc;
};

// y = K2 x at node v (x SoA [3][nn]).
template <typename T>
__device__ __forceinline__ void p2_apply(const P2View<T>& P, int64_t v, const T* __restrict__ x,
                                         T y[3]) {
    const int64_t nn = P.nn;
    T a0 = T(0), a1 = T(0), a2 = T(0);
    const int32_t k1 = P.rowptr[v + 1];
    for (int32_t k = P.rowptr[v]; k < k1; ++k) {
        const int64_t j = __ldg(P.cols + k);
        const T* b = P.K + 9 * (int64_t)k;
        const T x0 = x[j], x1 = x[nn + j], x2 = x[2 * nn + j];
        a0 = fma(b[0], x0, fma(b[1], x1, fma(b[2], x2, a0)));
        a1 = fma(b[3], x0, fma(b[4], x1, fma(b[5], x2, a1)));
        a2 = fma(b[6], x0, fma(b[7], x1, fma(b[8], x2, a2)));
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

// Velocity part of the FP64 block system (identity rows / zero columns on
// Dirichlet nodes already), one thread per block.
template <typename T>
__global__ void k_p2_vel_extract(int64_t nnzb, const double* __restrict__ A, T* __restrict__ K) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnzb;
         k += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) K[9 * k + 3 * r + c] = (T)A[16 * k + 4 * r + c];
    }
}

template <typename T>
__global__ void k_p2_dinv(int64_t nn, const int32_t* __restrict__ diag, const T* __restrict__ K,
                          T* __restrict__ Dinv) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn;
         v += (int64_t)gridDim.x * blockDim.x) {
        const T* b = K + 9 * (int64_t)diag[v];
        const double a00 = b[0], a11 = b[4], a22 = b[8];
        const double a01 = 0.5 * ((double)b[1] + (double)b[3]);
        const double a02 = 0.5 * ((double)b[2] + (double)b[6]);
        const double a12 = 0.5 * ((double)b[5] + (double)b[7]);
        const double c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22;
        const double c02 = a01 * a12 - a02 * a11, c11 = a00 * a22 - a02 * a02;
        const double c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
        const double det = a00 * c00 + a01 * c01 + a02 * c02;
        const double id = det != 0.0 ? 1.0 / det : 0.0;
        Dinv[0 * nn + v] = (T)(c00 * id);
        Dinv[1 * nn + v] = (T)(c01 * id);
        Dinv[2 * nn + v] = (T)(c02 * id);
        Dinv[3 * nn + v] = (T)(c11 * id);
        Dinv[4 * nn + v] = (T)(c12 * id);
        Dinv[5 * nn + v] = (T)(c22 * id);
    }
}

// Power iteration step: w = D^-1 K2 v / ||v||, ||w|| -> nrm.
template <typename T>
__global__ void k_p2_power(P2View<T> P, const T* __restrict__ Di, const T* __restrict__ v,
                           T* __restrict__ w, double* __restrict__ nrm, int first,
                           Reduction red) {
    const int64_t nn = P.nn;
    const double inv = first ? 1.0 : (*nrm > 0.0 ? 1.0 / *nrm : 0.0);
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        T y[3], z[3];
        p2_apply<T>(P, i, v, y);
        dinv_apply<T>(nn, i, Di, y, z);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const T o = P.mask[i] ? T(0) : (T)(z[c] * inv);
            w[c * nn + i] = o;
            acc[0] += (double)o * (double)o;
        }
    }
    double tot[1];
    if (grid_sum<1>(acc, red, tot) && threadIdx.x == 0) *nrm = sqrt(tot[0]);
}

// Degree-1 pre-smoothing from zero: x = d_0, r = b - K2 d_0.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_p2_resid_d0(LevelView<T> L, P2View<T> P, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    const int64_t nn = P.nn;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn;
         v += (int64_t)gridDim.x * blockDim.x) {
        T y[3];
        p2_apply<T>(P, v, L.d0, y);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            L.r[c * nn + v] = L.b[c * nn + v] - y[c];
            L.x[c * nn + v] = L.d0[c * nn + v];
        }
    }
}

// Post-smoothing residual r = b - K2 x and d_0 = D^-1 r / theta.
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_p2_resid_first(LevelView<T> L, P2View<T> P, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    const int64_t nn = P.nn;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nn;
         v += (int64_t)gridDim.x * blockDim.x) {
        T y[3], rr[3];
        p2_apply<T>(P, v, L.x, y);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            rr[c] = L.b[c * nn + v] - y[c];
            L.r[c * nn + v] = rr[c];
        }
        mg_first_dir<T>(L, v, rr);
    }
}

// b1(v) = r2(v) + 1/2 sum of r2 over the edges at v (P^T r), zero on the
// Dirichlet vertices; then the P1 level's first direction.
template <typename T>
__global__ void k_p2_restrict(LevelView<T> L, P2View<T> P, LevelView<T> C,
                              const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    const int64_t nn = P.nn, nv = P.nv, Nc = C.N;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nv;
         v += (int64_t)gridDim.x * blockDim.x) {
        T a[3] = {T(0), T(0), T(0)};
        if (!C.mask[v]) {
#pragma unroll
            for (int c = 0; c < 3; ++c) a[c] = P.mask[v] ? T(0) : L.r[c * nn + v];
            for (int32_t q = P.vinc_ptr[v]; q < P.vinc_ptr[v + 1]; ++q) {
                const int64_t e = nv + P.vinc[q];
                if (P.mask[e]) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) a[c] += T(0.5) * L.r[c * nn + e];
            }
        }
        C.b[v] = a[0];
        C.b[Nc + v] = a[1];
        C.b[2 * Nc + v] = a[2];
        mg_first_dir<T>(C, v, a);
    }
}

// x2 += P x1 on the P2 nodes that are not Dirichlet.
template <typename T>
__global__ void k_p2_prolong(LevelView<T> L, P2View<T> P, LevelView<T> C,
                             const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    const int64_t nn = P.nn, nv = P.nv, Nc = C.N;
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < nn;
         a += (int64_t)gridDim.x * blockDim.x) {
        if (P.mask[a]) continue;
        T s[3] = {T(0), T(0), T(0)};
        if (a < nv) {
            if (!C.mask[a])
#pragma unroll
                for (int c = 0; c < 3; ++c) s[c] = C.x[c * Nc + a];
        } else {
            const int64_t e = a - nv;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t p = P.ends[2 * e + h];
                if (C.mask[p]) continue;
#pragma unroll
                for (int c = 0; c < 3; ++c) s[c] += T(0.5) * C.x[c * Nc + p];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) L.x[c * nn + a] += s[c];
    }
}

// P^T K2 P at the vertex pair (v, v + off(d)), thread per (d, vertex):
// sum over a in S(v) (v with weight 1, its edges with 1/2) of the blocks of
// row a whose column b lies in S(w) (w itself 1, an edge at w 1/2).
template <typename T>
__global__ void k_p2_galerkin(P2View<T> P, int n1, const uint8_t* __restrict__ mask1,
                              T* __restrict__ K1) {
    const int64_t N1 = (int64_t)n1 * n1 * n1, nv = P.nv;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N1 * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N1);
        const int64_t v = t - d * N1;
        const int i = (int)(v % n1), j = (int)((v / n1) % n1), k = (int)(v / ((int64_t)n1 * n1));
        const int w = nbr(i, j, k, d, n1);
        double acc[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) acc[e] = 0.0;
        if (w >= 0 && !mask1[v] && !mask1[w]) {
            const int32_t q0 = P.vinc_ptr[v], q1 = P.vinc_ptr[v + 1];
            for (int32_t q = q0 - 1; q < q1; ++q) {
                const int64_t a = q < q0 ? v : nv + P.vinc[q];
                const double pa = q < q0 ? 1.0 : 0.5;
                for (int32_t kk = P.rowptr[a]; kk < P.rowptr[a + 1]; ++kk) {
                    const int64_t b = P.cols[kk];
                    double pb = 0.0;
                    if (b == w) {
                        pb = 1.0;
                    } else if (b >= nv) {
                        const int64_t e = b - nv;
                        if (P.ends[2 * e] == w || P.ends[2 * e + 1] == w) pb = 0.5;
                    }
                    if (pb == 0.0) continue;
                    const T* blk = P.K + 9 * (int64_t)kk;
#pragma unroll
                    for (int e = 0; e < 9; ++e) acc[e] += pa * pb * (double)blk[e];
                }
            }
        } else if (w >= 0 && d == 0 && mask1[v]) {
            acc[0] = acc[4] = acc[8] = 1.0;  // Dirichlet vertex: identity row
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) K1[kidx(9 * d + e, v)] = (T)acc[e];
    }
}

// Deterministic start vector of the power iteration (zero on Dirichlet nodes).
template <typename T>
__global__ void k_p2_power_init(int64_t nn, const uint8_t* __restrict__ mask, T* __restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)(i * 2654435761u) ^ 0x85EBCA6Bu;
        for (int c = 0; c < 3; ++c) {
            h = h * 1664525u + 1013904223u;
            v[c * nn + i] = mask[i] ? T(0) : (T)(0.5 + (double)(h >> 8) / 16777216.0);
        }
    }
}

template <typename T>
static MG<T>& mg_of_ctx(Ctx& c);
template <>
MG<double>& mg_of_ctx<double>(Ctx& c) { return c.mg64; }
template <>
MG<float>& mg_of_ctx<float>(Ctx& c) { return c.mg32; }

template <typename T>
static P2MG<T>& p2mg_of(Ctx& c);
template <>
P2MG<double>& p2mg_of<double>(Ctx& c) { return c.p2mg64; }
template <>
P2MG<float>& p2mg_of<float>(Ctx& c) { return c.p2mg32; }

template <typename T>
static P2View<T> p2view(const Ctx& c, const P2MG<T>& m) {
    return P2View<T>{c.np, c.nv, c.rowptr, c.cols, m.K, c.bnd, m.edge_ends, m.vinc_ptr, m.vinc};
}

// The P2 level as a LevelView (the vectors, D^-1 and 1/theta that the MINRES
// stages and mg_first_dir read; no stencil).
template <typename T>
LevelView<T> p2_level_view(Ctx& c) {
    P2MG<T>& m = p2mg_of<T>(c);
    LevelView<T> L{};
    L.n = 0;
    L.N = c.np;
    L.Di = m.Di;
    L.b = m.b;
    L.x = m.x;
    L.r = m.r;
    L.d0 = m.d0;
    L.d1 = m.d1;
    L.mask = c.bnd;
    L.coef = m.coef;
    return L;
}

template <typename T>
static void p2mg_build(Ctx& c, P2MG<T>& m) {
    if (m.built) return;
    const HostTopology& Tp = c.topo;
    const int64_t nn = c.np, ne = Tp.ne, nv = Tp.nv;
    m.K = dev_alloc<T>(c, (size_t)c.nnzb * 9);
    m.Di = dev_alloc<T>(c, (size_t)nn * 6);
    for (T** p : {&m.b, &m.x, &m.r, &m.d0, &m.d1}) *p = dev_alloc<T>(c, (size_t)nn * 3);
    m.coef = dev_alloc<double>(c, kCoefStride);
    m.lam = dev_alloc<double>(c, 1);
    m.edge_ends = dev_alloc<int32_t>(c, (size_t)std::max<int64_t>(1, 2 * ne));
    m.vinc_ptr = dev_alloc<int32_t>(c, (size_t)nv + 1);
    m.vinc = dev_alloc<int32_t>(c, (size_t)std::max<int64_t>(1, 2 * ne));
    FTS_CUDA(cudaMemcpyAsync(m.edge_ends, Tp.edge_ends.data(), 2 * ne * sizeof(int32_t),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemcpyAsync(m.vinc_ptr, Tp.vinc_ptr.data(), (nv + 1) * sizeof(int32_t),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemcpyAsync(m.vinc, Tp.vinc.data(), 2 * ne * sizeof(int32_t),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaMemsetAsync(m.x, 0, (size_t)nn * 3 * sizeof(T), c.stream));
    m.built = true;
}

template <typename T>
void p2mg_setup(Ctx& c) {
    P2MG<T>& m = p2mg_of<T>(c);
    p2mg_build<T>(c, m);
    const int64_t nn = c.np;
    if (!c.A64)
        throw CudaError(cudaErrorInvalidValue, "P2 multigrid set-up before the assembly",
                        __FILE__, __LINE__);
    k_p2_vel_extract<T><<<grid_for(c, c.nnzb), kThreads, 0, c.stream>>>(c.nnzb, c.A64, m.K);
    k_p2_dinv<T><<<grid_for(c, nn), kThreads, 0, c.stream>>>(nn, c.diag, m.K, m.Di);
    k_p2_power_init<T><<<grid_for(c, nn), kThreads, 0, c.stream>>>(nn, c.bnd, m.d0);
    c.launches += 3;
    const P2View<T> P = p2view<T>(c, m);
    T* v = m.d0;
    T* w = m.d1;
    for (int it = 0; it < kPowerIters; ++it) {
        k_p2_power<T><<<grid_for(c, nn), kThreads, 0, c.stream>>>(P, m.Di, v, w, m.lam, it == 0,
                                                                   c.red);
        c.launches += 1;
        std::swap(v, w);
    }
    FTS_CUDA(cudaGetLastError());
    double lam = 0.0;
    FTS_CUDA(cudaMemcpyAsync(&lam, m.lam, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FTS_CUDA(cudaStreamSynchronize(c.stream));
    lam = (lam > 0.0 && std::isfinite(lam) ? lam : 2.5) * kLamSafety;
    m.lam_host = lam;
    std::vector<double> coef(kCoefStride);
    cheb_table(lam, coef.data());
    FTS_CUDA(cudaMemcpyAsync(m.coef, coef.data(), coef.size() * sizeof(double),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaStreamSynchronize(c.stream));
}

template <typename T>
void p2mg_galerkin(Ctx& c, T* K1, const uint8_t* mask1, int n1) {
    P2MG<T>& m = p2mg_of<T>(c);
    const int64_t N1 = (int64_t)n1 * n1 * n1;
    k_p2_galerkin<T><<<grid_for(c, N1 * 8), kThreads, 0, c.stream>>>(p2view<T>(c, m), n1, mask1,
                                                                       K1);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

template <typename T>
void p2mg_vcycle(Ctx& c, const int* stop) {
    P2MG<T>& m = p2mg_of<T>(c);
    MG<T>& mg = mg_of_ctx<T>(c);
    const LevelView<T> L = p2_level_view<T>(c);
    const LevelView<T> C = level_view(mg, 0);
    const P2View<T> P = p2view<T>(c, m);
    const int g = grid_for(c, c.np);
    pdl_launch(k_p2_resid_d0<T>, g, kThreads, c.stream, L, P, stop);
    pdl_launch(k_p2_restrict<T>, grid_for(c, c.nv), kThreads, c.stream, L, P, C, stop);
    mg_vcycle<T>(c, mg, stop, false);
    pdl_launch(k_p2_prolong<T>, g, kThreads, c.stream, L, P, C, stop);
    pdl_launch(k_p2_resid_first<T>, g, kThreads, c.stream, L, P, stop);
    c.launches += 4;
}

template <typename T>
void p2mg_free(P2MG<T>& m) {
    for (void* p : {(void*)m.K, (void*)m.Di, (void*)m.b, (void*)m.x, (void*)m.r, (void*)m.d0,
                    (void*)m.d1, (void*)m.coef, (void*)m.lam, (void*)m.edge_ends,
                    (void*)m.vinc_ptr, (void*)m.vinc})
        if (p) cudaFree(p);
    m = P2MG<T>{};
}

template void p2mg_setup<double>(Ctx&);
template void p2mg_setup<float>(Ctx&);
template void p2mg_galerkin<double>(Ctx&, double*, const uint8_t*, int);
template void p2mg_galerkin<float>(Ctx&, float*, const uint8_t*, int);
template void p2mg_vcycle<double>(Ctx&, const int*);
template void p2mg_vcycle<float>(Ctx&, const int*);
template void p2mg_free<double>(P2MG<double>&);
template void p2mg_free<float>(P2MG<float>&);
template LevelView<double> p2_level_view<double>(Ctx&);
template LevelView<float> p2_level_view<float>(Ctx&);

}  // namespace fts
