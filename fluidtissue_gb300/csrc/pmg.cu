// Scalar multigrid V-cycle for the pressure block of the MINRES preconditioner
// on Kuhn lattices (structure and operator: pmg.cuh).  It runs on a second
// stream, concurrently with the velocity V-cycle of the same preconditioner
// application; both join before the stage that finishes the application.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "fts_device.cuh"
#include "pmg.cuh"
#include "pmg_device.cuh"

namespace fts {

__constant__ int c_pgal_start[16];
__constant__ unsigned short c_pgal_term[512];
__constant__ float c_pgal_w[512];

static void init_ptables(int device) {
    static bool done[64] = {};
    if (device < 64 && done[device]) return;
    std::vector<int> start;
    std::vector<unsigned short> term;
    std::vector<float> w;
    galerkin_terms(start, term, w);
    FTS_CUDA(cudaMemcpyToSymbol(c_pgal_start, start.data(), 16 * sizeof(int)));
    FTS_CUDA(cudaMemcpyToSymbol(c_pgal_term, term.data(), term.size() * sizeof(unsigned short)));
    FTS_CUDA(cudaMemcpyToSymbol(c_pgal_w, w.data(), w.size() * sizeof(float)));
    if (device < 64) done[device] = true;
}

// Entry Kp(f, f + off[e]) for any of the 15 directions.
template <typename T>
__device__ __forceinline__ T pentry(const T* __restrict__ K, int64_t N, int e, int64_t f, int n) {
    if (e < 8) return K[e * N + f];
    const int ep = e - 7;
    const int64_t w = f - (off_x(ep) + (int64_t)n * (off_y(ep) + (int64_t)n * off_z(ep)));
    return K[ep * N + w];
}

// ---------------------------------------------------------------------------
// Set-up kernels
// ---------------------------------------------------------------------------

// Fine level from the assembled system: the pressure entry (3,3) of the 4x4
// blocks, negated back to +(alpha D + eps M), plus w on the diagonal.  One
// thread per (node, stored direction).
template <typename T>
__global__ void k_pmg_extract(int n, const int32_t* __restrict__ rowptr,
                              const int32_t* __restrict__ cols, const double* __restrict__ A,
                              const int32_t* __restrict__ p2t_ptr,
                              const uint32_t* __restrict__ p2t, const ElemGeom* __restrict__ geom,
                              const double* __restrict__ mu, const OuterScalars* __restrict__ os,
                              T* __restrict__ K) {
    const int64_t N = (int64_t)n * n * n;
    const double ws = schur_scale(os);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((int64_t)n * n));
        const int w = nbr(i, j, k, d, n);
        double val = 0.0;
        if (w >= 0) {
            int lo = rowptr[v], hi = rowptr[v + 1] - 1;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (cols[mid] < w) lo = mid + 1;
                else hi = mid;
            }
            if (cols[lo] == w) val = -A[(int64_t)lo * 16 + 15];
        }
        if (d == 0) val += ws * lumped_inv_mu(v, p2t_ptr, p2t, geom, mu);
        K[d * N + v] = (T)val;
    }
}

// Fine level from the FP64 lattice half stencil: entry (3,3) of the 8 blocks.
template <typename T>
__global__ void k_pmg_extract_lat(int n, const double2* __restrict__ L,
                                  const int32_t* __restrict__ p2t_ptr,
                                  const uint32_t* __restrict__ p2t,
                                  const ElemGeom* __restrict__ geom,
                                  const double* __restrict__ mu,
                                  const OuterScalars* __restrict__ os, T* __restrict__ K) {
    const int64_t N = (int64_t)n * n * n;
    const double ws = schur_scale(os);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
        double val = -L[lat64_idx(d, 3, 1, v)].y;
        if (d == 0) val += ws * lumped_inv_mu(v, p2t_ptr, p2t, geom, mu);
        K[d * N + v] = (T)val;
    }
}

struct PRef {
    double mref[4][4];
};

// Fine level from the elements (matrix-free mode): sum over the elements
// holding v and v + off[d] of alpha h^2 vol g_a.g_b + eps vol Mref[a][b]
// (the pressure block of Flow.cpp's composition), plus w on the diagonal.
template <typename T, bool KUHN>
__global__ void k_pmg_from_elements(int n, const int32_t* __restrict__ p2t_ptr,
                                    const uint32_t* __restrict__ p2t,
                                    const int32_t* __restrict__ tets,
                                    const ElemGeom* __restrict__ geom,
                                    const double* __restrict__ mu, double alpha, double eps,
                                    PRef R, const OuterScalars* __restrict__ os,
                                    T* __restrict__ K) {
    const int64_t N = (int64_t)n * n * n;
    const double ws = schur_scale(os);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((int64_t)n * n));
        const int w = nbr(i, j, k, d, n);
        double val = 0.0;
        if (w >= 0) {
            auto add = [&](int64_t el, int a, int b) {
                const ElemGeom& G = geom[el];
                const double gg = G.g[a][0] * G.g[b][0] + G.g[a][1] * G.g[b][1] +
                                  G.g[a][2] * G.g[b][2];
                val += alpha * (G.hh * G.vol * gg) + eps * (G.vol * R.mref[a][b]);
            };
            if (KUHN) {  // generator's element order: the elements follow from the lattice
                kuhn_pair_elements(n, i, j, k, d, add);
            } else {
                for (int32_t q = p2t_ptr[v]; q < p2t_ptr[v + 1]; ++q) {
                    const uint32_t e = p2t[q];
                    const int64_t el = e >> 2;
                    const int4 tt = reinterpret_cast<const int4*>(tets)[el];
                    const int b =
                        tt.x == w ? 0 : (tt.y == w ? 1 : (tt.z == w ? 2 : (tt.w == w ? 3 : -1)));
                    if (b >= 0) add(el, (int)(e & 3), b);
                }
            }
        }
        if (d == 0) val += ws * lumped_inv_mu(v, p2t_ptr, p2t, geom, mu);
        K[d * N + v] = (T)val;
    }
}

// Galerkin coarse operator P^T Kp P, one thread per (coarse node, direction).
template <typename T>
__global__ void k_pmg_galerkin(int nf, const T* __restrict__ Kf, int nc, T* __restrict__ Kc) {
    const int64_t Nf = (int64_t)nf * nf * nf, Nc = (int64_t)nc * nc * nc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Nc * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int dJ = (int)(t / Nc);
        const int64_t I = t - dJ * Nc;
        const int ci = (int)(I % nc), cj = (int)((I / nc) % nc), ck = (int)(I / ((int64_t)nc * nc));
        T acc = T(0);
        if (nbr(ci, cj, ck, dJ, nc) >= 0) {
            for (int q = c_pgal_start[dJ]; q < c_pgal_start[dJ + 1]; ++q) {
                const int a = c_pgal_term[q] & 15, e = (c_pgal_term[q] >> 4) & 15;
                const int fi = 2 * ci + off_x(a), fj = 2 * cj + off_y(a), fk = 2 * ck + off_z(a);
                if (fi < 0 || fj < 0 || fk < 0 || fi >= nf || fj >= nf || fk >= nf) continue;
                const int64_t f = fi + (int64_t)nf * (fj + (int64_t)nf * fk);
                if (nbr(fi, fj, fk, e, nf) < 0) continue;
                acc += (T)c_pgal_w[q] * pentry<T>(Kf, Nf, e, f, nf);
            }
        }
        Kc[dJ * Nc + I] = acc;
    }
}

// D^-1 and the level's Gershgorin bound max_v sum_w |Kp(v, w)| / Kp(v, v)
// (non-negative doubles order like their bit patterns).
template <typename T>
__global__ void k_pmg_dinv(int n, const T* __restrict__ K, T* __restrict__ Di,
                           unsigned long long* __restrict__ gersh) {
    const int64_t N = (int64_t)n * n * n;
    double g = 0.0;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
         v += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((int64_t)n * n));
        const double kd = (double)K[v];
        double s = fabs(kd);
        for (int d = 1; d < 8; ++d) {
            if (nbr(i, j, k, d, n) >= 0) s += fabs((double)K[d * N + v]);
            const int w = nbr(i, j, k, d + 7, n);
            if (w >= 0) s += fabs((double)K[d * N + w]);
        }
        Di[v] = kd > 0.0 ? (T)(1.0 / kd) : T(0);
        if (kd > 0.0) g = fmax(g, s / kd);
    }
    for (int o = 16; o > 0; o >>= 1) g = fmax(g, __shfl_xor_sync(0xffffffffu, g, o));
    if ((threadIdx.x & 31) == 0 && g > 0.0)
        atomicMax(gersh, (unsigned long long)__double_as_longlong(g));
}

// ---------------------------------------------------------------------------
// V-cycle kernels (skip when the MINRES run has stopped)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_pmg_step(PView<T> L, int step, int mode, const T* __restrict__ din, T* __restrict__ dout,
           const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < L.N;
         v += (int64_t)gridDim.x * blockDim.x)
        pmg_step_node<T>(L, v, step, mode, din, dout, true);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_pmg_residual(PView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < L.N;
         v += (int64_t)gridDim.x * blockDim.x)
        pmg_resid_node<T>(L, v);
}

template <typename T, bool WR = true>
__global__ void __launch_bounds__(kThreads)
k_pmg_resid_first(PView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < L.N;
         v += (int64_t)gridDim.x * blockDim.x)
        pmg_resid_first_node<T, WR>(L, v);
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_pmg_resid_d0(PView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        pmg_resid_d0_node<T>(L, i);
}

template <typename T>
__global__ void k_pmg_add_d0(PView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        L.x[i] += L.d0[i];
}

template <typename T>
__global__ void k_pmg_restrict(PView<T> F, PView<T> C, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < C.N;
         I += (int64_t)gridDim.x * blockDim.x)
        pmg_restrict_node<T>(F, C, I);
}

template <typename T, bool FROM_D0 = false>
__global__ void k_pmg_prolong(PView<T> F, PView<T> C, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < F.N;
         f += (int64_t)gridDim.x * blockDim.x)
        pmg_prolong_node<T, FROM_D0>(F, C, f);
}

// Levels l0.. of one V-cycle in one CTA (__syncthreads between phases); the
// coarsest level by its dense inverse.
template <typename T>
struct PTailArgs {
    PView<T> lv[kMaxMGLevels];
    const T* cinv;
    int l0, nlev, skip_final;
};

template <typename T>
__global__ void __launch_bounds__(kPTailThreads, 1)
k_pmg_tail(const __grid_constant__ PTailArgs<T> a, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;  // uniform over the block
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int l = a.l0; l + 1 < a.nlev; ++l) {
        const PView<T> L = a.lv[l];
        for (int s = 1; s < kPSmooth; ++s) {
            const int mode = s == 1 ? kStepFromZero : kStepRegular;
            for (int64_t v = tid; v < L.N; v += nth)
                pmg_step_node<T>(L, v, s, mode, (s & 1) ? L.d0 : L.d1, (s & 1) ? L.d1 : L.d0,
                                 true);
            __syncthreads();
        }
        for (int64_t v = tid; v < L.N; v += nth) pmg_resid_node<T>(L, v);
        __syncthreads();
        const PView<T> C = a.lv[l + 1];
        for (int64_t v = tid; v < C.N; v += nth) pmg_restrict_node<T>(L, C, v);
        __syncthreads();
    }
    {
        const PView<T> L = a.lv[a.nlev - 1];
        const int N = (int)L.N;
        for (int i = tid; i < N; i += nth) {
            T s = T(0);
            for (int j = 0; j < N; ++j) s = fma(a.cinv[(int64_t)i * N + j], L.b[j], s);
            L.x[i] = s;
        }
        __syncthreads();
    }
    for (int l = a.nlev - 2; l >= a.l0; --l) {
        const PView<T> L = a.lv[l], C = a.lv[l + 1];
        for (int64_t v = tid; v < L.N; v += nth) pmg_prolong_node<T>(L, C, v);
        __syncthreads();
        for (int64_t v = tid; v < L.N; v += nth) pmg_resid_first_node<T>(L, v);
        __syncthreads();
        const int last = (l == 0 && a.skip_final) ? kPSmooth - 2 : kPSmooth - 1;
        for (int s = 1; s <= last; ++s) {
            const int mode = s == 1 ? kStepAfterFirst : kStepRegular;
            for (int64_t v = tid; v < L.N; v += nth)
                pmg_step_node<T>(L, v, s, mode, (s & 1) ? L.d0 : L.d1, (s & 1) ? L.d1 : L.d0,
                                 true);
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <typename T>
void pmg_build(Ctx& c, PMG<T>& pm) {
    if (pm.built) return;
    init_ptables(c.device);
    const std::vector<int> chain = mg_chain(c.topo.lattice_n);
    if (chain.size() > (size_t)kMaxMGLevels || chain.size() < 2) {
        c.last_error = "lattice size outside the pressure multigrid's range";
        throw (int)FTS_ERR_UNSUPPORTED;
    }
    for (const int n : chain) {
        PLevel<T> L;
        L.n = n;
        L.N = (int64_t)n * n * n;
        L.K = dev_alloc<T>(c, (size_t)L.N * 8);
        L.Di = dev_alloc<T>(c, (size_t)L.N);
        for (auto** p : {&L.b, &L.x, &L.r, &L.d0, &L.d1}) *p = dev_alloc<T>(c, (size_t)L.N);
        pm.L.push_back(L);
    }
    const int64_t Nc = pm.L.back().N;
    pm.cinv = dev_alloc<T>(c, (size_t)(Nc * Nc));
    pm.coef = dev_alloc<double>(c, pm.L.size() * kCoefStride);
    pm.gersh = dev_alloc<unsigned long long>(c, pm.L.size());
    FTS_CUDA(cudaMallocHost(&pm.h_gbits, pm.L.size() * sizeof(unsigned long long)));
    FTS_CUDA(cudaMallocHost(&pm.h_kc, (size_t)pm.L.back().N * 8 * sizeof(T)));
    FTS_CUDA(cudaEventCreateWithFlags(&pm.ev_copied, cudaEventDisableTiming));
    pm.tail_level = (int)pm.L.size() - 1;
    for (size_t l = 0; l + 1 < pm.L.size(); ++l)
        if (pm.L[l].N <= kPTailNodes) {
            pm.tail_level = (int)l;
            break;
        }
    pm.built = true;
}

// Chebyshev coefficients on [lam / 10, lam] (same recurrence as the velocity
// hierarchy's): 1/theta, then (rho_s rho_{s-1}, 2 rho_s / delta) for s >= 1.
static void pcheb_table(double lam, double* out) {
    const double lmax = lam, lmin = kPLowFrac * lam;
    const double th = 0.5 * (lmax + lmin), de = 0.5 * (lmax - lmin), sg = th / de;
    out[0] = 1.0 / th;
    double rho = 1.0 / sg;
    for (int s = 1; 2 * s < kCoefStride; ++s) {
        const double rprev = rho;
        rho = 1.0 / (2.0 * sg - rho);
        out[2 * s - 1] = rho * rprev;
        out[2 * s] = 2.0 * rho / de;
    }
}

// Inverse of the SPD matrix a (m x m, row-major) by Cholesky, in place.
// Returns false when a pivot is not positive.
static bool spd_inverse(std::vector<double>& a, int m) {
    std::vector<double> L((size_t)m * m, 0.0);
    for (int j = 0; j < m; ++j) {
        double d = a[(size_t)j * m + j];
        for (int k = 0; k < j; ++k) d -= L[(size_t)j * m + k] * L[(size_t)j * m + k];
        if (!(d > 0.0)) return false;
        const double ljj = std::sqrt(d);
        L[(size_t)j * m + j] = ljj;
        for (int i = j + 1; i < m; ++i) {
            double s = a[(size_t)i * m + j];
            for (int k = 0; k < j; ++k) s -= L[(size_t)i * m + k] * L[(size_t)j * m + k];
            L[(size_t)i * m + j] = s / ljj;
        }
    }
    // inverse column by column: L L^T x = e_c
    std::vector<double> inv((size_t)m * m), y(m);
    for (int c = 0; c < m; ++c) {
        for (int i = 0; i < m; ++i) {
            double s = i == c ? 1.0 : 0.0;
            for (int k = 0; k < i; ++k) s -= L[(size_t)i * m + k] * y[k];
            y[i] = s / L[(size_t)i * m + i];
        }
        for (int i = m - 1; i >= 0; --i) {
            double s = y[i];
            for (int k = i + 1; k < m; ++k) s -= L[(size_t)k * m + i] * inv[(size_t)k * m + c];
            inv[(size_t)i * m + c] = s / L[(size_t)i * m + i];
        }
    }
    a.swap(inv);
    return true;
}

static const int kHostOff[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1},
                                   {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

// Set-up kernels on stream st (after what st waits for), ending with the
// copies of the Gershgorin bounds and the coarsest stencil into pinned host
// buffers; pmg_setup_finish waits for them and completes the set-up on the host.
template <typename T>
void pmg_setup_enqueue(Ctx& c, PMG<T>& pm, cudaStream_t st) {
    PLevel<T>& F = pm.L[0];
    if (c.matfree) {
        const RefConstants R = ref_constants();
        PRef pr;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) pr.mref[a][b] = R.mref[a][b];
        if (c.topo.kuhn_elements)
            k_pmg_from_elements<T, true><<<grid_for(c, F.N * 8), kThreads, 0, st>>>(
                F.n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.par.alpha, c.par.eps, pr, c.os,
                F.K);
        else
            k_pmg_from_elements<T, false><<<grid_for(c, F.N * 8), kThreads, 0, st>>>(
                F.n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.par.alpha, c.par.eps, pr, c.os,
                F.K);
    } else if (c.use_lat64) {
        k_pmg_extract_lat<T><<<grid_for(c, F.N * 8), kThreads, 0, st>>>(
            F.n, c.lat64, c.p2t_ptr, c.p2t, c.geom, c.mu, c.os, F.K);
    } else {
        k_pmg_extract<T><<<grid_for(c, F.N * 8), kThreads, 0, st>>>(
            F.n, c.rowptr, c.cols, c.A64, c.p2t_ptr, c.p2t, c.geom, c.mu, c.os, F.K);
    }
    c.launches += 1;
    FTS_CUDA(cudaMemsetAsync(pm.gersh, 0, pm.L.size() * sizeof(unsigned long long), st));
    for (size_t l = 0; l < pm.L.size(); ++l) {
        PLevel<T>& L = pm.L[l];
        if (l > 0) {
            const PLevel<T>& P = pm.L[l - 1];
            k_pmg_galerkin<T><<<grid_for(c, L.N * 8), kThreads, 0, st>>>(P.n, P.K, L.n,
                                                                                L.K);
            c.launches += 1;
        }
        k_pmg_dinv<T><<<grid_for(c, L.N), kThreads, 0, st>>>(L.n, L.K, L.Di,
                                                                     pm.gersh + l);
        c.launches += 1;
    }
    FTS_CUDA(cudaGetLastError());
    const PLevel<T>& Cl = pm.L.back();
    FTS_CUDA(cudaMemcpyAsync(pm.h_gbits, pm.gersh, pm.L.size() * sizeof(unsigned long long),
                             cudaMemcpyDeviceToHost, st));
    FTS_CUDA(cudaMemcpyAsync(pm.h_kc, Cl.K, (size_t)Cl.N * 8 * sizeof(T), cudaMemcpyDeviceToHost,
                             st));
    FTS_CUDA(cudaEventRecord(pm.ev_copied, st));
}

template <typename T>
void pmg_setup_finish(Ctx& c, PMG<T>& pm, cudaStream_t st) {
    FTS_CUDA(cudaEventSynchronize(pm.ev_copied));
    const PLevel<T>& Cl = pm.L.back();
    const int m = (int)Cl.N;
    const unsigned long long* gbits = pm.h_gbits;
    const T* kc = pm.h_kc;
    std::vector<double> lam(pm.L.size());
    for (size_t l = 0; l < lam.size(); ++l) {
        double g;
        std::memcpy(&g, &gbits[l], sizeof(double));
        lam[l] = (g > 0.0 && std::isfinite(g)) ? g : 2.0;
    }
    pm.lam_host = lam;
    std::vector<double> coef(lam.size() * kCoefStride, 0.0);
    for (size_t l = 0; l < lam.size(); ++l) pcheb_table(lam[l], coef.data() + l * kCoefStride);
    // dense coarsest operator from its half stencil, inverted in FP64
    const int n = Cl.n;
    std::vector<double> dense((size_t)m * m, 0.0);
    for (int v = 0; v < m; ++v) {
        const int i = v % n, j = (v / n) % n, k = v / (n * n);
        for (int d = 0; d < 8; ++d) {
            const int a = i + kHostOff[d][0], b = j + kHostOff[d][1], cc = k + kHostOff[d][2];
            if (a >= n || b >= n || cc >= n) continue;
            const int w = a + n * (b + n * cc);
            const double val = (double)kc[(size_t)d * m + v];
            dense[(size_t)v * m + w] = val;
            dense[(size_t)w * m + v] = val;
        }
    }
    bool finite = true;
    for (const double v : dense) finite = finite && std::isfinite(v);
    if (!finite) {
        // non-finite inputs: the caller's input check reports them after the
        // set-up; the coarse solve is never used
        std::fill(dense.begin(), dense.end(), 0.0);
    } else if (!spd_inverse(dense, m)) {
        c.last_error = "pressure multigrid: coarsest operator is not positive definite "
                       "(viscosities must be positive)";
        throw (int)FTS_ERR_BAD_INPUT;
    }
    std::vector<T> cinv(dense.begin(), dense.end());
    FTS_CUDA(cudaMemcpyAsync(pm.coef, coef.data(), coef.size() * sizeof(double),
                             cudaMemcpyHostToDevice, st));
    FTS_CUDA(cudaMemcpyAsync(pm.cinv, cinv.data(), cinv.size() * sizeof(T),
                             cudaMemcpyHostToDevice, st));
    FTS_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
void pmg_setup(Ctx& c, PMG<T>& pm) {
    pmg_build<T>(c, pm);
    pmg_setup_enqueue<T>(c, pm, c.stream);
    pmg_setup_finish<T>(c, pm, c.stream);
}

template <typename T>
static void pvcycle_level(Ctx& c, PMG<T>& pm, size_t l, cudaStream_t st, const int* stop,
                          bool skip_final) {
    if ((int)l == pm.tail_level) {
        PTailArgs<T> a{};
        for (size_t k = 0; k < pm.L.size(); ++k) a.lv[k] = pview(pm, k);
        a.cinv = pm.cinv;
        a.l0 = (int)l;
        a.nlev = (int)pm.L.size();
        a.skip_final = skip_final ? 1 : 0;
        pdl_launch(k_pmg_tail<T>, 1, kPTailThreads, st, a, stop);
        c.launches += 1;
        return;
    }
    const PView<T> L = pview(pm, l), C = pview(pm, l + 1);
    const int g = grid_for(c, L.N);
    if (pmg_level_degree1(pm, l)) {
        // degree 1: x = d_0, r = b - Kp d_0; after the coarse correction
        // x = d_0 + P e, r = b - Kp x (not stored), d_0 = D^-1 r / theta,
        // x += d_0 (the caller's when skip_final)
        pdl_launch(k_pmg_resid_d0<T>, g, kThreads, st, L, stop);
        pdl_launch(k_pmg_restrict<T>, grid_for(c, C.N), kThreads, st, L, C, stop);
        pvcycle_level<T>(c, pm, l + 1, st, stop, false);
        pdl_launch(k_pmg_prolong<T, true>, g, kThreads, st, L, C, stop);
        pdl_launch(k_pmg_resid_first<T, false>, g, kThreads, st, L, stop);
        c.launches += 4;
        if (!skip_final) {
            pdl_launch(k_pmg_add_d0<T>, g, kThreads, st, L, stop);
            c.launches += 1;
        }
        return;
    }
    T* din = L.d0;
    T* dout = L.d1;
    for (int s = 1; s < kPSmooth; ++s) {
        pdl_launch(k_pmg_step<T>, g, kThreads, st, L, s, s == 1 ? kStepFromZero : kStepRegular, din,
                                              dout, stop);
        std::swap(din, dout);
    }
    pdl_launch(k_pmg_residual<T>, g, kThreads, st, L, stop);
    pdl_launch(k_pmg_restrict<T>, grid_for(c, C.N), kThreads, st, L, C, stop);
    c.launches += kPSmooth + 1;
    pvcycle_level<T>(c, pm, l + 1, st, stop, false);
    pdl_launch(k_pmg_prolong<T>, g, kThreads, st, L, C, stop);
    pdl_launch(k_pmg_resid_first<T>, g, kThreads, st, L, stop);
    c.launches += 2;
    din = L.d0;
    dout = L.d1;
    for (int s = 1; s < kPSmooth; ++s) {
        if (skip_final && s == kPSmooth - 1) break;
        pdl_launch(k_pmg_step<T>, g, kThreads, st, L, s, s == 1 ? kStepAfterFirst : kStepRegular,
                                              din, dout, stop);
        std::swap(din, dout);
        c.launches += 1;
    }
}

template <typename T>
void pmg_vcycle(Ctx& c, PMG<T>& pm, cudaStream_t stream, const int* stop, bool skip_final) {
    pvcycle_level<T>(c, pm, 0, stream, stop, skip_final);
    FTS_CUDA(cudaGetLastError());
}

template <typename T>
void pmg_free(PMG<T>& pm) {
    for (auto& L : pm.L)
        for (void* p : {(void*)L.K, (void*)L.Di, (void*)L.b, (void*)L.x, (void*)L.r, (void*)L.d0,
                        (void*)L.d1})
            if (p) cudaFree(p);
    for (void* p : {(void*)pm.coef, (void*)pm.gersh, (void*)pm.cinv})
        if (p) cudaFree(p);
    if (pm.h_gbits) cudaFreeHost(pm.h_gbits);
    if (pm.h_kc) cudaFreeHost(pm.h_kc);
    if (pm.ev_copied) cudaEventDestroy(pm.ev_copied);
    pm.L.clear();
    pm.coef = nullptr;
    pm.gersh = nullptr;
    pm.cinv = nullptr;
    pm.h_gbits = nullptr;
    pm.h_kc = nullptr;
    pm.ev_copied = nullptr;
    pm.tail_level = -1;
    pm.built = false;
}

template void pmg_setup<double>(Ctx&, PMG<double>&);
template void pmg_setup<float>(Ctx&, PMG<float>&);
template void pmg_build<double>(Ctx&, PMG<double>&);
template void pmg_build<float>(Ctx&, PMG<float>&);
template void pmg_setup_enqueue<double>(Ctx&, PMG<double>&, cudaStream_t);
template void pmg_setup_enqueue<float>(Ctx&, PMG<float>&, cudaStream_t);
template void pmg_setup_finish<double>(Ctx&, PMG<double>&, cudaStream_t);
template void pmg_setup_finish<float>(Ctx&, PMG<float>&, cudaStream_t);
template void pmg_vcycle<double>(Ctx&, PMG<double>&, cudaStream_t, const int*, bool);
template void pmg_vcycle<float>(Ctx&, PMG<float>&, cudaStream_t, const int*, bool);
template void pmg_free<double>(PMG<double>&);
template void pmg_free<float>(PMG<float>&);

}  // namespace fts
