// Geometric multigrid V-cycle for the velocity block K of the Stokes system on
// Kuhn lattices (the preconditioner of MINRES's velocity block; the reference
// has no preconditioner, src/growth/Flow.hpp:62).
//
// Structure.  On an n^3 Kuhn lattice (n odd) the coarse lattice is every other
// node; each fine node is either a coarse node or the midpoint of a coarse
// Kuhn edge, so the prolongation P is linear interpolation with weights 1 or
// 1/2 along the 14 Kuhn directions.  For even n the coarse lattice has n/2 + 1
// nodes per axis and its last layer sits on the fine boundary layer n - 1;
// those nodes are Dirichlet (their rows and columns of P vanish), so the same
// index formulas give the exact Galerkin operator on every interior node.  The Galerkin operator P^T K P keeps the
// 15-point Kuhn stencil.  K is symmetric, so every level stores only the self
// block and the 7 positive-direction 3x3 blocks per node (72 values) in tiles
// of 32 nodes: K[((node/32)*72 + 9d + 3r + c)*32 + node%32]; the block in the
// negative direction -e of node v is the transpose of node (v - e)'s block in
// direction +e.  Every load of a warp is one coalesced segment and no column
// indices are read.
//
// Smoother: Chebyshev polynomial of degree kSmooth in D^-1 K (D = 3x3 node
// blocks) on [lambda/10, lambda], lambda from power iteration; the same
// polynomial before and after the coarse correction keeps the V-cycle
// symmetric positive definite, as MINRES requires.  Coarsest level: Chebyshev
// of degree kCoarse in one CTA.
#include <cmath>
#include <cstring>
#include <vector>

#include "fts_device.cuh"
#include "mg.cuh"
#include "reduce.cuh"

namespace fts {

__constant__ int c_off[15][3];
__constant__ int c_gal_start[16];
__constant__ unsigned short c_gal_term[512];  // a | e << 4 | (weight code) << 8
__constant__ float c_gal_w[512];

static const int kOff[15][3] = {{0, 0, 0},  {1, 0, 0},   {0, 1, 0},   {0, 0, 1},   {1, 1, 0},
                                {1, 0, 1},  {0, 1, 1},   {1, 1, 1},   {-1, 0, 0},  {0, -1, 0},
                                {0, 0, -1}, {-1, -1, 0}, {-1, 0, -1}, {0, -1, -1}, {-1, -1, -1}};

static int dir_index(int dx, int dy, int dz) {
    for (int d = 0; d < 15; ++d)
        if (kOff[d][0] == dx && kOff[d][1] == dy && kOff[d][2] == dz) return d;
    return -1;
}

// Galerkin term table: coarse block (I, I + off[dJ]) = sum over terms (a, e, w)
// of w * K_f(f, dir e) with f = 2I + off[a], g = f + off[e] a child of I + off[dJ].
static void init_tables(int device) {
    static bool done[64] = {};
    if (device < 64 && done[device]) return;
    std::vector<int> start(16, 0);
    std::vector<unsigned short> term;
    std::vector<float> w;
    for (int dJ = 0; dJ < 15; ++dJ) {
        start[dJ] = (int)term.size();
        for (int a = 0; a < 15; ++a) {
            double wf = a == 0 ? 1.0 : 0.5;
            for (int e = 0; e < 15; ++e) {
                int q[3];
                for (int k = 0; k < 3; ++k) q[k] = kOff[a][k] + kOff[e][k] - 2 * kOff[dJ][k];
                int qi = dir_index(q[0], q[1], q[2]);
                if (qi < 0) continue;
                double wg = qi == 0 ? 1.0 : 0.5;
                term.push_back((unsigned short)(a | (e << 4)));
                w.push_back((float)(wf * wg));
            }
        }
    }
    start[15] = (int)term.size();
    FTS_CUDA(cudaMemcpyToSymbol(c_off, kOff, sizeof(kOff)));
    FTS_CUDA(cudaMemcpyToSymbol(c_gal_start, start.data(), 16 * sizeof(int)));
    FTS_CUDA(cudaMemcpyToSymbol(c_gal_term, term.data(), term.size() * sizeof(unsigned short)));
    FTS_CUDA(cudaMemcpyToSymbol(c_gal_w, w.data(), w.size() * sizeof(float)));
    if (device < 64) done[device] = true;
}

// Tiled stencil layout: 32 consecutive nodes share one tile of kStored x 32
// values (entry q = 9 d + 3 r + c, d = 0..7), so the loads of a warp stay
// inside one contiguous 9 KB (FP32) region.
constexpr int kStored = 72;
__device__ __forceinline__ int64_t kidx(int q, int64_t v) {
    return ((v >> 5) * kStored + q) * 32 + (v & 31);
}

// Entry x = 3r + c of the block K(f, f + off[e]) for any of the 15 directions.
template <typename T>
__device__ __forceinline__ T kblock(const T* __restrict__ K, int e, int x, int64_t f, int n) {
    if (e < 8) return K[kidx(9 * e + x, f)];
    const int ep = e - 7;  // positive direction; the block is stored at f - off[ep]
    const int64_t w = f - (c_off[ep][0] + (int64_t)n * (c_off[ep][1] + (int64_t)n * c_off[ep][2]));
    return K[kidx(9 * ep + 3 * (x % 3) + x / 3, w)];
}

__device__ __forceinline__ int nbr(int i, int j, int k, int d, int n) {
    int a = i + c_off[d][0], b = j + c_off[d][1], c = k + c_off[d][2];
    if (a < 0 || b < 0 || c < 0 || a >= n || b >= n || c >= n) return -1;
    return a + n * (b + n * c);
}

// ---------------------------------------------------------------------------
// Set-up kernels
// ---------------------------------------------------------------------------

// Fine level: velocity 3x3 part of the assembled node blocks, per direction.
template <typename T>
__global__ void k_mg_extract(int n, const int32_t* __restrict__ rowptr,
                             const int32_t* __restrict__ cols, const double* __restrict__ A,
                             T* __restrict__ K) {
    const int64_t N = (int64_t)n * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((int64_t)n * n));
        const int w = nbr(i, j, k, d, n);
        double blk[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (w >= 0) {
            int lo = rowptr[v], hi = rowptr[v + 1] - 1;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (cols[mid] < w) lo = mid + 1;
                else hi = mid;
            }
            if (cols[lo] == w) {
                const double* b = A + (int64_t)lo * 16;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) blk[3 * r + c] = b[4 * r + c];
            }
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) K[kidx(d * 9 + e, v)] = (T)blk[e];
    }
}

// Fine level straight from the elements (matrix-free mode: no block matrix
// exists).  One thread per (node v, stored direction d): the 3x3 block
// K(v, v + off[d]) = sum over elements holding both nodes of
// mu vol (delta_rc g_a.g_b + g_a[c] g_b[r]) (Flow.cpp:136-153); Dirichlet rows
// identity, Dirichlet columns zero.
template <typename T>
__global__ void k_mg_from_elements(int n, const int32_t* __restrict__ p2t_ptr,
                                   const uint32_t* __restrict__ p2t,
                                   const int32_t* __restrict__ tets,
                                   const ElemGeom* __restrict__ geom,
                                   const double* __restrict__ mu,
                                   const uint8_t* __restrict__ bnd, T* __restrict__ K) {
    const int64_t N = (int64_t)n * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((int64_t)n * n));
        const int w = nbr(i, j, k, d, n);
        double blk[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (bnd[v]) {
            if (d == 0) blk[0] = blk[4] = blk[8] = 1.0;
        } else if (w >= 0 && !bnd[w]) {
            for (int32_t q = p2t_ptr[v]; q < p2t_ptr[v + 1]; ++q) {
                const uint32_t e = p2t[q];
                const int64_t el = e >> 2;
                const int a = e & 3;
                const int4 tt = reinterpret_cast<const int4*>(tets)[el];
                const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
                int b = -1;
#pragma unroll
                for (int m = 0; m < 4; ++m)
                    if (ids[m] == w) b = m;
                if (b < 0) continue;
                const ElemGeom& G = geom[el];
                const double mv = mu[el] * G.vol;
                const double gg = G.g[a][0] * G.g[b][0] + G.g[a][1] * G.g[b][1] + G.g[a][2] * G.g[b][2];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int cc = 0; cc < 3; ++cc)
                        blk[3 * r + cc] += mv * ((r == cc ? gg : 0.0) + G.g[a][cc] * G.g[b][r]);
            }
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) K[kidx(d * 9 + e, v)] = (T)blk[e];
    }
}

// Dirichlet mask of a coarse level: node I is Dirichlet when the fine node 2I is.
__global__ void k_mg_coarse_mask(int nf, const uint8_t* __restrict__ mf, int nc,
                                 uint8_t* __restrict__ mc) {
    const int64_t Nc = (int64_t)nc * nc * nc;
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < Nc;
         v += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(v % nc), j = (int)((v / nc) % nc), k = (int)(v / ((int64_t)nc * nc));
        // coarse node I sits on fine node min(2I, nf-1): for even nf the last
        // coarse layer is the fine boundary layer
        const int fi = min(2 * i, nf - 1), fj = min(2 * j, nf - 1), fk = min(2 * k, nf - 1);
        mc[v] = mf[fi + nf * (fj + (int64_t)nf * fk)];
    }
}

// Galerkin coarse operator, one thread per (coarse node, coarse direction).
template <typename T>
__global__ void k_mg_galerkin(int nf, const T* __restrict__ Kf, const uint8_t* __restrict__ mf,
                              int nc, T* __restrict__ Kc, const uint8_t* __restrict__ mc) {
    const int64_t Nf = (int64_t)nf * nf * nf, Nc = (int64_t)nc * nc * nc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Nc * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int dJ = (int)(t / Nc);
        const int64_t I = t - dJ * Nc;
        const int ci = (int)(I % nc), cj = (int)((I / nc) % nc), ck = (int)(I / ((int64_t)nc * nc));
        T acc[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) acc[e] = T(0);
        const int J = nbr(ci, cj, ck, dJ, nc);
        if (mc[I]) {
            if (dJ == 0) acc[0] = acc[4] = acc[8] = T(1);
        } else if (J >= 0 && !mc[J]) {
            for (int q = c_gal_start[dJ]; q < c_gal_start[dJ + 1]; ++q) {
                const int a = c_gal_term[q] & 15, e = (c_gal_term[q] >> 4) & 15;
                const int fi = 2 * ci + c_off[a][0], fj = 2 * cj + c_off[a][1],
                          fk = 2 * ck + c_off[a][2];
                if (fi < 0 || fj < 0 || fk < 0 || fi >= nf || fj >= nf || fk >= nf) continue;
                const int64_t f = fi + (int64_t)nf * (fj + (int64_t)nf * fk);
                if (mf[f]) continue;
                const int g = nbr(fi, fj, fk, e, nf);
                if (g < 0 || mf[g]) continue;
                const T w = (T)c_gal_w[q];
#pragma unroll
                for (int x = 0; x < 9; ++x) acc[x] += w * kblock<T>(Kf, e, x, f, nf);
            }
        }
        if (dJ == 0) {  // the self block of a symmetric operator: symmetrise rounding
            T s01 = T(0.5) * (acc[1] + acc[3]), s02 = T(0.5) * (acc[2] + acc[6]),
              s12 = T(0.5) * (acc[5] + acc[7]);
            acc[1] = acc[3] = s01;
            acc[2] = acc[6] = s02;
            acc[5] = acc[7] = s12;
        }
#pragma unroll
        for (int x = 0; x < 9; ++x) Kc[kidx(dJ * 9 + x, I)] = acc[x];
    }
}

// Inverse of the symmetric 3x3 node block (D^-1), 6 values per node (SoA).
template <typename T>
__global__ void k_mg_dinv(int64_t N, const T* __restrict__ K, T* __restrict__ Dinv) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < N;
         v += (int64_t)gridDim.x * blockDim.x) {
        double a00 = K[kidx(0, v)], a11 = K[kidx(4, v)], a22 = K[kidx(8, v)];
        double a01 = 0.5 * ((double)K[kidx(1, v)] + (double)K[kidx(3, v)]);
        double a02 = 0.5 * ((double)K[kidx(2, v)] + (double)K[kidx(6, v)]);
        double a12 = 0.5 * ((double)K[kidx(5, v)] + (double)K[kidx(7, v)]);
        double c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22;
        double c02 = a01 * a12 - a02 * a11, c11 = a00 * a22 - a02 * a02;
        double c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
        double det = a00 * c00 + a01 * c01 + a02 * c02;
        double id = det != 0.0 ? 1.0 / det : 0.0;
        Dinv[0 * N + v] = (T)(c00 * id);
        Dinv[1 * N + v] = (T)(c01 * id);
        Dinv[2 * N + v] = (T)(c02 * id);
        Dinv[3 * N + v] = (T)(c11 * id);
        Dinv[4 * N + v] = (T)(c12 * id);
        Dinv[5 * N + v] = (T)(c22 * id);
    }
}

// y = K x at node v (3 components); x SoA [3][N].  32-bit lattice
// coordinates; interior nodes take the neighbour offsets without range checks.
template <typename T>
__device__ __forceinline__ void stencil_apply(int n, int64_t N, int64_t v64,
                                              const T* __restrict__ K,
                                              const T* __restrict__ x, T y[3]) {
    const int v = (int)v64;
    const int nn = n * n;
    const int k = v / nn;
    const int rem = v - k * nn;
    const int j = rem / n;
    const int i = rem - j * n;
    const bool inner = i > 0 && j > 0 && k > 0 && i < n - 1 && j < n - 1 && k < n - 1;
    T a0 = T(0), a1 = T(0), a2 = T(0);
#pragma unroll
    for (int d = 0; d < 8; ++d) {  // self and positive directions: own blocks
        const int w = inner ? v + c_off[d][0] + n * c_off[d][1] + nn * c_off[d][2]
                            : nbr(i, j, k, d, n);
        if (w < 0) continue;
        const T x0 = x[w], x1 = x[N + w], x2 = x[2 * N + w];
        const T* kb = K + kidx(d * 9, v64);
        a0 = fma(kb[0], x0, fma(kb[32], x1, fma(kb[64], x2, a0)));
        a1 = fma(kb[96], x0, fma(kb[128], x1, fma(kb[160], x2, a1)));
        a2 = fma(kb[192], x0, fma(kb[224], x1, fma(kb[256], x2, a2)));
    }
#pragma unroll
    for (int d = 1; d < 8; ++d) {  // negative directions: neighbour's block, transposed
        const int w = inner ? v - c_off[d][0] - n * c_off[d][1] - nn * c_off[d][2]
                            : nbr(i, j, k, d + 7, n);
        if (w < 0) continue;
        const T x0 = x[w], x1 = x[N + w], x2 = x[2 * N + w];
        const T* kb = K + kidx(d * 9, (int64_t)w);
        a0 = fma(kb[0], x0, fma(kb[96], x1, fma(kb[192], x2, a0)));
        a1 = fma(kb[32], x0, fma(kb[128], x1, fma(kb[224], x2, a1)));
        a2 = fma(kb[64], x0, fma(kb[160], x1, fma(kb[256], x2, a2)));
    }
    y[0] = a0;
    y[1] = a1;
    y[2] = a2;
}

template <typename T>
__device__ __forceinline__ void dinv_apply(int64_t N, int64_t v, const T* __restrict__ Di,
                                           const T r[3], T z[3]) {
    const T d0 = Di[v], d1 = Di[N + v], d2 = Di[2 * N + v], d3 = Di[3 * N + v],
            d4 = Di[4 * N + v], d5 = Di[5 * N + v];
    z[0] = d0 * r[0] + d1 * r[1] + d2 * r[2];
    z[1] = d1 * r[0] + d3 * r[1] + d4 * r[2];
    z[2] = d2 * r[0] + d4 * r[1] + d5 * r[2];
}

// Power iteration step: w = D^-1 K v / ||v||; the norm of w goes to lam[l].
template <typename T>
__global__ void k_mg_power(int n, const T* __restrict__ K, const T* __restrict__ Di,
                           const uint8_t* __restrict__ mask, const T* __restrict__ v,
                           T* __restrict__ w, double* __restrict__ nrm, int first, Reduction red) {
    const int64_t N = (int64_t)n * n * n;
    const double inv = first ? 1.0 : (*nrm > 0.0 ? 1.0 / *nrm : 0.0);
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        T y[3], z[3];
        stencil_apply<T>(n, N, i, K, v, y);
        dinv_apply<T>(N, i, Di, y, z);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            T o = mask[i] ? T(0) : (T)(z[c] * inv);
            w[c * N + i] = o;
            acc[0] += (double)o * (double)o;
        }
    }
    double tot[1];
    if (grid_sum<1>(acc, red, tot) && threadIdx.x == 0) *nrm = sqrt(tot[0]);
}

// Deterministic start vector for the power iteration (zero on Dirichlet nodes).
template <typename T>
__global__ void k_mg_power_init(int64_t N, const uint8_t* __restrict__ mask, T* __restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        uint32_t h = (uint32_t)(i * 2654435761u) ^ 0x9E3779B9u;
        for (int c = 0; c < 3; ++c) {
            h = h * 1664525u + 1013904223u;
            v[c * N + i] = mask[i] ? T(0) : (T)(0.5 + (double)(h >> 8) / 16777216.0);
        }
    }
}

// ---------------------------------------------------------------------------
// V-cycle kernels.  All skip when the MINRES run has stopped (*stop != 0).
// Chebyshev on [lmin, lmax] = [lambda*kLowFrac, lambda]:
//   theta = (lmax+lmin)/2, delta = (lmax-lmin)/2, sigma = theta/delta,
//   rho_0 = 1/sigma, rho_i = 1/(2 sigma - rho_{i-1});
//   d_0 = D^-1 r / theta;  d_i = rho_i rho_{i-1} d_{i-1} + (2 rho_i/delta) D^-1 r_i.
// ---------------------------------------------------------------------------
constexpr double kLowFrac = 0.1;
constexpr int kCoefStride = 64;      // per level: 1/theta, then (ca_s, cb_s) for s >= 1
constexpr int kCoarseThreads = 256;  // one CTA for the coarsest level (<= 9^3 nodes)

// Chebyshev coefficients of one level, computed once per solve on the host.
static void cheb_table(double lam, double* out) {
    const double lmax = lam, lmin = lam * kLowFrac;
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

// First smoothing step.  has_x = 0: from x = 0 (r = b, x = d).  has_x = 1: r
// already holds b - K x (computed by k_mg_residual, so that no thread reads x
// at a neighbour while x is updated here); x += d.
template <typename T>
__global__ void k_mg_smooth_first(int n, const T* __restrict__ K, const T* __restrict__ Di,
                                  const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                                  T* __restrict__ d, const double* __restrict__ coef, int has_x,
                                  const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t N = (int64_t)n * n * n;
    const T ith = (T)coef[0];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        T rr[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) rr[c] = has_x ? r[c * N + i] : b[c * N + i];
        T z[3];
        dinv_apply<T>(N, i, Di, rr, z);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            r[c * N + i] = rr[c];
            const T dd = z[c] * ith;
            d[c * N + i] = dd;
            x[c * N + i] = has_x ? x[c * N + i] + dd : dd;
        }
    }
}

// Later smoothing steps: r -= K d_in; d_out = ca d_in + cb D^-1 r; x += d_out.
// (has_x kernels must not read x at neighbours while another thread updates it:
// x is only touched at the thread's own node here.)
template <typename T>
__global__ void __launch_bounds__(kThreads, 4) k_mg_smooth_step(int n, const T* __restrict__ K, const T* __restrict__ Di,
                                 const T* __restrict__ din, T* __restrict__ dout,
                                 T* __restrict__ r, T* __restrict__ x,
                                 const double* __restrict__ coef, int step,
                                 const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t N = (int64_t)n * n * n;
    const T A = (T)coef[2 * step - 1], B = (T)coef[2 * step];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        T y[3], rr[3], z[3];
        stencil_apply<T>(n, N, i, K, din, y);
#pragma unroll
        for (int c = 0; c < 3; ++c) rr[c] = r[c * N + i] - y[c];
        dinv_apply<T>(N, i, Di, rr, z);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            r[c * N + i] = rr[c];
            const T dd = A * din[c * N + i] + B * z[c];
            dout[c * N + i] = dd;
            x[c * N + i] += dd;
        }
    }
}

// r = b - K x
template <typename T>
__global__ void __launch_bounds__(kThreads, 4) k_mg_residual(int n, const T* __restrict__ K, const T* __restrict__ b,
                              const T* __restrict__ x, T* __restrict__ r,
                              const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t N = (int64_t)n * n * n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        T y[3];
        stencil_apply<T>(n, N, i, K, x, y);
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c * N + i] = b[c * N + i] - y[c];
    }
}

// b_c(I) = sum_a w_a r_f(2I + off[a])  (P^T r), zero on Dirichlet nodes.
template <typename T>
__global__ void k_mg_restrict(int nf, const T* __restrict__ rf, const uint8_t* __restrict__ mf,
                              int nc, T* __restrict__ bc, const uint8_t* __restrict__ mc,
                              const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t Nf = (int64_t)nf * nf * nf, Nc = (int64_t)nc * nc * nc;
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < Nc;
         I += (int64_t)gridDim.x * blockDim.x) {
        T a0 = T(0), a1 = T(0), a2 = T(0);
        if (!mc[I]) {
            const int ci = (int)(I % nc), cj = (int)((I / nc) % nc),
                      ck = (int)(I / ((int64_t)nc * nc));
#pragma unroll
            for (int a = 0; a < 15; ++a) {
                const int f = nbr(2 * ci, 2 * cj, 2 * ck, a, nf);
                if (f < 0 || mf[f]) continue;
                const T w = a == 0 ? T(1) : T(0.5);
                a0 += w * rf[f];
                a1 += w * rf[Nf + f];
                a2 += w * rf[2 * Nf + f];
            }
        }
        bc[I] = a0;
        bc[Nc + I] = a1;
        bc[2 * Nc + I] = a2;
    }
}

// x_f(f) += sum_{parents J} w x_c(J)  (P e)
template <typename T>
__global__ void k_mg_prolong(int nf, T* __restrict__ xf, const uint8_t* __restrict__ mf, int nc,
                             const T* __restrict__ xc, const uint8_t* __restrict__ mc,
                             const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t Nf = (int64_t)nf * nf * nf, Nc = (int64_t)nc * nc * nc;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < Nf;
         f += (int64_t)gridDim.x * blockDim.x) {
        if (mf[f]) continue;
        const int fi = (int)(f % nf), fj = (int)((f / nf) % nf), fk = (int)(f / ((int64_t)nf * nf));
        const int Ai = fi >> 1, Aj = fj >> 1, Ak = fk >> 1;
        const int oi = fi & 1, oj = fj & 1, ok = fk & 1;
        T s0 = T(0), s1 = T(0), s2 = T(0);
        const int64_t A = Ai + (int64_t)nc * (Aj + (int64_t)nc * Ak);
        if ((oi | oj | ok) == 0) {
            if (!mc[A]) {
                s0 = xc[A];
                s1 = xc[Nc + A];
                s2 = xc[2 * Nc + A];
            }
        } else {
            const int64_t Bn = (Ai + oi) + (int64_t)nc * ((Aj + oj) + (int64_t)nc * (Ak + ok));
            if (!mc[A]) {
                s0 += T(0.5) * xc[A];
                s1 += T(0.5) * xc[Nc + A];
                s2 += T(0.5) * xc[2 * Nc + A];
            }
            if (!mc[Bn]) {
                s0 += T(0.5) * xc[Bn];
                s1 += T(0.5) * xc[Nc + Bn];
                s2 += T(0.5) * xc[2 * Nc + Bn];
            }
        }
        xf[f] += s0;
        xf[Nf + f] += s1;
        xf[2 * Nf + f] += s2;
    }
}

// Coarsest level: kCoarse Chebyshev steps from zero in a single CTA.
template <typename T>
__global__ void __launch_bounds__(kCoarseThreads) k_mg_coarse_solve(int n, const T* __restrict__ K, const T* __restrict__ Di,
                                  const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                                  T* __restrict__ d0, T* __restrict__ d1,
                                  const double* __restrict__ coef, int steps,
                                  const int* __restrict__ stop) {
    if (stop && *stop) return;
    const int64_t N = (int64_t)n * n * n;
    const T ith = (T)coef[0];
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
        T rr[3], z[3];
        for (int c = 0; c < 3; ++c) rr[c] = b[c * N + i];
        dinv_apply<T>(N, i, Di, rr, z);
        for (int c = 0; c < 3; ++c) {
            r[c * N + i] = rr[c];
            d0[c * N + i] = z[c] * ith;
            x[c * N + i] = z[c] * ith;
        }
    }
    __syncthreads();
    for (int s = 1; s < steps; ++s) {
        const T A = (T)coef[2 * s - 1], B = (T)coef[2 * s];
        const T* din = (s & 1) ? d0 : d1;
        T* dout = (s & 1) ? d1 : d0;
        for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
            T y[3], rr[3], z[3];
            stencil_apply<T>(n, N, i, K, din, y);
            for (int c = 0; c < 3; ++c) rr[c] = r[c * N + i] - y[c];
            dinv_apply<T>(N, i, Di, rr, z);
            for (int c = 0; c < 3; ++c) {
                r[c * N + i] = rr[c];
                const T dd = A * din[c * N + i] + B * z[c];
                dout[c * N + i] = dd;
                x[c * N + i] += dd;
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <typename T>
void mg_build(Ctx& c, MG<T>& mg) {
    if (mg.built) return;
    init_tables(c.device);
    const int n0 = c.topo.lattice_n;
    int n = n0;
    while (true) {
        MGLevel<T> L;
        L.n = n;
        L.N = (int64_t)n * n * n;
        L.K = dev_alloc<T>(c, (size_t)((L.N + 31) / 32) * 32 * kStored);
        L.Di = dev_alloc<T>(c, (size_t)L.N * 6);
        for (auto** p : {&L.b, &L.x, &L.r, &L.d0, &L.d1}) *p = dev_alloc<T>(c, (size_t)L.N * 3);
        L.mask = dev_alloc<uint8_t>(c, (size_t)L.N);
        mg.L.push_back(L);
        if (n < 5) break;
        n = mg_coarse_n(n);
    }
    mg.lam = dev_alloc<double>(c, mg.L.size() + 1);
    mg.coef = dev_alloc<double>(c, mg.L.size() * kCoefStride);
    FTS_CUDA(cudaMemcpyAsync(mg.L[0].mask, c.bnd, (size_t)mg.L[0].N, cudaMemcpyDeviceToDevice,
                             c.stream));
    for (size_t l = 1; l < mg.L.size(); ++l) {
        k_mg_coarse_mask<<<grid_for(c, mg.L[l].N), kThreads, 0, c.stream>>>(
            mg.L[l - 1].n, mg.L[l - 1].mask, mg.L[l].n, mg.L[l].mask);
        c.launches += 1;
    }
    FTS_CUDA(cudaGetLastError());
    mg.built = true;
}

// Per-solve set-up after assembly: fine operator, Galerkin hierarchy, D^-1,
// lambda_max per level.
template <typename T>
void mg_setup(Ctx& c, MG<T>& mg) {
    mg_build<T>(c, mg);
    MGLevel<T>& F = mg.L[0];
    if (c.matfree)
        k_mg_from_elements<T><<<grid_for(c, F.N * 8), kThreads, 0, c.stream>>>(
            F.n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.bnd, F.K);
    else
        k_mg_extract<T><<<grid_for(c, F.N * 8), kThreads, 0, c.stream>>>(F.n, c.rowptr, c.cols,
                                                                           c.A64, F.K);
    c.launches += 1;
    for (size_t l = 0; l < mg.L.size(); ++l) {
        MGLevel<T>& L = mg.L[l];
        if (l > 0) {
            MGLevel<T>& P = mg.L[l - 1];
            k_mg_galerkin<T><<<grid_for(c, L.N * 8), kThreads, 0, c.stream>>>(P.n, P.K, P.mask,
                                                                               L.n, L.K, L.mask);
            c.launches += 1;
        }
        k_mg_dinv<T><<<grid_for(c, L.N), kThreads, 0, c.stream>>>(L.N, L.K, L.Di);
        k_mg_power_init<T><<<grid_for(c, L.N), kThreads, 0, c.stream>>>(L.N, L.mask, L.d0);
        c.launches += 2;
        T* v = L.d0;
        T* w = L.d1;
        for (int it = 0; it < kPowerIters; ++it) {
            k_mg_power<T><<<grid_for(c, L.N), kThreads, 0, c.stream>>>(
                L.n, L.K, L.Di, L.mask, v, w, mg.lam + l, it == 0, c.red);
            c.launches += 1;
            T* t = v;
            v = w;
            w = t;
        }
    }
    FTS_CUDA(cudaGetLastError());
    // lambda_max ~ ||D^-1 K v|| for the normalised v of the last step; scale by
    // the safety factor on the host copy and write back.
    std::vector<double> lam(mg.L.size());
    FTS_CUDA(cudaMemcpyAsync(lam.data(), mg.lam, lam.size() * sizeof(double),
                             cudaMemcpyDeviceToHost, c.stream));
    FTS_CUDA(cudaStreamSynchronize(c.stream));
    // The power iteration normalises by the previous norm; the first step uses
    // the raw start vector, so use the last ratio only.
    for (auto& x : lam) x = (x > 0.0 && std::isfinite(x) ? x : 2.5) * kLamSafety;
    mg.lam_host = lam;
    std::vector<double> coef(lam.size() * kCoefStride);
    for (size_t l = 0; l < lam.size(); ++l) cheb_table(lam[l], coef.data() + l * kCoefStride);
    // A 3^3 coarsest lattice has a single interior node: x = D^-1 b is exact.
    if (mg.L.back().n == 3) coef[(lam.size() - 1) * kCoefStride] = 1.0;
    FTS_CUDA(cudaMemcpyAsync(mg.coef, coef.data(), coef.size() * sizeof(double),
                             cudaMemcpyHostToDevice, c.stream));
    FTS_CUDA(cudaStreamSynchronize(c.stream));
}

template <typename T>
static void vcycle_level(Ctx& c, MG<T>& mg, size_t l, const int* stop) {
    MGLevel<T>& L = mg.L[l];
    const int g = grid_for(c, L.N);
    const double* lam = mg.coef + l * kCoefStride;
    if (l + 1 == mg.L.size()) {
        k_mg_coarse_solve<T><<<1, kCoarseThreads, 0, c.stream>>>(
            L.n, L.K, L.Di, L.b, L.x, L.r, L.d0, L.d1, lam, L.n == 3 ? 1 : kCoarse, stop);
        c.launches += 1;
        return;
    }
    MGLevel<T>& C = mg.L[l + 1];
    // pre-smoothing from zero
    k_mg_smooth_first<T><<<g, kThreads, 0, c.stream>>>(L.n, L.K, L.Di, L.b, L.x, L.r, L.d0, lam,
                                                      0, stop);
    T* din = L.d0;
    T* dout = L.d1;
    for (int s = 1; s < kSmooth; ++s) {
        k_mg_smooth_step<T><<<g, kThreads, 0, c.stream>>>(L.n, L.K, L.Di, din, dout, L.r, L.x,
                                                         lam, s, stop);
        T* t = din;
        din = dout;
        dout = t;
    }
    k_mg_residual<T><<<g, kThreads, 0, c.stream>>>(L.n, L.K, L.b, L.x, L.r, stop);
    k_mg_restrict<T><<<grid_for(c, C.N), kThreads, 0, c.stream>>>(L.n, L.r, L.mask, C.n, C.b,
                                                                 C.mask, stop);
    c.launches += kSmooth + 2;
    vcycle_level<T>(c, mg, l + 1, stop);
    k_mg_prolong<T><<<g, kThreads, 0, c.stream>>>(L.n, L.x, L.mask, C.n, C.x, C.mask, stop);
    // post-smoothing from the corrected x
    k_mg_residual<T><<<g, kThreads, 0, c.stream>>>(L.n, L.K, L.b, L.x, L.r, stop);
    k_mg_smooth_first<T><<<g, kThreads, 0, c.stream>>>(L.n, L.K, L.Di, L.b, L.x, L.r, L.d0, lam,
                                                      1, stop);
    din = L.d0;
    dout = L.d1;
    for (int s = 1; s < kSmooth; ++s) {
        k_mg_smooth_step<T><<<g, kThreads, 0, c.stream>>>(L.n, L.K, L.Di, din, dout, L.r, L.x,
                                                         lam, s, stop);
        T* t = din;
        din = dout;
        dout = t;
    }
    c.launches += kSmooth + 2;
}

template <typename T>
void mg_vcycle(Ctx& c, MG<T>& mg, const int* stop) {
    vcycle_level<T>(c, mg, 0, stop);
    FTS_CUDA(cudaGetLastError());
}

template <typename T>
void mg_free(MG<T>& mg) {
    for (auto& L : mg.L)
        for (void* p : {(void*)L.K, (void*)L.Di, (void*)L.b, (void*)L.x, (void*)L.r, (void*)L.d0,
                        (void*)L.d1, (void*)L.mask})
            if (p) cudaFree(p);
    if (mg.lam) cudaFree(mg.lam);
    if (mg.coef) cudaFree(mg.coef);
    mg.coef = nullptr;
    mg.L.clear();
    mg.lam = nullptr;
    mg.built = false;
}

template void mg_setup<double>(Ctx&, MG<double>&);
template void mg_setup<float>(Ctx&, MG<float>&);
template void mg_vcycle<double>(Ctx&, MG<double>&, const int*);
template void mg_vcycle<float>(Ctx&, MG<float>&, const int*);
template void mg_free<double>(MG<double>&);
template void mg_free<float>(MG<float>&);

}  // namespace fts
