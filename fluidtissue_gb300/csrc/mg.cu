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
//
// Precision.  The FP32 hierarchy is built in FP32 (Galerkin products, D^-1)
// and the V-cycle then reads an FP16 copy of every stencil, scaled per level so
// that max |K| maps to 16384; the arithmetic stays FP32.  The stored half
// stencil is symmetric by construction, so the V-cycle stays an SPD
// preconditioner, of the FP16-rounded operator.  The FP64 hierarchy reads its
// FP64 stencils.
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include <cooperative_groups.h>

#include "fts_device.cuh"
#include "mg.cuh"
#include "mg_device.cuh"
#include "reduce.cuh"

namespace fts {

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
void galerkin_terms(std::vector<int>& start, std::vector<unsigned short>& term,
                    std::vector<float>& w) {
    start.assign(16, 0);
    term.clear();
    w.clear();
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
}

static void init_tables(int device) {
    static bool done[64] = {};
    if (device < 64 && done[device]) return;
    std::vector<int> start;
    std::vector<unsigned short> term;
    std::vector<float> w;
    galerkin_terms(start, term, w);
    FTS_CUDA(cudaMemcpyToSymbol(c_gal_start, start.data(), 16 * sizeof(int)));
    FTS_CUDA(cudaMemcpyToSymbol(c_gal_term, term.data(), term.size() * sizeof(unsigned short)));
    FTS_CUDA(cudaMemcpyToSymbol(c_gal_w, w.data(), w.size() * sizeof(float)));
    if (device < 64) done[device] = true;
}

// Entry x = 3r + c of the block K(f, f + off[e]) for any of the 15 directions.
template <typename T>
__device__ __forceinline__ T kblock(const T* __restrict__ K, int e, int x, int64_t f, int n) {
    if (e < 8) return K[kidx(9 * e + x, f)];
    const int ep = e - 7;  // positive direction; the block is stored at f - off[ep]
    const int64_t w = f - (off_x(ep) + (int64_t)n * (off_y(ep) + (int64_t)n * off_z(ep)));
    return K[kidx(9 * ep + 3 * (x % 3) + x / 3, w)];
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

// Fine level from the FP64 lattice half stencil: the velocity 3x3 part of the
// same 8 blocks per node.
template <typename T>
__global__ void k_mg_extract_lat(int n, const double2* __restrict__ L, T* __restrict__ K) {
    const int64_t N = (int64_t)n * n * n;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const double2 u = L[lat64_idx(d, r, 0, v)], w = L[lat64_idx(d, r, 1, v)];
            K[kidx(d * 9 + 3 * r, v)] = (T)u.x;
            K[kidx(d * 9 + 3 * r + 1, v)] = (T)u.y;
            K[kidx(d * 9 + 3 * r + 2, v)] = (T)w.x;
        }
    }
}

// Fine level straight from the elements (matrix-free mode: no block matrix
// exists).  One thread per (node v, stored direction d): the 3x3 block
// K(v, v + off[d]) = sum over elements holding both nodes of
// mu vol (delta_rc g_a.g_b + g_a[c] g_b[r]) (Flow.cpp:136-153); Dirichlet rows
// identity, Dirichlet columns zero.
template <typename T, bool KUHN>
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
            auto add = [&](int64_t el, int a, int b) {
                const ElemGeom& G = geom[el];
                const double mv = mu[el] * G.vol;
                const double gg = G.g[a][0] * G.g[b][0] + G.g[a][1] * G.g[b][1] + G.g[a][2] * G.g[b][2];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int cc = 0; cc < 3; ++cc)
                        blk[3 * r + cc] += mv * ((r == cc ? gg : 0.0) + G.g[a][cc] * G.g[b][r]);
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

// Galerkin coarse operator, one thread per (coarse node, coarse direction);
// the self block (115 terms against 15..27 for the others) is split over
// kGalSelfSplit threads whose partial sums k_mg_galerkin_self adds, so no
// thread walks far more terms than the rest.
constexpr int kGalSelfSplit = 4;

template <typename T>
__global__ void k_mg_galerkin(int nf, const T* __restrict__ Kf, const uint8_t* __restrict__ mf,
                              int nc, T* __restrict__ Kc, const uint8_t* __restrict__ mc,
                              T* __restrict__ self_part) {
    const int64_t Nf = (int64_t)nf * nf * nf, Nc = (int64_t)nc * nc * nc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < Nc * (7 + kGalSelfSplit);
         t += (int64_t)gridDim.x * blockDim.x) {
        const int vd = (int)(t / Nc);
        const int64_t I = t - vd * Nc;
        const int dJ = vd < kGalSelfSplit ? 0 : vd - kGalSelfSplit + 1;
        int q0 = c_gal_start[dJ], q1 = c_gal_start[dJ + 1];
        if (dJ == 0) {
            const int len = q1 - q0;
            q1 = q0 + (vd + 1) * len / kGalSelfSplit;
            q0 = q0 + vd * len / kGalSelfSplit;
        }
        const int ci = (int)(I % nc), cj = (int)((I / nc) % nc), ck = (int)(I / ((int64_t)nc * nc));
        T acc[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) acc[e] = T(0);
        const int J = nbr(ci, cj, ck, dJ, nc);
        if (!mc[I] && J >= 0 && !mc[J]) {
            for (int q = q0; q < q1; ++q) {
                const int a = c_gal_term[q] & 15, e = (c_gal_term[q] >> 4) & 15;
                const int fi = 2 * ci + off_x(a), fj = 2 * cj + off_y(a), fk = 2 * ck + off_z(a);
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
        if (dJ == 0) {
#pragma unroll
            for (int x = 0; x < 9; ++x) self_part[((int64_t)vd * 9 + x) * Nc + I] = acc[x];
        } else {
#pragma unroll
            for (int x = 0; x < 9; ++x) Kc[kidx(dJ * 9 + x, I)] = acc[x];
        }
    }
}

// The self blocks of a Galerkin product: the partial sums in a fixed order,
// identity on Dirichlet nodes, the symmetric part (symmetrising rounding).
template <typename T>
__global__ void k_mg_galerkin_self(int nc, const T* __restrict__ self_part, T* __restrict__ Kc,
                                   const uint8_t* __restrict__ mc) {
    const int64_t Nc = (int64_t)nc * nc * nc;
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < Nc;
         I += (int64_t)gridDim.x * blockDim.x) {
        T acc[9];
#pragma unroll
        for (int x = 0; x < 9; ++x) {
            T s = T(0);
            for (int p = 0; p < kGalSelfSplit; ++p) s += self_part[((int64_t)p * 9 + x) * Nc + I];
            acc[x] = s;
        }
        if (mc[I]) {
#pragma unroll
            for (int x = 0; x < 9; ++x) acc[x] = (x % 4 == 0) ? T(1) : T(0);
        } else {
            const T s01 = T(0.5) * (acc[1] + acc[3]), s02 = T(0.5) * (acc[2] + acc[6]),
                    s12 = T(0.5) * (acc[5] + acc[7]);
            acc[1] = acc[3] = s01;
            acc[2] = acc[6] = s02;
            acc[5] = acc[7] = s12;
        }
#pragma unroll
        for (int x = 0; x < 9; ++x) Kc[kidx(x, I)] = acc[x];
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

// Power iteration step: w = D^-1 K v / ||v||; the norm of w goes to lam[l].
template <typename T>
__global__ void k_mg_power(LevelView<T> L, const T* __restrict__ v, T* __restrict__ w,
                           double* __restrict__ nrm, int first, Reduction red) {
    const int64_t N = L.N;
    const double inv = first ? 1.0 : (*nrm > 0.0 ? 1.0 / *nrm : 0.0);
    const T ks = (T)*L.ks;
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N;
         i += (int64_t)gridDim.x * blockDim.x) {
        T y[3], z[3];
        stencil_apply<T>(L.n, N, i, L.K, v, y);
#pragma unroll
        for (int c = 0; c < 3; ++c) y[c] *= ks;
        dinv_apply<T>(N, i, L.Di, y, z);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            T o = L.mask[i] ? T(0) : (T)(z[c] * inv);
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

// max |K| of a level (bits of a non-negative float compare as unsigned).
__global__ void k_mg_absmax(int64_t n, const float* __restrict__ K, unsigned* __restrict__ out) {
    float m = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(K[i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

// FP16 copy of a level's stencil (layout of hidx), scaled so that max |K|
// maps to 16384.  Thread per (node, group): group g < 8 takes entries 0..7 of
// direction g, group 8 entry 8 of every direction.
__global__ void k_mg_to_half(int64_t nodes, const float* __restrict__ K,
                             const unsigned* __restrict__ maxbits, uint4* __restrict__ Kh,
                             double* __restrict__ scale) {
    const float mx = __uint_as_float(*maxbits);
    const float sc = mx > 0.f ? mx / 16384.f : 1.f;
    const float inv = 1.f / sc;
    if (blockIdx.x == 0 && threadIdx.x == 0) *scale = (double)sc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nodes * 9;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tile = t / (9 * 32);
        const int g = (int)((t / 32) % 9);
        const int64_t v = tile * 32 + (t & 31);
        __align__(16) __half h[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int q = g < 8 ? 9 * g + k : 9 * k + 8;
            h[k] = __float2half_rn(K[kidx(q, v)] * inv);
        }
        Kh[hidx(g, v)] = *reinterpret_cast<const uint4*>(h);
    }
}

__global__ void k_mg_unit_scale(int levels, double* __restrict__ scale) {
    for (int l = threadIdx.x; l < levels; l += blockDim.x) scale[l] = 1.0;
}

// ---------------------------------------------------------------------------
// V-cycle kernels.  All skip when the MINRES run has stopped (*stop != 0).
// Chebyshev on [lmin, lmax] = [lambda*kLowFrac, lambda]:
//   theta = (lmax+lmin)/2, delta = (lmax-lmin)/2, sigma = theta/delta,
//   rho_0 = 1/sigma, rho_i = 1/(2 sigma - rho_{i-1});
//   d_0 = D^-1 r / theta;  d_i = rho_i rho_{i-1} d_{i-1} + (2 rho_i/delta) D^-1 r_i.
// ---------------------------------------------------------------------------
#ifndef FTS_MG_LOW_FRAC
#define FTS_MG_LOW_FRAC 0.1
#endif
constexpr double kLowFrac = FTS_MG_LOW_FRAC;
constexpr int kCoarseThreads = 256;  // one CTA for the coarsest level (<= 9^3 nodes)

// Chebyshev coefficients of one level, computed once per solve on the host.
void cheb_table(double lam, double* out) {
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

// Levels of at most kClampNodes nodes (65^3 and below) run the clamped
// (branch-free) stencil body in their full-GPU kernels, the larger ones the
// split body: on those latency-bound levels a warp almost always holds a
// boundary node, and the split body then runs both bodies.
#ifndef FTS_MG_CLAMP_NODES
#define FTS_MG_CLAMP_NODES 300000
#endif
constexpr int64_t kClampNodes = FTS_MG_CLAMP_NODES;

template <typename T, int SK>
__global__ void __launch_bounds__(kThreads, 4)
k_mg_step(LevelView<T> L, int step, int mode, const T* __restrict__ din, T* __restrict__ dout,
          const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    T xo[3];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        mg_step_node<T, SK>(L, i, step, mode, din, dout, xo, true, true);
}

template <typename T, int SK>
__global__ void __launch_bounds__(kThreads, 4)
k_mg_residual(LevelView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        mg_resid_node<T, SK>(L, i);
}

template <typename T, int SK, bool WR = true>
__global__ void __launch_bounds__(kThreads, 4)
k_mg_resid_first(LevelView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        mg_resid_first_node<T, SK, WR>(L, i);
}

template <typename T>
__global__ void __launch_bounds__(kThreads, 4)
k_mg_resid_d0(LevelView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        mg_resid_d0_node<T>(L, i);
}

// x += d_0 (the degree-1 post-smoothing update).
template <typename T>
__global__ void k_mg_add_d0(LevelView<T> L, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < 3 * L.N;
         i += (int64_t)gridDim.x * blockDim.x)
        L.x[i] += L.d0[i];
}

template <typename T>
__global__ void k_mg_restrict(LevelView<T> F, LevelView<T> C, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < C.N;
         I += (int64_t)gridDim.x * blockDim.x)
        mg_restrict_node<T>(F, C, I);
}

template <typename T, bool FROM_D0 = false>
__global__ void k_mg_prolong(LevelView<T> F, LevelView<T> C, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < F.N;
         f += (int64_t)gridDim.x * blockDim.x)
        mg_prolong_node<T, FROM_D0>(F, C, f);
}

template <typename T>
__global__ void __launch_bounds__(kCoarseThreads)
k_mg_coarse_solve(LevelView<T> L, int steps, const int* __restrict__ stop) {
    pdl_wait();
    if (stop && *stop) return;
    mg_coarse_block<T>(L, steps);
}

// The levels l0.. of one V-cycle in one launch of a single thread-block
// cluster (16 CTAs of 512 threads where the device allows it, else 8): the
// small levels are latency bound as separate launches, so their phases are
// separated by hardware cluster barriers instead (barrier.cluster: release /
// acquire at cluster scope, covering the global-memory vectors the CTAs
// exchange).  Level l0's right-hand side and first direction are ready; its
// corrected x is the result.  skip_final (l0 == 0) leaves the last
// post-smoothing step of the finest level to the caller.
constexpr int kTailThreads = 512;
// Stencil body of the tail's levels: the clamped one, since nearly every warp
// of a small lattice holds a boundary node.
#ifndef FTS_TAIL_SK
#define FTS_TAIL_SK kSkClamped
#endif
constexpr int kTailSk = FTS_TAIL_SK;

template <typename T>
struct MGTailArgs {
    LevelView<T> lv[kMaxMGLevels];
    int l0, nlev, skip_final;
};

template <typename T>
__global__ void __launch_bounds__(kTailThreads, 1)
k_mg_tail(const __grid_constant__ MGTailArgs<T> a, const int* __restrict__ stop) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    pdl_wait();
    if (stop && *stop) return;  // uniform: nothing writes the flag during the V-cycle
    const int64_t tid = (int64_t)cl.block_rank() * blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)cl.num_blocks() * blockDim.x;
    T xo[3];
    for (int l = a.l0; l + 1 < a.nlev; ++l) {
        const LevelView<T> L = a.lv[l];
        for (int s = 1; s < kSmooth; ++s) {
            const int mode = s == 1 ? kStepFromZero : kStepRegular;
            for (int64_t v = tid; v < L.N; v += nth)
                mg_step_node<T, kTailSk>(L, v, s, mode, (s & 1) ? L.d0 : L.d1,
                                            (s & 1) ? L.d1 : L.d0, xo, true, true);
            cl.sync();
        }
        for (int64_t v = tid; v < L.N; v += nth) mg_resid_node<T, kTailSk>(L, v);
        cl.sync();
        const LevelView<T> C = a.lv[l + 1];
        for (int64_t v = tid; v < C.N; v += nth) mg_restrict_node<T>(L, C, v);
        cl.sync();
    }
    if (cl.block_rank() == 0) {
        const LevelView<T> L = a.lv[a.nlev - 1];
        mg_coarse_block<T, kTailSk>(L, L.n == 3 ? 1 : kCoarse);
    }
    cl.sync();
    for (int l = a.nlev - 2; l >= a.l0; --l) {
        const LevelView<T> L = a.lv[l], C = a.lv[l + 1];
        for (int64_t v = tid; v < L.N; v += nth) mg_prolong_node<T>(L, C, v);
        cl.sync();
        for (int64_t v = tid; v < L.N; v += nth) mg_resid_first_node<T, kTailSk>(L, v);
        cl.sync();
        const int last = (l == 0 && a.skip_final) ? kSmooth - 2 : kSmooth - 1;
        for (int s = 1; s <= last; ++s) {
            const int mode = s == 1 ? kStepAfterFirst : kStepRegular;
            for (int64_t v = tid; v < L.N; v += nth)
                mg_step_node<T, kTailSk>(L, v, s, mode, (s & 1) ? L.d0 : L.d1,
                                            (s & 1) ? L.d1 : L.d0, xo, true, true);
            cl.sync();
        }
    }
}

// Cluster size for the tail launch: 16 where the device and the kernel's
// resources allow it, else 8 (the portable maximum); 0 if neither fits.
template <typename T>
static int tail_cluster_size(Ctx& c) {
    FTS_CUDA(cudaFuncSetAttribute(k_mg_tail<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    for (int cs : {16, 8}) {
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3((unsigned)cs);
        lc.blockDim = dim3((unsigned)kTailThreads);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)cs;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        lc.attrs = attr;
        lc.numAttrs = 1;
        int clusters = 0;
        if (cudaOccupancyMaxActiveClusters(&clusters, k_mg_tail<T>, &lc) == cudaSuccess &&
            clusters > 0)
            return cs;
        (void)cudaGetLastError();
    }
    (void)c;
    return 0;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <typename T>
void mg_build(Ctx& c, MG<T>& mg) {
    if (mg.built) return;
    init_tables(c.device);
    // P2-P1: the hierarchy lives on the vertex lattice below the P2 level
    const int lattice_n = c.p2 ? c.topo.vertex_lattice_n : c.topo.lattice_n;
    for (const int n : mg_chain(lattice_n)) {
        MGLevel<T> L;
        L.n = n;
        L.N = (int64_t)n * n * n;
        const size_t stored = (size_t)((L.N + 31) / 32) * 32 * kStored;
        L.K = dev_alloc<T>(c, stored);
        // the set-up kernels write nodes < N only; the tile padding stays zero
        FTS_CUDA(cudaMemsetAsync(L.K, 0, stored * sizeof(T), c.stream));
        if (sizeof(typename MGStore<T>::type) == sizeof(T))
            L.Kh = reinterpret_cast<typename MGStore<T>::type*>(L.K);
        else
            L.Kh = dev_alloc<typename MGStore<T>::type>(c, stored);
        L.Di = dev_alloc<T>(c, (size_t)L.N * 6);
        for (auto** p : {&L.b, &L.x, &L.r, &L.d0, &L.d1}) *p = dev_alloc<T>(c, (size_t)L.N * 3);
        L.mask = dev_alloc<uint8_t>(c, (size_t)L.N);
        mg.L.push_back(L);
    }
    mg.lam = dev_alloc<double>(c, mg.L.size() + 1);
    mg.coef = dev_alloc<double>(c, mg.L.size() * kCoefStride);
    mg.scale = dev_alloc<double>(c, mg.L.size());
    mg.maxbits = dev_alloc<unsigned>(c, mg.L.size());
    if (mg.L.size() > 1)  // the largest coarse level's partial self blocks
        mg.gal_self = dev_alloc<T>(c, (size_t)kGalSelfSplit * 9 * (size_t)mg.L[1].N);
    if (mg.L.size() > (size_t)kMaxMGLevels) {
        c.last_error = "lattice too large for the multigrid hierarchy";
        throw (int)FTS_ERR_UNSUPPORTED;
    }
    // persistent launch for the small levels: the first level (below the
    // finest, unless the whole hierarchy is small) with at most tail_nodes<T>() nodes
    mg.tail_level = -1;
    for (size_t l = 0; l + 1 < mg.L.size(); ++l)
        if (mg.L[l].N <= tail_nodes<T>()) {
            mg.tail_level = (int)l;
            break;
        }
    if (mg.tail_level >= 0) {
        mg.tail_blocks = tail_cluster_size<T>(c);
        if (mg.tail_blocks == 0) mg.tail_level = -1;
    }
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

// The smoothing copy of level l's stencil (FP16 for the FP32 hierarchy).
static void mg_store(Ctx& c, MG<float>& mg, size_t l) {
    MGLevel<float>& L = mg.L[l];
    const int64_t stored = ((L.N + 31) / 32) * 32 * kStored;
    FTS_CUDA(cudaMemsetAsync(mg.maxbits + l, 0, sizeof(unsigned), c.stream));
    k_mg_absmax<<<grid_for(c, stored), kThreads, 0, c.stream>>>(stored, L.K, mg.maxbits + l);
    const int64_t nodes = ((L.N + 31) / 32) * 32;
    k_mg_to_half<<<grid_for(c, nodes * 9), kThreads, 0, c.stream>>>(
        nodes, L.K, mg.maxbits + l, reinterpret_cast<uint4*>(L.Kh), mg.scale + l);
    c.launches += 2;
}
static void mg_store(Ctx& c, MG<double>& mg, size_t l) {
    if (l == 0) {
        k_mg_unit_scale<<<1, 32, 0, c.stream>>>((int)mg.L.size(), mg.scale);
        c.launches += 1;
    }
}

// Per-solve set-up after assembly: fine operator, Galerkin hierarchy, D^-1,
// smoothing stencils, lambda_max per level.
template <typename T>
void mg_setup(Ctx& c, MG<T>& mg) {
    mg_build<T>(c, mg);
    MGLevel<T>& F = mg.L[0];
    if (c.matfree && c.topo.kuhn_elements)
        k_mg_from_elements<T, true><<<grid_for(c, F.N * 8), kThreads, 0, c.stream>>>(
            F.n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.bnd, F.K);
    else if (c.matfree)
        k_mg_from_elements<T, false><<<grid_for(c, F.N * 8), kThreads, 0, c.stream>>>(
            F.n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.bnd, F.K);
    else if (c.p2)
        p2mg_galerkin<T>(c, F.K, F.mask, F.n);
    else if (c.use_lat64)
        k_mg_extract_lat<T><<<grid_for(c, F.N * 8), kThreads, 0, c.stream>>>(F.n, c.lat64, F.K);
    else
        k_mg_extract<T><<<grid_for(c, F.N * 8), kThreads, 0, c.stream>>>(F.n, c.rowptr, c.cols,
                                                                           c.A64, F.K);
    c.launches += 1;
    // Each level's power iterations need only its own stencil and D^-1: with a
    // second stream (and the pressure set-up on it, whose kernels reduce
    // nothing through c.red) they run there, under the next levels' Galerkin
    // products on this stream.
    const bool side = c.aux_stream != nullptr && c.use_pmg;
    cudaStream_t ps = side ? c.aux_stream : c.stream;
    for (size_t l = 0; l < mg.L.size(); ++l) {
        MGLevel<T>& L = mg.L[l];
        if (l > 0) {
            MGLevel<T>& P = mg.L[l - 1];
            k_mg_galerkin<T><<<grid_for(c, L.N * (7 + kGalSelfSplit)), kThreads, 0, c.stream>>>(
                P.n, P.K, P.mask, L.n, L.K, L.mask, mg.gal_self);
            k_mg_galerkin_self<T><<<grid_for(c, L.N), kThreads, 0, c.stream>>>(L.n, mg.gal_self,
                                                                                L.K, L.mask);
            c.launches += 2;
        }
        k_mg_dinv<T><<<grid_for(c, L.N), kThreads, 0, c.stream>>>(L.N, L.K, L.Di);
        mg_store(c, mg, l);
        k_mg_power_init<T><<<grid_for(c, L.N), kThreads, 0, c.stream>>>(L.N, L.mask, L.d0);
        c.launches += 2;
        if (side) {
            FTS_CUDA(cudaEventRecord(c.ev_fork, c.stream));
            FTS_CUDA(cudaStreamWaitEvent(ps, c.ev_fork, 0));
        }
        const LevelView<T> V = level_view(mg, l);
        T* v = L.d0;
        T* w = L.d1;
        for (int it = 0; it < kPowerIters; ++it) {
            k_mg_power<T><<<grid_for(c, L.N), kThreads, 0, ps>>>(V, v, w, mg.lam + l, it == 0,
                                                                  c.red);
            c.launches += 1;
            T* t = v;
            v = w;
            w = t;
        }
    }
    if (side) {
        FTS_CUDA(cudaEventRecord(c.ev_join, ps));
        FTS_CUDA(cudaStreamWaitEvent(c.stream, c.ev_join, 0));
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

// One level of the V-cycle; L.d0 holds the first Chebyshev direction of L.b.
template <typename T>
static void vcycle_level(Ctx& c, MG<T>& mg, size_t l, const int* stop, int skip_final) {
    const LevelView<T> L = level_view(mg, l);
    const int g = grid_for(c, L.N);
    if ((int)l == mg.tail_level) {
        MGTailArgs<T> a{};
        for (size_t k = 0; k < mg.L.size(); ++k) a.lv[k] = level_view(mg, k);
        a.l0 = (int)l;
        a.nlev = (int)mg.L.size();
        a.skip_final = skip_final ? 1 : 0;
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3((unsigned)mg.tail_blocks);
        lc.blockDim = dim3((unsigned)kTailThreads);
        lc.stream = c.stream;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)mg.tail_blocks;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        lc.attrs = attr;
        lc.numAttrs = 2;
        FTS_CUDA(cudaLaunchKernelEx(&lc, k_mg_tail<T>, a, stop));
        c.launches += 1;
        return;
    }
    if (l + 1 == mg.L.size()) {
        pdl_launch(k_mg_coarse_solve<T>, 1, kCoarseThreads, c.stream, L, L.n == 3 ? 1 : kCoarse, stop);
        c.launches += 1;
        return;
    }
    const LevelView<T> C = level_view(mg, l + 1);
    if (mg_level_degree1(mg, l)) {
        // degree 1: x = d_0, r = b - K d_0; after the coarse correction
        // x = d_0 + P e, r = b - K x (not stored), d_0 = D^-1 r / theta,
        // x += d_0 (the caller's when skip_final)
        pdl_launch(k_mg_resid_d0<T>, g, kThreads, c.stream, L, stop);
        pdl_launch(k_mg_restrict<T>, grid_for(c, C.N), kThreads, c.stream, L, C, stop);
        vcycle_level<T>(c, mg, l + 1, stop, 0);
        pdl_launch(k_mg_prolong<T, true>, g, kThreads, c.stream, L, C, stop);
        c.launches += 3;
        if (skip_final == kSkipPost) return;  // the caller's stage 2 runs the residual
        pdl_launch(k_mg_resid_first<T, kSkSplit, false>, g, kThreads, c.stream, L, stop);
        c.launches += 1;
        if (!skip_final) {
            pdl_launch(k_mg_add_d0<T>, grid_for(c, 3 * L.N), kThreads, c.stream, L, stop);
            c.launches += 1;
        }
        return;
    }
    const bool clamp = L.N <= kClampNodes;
    auto step_kernel = clamp ? k_mg_step<T, kSkClamped> : k_mg_step<T, kSkSplit>;
    // pre-smoothing from zero (d_0 is already in L.d0)
    T* din = L.d0;
    T* dout = L.d1;
    for (int s = 1; s < kSmooth; ++s) {
        pdl_launch(step_kernel, g, kThreads, c.stream, L, s, s == 1 ? kStepFromZero : kStepRegular, din,
                   dout, stop);
        std::swap(din, dout);
    }
    pdl_launch(clamp ? k_mg_residual<T, kSkClamped> : k_mg_residual<T, kSkSplit>, g, kThreads,
               c.stream, L, stop);
    pdl_launch(k_mg_restrict<T>, grid_for(c, C.N), kThreads, c.stream, L, C, stop);
    c.launches += kSmooth + 1;
    vcycle_level<T>(c, mg, l + 1, stop, 0);
    pdl_launch(k_mg_prolong<T>, g, kThreads, c.stream, L, C, stop);
    // post-smoothing from the corrected x
    pdl_launch(clamp ? k_mg_resid_first<T, kSkClamped> : k_mg_resid_first<T, kSkSplit>, g,
               kThreads, c.stream, L, stop);
    c.launches += 2;
    din = L.d0;
    dout = L.d1;
    for (int s = 1; s < kSmooth; ++s) {
        if (skip_final && s == kSmooth - 1) break;
        pdl_launch(step_kernel, g, kThreads, c.stream, L, s, s == 1 ? kStepAfterFirst : kStepRegular, din,
                   dout, stop);
        std::swap(din, dout);
        c.launches += 1;
    }
}

template <typename T>
void mg_vcycle(Ctx& c, MG<T>& mg, const int* stop, int skip_final) {
    vcycle_level<T>(c, mg, 0, stop, skip_final);
    FTS_CUDA(cudaGetLastError());
}

template <typename T>
void mg_free(MG<T>& mg) {
    for (auto& L : mg.L) {
        if (L.Kh && (void*)L.Kh != (void*)L.K) cudaFree(L.Kh);
        for (void* p : {(void*)L.K, (void*)L.Di, (void*)L.b, (void*)L.x, (void*)L.r, (void*)L.d0,
                        (void*)L.d1, (void*)L.mask})
            if (p) cudaFree(p);
    }
    for (void* p : {(void*)mg.lam, (void*)mg.coef, (void*)mg.scale, (void*)mg.maxbits,
                    (void*)mg.gal_self})
        if (p) cudaFree(p);
    mg.tail_level = -1;
    mg.lam = nullptr;
    mg.coef = nullptr;
    mg.scale = nullptr;
    mg.maxbits = nullptr;
    mg.gal_self = nullptr;
    mg.L.clear();
    mg.built = false;
}

template void mg_setup<double>(Ctx&, MG<double>&);
template void mg_setup<float>(Ctx&, MG<float>&);
template void mg_vcycle<double>(Ctx&, MG<double>&, const int*, int);
template void mg_vcycle<float>(Ctx&, MG<float>&, const int*, int);
template void mg_free<double>(MG<double>&);
template void mg_free<float>(MG<float>&);

}  // namespace fts
