// Level-set update (LevelSet::update, src/fem/LevelSet.cpp:89-151, with the
// distance reset resetPhi_, :429-455) on one GPU:
//   1. Crank-Nicolson advection of phi by the nodal Stokes velocity:
//        (M + dt/2 A) phi' = (M - dt/2 A) phi,
//      M the P1 mass (assembled once), A(i,j) = int (V . grad phi_j) phi_i with
//      V interpolated at the quadrature points from the nodal values
//      (Assembler.hpp:179-190), both by the atomic-free node-row gather in
//      FP64 from element geometry stored once per mesh, then Jacobi-preconditioned BiCGSTAB (Eigen's algorithm and
//      stopping rule, LevelSet.hpp:145) with device-side scalars;
//   2. the distance reset: interface points on the edges whose end values
//      differ in sign bit (LevelSet.cpp:278-300), the pruned exact distance
//      search of dist.cu, the crossing edges' nodes keep the advected value, and
//      phi = 0.75 phi_kept + 0.25 phi_reset (LevelSet.cpp:17-18, :147).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "fts_device.cuh"
#include "reduce.cuh"

struct fts_dist;

namespace fts {

void dist_reset_device(fts_dist* D, const float* ifp, bool ifp_on_device, int32_t n_ifp,
                       double* phi_dev, int32_t method, cudaStream_t s, fts_dist_stats* st);

static std::string& g_ls_error() {
    static thread_local std::string e;
    return e;
}

constexpr int kLsThreads = 256;

struct LsConst {
    double phi[4][4];  // float-rounded basis table phi[a][q]
    double qw;
    double mq[4][4];   // qw sum_q phi_a(q) phi_j(q)
};

static LsConst ls_const() {
    const RefConstants R = ref_constants();
    LsConst c;
    std::memcpy(c.phi, R.phi, sizeof(c.phi));
    c.qw = 0.25 / 6.0;
    for (int a = 0; a < 4; ++a)
        for (int j = 0; j < 4; ++j) {
            double s = 0.0;
            for (int q = 0; q < 4; ++q) s += R.phi[a][q] * R.phi[j][q];
            c.mq[a][j] = c.qw * s;
        }
    return c;
}

// Element geometry in FP64 from float coordinates (Assembler.hpp:430-462).
__device__ __forceinline__ bool ls_geom(const float* __restrict__ xyz, const int ids[4],
                                        double g[4][3], double& detB) {
    double p[4][3];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int c = 0; c < 3; ++c) p[j][c] = (double)xyz[3 * (int64_t)ids[j] + c];
    double B[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        B[c][0] = p[1][c] - p[0][c];
        B[c][1] = p[2][c] - p[0][c];
        B[c][2] = p[3][c] - p[0][c];
    }
    const double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1];
    const double c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2];
    const double c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
    const double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
    detB = fabs(det);
    if (!(detB > 0.0)) return false;
    double cof[3][3];
    cof[0][0] = c00;
    cof[0][1] = c01;
    cof[0][2] = c02;
    cof[1][0] = B[0][2] * B[2][1] - B[0][1] * B[2][2];
    cof[1][1] = B[0][0] * B[2][2] - B[0][2] * B[2][0];
    cof[1][2] = B[0][1] * B[2][0] - B[0][0] * B[2][1];
    cof[2][0] = B[0][1] * B[1][2] - B[0][2] * B[1][1];
    cof[2][1] = B[0][2] * B[1][0] - B[0][0] * B[1][2];
    cof[2][2] = B[0][0] * B[1][1] - B[0][1] * B[1][0];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const double it0 = cof[r][0] / det, it1 = cof[r][1] / det, it2 = cof[r][2] / det;
        g[0][r] = -it0 - it1 - it2;
        g[1][r] = it0;
        g[2][r] = it1;
        g[3][r] = it2;
    }
    return true;
}

// Per-element geometry, computed once per mesh (the coordinates never change):
// gradients and |det B| (128 B).
struct LsGeom {
    double g[4][3];
    double detB;
    double pad[3];
};

__global__ void k_ls_geometry(int64_t nt, const int32_t* __restrict__ tets,
                              const float* __restrict__ xyz, LsGeom* __restrict__ geom,
                              int* __restrict__ bad) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int4 tt = reinterpret_cast<const int4*>(tets)[k];
        const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
        LsGeom G;
        if (!ls_geom(xyz, ids, G.g, G.detB)) {
            atomicOr(bad, 1);
            G.detB = 0.0;
        }
        G.pad[0] = G.pad[1] = G.pad[2] = 0.0;
        geom[k] = G;
    }
}

// feval . (qw) * detB with the reference's pairwise order.
__device__ __forceinline__ double ls_integ(const double f[4], double qw, double detB) {
    return ((f[0] * qw + f[2] * qw) + (f[1] * qw + f[3] * qw)) * detB;
}

// Row slot of every (node-element entry, column node b): slots[4 e + b] =
// position of the element's node b in the row of the entry's node, minus the
// row start (rows of at most 255 entries), once per mesh.
__global__ void k_ls_slots(int64_t np, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ cols, const int32_t* __restrict__ p2t_ptr,
                           const uint32_t* __restrict__ p2t, const int32_t* __restrict__ tets,
                           uint8_t* __restrict__ slots) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r0 = rowptr[i], r1 = rowptr[i + 1];
        for (int32_t e = p2t_ptr[i]; e < p2t_ptr[i + 1]; ++e) {
            const int4 tt = reinterpret_cast<const int4*>(tets)[p2t[e] >> 2];
            const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
            for (int b = 0; b < 4; ++b) {
                int32_t slot = r0;
                while (slot < r1 && cols[slot] != ids[b]) ++slot;
                slots[4 * (int64_t)e + b] = (uint8_t)(slot - r0);
            }
        }
    }
}

// Row gather of M (flow == NULL) or A (nodal velocity `flow`), one thread per
// node, from the stored element geometry.  With slots (k_ls_slots) the
// advection entries use the regrouped exact sum
//   int phi_a (V . grad phi_b) = |det B| sum_c (grad phi_b)_c sum_j V_jc mq[a][j]
// (V interpolated with the same float-rounded table: the quadrature sum
// reordered, 24 FMAs per node-element pair) and M_ab = |det B| mq[a][b];
// without, the reference's per-point expressions and a row search.
__global__ void k_ls_assemble(int64_t np, const int32_t* __restrict__ rowptr,
                              const int32_t* __restrict__ cols,
                              const int32_t* __restrict__ p2t_ptr,
                              const uint32_t* __restrict__ p2t, const int32_t* __restrict__ tets,
                              const LsGeom* __restrict__ geom, const double* __restrict__ flow,
                              LsConst K, const uint8_t* __restrict__ slots,
                              double* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r0 = rowptr[i], r1 = rowptr[i + 1];
        for (int32_t q = r0; q < r1; ++q) out[q] = 0.0;
        if (slots) {
            for (int32_t e = p2t_ptr[i]; e < p2t_ptr[i + 1]; ++e) {
                const uint32_t pe = p2t[e];
                const int64_t k = pe >> 2;
                const int a = pe & 3;
                const LsGeom& G = geom[k];
                const double detB = G.detB;
                const uint32_t sl = reinterpret_cast<const uint32_t*>(slots)[e];
                if (flow) {
                    const int4 tt = reinterpret_cast<const int4*>(tets)[k];
                    const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
                    double W[3] = {0.0, 0.0, 0.0};
#pragma unroll
                    for (int j = 0; j < 4; ++j)
#pragma unroll
                        for (int c = 0; c < 3; ++c) W[c] += K.mq[a][j] * flow[ids[j] + c * np];
#pragma unroll
                    for (int b = 0; b < 4; ++b)
                        out[r0 + ((sl >> (8 * b)) & 255u)] +=
                            detB * (G.g[b][0] * W[0] + G.g[b][1] * W[1] + G.g[b][2] * W[2]);
                } else {
#pragma unroll
                    for (int b = 0; b < 4; ++b)
                        out[r0 + ((sl >> (8 * b)) & 255u)] += detB * K.mq[a][b];
                }
            }
            continue;
        }
        for (int32_t e = p2t_ptr[i]; e < p2t_ptr[i + 1]; ++e) {
            const uint32_t pe = p2t[e];
            const int64_t k = pe >> 2;
            const int a = pe & 3;
            const int4 tt = reinterpret_cast<const int4*>(tets)[k];
            const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
            const LsGeom& G = geom[k];
            const double detB = G.detB;
            double g[4][3];
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int c = 0; c < 3; ++c) g[j][c] = G.g[j][c];
            double V[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
            if (flow) {
#pragma unroll
                for (int j = 0; j < 4; ++j)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const double vj = flow[ids[j] + c * np];
#pragma unroll
                        for (int q = 0; q < 4; ++q) V[c][q] += vj * K.phi[j][q];
                    }
            }
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                double f[4];
                if (flow) {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        f[q] = V[0][q] * (g[b][0] * K.phi[a][q]) + V[1][q] * (g[b][1] * K.phi[a][q]) +
                               V[2][q] * (g[b][2] * K.phi[a][q]);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; ++q) f[q] = K.phi[b][q] * K.phi[a][q];
                }
                const double v = ls_integ(f, K.qw, detB);
                int32_t slot = r0;
                while (slot < r1 && cols[slot] != ids[b]) ++slot;
                if (slot < r1) out[slot] += v;
            }
        }
    }
}

// L = M + h A, b = (M - h A) phi, inv = 1 / diag(L) (1 where the diagonal is 0,
// Eigen's DiagonalPreconditioner); x = phi (warm start).
__global__ void k_ls_system(int64_t np, const int32_t* __restrict__ rowptr,
                            const int32_t* __restrict__ cols, const double* __restrict__ M,
                            const double* __restrict__ A, double h,
                            const double* __restrict__ phi, double* __restrict__ L,
                            double* __restrict__ b, double* __restrict__ inv,
                            double* __restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0, d = 0.0;
        const int32_t q0 = rowptr[i], q1 = rowptr[i + 1];
#pragma unroll 4
        for (int32_t q = q0; q < q1; ++q) {  // unrolled: the loads of 4 entries in flight
            const double m = M[q], a = A[q];
            const int32_t j = cols[q];
            const double l = m + h * a;
            L[q] = l;
            acc += (m - h * a) * phi[j];
            if (j == i) d = l;
        }
        b[i] = acc;
        inv[i] = d != 0.0 ? 1.0 / d : 1.0;
        x[i] = phi[i];
    }
}

struct BjScalars {
    double rho, rho_old, alpha, w, beta, r0n, rr, bb, tol2;
    long long it, maxit;
    int stop, restart, restarts;
};

__device__ __forceinline__ double csr_row(const int32_t* __restrict__ rowptr,
                                          const int32_t* __restrict__ cols,
                                          const double* __restrict__ L,
                                          const double* __restrict__ v, int64_t i) {
    double acc = 0.0;
    const int32_t q0 = rowptr[i], q1 = rowptr[i + 1];
#pragma unroll 4
    for (int32_t q = q0; q < q1; ++q) acc += L[q] * v[cols[q]];
    return acc;
}

// r = b - L x, r0 = r (start, and Eigen's restart when rho collapses).
// Start: p = vv = 0, rho = r0.r, stop if ||b|| = 0 or already converged.
// Restart: rho = r0n = r.r, the iteration count resets on the first restart,
// beta from the previous rho.
__global__ void __launch_bounds__(kLsThreads)
k_bj_residual(int64_t np, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
              const double* __restrict__ L, const double* __restrict__ b,
              const double* __restrict__ x, double* __restrict__ r, double* __restrict__ r0,
              double* __restrict__ p, double* __restrict__ vv, int first, double tol,
              Reduction red, BjScalars* S) {
    double acc[2] = {0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double ri = b[i] - csr_row(rowptr, cols, L, x, i);
        r[i] = ri;
        r0[i] = ri;
        if (first) {
            p[i] = 0.0;
            vv[i] = 0.0;
        }
        acc[0] += ri * ri;
        acc[1] += b[i] * b[i];
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        S->r0n = tot[0];
        S->rr = tot[0];
        S->restart = 0;
        if (first) {
            S->bb = tot[1];
            S->tol2 = tol * tol * tot[1];
            S->alpha = 1.0;
            S->w = 1.0;
            S->rho_old = 1.0;
            S->rho = tot[0];
            S->beta = tot[0];
            S->it = 0;
            S->restarts = 0;
            S->stop = (tot[1] == 0.0 || tot[0] <= S->tol2 || S->maxit <= 0) ? 1 : 0;
        } else {
            S->rho = tot[0];
            if (S->restarts++ == 0) S->it = 0;
            S->beta = (S->rho / S->rho_old) * (S->alpha / S->w);
            S->stop = 0;
        }
    }
}

// p = r + beta (p - w vv), y = inv p.
__global__ void k_bj_p(int64_t np, const double* __restrict__ r, double* __restrict__ p,
                       const double* __restrict__ vv, const double* __restrict__ inv,
                       double* __restrict__ y, const BjScalars* __restrict__ S) {
    if (S->stop) return;
    const double beta = S->beta, w = S->w;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double pi = r[i] + beta * (p[i] - w * vv[i]);
        p[i] = pi;
        y[i] = inv[i] * pi;
    }
}

// vv = L y; alpha = rho / (r0 . vv).
__global__ void __launch_bounds__(kLsThreads)
k_bj_spmv1(int64_t np, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
           const double* __restrict__ L, const double* __restrict__ y,
           const double* __restrict__ r0, double* __restrict__ vv, Reduction red, BjScalars* S) {
    if (S->stop) return;
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = csr_row(rowptr, cols, L, y, i);
        vv[i] = v;
        acc[0] += r0[i] * v;
    }
    double tot[1];
    if (grid_sum<1>(acc, red, tot) && threadIdx.x == 0) S->alpha = S->rho / tot[0];
}

// s = r - alpha vv, z = inv s.
__global__ void k_bj_s(int64_t np, const double* __restrict__ r, const double* __restrict__ vv,
                       const double* __restrict__ inv, double* __restrict__ s,
                       double* __restrict__ z, const BjScalars* __restrict__ S) {
    if (S->stop) return;
    const double alpha = S->alpha;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double si = r[i] - alpha * vv[i];
        s[i] = si;
        z[i] = inv[i] * si;
    }
}

// t = L z; w = (t . s) / (t . t) (0 if t = 0).
__global__ void __launch_bounds__(kLsThreads)
k_bj_spmv2(int64_t np, const int32_t* __restrict__ rowptr, const int32_t* __restrict__ cols,
           const double* __restrict__ L, const double* __restrict__ z,
           const double* __restrict__ s, double* __restrict__ t, Reduction red, BjScalars* S) {
    if (S->stop) return;
    double acc[2] = {0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = csr_row(rowptr, cols, L, z, i);
        t[i] = v;
        acc[0] += v * v;
        acc[1] += v * s[i];
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0)
        S->w = tot[0] > 0.0 ? tot[1] / tot[0] : 0.0;
}

// x += alpha y + w z, r = s - w t; rr = r.r, rho_next = r0.r; the loop test
// and the next beta (or a restart when rho collapses).
__global__ void __launch_bounds__(kLsThreads)
k_bj_update(int64_t np, double* __restrict__ x, const double* __restrict__ y,
            const double* __restrict__ z, const double* __restrict__ s,
            const double* __restrict__ t, double* __restrict__ r, const double* __restrict__ r0,
            Reduction red, BjScalars* S) {
    if (S->stop) return;
    const double alpha = S->alpha, w = S->w;
    double acc[2] = {0.0, 0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += alpha * y[i] + w * z[i];
        const double ri = s[i] - w * t[i];
        r[i] = ri;
        acc[0] += ri * ri;
        acc[1] += r0[i] * ri;
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        S->rr = tot[0];
        S->it += 1;
        if (tot[0] <= S->tol2 || S->it >= S->maxit) {
            S->stop = 1;
            return;
        }
        S->rho_old = S->rho;
        S->rho = tot[1];
        const double eps2 = DBL_EPSILON * DBL_EPSILON;
        if (fabs(S->rho) < eps2 * S->r0n) {
            S->restart = 1;  // the host runs the restart residual
            S->stop = 1;
            return;
        }
        S->beta = (S->rho / S->rho_old) * (S->alpha / S->w);
    }
}

// Interface points on the edges (i < j) whose end values differ in sign bit,
// t = phi_i / (phi_i - phi_j) (0.5 if the difference is below FLT_MIN), the
// point (1 - t) p_i + t p_j in double, stored as float; both nodes flagged.
__global__ void k_ls_crossings(int64_t np, const int32_t* __restrict__ rowptr,
                               const int32_t* __restrict__ cols, const double* __restrict__ x,
                               const float* __restrict__ xyz, float* __restrict__ ifp,
                               unsigned* __restrict__ count, uint8_t* __restrict__ keep,
                               unsigned cap) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double xi = x[i];
        for (int32_t q = rowptr[i]; q < rowptr[i + 1]; ++q) {
            const int32_t j = cols[q];
            if (j <= i) continue;
            const double xj = x[j];
            if (signbit(xi) == signbit(xj)) continue;
            const double div = xi - xj;
            const double t = fabs(div) > (double)FLT_MIN ? xi / div : 0.5;
            const unsigned k = atomicAdd(count, 1u);
            if (k < cap)
#pragma unroll
                for (int c = 0; c < 3; ++c)
                    ifp[3 * (int64_t)k + c] = (float)((1.0 - t) * (double)xyz[3 * i + c] +
                                                      t * (double)xyz[3 * (int64_t)j + c]);
            keep[i] = 1;
            keep[j] = 1;
        }
    }
}

// phi = 0.75 (kept ? advected : reset) + 0.25 reset.
__global__ void k_ls_mix(int64_t np, const double* __restrict__ adv, const double* __restrict__ ifn,
                         const uint8_t* __restrict__ keep, double* __restrict__ phi) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double kept = keep[i] ? adv[i] : ifn[i];
        phi[i] = 0.75 * kept + 0.25 * ifn[i];
    }
}

__global__ void k_ls_check_velocity(int64_t n, const double* __restrict__ v,
                                    int* __restrict__ nan_flag, Reduction red,
                                    double* __restrict__ norm2) {
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double vi = v[i];
        if (isnan(vi) && i < 3 * (n / 4)) atomicOr(nan_flag, 1);
        acc[0] += vi * vi;
    }
    double tot[1];
    if (grid_sum<1>(acc, red, tot) && threadIdx.x == 0) *norm2 = tot[0];
}

// ---------------------------------------------------------------------------
// Surface tension (Flow::surfaceTension_, src/growth/Flow.cpp:307-341) and
// the LevelSet quantities it reads, from phi (current) and phi_reset (the last
// full distance reset, LevelSet::phi_ifn_, LevelSet.cpp:440):
//   normals = grad_nodes(phi_reset)                   LevelSet.cpp:453
//   k = div(normals / |normals|) by grad_nodes of each normalised component,
//       interpolated along the crossing edge          LevelSet.cpp:215-253
//   interface points on sign-bit crossing edges       LevelSet.cpp:261-300
//   patch areas: per mixed element, its crossing edges in the local order
//       01 02 03 12 13 23 make one triangle (3) or two (4: e0 e2 e3, e0 e1 e3),
//       0.5 |e1 x e2| added to each of the triangle's points, elements in
//       index order                                    LevelSet.cpp:326-420
//   grad / grad_nodes                                  Assembler.cpp:11-69
// Edges are (i, j) with i < j; the force is symmetric in the orientation.
// ---------------------------------------------------------------------------

// Element gradient of the nodal field u (Assembler::grad): FP64, stored float.
// comp >= 0: only component comp of the gradient of u_comp (u = [3][np] float
// fields), for the divergence.
__global__ void k_st_elem_grad(int64_t nt, const int32_t* __restrict__ tets,
                               const LsGeom* __restrict__ geom, const double* __restrict__ u,
                               float* __restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int4 tt = reinterpret_cast<const int4*>(tets)[k];
        const LsGeom& G = geom[k];
        const double u0 = u[tt.x], u1 = u[tt.y], u2 = u[tt.z], u3 = u[tt.w];
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[3 * k + c] = (float)(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(u0, G.g[0][c]),
                                                                  __dmul_rn(u1, G.g[1][c])),
                                                        __dmul_rn(u2, G.g[2][c])),
                                               __dmul_rn(u3, G.g[3][c])));
    }
}

__global__ void k_st_elem_div(int64_t nt, const int32_t* __restrict__ tets,
                              const LsGeom* __restrict__ geom, const float* __restrict__ gn,
                              int64_t np, float* __restrict__ out) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int4 tt = reinterpret_cast<const int4*>(tets)[k];
        const LsGeom& G = geom[k];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float* u = gn + c * np;
            const double u0 = u[tt.x], u1 = u[tt.y], u2 = u[tt.z], u3 = u[tt.w];
            out[3 * k + c] = (float)(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(u0, G.g[0][c]),
                                                                  __dmul_rn(u1, G.g[1][c])),
                                                        __dmul_rn(u2, G.g[2][c])),
                                               __dmul_rn(u3, G.g[3][c])));
        }
    }
}

__device__ __forceinline__ float st_norm3(float x, float y, float z) {
    return sqrtf(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
}

// Nodal average of element vectors (grad_nodes): float sums over the node's
// elements in index order / (float) count.  mode 0: normals (and their
// normalised components into gn[3][np]); mode 1: k = sum of the diagonal.
__global__ void k_st_node_avg(int64_t np, const int32_t* __restrict__ p2t_ptr,
                              const uint32_t* __restrict__ p2t, const float* __restrict__ ge,
                              int mode, float* __restrict__ nrm, float* __restrict__ gn,
                              float* __restrict__ kmesh) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        float sx = 0.f, sy = 0.f, sz = 0.f;
        for (int32_t q = p2t_ptr[i]; q < p2t_ptr[i + 1]; ++q) {
            const int64_t k = p2t[q] >> 2;
            sx = __fadd_rn(sx, ge[3 * k]);
            sy = __fadd_rn(sy, ge[3 * k + 1]);
            sz = __fadd_rn(sz, ge[3 * k + 2]);
        }
        const float cnt = (float)(p2t_ptr[i + 1] - p2t_ptr[i]);
        const float ax = __fdiv_rn(sx, cnt), ay = __fdiv_rn(sy, cnt), az = __fdiv_rn(sz, cnt);
        if (mode == 0) {
            nrm[3 * i] = ax;
            nrm[3 * i + 1] = ay;
            nrm[3 * i + 2] = az;
            const float nn = st_norm3(ax, ay, az);
            gn[i] = __fdiv_rn(ax, nn);
            gn[np + i] = __fdiv_rn(ay, nn);
            gn[2 * np + i] = __fdiv_rn(az, nn);
        } else {
            kmesh[i] = __fadd_rn(__fadd_rn(ax, ay), az);
        }
    }
}

__device__ __forceinline__ void st_point(const float* __restrict__ xyz, const double* __restrict__ phi,
                                         int a, int b, float p[3]) {
    double t = 0.5;
    const double div = phi[a] - phi[b];
    if (fabs(div) > (double)FLT_MIN) t = phi[a] / div;
#pragma unroll
    for (int c = 0; c < 3; ++c)
        p[c] = (float)__dadd_rn(__dmul_rn(1.0 - t, (double)xyz[3 * (int64_t)a + c]),
                                __dmul_rn(t, (double)xyz[3 * (int64_t)b + c]));
}

__constant__ int c_st_edge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

// The crossing edges (i, j), i < j, whose ends differ in sign bit, as (i, edge
// slot q) in list[]; nif counts them.
__global__ void k_st_cross_list(int64_t np, const int32_t* __restrict__ rowptr,
                                const int32_t* __restrict__ cols, const double* __restrict__ phi,
                                int2* __restrict__ list, unsigned cap, unsigned* __restrict__ nif) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const bool si = signbit(phi[i]);
        for (int32_t q = rowptr[i]; q < rowptr[i + 1]; ++q) {
            const int32_t j = cols[q];
            if (j <= i || signbit(phi[j]) == si) continue;
            const unsigned at = atomicAdd(nif, 1u);
            if (at < cap) list[at] = make_int2((int)i, q);
        }
    }
}

// Patch area of each crossing edge (i, j): a warp per edge, a lane per
// element of i (in index order, 32 at a time); a lane whose element holds j
// rebuilds the element's triangles (local edge order 01 02 03 12 13 23) and
// keeps those that contain the edge's point; lane 0 then adds the kept
// triangle areas in element order, A = (float)((double)A + 0.5 |cross|), the
// sequence of the element-by-element walk.  atot sums the areas (each
// triangle three times).
__global__ void k_st_areas(const int2* __restrict__ list, const unsigned* __restrict__ nif,
                           unsigned cap, const int32_t* __restrict__ cols,
                           const int32_t* __restrict__ p2t_ptr, const uint32_t* __restrict__ p2t,
                           const int32_t* __restrict__ tets, const float* __restrict__ xyz,
                           const double* __restrict__ phi, float* __restrict__ area,
                           double* __restrict__ atot, int* __restrict__ bad) {
    const int lane = threadIdx.x & 31;
    const unsigned n = min(*nif, cap);
    for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < n;
         w += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int2 ed = list[w];
        const int32_t i = ed.x, q = ed.y, j = cols[q];
        const int32_t e0 = p2t_ptr[i], e1 = p2t_ptr[i + 1];
        float A = 0.f;
        for (int32_t eb = e0; eb < e1; eb += 32) {
            double t[2] = {0.0, 0.0};
            int nt = 0;
            const int32_t e = eb + lane;
            if (e < e1) {
                const int64_t k = p2t[e] >> 2;
                const int4 tt = reinterpret_cast<const int4*>(tets)[k];
                const int ids[4] = {tt.x, tt.y, tt.z, tt.w};
                if (ids[0] == j || ids[1] == j || ids[2] == j || ids[3] == j) {
                    float pts[4][3];
                    int mine = -1, ne = 0;
                    bool over = false;
                    for (int m = 0; m < 6; ++m) {
                        const int a = ids[c_st_edge[m][0]], b = ids[c_st_edge[m][1]];
                        if (signbit(phi[a]) == signbit(phi[b])) continue;
                        if (ne == 4) {
                            over = true;
                            break;
                        }
                        const int lo = min(a, b), hi = max(a, b);
                        if (lo == i && hi == j) mine = ne;
                        st_point(xyz, phi, lo, hi, pts[ne]);
                        ++ne;
                    }
                    if (over || (ne != 3 && ne != 4)) {
                        atomicOr(bad, 1);
                    }
                    if (ne == 3 || ne == 4) {
                        const int tri[2][3] = {{0, ne == 3 ? 1 : 2, ne == 3 ? 2 : 3}, {0, 1, 3}};
                        for (int tr = 0; tr < (ne == 3 ? 1 : 2); ++tr) {
                            if (tri[tr][0] != mine && tri[tr][1] != mine && tri[tr][2] != mine)
                                continue;
                            const float* p0 = pts[tri[tr][0]];
                            const float* p1 = pts[tri[tr][1]];
                            const float* p2 = pts[tri[tr][2]];
                            const float e1x = __fsub_rn(p1[0], p0[0]), e1y = __fsub_rn(p1[1], p0[1]),
                                        e1z = __fsub_rn(p1[2], p0[2]);
                            const float e2x = __fsub_rn(p2[0], p0[0]), e2y = __fsub_rn(p2[1], p0[1]),
                                        e2z = __fsub_rn(p2[2], p0[2]);
                            const float cx = __fsub_rn(__fmul_rn(e1y, e2z), __fmul_rn(e1z, e2y));
                            const float cy = __fsub_rn(__fmul_rn(e1z, e2x), __fmul_rn(e1x, e2z));
                            const float cz = __fsub_rn(__fmul_rn(e1x, e2y), __fmul_rn(e1y, e2x));
                            t[nt++] = 0.5 * (double)st_norm3(cx, cy, cz);
                        }
                    }
                }
            }
            // the additions in element order (lane 0 replays them)
            for (int l = 0; l < 32; ++l) {
                const int c = __shfl_sync(0xffffffffu, nt, l);
                const double t0 = __shfl_sync(0xffffffffu, t[0], l);
                const double t1 = __shfl_sync(0xffffffffu, t[1], l);
                if (c >= 1) A = (float)((double)A + t0);
                if (c >= 2) A = (float)((double)A + t1);
            }
        }
        if (lane == 0) {
            area[q] = A;
            atomicAdd(atot, (double)A);
        }
    }
}

// Nodal force of each crossing edge (Flow.cpp:326-339), added to both ends.
__global__ void k_st_force(int64_t np, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ cols, const double* __restrict__ phi,
                           const float* __restrict__ area, const float* __restrict__ kmesh,
                           const float* __restrict__ nrm, float st, int rho,
                           double* __restrict__ force) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double pi = phi[i];
        for (int32_t q = rowptr[i]; q < rowptr[i + 1]; ++q) {
            const int32_t j = cols[q];
            if (j <= i || signbit(phi[j]) == signbit(pi)) continue;
            const float t = (float)(pi / (pi - phi[j]));
            const float kif = (float)__dadd_rn(__dmul_rn(1.0 - (double)t, (double)kmesh[i]),
                                               (double)__fmul_rn(t, kmesh[j]));
            const double A = (double)area[q];
            const int64_t ends[2] = {i, j};
#pragma unroll
            for (int m = 0; m < 2; ++m) {
                const int64_t v = ends[m];
                const float nx = nrm[3 * v], ny = nrm[3 * v + 1], nz = nrm[3 * v + 2];
                const float nn = st_norm3(nx, ny, nz);
                const double w = m == 0 ? 1.0 - (double)t : (double)t;
                const float sc = (float)__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(w, (double)st),
                                                                      (double)(-kif)), A),
                                                  (double)rho);
                atomicAdd(force + v, (double)__fmul_rn(sc, __fdiv_rn(nx, nn)));
                atomicAdd(force + np + v, (double)__fmul_rn(sc, __fdiv_rn(ny, nn)));
                atomicAdd(force + 2 * np + v, (double)__fmul_rn(sc, __fdiv_rn(nz, nn)));
            }
        }
    }
}

}  // namespace fts

using namespace fts;

struct fts_ls {
    int device = 0;
    int num_sms = 148;
    cudaStream_t stream = nullptr;
    HostTopology topo;
    int64_t np = 0, nt = 0, nnz = 0;
    float* xyz = nullptr;
    int32_t* tets = nullptr;
    int32_t* rowptr = nullptr;
    int32_t* cols = nullptr;
    int32_t* p2t_ptr = nullptr;
    uint32_t* p2t = nullptr;
    LsGeom* geom = nullptr;
    uint8_t* slots = nullptr;  // [4 * 4 nt] row offsets (NULL: rows too long)
    double* M = nullptr;
    double* A = nullptr;
    double* L = nullptr;
    double* flow = nullptr;
    double* phi = nullptr;
    double* vec[12] = {};  // x b r r0 p vv s t y z inv ifn
    uint8_t* keep = nullptr;
    float* ifp = nullptr;
    unsigned ifp_cap = 0;
    unsigned* count = nullptr;
    int* flag = nullptr;
    double* norm2 = nullptr;
    BjScalars* S = nullptr;
    BjScalars* S_host = nullptr;
    Reduction red{nullptr, nullptr};
    fts_dist* dist = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::string last_error;
    bool have_reset = false;  // vec[11] holds the last update's full reset values
    // surface tension (allocated by its first call)
    double* st_phi = nullptr;    // [np] current phi
    double* st_ifn = nullptr;    // [np] reset values given by the caller
    float* st_ge = nullptr;      // [3 nt] element gradients
    float* st_nrm = nullptr;     // [3 np] nodal normals (grad_nodes of phi_reset)
    float* st_gn = nullptr;      // [3][np] normalised components
    float* st_k = nullptr;       // [np] nodal curvature
    float* st_area = nullptr;    // [nnz] patch area per crossing edge slot
    int2* st_list = nullptr;     // crossing edges (node, edge slot)
    unsigned st_list_cap = 0;
    double* st_force = nullptr;  // [3 np]
    double* st_acc = nullptr;    // total area (x3)
};

namespace {

template <typename T>
T* ls_alloc(size_t n) {
    void* p = nullptr;
    FTS_CUDA(cudaMalloc(&p, n * sizeof(T) + 16));
    return static_cast<T*>(p);
}

void ls_free(fts_ls& S) {
    void* ptrs[] = {S.xyz, S.tets, S.rowptr, S.cols, S.p2t_ptr, S.p2t, S.geom, S.slots, S.M, S.A,
                    S.L,
                    S.flow, S.phi, S.keep, S.ifp, S.count, S.flag, S.norm2, S.S,
                    S.red.partials, S.red.ticket, S.st_phi, S.st_ifn, S.st_ge, S.st_nrm,
                    S.st_gn, S.st_k, S.st_area, S.st_force, S.st_acc, S.st_list};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (double* p : S.vec)
        if (p) cudaFree(p);
    if (S.S_host) cudaFreeHost(S.S_host);
    if (S.dist) fts_dist_destroy(S.dist);
    for (auto& e : S.ev)
        if (e) cudaEventDestroy(e);
    if (S.stream) cudaStreamDestroy(S.stream);
}

int grid_of(const fts_ls& S, int64_t work) {
    const int64_t need = std::max<int64_t>(1, (work + kLsThreads - 1) / kLsThreads);
    return (int)std::min<int64_t>(need, (int64_t)S.num_sms * 8);
}

}  // namespace

extern "C" {

int fts_ls_create(const fts_mesh* mesh, int32_t device, fts_ls** out) {
    if (!mesh || !out) return FTS_ERR_BAD_INPUT;
    *out = nullptr;
    fts_ls* S = new (std::nothrow) fts_ls();
    if (!S) return FTS_ERR_OOM;
    S->device = device;
    int rc = FTS_OK;
    try {
        std::string err;
        rc = build_topology(*mesh, S->topo, err);
        if (rc != FTS_OK) throw err;
        FTS_CUDA(cudaSetDevice(device));
        int sms = 0;
        FTS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        S->num_sms = sms > 0 ? sms : 148;
        FTS_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
        for (auto& e : S->ev) FTS_CUDA(cudaEventCreate(&e));
        const HostTopology& T = S->topo;
        S->np = T.np;
        S->nt = T.nt;
        S->nnz = T.rowptr[T.np];
        S->xyz = ls_alloc<float>(3 * S->np);
        S->tets = ls_alloc<int32_t>(4 * S->nt);
        S->rowptr = ls_alloc<int32_t>(S->np + 1);
        S->cols = ls_alloc<int32_t>(S->nnz);
        S->p2t_ptr = ls_alloc<int32_t>(S->np + 1);
        S->p2t = ls_alloc<uint32_t>(4 * S->nt);
        S->geom = ls_alloc<LsGeom>(S->nt);
        S->M = ls_alloc<double>(S->nnz);
        S->A = ls_alloc<double>(S->nnz);
        S->L = ls_alloc<double>(S->nnz);
        S->flow = ls_alloc<double>(4 * S->np);
        S->phi = ls_alloc<double>(S->np);
        for (auto& v : S->vec) v = ls_alloc<double>(S->np);
        S->keep = ls_alloc<uint8_t>(S->np);
        S->count = ls_alloc<unsigned>(1);
        S->flag = ls_alloc<int>(1);
        S->norm2 = ls_alloc<double>(1);
        S->S = ls_alloc<BjScalars>(1);
        FTS_CUDA(cudaMallocHost(&S->S_host, sizeof(BjScalars)));
        S->red.partials = ls_alloc<double>(kMaxPartials * 4);
        S->red.ticket = ls_alloc<unsigned>(1);
        FTS_CUDA(cudaMemset(S->red.ticket, 0, sizeof(unsigned)));
        FTS_CUDA(cudaMemcpy(S->xyz, mesh->xyz, 3 * S->np * sizeof(float), cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(S->tets, mesh->tets, 4 * S->nt * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(S->rowptr, T.rowptr.data(), (S->np + 1) * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(S->cols, T.cols.data(), S->nnz * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(S->p2t_ptr, T.p2t_ptr.data(), (S->np + 1) * sizeof(int32_t),
                            cudaMemcpyHostToDevice));
        FTS_CUDA(cudaMemcpy(S->p2t, T.p2t.data(), 4 * S->nt * sizeof(uint32_t),
                            cudaMemcpyHostToDevice));
        // the mass matrix, once per mesh (LevelSet.cpp:33-37)
        static const LsConst K = ls_const();
        FTS_CUDA(cudaMemset(S->flag, 0, sizeof(int)));
        k_ls_geometry<<<grid_of(*S, S->nt), kLsThreads, 0, S->stream>>>(S->nt, S->tets, S->xyz,
                                                                         S->geom, S->flag);
        if (T.max_row <= 255) {
            S->slots = ls_alloc<uint8_t>(16 * (size_t)S->nt);
            k_ls_slots<<<grid_of(*S, S->np), kLsThreads, 0, S->stream>>>(
                S->np, S->rowptr, S->cols, S->p2t_ptr, S->p2t, S->tets, S->slots);
        }
        k_ls_assemble<<<grid_of(*S, S->np), kLsThreads, 0, S->stream>>>(
            S->np, S->rowptr, S->cols, S->p2t_ptr, S->p2t, S->tets, S->geom, nullptr, K, S->slots,
            S->M);
        int bad = 0;
        FTS_CUDA(cudaMemcpyAsync(&bad, S->flag, sizeof(int), cudaMemcpyDeviceToHost, S->stream));
        FTS_CUDA(cudaStreamSynchronize(S->stream));
        if (bad) {
            err = "degenerate tetrahedron (det B == 0)";
            rc = FTS_ERR_DEGENERATE_ELEMENT;
            throw err;
        }
        rc = fts_dist_create(mesh->xyz, S->np, device, &S->dist);
        if (rc != FTS_OK) throw std::string(fts_dist_last_error(nullptr));
    } catch (const std::string& e) {
        g_ls_error() = e;
        if (rc == FTS_OK) rc = FTS_ERR_BAD_INPUT;
    } catch (const CudaError& e) {
        g_ls_error() = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        g_ls_error() = "host allocation failed";
        rc = FTS_ERR_OOM;
    }
    if (rc != FTS_OK) {
        ls_free(*S);
        delete S;
        return rc;
    }
    *out = S;
    return FTS_OK;
}

int fts_ls_update(fts_ls* S, const fts_ls_params* P, const double* flow, double* phi,
                  fts_ls_stats* stats) {
    if (!S || !P || !flow || !phi) return FTS_ERR_BAD_INPUT;
    const double t0 = wall_ms();
    fts_ls_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = FTS_OK;
    try {
        FTS_CUDA(cudaSetDevice(S->device));
        cudaStream_t s = S->stream;
        const int64_t np = S->np;
        const int g = grid_of(*S, np);
        int launches = 0;
        FTS_CUDA(cudaMemcpyAsync(S->flow, flow, 4 * np * sizeof(double), cudaMemcpyHostToDevice, s));
        FTS_CUDA(cudaMemcpyAsync(S->phi, phi, np * sizeof(double), cudaMemcpyHostToDevice, s));
        FTS_CUDA(cudaMemsetAsync(S->flag, 0, sizeof(int), s));
        k_ls_check_velocity<<<g, kLsThreads, 0, s>>>(4 * np, S->flow, S->flag, S->red, S->norm2);
        ++launches;
        int nanv = 0;
        double n2 = 0.0;
        FTS_CUDA(cudaMemcpyAsync(&nanv, S->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(&n2, S->norm2, sizeof(double), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        // LevelSet.cpp:91-93: nothing to advect (a NaN norm is not below FLT_MIN)
        if (P->dt < FLT_MIN || std::sqrt(n2) < FLT_MIN) {
            st.ms_total = wall_ms() - t0;
            if (stats) *stats = st;
            return FTS_OK;
        }
        if (nanv) {  // LevelSet.cpp:111-114
            S->last_error = "NaN in the velocity";
            st.status = FTS_ERR_NAN;
            st.ms_total = wall_ms() - t0;
            if (stats) *stats = st;
            return FTS_ERR_NAN;
        }
        static const LsConst K = ls_const();
        double* x = S->vec[0];
        double* b = S->vec[1];
        double* r = S->vec[2];
        double* r0 = S->vec[3];
        double* p = S->vec[4];
        double* vv = S->vec[5];
        double* sv = S->vec[6];
        double* t = S->vec[7];
        double* y = S->vec[8];
        double* z = S->vec[9];
        double* inv = S->vec[10];
        double* ifn = S->vec[11];
        FTS_CUDA(cudaEventRecord(S->ev[0], s));
        k_ls_assemble<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->p2t_ptr, S->p2t,
                                               S->tets, S->geom, S->flow, K, S->slots, S->A);
        k_ls_system<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->M, S->A, 0.5 * P->dt,
                                             S->phi, S->L, b, inv, x);
        FTS_CUDA(cudaEventRecord(S->ev[1], s));
        launches += 2;
        // Jacobi BiCGSTAB, device scalars; the host polls every few iterations
        BjScalars init{};
        const long long maxit = P->max_iter > 0 ? P->max_iter : 2 * np;
        init.maxit = maxit;
        FTS_CUDA(cudaMemcpyAsync(S->S, &init, sizeof(init), cudaMemcpyHostToDevice, s));
        const double tol = P->tol > 0.0 ? P->tol : DBL_EPSILON;
        k_bj_residual<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->L, b, x, r, r0, p, vv, 1,
                                               tol, S->red, S->S);
        ++launches;
        const int poll = 8;
        for (;;) {
            for (int u = 0; u < poll; ++u) {
                k_bj_p<<<g, kLsThreads, 0, s>>>(np, r, p, vv, inv, y, S->S);
                k_bj_spmv1<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->L, y, r0, vv,
                                                    S->red, S->S);
                k_bj_s<<<g, kLsThreads, 0, s>>>(np, r, vv, inv, sv, z, S->S);
                k_bj_spmv2<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->L, z, sv, t,
                                                    S->red, S->S);
                k_bj_update<<<g, kLsThreads, 0, s>>>(np, x, y, z, sv, t, r, r0, S->red, S->S);
                launches += 5;
            }
            FTS_CUDA(cudaGetLastError());
            FTS_CUDA(cudaMemcpyAsync(S->S_host, S->S, sizeof(BjScalars), cudaMemcpyDeviceToHost, s));
            FTS_CUDA(cudaStreamSynchronize(s));
            const BjScalars& H = *S->S_host;
            if (!H.stop) continue;
            if (H.restart) {
                k_bj_residual<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->L, b, x, r, r0,
                                                       p, vv, 0, tol, S->red, S->S);
                ++launches;
                continue;
            }
            break;
        }
        const BjScalars H = *S->S_host;
        if (H.bb == 0.0)  // Eigen: a zero right-hand side gives x = 0
            FTS_CUDA(cudaMemsetAsync(x, 0, np * sizeof(double), s));
        FTS_CUDA(cudaEventRecord(S->ev[2], s));
        st.iterations = H.it;
        st.error = H.bb > 0.0 ? std::sqrt(H.rr / H.bb) : 0.0;
        if (!(H.rr <= H.tol2) && H.bb != 0.0) {  // LevelSet.cpp:135-139: phi untouched
            S->last_error = "advection solve did not converge";
            rc = FTS_ERR_NOT_CONVERGED;
        } else if (!P->reset) {
            FTS_CUDA(cudaMemcpyAsync(phi, x, np * sizeof(double), cudaMemcpyDeviceToHost, s));
            FTS_CUDA(cudaStreamSynchronize(s));
        } else {
            // the distance reset (resetPhi_) of the advected phi
            const unsigned cap = (unsigned)std::min<int64_t>((S->nnz - np) / 2 + 1, 0x7fffffff);
            if (cap > S->ifp_cap) {
                if (S->ifp) cudaFree(S->ifp);
                S->ifp = nullptr;
                S->ifp = ls_alloc<float>(3 * (size_t)cap);
                S->ifp_cap = cap;
            }
            FTS_CUDA(cudaMemsetAsync(S->count, 0, sizeof(unsigned), s));
            FTS_CUDA(cudaMemsetAsync(S->keep, 0, np, s));
            k_ls_crossings<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, x, S->xyz, S->ifp,
                                                    S->count, S->keep, S->ifp_cap);
            ++launches;
            unsigned nif = 0;
            FTS_CUDA(cudaMemcpyAsync(&nif, S->count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
            FTS_CUDA(cudaStreamSynchronize(s));
            nif = std::min(nif, S->ifp_cap);
            FTS_CUDA(cudaMemcpyAsync(ifn, x, np * sizeof(double), cudaMemcpyDeviceToDevice, s));
            dist_reset_device(S->dist, S->ifp, true, (int32_t)nif, ifn, FTS_DIST_PRUNED, s, nullptr);
            k_ls_mix<<<g, kLsThreads, 0, s>>>(np, x, ifn, S->keep, S->phi);
            launches += nif > 0 ? 7 : 2;  // binning (5) and search, or the empty-set fill; mix
            S->have_reset = true;
            st.interface_points = nif;
            FTS_CUDA(cudaMemcpyAsync(phi, S->phi, np * sizeof(double), cudaMemcpyDeviceToHost, s));
        }
        FTS_CUDA(cudaEventRecord(S->ev[3], s));
        FTS_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        FTS_CUDA(cudaEventElapsedTime(&ms, S->ev[0], S->ev[1]));
        st.ms_assembly = ms;
        FTS_CUDA(cudaEventElapsedTime(&ms, S->ev[1], S->ev[2]));
        st.ms_solve = ms;
        FTS_CUDA(cudaEventElapsedTime(&ms, S->ev[2], S->ev[3]));
        st.ms_reset = ms;
        st.kernel_launches = launches;
    } catch (const CudaError& e) {
        S->last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        S->last_error = "host allocation failed";
        rc = FTS_ERR_OOM;
    }
    st.status = rc;
    st.ms_total = wall_ms() - t0;
    if (stats) *stats = st;
    return rc;
}

int fts_ls_reset_values(const fts_ls* S, double* phi_reset) {
    if (!S || !phi_reset) return FTS_ERR_BAD_INPUT;
    if (!S->have_reset) {
        const_cast<fts_ls*>(S)->last_error = "no update with a distance reset has run yet";
        return FTS_ERR_BAD_INPUT;
    }
    try {
        FTS_CUDA(cudaSetDevice(S->device));
        FTS_CUDA(cudaMemcpyAsync(phi_reset, S->vec[11], S->np * sizeof(double),
                                 cudaMemcpyDeviceToHost, S->stream));
        FTS_CUDA(cudaStreamSynchronize(S->stream));
    } catch (const CudaError& e) {
        const_cast<fts_ls*>(S)->last_error = e.what;
        return FTS_ERR_CUDA;
    }
    return FTS_OK;
}

int fts_ls_distance_reset(fts_ls* S, const double* phi, double* phi_reset) {
    if (!S || !phi || !phi_reset) return FTS_ERR_BAD_INPUT;
    try {
        FTS_CUDA(cudaSetDevice(S->device));
        cudaStream_t s = S->stream;
        const int64_t np = S->np;
        const int g = grid_of(*S, np);
        double* x = S->vec[0];
        double* ifn = S->vec[11];
        FTS_CUDA(cudaMemcpyAsync(x, phi, np * sizeof(double), cudaMemcpyHostToDevice, s));
        const unsigned cap = (unsigned)std::min<int64_t>((S->nnz - np) / 2 + 1, 0x7fffffff);
        if (cap > S->ifp_cap) {
            if (S->ifp) cudaFree(S->ifp);
            S->ifp = nullptr;
            S->ifp = ls_alloc<float>(3 * (size_t)cap);
            S->ifp_cap = cap;
        }
        FTS_CUDA(cudaMemsetAsync(S->count, 0, sizeof(unsigned), s));
        FTS_CUDA(cudaMemsetAsync(S->keep, 0, np, s));
        k_ls_crossings<<<g, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, x, S->xyz, S->ifp,
                                                S->count, S->keep, S->ifp_cap);
        FTS_CUDA(cudaGetLastError());
        unsigned nif = 0;
        FTS_CUDA(cudaMemcpyAsync(&nif, S->count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        nif = std::min(nif, S->ifp_cap);
        FTS_CUDA(cudaMemcpyAsync(ifn, x, np * sizeof(double), cudaMemcpyDeviceToDevice, s));
        dist_reset_device(S->dist, S->ifp, true, (int32_t)nif, ifn, FTS_DIST_PRUNED, s, nullptr);
        FTS_CUDA(cudaMemcpyAsync(phi_reset, ifn, np * sizeof(double), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        S->have_reset = true;
    } catch (const CudaError& e) {
        S->last_error = e.what;
        return e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    } catch (const std::bad_alloc&) {
        S->last_error = "host allocation failed";
        return FTS_ERR_OOM;
    }
    return FTS_OK;
}

int fts_ls_surface_tension(fts_ls* S, const double* phi, const double* phi_reset,
                           double surface_tension, int32_t node_density, double* force,
                           fts_st_stats* stats) {
    if (!S || !phi || !force) return FTS_ERR_BAD_INPUT;
    const double t0 = wall_ms();
    fts_st_stats st;
    std::memset(&st, 0, sizeof(st));
    int rc = FTS_OK;
    try {
        if (!phi_reset && !S->have_reset) {
            S->last_error = "phi_reset is NULL and no update with a distance reset has run";
            throw (int)FTS_ERR_BAD_INPUT;
        }
        FTS_CUDA(cudaSetDevice(S->device));
        cudaStream_t s = S->stream;
        const int64_t np = S->np, nt = S->nt;
        if (!S->st_phi) {
            S->st_phi = ls_alloc<double>(np);
            S->st_ifn = ls_alloc<double>(np);
            S->st_ge = ls_alloc<float>(3 * nt);
            S->st_nrm = ls_alloc<float>(3 * np);
            S->st_gn = ls_alloc<float>(3 * np);
            S->st_k = ls_alloc<float>(np);
            S->st_area = ls_alloc<float>(S->nnz);
            S->st_force = ls_alloc<double>(3 * np);
            S->st_acc = ls_alloc<double>(1);
            // every edge once at most
            S->st_list_cap = (unsigned)std::min<int64_t>((S->nnz - np) / 2 + 1, 0x7fffffff);
            S->st_list = ls_alloc<int2>(S->st_list_cap);
        }
        FTS_CUDA(cudaMemcpyAsync(S->st_phi, phi, np * sizeof(double), cudaMemcpyHostToDevice, s));
        const double* ifn = S->vec[11];
        if (phi_reset) {
            FTS_CUDA(cudaMemcpyAsync(S->st_ifn, phi_reset, np * sizeof(double),
                                     cudaMemcpyHostToDevice, s));
            ifn = S->st_ifn;
        }
        FTS_CUDA(cudaMemsetAsync(S->st_force, 0, 3 * np * sizeof(double), s));
        FTS_CUDA(cudaMemsetAsync(S->st_acc, 0, sizeof(double), s));
        FTS_CUDA(cudaMemsetAsync(S->count, 0, sizeof(unsigned), s));
        FTS_CUDA(cudaMemsetAsync(S->flag, 0, sizeof(int), s));
        const int ge = grid_of(*S, nt), gn = grid_of(*S, np);
        FTS_CUDA(cudaEventRecord(S->ev[0], s));
        k_st_elem_grad<<<ge, kLsThreads, 0, s>>>(nt, S->tets, S->geom, ifn, S->st_ge);
        k_st_node_avg<<<gn, kLsThreads, 0, s>>>(np, S->p2t_ptr, S->p2t, S->st_ge, 0, S->st_nrm,
                                                S->st_gn, S->st_k);
        k_st_elem_div<<<ge, kLsThreads, 0, s>>>(nt, S->tets, S->geom, S->st_gn, np, S->st_ge);
        k_st_node_avg<<<gn, kLsThreads, 0, s>>>(np, S->p2t_ptr, S->p2t, S->st_ge, 1, S->st_nrm,
                                                S->st_gn, S->st_k);
        k_st_cross_list<<<gn, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->st_phi, S->st_list,
                                                  S->st_list_cap, S->count);
        k_st_areas<<<S->num_sms * 8, kLsThreads, 0, s>>>(
            S->st_list, S->count, S->st_list_cap, S->cols, S->p2t_ptr, S->p2t, S->tets, S->xyz,
            S->st_phi, S->st_area, S->st_acc, S->flag);
        k_st_force<<<gn, kLsThreads, 0, s>>>(np, S->rowptr, S->cols, S->st_phi, S->st_area,
                                             S->st_k, S->st_nrm, (float)surface_tension,
                                             (int)node_density, S->st_force);
        FTS_CUDA(cudaGetLastError());
        FTS_CUDA(cudaEventRecord(S->ev[1], s));
        unsigned nif = 0;
        int bad = 0;
        double atot = 0.0;
        FTS_CUDA(cudaMemcpyAsync(&nif, S->count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(&bad, S->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(&atot, S->st_acc, sizeof(double), cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaMemcpyAsync(force, S->st_force, 3 * np * sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
        FTS_CUDA(cudaStreamSynchronize(s));
        float ms = 0.f;
        FTS_CUDA(cudaEventElapsedTime(&ms, S->ev[0], S->ev[1]));
        st.ms_kernels = ms;
        st.interface_points = nif;
        st.area = atot / 3.0;
        st.kernel_launches = 7;
        if (bad) {
            S->last_error = "an element crosses the interface on other than 3 or 4 edges";
            rc = FTS_ERR_BAD_INPUT;
        }
    } catch (int code) {
        rc = code;
    } catch (const CudaError& e) {
        S->last_error = e.what;
        rc = e.code == cudaErrorMemoryAllocation ? FTS_ERR_OOM : FTS_ERR_CUDA;
    }
    st.status = rc;
    st.ms_total = wall_ms() - t0;
    if (stats) *stats = st;
    return rc;
}

void fts_ls_destroy(fts_ls* S) {
    if (!S) return;
    cudaSetDevice(S->device);
    if (S->stream) cudaStreamSynchronize(S->stream);
    ls_free(*S);
    delete S;
}

const char* fts_ls_last_error(const fts_ls* S) {
    return S ? S->last_error.c_str() : g_ls_error().c_str();
}

}  // extern "C"
