// P2-P1 (Taylor-Hood) assembly of the Stokes system, the reference's velocity
// degree 2 (src/growth/Flow.cpp:20-94, :102-214, :345-399 with uDeg_ = 2;
// element integrals by bilin_without_p2t_ij, src/fem/Assembler.hpp:321-424).
//
// System nodes are the mesh vertices followed by the edges (the reference's
// DOF order "vertices, then edges", TetraMesh.cpp:219-258; the edge numbering
// differs, which changes nothing in the solution at the vertices).  Every
// node carries a 4x4 block row (ux, uy, uz, p) in the same symmetric form as
// P1: K (the symmetric-gradient viscous block, degree-4 rule), -B (velocity
// test x pressure trial, degree-3 rule), and -eps M on the pressure block
// (Taylor-Hood has no Brezzi-Pitkaranta term, Flow.cpp:190-192).  Edge nodes
// have no pressure: their pressure row and column are zero and the
// preconditioner gives them weight zero, so the placeholder never enters the
// iteration (a -1 diagonal would, through the rank-one pressure term of the
// preconditioner, and stalled the FP32 inner solve).  Dirichlet velocity rows
// and columns as in P1, on the vertices and edges of the boundary triangles.
//
// Element integrals come from reference tensors (RefP2) contracted with
// G = invB^T: int grad phi_a . grad phi_b = vol sum_mn (G^T G)_mn K[a][b][m][n]
// etc., the same quadrature sums regrouped.
#include <cstring>

#include "fts_device.cuh"

namespace fts {

struct P2Const {
    double K[10][10][3][3];
    double B[10][4][3];
    double N[10][4];
    double M[4][4];  // P1 mass on the degree-2 rule (mref)
};
__constant__ P2Const c_p2;

static void init_p2_tables(int device) {
    static bool done[64] = {};
    if (device < 64 && done[device]) return;
    const RefP2 R = ref_p2();
    const RefConstants P = ref_constants();
    P2Const h;
    std::memcpy(h.K, R.K, sizeof(h.K));
    std::memcpy(h.B, R.B, sizeof(h.B));
    std::memcpy(h.N, R.N, sizeof(h.N));
    std::memcpy(h.M, P.mref, sizeof(h.M));
    FTS_CUDA(cudaMemcpyToSymbol(c_p2, &h, sizeof(h)));
    if (device < 64) done[device] = true;
}

// G[r][c] = (invB^T)_rc = gradient of the P1 basis c+1 (ElemGeom.g[c+1][r]).
__device__ __forceinline__ void p2_jacobian(const ElemGeom& E, double G[3][3]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) G[r][c] = E.g[c + 1][r];
}

// One thread per system node i (a block row): the element contributions of
// every element holding i as local DOF a, added to the row's blocks in
// element order, then the Dirichlet masking.
__global__ void k_assemble_p2(int64_t nn, int64_t nv, const int32_t* __restrict__ rowptr,
                              const int32_t* __restrict__ cols,
                              const int32_t* __restrict__ xp2t_ptr,
                              const uint32_t* __restrict__ xp2t, const int32_t* __restrict__ dofs,
                              const ElemGeom* __restrict__ geom, const double* __restrict__ mu,
                              const uint8_t* __restrict__ bnd, double eps,
                              double* __restrict__ A) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c0 = rowptr[i], c1 = rowptr[i + 1];
        for (int64_t e = (int64_t)c0 * 16; e < (int64_t)c1 * 16; ++e) A[e] = 0.0;
        for (int32_t q = xp2t_ptr[i]; q < xp2t_ptr[i + 1]; ++q) {
            const int64_t k = xp2t[q] >> 4;
            const int a = (int)(xp2t[q] & 15);
            const ElemGeom& E = geom[k];
            double G[3][3];
            p2_jacobian(E, G);
            double GtG[3][3];
#pragma unroll
            for (int m = 0; m < 3; ++m)
#pragma unroll
                for (int n = 0; n < 3; ++n)
                    GtG[m][n] = G[0][m] * G[0][n] + G[1][m] * G[1][n] + G[2][m] * G[2][n];
            const double vol = E.vol, mv = mu[k] * vol;
            const int32_t* d = dofs + 10 * k;
            for (int b = 0; b < 10; ++b) {
                const int32_t j = d[b];
                int lo = c0, hi = c1 - 1;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (cols[mid] < j) lo = mid + 1;
                    else hi = mid;
                }
                double* blk = A + (int64_t)lo * 16;
                // viscous block: mu (delta_rc grad a . grad b + d_c phi_a d_r phi_b)
                double gg = 0.0;
                double T[3][3];  // T[m][n] = K[a][b][m][n]
#pragma unroll
                for (int m = 0; m < 3; ++m)
#pragma unroll
                    for (int n = 0; n < 3; ++n) {
                        T[m][n] = c_p2.K[a][b][m][n];
                        gg += GtG[m][n] * T[m][n];
                    }
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        double x = 0.0;
#pragma unroll
                        for (int m = 0; m < 3; ++m)
#pragma unroll
                            for (int n = 0; n < 3; ++n) x += G[c][m] * G[r][n] * T[m][n];
                        blk[4 * r + c] += mv * ((r == c ? gg : 0.0) + x);
                    }
                if (b < 4) {  // -B_r(a, b): velocity test a, pressure trial b
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        blk[4 * r + 3] -= vol * (G[r][0] * c_p2.B[a][b][0] + G[r][1] * c_p2.B[a][b][1] +
                                                 G[r][2] * c_p2.B[a][b][2]);
                }
                if (a < 4) {  // pressure row: -B_c(b, a)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        blk[12 + c] -= vol * (G[c][0] * c_p2.B[b][a][0] + G[c][1] * c_p2.B[b][a][1] +
                                              G[c][2] * c_p2.B[b][a][2]);
                    if (b < 4) blk[15] -= eps * (vol * c_p2.M[a][b]);
                }
            }
        }
        const bool bi = bnd[i] != 0;
        for (int32_t s = c0; s < c1; ++s) {
            const int32_t j = cols[s];
            double* blk = A + (int64_t)s * 16;
            const bool bj = bnd[j] != 0;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int r = e >> 2, c = e & 3;
                if (bi && r < 3) blk[e] = (j == i && r == c) ? 1.0 : 0.0;
                else if (c < 3 && bj) blk[e] = 0.0;
            }
        }
    }
}

// Right-hand side (Flow.cpp:392-396) for P2: F_al(i) = sum N(i,k) f_al(k) +
// sum C_al(i,k) s_k over the vertices k, C_al = int (2/3 mu) psi_k d_al phi_i;
// F_p(i) = sum M(i,k) s_k on the vertices.  b = (F_x, F_y, F_z, -F_p), zero on
// Dirichlet velocity rows and on the edge nodes' pressure.
__global__ void k_rhs_p2(int64_t nn, int64_t nv, const int32_t* __restrict__ xp2t_ptr,
                         const uint32_t* __restrict__ xp2t, const int32_t* __restrict__ dofs,
                         const ElemGeom* __restrict__ geom, const double* __restrict__ mu,
                         const double* __restrict__ s, const double* __restrict__ force,
                         const uint8_t* __restrict__ bnd, const OuterScalars* __restrict__ os,
                         V4<double>* __restrict__ b) {
    const double mean = os->sum;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn;
         i += (int64_t)gridDim.x * blockDim.x) {
        double F[4] = {0.0, 0.0, 0.0, 0.0};
        for (int32_t q = xp2t_ptr[i]; q < xp2t_ptr[i + 1]; ++q) {
            const int64_t k = xp2t[q] >> 4;
            const int a = (int)(xp2t[q] & 15);
            const ElemGeom& E = geom[k];
            double G[3][3];
            p2_jacobian(E, G);
            const double vol = E.vol, cm = (2.0 / 3 * mu[k]) * vol;
            const int32_t* d = dofs + 10 * k;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const double sv = s[d[kk]] - mean;
#pragma unroll
                for (int al = 0; al < 3; ++al) {
                    const double bint = G[al][0] * c_p2.B[a][kk][0] + G[al][1] * c_p2.B[a][kk][1] +
                                        G[al][2] * c_p2.B[a][kk][2];
                    F[al] += cm * bint * sv;
                    if (force) F[al] += vol * c_p2.N[a][kk] * force[al * nv + d[kk]];
                }
                if (a < 4) F[3] += vol * c_p2.M[a][kk] * sv;
            }
        }
        V4<double> o;
        const bool dd = bnd[i] != 0;
        o.x = dd ? 0.0 : F[0];
        o.y = dd ? 0.0 : F[1];
        o.z = dd ? 0.0 : F[2];
        o.w = i < nv ? -F[3] : 0.0;
        b[i] = o;
    }
}

void launch_assemble_p2(Ctx& c) {
    init_p2_tables(c.device);
    if (!c.A64) c.A64 = dev_alloc<double>(c, (size_t)c.nnzb * 16);
    k_assemble_p2<<<grid_for(c, c.np, 128), 128, 0, c.stream>>>(
        c.np, c.nv, c.rowptr, c.cols, c.xp2t_ptr, c.xp2t, c.dofs, c.geom, c.mu, c.bnd, c.par.eps,
        c.A64);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
    c.a64_valid = true;
}

void launch_rhs_p2(Ctx& c, bool have_force) {
    init_p2_tables(c.device);
    k_rhs_p2<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
        c.np, c.nv, c.xp2t_ptr, c.xp2t, c.dofs, c.geom, c.mu, c.s, have_force ? c.force : nullptr,
        c.bnd, c.os, c.b);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

}  // namespace fts
