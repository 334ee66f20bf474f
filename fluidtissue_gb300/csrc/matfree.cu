// Matrix-free element operator for the large single solve (operator_kind =
// FTS_OP_MATFREE, mixed precision, Kuhn lattices with the multigrid
// preconditioner).  No block matrix is stored: each element's rows are applied
// once and a thread per node adds the rows of the elements around it
// (atomic-free, deterministic):
//
//   velocity row a, component r:
//     mu V sum_c g_a[c] (G[r][c] + G[c][r])  -  V g_a[r] sum_b wq[b] p_b
//   pressure row a:
//     -wq[a] V div u  -  alpha h^2 V g_a . grad p  -  eps V sum_b mref[a][b] p_b
//
// with G[r][c] = sum_b u_{b,r} g_b[c] the element's velocity gradient — the
// same weak forms the assembled blocks hold (src/growth/Flow.cpp:54-72,
// :135-203, symmetric sign convention).  Dirichlet velocity rows are identity
// and Dirichlet velocity values are read as zero.
//
// FP32 inner operator: on meshes in the lattice generator's element order the
// geometry is recomputed from the coordinates, once per element: a thread per
// cube applies its 6 tetrahedra and writes the sums per cube corner
// (k_mf_cube), and a thread per node adds the corners it is of in the 8 cubes
// around it, fused with the MINRES dots (k_mf_gather_minres_A); otherwise a
// 64-byte FP32 record per element (gradients, volume, h^2, mu) built from the
// FP64 geometry, its rows applied by a thread per element (k_mf_elem32) and
// gathered in the node-element map's order (k_mf_gather_map_minres_A).
// FP64 outer residual: the stored FP64 ElemGeom, rows per element
// (k_mf_elem64) gathered in the map's order (k_mf_residual64).
#include <cfloat>

#include "fts_device.cuh"
#include "mg.cuh"
#include "mg_device.cuh"
#include "reduce.cuh"

namespace fts {

struct MfConst {
    float wq[4];
    float mref[4][4];
    double wqd[4];
    double mrefd[4][4];
};

static MfConst mf_const() {
    RefConstants R = ref_constants();
    MfConst m;
    for (int i = 0; i < 4; ++i) {
        m.wq[i] = (float)R.wq[i];
        m.wqd[i] = R.wq[i];
        for (int j = 0; j < 4; ++j) {
            m.mref[i][j] = (float)R.mref[i][j];
            m.mrefd[i][j] = R.mref[i][j];
        }
    }
    return m;
}

// FP32 element records for the inner operator, 64 B per element: gradients
// g[4][3], volume, h^2, mu (mu refreshed every solve), pad.
struct alignas(64) ElemF32 {
    float g[4][3];
    float vol, hh, mu, pad;
};

__global__ void k_mf_records(int64_t nt, const ElemGeom* __restrict__ geom,
                             const double* __restrict__ mu, ElemF32* __restrict__ rec) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const ElemGeom& G = geom[k];
        ElemF32 R;
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < 3; ++c) R.g[j][c] = (float)G.g[j][c];
        R.vol = (float)G.vol;
        R.hh = (float)G.hh;
        R.mu = (float)mu[k];
        R.pad = 0.f;
        rec[k] = R;
    }
}

// ---------------------------------------------------------------------------
// Kuhn-lattice form (elements in the order of the lattice generator: element
// 6c + t of cube c is the monotone path 0 -> e_p0 -> e_p0 + e_p1 -> (1,1,1) of
// axis permutation t).  A cube's 6 elements follow from its lattice position,
// and their geometry is recomputed in FP32 from the corner coordinates (edge
// vectors of nearby float coordinates are exact or nearly so), so one
// application reads 12 B of coordinates per node and 24 B of viscosity per
// cube, and writes and reads back 128 B of corner sums per cube — no element
// records, connectivity or node-element map.  Per node and element pair (the
// first version of this operator) the geometry was formed four times and the
// kernel took 4.94 ms at 257^3 against 2.04 ms for the two phases.
// ---------------------------------------------------------------------------
// FP32 geometry of a tetrahedron from its 4 vertices (the same formulas as the
// FP64 element geometry: B = [p1-p0, p2-p0, p3-p0], g = invB^T ghat, V = |det|/6,
// h = cbrt|det|, h^2 in float).
__device__ __forceinline__ void tet_geom_f32(const float p[4][3], float g[4][3], float& vol,
                                             float& hh) {
    float B[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        B[a][0] = p[1][a] - p[0][a];
        B[a][1] = p[2][a] - p[0][a];
        B[a][2] = p[3][a] - p[0][a];
    }
    const float c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1];
    const float c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2];
    const float c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
    const float det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
    float cof[3][3];
    cof[0][0] = c00;
    cof[0][1] = c01;
    cof[0][2] = c02;
    cof[1][0] = B[0][2] * B[2][1] - B[0][1] * B[2][2];
    cof[1][1] = B[0][0] * B[2][2] - B[0][2] * B[2][0];
    cof[1][2] = B[0][1] * B[2][0] - B[0][0] * B[2][1];
    cof[2][0] = B[0][1] * B[1][2] - B[0][2] * B[1][1];
    cof[2][1] = B[0][2] * B[1][0] - B[0][0] * B[1][2];
    cof[2][2] = B[0][0] * B[1][1] - B[0][1] * B[1][0];
    const float id = 1.f / det;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float it0 = cof[r][0] * id, it1 = cof[r][1] * id, it2 = cof[r][2] * id;
        g[0][r] = -it0 - it1 - it2;
        g[1][r] = it0;
        g[2][r] = it1;
        g[3][r] = it2;
    }
    const float adet = fabsf(det);
    vol = adet * (1.f / 6.f);
    const float h = cbrtf(adet);
    hh = h * h;
}

// The four rows a of one element applied to its nodal values u[4][4]
// (ux, uy, uz, p): the velocity gradient G and the pressure sums formed once,
// then per row the weak forms of the header.
template <typename T>
__device__ __forceinline__ void elem_apply4(const T g[4][3], T vol, T hh, T mu, const T u[4][4],
                                            T alpha, T eps, const T wq[4], const T mref[4][4],
                                            T y[4][4]) {
    T G[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            G[r][c] = u[0][r] * g[0][c] + u[1][r] * g[1][c] + u[2][r] * g[2][c] + u[3][r] * g[3][c];
    T gp[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) gp[c] = u[0][3] * g[0][c] + u[1][3] * g[1][c] + u[2][3] * g[2][c] + u[3][3] * g[3][c];
    const T pbar = wq[0] * u[0][3] + wq[1] * u[1][3] + wq[2] * u[2][3] + wq[3] * u[3][3];
    const T div = G[0][0] + G[1][1] + G[2][2];
    const T mv = mu * vol;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const T mp = mref[a][0] * u[0][3] + mref[a][1] * u[1][3] + mref[a][2] * u[2][3] + mref[a][3] * u[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
            y[a][r] = mv * (g[a][0] * (G[r][0] + G[0][r]) + g[a][1] * (G[r][1] + G[1][r]) +
                            g[a][2] * (G[r][2] + G[2][r])) -
                      vol * g[a][r] * pbar;
        y[a][3] = -wq[a] * vol * div - alpha * hh * vol * (g[a][0] * gp[0] + g[a][1] * gp[1] + g[a][2] * gp[2]) -
                  eps * vol * mp;
    }
}

// Phase 1 of the lattice matrix-free operator: a thread per cube (ci, cj, ck)
// of the (n-1)^3 cubes loads its 8 corners (corner q = dx + 2 dy + 4 dz),
// forms each of its 6 tetrahedra's geometry once (the monotone path
// 0 -> e_p0 -> e_p0 + e_p1 -> 7 of permutation t) and applies the element's
// four rows; the sums per corner and component go to
// out[(4 q + comp) * ncubes + cube] (coalesced for both phases).
__global__ void __launch_bounds__(kThreads)
k_mf_cube(int n, const float* __restrict__ xyz, const float* __restrict__ muf,
          const uint8_t* __restrict__ bnd, const V4<float>* __restrict__ Y, int ybuf, float alpha,
          float eps, MfConst K, const MinresScalars* __restrict__ s, float* __restrict__ out) {
    if (s->stop) return;
    const float wadd = (float)s->ycorr[ybuf];
    const int m = n - 1;
    const int nn = n * n;
    const int64_t ncubes = (int64_t)m * m * m;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncubes;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int ci = (int)(c % m), cj = (int)((c / m) % m), ck = (int)(c / ((int64_t)m * m));
        const int o = ci + n * (cj + n * ck);
        float p[8][3], u[8][4], acc[8][4];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int id = o + (q & 1) + n * ((q >> 1) & 1) + nn * (q >> 2);
            const float* xp = xyz + 3 * (int64_t)id;
            p[q][0] = __ldg(xp);
            p[q][1] = __ldg(xp + 1);
            p[q][2] = __ldg(xp + 2);
            const V4<float> xv = Y[id];
            const bool d = __ldg(bnd + id) != 0;
            u[q][0] = d ? 0.f : xv.x;
            u[q][1] = d ? 0.f : xv.y;
            u[q][2] = d ? 0.f : xv.z;
            u[q][3] = xv.w + wadd;
#pragma unroll
            for (int comp = 0; comp < 4; ++comp) acc[q][comp] = 0.f;
        }
#pragma unroll
        for (int t = 0; t < 6; ++t) {
            const int q1 = 1 << kuhn_p0(t), q2 = q1 | (1 << kuhn_p1(t));
            const int cq[4] = {0, q1, q2, 7};
            float pe[4][3], ue[4][4];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
#pragma unroll
                for (int a = 0; a < 3; ++a) pe[b][a] = p[cq[b]][a];
#pragma unroll
                for (int a = 0; a < 4; ++a) ue[b][a] = u[cq[b]][a];
            }
            float g[4][3], vol, hh, ye[4][4];
            tet_geom_f32(pe, g, vol, hh);
            elem_apply4<float>(g, vol, hh, __ldg(muf + 6 * c + t), ue, alpha, eps, K.wq, K.mref, ye);
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
                for (int comp = 0; comp < 4; ++comp) acc[cq[b]][comp] += ye[b][comp];
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
#pragma unroll
            for (int comp = 0; comp < 4; ++comp) out[(4 * q + comp) * ncubes + c] = acc[q][comp];
    }
}

// Phase 2: q = S (y + ycorr e_p) / beta at each node from the corner sums of
// the cubes around it (Dirichlet velocity rows identity), fused with the
// MINRES dots v.q and v.r1.
__global__ void __launch_bounds__(kThreads)
k_mf_gather_minres_A(int n, int64_t np, const float* __restrict__ cube,
                     const uint8_t* __restrict__ bnd, const V4<float>* __restrict__ Y, int ybuf,
                     const V4<float>* __restrict__ R1, V4<float>* __restrict__ q, Reduction red,
                     MinresScalars* s) {
    if (s->stop) return;
    const float tinv = (float)(1.0 / s->beta);
    const float wadd = (float)s->ycorr[ybuf];
    const int m = n - 1;
    const int nn = n * n;
    const int64_t ncubes = (int64_t)m * m * m;
    double acc[2] = {0.0, 0.0};
    for (int64_t v64 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v64 < np;
         v64 += (int64_t)gridDim.x * blockDim.x) {
        const int v = (int)v64;
        const int k = v / nn;
        const int rem = v - k * nn;
        const int j = rem / n;
        const int i = rem - j * n;
        float y[4] = {0.f, 0.f, 0.f, 0.f};
        // branch-free, so that all 32 loads are in flight at once: a cube
        // beyond the lattice is read at cube 0 and weighted by zero
#pragma unroll
        for (int corner = 0; corner < 8; ++corner) {
            const int dx = corner & 1, dy = (corner >> 1) & 1, dz = corner >> 2;
            const int ci = i - dx, cj = j - dy, ck = k - dz;
            const bool ok = ci >= 0 && cj >= 0 && ck >= 0 && ci < m && cj < m && ck < m;
            const int64_t cb = ok ? ci + (int64_t)m * (cj + (int64_t)m * ck) : 0;
            const float w = ok ? 1.f : 0.f;
#pragma unroll
            for (int comp = 0; comp < 4; ++comp)
                y[comp] = fmaf(w, __ldg(cube + (4 * corner + comp) * ncubes + cb), y[comp]);
        }
        const V4<float> yv = Y[v];
        if (bnd[v]) {
            y[0] = yv.x;
            y[1] = yv.y;
            y[2] = yv.z;
        }
        V4<float> o4;
        o4.x = y[0] * tinv;
        o4.y = y[1] * tinv;
        o4.z = y[2] * tinv;
        o4.w = y[3] * tinv;
        q[v] = o4;
        const V4<float> r1 = R1[v];
        const float v0 = yv.x * tinv, v1 = yv.y * tinv, v2 = yv.z * tinv, v3 = (yv.w + wadd) * tinv;
        acc[0] += (double)fmaf(v0, o4.x, fmaf(v1, o4.y, fmaf(v2, o4.z, v3 * o4.w)));
        acc[1] += (double)fmaf(v0, r1.x, fmaf(v1, r1.y, fmaf(v2, r1.z, v3 * r1.w)));
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
        s->alfa = tot[0] - c1 * tot[1];
    }
}

// The record form (any element order): a thread per element applies its four
// rows from its 64-byte record (k_mf_elem32, rows[4 k + a]); a thread per node
// adds the rows of its elements in the node-element map's order, fused with
// the MINRES dots (k_mf_gather_map_minres_A).
__global__ void __launch_bounds__(kThreads)
k_mf_elem32(int64_t nt, const int32_t* __restrict__ tets, const ElemF32* __restrict__ rec,
            const uint8_t* __restrict__ bnd, const V4<float>* __restrict__ Y, int ybuf,
            float alpha, float eps, MfConst K, const MinresScalars* __restrict__ s,
            V4<float>* __restrict__ rows) {
    if (s->stop) return;
    const float wadd = (float)s->ycorr[ybuf];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int4 t = __ldg(reinterpret_cast<const int4*>(tets) + k);
        const int ids[4] = {t.x, t.y, t.z, t.w};
        const float4* rp = reinterpret_cast<const float4*>(rec + k);
        const float4 r0 = __ldg(rp), r1v = __ldg(rp + 1), r2 = __ldg(rp + 2), r3 = __ldg(rp + 3);
        const float g[4][3] = {{r0.x, r0.y, r0.z}, {r0.w, r1v.x, r1v.y},
                               {r1v.z, r1v.w, r2.x}, {r2.y, r2.z, r2.w}};
        float u[4][4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const V4<float> xv = Y[ids[b]];
            const bool d = __ldg(bnd + ids[b]) != 0;
            u[b][0] = d ? 0.f : xv.x;
            u[b][1] = d ? 0.f : xv.y;
            u[b][2] = d ? 0.f : xv.z;
            u[b][3] = xv.w + wadd;
        }
        float y[4][4];
        elem_apply4<float>(g, r3.x, r3.y, r3.z, u, alpha, eps, K.wq, K.mref, y);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            V4<float> o;
            o.x = y[a][0];
            o.y = y[a][1];
            o.z = y[a][2];
            o.w = y[a][3];
            rows[4 * k + a] = o;
        }
    }
}

__global__ void __launch_bounds__(kThreads)
k_mf_gather_map_minres_A(int64_t np, const int32_t* __restrict__ p2t_ptr,
                         const uint32_t* __restrict__ p2t, const V4<float>* __restrict__ rows,
                         const uint8_t* __restrict__ bnd, const V4<float>* __restrict__ Y,
                         int ybuf, const V4<float>* __restrict__ R1, V4<float>* __restrict__ q,
                         Reduction red, MinresScalars* s) {
    if (s->stop) return;
    const float tinv = (float)(1.0 / s->beta);
    const float wadd = (float)s->ycorr[ybuf];
    double acc[2] = {0.0, 0.0};
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x) {
        float y[4] = {0.f, 0.f, 0.f, 0.f};
        for (int32_t qq = p2t_ptr[v]; qq < p2t_ptr[v + 1]; ++qq) {
            const uint32_t e = __ldg(p2t + qq);
            const V4<float> row = rows[4 * (int64_t)(e >> 2) + (e & 3)];
            y[0] += row.x;
            y[1] += row.y;
            y[2] += row.z;
            y[3] += row.w;
        }
        const V4<float> yv = Y[v];
        if (bnd[v]) {
            y[0] = yv.x;
            y[1] = yv.y;
            y[2] = yv.z;
        }
        V4<float> o;
        o.x = y[0] * tinv;
        o.y = y[1] * tinv;
        o.z = y[2] * tinv;
        o.w = y[3] * tinv;
        q[v] = o;
        const V4<float> r1 = R1[v];
        const float v0 = yv.x * tinv, v1 = yv.y * tinv, v2 = yv.z * tinv, v3 = (yv.w + wadd) * tinv;
        acc[0] += (double)fmaf(v0, o.x, fmaf(v1, o.y, fmaf(v2, o.z, v3 * o.w)));
        acc[1] += (double)fmaf(v0, r1.x, fmaf(v1, r1.y, fmaf(v2, r1.z, v3 * r1.w)));
    }
    double tot[2];
    if (grid_sum<2>(acc, red, tot) && threadIdx.x == 0) {
        const double c1 = s->iters >= 1 ? s->beta / s->oldb : 0.0;
        s->alfa = tot[0] - c1 * tot[1];
    }
}

__global__ void k_mu_f32(int64_t nt, const double* __restrict__ mu, float* __restrict__ muf) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x)
        muf[k] = (float)mu[k];
}

// FP64 outer residual r = b - S x (stored FP64 geometry), ||r||^2, ||b||^2, in
// two phases: a thread per element applies its four rows once
// (k_mf_elem64, rows[4 k + a]), and a thread per node adds the rows of its
// elements in the node-element map's order (k_mf_residual64) — the same row
// expressions and the same order of addition per node as gathering the rows
// element by element, without forming each element's velocity gradient four
// times (8.8 ms per residual at 129^3 for the one-phase form).
__global__ void __launch_bounds__(kThreads)
k_mf_elem64(int64_t nt, const int32_t* __restrict__ tets, const ElemGeom* __restrict__ geom,
            const double* __restrict__ mu, const uint8_t* __restrict__ bnd,
            const V4<double>* __restrict__ x, double alpha, double eps, MfConst K,
            V4<double>* __restrict__ rows) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int4 t = __ldg(reinterpret_cast<const int4*>(tets) + k);
        const int ids[4] = {t.x, t.y, t.z, t.w};
        const ElemGeom& G = geom[k];
        double g[4][3];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int c = 0; c < 3; ++c) g[j][c] = G.g[j][c];
        double u[4][4];
#pragma unroll
        for (int bb = 0; bb < 4; ++bb) {
            const V4<double> xv = x[ids[bb]];
            const bool d = __ldg(bnd + ids[bb]) != 0;
            u[bb][0] = d ? 0.0 : xv.x;
            u[bb][1] = d ? 0.0 : xv.y;
            u[bb][2] = d ? 0.0 : xv.z;
            u[bb][3] = xv.w;
        }
        double y[4][4];
        elem_apply4<double>(g, G.vol, G.hh, mu[k], u, alpha, eps, K.wqd, K.mrefd, y);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            V4<double> o;
            o.x = y[a][0];
            o.y = y[a][1];
            o.z = y[a][2];
            o.w = y[a][3];
            rows[4 * k + a] = o;
        }
    }
}

__global__ void __launch_bounds__(kThreads)
k_mf_residual64(int64_t np, const int32_t* __restrict__ p2t_ptr, const uint32_t* __restrict__ p2t,
                const V4<double>* __restrict__ rows, const uint8_t* __restrict__ bnd,
                const V4<double>* __restrict__ x, const V4<double>* __restrict__ b,
                V4<double>* __restrict__ r, Reduction red, OuterScalars* os) {
    double acc[2] = {0.0, 0.0};
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x) {
        double y[4] = {0.0, 0.0, 0.0, 0.0};
        for (int32_t qq = p2t_ptr[v]; qq < p2t_ptr[v + 1]; ++qq) {
            const uint32_t e = __ldg(p2t + qq);
            const V4<double> row = rows[4 * (int64_t)(e >> 2) + (e & 3)];
            y[0] += row.x;
            y[1] += row.y;
            y[2] += row.z;
            y[3] += row.w;
        }
        const V4<double> xv = x[v];
        if (bnd[v]) {
            y[0] = xv.x;
            y[1] = xv.y;
            y[2] = xv.z;
        }
        const V4<double> bv = b[v];
        V4<double> o;
        o.x = bv.x - y[0];
        o.y = bv.y - y[1];
        o.z = bv.z - y[2];
        o.w = bv.w - y[3];
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

// Pressure weight of the preconditioner per node (the velocity part is the
// multigrid V-cycle): 1 / (alpha D_ii + eps M_ii + s sum_e vol/(4 mu_e)), s =
// schur_scale.
__global__ void k_mf_pc(int64_t np, const int32_t* __restrict__ p2t_ptr,
                        const uint32_t* __restrict__ p2t, const ElemGeom* __restrict__ geom,
                        const double* __restrict__ mu, double alpha, double eps, MfConst K,
                        const OuterScalars* __restrict__ os, float* __restrict__ pc) {
    const double ws = schur_scale(os);
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < np;
         v += (int64_t)gridDim.x * blockDim.x) {
        double d = 0.0;
        for (int32_t qq = p2t_ptr[v]; qq < p2t_ptr[v + 1]; ++qq) {
            const uint32_t e = p2t[qq];
            const int64_t k = e >> 2;
            const int a = e & 3;
            const ElemGeom& G = geom[k];
            const double gg = G.g[a][0] * G.g[a][0] + G.g[a][1] * G.g[a][1] + G.g[a][2] * G.g[a][2];
            d += alpha * G.hh * G.vol * gg + eps * G.vol * K.mrefd[a][a];
        }
        d += ws * lumped_inv_mu(v, p2t_ptr, p2t, geom, mu);
        float* o = pc + 8 * v;
        o[0] = 1.f;
        o[1] = 0.f;
        o[2] = 0.f;
        o[3] = 1.f;
        o[4] = 0.f;
        o[5] = 1.f;
        o[6] = (float)(1.0 / d);
        o[7] = 0.f;
    }
}

void launch_mf_minres_A(Ctx& c, const V4<float>* Y, int ybuf, const V4<float>* R1, V4<float>* q) {
    static const MfConst K = mf_const();
    if (c.topo.kuhn_elements) {
        const int n = c.topo.lattice_n;
        const int64_t ncubes = (int64_t)(n - 1) * (n - 1) * (n - 1);
        if (!c.mf_cube) c.mf_cube = dev_alloc<float>(c, (size_t)ncubes * 32);
        k_mf_cube<<<grid_for(c, ncubes), kThreads, 0, c.stream>>>(
            n, c.xyz, c.mf_rec, c.bnd, Y, ybuf, (float)c.par.alpha, (float)c.par.eps, K, c.ms,
            c.mf_cube);
        k_mf_gather_minres_A<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
            n, c.np, c.mf_cube, c.bnd, Y, ybuf, R1, q, c.red, c.ms);
        c.launches += 2;
        return;
    }
    if (!c.mf_cube) c.mf_cube = dev_alloc<float>(c, (size_t)c.nt * 16);  // rows[4 nt]
    V4<float>* rows = reinterpret_cast<V4<float>*>(c.mf_cube);
    k_mf_elem32<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(
        c.nt, c.tets, reinterpret_cast<const ElemF32*>(c.mf_rec), c.bnd, Y, ybuf,
        (float)c.par.alpha, (float)c.par.eps, K, c.ms, rows);
    k_mf_gather_map_minres_A<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
        c.np, c.p2t_ptr, c.p2t, rows, c.bnd, Y, ybuf, R1, q, c.red, c.ms);
    c.launches += 2;
}

void launch_mf_residual64(Ctx& c) {
    static const MfConst K = mf_const();
    if (!c.mf_rows) c.mf_rows = dev_alloc<double>(c, (size_t)c.nt * 16);
    V4<double>* rows = reinterpret_cast<V4<double>*>(c.mf_rows);
    k_mf_elem64<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(
        c.nt, c.tets, c.geom, c.mu, c.bnd, c.x, c.par.alpha, c.par.eps, K, rows);
    k_mf_residual64<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
        c.np, c.p2t_ptr, c.p2t, rows, c.bnd, c.x, c.b, c.r, c.red, c.os);
    FTS_CUDA(cudaGetLastError());
    c.launches += 2;
}

void launch_mf_pc(Ctx& c) {
    static const MfConst K = mf_const();
    static_assert(sizeof(ElemF32) == 64, "64-byte element record");
    if (c.topo.kuhn_elements) {  // lattice form: FP32 viscosity only
        if (!c.mf_rec) c.mf_rec = dev_alloc<float>(c, (size_t)c.nt);
        k_mu_f32<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(c.nt, c.mu, c.mf_rec);
    } else {
        if (!c.mf_rec) c.mf_rec = dev_alloc<float>(c, (size_t)c.nt * 16);
        k_mf_records<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(
            c.nt, c.geom, c.mu, reinterpret_cast<ElemF32*>(c.mf_rec));
    }
    c.launches += 1;
    // with both V-cycles no node weight is read (velocity and pressure come
    // from the hierarchies)
    if (c.use_mg && c.use_pmg) return;
    k_mf_pc<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(c.np, c.p2t_ptr, c.p2t, c.geom, c.mu,
                                                         c.par.alpha, c.par.eps, K, c.os,
                                                         c.pc32);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

}  // namespace fts
