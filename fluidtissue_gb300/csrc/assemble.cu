// Element geometry, viscosity profile, mass source, right-hand side, block
// assembly and preconditioner set-up of the P1-P1 stabilised Stokes system.
//
// Reference arithmetic (paths relative to the reference project):
//   element geometry            src/fem/Assembler.hpp:430-462, h :193
//   weak forms / composition    src/growth/Flow.cpp:54-72, :135-203
//   viscosity profile           src/growth/ViscosityProfiles.hpp:27-72
//   source and RHS              src/growth/Flow.cpp:365-399
//
// The system is stored node-blocked: block (i,j) is the 4x4 coupling of the
// unknowns (ux,uy,uz,p) of nodes i and j, row-major.  Pressure rows are negated
// (the symmetric form  [K -B; -B^T -(alpha D + eps M)]  of the reference's
// [K -B; B^T alpha D + eps M], same solution), and the Dirichlet velocity rows
// and columns of boundary nodes are identity / zero instead of being removed
// (subSparse, Flow.cpp:206), which leaves the interior solution unchanged.
#include <cfloat>

#include "fts_device.cuh"
#include "mg_device.cuh"
#include "reduce.cuh"

namespace fts {

struct RefArgs {
    double wq[4];
    double mref[4][4];
};

static RefArgs ref_args() {
    RefConstants R = ref_constants();
    RefArgs a;
    for (int i = 0; i < 4; ++i) {
        a.wq[i] = R.wq[i];
        for (int j = 0; j < 4; ++j) a.mref[i][j] = R.mref[i][j];
    }
    return a;
}

// ---------------------------------------------------------------------------
// Geometry: detB = |det B|, invB^T, gradients, volume, h^2 (float), per element.
// ---------------------------------------------------------------------------
__global__ void k_geometry(int64_t nt, const float* __restrict__ xyz,
                           const int32_t* __restrict__ tets, ElemGeom* __restrict__ geom,
                           int* __restrict__ bad) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        int4 t = reinterpret_cast<const int4*>(tets)[k];
        int ids[4] = {t.x, t.y, t.z, t.w};
        double p[4][3];
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int a = 0; a < 3; ++a) p[j][a] = (double)xyz[3 * (int64_t)ids[j] + a];
        double B[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            B[a][0] = p[1][a] - p[0][a];
            B[a][1] = p[2][a] - p[0][a];
            B[a][2] = p[3][a] - p[0][a];
        }
        double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1];
        double c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2];
        double c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
        double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
        double adet = fabs(det);
        ElemGeom G;
        if (!(adet > 0.0) || !isfinite(adet)) {
            atomicOr(bad, 1);
            adet = 1.0;
            det = 1.0;
        }
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
        const double id = 1.0 / det;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            double it0 = cof[r][0] * id, it1 = cof[r][1] * id, it2 = cof[r][2] * id;
            G.g[0][r] = -it0 - it1 - it2;
            G.g[1][r] = it0;
            G.g[2][r] = it1;
            G.g[3][r] = it2;
        }
        G.vol = adet / 6.0;
        float h = (float)cbrt(adet);
        float hh = h * h;
        G.hh = (double)hh;
        G.pad[0] = G.pad[1] = 0.0;
        geom[k] = G;
    }
}

void launch_geometry(Ctx& c, int* bad) {
    k_geometry<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(c.nt, c.xyz, c.tets, c.geom, bad);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// ---------------------------------------------------------------------------
// setViscosity (ViscosityProfiles.hpp:27-72): mu_ext everywhere; on interior
// elements (all four nodes phi < 0, LevelSet.cpp:180-196) blended by the
// largest nodal growth factor.
// ---------------------------------------------------------------------------
__global__ void k_viscosity_profile(int64_t nt, const int32_t* __restrict__ tets,
                                    const double* __restrict__ phi,
                                    const double* __restrict__ gf, double mu_h, double mu_l,
                                    int profile, double maxGF, double* __restrict__ mu) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        int4 t = reinterpret_cast<const int4*>(tets)[k];
        double m = mu_l;
        if (phi[t.x] < 0.0 && phi[t.y] < 0.0 && phi[t.z] < 0.0 && phi[t.w] < 0.0) {
            double c3 = fmax(fmax(gf[t.x], gf[t.y]), fmax(gf[t.z], gf[t.w]));
            if (profile == 0) m = mu_l * (c3 / maxGF) + mu_h * (1.0 - c3 / maxGF);
            if (profile == 1) m = mu_h * (c3 / maxGF) + mu_l * (1.0 - c3 / maxGF);
            if (profile == 2) {
                c3 *= 4.0;
                if (c3 > maxGF) c3 = maxGF;
                m = mu_h * (c3 / maxGF) + mu_l * (1.0 - c3 / maxGF);
            }
        }
        mu[k] = m;
    }
}

void launch_viscosity_profile(Ctx& c) {
    const fts_params& P = c.par;
    double maxGF = P.rd_iterations > 0.0 ? P.gf_production : 1.0;
    k_viscosity_profile<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(
        c.nt, c.tets, c.phi, c.src, P.mu_interior, P.mu_exterior, P.mu_profile, maxGF, c.mu);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// min / max of mu over interior elements (the values Flow.cpp:241 prints).
__global__ void k_mu_minmax(int64_t nt, const int32_t* __restrict__ tets,
                            const double* __restrict__ phi, const double* __restrict__ mu,
                            Reduction red, OuterScalars* os) {
    // [0] interior min, [1] interior max, [2] min, [3] max
    double m[4] = {DBL_MAX, -DBL_MAX, DBL_MAX, -DBL_MAX};
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nt;
         k += (int64_t)gridDim.x * blockDim.x) {
        int4 t = reinterpret_cast<const int4*>(tets)[k];
        const double u = mu[k];
        if (phi[t.x] < 0.0 && phi[t.y] < 0.0 && phi[t.z] < 0.0 && phi[t.w] < 0.0) {
            m[0] = fmin(m[0], u);
            m[1] = fmax(m[1], u);
        }
        m[2] = fmin(m[2], u);
        m[3] = fmax(m[3], u);
    }
    // reduce through shuffles; partials via the ticket
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double other = __shfl_xor_sync(0xffffffffu, m[q], o);
            m[q] = (q & 1) ? fmax(m[q], other) : fmin(m[q], other);
        }
    }
    __shared__ double sm[4][32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int q = 0; q < 4; ++q) sm[q][wid] = m[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            for (int q = 0; q < 4; ++q)
                m[q] = (q & 1) ? fmax(m[q], sm[q][w]) : fmin(m[q], sm[q][w]);
        for (int q = 0; q < 4; ++q) red.partials[q * kMaxPartials + blockIdx.x] = m[q];
    }
    if (last_block(red) && threadIdx.x == 0) {
        double a[4] = {DBL_MAX, -DBL_MAX, DBL_MAX, -DBL_MAX};
        for (unsigned i = 0; i < gridDim.x; ++i)
            for (int q = 0; q < 4; ++q) {
                const double p = __ldcg(&red.partials[q * kMaxPartials + i]);
                a[q] = (q & 1) ? fmax(a[q], p) : fmin(a[q], p);
            }
        os->mu_min = a[0];
        os->mu_max = a[1];
        os->mu_all_min = a[2];
        os->mu_all_max = a[3];
    }
}

void launch_mu_minmax(Ctx& c) {
    k_mu_minmax<<<grid_for(c, c.nt), kThreads, 0, c.stream>>>(c.nt, c.tets, c.phi, c.mu, c.red,
                                                               c.os);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// ---------------------------------------------------------------------------
// Mass source (Flow.cpp:365-376): s_i = (c_i - sink) * growth on interior nodes
// with c_i > threshold; the mean over all nodes goes to os->sum (subtracted in
// the RHS kernel).
// ---------------------------------------------------------------------------
__global__ void k_source(int64_t np, const double* __restrict__ phi, const double* __restrict__ c,
                         double growth, double sink, double thr, double* __restrict__ s,
                         Reduction red, OuterScalars* os) {
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        double v = 0.0;
        if (phi[i] < 0.0 && c[i] > thr) v = (c[i] - sink) * growth;
        s[i] = v;
        acc[0] += v;
    }
    double tot[1];
    if (grid_sum<1>(acc, red, tot) && threadIdx.x == 0) os->sum = tot[0] / (double)np;
}

void launch_source(Ctx& c) {
    const fts_params& P = c.par;
    k_source<<<grid_for(c, c.nv), kThreads, 0, c.stream>>>(c.nv, c.phi, c.src, P.gf_growth,
                                                           P.level_sink, P.growth_threshold,
                                                           c.s, c.red, c.os);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// ---------------------------------------------------------------------------
// Right-hand side (Flow.cpp:392-396), gathered per node over its elements:
//   F_al(i) = sum_j N(i,j) f_al(j) + sum_j C_al(i,j) s_j,
//   C_al(i,j) = int (2/3 mu) psi_j d_al phi_i,    F_p(i) = sum_j M(i,j) s_j.
// Stored as b = (F_x, F_y, F_z, -F_p), zero on Dirichlet velocity rows.
// ---------------------------------------------------------------------------
__global__ void k_rhs(int64_t np, const int32_t* __restrict__ p2t_ptr,
                      const uint32_t* __restrict__ p2t, const int32_t* __restrict__ tets,
                      const ElemGeom* __restrict__ geom, const double* __restrict__ mu,
                      const double* __restrict__ s, const double* __restrict__ force,
                      const uint8_t* __restrict__ bnd, const OuterScalars* __restrict__ os,
                      RefArgs R, V4<double>* __restrict__ b) {
    const double mean = os->sum;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        double F[4] = {0.0, 0.0, 0.0, 0.0};
        for (int32_t q = p2t_ptr[i]; q < p2t_ptr[i + 1]; ++q) {
            uint32_t e = p2t[q];
            int64_t k = e >> 2;
            int a = e & 3;
            int4 t = reinterpret_cast<const int4*>(tets)[k];
            int ids[4] = {t.x, t.y, t.z, t.w};
            const ElemGeom& G = geom[k];
            double vol = G.vol;
            double sv[4], sw = 0.0, ms = 0.0;
#pragma unroll
            for (int bb = 0; bb < 4; ++bb) {
                sv[bb] = s[ids[bb]] - mean;
                sw += R.wq[bb] * sv[bb];
                ms += R.mref[a][bb] * sv[bb];
            }
            double cfac = (2.0 / 3 * mu[k]) * vol * sw;
#pragma unroll
            for (int al = 0; al < 3; ++al) F[al] += cfac * G.g[a][al];
            F[3] += vol * ms;
            if (force) {
#pragma unroll
                for (int al = 0; al < 3; ++al) {
                    double fm = 0.0;
#pragma unroll
                    for (int bb = 0; bb < 4; ++bb) fm += R.mref[a][bb] * force[al * np + ids[bb]];
                    F[al] += vol * fm;
                }
            }
        }
        V4<double> o;
        bool d = bnd[i] != 0;
        o.x = d ? 0.0 : F[0];
        o.y = d ? 0.0 : F[1];
        o.z = d ? 0.0 : F[2];
        o.w = -F[3];
        b[i] = o;
    }
}

void launch_rhs(Ctx& c, bool have_force) {
    k_rhs<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(c.np, c.p2t_ptr, c.p2t, c.tets, c.geom,
                                                        c.mu, c.s, have_force ? c.force : nullptr,
                                                        c.bnd, c.os, ref_args(), c.b);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// ---------------------------------------------------------------------------
// Block assembly: one warp per block row i (atomic-free, as the reference's
// node-row gather, Assembler.hpp:150-225).  The warp walks the elements around
// node i; for each element every lane owns two of the 4 x 16 entries it adds
// to row i (column node b = lane / 8), accumulated in a shared-memory copy of
// the row, which is then written out coalesced with the Dirichlet masking.
// ---------------------------------------------------------------------------
__global__ void k_assemble(int64_t np, const int32_t* __restrict__ rowptr,
                           const int32_t* __restrict__ cols, const int32_t* __restrict__ p2t_ptr,
                           const uint32_t* __restrict__ p2t, const int32_t* __restrict__ tets,
                           const ElemGeom* __restrict__ geom, const double* __restrict__ mu,
                           const uint8_t* __restrict__ bnd, double alpha, double eps, RefArgs R,
                           int max_row, double* __restrict__ A) {
    extern __shared__ double smem[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    double* buf = smem + (size_t)wib * max_row * 16;
    const int b = lane >> 3;        // column node (local index) handled by this lane
    const int e0 = (lane & 7) * 2;  // first of the two entries
    for (int64_t i = (int64_t)blockIdx.x * wpb + wib; i < np; i += (int64_t)gridDim.x * wpb) {
        const int32_t c0 = rowptr[i];
        const int ncol = rowptr[i + 1] - c0;
        for (int e = lane; e < ncol * 16; e += 32) buf[e] = 0.0;
        __syncwarp();
        for (int32_t q = p2t_ptr[i]; q < p2t_ptr[i + 1]; ++q) {
            const uint32_t pk = p2t[q];
            const int64_t k = pk >> 2;
            const int a = pk & 3;
            const int4 t = reinterpret_cast<const int4*>(tets)[k];
            const int tb = b == 0 ? t.x : (b == 1 ? t.y : (b == 2 ? t.z : t.w));
            // slot of node tb in row i (sorted columns)
            int lo = 0, hi = ncol - 1;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (cols[c0 + mid] < tb) lo = mid + 1;
                else hi = mid;
            }
            const ElemGeom* G = geom + k;
            const double ga0 = G->g[a][0], ga1 = G->g[a][1], ga2 = G->g[a][2];
            const double gb0 = G->g[b][0], gb1 = G->g[b][1], gb2 = G->g[b][2];
            const double vol = G->vol;
            const double gg = ga0 * gb0 + ga1 * gb1 + ga2 * gb2;
            const double mv = mu[k] * vol;
            const double ga[3] = {ga0, ga1, ga2}, gb[3] = {gb0, gb1, gb2};
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int e = e0 + u;
                const int r = e >> 2, cc = e & 3;
                double v;
                if (r < 3 && cc < 3) {
                    // K_{r,cc}(i,j) = mu vol (delta gg + d_cc phi_i d_r phi_j)
                    v = mv * ((r == cc ? gg : 0.0) + ga[cc] * gb[r]);
                } else if (r < 3) {
                    v = -(ga[r] * R.wq[b] * vol);  // -B_r(i,j)
                } else if (cc < 3) {
                    v = -(gb[cc] * R.wq[a] * vol);  // -B_cc(j,i) (negated pressure row)
                } else {
                    v = -(alpha * (G->hh * vol * gg) + eps * (vol * R.mref[a][b]));
                }
                buf[lo * 16 + e] += v;
            }
            __syncwarp();
        }
        const bool bi = bnd[i] != 0;
        for (int e = lane; e < ncol * 16; e += 32) {
            const int slot = e >> 4, rc = e & 15, r = rc >> 2, cc = rc & 3;
            const int32_t j = cols[c0 + slot];
            double v = buf[e];
            if (bi && r < 3) v = (j == i && r == cc) ? 1.0 : 0.0;
            else if (cc < 3 && bnd[j]) v = 0.0;
            A[(int64_t)(c0 + slot) * 16 + rc] = v;
        }
        __syncwarp();
    }
}

void launch_assemble(Ctx& c) {
    if (!c.A64) c.A64 = dev_alloc<double>(c, (size_t)c.nnzb * 16);
    int max_row = c.topo.max_row;
    size_t per_warp = (size_t)max_row * 16 * sizeof(double);
    int wpb = 8;
    while (wpb > 1 && per_warp * wpb > 160 * 1024) wpb >>= 1;
    size_t shmem = per_warp * wpb;
    FTS_CUDA(cudaFuncSetAttribute(k_assemble, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)shmem));
    int64_t blocks = (c.np + wpb - 1) / wpb;
    int64_t cap = (int64_t)c.num_sms * 16;
    int grid = (int)(blocks < cap ? blocks : cap);
    k_assemble<<<grid, wpb * 32, shmem, c.stream>>>(c.np, c.rowptr, c.cols, c.p2t_ptr, c.p2t,
                                                    c.tets, c.geom, c.mu, c.bnd, c.par.alpha,
                                                    c.par.eps, ref_args(), max_row, c.A64);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
    c.a64_valid = true;
}

void ensure_bsr64(Ctx& c) {
    if (c.a64_valid || c.matfree) return;
    if (c.p2) launch_assemble_p2(c);
    else launch_assemble(c);
}

// ---------------------------------------------------------------------------
// Lattice assembly (Kuhn lattices): one thread per (node v, stored direction
// d = 0..7) computes the 4x4 block (v, v + off[d]) by walking the elements of
// v and keeping those that also hold v + off[d] — the same terms, expressions
// and element order as k_assemble's row gather, so the block is bit-identical
// to the BSR's — with the same Dirichlet masking, and writes it to the FP64
// half stencil (lat64_idx) and the FP32 one (lat_idx of the Krylov kernels).
// The row gather's warp per row is latency bound on the element walk (66 ms at
// 129^3); here each thread walks one node's elements with no search and no
// shared-memory staging.
// ---------------------------------------------------------------------------
template <bool KUHN>
__global__ void __launch_bounds__(kThreads)
k_assemble_lat(int n, const int32_t* __restrict__ p2t_ptr, const uint32_t* __restrict__ p2t,
               const int32_t* __restrict__ tets, const ElemGeom* __restrict__ geom,
               const double* __restrict__ mu, const uint8_t* __restrict__ bnd, double alpha,
               double eps, RefArgs R, double2* __restrict__ L64, float4* __restrict__ L32) {
    const int64_t N = (int64_t)n * n * n;
    // direction-major: a warp's threads share d, so they walk alike (the self
    // block keeps all of a node's elements, the others about a quarter)
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < N * 8;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int d = (int)(t / N);
        const int64_t v = t - d * N;
        const int i = (int)(v % n), j = (int)((v / n) % n), k = (int)(v / ((int64_t)n * n));
        const int w = nbr(i, j, k, d, n);
        double blk[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) blk[e] = 0.0;
        if (w >= 0) {
            // the elements holding v and w, in the node-element map's order
            auto add = [&](int64_t el, int a, int b) {
                const ElemGeom* G = geom + el;
                const double ga[3] = {G->g[a][0], G->g[a][1], G->g[a][2]};
                const double gb[3] = {G->g[b][0], G->g[b][1], G->g[b][2]};
                const double vol = G->vol;
                const double gg = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
                const double mv = mu[el] * vol;
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int cc = 0; cc < 3; ++cc)
                        blk[4 * r + cc] += mv * ((r == cc ? gg : 0.0) + ga[cc] * gb[r]);
#pragma unroll
                for (int r = 0; r < 3; ++r) blk[4 * r + 3] += -(ga[r] * R.wq[b] * vol);
#pragma unroll
                for (int cc = 0; cc < 3; ++cc) blk[12 + cc] += -(gb[cc] * R.wq[a] * vol);
                blk[15] += -(alpha * (G->hh * vol * gg) + eps * (vol * R.mref[a][b]));
            };
            if (KUHN) {  // generator's element order: the elements follow from the lattice
                kuhn_pair_elements(n, i, j, k, d, add);
            } else {
                for (int32_t q = p2t_ptr[v]; q < p2t_ptr[v + 1]; ++q) {
                    const uint32_t pk = p2t[q];
                    const int64_t el = pk >> 2;
                    const int4 tt = reinterpret_cast<const int4*>(tets)[el];
                    const int b =
                        tt.x == w ? 0 : (tt.y == w ? 1 : (tt.z == w ? 2 : (tt.w == w ? 3 : -1)));
                    if (b >= 0) add(el, (int)(pk & 3), b);
                }
            }
            const bool bi = bnd[v] != 0, bw = bnd[w] != 0;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int r = e >> 2, cc = e & 3;
                if (bi && r < 3) blk[e] = (d == 0 && r == cc) ? 1.0 : 0.0;
                else if (cc < 3 && bw) blk[e] = 0.0;
            }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            L64[lat64_idx(d, r, 0, v)] = make_double2(blk[4 * r], blk[4 * r + 1]);
            L64[lat64_idx(d, r, 1, v)] = make_double2(blk[4 * r + 2], blk[4 * r + 3]);
            if (L32)  // NULL: the FP64 solve keeps no FP32 copy
                L32[((v >> 5) * 32 + d * 4 + r) * 32 + (v & 31)] =
                    make_float4((float)blk[4 * r], (float)blk[4 * r + 1], (float)blk[4 * r + 2],
                                (float)blk[4 * r + 3]);
        }
    }
}

void launch_assemble_lat(Ctx& c) {
    const int n = c.topo.lattice_n;
    const bool mixed = c.par.precision == FTS_PREC_MIXED;
    if (n <= 0 || (mixed && !c.lat_val))
        throw CudaError(cudaErrorInvalidValue, "lattice assembly without a lattice operator",
                        __FILE__, __LINE__);
    float4* L32 = mixed ? reinterpret_cast<float4*>(c.lat_val) : nullptr;
    const int64_t tiles = (c.np + 31) / 32;
    if (!c.lat64) {
        c.lat64 = dev_alloc<double2>(c, (size_t)tiles * 64 * 32);
        // tile padding past the last node stays zero
        FTS_CUDA(cudaMemsetAsync(c.lat64, 0, (size_t)tiles * 64 * 32 * sizeof(double2),
                                 c.stream));
    }
    if (c.topo.kuhn_elements)
        k_assemble_lat<true><<<grid_for(c, c.np * 8), kThreads, 0, c.stream>>>(
            n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.bnd, c.par.alpha, c.par.eps, ref_args(),
            c.lat64, L32);
    else
        k_assemble_lat<false><<<grid_for(c, c.np * 8), kThreads, 0, c.stream>>>(
            n, c.p2t_ptr, c.p2t, c.tets, c.geom, c.mu, c.bnd, c.par.alpha, c.par.eps, ref_args(),
            c.lat64, L32);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
    c.a64_valid = false;
}

// ---------------------------------------------------------------------------
// Block-diagonal SPD preconditioner: inverse of the node's 3x3 velocity block
// (identity on Dirichlet nodes) and, for pressure, the inverse of
// (alpha D + eps M)_ii + s sum_{e ni i} vol_e / (4 mu_e) (lumped 1/mu-weighted
// mass, a Schur-complement estimate; s = schur_scale).  pc[8 i + 0..5] = xx xy xz yy yz zz,
// pc[8 i + 6] = pressure weight.
// ---------------------------------------------------------------------------
// Diagonal block (i, i) of the BSR and of the FP64 lattice half stencil.
struct BsrDiag {
    const double* A;
    const int32_t* diag;
    __device__ __forceinline__ void load(int64_t i, double D[16]) const {
        const double* p = A + (int64_t)diag[i] * 16;
#pragma unroll
        for (int e = 0; e < 16; ++e) D[e] = p[e];
    }
};
struct LatDiag {
    const double2* L;
    __device__ __forceinline__ void load(int64_t i, double D[16]) const {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const double2 u = L[lat64_idx(0, r, 0, i)], w = L[lat64_idx(0, r, 1, i)];
            D[4 * r] = u.x;
            D[4 * r + 1] = u.y;
            D[4 * r + 2] = w.x;
            D[4 * r + 3] = w.y;
        }
    }
};

template <typename Diag>
__global__ void k_preconditioner(int64_t np, Diag dg, const int32_t* __restrict__ p2t_ptr,
                                 const uint32_t* __restrict__ p2t,
                                 const ElemGeom* __restrict__ geom, const double* __restrict__ mu,
                                 const OuterScalars* __restrict__ os,
                                 const uint8_t* __restrict__ bnd, double* __restrict__ pc) {
    const double ws = schur_scale(os);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        double D[16];
        dg.load(i, D);
        double o[8];
        if (bnd[i]) {
            o[0] = 1.0; o[1] = 0.0; o[2] = 0.0; o[3] = 1.0; o[4] = 0.0; o[5] = 1.0;
        } else {
            double a00 = D[0], a01 = 0.5 * (D[1] + D[4]), a02 = 0.5 * (D[2] + D[8]);
            double a11 = D[5], a12 = 0.5 * (D[6] + D[9]), a22 = D[10];
            double c00 = a11 * a22 - a12 * a12;
            double c01 = a02 * a12 - a01 * a22;
            double c02 = a01 * a12 - a02 * a11;
            double c11 = a00 * a22 - a02 * a02;
            double c12 = a01 * a02 - a00 * a12;
            double c22 = a00 * a11 - a01 * a01;
            double det = a00 * c00 + a01 * c01 + a02 * c02;
            double id = 1.0 / det;
            o[0] = c00 * id; o[1] = c01 * id; o[2] = c02 * id;
            o[3] = c11 * id; o[4] = c12 * id; o[5] = c22 * id;
        }
        const double w = ws * lumped_inv_mu(i, p2t_ptr, p2t, geom, mu);
        // a node without pressure (P2 edge node: zero pressure row) gets weight 0
        const double dp = -D[15] + w;
        o[6] = dp != 0.0 ? 1.0 / dp : 0.0;
        o[7] = 0.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) pc[8 * i + u] = o[u];
    }
}

// With both V-cycles (velocity and pressure multigrid) the node weights are
// never read, so they are not formed.
static bool pc_unused(const Ctx& c) { return c.use_mg && c.use_pmg; }

void launch_preconditioner(Ctx& c) {
    if (pc_unused(c)) return;
    if (c.use_lat64)
        k_preconditioner<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
            c.np, LatDiag{c.lat64}, c.p2t_ptr, c.p2t, c.geom, c.mu, c.os, c.bnd, c.pc64);
    else
        k_preconditioner<<<grid_for(c, c.np), kThreads, 0, c.stream>>>(
            c.np, BsrDiag{c.A64, c.diag}, c.p2t_ptr, c.p2t, c.geom, c.mu, c.os, c.bnd, c.pc64);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

// FP32 copies of the operator and preconditioner for the mixed-precision inner solve.
__global__ void k_to_f32(int64_t n, const double* __restrict__ in, float* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n / 2;
         i += (int64_t)gridDim.x * blockDim.x) {
        double2 v = reinterpret_cast<const double2*>(in)[i];
        reinterpret_cast<float2*>(out)[i] = make_float2((float)v.x, (float)v.y);
    }
}

// FP64 BSR -> FP32 sliced ELL: one warp per slice of 8 block rows; lane l
// handles row 8s + l/4, block row r = l%4, so every k writes 512 contiguous bytes.
__global__ void k_to_ell(int64_t np, int64_t nslices, const int32_t* __restrict__ rowptr,
                         const double* __restrict__ A, const int32_t* __restrict__ ell_ptr,
                         float* __restrict__ ell_val) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t s = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; s < nslices;
         s += warps) {
        const int32_t p0 = ell_ptr[s];
        const int32_t kmax = (ell_ptr[s + 1] - p0) >> 3;
        const int64_t row = 8 * s + (lane >> 2);
        const int r = lane & 3;
        const int32_t b0 = row < np ? rowptr[row] : 0;
        const int32_t len = row < np ? rowptr[row + 1] - b0 : 0;
        for (int32_t k = 0; k < kmax; ++k) {
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
            if (k < len) {
                const double* a = A + (int64_t)(b0 + k) * 16 + r * 4;
                const double2 a01 = *reinterpret_cast<const double2*>(a);
                const double2 a23 = *reinterpret_cast<const double2*>(a + 2);
                o = make_float4((float)a01.x, (float)a01.y, (float)a23.x, (float)a23.y);
            }
            reinterpret_cast<float4*>(ell_val)[((int64_t)p0 + 8 * k + (lane >> 2)) * 4 + r] = o;
        }
    }
}

// FP64 BSR -> FP32 lattice half stencil.  Thread t handles node v = 32 tile +
// (t % 32) and direction d = (t / 32) % 8; row r of the block goes to float4
// ((tile * 32 + 4 d + r) * 32 + v % 32), so a warp's store is 512 contiguous bytes.
__global__ void k_to_lat(int64_t tiles, const int32_t* __restrict__ src,
                         const double* __restrict__ A, float4* __restrict__ L) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tiles * 256;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t tile = t >> 8;
        const int d = (int)((t >> 5) & 7);
        const int lane = (int)(t & 31);
        const int32_t b = src[(tile * 32 + lane) * 8 + d];
        float4* out = L + (tile * 32 + 4 * d) * 32 + lane;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
            if (b >= 0) {
                const double2* a = reinterpret_cast<const double2*>(A + (int64_t)b * 16 + 4 * r);
                const double2 u = a[0], w = a[1];
                o = make_float4((float)u.x, (float)u.y, (float)w.x, (float)w.y);
            }
            out[r * 32] = o;
        }
    }
}

void launch_to_lat(Ctx& c) {
    if (!c.lat_val || !c.lat_src || !c.A64)
        throw CudaError(cudaErrorInvalidValue, "lattice copy without its map or the BSR",
                        __FILE__, __LINE__);
    const int64_t tiles = (c.np + 31) / 32;
    k_to_lat<<<grid_for(c, tiles * 256), kThreads, 0, c.stream>>>(
        tiles, c.lat_src, c.A64, reinterpret_cast<float4*>(c.lat_val));
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

void launch_to_f32(Ctx& c) {
    if ((c.use_lat && !c.lat_val) || (c.use_ell && !c.ell_val) ||
        (!c.use_lat && !c.use_ell && !c.A32) || !c.pc32)
        throw CudaError(cudaErrorInvalidValue, "FP32 operator copy used before allocation",
                        __FILE__, __LINE__);
    if (c.use_lat64) {
        // lat_val was written by the lattice assembly
        if (pc_unused(c)) return;
        k_to_f32<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(c.np * 8, c.pc64, c.pc32);
        FTS_CUDA(cudaGetLastError());
        c.launches += 1;
        return;
    }
    if (c.use_lat) {
        const int64_t tiles = (c.np + 31) / 32;
        k_to_lat<<<grid_for(c, tiles * 256), kThreads, 0, c.stream>>>(
            tiles, c.lat_src, c.A64, reinterpret_cast<float4*>(c.lat_val));
    } else if (c.use_ell)
        k_to_ell<<<grid_for(c, c.nslices * 32), kThreads, 0, c.stream>>>(
            c.np, c.nslices, c.rowptr, c.A64, c.ell_ptr, c.ell_val);
    else
        k_to_f32<<<grid_for(c, c.nnzb * 8), kThreads, 0, c.stream>>>(c.nnzb * 16, c.A64, c.A32);
    c.launches += 1;
    if (!pc_unused(c)) {
        k_to_f32<<<grid_for(c, c.np * 4), kThreads, 0, c.stream>>>(c.np * 8, c.pc64, c.pc32);
        c.launches += 1;
    }
    FTS_CUDA(cudaGetLastError());
}

// flow = [ux(np), uy(np), uz(np), p(np)], zero velocity on boundary nodes
// (Flow.cpp:290-300).
__global__ void k_scatter_flow(int64_t np, const V4<double>* __restrict__ x,
                               const uint8_t* __restrict__ bnd, double* __restrict__ flow) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np;
         i += (int64_t)gridDim.x * blockDim.x) {
        V4<double> v = x[i];
        bool d = bnd[i] != 0;
        flow[i] = d ? 0.0 : v.x;
        flow[np + i] = d ? 0.0 : v.y;
        flow[2 * np + i] = d ? 0.0 : v.z;
        flow[3 * np + i] = v.w;
    }
}

void launch_scatter_flow(Ctx& c, double* flow_out) {
    // the vertices are the first nv system nodes (P2: the edges follow)
    k_scatter_flow<<<grid_for(c, c.nv), kThreads, 0, c.stream>>>(c.nv, c.x, c.bnd, flow_out);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

__global__ void k_check_finite(int64_t n, const double* __restrict__ a, int* flag) {
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        bad = bad || !isfinite(a[i]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void k_any_abs_above(int64_t n, const double* __restrict__ a, double thr, int* flag) {
    bool hit = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        hit = hit || fabs(a[i]) > thr;
    if (__any_sync(0xffffffffu, hit) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

void launch_any_abs_above(Ctx& c, const double* a, int64_t n, double thr) {
    k_any_abs_above<<<grid_for(c, n), kThreads, 0, c.stream>>>(n, a, thr, c.err_flag);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

void launch_check_finite(Ctx& c, const double* a, int64_t n) {
    k_check_finite<<<grid_for(c, n), kThreads, 0, c.stream>>>(n, a, c.err_flag);
    FTS_CUDA(cudaGetLastError());
    c.launches += 1;
}

}  // namespace fts
