// ORACLE — test infrastructure only.
//
// A CPU restatement (C++/OpenMP, FP64, no Eigen) of fluidtissue's per-time-step
// P1-P1 Brezzi-Pitkaranta-stabilised Stokes solve, used as the parity checker
// and as the timed CPU baseline.  Only tests, the smoke check and the benchmark's
// CPU-baseline / reference arm may load it; the product path never does.
//
// Parity unpinned: the reference needs Eigen, CGAL, TBB and GMP, none of which
// exists on this machine, so it cannot be built and has no tests or golden
// vectors of its own.  This file restates its algorithm line by line (citations
// below, paths relative to the reference project) and is pinned instead by
// known-answer identities (mass = volume, K*const = 0, row sums of D = 0, ...)
// and by a direct sparse solve of the same system in the tests.
//
// Restated reference pieces:
//  * float-rounded P1 shape-function table at the 4-point degree-2 rule
//      src/fem/Quadrature.hpp:24-36, :102-112; src/fem/Tetrahedron.hpp:17-18, :27-51
//  * element geometry (detB = |det B|, invB^T)        src/fem/Assembler.hpp:430-462
//  * node-row gather assembly, row = test, col = trial src/fem/Assembler.hpp:134-229
//      h = (float)cbrt(detB) :193, integral = feval.dot(qw/6)*detB :143, :218
//  * weak forms and block composition                  src/growth/Flow.cpp:54-72, :135-203
//  * restriction to interior velocity + all pressure   src/growth/Flow.cpp:35-44, :206;
//                                                      src/fem/MathTypes.hpp:52-94
//  * interior dofs = nodes not on boundary triangles   src/fem/TetraMesh.cpp:266-269
//  * source, zero mean, RHS                            src/growth/Flow.cpp:365-399
//  * viscosity profiles                                src/growth/ViscosityProfiles.hpp:27-72
//  * interior nodes / elements (strict phi < 0)        src/fem/LevelSet.cpp:180-211
//  * un-preconditioned BiCGSTAB with ||r||/||b|| stop  src/growth/Flow.hpp:62, Flow.cpp:77-82, :266-285
//      (Eigen's BiCGSTAB, external and not vendored; restated from van der Vorst 1992)
//  * scatter to [ux(np), uy(np), uz(np), p(np)]        src/growth/Flow.cpp:290-300
//  * reaction-diffusion: interior submesh, lumped-mass  src/growth/RD.cpp:27-108, :116-172;
//    Laplacian, explicit Euler                         src/fem/Assembler.cpp:75-84
//  * distance reset of the level set (host path)       src/fem/EuclideanDistance.cu:16-38, :92-117
//  * level-set update: Crank-Nicolson advection,        src/fem/LevelSet.cpp:89-151, :261-300,
//    Jacobi-BiCGSTAB, distance reset and mixing          :429-455; Assembler.hpp:179-190
//  * P2-P1 (velocity degree 2): element integrals by     src/fem/Assembler.hpp:321-424,
//    quadrature at the rule of degree deg_i + deg_j     src/fem/Quadrature.hpp:24-56,
//    P2 / P1 basis tables float-rounded                 src/fem/Tetrahedron.hpp:56-115,
//    DOFs vertices then edges, boundary edges           src/fem/TetraMesh.cpp:219-290,
//    block system without the BP term                   src/growth/Flow.cpp:102-214, :345-399
//  * surface-tension load: element / nodal gradients     src/growth/Flow.cpp:307-341;
//    (Assembler.cpp:11-69), curvature, interface points  src/fem/LevelSet.cpp:215-253,
//    and interface-patch areas                           :261-300, :326-420, :453
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Reference element tables
// ---------------------------------------------------------------------------

// phi[a][q]: P1 basis a at quadrature point q, evaluated the way the reference
// does: the points are double, passed through std::function<float(float,float,
// float)>, so the arguments and the result are float while the expression
// 1.0 - x - y - z runs in double (Tetrahedron.hpp:27-31, Quadrature.hpp:108-112).
struct RefTables {
    double phi[4][4];
    double qw;  // 0.25 / 6.0 (Assembler.hpp:143)
    RefTables() {
        double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0;
        double b = (5.0 - std::sqrt(5.0)) / 20.0;
        double qp[3][4] = {{a, b, b, b}, {b, a, b, b}, {b, b, a, b}};
        for (int q = 0; q < 4; ++q) {
            float x = (float)qp[0][q], y = (float)qp[1][q], z = (float)qp[2][q];
            phi[0][q] = (double)(float)(1.0 - x - y - z);
            phi[1][q] = (double)x;
            phi[2][q] = (double)y;
            phi[3][q] = (double)z;
        }
        qw = 0.25 / 6.0;
    }
};
const RefTables& tables() {
    static RefTables t;
    return t;
}

// (f0 q + f1 q + f2 q + f3 q) * detB with a pairwise reduction of the
// 4-vector dot product.
inline double integ(const double f[4], double qw, double detB) {
    return ((f[0] * qw + f[2] * qw) + (f[1] * qw + f[3] * qw)) * detB;
}

// Element geometry (Assembler.hpp:430-462): B = [p2-p1, p3-p1, p4-p1] from the
// float coordinates cast to double, detB = |det B|, invB^T; g[j] = invB^T * ghat_j
// with ghat = (-1,-1,-1), e_x, e_y, e_z (Tetrahedron.hpp:33-50).
struct Geom {
    double detB;
    double g[4][3];
    float h;
};

inline bool element_geom(const float* xyz, const int32_t* t, Geom& G) {
    double p[4][3];
    for (int j = 0; j < 4; ++j)
        for (int a = 0; a < 3; ++a) p[j][a] = (double)xyz[3 * (int64_t)t[j] + a];
    double B[3][3];
    for (int a = 0; a < 3; ++a) {
        B[a][0] = p[1][a] - p[0][a];
        B[a][1] = p[2][a] - p[0][a];
        B[a][2] = p[3][a] - p[0][a];
    }
    double c00 = B[1][1] * B[2][2] - B[1][2] * B[2][1];
    double c01 = B[1][2] * B[2][0] - B[1][0] * B[2][2];
    double c02 = B[1][0] * B[2][1] - B[1][1] * B[2][0];
    double det = B[0][0] * c00 + B[0][1] * c01 + B[0][2] * c02;
    G.detB = std::fabs(det);
    if (G.detB == 0.0) return false;
    // inverse = adj(B)/det; (invB^T)(r,c) = inv(c,r) = cof(r,c)/det
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
    double it[3][3];  // invB^T
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) it[r][c] = cof[r][c] / det;
    for (int r = 0; r < 3; ++r) {
        G.g[0][r] = -it[r][0] - it[r][1] - it[r][2];
        G.g[1][r] = it[r][0];
        G.g[2][r] = it[r][1];
        G.g[3][r] = it[r][2];
    }
    G.h = (float)std::cbrt(G.detB);  // Assembler.hpp:193
    return true;
}

// Per node pair (i,j) quantities accumulated by the row gather for row i.
// K[al][be]: velocity block of the composed system (Flow.cpp:160-184):
//   K[0][0]=A11(i,j) K[0][1]=A12(i,j) K[0][2]=A13(i,j)
//   K[1][0]=A12(j,i) K[1][1]=A22(i,j) K[1][2]=A23(i,j)
//   K[2][0]=A13(j,i) K[2][1]=A23(j,i) K[2][2]=A33(i,j)
// Bv[al] = B_al(i,j) (velocity test i, pressure trial j), Bp[al] = B_al(j,i),
// M = M(i,j), D = D(i,j), C[al] = C_al(i,j) (2/3 mu weighted, Flow.cpp:383-390).
struct PairVals {
    double K[3][3];
    double Bv[3], Bp[3];
    double M, D;
    double C[3];
};

struct Topology {
    int64_t np = 0, nt = 0;
    std::vector<int64_t> p2t_ptr;  // np+1
    std::vector<int32_t> p2t;      // 4 nt, ascending tet index per node
    std::vector<int64_t> nb_ptr;   // np+1
    std::vector<int32_t> nb;       // sorted node neighbours incl. self
};

void build_topology(int64_t np, int64_t nt, const int32_t* tets, Topology& T) {
    T.np = np;
    T.nt = nt;
    T.p2t_ptr.assign(np + 1, 0);
    for (int64_t e = 0; e < 4 * nt; ++e) T.p2t_ptr[tets[e] + 1]++;
    for (int64_t i = 0; i < np; ++i) T.p2t_ptr[i + 1] += T.p2t_ptr[i];
    T.p2t.resize(4 * nt);
    std::vector<int64_t> fill(T.p2t_ptr.begin(), T.p2t_ptr.end() - 1);
    for (int64_t k = 0; k < nt; ++k)
        for (int j = 0; j < 4; ++j) T.p2t[fill[tets[4 * k + j]]++] = (int32_t)k;
    std::vector<int32_t> cnt(np);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < np; ++i) {
        int32_t buf[512];
        int n = 0;
        for (int64_t q = T.p2t_ptr[i]; q < T.p2t_ptr[i + 1] && n < 508; ++q)
            for (int j = 0; j < 4; ++j) buf[n++] = tets[4 * (int64_t)T.p2t[q] + j];
        std::sort(buf, buf + n);
        cnt[i] = (int32_t)(std::unique(buf, buf + n) - buf);
    }
    T.nb_ptr.assign(np + 1, 0);
    for (int64_t i = 0; i < np; ++i) T.nb_ptr[i + 1] = T.nb_ptr[i] + cnt[i];
    T.nb.resize(T.nb_ptr[np]);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < np; ++i) {
        int32_t buf[512];
        int n = 0;
        for (int64_t q = T.p2t_ptr[i]; q < T.p2t_ptr[i + 1] && n < 508; ++q)
            for (int j = 0; j < 4; ++j) buf[n++] = tets[4 * (int64_t)T.p2t[q] + j];
        std::sort(buf, buf + n);
        int u = (int)(std::unique(buf, buf + n) - buf);
        std::copy(buf, buf + u, T.nb.begin() + T.nb_ptr[i]);
    }
}

inline int find_col(const int32_t* cols, int n, int32_t c) {
    const int32_t* p = std::lower_bound(cols, cols + n, c);
    return (p != cols + n && *p == c) ? (int)(p - cols) : -1;
}

// Row gather of all pair quantities of row i (Assembler.hpp:150-225).
// mu: per element viscosity (data[k], Assembler.hpp:171-173).
bool gather_row(int64_t i, const Topology& T, const float* xyz, const int32_t* tets,
                const double* mu, std::vector<PairVals>& row) {
    const RefTables& R = tables();
    const double qw = R.qw;
    const int32_t* cols = T.nb.data() + T.nb_ptr[i];
    int ncol = (int)(T.nb_ptr[i + 1] - T.nb_ptr[i]);
    row.assign(ncol, PairVals());
    for (auto& pv : row) std::memset(&pv, 0, sizeof(PairVals));
    bool ok = true;
    for (int64_t q = T.p2t_ptr[i]; q < T.p2t_ptr[i + 1]; ++q) {
        int64_t k = T.p2t[q];
        const int32_t* t = tets + 4 * k;
        Geom G;
        if (!element_geom(xyz, t, G)) {
            ok = false;
            continue;
        }
        double Ve = mu ? mu[k] : 1.0;
        double Vc = 2.0 / 3 * Ve;  // 2.0/3*mu (Flow.cpp:386)
        float hh = G.h * G.h;       // (h*h) in float (Flow.cpp:195)
        int a = 0;
        if (t[1] == i) a = 1;
        else if (t[2] == i) a = 2;
        else if (t[3] == i) a = 3;
        const double* ga = G.g[a];
        const double* va = R.phi[a];
        for (int b = 0; b < 4; ++b) {
            int slot = find_col(cols, ncol, t[b]);
            PairVals& P = row[slot];
            const double* gb = G.g[b];
            const double* ub = R.phi[b];
            double f[4];
            // A11..A33 and the transposed off-diagonals (Flow.cpp:136-153)
            double kxx = ((2.0 * gb[0]) * ga[0] + gb[1] * ga[1] + gb[2] * ga[2]) * Ve;
            double kyy = (gb[0] * ga[0] + (2.0 * gb[1]) * ga[1] + gb[2] * ga[2]) * Ve;
            double kzz = (gb[0] * ga[0] + gb[1] * ga[1] + (2.0 * gb[2]) * ga[2]) * Ve;
            double kxy = (gb[0] * ga[1]) * Ve;  // A12(i,j): ux.*vy
            double kxz = (gb[0] * ga[2]) * Ve;  // A13(i,j)
            double kyz = (gb[1] * ga[2]) * Ve;  // A23(i,j)
            double kyx = (ga[0] * gb[1]) * Ve;  // A12(j,i)
            double kzx = (ga[0] * gb[2]) * Ve;  // A13(j,i)
            double kzy = (ga[1] * gb[2]) * Ve;  // A23(j,i)
            double kv[3][3] = {{kxx, kxy, kxz}, {kyx, kyy, kyz}, {kzx, kzy, kzz}};
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    for (int qq = 0; qq < 4; ++qq) f[qq] = kv[r][c];
                    P.K[r][c] += integ(f, qw, G.detB);
                }
            for (int al = 0; al < 3; ++al) {
                // B_al(i,j) = vx.*u : d_al phi_i * phi_j   (Flow.cpp:55-64)
                for (int qq = 0; qq < 4; ++qq) f[qq] = ga[al] * ub[qq];
                P.Bv[al] += integ(f, qw, G.detB);
                // B_al(j,i): test j, trial i
                for (int qq = 0; qq < 4; ++qq) f[qq] = gb[al] * va[qq];
                P.Bp[al] += integ(f, qw, G.detB);
                // C_al(i,j) = Ve * u.*v_al with Ve = 2/3 mu (Flow.cpp:385-390)
                for (int qq = 0; qq < 4; ++qq) f[qq] = Vc * (ub[qq] * ga[al]);
                P.C[al] += integ(f, qw, G.detB);
            }
            for (int qq = 0; qq < 4; ++qq) f[qq] = ub[qq] * va[qq];  // u.*v
            P.M += integ(f, qw, G.detB);
            double gg = gb[0] * ga[0] + gb[1] * ga[1] + gb[2] * ga[2];
            for (int qq = 0; qq < 4; ++qq) f[qq] = (double)hh * gg;  // (h*h)*(ux.*vx+...)
            P.D += integ(f, qw, G.detB);
        }
    }
    return ok;
}

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// CSR helpers
// ---------------------------------------------------------------------------
void spmv(int64_t n, const int64_t* rp, const int32_t* ci, const double* v, const double* x,
          double* y) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n; ++r) {
        double s = 0.0;
        for (int64_t q = rp[r]; q < rp[r + 1]; ++q) s += v[q] * x[ci[q]];
        y[r] = s;
    }
}

double dot(int64_t n, const double* a, const double* b) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

}  // namespace

extern "C" {

// Float-rounded basis table tab[a*4 + q] and the scaled weight (0.25/6).
void ora_ref_tables(double* tab, double* qw) {
    const RefTables& R = tables();
    for (int a = 0; a < 4; ++a)
        for (int q = 0; q < 4; ++q) tab[4 * a + q] = R.phi[a][q];
    if (qw) *qw = R.qw;
}

int ora_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void ora_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// Boundary nodes = nodes of triangles that belong to exactly one tetrahedron
// (the exterior boundary triangles; TetraMesh.cpp:266-269).
int ora_boundary_nodes(int64_t np, int64_t nt, const int32_t* tets, uint8_t* bnd) {
    for (int64_t e = 0; e < 4 * nt; ++e)
        if (tets[e] < 0 || tets[e] >= np) return 1;
    Topology T;
    build_topology(np, nt, tets, T);
    std::memset(bnd, 0, (size_t)np);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = tets + 4 * k;
        for (int f = 0; f < 4; ++f) {
            int32_t v[3], n = 0;
            for (int j = 0; j < 4; ++j)
                if (j != f) v[n++] = t[j];
            bool shared = false;
            for (int64_t q = T.p2t_ptr[v[0]]; q < T.p2t_ptr[v[0] + 1] && !shared; ++q) {
                int64_t k2 = T.p2t[q];
                if (k2 == k) continue;
                const int32_t* t2 = tets + 4 * k2;
                int hit = 0;
                for (int j = 0; j < 4; ++j) hit += (t2[j] == v[1]) + (t2[j] == v[2]);
                shared = (hit == 2);
            }
            if (!shared)
                for (int j = 0; j < 3; ++j) bnd[v[j]] = 1;  // benign race: all write 1
        }
    }
    return 0;
}

// setViscosity (ViscosityProfiles.hpp:27-72). profile: 0 INVERSE, 1 DIRECT,
// 2 DIRECT_RATE4X. mnmx (nullable) = {min, max} over interior elements, as the
// reference prints (FLT_MAX, FLT_MIN when there is none).
int ora_set_viscosity(int64_t np, int64_t nt, const int32_t* tets, const double* phi,
                      const double* gf, double mu_int, double mu_ext, int profile,
                      double rd_iterations, double gf_production, double* mu, double* mnmx) {
    (void)np;
    double mu_h = mu_int, mu_l = mu_ext;
    double maxGF = rd_iterations > 0.0 ? gf_production : 1.0;
    double mn = FLT_MAX, mx = FLT_MIN;
    for (int64_t k = 0; k < nt; ++k) {
        mu[k] = mu_l;
        const int32_t* t = tets + 4 * k;
        if (!(phi[t[0]] < 0.0 && phi[t[1]] < 0.0 && phi[t[2]] < 0.0 && phi[t[3]] < 0.0))
            continue;
        double c3 = std::max(std::max(gf[t[0]], gf[t[1]]), std::max(gf[t[2]], gf[t[3]]));
        if (profile == 0) mu[k] = mu_l * (c3 / maxGF) + mu_h * (1.0 - c3 / maxGF);
        if (profile == 1) mu[k] = mu_h * (c3 / maxGF) + mu_l * (1.0 - c3 / maxGF);
        if (profile == 2) {
            c3 *= 4.0;
            if (c3 > maxGF) c3 = maxGF;
            mu[k] = mu_h * (c3 / maxGF) + mu_l * (1.0 - c3 / maxGF);
        }
        mn = std::min(mn, mu[k]);
        mx = std::max(mx, mu[k]);
    }
    if (mnmx) {
        mnmx[0] = mn;
        mnmx[1] = mx;
    }
    return 0;
}

// Nodal mass source (Flow.cpp:365-376): s_i = (c_i - sink) * growth on interior
// nodes (phi < 0) with c_i > threshold, then s -= mean(s) over all nodes.
int ora_source(int64_t np, const double* phi, const double* c, double gf_growth,
               double level_sink, double growth_threshold, double* s) {
    double sum = 0.0;
    for (int64_t i = 0; i < np; ++i) {
        s[i] = 0.0;
        if (phi[i] < 0.0 && c[i] > growth_threshold) s[i] = (c[i] - level_sink) * gf_growth;
        sum += s[i];
    }
    double mean = sum / (double)np;
    for (int64_t i = 0; i < np; ++i) s[i] -= mean;
    return 0;
}

// Block pattern of the node graph: rowptr[np+1], cols[nnzb] (sorted, incl. self).
int ora_block_pattern_size(int64_t np, int64_t nt, const int32_t* tets, int64_t* nnzb) {
    Topology T;
    build_topology(np, nt, tets, T);
    *nnzb = T.nb_ptr[np];
    return 0;
}

// Node-pair blocks of the full (un-restricted) system in the reference's sign
// convention (Flow.cpp:160-203), 16 doubles per block, row-major over
// (ux, uy, uz, p) x (ux, uy, uz, p):
//   [ K            -B_al(i,j) ]
//   [ B_be(j,i)   alpha D(i,j) + eps M(i,j) ]
// plus the per-node right-hand side rhs[4*i + (0..2)] = (N f)_al(i) + (C_al s)(i),
// rhs[4*i + 3] = (M s)(i)  (Flow.cpp:392-396).  fst (nullable) = [fx, fy, fz]
// each of length np.  Returns 2 on a degenerate element.
int ora_assemble_blocks(int64_t np, int64_t nt, const float* xyz, const int32_t* tets,
                        const double* mu, const double* s, const double* fst, double alpha,
                        double eps, int64_t* rowptr, int32_t* cols, double* vals,
                        double* rhs) {
    Topology T;
    build_topology(np, nt, tets, T);
    for (int64_t i = 0; i <= np; ++i) rowptr[i] = T.nb_ptr[i];
    std::copy(T.nb.begin(), T.nb.end(), cols);
    int bad = 0;
#pragma omp parallel
    {
        std::vector<PairVals> row;
#pragma omp for schedule(dynamic, 256) reduction(| : bad)
        for (int64_t i = 0; i < np; ++i) {
            if (!gather_row(i, T, xyz, tets, mu, row)) bad |= 1;
            double F[4] = {0, 0, 0, 0};
            int64_t base = T.nb_ptr[i];
            for (size_t c = 0; c < row.size(); ++c) {
                const PairVals& P = row[c];
                double* b = vals + 16 * (base + (int64_t)c);
                for (int r = 0; r < 3; ++r) {
                    for (int cc = 0; cc < 3; ++cc) b[4 * r + cc] = P.K[r][cc];
                    b[4 * r + 3] = -P.Bv[r];
                    b[12 + r] = P.Bp[r];
                }
                b[15] = alpha * P.D + eps * P.M;
                int32_t j = T.nb[base + (int64_t)c];
                for (int al = 0; al < 3; ++al) {
                    double fj = fst ? fst[al * np + j] : 0.0;
                    F[al] += P.M * fj;  // N = M for P1 (Flow.cpp:70-72)
                }
                for (int al = 0; al < 3; ++al) F[al] += P.C[al] * s[j];
                F[3] += P.M * s[j];
            }
            for (int q = 0; q < 4; ++q) rhs[4 * i + q] = F[q];
        }
    }
    return bad ? 2 : 0;
}

// Size of the reduced system (Flow.cpp:35-44, :206): N = 3 nI + np.
int ora_reduced_size(int64_t np, const int64_t* rowptr, const int32_t* cols, const uint8_t* bnd,
                     int64_t* N, int64_t* nnz) {
    int64_t nI = 0;
    for (int64_t i = 0; i < np; ++i) nI += bnd[i] ? 0 : 1;
    int64_t z = 0;
    for (int64_t i = 0; i < np; ++i) {
        int64_t nint = 0, nall = rowptr[i + 1] - rowptr[i];
        for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q) nint += bnd[cols[q]] ? 0 : 1;
        int64_t rowlen = 3 * nint + nall;
        z += rowlen * (bnd[i] ? 1 : 4);
    }
    *N = 3 * nI + np;
    *nnz = z;
    return 0;
}

// Restriction subSparse(A_, sIdx_, sIdx_) / subDense(F, sIdx_) of the block
// system to the reference's reduced ordering [ux(I), uy(I), uz(I), p(0..np-1)].
// sidx[N] receives the full-system index 4-layout-free form of sIdx_:
// velocity a of node i -> a*np + i, pressure of node i -> 3*np + i.
int ora_reduce(int64_t np, const int64_t* rowptr, const int32_t* cols, const double* vals,
               const double* rhs, const uint8_t* bnd, int64_t* rrp, int32_t* rci, double* rv,
               double* rF, int32_t* sidx) {
    std::vector<int64_t> red(np, -1);
    int64_t nI = 0;
    for (int64_t i = 0; i < np; ++i)
        if (!bnd[i]) red[i] = nI++;
    // row order: ux(I), uy(I), uz(I), p(all)
    int64_t N = 3 * nI + np;
    std::vector<int64_t> rowlen(N);
    std::vector<int64_t> rownode(N);
    std::vector<int> rowcomp(N);
    for (int64_t i = 0; i < np; ++i) {
        if (red[i] >= 0)
            for (int a = 0; a < 3; ++a) {
                rownode[a * nI + red[i]] = i;
                rowcomp[a * nI + red[i]] = a;
            }
        rownode[3 * nI + i] = i;
        rowcomp[3 * nI + i] = 3;
    }
    for (int64_t r = 0; r < N; ++r) {
        int64_t i = rownode[r];
        int64_t nint = 0, nall = rowptr[i + 1] - rowptr[i];
        for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q) nint += bnd[cols[q]] ? 0 : 1;
        rowlen[r] = 3 * nint + nall;
    }
    rrp[0] = 0;
    for (int64_t r = 0; r < N; ++r) rrp[r + 1] = rrp[r] + rowlen[r];
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < N; ++r) {
        int64_t i = rownode[r];
        int rc = rowcomp[r];
        int64_t o = rrp[r];
        for (int cc = 0; cc < 3; ++cc)
            for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q) {
                int32_t j = cols[q];
                if (red[j] < 0) continue;
                rci[o] = (int32_t)(cc * nI + red[j]);
                rv[o++] = vals[16 * q + 4 * rc + cc];
            }
        for (int64_t q = rowptr[i]; q < rowptr[i + 1]; ++q) {
            rci[o] = (int32_t)(3 * nI + cols[q]);
            rv[o++] = vals[16 * q + 4 * rc + 3];
        }
        rF[r] = rhs[4 * i + rc];
        sidx[r] = (int32_t)(rc * np + i);
    }
    return 0;
}

int ora_spmv(int64_t N, const int64_t* rp, const int32_t* ci, const double* v, const double* x,
             double* y) {
    spmv(N, rp, ci, v, x, y);
    return 0;
}

// Un-preconditioned BiCGSTAB (van der Vorst 1992) as the reference configures
// Eigen's (Flow.hpp:62): stop when the updated residual satisfies
// ||r|| <= tol ||b||, at most maxit iterations (<= 0: 2N, Eigen's default),
// warm start from x; when rho collapses relative to ||r0||^2 the shadow
// residual is reset to the current residual.  Returns 0 on convergence, 1 on
// no convergence.  iters / err receive the iteration count and ||r||/||b||
// (the solver's own error() estimate).
int ora_bicgstab(int64_t N, const int64_t* rp, const int32_t* ci, const double* v, const double* b,
                 double* x, double tol, int64_t maxit, int64_t* iters, double* err) {
    std::vector<double> r(N), r0(N), p(N, 0.0), vv(N, 0.0), s(N), t(N);
    if (maxit <= 0) maxit = 2 * N;
    spmv(N, rp, ci, v, x, r.data());
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < N; ++q) r[q] = b[q] - r[q];
    double bb = dot(N, b, b);
    if (bb == 0.0) {
        std::fill(x, x + N, 0.0);
        if (iters) *iters = 0;
        if (err) *err = 0.0;
        return 0;
    }
    r0 = r;
    double r0n = dot(N, r.data(), r.data());
    double rr = r0n;
    double tol2 = tol * tol * bb;
    const double eps2 = DBL_EPSILON * DBL_EPSILON;
    double rho = 1.0, alpha = 1.0, w = 1.0;
    int64_t it = 0;
    int restarts = 0;
    while (rr > tol2 && it < maxit) {
        double rho_old = rho;
        rho = dot(N, r0.data(), r.data());
        if (std::fabs(rho) < eps2 * r0n) {
            // restart with the true residual as the new shadow vector
            spmv(N, rp, ci, v, x, r.data());
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) r[q] = b[q] - r[q];
            r0 = r;
            rho = r0n = dot(N, r.data(), r.data());
            if (restarts++ == 0) it = 0;
        }
        double beta = (rho / rho_old) * (alpha / w);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) p[q] = r[q] + beta * (p[q] - w * vv[q]);
        spmv(N, rp, ci, v, p.data(), vv.data());
        alpha = rho / dot(N, r0.data(), vv.data());
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) s[q] = r[q] - alpha * vv[q];
        spmv(N, rp, ci, v, s.data(), t.data());
        double tt = dot(N, t.data(), t.data());
        w = tt > 0.0 ? dot(N, t.data(), s.data()) / tt : 0.0;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            x[q] += alpha * p[q] + w * s[q];
            r[q] = s[q] - w * t[q];
        }
        rr = dot(N, r.data(), r.data());
        ++it;
    }
    if (iters) *iters = it;
    double e = std::sqrt(rr / bb);
    if (err) *err = e;
    return e <= tol ? 0 : 1;
}

// True relative residual ||b - A x|| / ||b|| with long-double accumulation.
double ora_true_residual(int64_t N, const int64_t* rp, const int32_t* ci, const double* v,
                         const double* b, const double* x) {
    long double rr = 0.0L, bb = 0.0L;
#pragma omp parallel for reduction(+ : rr, bb) schedule(static)
    for (int64_t r = 0; r < N; ++r) {
        long double s = 0.0L;
        for (int64_t q = rp[r]; q < rp[r + 1]; ++q) s += (long double)v[q] * x[ci[q]];
        long double d = (long double)b[r] - s;
        rr += d * d;
        bb += (long double)b[r] * b[r];
    }
    return bb > 0.0L ? (double)std::sqrt(rr / bb) : 0.0;
}

// Tight solve used to produce parity targets: MINRES (Paige & Saunders 1975)
// on the symmetric form J A x = J b of the reduced system, J = diag(+1 on the
// 3 nI velocity rows, -1 on the np pressure rows), preconditioned by the SPD
// diagonal minv[N] (inverse weights).  Restarted from the current iterate on the
// true residual until ||b - A x|| / ||b|| <= tol (long-double residual) or
// max_restarts.  Returns the true relative residual.
double ora_minres_tight(int64_t N, int64_t nI, const int64_t* rp, const int32_t* ci,
                        const double* v, const double* b, const double* minv, double* x,
                        double tol, int64_t maxit, int max_restarts, int64_t* iters_out) {
    std::vector<double> r1(N), r2(N), y(N), vv(N), w(N), w1(N), w2(N), jb(N);
    auto apply = [&](const double* in, double* out) {
        spmv(N, rp, ci, v, in, out);
#pragma omp parallel for schedule(static)
        for (int64_t q = 3 * nI; q < N; ++q) out[q] = -out[q];
    };
    for (int64_t q = 0; q < N; ++q) jb[q] = q < 3 * nI ? b[q] : -b[q];
    double bn = std::sqrt(dot(N, b, b));
    double tr = ora_true_residual(N, rp, ci, v, b, x);
    double inner_tol = tol;
    int64_t total = 0;
    for (int rs = 0; rs <= max_restarts && tr > tol && total < maxit; ++rs) {
        apply(x, r1.data());
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            r1[q] = jb[q] - r1[q];
            y[q] = minv[q] * r1[q];
        }
        r2 = r1;
        double beta1 = std::sqrt(dot(N, r1.data(), y.data()));
        if (!(beta1 > 0.0)) break;
        double rn0 = std::sqrt(dot(N, r1.data(), r1.data()));
        // the preconditioned target that corresponds to tol in the 2-norm,
        // adapted from the previous sweep's observed ratio
        double target = inner_tol * bn / rn0;
        double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1;
        double cs = -1.0, sn = 0.0;
        std::fill(w.begin(), w.end(), 0.0);
        std::fill(w2.begin(), w2.end(), 0.0);
        for (int64_t it = 1; total < maxit; ++it) {
            ++total;
            double s = 1.0 / beta;
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) vv[q] = s * y[q];
            apply(vv.data(), y.data());
            if (it >= 2) {
                double f = beta / oldb;
#pragma omp parallel for schedule(static)
                for (int64_t q = 0; q < N; ++q) y[q] -= f * r1[q];
            }
            double alfa = dot(N, vv.data(), y.data());
            double f2 = alfa / beta;
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) {
                y[q] -= f2 * r2[q];
                r1[q] = r2[q];
                r2[q] = y[q];
                y[q] = minv[q] * r2[q];
            }
            oldb = beta;
            beta = std::sqrt(dot(N, r2.data(), y.data()));
            double oldeps = epsln;
            double delta = cs * dbar + sn * alfa;
            double gbar = sn * dbar - cs * alfa;
            epsln = sn * beta;
            dbar = -cs * beta;
            double gamma = std::sqrt(gbar * gbar + beta * beta);
            if (gamma < DBL_MIN) gamma = DBL_MIN;
            cs = gbar / gamma;
            sn = beta / gamma;
            double phi = cs * phibar;
            phibar = sn * phibar;
            double ig = 1.0 / gamma;
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) {
                double wn = (vv[q] - oldeps * w1[q] - delta * w2[q]) * ig;
                w1[q] = w2[q];
                w2[q] = wn;
                x[q] += phi * wn;
            }
            if (phibar <= target * beta1) break;
        }
        double prev = tr;
        tr = ora_true_residual(N, rp, ci, v, b, x);
        if (tr > tol) {
            double ratio = tr / (inner_tol > 0 ? inner_tol : tol);
            inner_tol = tol / std::max(ratio, 1.0) * 0.5;
            if (tr > 0.9 * prev && rs > 2) break;  // stagnation
        }
    }
    if (iters_out) *iters_out = total;
    return tr;
}

// MINRES with the block-diagonal preconditioner of the GPU's Jacobi mode, on
// the symmetric form of the reduced system (used as the CPU baseline): for
// interior node m the 3x3 velocity block of rows (m, nI+m, 2nI+m) is inverted
// (vinv6[6m..]: xx xy xz yy yz zz), pressure row k is weighted by pinv[k], and
// the rank-one term crank * sum(r_p) is added to every pressure component.
// Runs at most maxit iterations from x (no restarts); returns the
// preconditioned residual reduction phibar / beta1.
double ora_minres_blockjacobi(int64_t N, int64_t nI, const int64_t* rp, const int32_t* ci,
                              const double* v, const double* b, const double* vinv6,
                              const double* pinv, double crank, double* x, double rtol,
                              int64_t maxit, int64_t* iters_out) {
    std::vector<double> r1(N), r2(N), y(N), vv(N), w(N, 0.0), w1(N, 0.0), w2(N, 0.0);
    const int64_t np = N - 3 * nI;
    auto apply = [&](const double* in, double* out) {
        spmv(N, rp, ci, v, in, out);
#pragma omp parallel for schedule(static)
        for (int64_t q = 3 * nI; q < N; ++q) out[q] = -out[q];
    };
    auto prec = [&](const double* in, double* out) {
#pragma omp parallel for schedule(static)
        for (int64_t m = 0; m < nI; ++m) {
            const double* B = vinv6 + 6 * m;
            const double a0 = in[m], a1 = in[nI + m], a2 = in[2 * nI + m];
            out[m] = B[0] * a0 + B[1] * a1 + B[2] * a2;
            out[nI + m] = B[1] * a0 + B[3] * a1 + B[4] * a2;
            out[2 * nI + m] = B[2] * a0 + B[4] * a1 + B[5] * a2;
        }
        double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
        for (int64_t k = 0; k < np; ++k) s += in[3 * nI + k];
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < np; ++k) out[3 * nI + k] = pinv[k] * in[3 * nI + k] + crank * s;
    };
    apply(x, r1.data());
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < N; ++q) r1[q] = (q < 3 * nI ? b[q] : -b[q]) - r1[q];
    r2 = r1;
    prec(r1.data(), y.data());
    const double beta1 = std::sqrt(dot(N, r1.data(), y.data()));
    double oldb = 0.0, beta = beta1, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0;
    int64_t it = 0;
    while (it < maxit && phibar > rtol * beta1 && beta1 > 0.0) {
        ++it;
        const double s = 1.0 / beta;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) vv[q] = s * y[q];
        apply(vv.data(), y.data());
        if (it >= 2) {
            const double f = beta / oldb;
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) y[q] -= f * r1[q];
        }
        const double alfa = dot(N, vv.data(), y.data());
        const double f2 = alfa / beta;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            y[q] -= f2 * r2[q];
            r1[q] = r2[q];
            r2[q] = y[q];
        }
        prec(r2.data(), y.data());
        oldb = beta;
        beta = std::sqrt(dot(N, r2.data(), y.data()));
        const double oldeps = epsln;
        const double delta = cs * dbar + sn * alfa;
        const double gbar = sn * dbar - cs * alfa;
        epsln = sn * beta;
        dbar = -cs * beta;
        double gamma = std::sqrt(gbar * gbar + beta * beta);
        if (gamma < DBL_MIN) gamma = DBL_MIN;
        cs = gbar / gamma;
        sn = beta / gamma;
        const double phi = cs * phibar;
        phibar = sn * phibar;
        const double ig = 1.0 / gamma;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            const double wn = (vv[q] - oldeps * w1[q] - delta * w2[q]) * ig;
            w1[q] = w2[q];
            w2[q] = wn;
            x[q] += phi * wn;
        }
    }
    if (iters_out) *iters_out = it;
    return beta1 > 0.0 ? phibar / beta1 : 0.0;
}

// Scatter of the reduced solution to flow = [ux(np), uy(np), uz(np), p(np)],
// zero on boundary velocity dofs (Flow.cpp:290-300).
int ora_scatter(int64_t np, int64_t N, const int32_t* sidx, const double* x, double* flow) {
    std::fill(flow, flow + 4 * np, 0.0);
    for (int64_t r = 0; r < N; ++r) flow[sidx[r]] = x[r];
    return 0;
}

// ---------------------------------------------------------------------------
// Reaction-diffusion (src/growth/RD.cpp:27-108, :116-172)
// ---------------------------------------------------------------------------
// Parameters, in this order: RD dt, Act, Da, DegA, Inh, Di, DegI,
// GF production, GF diffusion, GF degradation, GF inhibition.
//
// Interior nodes: phi < 0 (LevelSet.cpp:200-211), local index = rank in
// ascending global order; interior elements: all four nodes phi < 0
// (LevelSet.cpp:180-196).  On that submesh (Neumann boundary):
//   M(i,j) = int phi_i phi_j (float-rounded basis table), K(i,j) = int grad phi_i . grad phi_j
//   (Assembler weak forms u.*v and ux.*vx + uy.*vy + uz.*vz, RD.cpp:150-160),
//   L = diag(1 / rowsum M) K  (lump_mass, Assembler.cpp:75-84; RD.cpp:166-169);
// a row with no interior element stays empty.  Explicit Euler, iters steps
// (RD.cpp:74-92):
//   alive (max |act|, |inh| over all nodes >= FLT_MIN):
//     u2 = u.*u; de = 1 + Inh v + GFinh g
//     u' = u + dt (-Da L u + Act u2./de - DegA u);  v' = v + dt (-Di L v + u2 - DegI v)
//   g' = g + dt (-GFdiff L g - GFdeg g);  g'(sources) = GF production
// with g(sources) = GF production before the first step.  Afterwards act,
// inh, gf are zero on every non-interior node (RD.cpp:94-102).  Sources must be
// interior nodes here (the reference's map lookup would send any other node
// to its first interior node).  Returns 0, or -1 for a source outside the
// interior or a degenerate element.
int ora_rd_solve(int64_t np, int64_t nt, const float* xyz, const int32_t* tets,
                 const double* phi, const int32_t* src, int32_t nsrc, const double* prm,
                 int64_t iters, double* act, double* inh, double* gf) {
    const double dt = prm[0];
    if (iters == 0 || dt < FLT_MIN) return 0;
    const double Act = prm[1], Da = prm[2], DegA = prm[3], Inh = prm[4], Di = prm[5],
                 DegI = prm[6], GFprod = prm[7], GFdiff = prm[8], GFdeg = prm[9],
                 GFinh = prm[10];
    std::vector<int64_t> loc(np, -1);
    std::vector<int64_t> nodes;
    for (int64_t i = 0; i < np; ++i)
        if (phi[i] < 0.0) {
            loc[i] = (int64_t)nodes.size();
            nodes.push_back(i);
        }
    const int64_t n = (int64_t)nodes.size();
    for (int32_t s = 0; s < nsrc; ++s)
        if (src[s] < 0 || src[s] >= np || loc[src[s]] < 0) return -1;
    // node -> interior elements, rows of K and lumped M (row gather)
    std::vector<std::vector<int64_t>> n2e(n);
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = tets + 4 * k;
        if (phi[t[0]] < 0.0 && phi[t[1]] < 0.0 && phi[t[2]] < 0.0 && phi[t[3]] < 0.0)
            for (int a = 0; a < 4; ++a) n2e[loc[t[a]]].push_back(k);
    }
    const RefTables& R = tables();
    std::vector<std::vector<std::pair<int64_t, double>>> Lrow(n);
    bool ok = true;
#pragma omp parallel for schedule(dynamic, 256) reduction(&& : ok)
    for (int64_t i = 0; i < n; ++i) {
        std::vector<std::pair<int64_t, double>> row;  // (local col, K)
        double msum = 0.0;
        for (int64_t k : n2e[i]) {
            const int32_t* t = tets + 4 * k;
            Geom G;
            if (!element_geom(xyz, t, G)) {
                ok = false;
                continue;
            }
            int a = 0;
            while (t[a] != nodes[i]) ++a;
            for (int b = 0; b < 4; ++b) {
                double f[4];
                const double gg = G.g[b][0] * G.g[a][0] + G.g[b][1] * G.g[a][1] +
                                  G.g[b][2] * G.g[a][2];
                for (int q = 0; q < 4; ++q) f[q] = gg;
                const double kv = integ(f, R.qw, G.detB);
                for (int q = 0; q < 4; ++q) f[q] = R.phi[b][q] * R.phi[a][q];
                msum += integ(f, R.qw, G.detB);
                const int64_t j = loc[t[b]];
                bool found = false;
                for (auto& e : row)
                    if (e.first == j) {
                        e.second += kv;
                        found = true;
                    }
                if (!found) row.push_back({j, kv});
            }
        }
        std::sort(row.begin(), row.end());
        if (msum != 0.0)
            for (auto& e : row) e.second = e.second / msum;
        else
            row.clear();
        Lrow[i] = std::move(row);
    }
    if (!ok) return -1;
    bool alive = false;
    for (int64_t i = 0; i < np; ++i)
        alive = alive || std::fabs(act[i]) >= FLT_MIN || std::fabs(inh[i]) >= FLT_MIN;
    std::vector<double> u(n), v(n), g(n), un(n), vn(n), gn(n);
    for (int64_t i = 0; i < n; ++i) {
        u[i] = act[nodes[i]];
        v[i] = inh[nodes[i]];
        g[i] = gf[nodes[i]];
    }
    std::vector<char> is_src(n, 0);
    for (int32_t s = 0; s < nsrc; ++s) is_src[loc[src[s]]] = 1;
    for (int64_t i = 0; i < n; ++i)
        if (is_src[i]) g[i] = GFprod;
    for (int64_t it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            double lu = 0.0, lv = 0.0, lg = 0.0;
            for (const auto& e : Lrow[i]) {
                lu += e.second * u[e.first];
                lv += e.second * v[e.first];
                lg += e.second * g[e.first];
            }
            if (alive) {
                const double u2 = u[i] * u[i];
                const double de = 1.0 + Inh * v[i] + GFinh * g[i];
                un[i] = u[i] + dt * (-Da * lu + Act * (u2 / de) - DegA * u[i]);
                vn[i] = v[i] + dt * (-Di * lv + u2 - DegI * v[i]);
            } else {
                un[i] = u[i];
                vn[i] = v[i];
            }
            gn[i] = is_src[i] ? GFprod : g[i] + dt * (-GFdiff * lg - GFdeg * g[i]);
        }
        u.swap(un);
        v.swap(vn);
        g.swap(gn);
    }
    std::fill(act, act + np, 0.0);
    std::fill(inh, inh + np, 0.0);
    std::fill(gf, gf + np, 0.0);
    for (int64_t i = 0; i < n; ++i) {
        act[nodes[i]] = u[i];
        inh[nodes[i]] = v[i];
        gf[nodes[i]] = g[i];
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Distance reset (src/fem/EuclideanDistance.cu:16-38, :92-117, the host path):
// phi_n[k] = min_j sqrt(dx*dx + dy*dy + dz*dz) in float with dx = ifp_j - p_k,
// negated where the old phi_n[k] < 0; FLT_MAX when there is no point.  Nodes
// k0 <= k < k1 only (the CPU baseline times a sample).
// ---------------------------------------------------------------------------
int ora_dist_reset(int64_t np, const float* xyz, const float* ifp, int32_t n_ifp, int64_t k0,
                   int64_t k1, double* phi_n) {
    if (k0 < 0 || k1 > np || k0 > k1) return -1;
#pragma omp parallel for schedule(static)
    for (int64_t k = k0; k < k1; ++k) {
        const float p0 = xyz[3 * k], p1 = xyz[3 * k + 1], p2 = xyz[3 * k + 2];
        float dmin = FLT_MAX;
        for (int32_t j = 0; j < n_ifp; ++j) {
            const float dx = ifp[3 * j] - p0;
            const float dy = ifp[3 * j + 1] - p1;
            const float dz = ifp[3 * j + 2] - p2;
            const float d = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (d < dmin) dmin = d;
        }
        phi_n[k] = phi_n[k] < 0.0f ? -(double)dmin : (double)dmin;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Level-set update (src/fem/LevelSet.cpp:89-151 with resetPhi_ :429-455)
// ---------------------------------------------------------------------------
// Crank-Nicolson advection of phi by the nodal velocity (flow[0..3np)):
//   (M + dt/2 A) phi' = (M - dt/2 A) phi,
//   M(i,j) = int phi_i phi_j,  A(i,j) = int (V . grad phi_j) phi_i with V
//   interpolated at the quadrature points from the nodal values through the
//   float-rounded table (Assembler.hpp:179-190; weak form LevelSet.cpp:106-108),
// solved by Jacobi-preconditioned BiCGSTAB (Eigen's default preconditioner for
// BiCGSTAB<SparseMatrix>, LevelSet.hpp:145) from phi, stop ||r|| <= tol ||b||,
// at most maxit iterations (<= 0: 2N).  Then (reset != 0) the distance reset:
// interface points on the edges whose end values differ in sign bit
// (LevelSet.cpp:278-300), phi_ifn = +-distance to the nearest point
// (EuclideanDistance host path), the crossing edges' nodes keep the advected
// value, and phi = 0.75 phi_kept + 0.25 phi_ifn (LevelSet.cpp:17-18, :147).
// Returns 0; 1 if the solver did not converge (phi untouched); 2 for a NaN
// velocity (phi untouched); 3 for zero dt or zero flow (phi untouched, as the
// reference's early return).
namespace {

// Eigen-style BiCGSTAB with a diagonal (Jacobi) preconditioner.
int bicgstab_jacobi(int64_t N, const int64_t* rp, const int32_t* ci, const double* v,
                    const double* b, double* x, double tol, int64_t maxit, int64_t* iters,
                    double* err) {
    std::vector<double> r(N), r0(N), p(N, 0.0), vv(N, 0.0), s(N), t(N), y(N), z(N), inv(N);
    for (int64_t q = 0; q < N; ++q) {
        double d = 0.0;
        for (int64_t k = rp[q]; k < rp[q + 1]; ++k)
            if (ci[k] == q) d = v[k];
        inv[q] = d != 0.0 ? 1.0 / d : 1.0;
    }
    if (maxit <= 0) maxit = 2 * N;
    spmv(N, rp, ci, v, x, r.data());
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < N; ++q) r[q] = b[q] - r[q];
    const double bb = dot(N, b, b);
    if (bb == 0.0) {
        std::fill(x, x + N, 0.0);
        if (iters) *iters = 0;
        if (err) *err = 0.0;
        return 0;
    }
    r0 = r;
    double r0n = dot(N, r.data(), r.data());
    double rr = r0n;
    const double tol2 = tol * tol * bb;
    const double eps2 = DBL_EPSILON * DBL_EPSILON;
    double rho = 1.0, alpha = 1.0, w = 1.0;
    int64_t it = 0;
    int restarts = 0;
    while (rr > tol2 && it < maxit) {
        const double rho_old = rho;
        rho = dot(N, r0.data(), r.data());
        if (std::fabs(rho) < eps2 * r0n) {
            spmv(N, rp, ci, v, x, r.data());
#pragma omp parallel for schedule(static)
            for (int64_t q = 0; q < N; ++q) r[q] = b[q] - r[q];
            r0 = r;
            rho = r0n = dot(N, r.data(), r.data());
            if (restarts++ == 0) it = 0;
        }
        const double beta = (rho / rho_old) * (alpha / w);
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            p[q] = r[q] + beta * (p[q] - w * vv[q]);
            y[q] = inv[q] * p[q];
        }
        spmv(N, rp, ci, v, y.data(), vv.data());
        alpha = rho / dot(N, r0.data(), vv.data());
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            s[q] = r[q] - alpha * vv[q];
            z[q] = inv[q] * s[q];
        }
        spmv(N, rp, ci, v, z.data(), t.data());
        const double tt = dot(N, t.data(), t.data());
        w = tt > 0.0 ? dot(N, t.data(), s.data()) / tt : 0.0;
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < N; ++q) {
            x[q] += alpha * y[q] + w * z[q];
            r[q] = s[q] - w * t[q];
        }
        rr = dot(N, r.data(), r.data());
        ++it;
    }
    if (iters) *iters = it;
    const double e = std::sqrt(rr / bb);
    if (err) *err = e;
    return rr <= tol2 ? 0 : 1;
}

}  // namespace

int ora_ls_update(int64_t np, int64_t nt, const float* xyz, const int32_t* tets,
                  const double* flow, double* phi, double dt, double tol, int64_t maxit,
                  int reset, int64_t* iters, double* err, int64_t* n_ifp) {
    if (iters) *iters = 0;
    if (n_ifp) *n_ifp = 0;
    double fn = 0.0;
    for (int64_t q = 0; q < 4 * np; ++q) fn += flow[q] * flow[q];
    if (dt < FLT_MIN || std::sqrt(fn) < FLT_MIN) return 3;
    for (int64_t q = 0; q < 3 * np; ++q)
        if (std::isnan(flow[q])) return 2;
    Topology T;
    build_topology(np, nt, tets, T);
    const RefTables& R = tables();
    const int64_t nnz = T.nb_ptr[np];
    std::vector<double> Mv(nnz, 0.0), Av(nnz, 0.0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < np; ++i) {
        const int32_t* cols = T.nb.data() + T.nb_ptr[i];
        const int ncol = (int)(T.nb_ptr[i + 1] - T.nb_ptr[i]);
        for (int64_t q = T.p2t_ptr[i]; q < T.p2t_ptr[i + 1]; ++q) {
            const int64_t k = T.p2t[q];
            const int32_t* t = tets + 4 * k;
            Geom G;
            if (!element_geom(xyz, t, G)) continue;
            int a = 0;
            if (t[1] == i) a = 1;
            else if (t[2] == i) a = 2;
            else if (t[3] == i) a = 3;
            double V[3][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
            for (int j = 0; j < 4; ++j)
                for (int c = 0; c < 3; ++c)
                    for (int qq = 0; qq < 4; ++qq) V[c][qq] += flow[t[j] + c * np] * R.phi[j][qq];
            for (int b = 0; b < 4; ++b) {
                const int slot = find_col(cols, ncol, t[b]);
                double f[4];
                for (int qq = 0; qq < 4; ++qq) f[qq] = R.phi[b][qq] * R.phi[a][qq];
                Mv[T.nb_ptr[i] + slot] += integ(f, R.qw, G.detB);
                for (int qq = 0; qq < 4; ++qq)
                    f[qq] = V[0][qq] * (G.g[b][0] * R.phi[a][qq]) +
                            V[1][qq] * (G.g[b][1] * R.phi[a][qq]) +
                            V[2][qq] * (G.g[b][2] * R.phi[a][qq]);
                Av[T.nb_ptr[i] + slot] += integ(f, R.qw, G.detB);
            }
        }
    }
    const double h = 0.5 * dt;
    std::vector<double> L(nnz), rhs(np), x(phi, phi + np);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < np; ++i) {
        double sacc = 0.0;
        for (int64_t k = T.nb_ptr[i]; k < T.nb_ptr[i + 1]; ++k) {
            L[k] = Mv[k] + h * Av[k];
            sacc += (Mv[k] - h * Av[k]) * phi[T.nb[k]];
        }
        rhs[i] = sacc;
    }
    std::vector<int64_t> rp(T.nb_ptr.begin(), T.nb_ptr.end());
    int64_t it = 0;
    double e = 0.0;
    const int st = bicgstab_jacobi(np, rp.data(), T.nb.data(), L.data(), rhs.data(), x.data(),
                                   tol > 0.0 ? tol : DBL_EPSILON, maxit, &it, &e);
    if (iters) *iters = it;
    if (err) *err = e;
    if (st != 0) return 1;
    if (!reset) {
        std::copy(x.begin(), x.end(), phi);
        return 0;
    }
    // interface points on the crossing edges (i < j)
    std::vector<float> ifp;
    std::vector<char> keep(np, 0);
    for (int64_t i = 0; i < np; ++i)
        for (int64_t k = T.nb_ptr[i]; k < T.nb_ptr[i + 1]; ++k) {
            const int64_t j = T.nb[k];
            if (j <= i || std::signbit(x[i]) == std::signbit(x[j])) continue;
            double tt = 0.5;
            const double div = x[i] - x[j];
            if (std::fabs(div) > FLT_MIN) tt = x[i] / div;
            for (int c = 0; c < 3; ++c)
                ifp.push_back((float)((1.0 - tt) * (double)xyz[3 * i + c] +
                                      tt * (double)xyz[3 * j + c]));
            keep[i] = keep[j] = 1;
        }
    const int32_t nif = (int32_t)(ifp.size() / 3);
    if (n_ifp) *n_ifp = nif;
    std::vector<double> ifn(x);
    ora_dist_reset(np, xyz, ifp.data(), nif, 0, np, ifn.data());
    for (int64_t i = 0; i < np; ++i) {
        const double kept = keep[i] ? x[i] : ifn[i];
        phi[i] = 0.75 * kept + 0.25 * ifn[i];
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Surface tension (Flow::surfaceTension_, Flow.cpp:307-341) with the LevelSet
// quantities it reads.  Inputs: phi (the current level set) and phi_reset (the
// last full distance reset, LevelSet::phi_ifn_, LevelSet.cpp:440).
//  * element gradient of a nodal field (Assembler::grad, Assembler.cpp:11-42):
//    u0 g0 + u1 g1 + u2 g2 + u3 g3 in FP64, stored as float;
//  * nodal gradient (grad_nodes, Assembler.cpp:46-69): float sum of the
//    element gradients over the node's elements / (float) their count;
//  * normals = grad_nodes(phi_reset) (LevelSet.cpp:453);
//  * curvature k = div(grad_nodes(phi_reset) / |.|) by grad_nodes of each
//    normalised component (LevelSet.cpp:215-238), interpolated along the
//    crossing edge with t = phi0 / (phi0 - phi1) (:243-250);
//  * interface points on the edges whose end values differ in sign bit, at
//    t (0.5 when |phi0 - phi1| <= FLT_MIN), as float (LevelSet.cpp:261-300);
//  * patches: per element with mixed signs, its crossing edges in the local
//    order 01 02 03 12 13 23 give one triangle (3 crossings: e0 e1 e2) or two
//    (4 crossings: e0 e2 e3 and e0 e1 e3); each triangle adds 0.5 |e1 x e2|
//    (float cross product) to each of its three points, elements in index
//    order (LevelSet.cpp:326-420);
//  * force: f = (1 - t) st (-k) area rho n0/|n0| to e0 and t st (-k) area rho
//    n1/|n1| to e1, the scalar converted to float before it scales the float
//    normal (Flow.cpp:326-339).
// Edges are taken as (i, j) with i < j (the force is symmetric in the edge's
// orientation).  Returns 0; n_ifp = crossing edges, area = sum of the
// triangle areas (each triangle once).
// ---------------------------------------------------------------------------
namespace {

void elem_grad(int64_t nt, const float* xyz, const int32_t* tets, const double* u,
               std::vector<float>& g) {
    g.assign(3 * (size_t)nt, 0.f);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = tets + 4 * k;
        Geom G;
        if (!element_geom(xyz, t, G)) continue;
        for (int c = 0; c < 3; ++c)
            g[3 * k + c] = (float)(((u[t[0]] * G.g[0][c] + u[t[1]] * G.g[1][c]) +
                                    u[t[2]] * G.g[2][c]) + u[t[3]] * G.g[3][c]);
    }
}

void node_avg(const Topology& T, const std::vector<float>& ge, std::vector<float>& gn) {
    gn.assign(3 * (size_t)T.np, 0.f);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < T.np; ++i) {
        float s[3] = {0.f, 0.f, 0.f};
        for (int64_t q = T.p2t_ptr[i]; q < T.p2t_ptr[i + 1]; ++q)
            for (int c = 0; c < 3; ++c) s[c] += ge[3 * (size_t)T.p2t[q] + c];
        const float cnt = (float)(T.p2t_ptr[i + 1] - T.p2t_ptr[i]);
        for (int c = 0; c < 3; ++c) gn[3 * i + c] = s[c] / cnt;
    }
}

inline float norm3f(const float* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

inline void edge_point(const float* xyz, const double* phi, int32_t a, int32_t b, float out[3]) {
    double t = 0.5;
    const double div = phi[a] - phi[b];
    if (std::fabs(div) > FLT_MIN) t = phi[a] / div;
    for (int c = 0; c < 3; ++c)
        out[c] = (float)((1.0 - t) * (double)xyz[3 * (int64_t)a + c] +
                         t * (double)xyz[3 * (int64_t)b + c]);
}

const int kLocalEdge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

}  // namespace

int ora_surface_tension(int64_t np, int64_t nt, const float* xyz, const int32_t* tets,
                        const double* phi, const double* phi_reset, double st, int32_t rho,
                        double* force, int64_t* n_ifp, double* area_total) {
    Topology T;
    build_topology(np, nt, tets, T);
    std::vector<float> ge, normals, gn;
    elem_grad(nt, xyz, tets, phi_reset, ge);
    node_avg(T, ge, normals);
    // normalised nodal gradient components, then the divergence
    std::vector<double> comp[3];
    for (int c = 0; c < 3; ++c) comp[c].assign(np, 0.0);
    for (int64_t i = 0; i < np; ++i) {
        const float nn = norm3f(&normals[3 * i]);
        for (int c = 0; c < 3; ++c) comp[c][i] = (double)(normals[3 * i + c] / nn);
    }
    std::vector<float> kmesh(np, 0.f), dsum[3];
    for (int c = 0; c < 3; ++c) {
        std::vector<float> e;
        elem_grad(nt, xyz, tets, comp[c].data(), e);
        node_avg(T, e, dsum[c]);
    }
    for (int64_t i = 0; i < np; ++i)
        kmesh[i] = dsum[0][3 * i + 0] + dsum[1][3 * i + 1] + dsum[2][3 * i + 2];
    // crossing edges (i < j) and their slots
    std::vector<int64_t> slot_of;  // per CSR slot: interface point index or -1
    slot_of.assign(T.nb_ptr[np], -1);
    int64_t nif = 0;
    for (int64_t i = 0; i < np; ++i)
        for (int64_t q = T.nb_ptr[i]; q < T.nb_ptr[i + 1]; ++q) {
            const int32_t j = T.nb[q];
            if (j <= i || std::signbit(phi[i]) == std::signbit(phi[j])) continue;
            slot_of[q] = nif++;
        }
    auto point_of = [&](int32_t a, int32_t b) -> int64_t {
        if (a > b) std::swap(a, b);
        const int32_t* cols = T.nb.data() + T.nb_ptr[a];
        const int n = (int)(T.nb_ptr[a + 1] - T.nb_ptr[a]);
        return slot_of[T.nb_ptr[a] + find_col(cols, n, b)];
    };
    // patch areas, elements in index order
    std::vector<float> area(nif, 0.f);
    double atot = 0.0;
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = tets + 4 * k;
        int s = 0;
        for (int m = 0; m < 4; ++m) s += std::signbit(phi[t[m]]) ? 1 : 0;
        if (s == 0 || s == 4) continue;
        int64_t eif[4];
        float pts[4][3];
        int ne = 0;
        for (int e = 0; e < 6; ++e) {
            const int32_t a = t[kLocalEdge[e][0]], b = t[kLocalEdge[e][1]];
            if (std::signbit(phi[a]) == std::signbit(phi[b])) continue;
            if (ne == 4) return 1;
            eif[ne] = point_of(a, b);
            edge_point(xyz, phi, std::min(a, b), std::max(a, b), pts[ne]);
            ++ne;
        }
        if (ne != 3 && ne != 4) return 1;
        const int tri[2][3] = {{0, ne == 3 ? 1 : 2, ne == 3 ? 2 : 3}, {0, 1, 3}};
        for (int tr = 0; tr < (ne == 3 ? 1 : 2); ++tr) {
            const float* p0 = pts[tri[tr][0]];
            const float* p1 = pts[tri[tr][1]];
            const float* p2 = pts[tri[tr][2]];
            float e1[3], e2[3];
            for (int c = 0; c < 3; ++c) {
                e1[c] = p1[c] - p0[c];
                e2[c] = p2[c] - p0[c];
            }
            const float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                                 e1[0] * e2[1] - e1[1] * e2[0]};
            const double ha = 0.5 * (double)norm3f(cr);
            atot += ha;
            for (int m = 0; m < 3; ++m) {
                float& A = area[eif[tri[tr][m]]];
                A = (float)((double)A + ha);
            }
        }
    }
    // forces
    std::fill(force, force + 3 * np, 0.0);
    const float stf = (float)st;
    for (int64_t i = 0; i < np; ++i)
        for (int64_t q = T.nb_ptr[i]; q < T.nb_ptr[i + 1]; ++q) {
            if (slot_of[q] < 0) continue;
            const int32_t e0 = (int32_t)i, e1 = T.nb[q];
            const float t = (float)(phi[e0] / (phi[e0] - phi[e1]));
            const float kif = (float)((1.0 - (double)t) * (double)kmesh[e0] + (double)(t * kmesh[e1]));
            const float A = area[slot_of[q]];
            const int32_t ends[2] = {e0, e1};
            for (int m = 0; m < 2; ++m) {
                const float* nv = &normals[3 * (size_t)ends[m]];
                const float nn = norm3f(nv);
                const double w = m == 0 ? (1.0 - (double)t) : (double)t;
                const float sc = (float)(w * (double)stf * (double)(-kif) * (double)A * (double)rho);
                for (int c = 0; c < 3; ++c) force[c * np + ends[m]] += (double)(sc * (nv[c] / nn));
            }
        }
    if (n_ifp) *n_ifp = nif;
    if (area_total) *area_total = atot;
    return 0;
}

// ---------------------------------------------------------------------------
// P2-P1 system (the reference's velocity degree 2), in the reference's own
// form: unknowns [ux(nd), uy(nd), uz(nd), p(np)] with nd = np + ne (vertices,
// then edges), rows
//   [A11 A12 A13 -Bx; A12' A22 A23 -By; A13' A23' A33 -Bz; Bx' By' Bz' eps M]
// (Flow.cpp:160-203 with uDeg_ = 2), every P2 integral by the element loop of
// bilin_without_p2t_ij: for trial j, test i, feval at the quadrature points
// of the rule of degree deg_i + deg_j, dot (w/6), times |det B|
// (Assembler.hpp:321-424); M by the P1 path.  F = [N fx + Cx s; N fy + Cy s;
// N fz + Cz s; M s] (Flow.cpp:392-396).  The triplets are returned unsummed
// (setFromTriplets sums them); sidx = interior velocity DOFs of the three
// components and all pressure DOFs (Flow.cpp:35-44).
// ---------------------------------------------------------------------------
namespace {

const double kR3x[10] = {0.7784952948213300, 0.0738349017262234, 0.0738349017262234, 0.0738349017262234, 0.4062443438840510, 0.4062443438840510, 0.4062443438840510, 0.0937556561159491, 0.0937556561159491, 0.0937556561159491};
const double kR3y[10] = {0.0738349017262234, 0.7784952948213300, 0.0738349017262234, 0.0738349017262234, 0.4062443438840510, 0.0937556561159491, 0.0937556561159491, 0.4062443438840510, 0.4062443438840510, 0.0937556561159491};
const double kR3z[10] = {0.0738349017262234, 0.0738349017262234, 0.7784952948213300, 0.0738349017262234, 0.0937556561159491, 0.4062443438840510, 0.0937556561159491, 0.4062443438840510, 0.0937556561159491, 0.4062443438840510};
const double kR3w[10] = {0.0476331348432089, 0.0476331348432089, 0.0476331348432089, 0.0476331348432089, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610};
const double kR4x[20] = {0.9029422158182680, 0.0323525947272439, 0.0323525947272439, 0.0323525947272439, 0.2626825838877790, 0.6165965330619370, 0.2626825838877790, 0.6165965330619370, 0.2626825838877790, 0.6165965330619370, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.3097693042728620, 0.3097693042728620, 0.3097693042728620, 0.0706920871814129};
const double kR4y[20] = {0.0323525947272439, 0.9029422158182680, 0.0323525947272439, 0.0323525947272439, 0.6165965330619370, 0.2626825838877790, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.2626825838877790, 0.6165965330619370, 0.2626825838877790, 0.6165965330619370, 0.0603604415251421, 0.0603604415251421, 0.3097693042728620, 0.3097693042728620, 0.0706920871814129, 0.3097693042728620};
const double kR4z[20] = {0.0323525947272439, 0.0323525947272439, 0.9029422158182680, 0.0323525947272439, 0.0603604415251421, 0.0603604415251421, 0.6165965330619370, 0.2626825838877790, 0.0603604415251421, 0.0603604415251421, 0.6165965330619370, 0.2626825838877790, 0.0603604415251421, 0.0603604415251421, 0.2626825838877790, 0.6165965330619370, 0.3097693042728620, 0.0706920871814129, 0.3097693042728620, 0.3097693042728620};
const double kR4w[20] = {0.0070670747944695, 0.0070670747944695, 0.0070670747944695, 0.0070670747944695, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.1019369182898680, 0.1019369182898680, 0.1019369182898680, 0.1019369182898680};

// Basis tables at a rule: value[a][q], grad[a][c][q] (float-rounded).
struct Tab {
    int nq;
    double w[20];
    double p2[10][20], g2[10][3][20], p1[4][20];
};

Tab make_tab(int nq, const double* x, const double* y, const double* z, const double* w) {
    Tab T;
    T.nq = nq;
    for (int q = 0; q < nq; ++q) {
        T.w[q] = w[q] / 6.0;
        const float fx = (float)x[q], fy = (float)y[q], fz = (float)z[q];
        const double X = fx, Y = fy, Z = fz, L = 1.0 - X - Y - Z;
        const double v[10] = {L * (1.0 - 2.0 * X - 2.0 * Y - 2.0 * Z), X * (2.0 * X - 1.0),
                              Y * (2.0 * Y - 1.0), Z * (2.0 * Z - 1.0), 4.0 * X * L, 4.0 * Y * L,
                              4.0 * Z * L, 4.0 * X * Y, 4.0 * X * Z, 4.0 * Y * Z};
        const double sg = 4.0 * X + 4.0 * Y + 4.0 * Z - 3.0;
        const double gx[10] = {sg, 4.0 * X - 1.0, 0.0, 0.0, -8.0 * X - 4.0 * Y - 4.0 * Z + 4.0,
                               -4.0 * Y, -4.0 * Z, 4.0 * Y, 4.0 * Z, 0.0};
        const double gy[10] = {sg, 0.0, 4.0 * Y - 1.0, 0.0, -4.0 * X,
                               -4.0 * X - 8.0 * Y - 4.0 * Z + 4.0, -4.0 * Z, 4.0 * X, 0.0, 4.0 * Z};
        const double gz[10] = {sg, 0.0, 0.0, 4.0 * Z - 1.0, -4.0 * X, -4.0 * Y,
                               -4.0 * X - 4.0 * Y - 8.0 * Z + 4.0, 0.0, 4.0 * X, 4.0 * Y};
        for (int a = 0; a < 10; ++a) {
            T.p2[a][q] = (float)v[a];
            T.g2[a][0][q] = (float)gx[a];
            T.g2[a][1][q] = (float)gy[a];
            T.g2[a][2][q] = (float)gz[a];
        }
        T.p1[0][q] = (float)(1.0 - X - Y - Z);
        T.p1[1][q] = X;
        T.p1[2][q] = Y;
        T.p1[3][q] = Z;
    }
    return T;
}

struct P2Sys {
    std::vector<int64_t> r;
    std::vector<int32_t> c;
    std::vector<double> v;
    std::vector<double> F;
    std::vector<int64_t> sidx;
    int64_t nd = 0, ne = 0;
};

}  // namespace

// Builds the system; returns a handle, the triplet count, nd and the reduced size.
void* ora_p2_build(int64_t np, int64_t nt, const float* xyz, const int32_t* tets,
                   const uint8_t* bnd, const double* mu, const double* s_in, const double* fst,
                   double eps, int64_t* ntrip, int64_t* nd_out, int64_t* nred) {
    Topology T;
    build_topology(np, nt, tets, T);
    // edges: (i, j > i) of the node graph in row order
    std::vector<int64_t> eid(T.nb_ptr[np], -1);
    int64_t ne = 0;
    for (int64_t i = 0; i < np; ++i)
        for (int64_t q = T.nb_ptr[i]; q < T.nb_ptr[i + 1]; ++q)
            if (T.nb[q] > i) eid[q] = ne++;
    auto edge = [&](int32_t a, int32_t b) {
        if (a > b) std::swap(a, b);
        const int n = (int)(T.nb_ptr[a + 1] - T.nb_ptr[a]);
        return eid[T.nb_ptr[a] + find_col(T.nb.data() + T.nb_ptr[a], n, b)];
    };
    static const int le[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    const int64_t nd = np + ne;
    auto* S = new P2Sys;
    S->nd = nd;
    S->ne = ne;
    // boundary DOFs: boundary vertices (given) and the edges of boundary faces
    std::vector<char> dbnd(nd, 0);
    for (int64_t i = 0; i < np; ++i) dbnd[i] = bnd[i] ? 1 : 0;
    {
        static const int fc[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
        for (int64_t k = 0; k < nt; ++k) {
            const int32_t* t = tets + 4 * k;
            for (int f = 0; f < 4; ++f) {
                const int32_t v[3] = {t[fc[f][0]], t[fc[f][1]], t[fc[f][2]]};
                bool shared = false;
                for (int64_t q = T.p2t_ptr[v[0]]; q < T.p2t_ptr[v[0] + 1] && !shared; ++q) {
                    const int64_t k2 = T.p2t[q];
                    if (k2 == k) continue;
                    const int32_t* t2 = tets + 4 * k2;
                    int hit = 0;
                    for (int j = 0; j < 4; ++j) hit += (t2[j] == v[1]) + (t2[j] == v[2]);
                    shared = hit == 2;
                }
                if (shared) continue;
                for (int a = 0; a < 3; ++a)
                    for (int b = a + 1; b < 3; ++b) dbnd[np + edge(v[a], v[b])] = 1;
            }
        }
    }
    const Tab t4 = make_tab(20, kR4x, kR4y, kR4z, kR4w);
    const Tab t3 = make_tab(10, kR3x, kR3y, kR3z, kR3w);
    const RefTables& R1 = tables();
    // zero-mean source (Flow.cpp:376)
    std::vector<double> s(s_in, s_in + np);
    double mean = 0.0;
    for (double v : s) mean += v;
    mean /= (double)np;
    for (double& v : s) v -= mean;
    S->F.assign(3 * nd + np, 0.0);
    auto add = [&](int64_t r, int64_t c, double v) {
        S->r.push_back(r);
        S->c.push_back((int32_t)c);
        S->v.push_back(v);
    };
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = tets + 4 * k;
        int64_t dof[10];
        for (int j = 0; j < 4; ++j) dof[j] = t[j];
        for (int e = 0; e < 6; ++e) dof[4 + e] = np + edge(t[le[e][0]], t[le[e][1]]);
        Geom G;
        if (!element_geom(xyz, t, G)) continue;
        // invB^T (Geom.g[c+1][r] = invB^T(r, c)); global gradients at the points
        double it[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) it[r][c] = G.g[c + 1][r];
        auto grads = [&](const Tab& tb, double out[10][3][20]) {
            for (int a = 0; a < 10; ++a)
                for (int q = 0; q < tb.nq; ++q)
                    for (int r = 0; r < 3; ++r)
                        out[a][r][q] = it[r][0] * tb.g2[a][0][q] + it[r][1] * tb.g2[a][1][q] +
                                       it[r][2] * tb.g2[a][2][q];
        };
        static thread_local double g4[10][3][20], g3[10][3][20];
        grads(t4, g4);
        grads(t3, g3);
        const double detB = G.detB, m = mu[k];
        auto integ4 = [&](auto f) {
            double acc = 0.0;
            for (int q = 0; q < 20; ++q) acc += f(q) * t4.w[q];
            return acc * detB;
        };
        auto integ3 = [&](auto f) {
            double acc = 0.0;
            for (int q = 0; q < 10; ++q) acc += f(q) * t3.w[q];
            return acc * detB;
        };
        // viscous blocks: trial j (u), test i (v)
        for (int j = 0; j < 10; ++j)
            for (int i = 0; i < 10; ++i) {
                const auto& gu = g4[j];
                const auto& gv = g4[i];
                const double a11 = integ4([&](int q) { return (2.0 * gu[0][q] * gv[0][q] + gu[1][q] * gv[1][q] + gu[2][q] * gv[2][q]) * m; });
                const double a22 = integ4([&](int q) { return (gu[0][q] * gv[0][q] + 2.0 * gu[1][q] * gv[1][q] + gu[2][q] * gv[2][q]) * m; });
                const double a33 = integ4([&](int q) { return (gu[0][q] * gv[0][q] + gu[1][q] * gv[1][q] + 2.0 * gu[2][q] * gv[2][q]) * m; });
                const double a12 = integ4([&](int q) { return gu[0][q] * gv[1][q] * m; });
                const double a13 = integ4([&](int q) { return gu[0][q] * gv[2][q] * m; });
                const double a23 = integ4([&](int q) { return gu[1][q] * gv[2][q] * m; });
                const int64_t I = dof[i], J = dof[j];
                add(I, J, a11);
                add(nd + I, nd + J, a22);
                add(2 * nd + I, 2 * nd + J, a33);
                add(I, nd + J, a12);           // row x, column y: A12
                add(nd + J, I, a12);           // A12' in row y
                add(I, 2 * nd + J, a13);
                add(2 * nd + J, I, a13);
                add(nd + I, 2 * nd + J, a23);
                add(2 * nd + J, nd + I, a23);
            }
        // B (test P2 i, trial P1 j), N, C, degree 3
        for (int j = 0; j < 4; ++j)
            for (int i = 0; i < 10; ++i) {
                const int64_t I = dof[i], J = t[j];
                const double bx = integ3([&](int q) { return g3[i][0][q] * t3.p1[j][q]; });
                const double by = integ3([&](int q) { return g3[i][1][q] * t3.p1[j][q]; });
                const double bz = integ3([&](int q) { return g3[i][2][q] * t3.p1[j][q]; });
                add(I, 3 * nd + J, -bx);
                add(nd + I, 3 * nd + J, -by);
                add(2 * nd + I, 3 * nd + J, -bz);
                add(3 * nd + J, I, bx);
                add(3 * nd + J, nd + I, by);
                add(3 * nd + J, 2 * nd + I, bz);
                const double cm = 2.0 / 3 * m;
                const double nij = integ3([&](int q) { return t3.p2[i][q] * t3.p1[j][q]; });
                for (int al = 0; al < 3; ++al) {
                    const double cij = integ3([&](int q) { return cm * (t3.p1[j][q] * g3[i][al][q]); });
                    S->F[al * nd + I] += cij * s[J];
                    if (fst) S->F[al * nd + I] += nij * fst[al * np + J];
                }
            }
        // eps M and M s (P1, degree 2)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) {
                double f[4];
                for (int q = 0; q < 4; ++q) f[q] = R1.phi[b][q] * R1.phi[a][q];
                const double mab = integ(f, R1.qw, G.detB);
                add(3 * nd + t[a], 3 * nd + t[b], eps * mab);
                S->F[3 * nd + t[a]] += mab * s[t[b]];
            }
    }
    int64_t nI = 0;
    for (int64_t d = 0; d < nd; ++d) nI += dbnd[d] ? 0 : 1;
    S->sidx.resize(3 * nI + np);
    int64_t w = 0;
    for (int c = 0; c < 3; ++c)
        for (int64_t d = 0; d < nd; ++d)
            if (!dbnd[d]) S->sidx[w++] = c * nd + d;
    for (int64_t i = 0; i < np; ++i) S->sidx[w++] = 3 * nd + i;
    *ntrip = (int64_t)S->v.size();
    *nd_out = nd;
    *nred = (int64_t)S->sidx.size();
    return S;
}

void ora_p2_fetch(void* h, int64_t* rows, int32_t* cols, double* vals, double* F, int64_t* sidx) {
    auto* S = static_cast<P2Sys*>(h);
    std::copy(S->r.begin(), S->r.end(), rows);
    std::copy(S->c.begin(), S->c.end(), cols);
    std::copy(S->v.begin(), S->v.end(), vals);
    std::copy(S->F.begin(), S->F.end(), F);
    std::copy(S->sidx.begin(), S->sidx.end(), sidx);
}

void ora_p2_free(void* h) { delete static_cast<P2Sys*>(h); }

// Timing helper for the CPU baseline.
double ora_now_ms(void) { return now_ms(); }

}  // extern "C"
