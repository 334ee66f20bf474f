// Host-side mesh setup (once per context): validation, node -> tetrahedra map,
// block sparsity pattern of the node graph, Dirichlet flags, Kuhn-lattice
// detection.  OpenMP over nodes / tetrahedra.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "fts_internal.h"

namespace fts {

double wall_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

RefConstants ref_constants() {
    // The basis values pass through float (std::function<float(float,float,float)>,
    // Tetrahedron.hpp:17-18) while 1 - x - y - z is evaluated in double.
    RefConstants R;
    double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0;
    double b = (5.0 - std::sqrt(5.0)) / 20.0;
    double qp[3][4] = {{a, b, b, b}, {b, a, b, b}, {b, b, a, b}};
    double phi[4][4];
    for (int q = 0; q < 4; ++q) {
        float x = (float)qp[0][q], y = (float)qp[1][q], z = (float)qp[2][q];
        phi[0][q] = (double)(float)(1.0 - x - y - z);
        phi[1][q] = (double)x;
        phi[2][q] = (double)y;
        phi[3][q] = (double)z;
    }
    std::memcpy(R.phi, phi, sizeof(phi));
    for (int i = 0; i < 4; ++i) {
        double s = 0.0;
        for (int q = 0; q < 4; ++q) s += 0.25 * phi[i][q];
        R.wq[i] = s;
        for (int j = 0; j < 4; ++j) {
            double m = 0.0;
            for (int q = 0; q < 4; ++q) m += 0.25 * (phi[i][q] * phi[j][q]);
            R.mref[i][j] = m;
        }
    }
    return R;
}

// Quadrature rules of degree 3 (10 points) and 4 (20 points) on the unit
// tetrahedron as the reference lists them (Quadrature.hpp:37-56): the point
// coordinates and weights have to be these numbers for the element integrals
// to match.
namespace {
const double kQ3x[10] = {0.7784952948213300, 0.0738349017262234, 0.0738349017262234, 0.0738349017262234, 0.4062443438840510, 0.4062443438840510, 0.4062443438840510, 0.0937556561159491, 0.0937556561159491, 0.0937556561159491};
const double kQ3y[10] = {0.0738349017262234, 0.7784952948213300, 0.0738349017262234, 0.0738349017262234, 0.4062443438840510, 0.0937556561159491, 0.0937556561159491, 0.4062443438840510, 0.4062443438840510, 0.0937556561159491};
const double kQ3z[10] = {0.0738349017262234, 0.0738349017262234, 0.7784952948213300, 0.0738349017262234, 0.0937556561159491, 0.4062443438840510, 0.0937556561159491, 0.4062443438840510, 0.0937556561159491, 0.4062443438840510};
const double kQ3w[10] = {0.0476331348432089, 0.0476331348432089, 0.0476331348432089, 0.0476331348432089, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610, 0.1349112434378610};
const double kQ4x[20] = {0.9029422158182680, 0.0323525947272439, 0.0323525947272439, 0.0323525947272439, 0.2626825838877790, 0.6165965330619370, 0.2626825838877790, 0.6165965330619370, 0.2626825838877790, 0.6165965330619370, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.3097693042728620, 0.3097693042728620, 0.3097693042728620, 0.0706920871814129};
const double kQ4y[20] = {0.0323525947272439, 0.9029422158182680, 0.0323525947272439, 0.0323525947272439, 0.6165965330619370, 0.2626825838877790, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.0603604415251421, 0.2626825838877790, 0.6165965330619370, 0.2626825838877790, 0.6165965330619370, 0.0603604415251421, 0.0603604415251421, 0.3097693042728620, 0.3097693042728620, 0.0706920871814129, 0.3097693042728620};
const double kQ4z[20] = {0.0323525947272439, 0.0323525947272439, 0.9029422158182680, 0.0323525947272439, 0.0603604415251421, 0.0603604415251421, 0.6165965330619370, 0.2626825838877790, 0.0603604415251421, 0.0603604415251421, 0.6165965330619370, 0.2626825838877790, 0.0603604415251421, 0.0603604415251421, 0.2626825838877790, 0.6165965330619370, 0.3097693042728620, 0.0706920871814129, 0.3097693042728620, 0.3097693042728620};
const double kQ4w[20] = {0.0070670747944695, 0.0070670747944695, 0.0070670747944695, 0.0070670747944695, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.0469986689718877, 0.1019369182898680, 0.1019369182898680, 0.1019369182898680, 0.1019369182898680};

// P2 basis (vertices 0..3, then the edges 01 02 03 12 13 23) and its
// reference gradient at float (x, y, z): expressions in double, results
// rounded to float as the reference's std::function<float(float,float,float)>.
void p2_basis(float x, float y, float z, double phi[10], double g[10][3]) {
    const double X = x, Y = y, Z = z, L = 1.0 - X - Y - Z;
    phi[0] = (float)(L * (1.0 - 2.0 * X - 2.0 * Y - 2.0 * Z));
    phi[1] = (float)(X * (2.0 * X - 1.0));
    phi[2] = (float)(Y * (2.0 * Y - 1.0));
    phi[3] = (float)(Z * (2.0 * Z - 1.0));
    phi[4] = (float)(4.0 * X * L);
    phi[5] = (float)(4.0 * Y * L);
    phi[6] = (float)(4.0 * Z * L);
    phi[7] = (float)(4.0 * X * Y);
    phi[8] = (float)(4.0 * X * Z);
    phi[9] = (float)(4.0 * Y * Z);
    const double s = 4.0 * X + 4.0 * Y + 4.0 * Z - 3.0;
    const double gx[10] = {s, 4.0 * X - 1.0, 0.0, 0.0, -8.0 * X - 4.0 * Y - 4.0 * Z + 4.0,
                           -4.0 * Y, -4.0 * Z, 4.0 * Y, 4.0 * Z, 0.0};
    const double gy[10] = {s, 0.0, 4.0 * Y - 1.0, 0.0, -4.0 * X,
                           -4.0 * X - 8.0 * Y - 4.0 * Z + 4.0, -4.0 * Z, 4.0 * X, 0.0, 4.0 * Z};
    const double gz[10] = {s, 0.0, 0.0, 4.0 * Z - 1.0, -4.0 * X, -4.0 * Y,
                           -4.0 * X - 4.0 * Y - 8.0 * Z + 4.0, 0.0, 4.0 * X, 4.0 * Y};
    for (int a = 0; a < 10; ++a) {
        g[a][0] = (float)gx[a];
        g[a][1] = (float)gy[a];
        g[a][2] = (float)gz[a];
    }
}

void p1_basis(float x, float y, float z, double psi[4]) {
    psi[0] = (float)(1.0 - (double)x - (double)y - (double)z);
    psi[1] = x;
    psi[2] = y;
    psi[3] = z;
}
}  // namespace

RefP2 ref_p2() {
    RefP2 R;
    std::memset(&R, 0, sizeof(R));
    for (int q = 0; q < 20; ++q) {
        double phi[10], g[10][3];
        p2_basis((float)kQ4x[q], (float)kQ4y[q], (float)kQ4z[q], phi, g);
        for (int a = 0; a < 10; ++a)
            for (int b = 0; b < 10; ++b)
                for (int m = 0; m < 3; ++m)
                    for (int n = 0; n < 3; ++n) R.K[a][b][m][n] += kQ4w[q] * (g[a][m] * g[b][n]);
    }
    for (int q = 0; q < 10; ++q) {
        double phi[10], g[10][3], psi[4];
        const float x = (float)kQ3x[q], y = (float)kQ3y[q], z = (float)kQ3z[q];
        p2_basis(x, y, z, phi, g);
        p1_basis(x, y, z, psi);
        for (int a = 0; a < 10; ++a)
            for (int k = 0; k < 4; ++k) {
                R.N[a][k] += kQ3w[q] * (phi[a] * psi[k]);
                for (int m = 0; m < 3; ++m) R.B[a][k][m] += kQ3w[q] * (g[a][m] * psi[k]);
            }
    }
    return R;
}

void boundary_from_faces(const fts_mesh& m, const HostTopology& T, std::vector<uint8_t>& bnd) {
    const int64_t nt = m.nt;
    const int32_t* tets = m.tets;
    bnd.assign((size_t)m.np, 0);
    uint8_t* out = bnd.data();
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = tets + 4 * k;
        for (int f = 0; f < 4; ++f) {
            int32_t v[3];
            int n = 0;
            for (int j = 0; j < 4; ++j)
                if (j != f) v[n++] = t[j];
            bool shared = false;
            for (int32_t q = T.p2t_ptr[v[0]]; q < T.p2t_ptr[v[0] + 1] && !shared; ++q) {
                int64_t k2 = T.p2t[q] >> 2;
                if (k2 == k) continue;
                const int32_t* t2 = tets + 4 * k2;
                int hit = 0;
                for (int j = 0; j < 4; ++j) hit += (t2[j] == v[1]) + (t2[j] == v[2]);
                shared = (hit == 2);
            }
            if (!shared) {
                for (int j = 0; j < 3; ++j) {
#pragma omp atomic write
                    out[v[j]] = 1;
                }
            }
        }
    }
}

// A mesh is treated as the Kuhn lattice of n^3 nodes when np = n^3, node
// index = i + n j + n^2 k, and every node's graph neighbours are among its 14
// Kuhn lattice directions (+-e_x, +-e_y, +-e_z, +-(1,1,0), +-(1,0,1), +-(0,1,1),
// +-(1,1,1)).  Coordinates may be jittered; only connectivity matters.
static int32_t detect_lattice(const HostTopology& T) {
    int64_t n = (int64_t)std::llround(std::cbrt((double)T.np));
    if (n < 3 || n * n * n != T.np || T.nt != 6 * (n - 1) * (n - 1) * (n - 1)) return 0;
    bool ok = true;
#pragma omp parallel for schedule(static) reduction(&& : ok)
    for (int64_t v = 0; v < T.np; ++v) {
        int64_t i = v % n, j = (v / n) % n, k = v / (n * n);
        for (int32_t q = T.rowptr[v]; q < T.rowptr[v + 1]; ++q) {
            int64_t w = T.cols[q];
            int64_t di = w % n - i, dj = (w / n) % n - j, dk = w / (n * n) - k;
            bool good = (di >= -1 && di <= 1 && dj >= -1 && dj <= 1 && dk >= -1 && dk <= 1);
            // Kuhn directions have all non-zero components of one sign
            bool pos = di >= 0 && dj >= 0 && dk >= 0;
            bool neg = di <= 0 && dj <= 0 && dk <= 0;
            ok = ok && good && (pos || neg);
        }
    }
    return ok ? (int32_t)n : 0;
}

// Whether element 6c + t of cube c = (ci, cj, ck) is the path origin,
// origin + e_p0, origin + e_p0 + e_p1, origin + (1,1,1) of axis permutation t
// ({0,1,2} {0,2,1} {1,0,2} {1,2,0} {2,0,1} {2,1,0}), nodes in that order.
static bool kuhn_element_order(const fts_mesh& m, int32_t n) {
    static const int perm[6][2] = {{0, 1}, {0, 2}, {1, 0}, {1, 2}, {2, 0}, {2, 1}};
    const int64_t nn = n, cm = n - 1;
    const int64_t step[3] = {1, nn, nn * nn};
    if (m.nt != 6 * cm * cm * cm) return false;  // exactly the lattice's elements
    bool ok = true;
#pragma omp parallel for schedule(static) reduction(&& : ok)
    for (int64_t c = 0; c < cm * cm * cm; ++c) {
        const int64_t ci = c % cm, cj = (c / cm) % cm, ck = c / (cm * cm);
        const int64_t o = ci + nn * (cj + nn * ck);
        for (int t = 0; t < 6; ++t) {
            const int32_t* e = m.tets + 4 * (6 * c + t);
            const int64_t a = o + step[perm[t][0]], b = a + step[perm[t][1]];
            ok = ok && e[0] == o && e[1] == a && e[2] == b && e[3] == o + 1 + nn + nn * nn;
        }
    }
    return ok;
}

int build_topology(const fts_mesh& m, HostTopology& T, std::string& err) {
    if (m.np <= 0 || m.nt <= 0 || !m.xyz || !m.tets) {
        err = "mesh: np, nt, xyz and tets are required";
        return FTS_ERR_BAD_INPUT;
    }
    if (m.np >= (int64_t)1 << 31 || m.nt >= (int64_t)1 << 29) {
        err = "mesh: too many nodes or tetrahedra for 32-bit indices";
        return FTS_ERR_BAD_INPUT;
    }
    const int64_t np = m.np, nt = m.nt;
    T.np = np;
    T.nt = nt;
    bool bad = false;
#pragma omp parallel for schedule(static) reduction(|| : bad)
    for (int64_t e = 0; e < 4 * nt; ++e) bad = bad || m.tets[e] < 0 || m.tets[e] >= np;
    if (bad) {
        err = "mesh: tetrahedron node index out of range";
        return FTS_ERR_BAD_INPUT;
    }
    // node -> tetrahedra (counting sort keeps ascending tetrahedron order)
    T.p2t_ptr.assign((size_t)np + 1, 0);
    for (int64_t e = 0; e < 4 * nt; ++e) T.p2t_ptr[m.tets[e] + 1]++;
    for (int64_t i = 0; i < np; ++i) T.p2t_ptr[i + 1] += T.p2t_ptr[i];
    T.p2t.resize((size_t)(4 * nt));
    {
        std::vector<int32_t> fill(T.p2t_ptr.begin(), T.p2t_ptr.end() - 1);
        for (int64_t k = 0; k < nt; ++k)
            for (int j = 0; j < 4; ++j)
                T.p2t[fill[m.tets[4 * k + j]]++] = (uint32_t)((k << 2) | j);
    }
    int32_t maxp = 0;
    for (int64_t i = 0; i < np; ++i) maxp = std::max(maxp, T.p2t_ptr[i + 1] - T.p2t_ptr[i]);
    T.max_p2t = maxp;
    if (maxp == 0 || maxp > 4096) {
        err = "mesh: a node belongs to no tetrahedron or to more than 4096";
        return FTS_ERR_BAD_INPUT;
    }
    // node graph (sorted unique neighbours incl. self)
    std::vector<int32_t> cnt((size_t)np);
    auto neighbours = [&](int64_t i, std::vector<int32_t>& buf) {
        buf.clear();
        for (int32_t q = T.p2t_ptr[i]; q < T.p2t_ptr[i + 1]; ++q) {
            const int32_t* t = m.tets + 4 * (int64_t)(T.p2t[q] >> 2);
            for (int j = 0; j < 4; ++j) buf.push_back(t[j]);
        }
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    };
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t i = 0; i < np; ++i) {
            neighbours(i, buf);
            cnt[i] = (int32_t)buf.size();
        }
    }
    T.rowptr.assign((size_t)np + 1, 0);
    int64_t acc = 0;
    int32_t maxr = 0;
    for (int64_t i = 0; i < np; ++i) {
        T.rowptr[i] = (int32_t)acc;
        acc += cnt[i];
        maxr = std::max(maxr, cnt[i]);
    }
    if (acc >= (int64_t)1 << 31) {
        err = "mesh: node graph too large for 32-bit block indices";
        return FTS_ERR_BAD_INPUT;
    }
    T.rowptr[np] = (int32_t)acc;
    T.max_row = maxr;
    T.cols.resize((size_t)acc);
    T.diag.resize((size_t)np);
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t i = 0; i < np; ++i) {
            neighbours(i, buf);
            std::copy(buf.begin(), buf.end(), T.cols.begin() + T.rowptr[i]);
            T.diag[i] = T.rowptr[i] +
                        (int32_t)(std::lower_bound(buf.begin(), buf.end(), (int32_t)i) - buf.begin());
        }
    }
    if (m.boundary) {
        T.bnd.assign(m.boundary, m.boundary + np);
        for (auto& b : T.bnd) b = b ? 1 : 0;
    } else {
        boundary_from_faces(m, T, T.bnd);
    }
    int64_t nI = 0;
    for (int64_t i = 0; i < np; ++i) nI += T.bnd[i] ? 0 : 1;
    T.n_interior = nI;
    T.lattice_n = detect_lattice(T);
    T.kuhn_elements = T.lattice_n > 0 && kuhn_element_order(m, T.lattice_n);
    T.nv = np;
    return FTS_OK;
}

int extend_p2(const fts_mesh& m, HostTopology& T, std::string& err) {
    static const int kEdge[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
    const int64_t nv = T.np, nt = T.nt;
    // edge ids: the slots (i, j > i) of the vertex graph, in row order
    std::vector<int64_t> eid((size_t)T.rowptr[nv], -1);
    int64_t ne = 0;
    for (int64_t i = 0; i < nv; ++i)
        for (int32_t q = T.rowptr[i]; q < T.rowptr[i + 1]; ++q)
            if (T.cols[q] > i) eid[q] = ne++;
    const int64_t nn = nv + ne;
    if (nn >= (int64_t)1 << 31) {
        err = "mesh: too many P2 nodes for 32-bit indices";
        return FTS_ERR_BAD_INPUT;
    }
    // edge end vertices and the edges at each vertex (the P2 -> P1 transfer)
    T.edge_ends.assign((size_t)2 * ne, 0);
    for (int64_t i = 0; i < nv; ++i)
        for (int32_t q = T.rowptr[i]; q < T.rowptr[i + 1]; ++q)
            if (eid[q] >= 0) {
                T.edge_ends[2 * eid[q]] = (int32_t)i;
                T.edge_ends[2 * eid[q] + 1] = T.cols[q];
            }
    T.vinc_ptr.assign((size_t)nv + 1, 0);
    for (int64_t e = 0; e < ne; ++e) {
        T.vinc_ptr[T.edge_ends[2 * e] + 1]++;
        T.vinc_ptr[T.edge_ends[2 * e + 1] + 1]++;
    }
    for (int64_t i = 0; i < nv; ++i) T.vinc_ptr[i + 1] += T.vinc_ptr[i];
    T.vinc.assign((size_t)2 * ne, 0);
    {
        std::vector<int32_t> fill(T.vinc_ptr.begin(), T.vinc_ptr.end() - 1);
        for (int64_t e = 0; e < ne; ++e) {
            T.vinc[fill[T.edge_ends[2 * e]]++] = (int32_t)e;
            T.vinc[fill[T.edge_ends[2 * e + 1]]++] = (int32_t)e;
        }
    }
    auto edge_of = [&](int32_t a, int32_t b) -> int64_t {
        if (a > b) std::swap(a, b);
        const int32_t* c0 = T.cols.data() + T.rowptr[a];
        const int32_t* c1 = T.cols.data() + T.rowptr[a + 1];
        return eid[(size_t)(std::lower_bound(c0, c1, b) - T.cols.data())];
    };
    T.dofs.resize((size_t)nt * 10);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < nt; ++k) {
        const int32_t* t = m.tets + 4 * k;
        int32_t* d = T.dofs.data() + 10 * k;
        for (int j = 0; j < 4; ++j) d[j] = t[j];
        for (int e = 0; e < 6; ++e)
            d[4 + e] = (int32_t)(nv + edge_of(t[kEdge[e][0]], t[kEdge[e][1]]));
    }
    // system node -> (element, local DOF), ascending element per node
    T.xp2t_ptr.assign((size_t)nn + 1, 0);
    for (int64_t q = 0; q < 10 * nt; ++q) T.xp2t_ptr[T.dofs[q] + 1]++;
    for (int64_t i = 0; i < nn; ++i) T.xp2t_ptr[i + 1] += T.xp2t_ptr[i];
    T.xp2t.resize((size_t)nt * 10);
    {
        std::vector<int32_t> fill(T.xp2t_ptr.begin(), T.xp2t_ptr.end() - 1);
        for (int64_t k = 0; k < nt; ++k)
            for (int j = 0; j < 10; ++j)
                T.xp2t[fill[T.dofs[10 * k + j]]++] = (uint32_t)((k << 4) | j);
    }
    // boundary edges: the edges of the triangles that belong to one element
    std::vector<uint8_t> ebnd((size_t)ne, 0);
    {
        static const int kFace[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < nt; ++k) {
            const int32_t* t = m.tets + 4 * k;
            for (int f = 0; f < 4; ++f) {
                const int32_t v[3] = {t[kFace[f][0]], t[kFace[f][1]], t[kFace[f][2]]};
                bool shared = false;
                for (int32_t q = T.p2t_ptr[v[0]]; q < T.p2t_ptr[v[0] + 1] && !shared; ++q) {
                    const int64_t k2 = T.p2t[q] >> 2;
                    if (k2 == k) continue;
                    const int32_t* t2 = m.tets + 4 * k2;
                    int hit = 0;
                    for (int j = 0; j < 4; ++j) hit += (t2[j] == v[1]) + (t2[j] == v[2]);
                    shared = hit == 2;
                }
                if (shared) continue;
                for (int a = 0; a < 3; ++a)
                    for (int b = a + 1; b < 3; ++b) {
                        const int64_t e = edge_of(v[a], v[b]);
#pragma omp atomic write
                        ebnd[e] = 1;
                    }
            }
        }
    }
    // extended graph: the DOFs of the node's elements, sorted unique
    std::vector<int32_t> cnt((size_t)nn);
    auto row = [&](int64_t i, std::vector<int32_t>& buf) {
        buf.clear();
        for (int32_t q = T.xp2t_ptr[i]; q < T.xp2t_ptr[i + 1]; ++q) {
            const int32_t* d = T.dofs.data() + 10 * (int64_t)(T.xp2t[q] >> 4);
            buf.insert(buf.end(), d, d + 10);
        }
        std::sort(buf.begin(), buf.end());
        buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
    };
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t i = 0; i < nn; ++i) {
            row(i, buf);
            cnt[i] = (int32_t)buf.size();
        }
    }
    std::vector<int32_t> rowptr((size_t)nn + 1, 0);
    int64_t acc = 0;
    int32_t maxr = 0;
    for (int64_t i = 0; i < nn; ++i) {
        rowptr[i] = (int32_t)acc;
        acc += cnt[i];
        maxr = std::max(maxr, cnt[i]);
    }
    if (acc >= (int64_t)1 << 31) {
        err = "mesh: P2 node graph too large for 32-bit block indices";
        return FTS_ERR_BAD_INPUT;
    }
    rowptr[nn] = (int32_t)acc;
    std::vector<int32_t> cols((size_t)acc), diag((size_t)nn);
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(dynamic, 4096)
        for (int64_t i = 0; i < nn; ++i) {
            row(i, buf);
            std::copy(buf.begin(), buf.end(), cols.begin() + rowptr[i]);
            diag[i] = rowptr[i] +
                      (int32_t)(std::lower_bound(buf.begin(), buf.end(), (int32_t)i) - buf.begin());
        }
    }
    T.rowptr.swap(rowptr);
    T.cols.swap(cols);
    T.diag.swap(diag);
    T.max_row = maxr;
    T.bnd.resize((size_t)nn);
    for (int64_t e = 0; e < ne; ++e) T.bnd[nv + e] = ebnd[e];
    // the vertex element lists stay; the edge nodes have none
    T.p2t_ptr.resize((size_t)nn + 1, T.p2t_ptr[nv]);
    int64_t nI = 0;
    for (int64_t i = 0; i < nn; ++i) nI += T.bnd[i] ? 0 : 1;
    T.n_interior = nI;
    T.vertex_lattice_n = T.lattice_n;
    T.nv = nv;
    T.ne = ne;
    T.np = nn;
    T.lattice_n = 0;
    T.kuhn_elements = false;
    return FTS_OK;
}

}  // namespace fts
