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
    return FTS_OK;
}

}  // namespace fts
