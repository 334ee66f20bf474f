// Seeded synthetic inputs: Kuhn lattice meshes, analytic level sets, Gaussian
// growth factors and viscosity laws.  Host only (OpenMP); declared in
// include/fts_gen.h.
#include "fts_gen.h"

#include <cmath>
#include <cstddef>
#include <cstdint>

namespace {

inline uint64_t mix64(uint64_t z) {
    // splitmix64 finaliser
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

inline double uniform01(uint64_t seed, uint64_t stream, uint64_t index) {
    uint64_t h = mix64(seed ^ mix64(stream * 0xD1B54A32D192ED03ull ^ mix64(index)));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);  // 53 bits
}

// The 6 Kuhn tetrahedra of a cube: the monotone lattice paths from corner
// (0,0,0) to (1,1,1), one per axis permutation.
const int kPerm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};

inline double sq(double v) { return v * v; }

}  // namespace

extern "C" {

double fts_gen_uniform(uint64_t seed, uint64_t stream, uint64_t index) {
    return uniform01(seed, stream, index);
}

int fts_gen_kuhn_counts(int32_t n, int64_t* np, int64_t* nt) {
    if (n < 2 || !np || !nt) return 1;
    int64_t m = n - 1;
    *np = (int64_t)n * n * n;
    *nt = 6 * m * m * m;
    return 0;
}

int fts_gen_kuhn_mesh(int32_t n, double jitter, uint64_t seed, float* xyz, int32_t* tets,
                      uint8_t* boundary) {
    if (n < 2 || !xyz || !tets) return 1;
    const int64_t nn = n;
    const int64_t np = nn * nn * nn;
    const double h = 1.0 / (double)(n - 1);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < np; ++v) {
        int64_t ijk[3] = {v % nn, (v / nn) % nn, v / (nn * nn)};
        bool onb = false;
        for (int a = 0; a < 3; ++a) {
            bool face = (ijk[a] == 0 || ijk[a] == nn - 1);
            onb = onb || face;
            double x = (double)ijk[a] * h;
            if (!face && jitter != 0.0) {
                double u = uniform01(seed, 1 + (uint64_t)a, (uint64_t)v);
                x += (2.0 * u - 1.0) * jitter * h;
            }
            xyz[3 * v + a] = (float)x;
        }
        if (boundary) boundary[v] = onb ? 1 : 0;
    }
    const int64_t m = nn - 1;
    const int64_t ncube = m * m * m;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < ncube; ++c) {
        int64_t ci = c % m, cj = (c / m) % m, ck = c / (m * m);
        for (int t = 0; t < 6; ++t) {
            int64_t p[3] = {ci, cj, ck};
            int32_t* out = tets + 4 * (6 * c + t);
            out[0] = (int32_t)(p[0] + nn * (p[1] + nn * p[2]));
            for (int s = 0; s < 2; ++s) {
                p[kPerm[t][s]] += 1;
                out[1 + s] = (int32_t)(p[0] + nn * (p[1] + nn * p[2]));
            }
            out[3] = (int32_t)((ci + 1) + nn * ((cj + 1) + nn * (ck + 1)));
        }
    }
    return 0;
}

double fts_gen_shape_phi(const fts_gen_shape* s, double x, double y, double z) {
    switch (s->kind) {
        case FTS_SHAPE_SPHERE:
            return std::sqrt(sq(x - s->center[0]) + sq(y - s->center[1]) + sq(z - s->center[2])) -
                   s->radius;
        case FTS_SHAPE_ELLIPSOID: {
            // k0 (k0 - 1) / k1 with k0 = |p/a|, k1 = |p/a^2|: exact sign, first-order
            // distance near the surface.
            double px = x - s->center[0], py = y - s->center[1], pz = z - s->center[2];
            double k0 = std::sqrt(sq(px / s->axes[0]) + sq(py / s->axes[1]) + sq(pz / s->axes[2]));
            double k1 = std::sqrt(sq(px / (s->axes[0] * s->axes[0])) +
                                  sq(py / (s->axes[1] * s->axes[1])) +
                                  sq(pz / (s->axes[2] * s->axes[2])));
            if (k1 == 0.0) return -std::fmin(s->axes[0], std::fmin(s->axes[1], s->axes[2]));
            return k0 * (k0 - 1.0) / k1;
        }
        case FTS_SHAPE_TWO_SPHERES: {
            double d1 = std::sqrt(sq(x - s->center[0]) + sq(y - s->center[1]) +
                                  sq(z - s->center[2])) - s->radius;
            double d2 = std::sqrt(sq(x - s->center2[0]) + sq(y - s->center2[1]) +
                                  sq(z - s->center2[2])) - s->radius2;
            return std::fmin(d1, d2);
        }
        default:
            return 0.0;
    }
}

int fts_gen_surface_points(const fts_gen_shape* s, int32_t m, uint64_t seed, double* pts) {
    if (!s || m < 0 || (m > 0 && !pts)) return 1;
    const double two_pi = 6.283185307179586476925286766559;
    for (int32_t k = 0; k < m; ++k) {
        for (int attempt = 0; attempt < 64; ++attempt) {
            uint64_t idx = (uint64_t)k * 64 + (uint64_t)attempt;
            double zc = 2.0 * uniform01(seed, 101, idx) - 1.0;
            double th = two_pi * uniform01(seed, 102, idx);
            double rr = std::sqrt(std::fmax(0.0, 1.0 - zc * zc));
            double d[3] = {rr * std::cos(th), rr * std::sin(th), zc};
            double p[3];
            if (s->kind == FTS_SHAPE_SPHERE) {
                for (int a = 0; a < 3; ++a) p[a] = s->center[a] + s->radius * d[a];
            } else if (s->kind == FTS_SHAPE_ELLIPSOID) {
                for (int a = 0; a < 3; ++a) p[a] = s->center[a] + s->axes[a] * d[a];
            } else {
                double w1 = s->radius * s->radius, w2 = s->radius2 * s->radius2;
                bool first = uniform01(seed, 103, idx) * (w1 + w2) < w1;
                const double* c = first ? s->center : s->center2;
                double r = first ? s->radius : s->radius2;
                for (int a = 0; a < 3; ++a) p[a] = c[a] + r * d[a];
                const double* co = first ? s->center2 : s->center;
                double ro = first ? s->radius2 : s->radius;
                double dist = std::sqrt(sq(p[0] - co[0]) + sq(p[1] - co[1]) + sq(p[2] - co[2]));
                if (dist < ro && attempt < 63) continue;  // buried inside the other sphere
            }
            for (int a = 0; a < 3; ++a) pts[3 * k + a] = p[a];
            break;
        }
    }
    return 0;
}

int fts_gen_fields(const fts_gen_shape* s, int64_t np, int64_t nt, const float* xyz,
                   const int32_t* tets, int32_t ncentres, const double* centres, double sigma,
                   double amp, double* phi_node, double* c_node, double* phi_elem,
                   double* c_elem) {
    if (!s || !xyz || np <= 0 || ncentres < 0 || sigma <= 0.0) return 1;
    const double inv2s2 = 1.0 / (2.0 * sigma * sigma);
    auto gf = [&](double x, double y, double z) {
        double acc = 0.0;
        for (int32_t k = 0; k < ncentres; ++k) {
            double r2 = sq(x - centres[3 * k]) + sq(y - centres[3 * k + 1]) +
                        sq(z - centres[3 * k + 2]);
            acc += amp * std::exp(-r2 * inv2s2);
        }
        return acc;
    };
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < np; ++v) {
        double x = xyz[3 * v], y = xyz[3 * v + 1], z = xyz[3 * v + 2];
        if (phi_node) phi_node[v] = fts_gen_shape_phi(s, x, y, z);
        if (c_node) c_node[v] = gf(x, y, z);
    }
    if ((phi_elem || c_elem) && tets && nt > 0) {
#pragma omp parallel for schedule(static)
        for (int64_t e = 0; e < nt; ++e) {
            double c[3] = {0.0, 0.0, 0.0};
            for (int j = 0; j < 4; ++j) {
                int64_t v = tets[4 * e + j];
                for (int a = 0; a < 3; ++a) c[a] += (double)xyz[3 * v + a];
            }
            for (int a = 0; a < 3; ++a) c[a] *= 0.25;
            if (phi_elem) phi_elem[e] = fts_gen_shape_phi(s, c[0], c[1], c[2]);
            if (c_elem) c_elem[e] = gf(c[0], c[1], c[2]);
        }
    }
    return 0;
}

int fts_gen_viscosity(int64_t nt, const double* phi_elem, const double* c_elem, int32_t law,
                      double p0, double p1, double p2, double* mu) {
    if (!mu || nt < 0) return 1;
    if (law == FTS_MU_BAND && (!phi_elem || p2 <= 0.0)) return 1;
    if (law == FTS_MU_INVERSE && !c_elem) return 1;
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < nt; ++e) {
        double m;
        if (law == FTS_MU_BAND) {
            double t = 0.5 - phi_elem[e] / p2;
            t = t < 0.0 ? 0.0 : (t > 1.0 ? 1.0 : t);
            m = p1 + (p0 - p1) * t;
        } else if (law == FTS_MU_INVERSE) {
            m = 1.0 / (p0 + c_elem[e]);
            m = m < p1 ? p1 : (m > p2 ? p2 : m);
        } else {
            m = p0;
        }
        mu[e] = m;
    }
    return 0;
}

}  // extern "C"
