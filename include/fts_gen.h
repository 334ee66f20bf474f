/*
 * fts_gen.h — seeded synthetic inputs for the variable-viscosity Stokes solve.
 *
 * The reference builds its mesh by CGAL Delaunay of a node lattice
 * (src/fem/TetraMesh.cpp:23-165, :169-212) and gets phi, the growth factor and
 * the viscosity from the level-set / reaction-diffusion / viscosity-profile
 * modules (src/fem/LevelSet.cpp, src/growth/RD.cpp,
 * src/growth/ViscosityProfiles.hpp:27-72). None of those is on the Stokes path,
 * so these host-only helpers stand in for them: a Kuhn-split n^3 lattice on the
 * unit cube (float coordinates, as Mesh3D stores them: TetraMesh.hpp Vec3f),
 * analytic level sets, Gaussian growth factors centred on the interface and
 * pointwise viscosity laws. One generator feeds the oracle, the CUDA path, the
 * tests and the benchmark, so every consumer sees identical arrays.
 *
 * Everything here is deterministic for a given seed (a counter-based hash, no
 * global RNG state) and runs on the host with OpenMP. No GPU is touched.
 */
#ifndef FTS_GEN_H
#define FTS_GEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Node and tetrahedron counts of the Kuhn-split lattice with n nodes per axis:
 * np = n^3, nt = 6 (n-1)^3. Returns 0, or 1 for n < 2. */
int fts_gen_kuhn_counts(int32_t n, int64_t* np, int64_t* nt);

/* Kuhn-split lattice of [0,1]^3 with n nodes per axis.
 * Node (i,j,k) has index i + n*j + n*n*k and sits at (i,j,k)/(n-1), moved by a
 * uniform jitter in [-jitter*h, +jitter*h] (h = 1/(n-1)) along every axis in
 * which it is not on a cube face (so the cube faces stay planar and the hull is
 * still the cube). Each lattice cube is split into the 6 tetrahedra that share
 * its main diagonal. xyz: float[3*np]; tets: int32[4*nt];
 * boundary (nullable): uint8[np], 1 for nodes on the cube faces. */
int fts_gen_kuhn_mesh(int32_t n, double jitter, uint64_t seed,
                      float* xyz, int32_t* tets, uint8_t* boundary);

/* Analytic level sets (negative inside). */
enum {
    FTS_SHAPE_SPHERE = 0,      /* |x - c| - r */
    FTS_SHAPE_ELLIPSOID = 1,   /* first-order distance estimate to an axis-aligned ellipsoid */
    FTS_SHAPE_TWO_SPHERES = 2  /* min of two sphere distances (union) */
};

typedef struct fts_gen_shape {
    int32_t kind;
    double center[3];   /* sphere / ellipsoid centre; first sphere for TWO_SPHERES */
    double radius;      /* sphere radius; first radius for TWO_SPHERES */
    double axes[3];     /* ellipsoid semi-axes */
    double center2[3];  /* second sphere centre (TWO_SPHERES) */
    double radius2;     /* second sphere radius (TWO_SPHERES) */
} fts_gen_shape;

/* Level-set value at one point. */
double fts_gen_shape_phi(const fts_gen_shape* s, double x, double y, double z);

/* m seeded points on the zero level set (uniform direction on the unit sphere,
 * mapped onto the shape; for TWO_SPHERES the sphere is picked with probability
 * proportional to its area and points that fall inside the other sphere are
 * redrawn). pts: double[3*m]. */
int fts_gen_surface_points(const fts_gen_shape* s, int32_t m, uint64_t seed, double* pts);

/* Nodal and element-centroid fields.
 * phi_node[np], c_node[np]: level set and growth factor at nodes.
 * phi_elem[nt], c_elem[nt] (nullable): the same at element centroids (mean of
 * the 4 float node coordinates). Growth factor
 * c(x) = sum_k amp * exp(-|x - centre_k|^2 / (2 sigma^2)). */
int fts_gen_fields(const fts_gen_shape* s, int64_t np, int64_t nt,
                   const float* xyz, const int32_t* tets,
                   int32_t ncentres, const double* centres, double sigma, double amp,
                   double* phi_node, double* c_node, double* phi_elem, double* c_elem);

/* Pointwise viscosity laws evaluated per element.
 *  FTS_MU_BAND:     mu = mu_out + (mu_in - mu_out) * t,
 *                   t = clamp(0.5 - phi/band, 0, 1)   (p0 = mu_in, p1 = mu_out, p2 = band width)
 *  FTS_MU_INVERSE:  mu = clamp(1/(p0 + c), p1, p2)
 *  FTS_MU_CONSTANT: mu = p0 */
enum { FTS_MU_BAND = 0, FTS_MU_INVERSE = 1, FTS_MU_CONSTANT = 2 };
int fts_gen_viscosity(int64_t nt, const double* phi_elem, const double* c_elem,
                      int32_t law, double p0, double p1, double p2, double* mu);

/* Uniform double in [0,1) from (seed, stream, index); the same hash the
 * generator uses internally, exported so that workload parameters drawn in
 * host code share it. */
double fts_gen_uniform(uint64_t seed, uint64_t stream, uint64_t index);

#ifdef __cplusplus
}
#endif

#endif /* FTS_GEN_H */
