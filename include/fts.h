/*
 * fts.h — C ABI of libfts.so, the GB300-native variable-viscosity P1-P1
 * Stokes solve of fluidtissue (one Stokes step of the growth loop).
 *
 * It replaces the C++ class Flow (src/growth/Flow.hpp:15-63):
 *   Flow::init(const LevelSet&, const Parameters&)   -> fts_create
 *   Flow::solve(const LevelSet&, const VecXd&, VecXd&) -> fts_solve
 *   Flow::~Flow                                       -> fts_destroy
 * The same inputs go in — the tetrahedral mesh (Mesh3D::p float xyz, Mesh3D::t),
 * the nodal level set phi (LevelSet::getPhi), the nodal growth factor "source"
 * (growth.cpp:73-76) — and the same output comes out: flow[4*np] =
 * [ux(np), uy(np), uz(np), p(np)] with zero velocity on the exterior boundary
 * (Flow.cpp:290-300).
 *
 * Plain pointers and sizes only; no exceptions cross the boundary; every call
 * returns an fts_status.  A context is not re-entrant; distinct contexts may be
 * used from distinct host threads.  All work of a context runs on one GPU
 * (fts_params.device) and on one CUDA stream (fts_set_stream).
 */
#ifndef FTS_H
#define FTS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference returns 0 / -1 (Flow.cpp:84, :281-285); the
 * non-zero codes here refine its -1. */
typedef enum fts_status {
    FTS_OK = 0,
    FTS_ERR_BAD_INPUT = 1,          /* null pointer, size or index out of range, unsupported option */
    FTS_ERR_DEGENERATE_ELEMENT = 2, /* a tetrahedron with det B == 0 (Assembler.hpp:446-457) */
    FTS_ERR_NOT_CONVERGED = 3,      /* the solver stopped above the tolerance (Flow.cpp:281-285) */
    FTS_ERR_CUDA = 4,               /* a CUDA runtime call failed */
    FTS_ERR_OOM = 5,                /* device allocation failed */
    FTS_ERR_UNSUPPORTED = 6,        /* a reference option outside this path (P2; surface tension
                                       without its load) */
    FTS_ERR_NAN = 7,                /* NaN or Inf in the inputs or in the iteration */
    FTS_ERR_TIMEOUT = 8             /* a grid-barrier wait of a persistent launch ran out (a
                                       block did not arrive); the launch returned */
} fts_status;

/* Arithmetic of the solve. */
enum {
    FTS_PREC_FP64 = 0,  /* FP64 assembly, SpMV, Krylov (parity path) */
    FTS_PREC_MIXED = 1  /* FP32 inner Krylov (SpMV, preconditioner, vector updates) with an
                           FP64 outer refinement loop (residual, solution update, dot products) */
};

/* Krylov method. */
enum {
    FTS_SOLVER_MINRES = 0,   /* preconditioned MINRES on the symmetric form (default) */
    FTS_SOLVER_BICGSTAB = 1  /* un-preconditioned BiCGSTAB on the reference's form, as Flow.hpp:62 */
};

/* Preconditioner of MINRES: blockdiag(velocity part, pressure part) plus the
 * rank-one term of the constant pressure mode. */
enum {
    FTS_PC_AUTO = 0,           /* FTS_PC_MULTIGRID when the mesh is a Kuhn lattice that
                                  allows it, else FTS_PC_JACOBI */
    FTS_PC_JACOBI = 1,         /* velocity: node 3x3 block Jacobi; pressure: inverse of the
                                  diagonal of (alpha D + eps M) + lumped 1/mu mass (any mesh) */
    FTS_PC_MULTIGRID = 2,      /* velocity: geometric multigrid V-cycle; pressure: scalar
                                  multigrid V-cycle of (alpha D + eps M) + lumped 1/mu mass,
                                  run concurrently (Kuhn lattices only; batched solves use
                                  the pressure diagonal) */
    FTS_PC_MULTIGRID_DIAG = 3  /* velocity V-cycle, pressure diagonal as in FTS_PC_JACOBI */
};

/* Operator representation. */
enum {
    FTS_OP_AUTO = 0,       /* FTS_OP_STENCIL on Kuhn lattices, else FTS_OP_ASSEMBLED */
    FTS_OP_ASSEMBLED = 1,  /* node-blocked 4x4 BSR, assembled every solve; the FP32 inner
                              solve reads a sliced-ELL copy */
    FTS_OP_MATFREE = 2,    /* element-by-element operator for the FP32 inner solve */
    FTS_OP_STENCIL = 3     /* assembled BSR; the FP32 inner solve reads a symmetric half
                              stencil (self + 7 positive Kuhn directions, 8 blocks per
                              node) of it.  Kuhn lattices only. */
};

/* Mesh3D (src/fem/TetraMesh.hpp:49-62).  The library copies what it needs
 * during fts_create and keeps no pointer. */
typedef struct fts_mesh {
    int64_t np;               /* nodes */
    int64_t nt;               /* tetrahedra */
    const float* xyz;         /* [3*np] node coordinates x,y,z per node (Mesh3D::p, Vec3f) */
    const int32_t* tets;      /* [4*nt] node indices per tetrahedron (Mesh3D::t) */
    const uint8_t* boundary;  /* [np] nullable: 1 = node on an exterior boundary triangle.
                                 NULL: derived from the triangles that belong to exactly one
                                 tetrahedron (TetraMesh.cpp:266-269). */
} fts_mesh;

/* The Parameters keys the Stokes step reads (Flow.cpp:23, :77-82, :105,
 * :199, :223-228, :359-372; ViscosityProfiles.hpp:32-59), plus GB300 options.
 * Start from fts_params_default(). */
typedef struct fts_params {
    int32_t velocity_degree;    /* "Stokes velocity degree": 1 (P1-P1 stabilised) */
    double alpha;               /* "alpha": Brezzi-Pitkaranta weight of h^2 (grad p, grad q) */
    double eps;                 /* "eps": pressure mass regularisation */
    double tol;                 /* "Stokes tolerance": stop at ||b - A x|| <= tol ||b|| */
    int32_t max_iter;           /* "Max. CG iterations" (<= 0: 2 N as Eigen's default) */
    double mu_interior;         /* "Viscosity interior" */
    double mu_exterior;         /* "Viscosity exterior" */
    int32_t mu_profile;         /* "Viscosity profile": 0 INVERSE, 1 DIRECT, 2 DIRECT_RATE4X */
    double gf_growth;           /* "GF growth" */
    double level_sink;          /* "Level sink" */
    double growth_threshold;    /* "Growth threshold" */
    double rd_iterations;       /* "RD iterations" (selects maxGF and the early exit) */
    double gf_production;       /* "GF production" */
    double advection_dt;        /* "Advection dt" (< FLT_MIN: nothing to solve) */
    double surface_tension;     /* "Surface tension": > 0 needs the load from
                                   fts_ls_surface_tension in fts_solve's force */
    /* GB300 options */
    int32_t precision;          /* FTS_PREC_* */
    int32_t solver;             /* FTS_SOLVER_* */
    int32_t preconditioner;     /* FTS_PC_* */
    int32_t operator_kind;      /* FTS_OP_* */
    int32_t warm_start;         /* 1: start from the previous solution (USE_INITIAL_GUESS,
                                   Flow.cpp:15); 0: start from zero */
    int32_t device;             /* CUDA device ordinal */
    double inner_tol;           /* mixed precision: smallest relative reduction asked of
                                   each FP32 inner solve (<= 0: default 1e-5 for P1
                                   systems of >= 100,000 nodes and for batches, else
                                   1e-4) */
    int32_t verbose;            /* 1: print the reference's progress lines to stdout */
    int32_t time_kernels;       /* 1: bracket every operator application of the Krylov
                                   loop with CUDA events (fills fts_stats.ms_spmv) */
} fts_params;

/* Per-solve statistics (the quantities Flow.cpp prints, plus timings). */
typedef struct fts_stats {
    int32_t status;            /* fts_status of the call */
    int32_t solved;            /* 0 when an early exit left flow untouched (Flow.cpp:223-251) */
    int64_t iterations;        /* Krylov iterations, all precisions (Flow.cpp:270) */
    int64_t iterations_fp32;   /* of which in the FP32 inner solver */
    int32_t outer_iterations;  /* FP64 residual recomputations */
    double rel_residual;       /* true ||b - A x|| / ||b|| in FP64 at return */
    double error_estimate;     /* the solver's own estimate (Flow.cpp:271) */
    double mu_min, mu_max;     /* over interior elements (Flow.cpp:241) */
    double f_norm;             /* ||F|| (Flow.cpp:248) */
    double ms_assembly;        /* device time of viscosity, source, RHS and matrix assembly */
    double ms_solve;           /* device time of the Krylov solve */
    double ms_total;           /* wall time of the call */
    int64_t device_bytes;      /* device memory held by the context */
    int64_t kernel_launches;   /* kernels this library launched during the call */
    int64_t spmv_launches;     /* operator applications inside the Krylov loop */
    double ms_spmv;            /* their summed CUDA-event time (time_kernels = 1) */
    double spmv_bytes;         /* algorithmic bytes of one such application */
    double spmv_bytes_fp64;    /* the same for the FP64 operator */
} fts_stats;

typedef struct fts_ctx fts_ctx;

/* Defaults: P1, alpha 0.032, eps 1e-3, tol 1e-4 (parameters/summary.txt),
 * profile INVERSE with equal viscosities, FP64, MINRES, AUTO preconditioner and
 * operator, warm start on, device 0. */
void fts_params_default(fts_params* p);

/* Flow::init (src/growth/Flow.cpp:20-85): validates and uploads the mesh,
 * builds the dof map, the block sparsity pattern and the per-element geometry.
 * Returns FTS_ERR_DEGENERATE_ELEMENT if any tetrahedron is flat. */
int fts_create(const fts_mesh* mesh, const fts_params* params, fts_ctx** out);

/* Flow::solve (src/growth/Flow.cpp:89-94, :218-302) with host arrays:
 *   phi[np]    level set (interior = phi < 0, LevelSet.cpp:180-211)
 *   source[np] growth factor (or activator)
 *   mu[nt]     nullable: per-element viscosity; NULL = setViscosity's profile
 *              (ViscosityProfiles.hpp:27-72)
 *   force[3*np] nullable: nodal body force [fx(np), fy(np), fz(np)] (the
 *              surface-tension load slot of Flow.cpp:352-363, computed by
 *              fts_ls_surface_tension); required when "Surface tension" > 0
 *              (FTS_ERR_UNSUPPORTED without it)
 *   flow[4*np] output [ux, uy, uz, p]; left untouched by the early exits
 *   stats      nullable
 * The inputs are copied to the device, the system is assembled and solved on
 * the GPU and the result copied back; the call returns when flow is filled. */
int fts_solve(fts_ctx* ctx, const double* phi, const double* source, const double* mu,
              const double* force, double* flow, fts_stats* stats);

/* The same with device pointers (no host copies); flow may be device memory. */
int fts_solve_device(fts_ctx* ctx, const double* phi, const double* source, const double* mu,
                     const double* force, double* flow, fts_stats* stats);

/* Stream for all subsequent work of ctx (a cudaStream_t; NULL = the context's
 * own stream). */
int fts_set_stream(fts_ctx* ctx, void* stream);

/* Replace the solver options of an existing context (precision, solver,
 * preconditioner, tolerances, warm start); the mesh stays. */
int fts_update_params(fts_ctx* ctx, const fts_params* params);

/* Reset the warm-start vector (Flow::up_, Flow.cpp:47-48) to zero. */
int fts_reset_guess(fts_ctx* ctx);

/* Frees all device and host memory of ctx. */
void fts_destroy(fts_ctx* ctx);

/* Human-readable text of a status code. */
const char* fts_status_string(int status);

/* Last error message recorded on ctx (empty if none). */
const char* fts_last_error(const fts_ctx* ctx);

/* ---- inspection (tests and profiling) ---------------------------------- */

/* Sizes of the assembled node-block system: np, block nonzeros, and the
 * reference's reduced dimension N = 3 nI + np (Flow.cpp:35-44). */
int fts_get_sizes(const fts_ctx* ctx, int64_t* np, int64_t* nnzb, int64_t* n_reduced);

/* Copies the last assembled FP64 block matrix to host arrays: rowptr[np+1],
 * cols[nnzb], vals[16*nnzb] (row-major 4x4 per block over ux,uy,uz,p, in the
 * symmetric sign convention: pressure rows negated; boundary velocity rows and
 * columns replaced by identity / zero), rhs[4*np] (same convention). */
int fts_get_system(const fts_ctx* ctx, int32_t* rowptr, int32_t* cols, double* vals, double* rhs);

/* Applies the assembled operator: y = S x on host vectors of length 4*np,
 * node-interleaved (ux,uy,uz,p per node); precision FTS_PREC_FP64 or
 * FTS_PREC_MIXED (the FP32 copy). */
int fts_apply(fts_ctx* ctx, int32_t precision, const double* x, double* y);

/* ---- batched solves ------------------------------------------------------ */

/* Many independent Stokes solves (own mesh, viscosity and parameters each)
 * solved together: per-instance assembly, then the MINRES iteration of all
 * instances in one persistent cooperative launch with per-instance
 * convergence masks, the outer FP64 loop on the device, the sequence captured
 * as a CUDA graph.  Block-Jacobi + rank-one preconditioner (any mesh).  Each
 * instance is a Flow::solve (src/growth/Flow.cpp:89) of its own inputs. */
typedef struct fts_batch fts_batch;

/* Launch shape of the persistent kernel, chosen by the autotuner on the first
 * solve (threads per block, rows per work chunk, threads per block row = the
 * SpMV work split, co-resident blocks) and its measured time per sweep. */
typedef struct fts_batch_config {
    int32_t threads;
    int32_t chunk_rows;
    int32_t tpr;
    int32_t blocks;
    double ms_per_sweep;
    int32_t graph;  /* 1 when the outer loop runs as a captured CUDA graph */
    int32_t spmv_format;  /* operator storage of the Krylov SpMV phase: FTS_BATCH_BSR, or
                             FTS_BATCH_LATTICE (the FP32 lattice half stencil on Kuhn-lattice
                             instances, BSR on the others; mixed precision) */
} fts_batch_config;

enum { FTS_BATCH_BSR = 0, FTS_BATCH_LATTICE = 1 };

/* count instances; meshes[count], params[count] (same precision and device). */
int fts_batch_create(int32_t count, const fts_mesh* meshes, const fts_params* params,
                     fts_batch** out);
/* phi[i], source[i], flow[i] per instance (host); mu (nullable array) per
 * instance nullable; stats[count] (nullable).  Returns the first non-OK
 * instance status. */
int fts_batch_solve(fts_batch* b, const double* const* phi, const double* const* source,
                    const double* const* mu, double* const* flow, fts_stats* stats);
/* The same with device pointers. */
int fts_batch_solve_device(fts_batch* b, const double* const* phi, const double* const* source,
                           const double* const* mu, double* const* flow, fts_stats* stats);
int fts_batch_get_config(const fts_batch* b, fts_batch_config* cfg);
int fts_batch_set_stream(fts_batch* b, void* stream);
/* No counterpart in the reference (its solves are host code).  The longest
 * wait of any block at a grid barrier of the persistent launch (default 2 s);
 * when it runs out the launch records the error, every block returns and
 * fts_batch_solve reports FTS_ERR_TIMEOUT with the context still usable.
 * absent_block >= 0 is for failure-detection tests: that block of every later
 * persistent launch leaves at its first barrier without arriving, so the
 * others' waits run out (-1: none). */
int fts_batch_set_barrier_limit(fts_batch* b, double seconds, int32_t absent_block);
const char* fts_batch_last_error(const fts_batch* b);
void fts_batch_destroy(fts_batch* b);

/* ---- allocation-free residual ------------------------------------------- */

/* Largest system (block rows = nodes) fts_bsr_residual_noalloc accepts: its
 * reduction scratch is a fixed static device array of 256 KB. */
#define FTS_NOALLOC_MAX_NODES 1048576

/* No counterpart in the reference: an addition for callers that cannot
 * allocate device memory — applications that own all of the GPU's memory
 * through their own arena, or loops that must not stall on the device
 * synchronisation cudaMalloc / cudaFree can cause.  It computes the FP64
 * residual of a node-blocked system in the layout fts_get_system returns,
 * r = b - S x, with norms[0] = ||r||^2 and norms[1] = ||b||^2, and allocates
 * nothing: rowptr[np+1], cols[nnzb], vals[16*nnzb], x[4*np], b[4*np] (inputs)
 * and r[4*np], norms[2] (outputs) are device memory owned by the caller; the
 * reduction scratch is a static device array (every GPU that loads the library
 * holds it until exit).  np must be <= FTS_NOALLOC_MAX_NODES, else
 * FTS_ERR_BAD_INPUT.  Runs on `stream` (a cudaStream_t; NULL = the legacy
 * default stream) of the current device and returns without waiting for it.
 * Every call looks up the scratch array's device address in the current
 * context (nothing is cached, so the address stays right after a
 * cudaDeviceReset); the first call on a device also loads the library's module
 * there and should come before any stream capture.  Calls share the array:
 * calls whose kernels overlap on the GPU (different streams, not ordered)
 * race and their norms are wrong, so serialise them on one stream. */
int fts_bsr_residual_noalloc(int64_t np, const int32_t* rowptr, const int32_t* cols,
                             const double* vals, const double* x, const double* b, double* r,
                             double* norms, void* stream);

/* ------------------------------------------------------------------------
 * Reaction-diffusion: activator / inhibitor patterning and the growth factor,
 * replacing RD::solve (src/growth/RD.hpp:16-56, RD.cpp:27-108).  The system
 * lives on the interior submesh (nodes with phi < 0, elements with four such
 * nodes; LevelSet.cpp:180-211) with the lumped-mass Laplacian
 * L = diag(1 / rowsum M) K (RD.cpp:116-172, Assembler.cpp:75-84) and is
 * advanced by `iterations` explicit Euler steps of length dt (RD.cpp:74-92):
 *   u' = u + dt (-Da L u + Act u^2 / (1 + Inh v + GFinh g) - DegA u)
 *   v' = v + dt (-Di L v + u^2 - DegI v)       (only while u or v is non-zero)
 *   g' = g + dt (-GFdiff L g - GFdeg g),  g' = GF production on source nodes
 * All arithmetic FP64; all steps run in one persistent launch.
 * ------------------------------------------------------------------------ */
typedef struct fts_rd_params {
    double dt;                /* "RD dt" */
    int64_t iterations;       /* "RD iterations" */
    double act, da, dega;     /* "Act", "Da", "DegA" */
    double inh, di, degi;     /* "Inh", "Di", "DegI" */
    double gf_production;     /* "GF production" */
    double gf_diffusion;      /* "GF diffusion" */
    double gf_degradation;    /* "GF degradation" */
    double gf_inhibition;     /* "GF inhibition" */
} fts_rd_params;

typedef struct fts_rd_stats {
    int32_t status;
    int32_t alive;            /* activator / inhibitor were advanced (RD.cpp:60-62) */
    int64_t interior_nodes;
    int64_t interior_elements;
    int64_t steps;
    double ms_setup;          /* interior sets, Laplacian assembly, uploads */
    double ms_steps;          /* the Euler steps (device time) */
    double ms_total;          /* wall time of the call */
    int64_t kernel_launches;
} fts_rd_stats;

typedef struct fts_rd fts_rd;

/* RD's mesh (Mesh3D of the level set, RD.cpp:123-147) on `device`.  Returns
 * FTS_ERR_DEGENERATE_ELEMENT for a flat tetrahedron. */
int fts_rd_create(const fts_mesh* mesh, int32_t device, fts_rd** out);
/* RD::solve: activator, inhibitor, growth_factor [np] are the state (in/out,
 * host memory), phi [np] the level set, source_nodes the growth-factor
 * sources (Knots::getSourceNodes, global node indices; every one must be an
 * interior node, else FTS_ERR_BAD_INPUT).  iterations == 0 or dt < FLT_MIN
 * returns at once with the state untouched (RD.cpp:31-33); otherwise every
 * non-interior node of the three fields is zero on return (RD.cpp:94-102). */
int fts_rd_solve(fts_rd* rd, const fts_rd_params* params, const double* phi,
                 const int32_t* source_nodes, int32_t n_sources, double* activator,
                 double* inhibitor, double* growth_factor, fts_rd_stats* stats);
void fts_rd_destroy(fts_rd* rd);
const char* fts_rd_last_error(const fts_rd* rd);

/* ------------------------------------------------------------------------
 * Distance reset of the level set, replacing EuclideanDistance
 * (src/fem/EuclideanDistance.hpp:13-51, EuclideanDistance.cu:45-118): for
 * every mesh node p_k, phi_n[k] = min_j |ifp_j - p_k| over the interface
 * points (float, each distance from norm3df as in the reference's kernel),
 * negated where the old phi_n[k] < 0.  With no interface point the minimum is
 * FLT_MAX, as in the reference.
 *   FTS_DIST_PRUNED: the points binned on the device along a Morton curve of
 *     a 64^3 grid over their box, in blocks of 32 with bounding boxes; each
 *     node scans only the blocks that can hold its nearest point, and
 *     candidates within rounding of the minimum are re-evaluated with
 *     norm3df, so the result equals the exhaustive minimum.
 *   FTS_DIST_EXHAUSTIVE: the reference's algorithm (every node against every
 *     point), for comparison.
 * ------------------------------------------------------------------------ */
enum { FTS_DIST_PRUNED = 0, FTS_DIST_EXHAUSTIVE = 1 };

typedef struct fts_dist_stats {
    int32_t status;
    int32_t blocks;           /* point blocks */
    int64_t points_scanned;   /* point distances evaluated (all nodes) */
    double ms_setup;          /* uploads and the device binning of the points */
    double ms_kernel;         /* device time of the search kernel */
    double ms_total;
} fts_dist_stats;

typedef struct fts_dist fts_dist;

/* EuclideanDistance::init: node positions xyz[3 np] (float) on `device`. */
int fts_dist_create(const float* xyz, int64_t np, int32_t device, fts_dist** out);
/* EuclideanDistance::resetPhi: ifp[3 n_ifp] (float), phi_n[np] in/out (host). */
int fts_dist_reset(fts_dist* d, const float* ifp, int32_t n_ifp, double* phi_n, int32_t method,
                   fts_dist_stats* stats);
void fts_dist_destroy(fts_dist* d);
const char* fts_dist_last_error(const fts_dist* d);

/* ------------------------------------------------------------------------
 * Level-set update, replacing LevelSet::update (src/fem/LevelSet.cpp:89-151)
 * with its distance reset resetPhi_ (:429-455; the interface triangulation
 * and normals it also builds are not part of phi and are not computed):
 *   Crank-Nicolson advection (M + dt/2 A) phi' = (M - dt/2 A) phi with the
 *   nodal velocity of `flow` (A(i,j) = int (V . grad phi_j) phi_i), Jacobi-
 *   preconditioned BiCGSTAB from phi to ||r|| <= tol ||b|| (Eigen's algorithm,
 *   LevelSet.hpp:145), then (reset != 0) the distance reset to the edge
 *   crossings of the advected zero level set, the crossing edges' nodes keeping
 *   the advected value, and phi = 0.75 phi_kept + 0.25 phi_reset.
 * dt < FLT_MIN or ||flow|| < FLT_MIN: returns at once, phi untouched.  A NaN
 * velocity is FTS_ERR_NAN and an unconverged solve FTS_ERR_NOT_CONVERGED, phi
 * untouched (LevelSet.cpp:111-114, :135-139).  All arithmetic FP64.
 * ------------------------------------------------------------------------ */
typedef struct fts_ls_params {
    double dt;                /* "Advection dt" */
    double tol;               /* "Advection tolerance" (<= 0: machine epsilon) */
    int64_t max_iter;         /* "Max. CG iterations" (<= 0: 2 np) */
    int32_t reset;            /* 1: distance reset after the advection (the reference) */
} fts_ls_params;

typedef struct fts_ls_stats {
    int32_t status;
    int64_t iterations;       /* BiCGSTAB iterations (Eigen's count) */
    double error;             /* ||r|| / ||b|| at the stop */
    int64_t interface_points;
    double ms_assembly, ms_solve, ms_reset, ms_total;
    int64_t kernel_launches;
} fts_ls_stats;

typedef struct fts_ls fts_ls;

/* LevelSet's mesh on `device`; assembles the P1 mass matrix once
 * (LevelSet.cpp:33-37).  FTS_ERR_DEGENERATE_ELEMENT for a flat tetrahedron. */
int fts_ls_create(const fts_mesh* mesh, int32_t device, fts_ls** out);
/* flow[4 np] = [ux, uy, uz, p] (Flow::solve's output), phi[np] in/out (host). */
int fts_ls_update(fts_ls* ls, const fts_ls_params* params, const double* flow, double* phi,
                  fts_ls_stats* stats);
void fts_ls_destroy(fts_ls* ls);
const char* fts_ls_last_error(const fts_ls* ls);

/* The last update's full distance-reset values (LevelSet::phi_ifn_,
 * LevelSet.cpp:440, before the 0.75 / 0.25 mixing), host [np].
 * FTS_ERR_BAD_INPUT before any update with reset = 1. */
int fts_ls_reset_values(const fts_ls* ls, double* phi_reset);

/* The full distance reset of phi (LevelSet::resetPhi_, LevelSet.cpp:429-441:
 * phi_ifn_ before the crossing nodes keep their values): every node's signed
 * distance to the edge crossings of phi's zero level set (LevelSet.cpp:278-300),
 * sign from phi.  phi[np] in, phi_reset[np] out (host); the values also become
 * this context's reset values (fts_ls_surface_tension with phi_reset = NULL).
 * After LevelSet::update the crossing edges and their end values are those
 * the update's reset used, so this reproduces the level set's phi_ifn_ from
 * its phi alone. */
int fts_ls_distance_reset(fts_ls* ls, const double* phi, double* phi_reset);

/* ---------------------------------------------------------------------------
 * Surface tension: Flow::surfaceTension_ (src/growth/Flow.cpp:307-341) with the
 * LevelSet quantities it reads — normals = nodal gradient of phi_reset
 * (LevelSet.cpp:453, Assembler.cpp:46-69), curvature div(n/|n|) at the nodes
 * interpolated to the interface points (LevelSet.cpp:215-253), interface
 * points and the area of their interface-triangle patches (LevelSet.cpp:261-300,
 * :326-420).  The result is the nodal load `force` that fts_solve takes
 * (Flow.cpp:356-363, 392-395: F += N fx ...): pass it there with "Surface
 * tension" > 0.
 * ------------------------------------------------------------------------- */
typedef struct fts_st_stats {
    int32_t status;
    int64_t interface_points;  /* edges whose end values differ in sign bit */
    double area;               /* total area of the interface triangles */
    double ms_kernels;         /* device time */
    double ms_total;           /* wall time of the call */
    int64_t kernel_launches;
} fts_st_stats;

/* phi[np]: the current level set; phi_reset[np]: the last full reset values
 * (NULL: this context's from its last fts_ls_update with reset = 1);
 * surface_tension: "Surface tension"; node_density: "Node density" (the
 * reference's integer rho); force[3 np] out = [fx(np), fy(np), fz(np)]. */
int fts_ls_surface_tension(fts_ls* ls, const double* phi, const double* phi_reset,
                           double surface_tension, int32_t node_density, double* force,
                           fts_st_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* FTS_H */
