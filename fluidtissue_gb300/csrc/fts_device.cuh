// Device-side context and kernel interfaces of libfts (internal).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "fts.h"
#include "fts_internal.h"
#include "mg.cuh"
#include "p2mg.cuh"
#include "pmg.cuh"

struct fts_ctx;

namespace fts {

#define FTS_CUDA(call)                                                        \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) {                                              \
            throw ::fts::CudaError(e_, #call, __FILE__, __LINE__);            \
        }                                                                     \
    } while (0)

struct CudaError {
    cudaError_t code;
    std::string what;
    CudaError(cudaError_t c, const char* call, const char* file, int line)
        : code(c),
          what(std::string(call) + ": " + cudaGetErrorString(c) + " (" + file + ":" +
               std::to_string(line) + ")") {}
};

// Blocks per SM used for grid-stride kernels; grids are multiples of the SM
// count so every SM gets the same share.
constexpr int kThreads = 256;
constexpr int kMaxPartials = 4096;

// Mixed precision: the smallest relative reduction asked of one FP32 inner
// MINRES run (the parameter inner_tol overrides it).  Deeper inner runs mean
// fewer outer passes and restarts: 1e-5 for P1 systems of at least 100,000
// nodes and for batches (measured: 129^3 122 -> 116 iterations, 257^3 141 ->
// 139, 65^3 99 -> 99 with the set-up of one pass less, batch96 358 -> 325
// mean), 1e-4 for smaller systems and P2-P1 (17^3: 365 at 1e-4 against 436
// at 1e-5; P2-P1 33^3: 211 against 231).
constexpr double kInnerTolFloorLarge = 1e-5;
constexpr double kInnerTolFloorSmall = 1e-4;
constexpr int64_t kInnerTolLargeNodes = 100000;

// Node-interleaved vector element: (ux, uy, uz, p).
template <typename T>
struct alignas(4 * sizeof(T)) V4 {
    T x, y, z, w;
};

// Per-element geometry, 16 doubles (128 B): gradients of the 4 P1 basis
// functions (invB^T * ghat_j, Assembler.hpp:163-168), the element volume
// detB/6, and (float)h^2 with h = (float)cbrt(detB) (Assembler.hpp:193,
// Flow.cpp:195).
struct alignas(128) ElemGeom {
    double g[4][3];
    double vol;
    double hh;
    double pad[2];
};

// Unscaled Schur-complement weight of node v: the lumped 1/mu-weighted mass,
// sum over the node's elements of vol_e / (4 mu_e) (the caller multiplies by
// schur_scale).
__device__ __forceinline__ double lumped_inv_mu(int64_t v, const int32_t* __restrict__ p2t_ptr,
                                                const uint32_t* __restrict__ p2t,
                                                const ElemGeom* __restrict__ geom,
                                                const double* __restrict__ mu) {
    double w = 0.0;
    for (int32_t q = p2t_ptr[v]; q < p2t_ptr[v + 1]; ++q) {
        const int64_t k = p2t[q] >> 2;
        w += geom[k].vol / (4.0 * mu[k]);
    }
    return w;
}

// FP64 lattice half stencil (Kuhn lattices, mixed precision): entries
// (r, 2h) and (r, 2h + 1) of node v's 4x4 block towards direction d (0 = self,
// 1..7 positive Kuhn directions) as one double2; tiles of 32 nodes, so a
// warp's access to one (d, r, h) is 512 contiguous bytes; 1 KB per node.
__host__ __device__ __forceinline__ int64_t lat64_idx(int d, int r, int h, int64_t v) {
    return ((v >> 5) * 64 + d * 8 + r * 2 + h) * 32 + (v & 31);
}

// Scalar state of one MINRES run (Paige & Saunders 1975), kept on the device
// so that the iteration never waits on the host.
struct MinresScalars {
    double beta1, beta, oldb, alfa, dbar, epsln, oldeps, delta, gamma, phi, phibar, cs, sn;
    double target;
    double rtol;      // requested reduction of the preconditioned residual norm
    double crank;    // rank-one constant-pressure weight 1/(eps * volume)
    double ycorr[2]; // pressure shift of Y[0] / Y[1] (rank-one part of P^-1)
    double psum;     // sum of the pressure components of the Lanczos vector
    double pdot;     // its pressure part of n . P^-1 n (diagonal term)
    long long iters;
    long long maxit;
    int stop;
    int c_pending;
    int status;  // 0 running/converged, 1 max iterations, 2 NaN
    int pad;
};

// Scalars of the FP64 outer loop.
struct OuterScalars {
    double rr;     // ||b - S x||^2
    double bb;     // ||b||^2
    double scale;  // 1 / ||r|| used to normalise the FP32 inner right-hand side
    double sum;    // scratch reduction (source mean)
    double mu_min, mu_max;          // over the interior elements (Flow.cpp:241)
    double mu_all_min, mu_all_max;  // over every element (the Schur weight's scale)
    int nonfinite;
    int pad;
};

// Scale s of every Schur-complement estimate of the preconditioner (pressure
// weights, the pressure multigrid's fine operator): Kp = alpha D + eps M +
// s * lumped 1/mu mass.  The viscous term is 2 mu eps(u) : eps(v), so with
// constant viscosity B K^-1 B^T is about M / (2 mu): s = 1/2.  With viscosity
// contrast the weighted mass overestimates the Schur complement (the stiff
// side of an interface carries its nodes), and s falls with the contrast C =
// max mu / min mu over the elements: s = 1/2 / (1 + 1.5 log10 C), which
// matches the measured optimum of a uniform s on constant viscosity (1/2) and
// on contrast 200 (about 1/8).
#ifndef FTS_SCHUR_SCALE
#define FTS_SCHUR_SCALE 0.5
#endif
#ifndef FTS_SCHUR_CONTRAST
#define FTS_SCHUR_CONTRAST 1.5
#endif
__device__ __forceinline__ double schur_scale(const OuterScalars* os) {
    const double lo = os->mu_all_min, hi = os->mu_all_max;
    const double lc = (lo > 0.0 && hi > lo) ? log10(hi / lo) : 0.0;
    return FTS_SCHUR_SCALE / (1.0 + FTS_SCHUR_CONTRAST * lc);
}

struct Reduction {
    double* partials;   // [kMaxPartials * 4]
    unsigned* ticket;   // [1]
};

// Krylov work vectors of one precision (node-interleaved V4<T>, np each).
template <typename T>
struct KrylovWork {
    V4<T>* q = nullptr;
    V4<T>* R[2] = {nullptr, nullptr};
    V4<T>* Y[2] = {nullptr, nullptr};
    V4<T>* W[2] = {nullptr, nullptr};
    V4<T>* X = nullptr;  // correction accumulated by the inner solve
    V4<T>* r0 = nullptr; // right-hand side of the inner solve
};

struct Ctx {
    fts_params par{};
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    HostTopology topo;
    int64_t np = 0, nt = 0, nnzb = 0;  // np: system nodes (block rows)
    int64_t nv = 0;                    // mesh vertices (== np for P1-P1)
    bool p2 = false;                   // P2-P1: edges are system nodes too
    int32_t* dofs = nullptr;           // P2: [10 nt] element DOFs
    int32_t* xp2t_ptr = nullptr;       // P2: system node -> (element, local DOF)
    uint32_t* xp2t = nullptr;
    int num_sms = 148;
    std::string last_error;

    // mesh
    float* xyz = nullptr;
    int32_t* tets = nullptr;
    uint8_t* bnd = nullptr;
    int32_t* rowptr = nullptr;
    int32_t* cols = nullptr;
    int32_t* diag = nullptr;
    int32_t* p2t_ptr = nullptr;
    uint32_t* p2t = nullptr;
    ElemGeom* geom = nullptr;

    // per-solve inputs (device staging)
    double* phi = nullptr;
    double* src = nullptr;
    double* force = nullptr;
    double* mu = nullptr;
    double* s = nullptr;
    double* flow = nullptr;

    // system
    double* A64 = nullptr;
    float* A32 = nullptr;     // FP32 BSR copy (batch instances)
    // FP32 sliced-ELL copy (single solves): slices of 8 block rows; the k-th
    // blocks of a slice are contiguous (8 x 64 B), padding points at node 0
    // with zero values
    float* ell_val = nullptr;   // [slots * 16]
    int32_t* ell_col = nullptr; // [slots]
    int32_t* ell_ptr = nullptr; // [nslices + 1] first slot of each slice
    int64_t nslices = 0, ell_slots = 0;
    bool use_ell = false;
    // FP32 lattice half stencil (Kuhn lattices): per node the blocks to itself
    // and its 7 positive-direction neighbours, in tiles of 32 nodes x 128
    // values; the other 7 blocks are the neighbours' blocks transposed
    float* lat_val = nullptr;   // [ceil(np / 32) * 128 * 32]
    int32_t* lat_src = nullptr; // [ceil(np / 32) * 32 * 8] BSR block of (v, v + d) or -1
    bool use_lat = false;
    // FP64 half stencil of the same layout family (lat64_idx), assembled
    // straight from the elements in mixed precision on Kuhn lattices; the BSR
    // A64 is then assembled only when a caller asks for it (a64_valid)
    double2* lat64 = nullptr;
    bool use_lat64 = false;
    bool a64_valid = false;
    bool in_batch = false;
    double* pc64 = nullptr;   // 8 per node: inverse of the 3x3 velocity block (xx,xy,xz,yy,yz,zz),
    float* pc32 = nullptr;    // inverse pressure weight, pad
    V4<double>* b = nullptr;
    V4<double>* x = nullptr;
    V4<double>* r = nullptr;
    KrylovWork<double> w64;
    KrylovWork<float> w32;
    bool have32 = false;

    // scalars / reductions
    MinresScalars* ms = nullptr;
    MinresScalars* ms_host = nullptr;   // pinned
    OuterScalars* os = nullptr;
    OuterScalars* os_host = nullptr;    // pinned
    Reduction red{};
    int* err_flag = nullptr;
    double* bicg = nullptr;              // scalars of the reference-algorithm BiCGSTAB
    int bicg_restarts = 0;

    // operator representation: false = assembled BSR, true = element gather
    bool matfree = false;
    float* mf_rec = nullptr;   // FP32 element records of the matrix-free operator
    float* mf_cube = nullptr;  // matrix-free FP32 partial sums: per cube (lattice form) or
                               // per element row (record form)
    double* mf_rows = nullptr; // per-element rows of the FP64 matrix-free residual (16 per element)

    // preconditioner
    bool use_mg = false;
    MG<double> mg64;
    MG<float> mg32;
    P2MG<double> p2mg64;  // P2-P1: the P2 velocity level above the vertex hierarchy
    P2MG<float> p2mg32;
    // pressure-block V-cycle (Kuhn lattices with the velocity multigrid): runs
    // on aux_stream between the events ev_fork and ev_join of each application
    bool use_pmg = false;
    PMG<double> pmg64;
    PMG<float> pmg32;
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double volume = 0.0;  // sum of element volumes
    double crank = 0.0;   // 1 / (eps * volume), 0 when eps = 0

    // learned ratio between true and preconditioned residual reductions
    double pc_ratio64 = 10.0;
    double pc_ratio32 = 10.0;
    bool matrix_valid = false;

    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    int64_t device_bytes = 0;

    // launch accounting and optional per-application event timing of the
    // Krylov loop's operator kernel
    int64_t launches = 0;
    int64_t spmv_runs = 0;
    double ms_spmv = 0.0;
    static constexpr int kTimedPairs = 32;
    cudaEvent_t tev[2 * kTimedPairs] = {};
    bool tev_ready = false;
};

// ---- context lifecycle (api.cu) -------------------------------------------
void create(Ctx& c, const fts_mesh& m, const fts_params& p);   // throws CudaError / int
int create_context(const fts_mesh* mesh, const fts_params* params, fts_ctx** out, bool in_batch);
void free_all(Ctx& c);
int validate_params(const fts_params& p, std::string& err);
void ensure_fp32(Ctx& c);
void ensure_fp64_work(Ctx& c);
void build_lattice(Ctx& c);         // lattice half-stencil map and FP32 storage

// ---- assembly (assemble.cu) -----------------------------------------------
void launch_geometry(Ctx& c, int* bad);
void launch_viscosity_profile(Ctx& c);
void launch_mu_minmax(Ctx& c);
void launch_source(Ctx& c);
void launch_rhs(Ctx& c, bool have_force);
void launch_assemble(Ctx& c);       // FP64 BSR (allocated on first use)
void launch_to_lat(Ctx& c);         // FP32 lattice half stencil from the FP64 BSR
void launch_assemble_lat(Ctx& c);   // FP64 + FP32 lattice half stencils
void launch_assemble_p2(Ctx& c);    // P2-P1 FP64 BSR over vertices + edges (p2.cu)
void launch_rhs_p2(Ctx& c, bool have_force);
void ensure_bsr64(Ctx& c);          // BSR of the current system for callers that read it
void launch_preconditioner(Ctx& c);
void launch_to_f32(Ctx& c);
void launch_scatter_flow(Ctx& c, double* flow_out);
void launch_check_finite(Ctx& c, const double* a, int64_t n);
void launch_any_abs_above(Ctx& c, const double* a, int64_t n, double thr);

// ---- Krylov (krylov.cu) ------------------------------------------------------
// r = b - S x (FP64) and ||r||^2, ||b||^2 into c.os
void launch_residual64(Ctx& c);
// inner MINRES on S d = r0 in precision T; returns the number of iterations
template <typename T>
long long minres_inner(Ctx& c, double rtol, long long maxit, double* achieved, int* status);
void launch_prepare_inner32(Ctx& c);       // r0_32 = r * scale
void launch_update_x64(Ctx& c);            // x += d (FP64 inner)
void launch_update_x_from32(Ctx& c);       // x += d32 / scale
void launch_apply(Ctx& c, int precision, const V4<double>* in, V4<double>* out);
// matrix-free operator (matfree.cu)
void launch_mf_minres_A(Ctx& c, const V4<float>* Y, int ybuf, const V4<float>* R1, V4<float>* q);
void launch_mf_residual64(Ctx& c);
void launch_mf_pc(Ctx& c);
// the reference's un-preconditioned BiCGSTAB on c.x (bicgstab.cu)
long long bicgstab_solve(Ctx& c, double tol, long long maxit, double* err, int* status);
template <typename T>
void setup_preconditioner(Ctx& c);   // multigrid hierarchy when c.use_mg

template <typename T>
inline T* dev_alloc(Ctx& c, size_t n) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n * sizeof(T) + 16);
    if (e != cudaSuccess) throw CudaError(e, "cudaMalloc", __FILE__, __LINE__);
    c.device_bytes += (int64_t)(n * sizeof(T));
    return static_cast<T*>(p);
}

// Programmatic dependent launch: a kernel started by pdl_launch may be
// scheduled while the previous kernel of its stream drains (its launch and
// block start-up overlap the predecessor's tail).  Every such kernel calls
// pdl_wait() before it touches global memory; the wait returns once the
// predecessor has completed and its writes are visible (and at once for a
// kernel launched without the attribute).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void pdl_launch(void (*kern)(KArgs...), int grid, int block, cudaStream_t s,
                       Args&&... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3((unsigned)block);
    lc.dynamicSmemBytes = 0;
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    FTS_CUDA(cudaLaunchKernelEx(&lc, kern, static_cast<KArgs>(args)...));
}

inline int grid_for(const Ctx& c, int64_t work, int threads = kThreads, int per_sm = 8) {
    int64_t need = (work + threads - 1) / threads;
    int64_t cap = (int64_t)c.num_sms * per_sm;
    if (need < 1) need = 1;
    return (int)(need < cap ? need : cap);
}

}  // namespace fts

struct fts_ctx {
    fts::Ctx c;
};
