// Scalar multigrid for the pressure block of the Stokes preconditioner
// (internal).  The operator is  Kp = (alpha D + eps M) + diag(w),  the
// stabilisation block of the system plus the lumped 1/mu-weighted mass
// w_i = sum_{e ni i} vol_e / (4 mu_e), an SPD approximation of the Schur
// complement B K^-1 B^T + alpha D + eps M.  One V-cycle of Kp replaces the
// diagonal weight 1 / Kp_ii; the rank-one term for the constant pressure mode
// stays as it is.
//
// Hierarchy: the lattices of the velocity multigrid (same prolongation, same
// Galerkin term tables), no Dirichlet nodes: for even n the last coarse layer
// is a coarse node beyond the fine boundary, tied to the last fine layer by
// the weight 1/2 of its Kuhn edges.  Per level a scalar half stencil SoA
// K[d][N] (d = 0 self, 1..7 the positive Kuhn directions; the entry towards
// -e of node v is K[e][v - e]), the inverse diagonal, and the V-cycle vectors.
// Chebyshev smoothing of degree kPSmooth in D^-1 Kp on [kPLowFrac lambda, lambda] with
// lambda the Gershgorin bound max_i sum_j |Kp_ij| / Kp_ii of each level: an
// upper bound of the spectrum, so every smoother is convergent and the
// V-cycle is SPD whatever the coefficients.  Coarsest level (3^3 or 4^3
// nodes): exact, a dense inverse computed on the host in FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "mg.cuh"

namespace fts {

constexpr int kPSmooth = 2;          // Chebyshev degree of each pressure pre / post smoothing
#ifndef FTS_PMG_LOW_FRAC
#define FTS_PMG_LOW_FRAC 0.1
#endif
constexpr double kPLowFrac = FTS_PMG_LOW_FRAC;  // lower end of the smoothing interval / lambda

// Levels with at most this many nodes run in one launch of a single CTA.
constexpr int64_t kPTailNodes = 1000;
constexpr int kPTailThreads = 512;

template <typename T>
struct PLevel {
    int n = 0;
    int64_t N = 0;
    T* K = nullptr;   // [8][N] half stencil
    T* Di = nullptr;  // [N] 1 / K_ii
    T* b = nullptr;
    T* x = nullptr;
    T* r = nullptr;
    T* d0 = nullptr;
    T* d1 = nullptr;
};

template <typename T>
struct PMG {
    std::vector<PLevel<T>> L;
    double* coef = nullptr;              // device: Chebyshev coefficients per level
    unsigned long long* gersh = nullptr; // device: Gershgorin bound per level (double bits)
    T* cinv = nullptr;                   // device: dense inverse of the coarsest operator
    std::vector<double> lam_host;
    int tail_level = -1;                 // first level run by the single-CTA tail launch
    bool built = false;
    unsigned long long* h_gbits = nullptr;  // pinned: Gershgorin bounds per level
    T* h_kc = nullptr;                      // pinned: coarsest half stencil
    cudaEvent_t ev_copied = nullptr;        // both copied to the host
};

// The first kPDeg1Levels levels of the pressure hierarchy smooth with degree 1
// (as kDeg1Levels for the velocity hierarchy); level l does unless it is the
// coarsest or part of the single-CTA tail.
#ifndef FTS_PDEG1_LEVELS
#define FTS_PDEG1_LEVELS 1
#endif
constexpr int kPDeg1Levels = FTS_PDEG1_LEVELS;
template <typename T>
inline bool pmg_level_degree1(const PMG<T>& pm, size_t l) {
    return (int)l < kPDeg1Levels && (pm.tail_level < 0 || (int)l < pm.tail_level) &&
           l + 1 < pm.L.size();
}

// One level as the kernels see it.
template <typename T>
struct PView {
    int n;
    int64_t N;
    const T* K;
    const T* Di;
    T* b;
    T* x;
    T* r;
    T* d0;
    T* d1;
    const double* coef;
};

template <typename T>
inline PView<T> pview(const PMG<T>& pm, size_t l) {
    const PLevel<T>& L = pm.L[l];
    return PView<T>{L.n, L.N, L.K, L.Di, L.b, L.x, L.r, L.d0, L.d1, pm.coef + l * kCoefStride};
}

template <typename T>
void pmg_setup(Ctx& c, PMG<T>& pm);
// The same in two halves, so that the kernels can run on another stream while
// the caller enqueues other work: pmg_build (allocations, on c.stream), then
// pmg_setup_enqueue on stream st, then pmg_setup_finish (waits for st).
template <typename T>
void pmg_build(Ctx& c, PMG<T>& pm);
template <typename T>
void pmg_setup_enqueue(Ctx& c, PMG<T>& pm, cudaStream_t st);
template <typename T>
void pmg_setup_finish(Ctx& c, PMG<T>& pm, cudaStream_t st);
// V-cycle on pm.L[0].b on `stream`, whose first Chebyshev direction the
// caller has written; skip_final as for the velocity V-cycle.
template <typename T>
void pmg_vcycle(Ctx& c, PMG<T>& pm, cudaStream_t stream, const int* stop, bool skip_final);
template <typename T>
void pmg_free(PMG<T>& pm);

}  // namespace fts
