// Geometric multigrid hierarchy on Kuhn lattices (internal).
#pragma once

#include <cuda_fp16.h>

#include <cstdint>
#include <vector>

namespace fts {

struct Ctx;

constexpr int kSmooth = 2;        // Chebyshev degree of each pre / post smoothing
// The first kDeg1Levels levels (below the cluster tail) smooth with Chebyshev
// degree 1 instead of kSmooth: damped Jacobi with the level's 1/theta, one
// stencil pass before and one after the coarse correction instead of two; on
// the finest level the caller's final update is then pointwise.
#ifndef FTS_DEG1_LEVELS
#define FTS_DEG1_LEVELS 1
#endif
constexpr int kDeg1Levels = FTS_DEG1_LEVELS;
constexpr int kCoarse = 20;       // Chebyshev degree of the coarsest-level solve
constexpr int kPowerIters = 12;   // power iterations for lambda_max(D^-1 K)
constexpr double kLamSafety = 1.1;
constexpr int kCoefStride = 64;   // per level: 1/theta, then (ca_s, cb_s) for s >= 1
constexpr int kMaxMGLevels = 10;  // levels of one hierarchy (n <= 513)
// Levels with at most this many nodes run in one cluster launch (FP32 / FP64:
// a cluster has a tenth of the GPU's SMs, which the FP64 FMA rate feels first).
template <typename T>
constexpr int64_t tail_nodes() { return sizeof(T) == 4 ? 5000 : 1000; }

// Storage of the smoothing operator: the FP32 hierarchy keeps its stencils in
// FP16 (scaled per level by max|K| / 16384; arithmetic stays FP32), the FP64
// hierarchy in FP64.
template <typename T>
struct MGStore;
template <>
struct MGStore<float> {
    using type = __half;
};
template <>
struct MGStore<double> {
    using type = double;
};

template <typename T>
struct MGLevel {
    using KS = typename MGStore<T>::type;
    int n = 0;
    int64_t N = 0;
    T* K = nullptr;      // half stencil in T (Galerkin construction), tiles of 32 nodes x 72
    KS* Kh = nullptr;    // the stencil the V-cycle reads (== K when KS is T)
    T* Di = nullptr;     // [6][N] inverse 3x3 node blocks (xx xy xz yy yz zz)
    T* b = nullptr;      // [3][N] right-hand side
    T* x = nullptr;      // [3][N] solution
    T* r = nullptr;      // [3][N] residual
    T* d0 = nullptr;     // [3][N] Chebyshev directions
    T* d1 = nullptr;
    uint8_t* mask = nullptr;  // Dirichlet nodes
};

template <typename T>
struct MG {
    std::vector<MGLevel<T>> L;
    double* lam = nullptr;           // device: lambda_max per level (with safety factor)
    double* coef = nullptr;          // device: Chebyshev coefficients per level
    double* scale = nullptr;         // device: stencil scale per level (Kh * scale = K)
    unsigned* maxbits = nullptr;     // device: max |K| per level (float bits)
    T* gal_self = nullptr;           // device: partial self blocks of a Galerkin product
    std::vector<double> lam_host;
    bool built = false;
    // levels tail_level.. of every V-cycle run in one launch of a single
    // cluster of tail_blocks CTAs (cluster barriers between phases); -1: none
    int tail_level = -1;
    int tail_blocks = 0;
};

// Level l smooths with degree 1 (kDeg1Levels) unless it is the coarsest or
// part of the cluster tail (small levels keep kSmooth).
template <typename T>
inline bool mg_level_degree1(const MG<T>& mg, size_t l) {
    return (int)l < kDeg1Levels && (mg.tail_level < 0 || (int)l < mg.tail_level) &&
           l + 1 < mg.L.size();
}

// Chebyshev coefficients of one level for lambda_max = lam: 1/theta, then
// (ca_s, cb_s) for s >= 1 (kCoefStride values).
void cheb_table(double lam, double* out);

// Nodes per axis of the next coarser lattice.
inline int mg_coarse_n(int n) { return n % 2 ? (n + 1) / 2 : n / 2 + 1; }

// Nodes per axis of every level, finest first (coarsening stops below 5).
inline std::vector<int> mg_chain(int n) {
    std::vector<int> out;
    while (true) {
        out.push_back(n);
        if (n < 5) break;
        n = mg_coarse_n(n);
    }
    return out;
}

// Term table of the Galerkin product P^T K P on Kuhn lattices: for coarse
// direction dJ, terms start[dJ]..start[dJ+1]-1 of (a | e << 4, weight): the
// fine node f = 2I + off[a] and its direction e.
void galerkin_terms(std::vector<int>& start, std::vector<unsigned short>& term,
                    std::vector<float>& w);

template <typename T>
void mg_setup(Ctx& c, MG<T>& mg);
// V-cycle on mg.L[0].b, whose first Chebyshev direction L[0].d0 the caller has
// written.  skip_final: 0 runs the whole cycle; kSkipFinal leaves out the last
// post-smoothing step of the finest level (on a degree-1 finest level the
// update x + d_0), which the caller then runs fused with its own epilogue;
// kSkipPost on a degree-1 finest level also leaves out the post-smoothing
// residual (b - K x and its d_0), so the caller's epilogue starts from the
// prolongated x (elsewhere it acts as kSkipFinal).
enum : int { kSkipFinal = 1, kSkipPost = 2 };
template <typename T>
void mg_vcycle(Ctx& c, MG<T>& mg, const int* stop, int skip_final);
template <typename T>
void mg_free(MG<T>& mg);

}  // namespace fts
