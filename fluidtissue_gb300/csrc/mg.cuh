// Geometric multigrid hierarchy on Kuhn lattices (internal).
#pragma once

#include <cstdint>
#include <vector>

namespace fts {

struct Ctx;

constexpr int kSmooth = 2;        // Chebyshev degree of each pre / post smoothing
constexpr int kCoarse = 20;       // Chebyshev degree of the coarsest-level solve
constexpr int kPowerIters = 12;   // power iterations for lambda_max(D^-1 K)
constexpr double kLamSafety = 1.1;

template <typename T>
struct MGLevel {
    int n = 0;
    int64_t N = 0;
    T* K = nullptr;      // [15 directions][9 entries][N]
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
    std::vector<double> lam_host;
    bool built = false;
};

// Nodes per axis of the next coarser lattice.
inline int mg_coarse_n(int n) { return n % 2 ? (n + 1) / 2 : n / 2 + 1; }

template <typename T>
void mg_setup(Ctx& c, MG<T>& mg);
template <typename T>
void mg_vcycle(Ctx& c, MG<T>& mg, const int* stop);
template <typename T>
void mg_free(MG<T>& mg);

}  // namespace fts
