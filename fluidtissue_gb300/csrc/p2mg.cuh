// P2 -> P1 multigrid level for the Taylor-Hood (P2-P1) solve (internal).
//
// The velocity preconditioner of a P2-P1 system on a Kuhn lattice is a V-cycle
// whose finest level is the P2 velocity space (vertices and edge midpoints,
// the system's own nodes) and whose coarser levels are the P1 lattice
// hierarchy of mg.cu on the vertices.  Transfer: P e = e at a vertex and the
// mean of the two end values at an edge (exact interpolation of P1 fields in
// P2); restriction is P^T; the P1 finest operator is the Galerkin product
// P^T K2 P, which on a Kuhn lattice keeps the 15-point stencil of the P1
// hierarchy.  The P2 level smooths with degree-1 Chebyshev (damped 3x3 block
// Jacobi on [lambda / 10, lambda]), before and after the coarse correction;
// the update after it is the pointwise stage 2 of MINRES.
#pragma once

#include <cstdint>

namespace fts {

struct Ctx;

template <typename T>
struct P2MG {
    bool built = false;
    T* K = nullptr;            // [9 nnzb] velocity 3x3 part of every block of the system
    T* Di = nullptr;           // [6][nn] inverse diagonal 3x3 blocks
    T* b = nullptr;            // [3][nn] right-hand side
    T* x = nullptr;            // [3][nn]
    T* r = nullptr;            // [3][nn]
    T* d0 = nullptr;           // [3][nn] first Chebyshev direction
    T* d1 = nullptr;           // [3][nn] power-iteration buffer
    double* coef = nullptr;    // device: 1/theta, (ca_s, cb_s)
    double* lam = nullptr;     // device: lambda_max estimate
    int32_t* edge_ends = nullptr;  // [2 ne] end vertices of every edge
    int32_t* vinc_ptr = nullptr;   // [nv + 1] edges incident to each vertex
    int32_t* vinc = nullptr;       // [2 ne]
    double lam_host = 0.0;
};

// Per-solve set-up after the P2 assembly: velocity blocks, D^-1 and
// lambda_max of the P2 level (the P1 hierarchy then takes its finest operator
// from p2mg_galerkin).
template <typename T>
void p2mg_setup(Ctx& c);
// The P1 hierarchy's finest operator P^T K2 P into the level's half stencil
// (kidx layout) with the Dirichlet vertices as identity rows.
template <typename T>
void p2mg_galerkin(Ctx& c, T* K1, const uint8_t* mask1, int n1);
// One V-cycle on the P2 level's right-hand side b (whose d_0 the caller has
// written): pre-smoothing, restriction, the P1 V-cycle, prolongation and the
// post-smoothing residual with its d_0; the caller adds d_0 to x (stage 2).
template <typename T>
void p2mg_vcycle(Ctx& c, const int* stop);
template <typename T>
void p2mg_free(P2MG<T>& m);

}  // namespace fts
