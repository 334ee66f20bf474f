// Internal declarations shared by the host setup code (setup.cpp) and the
// CUDA translation units.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fts.h"

namespace fts {

// Host-side mesh topology built once per context (Flow::init's share of
// Mesh3D: p2t, the node graph and the interior-dof flags).
struct HostTopology {
    int64_t np = 0, nt = 0;
    std::vector<int32_t> rowptr;   // [np+1] block rows of the node graph
    std::vector<int32_t> cols;     // [nnzb] sorted neighbour nodes incl. self
    std::vector<int32_t> diag;     // [np] position of (i,i) in cols
    std::vector<int32_t> p2t_ptr;  // [np+1]
    std::vector<uint32_t> p2t;     // [4 nt] (tet << 2 | local index), ascending tet per node
    std::vector<uint8_t> bnd;      // [np] 1 = Dirichlet velocity node
    int32_t max_row = 0;           // longest block row
    int32_t max_p2t = 0;           // most tetrahedra around one node
    int32_t lattice_n = 0;         // n if the mesh is the Kuhn lattice of n^3 nodes (index
                                   // i + n j + n^2 k, Kuhn node graph), else 0
    bool kuhn_elements = false;    // lattice with element 6c + t = the monotone path of axis
                                   // permutation t in cube c (the lattice generator's order)
    int64_t n_interior = 0;        // nI (interior velocity nodes of the system)
    // P2-P1 (velocity degree 2): the system nodes are the np' = nv + ne
    // vertices and edges (velocity at all, pressure at the vertices only);
    // rowptr / cols / diag / bnd describe the extended graph and p2t_ptr has
    // empty lists for the edge nodes.
    int64_t nv = 0;                // mesh vertices (== np for P1)
    int64_t ne = 0;                // edges (P2 only)
    std::vector<int32_t> dofs;     // [10 nt] element DOFs: 4 vertices, then the edges
                                   // 01 02 03 12 13 23 as nv + edge id (Tetrahedron.hpp:61)
    std::vector<int32_t> xp2t_ptr; // [np'+1] system node -> (tet << 4 | local DOF 0..9)
    std::vector<uint32_t> xp2t;
    int32_t vertex_lattice_n = 0;  // P2: n if the vertices form the Kuhn lattice of n^3
    std::vector<int32_t> edge_ends;  // P2: [2 ne] end vertices of edge e (lower first)
    std::vector<int32_t> vinc_ptr;   // P2: [nv+1] edges incident to each vertex
    std::vector<int32_t> vinc;       // P2: [2 ne]
};

// Validates the mesh and builds the topology (OpenMP).  Returns an fts_status.
int build_topology(const fts_mesh& m, HostTopology& T, std::string& err);
// Turns a P1 topology into the P2-P1 one (edges numbered by their lower
// vertex's sorted neighbour list; boundary edges = edges of the boundary
// triangles, Mesh3D::initDofs, TetraMesh.cpp:219-290).
int extend_p2(const fts_mesh& m, HostTopology& T, std::string& err);

// Exterior-boundary nodes: nodes of the triangles that belong to exactly one
// tetrahedron (TetraMesh.cpp:266-269).
void boundary_from_faces(const fts_mesh& m, const HostTopology& T, std::vector<uint8_t>& bnd);

// Reference-element constants (float-rounded basis table at the 4-point rule,
// Quadrature.hpp:24-36, :102-112; Tetrahedron.hpp:17-18, :27-51):
//   wq[b]     = sum_q 0.25 phi_b(q)             (so that int psi_b = vol * wq[b])
//   mref[a][b] = sum_q 0.25 phi_a(q) phi_b(q)    (so that M_ab = vol * mref[a][b])
struct RefConstants {
    double wq[4];
    double mref[4][4];
    double phi[4][4];  // the float-rounded basis table phi[a][q]
};
RefConstants ref_constants();

// P2-P1 reference integrals (bilin_without_p2t_ij, Assembler.hpp:321-424): the
// rule of degree deg_i + deg_j (Quadrature.hpp:37-56), the P2 / P1 basis and
// gradient tables float-rounded as Tetrahedron.hpp:56-115 evaluates them, the
// weights as written.  With G = invB^T and vol = |det B| / 6:
//   int mu (grad phi_a)_m' (grad phi_b)_n' = mu vol sum_mn G_m'm G_n'n K[a][b][m][n]
//   int (grad phi_a)_r psi_k            = vol sum_m G_rm B[a][k][m]
//   int phi_a psi_k                     = vol N[a][k]
struct RefP2 {
    double K[10][10][3][3];  // sum_q w_q dphi_a/dxi_m dphi_b/dxi_n   (degree 4, 20 points)
    double B[10][4][3];      // sum_q w_q dphi_a/dxi_m psi_k          (degree 3, 10 points)
    double N[10][4];         // sum_q w_q phi_a psi_k                 (degree 3, 10 points)
};
RefP2 ref_p2();

double wall_ms();

}  // namespace fts
