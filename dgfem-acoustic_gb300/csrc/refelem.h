// Reference-element operators of the nodal DG scheme (host, FP64).
//
// The reference evaluates its operators per element with Gmsh quadrature
// (src/Mesh.cpp:691-751, :761-839). On straight-sided (affine) elements these
// reduce exactly to shared reference operators scaled by per-element
// geometry; this module builds them once, by exact integration of monomials
// on the reference simplex:
//   M_ref[i][j]   = int phi_i phi_j                (mass, Mesh.cpp:708-724)
//   K_r[i][j]     = int d_r(phi_i) phi_j           (weak stiffness, Mesh.cpp:734-751)
//   Dt_r          = M_ref^-1 K_r                   (volume operator per reference direction)
//   Mf[m][n]      = int_face psi_m psi_n           (face mass, Mesh.cpp:800-810)
//   LIFT_f        = M_ref^-1 E_f Mf                (face flux -> element nodes, Mesh.cpp:822-839)
// Node sets are equispaced Lagrange lattices (Gmsh's Lagrange nodes for
// orders 1..4). The solver's internal node order is the lattice order below;
// element corners keep the mesh's corner order.
#pragma once
#include <cstdint>
#include <vector>

namespace dgref {

constexpr int kMaxP = 4;

struct RefElement {
  int dim = 0, p = 0;
  int np = 0;   // nodes per element
  int nf = 0;   // faces per element
  int nfp = 0;  // nodes per face
  // lattice coordinates (i,j[,k]) of internal node n, ξ = lattice / p
  std::vector<int> lattice;  // np * dim
  // fmask[f][m]: internal node index of face node m of local face f
  std::vector<int> fmask;  // nf * nfp
  // face corner tables (Gmsh local face conventions)
  int face_corners[4][3] = {};
  // nbrnode[(lf*nperm + perm)*nfp + m]: neighbour-local node matching face node m
  int nperm = 0;
  std::vector<int> nbrnode;
  // permutation table: perm_table[perm][k] = position in the neighbour face of our corner k
  int perm_table[6][3] = {};
  // operators, row-major
  std::vector<double> Mref, Minv;  // np x np
  std::vector<double> Dt;          // dim x np x np  (Dt[r][i][j])
  std::vector<double> Mf;          // nfp x nfp
  std::vector<double> LIFT;        // np x (nf*nfp)
  double ref_measure = 0.0;        // reference element measure (1/2 or 1/6)
  double face_ref_measure = 0.0;   // reference face measure (1 or 1/2)
};

RefElement build(int dim, int p);

// Tables of the curved-element path, which follows the reference's own
// quadrature formulation element by element (src/Mesh.cpp:40-137 element
// Jacobians at the quadrature points, :209-260 face points, :691-839 mass,
// stiffness and face integrals). Internal node order; the face points of
// local face lf are the face rule's points mapped through that face's corner
// order (face_corners[lf]).
struct CurvedTables {
  int ng = 0, ngf = 0;
  std::vector<double> qw;   // [ng] element rule weights
  std::vector<double> qB;   // [ng][np] phi_j at the element points
  std::vector<double> qD;   // [dim][ng][np] d phi_j / d xi_r at the element points
  std::vector<double> fw;   // [ngf] face rule weights
  std::vector<double> fB;   // [nf][ngf][nfp] phi of face node m at the face points
  std::vector<double> fTu;  // [nf][ngf][np] d phi_j / du along the face parametrization
  std::vector<double> fTv;  // [nf][ngf][np] d phi_j / dv (3-D; empty in 2-D)
};
CurvedTables build_curved(const RefElement& re);

// Internal node index of lattice point (i,j[,k]); -1 if outside.
int lattice_index(const RefElement& re, const int* ijk);

// First three barycentric points of the degree-2p face rule that the
// reference's recipe reads (first point: normal sign; first three: 3-D
// tangent frame, Mesh.cpp:284-308,316-364). Values follow the oracle's rule
// (the reference's Gmsh rule is not available).
void face_rule_head(int p, double bary[3][3]);

// Sign of the recipe's normal relative to the right-hand normal of the face's
// corner order (+1 or -1): product of the derivative factors of the first two
// face vertex basis functions at the first face quadrature point.
int recipe_normal_sign(int dim, int p);

}  // namespace dgref
