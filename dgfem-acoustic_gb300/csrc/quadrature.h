// Quadrature rules of the curved-element path (host, FP64).
//
// The reference integrates every element and face with Gmsh's "Gauss(2p)"
// rules (src/Mesh.cpp:49-52, :213-215). Gmsh is not available here; these are
// the published rules of the same degrees that stand in for them, with a
// fixed point order: the first points of a face rule matter to the reference's
// recipe (the normal sign at the first point, the 3-D tangent frame from the
// first three points, Mesh.cpp:284-308, :316-364).
//   line        [-1, 1]:                   Gauss-Legendre, n points, ascending
//   triangle    (0,0), (1,0), (0,1):       Dunavant, degrees 1..8
//   tetrahedron (0,0,0), (1,0,0), ...:     4-point (deg 2), Keast 11 (deg 4),
//                                          Keast 24 (deg 6), Stroud conical
//                                          product 5x5x5 (deg 8, 9)
// On straight-sided elements every rule of sufficient degree gives the same
// operators; only curved elements depend on the choice.
#pragma once
#include <vector>

namespace dgref {

struct QRule {
  int n = 0, dim = 0;
  std::vector<double> x;  // n * dim reference coordinates
  std::vector<double> w;  // n weights
};

QRule gauss_legendre(int n);
QRule triangle_rule(int degree);
QRule tetrahedron_rule(int degree);

// The reference's rules for an order-p simplex: element rule of degree 2p;
// face rule: Gauss-Legendre with p + 1 points on [-1, 1] (2-D), the degree-2p
// triangle rule (3-D).
QRule element_rule(int dim, int p);
QRule face_rule(int dim, int p);

}  // namespace dgref
