// refcpu — CPU restatement of the reference solver numerics (test oracle and
// timed CPU baseline; see refcpu.h for scope). Built with -O3 -fopenmp
// -ffp-contract=off so that x86 and Arm hosts give identical results.
#include "refcpu.h"

#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Dense helpers (the reference calls Eigen: src/utils.cpp:384-448)
// ---------------------------------------------------------------------------

// Solve A x = b in place (A row-major n x n, copied), partial pivoting like
// Eigen's PartialPivLU used by eigen::solve (src/utils.cpp:384-389).
void lu_solve(std::vector<double> A, double* b, int n) {
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(A[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > best) best = std::fabs(A[i * n + k]), p = i;
    if (best == 0.0) throw std::runtime_error("singular matrix in lu_solve");
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[p * n + j]);
      std::swap(b[k], b[p]);
    }
    for (int i = k + 1; i < n; ++i) {
      double l = A[i * n + k] / A[k * n + k];
      A[i * n + k] = l;
      for (int j = k + 1; j < n; ++j) A[i * n + j] -= l * A[k * n + j];
      b[i] -= l * b[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= A[i * n + j] * b[j];
    b[i] = s / A[i * n + i];
  }
}

// General inverse in place (src/utils.cpp:391-396: Eigen inverse()).
void invert(double* A, int n) {
  std::vector<double> M(A, A + n * n), I(n * n, 0.0);
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(M[k * n + k]);
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(M[i * n + k]) > best) best = std::fabs(M[i * n + k]), p = i;
    if (best == 0.0) throw std::runtime_error("singular mass matrix");
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(M[k * n + j], M[p * n + j]), std::swap(I[k * n + j], I[p * n + j]);
    double d = M[k * n + k];
    for (int j = 0; j < n; ++j) M[k * n + j] /= d, I[k * n + j] /= d;
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      double l = M[i * n + k];
      if (l == 0.0) continue;
      for (int j = 0; j < n; ++j) M[i * n + j] -= l * M[k * n + j], I[i * n + j] -= l * I[k * n + j];
    }
  }
  std::copy(I.begin(), I.end(), A);
}

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double* a, const double* b, double* o) {
  o[0] = a[1] * b[2] - a[2] * b[1];
  o[1] = a[2] * b[0] - a[0] * b[2];
  o[2] = a[0] * b[1] - a[1] * b[0];
}
// Eigen's normalize() leaves a zero vector unchanged.
inline void normalize3(double* a) {
  double z = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (z > 0.0) {
    double s = std::sqrt(z);
    a[0] /= s, a[1] /= s, a[2] /= s;
  }
}

// ---------------------------------------------------------------------------
// Quadrature (stand-in for Gmsh "Gauss(2p)", src/Mesh.cpp:49-52,213-215)
// Reference elements as in Gmsh: line [-1,1]; triangle (0,0),(1,0),(0,1);
// tetrahedron (0,0,0),(1,0,0),(0,1,0),(0,0,1).
// ---------------------------------------------------------------------------
struct Rule {
  int n = 0, dim = 0;
  std::vector<double> x;  // n*dim reference coordinates
  std::vector<double> w;  // n weights
};

// Jacobi polynomial P_n^{(a,0)} and its derivative (three-term recurrence).
void jacobi(int n, double a, double x, double& p, double& dp) {
  double b = 0.0;
  double p0 = 1.0, p1 = 0.5 * (a - b + (a + b + 2.0) * x);
  double d0 = 0.0, d1 = 0.5 * (a + b + 2.0);
  if (n == 0) {
    p = 1.0, dp = 0.0;
    return;
  }
  for (int k = 2; k <= n; ++k) {
    double c = 2.0 * k + a + b;
    double a1 = 2.0 * k * (k + a + b) * (c - 2.0);
    double a2 = (c - 1.0) * (a * a - b * b);
    double a3 = (c - 2.0) * (c - 1.0) * c;
    double a4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * c;
    double p2 = ((a2 + a3 * x) * p1 - a4 * p0) / a1;
    double d2 = ((a2 + a3 * x) * d1 + a3 * p1 - a4 * d0) / a1;
    p0 = p1, p1 = p2, d0 = d1, d1 = d2;
  }
  p = p1, dp = d1;
}

// Gauss-Jacobi nodes/weights for weight (1-x)^a on [-1,1], ascending order.
void gauss_jacobi(int n, double a, std::vector<double>& x, std::vector<double>& w) {
  x.clear(), w.clear();
  const int M = 4000;
  double prev_x = -1.0 + 1e-12, prev_p, dummy;
  jacobi(n, a, prev_x, prev_p, dummy);
  for (int i = 1; i <= M && (int)x.size() < n; ++i) {
    double xi = -1.0 + 2.0 * i / M;
    if (i == M) xi = 1.0 - 1e-12;
    double pi;
    jacobi(n, a, xi, pi, dummy);
    if ((prev_p < 0) != (pi < 0)) {
      double lo = prev_x, hi = xi, plo = prev_p;
      for (int it = 0; it < 200; ++it) {
        double mid = 0.5 * (lo + hi), pm;
        jacobi(n, a, mid, pm, dummy);
        if ((pm < 0) == (plo < 0))
          lo = mid, plo = pm;
        else
          hi = mid;
      }
      double r = 0.5 * (lo + hi);
      for (int it = 0; it < 3; ++it) {
        double p, dp;
        jacobi(n, a, r, p, dp);
        r -= p / dp;
      }
      x.push_back(r);
    }
    prev_x = xi, prev_p = pi;
  }
  if ((int)x.size() != n) throw std::runtime_error("gauss_jacobi root search failed");
  for (double r : x) {
    double p, dp;
    jacobi(n, a, r, p, dp);
    w.push_back(std::pow(2.0, a + 1.0) / ((1.0 - r * r) * dp * dp));
  }
}

// Gauss-Legendre on the oracle's [0, 1] reference segment (line elements).
Rule line01_rule(int n);

Rule gauss_line(int n) {
  Rule r;
  r.n = n, r.dim = 1;
  gauss_jacobi(n, 0.0, r.x, r.w);
  return r;
}

Rule line01_rule(int n) {
  Rule r = gauss_line(n);
  for (int g = 0; g < n; ++g) r.x[g] = 0.5 * (r.x[g] + 1.0), r.w[g] *= 0.5;
  return r;
}

// Expand symmetric orbits given in barycentric coordinates. The first listed
// barycentric triple of the first orbit is the first point of the rule.
void push_bary_tri(Rule& r, double b0, double b1, double b2, double w) {
  r.x.push_back(b1), r.x.push_back(b2), r.w.push_back(0.5 * w), ++r.n;
}

// Degree 2p triangle rules (Dunavant), with the leading points ordered as the
// oracle's stand-in for Gmsh's first face quadrature points: for p >= 2 the
// first point has f(l0) f(l1) < 0, f being the derivative factor of the
// vertex basis function, i.e. the face normal built from the basis gradients
// of the first two face nodes (src/Mesh.cpp:344) points against the right-hand
// normal of the face's node order. The reference compensates exactly this
// with fc = -1 for p != 1 in 3-D (src/Mesh.cpp:366-367).
Rule tri_rule(int degree) {
  Rule r;
  r.dim = 2;
  auto s21 = [&](double a, double w, int first) {
    // orbit (a,a,1-2a); 'first' picks which permutation leads
    double c = 1.0 - 2.0 * a;
    double P[3][3] = {{c, a, a}, {a, c, a}, {a, a, c}};
    for (int k = 0; k < 3; ++k) {
      auto& p = P[(first + k) % 3];
      push_bary_tri(r, p[0], p[1], p[2], w);
    }
  };
  auto s111 = [&](double a, double b, double w) {
    double c = 1.0 - a - b;
    double P[6][3] = {{a, b, c}, {b, c, a}, {c, a, b}, {b, a, c}, {a, c, b}, {c, b, a}};
    for (auto& p : P) push_bary_tri(r, p[0], p[1], p[2], w);
  };
  switch (degree) {
    case 1:
    case 2:
      s21(1.0 / 6.0, 1.0 / 3.0, 0);  // (2/3,1/6,1/6) first
      break;
    case 3:
    case 4:
      s21(0.445948490915965, 0.223381589678011, 0);  // (0.108,0.446,0.446) first
      s21(0.091576213509771, 0.109951743655322, 0);
      break;
    case 5:
    case 6:
      s111(0.053145049844817, 0.310352451033784, 0.082851075618374);
      s21(0.249286745170910, 0.116786275726379, 0);
      s21(0.063089014491502, 0.050844906370207, 0);
      break;
    case 7:
    case 8: {
      // (0.0505, 0.8989, 0.0505) first
      double a = 0.050547228317031, c = 1.0 - 2.0 * a, w = 0.032458497623198;
      push_bary_tri(r, a, c, a, w);
      push_bary_tri(r, c, a, a, w);
      push_bary_tri(r, a, a, c, w);
      push_bary_tri(r, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0.144315607677787);
      s21(0.459292588292723, 0.095091634267285, 0);
      s21(0.170569307751760, 0.103217370534718, 0);
      s111(0.008394777409958, 0.263112829634638, 0.027230314174435);
      break;
    }
    default:
      throw std::runtime_error("triangle rule degree > 8 not available");
  }
  return r;
}

void push_bary_tet(Rule& r, const double* b, double w) {
  r.x.push_back(b[1]), r.x.push_back(b[2]), r.x.push_back(b[3]);
  r.w.push_back(w / 6.0), ++r.n;
}

// All distinct permutations of a barycentric quadruple.
void tet_orbit(Rule& r, double a, double b, double c, double d, double w) {
  double v[4] = {a, b, c, d};
  std::sort(v, v + 4);
  do {
    push_bary_tet(r, v, w);
  } while (std::next_permutation(v, v + 4));
}

// Degree 2p tetrahedron rules: 4-point (deg 2), Keast 11-point (deg 4),
// Keast 24-point (deg 6), Stroud conical product 5x5x5 (deg 8).
Rule tet_rule(int degree) {
  Rule r;
  r.dim = 3;
  if (degree <= 2) {
    double a = 0.1381966011250105;
    tet_orbit(r, a, a, a, 1 - 3 * a, 0.25);
  } else if (degree <= 4) {
    tet_orbit(r, 0.25, 0.25, 0.25, 0.25, -0.0789333333333333);
    double a = 0.0714285714285714;
    tet_orbit(r, a, a, a, 1 - 3 * a, 0.0457333333333333);
    double b = 0.399403576166799;
    tet_orbit(r, b, b, 0.5 - b, 0.5 - b, 0.149333333333333);
  } else if (degree <= 6) {
    double a1 = 0.214602871259151, a2 = 0.0406739585346113, a3 = 0.322337890142275;
    tet_orbit(r, a1, a1, a1, 1 - 3 * a1, 6 * 0.00665379170969465);
    tet_orbit(r, a2, a2, a2, 1 - 3 * a2, 6 * 0.00167953517588678);
    tet_orbit(r, a3, a3, a3, 1 - 3 * a3, 6 * 0.00922619692394239);
    double a = 0.0636610018750175, b = 0.269672331458316;
    tet_orbit(r, a, a, b, 1 - 2 * a - b, 6 * 0.00803571428571428);
  } else if (degree <= 9) {
    std::vector<double> xa, wa, xb, wb, xc, wc;
    gauss_jacobi(5, 0.0, xa, wa);
    gauss_jacobi(5, 1.0, xb, wb);
    gauss_jacobi(5, 2.0, xc, wc);
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j)
        for (int k = 0; k < 5; ++k) {
          double A = 0.5 * (1 + xa[i]), B = 0.5 * (1 + xb[j]), C = 0.5 * (1 + xc[k]);
          double w = wa[i] * 0.5 * wb[j] * 0.25 * wc[k] * 0.125;
          double wq = C, vq = B * (1 - C), uq = A * (1 - B) * (1 - C);
          r.x.push_back(uq), r.x.push_back(vq), r.x.push_back(wq);
          r.w.push_back(w), ++r.n;
        }
  } else {
    throw std::runtime_error("tetrahedron rule degree > 9 not available");
  }
  return r;
}

// ---------------------------------------------------------------------------
// Lagrange basis on an arbitrary nodal set (stand-in for Gmsh's Lagrange /
// GradLagrange basis functions, src/Mesh.cpp:64-67,230-232)
// ---------------------------------------------------------------------------
struct Basis {
  int dim = 0, order = 0, n = 0;
  std::vector<int> expo;   // n*dim monomial exponents
  std::vector<double> C;   // n x n: phi_i = sum_k C[k*n+i] m_k
  void build(int d, int p, const std::vector<double>& nodes) {
    dim = d, order = p;
    expo.clear();
    if (d == 1) {
      for (int a = 0; a <= p; ++a) expo.push_back(a);
    } else if (d == 2) {
      for (int s = 0; s <= p; ++s)
        for (int a = s; a >= 0; --a) expo.push_back(a), expo.push_back(s - a);
    } else {
      for (int s = 0; s <= p; ++s)
        for (int a = s; a >= 0; --a)
          for (int b = s - a; b >= 0; --b) expo.push_back(a), expo.push_back(b), expo.push_back(s - a - b);
    }
    n = (int)expo.size() / d;
    if ((int)nodes.size() != n * d) throw std::runtime_error("basis node count mismatch");
    // V[i][k] = m_k(x_i); C = V^-1
    C.assign(n * n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int k = 0; k < n; ++k) C[i * n + k] = mono(&nodes[i * d], k);
    invert(C.data(), n);
  }
  double mono(const double* x, int k) const {
    double v = 1.0;
    for (int d = 0; d < dim; ++d)
      for (int e = 0; e < expo[k * dim + d]; ++e) v *= x[d];
    return v;
  }
  double dmono(const double* x, int k, int dd) const {
    int e = expo[k * dim + dd];
    if (e == 0) return 0.0;
    double v = e;
    for (int d = 0; d < dim; ++d) {
      int ee = expo[k * dim + d] - (d == dd ? 1 : 0);
      for (int q = 0; q < ee; ++q) v *= x[d];
    }
    return v;
  }
  void eval(const double* x, double* phi) const {
    std::vector<double> m(n);
    for (int k = 0; k < n; ++k) m[k] = mono(x, k);
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += C[k * n + i] * m[k];
      phi[i] = s;
    }
  }
  void grad(const double* x, double* g /* n*dim */) const {
    std::vector<double> m(n);
    for (int d = 0; d < dim; ++d) {
      for (int k = 0; k < n; ++k) m[k] = dmono(x, k, d);
      for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s += C[k * n + i] * m[k];
        g[i * dim + d] = s;
      }
    }
  }
};

// Local faces in Gmsh's element conventions (getElementEdgeNodes /
// getElementFaceNodes, src/Mesh.cpp:178-181).
const int kTriEdges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kTetFaces[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};

// ---------------------------------------------------------------------------
// The mesh object (restates class Mesh, include/Mesh.h:38-310)
// ---------------------------------------------------------------------------
struct RefMesh {
  const refcpu_input* in = nullptr;
  int fc = 1, m_Dim = 3, m_elDim = 0, m_elOrder = 0, m_elNumNodes = 0, m_elNumIntPts = 0;
  int m_elNum = 0;
  int m_fDim = 0, m_fNumNodes = 0, m_fNumPerEl = 0, m_fNum = 0, m_fNumIntPts = 0;
  std::vector<double> m_elWeight, m_elBasisFcts, m_elJacobianDets, m_elGradBasisFcts;
  std::vector<double> m_fWeight, m_fBasisFcts, m_fJacobianDets, m_fNormals, m_fTangents, m_fBiTangents;
  std::vector<double> m_fIntPtCoords;
  std::vector<int64_t> m_fNodeIdx;          // [F][Nfp] global node index
  std::vector<int64_t> m_elFIds;            // [E][Nf]
  std::vector<std::vector<int64_t>> m_fNbrElIds, m_fNToElNIds;
  std::vector<int> m_elFOrientation;
  std::vector<char> m_fIsBoundary;
  std::vector<int> m_fBC;
  std::vector<std::vector<double>> RKR;
  std::vector<double> m_fFlux, m_elMassMatrices;
  std::vector<std::vector<double>> uGhost;
  std::vector<std::vector<std::vector<double>>> FluxGhost;
  // element local face node lists (element local node ids), Nf x Nfp
  std::vector<int> m_locFaceNodes;
  int nthreads = 1;

  inline double& elGradBasisFct(int64_t el, int g, int i, int x = 0) {
    return m_elGradBasisFcts[((el * m_elNumIntPts + g) * m_elNumNodes + i) * 3 + x];
  }
  inline double elBasisFct(int g, int i) const { return m_elBasisFcts[g * m_elNumNodes + i]; }
  inline double elJacobianDet(int64_t el, int g) const { return m_elJacobianDets[el * m_elNumIntPts + g]; }
  inline double fBasisFct(int g, int i) const { return m_fBasisFcts[g * m_fNumNodes + i]; }
  inline double& fNormal(int64_t f, int g, int x = 0) { return m_fNormals[(f * m_fNumIntPts + g) * 3 + x]; }
  inline double& fTangent(int64_t f, int g, int x = 0) { return m_fTangents[(f * m_fNumIntPts + g) * 3 + x]; }
  inline double& fBiTangent(int64_t f, int g, int x = 0) { return m_fBiTangents[(f * m_fNumIntPts + g) * 3 + x]; }
  inline double fJacobianDet(int64_t f, int g) const { return m_fJacobianDets[f * m_fNumIntPts + g]; }
  inline int64_t elFId(int64_t el, int f) const { return m_elFIds[el * m_fNumPerEl + f]; }
  inline int64_t fNbrElId(int64_t f, int k) const { return m_fNbrElIds[f][k]; }
  inline int64_t fNToElNId(int64_t f, int nf, int k) const {
    return m_fNToElNIds[f][nf * m_fNbrElIds[f].size() + k];
  }
  inline int& elFOrientation(int64_t el, int f) { return m_elFOrientation[el * m_fNumPerEl + f]; }
  inline double& fFlux(int64_t f, int n) { return m_fFlux[f * m_fNumNodes + n]; }
  inline double* elMassMatrix(int64_t el) { return &m_elMassMatrices[el * m_elNumNodes * m_elNumNodes]; }
  const double* X(int64_t node) const { return &in->xyz[3 * node]; }

  void setup(const refcpu_input* input);
  void precomputeMassMatrix();
  void getElStiffVector(int64_t el, std::vector<std::vector<double>>& Flux, double* out);
  void precomputeFlux(std::vector<double>& u, std::vector<std::vector<double>>& Flux, int eq);
  void getElFlux(int64_t el, double* F);
  void updateFlux(std::vector<std::vector<double>>& u, std::vector<std::vector<std::vector<double>>>& Flux);
};

void RefMesh::setup(const refcpu_input* input) {
  in = input;
  nthreads = std::max(1, in->num_threads);
  m_elDim = in->dim;
  m_elOrder = in->order;
  m_elNumNodes = in->nodes_per_elem;
  m_elNum = (int)in->n_elems;
  const int D = m_elDim, P = m_elOrder, Np = m_elNumNodes;
  if (D < 1 || D > 3) throw std::runtime_error("dim must be 1, 2 or 3");
  int expectNp = D == 1 ? P + 1 : D == 2 ? (P + 1) * (P + 2) / 2 : (P + 1) * (P + 2) * (P + 3) / 6;
  if (Np != expectNp) throw std::runtime_error("nodes_per_elem does not match order");
  const int nc = D + 1;

  // --- reference node set from element 0, snapped to the order-p lattice ---
  std::vector<double> refNodes(Np * D);
  auto local_coords = [&](int64_t el, int n, double* xi) {
    const int64_t* en = &in->elem_nodes[el * Np];
    double J[9] = {0}, rhs[3];
    for (int d = 0; d < D; ++d)
      for (int k = 0; k < D; ++k) J[d * D + k] = X(en[k + 1])[d] - X(en[0])[d];
    for (int d = 0; d < D; ++d) rhs[d] = X(en[n])[d] - X(en[0])[d];
    std::vector<double> A(J, J + D * D);
    lu_solve(A, rhs, D);
    for (int d = 0; d < D; ++d) xi[d] = rhs[d];
  };
  std::vector<int> lattice(Np * D);
  for (int n = 0; n < Np; ++n) {
    double xi[3];
    local_coords(0, n, xi);
    for (int d = 0; d < D; ++d) {
      double s = std::round(xi[d] * P);
      if (std::fabs(xi[d] * P - s) > 0.25) throw std::runtime_error("element 0 nodes are not a Lagrange lattice");
      lattice[n * D + d] = (int)s;
      refNodes[n * D + d] = s / P;
    }
  }
  for (int64_t el = 1; el < m_elNum; ++el)
    for (int n = nc; n < Np; ++n) {
      double xi[3];
      local_coords(el, n, xi);
      for (int d = 0; d < D; ++d)
        if (std::fabs(xi[d] * P - lattice[n * D + d]) > 0.25)
          throw std::runtime_error("elements do not share one local node ordering");
    }
  Basis elBasis;
  elBasis.build(D, P, refNodes);

  // --- volume quadrature, basis at points, Jacobians (Mesh.cpp:40-137) ---
  // lines: Gauss-Legendre with P + 1 points (degree 2P + 1), on the
  // oracle's [0, 1] reference segment
  Rule vr = D == 1 ? line01_rule(P + 1) : D == 2 ? tri_rule(2 * P) : tet_rule(2 * P);
  m_elNumIntPts = vr.n;
  const int Ng = vr.n;
  m_elWeight = vr.w;
  m_elBasisFcts.resize(Ng * Np);
  std::vector<double> ugrad(Ng * Np * D);
  for (int g = 0; g < Ng; ++g) {
    elBasis.eval(&vr.x[g * D], &m_elBasisFcts[g * Np]);
    elBasis.grad(&vr.x[g * D], &ugrad[g * Np * D]);
  }
  m_elJacobianDets.assign((size_t)m_elNum * Ng, 0.0);
  m_elGradBasisFcts.assign((size_t)m_elNum * Ng * Np * 3, 0.0);
  for (int64_t el = 0; el < m_elNum; ++el) {
    const int64_t* en = &in->elem_nodes[el * Np];
    for (int g = 0; g < Ng; ++g) {
      double J[9] = {0};  // J[x*D+u] = dx/du (isoparametric)
      for (int n = 0; n < Np; ++n)
        for (int x = 0; x < D; ++x)
          for (int u = 0; u < D; ++u) J[x * D + u] += X(en[n])[x] * ugrad[(g * Np + n) * D + u];
      // Gmsh's determinant of a line element in 3-D space is the length of
      // its tangent (positive); simplices keep the signed determinant
      double det = D == 1   ? std::fabs(J[0])
                   : D == 2 ? J[0] * J[3] - J[1] * J[2]
                            : J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                                  J[2] * (J[3] * J[7] - J[4] * J[6]);
      m_elJacobianDets[el * Ng + g] = det;
      // J^T grad_x = grad_u (src/Mesh.cpp:132-133)
      std::vector<double> JT(D * D);
      for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) JT[a * D + b] = J[b * D + a];
      for (int n = 0; n < Np; ++n) {
        double v[3] = {0, 0, 0};
        for (int u = 0; u < D; ++u) v[u] = ugrad[(g * Np + n) * D + u];
        lu_solve(JT, v, D);
        for (int x = 0; x < D; ++x) elGradBasisFct(el, g, n, x) = v[x];
      }
    }
  }

  // --- faces of all elements (Mesh.cpp:165-183) ---
  m_fDim = D - 1;
  m_fNumNodes = m_fDim == 0 ? 1 : m_fDim == 1 ? 1 + P : (P + 1) * (P + 2) / 2;
  m_fNumPerEl = D + 1;
  const int Nf = m_fNumPerEl, Nfp = m_fNumNodes;
  // element-local face node lists: corners in face order, then the rest
  m_locFaceNodes.assign(Nf * Nfp, -1);
  std::vector<double> faceRefNodes(Nf * Nfp * (D - 1));
  for (int lf = 0; lf < Nf; ++lf) {
    int corners[3];
    // lines: the faces are the two end points, local face lf = vertex lf
    for (int k = 0; k < D; ++k) corners[k] = D == 1 ? lf : D == 2 ? kTriEdges[lf][k] : kTetFaces[lf][k];
    int opp = 0;
    for (int v = 0; v < nc; ++v) {
      bool in_face = false;
      for (int k = 0; k < D; ++k) in_face |= corners[k] == v;
      if (!in_face) opp = v;
    }
    int cnt = 0;
    auto bary = [&](int n, int v) -> int {  // lattice barycentric * P
      if (v == 0) {
        int s = P;
        for (int d = 0; d < D; ++d) s -= lattice[n * D + d];
        return s;
      }
      return lattice[n * D + v - 1];
    };
    for (int k = 0; k < D; ++k) m_locFaceNodes[lf * Nfp + cnt++] = corners[k];
    // remaining face nodes ordered by their face coordinates, so that every
    // local face has the same node arrangement (one face basis serves all)
    std::vector<std::pair<int, int>> rest;  // (sort key, node)
    for (int n = nc; n < Np; ++n)
      if (bary(n, opp) == 0) {
        int key = D == 2 ? bary(n, corners[1]) : bary(n, corners[2]) * (P + 1) + bary(n, corners[1]);
        rest.push_back({key, n});
      }
    std::sort(rest.begin(), rest.end());
    for (auto& kn : rest) {
      if (cnt >= Nfp) throw std::runtime_error("too many face nodes");
      m_locFaceNodes[lf * Nfp + cnt++] = kn.second;
    }
    if (cnt != Nfp) throw std::runtime_error("face node count mismatch");
    for (int m = 0; m < Nfp; ++m) {
      int n = m_locFaceNodes[lf * Nfp + m];
      if (D == 1) {
        // point faces have no reference coordinates
      } else if (D == 2) {
        faceRefNodes[(lf * Nfp + m)] = 2.0 * bary(n, corners[1]) / P - 1.0;
      } else {
        faceRefNodes[(lf * Nfp + m) * 2 + 0] = (double)bary(n, corners[1]) / P;
        faceRefNodes[(lf * Nfp + m) * 2 + 1] = (double)bary(n, corners[2]) / P;
      }
    }
  }
  // All local faces share one face-node arrangement by construction; use face 0's.
  Basis fBasis;
  if (D > 1) fBasis.build(D - 1, P, std::vector<double>(faceRefNodes.begin(), faceRefNodes.begin() + Nfp * (D - 1)));
  for (int lf = 1; lf < Nf; ++lf)
    for (int k = 0; k < Nfp * (D - 1); ++k)
      if (std::fabs(faceRefNodes[lf * Nfp * (D - 1) + k] - faceRefNodes[k]) > 1e-12)
        throw std::runtime_error("local faces do not share one node arrangement");

  // --- unique faces in order of first occurrence (Mesh.cpp:981-1078) and
  //     face -> element connectivity (Mesh.cpp:1093-1130); hashing replaces
  //     the quadratic scans with the same result ---
  struct Key {
    int64_t a, b, c;
    bool operator==(const Key& o) const { return a == o.a && b == o.b && c == o.c; }
  };
  struct KeyHash {
    size_t operator()(const Key& k) const {
      uint64_t h = (uint64_t)k.a * 0x9E3779B97F4A7C15ull;
      h ^= (uint64_t)k.b + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
      h ^= (uint64_t)k.c + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
      return (size_t)h;
    }
  };
  std::unordered_map<Key, int64_t, KeyHash> faceOf;
  faceOf.reserve((size_t)m_elNum * Nf);
  m_elFIds.assign((size_t)m_elNum * Nf, -1);
  m_fNbrElIds.clear();
  m_fNodeIdx.clear();
  std::vector<int> upLocalFace;
  for (int64_t el = 0; el < m_elNum; ++el) {
    const int64_t* en = &in->elem_nodes[el * Np];
    for (int lf = 0; lf < Nf; ++lf) {
      int64_t v[3] = {en[m_locFaceNodes[lf * Nfp + 0]], D >= 2 ? en[m_locFaceNodes[lf * Nfp + 1]] : -1,
                      D == 3 ? en[m_locFaceNodes[lf * Nfp + 2]] : -1};
      std::sort(v, v + D);
      Key k{v[0], v[1], v[2]};
      auto it = faceOf.find(k);
      int64_t f;
      if (it == faceOf.end()) {
        f = (int64_t)m_fNbrElIds.size();
        faceOf.emplace(k, f);
        m_fNbrElIds.push_back({el});
        upLocalFace.push_back(lf);
        for (int m = 0; m < Nfp; ++m) m_fNodeIdx.push_back(en[m_locFaceNodes[lf * Nfp + m]]);
      } else {
        f = it->second;
        if (m_fNbrElIds[f].size() >= 2) throw std::runtime_error("non-manifold face (shared by > 2 elements)");
        m_fNbrElIds[f].push_back(el);
      }
      m_elFIds[el * Nf + lf] = f;
    }
  }
  m_fNum = (int)m_fNbrElIds.size();
  const int64_t F = m_fNum;

  // --- face quadrature, basis, Jacobians, tangential gradients (Mesh.cpp:209-260) ---
  // point faces (lines): one point of weight 1, face basis 1
  Rule fr;
  if (D == 1)
    fr.n = 1, fr.dim = 0, fr.w = {1.0};
  else
    fr = D == 2 ? gauss_line(P + 1) : tri_rule(2 * P);
  m_fNumIntPts = fr.n;
  const int Ngf = fr.n;
  m_fWeight = fr.w;
  m_fBasisFcts.resize(Ngf * Nfp);
  std::vector<double> fugrad(Ngf * Nfp * (D - 1));
  for (int g = 0; g < Ngf; ++g) {
    if (D == 1) {
      m_fBasisFcts[g * Nfp] = 1.0;
      continue;
    }
    fBasis.eval(&fr.x[g * (D - 1)], &m_fBasisFcts[g * Nfp]);
    fBasis.grad(&fr.x[g * (D - 1)], &fugrad[g * Nfp * (D - 1)]);
  }
  m_fJacobianDets.assign(F * Ngf, 0.0);
  m_fIntPtCoords.assign(F * Ngf * 3, 0.0);
  std::vector<double> fGrad(F * Ngf * Nfp * 3, 0.0);  // tangential gradients
  for (int64_t f = 0; f < F; ++f) {
    const int64_t* fn = &m_fNodeIdx[f * Nfp];
    for (int g = 0; g < Ngf; ++g) {
      double T[2][3] = {{0, 0, 0}, {0, 0, 0}}, xg[3] = {0, 0, 0};
      for (int n = 0; n < Nfp; ++n) {
        for (int x = 0; x < 3; ++x) {
          xg[x] += X(fn[n])[x] * fBasisFct(g, n);
          for (int u = 0; u < D - 1; ++u) T[u][x] += X(fn[n])[x] * fugrad[(g * Nfp + n) * (D - 1) + u];
        }
      }
      for (int x = 0; x < 3; ++x) m_fIntPtCoords[(f * Ngf + g) * 3 + x] = xg[x];
      double det;
      if (D == 1) {
        det = 1.0;  // Gmsh's Jacobian determinant of a point element
      } else if (D == 2) {
        det = std::sqrt(dot3(T[0], T[0]));
        for (int n = 0; n < Nfp; ++n) {
          double c = fugrad[g * Nfp + n] / (det * det);
          for (int x = 0; x < 3; ++x) fGrad[((f * Ngf + g) * Nfp + n) * 3 + x] = c * T[0][x];
        }
      } else {
        double nrm[3];
        cross3(T[0], T[1], nrm);
        det = std::sqrt(dot3(nrm, nrm));
        // grad = T (T^T T)^-1 grad_uv
        double a = dot3(T[0], T[0]), b = dot3(T[0], T[1]), c = dot3(T[1], T[1]);
        double id = 1.0 / (a * c - b * b);
        for (int n = 0; n < Nfp; ++n) {
          double gu = fugrad[(g * Nfp + n) * 2], gv = fugrad[(g * Nfp + n) * 2 + 1];
          double cu = (c * gu - b * gv) * id, cv = (-b * gu + a * gv) * id;
          for (int x = 0; x < 3; ++x) fGrad[((f * Ngf + g) * Nfp + n) * 3 + x] = cu * T[0][x] + cv * T[1][x];
        }
      }
      m_fJacobianDets[f * Ngf + g] = det;
    }
  }

  // --- normals, tangents, bitangents (Mesh.cpp:277-367) ---
  m_fNormals.clear(), m_fTangents.clear(), m_fBiTangents.clear();
  m_fNormals.reserve(F * Ngf * 3), m_fTangents.reserve(F * Ngf * 3), m_fBiTangents.reserve(F * Ngf * 3);
  auto fg = [&](int64_t f, int g, int n) { return &fGrad[((f * Ngf + g) * Nfp + n) * 3]; };
  for (int64_t f = 0; f < F; ++f) {
    double Tv[3] = {0, 0, 0}, Bv[3] = {0, 0, 0};
    if (m_fDim == 2) {
      const double* p1 = &m_fIntPtCoords[(f * Ngf + 0) * 3];
      const double* p2 = &m_fIntPtCoords[(f * Ngf + 1) * 3];
      const double* p3 = &m_fIntPtCoords[(f * Ngf + 2) * 3];
      double h = std::sqrt(std::pow(p2[0] - p1[0], 2) + std::pow(p2[1] - p1[1], 2) + std::pow(p2[2] - p1[2], 2));
      double i = ((p2[0] - p1[0]) * (p3[0] - p1[0]) + (p2[1] - p1[1]) * (p3[1] - p1[1]) +
                  (p2[2] - p1[2]) * (p3[2] - p1[2])) /
                 h;
      double j = std::sqrt(std::pow(p3[0] - p1[0], 2) + std::pow(p3[1] - p1[1], 2) + std::pow(p3[2] - p1[2], 2) -
                           std::pow(i, 2));
      double u1 = 0, v1 = 0, u2 = h, v2 = 0, u3 = i, v3 = j;
      double delta = std::fabs(u2 - u1) * std::fabs(v3 - v1) - std::fabs(v2 - v1) * std::fabs(u3 - u1);
      for (int x = 0; x < 3; ++x) {
        Tv[x] = (std::fabs(v3 - v1) * (p2[x] - p1[x]) - std::fabs(v2 - v1) * (p3[x] - p1[x])) / delta;
        Bv[x] = -(std::fabs(u3 - u1) * (p2[x] - p1[x]) - std::fabs(u2 - u1) * (p3[x] - p1[x])) / delta;
      }
    }
    for (int g = 0; g < Ngf; ++g) {
      double normal[3], tangent[3], bitangent[3];
      if (m_fDim == 0) {
        // Mesh.cpp:320-325: every point face has the normal (1, 0, 0)
        normal[0] = 1.0, normal[1] = normal[2] = 0.0;
        tangent[0] = tangent[1] = tangent[2] = 0.0;
        bitangent[0] = bitangent[1] = bitangent[2] = 0.0;
      } else if (m_fDim == 1) {
        const double plane[3] = {0, 0, -1};
        cross3(fg(f, g, 0), plane, normal);
        if (dot3(fg(f, g, 0), fg(f, 0, 0)) < 0)
          for (int x = 0; x < 3; ++x) normal[x] *= -1.0;
        tangent[0] = -normal[1], tangent[1] = normal[0], tangent[2] = 0;
        bitangent[0] = bitangent[1] = bitangent[2] = 0;
      } else {
        cross3(fg(f, g, 0), fg(f, g, 1), normal);
        if (g != 0 && dot3(&m_fNormals[(f * Ngf) * 3], normal) < 0)
          for (int x = 0; x < 3; ++x) normal[x] *= -1.0;
        for (int x = 0; x < 3; ++x) tangent[x] = Tv[x], bitangent[x] = Bv[x];
      }
      normalize3(normal), normalize3(tangent), normalize3(bitangent);
      m_fNormals.insert(m_fNormals.end(), normal, normal + 3);
      m_fTangents.insert(m_fTangents.end(), tangent, tangent + 3);
      m_fBiTangents.insert(m_fBiTangents.end(), bitangent, bitangent + 3);
    }
  }
  fc = (m_elDim == 3 && m_elOrder != 1) ? -1 : 1;

  // --- face node -> element node maps by node identity (Mesh.cpp:416-431) ---
  m_fNToElNIds.assign(F, {});
  for (int64_t f = 0; f < F; ++f)
    for (int nf = 0; nf < Nfp; ++nf)
      for (int64_t el : m_fNbrElIds[f]) {
        const int64_t* en = &in->elem_nodes[el * Np];
        for (int nel = 0; nel < Np; ++nel)
          if (m_fNodeIdx[f * Nfp + nf] == en[nel]) m_fNToElNIds[f].push_back(nel);
      }
  for (int64_t f = 0; f < F; ++f)
    if ((int64_t)m_fNToElNIds[f].size() != Nfp * (int64_t)m_fNbrElIds[f].size())
      throw std::runtime_error("face nodes are not shared node by node with the neighbour (non-conforming mesh)");

  // --- orientation (Mesh.cpp:452-477): first node of the element's local
  //     face minus the barycentre of the primary nodes, against n(g=0) ---
  m_elFOrientation.assign((size_t)m_elNum * Nf, 1);
  for (int64_t el = 0; el < m_elNum; ++el) {
    const int64_t* en = &in->elem_nodes[el * Np];
    double bc[3] = {0, 0, 0};
    for (int v = 0; v < nc; ++v)
      for (int x = 0; x < 3; ++x) bc[x] += X(en[v])[x];
    for (int x = 0; x < 3; ++x) bc[x] /= nc;
    for (int lf = 0; lf < Nf; ++lf) {
      const double* xn = X(en[m_locFaceNodes[lf * Nfp]]);
      double dp = 0.0;
      for (int x = 0; x < m_Dim; ++x) dp += (xn[x] - bc[x]) * fNormal(elFId(el, lf), 0, x);
      elFOrientation(el, lf) = (dp >= 0) ? 1 : -1;
    }
  }
  // The neighbour "reclassification" at Mesh.cpp:491-509 tests
  // m_fNbrElIds.size() == 2 (the face count) and never fires; nothing to do.

  // --- boundary flags, outward boundary normals (Mesh.cpp:536-568) ---
  m_fIsBoundary.assign(F, 0);
  for (int64_t f = 0; f < F; ++f) {
    if (m_fNbrElIds[f].size() < 2) {
      m_fIsBoundary[f] = 1;
      int64_t el = fNbrElId(f, 0);
      for (int lf = 0; lf < Nf; ++lf)
        if (elFId(el, lf) == f) {
          for (int g = 0; g < Ngf; ++g)
            for (int x = 0; x < 3; ++x) fNormal(f, g, x) *= elFOrientation(el, lf);
          elFOrientation(el, lf) = 1;
        }
    }
  }

  // --- BC codes: group whose node list holds the face's first node; groups in
  //     ascending tag order, last match wins; default Absorbing (Mesh.cpp:579-605) ---
  m_fBC.assign(F, 0);
  std::vector<char> inGroup(in->n_nodes, 0);
  for (int gi = 0; gi < in->n_groups; ++gi) {
    std::fill(inGroup.begin(), inGroup.end(), 0);
    for (int64_t k = in->group_offsets[gi]; k < in->group_offsets[gi + 1]; ++k) inGroup[in->group_nodes[k]] = 1;
    for (int64_t f = 0; f < F; ++f)
      if (m_fIsBoundary[f] && inGroup[m_fNodeIdx[f * Nfp]]) m_fBC[f] = in->group_bc[gi] == 1 ? 1 : 0;
  }

  // --- RKR (Mesh.cpp:619-666) ---
  RKR.assign(F * Ngf, {});
  for (int64_t f = 0; f < F; ++f) {
    if (!m_fIsBoundary[f] || m_fBC[f] != 0) continue;
    for (int g = 0; g < Ngf; ++g) {
      int64_t i = f * Ngf + g;
      double nx = fNormal(f, g, 0), ny = fNormal(f, g, 1), nz = fNormal(f, g, 2);
      double tx = fTangent(f, g, 0), ty = fTangent(f, g, 1), tz = fTangent(f, g, 2);
      double sx = fBiTangent(f, g, 0), sy = fBiTangent(f, g, 1), sz = fBiTangent(f, g, 2);
      double c0 = in->c0, rho0 = in->rho0;
      double vx0 = in->v0[0], vy0 = in->v0[1], vz0 = in->v0[2];
      double vn0 = vx0 * nx + vy0 * ny + vz0 * nz;
      double lambda = (vn0 < 0) ? 0 : -1;
      auto& R = RKR[i];
      R.resize(16);
      R[0] = 0.25 * (c0 + vn0);
      R[1] = 0.25 * (c0 * rho0 * (c0 + vn0) * nx);
      R[2] = 0.25 * (c0 * rho0 * (c0 + vn0) * ny);
      R[3] = 0.25 * (c0 * rho0 * (c0 + vn0) * nz);
      R[4] = 0.25 * (nx * (c0 + vn0) / (rho0 * c0));
      R[5] = 0.25 * ((c0 + vn0) * nx * nx - vn0 * lambda * (tx * tx + sx * sx));
      R[6] = 0.25 * ((c0 + vn0) * nx * ny - vn0 * lambda * (ty * tx + sy * sx));
      R[7] = 0.25 * ((c0 + vn0) * nx * nz - vn0 * lambda * (tz * tx + sz * sx));
      R[8] = 0.25 * (ny * (c0 + vn0) / (rho0 * c0));
      R[9] = 0.25 * ((c0 + vn0) * ny * nx - vn0 * lambda * (tx * ty + sx * sy));
      R[10] = 0.25 * ((c0 + vn0) * ny * ny - vn0 * lambda * (ty * ty + sy * sy));
      R[11] = 0.25 * ((c0 + vn0) * ny * nz - vn0 * lambda * (tz * ty + sz * sy));
      R[12] = 0.25 * (nz * (c0 + vn0) / (rho0 * c0));
      R[13] = 0.25 * ((c0 + vn0) * nz * nx - vn0 * lambda * (tx * tz + sx * sz));
      R[14] = 0.25 * ((c0 + vn0) * nz * ny - vn0 * lambda * (ty * tz + sy * sz));
      R[15] = 0.25 * ((c0 + vn0) * nz * nz - vn0 * lambda * (tz * tz + sz * sz));
    }
  }

  // --- work storage (Mesh.cpp:674-679) ---
  m_fFlux.assign(F * Nfp, 0.0);
  uGhost.assign(4, std::vector<double>(F * Ngf, 0.0));
  FluxGhost.assign(4, std::vector<std::vector<double>>(F * Ngf, std::vector<double>(3, 0.0)));
}

// src/Mesh.cpp:691-724
void RefMesh::precomputeMassMatrix() {
  const int Np = m_elNumNodes, Ng = m_elNumIntPts;
  m_elMassMatrices.assign((size_t)m_elNum * Np * Np, 0.0);
  for (int64_t el = 0; el < m_elNum; ++el) {
    double* M = elMassMatrix(el);
    for (int i = 0; i < Np; ++i)
      for (int j = 0; j < Np; ++j) {
        M[i * Np + j] = 0.0;
        for (int g = 0; g < Ng; g++)
          M[i * Np + j] += elBasisFct(g, i) * elBasisFct(g, j) * m_elWeight[g] * elJacobianDet(el, g);
      }
    invert(M, Np);
  }
}

// src/Mesh.cpp:734-751
void RefMesh::getElStiffVector(int64_t el, std::vector<std::vector<double>>& Flux, double* out) {
  const int Np = m_elNumNodes, Ng = m_elNumIntPts;
  for (int i = 0; i < Np; ++i) {
    out[i] = 0.0;
    for (int j = 0; j < Np; ++j) {
      int64_t jId = el * Np + j;
      for (int g = 0; g < Ng; g++)
        out[i] += dot3(Flux[jId].data(), &elGradBasisFct(el, g, i)) * elBasisFct(g, j) * m_elWeight[g] *
                  elJacobianDet(el, g);
    }
  }
}

// src/Mesh.cpp:761-813, with its nested OpenMP region. Under libgomp's default
// max-active-levels of 1 the inner 'parallel for' of an active outer team is
// a team of one, so every outer thread runs the whole face loop. The inner
// team is pinned to one thread so that a one-thread (inactive) outer region
// behaves the same way instead of sharing FIntPts across an inner team.
void RefMesh::precomputeFlux(std::vector<double>& u, std::vector<std::vector<double>>& Flux, int eq) {
  const int Nfp = m_fNumNodes, Ngf = m_fNumIntPts;
  const double c0 = in->c0;
#pragma omp parallel num_threads(nthreads)
  {
    int64_t elUp, elDn;
    std::vector<double> FIntPts(Ngf, 0);
    std::vector<double> Fnum(m_Dim, 0);
#pragma omp parallel for schedule(static) num_threads(1)
    for (int f = 0; f < m_fNum; ++f) {
      std::fill(FIntPts.begin(), FIntPts.end(), 0);
      if (m_fIsBoundary[f]) {
        for (int g = 0; g < Ngf; ++g) FIntPts[g] = FluxGhost[eq][(int64_t)f * Ngf + g][0];
      } else {
        for (int i = 0; i < Nfp; ++i) {
          elUp = fNbrElId(f, 0) * m_elNumNodes + fNToElNId(f, i, 0);
          elDn = fNbrElId(f, 1) * m_elNumNodes + fNToElNId(f, i, 1);
          for (int g = 0; g < Ngf; ++g) {
            for (int x = 0; x < m_Dim; ++x)
              Fnum[x] = 0.5 * ((Flux[elUp][x] + Flux[elDn][x]) + fc * c0 * fNormal(f, g, x) * (u[elUp] - u[elDn]));
#pragma omp atomic update
            FIntPts[g] += dot3(&fNormal(f, g), Fnum.data()) * fBasisFct(g, i);
          }
        }
      }
      for (int n = 0; n < Nfp; ++n) {
        fFlux(f, n) = 0;
        for (int g = 0; g < Ngf; ++g) {
#pragma omp atomic update
          fFlux(f, n) += m_fWeight[g] * fBasisFct(g, n) * FIntPts[g] * fJacobianDet(f, g);
        }
      }
    }
  }
}

// src/Mesh.cpp:822-839
void RefMesh::getElFlux(int64_t el, double* F) {
  std::fill(F, F + m_elNumNodes, 0);
  for (int f = 0; f < m_fNumPerEl; ++f) {
    int64_t fid = elFId(el, f);
    int i = (el == fNbrElId(fid, 0)) ? 0 : 1;
    for (int nf = 0; nf < m_fNumNodes; ++nf) F[fNToElNId(fid, nf, i)] += elFOrientation(el, f) * fFlux(fid, nf);
  }
}

// src/Mesh.cpp:851-975
void RefMesh::updateFlux(std::vector<std::vector<double>>& u, std::vector<std::vector<std::vector<double>>>& Flux) {
  const int Np = m_elNumNodes, Nfp = m_fNumNodes, Ngf = m_fNumIntPts;
  const double* v0 = in->v0;
  const double c0 = in->c0, rho0 = in->rho0;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int el = 0; el < m_elNum; ++el) {
    for (int n = 0; n < Np; ++n) {
      int64_t i = (int64_t)el * Np + n;
      Flux[0][i] = {v0[0] * u[0][i] + rho0 * c0 * c0 * u[1][i], v0[1] * u[0][i] + rho0 * c0 * c0 * u[2][i],
                    v0[2] * u[0][i] + rho0 * c0 * c0 * u[3][i]};
      Flux[1][i] = {v0[0] * u[1][i] + u[0][i] / rho0, v0[1] * u[1][i], v0[2] * u[1][i]};
      Flux[2][i] = {v0[0] * u[2][i], v0[1] * u[2][i] + u[0][i] / rho0, v0[2] * u[2][i]};
      Flux[3][i] = {v0[0] * u[3][i], v0[1] * u[3][i], v0[2] * u[3][i] + u[0][i] / rho0};
    }
    for (int f = 0; f < m_fNumPerEl; ++f) {
      int64_t fId = elFId(el, f);
      if (!m_fIsBoundary[fId]) continue;
      for (int g = 0; g < Ngf; ++g) {
        int64_t gId = fId * Ngf + g;
        uGhost[0][gId] = uGhost[1][gId] = uGhost[2][gId] = uGhost[3][gId] = 0;
        for (int n = 0; n < Nfp; ++n) {
          int64_t nId = (int64_t)el * Np + fNToElNId(fId, n, 0);
#pragma omp atomic
          uGhost[0][gId] += u[0][nId] * fBasisFct(g, n);
#pragma omp atomic
          uGhost[1][gId] += u[1][nId] * fBasisFct(g, n);
#pragma omp atomic
          uGhost[2][gId] += u[2][nId] * fBasisFct(g, n);
#pragma omp atomic
          uGhost[3][gId] += u[3][nId] * fBasisFct(g, n);
        }
        if (m_fBC[fId] == 1) {
          double nx = fNormal(fId, g, 0), ny = fNormal(fId, g, 1), nz = fNormal(fId, g, 2);
          double dot = nx * uGhost[1][gId] + ny * uGhost[2][gId] + nz * uGhost[3][gId];
#pragma omp atomic
          uGhost[1][gId] -= dot * nx;
#pragma omp atomic
          uGhost[2][gId] -= dot * ny;
#pragma omp atomic
          uGhost[3][gId] -= dot * nz;
          FluxGhost[0][gId] = {v0[0] * uGhost[0][gId] + rho0 * c0 * c0 * uGhost[1][gId],
                               v0[1] * uGhost[0][gId] + rho0 * c0 * c0 * uGhost[2][gId],
                               v0[2] * uGhost[0][gId] + rho0 * c0 * c0 * uGhost[3][gId]};
          FluxGhost[1][gId] = {v0[0] * uGhost[1][gId] + uGhost[0][gId] / rho0, v0[1] * uGhost[1][gId],
                               v0[2] * uGhost[1][gId]};
          FluxGhost[2][gId] = {v0[0] * uGhost[2][gId], v0[1] * uGhost[2][gId] + uGhost[0][gId] / rho0,
                               v0[2] * uGhost[2][gId]};
          FluxGhost[3][gId] = {v0[0] * uGhost[3][gId], v0[1] * uGhost[3][gId],
                               v0[2] * uGhost[3][gId] + uGhost[0][gId] / rho0};
          for (int eq = 0; eq < 4; ++eq) FluxGhost[eq][gId][0] = dot3(&fNormal(fId, g), &FluxGhost[eq][gId][0]);
        } else {
          const auto& R = RKR[gId];
          FluxGhost[0][gId][0] = R[0] * uGhost[0][gId] + R[1] * uGhost[1][gId] + R[2] * uGhost[2][gId] + R[3] * uGhost[3][gId];
          FluxGhost[1][gId][0] = R[4] * uGhost[0][gId] + R[5] * uGhost[1][gId] + R[6] * uGhost[2][gId] + R[7] * uGhost[3][gId];
          FluxGhost[2][gId][0] = R[8] * uGhost[0][gId] + R[9] * uGhost[1][gId] + R[10] * uGhost[2][gId] + R[11] * uGhost[3][gId];
          FluxGhost[3][gId][0] = R[12] * uGhost[0][gId] + R[13] * uGhost[1][gId] + R[14] * uGhost[2][gId] + R[15] * uGhost[3][gId];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Solver (src/solver.cpp)
// ---------------------------------------------------------------------------
struct Solver {
  RefMesh& mesh;
  const refcpu_input* in;
  int Np = 0;
  int64_t numNodes = 0;
  std::vector<double> elFlux, elStiffvector;
  std::vector<std::vector<std::vector<double>>> Flux;
  explicit Solver(RefMesh& m) : mesh(m), in(m.in) {
    Np = mesh.m_elNumNodes;
    numNodes = (int64_t)mesh.m_elNum * Np;
    elFlux.resize(Np);
    elStiffvector.resize(Np);
    Flux.assign(4, std::vector<std::vector<double>>(numNodes, std::vector<double>(3)));
  }
  // src/solver.cpp:38-57
  void numStep(std::vector<std::vector<double>>& u, double beta) {
    const int T = mesh.nthreads;
    const double dt = in->dt;
    for (int eq = 0; eq < 4; ++eq) {
      mesh.precomputeFlux(u[eq], Flux[eq], eq);
#pragma omp parallel for schedule(static) firstprivate(elFlux, elStiffvector) num_threads(T)
      for (int el = 0; el < mesh.m_elNum; ++el) {
        mesh.getElFlux(el, elFlux.data());
        mesh.getElStiffVector(el, Flux[eq], elStiffvector.data());
        for (int i = 0; i < Np; ++i) elStiffvector[i] -= elFlux[i];
        // y = beta*y + dt * M^-T x (column-major map of row-major storage)
        const double* M = mesh.elMassMatrix(el);
        double* y = &u[eq][(int64_t)el * Np];
        double tmp[64];
        for (int i = 0; i < Np; ++i) tmp[i] = 0.0;
        for (int j = 0; j < Np; ++j)
          for (int i = 0; i < Np; ++i) tmp[i] += M[j * Np + i] * elStiffvector[j];
        for (int i = 0; i < Np; ++i) y[i] = beta * y[i] + dt * tmp[i];
      }
    }
  }
};

// include/configParser.h:38-58
double interpolate_value(const double* tab, int64_t rows, double t) {
  if (rows <= 0) return 0.0;
  size_t lo = 0, hi = rows - 1, m = 0;
  double tmin = tab[lo * 2], tmax = tab[hi * 2];
  int guard = 0;
  while (lo <= hi && t >= tmin && t <= tmax) {
    m = (lo + hi) / 2;
    if (t < tab[m * 2])
      hi = m;
    else
      lo = m;
    if (hi == lo + 1) return tab[lo * 2 + 1] + ((tab[hi * 2 + 1] - tab[lo * 2 + 1]) / (tab[hi * 2] - tab[lo * 2])) * (t - tab[lo * 2]);
    if (++guard > 200) break;  // one-row table: the reference loops forever here
  }
  return 0.0;
}

void node_coords(const refcpu_input* in, int64_t n, double* c) {
  int64_t node = in->elem_nodes[n];
  for (int x = 0; x < 3; ++x) c[x] = in->xyz[3 * node + x];
}

void apply_ic(const refcpu_input* in, std::vector<std::vector<double>>& u) {
  int64_t N = in->n_elems * in->nodes_per_elem;
  for (int i = 0; i < in->n_ic; ++i) {
    const double* ic = &in->ic[5 * i];
    double x = ic[0], y = ic[1], z = ic[2], size = ic[3], amp = ic[4];
    for (int64_t n = 0; n < N; n++) {
      double c[3];
      node_coords(in, n, c);
      u[0][n] += amp * std::exp(-((c[0] - x) * (c[0] - x) + (c[1] - y) * (c[1] - y) + (c[2] - z) * (c[2] - z)) / size);
    }
  }
}

void check_input(const refcpu_input* in) {
  if (!in || !in->xyz || !in->elem_nodes) throw std::runtime_error("null mesh arrays");
  if (in->n_elems <= 0) throw std::runtime_error("mesh has no elements");
  if (in->order < 1 || in->order > 4) throw std::runtime_error("order must be 1..4");
  if (in->dt <= 0) throw std::runtime_error("time step must be positive");
}

}  // namespace

extern "C" {

const char* refcpu_last_error(void) { return g_err.c_str(); }

void refcpu_count_steps(double t_start, double t_end, double dt, double t_rate, int64_t* n_steps, int64_t* n_snap) {
  int64_t ns = 0, nsn = 0;
  for (double t = t_start, step = 0, tDisplay = 0; t <= t_end; t += dt, tDisplay += dt, ++step) {
    if (tDisplay >= t_rate || step == 0) {
      tDisplay = 0;
      ++nsn;
    }
    ++ns;
  }
  *n_steps = ns;
  *n_snap = nsn;
}

int refcpu_initial_state(const refcpu_input* in, double* uout) {
  try {
    check_input(in);
    int64_t N = in->n_elems * in->nodes_per_elem;
    std::vector<std::vector<double>> u(4, std::vector<double>(N, 0.0));
    apply_ic(in, u);
    for (int q = 0; q < 4; ++q) std::copy(u[q].begin(), u[q].end(), uout + q * N);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int refcpu_faces(const refcpu_input* in, int64_t* face_id, int64_t* nbr, int* orient, int* bc, int* penalty) {
  try {
    check_input(in);
    RefMesh mesh;
    mesh.setup(in);
    const int Nf = mesh.m_fNumPerEl;
    for (int64_t el = 0; el < mesh.m_elNum; ++el)
      for (int lf = 0; lf < Nf; ++lf) {
        int64_t f = mesh.elFId(el, lf), k = el * Nf + lf;
        if (face_id) face_id[k] = f;
        bool b = mesh.m_fIsBoundary[f];
        if (nbr) nbr[k] = b ? -1 : (mesh.fNbrElId(f, 0) == el ? mesh.fNbrElId(f, 1) : mesh.fNbrElId(f, 0));
        if (orient) orient[k] = mesh.elFOrientation(el, lf);
        if (bc) bc[k] = b ? mesh.m_fBC[f] : -1;
        if (penalty) {
          if (b) {
            penalty[k] = 0;
          } else {
            int64_t up = mesh.fNbrElId(f, 0);
            int lfu = 0;
            for (int q = 0; q < Nf; ++q)
              if (mesh.elFId(up, q) == f) lfu = q;
            penalty[k] = mesh.fc * mesh.elFOrientation(up, lfu);
          }
        }
      }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int refcpu_stage(const refcpu_input* in, const double* uin, double* kout) {
  try {
    check_input(in);
    RefMesh mesh;
    mesh.setup(in);
    mesh.precomputeMassMatrix();
    Solver s(mesh);
    int64_t N = s.numNodes;
    std::vector<std::vector<double>> k(4, std::vector<double>(N));
    for (int q = 0; q < 4; ++q) std::copy(uin + q * N, uin + (q + 1) * N, k[q].begin());
    mesh.updateFlux(k, s.Flux);
    s.numStep(k, 0.0);
    for (int q = 0; q < 4; ++q) std::copy(k[q].begin(), k[q].end(), kout + q * N);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int refcpu_run(const refcpu_input* in, refcpu_output* out) {
  try {
    check_input(in);
    auto t0 = std::chrono::steady_clock::now();
    RefMesh mesh;
    mesh.setup(in);
    mesh.precomputeMassMatrix();
    Solver s(mesh);
    const int Np = s.Np;
    const int64_t numNodes = s.numNodes;
    const int T = mesh.nthreads;
    const double c0 = in->c0;

    // penalty-sign histogram over interior faces
    out->penalty_sign_hist[0] = out->penalty_sign_hist[1] = 0;
    out->n_faces = mesh.m_fNum;
    out->n_boundary_faces = 0;
    for (int64_t f = 0; f < mesh.m_fNum; ++f) {
      if (mesh.m_fIsBoundary[f]) {
        ++out->n_boundary_faces;
        continue;
      }
      int64_t up = mesh.fNbrElId(f, 0);
      for (int q = 0; q < mesh.m_fNumPerEl; ++q)
        if (mesh.elFId(up, q) == f) out->penalty_sign_hist[mesh.fc * mesh.elFOrientation(up, q) > 0 ? 1 : 0]++;
    }

    std::vector<std::vector<double>> u(4, std::vector<double>(numNodes, 0.0));
    apply_ic(in, u);

    // source / observer node sets (src/solver.cpp:339-383)
    std::vector<std::vector<int64_t>> srcIdx(in->n_src);
    for (int i = 0; i < in->n_src; ++i) {
      const double* sp = &in->src_params[8 * i];
      for (int64_t n = 0; n < numNodes; n++) {
        double c[3];
        node_coords(in, n, c);
        if (std::pow(c[0] - sp[0], 2) + std::pow(c[1] - sp[1], 2) + std::pow(c[2] - sp[2], 2) < std::pow(sp[3], 2))
          srcIdx[i].push_back(n);
      }
    }
    std::vector<std::vector<int64_t>> obsIdx(in->n_obs);
    std::vector<std::vector<double>> obsDist(in->n_obs);
    for (int i = 0; i < in->n_obs; ++i) {
      const double* o = &in->obs[4 * i];
      for (int64_t n = 0; n < numNodes; n++) {
        double c[3];
        node_coords(in, n, c);
        double d = std::sqrt(std::pow(c[0] - o[0], 2) + std::pow(c[1] - o[1], 2) + std::pow(c[2] - o[2], 2));
        if (d < o[3]) obsIdx[i].push_back(n), obsDist[i].push_back(d);
      }
    }
    std::vector<double> g_p(numNodes), g_rho(numNodes), g_v(3 * numNodes);
    auto t1 = std::chrono::steady_clock::now();
    out->setup_seconds = std::chrono::duration<double>(t1 - t0).count();

    std::vector<std::vector<double>> k1, k2, k3, k4;
    int64_t step_i = 0, nsnap = 0;
    for (double t = in->t_start, step = 0, tDisplay = 0; t <= in->t_end; t += in->dt, tDisplay += in->dt, ++step) {
      if (in->max_steps >= 0 && step_i >= in->max_steps) break;
      if (tDisplay >= in->t_rate || step == 0) {
        tDisplay = 0;
#pragma omp parallel for schedule(static) num_threads(T)
        for (int el = 0; el < mesh.m_elNum; ++el)
          for (int n = 0; n < Np; ++n) {
            int64_t elN = (int64_t)el * Np + n;
            g_p[elN] = u[0][elN];
            g_rho[elN] = u[0][elN] / (c0 * c0);
            g_v[3 * elN + 0] = u[1][elN];
            g_v[3 * elN + 1] = u[2][elN];
            g_v[3 * elN + 2] = u[3][elN];
          }
        if (out->snapshot_steps) out->snapshot_steps[nsnap] = step_i;
        ++nsnap;
      }
      // sources (src/solver.cpp:455-483)
      for (int src = 0; src < in->n_src; ++src) {
        const double* sp = &in->src_params[8 * src];
        int kind = in->src_kind[src];
        if (kind == REFCPU_SRC_SINE) {
          double amp = sp[4], freq = sp[5], phase = sp[6], duration = sp[7];
          if (t < duration)
            for (int64_t n : srcIdx[src]) u[0][n] = amp * std::sin(2 * M_PI * freq * t + phase);
        } else if (kind == REFCPU_SRC_CALLBACK) {
          double duration = sp[7];
          if (t < duration)
            for (int64_t n : srcIdx[src]) u[0][n] = in->src_fn(src, t, in->src_user);
        } else {
          const double* tab = &in->src_table[2 * in->src_table_offsets[src]];
          int64_t rows = in->src_table_offsets[src + 1] - in->src_table_offsets[src];
          for (int64_t n : srcIdx[src]) u[0][n] = interpolate_value(tab, rows, t);
        }
      }
      if (in->method == 0) {
        // RK4 (src/solver.cpp:488-516)
        k1 = k2 = k3 = k4 = u;
        mesh.updateFlux(k1, s.Flux);
        s.numStep(k1, 0);
        for (int eq = 0; eq < 4; ++eq)
          for (int64_t i = 0; i < numNodes; ++i) k2[eq][i] += 0.5 * k1[eq][i];
        mesh.updateFlux(k2, s.Flux);
        s.numStep(k2, 0);
        for (int eq = 0; eq < 4; ++eq)
          for (int64_t i = 0; i < numNodes; ++i) k3[eq][i] += 0.5 * k2[eq][i];
        mesh.updateFlux(k3, s.Flux);
        s.numStep(k3, 0);
        for (int eq = 0; eq < 4; ++eq)
          for (int64_t i = 0; i < numNodes; ++i) k4[eq][i] += 1 * k3[eq][i];
        mesh.updateFlux(k4, s.Flux);
        s.numStep(k4, 0);
        for (int eq = 0; eq < 4; ++eq)
          for (int64_t i = 0; i < numNodes; ++i) u[eq][i] += (k1[eq][i] + 2 * k2[eq][i] + 2 * k3[eq][i] + k4[eq][i]) / 6.0;
      } else {
        // Euler1 (src/solver.cpp:229-230): u = dt M^-1 (S - F) + u
        mesh.updateFlux(u, s.Flux);
        s.numStep(u, 1);
      }
      // residuals (src/solver.cpp:518-545)
      double residual[5] = {0, 0, 0, 0, 0};
#pragma omp parallel for schedule(static) num_threads(T)
      for (int el = 0; el < mesh.m_elNum; ++el)
        for (int n = 0; n < Np; ++n) {
          int64_t elN = (int64_t)el * Np + n;
#pragma omp atomic update
          residual[0] += std::pow(g_p[elN] - u[0][elN], 2);
#pragma omp atomic update
          residual[1] += std::pow(g_rho[elN] - u[0][elN] / (c0 * c0), 2);
#pragma omp atomic update
          residual[2] += std::pow(g_v[3 * elN + 0] - u[1][elN], 2);
#pragma omp atomic update
          residual[3] += std::pow(g_v[3 * elN + 1] - u[2][elN], 2);
#pragma omp atomic update
          residual[4] += std::pow(g_v[3 * elN + 2] - u[3][elN], 2);
        }
      if (out->times) out->times[step_i] = t;
      for (int eq = 0; eq < 5; ++eq) {
        residual[eq] /= (double)(mesh.m_elNum * Np);
        if (out->residuals) out->residuals[step_i * 5 + eq] = residual[eq];
      }
      // observers (src/solver.cpp:552-573)
      for (int obs = 0; obs < in->n_obs; ++obs) {
        double p = 0, rho = 0, w_sum = 0, v[3] = {0, 0, 0};
        for (size_t n = 0; n < obsIdx[obs].size(); ++n) {
          double w = 1.0 / (std::pow(obsDist[obs][n], 2) + 1.0e-12);
          p += u[0][obsIdx[obs][n]] * w;
          v[0] += u[1][obsIdx[obs][n]] * w;
          v[1] += u[2][obsIdx[obs][n]] * w;
          v[2] += u[3][obsIdx[obs][n]] * w;
          w_sum += w;
        }
        p /= w_sum;
        rho = p / std::pow(c0, 2);
        v[0] /= w_sum, v[1] /= w_sum, v[2] /= w_sum;
        if (out->obs_trace) {
          double* o = &out->obs_trace[(step_i * in->n_obs + obs) * 5];
          o[0] = rho, o[1] = p, o[2] = v[0], o[3] = v[1], o[4] = v[2];
        }
      }
      ++step_i;
    }
    auto t2 = std::chrono::steady_clock::now();
    out->loop_seconds = std::chrono::duration<double>(t2 - t1).count();
    out->steps_done = step_i;
    out->n_snap = nsnap;
    if (out->state)
      for (int q = 0; q < 4; ++q) std::copy(u[q].begin(), u[q].end(), out->state + q * numNodes);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

int refcpu_rule(int kind, int degree, int* n, double* x, double* w) {
  try {
    Rule r = kind == 1 ? gauss_line(degree) : kind == 2 ? tri_rule(degree) : tet_rule(degree);
    *n = r.n;
    if (x) std::copy(r.x.begin(), r.x.end(), x);
    if (w) std::copy(r.w.begin(), r.w.end(), w);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"
