// Quadrature rules of the curved-element path; see quadrature.h.
#include "quadrature.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace dgref {
namespace {

// Jacobi polynomial P_n^(a,0)(x) and its derivative by the three-term
// recurrence (and its derivative).
void jacobi_a0(int n, double a, double x, double& p, double& dp) {
  double pm = 1.0, dpm = 0.0;
  if (n == 0) {
    p = pm, dp = dpm;
    return;
  }
  double pc = 0.5 * ((a + 2.0) * x + a), dpc = 0.5 * (a + 2.0);
  for (int k = 2; k <= n; ++k) {
    const double s = 2.0 * k + a;
    const double den = 2.0 * k * (k + a) * (s - 2.0);
    const double lin = (s - 1.0) * (s * (s - 2.0) * x + a * a);
    const double back = 2.0 * (k + a - 1.0) * (k - 1.0) * s;
    const double pn = (lin * pc - back * pm) / den;
    const double dpn = (lin * dpc + (s - 1.0) * s * (s - 2.0) * pc - back * dpm) / den;
    pm = pc, dpm = dpc, pc = pn, dpc = dpn;
  }
  p = pc, dp = dpc;
}

// Gauss-Jacobi rule for the weight (1 - x)^a on [-1, 1]: Newton's method on
// P_n^(a,0) with the roots already found divided out, from Chebyshev starting
// points; ascending nodes.
void gauss_jacobi_a0(int n, double a, std::vector<double>& x, std::vector<double>& w) {
  x.clear(), w.clear();
  for (int k = 0; k < n; ++k) {
    double r = -std::cos((2.0 * k + 1.0) * M_PI / (2.0 * n));
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      jacobi_a0(n, a, r, p, dp);
      double s = 0.0;
      for (double q : x) s += 1.0 / (r - q);
      const double step = p / (dp - p * s);
      r -= step;
      if (std::fabs(step) <= 1e-17 * (1.0 + std::fabs(r))) break;
    }
    // polish on the undeflated polynomial
    for (int it = 0; it < 3; ++it) {
      double p, dp;
      jacobi_a0(n, a, r, p, dp);
      r -= p / dp;
    }
    x.push_back(r);
  }
  std::sort(x.begin(), x.end());
  for (double r : x) {
    double p, dp;
    jacobi_a0(n, a, r, p, dp);
    w.push_back(std::pow(2.0, a + 1.0) / ((1.0 - r * r) * dp * dp));
  }
}

// Triangle points from barycentric coordinates (b0, b1, b2) -> (b1, b2);
// published weights are normalised to area 1, the rule's to 1/2.
struct TriBuilder {
  QRule r;
  TriBuilder() { r.dim = 2; }
  void point(double b0, double b1, double b2, double wt) {
    (void)b0;
    r.x.push_back(b1), r.x.push_back(b2), r.w.push_back(0.5 * wt), ++r.n;
  }
  // orbit of (a, a, 1 - 2a): the three points, starting from rotation `lead`
  void orbit3(double a, double wt, int lead) {
    const double c = 1.0 - 2.0 * a;
    const double pts[3][3] = {{c, a, a}, {a, c, a}, {a, a, c}};
    for (int k = 0; k < 3; ++k) {
      const double* q = pts[(lead + k) % 3];
      point(q[0], q[1], q[2], wt);
    }
  }
  // orbit of (a, b, 1 - a - b): the six points in a fixed order
  void orbit6(double a, double b, double wt) {
    const double c = 1.0 - a - b;
    const double pts[6][3] = {{a, b, c}, {b, c, a}, {c, a, b}, {b, a, c}, {a, c, b}, {c, b, a}};
    for (const auto& q : pts) point(q[0], q[1], q[2], wt);
  }
};

// Tetrahedron points from barycentric quadruples (b0..b3) -> (b1, b2, b3);
// published weights are normalised to volume 1, the rule's to 1/6.
struct TetBuilder {
  QRule r;
  TetBuilder() { r.dim = 3; }
  // all distinct permutations of the quadruple, in lexicographic order
  void orbit(double a, double b, double c, double d, double wt) {
    double v[4] = {a, b, c, d};
    std::sort(v, v + 4);
    do {
      r.x.push_back(v[1]), r.x.push_back(v[2]), r.x.push_back(v[3]);
      r.w.push_back(wt / 6.0), ++r.n;
    } while (std::next_permutation(v, v + 4));
  }
};

}  // namespace

QRule gauss_legendre(int n) {
  QRule r;
  r.dim = 1;
  gauss_jacobi_a0(n, 0.0, r.x, r.w);
  r.n = n;
  return r;
}

QRule triangle_rule(int degree) {
  TriBuilder t;
  if (degree <= 2) {
    t.orbit3(1.0 / 6.0, 1.0 / 3.0, 0);
  } else if (degree <= 4) {
    t.orbit3(0.445948490915965, 0.223381589678011, 0);
    t.orbit3(0.091576213509771, 0.109951743655322, 0);
  } else if (degree <= 6) {
    t.orbit6(0.053145049844817, 0.310352451033784, 0.082851075618374);
    t.orbit3(0.249286745170910, 0.116786275726379, 0);
    t.orbit3(0.063089014491502, 0.050844906370207, 0);
  } else if (degree <= 8) {
    // the (a, 1 - 2a, a) point leads
    const double a = 0.050547228317031, c = 1.0 - 2.0 * a, wa = 0.032458497623198;
    t.point(a, c, a, wa);
    t.point(c, a, a, wa);
    t.point(a, a, c, wa);
    t.point(1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 0.144315607677787);
    t.orbit3(0.459292588292723, 0.095091634267285, 0);
    t.orbit3(0.170569307751760, 0.103217370534718, 0);
    t.orbit6(0.008394777409958, 0.263112829634638, 0.027230314174435);
  } else {
    throw std::runtime_error("triangle rules above degree 8 are not available");
  }
  return t.r;
}

QRule tetrahedron_rule(int degree) {
  TetBuilder t;
  if (degree <= 2) {
    const double a = 0.1381966011250105;
    t.orbit(a, a, a, 1.0 - 3.0 * a, 0.25);
  } else if (degree <= 4) {
    t.orbit(0.25, 0.25, 0.25, 0.25, -0.0789333333333333);
    const double a = 0.0714285714285714;
    t.orbit(a, a, a, 1.0 - 3.0 * a, 0.0457333333333333);
    const double b = 0.399403576166799;
    t.orbit(b, b, 0.5 - b, 0.5 - b, 0.149333333333333);
  } else if (degree <= 6) {
    const double a1 = 0.214602871259151, a2 = 0.0406739585346113, a3 = 0.322337890142275;
    t.orbit(a1, a1, a1, 1.0 - 3.0 * a1, 6.0 * 0.00665379170969465);
    t.orbit(a2, a2, a2, 1.0 - 3.0 * a2, 6.0 * 0.00167953517588678);
    t.orbit(a3, a3, a3, 1.0 - 3.0 * a3, 6.0 * 0.00922619692394239);
    const double a = 0.0636610018750175, b = 0.269672331458316;
    t.orbit(a, a, b, 1.0 - 2.0 * a - b, 6.0 * 0.00803571428571428);
  } else if (degree <= 9) {
    // Stroud conical product of 5-point Gauss-Jacobi rules with weights
    // (1-x)^0, (1-x)^1, (1-x)^2 (Duffy collapse of the unit cube)
    std::vector<double> xa, wa, xb, wb, xc, wc;
    gauss_jacobi_a0(5, 0.0, xa, wa);
    gauss_jacobi_a0(5, 1.0, xb, wb);
    gauss_jacobi_a0(5, 2.0, xc, wc);
    QRule& r = t.r;
    for (int i = 0; i < 5; ++i)
      for (int j = 0; j < 5; ++j)
        for (int k = 0; k < 5; ++k) {
          const double A = 0.5 * (1.0 + xa[i]), B = 0.5 * (1.0 + xb[j]), Cc = 0.5 * (1.0 + xc[k]);
          const double wt = wa[i] * 0.5 * wb[j] * 0.25 * wc[k] * 0.125;
          r.x.push_back(A * (1.0 - B) * (1.0 - Cc)), r.x.push_back(B * (1.0 - Cc)), r.x.push_back(Cc);
          r.w.push_back(wt), ++r.n;
        }
  } else {
    throw std::runtime_error("tetrahedron rules above degree 9 are not available");
  }
  return t.r;
}

QRule element_rule(int dim, int p) { return dim == 2 ? triangle_rule(2 * p) : tetrahedron_rule(2 * p); }

QRule face_rule(int dim, int p) { return dim == 2 ? gauss_legendre(p + 1) : triangle_rule(2 * p); }

}  // namespace dgref
