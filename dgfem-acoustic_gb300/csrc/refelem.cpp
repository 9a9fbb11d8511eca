#include "refelem.h"

#include "quadrature.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace dgref {

namespace {

double fact(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; ++i) f *= i;
  return f;
}

// Exact integral of x^a y^b [z^c] over the unit reference simplex of dim d.
double mono_int(int d, const int* e) {
  double num = 1.0;
  int s = 0;
  for (int k = 0; k < d; ++k) num *= fact(e[k]), s += e[k];
  return num / fact(s + d);
}

// Gauss-Jordan inverse with partial pivoting (row-major, in place).
void invert(std::vector<double>& A, int n) {
  std::vector<double> I(n * n, 0.0);
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > std::fabs(A[piv * n + k])) piv = i;
    if (A[piv * n + k] == 0.0) throw std::runtime_error("singular reference matrix");
    if (piv != k)
      for (int j = 0; j < n; ++j) std::swap(A[k * n + j], A[piv * n + j]), std::swap(I[k * n + j], I[piv * n + j]);
    double d = A[k * n + k];
    for (int j = 0; j < n; ++j) A[k * n + j] /= d, I[k * n + j] /= d;
    for (int i = 0; i < n; ++i) {
      if (i == k || A[i * n + k] == 0.0) continue;
      double l = A[i * n + k];
      for (int j = 0; j < n; ++j) A[i * n + j] -= l * A[k * n + j], I[i * n + j] -= l * I[k * n + j];
    }
  }
  A = I;
}

// Monomial exponents of total degree <= p in d variables.
std::vector<int> monomials(int d, int p) {
  std::vector<int> e;
  if (d == 1) {
    for (int a = 0; a <= p; ++a) e.push_back(a);
  } else if (d == 2) {
    for (int s = 0; s <= p; ++s)
      for (int a = s; a >= 0; --a) e.push_back(a), e.push_back(s - a);
  } else {
    for (int s = 0; s <= p; ++s)
      for (int a = s; a >= 0; --a)
        for (int b = s - a; b >= 0; --b) e.push_back(a), e.push_back(b), e.push_back(s - a - b);
  }
  return e;
}

// Lagrange basis coefficients on nodes (d coords each): C = V^-1, phi_i = sum_k C[k][i] m_k.
std::vector<double> lagrange_coeffs(int d, int p, const std::vector<double>& nodes, const std::vector<int>& ex) {
  int n = (int)ex.size() / d;
  std::vector<double> V(n * n);
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < n; ++k) {
      double v = 1.0;
      for (int a = 0; a < d; ++a) v *= std::pow(nodes[i * d + a], ex[k * d + a]);
      V[i * n + k] = v;
    }
  invert(V, n);
  return V;
}

// Gram of the Lagrange basis under the bilinear form given by monomial moments.
template <class MomentFn>
std::vector<double> gram(int n, const std::vector<double>& Ca, const std::vector<double>& Cb, MomentFn mom) {
  std::vector<double> G(n * n, 0.0), Mk(n * n);
  for (int k = 0; k < n; ++k)
    for (int l = 0; l < n; ++l) Mk[k * n + l] = mom(k, l);
  // G[i][j] = sum_kl Ca[k][i] Mk[k][l] Cb[l][j]
  std::vector<double> T(n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int l = 0; l < n; ++l) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += Ca[k * n + i] * Mk[k * n + l];
      T[i * n + l] = s;
    }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int l = 0; l < n; ++l) s += T[i * n + l] * Cb[l * n + j];
      G[i * n + j] = s;
    }
  return G;
}

// Equispaced vertex basis function of order p as a function of its
// barycentric coordinate, and its derivative.
double vertex_fn_deriv(int p, double lam) {
  // phi(l) = prod_{k<p} (p l - k)/(p - k)
  double d = 0.0;
  for (int q = 0; q < p; ++q) {
    double term = (double)p / (p - q);
    for (int k = 0; k < p; ++k)
      if (k != q) term *= (p * lam - k) / (double)(p - k);
    d += term;
  }
  return d;
}

double first_gauss_point(int n) {
  // smallest root of the Legendre polynomial P_n (ascending order)
  double x = -std::cos(M_PI * (0.75) / (n + 0.5));
  for (int it = 0; it < 100; ++it) {
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= n; ++k) {
      double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
      p0 = p1, p1 = p2;
    }
    double dp = n * (x * p1 - p0) / (x * x - 1.0);
    double dx = p1 / dp;
    x -= dx;
    if (std::fabs(dx) < 1e-16) break;
  }
  return x;
}

const int kTriEdges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kTetFaces[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {3, 1, 2}};

}  // namespace

int lattice_index(const RefElement& re, const int* ijk) {
  int p = re.p;
  if (re.dim == 1) return (ijk[0] >= 0 && ijk[0] <= p) ? ijk[0] : -1;
  if (re.dim == 2) {
    int i = ijk[0], j = ijk[1];
    if (i < 0 || j < 0 || i + j > p) return -1;
    int idx = 0;
    for (int jj = 0; jj < j; ++jj) idx += p - jj + 1;
    return idx + i;
  }
  int i = ijk[0], j = ijk[1], k = ijk[2];
  if (i < 0 || j < 0 || k < 0 || i + j + k > p) return -1;
  int idx = 0;
  for (int kk = 0; kk < k; ++kk) idx += (p - kk + 1) * (p - kk + 2) / 2;
  for (int jj = 0; jj < j; ++jj) idx += p - k - jj + 1;
  return idx + i;
}

void face_rule_head(int p, double bary[3][3]) {
  // Leading points of the oracle's degree-2p triangle rules (tri_rule in
  // oracle/refcpu.cpp): orbit heads chosen there.
  const double a2 = 1.0 / 6.0, c2 = 1.0 - 2.0 * a2;
  const double a4 = 0.445948490915965, c4 = 1.0 - 2.0 * a4;
  const double a6 = 0.053145049844817, b6 = 0.310352451033784, c6 = 1.0 - a6 - b6;
  const double a8 = 0.050547228317031, c8 = 1.0 - 2.0 * a8;
  double P[3][3];
  switch (p) {
    case 1: {
      double q[3][3] = {{c2, a2, a2}, {a2, c2, a2}, {a2, a2, c2}};
      std::copy(&q[0][0], &q[0][0] + 9, &P[0][0]);
      break;
    }
    case 2: {
      double q[3][3] = {{c4, a4, a4}, {a4, c4, a4}, {a4, a4, c4}};
      std::copy(&q[0][0], &q[0][0] + 9, &P[0][0]);
      break;
    }
    case 3: {
      double q[3][3] = {{a6, b6, c6}, {b6, c6, a6}, {c6, a6, b6}};
      std::copy(&q[0][0], &q[0][0] + 9, &P[0][0]);
      break;
    }
    default: {
      double q[3][3] = {{a8, c8, a8}, {c8, a8, a8}, {a8, a8, c8}};
      std::copy(&q[0][0], &q[0][0] + 9, &P[0][0]);
      break;
    }
  }
  std::copy(&P[0][0], &P[0][0] + 9, &bary[0][0]);
}

int recipe_normal_sign(int dim, int p) {
  if (dim == 2) {
    double s = first_gauss_point(p + 1);
    double lam0 = 0.5 * (1.0 - s);
    return vertex_fn_deriv(p, lam0) > 0 ? 1 : -1;
  }
  double b[3][3];
  face_rule_head(p, b);
  double f = vertex_fn_deriv(p, b[0][0]) * vertex_fn_deriv(p, b[0][1]);
  return f > 0 ? 1 : -1;
}

RefElement build(int dim, int p) {
  if (dim < 1 || dim > 3) throw std::runtime_error("dim must be 1, 2 or 3");
  if (p < 1 || p > kMaxP) throw std::runtime_error("order must be 1..4");
  RefElement re;
  re.dim = dim, re.p = p;
  re.np = dim == 1 ? p + 1 : dim == 2 ? (p + 1) * (p + 2) / 2 : (p + 1) * (p + 2) * (p + 3) / 6;
  re.nf = dim + 1;
  re.nfp = dim == 1 ? 1 : dim == 2 ? p + 1 : (p + 1) * (p + 2) / 2;
  re.ref_measure = dim == 1 ? 1.0 : dim == 2 ? 0.5 : 1.0 / 6.0;
  re.face_ref_measure = dim == 3 ? 0.5 : 1.0;  // a point face has measure 1
  // lattice in internal order
  re.lattice.clear();
  if (dim == 1) {
    for (int i = 0; i <= p; ++i) re.lattice.push_back(i);
  } else if (dim == 2) {
    for (int j = 0; j <= p; ++j)
      for (int i = 0; i <= p - j; ++i) re.lattice.push_back(i), re.lattice.push_back(j);
  } else {
    for (int k = 0; k <= p; ++k)
      for (int j = 0; j <= p - k; ++j)
        for (int i = 0; i <= p - j - k; ++i) re.lattice.push_back(i), re.lattice.push_back(j), re.lattice.push_back(k);
  }
  const int np = re.np, nf = re.nf, nfp = re.nfp, D = dim;
  // vertex barycentric (times p) of internal node n
  auto bary = [&](int n, int v) {
    if (v == 0) {
      int s = p;
      for (int d = 0; d < D; ++d) s -= re.lattice[n * D + d];
      return s;
    }
    return re.lattice[n * D + v - 1];
  };
  for (int f = 0; f < nf; ++f)
    // lines: local face f is the end point at vertex f
    for (int k = 0; k < D; ++k) re.face_corners[f][k] = D == 1 ? f : D == 2 ? kTriEdges[f][k] : kTetFaces[f][k];
  // face lattice: (a1, a2) with a0 = p - a1 - a2, a2 outer
  std::vector<int> flat;  // nfp * 3 face barycentrics (a0,a1,a2)
  if (D == 1) {
    flat.push_back(p), flat.push_back(0), flat.push_back(0);
  } else if (D == 2) {
    for (int a1 = 0; a1 <= p; ++a1) flat.push_back(p - a1), flat.push_back(a1), flat.push_back(0);
  } else {
    for (int a2 = 0; a2 <= p; ++a2)
      for (int a1 = 0; a1 <= p - a2; ++a1) flat.push_back(p - a1 - a2), flat.push_back(a1), flat.push_back(a2);
  }
  auto face_index = [&](int a0, int a1, int a2) {
    for (int m = 0; m < nfp; ++m)
      if (flat[m * 3] == a0 && flat[m * 3 + 1] == a1 && flat[m * 3 + 2] == a2) return m;
    return -1;
  };
  re.fmask.assign(nf * nfp, -1);
  for (int f = 0; f < nf; ++f) {
    const int* c = re.face_corners[f];
    for (int m = 0; m < nfp; ++m) {
      for (int n = 0; n < np; ++n) {
        bool ok = true;
        int sum = 0;
        for (int k = 0; k < D; ++k) ok &= bary(n, c[k]) == flat[m * 3 + k], sum += bary(n, c[k]);
        if (ok && sum == p) {
          re.fmask[f * nfp + m] = n;
          break;
        }
      }
      if (re.fmask[f * nfp + m] < 0) throw std::runtime_error("face mask construction failed");
    }
  }
  // permutations of the face corners: our corner k sits at neighbour position perm[k]
  re.nperm = D == 1 ? 1 : D == 2 ? 2 : 6;
  const int perms3[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int perms2[2][3] = {{0, 1, 2}, {1, 0, 2}};
  for (int q = 0; q < re.nperm; ++q)
    for (int k = 0; k < 3; ++k) re.perm_table[q][k] = D == 3 ? perms3[q][k] : perms2[q][k];
  re.nbrnode.assign(nf * re.nperm * nfp, -1);
  for (int lf = 0; lf < nf; ++lf)
    for (int q = 0; q < re.nperm; ++q)
      for (int m = 0; m < nfp; ++m) {
        int b[3] = {0, 0, 0};
        for (int k = 0; k < D; ++k) b[re.perm_table[q][k]] = flat[m * 3 + k];
        int mn = face_index(b[0], b[1], b[2]);
        re.nbrnode[(lf * re.nperm + q) * nfp + m] = re.fmask[lf * nfp + mn];
      }
  // volume operators
  std::vector<double> nodes(np * D);
  for (int n = 0; n < np; ++n)
    for (int d = 0; d < D; ++d) nodes[n * D + d] = (double)re.lattice[n * D + d] / p;
  auto ex = monomials(D, p);
  auto C = lagrange_coeffs(D, p, nodes, ex);
  re.Mref = gram(np, C, C, [&](int k, int l) {
    int e[3];
    for (int d = 0; d < D; ++d) e[d] = ex[k * D + d] + ex[l * D + d];
    return mono_int(D, e);
  });
  re.Minv = re.Mref;
  invert(re.Minv, np);
  re.Dt.assign(D * np * np, 0.0);
  for (int r = 0; r < D; ++r) {
    // K_r[i][j] = int d_r(phi_i) phi_j
    auto K = gram(np, C, C, [&](int k, int l) {
      int a = ex[k * D + r];
      if (a == 0) return 0.0;
      int e[3];
      for (int d = 0; d < D; ++d) e[d] = ex[k * D + d] + ex[l * D + d] - (d == r ? 1 : 0);
      return a * mono_int(D, e);
    });
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) {
        double s = 0.0;
        for (int k = 0; k < np; ++k) s += re.Minv[i * np + k] * K[k * np + j];
        re.Dt[(r * np + i) * np + j] = s;
      }
  }
  // face mass on the face lattice (face coordinates a1/p [, a2/p]); a point
  // face (lines) has the 1 x 1 mass 1
  if (D == 1) {
    re.Mf.assign(1, 1.0);
  } else {
    std::vector<double> fnodes(nfp * (D - 1));
    for (int m = 0; m < nfp; ++m)
      for (int d = 0; d < D - 1; ++d) fnodes[m * (D - 1) + d] = (double)flat[m * 3 + 1 + d] / p;
    auto fex = monomials(D - 1, p);
    auto FC = lagrange_coeffs(D - 1, p, fnodes, fex);
    re.Mf = gram(nfp, FC, FC, [&](int k, int l) {
      int e[3];
      for (int d = 0; d < D - 1; ++d) e[d] = fex[k * (D - 1) + d] + fex[l * (D - 1) + d];
      return mono_int(D - 1, e);
    });
  }
  // LIFT = Minv E_f Mf, columns grouped by face
  re.LIFT.assign(np * nf * nfp, 0.0);
  for (int f = 0; f < nf; ++f)
    for (int i = 0; i < np; ++i)
      for (int m = 0; m < nfp; ++m) {
        double s = 0.0;
        for (int mm = 0; mm < nfp; ++mm) s += re.Minv[i * np + re.fmask[f * nfp + mm]] * re.Mf[mm * nfp + m];
        re.LIFT[i * (nf * nfp) + f * nfp + m] = s;
      }
  return re;
}

CurvedTables build_curved(const RefElement& re) {
  const int D = re.dim, p = re.p, np = re.np, nf = re.nf, nfp = re.nfp;
  std::vector<double> nodes(np * D);
  for (int n = 0; n < np; ++n)
    for (int d = 0; d < D; ++d) nodes[n * D + d] = (double)re.lattice[n * D + d] / p;
  const auto ex = monomials(D, p);
  const auto C = lagrange_coeffs(D, p, nodes, ex);
  const int nm = (int)ex.size() / D;
  // phi_j(xi) and d phi_j / d xi_r
  auto eval = [&](const double* xi, double* phi, double* dphi /* [D][np] */) {
    std::vector<double> m(nm), dm(D * nm);
    for (int k = 0; k < nm; ++k) {
      double v = 1.0;
      for (int d = 0; d < D; ++d) v *= std::pow(xi[d], ex[k * D + d]);
      m[k] = v;
      for (int r = 0; r < D; ++r) {
        const int a = ex[k * D + r];
        double g = 0.0;
        if (a > 0) {
          g = a * std::pow(xi[r], a - 1);
          for (int d = 0; d < D; ++d)
            if (d != r) g *= std::pow(xi[d], ex[k * D + d]);
        }
        dm[r * nm + k] = g;
      }
    }
    for (int j = 0; j < np; ++j) {
      double s = 0.0;
      for (int k = 0; k < nm; ++k) s += C[k * np + j] * m[k];
      if (phi) phi[j] = s;
      for (int r = 0; r < D && dphi; ++r) {
        double g = 0.0;
        for (int k = 0; k < nm; ++k) g += C[k * np + j] * dm[r * nm + k];
        dphi[r * np + j] = g;
      }
    }
  };
  CurvedTables t;
  const QRule er = element_rule(D, p), fr = face_rule(D, p);
  t.ng = er.n, t.ngf = fr.n;
  t.qw = er.w, t.fw = fr.w;
  t.qB.assign((size_t)t.ng * np, 0.0);
  t.qD.assign((size_t)D * t.ng * np, 0.0);
  std::vector<double> dphi(D * np);
  for (int g = 0; g < t.ng; ++g) {
    eval(&er.x[g * D], &t.qB[(size_t)g * np], dphi.data());
    for (int r = 0; r < D; ++r)
      for (int j = 0; j < np; ++j) t.qD[((size_t)r * t.ng + g) * np + j] = dphi[r * np + j];
  }
  // reference coordinates of the mesh corners: vertex 0 at the origin,
  // vertex k at the unit vector e_k
  auto corner = [&](int c, double* xi) {
    for (int d = 0; d < D; ++d) xi[d] = (c > 0 && d == c - 1) ? 1.0 : 0.0;
  };
  t.fB.assign((size_t)nf * t.ngf * nfp, 0.0);
  t.fTu.assign((size_t)nf * t.ngf * np, 0.0);
  if (D == 3) t.fTv.assign((size_t)nf * t.ngf * np, 0.0);
  std::vector<double> phi(np);
  for (int lf = 0; lf < nf; ++lf) {
    double c0[3], c1[3], c2[3] = {0, 0, 0};
    corner(re.face_corners[lf][0], c0), corner(re.face_corners[lf][1], c1);
    if (D == 3) corner(re.face_corners[lf][2], c2);
    double du[3], dv[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) {
      // 2-D: u in [-1, 1] from corner 0 to corner 1; 3-D: (u, v) on the
      // unit triangle with corners 0, 1, 2 at (0,0), (1,0), (0,1)
      du[d] = D == 2 ? 0.5 * (c1[d] - c0[d]) : c1[d] - c0[d];
      if (D == 3) dv[d] = c2[d] - c0[d];
    }
    for (int g = 0; g < t.ngf; ++g) {
      double xi[3];
      if (D == 2) {
        const double u = fr.x[g];
        for (int d = 0; d < D; ++d) xi[d] = c0[d] * 0.5 * (1.0 - u) + c1[d] * 0.5 * (1.0 + u);
      } else {
        const double u = fr.x[g * 2], v = fr.x[g * 2 + 1];
        for (int d = 0; d < D; ++d) xi[d] = c0[d] * (1.0 - u - v) + c1[d] * u + c2[d] * v;
      }
      eval(xi, phi.data(), dphi.data());
      for (int m = 0; m < nfp; ++m) t.fB[((size_t)lf * t.ngf + g) * nfp + m] = phi[re.fmask[lf * nfp + m]];
      for (int j = 0; j < np; ++j) {
        double a = 0.0, b = 0.0;
        for (int r = 0; r < D; ++r) a += dphi[r * np + j] * du[r], b += dphi[r * np + j] * dv[r];
        t.fTu[((size_t)lf * t.ngf + g) * np + j] = a;
        if (D == 3) t.fTv[((size_t)lf * t.ngf + g) * np + j] = b;
      }
    }
  }
  return t;
}

}  // namespace dgref
