// Curved (non-affine) elements: setup of the per-element quadrature data and
// the per-stage right-hand side; see curved.cuh.
//
// The right-hand side follows the reference's formulation element by element
// (src/Mesh.cpp:734-975, src/solver.cpp:38-57) with the LEE flux being linear
// in the state, so that the nodal fluxes interpolated to a quadrature point
// equal the flux of the interpolated state:
//   S_i  = sum_g sum_r dphi_i/dxi_r(g) sum_d A_g[r][d] F_d(u(x_g))
//   face: per face point, the numerical flux of Mesh.cpp:761-813 with the
//         point's own normal (interior: central flux plus penalty s_f c0/2
//         times the jump; boundary: the ghost flux of Mesh.cpp:851-975 on the
//         interpolated trace, reflecting or RKR), weighted by w_g |J_f,g| and
//         tested with the face basis
//   rhs  = M^-T (S - sum_faces ...)
// One block per curved element; the elements are few next to the affine
// ones (the boundary layer of a curved geometry), so the kernel is written
// for clarity, not for the roofline.
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "ctx.h"
#include "curved.cuh"

namespace {

struct GeomDev {
  int D, np, nf, nfp, ng, ngf;
  const double* xyz;
  const int64_t* en;
  const int* perm;
  const double* det_aff;
  const int64_t* celem;
  const double *qw, *qB, *qD, *fw, *fB, *fTu, *fTv;
  const short* fmask;
  double *A, *Minv, *F, *TB;
  int* err;
};

__device__ void unit3(double* a) {
  const double z = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (z > 0.0) {
    const double r = sqrt(z);
    a[0] /= r, a[1] /= r, a[2] /= r;
  }
}

// One block per curved element: Jacobians at the element points, the mass
// matrix and its inverse, the face-point normals and weights, the 3-D face
// tangent frames.
__global__ void __launch_bounds__(128) k_curved_geom(GeomDev s) {
  extern __shared__ __align__(16) double smd[];
  __shared__ int piv;
  const int np = s.np, D = s.D, ng = s.ng, w2 = 2 * s.np;
  double* sx = smd;               // [np][3] node coordinates, internal order
  double* sw = sx + 3 * np;       // [ng] w_g det J_g
  double* aug = sw + ng;          // [np][2 np]
  double* col = aug + np * w2;    // [np] elimination factors
  const int slot = blockIdx.x, tid = threadIdx.x, NT = blockDim.x;
  const int64_t e = s.celem[slot];
  const double sg = s.det_aff[e] > 0.0 ? 1.0 : -1.0;
  for (int n = tid; n < np; n += NT) {
    const int64_t node = s.en[e * np + n];
    const int ii = s.perm[n];
    for (int d = 0; d < 3; ++d) sx[ii * 3 + d] = s.xyz[node * 3 + d];
  }
  __syncthreads();
  for (int g = tid; g < ng; g += NT) {
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // J[d][r] = dx_d / dxi_r
    for (int j = 0; j < np; ++j)
      for (int r = 0; r < D; ++r) {
        const double dphi = s.qD[((size_t)r * ng + g) * np + j];
        for (int d = 0; d < D; ++d) J[d][r] += sx[j * 3 + d] * dphi;
      }
    double det, Gi[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (D == 2) {
      det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      Gi[0][0] = J[1][1] / det, Gi[0][1] = -J[0][1] / det;
      Gi[1][0] = -J[1][0] / det, Gi[1][1] = J[0][0] / det;
    } else {
      det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
            J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      Gi[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
      Gi[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
      Gi[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
      Gi[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
      Gi[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
      Gi[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
      Gi[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
      Gi[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
      Gi[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    }
    if (!(det * sg > 0.0)) atomicOr(s.err, 1);  // degenerate or inverted inside the element
    const double wd = s.qw[g] * det;
    sw[g] = wd;
    double* A = s.A + ((size_t)slot * ng + g) * D * D;
    for (int r = 0; r < D; ++r)
      for (int d = 0; d < D; ++d) A[r * D + d] = wd * Gi[r][d];
  }
  __syncthreads();
  for (int idx = tid; idx < np * np; idx += NT) {
    const int i = idx / np, j = idx - (idx / np) * np;
    double m = 0.0;
    for (int g = 0; g < ng; ++g) m += s.qB[(size_t)g * np + i] * s.qB[(size_t)g * np + j] * sw[g];
    aug[i * w2 + j] = m;
    aug[i * w2 + np + j] = i == j ? 1.0 : 0.0;
  }
  __syncthreads();
  // Gauss-Jordan elimination with partial pivoting
  for (int k = 0; k < np; ++k) {
    if (tid == 0) {
      int p = k;
      double best = fabs(aug[k * w2 + k]);
      for (int i = k + 1; i < np; ++i) {
        const double v = fabs(aug[i * w2 + k]);
        if (v > best) best = v, p = i;
      }
      piv = p;
      if (!(best > 0.0)) atomicOr(s.err, 2);  // singular mass matrix
    }
    __syncthreads();
    const int p = piv;
    if (p != k)
      for (int j = tid; j < w2; j += NT) {
        const double t = aug[k * w2 + j];
        aug[k * w2 + j] = aug[p * w2 + j];
        aug[p * w2 + j] = t;
      }
    __syncthreads();
    const double inv = 1.0 / aug[k * w2 + k];
    for (int i = tid; i < np; i += NT) col[i] = aug[i * w2 + k];
    __syncthreads();
    for (int j = tid; j < w2; j += NT) aug[k * w2 + j] *= inv;
    __syncthreads();
    for (int idx = tid; idx < np * w2; idx += NT) {
      const int i = idx / w2, j = idx - (idx / w2) * w2;
      if (i != k) aug[i * w2 + j] -= col[i] * aug[k * w2 + j];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < np * np; idx += NT) {
    const int i = idx / np, j = idx - (idx / np) * np;
    s.Minv[((size_t)slot * np + i) * np + j] = aug[i * w2 + np + j];
  }
  // face points: outward unit normal (the same sign rule as the straight-sided
  // faces: the element's orientation times the right-hand normal of the face
  // corner order) and w_g |J_f,g|
  for (int idx = tid; idx < s.nf * s.ngf; idx += NT) {
    const int lf = idx / s.ngf, g = idx - (idx / s.ngf) * s.ngf;
    double tu[3] = {0, 0, 0}, tv[3] = {0, 0, 0};
    const double* fu = s.fTu + ((size_t)lf * s.ngf + g) * np;
    const double* fv = D == 3 ? s.fTv + ((size_t)lf * s.ngf + g) * np : nullptr;
    for (int j = 0; j < np; ++j)
      for (int d = 0; d < 3; ++d) {
        tu[d] += sx[j * 3 + d] * fu[j];
        if (D == 3) tv[d] += sx[j * 3 + d] * fv[j];
      }
    double n[3] = {0, 0, 0}, jf;
    if (D == 2) {
      jf = sqrt(tu[0] * tu[0] + tu[1] * tu[1]);
      n[0] = sg * tu[1] / jf, n[1] = -sg * tu[0] / jf;
    } else {
      const double c[3] = {tu[1] * tv[2] - tu[2] * tv[1], tu[2] * tv[0] - tu[0] * tv[2], tu[0] * tv[1] - tu[1] * tv[0]};
      jf = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      for (int d = 0; d < 3; ++d) n[d] = sg * c[d] / jf;
    }
    double* F = s.F + (((size_t)slot * s.nf + lf) * s.ngf + g) * (D + 1);
    for (int d = 0; d < D; ++d) F[d] = n[d];
    F[D] = s.fw[g] * jf;
  }
  if (D == 3) {
    for (int lf = tid; lf < s.nf; lf += NT) {
      double P[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int k = 0; k < 3; ++k)
        for (int m = 0; m < s.nfp; ++m) {
          const double b = s.fB[((size_t)lf * s.ngf + k) * s.nfp + m];
          const int node = s.fmask[lf * s.nfp + m];
          for (int d = 0; d < 3; ++d) P[k][d] += b * sx[node * 3 + d];
        }
      const double h = sqrt((P[1][0] - P[0][0]) * (P[1][0] - P[0][0]) + (P[1][1] - P[0][1]) * (P[1][1] - P[0][1]) +
                            (P[1][2] - P[0][2]) * (P[1][2] - P[0][2]));
      const double ii = ((P[1][0] - P[0][0]) * (P[2][0] - P[0][0]) + (P[1][1] - P[0][1]) * (P[2][1] - P[0][1]) +
                         (P[1][2] - P[0][2]) * (P[2][2] - P[0][2])) / h;
      const double jj = sqrt((P[2][0] - P[0][0]) * (P[2][0] - P[0][0]) + (P[2][1] - P[0][1]) * (P[2][1] - P[0][1]) +
                             (P[2][2] - P[0][2]) * (P[2][2] - P[0][2]) - ii * ii);
      const double delta = fabs(h) * fabs(jj);
      double t[3], sb[3];
      for (int d = 0; d < 3; ++d) {
        t[d] = (fabs(jj) * (P[1][d] - P[0][d])) / delta;
        sb[d] = -(fabs(ii) * (P[1][d] - P[0][d]) - fabs(h) * (P[2][d] - P[0][d])) / delta;
      }
      unit3(t), unit3(sb);
      double* TB = s.TB + ((size_t)slot * s.nf + lf) * 6;
      for (int d = 0; d < 3; ++d) TB[d] = t[d], TB[3 + d] = sb[d];
    }
  }
}

__global__ void k_f64_to_f32(const double* src, int64_t n, float* dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

template <typename T>
struct RhsDev {
  const T* y_in;
  int64_t stride;
  const T* geoF;
  int recf;
  const int* geoI;
  int reci;
  const int* bcode;
  const short* fmask;
  const short* nbrnode;
  const int64_t* celem;
  const T *A, *Minv, *F, *TB, *qB, *qD, *fB;
  T* rhs;
  int64_t ncurved;
  int ng, ngf;
  dgk::Phys ph;
};

template <typename T, int D, int P>
__global__ void __launch_bounds__(128) k_curved_rhs(const RhsDev<T> c) {
  using S = dgk::Shape<D, P>;
  constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM;
  extern __shared__ __align__(16) unsigned char smr[];
  const int ng = c.ng, ngf = c.ngf;
  T* su = reinterpret_cast<T*>(smr);  // [NV][NP] element state
  T* sS = su + NV * NP;               // [NV][NP] S - face terms
  T* sH = sS + NV * NP;               // [ng][D][NV] contracted fluxes at the element points
  T* sUm = sH + ng * D * NV;          // [NV][NFP] own trace
  T* sUp = sUm + NV * NFP;            // [NV][NFP] neighbour trace
  T* sFI = sUp + NV * NFP;            // [ngf][NV] weighted flux at the face points
  const int slot = blockIdx.x, tid = threadIdx.x, NT = blockDim.x;
  const int64_t e = c.celem[slot];
  const T rhoc2 = (T)c.ph.rhoc2, inv_rho0 = (T)c.ph.inv_rho0, half_c0 = (T)c.ph.half_c0;
  const T c0 = (T)c.ph.c0, rho0 = (T)c.ph.rho0;
  const T* rec = c.geoF + e * c.recf + S::PHYS_OFF;
  T v0[3] = {rec[0], rec[1], D == 3 ? rec[2] : (T)0};
  for (int i = tid; i < NV * NP; i += NT) {
    const int q = i / NP, j = i - (i / NP) * NP;
    su[i] = c.y_in[q * c.stride + e * NP + j];
  }
  __syncthreads();
  // ---- volume: fluxes at the element points, contracted with A_g ----
  for (int g = tid; g < ng; g += NT) {
    T ug[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) ug[q] = 0;
    for (int j = 0; j < NP; ++j) {
      const T b = c.qB[(size_t)g * NP + j];
#pragma unroll
      for (int q = 0; q < NV; ++q) ug[q] += b * su[q * NP + j];
    }
    T Fq[NV][D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      Fq[0][d] = v0[d] * ug[0] + rhoc2 * ug[1 + d];
#pragma unroll
      for (int a = 0; a < D; ++a) Fq[1 + a][d] = v0[d] * ug[1 + a] + (a == d ? ug[0] * inv_rho0 : (T)0);
    }
    const T* Ag = c.A + ((size_t)slot * ng + g) * D * D;
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        T h = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) h += Ag[r * D + d] * Fq[q][d];
        sH[(g * D + r) * NV + q] = h;
      }
  }
  __syncthreads();
  for (int i = tid; i < NV * NP; i += NT) {
    const int q = i / NP, ii = i - (i / NP) * NP;
    T s = 0;
    for (int g = 0; g < ng; ++g)
#pragma unroll
      for (int r = 0; r < D; ++r) s += c.qD[((size_t)r * ng + g) * NP + ii] * sH[(g * D + r) * NV + q];
    sS[i] = s;
  }
  __syncthreads();
  // ---- faces ----
  for (int lf = 0; lf < NF; ++lf) {
    const int nbr = c.geoI[e * c.reci + lf], code = c.geoI[e * c.reci + NF + lf];
    const bool bnd = (code & dgk::kCodeBoundary) != 0;
    for (int i = tid; i < NV * NFP; i += NT) {
      const int q = i / NFP, m = i - (i / NFP) * NFP;
      sUm[i] = su[q * NP + c.fmask[lf * NFP + m]];
      if (!bnd) {
        const int nn = c.nbrnode[((code & dgk::kCodeLfMask) * NPERM + ((code >> dgk::kCodePermShift) & dgk::kCodePermMask)) *
                                     NFP + m];
        sUp[i] = c.y_in[q * c.stride + (int64_t)nbr * NP + nn];
      }
    }
    __syncthreads();
    const T* Fr = c.F + ((size_t)slot * NF + lf) * ngf * (D + 1);
    for (int g = tid; g < ngf; g += NT) {
      const T* fb = c.fB + ((size_t)lf * ngf + g) * NFP;
      T n[3] = {Fr[g * (D + 1)], Fr[g * (D + 1) + 1], D == 3 ? Fr[g * (D + 1) + 2] : (T)0};
      const T W = Fr[g * (D + 1) + D];
      T vn0 = v0[0] * n[0] + v0[1] * n[1];
      if (D == 3) vn0 += v0[2] * n[2];
      T fi[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) fi[q] = 0;
      if (!bnd) {
        const T hc = (code & dgk::kCodeNegPenalty) ? -half_c0 : half_c0;
        for (int m = 0; m < NFP; ++m) {
          T avg[NV], dif[NV], h[NV];
#pragma unroll
          for (int q = 0; q < NV; ++q) {
            const T um = sUm[q * NFP + m], up = sUp[q * NFP + m];
            avg[q] = um + up, dif[q] = um - up;
          }
          T nv = n[0] * avg[1] + n[1] * avg[2];
          if (D == 3) nv += n[2] * avg[3];
          h[0] = (T)0.5 * (vn0 * avg[0] + rhoc2 * nv) + hc * dif[0];
#pragma unroll
          for (int d = 0; d < D; ++d) h[1 + d] = (T)0.5 * (vn0 * avg[1 + d] + n[d] * avg[0] * inv_rho0) + hc * dif[1 + d];
#pragma unroll
          for (int q = 0; q < NV; ++q) fi[q] += fb[m] * h[q];
        }
      } else {
        T ug[4] = {0, 0, 0, 0};
        for (int m = 0; m < NFP; ++m)
#pragma unroll
          for (int q = 0; q < NV; ++q) ug[q] += fb[m] * sUm[q * NFP + m];
        if (c.bcode[nbr] == 1) {
          // reflecting wall: the trace without its normal velocity, then n.F
          T dot = n[0] * ug[1] + n[1] * ug[2];
          if (D == 3) dot += n[2] * ug[3];
          T vr[3];
#pragma unroll
          for (int d = 0; d < D; ++d) vr[d] = ug[1 + d] - dot * n[d];
          T nvr = n[0] * vr[0] + n[1] * vr[1];
          if (D == 3) nvr += n[2] * vr[2];
          fi[0] = vn0 * ug[0] + rhoc2 * nvr;
#pragma unroll
          for (int d = 0; d < D; ++d) fi[1 + d] = vn0 * vr[d] + n[d] * ug[0] * inv_rho0;
        } else {
          // absorbing: RKR at this point (Mesh.cpp:619-666)
          T t[3] = {0, 0, 0}, sb[3] = {0, 0, 0};
          if (D == 2) {
            t[0] = -n[1], t[1] = n[0];
            const T z = t[0] * t[0] + t[1] * t[1];
            if (z > (T)0) {
              const T r = sqrt(z);
              t[0] /= r, t[1] /= r;
            }
          } else {
            const T* tb = c.TB + ((size_t)slot * NF + lf) * 6;
#pragma unroll
            for (int d = 0; d < 3; ++d) t[d] = tb[d], sb[d] = tb[3 + d];
          }
          const T lam = vn0 < (T)0 ? (T)0 : (T)-1, cv = c0 + vn0;
          T R[NV][NV];
          R[0][0] = (T)0.25 * cv;
#pragma unroll
          for (int a = 0; a < D; ++a) R[0][1 + a] = (T)0.25 * (c0 * rho0 * cv * n[a]);
#pragma unroll
          for (int a = 0; a < D; ++a) {
            R[1 + a][0] = (T)0.25 * (n[a] * cv / (rho0 * c0));
#pragma unroll
            for (int b = 0; b < D; ++b)
              R[1 + a][1 + b] = (T)0.25 * (cv * n[a] * n[b] - vn0 * lam * (t[b] * t[a] + sb[b] * sb[a]));
          }
#pragma unroll
          for (int a = 0; a < NV; ++a) {
            T acc = 0;
#pragma unroll
            for (int b = 0; b < NV; ++b) acc += R[a][b] * ug[b];
            fi[a] = acc;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < NV; ++q) sFI[g * NV + q] = W * fi[q];
    }
    __syncthreads();
    for (int i = tid; i < NV * NFP; i += NT) {
      const int q = i / NFP, m = i - (i / NFP) * NFP;
      T fl = 0;
      for (int g = 0; g < ngf; ++g) fl += c.fB[((size_t)lf * ngf + g) * NFP + m] * sFI[g * NV + q];
      sS[q * NP + c.fmask[lf * NFP + m]] -= fl;
    }
    __syncthreads();
  }
  // ---- M^-T (S - F) ----
  const T* Mi = c.Minv + (size_t)slot * NP * NP;
  for (int i = tid; i < NV * NP; i += NT) {
    const int q = i / NP, ii = i - (i / NP) * NP;
    T r = 0;
    for (int j = 0; j < NP; ++j) r += Mi[j * NP + ii] * sS[q * NP + j];
    c.rhs[(q * c.ncurved + slot) * NP + ii] = r;
  }
}

template <typename T, int D, int P>
cudaError_t launch_rhs_dp(const RhsDev<T>& d, int nblocks, cudaStream_t st) {
  using S = dgk::Shape<D, P>;
  const size_t smem =
      sizeof(T) * (2 * S::NV * S::NP + (size_t)d.ng * D * S::NV + 2 * S::NV * S::NFP + (size_t)d.ngf * S::NV);
  k_curved_rhs<T, D, P><<<nblocks, 128, smem, st>>>(d);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_rhs_t(dg_ctx* c, const T* y_in) {
  RhsDev<T> d{};
  d.y_in = y_in;
  d.stride = c->Epad * c->np;
  d.geoF = (const T*)c->geoF;
  d.recf = sizeof(T) == 4 ? c->sh.recf32 : c->sh.recf64;
  d.geoI = c->geoI;
  d.reci = c->sh.reci;
  d.bcode = c->d_bcode;
  d.fmask = c->fmask;
  d.nbrnode = c->nbrnode;
  d.celem = c->celem;
  d.A = (const T*)c->cA, d.Minv = (const T*)c->cMinv, d.F = (const T*)c->cF, d.TB = (const T*)c->cTB;
  d.qB = (const T*)c->cqB, d.qD = (const T*)c->cqD, d.fB = (const T*)c->cfB;
  d.rhs = (T*)c->crhs;
  d.ncurved = c->ncurved;
  d.ng = c->cng, d.ngf = c->cngf;
  d.ph = c->ph;
  const int nb = (int)c->ncurved;
  switch (c->dim * 10 + c->order) {
    case 22: return launch_rhs_dp<T, 2, 2>(d, nb, c->stream);
    case 23: return launch_rhs_dp<T, 2, 3>(d, nb, c->stream);
    case 24: return launch_rhs_dp<T, 2, 4>(d, nb, c->stream);
    case 32: return launch_rhs_dp<T, 3, 2>(d, nb, c->stream);
    case 33: return launch_rhs_dp<T, 3, 3>(d, nb, c->stream);
    case 34: return launch_rhs_dp<T, 3, 4>(d, nb, c->stream);
  }
  return cudaErrorInvalidValue;
}

#define CURVED_CK(x)                                                                                \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA (curved setup): ") + cudaGetErrorString(e_)); \
  } while (0)

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

namespace dgc {

int setup_curved(dg_ctx* c, const double* xyz, const int64_t* en, const int* perm, const double* det_aff,
                 const int* curved_flag, cudaStream_t st) {
  std::vector<void*> scratch;
  auto tmp = [&](size_t bytes) {
    void* p = nullptr;
    if (cudaMalloc(&p, bytes + 16) != cudaSuccess) throw std::runtime_error("device allocation failed (curved setup)");
    scratch.push_back(p);
    return p;
  };
  auto own = [&](void** p, size_t bytes) { CURVED_CK(dev_alloc(c, p, bytes)); };
  try {
    const int64_t E = c->E, Epad = c->Epad;
    std::vector<int> flag(E);
    CURVED_CK(cudaMemcpyAsync(flag.data(), curved_flag, E * sizeof(int), cudaMemcpyDeviceToHost, st));
    CURVED_CK(cudaStreamSynchronize(st));
    std::vector<int64_t> celem;
    std::vector<int> cslot(Epad, -1);
    for (int64_t e = 0; e < E; ++e)
      if (flag[e]) cslot[e] = (int)celem.size(), celem.push_back(e);
    c->ncurved = (int64_t)celem.size();
    if (c->ncurved == 0) return DG_OK;
    if (c->order < 2) throw std::runtime_error("curved elements need order >= 2");
    if (c->dim == 1) {
      c->err = "mesh setup failed: 1-D elements must have equispaced nodes;";
      return DG_ERR_MESH;
    }
    const int D = c->dim, np = c->np, nf = c->nf, nfp = c->nfp, NV = c->nv;
    const int64_t nc = c->ncurved;
    const dgref::CurvedTables tb = dgref::build_curved(c->re);
    const int ng = tb.ng, ngf = tb.ngf;
    c->cng = ng, c->cngf = ngf;
    own((void**)&c->cslot, Epad * sizeof(int));
    own((void**)&c->celem, nc * sizeof(int64_t));
    CURVED_CK(cudaMemcpyAsync(c->cslot, cslot.data(), Epad * sizeof(int), cudaMemcpyHostToDevice, st));
    CURVED_CK(cudaMemcpyAsync(c->celem, celem.data(), nc * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    auto up = [&](const std::vector<double>& v) {
      double* p = (double*)tmp(std::max<size_t>(1, v.size()) * sizeof(double));
      if (!v.empty()) CURVED_CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st));
      return p;
    };
    GeomDev g{};
    g.D = D, g.np = np, g.nf = nf, g.nfp = nfp, g.ng = ng, g.ngf = ngf;
    g.xyz = xyz, g.en = en, g.perm = perm, g.det_aff = det_aff, g.celem = c->celem;
    g.qw = up(tb.qw), g.qB = up(tb.qB), g.qD = up(tb.qD), g.fw = up(tb.fw), g.fB = up(tb.fB);
    g.fTu = up(tb.fTu), g.fTv = up(tb.fTv);
    std::vector<short> fm(c->re.fmask.begin(), c->re.fmask.end());
    short* dfm = (short*)tmp(fm.size() * sizeof(short));
    CURVED_CK(cudaMemcpyAsync(dfm, fm.data(), fm.size() * sizeof(short), cudaMemcpyHostToDevice, st));
    g.fmask = dfm;
    const int64_t nA = nc * ng * D * D, nM = nc * np * np, nF = nc * nf * ngf * (D + 1), nT = nc * nf * 6;
    g.A = (double*)tmp(nA * sizeof(double));
    g.Minv = (double*)tmp(nM * sizeof(double));
    g.F = (double*)tmp(nF * sizeof(double));
    g.TB = (double*)tmp(nT * sizeof(double));
    CURVED_CK(cudaMemsetAsync(g.TB, 0, nT * sizeof(double), st));
    g.err = (int*)tmp(sizeof(int));
    CURVED_CK(cudaMemsetAsync(g.err, 0, sizeof(int), st));
    const size_t smem = sizeof(double) * (3 * np + ng + 2 * np * np + np);
    if (smem > 48 * 1024) CURVED_CK(cudaFuncSetAttribute(k_curved_geom, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_curved_geom<<<(unsigned)nc, 128, smem, st>>>(g);
    CURVED_CK(cudaGetLastError());
    int herr = 0;
    CURVED_CK(cudaMemcpyAsync(&herr, g.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CURVED_CK(cudaStreamSynchronize(st));
    if (herr) {
      c->err = "mesh setup failed:";
      if (herr & 1) c->err += " curved element degenerate or inverted at a quadrature point;";
      if (herr & 2) c->err += " singular mass matrix of a curved element;";
      for (void* p : scratch) cudaFree(p);
      return DG_ERR_MESH;
    }
    // working precision
    auto keep = [&](const double* src, int64_t n, void** dst) {
      if (c->prec == DG_FP64) {
        own(dst, n * sizeof(double));
        CURVED_CK(cudaMemcpyAsync(*dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      } else {
        own(dst, n * sizeof(float));
        k_f64_to_f32<<<nblk(n, 256), 256, 0, st>>>(src, n, (float*)*dst);
        CURVED_CK(cudaGetLastError());
      }
    };
    keep(g.A, nA, &c->cA);
    keep(g.Minv, nM, &c->cMinv);
    keep(g.F, nF, &c->cF);
    keep(g.TB, nT, &c->cTB);
    keep(g.qB, (int64_t)tb.qB.size(), &c->cqB);
    keep(g.qD, (int64_t)tb.qD.size(), &c->cqD);
    keep(g.fB, (int64_t)tb.fB.size(), &c->cfB);
    own(&c->crhs, (size_t)NV * nc * np * c->tsize);
    CURVED_CK(cudaMemsetAsync(c->crhs, 0, (size_t)NV * nc * np * c->tsize, st));
    CURVED_CK(cudaStreamSynchronize(st));
    for (void* p : scratch) cudaFree(p);
    return DG_OK;
  } catch (const std::exception& ex) {
    cudaStreamSynchronize(st);
    for (void* p : scratch) cudaFree(p);
    c->err = ex.what();
    return DG_ERR_CUDA;
  }
}

cudaError_t launch_curved(dg_ctx* c, const void* y_in) {
  if (c->ncurved == 0) return cudaSuccess;
  if (c->prec == DG_FP32) return launch_rhs_t<float>(c, (const float*)y_in);
  return launch_rhs_t<double>(c, (const double*)y_in);
}

}  // namespace dgc
