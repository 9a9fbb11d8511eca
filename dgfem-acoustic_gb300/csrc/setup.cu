// GPU FP64 setup: element geometry, face connectivity, face geometry,
// penalty signs, BC codes and boundary flux matrices.
//
// Restates, for straight-sided elements, the setup of the reference's Mesh
// constructor (src/Mesh.cpp:20-686) with linear-time algorithms:
//   * element Jacobians and their inverses (Mesh.cpp:74-137);
//   * unique faces and face->element connectivity (Mesh.cpp:981-1130, both
//     quadratic scans there) by hashing the sorted corner triples;
//   * face normals, their orientation and the outward boundary normals
//     (Mesh.cpp:316-367, :452-568): each element uses its own outward normal,
//     and the interior penalty sign of the reference, s_f = fc * orient(up, f)
//     with up the lower-numbered neighbour, is fc * kappa * sign(det J_up)
//     where kappa is the sign of the recipe's normal relative to the
//     right-hand normal of the face's corner order (see refelem.h);
//   * BC codes from the first node of the face, groups applied in ascending
//     physical tag order, last match wins, default Absorbing (Mesh.cpp:579-605);
//   * the absorbing-boundary matrix RKR with the 3-D tangent frame built from
//     the first three face quadrature points (Mesh.cpp:284-308, :619-666), and
//     the reflecting-wall flux (Mesh.cpp:911-949) as a matrix on the trace.
#include <cub/cub.cuh>

#include <cmath>
#include <cstring>
#include <stdexcept>

#include "ctx.h"
#include "curved.cuh"

namespace {

constexpr unsigned long long kEmpty = 0xFFFFFFFFFFFFFFFFull;

struct SetupDev {
  int dim, order, np, nf, nfp, nv, nperm;
  int64_t E, nnodes;
  const double* xyz;
  const int64_t* en;  // [E][np] mesh local order
  const int* perm;    // [np] mesh local -> internal (from element 0)
  int face_corners[4][3];
  int perm_table[6][3];
  int fc_kappa;       // fc * kappa
  double head[3][3];  // leading face quadrature barycentrics (3-D tangent frame)
  double v0[3], rho0, c0;
  int ngroups;
  const int* gbc;
  const unsigned* gmask;  // [nnodes] bit g set: node in group g
  const double* ev0;      // [E][3] per-element mean flow, or null (v0 above for all)
  const double* escale;   // [E] per-element time-step scale, or null (1)
};

__device__ __forceinline__ const double* elem_v0(const SetupDev& s, int64_t e) { return s.ev0 ? s.ev0 + 3 * e : s.v0; }

__device__ __forceinline__ const double* X(const SetupDev& s, int64_t node) { return s.xyz + 3 * node; }

// Per element: J = [x_k - x_0], det J, G = J^-1, and the lattice check of
// every element node against the shared node permutation. An element whose
// high-order nodes leave the straight-sided lattice by more than 1e-9 lattice
// spacings is curved (curved[e] = 1); the node order is still read from the
// nearest lattice points, up to a quarter spacing away.
__global__ void k_elem_geom(SetupDev s, double* det, double* G, int* curved, int* err) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.E) return;
  const int D = s.dim;
  const int64_t* en = s.en + e * s.np;
  const double* x0 = X(s, en[0]);
  double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // J[d][k] = dx_d/dxi_k
  for (int k = 0; k < D; ++k) {
    const double* xk = X(s, en[k + 1]);
    for (int d = 0; d < D; ++d) J[d][k] = xk[d] - x0[d];
  }
  double Gi[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  double dt;
  if (D == 1) {
    dt = J[0][0];
    Gi[0][0] = 1.0 / dt;
  } else if (D == 2) {
    dt = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Gi[0][0] = J[1][1] / dt, Gi[0][1] = -J[0][1] / dt;
    Gi[1][0] = -J[1][0] / dt, Gi[1][1] = J[0][0] / dt;
  } else {
    dt = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    Gi[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / dt;
    Gi[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / dt;
    Gi[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / dt;
    Gi[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / dt;
    Gi[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / dt;
    Gi[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / dt;
    Gi[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / dt;
    Gi[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / dt;
    Gi[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / dt;
  }
  det[e] = dt;
  if (!(fabs(dt) > 0.0)) atomicOr(err, 1);  // degenerate element
  for (int r = 0; r < D; ++r)
    for (int d = 0; d < D; ++d) G[e * D * D + r * D + d] = Gi[r][d];
  // lattice check: node n must sit at the internal lattice point perm[n]
  int is_curved = 0;
  for (int n = D + 1; n < s.np; ++n) {
    const double* xn = X(s, en[n]);
    double rel[3] = {0, 0, 0};
    for (int d = 0; d < D; ++d) rel[d] = xn[d] - x0[d];
    int lat[3] = {0, 0, 0};
    bool ok = true;
    for (int r = 0; r < D; ++r) {
      double xi = 0.0;
      for (int d = 0; d < D; ++d) xi += Gi[r][d] * rel[d];
      double l = xi * s.order, lr = rint(l);
      if (fabs(l - lr) > 1e-9) is_curved = 1;
      if (!(fabs(l - lr) <= 0.25)) ok = false;
      lat[r] = (int)lr;
    }
    // internal index of the lattice point (same enumeration as dgref::lattice_index)
    int p = s.order, idx = -1;
    if (D == 1) {
      if (lat[0] >= 0 && lat[0] <= p) idx = lat[0];
    } else if (D == 2) {
      if (lat[0] >= 0 && lat[1] >= 0 && lat[0] + lat[1] <= p) {
        idx = 0;
        for (int jj = 0; jj < lat[1]; ++jj) idx += p - jj + 1;
        idx += lat[0];
      }
    } else if (lat[0] >= 0 && lat[1] >= 0 && lat[2] >= 0 && lat[0] + lat[1] + lat[2] <= p) {
      idx = 0;
      for (int kk = 0; kk < lat[2]; ++kk) idx += (p - kk + 1) * (p - kk + 2) / 2;
      for (int jj = 0; jj < lat[1]; ++jj) idx += p - lat[2] - jj + 1;
      idx += lat[0];
    }
    if (!ok) atomicOr(err, 2);                 // node too far from any lattice point
    else if (idx != s.perm[n]) atomicOr(err, 4);  // element node order differs from element 0
  }
  curved[e] = is_curved;
}

__global__ void k_mark_corners(SetupDev s, int* mark) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.E * (s.dim + 1)) return;
  int64_t e = i / (s.dim + 1);
  int v = (int)(i - e * (s.dim + 1));
  mark[s.en[e * s.np + v]] = 1;
}

__device__ __forceinline__ unsigned long long face_key(const SetupDev& s, const int* vid, int64_t e, int lf) {
  const int64_t* en = s.en + e * s.np;
  if (s.dim == 1) return (unsigned long long)vid[en[s.face_corners[lf][0]]];  // a point face: its vertex
  unsigned long long a = vid[en[s.face_corners[lf][0]]], b = vid[en[s.face_corners[lf][1]]];
  unsigned long long c = s.dim == 3 ? (unsigned long long)vid[en[s.face_corners[lf][2]]] : 0ull;
  // sort (a, b[, c])
  if (a > b) { unsigned long long t = a; a = b; b = t; }
  if (s.dim == 3) {
    if (b > c) { unsigned long long t = b; b = c; c = t; }
    if (a > b) { unsigned long long t = a; a = b; b = t; }
  }
  return (a << 42) | (b << 21) | c;
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return k;
}

// Insert every element face into an open-addressing table keyed by its sorted
// corner vertex ids; each slot records up to two (element, local face) owners.
__global__ void k_face_insert(SetupDev s, const int* vid, unsigned long long* keys, int* cnt, int64_t* owner,
                              unsigned long long mask, int* err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.E * s.nf) return;
  int64_t e = i / s.nf;
  int lf = (int)(i - e * s.nf);
  unsigned long long key = face_key(s, vid, e, lf);
  unsigned long long slot = mix64(key) & mask;
  for (unsigned long long probe = 0; probe <= mask; ++probe) {
    unsigned long long prev = atomicCAS(&keys[slot], kEmpty, key);
    if (prev == kEmpty || prev == key) {
      int c = atomicAdd(&cnt[slot], 1);
      if (c < 2)
        owner[2 * slot + c] = i;
      else
        atomicOr(err, 8);  // face shared by more than two elements
      return;
    }
    slot = (slot + 1) & mask;
  }
  atomicOr(err, 16);  // table full (cannot happen with the chosen capacity)
}

__global__ void k_face_match(SetupDev s, const int* vid, const unsigned long long* keys, const int* cnt,
                             const int64_t* owner, unsigned long long mask, int64_t* partner, int* bflag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.E * s.nf) return;
  int64_t e = i / s.nf;
  int lf = (int)(i - e * s.nf);
  unsigned long long key = face_key(s, vid, e, lf);
  unsigned long long slot = mix64(key) & mask;
  int64_t p = -1;
  for (unsigned long long probe = 0; probe <= mask; ++probe) {
    if (keys[slot] == key) {
      if (cnt[slot] == 2) p = owner[2 * slot] == i ? owner[2 * slot + 1] : owner[2 * slot];
      break;
    }
    if (keys[slot] == kEmpty) break;
    slot = (slot + 1) & mask;
  }
  partner[i] = p;
  bflag[i] = p < 0 ? 1 : 0;
}

__device__ void normalize3(double* a) {
  double z = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  if (z > 0.0) {
    double r = sqrt(z);
    a[0] /= r, a[1] /= r, a[2] /= r;
  }
}

// Face geometry, codes and boundary matrices of every (element, local face).
__global__ void k_face_geom(SetupDev s, const double* det, const int64_t* partner, const int* bidx, double* geoF,
                            int recf, int* geoI, int reci, double* bmat, int* bcode, int* err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= s.E * s.nf) return;
  const int D = s.dim, NV = s.nv;
  int64_t e = i / s.nf;
  int lf = (int)(i - e * s.nf);
  const int64_t* en = s.en + e * s.np;
  int64_t cn[3] = {en[s.face_corners[lf][0]], en[s.face_corners[lf][1]], D == 3 ? en[s.face_corners[lf][2]] : -1};
  const double* x0 = X(s, cn[0]);
  const double* x1 = D >= 2 ? X(s, cn[1]) : x0;
  double sg = det[e] > 0 ? 1.0 : -1.0;
  double n[3] = {0, 0, 0}, Jf;
  if (D == 1) {
    // point face (Mesh.cpp:320-325 and the outward flip of :536-568): the
    // element's outward direction along x; Gmsh's point Jacobian is 1
    Jf = 1.0;
    n[0] = lf == 1 ? sg : -sg;
  } else if (D == 2) {
    double tx = x1[0] - x0[0], ty = x1[1] - x0[1];
    Jf = sqrt(tx * tx + ty * ty);
    n[0] = sg * ty / Jf, n[1] = -sg * tx / Jf;
  } else {
    const double* x2 = X(s, cn[2]);
    double a[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]}, b[3] = {x2[0] - x0[0], x2[1] - x0[1], x2[2] - x0[2]};
    double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    Jf = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    for (int d = 0; d < 3; ++d) n[d] = sg * c[d] / Jf;
  }
  double* gf = geoF + e * recf + D * D + lf * (D + 1);
  for (int d = 0; d < D; ++d) gf[d] = n[d];
  gf[D] = Jf / fabs(det[e]);
  int64_t p = partner[i];
  int nbr, code;
  if (p >= 0) {
    int64_t e2 = p / s.nf;
    int lf2 = (int)(p - e2 * s.nf);
    const int64_t* en2 = s.en + e2 * s.np;
    int64_t hn[3] = {en2[s.face_corners[lf2][0]], en2[s.face_corners[lf2][1]],
                     D == 3 ? en2[s.face_corners[lf2][2]] : -1};
    int q = -1, nperm = D == 2 ? 2 : 6;
    for (int t = 0; t < nperm && q < 0; ++t) {
      bool ok = true;
      for (int k = 0; k < D; ++k) ok &= cn[k] == hn[s.perm_table[t][k]];
      if (ok) q = t;
    }
    if (q < 0) {
      atomicOr(err, 32);  // corner correspondence failed
      q = 0;
    }
    int64_t up = e < e2 ? e : e2;
    int sf = s.fc_kappa * (det[up] > 0 ? 1 : -1);
    if (D == 1) {
      // s_f = orientation of the face seen from up (fc = 1): +1 at its
      // right end point, -1 at its left one
      const int lfu = up == e ? lf : lf2;
      sf = (lfu == 1 ? 1 : -1) * (det[up] > 0 ? 1 : -1);
    }
    nbr = (int)e2;
    code = lf2 | (q << dgk::kCodePermShift) | (sf < 0 ? dgk::kCodeNegPenalty : 0);
  } else {
    int b = bidx[i];
    nbr = b;
    code = dgk::kCodeBoundary;
    unsigned m = s.gmask[cn[0]];
    int bc = 0;
    for (int g = 0; g < s.ngroups; ++g)
      if ((m >> g) & 1u) bc = s.gbc[g] == 1 ? 1 : 0;
    bcode[b] = bc;
    const double* v0 = elem_v0(s, e);
    double v0n = v0[0] * n[0] + v0[1] * n[1] + v0[2] * n[2];
    double R[4][4];
    if (bc == 1) {
      // reflecting wall: remove the normal velocity of the trace, then n.F
      double nn = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
      double rc2 = s.rho0 * s.c0 * s.c0;
      R[0][0] = v0n;
      for (int j = 0; j < 3; ++j) R[0][1 + j] = rc2 * (n[j] - nn * n[j]);
      for (int a = 0; a < 3; ++a) {
        R[1 + a][0] = n[a] / s.rho0;
        for (int j = 0; j < 3; ++j) R[1 + a][1 + j] = v0n * ((a == j ? 1.0 : 0.0) - n[a] * n[j]);
      }
    } else {
      double t[3] = {0, 0, 0}, sb[3] = {0, 0, 0};
      if (D == 1) {
        // point faces carry no tangent frame (Mesh.cpp:320-325)
      } else if (D == 2) {
        t[0] = -n[1], t[1] = n[0];
        normalize3(t);
      } else {
        const double* x2 = X(s, cn[2]);
        double P[3][3];
        for (int k = 0; k < 3; ++k)
          for (int d = 0; d < 3; ++d) P[k][d] = s.head[k][0] * x0[d] + s.head[k][1] * x1[d] + s.head[k][2] * x2[d];
        double h = sqrt((P[1][0] - P[0][0]) * (P[1][0] - P[0][0]) + (P[1][1] - P[0][1]) * (P[1][1] - P[0][1]) +
                        (P[1][2] - P[0][2]) * (P[1][2] - P[0][2]));
        double ii = ((P[1][0] - P[0][0]) * (P[2][0] - P[0][0]) + (P[1][1] - P[0][1]) * (P[2][1] - P[0][1]) +
                     (P[1][2] - P[0][2]) * (P[2][2] - P[0][2])) / h;
        double jj = sqrt((P[2][0] - P[0][0]) * (P[2][0] - P[0][0]) + (P[2][1] - P[0][1]) * (P[2][1] - P[0][1]) +
                         (P[2][2] - P[0][2]) * (P[2][2] - P[0][2]) - ii * ii);
        double delta = fabs(h) * fabs(jj);
        for (int d = 0; d < 3; ++d) {
          t[d] = (fabs(jj) * (P[1][d] - P[0][d])) / delta;
          sb[d] = -(fabs(ii) * (P[1][d] - P[0][d]) - fabs(h) * (P[2][d] - P[0][d])) / delta;
        }
        normalize3(t);
        normalize3(sb);
      }
      double lam = v0n < 0 ? 0.0 : -1.0, cv = s.c0 + v0n;
      R[0][0] = 0.25 * cv;
      for (int a = 0; a < 3; ++a) R[0][1 + a] = 0.25 * (s.c0 * s.rho0 * cv * n[a]);
      for (int a = 0; a < 3; ++a) {
        R[1 + a][0] = 0.25 * (n[a] * cv / (s.rho0 * s.c0));
        for (int b = 0; b < 3; ++b) R[1 + a][1 + b] = 0.25 * (cv * n[a] * n[b] - v0n * lam * (t[b] * t[a] + sb[b] * sb[a]));
      }
    }
    for (int a = 0; a < NV; ++a)
      for (int b2 = 0; b2 < NV; ++b2) bmat[(int64_t)b * NV * NV + a * NV + b2] = R[a][b2];
  }
  geoI[e * reci + lf] = nbr;
  geoI[e * reci + s.nf + lf] = code;
}

// Places G (d xi / dx) at the head of each element's geometry record and the
// element's mean flow and time-step scale after the face entries.
__global__ void k_place_elem(SetupDev s, const double* G, double* geoF, int recf) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= s.E) return;
  const int D = s.dim;
  for (int k = 0; k < D * D; ++k) geoF[e * recf + k] = G[e * D * D + k];
  const int off = D * D + s.nf * (D + 1);
  const double* v0 = elem_v0(s, e);
  for (int d = 0; d < D; ++d) geoF[e * recf + off + d] = v0[d];
  geoF[e * recf + off + D] = s.escale ? s.escale[e] : 1.0;
}

__global__ void k_to_f32(const double* src, int64_t n, float* dst) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float)src[i];
}

// FP32 records have their own padded length.
__global__ void k_geo_to_f32(const double* g64, int recf64, float* g32, int recf32, int64_t Epad, int raw) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= Epad * raw) return;
  int64_t e = i / raw;
  int k = (int)(i - e * raw);
  g32[e * recf32 + k] = (float)g64[e * recf64 + k];
}

__global__ void k_penalty_hist(const int* geoI, int reci, int nf, int64_t E, unsigned long long* hist) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= E * nf) return;
  int64_t e = i / nf;
  int lf = (int)(i - e * nf);
  int code = geoI[e * reci + nf + lf];
  if (code & dgk::kCodeBoundary) return;
  if ((int64_t)geoI[e * reci + lf] < e) return;  // count each interior face once (at its lower element)
  atomicAdd(&hist[(code & dgk::kCodeNegPenalty) ? 0 : 1], 1ull);
}

struct Scratch {
  std::vector<void*> p;
  ~Scratch() {
    for (void* q : p) cudaFree(q);
  }
  template <class T>
  T* alloc(size_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, n * sizeof(T) + 16) != cudaSuccess) throw std::runtime_error("device allocation failed (setup)");
    p.push_back(q);
    return (T*)q;
  }
};

#define SETUP_CK(x)                                                                              \
  do {                                                                                           \
    cudaError_t e_ = (x);                                                                        \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

inline unsigned blocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

namespace dgc {

int run_setup(dg_ctx* c, const dg_mesh_desc* mesh, const double* elem_v0, const double* elem_scale) {
  try {
    Scratch S;
    cudaStream_t st = c->stream;
    const int D = c->dim, np = c->np, nf = c->nf, NV = c->nv;
    const int64_t E = c->E, N = c->nnodes, Epad = c->Epad;
    // ---- inputs ----
    double* xyz = S.alloc<double>(3 * N);
    int64_t* en = S.alloc<int64_t>(E * np);
    int* perm = S.alloc<int>(np);
    unsigned* gmask = S.alloc<unsigned>(N);
    int* gbc = S.alloc<int>(32);
    std::vector<unsigned> hmask(N, 0u);
    for (int g = 0; g < mesh->n_groups; ++g)
      for (int64_t k = mesh->group_offsets[g]; k < mesh->group_offsets[g + 1]; ++k) {
        int64_t node = mesh->group_nodes[k];
        if (node < 0 || node >= N) throw std::runtime_error("group node index out of range");
        hmask[node] |= 1u << g;
      }
    std::vector<int> hgbc(32, 0);
    for (int g = 0; g < mesh->n_groups; ++g) hgbc[g] = mesh->group_bc[g];
    SETUP_CK(cudaMemcpyAsync(xyz, mesh->xyz, 3 * N * sizeof(double), cudaMemcpyHostToDevice, st));
    SETUP_CK(cudaMemcpyAsync(en, mesh->elem_nodes, E * np * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    SETUP_CK(cudaMemcpyAsync(perm, c->perm_c2i.data(), np * sizeof(int), cudaMemcpyHostToDevice, st));
    SETUP_CK(cudaMemcpyAsync(gmask, hmask.data(), N * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    SETUP_CK(cudaMemcpyAsync(gbc, hgbc.data(), 32 * sizeof(int), cudaMemcpyHostToDevice, st));

    SetupDev sd{};
    sd.dim = D, sd.order = c->order, sd.np = np, sd.nf = nf, sd.nfp = c->nfp, sd.nv = NV, sd.nperm = c->re.nperm;
    sd.E = E, sd.nnodes = N, sd.xyz = xyz, sd.en = en, sd.perm = perm;
    std::memcpy(sd.face_corners, c->re.face_corners, sizeof(sd.face_corners));
    std::memcpy(sd.perm_table, c->re.perm_table, sizeof(sd.perm_table));
    int fc = (D == 3 && c->order != 1) ? -1 : 1;
    sd.fc_kappa = fc * dgref::recipe_normal_sign(D, c->order);
    dgref::face_rule_head(c->order, sd.head);
    for (int d = 0; d < 3; ++d) sd.v0[d] = c->ph.v0[d];
    sd.rho0 = c->ph.rho0, sd.c0 = c->ph.c0;
    sd.ngroups = mesh->n_groups, sd.gbc = gbc, sd.gmask = gmask;
    sd.ev0 = nullptr, sd.escale = nullptr;
    if (elem_v0) {
      double* d = S.alloc<double>(3 * E);
      SETUP_CK(cudaMemcpyAsync(d, elem_v0, 3 * E * sizeof(double), cudaMemcpyHostToDevice, st));
      sd.ev0 = d;
    }
    if (elem_scale) {
      double* d = S.alloc<double>(E);
      SETUP_CK(cudaMemcpyAsync(d, elem_scale, E * sizeof(double), cudaMemcpyHostToDevice, st));
      sd.escale = d;
    }

    int* err = S.alloc<int>(1);
    SETUP_CK(cudaMemsetAsync(err, 0, sizeof(int), st));
    // ---- element geometry ----
    double* det = S.alloc<double>(E);
    double* G = S.alloc<double>(E * D * D);
    int* curved = S.alloc<int>(E);
    k_elem_geom<<<blocks(E, 128), 128, 0, st>>>(sd, det, G, curved, err);
    SETUP_CK(cudaGetLastError());
    // ---- compact vertex ids ----
    int* mark = S.alloc<int>(N + 1);
    int* vid = S.alloc<int>(N + 1);
    SETUP_CK(cudaMemsetAsync(mark, 0, (N + 1) * sizeof(int), st));
    k_mark_corners<<<blocks(E * (D + 1), 256), 256, 0, st>>>(sd, mark);
    size_t tmp_bytes = 0;
    SETUP_CK(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, mark, vid, (int)(N + 1), st));
    void* tmp = S.alloc<unsigned char>(tmp_bytes);
    SETUP_CK(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, mark, vid, (int)(N + 1), st));
    int nvert = 0;
    SETUP_CK(cudaMemcpyAsync(&nvert, vid + N, sizeof(int), cudaMemcpyDeviceToHost, st));
    SETUP_CK(cudaStreamSynchronize(st));
    if (nvert >= (1 << 21)) throw std::runtime_error("meshes with more than 2^21 vertices are not supported");
    // ---- face matching ----
    int64_t nef = E * nf;
    unsigned long long cap = 1;
    while (cap < (unsigned long long)(2 * nef)) cap <<= 1;
    unsigned long long* keys = S.alloc<unsigned long long>(cap);
    int* cnt = S.alloc<int>(cap);
    int64_t* owner = S.alloc<int64_t>(2 * cap);
    SETUP_CK(cudaMemsetAsync(keys, 0xFF, cap * sizeof(unsigned long long), st));
    SETUP_CK(cudaMemsetAsync(cnt, 0, cap * sizeof(int), st));
    k_face_insert<<<blocks(nef, 256), 256, 0, st>>>(sd, vid, keys, cnt, owner, cap - 1, err);
    SETUP_CK(cudaGetLastError());
    int64_t* partner = S.alloc<int64_t>(nef);
    int* bflag = S.alloc<int>(nef + 1);
    int* bidx = S.alloc<int>(nef + 1);
    SETUP_CK(cudaMemsetAsync(bflag + nef, 0, sizeof(int), st));
    k_face_match<<<blocks(nef, 256), 256, 0, st>>>(sd, vid, keys, cnt, owner, cap - 1, partner, bflag);
    SETUP_CK(cudaGetLastError());
    size_t tmp2 = 0;
    SETUP_CK(cub::DeviceScan::ExclusiveSum(nullptr, tmp2, bflag, bidx, (int)(nef + 1), st));
    void* t2 = S.alloc<unsigned char>(tmp2);
    SETUP_CK(cub::DeviceScan::ExclusiveSum(t2, tmp2, bflag, bidx, (int)(nef + 1), st));
    int nb = 0;
    SETUP_CK(cudaMemcpyAsync(&nb, bidx + nef, sizeof(int), cudaMemcpyDeviceToHost, st));
    SETUP_CK(cudaStreamSynchronize(st));
    c->n_bfaces = nb;
    c->n_faces = (nef + nb) / 2;
    // ---- face geometry, codes, boundary matrices (FP64) ----
    const int recf64 = c->sh.recf64, reci = c->sh.reci;
    double* geo64 = S.alloc<double>(Epad * recf64);
    SETUP_CK(cudaMemsetAsync(geo64, 0, Epad * recf64 * sizeof(double), st));
    void* geoI = nullptr;
    SETUP_CK(dev_alloc(c, &geoI, Epad * reci * sizeof(int)));
    c->geoI = (int*)geoI;
    SETUP_CK(cudaMemsetAsync(c->geoI, 0, Epad * reci * sizeof(int), st));
    int64_t nbm = (int64_t)(nb > 0 ? nb : 1) * NV * NV;
    double* bm64 = S.alloc<double>(nbm);
    SETUP_CK(dev_alloc(c, (void**)&c->d_bcode, (nb > 0 ? nb : 1) * sizeof(int)));
    int* bcode = c->d_bcode;
    k_place_elem<<<blocks(E, 256), 256, 0, st>>>(sd, G, geo64, recf64);
    k_face_geom<<<blocks(nef, 128), 128, 0, st>>>(sd, det, partner, bidx, geo64, recf64, c->geoI, reci, bm64, bcode,
                                                   err);
    SETUP_CK(cudaGetLastError());
    // ---- store in the working precision ----
    if (c->prec == DG_FP64) {
      SETUP_CK(dev_alloc(c, &c->geoF, Epad * recf64 * sizeof(double)));
      SETUP_CK(cudaMemcpyAsync(c->geoF, geo64, Epad * recf64 * sizeof(double), cudaMemcpyDeviceToDevice, st));
      SETUP_CK(dev_alloc(c, &c->bmat, nbm * sizeof(double)));
      SETUP_CK(cudaMemcpyAsync(c->bmat, bm64, nbm * sizeof(double), cudaMemcpyDeviceToDevice, st));
    } else {
      const int recf32 = c->sh.recf32, raw = D * D + nf * (D + 1) + D + 1;
      SETUP_CK(dev_alloc(c, &c->geoF, Epad * recf32 * sizeof(float)));
      SETUP_CK(cudaMemsetAsync(c->geoF, 0, Epad * recf32 * sizeof(float), st));
      k_geo_to_f32<<<blocks(Epad * raw, 256), 256, 0, st>>>(geo64, recf64, (float*)c->geoF, recf32, Epad, raw);
      SETUP_CK(dev_alloc(c, &c->bmat, nbm * sizeof(float)));
      k_to_f32<<<blocks(nbm, 256), 256, 0, st>>>(bm64, nbm, (float*)c->bmat);
      SETUP_CK(cudaGetLastError());
    }
    // ---- checks and statistics ----
    unsigned long long* hist = S.alloc<unsigned long long>(2);
    SETUP_CK(cudaMemsetAsync(hist, 0, 2 * sizeof(unsigned long long), st));
    k_penalty_hist<<<blocks(nef, 256), 256, 0, st>>>(c->geoI, reci, nf, E, hist);
    int herr = 0;
    unsigned long long hh[2];
    SETUP_CK(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    SETUP_CK(cudaMemcpyAsync(hh, hist, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    SETUP_CK(cudaStreamSynchronize(st));
    c->info.penalty_sign_hist[0] = (int64_t)hh[0];
    c->info.penalty_sign_hist[1] = (int64_t)hh[1];
    if (herr) {
      std::string m = "mesh setup failed:";
      if (herr & 1) m += " degenerate element;";
      if (herr & 2) m += " element too distorted (a high-order node more than a quarter lattice spacing off its straight-sided position);";
      if (herr & 4) m += " elements do not share one local node ordering;";
      if (herr & 8) m += " face shared by more than two elements;";
      if (herr & 16) m += " face hash table overflow;";
      if (herr & 32) m += " inconsistent face corners;";
      c->err = m;
      return DG_ERR_MESH;
    }
    // ---- curved elements: per-element quadrature data ----
    int rc = setup_curved(c, xyz, en, perm, det, curved, st);
    if (rc != DG_OK) return rc;
    return DG_OK;
  } catch (const std::exception& ex) {
    c->err = ex.what();
    return DG_ERR_CUDA;
  }
}

}  // namespace dgc
