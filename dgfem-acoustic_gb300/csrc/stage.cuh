// Fused RK4 stage kernel: semi-discrete LEE right-hand side (volume term,
// face numerical flux with absorbing/reflecting boundaries, LIFT) and the
// stage update, for one (dim, order, precision).
//
// What one launch computes, per element e (the reference's per-stage work,
// src/Mesh.cpp:734-975 + src/solver.cpp:38-57 + :488-516):
//   L_q(i) = sum_r sum_d G_rd (A_d W^r)_q(i)  -  sum_f sJ_f sum_m LIFT_f(i,m) h_q(f,m)
//   W^r(i) = sum_j Dt_r(i,j) y(j)            (weak volume term; Dt_r = M^-1 K_r)
//   A_d    : LEE flux Jacobians (F_p = v0 p + rho0 c0^2 v, F_v = v0 v + p/rho0 e)
//   h      : interior  1/2 n.(F(y-) + F(y+)) + 1/2 s_f c0 (y- - y+)
//            boundary  B_f y-  (RKR for absorbing, reflect-then-flux for reflecting)
//   k = dt L, followed by the stage's RK4 update.
// Layout and mapping: a block owns a tile of ET consecutive elements and
// runs persistently over tiles. Each element is handled by NSPLIT threads,
// each owning NC output nodes. The tile's stage input, geometry, the shared
// reference operators and the face fluxes live in shared memory; neighbour
// traces are gathered from global memory (L2). All global state traffic is
// coalesced (tile-contiguous copies in, tile-contiguous stores out).
#pragma once
#include <cstdint>

#include "dg_internal.cuh"

namespace dgk {

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

template <int N, int VEC>
struct Align {
  static constexpr int v = (N + VEC - 1) / VEC * VEC;
};

template <typename T, int D, int P>
struct StageSmem {
  using S = ShapeT<D, P, T>;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NK = NF * NFP;
  static constexpr int NPP = NP | 1;  // odd element strides: conflict-free per-element reads
  static constexpr int NKP = NK | 1;
  static constexpr int VEC = S::VEC;
  static constexpr int oD = 0;
  static constexpr int oL = oD + Align<D * NP * NP, VEC>::v;
  static constexpr int oY = oL + Align<NK * NP, VEC>::v;
  static constexpr int oH = oY + Align<NV * S::ET * NPP, VEC>::v;
  static constexpr int oGF = oH + Align<NV * S::ET * NKP, VEC>::v;
  static constexpr int nT = oGF + S::ET * S::RECF;  // T elements
  static constexpr int nI = S::ET * S::RECI;        // ints
  static constexpr int nS = NK + NF * S::NPERM * NFP;  // shorts
  static constexpr size_t bytes_red = (S::NT / 32) * 5 * sizeof(double);
  static constexpr size_t bytes =
      ((size_t)nT * sizeof(T) + nI * sizeof(int) + ((nS * sizeof(short) + 15) / 16 * 16) + bytes_red + 15) / 16 * 16;
};

template <typename T, int D, int P>
__global__ void __launch_bounds__(ShapeT<D, P, T>::NT) stage_kernel(const StageArgs<T> a) {
  using S = ShapeT<D, P, T>;
  using M = StageSmem<T, D, P>;
  constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM;
  constexpr int NC = S::NC, NSPLIT = S::NSPLIT, ET = S::ET, NT = S::NT, RECF = S::RECF, RECI = S::RECI;
  constexpr int NK = M::NK, NPP = M::NPP, NKP = M::NKP;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sT = reinterpret_cast<T*>(smem_raw);
  T* sD = sT + M::oD;
  T* sL = sT + M::oL;
  T* sY = sT + M::oY;
  T* sH = sT + M::oH;
  T* sGF = sT + M::oGF;
  int* sGI = reinterpret_cast<int*>(sT + M::nT);
  short* sFm = reinterpret_cast<short*>(sGI + M::nI);
  short* sNb = sFm + NK;
  double* sRed = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(smem_raw) + M::bytes - M::bytes_red - 0);

  const int tid = threadIdx.x;
  // shared reference operators, loaded once per persistent block
  for (int i = tid; i < D * NP * NP; i += NT) sD[i] = a.Dt[i];
  for (int i = tid; i < NK * NP; i += NT) sL[i] = a.LIFT[i];
  for (int i = tid; i < NK; i += NT) sFm[i] = a.fmask[i];
  for (int i = tid; i < NF * NPERM * NFP; i += NT) sNb[i] = a.nbrnode[i];

  const T rhoc2 = (T)a.ph.rhoc2, inv_rho0 = (T)a.ph.inv_rho0, half_c0 = (T)a.ph.half_c0;
  const T dt = (T)a.dt;
  const int64_t stride = a.stride;
  ResAcc<T> racc;

  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
    const int64_t e0 = (int64_t)tile * ET;
    // ---- stage input and geometry of the tile (coalesced) ----
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const T* src = a.y_in + q * stride + e0 * NP;
      for (int i = tid; i < ET * NP; i += NT) {
        int e = i / NP, j = i - e * NP;
        sY[(q * ET + e) * NPP + j] = ldg(src + i);
      }
    }
    for (int i = tid; i < ET * RECF; i += NT) sGF[i] = ldg(a.geoF + e0 * RECF + i);
    for (int i = tid; i < ET * RECI; i += NT) sGI[i] = ldg(a.geoI + e0 * RECI + i);
    __syncthreads();

    // ---- face numerical fluxes h (scaled by sJ) for every face node of the tile ----
    for (int it = tid; it < ET * NK; it += NT) {
      const int e = it / NK, k = it - e * NK;
      const int f = k / NFP, m = k - f * NFP;
      const int node = sFm[k];
      T um[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) um[q] = sY[(q * ET + e) * NPP + node];
      const int nbr = sGI[e * RECI + f];
      const int code = sGI[e * RECI + NF + f];
      const T* gf = sGF + e * RECF + D * D + f * (D + 1);
      T n[3];
#pragma unroll
      for (int d = 0; d < D; ++d) n[d] = gf[d];
      const T sJ = gf[D];
      T h[NV];
      if (code & kCodeBoundary) {
        const T* B = a.bmat + (int64_t)nbr * NV * NV;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          T s = 0;
#pragma unroll
          for (int qq = 0; qq < NV; ++qq) s += ldg(B + q * NV + qq) * um[qq];
          h[q] = s;
        }
      } else {
        const int lfn = code & kCodeLfMask, perm = (code >> kCodePermShift) & kCodePermMask;
        const int nn = sNb[(lfn * NPERM + perm) * NFP + m];
        T up[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) up[q] = ldg(a.y_in + q * stride + (int64_t)nbr * NP + nn);
        const T hc = (code & kCodeNegPenalty) ? -half_c0 : half_c0;
        const T* ev0 = sGF + e * RECF + S::PHYS_OFF;
        T vn0 = ev0[0] * n[0];
        #pragma unroll
        for (int d = 1; d < D; ++d) vn0 += ev0[d] * n[d];
        T avg[NV], dif[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) avg[q] = um[q] + up[q], dif[q] = um[q] - up[q];
        T nv = n[0] * avg[1];
        #pragma unroll
        for (int d = 1; d < D; ++d) nv += n[d] * avg[1 + d];
        h[0] = (T)0.5 * (vn0 * avg[0] + rhoc2 * nv) + hc * dif[0];
#pragma unroll
        for (int d = 0; d < D; ++d) h[1 + d] = (T)0.5 * (vn0 * avg[1 + d] + n[d] * avg[0] * inv_rho0) + hc * dif[1 + d];
      }
#pragma unroll
      for (int q = 0; q < NV; ++q) sH[(q * ET + e) * NKP + k] = sJ * h[q];
    }
    __syncthreads();

    // ---- volume term and lifting for this thread's nodes ----
    const int e = tid / NSPLIT, s = tid - (tid / NSPLIT) * NSPLIT;
    const int i0 = s * NC;
    T Lv[NC][NV];
    {
      T W[D][NC][NV];
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int ii = 0; ii < NC; ++ii)
#pragma unroll
          for (int q = 0; q < NV; ++q) W[r][ii][q] = 0;
#pragma unroll 5
      for (int j = 0; j < NP; ++j) {
        T yq[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) yq[q] = sY[(q * ET + e) * NPP + j];
#pragma unroll
        for (int r = 0; r < D; ++r) {
          const T* drow = sD + (r * NP + j) * NP;
#pragma unroll
          for (int ii = 0; ii < NC; ++ii) {
            const int i = (i0 + ii < NP) ? i0 + ii : NP - 1;
            const T dv = drow[i];
#pragma unroll
            for (int q = 0; q < NV; ++q) W[r][ii][q] += dv * yq[q];
          }
        }
      }
      const T* G = sGF + e * RECF;
      const T* ev0 = G + S::PHYS_OFF;
      T gv0[D];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        gv0[r] = G[r * D + 0] * ev0[0];
        #pragma unroll
        for (int d = 1; d < D; ++d) gv0[r] += G[r * D + d] * ev0[d];
      }
#pragma unroll
      for (int ii = 0; ii < NC; ++ii) {
        T vp = 0, vv[D];
#pragma unroll
        for (int d = 0; d < D; ++d) vv[d] = 0;
#pragma unroll
        for (int r = 0; r < D; ++r) {
          T gw = 0;
#pragma unroll
          for (int d = 0; d < D; ++d) gw += G[r * D + d] * W[r][ii][1 + d];
          vp += gv0[r] * W[r][ii][0] + rhoc2 * gw;
#pragma unroll
          for (int d = 0; d < D; ++d) vv[d] += gv0[r] * W[r][ii][1 + d] + G[r * D + d] * W[r][ii][0] * inv_rho0;
        }
        Lv[ii][0] = vp;
#pragma unroll
        for (int d = 0; d < D; ++d) Lv[ii][1 + d] = vv[d];
      }
    }
#pragma unroll 4
    for (int k = 0; k < NK; ++k) {
      T hq[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) hq[q] = sH[(q * ET + e) * NKP + k];
      const T* lrow = sL + k * NP;
#pragma unroll
      for (int ii = 0; ii < NC; ++ii) {
        const int i = (i0 + ii < NP) ? i0 + ii : NP - 1;
        const T lv = lrow[i];
#pragma unroll
        for (int q = 0; q < NV; ++q) Lv[ii][q] -= lv * hq[q];
      }
    }
    curved_override<T, NC, NV, NP>(a, e0 + e, i0, Lv);
    const T dte = dt * sGF[e * RECF + S::PHYS_OFF + D];  // dt times the element's step scale
    __syncthreads();  // every thread is done reading sY / sH of this tile
#pragma unroll
    for (int ii = 0; ii < NC; ++ii)
      if (i0 + ii < NP)
#pragma unroll
        for (int q = 0; q < NV; ++q) sY[(q * ET + e) * NPP + i0 + ii] = dte * Lv[ii][q];
    __syncthreads();

    // ---- stage update over the tile's contiguous DOFs ----
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      const int64_t base = q * stride + e0 * NP;
      for (int i = tid; i < ET * NP; i += NT) {
        const int el = i / NP, j = i - el * NP;
        const T kv = sY[(q * ET + el) * NPP + j];
        const int64_t g = base + i;
        switch (a.stage) {
          case 0:
            a.k_out[g] = kv;
            break;
          case 1:
            a.acc[g] = kv;
            a.y_out[g] = a.u[g] + (T)0.5 * kv;
            break;
          case 2:
            a.acc[g] = a.acc[g] + (T)2 * kv;
            a.y_out[g] = a.u[g] + (T)0.5 * kv;
            break;
          case 3:
            a.acc[g] = a.acc[g] + (T)2 * kv;
            a.y_out[g] = a.u[g] + kv;
            break;
          case 4: {
            const T un = a.u[g] + rk4_sixth(a.acc[g] + kv);
            a.u[g] = un;
            racc.add(q, a.snap[g], un, a.c0sq);
            break;
          }
          default:
            a.y_out[g] = a.u[g] + kv;
            break;
        }
      }
    }
    __syncthreads();
  }

  if (a.stage == 4) {
    // block reduction of the residual partial sums (fixed order: deterministic)
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      double v = racc.get(c, a.c0sq);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if ((tid & 31) == 0) sRed[(tid >> 5) * 5 + c] = v;
    }
    __syncthreads();
    if (tid < 5) {
      double v = 0.0;
      for (int w = 0; w < NT / 32; ++w) v += sRed[w * 5 + tid];
      a.partials[blockIdx.x * 5 + tid] = v;
    }
  }
}

template <typename T, int D, int P>
cudaError_t launch_stage_impl(const StageArgs<T>& a, int grid, cudaStream_t s) {
  using M = StageSmem<T, D, P>;
  auto kfn = stage_kernel<T, D, P>;
  static bool configured = false;
  if (!configured) {
    cudaError_t err = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)M::bytes);
    if (err != cudaSuccess) return err;
    configured = true;
  }
  kfn<<<grid, ShapeT<D, P, T>::NT, M::bytes, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int D, int P>
int blocks_per_sm_impl() {
  using M = StageSmem<T, D, P>;
  auto kfn = stage_kernel<T, D, P>;
  if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)M::bytes) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kfn, ShapeT<D, P, T>::NT, M::bytes) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return nb < 1 ? 1 : nb;
}

}  // namespace dgk
