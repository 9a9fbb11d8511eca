// Constant-operator fused RK4 stage kernel (sm_103a, FP32 state).
//
// Same arithmetic as the reference's per-stage work (src/Mesh.cpp:734-975,
// src/solver.cpp:38-57, :488-516), organised so that the reference operators
// never pass through the load/store pipe:
//
//   * each warp owns one chunk of NC output nodes (chunk S, warp-uniform) of
//     32 consecutive elements (lane = element); the chunk is a template
//     parameter of the warp's code path, so every operator entry Dt_r[i][j]
//     and LIFT[k][i] it touches has a compile-time address in constant memory
//     and enters the FMA as a constant-bank operand;
//   * per node j a thread loads its element's NV stage values (element-minor
//     copy of the tile: conflict-free), forms the D x NV contravariant fluxes
//     sum_d G_rd F_{q,d} in registers and accumulates NC x D x NV FMAs;
//   * face fluxes as in the pipelined kernel (cp.async neighbour gathers,
//     Lax-Friedrichs / boundary matrix in shared memory), lifted with
//     constant LIFT entries;
//   * dt L goes to shared memory in the tile's [q][e][i] layout and the RK
//     update runs as one coalesced float4 pass over the tile, reading u, the
//     accumulator and the snapshot from global memory (prefetched to L2 when
//     the tile starts) and writing the results straight back.
// Tiles (stage input, geometry records) arrive by TMA bulk copies into a
// double buffer as in the pipelined kernel. Every wait is bounded.
#pragma once
#include <cstdint>

#include "stage2.cuh"

namespace dgk {

// Reference operators of every (dim, order) in constant memory: per shape,
// Dt [D][NP i][NP j] then LIFT [NF*NFP k][NP i] (FP32).
template <int D, int P>
struct COpsOff;
template <> struct COpsOff<2, 1> { static constexpr int v = 0; };
template <> struct COpsOff<2, 2> { static constexpr int v = 36; };
template <> struct COpsOff<2, 3> { static constexpr int v = 36 + 126; };
template <> struct COpsOff<2, 4> { static constexpr int v = 36 + 126 + 320; };
template <> struct COpsOff<3, 1> { static constexpr int v = 36 + 126 + 320 + 675; };
template <> struct COpsOff<3, 2> { static constexpr int v = 1157 + 96; };
template <> struct COpsOff<3, 3> { static constexpr int v = 1157 + 96 + 540; };
template <> struct COpsOff<3, 4> { static constexpr int v = 1157 + 96 + 540 + 2000; };
constexpr int kCOpsTotal = 1157 + 96 + 540 + 2000 + 5775;

// defined here: the constant-operator kernels and the upload live in one
// translation unit (stage3.cu)
__constant__ float c_ops[kCOpsTotal];

template <int D_, int P, int NC_, int EG_>
struct C3Cfg {
  using S = ShapeT<D_, P, float>;
  static constexpr int D = D_;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM, NK = NF * NFP;
  static constexpr int NC = NC_;
  static constexpr int NSPLIT = (NP + NC - 1) / NC;
  static constexpr int EG = EG_;             // groups of 32 elements per tile
  static constexpr int ET = 32 * EG;
  static constexpr int NT = 32 * EG * NSPLIT;
  static constexpr int RECF = S::RECF, RECI = S::RECI;
  static constexpr int NKP = NK | 1;
  // face buffer: the variables of a face node side by side (see stage2.cuh)
  static constexpr int NVQ = NV;  // 2-D: three words, no padding (it would cost occupancy)
  static constexpr int SN_EL = NKP * NVQ, SN_K = NVQ, SN_Q = 1;
  static constexpr size_t SN_WORDS = (size_t)ET * NKP * NVQ;
  static constexpr bool UNROLL = NP <= 16;  // compile-time operator addresses
  static constexpr int OFF_DT = COpsOff<D_, P>::v, OFF_L = OFF_DT + D * NP * NP;
  static constexpr uint32_t YSEG = ET * NP * sizeof(float);
  static constexpr uint32_t GFB = ET * RECF * sizeof(float);
  static constexpr uint32_t GIB = ET * RECI * sizeof(int);
  // shared memory (bytes)
  static constexpr size_t oBar = 0;
  static constexpr size_t oFm = 64;
  static constexpr size_t oNb = oFm + RoundUp<NK * 2, 16>::v;
  static constexpr size_t oY = RoundUp<oNb + NF * NPERM * NFP * 2, 128>::v;  // 2 x [NV][ET][NP]
  static constexpr size_t oYT = oY + 2 * (size_t)NV * YSEG;                   // [NV][NP][ET]
  static constexpr size_t oGF = oYT + (size_t)NV * YSEG;                      // 2 x [ET][RECF]
  static constexpr size_t oGI = oGF + 2 * (size_t)GFB;                        // 2 x [ET][RECI]
  static constexpr size_t oN = RoundUp<oGI + 2 * (size_t)GIB, 128>::v;       // [NV][ET][NKP], then dt L [NV][ET][NP]
  static constexpr size_t oR = RoundUp<oN + SN_WORDS * 4, 16>::v;
  static constexpr size_t bytes = oR + (NT / 32) * 5 * sizeof(double);
  static_assert((size_t)NV * ET * NP <= SN_WORDS, "dt L must fit in the face-flux buffer");
  static_assert((ET * NP) % 4 == 0, "tile segments must be float4 multiples");
};

// Volume and lift terms of output chunk S for this thread's element.
template <class C, int S>
__device__ __forceinline__ void chunk_rhs(const float* sYT, const float* sN, int e, const float (&g)[C::D][C::D],
                                          const float (&gv0)[C::D], float rhoc2, float inv_rho0,
                                          float (&Lv)[C::NC][C::NV]) {
  constexpr int D = C::D, NP = C::NP, NV = C::NV, NC = C::NC, ET = C::ET, NK = C::NK;
  constexpr int I0 = S * NC;
#pragma unroll
  for (int ii = 0; ii < NC; ++ii)
#pragma unroll
    for (int q = 0; q < NV; ++q) Lv[ii][q] = 0.f;
#pragma unroll(C::UNROLL ? NP : 1)
  for (int j = 0; j < NP; ++j) {
    float y[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) y[q] = sYT[(q * NP + j) * ET + e];
    // contravariant fluxes: Fr[r][0] = gv0_r p + rho c^2 (G v)_r,
    // Fr[r][1+d] = gv0_r v_d + G_rd p / rho0
    float fr[D][NV];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float gw = g[r][0] * y[1] + g[r][1] * y[2];
      if (D == 3) gw += g[r][2] * y[3];
      fr[r][0] = gv0[r] * y[0] + rhoc2 * gw;
      const float pr = y[0] * inv_rho0;
#pragma unroll
      for (int d = 0; d < D; ++d) fr[r][1 + d] = gv0[r] * y[1 + d] + g[r][d] * pr;
    }
    // unrolled (small elements): every operator address is a compile-time
    // constant and enters the FMA as a constant-bank operand; otherwise one
    // uniform constant load per entry feeds NV FMAs
#pragma unroll
    for (int ii = 0; ii < NC; ++ii) {
      if (I0 + ii >= NP) break;
#pragma unroll
      for (int r = 0; r < D; ++r) {
        const float dv = c_ops[C::OFF_DT + (r * NP + I0 + ii) * NP + j];
#pragma unroll
        for (int q = 0; q < NV; ++q) Lv[ii][q] = fmaf(dv, fr[r][q], Lv[ii][q]);
      }
    }
  }
#pragma unroll(C::UNROLL ? NK : 1)
  for (int k = 0; k < NK; ++k) {
    float h[C::NVQ];
    vload<float, C::NVQ>(h, sN + (size_t)e * C::SN_EL + k * C::NVQ);
#pragma unroll
    for (int ii = 0; ii < NC; ++ii) {
      if (I0 + ii >= NP) break;
      const float lv = c_ops[C::OFF_L + k * NP + I0 + ii];
#pragma unroll
      for (int q = 0; q < NV; ++q) Lv[ii][q] = fmaf(-lv, h[q], Lv[ii][q]);
    }
  }
}

template <class C, int S>
__device__ __forceinline__ void chunk_dispatch(int s, const float* sYT, const float* sN, int e,
                                               const float (&g)[C::D][C::D], const float (&gv0)[C::D], float rhoc2,
                                               float inv_rho0, float (&Lv)[C::NC][C::NV]) {
  if constexpr (S < C::NSPLIT) {
    if (s == S)
      chunk_rhs<C, S>(sYT, sN, e, g, gv0, rhoc2, inv_rho0, Lv);
    else
      chunk_dispatch<C, S + 1>(s, sYT, sN, e, g, gv0, rhoc2, inv_rho0, Lv);
  }
}

template <int D, int P, int NC_, int EG_>
__global__ void __launch_bounds__(C3Cfg<D, P, NC_, EG_>::NT) stage3_kernel(const StageArgs<float> a, int* err) {
  using C = C3Cfg<D, P, NC_, EG_>;
  using T = float;
  constexpr int NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM, NK = C::NK;
  constexpr int NC = C::NC, ET = C::ET, NT = C::NT, RECF = C::RECF, RECI = C::RECI;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::oBar);
  short* sFm = reinterpret_cast<short*>(sm + C::oFm);
  short* sNb = reinterpret_cast<short*>(sm + C::oNb);
  T* sYb = reinterpret_cast<T*>(sm + C::oY);
  T* sYT = reinterpret_cast<T*>(sm + C::oYT);
  T* sGFb = reinterpret_cast<T*>(sm + C::oGF);
  int* sGIb = reinterpret_cast<int*>(sm + C::oGI);
  T* sN = reinterpret_cast<T*>(sm + C::oN);
  T* sK = sN;  // dt L after the lift: [NV][ET][NP]
  double* sRed = reinterpret_cast<double*>(sm + C::oR);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int s = warp % C::NSPLIT;                 // output chunk of this warp
  const int e = (warp / C::NSPLIT) * 32 + lane;   // element of this thread in the tile
  const int stage = a.stage;
  const int64_t stride = a.stride;

  auto issue_tile = [&](int tile, int b) {
    const int64_t e0 = (int64_t)tile * ET;
    mbar_expect_tx(&bar[b], NV * C::YSEG + C::GFB + C::GIB);
#pragma unroll
    for (int q = 0; q < NV; ++q)
      tma_load_1d(sYb + ((size_t)b * NV + q) * ET * NP, a.y_in + q * stride + e0 * NP, C::YSEG, &bar[b]);
    tma_load_1d(sGFb + (size_t)b * ET * RECF, a.geoF + e0 * RECF, C::GFB, &bar[b]);
    tma_load_1d(sGIb + (size_t)b * ET * RECI, a.geoI + e0 * RECI, C::GIB, &bar[b]);
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  for (int i = tid; i < NK; i += NT) sFm[i] = a.fmask[i];
  for (int i = tid; i < NF * NPERM * NFP; i += NT) sNb[i] = a.nbrnode[i];
  __syncthreads();
  // thread 0: tile buffers armed and not yet observed (bit b) and the armed
  // phase's parity (bit 2+b); drained on exit
  uint32_t pend = 0;
  if (tid == 0 && (int)blockIdx.x < a.ntiles) issue_tile(blockIdx.x, 0), pend = 1u;

  const T rhoc2 = (T)a.ph.rhoc2, inv_rho0 = (T)a.ph.inv_rho0, half_c0 = (T)a.ph.half_c0;
  const T dt = (T)a.dt;
  ResAcc<float> racc;
  bool ok = true;
  const int nepi = (stage == 2 || stage == 3) ? 2 : (stage == 4 ? 3 : 0);

  int it = 0;
  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int64_t e0 = (int64_t)tile * ET;
    const bool got = mbar_wait(&bar[b], (it >> 1) & 1, a.wait_limit);
    if (tid == 0 && got) pend &= ~(1u << b);
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    const T* sY = sYb + (size_t)b * NV * ET * NP;
    const T* sGF = sGFb + (size_t)b * ET * RECF;
    const int* sGI = sGIb + (size_t)b * ET * RECI;
    if (tid == 0) {
      fence_proxy_async();
      const int nt = tile + gridDim.x;
      if (nt < a.ntiles)
        issue_tile(nt, b ^ 1), pend = (pend & ~(0x5u << (b ^ 1))) | (1u << (b ^ 1)) |
                                      ((uint32_t)(((it + 1) >> 1) & 1) << (2 + (b ^ 1)));
    }
    // RK operands of this tile towards L2 (read by the coalesced epilogue)
    if (tid < NV * nepi) {
      const int k = tid / NV, q = tid - (tid / NV) * NV;
      const T* src = k == 0 ? a.u : (k == 1 ? a.acc : a.snap);
      prefetch_l2(src + q * stride + e0 * NP, C::YSEG);
    }
    // ---- neighbour traces (asynchronous) ----
    gather_traces<C, T>(a.y_in, stride, sGI, sNb, sN, tid, e0);
    cp_async_commit();
    // ---- element-minor copy of the stage input ----
    for (int w = tid; w < NV * ET * NP; w += NT) {
      const int q = w / (ET * NP), r = w - q * (ET * NP);
      const int el = r / NP, j = r - (r / NP) * NP;
      sYT[(q * NP + j) * ET + el] = sY[w];
    }
    __syncthreads();

    // ---- per-element metric, mean flow and time-step scale ----
    const T* G = sGF + e * RECF;
    T g[D][D], gv0[D];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int d = 0; d < D; ++d) g[r][d] = G[r * D + d];
    {
      const T* ev0 = G + C::S::PHYS_OFF;
#pragma unroll
      for (int r = 0; r < D; ++r) {
        gv0[r] = g[r][0] * ev0[0] + g[r][1] * ev0[1];
        if (D == 3) gv0[r] += g[r][2] * ev0[2];
      }
    }
    const T dte = dt * G[C::S::PHYS_OFF + D];

    cp_async_wait_all();
    __syncthreads();
    // ---- face numerical fluxes (in place of the gathered traces) ----
    face_fluxes<C, T>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, tid, rhoc2, inv_rho0, half_c0, e0);
    __syncthreads();

    // ---- volume and lift for this warp's node chunk ----
    T Lv[NC][NV];
    chunk_dispatch<C, 0>(s, sYT, sN, e, g, gv0, rhoc2, inv_rho0, Lv);
    __syncthreads();  // sN is read by every chunk before dt L overwrites it
#pragma unroll
    for (int ii = 0; ii < NC; ++ii) {
      const int i = s * NC + ii;
      if (i >= NP) break;
#pragma unroll
      for (int q = 0; q < NV; ++q) sK[(q * ET + e) * NP + i] = dte * Lv[ii][q];
    }
    __syncthreads();

    // ---- RK update: one coalesced float4 pass over the tile ----
    for (int w4 = tid; w4 < NV * ET * NP / 4; w4 += NT) {
      const int w = w4 * 4;
      const int q = w / (ET * NP), off = w - q * (ET * NP);
      const int64_t gidx = q * stride + e0 * NP + off;
      const float4 kv = *reinterpret_cast<const float4*>(sK + w);
      float4 o1, o2;
      switch (stage) {
        case 0:
          *reinterpret_cast<float4*>(a.k_out + gidx) = kv;
          break;
        case 1: {
          const float4 xu = *reinterpret_cast<const float4*>(sY + w);
          o2 = make_float4(xu.x + 0.5f * kv.x, xu.y + 0.5f * kv.y, xu.z + 0.5f * kv.z, xu.w + 0.5f * kv.w);
          *reinterpret_cast<float4*>(a.acc + gidx) = kv;
          *reinterpret_cast<float4*>(a.y_out + gidx) = o2;
          break;
        }
        case 2:
        case 3: {
          const float4 xu = __ldcs(reinterpret_cast<const float4*>(a.u + gidx));
          const float4 xa = __ldcs(reinterpret_cast<const float4*>(a.acc + gidx));
          const float c = stage == 2 ? 0.5f : 1.0f;
          o1 = make_float4(xa.x + 2.f * kv.x, xa.y + 2.f * kv.y, xa.z + 2.f * kv.z, xa.w + 2.f * kv.w);
          o2 = make_float4(xu.x + c * kv.x, xu.y + c * kv.y, xu.z + c * kv.z, xu.w + c * kv.w);
          *reinterpret_cast<float4*>(a.acc + gidx) = o1;
          *reinterpret_cast<float4*>(a.y_out + gidx) = o2;
          break;
        }
        case 4: {
          const float4 xu = __ldcs(reinterpret_cast<const float4*>(a.u + gidx));
          const float4 xa = __ldcs(reinterpret_cast<const float4*>(a.acc + gidx));
          const float4 xs = __ldcs(reinterpret_cast<const float4*>(a.snap + gidx));
          const float un[4] = {xu.x + rk4_sixth(xa.x + kv.x), xu.y + rk4_sixth(xa.y + kv.y),
                               xu.z + rk4_sixth(xa.z + kv.z), xu.w + rk4_sixth(xa.w + kv.w)};
          const float sn[4] = {xs.x, xs.y, xs.z, xs.w};
#pragma unroll
          for (int v = 0; v < 4; ++v) racc.add(q, sn[v], un[v], a.c0sq);
          *reinterpret_cast<float4*>(a.u + gidx) = make_float4(un[0], un[1], un[2], un[3]);
          break;
        }
        default: {
          const float4 xu = *reinterpret_cast<const float4*>(sY + w);
          o2 = make_float4(xu.x + kv.x, xu.y + kv.y, xu.z + kv.z, xu.w + kv.w);
          *reinterpret_cast<float4*>(a.y_out + gidx) = o2;
          break;
        }
      }
    }
    __syncthreads();  // tile buffers and dt L are free again
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i)
      if (pend & (1u << i)) mbar_wait(&bar[i], (pend >> (2 + i)) & 1u);
    if (!ok) atomicOr(err, 1);
  }

  if (stage == 4) {
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      double v = racc.get(c, a.c0sq);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if (lane == 0) sRed[warp * 5 + c] = v;
    }
    __syncthreads();
    if (tid < 5) {
      double v = 0.0;
      for (int w = 0; w < NT / 32; ++w) v += sRed[w * 5 + tid];
      a.partials[blockIdx.x * 5 + tid] = v;
    }
  }
}

template <int D, int P, int NC_, int EG_>
struct Stage3 {
  using C = C3Cfg<D, P, NC_, EG_>;
  static cudaError_t set_attrs() {
    auto kfn = stage3_kernel<D, P, NC_, EG_>;
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    return e;
  }
  static cudaError_t launch(const StageArgs<float>& a, int grid, int* err, cudaStream_t s) {
    static bool configured = false;
    if (!configured) {
      cudaError_t e = set_attrs();
      if (e != cudaSuccess) return e;
      configured = true;
    }
    stage3_kernel<D, P, NC_, EG_><<<grid, C::NT, C::bytes, s>>>(a, err);
    return cudaGetLastError();
  }
  static int blocks_per_sm() {
    if (set_attrs() != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stage3_kernel<D, P, NC_, EG_>, C::NT, C::bytes) !=
        cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return nb;
  }
};

}  // namespace dgk
