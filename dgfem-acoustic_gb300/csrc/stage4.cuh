// Wide-chunk pipelined RK4 stage kernel (sm_103a, FP32 state).
//
// Same arithmetic as the reference's per-stage work (src/Mesh.cpp:734-975,
// src/solver.cpp:38-57, :488-516) and the same tile pipeline as the
// pipelined kernel (stage2.cuh: persistent blocks, TMA bulk copies of the
// stage input and geometry into a double buffer, cp.async neighbour gathers,
// face fluxes per run of a face's nodes). What differs is how a thread
// applies the reference operators and how the RK update reaches memory; on
// the pipelined kernel the shared-memory pipe was the limit (2-D p = 4:
// 4,900 instructions and 1,250 shared-memory loads per element and stage,
// issue 43 %, short-scoreboard and MIO-throttle the top stalls):
//
//   * operator rows padded with zeros to NPR = NSPLIT x NC entries, so that
//     every thread's chunk of NC output nodes (6 to 10 here, against 2 to 5)
//     starts on a vector boundary: its operator entries for one input node
//     arrive in 16-byte (or 8-byte) shared-memory loads;
//   * the FMAs run as packed pairs over a thread's node pairs (__ffma2_rn:
//     per component the rounding of fmaf);
//   * FORM selects the volume contraction: kWForm contracts the stage input
//     per reference direction, W_r[i][q] = sum_j Dt_r[i][j] y_q[j], and mixes
//     the directions with the element metric afterwards (D x NC x NV
//     accumulators); kFluxForm forms the contravariant fluxes
//     F_rq(y_j) = sum_d G_rd F_{q,d}(y_j) per input node first and
//     accumulates L[i][q] += Dt_r[i][j] F_rq (NC x NV accumulators, the
//     fluxes recomputed by each of an element's NSPLIT threads);
//   * STAGED = false leaves the RK operands (u, accumulator, residual
//     snapshot) out of shared memory, which lets about twice as many blocks
//     share an SM: they are prefetched to L2 when the tile starts, dt*L is
//     written to shared memory in the tile's [q][e][i] layout (over the face
//     buffer, free after the lift), and one coalesced float4 pass over the
//     tile reads the operands from L2 and writes the results. STAGED = true
//     copies them into shared memory by TMA (as the pipelined kernel does)
//     and updates from registers.
#pragma once
#include <cstdint>

#include "stage2.cuh"

namespace dgk {

// volume forms: flux form, W form, W form with two elements per thread
constexpr int kFluxForm = 0, kWForm = 1, kWForm2 = 2;

// Compile-time configuration: element shape (D, P), nodes per thread NC
// (even), elements per tile ET, the volume form and the operand staging.
// Shared-memory layout names follow Pipe's (pipe_loop reads them).
template <int D_, int P, int NC_, int ET_, int FORM_, bool STAGED_>
struct Wide {
  using T = float;
  using S = ShapeT<D_, P, float>;
  static constexpr bool kStaged = STAGED_;
  static constexpr int FORM = FORM_;
  static constexpr int D = D_;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM, NK = NF * NFP;
  static constexpr int NC = NC_;
  static constexpr int NSPLIT = (NP + NC - 1) / NC;
  static constexpr int NPR = NSPLIT * NC;                 // operator row stride (zero padded)
  static constexpr int OVW = NC % 4 == 0 ? 4 : 2;         // operator load width
  static constexpr int NH = NC / 2;                       // node pairs of a thread
  static constexpr int ET = ET_;
  static constexpr int NT = ET * NSPLIT;
  static constexpr int RECF = S::RECF, RECI = S::RECI;
  // register RK update (staged operands): vector width such that chunk
  // starts s*NC and element starts e*NP lie on VW-element boundaries and no
  // vector crosses the element's last node
  static constexpr int VW = (NP % 4 == 0 && NC % 4 == 0) ? 4 : (NP % 2 == 0) ? 2 : 1;
  static constexpr uint32_t YSEG = ET * NP * sizeof(float);
  static constexpr uint32_t GFB = ET * RECF * sizeof(float);
  static constexpr uint32_t GIB = ET * RECI * sizeof(int);
  // face buffer: [ET][NKP][NV], a face node's variables side by side (odd
  // element stride NKP x NV words: the elements of a warp meet distinct banks)
  static constexpr int NKP = NK | 1;
  static constexpr int NVQ = NV;
  static constexpr int SN_EL = NKP * NVQ, SN_K = NVQ, SN_Q = 1;
  static constexpr size_t SN_WORDS = (size_t)ET * NKP * NVQ;
  // shared memory layout (bytes)
  static constexpr size_t oBar = 0;                                           // 3 mbarriers
  static constexpr size_t oD = 64;                                            // Dt [D][NP j][NPR i]
  static constexpr size_t oL = RoundUp<oD + D * NP * NPR * 4, 16>::v;         // -LIFT [NK][NPR]
  static constexpr size_t oFm = RoundUp<oL + NK * NPR * 4, 16>::v;            // fmask
  static constexpr size_t oNb = oFm + RoundUp<NK * 2, 16>::v;                 // nbrnode
  static constexpr size_t oY = RoundUp<oNb + NF * NPERM * NFP * 2, 128>::v;   // 2 x [NV][ET][NP]
  static constexpr size_t oGF = oY + 2 * (size_t)NV * YSEG;                  // 2 x [ET][RECF]
  static constexpr size_t oGI = oGF + 2 * (size_t)GFB;                        // 2 x [ET][RECI]
  static constexpr size_t oE = RoundUp<oGI + 2 * (size_t)GIB, 128>::v;       // [3][NV][ET][NP] (staged)
  static constexpr size_t oN = oE + (kStaged ? 3 * (size_t)NV * YSEG : 0);    // [ET][NKP][NV]
  static constexpr size_t oR = RoundUp<oN + SN_WORDS * 4, 16>::v;            // [NT/32][5] double
  static constexpr size_t bytes = oR + (NT / 32) * 5 * sizeof(double);
  static_assert(NC % 2 == 0, "nodes per thread come in pairs");
  static_assert(NT % 32 == 0, "threads per block must be a multiple of 32");
  static_assert(YSEG % 16 == 0, "tile segments must be 16-byte multiples");
  static_assert(NPR % OVW == 0, "operator rows must be whole vectors");
  static_assert(SN_WORDS >= (size_t)NV * ET * NP, "dt*L of a tile must fit in the face buffer");
};

// The RK update of a tile in one coalesced float4 pass over its
// [q][e][i] layout: the thread's items w = tid + k*NT are taken G at a time.
// wide_rk_load loads the operands of one group (u, accumulator and
// snapshot from global memory, where the tile start prefetched them to L2;
// in stages 1 and 5 u from the tile's stage input sY); wide_rk_store
// combines them with dt*L from sK and writes the results. The first group's
// loads are issued before the lift, so that their latency overlaps it.
constexpr int kRkGroup = 3;
struct RkOps {
  float4 x0[kRkGroup], x1[kRkGroup], x2[kRkGroup];
};

template <class C>
__device__ __forceinline__ void wide_rk_load(const StageArgs<float>& a, const float* sY, int64_t e0, int tid, int k0,
                                             RkOps& o) {
  constexpr int NP = C::NP, ET = C::ET, NT = C::NT, SEG4 = ET * NP / 4, TILE4 = C::NV * SEG4;
  constexpr int IT = (TILE4 + NT - 1) / NT;  // float4 items of a thread
  const int stage = a.stage;
  const bool ld_y = stage == 1 || stage == 5, ld_ua = stage >= 2 && stage <= 4, ld_s = stage == 4;
#pragma unroll
  for (int g = 0; g < kRkGroup; ++g) {
    const int w = tid + (k0 + g) * NT;
    const int qq = w / SEG4, r4 = w - (w / SEG4) * SEG4;
    const int64_t gi = qq * a.stride + e0 * NP + (int64_t)r4 * 4;
    o.x0[g] = o.x1[g] = o.x2[g] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (tid < NT && k0 + g < IT && w < TILE4) {
      if (ld_y) o.x0[g] = *reinterpret_cast<const float4*>(sY + qq * ET * NP + r4 * 4);
      if (ld_ua) {
        o.x0[g] = __ldcs(reinterpret_cast<const float4*>(a.u + gi));
        o.x1[g] = __ldcs(reinterpret_cast<const float4*>(a.acc + gi));
      }
      if (ld_s) o.x2[g] = __ldcs(reinterpret_cast<const float4*>(a.snap + gi));
    }
  }
}

template <class C>
__device__ __forceinline__ void wide_rk_store(const StageArgs<float>& a, const float* sK, int64_t e0, int tid, int k0,
                                              const RkOps& o, ResAcc<float>& racc) {
  constexpr int NP = C::NP, ET = C::ET, NT = C::NT, SEG4 = ET * NP / 4, TILE4 = C::NV * SEG4;
  constexpr int IT = (TILE4 + NT - 1) / NT;
  const int stage = a.stage;
#pragma unroll
  for (int g = 0; g < kRkGroup; ++g) {
    const int w = tid + (k0 + g) * NT;
    if (!(tid < NT && k0 + g < IT && w < TILE4)) continue;
    const int qq = w / SEG4, r4 = w - (w / SEG4) * SEG4;
    const int64_t gi = qq * a.stride + e0 * NP + (int64_t)r4 * 4;
    const float4 v = *reinterpret_cast<const float4*>(sK + qq * ET * NP + r4 * 4);
    switch (stage) {
      case 0:
        *reinterpret_cast<float4*>(a.k_out + gi) = v;
        break;
      case 1: {
        const float4 y = o.x0[g];
        *reinterpret_cast<float4*>(a.acc + gi) = v;
        *reinterpret_cast<float4*>(a.y_out + gi) =
            make_float4(y.x + 0.5f * v.x, y.y + 0.5f * v.y, y.z + 0.5f * v.z, y.w + 0.5f * v.w);
        break;
      }
      case 2:
      case 3: {
        const float4 u = o.x0[g], ac = o.x1[g];
        const float c = stage == 2 ? 0.5f : 1.0f;
        *reinterpret_cast<float4*>(a.acc + gi) =
            make_float4(ac.x + 2.f * v.x, ac.y + 2.f * v.y, ac.z + 2.f * v.z, ac.w + 2.f * v.w);
        *reinterpret_cast<float4*>(a.y_out + gi) = make_float4(u.x + c * v.x, u.y + c * v.y, u.z + c * v.z, u.w + c * v.w);
        break;
      }
      case 4: {
        const float4 u = o.x0[g], ac = o.x1[g], sn = o.x2[g];
        const float4 un = make_float4(u.x + rk4_sixth(ac.x + v.x), u.y + rk4_sixth(ac.y + v.y),
                                      u.z + rk4_sixth(ac.z + v.z), u.w + rk4_sixth(ac.w + v.w));
        *reinterpret_cast<float4*>(a.u + gi) = un;
        racc.add(qq, sn.x, un.x, a.c0sq);
        racc.add(qq, sn.y, un.y, a.c0sq);
        racc.add(qq, sn.z, un.z, a.c0sq);
        racc.add(qq, sn.w, un.w, a.c0sq);
        break;
      }
      default: {
        const float4 y = o.x0[g];
        *reinterpret_cast<float4*>(a.y_out + gi) = make_float4(y.x + v.x, y.y + v.y, y.z + v.z, y.w + v.w);
        break;
      }
    }
  }
}

// One tile of the wide-chunk stage for elements e0 .. e0+ET-1 (see the file
// comment); the arguments are pipe_tile's. sD holds Dt [D][NP j][NPR i], sL
// the negated LIFT [NK][NPR i], both zero past NP.
template <class C>
__device__ __forceinline__ void wide_tile(const StageArgs<float>& a, int64_t e0, float* sY, const float* sGF,
                                          const int* sGI, const float* sE, float* sN, const float* sD, const float* sL,
                                          const short* sFm, const short* sNb, uint64_t* bar_epi, uint32_t epi_parity,
                                          int nepi, int tid, bool& ok, ResAcc<float>& racc) {
  constexpr int D = C::D, NP = C::NP, NV = C::NV, NK = C::NK, NC = C::NC, NH = C::NH, NSPLIT = C::NSPLIT;
  constexpr int ET = C::ET, RECF = C::RECF, NPR = C::NPR, OVW = C::OVW, NVQ = C::NVQ;
  const float rhoc2 = a.f_rhoc2, inv_rho0 = a.f_inv_rho0, half_c0 = a.f_half_c0;
  // a block larger than this shape's NT (the mixed-order kernel) leaves its
  // other threads idle in this tile; they only take part in the barriers
  const bool active = tid < C::NT;
  const int e = active ? tid / NSPLIT : 0, s = active ? tid - (tid / NSPLIT) * NSPLIT : 0;
  const int i0 = s * NC;
  if constexpr (!C::kStaged) {
    // RK operands of this tile towards L2 (read by the coalesced update)
    if (tid < NV * nepi) {
      const int k = tid / NV, q = tid - (tid / NV) * NV;
      const float* src = k == 0 ? a.u : (k == 1 ? a.acc : a.snap);
      prefetch_l2(src + q * a.stride + e0 * NP, C::YSEG);
    }
  }
  // ---- neighbour traces: asynchronous gathers into sN ----
  if (active) gather_traces<C, float>(a.y_in, a.stride, sGI, sNb, sN, tid, e0);
  cp_async_commit();

  // element coefficients: gv0_r = sum_d G_rd v0_d, rho0 c0^2 G, G / rho0
  float gv0[D], cp[D][D], cv[D][D];
  {
    const float* G = sGF + e * RECF;
    const float* ev0 = G + C::S::PHYS_OFF;
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float x = G[r * D] * ev0[0];
#pragma unroll
      for (int d = 1; d < D; ++d) x = fmaf(G[r * D + d], ev0[d], x);
      gv0[r] = x;
#pragma unroll
      for (int d = 0; d < D; ++d) cp[r][d] = rhoc2 * G[r * D + d], cv[r][d] = G[r * D + d] * inv_rho0;
    }
  }
  float2 L2[NH][NV];
#pragma unroll
  for (int h = 0; h < NH; ++h)
#pragma unroll
    for (int q = 0; q < NV; ++q) L2[h][q] = make_float2(0.f, 0.f);
  const float* ye = sY + e * NP;
  if (active) {
    if constexpr (C::FORM == kFluxForm) {
      // ---- volume term: L[i][q] = sum_j sum_r Dt_r[i][j] F_rq(y_j) ----
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        float y[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) y[q] = ye[q * ET * NP + j];
#pragma unroll
        for (int r = 0; r < D; ++r) {
          // pressure: gv0_r p + rho0 c0^2 sum_d G_rd v_d; v_d: gv0_r v_d + G_rd p / rho0
          float F[NV];
          F[0] = gv0[r] * y[0];
#pragma unroll
          for (int d = 0; d < D; ++d) F[0] = fmaf(cp[r][d], y[1 + d], F[0]);
#pragma unroll
          for (int d = 0; d < D; ++d) F[1 + d] = fmaf(cv[r][d], y[0], gv0[r] * y[1 + d]);
          float dv[NC];
#pragma unroll
          for (int c = 0; c < NC; c += OVW) vload<float, OVW>(dv + c, sD + (r * NP + j) * NPR + i0 + c);
#pragma unroll
          for (int h = 0; h < NH; ++h) {
            const float2 dp = make_float2(dv[2 * h], dv[2 * h + 1]);
#pragma unroll
            for (int q = 0; q < NV; ++q) L2[h][q] = __ffma2_rn(dp, make_float2(F[q], F[q]), L2[h][q]);
          }
        }
      }
    } else {
      // ---- volume term: W_r[i][q] = sum_j Dt_r[i][j] y_q[j], then the
      // metric mixing L[i][0] = sum_r gv0_r W_r[i][0] + rho0 c0^2 G_rd W_r[i][1+d],
      // L[i][1+d] = sum_r gv0_r W_r[i][1+d] + G_rd W_r[i][0] / rho0 ----
      float2 W2[D][NH][NV];
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int h = 0; h < NH; ++h)
#pragma unroll
          for (int q = 0; q < NV; ++q) W2[r][h][q] = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < NP; ++j) {
        float y[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) y[q] = ye[q * ET * NP + j];
#pragma unroll
        for (int r = 0; r < D; ++r) {
          float dv[NC];
#pragma unroll
          for (int c = 0; c < NC; c += OVW) vload<float, OVW>(dv + c, sD + (r * NP + j) * NPR + i0 + c);
#pragma unroll
          for (int h = 0; h < NH; ++h) {
            const float2 dp = make_float2(dv[2 * h], dv[2 * h + 1]);
#pragma unroll
            for (int q = 0; q < NV; ++q) W2[r][h][q] = __ffma2_rn(dp, make_float2(y[q], y[q]), W2[r][h][q]);
          }
        }
      }
#pragma unroll
      for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int r = 0; r < D; ++r) {
          const float2 g0 = make_float2(gv0[r], gv0[r]);
          L2[h][0] = __ffma2_rn(g0, W2[r][h][0], L2[h][0]);
#pragma unroll
          for (int d = 0; d < D; ++d) {
            L2[h][0] = __ffma2_rn(make_float2(cp[r][d], cp[r][d]), W2[r][h][1 + d], L2[h][0]);
            L2[h][1 + d] = __ffma2_rn(g0, W2[r][h][1 + d], L2[h][1 + d]);
            L2[h][1 + d] = __ffma2_rn(make_float2(cv[r][d], cv[r][d]), W2[r][h][0], L2[h][1 + d]);
          }
        }
    }
  }
  cp_async_wait_all();
  __syncthreads();

  // ---- face numerical fluxes (in place of the gathered traces) ----
  if (active) face_fluxes<C, float>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, tid, rhoc2, inv_rho0, half_c0, e0);
  __syncthreads();

  // operands of the first group of RK-update items, in flight during the lift
  RkOps rk;
  if constexpr (!C::kStaged) wide_rk_load<C>(a, sY, e0, tid, 0, rk);

  // ---- lifting (sL holds -LIFT: the products accumulate) ----
  if (active) {
    const float* hrow = sN + (size_t)e * C::SN_EL;
#pragma unroll
    for (int k = 0; k < NK; ++k) {
      float hq[NVQ];
      vload<float, NVQ>(hq, hrow + k * NVQ);
      float lv[NC];
#pragma unroll
      for (int c = 0; c < NC; c += OVW) vload<float, OVW>(lv + c, sL + k * NPR + i0 + c);
#pragma unroll
      for (int h = 0; h < NH; ++h) {
        const float2 lp = make_float2(lv[2 * h], lv[2 * h + 1]);
#pragma unroll
        for (int q = 0; q < NV; ++q) L2[h][q] = __ffma2_rn(lp, make_float2(hq[q], hq[q]), L2[h][q]);
      }
    }
  }
  const float dte = a.f_dt * sGF[e * RECF + C::S::PHYS_OFF + D];  // dt times the element's step scale

  if constexpr (!C::kStaged) {
    // ---- dt*L into the face buffer ([q][e][i]), then the coalesced update ----
    float* sK = sN;
    __syncthreads();  // every thread has read the face fluxes
    if (active) {
#pragma unroll
      for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int i = i0 + 2 * h + u;
          if (i < NP)
#pragma unroll
            for (int q = 0; q < NV; ++q) sK[(q * ET + e) * NP + i] = dte * (u ? L2[h][q].y : L2[h][q].x);
        }
    }
    __syncthreads();
    if (ok) {
      constexpr int IT = (C::NV * ET * NP / 4 + C::NT - 1) / C::NT;
#pragma unroll
      for (int k0 = 0; k0 < IT; k0 += kRkGroup) {
        if (k0 > 0) wide_rk_load<C>(a, sY, e0, tid, k0, rk);
        wide_rk_store<C>(a, sK, e0, tid, k0, rk, racc);
      }
    }
  } else {
    // ---- RK update from registers ----
    if (nepi > 0 && ok && !mbar_wait(bar_epi, epi_parity, a.wait_limit)) ok = false;
    // after a timeout the operand buffer may still be landing: no RK update
    if (!active || !ok) return;
    float Lv[NC][NV];
#pragma unroll
    for (int h = 0; h < NH; ++h)
#pragma unroll
      for (int q = 0; q < NV; ++q) Lv[2 * h][q] = L2[h][q].x, Lv[2 * h + 1][q] = L2[h][q].y;
    rk_update_regs<float, NC, NV, C::VW, ET, NP>(a, e0, e, i0, Lv, (nepi > 0) ? sE : sY, sE, dte, racc);
  }
}

// Two elements per thread (W form, operands not staged): a thread owns the
// same chunk of NC output nodes of elements e and e + ET/2 of the tile, so
// that every operator entry it loads from shared memory feeds 2 x NV FMAs
// instead of NV (the volume and lift phases take half the operator
// wavefronts per element); ET/2 x NSPLIT threads per tile.
template <int D_, int P, int NC_, int ET_>
struct WideEB : Wide<D_, P, NC_, ET_, kWForm, false> {
  using Base = Wide<D_, P, NC_, ET_, kWForm, false>;
  static constexpr int EB = 2;
  static constexpr int NT = ET_ / 2 * Base::NSPLIT;
  static_assert(NT % 32 == 0, "threads per block must be a multiple of 32");
  static_assert(ET_ % 2 == 0, "two elements per thread");
};

template <class C>
__device__ __forceinline__ void wide_mix(const float* sGF, int e, float rhoc2, float inv_rho0,
                                         const float2 (&W2)[C::D][C::NH][C::NV], float2 (&L2)[C::NH][C::NV]) {
  constexpr int D = C::D, NH = C::NH, RECF = C::RECF;
  const float* G = sGF + e * RECF;
  const float* ev0 = G + C::S::PHYS_OFF;
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float x = G[r * D] * ev0[0];
#pragma unroll
    for (int d = 1; d < D; ++d) x = fmaf(G[r * D + d], ev0[d], x);
    const float2 g0 = make_float2(x, x);
#pragma unroll
    for (int h = 0; h < NH; ++h) {
      L2[h][0] = __ffma2_rn(g0, W2[r][h][0], L2[h][0]);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const float cpv = rhoc2 * G[r * D + d], cvv = G[r * D + d] * inv_rho0;
        L2[h][0] = __ffma2_rn(make_float2(cpv, cpv), W2[r][h][1 + d], L2[h][0]);
        L2[h][1 + d] = __ffma2_rn(g0, W2[r][h][1 + d], L2[h][1 + d]);
        L2[h][1 + d] = __ffma2_rn(make_float2(cvv, cvv), W2[r][h][0], L2[h][1 + d]);
      }
    }
  }
}

// One tile of the two-elements-per-thread stage (see WideEB); the arguments
// are pipe_tile's.
template <class C>
__device__ __forceinline__ void wide_eb_tile(const StageArgs<float>& a, int64_t e0, float* sY, const float* sGF,
                                             const int* sGI, const float* sE, float* sN, const float* sD,
                                             const float* sL, const short* sFm, const short* sNb, uint64_t* bar_epi,
                                             uint32_t epi_parity, int nepi, int tid, bool& ok, ResAcc<float>& racc) {
  constexpr int D = C::D, NP = C::NP, NV = C::NV, NK = C::NK, NC = C::NC, NH = C::NH, NSPLIT = C::NSPLIT;
  constexpr int ET = C::ET, RECF = C::RECF, NPR = C::NPR, OVW = C::OVW, NVQ = C::NVQ, EH = ET / 2;
  const float rhoc2 = a.f_rhoc2, inv_rho0 = a.f_inv_rho0, half_c0 = a.f_half_c0;
  const bool active = tid < C::NT;
  const int ep = active ? tid / NSPLIT : 0, s = active ? tid - (tid / NSPLIT) * NSPLIT : 0;
  const int ea = ep, eb = ep + EH;  // the thread's two elements
  const int i0 = s * NC;
  // RK operands of this tile towards L2 (read by the coalesced update)
  if (tid < NV * nepi) {
    const int k = tid / NV, q = tid - (tid / NV) * NV;
    const float* src = k == 0 ? a.u : (k == 1 ? a.acc : a.snap);
    prefetch_l2(src + q * a.stride + e0 * NP, C::YSEG);
  }
  // ---- neighbour traces: asynchronous gathers into sN ----
  if (active) gather_traces<C, float>(a.y_in, a.stride, sGI, sNb, sN, tid, e0);
  cp_async_commit();

  float2 La[NH][NV], Lb[NH][NV];
#pragma unroll
  for (int h = 0; h < NH; ++h)
#pragma unroll
    for (int q = 0; q < NV; ++q) La[h][q] = Lb[h][q] = make_float2(0.f, 0.f);
  if (active) {
    // ---- volume term per reference direction for both elements, then
    // the metric mixing per element ----
    float2 Wa[D][NH][NV], Wb[D][NH][NV];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) Wa[r][h][q] = Wb[r][h][q] = make_float2(0.f, 0.f);
    const float* ya = sY + ea * NP;
    const float* yb = sY + eb * NP;
#pragma unroll 4
    for (int j = 0; j < NP; ++j) {
      float y1[NV], y2[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) y1[q] = ya[q * ET * NP + j], y2[q] = yb[q * ET * NP + j];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float dv[NC];
#pragma unroll
        for (int c = 0; c < NC; c += OVW) vload<float, OVW>(dv + c, sD + (r * NP + j) * NPR + i0 + c);
#pragma unroll
        for (int h = 0; h < NH; ++h) {
          const float2 dp = make_float2(dv[2 * h], dv[2 * h + 1]);
#pragma unroll
          for (int q = 0; q < NV; ++q) {
            Wa[r][h][q] = __ffma2_rn(dp, make_float2(y1[q], y1[q]), Wa[r][h][q]);
            Wb[r][h][q] = __ffma2_rn(dp, make_float2(y2[q], y2[q]), Wb[r][h][q]);
          }
        }
      }
    }
    wide_mix<C>(sGF, ea, rhoc2, inv_rho0, Wa, La);
    wide_mix<C>(sGF, eb, rhoc2, inv_rho0, Wb, Lb);
  }
  cp_async_wait_all();
  __syncthreads();

  // ---- face numerical fluxes (in place of the gathered traces) ----
  if (active) face_fluxes<C, float>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, tid, rhoc2, inv_rho0, half_c0, e0);
  __syncthreads();

  // operands of the first group of RK-update items, in flight during the lift
  RkOps rk;
  wide_rk_load<C>(a, sY, e0, tid, 0, rk);

  // ---- lifting for both elements (sL holds -LIFT) ----
  if (active) {
    const float* ha = sN + (size_t)ea * C::SN_EL;
    const float* hb = sN + (size_t)eb * C::SN_EL;
#pragma unroll 4
    for (int k = 0; k < NK; ++k) {
      float h1[NVQ], h2[NVQ];
      vload<float, NVQ>(h1, ha + k * NVQ);
      vload<float, NVQ>(h2, hb + k * NVQ);
      float lv[NC];
#pragma unroll
      for (int c = 0; c < NC; c += OVW) vload<float, OVW>(lv + c, sL + k * NPR + i0 + c);
#pragma unroll
      for (int h = 0; h < NH; ++h) {
        const float2 lp = make_float2(lv[2 * h], lv[2 * h + 1]);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          La[h][q] = __ffma2_rn(lp, make_float2(h1[q], h1[q]), La[h][q]);
          Lb[h][q] = __ffma2_rn(lp, make_float2(h2[q], h2[q]), Lb[h][q]);
        }
      }
    }
  }
  // ---- dt*L into the face buffer ([q][e][i]), then the coalesced update ----
  const float dta = a.f_dt * sGF[ea * RECF + C::S::PHYS_OFF + D];
  const float dtb = a.f_dt * sGF[eb * RECF + C::S::PHYS_OFF + D];
  float* sK = sN;
  __syncthreads();  // every thread has read the face fluxes
  if (active) {
#pragma unroll
    for (int h = 0; h < NH; ++h)
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int i = i0 + 2 * h + u;
        if (i < NP)
#pragma unroll
          for (int q = 0; q < NV; ++q) {
            sK[(q * ET + ea) * NP + i] = dta * (u ? La[h][q].y : La[h][q].x);
            sK[(q * ET + eb) * NP + i] = dtb * (u ? Lb[h][q].y : Lb[h][q].x);
          }
      }
  }
  __syncthreads();
  if (ok) {
    constexpr int IT = (C::NV * ET * NP / 4 + C::NT - 1) / C::NT;
#pragma unroll
    for (int k0 = 0; k0 < IT; k0 += kRkGroup) {
      if (k0 > 0) wide_rk_load<C>(a, sY, e0, tid, k0, rk);
      wide_rk_store<C>(a, sK, e0, tid, k0, rk, racc);
    }
  }
}

struct WideEBTileOps {
  template <class C, typename T>
  __device__ static void load_ops(T* sD, T* sL, const StageArgs<T>& a, int tid, int nthreads = C::NT);
  template <class C, typename T>
  __device__ static void run(const StageArgs<T>& a, int64_t e0, T* sY, const T* sGF, const int* sGI, const T* sE,
                             T* sN, const T* sD, const T* sL, const short* sFm, const short* sNb, uint64_t* bar_epi,
                             uint32_t epi_parity, int nepi, int tid, bool& ok, ResAcc<T>& racc) {
    wide_eb_tile<C>(a, e0, sY, sGF, sGI, sE, sN, sD, sL, sFm, sNb, bar_epi, epi_parity, nepi, tid, ok, racc);
  }
};

// Operator tables (zero-padded rows) and tile body of the wide-chunk kernel.
struct WideTileOps {
  template <class C, typename T>
  __device__ static void load_ops(T* sD, T* sL, const StageArgs<T>& a, int tid, int nthreads = C::NT) {
    constexpr int NP = C::NP, NPR = C::NPR;
    for (int w = tid; w < C::D * NP * NPR; w += nthreads) {
      const int row = w / NPR, i = w - (w / NPR) * NPR;
      sD[w] = i < NP ? a.Dt[row * NP + i] : (T)0;
    }
    for (int w = tid; w < C::NK * NPR; w += nthreads) {
      const int k = w / NPR, i = w - (w / NPR) * NPR;
      sL[w] = i < NP ? -a.LIFT[k * NP + i] : (T)0;
    }
  }
  template <class C, typename T>
  __device__ static void run(const StageArgs<T>& a, int64_t e0, T* sY, const T* sGF, const int* sGI, const T* sE,
                             T* sN, const T* sD, const T* sL, const short* sFm, const short* sNb, uint64_t* bar_epi,
                             uint32_t epi_parity, int nepi, int tid, bool& ok, ResAcc<T>& racc) {
    wide_tile<C>(a, e0, sY, sGF, sGI, sE, sN, sD, sL, sFm, sNb, bar_epi, epi_parity, nepi, tid, ok, racc);
  }
};

template <class C, typename T>
__device__ void WideEBTileOps::load_ops(T* sD, T* sL, const StageArgs<T>& a, int tid, int nthreads) {
  WideTileOps::load_ops<C, T>(sD, sL, a, tid, nthreads);
}

// configuration and tile body of a variant (FORM kWForm2: two elements per
// thread, operands not staged)
template <int D, int P, int NC_, int ET_, int FORM, bool STAGED>
struct Stage4Sel {
  using C = Wide<D, P, NC_, ET_, FORM, STAGED>;
  using Ops = WideTileOps;
};
template <int D, int P, int NC_, int ET_, bool STAGED>
struct Stage4Sel<D, P, NC_, ET_, kWForm2, STAGED> {
  using C = WideEB<D, P, NC_, ET_>;
  using Ops = WideEBTileOps;
};

template <int D, int P, int NC_, int ET_, int FORM, bool STAGED>
__global__ void __launch_bounds__(Stage4Sel<D, P, NC_, ET_, FORM, STAGED>::C::NT)
    stage4_kernel(const StageArgs<float> a, int* err) {
  extern __shared__ __align__(128) unsigned char sm[];
  using Sel = Stage4Sel<D, P, NC_, ET_, FORM, STAGED>;
  pipe_loop<typename Sel::C, float, typename Sel::Ops>(a, err, sm);
}

template <int D, int P, int NC_, int ET_, int FORM, bool STAGED>
struct Stage4 {
  using C = typename Stage4Sel<D, P, NC_, ET_, FORM, STAGED>::C;
  static cudaError_t set_attrs() {
    auto kfn = stage4_kernel<D, P, NC_, ET_, FORM, STAGED>;
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
    stage4_kernel<D, P, NC_, ET_, FORM, STAGED><<<grid, C::NT, C::bytes, s>>>(a, err);
    return cudaGetLastError();
  }
  static int blocks_per_sm() {
    // a configuration larger than an SM's shared memory is reported as
    // unavailable; the failed query leaves no sticky launch error
    if (set_attrs() != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stage4_kernel<D, P, NC_, ET_, FORM, STAGED>, C::NT,
                                                      C::bytes) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return nb;
  }
};

}  // namespace dgk
