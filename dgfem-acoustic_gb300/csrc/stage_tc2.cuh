// Tensor-core fused RK4 stage kernel, two-chunk form (sm_103a, FP32 state,
// tcgen05 TF32 with two-term splits of both operands), built so that two
// blocks share an SM.
//
// Same arithmetic as stage_tc.cuh (the RHS of a tile of ET elements is one
// GEMM D = A B^T with rows m = (q,e), K = the contravariant volume fluxes
// (r,j) then the scaled face fluxes k, N = output node i; B = [Dt_1..Dt_D |
// -LIFT], TF32 products of the split operands, FP32 accumulate),
// following src/Mesh.cpp:734-975, src/solver.cpp:38-57 and :488-516. What
// differs is the resource plan. One pipeline per block holds every phase of
// a tile in sequence (TMA load, neighbour gathers, A construction, MMA,
// epilogue); at 3-D p = 4 the single block per SM that the one-chunk kernel
// fits (384 tensor-memory columns, 170 KB of shared memory) left the SM idle
// through each phase's latency. Here:
//   * K is applied in at most two chunks, A (head and tail) for one chunk at
//     a time, so that a block's tensor memory (D + 2 KC columns) is at most
//     256 columns: two blocks per SM, each hiding the other's waits; the
//     second chunk's correction products go to a second accumulator in the
//     A region's free columns (tc2_mma_chunk);
//   * the tile buffer is single: the next tile's TMA load is issued as soon as
//     the current tile's stage input has been turned into A and face fluxes
//     (it overlaps the last MMA chunk and the epilogue);
//   * the RK operands are not staged: the epilogue writes dt*L of the tile
//     into shared memory in the state's [q][e][i] layout, then one coalesced
//     float4 pass over the tile reads u, the accumulator and the snapshot
//     from global memory (prefetched to L2 when the tile starts; a thread's
//     first items loaded before the last chunk's wait) and writes the new
//     values straight back;
//   * the MMAs are issued by one converged warp as an unrolled run (one lane
//     executes them), the neighbour gathers share the phase of the first
//     chunk's volume columns, and A's tails go to the MMAs unrounded (the
//     schedule was set by timing each phase of a tile on the SM clock).
// 3-D p = 4: 109 KB of shared memory and 256 tensor-memory columns per block.
// Every wait is bounded (StageArgs::wait_limit polling rounds); a block that
// gives up issues no further copy or MMA, waits (default limit) for its own
// copies and MMAs in flight, frees its tensor memory, sets the error flag
// and returns.
#pragma once
#include <cstdint>

#include "stage_tc.cuh"

namespace dgk {

template <int D_, int P, int NPART_>
struct Tc2Cfg {
  using T = float;
  using S = ShapeT<D_, P, float>;
  static constexpr int D = D_;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM, NK = NF * NFP;
  static constexpr int ET = 32;            // elements per tile
  static constexpr int ROWS = NV * ET;     // used rows of the M = 128 tile
  static constexpr int NPART = NPART_;     // threads per row: columns split NPART ways
  static constexpr int NT = 128 * NPART;   // lane quarters x parts
  static constexpr int RECF = S::RECF, RECI = S::RECI;
  // RK update: the first kRkEarly float4 items of a thread have their
  // operands loaded before the last MMA chunk's wait (0: none); the
  // accumulator columns are read in kEpiPasses passes (registers)
  static constexpr int kRkEarly = 2;
  // the other items' operand loads issued before the epilogue's barrier
  // (after the accumulator columns are read, whose registers are free then)
  static constexpr bool kRkRestEarly = true;
  static constexpr int kEpiPasses = 2;
  // A's tail (x - TF32(x)) handed to the MMA as FP32 bits: the tensor core
  // reads its TF32 bits, which drops the second rounding instruction per A
  // value (tail error at most 2^-21 of the value instead of 2^-22)
  static constexpr bool kRawTail = true;
  // neighbour gathers issued after the barrier that publishes the
  // per-element values, in the same phase as the first chunk's volume
  // columns (the pressure rows' warps, with more volume columns, take fewer
  // gather items), rather than before it
  static constexpr bool kGatherWithVolume = true;
  // face buffer: one plane per variable [NV][ET][NKP] (gather_traces /
  // face_fluxes strides); it also holds dt*L of the tile [NV][ET][NP] in the
  // epilogue
  static constexpr int NKP = NK | 1;
  static constexpr int NVQ = 1, SN_EL = NKP, SN_K = 1, SN_Q = ET * NKP;
  static constexpr int NPP = RoundUpTc<NP, 4>::v;       // volume block width per direction
  static constexpr int KV = D * NPP;                     // volume columns
  static constexpr int KF = RoundUpTc<NK, 4>::v;         // face columns
  static constexpr int KT = RoundUpTc<KV + KF, 8>::v;    // K (multiple of the TF32 MMA depth 8)
  static constexpr int NN = RoundUpTc<NP, 16>::v;        // N (multiple of 16 for M = 128)
  // K chunks: D + A head + A tail within 256 columns. The first chunk is as
  // wide as that allows (KC); a second chunk takes the rest (KC2), and its
  // A leaves room in the A region for a second accumulator DC that takes
  // its correction products (see tc2_mma_chunk)
  static constexpr int KCMAX = (256 - NN) / 2 / 8 * 8;
  static constexpr int NCH = KT <= KCMAX ? 1 : 2;
  static constexpr int KC = NCH == 1 ? KT : KCMAX;
  static constexpr int KC2 = KT - KC;
  static constexpr int COL_D = 0, COL_AH = NN, COL_AL = NN + KC;  // tensor-memory columns
  static constexpr int COL_AL2 = NN + KC2, COL_DC = NN + 2 * KC2;  // second chunk: A tail, DC
  static constexpr int TCOLS = Pow2Cols<NN + 2 * KC>::v;
  static constexpr int GT = D * D + D + 1;               // per-element values of the row phase
  static constexpr int VWY = (NP % 4 == 0) ? 4 : (NP % 2 == 0) ? 2 : 1;
  static constexpr uint32_t YSEG = ET * NP * sizeof(float);
  static constexpr uint32_t GFB = ET * RECF * sizeof(float);
  static constexpr uint32_t GIB = ET * RECI * sizeof(int);
  static constexpr int TILE4 = NV * ET * NP / 4;         // float4 of one tile
  // B with only the 8-row groups that hold nodes (as in stage_tc.cuh)
  static constexpr int NG = (NP + 7) / 8;
  static constexpr uint32_t BBYTES = (KT / 4) * NG * 128;
  static constexpr uint32_t BSLACK = (NN / 8 - NG) * 128;
  static constexpr uint32_t LBO = NG * 128, SBO = 128;
  // shared memory layout (bytes)
  static constexpr size_t oBar = 0;                        // 2 mbarriers + tensor-memory address
  static constexpr size_t oBh = 128;
  static constexpr size_t oBl = oBh + BBYTES;
  static constexpr size_t oFm = RoundUpTc<oBl + BBYTES + BSLACK, 16>::v;
  static constexpr size_t oNb = oFm + RoundUpTc<NK * 2, 16>::v;
  static constexpr size_t oGT = RoundUpTc<oNb + NF * NPERM * NFP * 2, 16>::v;   // [GT][ET+1]
  static constexpr size_t oY = RoundUpTc<oGT + GT * (ET + 1) * 4, 128>::v;     // [NV][ET][NP]
  static constexpr size_t oGF = oY + (size_t)NV * YSEG;
  static constexpr size_t oGI = oGF + GFB;
  static constexpr size_t oN = RoundUpTc<oGI + GIB, 128>::v;                   // [NV][ET][NKP]
  static constexpr size_t oR = RoundUpTc<oN + (size_t)NV * ET * NKP * 4, 16>::v;  // [NT/32][5] double
  static constexpr size_t bytes = oR + (NT / 32) * 5 * sizeof(double);
  static_assert(KT <= 2 * KCMAX, "K must fit in two chunks");
  static_assert(NCH == 1 || COL_DC + NN <= NN + 2 * KC, "the second accumulator must fit in the A region");
  static_assert(ROWS <= 128, "rows of a tile exceed the MMA height");
  static_assert(NN + 2 * KC <= 256, "tensor memory of a block exceeds 256 columns");
  static_assert(NV * ET * NP <= NV * ET * NKP, "dt*L of a tile must fit in the face buffer");
  static_assert((ET * NP) % 4 == 0, "tile segments must be float4 multiples");
  static_assert(YSEG % 16 == 0, "tile segments must be 16-byte multiples");
  static_assert(bytes <= 227 * 1024, "shared memory of one block exceeds 227 KB");
};

// Head and tail of 4 A values (split4, or with the tail as FP32 bits: kRawTail)
template <class C>
__device__ __forceinline__ void tc2_split4(const float* x, uint32_t* hi, uint32_t* lo) {
  if constexpr (C::kRawTail) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      hi[u] = tf32_rna(x[u]);
      lo[u] = __float_as_uint(x[u] - __uint_as_float(hi[u]));
    }
  } else {
    split4(x, hi, lo);
  }
}

// Volume columns [kc0, kc1) of row (Q, e) into tensor memory, the variable
// Q fixed at compile time (each warp owns rows of one variable):
//   A_vol[(Q,e)][r*NPP + j] = sum_d G_rd F_{Q,d}(y_j)
//   Q = 0 (pressure):  gv0_r p_j + sum_d (rho0 c0^2 G_rd) v_d,j
//   Q = 1+d (v_d):     gv0_r v_d,j + (G_rd / rho0) p_j
// with gv0_r = sum_d G_rd v0_d, each value split into a TF32 head and a
// TF32 tail at columns COL_AH / col_al + (col - kc0). cf holds the element's
// coefficients: gv0 (D values), then rho0 c0^2 G (D*D, Q = 0) or G_rQ / rho0
// (D, Q > 0). The thread takes the 4-node groups j0 = 4*(part + t*NPART);
// the last group of an NP that is not a multiple of 4 reads the last node
// again (its columns meet zero rows of B).
template <class C, int Q>
__device__ __forceinline__ void tc2_build_vol(const float* sY, const float* cf, int e, int part, uint32_t trow,
                                              int kc0, int kc1, int col_al) {
  constexpr int D = C::D, NP = C::NP, NPP = C::NPP, ET = C::ET;
  const float* yp_row = sY + e * NP;                               // pressure
  const float* yq_row = sY + (Q == 0 ? 1 : Q) * ET * NP + e * NP;  // v_x (Q = 0) or v_Q
#pragma unroll 1
  for (int g4 = part; g4 < NPP / 4; g4 += C::NPART) {
    const int j0 = g4 * 4;
    bool any = false;
#pragma unroll
    for (int r = 0; r < D; ++r) any |= (r * NPP + j0 >= kc0 && r * NPP + j0 < kc1);
    if (!any) continue;  // warp-uniform
    float yp[4], yv[Q == 0 ? D : 1][4];
    if (j0 + 4 <= NP) {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        yp[u] = yp_row[j0 + u];
#pragma unroll
        for (int d = 0; d < (Q == 0 ? D : 1); ++d) yv[d][u] = yq_row[d * ET * NP + j0 + u];
      }
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int j = j0 + u < NP ? j0 + u : NP - 1;
        yp[u] = yp_row[j];
#pragma unroll
        for (int d = 0; d < (Q == 0 ? D : 1); ++d) yv[d][u] = yq_row[d * ET * NP + j];
      }
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
      const int col = r * NPP + j0;
      if (col < kc0 || col >= kc1) continue;  // warp-uniform
      float fr[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        float x;
        if constexpr (Q == 0) {
          x = cf[r] * yp[u];
#pragma unroll
          for (int d = 0; d < D; ++d) x = fmaf(cf[D + r * D + d], yv[d][u], x);
        } else {
          x = fmaf(cf[D + r], yp[u], cf[r] * yv[0][u]);
        }
        // a column past NP (the clamped last node's value, finite) meets
        // a zero row of B: no mask needed
        fr[u] = x;
      }
      uint32_t hi[4], lo[4];
      tc2_split4<C>(fr, hi, lo);
      tmem_st4(trow + C::COL_AH + (col - kc0), hi);
      tmem_st4(trow + col_al + (col - kc0), lo);
    }
  }
}

// The element's coefficients of row variable q (see tc2_build_vol) from the
// element-minor per-element values sGT [GT][ET+1]: G (D*D), v0 (D).
template <class C>
__device__ __forceinline__ void tc2_coeffs(const float* sGT, int q, int e, float rhoc2, float inv_rho0,
                                           float (&cf)[C::D + C::D * C::D]) {
  constexpr int D = C::D, ET = C::ET;
  float g[D][D], v0[D];
#pragma unroll
  for (int r = 0; r < D; ++r)
#pragma unroll
    for (int d = 0; d < D; ++d) g[r][d] = sGT[(r * D + d) * (ET + 1) + e];
#pragma unroll
  for (int d = 0; d < D; ++d) v0[d] = sGT[(D * D + d) * (ET + 1) + e];
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float x = g[r][0] * v0[0];
#pragma unroll
    for (int d = 1; d < D; ++d) x = fmaf(g[r][d], v0[d], x);
    cf[r] = x;
  }
  if (q == 0) {
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int d = 0; d < D; ++d) cf[D + r * D + d] = rhoc2 * g[r][d];
  } else {
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float x = g[r][0];
#pragma unroll
      for (int d = 1; d < D; ++d)
        if (q == 1 + d) x = g[r][d];
      cf[D + r] = x * inv_rho0;
    }
  }
}

// tc2_build_vol for the row's variable q (warp-uniform).
template <class C>
__device__ __forceinline__ void tc2_build_vol_q(int q, const float* sY, const float* cf, int e, int part,
                                                uint32_t trow, int kc0, int kc1, int col_al) {
  switch (q) {
    case 0: tc2_build_vol<C, 0>(sY, cf, e, part, trow, kc0, kc1, col_al); break;
    case 1: tc2_build_vol<C, 1>(sY, cf, e, part, trow, kc0, kc1, col_al); break;
    case 2: tc2_build_vol<C, 2>(sY, cf, e, part, trow, kc0, kc1, col_al); break;
    default:
      if constexpr (C::D == 3) tc2_build_vol<C, 3>(sY, cf, e, part, trow, kc0, kc1, col_al);
      break;
  }
}

// Face columns (and the zero padding after them) of [kc0, kc1) of this
// thread's row from the face-flux plane of variable q.
template <class C>
__device__ __forceinline__ void tc2_build_face(const float* sN, int q, int e, int part, uint32_t trow, int kc0,
                                               int kc1, int col_al) {
  constexpr int KV = C::KV, NK = C::NK;
  const float* hrow = sN + (size_t)(q * C::ET + e) * C::NKP;
  for (int c4 = part; c4 < (C::KT - KV) / 4; c4 += C::NPART) {
    const int col = KV + c4 * 4;
    if (col < kc0 || col >= kc1) continue;  // warp-uniform
    float x[4];
    if constexpr (C::KT - KV == NK) {  // no padding columns
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = hrow[c4 * 4 + u];
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = (c4 * 4 + u < NK) ? hrow[c4 * 4 + u] : 0.f;
    }
    uint32_t hi[4], lo[4];
    tc2_split4<C>(x, hi, lo);
    tmem_st4(trow + C::COL_AH + (col - kc0), hi);
    tmem_st4(trow + col_al + (col - kc0), lo);
  }
}

// One chunk's MMAs (issued by one thread) over K columns [kc0, kc1), then a
// commit to bar: the correction products A_lo B_hi and A_hi B_lo into the
// accumulator at column dcorr, then the head products A_hi B_hi into D. Each
// MMA's FP32 accumulation rounds relative to the accumulator it adds to, so
// the small correction products must not be added to an accumulator that
// already holds a large sum: the first chunk adds them to D before its head
// products (D still small), the second chunk to its own accumulator DC,
// which the epilogue adds to D. (The operator is split exactly, split_op22;
// the dropped A_lo B_lo is below 2^-22 of a product.)
//
// The whole issuing warp runs this in converged control flow and only its
// lane 0 executes the MMAs (single-thread instructions): every operand is a
// compile-time offset from warp-uniform bases (B descriptors: the start
// address field advanced by the K step's byte offset / 16; operand
// addresses stay below 256 KB, so the 14-bit field does not carry), and the
// loops unroll into a straight run of MMAs. (Issued from one divergent
// thread with descriptors built per MMA, a 39-MMA chunk took about 100
// cycles per MMA, several times the tensor core's time for it.)
template <class C, int KC0, int KC1, int COL_AL_, int DCORR, bool FIRST>
__device__ __forceinline__ void tc2_mma_chunk(uint32_t tbase, uint64_t dbh, uint64_t dbl, uint32_t idesc,
                                              bool lane0, uint64_t* bar) {
#pragma unroll
  for (int pass = 0; pass < 3; ++pass) {
    const uint32_t acol = pass == 0 ? COL_AL_ : C::COL_AH;
    const uint64_t db = pass == 1 ? dbl : dbh;
    const uint32_t dcol = pass < 2 ? DCORR : C::COL_D;
    // the first MMA into an accumulator that starts empty overwrites it
    const bool init0 = pass == 0 && (FIRST || DCORR != C::COL_D);
#pragma unroll
    for (int ks = 0; ks < (KC1 - KC0) / 8; ++ks) {
      const uint64_t off = (uint64_t)(((KC0 / 8 + ks) * 2 * C::LBO) >> 4);
      if (lane0) umma_tf32_ts(tbase + dcol, tbase + acol + ks * 8, db + off, idesc, (init0 && ks == 0) ? 0u : 1u);
    }
  }
  if (lane0) umma_commit(bar);
  __syncwarp();
}

// The RK update of a tile (elements e0 ..) from dt*L in sK, one coalesced
// float4 pass: the thread's items are taken G at a time, the operands of all
// G (u, accumulator, snapshot or stage input from global memory, prefetched
// to L2 when the tile started) loaded before any update is computed and
// stored, so that their loads are in flight together. The first group's
// loads are issued early (tc2_rk_load before the last MMA chunk's wait), so
// that their latency overlaps that wait.
template <class C, int G_>
struct Tc2RkGroup {
  static constexpr int G = G_;  // items whose loads are in flight together
  float4 x0[G], x1[G], x2[G];
  int64_t gi[G];  // offset in the state arrays
  int so[G];      // offset in sK
  int qv[G];      // variable
  bool in[G];
};

template <class C, int G>
__device__ __forceinline__ void tc2_rk_load(const StageArgs<float>& a, int64_t e0, int wt, int k0,
                                            Tc2RkGroup<C, G>& r) {
  constexpr int NP = C::NP, NT = C::NT, SEG4 = C::ET * NP / 4;
  constexpr int IT = (C::TILE4 + NT - 1) / NT;  // float4 items of the thread
  const int stage = a.stage;
  const bool ld_y = stage == 1 || stage == 5, ld_ua = stage >= 2 && stage <= 4, ld_s = stage == 4;
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int w = wt + (k0 + g) * NT;
    r.in[g] = k0 + g < IT && w < C::TILE4;
    const int qq = w / SEG4, r4 = w - (w / SEG4) * SEG4;
    r.qv[g] = qq;
    r.so[g] = qq * C::ET * NP + r4 * 4;
    r.gi[g] = qq * a.stride + e0 * NP + (int64_t)r4 * 4;
    r.x0[g] = r.x1[g] = r.x2[g] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (r.in[g]) {
      if (ld_y) r.x0[g] = *reinterpret_cast<const float4*>(a.y_in + r.gi[g]);
      if (ld_ua) {
        r.x0[g] = *reinterpret_cast<const float4*>(a.u + r.gi[g]);
        r.x1[g] = *reinterpret_cast<const float4*>(a.acc + r.gi[g]);
      }
      if (ld_s) r.x2[g] = *reinterpret_cast<const float4*>(a.snap + r.gi[g]);
    }
  }
}

template <class C, int G>
__device__ __forceinline__ void tc2_rk_finish(const StageArgs<float>& a, const float* sK, const Tc2RkGroup<C, G>& r,
                                              ResAcc<float>& racc) {
  const int stage = a.stage;
#pragma unroll
  for (int g = 0; g < G; ++g) {
    if (!r.in[g]) continue;
    const float4 v = *reinterpret_cast<const float4*>(sK + r.so[g]);
    switch (stage) {
      case 0:
        *reinterpret_cast<float4*>(a.k_out + r.gi[g]) = v;
        break;
      case 1: {
        const float4 y = r.x0[g];
        *reinterpret_cast<float4*>(a.acc + r.gi[g]) = v;
        *reinterpret_cast<float4*>(a.y_out + r.gi[g]) =
            make_float4(y.x + 0.5f * v.x, y.y + 0.5f * v.y, y.z + 0.5f * v.z, y.w + 0.5f * v.w);
        break;
      }
      case 2:
      case 3: {
        const float4 u = r.x0[g], ac = r.x1[g];
        const float c = stage == 2 ? 0.5f : 1.0f;
        *reinterpret_cast<float4*>(a.acc + r.gi[g]) =
            make_float4(ac.x + 2.f * v.x, ac.y + 2.f * v.y, ac.z + 2.f * v.z, ac.w + 2.f * v.w);
        *reinterpret_cast<float4*>(a.y_out + r.gi[g]) =
            make_float4(u.x + c * v.x, u.y + c * v.y, u.z + c * v.z, u.w + c * v.w);
        break;
      }
      case 4: {
        const float4 u = r.x0[g], ac = r.x1[g], sn = r.x2[g];
        const float4 un = make_float4(u.x + rk4_sixth(ac.x + v.x), u.y + rk4_sixth(ac.y + v.y),
                                      u.z + rk4_sixth(ac.z + v.z), u.w + rk4_sixth(ac.w + v.w));
        *reinterpret_cast<float4*>(a.u + r.gi[g]) = un;
        racc.add(r.qv[g], sn.x, un.x, a.c0sq);
        racc.add(r.qv[g], sn.y, un.y, a.c0sq);
        racc.add(r.qv[g], sn.z, un.z, a.c0sq);
        racc.add(r.qv[g], sn.w, un.w, a.c0sq);
        break;
      }
      default: {
        const float4 y = r.x0[g];
        *reinterpret_cast<float4*>(a.y_out + r.gi[g]) = make_float4(y.x + v.x, y.y + v.y, y.z + v.z, y.w + v.w);
        break;
      }
    }
  }
}

template <int D, int P, int NPART>
__global__ void __launch_bounds__(Tc2Cfg<D, P, NPART>::NT, 2)
    stage_tc2_kernel(const StageArgs<float> a, int* err) {
  using C = Tc2Cfg<D, P, NPART>;
  constexpr int NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM, NK = C::NK;
  constexpr int ET = C::ET, NT = C::NT, RECF = C::RECF, KV = C::KV, KT = C::KT, KC = C::KC, NCH = C::NCH;
  constexpr int NN = C::NN, GT = C::GT;
  // float4 items of the RK update per thread, and those loaded early
  constexpr bool EARLY = C::kRkEarly > 0;
  constexpr int RK_IT = (C::TILE4 + NT - 1) / NT, RK_G0 = RK_IT < 3 ? RK_IT : 3;
  constexpr int RK_E = EARLY ? (RK_IT < C::kRkEarly ? RK_IT : C::kRkEarly) : RK_G0;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::oBar);  // 0: tile copy, 1: MMA chunks
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + C::oBar + 64);
  unsigned char* sBh = sm + C::oBh;
  unsigned char* sBl = sm + C::oBl;
  short* sFm = reinterpret_cast<short*>(sm + C::oFm);
  short* sNb = reinterpret_cast<short*>(sm + C::oNb);
  float* sGT = reinterpret_cast<float*>(sm + C::oGT);
  float* sY = reinterpret_cast<float*>(sm + C::oY);
  float* sGF = reinterpret_cast<float*>(sm + C::oGF);
  int* sGI = reinterpret_cast<int*>(sm + C::oGI);
  float* sN = reinterpret_cast<float*>(sm + C::oN);
  float* sK = sN;  // dt*L of the tile [NV][ET][NP] once the face fluxes are consumed
  double* sRed = reinterpret_cast<double*>(sm + C::oR);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int lq = warp & 3, part = warp >> 2;  // tensor-memory lane quarter, column part
  const int m = lq * 32 + lane;               // tile row = (q, e)
  // Work shared by the whole block (gathers, face fluxes, per-element
  // values, RK update) is handed out by rank: the pressure rows' warps (lane
  // quarter 0), whose volume columns cost twice those of a velocity row,
  // come last, so that the items left over by an uneven split go elsewhere.
  const int wt = (lq == 0 ? 3 * NPART + part : 3 * part + lq - 1) * 32 + lane;
  // One thread (the first of the last warp: velocity or unused rows) issues
  // the TMA copies and the MMAs and polls their mbarriers.
  const bool leader = tid == NT - 32;
  const bool row_ok = lq * 32 < C::ROWS;      // warp-uniform
  const int q = m / ET, e = m - (m / ET) * ET;
  const int stage = a.stage;
  const int64_t stride = a.stride;
  const int nepi = (stage == 2 || stage == 3) ? 2 : (stage == 4 ? 3 : 0);  // u, acc, snapshot read by the epilogue

  auto issue_tile = [&](int tile) {
    const int64_t e0 = (int64_t)tile * ET;
    mbar_expect_tx(&bar[0], NV * C::YSEG + C::GFB + C::GIB);
#pragma unroll
    for (int qq = 0; qq < NV; ++qq)
      tma_load_1d(sY + (size_t)qq * ET * NP, a.y_in + qq * stride + e0 * NP, C::YSEG, &bar[0]);
    tma_load_1d(sGF, a.geoF + e0 * RECF, C::GFB, &bar[0]);
    tma_load_1d(sGI, a.geoI + e0 * C::RECI, C::GIB, &bar[0]);
  };

  // ---- setup: barriers, tensor memory, operator B (hi/lo), node tables ----
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"((uint32_t)C::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int idx = tid; idx < C::NG * 8 * KT; idx += NT) {
    const int n = idx / KT, k = idx - (idx / KT) * KT;
    float x = 0.f;
    if (n < NP) {
      if (k < KV) {
        const int r = k / C::NPP, j = k - (k / C::NPP) * C::NPP;
        if (j < NP) x = a.Dt[(r * NP + j) * NP + n];
      } else if (k - KV < NK) {
        x = -a.LIFT[(k - KV) * NP + n];
      }
    }
    const uint32_t off = (uint32_t)((k / 4) * C::NG + n / 8) * 128 + (n % 8) * 16 + (k % 4) * 4;
    uint32_t h, l;
    split_op22(x, h, l);
    *reinterpret_cast<uint32_t*>(sBh + off) = h;
    *reinterpret_cast<uint32_t*>(sBl + off) = l;
  }
  for (int i = tid; i < (int)(C::BSLACK / 4); i += NT) reinterpret_cast<float*>(sBl + C::BBYTES)[i] = 0.f;
  for (int i = tid; i < NK; i += NT) sFm[i] = a.fmask[i];
  for (int i = tid; i < NF * NPERM * NFP; i += NT) sNb[i] = a.nbrnode[i];
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B is read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t trow = tbase + ((uint32_t)(lq * 32) << 16);
  if (!row_ok) {
    // rows past NV*ET (2-D) feed only accumulator rows that are never read;
    // they are zeroed once so that they hold finite values
    const uint32_t z[4] = {0u, 0u, 0u, 0u};
    for (int c = 4 * part; c < 2 * KC; c += 4 * NPART) tmem_st4(trow + C::COL_AH + c, z);
    tmem_wait_st();
  }

  const float rhoc2 = (float)a.ph.rhoc2, inv_rho0 = (float)a.ph.inv_rho0, half_c0 = (float)a.ph.half_c0;
  const float dt = (float)a.dt;
  ResAcc<float> racc;
  bool ok = true;
  // leader: barriers whose armed phase was not yet observed complete (bit
  // i) and that phase's parity (bit 4+i); drained before the block exits
  uint32_t pend = 0;
  auto arm = [&](int i, uint32_t parity) { pend = (pend & ~(0x11u << i)) | (1u << i) | ((parity & 1u) << (4 + i)); };
  uint32_t mma_phase = 0;  // MMA commits waited for so far (bar[1] parity)
  if (leader && (int)blockIdx.x < a.ntiles) issue_tile(blockIdx.x), arm(0, 0);
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
  const uint64_t dbh = umma_desc(smem_u32(sBh), C::LBO, C::SBO), dbl = umma_desc(smem_u32(sBl), C::LBO, C::SBO);
  // the MMA warp (the leader's), as a warp-uniform value
  const bool mma_warp = __shfl_sync(0xffffffffu, warp, 0) == NT / 32 - 1;
  static_assert(NCH == 1 || KV >= KC, "face columns must lie in the last K chunk");

  // Each mbarrier is polled by the leader alone; the block learns the outcome
  // from the barrier that follows (__syncthreads_or), which orders the
  // copied data or the finished MMAs before every thread's use of them.
  int it = 0;
  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++it) {
    const int64_t e0 = (int64_t)tile * ET;
    bool got = true;
    if (leader) {
      got = mbar_wait(&bar[0], it & 1, a.wait_limit);
      if (got) pend &= ~1u;
    }
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    // RK operands of this tile towards L2 (read by the coalesced epilogue)
    if (wt < NV * nepi) {
      const int k = wt / NV, qq = wt - (wt / NV) * NV;
      const float* src = k == 0 ? a.u : (k == 1 ? a.acc : a.snap);
      prefetch_l2(src + qq * stride + e0 * NP, C::YSEG);
    }
    // ---- neighbour traces (asynchronous) ----
    if constexpr (!C::kGatherWithVolume) {
      gather_traces<C, float>(a.y_in, stride, sGI, sNb, sN, wt, e0);
      cp_async_commit();
    }
    // ---- per-element values of the row phase, element-minor ----
    for (int w = wt; w < ET * GT; w += NT) {
      const int el = w / GT, v = w - (w / GT) * GT;
      const int src = v < D * D ? v : C::S::PHYS_OFF + (v - D * D);
      sGT[v * (ET + 1) + el] = sGF[el * RECF + src];
    }
    __syncthreads();
    if constexpr (C::kGatherWithVolume) {
      gather_traces<C, float>(a.y_in, stride, sGI, sNb, sN, wt, e0);
      cp_async_commit();
    }
    float cf[D + D * D];
    Tc2RkGroup<C, RK_E> rk0;  // the first RK-update operands
    if (row_ok) {
      tc2_coeffs<C>(sGT, q, e, rhoc2, inv_rho0, cf);
      // ---- volume columns of the first chunk ----
      tc2_build_vol_q<C>(q, sY, cf, e, part, trow, 0, KC, C::COL_AL);
    }
    // one barrier for both: the first chunk's A is in tensor memory, and
    // every thread's neighbour gathers have landed
    cp_async_wait_all();
    tmem_wait_st();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if constexpr (NCH == 2) {
      if (mma_warp) tc2_mma_chunk<C, 0, KC, C::COL_AL, C::COL_D, true>(tbase, dbh, dbl, idesc, leader, &bar[1]);
      if (leader) arm(1, mma_phase);
    }
    // ---- face numerical fluxes (in place of the gathered traces; they
    // overlap the first chunk's MMAs) ----
    face_fluxes<C, float>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, wt, rhoc2, inv_rho0, half_c0, e0);
    if constexpr (NCH == 2) {
      // the first chunk's MMAs have read A before it is overwritten
      bool gm = true;
      if (leader) {
        gm = mbar_wait(&bar[1], mma_phase & 1, a.wait_limit);
        if (gm) pend &= ~2u;
      }
      ++mma_phase;
      if (__syncthreads_or(!gm)) {  // also: the face fluxes are in sN
        ok = false;
        break;
      }
      tc_fence_after();
      if (row_ok) tc2_build_vol_q<C>(q, sY, cf, e, part, trow, KC, KT, C::COL_AL2);
    } else {
      __syncthreads();  // the face fluxes are in sN
    }
    if (row_ok) tc2_build_face<C>(sN, q, e, part, trow, NCH == 2 ? KC : 0, KT, NCH == 2 ? C::COL_AL2 : C::COL_AL);
    // the first RK-operand loads, in flight through the last chunk's MMAs
    if constexpr (EARLY) tc2_rk_load<C>(a, e0, wt, 0, rk0);
    tmem_wait_st();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    bool gm2 = true;
    if (mma_warp) {
      if constexpr (NCH == 2)
        tc2_mma_chunk<C, KC, KT, C::COL_AL2, C::COL_DC, false>(tbase, dbh, dbl, idesc, leader, &bar[1]);
      else
        tc2_mma_chunk<C, 0, KT, C::COL_AL, C::COL_D, true>(tbase, dbh, dbl, idesc, leader, &bar[1]);
    }
    if (leader) {
      arm(1, mma_phase);
      // the tile buffer has been consumed: the next tile's copies overlap
      // this chunk's MMAs and the epilogue
      fence_proxy_async();
      const int nt = tile + gridDim.x;
      if (nt < a.ntiles) issue_tile(nt), arm(0, (it + 1) & 1);
      gm2 = mbar_wait(&bar[1], mma_phase & 1, a.wait_limit);
      if (gm2) pend &= ~2u;
    }
    ++mma_phase;
    if (__syncthreads_or(!gm2)) {
      ok = false;
      break;
    }
    tc_fence_after();

    // ---- epilogue 1: dt*L of this thread's row into sK ([q][e][i]), the
    // accumulator columns in kEpiPasses passes ----
    if (row_ok) {
      const float dte = dt * sGT[(D * D + D) * (ET + 1) + e];
      float* kr = sK + (size_t)(q * ET + e) * NP;
      constexpr int NCHK = (NN / 4 + NPART - 1) / NPART, NPASS = C::kEpiPasses;
      constexpr int NHALF = (NCHK + NPASS - 1) / NPASS;
#pragma unroll
      for (int h = 0; h < NPASS; ++h) {
        uint32_t dr[NHALF][4], dc[NHALF][4];
#pragma unroll
        for (int tt = 0; tt < NHALF; ++tt) {
          const int c4 = part + (h * NHALF + tt) * NPART;
          if (h * NHALF + tt < NCHK && c4 * 4 < NP) {  // warp-uniform condition
            tmem_ld4_async(trow + C::COL_D + c4 * 4, dr[tt]);
            if constexpr (NCH == 2) tmem_ld4_async(trow + C::COL_DC + c4 * 4, dc[tt]);
          }
        }
#pragma unroll
        for (int tt = 0; tt < NHALF; ++tt)
          if (h * NHALF + tt < NCHK && (part + (h * NHALF + tt) * NPART) * 4 < NP) {
            tmem_wait_ld4(dr[tt]);
            if constexpr (NCH == 2) tmem_wait_ld4(dc[tt]);
          }
#pragma unroll
        for (int tt = 0; tt < NHALF; ++tt) {
          const int i0 = (part + (h * NHALF + tt) * NPART) * 4;
          if (h * NHALF + tt >= NCHK || i0 >= NP) break;  // warp-uniform
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            float x = __uint_as_float(dr[tt][u]);
            if constexpr (NCH == 2) x += __uint_as_float(dc[tt][u]);
            if (i0 + u < NP) kr[i0 + u] = dte * x;
          }
        }
      }
    }
    constexpr int RK_N1 = RK_IT > RK_E ? RK_IT - RK_E : 1;
    Tc2RkGroup<C, RK_N1> rk1;  // the thread's other items
    if constexpr (RK_IT > RK_E && C::kRkRestEarly) tc2_rk_load<C>(a, e0, wt, RK_E, rk1);
    tc_fence_before();
    __syncthreads();

    // ---- epilogue 2: RK update, one coalesced float4 pass over the tile:
    // the early group, then the thread's other items in one group ----
    if constexpr (!EARLY) tc2_rk_load<C>(a, e0, wt, 0, rk0);
    tc2_rk_finish<C>(a, sK, rk0, racc);
    if constexpr (RK_IT > RK_E) {
      if constexpr (!C::kRkRestEarly) tc2_rk_load<C>(a, e0, wt, RK_E, rk1);
      tc2_rk_finish<C>(a, sK, rk1, racc);
    }
    // no barrier here: the next tile's first barrier (after its copy wait)
    // comes before its gathers reuse sK (the face buffer)
  }

  // ---- teardown: own copies and tensor-core work first, then the memory ----
  if (leader) {
    // after a timeout: bounded waits (default limit) for the copies and the
    // MMA group still armed, so that nothing lands in freed memory
    for (int i = 0; i < 2; ++i)
      if (pend & (1u << i)) mbar_wait(&bar[i], (pend >> (4 + i)) & 1u);
    if (!ok) atomicOr(err, 1);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"((uint32_t)C::TCOLS)
                 : "memory");

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

template <int D, int P, int NPART>
struct StageTc2 {
  using C = Tc2Cfg<D, P, NPART>;
  static int blocks_per_sm() {
    auto kfn = stage_tc2_kernel<D, P, NPART>;
    if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes) != cudaSuccess ||
        cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
            cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    // from the SM's limits (the occupancy query answers 1 for kernels that
    // use tensor memory): shared memory, threads, registers and the 512
    // tensor-memory columns the resident blocks share
    int dev = 0, smem_sm = 0, smem_res = 0, thr_sm = 0, regs_sm = 0;
    cudaFuncAttributes fa{};
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&smem_res, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, kfn) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    int nb = smem_sm / ((int)C::bytes + smem_res);
    nb = nb < thr_sm / C::NT ? nb : thr_sm / C::NT;
    const int regs_block = ((fa.numRegs + 7) / 8 * 8) * C::NT;
    if (regs_block > 0) nb = nb < regs_sm / regs_block ? nb : regs_sm / regs_block;
    const int by_tmem = 512 / C::TCOLS;
    nb = nb < by_tmem ? nb : by_tmem;
    return nb > 0 ? nb : 0;
  }
  static cudaError_t launch(const StageArgs<float>& a, int grid, int* err, cudaStream_t s) {
    auto kfn = stage_tc2_kernel<D, P, NPART>;
    static bool configured = false;
    if (!configured) {
      cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
      if (e != cudaSuccess) return e;
      configured = true;
    }
    kfn<<<grid, C::NT, C::bytes, s>>>(a, err);
    return cudaGetLastError();
  }
};

}  // namespace dgk
