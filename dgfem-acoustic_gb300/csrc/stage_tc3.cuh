// Warp-specialised tensor-core fused RK4 stage kernel (sm_103a, FP32 state,
// tcgen05 TF32 with two-term splits of both operands), tetrahedra.
//
// Same arithmetic as stage_tc.cuh / stage_tc2.cuh (the RHS of a tile of 32
// elements is one GEMM D = A B^T with rows m = (q,e), K = the contravariant
// volume fluxes (r,j) then the scaled face fluxes k, N = output node i;
// B = [Dt_1..Dt_D | -LIFT]; TF32 products of the split operands, FP32
// accumulation), following src/Mesh.cpp:734-975, src/solver.cpp:38-57 and
// :488-516. What differs is the schedule. In the two-chunk kernel every
// phase of a tile ran in sequence behind block-wide barriers (ncu, 3-D p = 4:
// issue 43 %, the warps stalled on barriers first): the A rows of the
// pressure variable cost more than the velocity rows, one thread issued the
// MMAs while the others waited, and the RK update waited for the last MMA.
// Here one block per SM holds three roles that hand work to each other
// through mbarriers:
//
//   * 8 or 16 builder warps (2 or 4 per tensor-memory lane quarter): the tile's copy
//     wait, neighbour gathers, face fluxes, and A in K chunks (one chunk per
//     reference direction, then the face columns) into two alternating
//     tensor-memory regions; a chunk is handed to the MMA thread as soon as
//     it is written, and the builders go on with the next chunk (or the next
//     tile) while the tensor cores work;
//   * 1 MMA thread: per chunk the correction products (into D for the first
//     chunk, while D is small, into a second accumulator DC for the others)
//     and the head products into D; accumulators D and DC are double
//     buffered, so the MMAs of a tile start while the previous tile's
//     accumulators are read;
//   * 4 epilogue warps (1 per lane quarter): per tile a TMA copy of the RK
//     operands (u, accumulator, snapshot) into shared memory, the
//     accumulator rows (tcgen05.ld), the RK update in shared memory and TMA
//     bulk stores of the results.
//
// Each role decides from one elected thread's bounded mbarrier waits; the
// outcome reaches the role's other threads through a named barrier with an
// OR reduction, so a role leaves its loop as a whole. A role that gives up
// sets a shared abort flag that the others' waits also watch; at the end the
// MMA thread waits (bounded) for its MMAs, the copy issuers for their copies,
// and the tensor memory is freed.
#pragma once
#include <cstdint>

#include "stage_tc2.cuh"

namespace dgk {

template <int D_, int P, int NPART_>
struct Tc3Cfg {
  using T = float;
  using S = ShapeT<D_, P, float>;
  static constexpr int D = D_;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM, NK = NF * NFP;
  static constexpr int ET = 32;                   // elements per tile
  static constexpr int ROWS = NV * ET;            // rows of the M = 128 tile
  static constexpr int NPART = NPART_;            // builder threads per row (warps per lane quarter)
  static constexpr int NB = 128 * NPART;          // builder threads
  static constexpr int NE = 128;                  // epilogue threads: 4 warps, 1 per lane quarter
  static constexpr int NTHREADS = NB + NE + 32;   // + the MMA warp
  static constexpr int NT = NB;                   // threads of the shared face-flux and gather helpers
  static constexpr int RECF = S::RECF, RECI = S::RECI;
  // face buffer: one plane per variable [NV][ET][NKP] (face_fluxes strides)
  static constexpr int NKP = NK | 1;
  static constexpr int NVQ = 1, SN_EL = NKP, SN_K = 1, SN_Q = ET * NKP;
  static constexpr int NPP = RoundUpTc<NP, 8>::v;  // volume columns per direction (whole MMA K steps)
  static constexpr int KV = D * NPP;
  static constexpr int KF = RoundUpTc<NK, 8>::v;   // face columns
  static constexpr int KT = KV + KF;
  static constexpr int NCH = D + 1;                // K chunks: one per direction, then the face columns
  static constexpr int KCMAX = NPP > KF ? NPP : KF;
  static constexpr int NN = RoundUpTc<NP, 16>::v;  // N (multiple of 16 for M = 128)
  // tensor memory: D and DC of two tiles, two A regions (head, then tail)
  static constexpr int COL_D = 0, COL_DC = 2 * NN, COL_A = 4 * NN, AREG = 2 * KCMAX;
  static constexpr int TCOLS = 512;
  static constexpr int GT = D * D + D + 1;         // per-element values of the builders
  static constexpr uint32_t YSEG = ET * NP * sizeof(float);
  static constexpr uint32_t GFB = ET * RECF * sizeof(float);
  static constexpr uint32_t GIB = ET * RECI * sizeof(int);
  // B with only the 8-row groups that hold nodes (as in stage_tc.cuh)
  static constexpr int NG = (NP + 7) / 8;
  static constexpr uint32_t BBYTES = (KT / 4) * NG * 128;
  static constexpr uint32_t BSLACK = (NN / 8 - NG) * 128;
  static constexpr uint32_t LBO = NG * 128, SBO = 128;
  // mbarriers
  static constexpr int BAR_TILE = 0, BAR_AREADY = 2, BAR_AFREE = 4, BAR_DREADY = 6, BAR_DFREE = 8, BAR_EPI = 10,
                       BAR_DRAIN = 11, NBARS = 12;
  // shared memory layout (bytes)
  static constexpr size_t oBar = 0;
  static constexpr size_t oMisc = 128;  // tensor-memory address, abort flag
  static constexpr size_t oBh = 256;
  static constexpr size_t oBl = oBh + BBYTES;
  static constexpr size_t oFm = RoundUpTc<oBl + BBYTES + BSLACK, 16>::v;
  static constexpr size_t oNb = oFm + RoundUpTc<NK * 2, 16>::v;
  static constexpr size_t oGT = RoundUpTc<oNb + NF * NPERM * NFP * 2, 16>::v;  // [GT][ET+1]
  static constexpr size_t TILEB = RoundUpTc<NV * YSEG + GFB + GIB, 128>::v;   // [NV][ET][NP], GF, GI
  static constexpr size_t oY = RoundUpTc<oGT + GT * (ET + 1) * 4, 128>::v;     // 2 tiles
  static constexpr size_t oN = oY + 2 * TILEB;                                 // [NV][ET][NKP]
  static constexpr size_t oE = RoundUpTc<oN + (size_t)NV * ET * NKP * 4, 128>::v;  // [3][NV][ET][NP]
  static constexpr size_t oR = oE + 3 * (size_t)NV * YSEG;                     // [warps][5] double
  static constexpr size_t bytes = oR + (NTHREADS / 32) * 5 * sizeof(double);
  // requested per block: at least 118 KB, so that no second block (which
  // would wait for the first one's tensor memory) shares an SM
  static constexpr size_t launch_bytes = bytes > 118 * 1024 ? bytes : 118 * 1024;
  static_assert(D == 3, "the warp-specialised kernel is built for tetrahedra");
  static_assert(ROWS == 128, "rows of a tile must fill the MMA height");
  static_assert(COL_A + 2 * AREG <= TCOLS, "tensor memory of the block exceeds 512 columns");
  static_assert(YSEG % 16 == 0 && GFB % 16 == 0 && GIB % 16 == 0, "copy segments must be 16-byte multiples");
  static_assert(bytes <= 227 * 1024, "shared memory of one block exceeds 227 KB");
};

// Named barrier of a role (id, count threads); with an OR over the threads'
// predicates.
__device__ __forceinline__ void role_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ bool role_sync_or(int id, int count, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(id), "r"(count)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait for the phase with the given parity that also gives up when
// another role has set the abort flag.
__device__ __forceinline__ bool mbar_wait_abort(uint64_t* bar, uint32_t parity, int limit, const volatile int* abort) {
  const uint32_t a = smem_u32(bar);
  for (int it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(kWaitHintNs)
        : "memory");
    if (ok) return true;
    if ((it & 63) == 63 && *abort) return false;
  }
  return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t ta, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(ta)
      : "memory");
}
// waits for the thread's outstanding tcgen05.ld; the registers are operands
// so that no use of them is scheduled before the wait
__device__ __forceinline__ void tmem_wait_ld16(uint32_t* r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15])::
                   "memory");
}

// Volume columns of reference direction r for row (Q, e) into one A region
// (head at ahi, tail at alo, local column j): the thread takes the 4-node
// groups j0 = 4 (part + t NPART); columns past NP repeat the last node
// (finite values that meet zero rows of B).
//   Q = 0 (pressure): gv0_r p_j + sum_d (rho0 c0^2 G_rd) v_d,j
//   Q = 1+d (v_d):    gv0_r v_d,j + (G_rd / rho0) p_j
template <class C, int Q>
__device__ __forceinline__ void tc3_build_vol(const float* sY, const float* cf, int e, int part, int r, uint32_t ahi,
                                              uint32_t alo) {
  constexpr int D = C::D, NP = C::NP, ET = C::ET, NG4 = C::NPP / 4;
  const float* yp_row = sY + e * NP;
  const float* yq_row = sY + (Q == 0 ? 1 : Q) * ET * NP + e * NP;
  float cr[1 + D];
  cr[0] = cf[r];
  if constexpr (Q == 0) {
#pragma unroll
    for (int d = 0; d < D; ++d) cr[1 + d] = cf[D + r * D + d];
  } else {
    cr[1] = cf[D + r];
  }
#pragma unroll
  for (int t = 0; t < (NG4 + C::NPART - 1) / C::NPART; ++t) {
    const int g4 = part + t * C::NPART;
    if (g4 >= NG4) break;
    const int j0 = 4 * g4;
    float fr[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int j = j0 + u < NP ? j0 + u : NP - 1;
      const float yp = yp_row[j];
      float x;
      if constexpr (Q == 0) {
        x = cr[0] * yp;
#pragma unroll
        for (int d = 0; d < D; ++d) x = fmaf(cr[1 + d], yq_row[d * ET * NP + j], x);
      } else {
        x = fmaf(cr[1], yp, cr[0] * yq_row[j]);
      }
      fr[u] = x;  // past NP: the last node's value, against a zero row of B
    }
    uint32_t hi[4], lo[4];
    split4(fr, hi, lo);
    tmem_st4(ahi + j0, hi);
    tmem_st4(alo + j0, lo);
  }
}

template <class C>
__device__ __forceinline__ void tc3_build_vol_q(int q, const float* sY, const float* cf, int e, int part, int r,
                                                uint32_t ahi, uint32_t alo) {
  switch (q) {
    case 0: tc3_build_vol<C, 0>(sY, cf, e, part, r, ahi, alo); break;
    case 1: tc3_build_vol<C, 1>(sY, cf, e, part, r, ahi, alo); break;
    case 2: tc3_build_vol<C, 2>(sY, cf, e, part, r, ahi, alo); break;
    default: tc3_build_vol<C, 3>(sY, cf, e, part, r, ahi, alo); break;
  }
}

// Face columns of row (q, e) (and the zero padding after them) from the
// face-flux plane of variable q into one A region.
template <class C>
__device__ __forceinline__ void tc3_build_face(const float* sN, int q, int e, int part, uint32_t ahi, uint32_t alo) {
  constexpr int NK = C::NK, NG4 = C::KF / 4;
  const float* hrow = sN + (size_t)(q * C::ET + e) * C::NKP;
#pragma unroll
  for (int t = 0; t < (NG4 + C::NPART - 1) / C::NPART; ++t) {
    const int c4 = part + t * C::NPART;
    if (c4 >= NG4) break;
    const int k0 = 4 * c4;
    float x[4];
    if constexpr (C::KF == NK) {  // no padding columns
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = hrow[k0 + u];
    } else {
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = k0 + u < NK ? hrow[k0 + u] : 0.f;
    }
    uint32_t hi[4], lo[4];
    split4(x, hi, lo);
    tmem_st4(ahi + k0, hi);
    tmem_st4(alo + k0, lo);
  }
}

template <int D, int P, int NPART>
__global__ void __launch_bounds__(Tc3Cfg<D, P, NPART>::NTHREADS, 1)
    stage_tc3_kernel(const StageArgs<float> a, int* err) {
  using C = Tc3Cfg<D, P, NPART>;
  constexpr int NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM, NK = C::NK;
  constexpr int ET = C::ET, NB = C::NB, NE = C::NE, RECF = C::RECF, RECI = C::RECI;
  constexpr int KV = C::KV, KT = C::KT, NCH = C::NCH, NN = C::NN, GT = C::GT, NPP = C::NPP, KCMAX = C::KCMAX;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::oBar);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + C::oMisc);
  volatile int* sAbort = reinterpret_cast<volatile int*>(sm + C::oMisc + 4);
  unsigned char* sBh = sm + C::oBh;
  unsigned char* sBl = sm + C::oBl;
  short* sFm = reinterpret_cast<short*>(sm + C::oFm);
  short* sNb = reinterpret_cast<short*>(sm + C::oNb);
  float* sGT = reinterpret_cast<float*>(sm + C::oGT);
  unsigned char* sTiles = sm + C::oY;
  float* sN = reinterpret_cast<float*>(sm + C::oN);
  float* sE = reinterpret_cast<float*>(sm + C::oE);
  double* sRed = reinterpret_cast<double*>(sm + C::oR);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int stage = a.stage;
  const int64_t stride = a.stride;
  // operand arrays the epilogue reads: stage 0 none; 1 and 5 the stage input
  // (u); 2-3 u and the accumulator; 4 u, the accumulator and the snapshot
  const int nepi = stage == 0 ? 0 : (stage == 1 || stage == 5) ? 1 : (stage == 4 ? 3 : 2);
  // tiles of this block: blockIdx.x + i * gridDim.x
  const int nmine = (int)blockIdx.x < a.ntiles ? (a.ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  // ---- setup: barriers, tensor memory, operator B (hi/lo), node tables ----
  if (tid == 0) {
    for (int i = 0; i < C::NBARS; ++i)
      mbar_init(&bar[i], i == C::BAR_AREADY || i == C::BAR_AREADY + 1 ? NB
                         : (i == C::BAR_DFREE || i == C::BAR_DFREE + 1) ? NE
                                                                        : 1);
    *sAbort = 0;
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"((uint32_t)C::TCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int idx = tid; idx < C::NG * 8 * KT; idx += C::NTHREADS) {
    const int n = idx / KT, k = idx - (idx / KT) * KT;
    float x = 0.f;
    if (n < NP) {
      if (k < KV) {
        const int r = k / NPP, j = k - (k / NPP) * NPP;
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
  for (int i = tid; i < (int)(C::BSLACK / 4); i += C::NTHREADS) reinterpret_cast<float*>(sBl + C::BBYTES)[i] = 0.f;
  for (int i = tid; i < NK; i += C::NTHREADS) sFm[i] = a.fmask[i];
  for (int i = tid; i < NF * NPERM * NFP; i += C::NTHREADS) sNb[i] = a.nbrnode[i];
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B is read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const float rhoc2 = a.f_rhoc2, inv_rho0 = a.f_inv_rho0, half_c0 = a.f_half_c0;
  ResAcc<float> racc;

  constexpr int NBW = NB / 32;  // builder warps
  if (warp < NBW) {
    // ===================== builders =====================
    const int lq = warp & 3, part = warp >> 2;
    const int m = lq * 32 + lane, q = m / ET, e = m - (m / ET) * ET;
    const uint32_t trow = tbase + ((uint32_t)(lq * 32) << 16);
    // shared work (gathers, face fluxes, per-element values) by a rank that
    // puts the pressure rows' warps (lane quarter 0) last
    const int wt = (lq == 0 ? 3 * C::NPART + part : 3 * part + lq - 1) * 32 + lane;
    // the copy issuer and waiter: a velocity-row warp's first thread (the
    // pressure rows' warps have the most A columns to build)
    const bool lead = tid == (NBW - 1) * 32;
    // lead: tile buffers whose copy was issued and not yet observed (bit b)
    // and that copy's phase parity (bit 4+b)
    uint32_t pend = 0;
    auto issue_tile = [&](int i) {
      const int b = i & 1;
      const int64_t e0 = (int64_t)((int)blockIdx.x + i * (int)gridDim.x) * ET;
      unsigned char* t = sTiles + b * C::TILEB;
      uint64_t* tb = &bar[C::BAR_TILE + b];
      mbar_expect_tx(tb, NV * C::YSEG + C::GFB + C::GIB);
#pragma unroll
      for (int qq = 0; qq < NV; ++qq)
        tma_load_1d(t + qq * C::YSEG, a.y_in + qq * stride + e0 * NP, C::YSEG, tb);
      tma_load_1d(t + NV * C::YSEG, a.geoF + e0 * RECF, C::GFB, tb);
      tma_load_1d(t + NV * C::YSEG + C::GFB, a.geoI + e0 * RECI, C::GIB, tb);
      pend = (pend & ~(0x11u << b)) | (1u << b) | ((uint32_t)((i >> 1) & 1) << (4 + b));
    };
    if (lead) {
      if (nmine > 0) issue_tile(0);
      if (nmine > 1) issue_tile(1);
    }
    for (int i = 0; i < nmine; ++i) {
      const int b = i & 1;
      const int64_t e0 = (int64_t)((int)blockIdx.x + i * (int)gridDim.x) * ET;
      bool got = true;
      if (lead) {
        got = mbar_wait_abort(&bar[C::BAR_TILE + b], (i >> 1) & 1, a.wait_limit, sAbort);
        if (got) pend &= ~(1u << b);
      }
      if (role_sync_or(1, NB, !got)) {
        *sAbort = 1;
        break;
      }
      float* sY = reinterpret_cast<float*>(sTiles + b * C::TILEB);
      const float* sGF = reinterpret_cast<const float*>(sTiles + b * C::TILEB + NV * C::YSEG);
      const int* sGI = reinterpret_cast<const int*>(sTiles + b * C::TILEB + NV * C::YSEG + C::GFB);
      // ---- neighbour traces (asynchronous) and the per-element values ----
      gather_traces<C, float>(a.y_in, stride, sGI, sNb, sN, wt, e0);
      cp_async_commit();
      for (int w = wt; w < ET * GT; w += NB) {
        const int el = w / GT, v = w - (w / GT) * GT;
        const int src = v < D * D ? v : C::S::PHYS_OFF + (v - D * D);
        sGT[v * (ET + 1) + el] = sGF[el * RECF + src];
      }
      role_sync(1, NB);
      float cf[D + D * D];
      tc2_coeffs<C>(sGT, q, e, rhoc2, inv_rho0, cf);
      bool fail = false;
#pragma unroll 1
      for (int c = 0; c < NCH; ++c) {
        const int g = i * NCH + c;  // chunk counter of this block
        const int reg = g & 1;
        if (g >= 2) {
          // the MMAs of chunk g - 2 have read this region
          bool fr = true;
          if (lead) fr = mbar_wait_abort(&bar[C::BAR_AFREE + reg], ((g >> 1) - 1) & 1, a.wait_limit, sAbort);
          if (role_sync_or(1, NB, !fr)) {
            fail = true;
            break;
          }
          tc_fence_after();
        }
        const uint32_t ahi = trow + C::COL_A + reg * C::AREG, alo = ahi + KCMAX;
        if (c < D)
          tc3_build_vol_q<C>(q, sY, cf, e, part, c, ahi, alo);
        else
          tc3_build_face<C>(sN, q, e, part, ahi, alo);
        tmem_wait_st();
        tc_fence_before();
        mbar_arrive(&bar[C::BAR_AREADY + reg]);
        if (c == 0) {
          // ---- face numerical fluxes (in place of the gathered traces) ----
          cp_async_wait_all();
          role_sync(1, NB);
          face_fluxes<C, float>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, wt, rhoc2, inv_rho0, half_c0, e0);
          role_sync(1, NB);
        }
        if (c == D - 1) {
          // the tile's stage input and geometry are consumed: the copy of the
          // tile after next goes into this buffer
          role_sync(1, NB);
          if (lead && i + 2 < nmine) {
            fence_proxy_async();
            issue_tile(i + 2);
          }
        }
      }
      if (fail) {
        *sAbort = 1;
        break;
      }
    }
    if (lead) {
      // copies still in flight after a give-up: bounded waits (full limit)
      for (int b = 0; b < 2; ++b)
        if (pend & (1u << b)) mbar_wait(&bar[C::BAR_TILE + b], (pend >> (4 + b)) & 1u);
    }
  } else if (warp < NBW + 4) {
    // ===================== epilogue =====================
    const int lq = warp & 3;
    const int m = lq * 32 + lane, q = m / ET, e = m - (m / ET) * ET;
    const uint32_t trow = tbase + ((uint32_t)(lq * 32) << 16);
    const bool elead = tid == NB;
    const float* src_k[3] = {(stage == 1 || stage == 5) ? a.y_in : a.u, a.acc, a.snap};
    bool epend = false;  // operand copy issued and not yet observed (its phase parity in epar)
    uint32_t epar = 0;
    for (int i = 0; i < nmine; ++i) {
      const int b = i & 1;
      const int64_t e0 = (int64_t)((int)blockIdx.x + i * (int)gridDim.x) * ET;
      // ---- RK operands of this tile into sE, once the previous tile's
      // stores have finished reading it ----
      if (elead) bulk_wait_read();
      if (elead && nepi > 0) {
        mbar_expect_tx(&bar[C::BAR_EPI], nepi * NV * C::YSEG);
        for (int k = 0; k < nepi; ++k)
#pragma unroll
          for (int qq = 0; qq < NV; ++qq)
            tma_load_1d(sE + ((size_t)k * NV + qq) * ET * NP, src_k[k] + qq * stride + e0 * NP, C::YSEG,
                        &bar[C::BAR_EPI]);
        epend = true, epar = (uint32_t)(i & 1);
      }
      const float dte = a.f_dt * a.geoF[(e0 + e) * RECF + C::S::PHYS_OFF + D];
      // ---- this tile's accumulators and RK operands ----
      bool ok = true;
      if (elead) {
        ok = mbar_wait_abort(&bar[C::BAR_DREADY + b], (i >> 1) & 1, a.wait_limit, sAbort);
        if (ok && nepi > 0) {
          ok = mbar_wait_abort(&bar[C::BAR_EPI], i & 1, a.wait_limit, sAbort);
          if (ok) epend = false;
        }
      }
      if (role_sync_or(2, NE, !ok)) {
        *sAbort = 1;
        break;
      }
      tc_fence_after();
      // ---- RK update in shared memory, 16 accumulator columns at a time,
      // then bulk stores ----
      float* s0 = sE + (size_t)(q * ET + e) * NP;           // u (or the stage input), then results
      float* s1 = sE + (size_t)((NV + q) * ET + e) * NP;    // accumulator
      const float* s2 = sE + (size_t)((2 * NV + q) * ET + e) * NP;  // snapshot
#pragma unroll
      for (int c16 = 0; c16 < NN / 16; ++c16) {
        uint32_t r1[16], r2[16];
        tmem_ld16(trow + C::COL_D + b * NN + c16 * 16, r1);
        tmem_ld16(trow + C::COL_DC + b * NN + c16 * 16, r2);
        tmem_wait_ld16(r1);
        tmem_wait_ld16(r2);
        if (c16 == NN / 16 - 1) {
          tc_fence_before();
          mbar_arrive(&bar[C::BAR_DFREE + b]);  // the MMAs of the tile after next may write them
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int n = c16 * 16 + u;
          if (n >= NP) break;
          const float k = dte * (__uint_as_float(r1[u]) + __uint_as_float(r2[u]));
          switch (stage) {
            case 0:
              s0[n] = k;
              break;
            case 1: {
              const float uu = s0[n];
              s1[n] = k;
              s0[n] = uu + 0.5f * k;
              break;
            }
            case 2:
            case 3: {
              const float uu = s0[n], ac = s1[n];
              s1[n] = ac + 2.f * k;
              s0[n] = uu + (stage == 2 ? 0.5f * k : k);
              break;
            }
            case 4: {
              const float un = s0[n] + rk4_sixth(s1[n] + k);
              racc.add(q, s2[n], un, a.c0sq);
              s0[n] = un;
              break;
            }
            default:
              s0[n] = s0[n] + k;
              break;
          }
        }
      }
      fence_proxy_async();  // the results are read by the bulk stores
      role_sync(2, NE);
      if (elead) {
        float* dst0 = stage == 0 ? a.k_out : stage == 4 ? a.u : a.y_out;
#pragma unroll
        for (int qq = 0; qq < NV; ++qq)
          tma_store_1d(dst0 + qq * stride + e0 * NP, sE + (size_t)qq * ET * NP, C::YSEG);
        if (stage >= 1 && stage <= 3)
#pragma unroll
          for (int qq = 0; qq < NV; ++qq)
            tma_store_1d(a.acc + qq * stride + e0 * NP, sE + (size_t)(NV + qq) * ET * NP, C::YSEG);
        bulk_commit();
      }
    }
    if (elead) {
      if (epend) mbar_wait(&bar[C::BAR_EPI], epar);  // a copy still in flight after a give-up
      bulk_wait_all();
    }
  } else if (lane == 0) {
    // ===================== MMA issue =====================
    const uint32_t idesc =
        (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    const uint32_t bh = smem_u32(sBh), bl = smem_u32(sBl);
    bool fail = false;
    for (int i = 0; i < nmine && !fail; ++i) {
      const int b = i & 1;
      const uint32_t d_acc = tbase + C::COL_D + b * NN, dc_acc = tbase + C::COL_DC + b * NN;
#pragma unroll 1
      for (int c = 0; c < NCH; ++c) {
        const int g = i * NCH + c;
        const int reg = g & 1;
        bool ok = mbar_wait_abort(&bar[C::BAR_AREADY + reg], (g >> 1) & 1, a.wait_limit, sAbort);
        // the epilogue has read this accumulator pair two tiles ago
        if (ok && c == 0 && i >= 2)
          ok = mbar_wait_abort(&bar[C::BAR_DFREE + b], ((i >> 1) - 1) & 1, a.wait_limit, sAbort);
        if (!ok) {
          *sAbort = 1;
          fail = true;
          break;
        }
        tc_fence_after();
        const int k0 = c < D ? c * NPP : KV;
        const int nk = (c < D ? NPP : C::KF) / 8;
        const uint32_t ahi = tbase + C::COL_A + reg * C::AREG, alo = ahi + KCMAX;
        const uint32_t dcorr = c == 0 ? d_acc : dc_acc;
        // the correction products first (A_lo B_hi, A_hi B_lo), then the
        // head products A_hi B_hi into D; the first MMA into D (chunk 0)
        // and into DC (chunk 1) overwrites it
#pragma unroll
        for (int pass = 0; pass < 3; ++pass) {
          const uint32_t acol = pass == 0 ? alo : ahi;
          const uint32_t bsrc = (pass == 1 ? bl : bh) + (uint32_t)(k0 / 8) * 2 * C::LBO;
          const uint32_t dcol = pass < 2 ? dcorr : d_acc;
          const bool init0 = pass == 0 && c <= 1;
#pragma unroll 1
          for (int ks = 0; ks < nk; ++ks)
            umma_tf32_ts(dcol, acol + ks * 8, umma_desc(bsrc + ks * 2 * C::LBO, C::LBO, C::SBO), idesc,
                         (init0 && ks == 0) ? 0u : 1u);
        }
        umma_commit(&bar[C::BAR_AFREE + reg]);
        if (c == NCH - 1) umma_commit(&bar[C::BAR_DREADY + b]);
      }
    }
    // every MMA of this thread has completed before the memory is freed
    umma_commit(&bar[C::BAR_DRAIN]);
    mbar_wait(&bar[C::BAR_DRAIN], 0u);
  }

  // ---- teardown ----
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"((uint32_t)C::TCOLS)
                 : "memory");
  if (tid == 0 && *sAbort) atomicOr(err, 1);
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
      for (int w = 0; w < C::NTHREADS / 32; ++w) v += sRed[w * 5 + tid];
      a.partials[blockIdx.x * 5 + tid] = v;
    }
  }
}

template <int D, int P, int NPART>
struct StageTc3 {
  using C = Tc3Cfg<D, P, NPART>;
  static cudaError_t set_attrs() {
    auto kfn = stage_tc3_kernel<D, P, NPART>;
    cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::launch_bytes);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    return e;
  }
  // one block per SM: it holds all 512 tensor-memory columns
  static int blocks_per_sm() {
    if (set_attrs() != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return 1;
  }
  static cudaError_t launch(const StageArgs<float>& a, int grid, int* err, cudaStream_t s) {
    static bool configured = false;
    if (!configured) {
      cudaError_t e = set_attrs();
      if (e != cudaSuccess) return e;
      configured = true;
    }
    stage_tc3_kernel<D, P, NPART><<<grid, C::NTHREADS, C::launch_bytes, s>>>(a, err);
    return cudaGetLastError();
  }
};

}  // namespace dgk
