// Tensor-core fused RK4 stage kernel (sm_103a, FP32 state, tcgen05 TF32
// with two-term splits of both operands).
//
// Same arithmetic as the reference's per-stage work (src/Mesh.cpp:734-975,
// src/solver.cpp:38-57, :488-516), written as one small GEMM per tile of
// ET elements. The RHS of variable q of element e is linear in two sets of
// per-element values: the contravariant volume fluxes
//   A_vol[(q,e)][(r,j)] = sum_d G_rd F_{q,d}(y_j)   (r = reference direction)
// and the scaled face fluxes
//   A_face[(q,e)][k]    = sJ_f h_q(k)               (k = face node)
// so that
//   L[(q,e)][i] = sum_{r,j} Dt_r[i][j] A_vol + sum_k (-LIFT[k][i]) A_face,
// i.e. D = A B^T with rows m = (q,e) (M = 128), K = (r,j) then k, N = i.
//
// Per tile:
//   * TMA bulk copies land the tile (stage input, geometry records) in a
//     double buffer, and the RK operands (u, accumulator, snapshot) in a third
//     buffer, as in the pipelined kernel; neighbour traces are gathered with
//     cp.async and turned into face fluxes in shared memory;
//   * each thread owns one row (q,e): it computes the row's A entries, splits
//     each into a TF32 head and a TF32 tail (x ~ hi + lo, |x - hi - lo| <=
//     2^-22 |x|) and writes both to tensor memory (tcgen05.st), so A never
//     occupies shared memory;
//   * one thread issues the MMAs D = A_lo B_hi + A_hi B_lo + A_hi B_hi, the
//     correction products first while D is small (tcgen05.mma kind::tf32, A
//     from tensor memory, B = [Dt_1..Dt_D | -LIFT] rounded to 22 significand
//     bits and split exactly into head and tail, kept in shared memory in the
//     canonical K-major no-swizzle layout), completion signalled on an
//     mbarrier;
//   * the epilogue reads the row's accumulator (tcgen05.ld), applies the RK
//     update in shared memory and writes the tile back with TMA bulk stores.
// The errors are the data split (2^-22), the dropped A_lo B_lo (< 2^-22),
// the operator's 22-bit rounding (2^-23, fixed) and the FP32 accumulation.
// Every wait is bounded; on timeout the block records an error flag, waits
// (bounded) for its own tensor-core work and copies, frees its tensor memory
// and returns.
#pragma once
#include <cstdint>

#include "stage2.cuh"

namespace dgk {

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// tcgen05 shared-memory matrix descriptor: canonical K-major layout without
// swizzle, made of 8-row x 16-byte core matrices; lbo = byte distance between
// core matrices adjacent along K, sbo = along M/N.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version (tcgen05)
  return d;
}

// D[tmem] (+)= A[tmem] * B[smem]^T, kind::tf32, FP32 accumulate.
__device__ __forceinline__ void umma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_st4(uint32_t ta, const uint32_t* v) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(ta), "r"(v[0]), "r"(v[1]),
               "r"(v[2]), "r"(v[3])
               : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
// 4 accumulator columns of this warp's lane quarter without waiting; the
// registers are valid after tmem_wait_ld4 on them
__device__ __forceinline__ void tmem_ld4_async(uint32_t ta, uint32_t* r) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(ta)
               : "memory");
}
// waits for every outstanding tcgen05.ld of the thread; the registers are
// operands so that no use of them is scheduled before the wait
__device__ __forceinline__ void tmem_wait_ld4(uint32_t* r) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3])::"memory");
}

// 1-D TMA bulk store shared -> global (bytes % 16 == 0, 16-byte aligned).
__device__ __forceinline__ void tma_store_1d(void* dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Splits four values into TF32 heads and TF32 tails, both rounded to
// nearest: x - hi is exact in FP32, and rounding it (instead of letting the
// MMA drop its low 13 bits) keeps the tail's error unbiased.
__device__ __forceinline__ void split4(const float* x, uint32_t* hi, uint32_t* lo) {
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    hi[u] = tf32_rna(x[u]);
    lo[u] = tf32_rna(x[u] - __uint_as_float(hi[u]));
  }
}

// An operator entry as an exact pair of TF32 values: x is first rounded to
// nearest at 22 significand bits (an error of at most 2^-23 |x|, fixed for
// the whole run), so that head = TF32(x22) and tail = x22 - head (at most 11
// significand bits) represent it without further error.
__device__ __forceinline__ void split_op22(float x, uint32_t& hi, uint32_t& lo) {
  uint32_t u = __float_as_uint(x);
  u = (u + 1u + ((u >> 2) & 1u)) & ~3u;  // round to nearest even at bit 2
  const float x22 = __uint_as_float(u);
  hi = tf32_rna(x22);
  lo = __float_as_uint(x22 - __uint_as_float(hi));
}

template <int N, int A>
struct RoundUpTc {
  static constexpr int v = (N + A - 1) / A * A;
};

template <int X>
struct Pow2Cols {  // tensor-memory allocation: a power of two >= 32 columns
  static constexpr int v = X <= 32 ? 32 : X <= 64 ? 64 : X <= 128 ? 128 : X <= 256 ? 256 : 512;
};

// Four consecutive row entries row[j0 .. j0+3] of a row of NP values in
// shared memory (row start 4*VW-byte aligned when VW > 1), in VW-wide
// vectors; entries past NP (the last group of a row whose NP is not a
// multiple of 4) read into the next row or pad and must be masked by the
// caller.
template <int NP, int VW>
__device__ __forceinline__ void load4(float* v, const float* row, int j0) {
  if constexpr (VW == 4) {
    const float4 x = *reinterpret_cast<const float4*>(row + j0);
    v[0] = x.x, v[1] = x.y, v[2] = x.z, v[3] = x.w;
  } else if constexpr (VW == 2) {
    const float2 x = *reinterpret_cast<const float2*>(row + j0);
    const float2 y = *reinterpret_cast<const float2*>(row + j0 + 2);
    v[0] = x.x, v[1] = x.y, v[2] = y.x, v[3] = y.y;
  } else {
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = row[j0 + u < NP ? j0 + u : NP - 1];
  }
}

// Stores the entries of v that fall inside the row (j0 + u < NP).
template <int NP, int VW>
__device__ __forceinline__ void store4(float* row, int j0, const float* v) {
  if constexpr (VW == 4) {
    *reinterpret_cast<float4*>(row + j0) = make_float4(v[0], v[1], v[2], v[3]);
  } else if constexpr (VW == 2) {
    *reinterpret_cast<float2*>(row + j0) = make_float2(v[0], v[1]);
    if (j0 + 2 < NP) *reinterpret_cast<float2*>(row + j0 + 2) = make_float2(v[2], v[3]);
  } else {
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (j0 + u < NP) row[j0 + u] = v[u];
  }
}

template <int D_, int P, int NPART_>
struct TcCfg {
  using T = float;
  using S = ShapeT<D_, P, float>;
  static constexpr int D = D_;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM, NK = NF * NFP;
  static constexpr int ET = 32;            // elements per tile
  static constexpr int ROWS = NV * ET;     // used rows of the M = 128 tile
  static constexpr int NPART = NPART_;     // threads per row: columns split NPART ways
  static constexpr int NT = 128 * NPART;   // lane quarters x parts
  static constexpr int RECF = S::RECF, RECI = S::RECI;
  static constexpr int NKP = NK | 1;
  // face buffer: one plane per variable (the face rows read one variable's
  // face nodes side by side)
  static constexpr int NVQ = 1, SN_EL = NKP, SN_K = 1, SN_Q = ET * NKP;
  static constexpr int NPP = RoundUpTc<NP, 4>::v;       // volume block width per direction
  static constexpr int KV = D * NPP;                     // volume columns
  static constexpr int KF = RoundUpTc<NK, 4>::v;         // face columns
  static constexpr int KT = RoundUpTc<KV + KF, 8>::v;    // K (multiple of the TF32 MMA depth 8)
  static constexpr int NN = RoundUpTc<NP, 16>::v;        // N (multiple of 16 for M = 128)
  static constexpr int COL_D = 0, COL_AH = NN, COL_AL = NN + KT;  // tensor-memory columns
  static constexpr int TCOLS = Pow2Cols<NN + 2 * KT>::v;
  static constexpr int GT = D * D + D + 1;               // per-element values of the row phase
  static constexpr int VWY = (NP % 4 == 0) ? 4 : (NP % 2 == 0) ? 2 : 1;
  static constexpr uint32_t YSEG = ET * NP * sizeof(float);
  static constexpr uint32_t GFB = ET * RECF * sizeof(float);
  static constexpr uint32_t GIB = ET * RECI * sizeof(int);
  // B is stored with only the 8-row groups that hold nodes (NG of NN/8): the
  // MMA reads NN rows per K chunk, and the rows past NG*8 run into the next
  // chunk (or the slack after B lo); they only feed accumulator columns >= NP,
  // which are never read
  static constexpr int NG = (NP + 7) / 8;
  static constexpr uint32_t BBYTES = (KT / 4) * NG * 128;  // one operand copy (hi or lo)
  static constexpr uint32_t BSLACK = (NN / 8 - NG) * 128;
  static constexpr uint32_t LBO = NG * 128, SBO = 128;
  // shared memory layout (bytes)
  static constexpr size_t oBar = 0;                        // 5 mbarriers + tensor-memory address
  static constexpr size_t oBh = 128;                       // B hi, canonical layout
  static constexpr size_t oBl = oBh + BBYTES;              // B lo
  static constexpr size_t oFm = RoundUpTc<oBl + BBYTES + BSLACK, 16>::v;
  static constexpr size_t oNb = oFm + RoundUpTc<NK * 2, 16>::v;
  static constexpr size_t oGT = RoundUpTc<oNb + NF * NPERM * NFP * 2, 16>::v;  // [GT][ET+1]
  static constexpr size_t oY = RoundUpTc<oGT + GT * (ET + 1) * 4, 128>::v;    // 2 x [NV][ET][NP]
  static constexpr size_t oGF = oY + 2 * (size_t)NV * YSEG;
  static constexpr size_t oGI = oGF + 2 * (size_t)GFB;
  static constexpr size_t oE = RoundUpTc<oGI + 2 * (size_t)GIB, 128>::v;    // [2][NV][ET][NP]
  static constexpr size_t oN = oE + 2 * (size_t)NV * YSEG;                   // [NV][ET][NKP]
  static constexpr size_t oR = RoundUpTc<oN + (size_t)NV * ET * NKP * 4, 16>::v;  // [NT/32][5] double
  static constexpr size_t bytes = oR + (NT / 32) * 5 * sizeof(double);
  static_assert(ROWS <= 128, "rows of a tile exceed the MMA height");
  static_assert(NN + 2 * KT <= 512, "tensor-memory columns exceed the SM's 512");
  static_assert(YSEG % 16 == 0, "tile segments must be 16-byte multiples");
  static_assert(bytes <= 227 * 1024, "shared memory of one block exceeds 227 KB");
};

template <int D, int P, int NPART>
__global__ void __launch_bounds__(TcCfg<D, P, NPART>::NT) stage_tc_kernel(const StageArgs<float> a, int* err) {
  using C = TcCfg<D, P, NPART>;
  using T = float;
  constexpr int NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM, NK = C::NK;
  constexpr int ET = C::ET, NT = C::NT, RECF = C::RECF, NPP = C::NPP, KV = C::KV, KF = C::KF, KT = C::KT;
  constexpr int NN = C::NN, GT = C::GT;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::oBar);  // 0,1: tile buffers, 2: RK operands, 3: MMA
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + C::oBar + 64);
  unsigned char* sBh = sm + C::oBh;
  unsigned char* sBl = sm + C::oBl;
  short* sFm = reinterpret_cast<short*>(sm + C::oFm);
  short* sNb = reinterpret_cast<short*>(sm + C::oNb);
  T* sGT = reinterpret_cast<T*>(sm + C::oGT);
  T* sYb = reinterpret_cast<T*>(sm + C::oY);
  T* sGFb = reinterpret_cast<T*>(sm + C::oGF);
  int* sGIb = reinterpret_cast<int*>(sm + C::oGI);
  T* sE = reinterpret_cast<T*>(sm + C::oE);
  T* sN = reinterpret_cast<T*>(sm + C::oN);
  double* sRed = reinterpret_cast<double*>(sm + C::oR);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int lq = warp & 3, part = warp >> 2;  // tensor-memory lane quarter, column part
  const int m = lq * 32 + lane;               // tile row = (q, e)
  const bool row_ok = lq * 32 < C::ROWS;      // warp-uniform
  const int q = m / ET, e = m - (m / ET) * ET;
  const int stage = a.stage;
  const int64_t stride = a.stride;
  // RK operands staged by TMA: u and the accumulator (stages 2-4); the
  // residual snapshot of stage 4 is read straight from global memory
  const int nepi = (stage >= 2 && stage <= 4) ? 2 : 0;

  auto issue_tile = [&](int tile, int b) {
    const int64_t e0 = (int64_t)tile * ET;
    mbar_expect_tx(&bar[b], NV * C::YSEG + C::GFB + C::GIB);
#pragma unroll
    for (int qq = 0; qq < NV; ++qq)
      tma_load_1d(sYb + ((size_t)b * NV + qq) * ET * NP, a.y_in + qq * stride + e0 * NP, C::YSEG, &bar[b]);
    tma_load_1d(sGFb + (size_t)b * ET * RECF, a.geoF + e0 * RECF, C::GFB, &bar[b]);
    tma_load_1d(sGIb + (size_t)b * ET * C::RECI, a.geoI + e0 * C::RECI, C::GIB, &bar[b]);
  };
  auto issue_epi = [&](int tile) {
    const int64_t e0 = (int64_t)tile * ET;
    mbar_expect_tx(&bar[2], nepi * NV * C::YSEG);
    for (int k = 0; k < nepi; ++k) {
      const T* src = k == 0 ? a.u : a.acc;
#pragma unroll
      for (int qq = 0; qq < NV; ++qq)
        tma_load_1d(sE + ((size_t)k * NV + qq) * ET * NP, src + qq * stride + e0 * NP, C::YSEG, &bar[2]);
    }
  };

  // ---- setup: barriers, tensor memory, operator B (hi/lo), node tables ----
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) mbar_init(&bar[i], 1);
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
  for (int i = tid; i < (int)(C::BSLACK / 4); i += NT)
    reinterpret_cast<float*>(sBl + C::BBYTES)[i] = 0.f;
  for (int i = tid; i < NK; i += NT) sFm[i] = a.fmask[i];
  for (int i = tid; i < NF * NPERM * NFP; i += NT) sNb[i] = a.nbrnode[i];
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // B is read by the tensor cores
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t trow = tbase + ((uint32_t)(lq * 32) << 16);
  // A columns that no tile writes are zero: padding past KV + KF, and every
  // column of the rows past ROWS
  {
    const uint32_t z[4] = {0u, 0u, 0u, 0u};
    if (row_ok) {
      for (int c = KV + KF + 4 * part; c < KT; c += 4 * NPART) {
        tmem_st4(trow + C::COL_AH + c, z);
        tmem_st4(trow + C::COL_AL + c, z);
      }
    } else {
      for (int c = 4 * part; c < KT; c += 4 * NPART) {
        tmem_st4(trow + C::COL_AH + c, z);
        tmem_st4(trow + C::COL_AL + c, z);
      }
    }
    tmem_wait_st();
  }

  const T rhoc2 = (T)a.ph.rhoc2, inv_rho0 = (T)a.ph.inv_rho0, half_c0 = (T)a.ph.half_c0;
  const T dt = (T)a.dt;
  float red_a = 0.f;  // this row's residual sum of (snapshot - u)^2 (FP32, see ResAcc)
  bool ok = true;
  // thread 0: barriers whose armed phase was not yet observed complete (bit i)
  // and that phase's parity (bit 4+i); drained before the block exits
  uint32_t pend = 0;
  auto arm = [&](int i, int parity) { pend = (pend & ~(0x11u << i)) | (1u << i) | ((uint32_t)(parity & 1) << (4 + i)); };
  auto seen = [&](int i) { pend &= ~(1u << i); };
  if (tid == 0 && (int)blockIdx.x < a.ntiles) issue_tile(blockIdx.x, 0), arm(0, 0);
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(NN >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);

  int it = 0;
  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int64_t e0 = (int64_t)tile * ET;
    bool got = mbar_wait(&bar[b], (it >> 1) & 1, a.wait_limit);
    if (tid == 0 && got) seen(b);
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    T* sY = sYb + (size_t)b * NV * ET * NP;
    const T* sGF = sGFb + (size_t)b * ET * RECF;
    const int* sGI = sGIb + (size_t)b * ET * C::RECI;
    if (tid == 0) {
      fence_proxy_async();
      const int nt = tile + gridDim.x;
      if (nt < a.ntiles) issue_tile(nt, b ^ 1), arm(b ^ 1, (it + 1) >> 1);
      bulk_wait_read();  // the previous tile's stores have read the operand buffer
      if (nepi > 0) issue_epi(tile), arm(2, it);
    }
    // ---- neighbour traces (asynchronous) ----
    gather_traces<C, T>(a.y_in, stride, sGI, sNb, sN, tid, e0);
    cp_async_commit();
    // ---- per-element values of the row phase, element-minor ----
    for (int w = tid; w < ET * GT; w += NT) {
      const int el = w / GT, v = w - (w / GT) * GT;
      const int src = v < D * D ? v : C::S::PHYS_OFF + (v - D * D);
      sGT[v * (ET + 1) + el] = sGF[el * RECF + src];
    }
    __syncthreads();

    // ---- volume rows: A_vol[(q,e)][(r,j)] -> tensor memory ----
    T g[D][D], gv0[D];
    if (row_ok) {
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int d = 0; d < D; ++d) g[r][d] = sGT[(r * D + d) * (ET + 1) + e];
      T v0[D];
#pragma unroll
      for (int d = 0; d < D; ++d) v0[d] = sGT[(D * D + d) * (ET + 1) + e];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        gv0[r] = g[r][0] * v0[0] + g[r][1] * v0[1];
        if (D == 3) gv0[r] += g[r][2] * v0[2];
      }
      const T* ye = sY + e * NP;
      for (int g4 = part; g4 < NPP / 4; g4 += NPART) {
        const int j0 = g4 * 4;
        T yp[4], yv[D][4];
        // p and the velocity components this row needs (all of them for the
        // p row); lanes are consecutive elements, so vector loads keep the
        // NP-word stride free of bank conflicts
        load4<NP, C::VWY>(yp, ye, j0);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          if (q == 0 || q == 1 + d)
            load4<NP, C::VWY>(yv[d], ye + (1 + d) * ET * NP, j0);
          else
            yv[d][0] = yv[d][1] = yv[d][2] = yv[d][3] = (T)0;
        }
        T fr[D][4];
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
#pragma unroll
          for (int r = 0; r < D; ++r) {
            T x;
            if (q == 0) {
              T gw = g[r][0] * yv[0][jj] + g[r][1] * yv[1][jj];
              if (D == 3) gw += g[r][2] * yv[2][jj];
              x = gv0[r] * yp[jj] + rhoc2 * gw;
            } else {
              const int dq = q - 1;
              T gr = g[r][0];
              T vq = yv[0][jj];
#pragma unroll
              for (int d = 1; d < D; ++d)
                if (dq == d) gr = g[r][d], vq = yv[d][jj];
              x = gv0[r] * vq + gr * yp[jj] * inv_rho0;
            }
            fr[r][jj] = (j0 + jj < NP) ? x : (T)0;
          }
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
          uint32_t hi[4], lo[4];
          split4(fr[r], hi, lo);
          tmem_st4(trow + C::COL_AH + r * NPP + j0, hi);
          tmem_st4(trow + C::COL_AL + r * NPP + j0, lo);
        }
      }
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- face numerical fluxes (in place of the gathered traces) ----
    face_fluxes<C, T>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, tid, rhoc2, inv_rho0, half_c0, e0);
    __syncthreads();

    // ---- face rows: A_face[(q,e)][k] -> tensor memory ----
    if (row_ok) {
      const T* hrow = sN + (size_t)(q * ET + e) * C::NKP;
      for (int c4 = part; c4 < KF / 4; c4 += NPART) {
        T x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = (c4 * 4 + u < NK) ? hrow[c4 * 4 + u] : (T)0;
        uint32_t hi[4], lo[4];
        split4(x, hi, lo);
        tmem_st4(trow + C::COL_AH + KV + c4 * 4, hi);
        tmem_st4(trow + C::COL_AL + KV + c4 * 4, lo);
      }
    }
    tmem_wait_st();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    // ---- D = A_lo B_hi + A_hi B_lo + A_hi B_hi: the correction products
    // first, while D is small (each MMA's accumulation rounds relative to D) ----
    if (tid == 0) {
      const uint32_t bh = smem_u32(sBh), bl = smem_u32(sBl);
#pragma unroll 1
      for (int pass = 0; pass < 3; ++pass) {
        const uint32_t acol = pass == 0 ? C::COL_AL : C::COL_AH;
        const uint32_t bsrc = pass == 1 ? bl : bh;
#pragma unroll 1
        for (int ks = 0; ks < KT / 8; ++ks)
          umma_tf32_ts(tbase + C::COL_D, tbase + acol + ks * 8, umma_desc(bsrc + ks * 2 * C::LBO, C::LBO, C::SBO),
                       idesc, (pass > 0 || ks > 0) ? 1u : 0u);
      }
      umma_commit(&bar[3]);
      arm(3, it);
    }
    got = mbar_wait(&bar[3], it & 1, a.wait_limit);
    if (tid == 0 && got) seen(3);
    if (nepi > 0 && got) {
      got = mbar_wait(&bar[2], it & 1, a.wait_limit);
      if (tid == 0 && got) seen(2);
    }
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    tc_fence_after();

    // ---- epilogue: RK update of this row's nodes in the operand buffer ----
    if (row_ok) {
      constexpr int VW = C::VWY;
      const T dte = dt * sGT[(D * D + D) * (ET + 1) + e];
      T* r0 = sE + (size_t)(q * ET + e) * NP;                  // slot 0 row: u in, new y or u out
      T* r1 = sE + (size_t)(NV * ET + q * ET + e) * NP;        // slot 1 row: acc in, new acc out
      const T* ry = sY + (size_t)(q * ET + e) * NP;            // stage input row (u in stages 1, 5)
      const T* gs = a.snap + q * stride + (e0 + e) * NP;      // residual snapshot row (stage 4)
      // this thread's accumulator chunks (columns part*4, (part+NPART)*4, ...
      // below NP): every load issued first, one wait
      constexpr int NCH = (NN / 4 + NPART - 1) / NPART;
      uint32_t dr[NCH][4];
#pragma unroll
      for (int t = 0; t < NCH; ++t) {
        const int c4 = part + t * NPART;
        if (c4 * 4 < NP) tmem_ld4_async(trow + C::COL_D + c4 * 4, dr[t]);  // warp-uniform condition
      }
#pragma unroll
      for (int t = 0; t < NCH; ++t)
        if ((part + t * NPART) * 4 < NP) tmem_wait_ld4(dr[t]);
#pragma unroll
      for (int t = 0; t < NCH; ++t) {
        const int c4 = part + t * NPART;
        const int i0 = c4 * 4;
        if (i0 >= NP) break;  // warp-uniform
        T kv[4], x0[4], x1[4], o0[4], o1[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) kv[u] = dte * __uint_as_float(dr[t][u]);
        switch (stage) {
          case 0:
            store4<NP, VW>(r0, i0, kv);
            break;
          case 1:
            load4<NP, VW>(x0, ry, i0);
#pragma unroll
            for (int u = 0; u < 4; ++u) o1[u] = x0[u] + (T)0.5 * kv[u];
            store4<NP, VW>(r0, i0, kv);
            store4<NP, VW>(r1, i0, o1);
            break;
          case 2:
          case 3:
            load4<NP, VW>(x0, r0, i0);
            load4<NP, VW>(x1, r1, i0);
#pragma unroll
            for (int u = 0; u < 4; ++u)
              o1[u] = x1[u] + (T)2 * kv[u], o0[u] = x0[u] + (stage == 2 ? (T)0.5 * kv[u] : kv[u]);
            store4<NP, VW>(r1, i0, o1);
            store4<NP, VW>(r0, i0, o0);
            break;
          case 4:
            load4<NP, VW>(x0, r0, i0);
            load4<NP, VW>(x1, r1, i0);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              o0[u] = x0[u] + rk4_sixth(x1[u] + kv[u]);
              if (i0 + u < NP) {
                const float dn = gs[i0 + u] - o0[u];
                red_a = fmaf(dn, dn, red_a);
              }
            }
            store4<NP, VW>(r0, i0, o0);
            break;
          default:
            load4<NP, VW>(x0, ry, i0);
#pragma unroll
            for (int u = 0; u < 4; ++u) o0[u] = x0[u] + kv[u];
            store4<NP, VW>(r0, i0, o0);
            break;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the bulk stores read these values
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      // outputs per stage: (slot, destination)
      T* dst0 = nullptr;
      T* dst1 = nullptr;
      switch (stage) {
        case 0: dst0 = a.k_out; break;
        case 1: dst0 = a.acc, dst1 = a.y_out; break;
        case 2:
        case 3: dst0 = a.y_out, dst1 = a.acc; break;
        case 4: dst0 = a.u; break;
        default: dst0 = a.y_out; break;
      }
#pragma unroll
      for (int qq = 0; qq < NV; ++qq) {
        tma_store_1d(dst0 + qq * stride + e0 * NP, sE + (size_t)qq * ET * NP, C::YSEG);
        if (dst1) tma_store_1d(dst1 + qq * stride + e0 * NP, sE + ((size_t)NV + qq) * ET * NP, C::YSEG);
      }
      bulk_commit();
    }
  }

  // ---- teardown: own copies and tensor-core work first, then the memory ----
  if (tid == 0) {
    bulk_wait_all();
    // after a timeout: bounded waits for the copies and the MMA group still
    // armed, so that nothing lands in freed shared or tensor memory
    for (int i = 0; i < 4; ++i)
      if (pend & (1u << i)) mbar_wait(&bar[i], (pend >> (4 + i)) & 1u);
  }
  if (!ok && tid == 0) atomicOr(err, 1);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"((uint32_t)C::TCOLS)
                 : "memory");

  if (stage == 4) {
    // residual components: 0 p, 1 p/c0^2, 2.. velocity components
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const double ra = (double)red_a;
      double v = !row_ok ? 0.0
                         : (c == 0 ? (q == 0 ? ra : 0.0)
                                   : c == 1 ? (q == 0 ? ra / (a.c0sq * a.c0sq) : 0.0) : (q == c - 1 ? ra : 0.0));
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
struct StageTc {
  using C = TcCfg<D, P, NPART>;
  static int blocks_per_sm() {
    auto kfn = stage_tc_kernel<D, P, NPART>;
    // the largest shared-memory carve-out, so that the occupancy query and
    // the launches see the same per-SM capacity
    if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes) != cudaSuccess ||
        cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
            cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    // The runtime's occupancy query answers 1 block per SM for kernels that
    // use tensor memory; the block count is taken from the SM's limits
    // instead: shared memory, threads, registers, and the 512 tensor-memory
    // columns that the resident blocks share. Blocks never wait on one
    // another, so a grid larger than what is resident is only slower.
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
    auto kfn = stage_tc_kernel<D, P, NPART>;
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
