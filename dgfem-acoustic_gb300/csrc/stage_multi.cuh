// One persistent launch per RK stage for a batch of 2-D instances of mixed
// order (p = 2, 3, 4): the batched ensemble's stage kernel (FP32 state).
//
// The batch keeps one disjoint-union mesh per element order (batch.cu). This
// kernel advances all of them in one launch: its blocks take tiles from a
// work queue over every order's tiles (an atomic counter; order after order)
// and run each tile with the wide-chunk kernel's per-tile code for that
// order (wide_tile in stage4.cuh) with that order's own tile shape; the
// block has the largest shape's thread count and the threads past a shape's
// count idle in its tiles (the shapes below all have 64 threads):
//   p = 2: 64 elements per tile, 6 nodes per thread, one thread per element;
//   p = 3: 32 elements per tile, 6 nodes per thread, two per element;
//   p = 4: 32 elements per tile, 8 nodes per thread, two per element;
// all with the volume contraction per reference direction (W form) and the
// RK operands read from L2 by the coalesced update (not staged). Every
// order's reference operators sit in shared memory. The tile buffers are two
// fixed slots sized for the largest order (consecutive queue items may be of
// different orders; the next item's stage input and geometry arrive by TMA
// while the current one computes), then the face-flux buffer, also sized for
// the largest order. Every wait is bounded; after a timeout a block records
// the error, drains its own copies (bounded) and stops taking work.
#pragma once
#include <cstdint>

#include "stage4.cuh"

namespace dgk {

using MultiC2 = Wide<2, 2, 6, 64, kWForm, false>;
using MultiC3 = Wide<2, 3, 6, 32, kWForm, false>;
using MultiC4 = Wide<2, 4, 8, 32, kWForm, false>;
constexpr int kMultiNT = 64;
// blocks per SM the register budget is set for (the shared memory's limit)
constexpr int kMultiMinBlocks = 6;

template <typename A, typename B>
constexpr A cmax(A x, B y) {
  return x > (A)y ? x : (A)y;
}

// operator tables of an order: the [oD, oY) section of its Pipe layout
template <class C>
constexpr size_t multi_ops_bytes() {
  return C::oY - C::oD;
}
template <class C>
constexpr size_t multi_slot_bytes() {
  return RoundUp<C::NV * C::YSEG + C::GFB + C::GIB, 128>::v;
}
template <class C>
constexpr size_t multi_epi_bytes() {
  return C::kStaged ? 3 * (size_t)C::NV * C::YSEG : 0;
}
template <class C>
constexpr size_t multi_nbuf_bytes() {
  return C::SN_WORDS * 4;
}

struct MultiLayout {
  static constexpr size_t oBar = 0;  // 3 mbarriers, then the next work item
  static constexpr size_t oItem = 32;
  static constexpr size_t oOps2 = 64;
  static constexpr size_t oOps3 = RoundUp<oOps2 + multi_ops_bytes<MultiC2>(), 128>::v;
  static constexpr size_t oOps4 = RoundUp<oOps3 + multi_ops_bytes<MultiC3>(), 128>::v;
  static constexpr size_t SLOT =
      cmax(cmax(multi_slot_bytes<MultiC2>(), multi_slot_bytes<MultiC3>()), multi_slot_bytes<MultiC4>());
  static constexpr size_t oSlot = RoundUp<oOps4 + multi_ops_bytes<MultiC4>(), 128>::v;  // 2 slots
  static constexpr size_t oE = oSlot + 2 * SLOT;
  static constexpr size_t EPI =
      cmax(cmax(multi_epi_bytes<MultiC2>(), multi_epi_bytes<MultiC3>()), multi_epi_bytes<MultiC4>());
  static constexpr size_t oN = RoundUp<oE + EPI, 128>::v;
  static constexpr size_t NBUF =
      cmax(cmax(multi_nbuf_bytes<MultiC2>(), multi_nbuf_bytes<MultiC3>()), multi_nbuf_bytes<MultiC4>());
  static constexpr size_t oR = RoundUp<oN + NBUF, 16>::v;  // [warps][5] double
  static constexpr size_t bytes = oR + (size_t)(kMultiNT / 32) * 5 * sizeof(double);
};

static_assert(MultiC2::NT <= kMultiNT && MultiC3::NT <= kMultiNT && MultiC4::NT <= kMultiNT,
              "the block holds every order's tile shape");
static_assert(kMultiNT % 32 == 0 && MultiC2::NT % 32 == 0 && MultiC3::NT % 32 == 0 && MultiC4::NT % 32 == 0,
              "idle threads of a tile are whole warps");

// Operator tables of one order in shared memory (same relative layout as in
// the order's pipelined kernel).
template <class C>
struct OpsSm {
  const float* sD;
  const float* sL;
  const short* sFm;
  const short* sNb;
  __device__ static OpsSm at(unsigned char* base) {
    OpsSm o;
    o.sD = reinterpret_cast<const float*>(base);
    o.sL = reinterpret_cast<const float*>(base + (C::oL - C::oD));
    o.sFm = reinterpret_cast<const short*>(base + (C::oFm - C::oD));
    o.sNb = reinterpret_cast<const short*>(base + (C::oNb - C::oD));
    return o;
  }
  __device__ static void load(unsigned char* base, const StageArgs<float>& a, int tid) {
    constexpr int NK = C::NK, NF = C::NF, NFP = C::NFP, NPERM = C::NPERM;
    float* sD = reinterpret_cast<float*>(base);
    float* sL = reinterpret_cast<float*>(base + (C::oL - C::oD));
    short* sFm = reinterpret_cast<short*>(base + (C::oFm - C::oD));
    short* sNb = reinterpret_cast<short*>(base + (C::oNb - C::oD));
    WideTileOps::load_ops<C, float>(sD, sL, a, tid, kMultiNT);
    for (int i = tid; i < NK; i += kMultiNT) sFm[i] = a.fmask[i];
    for (int i = tid; i < NF * NPERM * NFP; i += kMultiNT) sNb[i] = a.nbrnode[i];
  }
};

// order slot and tile of a work item (items run order after order)
__device__ __forceinline__ int multi_slot(const MultiArgs& m, int item, int* tile) {
  int t = item;
#pragma unroll
  for (int g = 0; g < kMultiOrders; ++g) {
    if (t < m.g[g].ntiles) {
      *tile = t;
      return g;
    }
    t -= m.g[g].ntiles;
  }
  *tile = 0;
  return -1;
}

template <class C>
__device__ __forceinline__ void multi_issue_tile(const StageArgs<float>& a, int tile, unsigned char* slot,
                                                 uint64_t* bar) {
  constexpr int NV = C::NV, ET = C::ET, NP = C::NP, RECF = C::RECF, RECI = C::RECI;
  const int64_t e0 = (int64_t)tile * ET;
  float* sY = reinterpret_cast<float*>(slot);
  float* sGF = reinterpret_cast<float*>(slot + NV * C::YSEG);
  int* sGI = reinterpret_cast<int*>(slot + NV * C::YSEG + C::GFB);
  mbar_expect_tx(bar, NV * C::YSEG + C::GFB + C::GIB);
#pragma unroll
  for (int q = 0; q < NV; ++q) tma_load_1d(sY + q * ET * NP, a.y_in + q * a.stride + e0 * NP, C::YSEG, bar);
  tma_load_1d(sGF, a.geoF + e0 * RECF, C::GFB, bar);
  tma_load_1d(sGI, a.geoI + e0 * RECI, C::GIB, bar);
}

template <class C>
__device__ __forceinline__ void multi_issue_epi(const StageArgs<float>& a, int tile, float* sE, int nepi,
                                                uint64_t* bar) {
  constexpr int NV = C::NV, ET = C::ET, NP = C::NP;
  const int64_t e0 = (int64_t)tile * ET;
  mbar_expect_tx(bar, nepi * NV * C::YSEG);
  for (int k = 0; k < nepi; ++k) {
    const float* src = k == 0 ? a.u : (k == 1 ? a.acc : a.snap);
#pragma unroll
    for (int q = 0; q < NV; ++q)
      tma_load_1d(sE + ((size_t)k * NV + q) * ET * NP, src + q * a.stride + e0 * NP, C::YSEG, bar);
  }
}

template <class C>
__device__ __forceinline__ void multi_run_tile(const StageArgs<float>& a, int tile, unsigned char* slot, float* sE,
                                               float* sN, unsigned char* ops, uint64_t* bar_epi, uint32_t epi_parity,
                                               int nepi, int tid, bool& ok, ResAcc<float>& racc) {
  const OpsSm<C> o = OpsSm<C>::at(ops);
  float* sY = reinterpret_cast<float*>(slot);
  const float* sGF = reinterpret_cast<const float*>(slot + C::NV * C::YSEG);
  const int* sGI = reinterpret_cast<const int*>(slot + C::NV * C::YSEG + C::GFB);
  wide_tile<C>(a, (int64_t)tile * C::ET, sY, sGF, sGI, sE, sN, o.sD, o.sL, o.sFm, o.sNb, bar_epi, epi_parity, nepi,
               tid, ok, racc);
}

__global__ void __launch_bounds__(kMultiNT, kMultiMinBlocks) stage_multi_kernel(const MultiArgs m, int* err) {
  using L = MultiLayout;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + L::oBar);  // [0],[1]: slots, [2]: RK operands
  int* sItem = reinterpret_cast<int*>(sm + L::oItem);         // next work item
  unsigned char* ops2 = sm + L::oOps2;
  unsigned char* ops3 = sm + L::oOps3;
  unsigned char* ops4 = sm + L::oOps4;
  unsigned char* slots = sm + L::oSlot;
  float* sE = reinterpret_cast<float*>(sm + L::oE);
  float* sN = reinterpret_cast<float*>(sm + L::oN);
  double* sRed = reinterpret_cast<double*>(sm + L::oR);
  const int tid = threadIdx.x;
  const int stage = m.g[0].stage;
  const int nepi = (stage == 2 || stage == 3) ? 2 : (stage == 4 ? 3 : 0);

  auto issue = [&](int item, int b) {
    int tile;
    const int g = multi_slot(m, item, &tile);
    unsigned char* slot = slots + (size_t)b * L::SLOT;
    if (g == 0) multi_issue_tile<MultiC2>(m.g[0], tile, slot, &bar[b]);
    if (g == 1) multi_issue_tile<MultiC3>(m.g[1], tile, slot, &bar[b]);
    if (g == 2) multi_issue_tile<MultiC4>(m.g[2], tile, slot, &bar[b]);
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_mbar_init();
  }
  if (m.g[0].ntiles > 0) OpsSm<MultiC2>::load(ops2, m.g[0], tid);
  if (m.g[1].ntiles > 0) OpsSm<MultiC3>::load(ops3, m.g[1], tid);
  if (m.g[2].ntiles > 0) OpsSm<MultiC4>::load(ops4, m.g[2], tid);
  // thread 0: slots (bits 0, 1) and RK operands (bit 2) armed and not yet
  // observed complete, drained on exit
  uint32_t pend = 0;
  // thread 0 claims items one ahead of the prefetch: the queue's atomic
  // round trip overlaps a tile's work instead of delaying the next copy
  int ahead = 0;
  if (tid == 0) {
    const int first = (int)atomicAdd(m.queue, 1u);
    *sItem = first;
    if (first < m.ntiles_total) {
      issue(first, 0), pend = 1u;
      ahead = (int)atomicAdd(m.queue, 1u);
    }
  }
  __syncthreads();

  // stage 4: racc holds the residual sums of order rg; a block's items come
  // in order after order, so each order's row is written once, when the
  // block moves on to the next order or finishes (orders bit-set in wrote)
  ResAcc<float> racc;
  int rg = -1;
  unsigned wrote = 0;
  auto put_row = [&](int g, bool zero) {
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      double v = zero ? 0.0 : racc.get(c, m.g[g].c0sq);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
      if ((tid & 31) == 0) sRed[(tid >> 5) * 5 + c] = v;
    }
    __syncthreads();
    if (tid < 5) {
      double v = 0.0;
      for (int w = 0; w < kMultiNT / 32; ++w) v += sRed[w * 5 + tid];
      m.g[g].partials[blockIdx.x * 5 + tid] = v;
    }
    __syncthreads();
    racc = ResAcc<float>();
    wrote |= 1u << g;
  };
  bool ok = true;
  int it = 0;
  for (;; ++it) {
    const int item = *sItem;  // written before the barrier that ended the previous item
    if (item >= m.ntiles_total) break;
    const int b = it & 1;
    const bool got = mbar_wait(&bar[b], (it >> 1) & 1, m.wait_limit);
    if (tid == 0 && got) pend &= ~(1u << b);
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    int tile;
    const int g = multi_slot(m, item, &tile);
    if (stage == 4 && g != rg) {  // block-uniform
      if (rg >= 0) put_row(rg, false);
      rg = g;
    }
    if (tid == 0) {
      fence_proxy_async();
      const int next = ahead;
      *sItem = next;
      if (next < m.ntiles_total) {
        issue(next, b ^ 1), pend |= 1u << (b ^ 1);
        ahead = (int)atomicAdd(m.queue, 1u);
      }
      if (nepi > 0) {
        if (g == 0 && MultiC2::kStaged) multi_issue_epi<MultiC2>(m.g[0], tile, sE, nepi, &bar[2]), pend |= 4u;
        if (g == 1 && MultiC3::kStaged) multi_issue_epi<MultiC3>(m.g[1], tile, sE, nepi, &bar[2]), pend |= 4u;
        if (g == 2 && MultiC4::kStaged) multi_issue_epi<MultiC4>(m.g[2], tile, sE, nepi, &bar[2]), pend |= 4u;
      }
    }
    unsigned char* slot = slots + (size_t)b * L::SLOT;
    if (g == 0)
      multi_run_tile<MultiC2>(m.g[0], tile, slot, sE, sN, ops2, &bar[2], (uint32_t)(it & 1), nepi, tid, ok, racc);
    else if (g == 1)
      multi_run_tile<MultiC3>(m.g[1], tile, slot, sE, sN, ops3, &bar[2], (uint32_t)(it & 1), nepi, tid, ok, racc);
    else
      multi_run_tile<MultiC4>(m.g[2], tile, slot, sE, sN, ops4, &bar[2], (uint32_t)(it & 1), nepi, tid, ok, racc);
    if (tid == 0 && ok) pend &= ~4u;  // the RK operands arrived (waited inside the tile)
    if (__syncthreads_or(!ok)) {      // buffers of this item are free again
      ok = false;
      break;
    }
  }
  if (tid == 0) {
    // after a timeout: bounded waits for this block's copies still in flight
    for (int i = 0; i < 2; ++i)
      if (pend & (1u << i)) mbar_wait(&bar[i], (uint32_t)(((it + (i != (it & 1))) >> 1) & 1));
    if (pend & 4u) mbar_wait(&bar[2], (uint32_t)(it & 1));
    if (!ok) atomicOr(err, 1);
  }

  if (stage == 4) {
    // residual partial sums per order (one row per block in each order's
    // partials array; a block that ran no tile of an order writes zeros)
    if (rg >= 0) put_row(rg, false);
#pragma unroll
    for (int g = 0; g < kMultiOrders; ++g)
      if (m.g[g].ntiles > 0 && !(wrote & (1u << g))) put_row(g, true);
  }
}

}  // namespace dgk
