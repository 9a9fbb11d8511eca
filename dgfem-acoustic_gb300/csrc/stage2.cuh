// Pipelined fused RK4 stage kernel (sm_103a).
//
// Same arithmetic as the reference's per-stage work (src/Mesh.cpp:734-975,
// src/solver.cpp:38-57, :488-516), organised for memory-level parallelism:
//
//   persistent blocks, one tile of ET consecutive elements at a time;
//   * the tile's stage input and geometry records arrive by TMA bulk copies
//     (cp.async.bulk, mbarrier completion) into a double buffer: the next
//     tile is in flight while the current one computes;
//   * the tile's RK operands (u, accumulator, residual snapshot) arrive by a
//     second TMA group issued at tile start and consumed by the epilogue;
//   * neighbour traces are gathered with per-thread cp.async (LDGSTS) issued
//     before the volume contraction and awaited after it;
//   * volume contraction W^r = Dt_r y (shared operators, register blocked:
//     each thread owns NC output nodes of one element), flux mixing, face
//     numerical fluxes, LIFT, and the RK update straight from registers with
//     vectorised coalesced stores.
// Every mbarrier wait is bounded; on timeout the block records an error flag
// and finishes its loop without further waiting.
#pragma once
#include <cstdint>
#include <type_traits>

#include "dg_internal.cuh"

namespace dgk {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// 1-D TMA bulk copy global -> shared, completion counted on bar (bytes % 16 == 0,
// both addresses 16-byte aligned).
__device__ __forceinline__ void tma_load_1d(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bulk prefetch of bytes at p into L2 (no completion to wait for).
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Bounded wait for the phase with the given parity: at most `limit` polling
// rounds (none when limit <= 0); false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = kWaitRounds) {
  const uint32_t a = smem_u32(bar);
  for (int it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(kWaitHintNs)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit_wait_all() {
  asm volatile("cp.async.commit_group;\n cp.async.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// VW-wide vector load/store of T (VW in {1, 2, 4}; addresses VW-aligned).
template <typename T, int VW>
__device__ __forceinline__ void vload(T* r, const T* p) {
  if constexpr (VW == 4 && sizeof(T) == 8) {
    const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
    r[0] = a.x, r[1] = a.y, r[2] = b.x, r[3] = b.y;
  } else if constexpr (VW == 4 && sizeof(T) == 4) {
    float4 v = *reinterpret_cast<const float4*>(p);
    r[0] = v.x, r[1] = v.y, r[2] = v.z, r[3] = v.w;
  } else if constexpr (VW == 2 && sizeof(T) == 4) {
    float2 v = *reinterpret_cast<const float2*>(p);
    r[0] = v.x, r[1] = v.y;
  } else if constexpr (VW == 2 && sizeof(T) == 8) {
    double2 v = *reinterpret_cast<const double2*>(p);
    r[0] = v.x, r[1] = v.y;
  } else {
#pragma unroll
    for (int v = 0; v < VW; ++v) r[v] = p[v];
  }
}
template <typename T, int VW>
__device__ __forceinline__ void vstore(T* p, const T* r) {
  if constexpr (VW == 4 && sizeof(T) == 8) {
    reinterpret_cast<double2*>(p)[0] = make_double2(r[0], r[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(r[2], r[3]);
  } else if constexpr (VW == 4 && sizeof(T) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
  } else if constexpr (VW == 2 && sizeof(T) == 4) {
    *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
  } else if constexpr (VW == 2 && sizeof(T) == 8) {
    *reinterpret_cast<double2*>(p) = make_double2(r[0], r[1]);
  } else {
#pragma unroll
    for (int v = 0; v < VW; ++v) p[v] = r[v];
  }
}

// The NC entries row[i0 .. i0+NC) of an operator row in shared memory, in
// VW-wide vectors when the chunk is aligned; entries past the row end
// (last chunk of a node split that does not divide NP) repeat the last entry.
template <typename T, int NC, int VW, int NP>
__device__ __forceinline__ void load_chunk(T* out, const T* row, int i0) {
  if constexpr (VW > 1) {
#pragma unroll
    for (int c = 0; c < NC; c += VW) vload<T, VW>(out + c, row + i0 + c);
  } else {
#pragma unroll
    for (int ii = 0; ii < NC; ++ii) out[ii] = row[(i0 + ii < NP) ? i0 + ii : NP - 1];
  }
}

template <int N, int A>
struct RoundUp {
  static constexpr int v = (N + A - 1) / A * A;
};

// Per-tile helpers shared by the pipelined and the tensor-core stage kernels.
// C provides the element shape (D, NP, NF, NFP, NV, NPERM, NK), the tile
// (ET elements, NT threads), the record sizes and the face buffer's strides:
// entry (variable q, element el, face node k) of sN sits at
// el * SN_EL + k * SN_K + q * SN_Q, either one plane per variable
// [NV][ET][NKP] (SN_Q = ET * NKP) or the variables of a face node side by side
// [ET][NKP][NVQ] (SN_Q = 1, NVQ = NV), so that the
// lifting reads all variables of a node with one vector load.
// Tile buffers: sY [NV][ET][NP], sGF [ET][RECF], sGI [ET][RECI], sN.

// Face work is split into items of one element face and MC of its NFP nodes
// (nodes ch, ch + FCH, ...: the items of neighbouring threads take
// neighbouring face nodes, so that their writes to sN are consecutive); the
// face's data (neighbour, code, normal, scale, mean-flow component, boundary
// matrix) is read once per item. FCH, the items per face, is the smallest
// divisor of NFP for which the items fill the block (equal items: measured
// faster than uneven ones on the 3-D p = 3 kernels).
constexpr int face_runs(int nfp, int items_per_run, int nt) {
  for (int d = 1; d <= nfp; ++d)
    if (nfp % d == 0 && items_per_run * d >= nt) return d;
  return nfp;
}
template <class C>
struct FaceSplit {
  static constexpr int FCH = face_runs(C::NFP, C::ET * C::NF, C::NT);
  static constexpr int MC = C::NFP / FCH;
  static constexpr int ITEMS = C::ET * C::NF * FCH;
};

// Issues cp.async gathers of the neighbour traces of every interior face
// node of the tile whose neighbour lies outside the tile (elements e0 ..
// e0+ET-1) into sN (the caller commits and waits); traces of neighbours
// inside the tile are read from the tile itself by face_fluxes.
template <class C, typename T>
__device__ __forceinline__ void gather_traces(const T* __restrict__ y_in, int64_t stride, const int* sGI,
                                              const short* sNb, T* sN, int tid, int64_t e0) {
  constexpr int NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM;
  constexpr int ET = C::ET, NT = C::NT, RECI = C::RECI;
  using FS = FaceSplit<C>;
  for (int it = tid; it < FS::ITEMS; it += NT) {
    const int el = it / (NF * FS::FCH), rem = it - el * (NF * FS::FCH);
    const int f = rem / FS::FCH, ch = rem - f * FS::FCH;
    const int code = sGI[el * RECI + NF + f];
    const int nbr = sGI[el * RECI + f];
    if ((code & kCodeBoundary) || (uint64_t)((int64_t)nbr - e0) < (uint64_t)ET) continue;
    const short* nbt = sNb + ((code & kCodeLfMask) * NPERM + ((code >> kCodePermShift) & kCodePermMask)) * NFP;
    const T* src0 = y_in + (int64_t)nbr * NP;
    T* dst0 = sN + (size_t)el * C::SN_EL + f * NFP * C::SN_K;
#pragma unroll
    for (int mm = 0; mm < FS::MC; ++mm) {
      const int m = mm * FS::FCH + ch;
      const T* src = src0 + nbt[m];
      T* dst = dst0 + m * C::SN_K;
#pragma unroll
      for (int q = 0; q < NV; ++q) {
        if (sizeof(T) == 4)
          cp_async4(dst + q * C::SN_Q, src + q * stride);
        else
          cp_async8(dst + q * C::SN_Q, src + q * stride);
      }
    }
  }
}

// Face numerical fluxes of every face node of the tile, scaled by the face
// scale sJ, written in place of the gathered traces in sN: the interior
// Lax-Friedrichs flux (src/Mesh.cpp:761-813) or the boundary matrix
// (absorbing RKR / reflecting, src/Mesh.cpp:882-972). The neighbour trace
// comes from the tile when the neighbour is one of its elements, else from
// the gathered copy.
template <class C, typename T>
__device__ __forceinline__ void face_fluxes(const T* __restrict__ bmat, const T* sY, const T* sGF, const int* sGI,
                                            const short* sFm, const short* sNb, T* sN, int tid, T rhoc2, T inv_rho0,
                                            T half_c0, int64_t e0) {
  constexpr int D = C::D, NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM;
  constexpr int ET = C::ET, NT = C::NT, RECF = C::RECF, RECI = C::RECI;
  using FS = FaceSplit<C>;
  for (int it = tid; it < FS::ITEMS; it += NT) {
    const int el = it / (NF * FS::FCH), rem = it - el * (NF * FS::FCH);
    const int f = rem / FS::FCH, ch = rem - f * FS::FCH;
    const int nbr = sGI[el * RECI + f];
    const int code = sGI[el * RECI + NF + f];
    const T* gf = sGF + el * RECF + D * D + f * (D + 1);
    T n[3];
#pragma unroll
    for (int d = 0; d < D; ++d) n[d] = gf[d];
    const T sJ = gf[D];
    const T* ye = sY + el * NP;
    T* srow = sN + (size_t)el * C::SN_EL + f * NFP * C::SN_K;
    const short* fm = sFm + f * NFP;
    // h holds the flux already scaled by sJ (the per-face coefficients
    // below carry the scale)
    auto put = [&](int m, const T (&h)[NV]) {
      T* slot = srow + m * C::SN_K;
      if constexpr (C::SN_Q == 1) {
        T hv[C::NVQ];
#pragma unroll
        for (int q = 0; q < C::NVQ; ++q) hv[q] = q < NV ? h[q < NV ? q : 0] : (T)0;
        vstore<T, C::NVQ>(slot, hv);
      } else {
#pragma unroll
        for (int q = 0; q < NV; ++q) slot[(size_t)q * C::SN_Q] = h[q];
      }
    };
    if (code & kCodeBoundary) {
      T B[NV][NV];  // sJ * the boundary matrix
      const T* Bg = bmat + (int64_t)nbr * NV * NV;
#pragma unroll
      for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int qq = 0; qq < NV; ++qq) B[q][qq] = sJ * __ldg(Bg + q * NV + qq);
#pragma unroll
      for (int mm = 0; mm < FS::MC; ++mm) {
        const int m = mm * FS::FCH + ch;
          const int node = fm[m];
        T um[NV], h[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) um[q] = ye[q * ET * NP + node];
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          T acc = 0;
#pragma unroll
          for (int qq = 0; qq < NV; ++qq) acc += B[q][qq] * um[qq];
          h[q] = acc;
        }
        put(m, h);
      }
    } else {
      const int64_t rel = (int64_t)nbr - e0;
      const bool in_tile = (uint64_t)rel < (uint64_t)ET;
      const short* nbt = sNb + ((code & kCodeLfMask) * NPERM + ((code >> kCodePermShift) & kCodePermMask)) * NFP;
      const T* yn = sY + (in_tile ? (int)rel : 0) * NP;
      const T hc = (code & kCodeNegPenalty) ? -half_c0 : half_c0;
      const T* ev0 = sGF + el * RECF + C::S::PHYS_OFF;
      T vn0 = ev0[0] * n[0];
#pragma unroll
      for (int d = 1; d < D; ++d) vn0 += ev0[d] * n[d];
      // sJ h = (sJ vn0 / 2) avg + (sJ n / 2) (rho0 c0^2 avg_v, avg_p / rho0)
      //        + (sJ hc) dif
      const T hsJ = (T)0.5 * sJ;
      const T a0 = hsJ * vn0, hcs = sJ * hc;
      T np_[3], nu_[3];
#pragma unroll
      for (int d = 0; d < D; ++d) np_[d] = hsJ * rhoc2 * n[d], nu_[d] = hsJ * inv_rho0 * n[d];
#pragma unroll
      for (int mm = 0; mm < FS::MC; ++mm) {
        const int m = mm * FS::FCH + ch;
          const int node = fm[m];
        T um[NV], up[NV], h[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) um[q] = ye[q * ET * NP + node];
        if (in_tile) {
          const int nn = nbt[m];
#pragma unroll
          for (int q = 0; q < NV; ++q) up[q] = yn[q * ET * NP + nn];
        } else {
          const T* slot = srow + m * C::SN_K;
          if constexpr (C::SN_Q == 1) {
            T hv[C::NVQ];  // the node's gathered variables in one vector load
            vload<T, C::NVQ>(hv, slot);
#pragma unroll
            for (int q = 0; q < NV; ++q) up[q] = hv[q];
          } else {
#pragma unroll
            for (int q = 0; q < NV; ++q) up[q] = slot[(size_t)q * C::SN_Q];
          }
        }
        T avg[NV], dif[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) avg[q] = um[q] + up[q], dif[q] = um[q] - up[q];
        T x = a0 * avg[0];
#pragma unroll
        for (int d = 0; d < D; ++d) x += np_[d] * avg[1 + d];
        h[0] = x + hcs * dif[0];
#pragma unroll
        for (int d = 0; d < D; ++d) h[1 + d] = a0 * avg[1 + d] + nu_[d] * avg[0] + hcs * dif[1 + d];
        put(m, h);
      }
    }
  }
}

// Compile-time configuration: element shape (D, P), precision T, nodes per
// thread NC and elements per tile ET.
template <typename T, int D_, int P, int NC_, int ET_>
struct Pipe {
  using S = ShapeT<D_, P, T>;
  static constexpr bool kStaged = true;  // RK operands staged in shared memory by TMA
  static constexpr int D = D_;
  static constexpr int NP = S::NP, NF = S::NF, NFP = S::NFP, NV = S::NV, NPERM = S::NPERM, NK = NF * NFP;
  static constexpr int NC = NC_;
  static constexpr int NSPLIT = (NP + NC - 1) / NC;
  static constexpr int ET = ET_;
  static constexpr int NT = ET * NSPLIT;
  static constexpr int RECF = S::RECF, RECI = S::RECI;
  static constexpr int Q4 = 4;  // variables per face node slot (vz slot unused in 2-D)
  // epilogue vector width: chunks of NC nodes start on VW-element boundaries
  // when NP is a multiple of NC (16-byte vectors at most)
  static constexpr int VWMAX = 16 / (int)sizeof(T);
  static constexpr int VW = (NP % NC != 0) ? 1 : (NC % 4 == 0 && VWMAX >= 4) ? 4 : (NC % 2 == 0) ? 2 : 1;
  // byte sizes of the TMA segments
  static constexpr uint32_t YSEG = ET * NP * sizeof(T);  // one variable of the tile
  static constexpr uint32_t GFB = ET * RECF * sizeof(T);
  static constexpr uint32_t GIB = ET * RECI * sizeof(int);
  // shared memory layout (bytes)
  static constexpr size_t oBar = 0;                                        // 3 mbarriers
  static constexpr size_t oD = 64;                                          // Dt [D][NP j][NP i]
  static constexpr size_t oL = RoundUp<oD + D * NP * NP * sizeof(T), 16>::v;  // LIFT [NK][NP]
  static constexpr size_t oFm = RoundUp<oL + NK * NP * sizeof(T), 16>::v;     // fmask
  static constexpr size_t oNb = oFm + RoundUp<NK * 2, 16>::v;                 // nbrnode
  static constexpr size_t oY = RoundUp<oNb + NF * NPERM * NFP * 2, 128>::v;   // 2 x [NV][ET][NP]
  static constexpr size_t oGF = oY + 2 * (size_t)NV * YSEG;                  // 2 x [ET][RECF]
  static constexpr size_t oGI = oGF + 2 * (size_t)GFB;                        // 2 x [ET][RECI]
  static constexpr size_t oE = RoundUp<oGI + 2 * (size_t)GIB, 128>::v;       // [3][NV][ET][NP]
  // neighbour traces / face fluxes, the variables of a face node side by
  // side; element stride NKP (odd) x NVQ so that the elements of a warp read
  // distinct banks
  static constexpr int NKP = NK | 1;
  static constexpr int NVQ = NV;  // 2-D: three words, no padding (it would cost occupancy)
  static constexpr int SN_EL = NKP * NVQ, SN_K = NVQ, SN_Q = 1;
  static constexpr size_t SN_WORDS = (size_t)ET * NKP * NVQ;
  static constexpr size_t oN = oE + 3 * (size_t)NV * YSEG;                    // [ET][NKP][NVQ]
  static constexpr size_t oR = RoundUp<oN + SN_WORDS * sizeof(T), 16>::v;   // [NT/32][5] double
  static constexpr size_t bytes = oR + (NT / 32) * 5 * sizeof(double);
  static_assert(NT % 32 == 0, "threads per block must be a multiple of 32");
  static_assert((ET * NP * sizeof(T)) % 16 == 0, "tile segments must be 16-byte multiples");
};

// RK update of this thread's chunk of output nodes (i0 .. i0+NC of element
// e0 + e, every variable) from the operator result Lv in registers: stage 0
// writes dt*L; RK4 stages 1-3 write the accumulator and the next stage input;
// stage 4 writes the new state and adds to the residual sums; stage 5
// (Euler) writes u + dt*L. The tile's u (eu), accumulator and snapshot (in sE
// after eu's slot) are in shared memory in the [q][e][i] layout; dte is dt
// times the element's step scale. Global stores are VW-wide vectors (the
// chunk and element starts must be VW-aligned, NP a multiple of VW).
template <typename T, int NC, int NV, int VW, int ET, int NP>
__device__ __forceinline__ void rk_update_regs(const StageArgs<T>& a, int64_t e0, int e, int i0, const T (&Lv)[NC][NV],
                                               const T* eu, const T* sE, T dte, ResAcc<T>& racc) {
  const int64_t stride = a.stride;
  const T* ea = sE + (size_t)NV * ET * NP;
  const T* es = sE + (size_t)2 * NV * ET * NP;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
#pragma unroll
    for (int c0 = 0; c0 < NC; c0 += VW) {
      const int i = i0 + c0;
      if (i >= NP) continue;
      const int lidx = (q * ET + e) * NP + i;
      const int64_t g = q * stride + (e0 + e) * NP + i;
      T kv[VW], o1[VW], o2[VW], xu[VW], xa[VW];
#pragma unroll
      for (int v = 0; v < VW; ++v) kv[v] = dte * Lv[c0 + v][q];
      switch (a.stage) {
        case 0:
          vstore<T, VW>(a.k_out + g, kv);
          break;
        case 1:
          vload<T, VW>(xu, eu + lidx);
#pragma unroll
          for (int v = 0; v < VW; ++v) o1[v] = kv[v], o2[v] = xu[v] + (T)0.5 * kv[v];
          vstore<T, VW>(a.acc + g, o1);
          vstore<T, VW>(a.y_out + g, o2);
          break;
        case 2:
        case 3:
          vload<T, VW>(xu, eu + lidx);
          vload<T, VW>(xa, ea + lidx);
#pragma unroll
          for (int v = 0; v < VW; ++v)
            o1[v] = xa[v] + (T)2 * kv[v], o2[v] = xu[v] + (a.stage == 2 ? (T)0.5 * kv[v] : kv[v]);
          vstore<T, VW>(a.acc + g, o1);
          vstore<T, VW>(a.y_out + g, o2);
          break;
        case 4: {
          T xs[VW];
          vload<T, VW>(xu, eu + lidx);
          vload<T, VW>(xa, ea + lidx);
          vload<T, VW>(xs, es + lidx);
#pragma unroll
          for (int v = 0; v < VW; ++v) {
            const T un = xu[v] + rk4_sixth(xa[v] + kv[v]);
            o1[v] = un;
            racc.add(q, xs[v], un, a.c0sq);
          }
          vstore<T, VW>(a.u + g, o1);
          break;
        }
        default:
          vload<T, VW>(xu, eu + lidx);
#pragma unroll
          for (int v = 0; v < VW; ++v) o2[v] = xu[v] + kv[v];
          vstore<T, VW>(a.y_out + g, o2);
          break;
      }
    }
  }
}

// One tile of the pipelined stage for elements e0 .. e0+ET-1: neighbour
// gathers, volume term, face fluxes, lift and the RK update. The tile's stage
// input and geometry records (sY, sGF, sGI) have arrived; its RK operands sE
// (u, accumulator, snapshot: nepi of them) arrive on bar_epi with phase parity
// epi_parity. sD holds Dt, sL the negated LIFT table. The caller
// synchronises the block before the buffers are reused.
template <class C, typename T>
__device__ __forceinline__ void pipe_tile(const StageArgs<T>& a, int64_t e0, T* sY, const T* sGF, const int* sGI,
                                          const T* sE, T* sN, const T* sD, const T* sL, const short* sFm,
                                          const short* sNb, uint64_t* bar_epi, uint32_t epi_parity, int nepi, int tid,
                                          bool& ok, ResAcc<T>& racc) {
  constexpr int D = C::D, NP = C::NP, NV = C::NV, NK = C::NK;
  constexpr int NC = C::NC, NSPLIT = C::NSPLIT, ET = C::ET, RECF = C::RECF;
  const int64_t stride = a.stride;
  const T rhoc2 = (T)a.ph.rhoc2, inv_rho0 = (T)a.ph.inv_rho0, half_c0 = (T)a.ph.half_c0;
  const T dt = (T)a.dt;
  // a block larger than this shape's NT (the mixed-order kernel) leaves its
  // other threads idle in this tile; they only take part in the barriers
  const bool active = tid < C::NT;
  const int e = active ? tid / NSPLIT : 0, s = active ? tid - (tid / NSPLIT) * NSPLIT : 0;
  const int i0 = s * NC;
  // ---- neighbour traces: asynchronous gathers into sN ----
  if (active) gather_traces<C, T>(a.y_in, stride, sGI, sNb, sN, tid, e0);
  cp_async_commit();

  // ---- volume term for this thread's nodes ----
  T Lv[NC][NV];
  if (active) {
    T W[D][NC][NV];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int ii = 0; ii < NC; ++ii)
#pragma unroll
        for (int q = 0; q < NV; ++q) W[r][ii][q] = 0;
    const T* ye = sY + e * NP;
    if constexpr (std::is_same<T, float>::value && NC >= 2) {
      // FP32: the FMAs of node pairs as packed pairs (per component the
      // rounding of fmaf, the same result); an odd last node stays scalar
      constexpr int NH = NC / 2;
      float2 W2[D][NH][NV];
      float W1[D][NV];
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          W1[r][q] = 0.f;
#pragma unroll
          for (int h = 0; h < NH; ++h) W2[r][h][q] = make_float2(0.f, 0.f);
        }
#pragma unroll 4
      for (int j = 0; j < NP; ++j) {
        float yq[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) yq[q] = ye[q * ET * NP + j];
#pragma unroll
        for (int r = 0; r < D; ++r) {
          float dv[NC];
          load_chunk<float, NC, C::VW, NP>(dv, sD + (r * NP + j) * NP, i0);
#pragma unroll
          for (int h = 0; h < NH; ++h) {
            const float2 dp = make_float2(dv[2 * h], dv[2 * h + 1]);
#pragma unroll
            for (int q = 0; q < NV; ++q) W2[r][h][q] = __ffma2_rn(dp, make_float2(yq[q], yq[q]), W2[r][h][q]);
          }
          if constexpr (NC % 2 != 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) W1[r][q] += dv[NC - 1] * yq[q];
          }
        }
      }
#pragma unroll
      for (int r = 0; r < D; ++r)
#pragma unroll
        for (int q = 0; q < NV; ++q) {
#pragma unroll
          for (int h = 0; h < NH; ++h) W[r][2 * h][q] = W2[r][h][q].x, W[r][2 * h + 1][q] = W2[r][h][q].y;
          if constexpr (NC % 2 != 0) W[r][NC - 1][q] = W1[r][q];
        }
    } else {
#pragma unroll 4
      for (int j = 0; j < NP; ++j) {
        T yq[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) yq[q] = ye[q * ET * NP + j];
#pragma unroll
        for (int r = 0; r < D; ++r) {
          T dv[NC];
          load_chunk<T, NC, C::VW, NP>(dv, sD + (r * NP + j) * NP, i0);
#pragma unroll
          for (int ii = 0; ii < NC; ++ii)
#pragma unroll
            for (int q = 0; q < NV; ++q) W[r][ii][q] += dv[ii] * yq[q];
        }
      }
    }
    const T* G = sGF + e * RECF;
    T g[D][D];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
      for (int d = 0; d < D; ++d) g[r][d] = G[r * D + d];
    const T* ev0 = G + C::S::PHYS_OFF;
    T gv0[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      gv0[r] = g[r][0] * ev0[0];
      #pragma unroll
      for (int d = 1; d < D; ++d) gv0[r] += g[r][d] * ev0[d];
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
        for (int d = 0; d < D; ++d) gw += g[r][d] * W[r][ii][1 + d];
        vp += gv0[r] * W[r][ii][0] + rhoc2 * gw;
#pragma unroll
        for (int d = 0; d < D; ++d) vv[d] += gv0[r] * W[r][ii][1 + d] + g[r][d] * W[r][ii][0] * inv_rho0;
      }
      Lv[ii][0] = vp;
#pragma unroll
      for (int d = 0; d < D; ++d) Lv[ii][1 + d] = vv[d];
    }
  }
  cp_async_wait_all();
  __syncthreads();

  // ---- face numerical fluxes (in place of the gathered traces) ----
  if (active) face_fluxes<C, T>(a.bmat, sY, sGF, sGI, sFm, sNb, sN, tid, rhoc2, inv_rho0, half_c0, e0);
  __syncthreads();

  // ---- lifting (sL holds -LIFT: the products accumulate) ----
  if (active) {
    const T* hrow = sN + (size_t)e * C::SN_EL;
    if constexpr (std::is_same<T, float>::value && NC >= 2) {
      constexpr int NH = NC / 2;
      float2 L2[NH][NV];
#pragma unroll
      for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) L2[h][q] = make_float2(Lv[2 * h][q], Lv[2 * h + 1][q]);
#pragma unroll 4
      for (int k = 0; k < NK; ++k) {
        float hq[C::NVQ];
        vload<float, C::NVQ>(hq, hrow + k * C::NVQ);
        float lv[NC];
        load_chunk<float, NC, C::VW, NP>(lv, sL + k * NP, i0);
#pragma unroll
        for (int h = 0; h < NH; ++h) {
          const float2 lp = make_float2(lv[2 * h], lv[2 * h + 1]);
#pragma unroll
          for (int q = 0; q < NV; ++q) L2[h][q] = __ffma2_rn(lp, make_float2(hq[q], hq[q]), L2[h][q]);
        }
        if constexpr (NC % 2 != 0) {
#pragma unroll
          for (int q = 0; q < NV; ++q) Lv[NC - 1][q] += lv[NC - 1] * hq[q];
        }
      }
#pragma unroll
      for (int h = 0; h < NH; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) Lv[2 * h][q] = L2[h][q].x, Lv[2 * h + 1][q] = L2[h][q].y;
    } else {
#pragma unroll 4
      for (int k = 0; k < NK; ++k) {
        T hq[C::NVQ];
        vload<T, C::NVQ>(hq, hrow + k * C::NVQ);
        T lv[NC];
        load_chunk<T, NC, C::VW, NP>(lv, sL + k * NP, i0);
#pragma unroll
        for (int ii = 0; ii < NC; ++ii)
#pragma unroll
          for (int q = 0; q < NV; ++q) Lv[ii][q] += lv[ii] * hq[q];
      }
    }
  }

  if (active) curved_override<T, NC, NV, NP>(a, e0 + e, i0, Lv);
  // ---- RK update from registers (vectorised when the node chunk allows) ----
  if (nepi > 0 && ok && !mbar_wait(bar_epi, epi_parity, a.wait_limit)) ok = false;
  // after a timeout the operand buffer may still be landing: no RK update
  if (!active || !ok) return;
  rk_update_regs<T, NC, NV, C::VW, ET, NP>(a, e0, e, i0, Lv, (nepi > 0) ? sE : sY, sE,
                                           dt * sGF[e * RECF + C::S::PHYS_OFF + D], racc);
}

// Operator tables and tile body of the pipelined kernel: Dt [D][NP j][NP i]
// and the negated LIFT [NK][NP i] in shared memory, pipe_tile per tile.
struct PipeTileOps {
  template <class C, typename T>
  __device__ static void load_ops(T* sD, T* sL, const StageArgs<T>& a, int tid) {
    for (int i = tid; i < C::D * C::NP * C::NP; i += C::NT) sD[i] = a.Dt[i];
    for (int i = tid; i < C::NK * C::NP; i += C::NT) sL[i] = -a.LIFT[i];  // negated for pipe_tile's lift
  }
  template <class C, typename T>
  __device__ static void run(const StageArgs<T>& a, int64_t e0, T* sY, const T* sGF, const int* sGI, const T* sE,
                             T* sN, const T* sD, const T* sL, const short* sFm, const short* sNb, uint64_t* bar_epi,
                             uint32_t epi_parity, int nepi, int tid, bool& ok, ResAcc<T>& racc) {
    pipe_tile<C, T>(a, e0, sY, sGF, sGI, sE, sN, sD, sL, sFm, sNb, bar_epi, epi_parity, nepi, tid, ok, racc);
  }
};

// The persistent tile loop of the pipelined kernels: C gives the shape and
// the shared-memory layout (oBar, oD, oL, oFm, oNb, oY, oGF, oGI, oE, oN,
// oR), Ops the operator tables and the per-tile body.
template <class C, typename T, class Ops>
__device__ __forceinline__ void pipe_loop(const StageArgs<T>& a, int* err, unsigned char* sm) {
  constexpr int NP = C::NP, NF = C::NF, NFP = C::NFP, NV = C::NV, NPERM = C::NPERM, NK = C::NK;
  constexpr int ET = C::ET, NT = C::NT, RECF = C::RECF, RECI = C::RECI;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + C::oBar);  // [0],[1]: tile buffers, [2]: epilogue operands
  T* sD = reinterpret_cast<T*>(sm + C::oD);
  T* sL = reinterpret_cast<T*>(sm + C::oL);
  short* sFm = reinterpret_cast<short*>(sm + C::oFm);
  short* sNb = reinterpret_cast<short*>(sm + C::oNb);
  T* sYb = reinterpret_cast<T*>(sm + C::oY);
  T* sGFb = reinterpret_cast<T*>(sm + C::oGF);
  int* sGIb = reinterpret_cast<int*>(sm + C::oGI);
  T* sE = reinterpret_cast<T*>(sm + C::oE);
  T* sN = reinterpret_cast<T*>(sm + C::oN);
  double* sRed = reinterpret_cast<double*>(sm + C::oR);

  const int tid = threadIdx.x;
  const int stage = a.stage;
  const int64_t stride = a.stride;
  // epilogue operands: stage 1 reads u through the stage input, 2-3 need u and
  // acc, 4 needs u, acc and the snapshot, 5 (Euler) reads u as the input.
  const int nepi = (stage == 2 || stage == 3) ? 2 : (stage == 4 ? 3 : 0);
  const T* epi_src[3] = {a.u, a.acc, a.snap};

  auto issue_tile = [&](int tile, int b) {
    const int64_t e0 = (int64_t)tile * ET;
    mbar_expect_tx(&bar[b], NV * C::YSEG + C::GFB + C::GIB);
#pragma unroll
    for (int q = 0; q < NV; ++q)
      tma_load_1d(sYb + ((size_t)b * NV + q) * ET * NP, a.y_in + q * stride + e0 * NP, C::YSEG, &bar[b]);
    tma_load_1d(sGFb + (size_t)b * ET * RECF, a.geoF + e0 * RECF, C::GFB, &bar[b]);
    tma_load_1d(sGIb + (size_t)b * ET * RECI, a.geoI + e0 * RECI, C::GIB, &bar[b]);
  };
  auto issue_epi = [&](int tile) {
    const int64_t e0 = (int64_t)tile * ET;
    mbar_expect_tx(&bar[2], nepi * NV * C::YSEG);
    for (int k = 0; k < nepi; ++k)
#pragma unroll
      for (int q = 0; q < NV; ++q)
        tma_load_1d(sE + ((size_t)k * NV + q) * ET * NP, epi_src[k] + q * stride + e0 * NP, C::YSEG, &bar[2]);
  };

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    fence_mbar_init();
  }
  Ops::template load_ops<C, T>(sD, sL, a, tid);
  for (int i = tid; i < NK; i += NT) sFm[i] = a.fmask[i];
  for (int i = tid; i < NF * NPERM * NFP; i += NT) sNb[i] = a.nbrnode[i];
  __syncthreads();
  // thread 0: barriers whose armed phase was not yet observed complete (bit
  // i) and that phase's parity (bit 4+i); drained before the block exits
  uint32_t pend = 0;
  auto arm = [&](int i, int parity) { pend = (pend & ~(0x11u << i)) | (1u << i) | ((uint32_t)(parity & 1) << (4 + i)); };
  if (tid == 0 && (int)blockIdx.x < a.ntiles) issue_tile(blockIdx.x, 0), arm(0, 0);

  ResAcc<T> racc;
  bool ok = true;

  int it = 0;
  for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++it) {
    const int b = it & 1;
    const int64_t e0 = (int64_t)tile * ET;
    const bool got = mbar_wait(&bar[b], (it >> 1) & 1, a.wait_limit);
    if (tid == 0 && got) pend &= ~(1u << b);
    // a tile whose copy has not arrived holds no valid neighbour indices: the
    // whole block stops before anything reads them (and issues no copy)
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    T* sY = sYb + (size_t)b * NV * ET * NP;
    const T* sGF = sGFb + (size_t)b * ET * RECF;
    const int* sGI = sGIb + (size_t)b * ET * RECI;
    if (tid == 0) {
      // the other buffer and the operand buffer were released at the
      // previous tile's end
      fence_proxy_async();
      const int nt = tile + gridDim.x;
      if (nt < a.ntiles) issue_tile(nt, b ^ 1), arm(b ^ 1, (it + 1) >> 1);
      if (C::kStaged && nepi > 0) issue_epi(tile), arm(2, it);
    }
    Ops::template run<C, T>(a, e0, sY, sGF, sGI, sE, sN, sD, sL, sFm, sNb, &bar[2], (uint32_t)(it & 1), nepi, tid, ok,
                            racc);
    if (tid == 0 && ok) pend &= ~4u;  // thread 0 observed the operand copies (inside the tile)
    if (__syncthreads_or(!ok)) {      // buffers of this tile are free again
      ok = false;
      break;
    }
  }
  if (tid == 0) {
    // after a timeout: bounded waits (full limit) for the copies still in
    // flight, so that none lands in shared memory after the block has left
    for (int i = 0; i < 3; ++i)
      if (pend & (1u << i)) mbar_wait(&bar[i], (pend >> (4 + i)) & 1u);
    if (!ok) atomicOr(err, 1);
  }

  if (stage == 4) {
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


template <typename T, int D, int P, int NC_, int ET_>
__global__ void __launch_bounds__(Pipe<T, D, P, NC_, ET_>::NT) stage2_kernel(const StageArgs<T> a, int* err) {
  extern __shared__ __align__(128) unsigned char sm[];
  pipe_loop<Pipe<T, D, P, NC_, ET_>, T, PipeTileOps>(a, err, sm);
}

template <typename T, int D, int P, int NC_, int ET_>
struct Stage2 {
  using C = Pipe<T, D, P, NC_, ET_>;
  static cudaError_t launch(const StageArgs<T>& a, int grid, int* err, cudaStream_t s) {
    auto kfn = stage2_kernel<T, D, P, NC_, ET_>;
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
  static int blocks_per_sm() {
    auto kfn = stage2_kernel<T, D, P, NC_, ET_>;
    // a configuration larger than the shared memory of an SM is reported as
    // unavailable; the failed query must not leave a sticky launch error
    // the largest shared-memory carve-out, so that the occupancy query and
    // the launches see the same per-SM capacity
    if (cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)C::bytes) != cudaSuccess ||
        cudaFuncSetAttribute(kfn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
            cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kfn, C::NT, C::bytes) != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    return nb;
  }
};

}  // namespace dgk
