// Internal declarations shared by the CUDA translation units of the solver.
//
// Device data layout (all per-element arrays padded to Epad = tiles * ET):
//   state   T [n_var][Epad*Np]  per variable, element-major, internal lattice
//                               node order inside an element
//   geoF    T [Epad][RECF]      G = d(xi)/dx (dim*dim), then per local face:
//                               outward unit normal (dim) and sJ = J_f/|det J|,
//                               then the element's mean flow v0 (dim) and its
//                               time-step scale (1 for a single run; the
//                               instance's dt in a batch)
//   geoI    int [Epad][RECI]    per local face: neighbour element (interior)
//                               or boundary-face index; then per local face the
//                               face code (neighbour local face, corner
//                               permutation, penalty sign, boundary flag)
//   bmat    T [n_bfaces][n_var*n_var]  boundary flux matrix (RKR or reflecting)
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace dgk {

// Polling rounds of a bounded device wait (mbarrier try_wait) before it
// gives up and the kernel reports DG_ERR_TIMEOUT.
constexpr int kWaitRounds = 1 << 20;
// Suspend-time hint of each polling round (ns): a waiting thread sleeps until
// the phase completes or this time has passed, instead of spinning and taking
// issue slots from the warps that work; a wait ends after at most
// kWaitRounds x kWaitHintNs (about a second).
constexpr uint32_t kWaitHintNs = 1000;

constexpr int kCodeLfMask = 0x3;       // neighbour local face
constexpr int kCodePermShift = 2;      // corner permutation index (3 bits)
constexpr int kCodePermMask = 0x7;
constexpr int kCodeNegPenalty = 1 << 5;  // penalty sign s_f = -1
constexpr int kCodeBoundary = 1 << 6;    // boundary face; nbr slot holds the boundary index

// Compile-time shape of a (dim, order) pair.
template <int D, int P>
struct Shape {
  static constexpr int NP = D == 1 ? P + 1 : D == 2 ? (P + 1) * (P + 2) / 2 : (P + 1) * (P + 2) * (P + 3) / 6;
  static constexpr int NF = D + 1;
  static constexpr int NFP = D == 1 ? 1 : D == 2 ? P + 1 : (P + 1) * (P + 2) / 2;
  static constexpr int NV = D + 1;
  static constexpr int NPERM = D == 1 ? 1 : D == 2 ? 2 : 6;
  // threads per element: each owns a chunk of NC output nodes
  static constexpr int NCMAX = D == 2 ? 6 : 5;
  static constexpr int NSPLIT = (NP + NCMAX - 1) / NCMAX;
  static constexpr int NC = (NP + NSPLIT - 1) / NSPLIT;
  // elements per tile: a multiple of 4 (16-byte tile boundaries) with
  // ET * NSPLIT a multiple of the warp size
  static constexpr int ET = NSPLIT <= 2 ? 128 / NSPLIT : 32;
  static constexpr int NT = ET * NSPLIT;  // threads per block
  static constexpr int PHYS_OFF = D * D + NF * (D + 1);  // v0 (D), dt scale
  static constexpr int RECF_RAW = PHYS_OFF + D + 1;
  static constexpr int RECI = ((2 * NF) + 3) / 4 * 4;
};

template <int D, int P, typename T>
struct ShapeT : Shape<D, P> {
  static constexpr int VEC = 16 / sizeof(T);
  static constexpr int RECF = (Shape<D, P>::RECF_RAW + VEC - 1) / VEC * VEC;
};

// Residual partial sums of one thread: mean over the state of
// (snapshot - u)^2 for p, p/c0^2 and the velocity components
// (src/solver.cpp:518-545). FP64 states follow the reference's formula in
// FP64. FP32 states square the FP32 differences and sum them in FP32 (GB300's
// FP64 rate made this diagnostic the most expensive part of the last RK
// stage); the density sum is p's sum / c0^4, the same quantity in exact
// arithmetic. The block reduction that follows is in FP64.
template <typename T>
struct ResAcc;
template <>
struct ResAcc<double> {
  double r[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  __device__ __forceinline__ void add(int q, double s, double u, double c0sq) {
    const double dn = s - u;
    if (q == 0) {
      r[0] += dn * dn;
      const double dr = s / c0sq - u / c0sq;
      r[1] += dr * dr;
    } else if (q == 1) {
      r[2] += dn * dn;
    } else if (q == 2) {
      r[3] += dn * dn;
    } else {
      r[4] += dn * dn;
    }
  }
  __device__ __forceinline__ double get(int c, double) const { return r[c]; }
};
template <>
struct ResAcc<float> {
  float r[4] = {0.f, 0.f, 0.f, 0.f};  // p, vx, vy, vz
  __device__ __forceinline__ void add(int q, float s, float u, double) {
    const float dn = s - u;
    if (q == 0)
      r[0] = fmaf(dn, dn, r[0]);
    else if (q == 1)
      r[1] = fmaf(dn, dn, r[1]);
    else if (q == 2)
      r[2] = fmaf(dn, dn, r[2]);
    else
      r[3] = fmaf(dn, dn, r[3]);
  }
  __device__ __forceinline__ double get(int c, double c0sq) const {
    return c == 0 ? (double)r[0] : c == 1 ? (double)r[0] / (c0sq * c0sq) : (double)r[c - 1];
  }
};

// The RK4 combine's division by 6 (src/solver.cpp:509-516): FP64 divides,
// as the reference does; FP32 multiplies by the FP32 reciprocal (within an
// ulp of the division, without the division's instruction sequence, which
// made the last stage the slowest).
__device__ __forceinline__ double rk4_sixth(double x) { return x / 6.0; }
__device__ __forceinline__ float rk4_sixth(float x) { return x * (1.0f / 6.0f); }

// Physical constants used by the kernels.
struct Phys {
  double v0[3];
  double rho0, c0, rhoc2, inv_rho0, half_c0;
};

template <typename T>
struct StageArgs {
  const T* y_in;   // stage input
  T* y_out;        // next stage input (stages 1-3)
  T* u;            // state at step start (updated in stage 4)
  T* acc;          // RK accumulator
  const T* snap;   // residual reference (stage 4)
  T* k_out;        // stage 0: dt*L(y_in)
  double* partials;  // [gridDim][5] residual partial sums (stage 4)
  const T* geoF;
  const int* geoI;
  const T* bmat;
  const T* Dt;     // [D][NP(j)][NP(i)]
  const T* LIFT;   // [NF*NFP(k)][NP(i)]
  const short* fmask;   // [NF*NFP]
  const short* nbrnode; // [NF*NPERM*NFP]
  int64_t stride;  // Epad*NP
  // curved elements: per element its slot in crhs (-1: straight-sided); null
  // when the mesh has none. crhs [NV][cstride] holds M^-T (S - F) of the
  // curved elements (curved.cu), computed before the stage kernel runs.
  const int* cslot;
  const T* crhs;
  int64_t cstride;  // ncurved*NP
  int ntiles;
  int stage;       // 0: k only, 1..4: RK4 stages, 5: Euler (y_out = u + k)
  int wait_limit;  // polling rounds of a bounded device wait before it gives up
  double dt;
  double c0sq;
  Phys ph;
  // FP32 copies of rho0 c0^2, 1/rho0, c0/2 and dt (rounded once on the host,
  // so that FP32 kernels convert nothing per tile)
  float f_rhoc2, f_inv_rho0, f_half_c0, f_dt;
};

// The stage kernels' operator result Lv of this thread's node chunk is
// replaced by the curved-element right-hand side where the element is
// curved.
template <typename T, int NC, int NV, int NP>
__device__ __forceinline__ void curved_override(const StageArgs<T>& a, int64_t el, int i0, T (&Lv)[NC][NV]) {
  if (a.cslot == nullptr) return;
  const int cs = a.cslot[el];
  if (cs < 0) return;
  const T* r = a.crhs + (int64_t)cs * NP;
#pragma unroll
  for (int ii = 0; ii < NC; ++ii)
    if (i0 + ii < NP)
#pragma unroll
      for (int q = 0; q < NV; ++q) Lv[ii][q] = r[q * a.cstride + i0 + ii];
}

// Stage launchers and occupancy queries; defined in stage_{f32,f64}_{2,3}d.cu.
cudaError_t launch_stage_f32_2d(int order, const StageArgs<float>& a, int grid, cudaStream_t s);
cudaError_t launch_stage_f32_3d(int order, const StageArgs<float>& a, int grid, cudaStream_t s);
cudaError_t launch_stage_f64_2d(int order, const StageArgs<double>& a, int grid, cudaStream_t s);
cudaError_t launch_stage_f64_3d(int order, const StageArgs<double>& a, int grid, cudaStream_t s);
int blocks_per_sm_f32_2d(int order);
int blocks_per_sm_f32_3d(int order);
int blocks_per_sm_f64_2d(int order);
int blocks_per_sm_f64_3d(int order);

// Pipelined stage kernel (stage2.cuh): variants differ in nodes per thread
// and elements per tile; the context picks one by timing (autotuning).
struct Stage2Info {
  int nc, et, nt, smem_bytes, blocks_per_sm, n_variants;
};
cudaError_t launch_stage2_f32_2d(int order, int variant, const StageArgs<float>& a, int grid, int* err, cudaStream_t s);
cudaError_t launch_stage2_f32_3d(int order, int variant, const StageArgs<float>& a, int grid, int* err, cudaStream_t s);
cudaError_t launch_stage2_f64_2d(int order, int variant, const StageArgs<double>& a, int grid, int* err, cudaStream_t s);
cudaError_t launch_stage2_f64_3d(int order, int variant, const StageArgs<double>& a, int grid, int* err, cudaStream_t s);
Stage2Info stage2_info_f32_2d(int order, int variant);
Stage2Info stage2_info_f32_3d(int order, int variant);
Stage2Info stage2_info_f64_2d(int order, int variant);
Stage2Info stage2_info_f64_3d(int order, int variant);
// 1-D (line elements, stage_1d.cu): the same families for both precisions.
cudaError_t launch_stage_f32_1d(int order, const StageArgs<float>& a, int grid, cudaStream_t s);
cudaError_t launch_stage_f64_1d(int order, const StageArgs<double>& a, int grid, cudaStream_t s);
int blocks_per_sm_f32_1d(int order);
int blocks_per_sm_f64_1d(int order);
cudaError_t launch_stage2_f32_1d(int order, int variant, const StageArgs<float>& a, int grid, int* err, cudaStream_t s);
cudaError_t launch_stage2_f64_1d(int order, int variant, const StageArgs<double>& a, int grid, int* err, cudaStream_t s);
Stage2Info stage2_info_f32_1d(int order, int variant);
Stage2Info stage2_info_f64_1d(int order, int variant);
// Tensor-core stage kernels (FP32 state only): variant ids kTcVariant,
// kTcVariant + 1, kTcVariant + 2 of the context's kernel selection are the
// one-chunk kernel (stage_tc.cuh; 2, 4 or 8 threads per tile row: 256, 512 or
// 1024 per block), kTcVariant + 3 and kTcVariant + 4 the two-chunk kernel
// (stage_tc2.cuh, two blocks per SM; 2 or 4 threads per tile row),
// kTcVariant + 5 and kTcVariant + 6 the warp-specialised kernel
// (stage_tc3.cuh; 2 or 4 builder threads per tile row).
constexpr int kTcVariant = 16;
constexpr int kTcVariants = 7;
inline bool is_tc_variant(int v) { return v >= kTcVariant && v < kTcVariant + kTcVariants; }
inline bool is_tc2_variant(int v) { return v >= kTcVariant + 3 && v < kTcVariant + 5; }
inline bool is_tc3_variant(int v) { return v >= kTcVariant + 5 && v < kTcVariant + 7; }
inline int tc_npart(int v) {
  return is_tc3_variant(v) ? 2 << (v - kTcVariant - 5) : is_tc2_variant(v) ? 2 << (v - kTcVariant - 3) : 2 << (v - kTcVariant);
}
cudaError_t launch_stage_tc(int dim, int order, int npart, const StageArgs<float>& a, int grid, int* err,
                            cudaStream_t s);
Stage2Info stage_tc_info(int dim, int order, int npart);
cudaError_t launch_stage_tc2(int dim, int order, int npart, const StageArgs<float>& a, int grid, int* err,
                             cudaStream_t s);
Stage2Info stage_tc2_info(int dim, int order, int npart);
// Warp-specialised tensor-core kernel (stage_tc3.cuh, tetrahedra of orders 3
// and 4, one block per SM): variants kTcVariant + 5 and kTcVariant + 6 (2 or
// 4 builder threads per tile row).
cudaError_t launch_stage_tc3(int dim, int order, int npart, const StageArgs<float>& a, int grid, int* err,
                             cudaStream_t s);
Stage2Info stage_tc3_info(int dim, int order, int npart);
// Constant-operator stage kernel (stage3.cuh, FP32 state only): variant ids
// kStage3Variant + k of the context's kernel selection; the operators are
// uploaded to constant memory once per device and element type.
constexpr int kStage3Variant = 32;
cudaError_t stage3_upload_ops(int dim, int order, const float* Dt, const float* LIFT);
cudaError_t launch_stage3(int dim, int order, int variant, const StageArgs<float>& a, int grid, int* err,
                          cudaStream_t s);
Stage2Info stage3_info(int dim, int order, int variant);
// Wide-chunk stage kernel (stage4.cuh, FP32 state): variant ids
// kWideVariant + k of the context's kernel selection.
constexpr int kWideVariant = 48;
inline bool is_stage3_variant(int v) { return v >= kStage3Variant && v < kWideVariant; }
inline bool is_wide_variant(int v) { return v >= kWideVariant && v < kWideVariant + 16; }
cudaError_t launch_stage4(int dim, int order, int variant, const StageArgs<float>& a, int grid, int* err,
                          cudaStream_t s);
Stage2Info stage4_info(int dim, int order, int variant);
// Mixed-order stage kernel of the batched ensemble (stage_multi.cuh): 2-D,
// FP32, orders 2-4, one launch per RK stage over every order's tiles.
// Per-launch description: one StageArgs per order slot (slot k holds order
// k + 2; ntiles 0 for an order the batch does not hold, stage set in every
// slot) and the work-queue counter of the launch (zero when it starts).
constexpr int kMultiOrders = 3;
struct MultiArgs {
  StageArgs<float> g[kMultiOrders];
  int ntiles_total;
  unsigned* queue;
  int wait_limit;  // polling rounds of a bounded wait for a work item's copies
};
int stage_multi_elems_per_tile(int order);
int stage_multi_blocks_per_sm();
cudaError_t launch_stage_multi(const MultiArgs& m, int grid, int* err, cudaStream_t s);
// element padding: every tile size divides this
constexpr int kElemAlign = 128;

// Host-side shape queries for a runtime (dim, order).
struct ShapeInfo {
  int np, nf, nfp, nv, nperm, et, nt, recf32, recf64, reci;
};
inline ShapeInfo shape_info(int dim, int order) {
#define DGK_SHAPE(D, P)                                                                                  \
  if (dim == D && order == P)                                                                            \
    return ShapeInfo{Shape<D, P>::NP,     Shape<D, P>::NF,     Shape<D, P>::NFP,           Shape<D, P>::NV, \
                     Shape<D, P>::NPERM,  Shape<D, P>::ET,     Shape<D, P>::NT,            ShapeT<D, P, float>::RECF, \
                     ShapeT<D, P, double>::RECF, Shape<D, P>::RECI};
  DGK_SHAPE(1, 1) DGK_SHAPE(1, 2) DGK_SHAPE(1, 3) DGK_SHAPE(1, 4)
  DGK_SHAPE(2, 1) DGK_SHAPE(2, 2) DGK_SHAPE(2, 3) DGK_SHAPE(2, 4)
  DGK_SHAPE(3, 1) DGK_SHAPE(3, 2) DGK_SHAPE(3, 3) DGK_SHAPE(3, 4)
#undef DGK_SHAPE
  return ShapeInfo{0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
