// Instantiations of the constant-operator stage kernel (FP32 state), 2-D and
// 3-D, orders 1..4, and the upload of the reference operators into constant
// memory. Variants (nodes per thread NC, groups of 32 elements per tile EG)
// are offered to the context's kernel selection as kStage3Variant + k.
#include <mutex>

#include "stage3.cuh"

namespace dgk {

namespace {
struct V3 {
  int nc, eg;
};
// per (dim, order): candidate (NC, EG)
#define DGK_S3_VARIANTS(X)                                   \
  X(2, 1, 3, 4) X(2, 1, 3, 2)                               \
  X(2, 2, 6, 4) X(2, 2, 3, 4) X(2, 2, 6, 2)                 \
  X(2, 3, 5, 2) X(2, 3, 5, 4) X(2, 3, 4, 2)                 \
  X(2, 4, 5, 2) X(2, 4, 5, 1) X(2, 4, 8, 2)                 \
  X(3, 1, 4, 2) X(3, 1, 2, 2)                               \
  X(3, 2, 5, 2) X(3, 2, 5, 1)                               \
  X(3, 3, 5, 1) X(3, 3, 5, 2) X(3, 3, 7, 1)                 \
  X(3, 4, 5, 1) X(3, 4, 7, 1)

std::mutex g_mu;
bool g_loaded[64][8] = {};  // per device, per (dim, order) slot
}  // namespace

cudaError_t stage3_upload_ops(int dim, int order, const float* Dt, const float* LIFT) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || order < 1 || order > 4 || (dim != 2 && dim != 3)) return cudaErrorInvalidValue;
  const int slot = (dim - 2) * 4 + order - 1;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_loaded[dev][slot]) return cudaSuccess;
  int off = 0, np = 0, nk = 0;
#define DGK_S3_OFF(D, P)                                               \
  if (dim == D && order == P) {                                       \
    off = COpsOff<D, P>::v, np = Shape<D, P>::NP, nk = Shape<D, P>::NF * Shape<D, P>::NFP; \
  }
  DGK_S3_OFF(2, 1) DGK_S3_OFF(2, 2) DGK_S3_OFF(2, 3) DGK_S3_OFF(2, 4)
  DGK_S3_OFF(3, 1) DGK_S3_OFF(3, 2) DGK_S3_OFF(3, 3) DGK_S3_OFF(3, 4)
#undef DGK_S3_OFF
  e = cudaMemcpyToSymbol(c_ops, Dt, sizeof(float) * dim * np * np, sizeof(float) * off);
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbol(c_ops, LIFT, sizeof(float) * nk * np, sizeof(float) * (off + dim * np * np));
  if (e == cudaSuccess) g_loaded[dev][slot] = true;
  return e;
}

cudaError_t launch_stage3(int dim, int order, int variant, const StageArgs<float>& a, int grid, int* err,
                          cudaStream_t s) {
  int k = 0;
#define DGK_S3_LAUNCH(DD, PP, CC, GG)                                                \
  if (dim == DD && order == PP) {                                                    \
    if (k == variant) return Stage3<DD, PP, CC, GG>::launch(a, grid, err, s);       \
    ++k;                                                                             \
  }
  DGK_S3_VARIANTS(DGK_S3_LAUNCH)
#undef DGK_S3_LAUNCH
  return cudaErrorInvalidValue;
}

Stage2Info stage3_info(int dim, int order, int variant) {
  int k = 0, n = 0;
#define DGK_S3_COUNT(DD, PP, CC, GG) \
  if (dim == DD && order == PP) ++n;
  DGK_S3_VARIANTS(DGK_S3_COUNT)
#undef DGK_S3_COUNT
#define DGK_S3_INFO(DD, PP, CC, GG)                                                                         \
  if (dim == DD && order == PP) {                                                                          \
    if (k == variant) {                                                                                    \
      using Cf = C3Cfg<DD, PP, CC, GG>;                                                                    \
      return Stage2Info{Cf::NC, Cf::ET, Cf::NT, (int)Cf::bytes, Stage3<DD, PP, CC, GG>::blocks_per_sm(), n}; \
    }                                                                                                      \
    ++k;                                                                                                   \
  }
  DGK_S3_VARIANTS(DGK_S3_INFO)
#undef DGK_S3_INFO
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
