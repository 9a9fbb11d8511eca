// Instantiations of the wide-chunk stage kernel (stage4.cuh; FP32 state,
// triangles of orders 1..4, tetrahedra of orders 3 and 4). Variants (nodes per thread NC, elements per
// tile ET, volume form, operand staging) are offered to the context's kernel
// selection as kWideVariant + k.
#include "stage4.cuh"

namespace dgk {

namespace {
// per (dim, order): candidate (NC, ET, volume form, operands staged); form
// W2 is the W form with two elements per thread
constexpr int F = kFluxForm, W = kWForm, W2 = kWForm2;
#define DGK_S4_VARIANTS(X)                                                                            \
  X(2, 1, 4, 128, W, false) X(2, 1, 4, 128, F, true)                                                  \
  X(2, 2, 6, 64, W, false) X(2, 2, 6, 64, F, false) X(2, 2, 6, 64, F, true) X(2, 2, 6, 128, W, false)   \
  X(2, 2, 4, 64, W, false)                                                                            \
  X(2, 3, 6, 32, W, false) X(2, 3, 6, 32, F, false) X(2, 3, 6, 32, F, true) X(2, 3, 6, 64, W, false)    \
  X(2, 3, 4, 32, W, false) X(2, 3, 10, 64, W, false)                                                  \
  X(2, 4, 8, 32, W, false) X(2, 4, 8, 32, F, false) X(2, 4, 8, 32, F, true) X(2, 4, 8, 64, W, false)    \
  X(2, 4, 4, 32, W, false) X(2, 4, 6, 32, W, false)                                                   \
  X(3, 3, 2, 32, W, false) X(3, 3, 4, 32, W, false) X(3, 3, 4, 32, F, false) X(3, 3, 2, 32, W2, false)  \
  X(3, 4, 6, 32, W, false) X(3, 4, 4, 32, W, false)
}  // namespace

cudaError_t launch_stage4(int dim, int order, int variant, const StageArgs<float>& a, int grid, int* err,
                          cudaStream_t s) {
  int k = 0;
#define DGK_S4_LAUNCH(DD, PP, CC, EE, FF, SS)                                          \
  if (dim == DD && order == PP) {                                                      \
    if (k == variant) return Stage4<DD, PP, CC, EE, FF, SS>::launch(a, grid, err, s); \
    ++k;                                                                               \
  }
  DGK_S4_VARIANTS(DGK_S4_LAUNCH)
#undef DGK_S4_LAUNCH
  return cudaErrorInvalidValue;
}

Stage2Info stage4_info(int dim, int order, int variant) {
  int k = 0, n = 0;
#define DGK_S4_COUNT(DD, PP, CC, EE, FF, SS) \
  if (dim == DD && order == PP) ++n;
  DGK_S4_VARIANTS(DGK_S4_COUNT)
#undef DGK_S4_COUNT
#define DGK_S4_INFO(DD, PP, CC, EE, FF, SS)                                                   \
  if (dim == DD && order == PP) {                                                            \
    if (k == variant) {                                                                      \
      using Cf = typename Stage4Sel<DD, PP, CC, EE, FF, SS>::C;                              \
      return Stage2Info{Cf::NC, Cf::ET, Cf::NT, (int)Cf::bytes,                              \
                        Stage4<DD, PP, CC, EE, FF, SS>::blocks_per_sm(), n};                 \
    }                                                                                        \
    ++k;                                                                                     \
  }
  DGK_S4_VARIANTS(DGK_S4_INFO)
#undef DGK_S4_INFO
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
