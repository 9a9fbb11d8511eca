// Instantiations of the tensor-core stage kernel (FP32 state), 2-D and 3-D,
// orders 1..4. It is offered to the context's kernel selection as variant
// kTcVariant next to the CUDA-core variants.
#include "stage_tc.cuh"

namespace dgk {

#define DGK_TC_CASES(X) X(2, 1) X(2, 2) X(2, 3) X(2, 4) X(3, 1) X(3, 2) X(3, 3) X(3, 4)

cudaError_t launch_stage_tc(int dim, int order, const StageArgs<float>& a, int grid, int* err, cudaStream_t s) {
#define DGK_TC_LAUNCH(D, P) \
  if (dim == D && order == P) return StageTc<D, P>::launch(a, grid, err, s);
  DGK_TC_CASES(DGK_TC_LAUNCH)
#undef DGK_TC_LAUNCH
  return cudaErrorInvalidValue;
}

Stage2Info stage_tc_info(int dim, int order) {
#define DGK_TC_INFO(D, P)                                                                                     \
  if (dim == D && order == P) {                                                                               \
    using C = TcCfg<D, P>;                                                                                    \
    return Stage2Info{C::NP, C::ET, C::NT, (int)C::bytes, StageTc<D, P>::blocks_per_sm(), 1};                 \
  }
  DGK_TC_CASES(DGK_TC_INFO)
#undef DGK_TC_INFO
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
