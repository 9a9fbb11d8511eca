// Instantiations of the tensor-core stage kernel (FP32 state), 2-D and 3-D,
// orders 1..4, with 2, 4 or 8 threads per tile row (256, 512 or 1024 threads
// per block). They are offered to the context's kernel selection as variants
// kTcVariant .. kTcVariant + 2 next to the CUDA-core variants.
#include "stage_tc.cuh"

namespace dgk {

#define DGK_TC_CASES(X) X(2, 1) X(2, 2) X(2, 3) X(2, 4) X(3, 1) X(3, 2) X(3, 3) X(3, 4)

cudaError_t launch_stage_tc(int dim, int order, int npart, const StageArgs<float>& a, int grid, int* err,
                            cudaStream_t s) {
#define DGK_TC_LAUNCH(D, P)                                                  \
  if (dim == D && order == P)                                                \
    return npart == 8   ? StageTc<D, P, 8>::launch(a, grid, err, s)          \
           : npart == 4 ? StageTc<D, P, 4>::launch(a, grid, err, s)          \
           : npart == 2 ? StageTc<D, P, 2>::launch(a, grid, err, s) : cudaErrorInvalidValue;
  DGK_TC_CASES(DGK_TC_LAUNCH)
#undef DGK_TC_LAUNCH
  return cudaErrorInvalidValue;
}

template <int D, int P, int NPART>
static Stage2Info tc_info() {
  using C = TcCfg<D, P, NPART>;
  return Stage2Info{C::NP, C::ET, C::NT, (int)C::bytes, StageTc<D, P, NPART>::blocks_per_sm(), 1};
}

Stage2Info stage_tc_info(int dim, int order, int npart) {
#define DGK_TC_INFO(D, P)                                         \
  if (dim == D && order == P) {                                   \
    if (npart == 2) return tc_info<D, P, 2>();                    \
    if (npart == 4) return tc_info<D, P, 4>();                    \
    if (npart == 8) return tc_info<D, P, 8>();                    \
  }
  DGK_TC_CASES(DGK_TC_INFO)
#undef DGK_TC_INFO
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
