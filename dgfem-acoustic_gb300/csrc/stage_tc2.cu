// Instantiations of the two-chunk tensor-core stage kernel (FP32 state,
// stage_tc2.cuh), 2-D and 3-D, orders 1..4, with 2 or 4 threads per tile row
// (256 or 512 threads per block). They are offered to the context's kernel
// selection as variants kTcVariant + 3 and kTcVariant + 4.
#include "stage_tc2.cuh"

namespace dgk {

#define DGK_TC_CASES(X) X(2, 1) X(2, 2) X(2, 3) X(2, 4) X(3, 1) X(3, 2) X(3, 3) X(3, 4)

cudaError_t launch_stage_tc2(int dim, int order, int npart, const StageArgs<float>& a, int grid, int* err,
                             cudaStream_t s) {
#define DGK_TC2_LAUNCH(D, P)                                                 \
  if (dim == D && order == P)                                                \
    return npart == 4   ? StageTc2<D, P, 4>::launch(a, grid, err, s)         \
           : npart == 2 ? StageTc2<D, P, 2>::launch(a, grid, err, s) : cudaErrorInvalidValue;
  DGK_TC_CASES(DGK_TC2_LAUNCH)
#undef DGK_TC2_LAUNCH
  return cudaErrorInvalidValue;
}

template <int D, int P, int NPART>
static Stage2Info tc2_info() {
  using C = Tc2Cfg<D, P, NPART>;
  return Stage2Info{C::NP, C::ET, C::NT, (int)C::bytes, StageTc2<D, P, NPART>::blocks_per_sm(), 1};
}

Stage2Info stage_tc2_info(int dim, int order, int npart) {
#define DGK_TC2_INFO(D, P)                                        \
  if (dim == D && order == P) {                                   \
    if (npart == 2) return tc2_info<D, P, 2>();                   \
    if (npart == 4) return tc2_info<D, P, 4>();                   \
  }
  DGK_TC_CASES(DGK_TC2_INFO)
#undef DGK_TC2_INFO
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
