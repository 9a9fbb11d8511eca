// Instantiations of the stage kernels for 1-D line meshes, FP32 and FP64,
// orders 1..4: the baseline kernel and one pipelined variant (all Np nodes of
// an element in one thread, 128 elements per tile).
#include "stage.cuh"
#include "stage2.cuh"

namespace dgk {

#define DGK_1D_ORDERS(X) X(1) X(2) X(3) X(4)

cudaError_t launch_stage_f32_1d(int order, const StageArgs<float>& a, int grid, cudaStream_t s) {
#define X(P) \
  if (order == P) return launch_stage_impl<float, 1, P>(a, grid, s);
  DGK_1D_ORDERS(X)
#undef X
  return cudaErrorInvalidValue;
}
cudaError_t launch_stage_f64_1d(int order, const StageArgs<double>& a, int grid, cudaStream_t s) {
#define X(P) \
  if (order == P) return launch_stage_impl<double, 1, P>(a, grid, s);
  DGK_1D_ORDERS(X)
#undef X
  return cudaErrorInvalidValue;
}
int blocks_per_sm_f32_1d(int order) {
#define X(P) \
  if (order == P) return blocks_per_sm_impl<float, 1, P>();
  DGK_1D_ORDERS(X)
#undef X
  return 1;
}
int blocks_per_sm_f64_1d(int order) {
#define X(P) \
  if (order == P) return blocks_per_sm_impl<double, 1, P>();
  DGK_1D_ORDERS(X)
#undef X
  return 1;
}
cudaError_t launch_stage2_f32_1d(int order, int variant, const StageArgs<float>& a, int grid, int* err, cudaStream_t s) {
#define X(P) \
  if (order == P && variant == 0) return Stage2<float, 1, P, P + 1, 128>::launch(a, grid, err, s);
  DGK_1D_ORDERS(X)
#undef X
  return cudaErrorInvalidValue;
}
cudaError_t launch_stage2_f64_1d(int order, int variant, const StageArgs<double>& a, int grid, int* err,
                                 cudaStream_t s) {
#define X(P) \
  if (order == P && variant == 0) return Stage2<double, 1, P, P + 1, 128>::launch(a, grid, err, s);
  DGK_1D_ORDERS(X)
#undef X
  return cudaErrorInvalidValue;
}
template <typename T, int P>
static Stage2Info info_1d() {
  using C = Pipe<T, 1, P, P + 1, 128>;
  return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<T, 1, P, P + 1, 128>::blocks_per_sm(), 1};
}
Stage2Info stage2_info_f32_1d(int order, int variant) {
#define X(P) \
  if (order == P && variant == 0) return info_1d<float, P>();
  DGK_1D_ORDERS(X)
#undef X
  return Stage2Info{0, 0, 0, 0, 0, 0};
}
Stage2Info stage2_info_f64_1d(int order, int variant) {
#define X(P) \
  if (order == P && variant == 0) return info_1d<double, P>();
  DGK_1D_ORDERS(X)
#undef X
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
