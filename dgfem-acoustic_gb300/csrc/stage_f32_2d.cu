// Instantiations of the fused stage kernels: float, 2-D, orders 1..4.
// Generated variant table: (nodes per thread NC, elements per tile ET).
#include "stage.cuh"
#include "stage2.cuh"

namespace dgk {

cudaError_t launch_stage_f32_2d(int order, const StageArgs<float>& a, int grid, cudaStream_t s) {
  switch (order) {
    case 1: return launch_stage_impl<float, 2, 1>(a, grid, s);
    case 2: return launch_stage_impl<float, 2, 2>(a, grid, s);
    case 3: return launch_stage_impl<float, 2, 3>(a, grid, s);
    case 4: return launch_stage_impl<float, 2, 4>(a, grid, s);
  }
  return cudaErrorInvalidValue;
}

int blocks_per_sm_f32_2d(int order) {
  switch (order) {
    case 1: return blocks_per_sm_impl<float, 2, 1>();
    case 2: return blocks_per_sm_impl<float, 2, 2>();
    case 3: return blocks_per_sm_impl<float, 2, 3>();
    case 4: return blocks_per_sm_impl<float, 2, 4>();
  }
  return 1;
}

cudaError_t launch_stage2_f32_2d(int order, int variant, const StageArgs<float>& a, int grid, int* err, cudaStream_t s) {
  if (order == 1 && variant == 0) return Stage2<float, 2, 1, 3, 128>::launch(a, grid, err, s);
  if (order == 2 && variant == 0) return Stage2<float, 2, 2, 6, 128>::launch(a, grid, err, s);
  if (order == 2 && variant == 1) return Stage2<float, 2, 2, 3, 64>::launch(a, grid, err, s);
  if (order == 3 && variant == 0) return Stage2<float, 2, 3, 5, 64>::launch(a, grid, err, s);
  if (order == 3 && variant == 1) return Stage2<float, 2, 3, 4, 32>::launch(a, grid, err, s);
  if (order == 3 && variant == 2) return Stage2<float, 2, 3, 2, 32>::launch(a, grid, err, s);
  if (order == 4 && variant == 0) return Stage2<float, 2, 4, 5, 32>::launch(a, grid, err, s);
  if (order == 4 && variant == 1) return Stage2<float, 2, 4, 4, 32>::launch(a, grid, err, s);
  return cudaErrorInvalidValue;
}

Stage2Info stage2_info_f32_2d(int order, int variant) {
  if (order == 1 && variant == 0) { using C = Pipe<float, 2, 1, 3, 128>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 1, 3, 128>::blocks_per_sm(), 1}; }
  if (order == 2 && variant == 0) { using C = Pipe<float, 2, 2, 6, 128>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 2, 6, 128>::blocks_per_sm(), 2}; }
  if (order == 2 && variant == 1) { using C = Pipe<float, 2, 2, 3, 64>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 2, 3, 64>::blocks_per_sm(), 2}; }
  if (order == 3 && variant == 0) { using C = Pipe<float, 2, 3, 5, 64>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 3, 5, 64>::blocks_per_sm(), 3}; }
  if (order == 3 && variant == 1) { using C = Pipe<float, 2, 3, 4, 32>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 3, 4, 32>::blocks_per_sm(), 3}; }
  if (order == 3 && variant == 2) { using C = Pipe<float, 2, 3, 2, 32>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 3, 2, 32>::blocks_per_sm(), 3}; }
  if (order == 4 && variant == 0) { using C = Pipe<float, 2, 4, 5, 32>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 4, 5, 32>::blocks_per_sm(), 2}; }
  if (order == 4 && variant == 1) { using C = Pipe<float, 2, 4, 4, 32>; return Stage2Info{C::NC, C::ET, C::NT, (int)C::bytes, Stage2<float, 2, 4, 4, 32>::blocks_per_sm(), 2}; }
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
