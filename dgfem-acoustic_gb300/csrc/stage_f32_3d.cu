// Instantiations of the fused stage kernel: float, 3-D, orders 1..4.
#include "stage.cuh"

namespace dgk {

cudaError_t launch_stage_f32_3d(int order, const StageArgs<float>& a, int grid, cudaStream_t s) {
  switch (order) {
    case 1: return launch_stage_impl<float, 3, 1>(a, grid, s);
    case 2: return launch_stage_impl<float, 3, 2>(a, grid, s);
    case 3: return launch_stage_impl<float, 3, 3>(a, grid, s);
    case 4: return launch_stage_impl<float, 3, 4>(a, grid, s);
  }
  return cudaErrorInvalidValue;
}

int blocks_per_sm_f32_3d(int order) {
  switch (order) {
    case 1: return blocks_per_sm_impl<float, 3, 1>();
    case 2: return blocks_per_sm_impl<float, 3, 2>();
    case 3: return blocks_per_sm_impl<float, 3, 3>();
    case 4: return blocks_per_sm_impl<float, 3, 4>();
  }
  return 1;
}

}  // namespace dgk
