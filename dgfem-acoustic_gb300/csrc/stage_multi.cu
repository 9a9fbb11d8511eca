// Launcher of the mixed-order stage kernel of the batched ensemble
// (stage_multi.cuh).
#include "stage_multi.cuh"

namespace dgk {

namespace {
cudaError_t multi_attrs() {
  cudaError_t e = cudaFuncSetAttribute(stage_multi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)MultiLayout::bytes);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(stage_multi_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
  return e;
}
}  // namespace

int stage_multi_elems_per_tile(int order) {
  return order == 2 ? MultiC2::ET : order == 3 ? MultiC3::ET : order == 4 ? MultiC4::ET : 0;
}

int stage_multi_blocks_per_sm() {
  if (multi_attrs() != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stage_multi_kernel, kMultiNT, MultiLayout::bytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nb;
}

cudaError_t launch_stage_multi(const MultiArgs& m, int grid, int* err, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaError_t e = multi_attrs();
    if (e != cudaSuccess) return e;
    configured = true;
  }
  stage_multi_kernel<<<grid, kMultiNT, MultiLayout::bytes, s>>>(m, err);
  return cudaGetLastError();
}

}  // namespace dgk
