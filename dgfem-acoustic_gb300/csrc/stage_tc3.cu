// Instantiations of the warp-specialised tensor-core stage kernel (FP32
// state, stage_tc3.cuh), tetrahedra of orders 3 and 4, with 2 or 4 builder
// threads per tile row (8 or 16 builder warps). They are offered to the
// context's kernel selection as variants kTcVariant + 5 and kTcVariant + 6.
#include "stage_tc3.cuh"

namespace dgk {

cudaError_t launch_stage_tc3(int dim, int order, int npart, const StageArgs<float>& a, int grid, int* err,
                             cudaStream_t s) {
  if (dim == 3 && order == 3) {
    if (npart == 2) return StageTc3<3, 3, 2>::launch(a, grid, err, s);
    if (npart == 4) return StageTc3<3, 3, 4>::launch(a, grid, err, s);
  }
  if (dim == 3 && order == 4) {
    if (npart == 2) return StageTc3<3, 4, 2>::launch(a, grid, err, s);
    if (npart == 4) return StageTc3<3, 4, 4>::launch(a, grid, err, s);
  }
  return cudaErrorInvalidValue;
}

template <int D, int P, int NPART>
static Stage2Info tc3_info() {
  using C = Tc3Cfg<D, P, NPART>;
  return Stage2Info{C::NP, C::ET, C::NTHREADS, (int)C::launch_bytes, StageTc3<D, P, NPART>::blocks_per_sm(), 1};
}

Stage2Info stage_tc3_info(int dim, int order, int npart) {
  if (dim == 3 && order == 3) return npart == 2 ? tc3_info<3, 3, 2>() : tc3_info<3, 3, 4>();
  if (dim == 3 && order == 4) return npart == 2 ? tc3_info<3, 4, 2>() : tc3_info<3, 4, 4>();
  return Stage2Info{0, 0, 0, 0, 0, 0};
}

}  // namespace dgk
