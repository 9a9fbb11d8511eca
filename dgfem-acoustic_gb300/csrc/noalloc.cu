// Allocation-free residual diagnostic (dg_residuals_noalloc in
// include/dgfem_gb300.h).
//
// Some callers cannot allocate device memory at the point where they need
// the diagnostic: code running inside a pre-planned memory budget (a host
// framework that owns every allocation), real-time loops that must not call
// into the allocator, or callers that hand the library device buffers they
// manage themselves. For them this entry point computes the five residual
// means of the reference's time loop (src/solver.cpp:518-545) between a state
// and a snapshot that the caller passes as device arrays, writing the result
// to a caller-provided device array, and allocates nothing.
//
// Its only scratch is the file-scope array below (kMaxChunks rows of five
// partial sums, 160 KiB), which every GPU that loads this library holds until
// the process exits. Each block reduces one fixed-size chunk of kChunk nodes,
// so a call may cover at most kChunk * kMaxChunks nodes per variable; larger
// inputs are rejected with DG_ERR_ARG. The fixed chunking also makes the
// result independent of the GPU's SM count (bitwise reproducible).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>

#include "../../include/dgfem_gb300.h"

namespace dgc {
void set_global_error(const std::string& m);
}

namespace {

constexpr int kChunk = 16384;      // nodes of one variable reduced by one block
constexpr int kMaxChunks = 4096;   // rows of the scratch array
constexpr int kThreads = 256;

// Shared by every call on a device; the last call's partial sums stay here.
static __device__ __align__(256) double g_res_partials[kMaxChunks * 5];

template <typename T>
__global__ void k_res_partials(const T* u, const T* snap, int n_var, int64_t n, int64_t stride, double c0sq,
                               double* part) {
  __shared__ double sh[kThreads / 32][5];
  const int64_t begin = (int64_t)blockIdx.x * kChunk;
  const int64_t end = begin + kChunk < n ? begin + kChunk : n;
  double r[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int q = 0; q < n_var; ++q)
    for (int64_t i = begin + threadIdx.x; i < end; i += kThreads) {
      const double s = (double)snap[q * stride + i], v = (double)u[q * stride + i];
      const double d = s - v;
      if (q == 0) {
        r[0] += d * d;
        const double dr = s / c0sq - v / c0sq;
        r[1] += dr * dr;
      } else {
        r[1 + q] += d * d;
      }
    }
  for (int c = 0; c < 5; ++c) {
    double x = r[c];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5][c] = x;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double x = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) x += sh[w][threadIdx.x];
    part[blockIdx.x * 5 + threadIdx.x] = x;  // every row in use is written before it is read
  }
}

__global__ void k_res_final(const double* part, int nchunks, double inv_n, double* out) {
  // one warp per component, fixed summation order
  const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (c >= 5) return;
  double x = 0.0;
  for (int b = lane; b < nchunks; b += 32) x += part[b * 5 + c];
  for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
  if (lane == 0) out[c] = x * inv_n;
}

// Device address of the scratch array for the current device, looked up on
// every call with that device current. The lookup allocates nothing, and not
// caching it keeps the address right after a cudaDeviceReset (which reloads
// the module, so the array may move).
cudaError_t scratch_for_current_device(double** p) {
  void* a = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&a, g_res_partials);
  if (e != cudaSuccess) return e;
  *p = static_cast<double*>(a);
  return cudaSuccess;
}

}  // namespace

extern "C" int dg_residuals_noalloc(const void* u, const void* snap, int precision, int n_var, int64_t n_per_var,
                                    int64_t var_stride, double c0, double* res, void* stream) {
  if (!u || !snap || !res || n_var < 1 || n_var > 4 || n_per_var <= 0 || var_stride < n_per_var || !(c0 > 0) ||
      (precision != DG_FP32 && precision != DG_FP64)) {
    dgc::set_global_error("dg_residuals_noalloc: invalid argument");
    return DG_ERR_ARG;
  }
  const int64_t nchunks = (n_per_var + kChunk - 1) / kChunk;
  if (nchunks > kMaxChunks) {
    dgc::set_global_error("dg_residuals_noalloc: " + std::to_string(n_per_var) + " nodes per variable exceed the " +
                          std::to_string((int64_t)kChunk * kMaxChunks) + "-node limit of its fixed scratch");
    return DG_ERR_ARG;
  }
  double* part = nullptr;
  cudaError_t e = scratch_for_current_device(&part);
  if (e != cudaSuccess) {
    dgc::set_global_error(std::string("dg_residuals_noalloc: CUDA: ") + cudaGetErrorString(e));
    return DG_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double c0sq = c0 * c0;
  if (precision == DG_FP32)
    k_res_partials<float><<<(unsigned)nchunks, kThreads, 0, s>>>(static_cast<const float*>(u),
                                                                 static_cast<const float*>(snap), n_var, n_per_var,
                                                                 var_stride, c0sq, part);
  else
    k_res_partials<double><<<(unsigned)nchunks, kThreads, 0, s>>>(static_cast<const double*>(u),
                                                                  static_cast<const double*>(snap), n_var, n_per_var,
                                                                  var_stride, c0sq, part);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    k_res_final<<<1, 5 * 32, 0, s>>>(part, (int)nchunks, 1.0 / (double)n_per_var, res);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    dgc::set_global_error(std::string("dg_residuals_noalloc: CUDA: ") + cudaGetErrorString(e));
    return DG_ERR_CUDA;
  }
  // components of variables the state does not carry (vz in 2-D) come out as
  // zero: their partial sums are written as zero like every other component
  return DG_OK;
}
