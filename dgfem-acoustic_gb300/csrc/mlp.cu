// Learned spectral surrogate: a small fully connected network (GELU hidden
// layers, linear output) that maps source and mean-flow parameters to
// observer log-spectra, trained and evaluated on the GPU by the kernels of
// this file (dg_mlp_* in include/dgfem_gb300.h). It has no counterpart in the
// reference: the reference answers every parameter query with a full DG run,
// which remains the fallback and the measure of the network's error.
//
// Numerics: weights are held in BF16 for the forward and backward passes
// (FP32 master copies for the optimiser), activations and gradients in FP32,
// every sum accumulated in FP32.
//
// Kernels: one GEMM serves the three products of a layer: Z = X W^T
// (forward), dX = dZ W (input gradient) and dW = dZ^T X (weight gradient),
// on the CUDA cores (k_gemm: 64 x 64 output tile, 16-deep K slices staged in
// shared memory, 4 x 4 outputs per thread; the default) or on the tensor
// cores (k_gemm_tc, tcgen05 kind::tf32; dg_mlp_set_tensor_cores). At this
// network's sizes (layers of at most 512, 256-2000 rows) the CUDA-core GEMM
// is the faster: the tensor-core one stages and splits each K slice and waits
// for its MMAs before the next (GB300, the 6-256-256-256-256-512 network:
// forward of 2000 rows 0.31 against 0.63 ms, a training step of 256 rows
// 0.68 against 0.87 ms, host arrays);
// element-wise GELU and its derivative, the MSE gradient, bias reductions
// and an Adam step complete the training loop.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/dgfem_gb300.h"
#include "stage_tc.cuh"  // tcgen05, mbarrier and shared-memory descriptor helpers

namespace dgc {
void set_global_error(const std::string& m);
}

namespace {

constexpr int BM = 64, BN = 64, BK = 16, GT = 256;

template <typename T>
__device__ __forceinline__ float ldf(const T* p) {
  if constexpr (sizeof(T) == 2)
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(p));
  else
    return *p;
}

// C[m][n] = sum_k A(m,k) B(k,n) (+ bias[n]); A(m,k) = A[m*sam + k*sak],
// B(k,n) = B[k*sbk + n*sbn]. Epilogue: mode 0 stores C to Z and GELU(C) to Y
// (hidden layer), mode 1 stores C to Y (output layer or gradient).
template <typename TA, typename TB>
__global__ void __launch_bounds__(GT) k_gemm(int M, int N, int K, const TA* __restrict__ A, int64_t sam, int64_t sak,
                                             const TB* __restrict__ B, int64_t sbk, int64_t sbn,
                                             const float* __restrict__ bias, float* __restrict__ Z,
                                             float* __restrict__ Y, int ldc, int mode) {
  __shared__ float sA[BK][BM + 4];
  __shared__ float sB[BK][BN + 4];
  const int tid = threadIdx.x;
  const int tm = tid / 16, tn = tid % 16;  // 16 x 16 threads, 4 x 4 outputs each
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += BK) {
    for (int i = tid; i < BM * BK; i += GT) {
      const int mm = i / BK, kk = i % BK;
      const int m = m0 + mm, k = k0 + kk;
      sA[kk][mm] = (m < M && k < K) ? ldf(A + (int64_t)m * sam + (int64_t)k * sak) : 0.f;
    }
    for (int i = tid; i < BN * BK; i += GT) {
      const int kk = i / BN, nn = i % BN;
      const int n = n0 + nn, k = k0 + kk;
      sB[kk][nn] = (n < N && k < K) ? ldf(B + (int64_t)k * sbk + (int64_t)n * sbn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tm * 4 + i], b[i] = sB[kk][tn * 4 + i];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tm * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tn * 4 + j;
      if (n >= N) continue;
      float c = acc[i][j] + (bias ? bias[n] : 0.f);
      if (mode == 0) {
        Z[(int64_t)m * ldc + n] = c;
        Y[(int64_t)m * ldc + n] = 0.5f * c * (1.f + erff(c * 0.70710678118654752f));
      } else {
        Y[(int64_t)m * ldc + n] = c;
      }
    }
  }
}

// Tensor-core GEMM (sm_103a tcgen05, kind::tf32), same contract as k_gemm:
// C[m][n] = sum_k A(m,k) B(k,n) (+ bias[n]) over a 128 x 64 output tile per
// block of 128 threads, K in slices of 32. Each slice is staged in shared
// memory in the canonical K-major no-swizzle layout (8-row x 16-byte core
// matrices): A (FP32 activations or gradients) as a TF32 head and tail, B
// the same when it is FP32 (activations, in the weight gradient) and as it
// is when it holds BF16 weights (exact in TF32). One thread issues the
// slice's MMAs, A_lo B_hi (+ A_hi B_lo) + A_hi B_hi, accumulating in FP32 in
// 64 tensor-memory columns, and commits to an mbarrier that the block waits
// for (bounded) before the next slice overwrites the operands; the epilogue
// reads the accumulator rows (tcgen05.ld, one lane quarter per warp) and
// applies k_gemm's epilogue. A block whose wait gives up sets *err, waits
// (default limit) for its MMAs in flight and frees its tensor memory.
constexpr int TBM = 128, TBN = 64, TBK = 32, TGT = 128;
constexpr uint32_t T_LBO_A = (TBM / 8) * 128, T_LBO_B = (TBN / 8) * 128;  // K-adjacent core matrices
constexpr uint32_t T_ABYTES = TBM * TBK * 4, T_BBYTES = TBN * TBK * 4;
constexpr size_t T_SMEM = 2 * (size_t)T_ABYTES + 2 * (size_t)T_BBYTES + 32;  // + mbarrier, tensor-memory slot

// byte offset of (row, k) in a [rows][TBK] operand slice (core matrices of
// 8 rows x 4 values, row groups adjacent, then K groups)
__device__ __forceinline__ uint32_t tc_off(int row, int k, int rows) {
  return (uint32_t)(((k >> 2) * (rows >> 3) + (row >> 3)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::tf32, FP32 accumulate.
__device__ __forceinline__ void umma_tf32_ss(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                             uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

template <typename TB>
__global__ void __launch_bounds__(TGT) k_gemm_tc(int M, int N, int K, const float* __restrict__ A, int64_t sam,
                                                 int64_t sak, const TB* __restrict__ B, int64_t sbk, int64_t sbn,
                                                 const float* __restrict__ bias, float* __restrict__ Z,
                                                 float* __restrict__ Y, int ldc, int mode, int* __restrict__ err) {
  constexpr bool BSPLIT = sizeof(TB) == 4;
  extern __shared__ __align__(128) unsigned char smt[];
  unsigned char* sAh = smt;
  unsigned char* sAl = sAh + T_ABYTES;
  unsigned char* sBh = sAl + T_ABYTES;
  unsigned char* sBl = sBh + T_BBYTES;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sBl + T_BBYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sBl + T_BBYTES + 16);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * TBM, n0 = blockIdx.x * TBN;
  if (tid == 0) {
    dgk::mbar_init(bar, 1);
    dgk::fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dgk::smem_u32(tslot)),
                 "r"((uint32_t)TBN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  dgk::tc_fence_before();
  __syncthreads();
  dgk::tc_fence_after();
  const uint32_t tbase = *tslot;
  const uint32_t idesc =
      (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TBN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
  const uint64_t dah = dgk::umma_desc(dgk::smem_u32(sAh), T_LBO_A, 128);
  const uint64_t dal = dgk::umma_desc(dgk::smem_u32(sAl), T_LBO_A, 128);
  const uint64_t dbh = dgk::umma_desc(dgk::smem_u32(sBh), T_LBO_B, 128);
  const uint64_t dbl = dgk::umma_desc(dgk::smem_u32(sBl), T_LBO_B, 128);
  bool ok = true, pend = false;  // pend: a commit not yet observed complete (thread 0)
  uint32_t phase = 0;
  for (int k0 = 0; k0 < K; k0 += TBK) {
    // ---- the slice's operands, zero outside the matrices ----
    for (int i = tid; i < TBM * TBK; i += TGT) {
      const int mm = i / TBK, kk = i - (i / TBK) * TBK, m = m0 + mm, k = k0 + kk;
      const float x = (m < M && k < K) ? A[(int64_t)m * sam + (int64_t)k * sak] : 0.f;
      const uint32_t h = dgk::tf32_rna(x), off = tc_off(mm, kk, TBM);
      *reinterpret_cast<uint32_t*>(sAh + off) = h;
      *reinterpret_cast<uint32_t*>(sAl + off) = dgk::tf32_rna(x - __uint_as_float(h));
    }
    for (int i = tid; i < TBN * TBK; i += TGT) {
      const int nn = i / TBK, kk = i - (i / TBK) * TBK, n = n0 + nn, k = k0 + kk;
      const float x = (n < N && k < K) ? ldf(B + (int64_t)k * sbk + (int64_t)n * sbn) : 0.f;
      const uint32_t off = tc_off(nn, kk, TBN);
      if constexpr (BSPLIT) {
        const uint32_t h = dgk::tf32_rna(x);
        *reinterpret_cast<uint32_t*>(sBh + off) = h;
        *reinterpret_cast<uint32_t*>(sBl + off) = dgk::tf32_rna(x - __uint_as_float(h));
      } else {
        *reinterpret_cast<uint32_t*>(sBh + off) = __float_as_uint(x);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // read by the tensor cores
    dgk::tc_fence_before();
    __syncthreads();
    dgk::tc_fence_after();
    bool got = true;
    if (tid == 0) {
#pragma unroll
      for (int ks = 0; ks < TBK / 8; ++ks) {
        const uint64_t oa = (uint64_t)((ks * 2 * T_LBO_A) >> 4), ob = (uint64_t)((ks * 2 * T_LBO_B) >> 4);
        umma_tf32_ss(tbase, dal + oa, dbh + ob, idesc, (k0 == 0 && ks == 0) ? 0u : 1u);
        if constexpr (BSPLIT) umma_tf32_ss(tbase, dah + oa, dbl + ob, idesc, 1u);
        umma_tf32_ss(tbase, dah + oa, dbh + ob, idesc, 1u);
      }
      dgk::umma_commit(bar);
      got = dgk::mbar_wait(bar, phase & 1u);
      pend = !got;
    }
    ++phase;
    if (__syncthreads_or(!got)) {
      ok = false;
      break;
    }
    dgk::tc_fence_after();
  }
  if (ok) {
    // ---- epilogue: row m0 + 32 warp + lane, TBN columns ----
    const int m = m0 + warp * 32 + lane;
    const uint32_t trow = tbase + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < TBN; c0 += 16) {
      uint32_t r[4][4];
#pragma unroll
      for (int t = 0; t < 4; ++t) dgk::tmem_ld4_async(trow + c0 + 4 * t, r[t]);
#pragma unroll
      for (int t = 0; t < 4; ++t) dgk::tmem_wait_ld4(r[t]);
      if (m >= M) continue;
#pragma unroll
      for (int t = 0; t < 4; ++t)
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int n = n0 + c0 + 4 * t + u;
          if (n >= N) continue;
          const float c = __uint_as_float(r[t][u]) + (bias ? bias[n] : 0.f);
          if (mode == 0) {
            Z[(int64_t)m * ldc + n] = c;
            Y[(int64_t)m * ldc + n] = 0.5f * c * (1.f + erff(c * 0.70710678118654752f));
          } else {
            Y[(int64_t)m * ldc + n] = c;
          }
        }
    }
  }
  // ---- teardown: the MMAs in flight after a give-up, then the memory ----
  if (tid == 0 && pend) dgk::mbar_wait(bar, (phase - 1) & 1u);
  if (tid == 0 && !ok) atomicOr(err, 1);
  dgk::tc_fence_before();
  __syncthreads();
  dgk::tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"((uint32_t)TBN)
                 : "memory");
}

// dZ = dY * GELU'(Z), GELU'(z) = Phi(z) + z phi(z)
__global__ void k_gelu_bwd(const float* __restrict__ Z, const float* __restrict__ dY, float* __restrict__ dZ,
                           int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float z = Z[i];
  const float cdf = 0.5f * (1.f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  dZ[i] = dY[i] * (cdf + z * pdf);
}

// MSE over all outputs: dY = 2 (Y - T) / n, per-block partial sums of (Y-T)^2
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, float* __restrict__ dY, int64_t n,
                      double* __restrict__ part) {
  __shared__ double sh[GT / 32];
  double s = 0.0;
  const float sc = 2.f / (float)n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    dY[i] = sc * d;
    s += (double)d * d;
  }
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < GT / 32; ++w) t += sh[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_sum_parts(const double* part, int n, double scale, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < n; ++i) t += part[i];
    *out = t * scale;
  }
}

// db[n] = sum_b dZ[b][n]
__global__ void k_colsum(const float* __restrict__ dZ, int B, int N, float* __restrict__ db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int b = 0; b < B; ++b) s += dZ[(int64_t)b * N + n];
  db[n] = s;
}

__global__ void k_gather_rows(const float* __restrict__ src, const int* __restrict__ idx, int n, int w,
                              float* __restrict__ dst) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)n * w) return;
  const int r = (int)(i / w), c = (int)(i % w);
  dst[i] = src[(int64_t)idx[r] * w + c];
}

// Adam on the FP32 master parameters with decoupled weight decay wd (AdamW);
// weights are re-rounded to BF16 afterwards
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int64_t n, float lr, float b1, float b2, float eps, float c1, float c2,
                       float wd) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float v = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a, m2[i] = v;
  p[i] -= lr * ((a / c1) / (sqrtf(v / c2) + eps) + wd * p[i]);
}

__global__ void k_to_bf16(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

struct dg_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<int> w;                  // widths, n_layers + 1
  std::vector<int64_t> woff, boff;     // offsets of W_l and b_l in the flat parameter vector
  std::vector<int64_t> hoff;           // offsets of W_l in the BF16 copy
  int64_t n_params = 0, n_wts = 0;
  float *p = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // FP32 master, gradient, Adam moments
  __nv_bfloat16* wh = nullptr;          // BF16 weights
  // activations for a batch of up to cap rows: per layer input X_l, pre-activation Z_l
  int64_t cap = 0;
  std::vector<float*> X, Z;
  float *dA = nullptr, *dB = nullptr;  // gradient ping-pong buffers [cap][max width]
  double *part = nullptr, *loss = nullptr;
  // training set
  float *tx = nullptr, *ty = nullptr, *bx = nullptr, *by = nullptr;
  int* bidx = nullptr;
  int64_t n_data = 0, bcap = 0;
  int64_t step = 0;  // Adam steps taken
  int tc = 0;             // GEMMs on the tensor cores (k_gemm_tc), else k_gemm
  int* d_err = nullptr;   // set by a tensor-core GEMM whose wait gave up
  std::string err;
};

namespace {

int fail(dg_mlp* m, int code, const std::string& msg) {
  if (m) m->err = msg;
  dgc::set_global_error(msg);
  return code;
}

#define MCK(m, x)                                                                                   \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess) return fail((m), DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

int max_width(const dg_mlp* m) {
  int mw = 0;
  for (int v : m->w) mw = v > mw ? v : mw;
  return mw;
}

int ensure_cap(dg_mlp* m, int64_t n) {
  if (n <= m->cap) return DG_OK;
  for (float* q : m->X) cudaFree(q);
  for (float* q : m->Z) cudaFree(q);
  cudaFree(m->dA), cudaFree(m->dB);
  m->X.assign(m->w.size(), nullptr);
  m->Z.assign(m->w.size(), nullptr);
  const int L = (int)m->w.size() - 1;
  for (int l = 0; l <= L; ++l) {
    MCK(m, cudaMalloc(&m->X[l], n * m->w[l] * sizeof(float)));
    if (l >= 1) MCK(m, cudaMalloc(&m->Z[l], n * m->w[l] * sizeof(float)));
  }
  MCK(m, cudaMalloc(&m->dA, n * max_width(m) * sizeof(float)));
  MCK(m, cudaMalloc(&m->dB, n * max_width(m) * sizeof(float)));
  m->cap = n;
  return DG_OK;
}

// One GEMM of a layer (k_gemm's contract) on the tensor cores or the CUDA
// cores, on the network's stream.
template <typename TB>
int gemm(dg_mlp* m, int M, int N, int K, const float* A, int64_t sam, int64_t sak, const TB* B, int64_t sbk,
         int64_t sbn, const float* bias, float* Z, float* Y, int ldc, int mode) {
  if (m->tc) {
    static bool configured = false;
    if (!configured) {
      MCK(m, cudaFuncSetAttribute(k_gemm_tc<TB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T_SMEM));
      configured = true;
    }
    dim3 grid(nblk(N, TBN), nblk(M, TBM));
    k_gemm_tc<TB><<<grid, TGT, T_SMEM, m->stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, Z, Y, ldc, mode, m->d_err);
  } else {
    dim3 grid(nblk(N, BN), nblk(M, BM));
    k_gemm<float, TB><<<grid, GT, 0, m->stream>>>(M, N, K, A, sam, sak, B, sbk, sbn, bias, Z, Y, ldc, mode);
  }
  MCK(m, cudaGetLastError());
  return DG_OK;
}

// After a stream synchronisation: DG_ERR_TIMEOUT (and the flag cleared) when
// a tensor-core GEMM gave up waiting for its MMAs.
int check_gemm_waits(dg_mlp* m) {
  int h = 0;
  MCK(m, cudaMemcpyAsync(&h, m->d_err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  MCK(m, cudaStreamSynchronize(m->stream));
  if (h == 0) return DG_OK;
  MCK(m, cudaMemsetAsync(m->d_err, 0, sizeof(int), m->stream));
  MCK(m, cudaStreamSynchronize(m->stream));
  return fail(m, DG_ERR_TIMEOUT, "dg_mlp: a tensor-core GEMM timed out waiting for its MMAs");
}

int refresh_bf16(dg_mlp* m) {
  const int L = (int)m->w.size() - 1;
  for (int l = 0; l < L; ++l) {
    const int64_t nw = (int64_t)m->w[l + 1] * m->w[l];
    k_to_bf16<<<nblk(nw, 256), 256, 0, m->stream>>>(m->p + m->woff[l], m->wh + m->hoff[l], nw);
  }
  MCK(m, cudaGetLastError());
  return DG_OK;
}

// Forward pass of n rows already in X[0]; output in X[L].
int forward(dg_mlp* m, int64_t n) {
  const int L = (int)m->w.size() - 1;
  for (int l = 0; l < L; ++l) {
    const int K = m->w[l], N = m->w[l + 1];
    const bool last = l == L - 1;
    const int rc = gemm<__nv_bfloat16>(m, (int)n, N, K, m->X[l], K, 1, m->wh + m->hoff[l], 1, K, m->p + m->boff[l],
                                       m->Z[l + 1], m->X[l + 1], N, last ? 1 : 0);
    if (rc != DG_OK) return rc;
  }
  return DG_OK;
}

// Backward pass for n rows with dY (gradient of the loss w.r.t. the output)
// in dA; writes the parameter gradient to m->g.
int backward(dg_mlp* m, int64_t n) {
  const int L = (int)m->w.size() - 1;
  float* dcur = m->dA;   // gradient w.r.t. the output of layer l (post-activation)
  float* dnext = m->dB;
  for (int l = L - 1; l >= 0; --l) {
    const int K = m->w[l], N = m->w[l + 1];
    float* dZ = dcur;
    if (l < L - 1) {  // hidden layer: through GELU
      k_gelu_bwd<<<nblk(n * N, 256), 256, 0, m->stream>>>(m->Z[l + 1], dcur, dnext, n * N);
      dZ = dnext;
      std::swap(dcur, dnext);  // dcur now holds dZ
    }
    // dW[N][K] = dZ^T X: rows n of W, columns k, summed over the batch
    int rc = gemm<float>(m, N, K, (int)n, dZ, 1, N, m->X[l], K, 1, nullptr, nullptr, m->g + m->woff[l], K, 1);
    if (rc != DG_OK) return rc;
    k_colsum<<<nblk(N, 128), 128, 0, m->stream>>>(dZ, (int)n, N, m->g + m->boff[l]);
    if (l > 0) {
      // dX[n][K] = dZ W
      rc = gemm<__nv_bfloat16>(m, (int)n, K, N, dZ, N, 1, m->wh + m->hoff[l], K, 1, nullptr, nullptr, dnext, K, 1);
      if (rc != DG_OK) return rc;
      std::swap(dcur, dnext);
    }
  }
  MCK(m, cudaGetLastError());
  return DG_OK;
}

// loss and dY (into dA) for n rows of targets T
int mse(dg_mlp* m, const float* T, int64_t n) {
  const int L = (int)m->w.size() - 1;
  const int64_t cnt = n * m->w[L];
  const int nb = 64;
  k_mse<<<nb, GT, 0, m->stream>>>(m->X[L], T, m->dA, cnt, m->part);
  k_sum_parts<<<1, 32, 0, m->stream>>>(m->part, nb, 1.0 / (double)cnt, m->loss);
  MCK(m, cudaGetLastError());
  return DG_OK;
}

}  // namespace

extern "C" {

int dg_mlp_create(int n_layers, const int* widths, int device, dg_mlp** out) {
  if (!out || !widths || n_layers < 1 || n_layers > 16) return fail(nullptr, DG_ERR_ARG, "dg_mlp_create: invalid argument");
  *out = nullptr;
  for (int l = 0; l <= n_layers; ++l)
    if (widths[l] < 1 || widths[l] > 8192) return fail(nullptr, DG_ERR_ARG, "dg_mlp_create: invalid layer width");
  dg_mlp* m = new dg_mlp();
  m->device = device;
  m->w.assign(widths, widths + n_layers + 1);
  for (int l = 0; l < n_layers; ++l) {
    m->woff.push_back(m->n_params);
    m->n_params += (int64_t)widths[l + 1] * widths[l];
    m->boff.push_back(m->n_params);
    m->n_params += widths[l + 1];
    m->hoff.push_back(m->n_wts);
    m->n_wts += (int64_t)widths[l + 1] * widths[l];
  }
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  for (float** q : {&m->p, &m->g, &m->m1, &m->m2})
    if (e == cudaSuccess) e = cudaMalloc(q, m->n_params * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->wh, m->n_wts * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc(&m->part, 64 * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&m->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(m->d_err, 0, sizeof(int), m->stream);
  // on the network's own (non-blocking) stream: a legacy-stream memset would
  // not be ordered with the uploads that follow
  for (float* q : {m->p, m->g, m->m1, m->m2})
    if (e == cudaSuccess) e = cudaMemsetAsync(q, 0, m->n_params * sizeof(float), m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    std::string msg = std::string("dg_mlp_create: CUDA: ") + cudaGetErrorString(e);
    dg_mlp_destroy(m);
    return fail(nullptr, DG_ERR_CUDA, msg);
  }
  *out = m;
  return DG_OK;
}

int dg_mlp_destroy(dg_mlp* m) {
  if (!m) return DG_OK;
  cudaSetDevice(m->device);
  for (float* q : m->X) cudaFree(q);
  for (float* q : m->Z) cudaFree(q);
  for (void* q : {(void*)m->p, (void*)m->g, (void*)m->m1, (void*)m->m2, (void*)m->wh, (void*)m->dA, (void*)m->dB,
                  (void*)m->part, (void*)m->loss, (void*)m->tx, (void*)m->ty, (void*)m->bx, (void*)m->by,
                  (void*)m->bidx, (void*)m->d_err})
    cudaFree(q);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return DG_OK;
}

const char* dg_mlp_last_error(dg_mlp* m) { return m ? m->err.c_str() : dg_last_error(nullptr); }

int64_t dg_mlp_param_count(dg_mlp* m) { return m ? m->n_params : 0; }

int dg_mlp_set_params(dg_mlp* m, const float* params) {
  if (!m || !params) return fail(m, DG_ERR_ARG, "dg_mlp_set_params: invalid argument");
  cudaSetDevice(m->device);
  MCK(m, cudaMemcpyAsync(m->p, params, m->n_params * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(m, cudaMemsetAsync(m->m1, 0, m->n_params * sizeof(float), m->stream));
  MCK(m, cudaMemsetAsync(m->m2, 0, m->n_params * sizeof(float), m->stream));
  m->step = 0;
  int rc = refresh_bf16(m);
  if (rc != DG_OK) return rc;
  MCK(m, cudaStreamSynchronize(m->stream));
  return DG_OK;
}

int dg_mlp_get_params(dg_mlp* m, float* params) {
  if (!m || !params) return fail(m, DG_ERR_ARG, "dg_mlp_get_params: invalid argument");
  cudaSetDevice(m->device);
  MCK(m, cudaMemcpyAsync(params, m->p, m->n_params * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(m, cudaStreamSynchronize(m->stream));
  return DG_OK;
}

int dg_mlp_forward_device(dg_mlp* m, const float* x, int64_t n, float* y, void* stream) {
  if (!m || !x || !y || n < 1) return fail(m, DG_ERR_ARG, "dg_mlp_forward_device: invalid argument");
  cudaSetDevice(m->device);
  int rc = ensure_cap(m, n);
  if (rc != DG_OK) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
  cudaStream_t keep = m->stream;
  m->stream = s;
  const int L = (int)m->w.size() - 1;
  cudaError_t e = cudaMemcpyAsync(m->X[0], x, n * m->w[0] * sizeof(float), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) rc = forward(m, n);
  if (e == cudaSuccess && rc == DG_OK)
    e = cudaMemcpyAsync(y, m->X[L], n * m->w[L] * sizeof(float), cudaMemcpyDeviceToDevice, s);
  m->stream = keep;
  if (e != cudaSuccess) return fail(m, DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  return rc;
}

int dg_mlp_forward(dg_mlp* m, const float* x, int64_t n, float* y) {
  if (!m || !x || !y || n < 1) return fail(m, DG_ERR_ARG, "dg_mlp_forward: invalid argument");
  cudaSetDevice(m->device);
  int rc = ensure_cap(m, n);
  if (rc != DG_OK) return rc;
  const int L = (int)m->w.size() - 1;
  MCK(m, cudaMemcpyAsync(m->X[0], x, n * m->w[0] * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  rc = forward(m, n);
  if (rc != DG_OK) return rc;
  MCK(m, cudaMemcpyAsync(y, m->X[L], n * m->w[L] * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  MCK(m, cudaStreamSynchronize(m->stream));
  return check_gemm_waits(m);
}

int dg_mlp_gradient(dg_mlp* m, const float* x, const float* t, int64_t n, float* grad, double* loss) {
  if (!m || !x || !t || !grad || n < 1) return fail(m, DG_ERR_ARG, "dg_mlp_gradient: invalid argument");
  cudaSetDevice(m->device);
  int rc = ensure_cap(m, n);
  if (rc != DG_OK) return rc;
  const int L = (int)m->w.size() - 1;
  float* dt = nullptr;
  MCK(m, cudaMalloc(&dt, n * m->w[L] * sizeof(float)));
  cudaError_t e = cudaMemcpyAsync(m->X[0], x, n * m->w[0] * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dt, t, n * m->w[L] * sizeof(float), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) {
    rc = forward(m, n);
    if (rc == DG_OK) rc = mse(m, dt, n);
    if (rc == DG_OK) rc = backward(m, n);
    if (rc == DG_OK) e = cudaMemcpyAsync(grad, m->g, m->n_params * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
    if (rc == DG_OK && e == cudaSuccess && loss)
      e = cudaMemcpyAsync(loss, m->loss, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  }
  cudaFree(dt);
  if (e != cudaSuccess) return fail(m, DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  if (rc == DG_OK) rc = check_gemm_waits(m);
  return rc;
}

int dg_mlp_set_data(dg_mlp* m, const float* x, const float* t, int64_t n) {
  if (!m || !x || !t || n < 1) return fail(m, DG_ERR_ARG, "dg_mlp_set_data: invalid argument");
  cudaSetDevice(m->device);
  const int L = (int)m->w.size() - 1;
  cudaFree(m->tx), cudaFree(m->ty);
  m->tx = m->ty = nullptr;
  MCK(m, cudaMalloc(&m->tx, n * m->w[0] * sizeof(float)));
  MCK(m, cudaMalloc(&m->ty, n * m->w[L] * sizeof(float)));
  MCK(m, cudaMemcpyAsync(m->tx, x, n * m->w[0] * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(m, cudaMemcpyAsync(m->ty, t, n * m->w[L] * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MCK(m, cudaStreamSynchronize(m->stream));
  m->n_data = n;
  return DG_OK;
}

int dg_mlp_train(dg_mlp* m, int64_t n_steps, int batch, double lr, double lr_final, double weight_decay, uint64_t seed,
                 double* losses) {
  if (!m || n_steps < 0 || batch < 1 || !(lr > 0) || !(lr_final > 0) || !(weight_decay >= 0))
    return fail(m, DG_ERR_ARG, "dg_mlp_train: invalid argument");
  if (m->n_data < batch) return fail(m, DG_ERR_ARG, "dg_mlp_train: fewer training rows than one batch");
  cudaSetDevice(m->device);
  int rc = ensure_cap(m, batch);
  if (rc != DG_OK) return rc;
  const int L = (int)m->w.size() - 1;
  if (m->bcap < batch) {
    cudaFree(m->by), cudaFree(m->bidx);
    m->by = nullptr, m->bidx = nullptr;
    MCK(m, cudaMalloc(&m->by, (int64_t)batch * m->w[L] * sizeof(float)));
    m->bcap = batch;
  }
  // one permutation of the training rows per epoch, drawn on the host
  const int64_t nd = m->n_data, steps_per_epoch = nd / batch;
  std::vector<int> perm(nd);
  std::mt19937_64 rng(seed);
  MCK(m, cudaMalloc(&m->bidx, nd * sizeof(int)));
  double* d_losses = nullptr;
  MCK(m, cudaMalloc(&d_losses, (n_steps > 0 ? n_steps : 1) * sizeof(double)));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  cudaError_t e = cudaSuccess;
  for (int64_t s = 0; s < n_steps && rc == DG_OK && e == cudaSuccess; ++s) {
    const int64_t within = s % steps_per_epoch;
    if (within == 0) {
      for (int64_t i = 0; i < nd; ++i) perm[i] = (int)i;
      std::shuffle(perm.begin(), perm.end(), rng);
      e = cudaMemcpyAsync(m->bidx, perm.data(), nd * sizeof(int), cudaMemcpyHostToDevice, m->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);  // perm is rewritten next epoch
      if (e != cudaSuccess) break;
    }
    const int* idx = m->bidx + within * batch;
    k_gather_rows<<<nblk((int64_t)batch * m->w[0], 256), 256, 0, m->stream>>>(m->tx, idx, batch, m->w[0], m->X[0]);
    k_gather_rows<<<nblk((int64_t)batch * m->w[L], 256), 256, 0, m->stream>>>(m->ty, idx, batch, m->w[L], m->by);
    rc = forward(m, batch);
    if (rc == DG_OK) rc = mse(m, m->by, batch);
    if (rc == DG_OK) e = cudaMemcpyAsync(d_losses + s, m->loss, sizeof(double), cudaMemcpyDeviceToDevice, m->stream);
    if (rc == DG_OK && e == cudaSuccess) rc = backward(m, batch);
    if (rc != DG_OK || e != cudaSuccess) break;
    // cosine decay from lr to lr_final
    const double frac = n_steps > 1 ? (double)s / (double)(n_steps - 1) : 1.0;
    const double lrs = lr_final + 0.5 * (lr - lr_final) * (1.0 + std::cos(3.14159265358979323846 * frac));
    m->step += 1;
    const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
    k_adam<<<nblk(m->n_params, 256), 256, 0, m->stream>>>(m->p, m->g, m->m1, m->m2, m->n_params, (float)lrs, b1, b2,
                                                          eps, c1, c2, (float)weight_decay);
    rc = refresh_bf16(m);
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (e == cudaSuccess && rc == DG_OK && losses && n_steps > 0)
    e = cudaMemcpyAsync(losses, d_losses, n_steps * sizeof(double), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(d_losses);
  cudaFree(m->bidx);
  m->bidx = nullptr;
  if (e != cudaSuccess) return fail(m, DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e));
  if (rc == DG_OK) rc = check_gemm_waits(m);
  return rc;
}

int dg_mlp_set_tensor_cores(dg_mlp* m, int on) {
  if (!m) return fail(m, DG_ERR_ARG, "dg_mlp_set_tensor_cores: invalid argument");
  m->tc = on ? 1 : 0;
  return DG_OK;
}

int dg_mlp_tensor_cores(const dg_mlp* m) { return m && m->tc ? 1 : 0; }

}  // extern "C"
