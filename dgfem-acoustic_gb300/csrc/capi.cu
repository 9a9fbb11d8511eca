// C ABI of the GB300 DG solver (include/dgfem_gb300.h): context lifetime,
// state I/O in the reference layout, sources, observers, the per-step CUDA
// graph (source injection -> four fused RK4 stages -> residual and observer
// reductions) and benchmarking.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "ctx.h"
#include "curved.cuh"

namespace {

thread_local std::string g_create_error;

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// auxiliary kernels
// ---------------------------------------------------------------------------

// reference layout [4][E*np] (double, mesh local node order) -> internal
template <typename T>
__global__ void k_ref_to_int(const double* ref, T* out, const int* perm, int64_t E, int np, int nv, int64_t stride) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)nv * E * np) return;
  int q = (int)(i / (E * np));
  int64_t r = i - (int64_t)q * E * np;
  int64_t e = r / np;
  int n = (int)(r - e * np);
  out[q * stride + e * np + perm[n]] = (T)ref[i];
}

template <typename T>
__global__ void k_int_to_ref(const T* in, double* ref, const int* perm, int64_t E, int np, int nv, int64_t stride) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= 4 * E * np) return;
  int q = (int)(i / (E * np));
  int64_t r = i - (int64_t)q * E * np;
  int64_t e = r / np;
  int n = (int)(r - e * np);
  ref[i] = q < nv ? (double)in[q * stride + e * np + perm[n]] : 0.0;
}

// Hard overwrite of the pressure at source nodes (src/solver.cpp:455-483):
// per node, the last source (in order) that is active at this step wins.
template <typename T>
__global__ void k_inject(T* up, const int64_t* dof, const int* off, const int* ids, const double* val, int nsrc,
                         int64_t nrows, const int64_t* step, int64_t ndof) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= ndof) return;
  int64_t s = step[0];
  if (s < 0 || s >= nrows) return;
  const double* row = val + s * nsrc;
  double v = 0.0;
  bool any = false;
  for (int k = off[i]; k < off[i + 1]; ++k) {
    double x = row[ids[k]];
    if (!isnan(x)) v = x, any = true;
  }
  if (any) up[dof[i]] = (T)v;
}

// Block sizes of the finalize kernel: 256 threads when an observer holds
// more node slots than the small block (one slot per thread), else 64.
constexpr int kFinalizeThreads = 256, kFinalizeThreadsSmall = 64;

// Block sums of five FP64 values per thread by a halving tree in shared
// memory, each level with only the warps it needs (GB300's FP64 rate makes
// per-warp shuffle trees, which add on every lane at every level, the larger
// cost). The sums end in red[c][0]; every thread of the block calls it.
template <int NT>
__device__ __forceinline__ void block_sum5(double (&red)[5][NT], const double (&acc)[5], int tid) {
#pragma unroll
  for (int c = 0; c < 5; ++c) red[c][tid] = acc[c];
  __syncthreads();
#pragma unroll
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (tid < s) {
#pragma unroll
      for (int c = 0; c < 5; ++c) red[c][tid] += red[c][tid + s];
    }
    __syncthreads();
  }
}

// Residuals (block 0) and observer IDW samples (then, per observer o, the
// blocks bfirst[o] .. bfirst[o+1]-1 of the observer blocks, bmap giving each
// block's observer; each block sums a strided share of the observer's node
// slots) of the step just completed (src/solver.cpp:518-573). With more than
// one block per observer, the blocks store partial sums and the observer's
// last block to finish (counted with an atomic per observer) combines them in
// block order: the result does not depend on the blocks' timing. Without
// bmap every observer has one block.
template <typename T, int NT>
__global__ void __launch_bounds__(NT)
    k_finalize(const double* partials, int nparts, double inv_count, double* res, const T* u, int64_t stride, int nv,
               const int64_t* odof, const int64_t* ooff, const double* ow, double* obs, int n_obs, const int* bmap,
               const int* bfirst, double* obs_part, unsigned* obs_cnt, const int64_t* step, int64_t cap) {
  __shared__ double red[5][NT];
  __shared__ bool last;
  int64_t slot = step[0] - step[1];
  if (slot < 0 || slot >= cap) return;
  const int tid = threadIdx.x;
  if (blockIdx.x == 0) {
    double acc[5] = {0, 0, 0, 0, 0};
    for (int b = tid; b < nparts; b += NT)
      for (int c = 0; c < 5; ++c) acc[c] += partials[b * 5 + c];
    block_sum5<NT>(red, acc, tid);
    if (tid < 5) res[slot * 5 + tid] = red[tid][0] * inv_count;
    return;
  }
  const int ob = blockIdx.x - 1;
  const int o = bmap ? bmap[ob] : ob;
  if (o >= n_obs) return;
  const int first = bmap ? bfirst[o] : ob, nb = bmap ? bfirst[o + 1] - first : 1, part = ob - first;
  double acc[5] = {0, 0, 0, 0, 0};  // p, vx, vy, vz, w
  const int64_t step_k = (int64_t)NT * nb;
#pragma unroll 4
  for (int64_t k = ooff[o] + (int64_t)part * NT + tid; k < ooff[o + 1]; k += step_k) {
    double w = ow[k];
    int64_t d = odof[k];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (q < nv) acc[q] += (double)u[q * stride + d] * w;
    acc[4] += w;
  }
  block_sum5<NT>(red, acc, tid);
  if (nb == 1) {
    if (tid < 4) obs[(slot * n_obs + o) * 4 + tid] = red[tid][0] / red[4][0];
    return;
  }
  if (tid < 5) {
    obs_part[(int64_t)ob * 5 + tid] = red[tid][0];
    __threadfence();
  }
  __syncthreads();
  if (tid == 0) last = atomicAdd(obs_cnt + o, 1u) == (unsigned)(nb - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (tid < 4) {
    double v = 0.0, w = 0.0;
    for (int b = first; b < first + nb; ++b) {
      v += __ldcg(obs_part + (int64_t)b * 5 + tid);
      w += __ldcg(obs_part + (int64_t)b * 5 + 4);
    }
    obs[(slot * n_obs + o) * 4 + tid] = v / w;
  }
  if (tid == 0) obs_cnt[o] = 0u;  // for the next step
}

__global__ void k_advance(int64_t* step) { step[0] += 1; }

template <typename T, int NT>
void launch_finalize_nt(dg_ctx* c, int nparts, double inv_count, int64_t stride) {
  k_finalize<T, NT><<<1 + c->obs_blocks, NT, 0, c->stream>>>(
      c->partials, nparts, inv_count, c->d_res, (const T*)c->u, stride, c->nv, c->d_obs_dof, c->d_obs_off, c->d_obs_w,
      c->d_obs, c->n_obs, c->d_obs_bmap, c->d_obs_bfirst, c->d_obs_part, c->d_obs_cnt, c->d_step, c->out_cap);
}
template <typename T>
void launch_finalize(dg_ctx* c, int nparts, double inv_count, int64_t stride) {
  if (c->obs_small)
    launch_finalize_nt<T, kFinalizeThreadsSmall>(c, nparts, inv_count, stride);
  else
    launch_finalize_nt<T, kFinalizeThreads>(c, nparts, inv_count, stride);
}

// Euler1 commit: u = y (computed as u + k by the stage kernel) with residuals.
template <typename T>
__global__ void k_euler_commit(T* u, const T* y, const T* snap, int64_t n, int64_t stride, int nv, double c0sq,
                               double* partials) {
  __shared__ double sh[32][5];
  dgk::ResAcc<T> racc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int q = (int)(i / stride);
    T un = y[i];
    u[i] = un;
    racc.add(q, snap[i], un, c0sq);
  }
  const int tid = threadIdx.x;
  for (int c = 0; c < 5; ++c) {
    double v = racc.get(c, c0sq);
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if ((tid & 31) == 0) sh[tid >> 5][c] = v;
  }
  __syncthreads();
  if (tid < 5) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[w][tid];
    partials[blockIdx.x * 5 + tid] = v;
  }
}

// Element means of p, p/c0^2 and v (src/Mesh.cpp:1196-1212), mesh node order.
template <typename T>
__global__ void k_cell_means(const T* u, const int* perm, int64_t E, int np, int nv, int64_t stride, double c0sq,
                             double* out) {
  int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  double p = 0, rho = 0, v[3] = {0, 0, 0};
  for (int n = 0; n < np; ++n) {
    int64_t g = e * np + perm[n];
    double pv = (double)u[g];
    p += pv;
    rho += pv / c0sq;
    for (int d = 0; d < nv - 1; ++d) v[d] += (double)u[(1 + d) * stride + g];
  }
  out[e * 5 + 0] = p / np;
  out[e * 5 + 1] = rho / np;
  for (int d = 0; d < 3; ++d) out[e * 5 + 2 + d] = v[d] / np;
}

__global__ void k_flush(unsigned* buf, int64_t n, unsigned v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    buf[i] = v + (unsigned)i;
}

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------

int fail(dg_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(c, x)                                                                               \
  do {                                                                                         \
    cudaError_t e_ = (x);                                                                      \
    if (e_ != cudaSuccess) return fail((c), DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
dgk::StageArgs<T> stage_args(dg_ctx* c, int stage, const T* y_in, T* y_out, T* k_out, double dt) {
  dgk::StageArgs<T> a{};
  a.y_in = y_in;
  a.y_out = y_out;
  a.u = (T*)c->u;
  a.acc = (T*)c->acc;
  a.snap = (const T*)c->snap;
  a.k_out = k_out;
  a.partials = c->partials;
  a.geoF = (const T*)c->geoF;
  a.geoI = c->geoI;
  a.bmat = (const T*)c->bmat;
  a.Dt = (const T*)c->Dt;
  a.LIFT = (const T*)c->LIFT;
  a.cslot = c->ncurved > 0 ? c->cslot : nullptr;
  a.crhs = (const T*)c->crhs;
  a.cstride = c->ncurved * c->np;
  a.fmask = c->fmask;
  a.nbrnode = c->nbrnode;
  a.stride = c->Epad * c->np;
  a.ntiles = c->variant >= 0 ? (int)(c->Epad / c->s2.et) : (int)c->ntiles;
  a.stage = stage;
  a.wait_limit = c->wait_limit;
  a.dt = dt;
  a.c0sq = c->c0sq;
  a.ph = c->ph;
  a.f_rhoc2 = (float)c->ph.rhoc2, a.f_inv_rho0 = (float)c->ph.inv_rho0, a.f_half_c0 = (float)c->ph.half_c0;
  a.f_dt = (float)dt;
  return a;
}

template <typename T>
cudaError_t launch_stage_t(dg_ctx* c, int stage, const T* y_in, T* y_out, T* k_out, double dt) {
  const dgk::StageArgs<T> a = stage_args<T>(c, stage, y_in, y_out, k_out, dt);
  if (dgk::is_tc_variant(c->variant)) {
    if constexpr (sizeof(T) == 4)
      return dgk::is_tc3_variant(c->variant)
                 ? dgk::launch_stage_tc3(c->dim, c->order, dgk::tc_npart(c->variant), a, c->grid2, c->d_err, c->stream)
             : dgk::is_tc2_variant(c->variant)
                 ? dgk::launch_stage_tc2(c->dim, c->order, dgk::tc_npart(c->variant), a, c->grid2, c->d_err, c->stream)
                 : dgk::launch_stage_tc(c->dim, c->order, dgk::tc_npart(c->variant), a, c->grid2, c->d_err, c->stream);
    return cudaErrorInvalidValue;
  }
  if (dgk::is_stage3_variant(c->variant)) {
    if constexpr (sizeof(T) == 4)
      return dgk::launch_stage3(c->dim, c->order, c->variant - dgk::kStage3Variant, a, c->grid2, c->d_err, c->stream);
    return cudaErrorInvalidValue;
  }
  if (dgk::is_wide_variant(c->variant)) {
    if constexpr (sizeof(T) == 4)
      return dgk::launch_stage4(c->dim, c->order, c->variant - dgk::kWideVariant, a, c->grid2, c->d_err, c->stream);
    return cudaErrorInvalidValue;
  }
  if (c->variant >= 0) {
    if constexpr (sizeof(T) == 4)
      return c->dim == 1   ? dgk::launch_stage2_f32_1d(c->order, c->variant, a, c->grid2, c->d_err, c->stream)
             : c->dim == 2 ? dgk::launch_stage2_f32_2d(c->order, c->variant, a, c->grid2, c->d_err, c->stream)
                           : dgk::launch_stage2_f32_3d(c->order, c->variant, a, c->grid2, c->d_err, c->stream);
    else
      return c->dim == 1   ? dgk::launch_stage2_f64_1d(c->order, c->variant, a, c->grid2, c->d_err, c->stream)
             : c->dim == 2 ? dgk::launch_stage2_f64_2d(c->order, c->variant, a, c->grid2, c->d_err, c->stream)
                           : dgk::launch_stage2_f64_3d(c->order, c->variant, a, c->grid2, c->d_err, c->stream);
  }
  if constexpr (sizeof(T) == 4)
    return c->dim == 1   ? dgk::launch_stage_f32_1d(c->order, a, c->grid, c->stream)
           : c->dim == 2 ? dgk::launch_stage_f32_2d(c->order, a, c->grid, c->stream)
                         : dgk::launch_stage_f32_3d(c->order, a, c->grid, c->stream);
  else
    return c->dim == 1   ? dgk::launch_stage_f64_1d(c->order, a, c->grid, c->stream)
           : c->dim == 2 ? dgk::launch_stage_f64_2d(c->order, a, c->grid, c->stream)
                         : dgk::launch_stage_f64_3d(c->order, a, c->grid, c->stream);
}

cudaError_t launch_stage(dg_ctx* c, int stage, const void* y_in, void* y_out, void* k_out, double dt) {
  // curved elements first: their right-hand side from the same stage input
  if (c->ncurved > 0) {
    cudaError_t e = dgc::launch_curved(c, y_in);
    if (e != cudaSuccess) return e;
  }
  if (c->prec == DG_FP32) return launch_stage_t<float>(c, stage, (const float*)y_in, (float*)y_out, (float*)k_out, dt);
  return launch_stage_t<double>(c, stage, (const double*)y_in, (double*)y_out, (double*)k_out, dt);
}

// Source overwrite before a step (k_inject on c->stream).
cudaError_t enqueue_inject(dg_ctx* c) {
  if (c->n_src_dofs > 0) {
    if (c->prec == DG_FP32)
      k_inject<float><<<nblk(c->n_src_dofs, 128), 128, 0, c->stream>>>(
          (float*)c->u, c->d_src_dof, c->d_src_off, c->d_src_ids, c->d_srcval, c->n_src, c->srcval_steps, c->d_step,
          c->n_src_dofs);
    else
      k_inject<double><<<nblk(c->n_src_dofs, 128), 128, 0, c->stream>>>(
          (double*)c->u, c->d_src_dof, c->d_src_off, c->d_src_ids, c->d_srcval, c->n_src, c->srcval_steps, c->d_step,
          c->n_src_dofs);
    return cudaGetLastError();
  }
  return cudaSuccess;
}

// Residual means (from nparts rows of stage-4 partial sums) and observer
// samples after a step, then the step counter (on c->stream).
cudaError_t enqueue_finalize(dg_ctx* c, int nparts) {
  const int64_t stride = c->Epad * c->np;
  double inv_count = 1.0 / (double)(c->E * c->np);
  // an observer with thousands of node slots is summed by several blocks:
  // the sums are FP64, whose rate per SM on GB300 bounds a single block
  if (c->prec == DG_FP32)
    launch_finalize<float>(c, nparts, inv_count, stride);
  else
    launch_finalize<double>(c, nparts, inv_count, stride);
  cudaError_t err = cudaGetLastError();
  if (err != cudaSuccess) return err;
  k_advance<<<1, 1, 0, c->stream>>>(c->d_step);
  return cudaGetLastError();
}

// One time step on c->stream. kind 0: RK4, 1: Euler1. ev (optional, 8
// events) brackets the stage launches for kernel timing.
cudaError_t enqueue_step(dg_ctx* c, int kind, double dt, cudaEvent_t* ev) {
  cudaError_t err;
  const int64_t stride = c->Epad * c->np;
  if ((err = enqueue_inject(c)) != cudaSuccess) return err;
  int nparts = c->variant >= 0 ? c->grid2 : c->grid;
  if (kind == 0) {
    const void* in[4] = {c->u, c->y0, c->y1, c->y0};
    void* out[4] = {c->y0, c->y1, c->y0, nullptr};
    for (int s = 0; s < 4; ++s) {
      if (ev) cudaEventRecord(ev[2 * s], c->stream);
      if ((err = launch_stage(c, s + 1, in[s], out[s], nullptr, dt)) != cudaSuccess) return err;
      if (ev) cudaEventRecord(ev[2 * s + 1], c->stream);
    }
  } else {
    if (ev) cudaEventRecord(ev[0], c->stream);
    if ((err = launch_stage(c, 5, c->u, c->y0, nullptr, dt)) != cudaSuccess) return err;
    if (ev) cudaEventRecord(ev[1], c->stream);
    const int cb = 2 * c->num_sms;
    nparts = cb;
    int64_t n = (int64_t)c->nv * stride;
    if (c->prec == DG_FP32)
      k_euler_commit<float><<<cb, 256, 0, c->stream>>>((float*)c->u, (const float*)c->y0, (const float*)c->snap, n,
                                                       stride, c->nv, c->c0sq, c->partials);
    else
      k_euler_commit<double><<<cb, 256, 0, c->stream>>>((double*)c->u, (const double*)c->y0, (const double*)c->snap,
                                                        n, stride, c->nv, c->c0sq, c->partials);
    if ((err = cudaGetLastError()) != cudaSuccess) return err;
  }
  return enqueue_finalize(c, nparts);
}

int ensure_out_cap(dg_ctx* c, int64_t n) {
  if (n <= c->out_cap) return DG_OK;
  int64_t cap = std::max<int64_t>(n, 1024);
  if (c->d_res) cudaFree(c->d_res);
  if (c->d_obs) cudaFree(c->d_obs);
  c->d_res = nullptr, c->d_obs = nullptr;
  CK(c, cudaMalloc(&c->d_res, cap * 5 * sizeof(double)));
  CK(c, cudaMalloc(&c->d_obs, cap * std::max(1, c->n_obs) * 4 * sizeof(double)));
  c->out_cap = cap;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  return DG_OK;
}

int build_graph(dg_ctx* c, int kind, double dt) {
  if (c->graph && c->graph_dt == dt && c->graph_kind == kind) return DG_OK;
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = enqueue_step(c, kind, dt, nullptr);
  cudaError_t err2 = cudaStreamEndCapture(c->stream, &g);
  if (err != cudaSuccess) return fail(c, DG_ERR_CUDA, std::string("CUDA (capture): ") + cudaGetErrorString(err));
  CK(c, err2);
  err = cudaGraphInstantiate(&c->graph, g, 0);
  cudaGraphDestroy(g);
  CK(c, err);
  c->graph_dt = dt;
  c->graph_kind = kind;
  return DG_OK;
}

int run_steps(dg_ctx* c, int kind, int64_t n_steps, double dt, double* residuals, double* obs) {
  if (!c) return DG_ERR_ARG;
  if (n_steps < 0 || !(dt > 0)) return fail(c, DG_ERR_ARG, "n_steps must be >= 0 and dt > 0");
  if (n_steps == 0) return DG_OK;
  int rc = ensure_out_cap(c, n_steps);
  if (rc) return rc;
  rc = build_graph(c, kind, dt);
  if (rc) return rc;
  int64_t st[2] = {c->step, c->step};
  CK(c, cudaMemcpyAsync(c->d_step, st, sizeof(st), cudaMemcpyHostToDevice, c->stream));
  for (int64_t i = 0; i < n_steps; ++i) CK(c, cudaGraphLaunch(c->graph, c->stream));
  std::vector<double> res(n_steps * 5);
  CK(c, cudaMemcpyAsync(res.data(), c->d_res, n_steps * 5 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (obs && c->n_obs > 0)
    CK(c, cudaMemcpyAsync(obs, c->d_obs, n_steps * c->n_obs * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  int herr = 0;
  CK(c, cudaMemcpyAsync(&herr, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->step += n_steps;
  if (residuals) std::memcpy(residuals, res.data(), res.size() * sizeof(double));
  if (herr) {
    // the kernels that gave up drained their own copies before exiting; the
    // flag is cleared so that the context stays usable
    CK(c, cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return fail(c, DG_ERR_TIMEOUT, "a bounded device wait gave up (TMA copy did not complete)");
  }
  for (double v : res)
    if (!std::isfinite(v)) return fail(c, DG_ERR_NONFINITE, "non-finite values in the state (residual is NaN/Inf)");
  return DG_OK;
}

template <typename T>
void to_dev_ops(const dgref::RefElement& re, std::vector<T>& Dt, std::vector<T>& L) {
  const int np = re.np, D = re.dim, nk = re.nf * re.nfp;
  Dt.resize(D * np * np);
  for (int r = 0; r < D; ++r)
    for (int j = 0; j < np; ++j)
      for (int i = 0; i < np; ++i) Dt[(r * np + j) * np + i] = (T)re.Dt[(r * np + i) * np + j];
  L.resize(nk * np);
  for (int k = 0; k < nk; ++k)
    for (int i = 0; i < np; ++i) L[k * np + i] = (T)re.LIFT[i * nk + k];
}


// The tensor-core, constant-operator and flux-form kernels have no
// curved-element path; the baseline and pipelined kernels take the curved
// right-hand side.
bool variant_handles_mesh(const dg_ctx* c, int v) {
  return c->ncurved == 0 || !(dgk::is_tc_variant(v) || v >= dgk::kStage3Variant);
}

dgk::Stage2Info stage2_info(const dg_ctx* c, int v) {
  if (dgk::is_wide_variant(v))
    return c->prec == DG_FP32 ? dgk::stage4_info(c->dim, c->order, v - dgk::kWideVariant)
                              : dgk::Stage2Info{0, 0, 0, 0, 0, 0};
  if (v >= dgk::kStage3Variant)
    return c->prec == DG_FP32 && dgk::is_stage3_variant(v) ? dgk::stage3_info(c->dim, c->order, v - dgk::kStage3Variant)
                                                           : dgk::Stage2Info{0, 0, 0, 0, 0, 0};
  if (dgk::is_tc_variant(v))
    return c->prec != DG_FP32        ? dgk::Stage2Info{0, 0, 0, 0, 0, 0}
           : dgk::is_tc3_variant(v) ? dgk::stage_tc3_info(c->dim, c->order, dgk::tc_npart(v))
           : dgk::is_tc2_variant(v) ? dgk::stage_tc2_info(c->dim, c->order, dgk::tc_npart(v))
                                    : dgk::stage_tc_info(c->dim, c->order, dgk::tc_npart(v));
  if (c->prec == DG_FP32)
    return c->dim == 1   ? dgk::stage2_info_f32_1d(c->order, v)
           : c->dim == 2 ? dgk::stage2_info_f32_2d(c->order, v)
                         : dgk::stage2_info_f32_3d(c->order, v);
  return c->dim == 1   ? dgk::stage2_info_f64_1d(c->order, v)
         : c->dim == 2 ? dgk::stage2_info_f64_2d(c->order, v)
                       : dgk::stage2_info_f64_3d(c->order, v);
}

// Selects the stage kernel: -1 baseline, k >= 0 pipelined variant k,
// kTcVariant .. kTcVariant + 6 the tensor-core kernels, kStage3Variant + k
// constant-operator variant k, kWideVariant + k flux-form variant k (the
// last three FP32).
bool set_variant(dg_ctx* c, int v) {
  if (v < 0) {
    c->variant = -1;
    return true;
  }
  if (!variant_handles_mesh(c, v)) return false;
  dgk::Stage2Info si = stage2_info(c, v);
  if (si.nc == 0 || si.blocks_per_sm <= 0 || c->Epad % si.et != 0) return false;
  if (dgk::is_stage3_variant(v)) {
    // the constant-operator kernels read Dt [r][i][j] and LIFT [k][i] from
    // constant memory (uploaded once per device and element type)
    const int np = c->re.np, D = c->re.dim, nk = c->re.nf * c->re.nfp;
    std::vector<float> dt((size_t)D * np * np), lift((size_t)nk * np);
    for (size_t i = 0; i < dt.size(); ++i) dt[i] = (float)c->re.Dt[i];
    for (int k = 0; k < nk; ++k)
      for (int i = 0; i < np; ++i) lift[(size_t)k * np + i] = (float)c->re.LIFT[(size_t)i * nk + k];
    if (dgk::stage3_upload_ops(c->dim, c->order, dt.data(), lift.data()) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
  }
  c->variant = v;
  c->s2 = si;
  c->grid2 = (int)std::min<int64_t>(c->Epad / si.et, (int64_t)si.blocks_per_sm * c->num_sms);
  if (c->graph) cudaGraphExecDestroy(c->graph), c->graph = nullptr;
  return true;
}

// Autotuner results, cached per (GPU model, dimension, order, precision,
// mesh size class): in the process, and in the file named by
// DGFEM_TUNE_CACHE when it is set (one "key<TAB>variant" line per result;
// a later line for the same key wins).
struct TuneCache {
  std::mutex mu;
  std::map<std::string, int> entries;
  std::map<std::string, bool> files_read;
  int64_t hits = 0, misses = 0;
};
TuneCache& tune_cache() {
  static TuneCache tc;
  return tc;
}

std::string tune_key(const dg_ctx* c) {
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess) {
    cudaGetLastError();
    return std::string();
  }
  int size_class = 0;
  while (size_class < 62 && ((int64_t)1 << (size_class + 1)) <= c->Epad) ++size_class;
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s|cc%d.%d|sm%d|d%d|p%d|%s|e2^%d", prop.name, prop.major, prop.minor,
                prop.multiProcessorCount, c->dim, c->order, c->prec == DG_FP32 ? "fp32" : "fp64", size_class);
  for (char* q = buf; *q; ++q)
    if (*q == '\t' || *q == '\n') *q = ' ';
  return buf;
}

// caller holds the cache lock
void tune_cache_read_file(TuneCache& tc, const char* path) {
  if (!path || !*path || tc.files_read[path]) return;
  tc.files_read[path] = true;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  char line[768];
  while (std::fgets(line, sizeof(line), f)) {
    char* tab = std::strrchr(line, '\t');
    if (!tab) continue;
    *tab = 0;
    char* end = nullptr;
    long v = std::strtol(tab + 1, &end, 10);
    if (end == tab + 1) continue;
    tc.entries[line] = (int)v;
  }
  std::fclose(f);
}

bool tune_cache_lookup(const std::string& key, int* v) {
  if (key.empty()) return false;
  TuneCache& tc = tune_cache();
  std::lock_guard<std::mutex> lk(tc.mu);
  tune_cache_read_file(tc, std::getenv("DGFEM_TUNE_CACHE"));
  auto it = tc.entries.find(key);
  if (it == tc.entries.end()) {
    ++tc.misses;
    return false;
  }
  ++tc.hits;
  *v = it->second;
  return true;
}

void tune_cache_store(const std::string& key, int v) {
  if (key.empty()) return;
  TuneCache& tc = tune_cache();
  std::lock_guard<std::mutex> lk(tc.mu);
  tc.entries[key] = v;
  const char* path = std::getenv("DGFEM_TUNE_CACHE");
  if (!path || !*path) return;
  if (FILE* f = std::fopen(path, "a")) {
    std::fprintf(f, "%s\t%d\n", key.c_str(), v);
    std::fclose(f);
  }
}

// Autotuner: times RK stages 1-3 (stage input, u and accumulator reads;
// accumulator and next-stage writes) of every kernel variant on this mesh
// and keeps the fastest. want >= -1 forces a variant instead; want == -3
// takes a cached result for this GPU model, element type, precision and mesh
// size class where one exists (what context creation does) and times the
// variants otherwise; want == -2 always times them. Timed results are cached.
int select_variant(dg_ctx* c, int want) {
  if (want >= -1) {
    if (!set_variant(c, want)) return fail(c, DG_ERR_ARG, "stage kernel variant not available");
    return DG_OK;
  }
  const std::string key = tune_key(c);
  if (want == -3) {
    int v = -1;
    if (tune_cache_lookup(key, &v) && set_variant(c, v)) return DG_OK;
  }
  std::vector<int> cands{-1};
  for (int v = 0; v < 8; ++v) {
    dgk::Stage2Info si = stage2_info(c, v);
    if (si.nc == 0) break;
    if (si.blocks_per_sm > 0) cands.push_back(v);
  }
  for (int v = dgk::kTcVariant; v < dgk::kTcVariant + dgk::kTcVariants; ++v) {
    dgk::Stage2Info si = stage2_info(c, v);
    if (si.nc > 0 && si.blocks_per_sm > 0) cands.push_back(v);
  }
  for (int k = 0; k < 8; ++k) {
    dgk::Stage2Info si = stage2_info(c, dgk::kStage3Variant + k);
    if (si.nc == 0) break;
    if (si.blocks_per_sm > 0) cands.push_back(dgk::kStage3Variant + k);
  }
  for (int k = 0; k < 16; ++k) {
    dgk::Stage2Info si = stage2_info(c, dgk::kWideVariant + k);
    if (si.nc == 0) break;
    if (si.blocks_per_sm > 0) cands.push_back(dgk::kWideVariant + k);
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // the caches are flushed before each timed repetition (a write larger than
  // L2), as a stage of a real step finds them after the other stages' traffic
  const int64_t flush_words = (int64_t)64 << 20;  // 256 MiB
  unsigned* flush = nullptr;
  if (cudaMalloc(&flush, flush_words * sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    flush = nullptr;
  }
  float best = 1e30f;
  int best_v = -1;
  // the four stages of an RK step (their operand mixes differ); stage 4
  // updates a stage buffer in place of the state, which stays untouched
  auto rk_stages = [&]() {
    cudaError_t err = cudaSuccess;
    for (int st = 1; st <= 3 && err == cudaSuccess; ++st) err = launch_stage(c, st, c->y0, c->y1, nullptr, 1e-30);
    if (err == cudaSuccess) {
      void* u = c->u;
      c->u = c->y1;
      err = launch_stage(c, 4, c->y0, nullptr, nullptr, 1e-30);
      c->u = u;
    }
    return err;
  };
  for (int v : cands) {
    if (!set_variant(c, v)) continue;
    // once to warm up, then three times timed
    cudaError_t err = rk_stages();
    float tot = 0.f;
    for (int r = 0; r < 3 && err == cudaSuccess; ++r) {
      if (flush) k_flush<<<2 * c->num_sms, 512, 0, c->stream>>>(flush, flush_words, (unsigned)r);
      cudaEventRecord(e0, c->stream);
      err = rk_stages();
      cudaEventRecord(e1, c->stream);
      if (err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
      float ms = 0.f;
      if (err == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
      tot += ms;
    }
    if (err != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (flush) cudaFree(flush);
      return fail(c, DG_ERR_CUDA, std::string("CUDA (autotune): ") + cudaGetErrorString(err));
    }
    if (tot < best) best = tot, best_v = v;
  }
  if (flush) cudaFree(flush);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  // the timing runs wrote the accumulator, the stage buffers and the
  // residual partial sums only; clear the buffers
  const size_t nb = (size_t)c->nv * c->Epad * c->np * c->tsize;
  cudaMemsetAsync(c->acc, 0, nb, c->stream);
  cudaMemsetAsync(c->y0, 0, nb, c->stream);
  cudaMemsetAsync(c->y1, 0, nb, c->stream);
  cudaStreamSynchronize(c->stream);
  set_variant(c, best_v);
  tune_cache_store(key, best_v);
  return DG_OK;
}

}  // namespace

namespace dgc {
void set_global_error(const std::string& m) { g_create_error = m; }
cudaError_t enqueue_step(dg_ctx* c, int kind, double dt, cudaEvent_t* ev) { return ::enqueue_step(c, kind, dt, ev); }
cudaError_t enqueue_inject(dg_ctx* c) { return ::enqueue_inject(c); }
cudaError_t enqueue_finalize(dg_ctx* c, int nparts) { return ::enqueue_finalize(c, nparts); }
dgk::StageArgs<float> stage_args_f32(dg_ctx* c, int stage, const float* y_in, float* y_out, double dt) {
  return ::stage_args<float>(c, stage, y_in, y_out, nullptr, dt);
}
int ensure_out_cap(dg_ctx* c, int64_t n) { return ::ensure_out_cap(c, n); }
int create_ctx(const dg_mesh_desc* mesh, const dg_phys* phys, int precision, int device, const double* elem_v0,
               const double* elem_scale, dg_ctx** out, std::string* err);

cudaError_t dev_alloc(dg_ctx* c, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes + 64);
  if (e == cudaSuccess) {
    c->allocs.push_back(*p);
    c->device_bytes += (int64_t)bytes;
  }
  return e;
}
}  // namespace dgc

extern "C" {

const char* dg_last_error(const dg_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

int dg_create(const dg_mesh_desc* mesh, const dg_phys* phys, int precision, int device, dg_ctx** out) {
  std::string e;
  int rc = dgc::create_ctx(mesh, phys, precision, device, nullptr, nullptr, out, &e);
  if (rc != DG_OK) g_create_error = e;
  return rc;
}

}  // extern "C"

int dgc::create_ctx(const dg_mesh_desc* mesh, const dg_phys* phys, int precision, int device, const double* elem_v0,
                    const double* elem_scale, dg_ctx** out, std::string* err) {
  if (!out) return DG_ERR_ARG;
  *out = nullptr;
  auto bad = [&](int code, const std::string& m) {
    *err = m;
    return code;
  };
  if (!mesh || !phys || !mesh->xyz || !mesh->elem_nodes) return bad(DG_ERR_ARG, "null mesh or physics");
  if (mesh->dim < 1 || mesh->dim > 3) return bad(DG_ERR_ARG, "dim must be 1, 2 or 3");
  if (mesh->dim == 1)
    for (int64_t k = 0; k < mesh->n_nodes; ++k)
      if (mesh->xyz[3 * k + 1] != 0.0 || mesh->xyz[3 * k + 2] != 0.0)
        return bad(DG_ERR_MESH, "1-D meshes must lie on the x axis (y = z = 0)");
  if (mesh->order < 1 || mesh->order > 4) return bad(DG_ERR_ARG, "order must be 1..4");
  if (precision != DG_FP64 && precision != DG_FP32) return bad(DG_ERR_ARG, "precision must be DG_FP64 or DG_FP32");
  if (mesh->n_elems <= 0 || mesh->n_nodes <= 0) return bad(DG_ERR_ARG, "empty mesh");
  if (mesh->n_groups < 0 || mesh->n_groups > 32) return bad(DG_ERR_ARG, "at most 32 boundary groups");
  if (mesh->n_groups > 0 && (!mesh->group_bc || !mesh->group_offsets || !mesh->group_nodes))
    return bad(DG_ERR_ARG, "null group arrays");
  if (!(phys->rho0 > 0) || !(phys->c0 > 0)) return bad(DG_ERR_ARG, "rho0 and c0 must be positive");
  auto* c = new dg_ctx;
  c->dim = mesh->dim, c->order = mesh->order, c->prec = precision, c->device = device;
  try {
    c->re = dgref::build(c->dim, c->order);
  } catch (const std::exception& e) {
    delete c;
    return bad(DG_ERR_ARG, e.what());
  }
  c->sh = dgk::shape_info(c->dim, c->order);
  c->np = c->re.np, c->nf = c->re.nf, c->nfp = c->re.nfp, c->nv = c->dim + 1;
  if (mesh->nodes_per_elem != c->np) {
    delete c;
    return bad(DG_ERR_ARG, "nodes_per_elem does not match dim/order");
  }
  c->E = mesh->n_elems, c->nnodes = mesh->n_nodes;
  c->Epad = (c->E + dgk::kElemAlign - 1) / dgk::kElemAlign * dgk::kElemAlign;
  c->ntiles = c->Epad / c->sh.et;
  if (c->Epad >= (int64_t)1 << 31) {
    delete c;
    return bad(DG_ERR_ARG, "too many elements");
  }
  c->tsize = precision == DG_FP32 ? 4 : 8;
  for (int d = 0; d < 3; ++d) c->ph.v0[d] = phys->v0[d];
  c->ph.rho0 = phys->rho0, c->ph.c0 = phys->c0;
  c->ph.rhoc2 = phys->rho0 * phys->c0 * phys->c0;
  c->ph.inv_rho0 = 1.0 / phys->rho0;
  c->ph.half_c0 = 0.5 * phys->c0;
  c->c0sq = phys->c0 * phys->c0;
  // node permutation from element 0 (checked on every element by the setup)
  {
    const int D = c->dim, np = c->np;
    for (int64_t k = 0; k < (int64_t)c->E * np; ++k)
      if (mesh->elem_nodes[k] < 0 || mesh->elem_nodes[k] >= mesh->n_nodes) {
        delete c;
        return bad(DG_ERR_ARG, "element node index out of range");
      }
    const int64_t* en = mesh->elem_nodes;
    const double* x0 = mesh->xyz + 3 * en[0];
    double J[3][3] = {{0}}, Gi[3][3] = {{0}};
    for (int k = 0; k < D; ++k)
      for (int d = 0; d < D; ++d) J[d][k] = mesh->xyz[3 * en[k + 1] + d] - x0[d];
    if (D == 1) {
      Gi[0][0] = 1.0 / J[0][0];
    } else if (D == 2) {
      double dt = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      Gi[0][0] = J[1][1] / dt, Gi[0][1] = -J[0][1] / dt, Gi[1][0] = -J[1][0] / dt, Gi[1][1] = J[0][0] / dt;
    } else {
      double dt = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                  J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
      Gi[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / dt;
      Gi[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / dt;
      Gi[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / dt;
      Gi[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / dt;
      Gi[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / dt;
      Gi[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / dt;
      Gi[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / dt;
      Gi[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / dt;
      Gi[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / dt;
    }
    c->perm_c2i.assign(np, -1);
    std::vector<int> used(np, 0);
    for (int n = 0; n < np; ++n) {
      int lat[3] = {0, 0, 0};
      for (int r = 0; r < D; ++r) {
        double xi = 0.0;
        for (int d = 0; d < D; ++d) xi += Gi[r][d] * (mesh->xyz[3 * en[n] + d] - x0[d]);
        lat[r] = (int)std::lround(xi * c->order);
      }
      int idx = dgref::lattice_index(c->re, lat);
      if (idx < 0 || used[idx]) {
        delete c;
        return bad(DG_ERR_MESH, "element 0 nodes do not form a straight-sided Lagrange lattice");
      }
      used[idx] = 1;
      c->perm_c2i[n] = idx;
    }
  }
  // device, stream, buffers
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    std::string m = std::string("CUDA: ") + cudaGetErrorString(e);
    dg_destroy(c);
    return bad(DG_ERR_CUDA, m);
  }
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(t0, c->stream);
  int rc = dgc::run_setup(c, mesh, elem_v0, elem_scale);
  if (rc != DG_OK) {
    std::string m = c->err;
    dg_destroy(c);
    return bad(rc, m);
  }
  // blocks per SM for the persistent stage kernel
  int bps = 1;
  if (c->prec == DG_FP32)
    bps = c->dim == 1   ? dgk::blocks_per_sm_f32_1d(c->order)
          : c->dim == 2 ? dgk::blocks_per_sm_f32_2d(c->order)
                        : dgk::blocks_per_sm_f32_3d(c->order);
  else
    bps = c->dim == 1   ? dgk::blocks_per_sm_f64_1d(c->order)
          : c->dim == 2 ? dgk::blocks_per_sm_f64_2d(c->order)
                        : dgk::blocks_per_sm_f64_3d(c->order);
  c->grid = (int)std::min<int64_t>(c->ntiles, (int64_t)bps * c->num_sms);
  const size_t ts = c->tsize;
  const int64_t nstate = (int64_t)c->nv * c->Epad * c->np;
  void** bufs[6] = {&c->u, &c->acc, &c->y0, &c->y1, &c->snap, &c->kbuf};
  for (auto b : bufs) {
    e = dgc::dev_alloc(c, b, nstate * ts);
    if (e == cudaSuccess) e = cudaMemsetAsync(*b, 0, nstate * ts, c->stream);
    if (e != cudaSuccess) break;
  }
  std::vector<short> fm(c->re.fmask.begin(), c->re.fmask.end()), nb(c->re.nbrnode.begin(), c->re.nbrnode.end());
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->fmask, fm.size() * sizeof(short));
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->nbrnode, nb.size() * sizeof(short));
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->fmask, fm.data(), fm.size() * sizeof(short), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->nbrnode, nb.data(), nb.size() * sizeof(short), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) {
    if (c->prec == DG_FP32) {
      std::vector<float> Dt, L;
      to_dev_ops(c->re, Dt, L);
      e = dgc::dev_alloc(c, &c->Dt, Dt.size() * 4);
      if (e == cudaSuccess) e = dgc::dev_alloc(c, &c->LIFT, L.size() * 4);
      if (e == cudaSuccess) e = cudaMemcpyAsync(c->Dt, Dt.data(), Dt.size() * 4, cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(c->LIFT, L.data(), L.size() * 4, cudaMemcpyHostToDevice, c->stream);
    } else {
      std::vector<double> Dt, L;
      to_dev_ops(c->re, Dt, L);
      e = dgc::dev_alloc(c, &c->Dt, Dt.size() * 8);
      if (e == cudaSuccess) e = dgc::dev_alloc(c, &c->LIFT, L.size() * 8);
      if (e == cudaSuccess) e = cudaMemcpyAsync(c->Dt, Dt.data(), Dt.size() * 8, cudaMemcpyHostToDevice, c->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(c->LIFT, L.data(), L.size() * 8, cudaMemcpyHostToDevice, c->stream);
    }
  }
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->d_perm, c->np * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->d_perm, c->perm_c2i.data(), c->np * sizeof(int), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->d_ref, 4 * c->E * c->np * sizeof(double));
  c->max_grid = std::max(c->grid, 2 * c->num_sms);
  for (int v = 0; v < 8; ++v) {
    dgk::Stage2Info si = stage2_info(c, v);
    if (si.nc == 0) break;
    c->max_grid = std::max<int>(c->max_grid, (int)std::min<int64_t>(c->Epad / si.et, (int64_t)si.blocks_per_sm * c->num_sms));
  }
  for (int v = dgk::kTcVariant; v < dgk::kTcVariant + dgk::kTcVariants; ++v) {
    dgk::Stage2Info si = stage2_info(c, v);
    if (si.nc > 0)
      c->max_grid = std::max<int>(c->max_grid, (int)std::min<int64_t>(c->Epad / si.et, (int64_t)si.blocks_per_sm * c->num_sms));
  }
  for (int k = 0; k < 8; ++k) {
    dgk::Stage2Info si = stage2_info(c, dgk::kStage3Variant + k);
    if (si.nc == 0) break;
    c->max_grid = std::max<int>(c->max_grid, (int)std::min<int64_t>(c->Epad / si.et, (int64_t)si.blocks_per_sm * c->num_sms));
  }
  for (int k = 0; k < 16; ++k) {
    dgk::Stage2Info si = stage2_info(c, dgk::kWideVariant + k);
    if (si.nc == 0) break;
    c->max_grid = std::max<int>(c->max_grid, (int)std::min<int64_t>(c->Epad / si.et, (int64_t)si.blocks_per_sm * c->num_sms));
  }
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->partials, c->max_grid * 5 * sizeof(double));
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = dgc::dev_alloc(c, (void**)&c->d_step, 2 * sizeof(int64_t));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_step, 0, 2 * sizeof(int64_t), c->stream);
  cudaEventRecord(t1, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    std::string m = std::string("CUDA: ") + cudaGetErrorString(e);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    dg_destroy(c);
    return bad(DG_ERR_CUDA, m);
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, t0, t1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  c->info.dim = c->dim, c->info.order = c->order, c->info.nodes_per_elem = c->np, c->info.n_var = c->nv;
  c->info.precision = c->prec, c->info.n_elems = c->E, c->info.n_faces = c->n_faces;
  c->info.n_curved = c->ncurved;
  c->info.n_boundary_faces = c->n_bfaces;
  c->info.device_bytes = c->device_bytes;
  c->info.setup_ms = ms;
  {
    // DGFEM_STAGE_VARIANT forces a kernel where it exists for this context
    // (e.g. the tensor-core kernel only for FP32); elsewhere the autotuner picks
    const char* ev = std::getenv("DGFEM_STAGE_VARIANT");
    int want = ev ? std::atoi(ev) : -3;
    int rc2 = select_variant(c, want);
    if (rc2 == DG_ERR_ARG && ev) rc2 = select_variant(c, -3);
    if (rc2 != DG_OK) {
      std::string m = c->err;
      dg_destroy(c);
      return bad(rc2, m);
    }
  }
  c->info.kernel_variant = c->variant;
  c->info.kernel_grid = c->variant >= 0 ? c->grid2 : c->grid;
  *out = c;
  return DG_OK;
}

extern "C" {

int dg_destroy(dg_ctx* c) {
  if (!c) return DG_OK;
  if (c->graph) cudaGraphExecDestroy(c->graph);
  for (void* p : c->allocs) cudaFree(p);
  void* extra[] = {c->d_res, c->d_obs, c->d_src_dof, c->d_src_off, c->d_src_ids, c->d_srcval,
                   c->d_obs_dof, c->d_obs_off, c->d_obs_w, c->d_obs_part, c->d_obs_cnt, c->d_obs_bmap,
                   c->d_obs_bfirst};
  for (void* p : extra)
    if (p) cudaFree(p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return DG_OK;
}

int dg_get_info(const dg_ctx* c, dg_info_t* info) {
  if (!c || !info) return DG_ERR_ARG;
  *info = c->info;
  info->device_bytes = c->device_bytes;
  return DG_OK;
}

int dg_set_state(dg_ctx* c, const double* u) {
  if (!c || !u) return DG_ERR_ARG;
  const int64_t n = 4 * c->E * c->np;
  if (c->dim == 2)
    for (int64_t i = 3 * c->E * c->np; i < n; ++i)
      if (u[i] != 0.0) return fail(c, DG_ERR_ARG, "2-D state must have vz = 0");
  CK(c, cudaMemcpyAsync(c->d_ref, u, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  // the padding elements past E take part in every stage (their geometry is
  // zero, so a finite state stays zero there); they are cleared so that a
  // non-finite state of an earlier run cannot stay behind in them
  if (c->Epad > c->E) {
    const size_t w = c->prec == DG_FP32 ? 4 : 8;
    for (int q = 0; q < c->nv; ++q)
      CK(c, cudaMemsetAsync((char*)c->u + ((size_t)q * c->Epad + c->E) * c->np * w, 0,
                            (size_t)(c->Epad - c->E) * c->np * w, c->stream));
  }
  int64_t m = (int64_t)c->nv * c->E * c->np;
  if (c->prec == DG_FP32)
    k_ref_to_int<float><<<nblk(m, 256), 256, 0, c->stream>>>(c->d_ref, (float*)c->u, c->d_perm, c->E, c->np, c->nv,
                                                             c->Epad * c->np);
  else
    k_ref_to_int<double><<<nblk(m, 256), 256, 0, c->stream>>>(c->d_ref, (double*)c->u, c->d_perm, c->E, c->np, c->nv,
                                                              c->Epad * c->np);
  CK(c, cudaGetLastError());
  CK(c, cudaStreamSynchronize(c->stream));
  return DG_OK;
}

int dg_get_state(dg_ctx* c, double* u) {
  if (!c || !u) return DG_ERR_ARG;
  const int64_t n = 4 * c->E * c->np;
  if (c->prec == DG_FP32)
    k_int_to_ref<float><<<nblk(n, 256), 256, 0, c->stream>>>((const float*)c->u, c->d_ref, c->d_perm, c->E, c->np,
                                                             c->nv, c->Epad * c->np);
  else
    k_int_to_ref<double><<<nblk(n, 256), 256, 0, c->stream>>>((const double*)c->u, c->d_ref, c->d_perm, c->E, c->np,
                                                              c->nv, c->Epad * c->np);
  CK(c, cudaGetLastError());
  CK(c, cudaMemcpyAsync(u, c->d_ref, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return DG_OK;
}

int dg_set_sources(dg_ctx* c, int n_src, const int64_t* offsets, const int64_t* dofs) {
  if (!c || n_src < 0 || (n_src > 0 && !offsets)) return DG_ERR_ARG;
  // sources may cover no dof at all (a radius with no node inside): then
  // dofs may be null
  if (n_src > 0 && offsets[n_src] > 0 && !dofs) return fail(c, DG_ERR_ARG, "dg_set_sources: dofs is null");
  // unique internal dofs, each with the ordered list of sources covering it
  std::map<int64_t, std::vector<int>> cover;
  const int64_t ndof = c->E * c->np;
  for (int s = 0; s < n_src; ++s)
    for (int64_t k = offsets[s]; k < offsets[s + 1]; ++k) {
      int64_t d = dofs[k];
      if (d < 0 || d >= ndof) return fail(c, DG_ERR_ARG, "source dof out of range");
      int64_t e = d / c->np;
      int n = (int)(d - e * c->np);
      int64_t idof = e * c->np + c->perm_c2i[n];
      auto& v = cover[idof];
      if (v.empty() || v.back() != s) v.push_back(s);
    }
  std::vector<int64_t> hd;
  std::vector<int> ho(1, 0), hi;
  for (auto& kv : cover) {
    hd.push_back(kv.first);
    for (int s : kv.second) hi.push_back(s);
    ho.push_back((int)hi.size());
  }
  for (void* p : {(void*)c->d_src_dof, (void*)c->d_src_off, (void*)c->d_src_ids})
    if (p) cudaFree(p);
  c->d_src_dof = nullptr, c->d_src_off = nullptr, c->d_src_ids = nullptr;
  c->n_src = n_src;
  c->n_src_dofs = (int64_t)hd.size();
  if (c->graph) cudaGraphExecDestroy(c->graph), c->graph = nullptr;
  if (hd.empty()) return DG_OK;
  CK(c, cudaMalloc(&c->d_src_dof, hd.size() * sizeof(int64_t)));
  CK(c, cudaMalloc(&c->d_src_off, ho.size() * sizeof(int)));
  CK(c, cudaMalloc(&c->d_src_ids, hi.size() * sizeof(int)));
  CK(c, cudaMemcpyAsync(c->d_src_dof, hd.data(), hd.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  CK(c, cudaMemcpyAsync(c->d_src_off, ho.data(), ho.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  CK(c, cudaMemcpyAsync(c->d_src_ids, hi.data(), hi.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return DG_OK;
}

int dg_set_source_values(dg_ctx* c, int64_t n_steps, const double* values) {
  if (!c || n_steps < 0 || (n_steps > 0 && c->n_src > 0 && !values)) return DG_ERR_ARG;
  if (c->d_srcval) cudaFree(c->d_srcval), c->d_srcval = nullptr;
  c->srcval_steps = 0;
  if (c->graph) cudaGraphExecDestroy(c->graph), c->graph = nullptr;
  if (n_steps == 0 || c->n_src == 0) return DG_OK;
  CK(c, cudaMalloc(&c->d_srcval, n_steps * c->n_src * sizeof(double)));
  CK(c, cudaMemcpyAsync(c->d_srcval, values, n_steps * c->n_src * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  c->srcval_steps = n_steps;
  return DG_OK;
}

int dg_set_observers(dg_ctx* c, int n_obs, const int64_t* offsets, const int64_t* dofs, const double* weights) {
  if (!c || n_obs < 0 || (n_obs > 0 && !offsets)) return DG_ERR_ARG;
  if (n_obs > 0 && offsets[n_obs] > 0 && (!dofs || !weights))
    return fail(c, DG_ERR_ARG, "dg_set_observers: dofs or weights is null");
  for (void* p : {(void*)c->d_obs_dof, (void*)c->d_obs_off, (void*)c->d_obs_w, (void*)c->d_obs_part,
                  (void*)c->d_obs_cnt, (void*)c->d_obs_bmap, (void*)c->d_obs_bfirst})
    if (p) cudaFree(p);
  c->d_obs_dof = nullptr, c->d_obs_off = nullptr, c->d_obs_w = nullptr, c->d_obs_part = nullptr;
  c->d_obs_cnt = nullptr, c->d_obs_bmap = nullptr, c->d_obs_bfirst = nullptr;
  c->obs_blocks = n_obs;
  c->obs_small = true;
  c->n_obs = n_obs;
  if (c->d_obs) cudaFree(c->d_obs), c->d_obs = nullptr;
  if (c->d_res) cudaFree(c->d_res), c->d_res = nullptr;
  c->out_cap = 0;
  if (c->graph) cudaGraphExecDestroy(c->graph), c->graph = nullptr;
  if (n_obs == 0) return DG_OK;
  int64_t total = offsets[n_obs];
  std::vector<int64_t> hd(std::max<int64_t>(total, 1));
  const int64_t ndof = c->E * c->np;
  for (int64_t k = 0; k < total; ++k) {
    int64_t d = dofs[k];
    if (d < 0 || d >= ndof) return fail(c, DG_ERR_ARG, "observer dof out of range");
    int64_t e = d / c->np;
    hd[k] = e * c->np + c->perm_c2i[d - e * c->np];
  }
  CK(c, cudaMalloc(&c->d_obs_dof, hd.size() * sizeof(int64_t)));
  CK(c, cudaMalloc(&c->d_obs_off, (n_obs + 1) * sizeof(int64_t)));
  CK(c, cudaMalloc(&c->d_obs_w, std::max<int64_t>(total, 1) * sizeof(double)));
  CK(c, cudaMemcpyAsync(c->d_obs_dof, hd.data(), hd.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  CK(c, cudaMemcpyAsync(c->d_obs_off, offsets, (n_obs + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (total > 0) {
    CK(c, cudaMemcpyAsync(c->d_obs_w, weights, total * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  // blocks per observer: one node slot per thread, at most 64 blocks each
  int64_t most = 0;
  for (int o = 0; o < n_obs; ++o) most = std::max<int64_t>(most, offsets[o + 1] - offsets[o]);
  c->obs_small = most <= kFinalizeThreadsSmall;
  if (most > kFinalizeThreads) {
    std::vector<int> bfirst(n_obs + 1, 0), bmap;
    for (int o = 0; o < n_obs; ++o) {
      const int64_t n = offsets[o + 1] - offsets[o];
      const int b = (int)std::min<int64_t>(64, std::max<int64_t>(1, (n + kFinalizeThreads - 1) / kFinalizeThreads));
      bfirst[o + 1] = bfirst[o] + b;
      for (int k = 0; k < b; ++k) bmap.push_back(o);
    }
    const int nb = bfirst[n_obs];
    CK(c, cudaMalloc(&c->d_obs_part, (size_t)nb * 5 * sizeof(double)));
    CK(c, cudaMalloc(&c->d_obs_cnt, (size_t)n_obs * sizeof(unsigned)));
    CK(c, cudaMalloc(&c->d_obs_bmap, (size_t)nb * sizeof(int)));
    CK(c, cudaMalloc(&c->d_obs_bfirst, (size_t)(n_obs + 1) * sizeof(int)));
    CK(c, cudaMemsetAsync(c->d_obs_cnt, 0, (size_t)n_obs * sizeof(unsigned), c->stream));
    CK(c, cudaMemcpyAsync(c->d_obs_bmap, bmap.data(), (size_t)nb * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->d_obs_bfirst, bfirst.data(), (size_t)(n_obs + 1) * sizeof(int), cudaMemcpyHostToDevice,
                          c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    c->obs_blocks = nb;
  }
  return DG_OK;
}

int dg_snapshot(dg_ctx* c) {
  if (!c) return DG_ERR_ARG;
  CK(c, cudaMemcpyAsync(c->snap, c->u, (size_t)c->nv * c->Epad * c->np * c->tsize, cudaMemcpyDeviceToDevice,
                        c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return DG_OK;
}

int dg_run(dg_ctx* c, int64_t n_steps, double dt, double* residuals, double* obs) {
  return run_steps(c, 0, n_steps, dt, residuals, obs);
}

int dg_run_euler(dg_ctx* c, int64_t n_steps, double dt, double* residuals, double* obs) {
  return run_steps(c, 1, n_steps, dt, residuals, obs);
}

int64_t dg_step_index(const dg_ctx* c) { return c ? c->step : -1; }

int dg_set_step_index(dg_ctx* c, int64_t step) {
  if (!c || step < 0) return DG_ERR_ARG;
  c->step = step;
  return DG_OK;
}

int dg_rhs(dg_ctx* c, const double* u, double dt, double* k) {
  if (!c || !u || !k) return DG_ERR_ARG;
  const int64_t n = 4 * c->E * c->np, m = (int64_t)c->nv * c->E * c->np, stride = c->Epad * c->np;
  CK(c, cudaMemcpyAsync(c->d_ref, u, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  if (c->prec == DG_FP32)
    k_ref_to_int<float><<<nblk(m, 256), 256, 0, c->stream>>>(c->d_ref, (float*)c->y1, c->d_perm, c->E, c->np, c->nv,
                                                             stride);
  else
    k_ref_to_int<double><<<nblk(m, 256), 256, 0, c->stream>>>(c->d_ref, (double*)c->y1, c->d_perm, c->E, c->np,
                                                              c->nv, stride);
  CK(c, cudaGetLastError());
  CK(c, launch_stage(c, 0, c->y1, nullptr, c->kbuf, dt));
  if (c->prec == DG_FP32)
    k_int_to_ref<float><<<nblk(n, 256), 256, 0, c->stream>>>((const float*)c->kbuf, c->d_ref, c->d_perm, c->E, c->np,
                                                             c->nv, stride);
  else
    k_int_to_ref<double><<<nblk(n, 256), 256, 0, c->stream>>>((const double*)c->kbuf, c->d_ref, c->d_perm, c->E,
                                                              c->np, c->nv, stride);
  CK(c, cudaGetLastError());
  CK(c, cudaMemcpyAsync(k, c->d_ref, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  return DG_OK;
}

int dg_cell_means(dg_ctx* c, double* p, double* rho, double* v) {
  if (!c) return DG_ERR_ARG;
  std::vector<double> h(c->E * 5);
  if (c->prec == DG_FP32)
    k_cell_means<float><<<nblk(c->E, 128), 128, 0, c->stream>>>((const float*)c->u, c->d_perm, c->E, c->np, c->nv,
                                                                c->Epad * c->np, c->c0sq, c->d_ref);
  else
    k_cell_means<double><<<nblk(c->E, 128), 128, 0, c->stream>>>((const double*)c->u, c->d_perm, c->E, c->np, c->nv,
                                                                 c->Epad * c->np, c->c0sq, c->d_ref);
  CK(c, cudaGetLastError());
  CK(c, cudaMemcpyAsync(h.data(), c->d_ref, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  for (int64_t e = 0; e < c->E; ++e) {
    if (p) p[e] = h[e * 5];
    if (rho) rho[e] = h[e * 5 + 1];
    if (v)
      for (int d = 0; d < 3; ++d) v[e * 3 + d] = h[e * 5 + 2 + d];
  }
  return DG_OK;
}

int dg_face_info(dg_ctx* c, int64_t* nbr, int* penalty, int* bc) {
  if (!c) return DG_ERR_ARG;
  const int reci = c->sh.reci, nf = c->nf;
  std::vector<int> gi(c->E * reci);
  CK(c, cudaMemcpyAsync(gi.data(), c->geoI, gi.size() * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  std::vector<int> bcodes(std::max<int64_t>(c->n_bfaces, 1));
  if (c->n_bfaces > 0) {
    CK(c, cudaMemcpyAsync(bcodes.data(), c->d_bcode, c->n_bfaces * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
  }
  for (int64_t e = 0; e < c->E; ++e)
    for (int lf = 0; lf < nf; ++lf) {
      int nb = gi[e * reci + lf], code = gi[e * reci + nf + lf];
      bool b = code & dgk::kCodeBoundary;
      if (nbr) nbr[e * nf + lf] = b ? -1 : nb;
      if (penalty) penalty[e * nf + lf] = b ? 0 : ((code & dgk::kCodeNegPenalty) ? -1 : 1);
      if (bc) bc[e * nf + lf] = b ? bcodes[nb] : -1;
    }
  return DG_OK;
}

void* dg_stream(dg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int dg_kernel_info(dg_ctx* c, int variant, int* out) {
  if (!c || !out) return fail(c, DG_ERR_ARG, "dg_kernel_info: invalid argument");
  for (int i = 0; i < 5; ++i) out[i] = 0;
  if (variant < 0) {
    out[0] = (int)c->sh.et, out[1] = c->sh.nt, out[4] = c->grid;
    return DG_OK;
  }
  dgk::Stage2Info si = stage2_info(c, variant);
  // available exactly when dg_tune accepts it
  if (!variant_handles_mesh(c, variant) || si.nc == 0 || si.blocks_per_sm <= 0 || c->Epad % si.et != 0) return DG_OK;
  out[0] = si.et, out[1] = si.nt, out[2] = si.smem_bytes, out[3] = si.blocks_per_sm;
  out[4] = (int)std::min<int64_t>(c->Epad / si.et, (int64_t)si.blocks_per_sm * c->num_sms);
  return DG_OK;
}

int dg_host_alloc(size_t bytes, void** out) {
  if (!out) return DG_ERR_ARG;
  *out = nullptr;
  if (bytes == 0) return DG_ERR_ARG;
  if (cudaMallocHost(out, bytes) != cudaSuccess) {
    cudaGetLastError();
    *out = nullptr;
    return DG_ERR_CUDA;
  }
  return DG_OK;
}

int dg_host_free(void* p) {
  if (!p) return DG_OK;
  return cudaFreeHost(p) == cudaSuccess ? DG_OK : DG_ERR_CUDA;
}

int dg_tune_cache_stats(int64_t* hits, int64_t* misses, int64_t* entries) {
  TuneCache& tc = tune_cache();
  std::lock_guard<std::mutex> lk(tc.mu);
  if (hits) *hits = tc.hits;
  if (misses) *misses = tc.misses;
  if (entries) *entries = (int64_t)tc.entries.size();
  return DG_OK;
}

void dg_tune_cache_clear(void) {
  TuneCache& tc = tune_cache();
  std::lock_guard<std::mutex> lk(tc.mu);
  tc.entries.clear();
  tc.files_read.clear();
  tc.hits = tc.misses = 0;
}

int dg_tune(dg_ctx* c, int variant) {
  if (!c || variant < -3) return DG_ERR_ARG;
  int rc = select_variant(c, variant);
  c->info.kernel_variant = c->variant;
  c->info.kernel_grid = c->variant >= 0 ? c->grid2 : c->grid;
  return rc;
}

int dg_set_wait_limit(dg_ctx* c, int rounds) {
  if (!c || rounds < 0) return DG_ERR_ARG;
  c->wait_limit = rounds;
  // the per-step graph holds the kernel arguments: captured again on the
  // next run
  if (c->graph) {
    cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
  }
  return DG_OK;
}

int dg_bench_steps(dg_ctx* c, int64_t n_steps, double dt, int64_t flush_bytes, double* step_ms, double* kernel_ms) {
  if (!c || n_steps <= 0 || !(dt > 0)) return DG_ERR_ARG;
  int rc = ensure_out_cap(c, n_steps);
  if (rc) return rc;
  rc = build_graph(c, 0, dt);
  if (rc) return rc;
  unsigned* flush = nullptr;
  int64_t nflush = flush_bytes / 4;
  if (nflush > 0) CK(c, cudaMalloc(&flush, nflush * 4));
  int64_t st[2] = {c->step, c->step};
  CK(c, cudaMemcpyAsync(c->d_step, st, sizeof(st), cudaMemcpyHostToDevice, c->stream));
  std::vector<cudaEvent_t> ev(2 * n_steps);
  for (auto& x : ev) cudaEventCreate(&x);
  for (int64_t i = 0; i < n_steps; ++i) {
    if (flush) k_flush<<<2 * c->num_sms, 512, 0, c->stream>>>(flush, nflush, (unsigned)i);
    cudaEventRecord(ev[2 * i], c->stream);
    cudaGraphLaunch(c->graph, c->stream);
    cudaEventRecord(ev[2 * i + 1], c->stream);
  }
  CK(c, cudaStreamSynchronize(c->stream));
  double tot = 0.0;
  for (int64_t i = 0; i < n_steps; ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    tot += ms;
  }
  c->step += n_steps;
  if (step_ms) *step_ms = tot / n_steps;
  if (kernel_ms) {
    // second pass without the graph: events around each stage launch
    std::vector<cudaEvent_t> se(8 * n_steps);
    for (auto& x : se) cudaEventCreate(&x);
    st[0] = st[1] = c->step;
    CK(c, cudaMemcpyAsync(c->d_step, st, sizeof(st), cudaMemcpyHostToDevice, c->stream));
    for (int64_t i = 0; i < n_steps; ++i) {
      if (flush) k_flush<<<2 * c->num_sms, 512, 0, c->stream>>>(flush, nflush, (unsigned)i);
      cudaError_t err = enqueue_step(c, 0, dt, &se[8 * i]);
      if (err != cudaSuccess) {
        for (auto& x : se) cudaEventDestroy(x);
        return fail(c, DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(err));
      }
    }
    CK(c, cudaStreamSynchronize(c->stream));
    double kt = 0.0;
    for (int64_t i = 0; i < 4 * n_steps; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, se[2 * i], se[2 * i + 1]);
      kt += ms;
    }
    for (auto& x : se) cudaEventDestroy(x);
    c->step += n_steps;
    *kernel_ms = kt / n_steps;
  }
  for (auto& x : ev) cudaEventDestroy(x);
  if (flush) cudaFree(flush);
  return DG_OK;
}

}  // extern "C"
