// Batched ensemble of independent solver instances (dg_batch_* in
// include/dgfem_gb300.h). No counterpart in the reference, which runs one
// case per process. Here hundreds of
// independent LEE runs (different meshes, orders, sources, mean flows and time
// steps) advanced together so that the GPU is filled even when each instance
// is small.
//
// Instances of one element type (dim, order) are concatenated into one
// disjoint-union mesh and solved by one context whose geometry records carry
// each element's own mean flow and time step. Every step is one CUDA graph.
// For 2-D FP32 instances of orders 2-4 (the ensemble study) every RK stage of
// all instances is one persistent launch of the mixed-order stage kernel
// (stage_multi.cuh), whose blocks take tiles of every order from a work
// queue; otherwise the per-type contexts run their source injection, four
// fused RK4 stages and observer reductions on their own streams as parallel
// branches of the graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "ctx.h"
#include "dg_internal.cuh"

namespace dgc {
int create_ctx(const dg_mesh_desc* mesh, const dg_phys* phys, int precision, int device, const double* elem_v0,
               const double* elem_scale, dg_ctx** out, std::string* err);
cudaError_t enqueue_step(dg_ctx* c, int kind, double dt, cudaEvent_t* ev);
cudaError_t enqueue_inject(dg_ctx* c);
cudaError_t enqueue_finalize(dg_ctx* c, int nparts);
dgk::StageArgs<float> stage_args_f32(dg_ctx* c, int stage, const float* y_in, float* y_out, double dt);
int ensure_out_cap(dg_ctx* c, int64_t n);
void set_global_error(const std::string& m);
}  // namespace dgc

struct dg_batch {
  struct Group {
    dg_ctx* ctx = nullptr;
    int dim = 0, order = 0, np = 0;
    std::vector<int> inst;            // member instances in order
    std::vector<double> state;        // reference-layout staging [4][E*np]
    bool state_dirty = false, state_valid = false;
    cudaEvent_t join = nullptr;
  };
  std::vector<Group> groups;
  std::vector<int> inst_group;
  std::vector<int64_t> inst_elem_off, inst_E;
  // per-instance sources and observers (instance-local dofs)
  struct Src {
    std::vector<int64_t> off{0}, dofs;
    int n = 0;
    int64_t steps = 0;
    std::vector<double> values;  // [steps][n]
  };
  struct Obs {
    std::vector<int64_t> off{0}, dofs;
    std::vector<double> w;
    int n = 0;
  };
  std::vector<Src> src;
  std::vector<Obs> obs;
  bool sources_dirty = true, observers_dirty = true;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t graph = nullptr;
  // one launch per RK stage for all element orders (2-D FP32, orders 2-4):
  // slot k -> group holding order k + 2 (or -1), the four stages' work-queue
  // counters, the launch's grid
  bool fused_ok = false, fused = false;
  int slot_group[dgk::kMultiOrders] = {-1, -1, -1};
  unsigned* d_queue = nullptr;
  int fused_grid = 0;
  int64_t step = 0, total_dofs = 0;
  std::string err;
};

namespace {

int fail(dg_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}

#define BCK(b, x)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (x);                                                                        \
    if (e_ != cudaSuccess) return fail((b), DG_ERR_CUDA, std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

// Pushes staged states, sources and observers to the group contexts.
int sync_inputs(dg_batch* b) {
  for (auto& g : b->groups)
    if (g.state_dirty) {
      int rc = dg_set_state(g.ctx, g.state.data());
      if (rc) return fail(b, rc, dg_last_error(g.ctx));
      g.state_dirty = false;
    }
  if (b->sources_dirty) {
    for (auto& g : b->groups) {
      std::vector<int64_t> off{0}, dofs;
      int64_t steps = 0;
      int nsrc = 0;
      for (int i : g.inst) {
        steps = std::max(steps, b->src[i].steps);
        nsrc += b->src[i].n;
      }
      std::vector<double> vals(std::max<int64_t>(steps * nsrc, 1), std::nan(""));
      int col = 0;
      for (int i : g.inst) {
        const auto& s = b->src[i];
        const int64_t base = b->inst_elem_off[i] * g.np;
        for (int k = 0; k < s.n; ++k) {
          for (int64_t t = s.off[k]; t < s.off[k + 1]; ++t) dofs.push_back(base + s.dofs[t]);
          off.push_back((int64_t)dofs.size());
          for (int64_t st = 0; st < s.steps; ++st) vals[st * nsrc + col + k] = s.values[st * s.n + k];
        }
        col += s.n;
      }
      int rc = dg_set_sources(g.ctx, nsrc, off.data(), dofs.data());
      if (!rc) rc = dg_set_source_values(g.ctx, nsrc > 0 ? steps : 0, vals.data());
      if (rc) return fail(b, rc, dg_last_error(g.ctx));
    }
    b->sources_dirty = false;
    if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
  }
  if (b->observers_dirty) {
    for (auto& g : b->groups) {
      std::vector<int64_t> off{0}, dofs;
      std::vector<double> w;
      int nobs = 0;
      for (int i : g.inst) {
        const auto& o = b->obs[i];
        const int64_t base = b->inst_elem_off[i] * g.np;
        for (int k = 0; k < o.n; ++k) {
          for (int64_t t = o.off[k]; t < o.off[k + 1]; ++t) dofs.push_back(base + o.dofs[t]), w.push_back(o.w[t]);
          off.push_back((int64_t)dofs.size());
        }
        nobs += o.n;
      }
      int rc = dg_set_observers(g.ctx, nobs, off.data(), dofs.data(), w.data());
      if (rc) return fail(b, rc, dg_last_error(g.ctx));
    }
    b->observers_dirty = false;
    if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
  }
  return DG_OK;
}

// One graph per step with one launch per RK stage for every element order:
// queue counters reset, per-order source injection, the four mixed-order
// stage kernels, per-order residual and observer reductions (all on the
// batch's stream; the group contexts' work is enqueued there).
int build_fused_graph(dg_batch* b) {
  cudaGraph_t graph = nullptr;
  BCK(b, cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaMemsetAsync(b->d_queue, 0, 4 * sizeof(unsigned), b->main);
  std::vector<cudaStream_t> keep;
  for (auto& g : b->groups) keep.push_back(g.ctx->stream), g.ctx->stream = b->main;
  for (auto& g : b->groups)
    if (err == cudaSuccess) err = dgc::enqueue_inject(g.ctx);
  int* derr = nullptr;
  for (int st = 1; st <= 4 && err == cudaSuccess; ++st) {
    dgk::MultiArgs m{};
    m.ntiles_total = 0;
    m.queue = b->d_queue + (st - 1);
    m.wait_limit = dgk::kWaitRounds;
    for (int k = 0; k < dgk::kMultiOrders; ++k) {
      m.g[k].stage = st;
      m.g[k].ntiles = 0;
      if (b->slot_group[k] < 0) continue;
      dg_ctx* c = b->groups[b->slot_group[k]].ctx;
      const float* in[4] = {(const float*)c->u, (const float*)c->y0, (const float*)c->y1, (const float*)c->y0};
      float* out[4] = {(float*)c->y0, (float*)c->y1, (float*)c->y0, nullptr};
      // every instance's own dt sits in its elements' step scale
      m.g[k] = dgc::stage_args_f32(c, st, in[st - 1], out[st - 1], 1.0);
      m.g[k].ntiles = (int)(c->Epad / dgk::stage_multi_elems_per_tile(k + 2));
      m.ntiles_total += m.g[k].ntiles;
      if (!derr) derr = c->d_err;
    }
    err = dgk::launch_stage_multi(m, b->fused_grid, derr, b->main);
  }
  for (auto& g : b->groups)
    if (err == cudaSuccess) err = dgc::enqueue_finalize(g.ctx, b->fused_grid);
  for (size_t i = 0; i < b->groups.size(); ++i) b->groups[i].ctx->stream = keep[i];
  cudaError_t err2 = cudaStreamEndCapture(b->main, &graph);
  if (err != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail(b, DG_ERR_CUDA, std::string("CUDA (capture): ") + cudaGetErrorString(err));
  }
  BCK(b, err2);
  err = cudaGraphInstantiate(&b->graph, graph, 0);
  cudaGraphDestroy(graph);
  BCK(b, err);
  return DG_OK;
}

// One graph per step: every group's step as a parallel branch.
int build_graph(dg_batch* b, int64_t n_steps) {
  for (auto& g : b->groups) {
    int rc = dgc::ensure_out_cap(g.ctx, n_steps);
    if (rc) return fail(b, rc, dg_last_error(g.ctx));
  }
  if (b->graph) return DG_OK;
  if (b->fused) return build_fused_graph(b);
  cudaGraph_t graph = nullptr;
  BCK(b, cudaStreamBeginCapture(b->main, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaEventRecord(b->fork, b->main);
  for (auto& g : b->groups) {
    if (err == cudaSuccess) err = cudaStreamWaitEvent(g.ctx->stream, b->fork, 0);
    // every instance's own dt sits in its elements' step scale
    if (err == cudaSuccess) err = dgc::enqueue_step(g.ctx, 0, 1.0, nullptr);
    if (err == cudaSuccess) err = cudaEventRecord(g.join, g.ctx->stream);
    if (err == cudaSuccess) err = cudaStreamWaitEvent(b->main, g.join, 0);
  }
  cudaError_t err2 = cudaStreamEndCapture(b->main, &graph);
  if (err != cudaSuccess) return fail(b, DG_ERR_CUDA, std::string("CUDA (capture): ") + cudaGetErrorString(err));
  BCK(b, err2);
  err = cudaGraphInstantiate(&b->graph, graph, 0);
  cudaGraphDestroy(graph);
  BCK(b, err);
  return DG_OK;
}

int launch_steps(dg_batch* b, int64_t n_steps, cudaEvent_t* ev) {
  for (auto& g : b->groups) {
    int64_t st[2] = {b->step, b->step};
    BCK(b, cudaMemcpyAsync(g.ctx->d_step, st, sizeof(st), cudaMemcpyHostToDevice, b->main));
  }
  for (int64_t i = 0; i < n_steps; ++i) {
    if (ev) cudaEventRecord(ev[2 * i], b->main);
    BCK(b, cudaGraphLaunch(b->graph, b->main));
    if (ev) cudaEventRecord(ev[2 * i + 1], b->main);
  }
  return DG_OK;
}

}  // namespace

extern "C" {

const char* dg_batch_last_error(const dg_batch* b) { return b ? b->err.c_str() : dg_last_error(nullptr); }

int dg_batch_create(int n, const dg_mesh_desc* meshes, const dg_phys* phys, const double* dts, int precision,
                    int device, dg_batch** out) {
  if (!out || n <= 0 || !meshes || !phys || !dts) {
    dgc::set_global_error("dg_batch_create: invalid argument");
    return DG_ERR_ARG;
  }
  *out = nullptr;
  for (int i = 1; i < n; ++i)
    if (phys[i].rho0 != phys[0].rho0 || phys[i].c0 != phys[0].c0) {
      dgc::set_global_error("dg_batch_create: all instances must share rho0 and c0");
      return DG_ERR_ARG;
    }
  for (int i = 0; i < n; ++i)
    if (!(dts[i] > 0)) {
      dgc::set_global_error("dg_batch_create: time steps must be positive");
      return DG_ERR_ARG;
    }
  auto* b = new dg_batch;
  b->inst_group.assign(n, -1);
  b->inst_elem_off.assign(n, 0);
  b->inst_E.assign(n, 0);
  b->src.assign(n, {});
  b->obs.assign(n, {});
  std::map<std::pair<int, int>, int> gid;
  for (int i = 0; i < n; ++i) {
    auto key = std::make_pair(meshes[i].dim, meshes[i].order);
    if (!gid.count(key)) {
      gid[key] = (int)b->groups.size();
      b->groups.emplace_back();
      b->groups.back().dim = key.first, b->groups.back().order = key.second;
      b->groups.back().np = meshes[i].nodes_per_elem;
    }
    b->inst_group[i] = gid[key];
    b->groups[gid[key]].inst.push_back(i);
  }
  auto bail = [&](int code, const std::string& m) {
    dgc::set_global_error("dg_batch_create: " + m);
    dg_batch_destroy(b);
    return code;
  };
  for (auto& g : b->groups) {
    // disjoint union of the member meshes
    std::vector<double> xyz, v0, scale;
    std::vector<int64_t> en, goff{0}, gnodes;
    std::vector<int> gbc;
    const dg_mesh_desc& m0 = meshes[g.inst[0]];
    const int ngr = m0.n_groups;
    std::vector<std::vector<int64_t>> gn(ngr);
    int64_t node_off = 0, elem_off = 0;
    for (int i : g.inst) {
      const dg_mesh_desc& m = meshes[i];
      if (m.nodes_per_elem != g.np || m.n_groups != ngr) return bail(DG_ERR_ARG, "instances of one element type must have the same boundary group structure");
      for (int k = 0; k < ngr; ++k)
        if (m.group_bc[k] != m0.group_bc[k]) return bail(DG_ERR_ARG, "instances of one element type must use the same BC per group");
      xyz.insert(xyz.end(), m.xyz, m.xyz + 3 * m.n_nodes);
      for (int64_t k = 0; k < m.n_elems * g.np; ++k) en.push_back(m.elem_nodes[k] + node_off);
      for (int k = 0; k < ngr; ++k)
        for (int64_t t = m.group_offsets[k]; t < m.group_offsets[k + 1]; ++t) gn[k].push_back(m.group_nodes[t] + node_off);
      for (int64_t e = 0; e < m.n_elems; ++e) {
        for (int d = 0; d < 3; ++d) v0.push_back(phys[i].v0[d]);
        scale.push_back(dts[i]);
      }
      b->inst_elem_off[i] = elem_off;
      b->inst_E[i] = m.n_elems;
      node_off += m.n_nodes;
      elem_off += m.n_elems;
    }
    for (int k = 0; k < ngr; ++k) {
      gbc.push_back(m0.group_bc[k]);
      gnodes.insert(gnodes.end(), gn[k].begin(), gn[k].end());
      goff.push_back((int64_t)gnodes.size());
    }
    dg_mesh_desc md = m0;
    md.n_nodes = node_off, md.xyz = xyz.data(), md.n_elems = elem_off, md.elem_nodes = en.data();
    md.n_groups = ngr, md.group_bc = gbc.data(), md.group_offsets = goff.data(), md.group_nodes = gnodes.data();
    dg_phys ph = phys[g.inst[0]];
    std::string e;
    int rc = dgc::create_ctx(&md, &ph, precision, device, v0.data(), scale.data(), &g.ctx, &e);
    if (rc) return bail(rc, e);
    g.state.assign(4 * elem_off * g.np, 0.0);
    b->total_dofs += elem_off * g.np * (g.dim + 1);
    if (cudaEventCreateWithFlags(&g.join, cudaEventDisableTiming) != cudaSuccess) return bail(DG_ERR_CUDA, "event");
  }
  if (cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    return bail(DG_ERR_CUDA, "stream/event creation failed");
  // one launch per stage for all orders: 2-D FP32 instances of orders 2-4
  b->fused_ok = precision == DG_FP32;
  for (size_t k = 0; k < b->groups.size(); ++k) {
    const auto& g = b->groups[k];
    if (g.dim != 2 || g.order < 2 || g.order > 4 || g.ctx->ncurved > 0)
      b->fused_ok = false;
    else
      b->slot_group[g.order - 2] = (int)k;
  }
  if (b->fused_ok) {
    const int bps = dgk::stage_multi_blocks_per_sm();
    int64_t tiles = 0;
    int cap = 1 << 30;
    for (auto& g : b->groups) {
      tiles += g.ctx->Epad / dgk::stage_multi_elems_per_tile(g.order);
      cap = std::min(cap, g.ctx->max_grid);  // rows of every order's partial-sum array
    }
    b->fused_grid = (int)std::min<int64_t>(std::min<int64_t>(tiles, (int64_t)bps * b->groups[0].ctx->num_sms), cap);
    if (bps <= 0 || b->fused_grid <= 0 || cudaMalloc(&b->d_queue, 4 * sizeof(unsigned)) != cudaSuccess) {
      cudaGetLastError();
      b->fused_ok = false;
    }
  }
  // one launch per stage is the default where the batch allows it (measured
  // faster than one kernel per order on the 256-instance ensemble: 2.33
  // against 2.45 ms per step); DGFEM_BATCH_FUSED=0 or dg_batch_set_fused(b, 0)
  // selects one kernel per order
  const char* ev = std::getenv("DGFEM_BATCH_FUSED");
  b->fused = b->fused_ok && !(ev && std::strcmp(ev, "0") == 0);
  *out = b;
  return DG_OK;
}

int dg_batch_destroy(dg_batch* b) {
  if (!b) return DG_OK;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (auto& g : b->groups) {
    if (g.join) cudaEventDestroy(g.join);
    if (g.ctx) dg_destroy(g.ctx);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->main) cudaStreamDestroy(b->main);
  if (b->d_queue) cudaFree(b->d_queue);
  delete b;
  return DG_OK;
}

int dg_batch_set_fused(dg_batch* b, int on) {
  if (!b) return DG_ERR_ARG;
  if (on && !b->fused_ok)
    return fail(b, DG_ERR_ARG, "one launch per stage needs FP32 2-D straight-sided instances of orders 2-4 only");
  if (b->fused != (on != 0)) {
    b->fused = on != 0;
    if (b->graph) cudaGraphExecDestroy(b->graph), b->graph = nullptr;
  }
  return DG_OK;
}

int dg_batch_fused(const dg_batch* b) { return b && b->fused ? 1 : 0; }

int dg_batch_info(const dg_batch* b, int* n_groups, int64_t* total_dofs) {
  if (!b) return DG_ERR_ARG;
  if (n_groups) *n_groups = (int)b->groups.size();
  if (total_dofs) *total_dofs = b->total_dofs;
  return DG_OK;
}

int dg_batch_set_state(dg_batch* b, int inst, const double* u) {
  if (!b || !u || inst < 0 || inst >= (int)b->inst_group.size()) return DG_ERR_ARG;
  auto& g = b->groups[b->inst_group[inst]];
  const int64_t N = (int64_t)g.state.size() / 4, n = b->inst_E[inst] * g.np, off = b->inst_elem_off[inst] * g.np;
  for (int q = 0; q < 4; ++q) std::memcpy(&g.state[q * N + off], u + q * n, n * sizeof(double));
  g.state_dirty = true;
  return DG_OK;
}

int dg_batch_get_state(dg_batch* b, int inst, double* u) {
  if (!b || !u || inst < 0 || inst >= (int)b->inst_group.size()) return DG_ERR_ARG;
  int rc = sync_inputs(b);
  if (rc) return rc;
  auto& g = b->groups[b->inst_group[inst]];
  const int64_t N = (int64_t)g.state.size() / 4, n = b->inst_E[inst] * g.np, off = b->inst_elem_off[inst] * g.np;
  if (!g.state_valid) {
    rc = dg_get_state(g.ctx, g.state.data());
    if (rc) return fail(b, rc, dg_last_error(g.ctx));
    g.state_valid = true;
  }
  for (int q = 0; q < 4; ++q) std::memcpy(u + q * n, &g.state[q * N + off], n * sizeof(double));
  return DG_OK;
}

int dg_batch_set_sources(dg_batch* b, int inst, int n_src, const int64_t* offsets, const int64_t* dofs,
                         int64_t n_steps, const double* values) {
  if (!b || inst < 0 || inst >= (int)b->inst_group.size() || n_src < 0 || n_steps < 0) return DG_ERR_ARG;
  auto& s = b->src[inst];
  const int64_t nd = b->inst_E[inst] * b->groups[b->inst_group[inst]].np;
  s.n = n_src;
  s.steps = n_src > 0 ? n_steps : 0;
  s.off.assign(offsets, offsets + n_src + 1);
  s.dofs.assign(dofs, dofs + (n_src > 0 ? offsets[n_src] : 0));
  for (auto d : s.dofs)
    if (d < 0 || d >= nd) return fail(b, DG_ERR_ARG, "source dof out of range");
  s.values.assign(values, values + s.steps * n_src);
  b->sources_dirty = true;
  return DG_OK;
}

int dg_batch_set_observers(dg_batch* b, int inst, int n_obs, const int64_t* offsets, const int64_t* dofs,
                           const double* weights) {
  if (!b || inst < 0 || inst >= (int)b->inst_group.size() || n_obs < 0) return DG_ERR_ARG;
  auto& o = b->obs[inst];
  const int64_t nd = b->inst_E[inst] * b->groups[b->inst_group[inst]].np;
  o.n = n_obs;
  o.off.assign(offsets, offsets + n_obs + 1);
  int64_t tot = n_obs > 0 ? offsets[n_obs] : 0;
  o.dofs.assign(dofs, dofs + tot);
  o.w.assign(weights, weights + tot);
  for (auto d : o.dofs)
    if (d < 0 || d >= nd) return fail(b, DG_ERR_ARG, "observer dof out of range");
  b->observers_dirty = true;
  return DG_OK;
}

int dg_batch_run(dg_batch* b, int64_t n_steps, double* obs) {
  if (!b || n_steps < 0) return DG_ERR_ARG;
  if (n_steps == 0) return DG_OK;
  int rc = sync_inputs(b);
  if (!rc) rc = build_graph(b, n_steps);
  if (!rc) rc = launch_steps(b, n_steps, nullptr);
  if (rc) return rc;
  BCK(b, cudaStreamSynchronize(b->main));
  b->step += n_steps;
  for (auto& g : b->groups) {
    g.state_valid = false;
    g.ctx->step = b->step;
  }
  if (obs) {
    // per instance, in instance order: [n_steps][n_obs_i][4]
    std::vector<int64_t> inst_out(b->inst_group.size(), 0);
    int64_t acc = 0;
    for (size_t i = 0; i < b->inst_group.size(); ++i) inst_out[i] = acc, acc += n_steps * b->obs[i].n * 4;
    for (auto& g : b->groups) {
      int nobs = g.ctx->n_obs;
      if (nobs == 0) continue;
      std::vector<double> h(n_steps * nobs * 4);
      BCK(b, cudaMemcpy(h.data(), g.ctx->d_obs, h.size() * sizeof(double), cudaMemcpyDeviceToHost));
      int col = 0;
      for (int i : g.inst) {
        const int ni = b->obs[i].n;
        for (int64_t s = 0; s < n_steps; ++s)
          for (int k = 0; k < ni; ++k)
            for (int c = 0; c < 4; ++c) obs[inst_out[i] + (s * ni + k) * 4 + c] = h[(s * nobs + col + k) * 4 + c];
        col += ni;
      }
    }
  }
  int herr = 0;
  for (auto& g : b->groups) {
    BCK(b, cudaMemcpy(&herr, g.ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (herr) {
      BCK(b, cudaMemset(g.ctx->d_err, 0, sizeof(int)));  // the batch stays usable
      return fail(b, DG_ERR_TIMEOUT, "a bounded device wait gave up");
    }
  }
  return DG_OK;
}

int dg_batch_bench(dg_batch* b, int64_t n_steps, double* step_ms) {
  if (!b || n_steps <= 0) return DG_ERR_ARG;
  int rc = sync_inputs(b);
  if (!rc) rc = build_graph(b, n_steps);
  if (rc) return rc;
  std::vector<cudaEvent_t> ev(2 * n_steps);
  for (auto& e : ev) cudaEventCreate(&e);
  rc = launch_steps(b, n_steps, ev.data());
  if (!rc && cudaStreamSynchronize(b->main) != cudaSuccess) rc = fail(b, DG_ERR_CUDA, "synchronize failed");
  double tot = 0.0;
  for (int64_t i = 0; !rc && i < n_steps; ++i) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
    tot += ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  b->step += n_steps;
  for (auto& g : b->groups) g.state_valid = false, g.ctx->step = b->step;
  if (step_ms) *step_ms = tot / n_steps;
  return DG_OK;
}

}  // extern "C"
