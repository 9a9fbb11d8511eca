// The solver context behind the C ABI (include/dgfem_gb300.h).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/dgfem_gb300.h"
#include "dg_internal.cuh"
#include "refelem.h"

struct dg_ctx {
  // problem
  int dim = 0, order = 0, prec = DG_FP64, device = 0;
  int np = 0, nv = 0, nf = 0, nfp = 0;
  int64_t E = 0, Epad = 0, ntiles = 0, nnodes = 0;
  int64_t n_faces = 0, n_bfaces = 0;
  dgref::RefElement re;
  dgk::ShapeInfo sh{};
  dgk::Phys ph{};
  double c0sq = 1.0;
  std::vector<int> perm_c2i;  // mesh local node -> internal node
  // device
  cudaStream_t stream = nullptr;
  int num_sms = 0, grid = 0;
  // stage kernel selection: -1 = baseline kernel (stage.cuh), k >= 0 = pipelined variant k (stage2.cuh)
  int variant = -1, grid2 = 0, max_grid = 0;
  dgk::Stage2Info s2{};
  int* d_err = nullptr;  // device error flags of bounded waits
  int wait_limit = dgk::kWaitRounds;  // polling rounds of a bounded device wait (dg_set_wait_limit)
  size_t tsize = 8;
  void* u = nullptr;     // state            [nv][Epad*np]
  void* acc = nullptr;   // RK accumulator
  void* y0 = nullptr;    // stage inputs (double buffered)
  void* y1 = nullptr;
  void* snap = nullptr;  // residual reference
  void* kbuf = nullptr;  // dg_rhs output
  void* geoF = nullptr;  // [Epad][recf]
  int* geoI = nullptr;   // [Epad][reci]
  void* bmat = nullptr;  // [n_bfaces][nv*nv]
  int* d_bcode = nullptr;  // [n_bfaces] 1 reflecting, 0 absorbing
  void* Dt = nullptr;    // [dim][np][np] (j-major rows: Dt[r][j][i])
  void* LIFT = nullptr;  // [nf*nfp][np]
  short* fmask = nullptr;
  short* nbrnode = nullptr;
  int* d_perm = nullptr;       // [np] mesh local -> internal
  double* d_ref = nullptr;     // [4][E*np] staging for reference-layout I/O
  double* partials = nullptr;  // [grid][5]
  int64_t* d_step = nullptr;   // [0] global step, [1] first step of the current run
  double* d_res = nullptr;     // [out_cap][5]
  double* d_obs = nullptr;     // [out_cap][n_obs][4]
  int64_t out_cap = 0;
  int64_t step = 0;
  // sources: unique internal dofs, CSR list of covering sources per dof
  int n_src = 0;
  int64_t n_src_dofs = 0;
  int64_t* d_src_dof = nullptr;
  int* d_src_off = nullptr;
  int* d_src_ids = nullptr;
  double* d_srcval = nullptr;
  int64_t srcval_steps = 0;
  // observers
  int n_obs = 0;
  int64_t* d_obs_dof = nullptr;
  int64_t* d_obs_off = nullptr;
  double* d_obs_w = nullptr;
  // observer blocks of the finalize kernel (obs_blocks in all); when an
  // observer has more node slots than a block has threads, blocks
  // bfirst[o] .. bfirst[o+1]-1 sum observer o (bmap: block -> observer),
  // with per-block partial sums [obs_blocks][5] and per observer the count
  // of its blocks done (the last one combines them in block order)
  int obs_blocks = 0;
  int* d_obs_bmap = nullptr;
  int* d_obs_bfirst = nullptr;
  bool obs_small = true;  // every observer within the small finalize block
  double* d_obs_part = nullptr;
  unsigned* d_obs_cnt = nullptr;
  // curved elements (curved.cu): slot table, per-element quadrature data and
  // the per-stage right-hand side of those elements
  int64_t ncurved = 0;
  int cng = 0, cngf = 0;
  int* cslot = nullptr;      // [Epad] slot of a curved element, -1 otherwise (null: none)
  int64_t* celem = nullptr;  // [ncurved] element of each slot
  void* cA = nullptr;        // [ncurved][ng][dim][dim]
  void* cMinv = nullptr;     // [ncurved][np][np]
  void* cF = nullptr;        // [ncurved][nf][ngf][dim+1]
  void* cTB = nullptr;       // [ncurved][nf][6]
  void* cqB = nullptr;       // [ng][np]
  void* cqD = nullptr;       // [dim][ng][np]
  void* cfB = nullptr;       // [nf][ngf][nfp]
  void* crhs = nullptr;      // [nv][ncurved][np]
  // per-step graph
  cudaGraphExec_t graph = nullptr;
  double graph_dt = 0.0;
  int graph_kind = -1;  // 0 = RK4, 1 = Euler
  // bookkeeping
  std::string err;
  dg_info_t info{};
  int64_t device_bytes = 0;
  std::vector<void*> allocs;
};

namespace dgc {
// FP64 GPU setup of geometry, connectivity and boundary data (setup.cu).
int run_setup(dg_ctx* c, const dg_mesh_desc* mesh, const double* elem_v0, const double* elem_scale);
// Allocation helper that records the buffer for dg_destroy.
cudaError_t dev_alloc(dg_ctx* c, void** p, size_t bytes);
}  // namespace dgc
