/*
 * dgfem_gb300.h — C ABI of the GB300-native DG solver core.
 *
 * The reference (DGFEM-Acoustic) has no plugin API: its seam is the
 * in-process call solver::rungeKutta(u, mesh, config) (include/solver.h:25,
 * src/solver.cpp:311) on a Mesh built by Mesh::Mesh(config)
 * (src/Mesh.cpp:20-686), driven by the dgalerkin executable
 * (src/dgalerkin.cpp:14-85). This ABI splits that call into the pieces a host
 * driver (the project's dgalerkin) needs, with plain C types only:
 *
 *   dg_create           replaces Mesh::Mesh + Mesh::precomputeMassMatrix
 *                       (src/Mesh.cpp:20-724): GPU FP64 setup of geometry,
 *                       face connectivity, normals, penalty signs, BC codes
 *                       and boundary matrices (RKR, Mesh.cpp:619-666)
 *   dg_set_state / dg_get_state
 *                       the solution vector u[4][E*Np] of src/dgalerkin.cpp:51
 *                       (per-variable, element-major, the mesh's local node
 *                       order); vz is carried as zero in 2-D
 *   dg_set_sources / dg_set_source_values
 *                       source node sets (src/solver.cpp:339-358) and the
 *                       per-step values written by the hard overwrite
 *                       (src/solver.cpp:455-483)
 *   dg_set_observers    observer node sets and IDW weights (src/solver.cpp:360-383)
 *   dg_snapshot         the residual reference copy taken at output steps
 *                       (src/solver.cpp:421-439)
 *   dg_run              n time steps of classic RK4 (src/solver.cpp:413-574):
 *                       source injection, four RHS stages (Mesh::updateFlux,
 *                       numStep: src/Mesh.cpp:734-975, src/solver.cpp:38-57),
 *                       the combine, the residuals and observer samples
 *   dg_run_euler        n steps of forward Euler (src/solver.cpp:153-302)
 *   dg_rhs              one numStep with beta = 0 after updateFlux:
 *                       k = dt M^-1 (S - F) (src/solver.cpp:38-57)
 *   dg_cell_means       element means written to the VTU files (src/Mesh.cpp:1196-1212)
 *
 * Conventions: every call returns DG_OK (0) or an error code; nothing aborts
 * or throws. dg_last_error(ctx) returns the message of the last failure on
 * ctx (ctx may be NULL for dg_create failures). One context owns one CUDA
 * stream and all its device memory; a context is not thread-safe, distinct
 * contexts may be used concurrently. Device memory is allocated in dg_create,
 * dg_set_sources, dg_set_observers and on the first dg_run that needs more
 * per-step output room.
 */
#ifndef DGFEM_GB300_H
#define DGFEM_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DG_OK = 0,
  DG_ERR_ARG = 1,       /* invalid argument or call order */
  DG_ERR_CUDA = 2,      /* CUDA runtime error (no device, out of memory, launch failure) */
  DG_ERR_MESH = 3,      /* unsupported or inconsistent mesh (non-conforming, inverted, ...) */
  DG_ERR_NONFINITE = 4, /* NaN/Inf detected in the state */
  DG_ERR_TIMEOUT = 5    /* a bounded device wait gave up */
};

enum { DG_FP64 = 0, DG_FP32 = 1 };

typedef struct dg_ctx dg_ctx;

typedef struct {
  int dim;            /* 2 (triangles) or 3 (tetrahedra) */
  int order;          /* Lagrange order 1..4 */
  int nodes_per_elem; /* Np */
  int64_t n_nodes;
  const double* xyz;         /* [n_nodes][3] node coordinates */
  int64_t n_elems;
  const int64_t* elem_nodes; /* [n_elems][Np] node indices; corners first (Gmsh order) */
  /* boundary physical groups with a BC type, in ascending physical tag order
   * (the order in which src/Mesh.cpp:582-605 applies them; last match wins) */
  int n_groups;                 /* <= 32 */
  const int* group_bc;          /* 1 = Reflecting, 0 = Absorbing */
  const int64_t* group_offsets; /* [n_groups+1] */
  const int64_t* group_nodes;   /* node indices of each group */
} dg_mesh_desc;

typedef struct {
  double v0[3]; /* mean flow */
  double rho0;
  double c0;
} dg_phys;

typedef struct {
  int dim, order, nodes_per_elem, n_var, precision;
  int64_t n_elems, n_faces, n_boundary_faces;
  int64_t penalty_sign_hist[2]; /* interior faces with s_f = -1, +1 */
  int64_t device_bytes;
  double setup_ms;
  int kernel_variant; /* stage kernel in use: -1 baseline, 0..15 pipelined variant k, 16..18 tensor-core
                         kernel, 32.. constant-operator variant */
  int kernel_grid;    /* blocks of each stage-kernel launch (persistent blocks for variants >= 0) */
  int64_t n_curved;   /* curved elements (high-order nodes off the straight-sided lattice), integrated
                         element by element with the reference's quadrature formulation */
} dg_info_t;

int dg_create(const dg_mesh_desc* mesh, const dg_phys* phys, int precision, int device, dg_ctx** out);
int dg_destroy(dg_ctx* ctx);
const char* dg_last_error(const dg_ctx* ctx);
int dg_get_info(const dg_ctx* ctx, dg_info_t* info);

int dg_set_state(dg_ctx* ctx, const double* u);
int dg_get_state(dg_ctx* ctx, double* u);

/* Source node sets: dofs are e*Np + n in the mesh's local node order.
 * Sources are applied in index order; a later active source overwrites an
 * earlier one on shared nodes. */
int dg_set_sources(dg_ctx* ctx, int n_src, const int64_t* offsets, const int64_t* dofs);
/* values[step][src] for global steps [0, n_steps); NaN = source inactive at that step */
int dg_set_source_values(dg_ctx* ctx, int64_t n_steps, const double* values);
/* Observer node sets with their IDW weights w = 1/(d^2 + 1e-12). */
int dg_set_observers(dg_ctx* ctx, int n_obs, const int64_t* offsets, const int64_t* dofs, const double* weights);

int dg_snapshot(dg_ctx* ctx);
/* Runs n_steps RK4 steps from the current global step index. residuals
 * [n_steps][5] (p, rho, vx, vy, vz) and obs [n_steps][n_obs][4] (p, vx, vy, vz)
 * are filled when non-NULL. */
int dg_run(dg_ctx* ctx, int64_t n_steps, double dt, double* residuals, double* obs);
int dg_run_euler(dg_ctx* ctx, int64_t n_steps, double dt, double* residuals, double* obs);
int64_t dg_step_index(const dg_ctx* ctx);
int dg_set_step_index(dg_ctx* ctx, int64_t step);

/* k = dt * M^-1 (S - F) of state u (both [4][E*Np]); the context state is unchanged. */
int dg_rhs(dg_ctx* ctx, const double* u, double dt, double* k);
/* element means of p, p/c0^2 and v ([E], [E], [E][3]) */
int dg_cell_means(dg_ctx* ctx, double* p, double* rho, double* v);

/* Per element local face (n_elems x (dim+1), local faces in Gmsh order):
 * neighbour element (-1 on the boundary), penalty sign s_f (0 on the
 * boundary) and BC code (1 reflecting, 0 absorbing, -1 interior). */
int dg_face_info(dg_ctx* ctx, int64_t* nbr, int* penalty, int* bc);

/* Asynchronous VTU snapshots (replaces the time loop's synchronous
 * Mesh::writeVTUb, src/Mesh.cpp:1136-1230, src/solver.cpp:451). A writer
 * holds the VTK mesh part of every file (points [n_points][3]; cells
 * [n_elems][dim+1]: the point index of each element corner, the reference's
 * node tag - 1) and n_slots (0: 3) pinned snapshot slots.
 * dg_vtu_write_async computes the cell means (p, p/c0^2, velocity; the
 * reference's formula) of the context's state as of the steps enqueued so
 * far, on the GPU, and returns; a background thread writes `path` (VTK XML,
 * appended raw data; compression 1: zlib blocks as VTK's default writer,
 * 0: uncompressed, -1: zlib when the system library loads). It blocks only
 * while every slot is in flight. dg_vtu_writer_flush waits for every file
 * and returns the first failure (message in dg_vtu_writer_last_error).
 * Destroy the writer before its context. */
typedef struct dg_vtu_writer dg_vtu_writer;
int dg_vtu_writer_create(dg_ctx* ctx, int64_t n_points, const double* points, const int64_t* cells, int compression,
                         int n_slots, dg_vtu_writer** out);
int dg_vtu_write_async(dg_vtu_writer* w, const char* path);
int dg_vtu_writer_flush(dg_vtu_writer* w);
int dg_vtu_writer_destroy(dg_vtu_writer* w);
const char* dg_vtu_writer_last_error(const dg_vtu_writer* w);
int dg_vtu_writer_stats(const dg_vtu_writer* w, int64_t* files_written, int* compressed);

/* Stage kernel selection. variant -2: time every variant on this mesh (the
 * four RK stages of a step; the state is left untouched, the stage buffers
 * and the accumulator are cleared) and keep the fastest; -3: the same, unless the tune cache holds a result for
 * this GPU model, element type, precision and mesh size class (what
 * dg_create does; the environment variable DGFEM_STAGE_VARIANT overrides it
 * there); -1: baseline kernel; k >= 0:
 * pipelined variant k (TMA-staged tiles; the variants differ in output nodes
 * per thread and elements per tile); 16, 17, 18: tensor-core kernel with 256,
 * 512 or 1024 threads per block (FP32 contexts only: tcgen05 TF32 MMAs of
 * head/tail-split operands, FP32-level results); 19, 20: the two-chunk
 * tensor-core kernel (K applied in at most two chunks so that two blocks
 * share an SM) with 256 or 512 threads per block (FP32 only); 32 + k: constant-operator variant k (FP32
 * contexts only: operators in constant memory). Returns
 * DG_ERR_ARG for a variant that does not exist for this element type or
 * precision. */
int dg_tune(dg_ctx* ctx, int variant);

/* Polling rounds that each bounded device wait of the stage kernels (the
 * mbarrier waits for their TMA copies and tensor-core work) makes before it
 * gives up (default 2^20; 0 gives up at once). A kernel whose wait gives up
 * issues no further copy, waits with the default limit for the copies it
 * already issued, sets the context's error flag and returns; the dg_run call
 * then returns DG_ERR_TIMEOUT and clears the flag, and the context stays
 * usable. For tests of that failure path and for diagnosing a stalled
 * device. No reference counterpart (the reference aborts through
 * Fatal_Error, include/err.h:5-9). */
int dg_set_wait_limit(dg_ctx* ctx, int rounds);

/* Page-locked (pinned) host memory for the host arrays of dg_set_state,
 * dg_get_state, dg_run and friends: copies from and to it run at the
 * host-device link's rate instead of through a staging buffer. No reference
 * counterpart (the reference has no device). */
int dg_host_alloc(size_t bytes, void** out);
int dg_host_free(void* p);

/* The autotuner's result cache (process-wide; keyed by GPU model, dimension,
 * order, precision and the mesh's size class floor(log2(padded elements))).
 * Every timed selection stores its winner; when DGFEM_TUNE_CACHE names a
 * file, results are also appended to it and read back from it on the first
 * lookup, so later processes skip the timing. Replaces no reference
 * interface (the reference has no kernel selection). */
int dg_tune_cache_stats(int64_t* hits, int64_t* misses, int64_t* entries);
/* Forgets the in-process entries and counters (the file is left as is and
 * is read again on the next lookup). */
void dg_tune_cache_clear(void);

/* Launch shape of stage-kernel variant `variant` (as in dg_tune) for this
 * context: out[0] elements per tile (0: not available), out[1] threads per
 * block, out[2] dynamic shared memory bytes, out[3] resident blocks per SM
 * (the occupancy query, capped by tensor memory for the tensor-core kernel),
 * out[4] the grid a launch would use. */
int dg_kernel_info(dg_ctx* ctx, int variant, int* out);

/* The CUDA stream (cudaStream_t) all work of ctx is issued on. */
void* dg_stream(dg_ctx* ctx);
/* Timed RK4 steps for benchmarking: runs n_steps with the per-step graph and
 * returns the per-step device time from CUDA events on ctx's stream; when
 * kernel_ms is non-NULL also the summed time of the four stage kernels,
 * timed with events around each stage launch in a second pass. flush_bytes > 0
 * writes a scratch buffer of that size between steps (outside the timing). */
int dg_bench_steps(dg_ctx* ctx, int64_t n_steps, double dt, int64_t flush_bytes, double* step_ms,
                   double* kernel_ms);

/* Allocation-free residual diagnostic. No counterpart in the reference: it
 * serves callers that cannot allocate device memory where they need the
 * diagnostic (code inside a host framework that owns every allocation, loops
 * that must not call the allocator, callers that manage their own device
 * buffers). It needs no context.
 *
 * Computes, on `stream`, the five residual means of the reference's time loop
 * between a state u and a snapshot (res[0] p, res[1] p/c0^2, res[2..4] vx, vy,
 * vz; variables beyond n_var give 0) from caller-owned device arrays laid out
 * as n_var planes of var_stride elements (float for DG_FP32, double for
 * DG_FP64), each with n_per_var nodes, and writes them to the caller-owned
 * device array res[5]. It allocates nothing and does not synchronise.
 *
 * Its only scratch is a fixed 160 KiB array inside the library that every GPU
 * loading the library holds until the process exits; n_per_var is therefore
 * limited to 67,108,864 nodes (DG_ERR_ARG beyond). Every call looks up that
 * array's device address with the calling thread's current device (so a
 * cudaDeviceReset between calls is harmless); the first call on a device may
 * load the library's device code, so make it before any stream capture. All
 * calls share the array, so calls that overlap on the GPU (concurrent
 * streams) race; calls in one stream are safe back to back (each call writes
 * every scratch row it reads). Errors are reported through
 * dg_last_error(NULL). */
int dg_residuals_noalloc(const void* u, const void* snap, int precision, int n_var, int64_t n_per_var,
                         int64_t var_stride, double c0, double* res, void* stream);

/* ---- batched ensembles --------------------------------------------------
 * No counterpart in the reference (one case per process): n independent
 * instances (own mesh, order, mean flow, sources, observers and time step;
 * shared rho0 and c0) advanced together. Instances of one element type are
 * solved as one disjoint-union mesh; each step is one CUDA graph with one
 * branch per element type. Instances of one element type must have the same
 * boundary group structure (same number of groups, same BC per group).
 * dofs below are instance-local (e*Np + n, mesh local node order). */
typedef struct dg_batch dg_batch;
int dg_batch_create(int n, const dg_mesh_desc* meshes, const dg_phys* phys, const double* dt, int precision,
                    int device, dg_batch** out);
int dg_batch_destroy(dg_batch* b);
const char* dg_batch_last_error(const dg_batch* b);
int dg_batch_info(const dg_batch* b, int* n_groups, int64_t* total_dofs);
int dg_batch_set_state(dg_batch* b, int inst, const double* u);
int dg_batch_get_state(dg_batch* b, int inst, double* u);
/* values[step][src] for the instance's global steps [0, n_steps); NaN = inactive */
int dg_batch_set_sources(dg_batch* b, int inst, int n_src, const int64_t* offsets, const int64_t* dofs,
                         int64_t n_steps, const double* values);
int dg_batch_set_observers(dg_batch* b, int inst, int n_obs, const int64_t* offsets, const int64_t* dofs,
                           const double* weights);
/* n_steps RK4 steps of every instance (each with its own dt); obs receives,
 * instance after instance, [n_steps][n_obs_i][4] (p, vx, vy, vz) */
int dg_batch_run(dg_batch* b, int64_t n_steps, double* obs);
/* timed steps (CUDA events around each per-step graph launch) */
int dg_batch_bench(dg_batch* b, int64_t n_steps, double* step_ms);
/* A batch of FP32 2-D straight-sided instances of orders 2-4 runs each RK
 * stage of all its instances as one persistent launch whose blocks take
 * element tiles of every order from a work queue (on = 1, the default for
 * such a batch); on = 0 (also selected at creation by the environment
 * variable DGFEM_BATCH_FUSED=0) runs one stage kernel per element order, as
 * parallel branches of the step's graph, which is also what every other
 * batch runs. Returns DG_ERR_ARG when on != 0 and the batch holds other
 * element types or FP64. */
int dg_batch_set_fused(dg_batch* b, int on);
/* 1 when the batch runs one launch per stage for all orders, else 0 */
int dg_batch_fused(const dg_batch* b);

/* ------------------------------------------------------------------------
 * Learned spectral surrogate (no counterpart in the reference, which answers
 * every parameter query with a DG run; DG stays the fallback and the
 * measure of the surrogate's error). A fully connected network: widths[0] inputs,
 * n_layers - 1 GELU hidden layers, a linear output layer of widths[n_layers];
 * BF16 weights in the forward/backward passes, FP32 master weights, FP32
 * accumulation. Parameters are one flat FP32 vector, layer after layer:
 * W_l [widths[l+1]][widths[l]] (row-major) then b_l [widths[l+1]].
 * ------------------------------------------------------------------------ */
typedef struct dg_mlp dg_mlp;
int dg_mlp_create(int n_layers, const int* widths, int device, dg_mlp** out);
int dg_mlp_destroy(dg_mlp* m);
const char* dg_mlp_last_error(dg_mlp* m);
int64_t dg_mlp_param_count(dg_mlp* m);
/* host FP32 parameters in/out; setting them resets the optimiser state */
int dg_mlp_set_params(dg_mlp* m, const float* params);
int dg_mlp_get_params(dg_mlp* m, float* params);
/* n rows of inputs [n][widths[0]] -> outputs [n][widths[n_layers]]: host
 * arrays (synchronous), or device arrays on the given CUDA stream (NULL: the
 * network's own stream; asynchronous) */
int dg_mlp_forward(dg_mlp* m, const float* x, int64_t n, float* y);
int dg_mlp_forward_device(dg_mlp* m, const float* x, int64_t n, float* y, void* stream);
/* gradient of the mean squared error over the n x widths[n_layers] outputs
 * against targets t, written as one flat vector like the parameters */
int dg_mlp_gradient(dg_mlp* m, const float* x, const float* t, int64_t n, float* grad, double* loss);
/* training rows (host arrays, copied to the device once) */
int dg_mlp_set_data(dg_mlp* m, const float* x, const float* t, int64_t n);
/* n_steps Adam steps (beta 0.9/0.999, eps 1e-8, decoupled weight decay
 * weight_decay, 0 for plain Adam) on shuffled mini-batches (one permutation
 * per epoch from seed), learning rate decaying from lr to lr_final on a
 * cosine; losses (optional) receives each step's batch loss */
int dg_mlp_train(dg_mlp* m, int64_t n_steps, int batch, double lr, double lr_final, double weight_decay, uint64_t seed,
                 double* losses);
/* The layers' GEMMs on the tensor cores (on != 0: tcgen05 kind::tf32,
 * activations and gradients as TF32 head + tail, BF16 weights exact in TF32,
 * FP32 accumulation; a wait for the MMAs that runs out makes the synchronous
 * calls return DG_ERR_TIMEOUT) or on the CUDA cores (0, the default, faster
 * at the surrogate's sizes). */
int dg_mlp_set_tensor_cores(dg_mlp* m, int on);
int dg_mlp_tensor_cores(const dg_mlp* m);

#ifdef __cplusplus
}
#endif
#endif
