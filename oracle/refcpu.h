/*
 * refcpu — CPU restatement of the reference DGFEM-Acoustic solver numerics.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the parity oracle and the timed
 * CPU baseline. Only tests/, __graft_entry__.smoke() and bench.py (its
 * cpu_baseline leg and its --impl reference arm) may load it. The product
 * (the dgfem GB300 library and the dgalerkin executable) never links it.
 *
 * It follows, function by function:
 *   src/Mesh.cpp:20-686   mesh setup (geometry, faces, connectivity, normals,
 *                          orientation, boundary flags, BC codes, RKR)
 *   src/Mesh.cpp:691-724  mass matrices and their inverses
 *   src/Mesh.cpp:734-975  stiffness vector, face flux, element flux, nodal flux
 *                          and ghost states
 *   src/solver.cpp:38-57  numStep
 *   src/solver.cpp:311-582 rungeKutta (sources, RK4 stages, residuals, observers)
 *   src/solver.cpp:66-302 forwardEuler
 *   src/dgalerkin.cpp:51-70 Gaussian initial conditions
 *   include/configParser.h:38-58 file-source interpolation
 * with the loop structure, storage layout (vector<vector<vector<double>>> for
 * the nodal flux) and OpenMP pragmas of the reference, so that it can be
 * timed as the reference CPU path.
 *
 * Gmsh's role (Lagrange basis, Gauss(2p) quadrature, Jacobians, face
 * extraction) is played by the oracle's own code: a monomial-Vandermonde
 * Lagrange basis on the element's own node set, symmetric degree-2p simplex
 * rules and Gauss-Legendre lines. On straight-sided elements every integrand
 * is a polynomial of degree <= 2p, so any exact rule reproduces the reference
 * up to roundoff. Parity with the reference binary is pinned by the golden
 * residual trace of cases/2d_hilltop (residuals.csv); the penalty sign and the
 * 3-D tangent frame depend on Gmsh's first face quadrature points, which the
 * oracle chooses as documented in its source (parity with the binary in 3-D
 * with p >= 2 rests on that choice).
 */
#ifndef DG_REFCPU_H
#define DG_REFCPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Source kinds (after dipole/quadrupole expansion into monopoles,
 * src/configParser.cpp:87-115). */
enum { REFCPU_SRC_SINE = 0, REFCPU_SRC_CALLBACK = 1, REFCPU_SRC_TABLE = 2 };

typedef double (*refcpu_src_fn)(int src, double t, void* user);

typedef struct {
  /* mesh: nodes, elements (node indices in the mesh file's local order) */
  int dim;   /* 2 or 3 */
  int order; /* polynomial order p (1..4) */
  int nodes_per_elem;
  int64_t n_nodes;
  const double* xyz; /* [n_nodes][3] */
  int64_t n_elems;
  const int64_t* elem_nodes; /* [n_elems][nodes_per_elem] */
  /* boundary groups with a recognised BC type, ascending physical tag order */
  int n_groups;
  const int* group_bc;            /* 1 = Reflecting, 0 = Absorbing */
  const int64_t* group_offsets;   /* [n_groups+1] */
  const int64_t* group_nodes;     /* node indices */
  /* physics and time */
  double v0[3], rho0, c0;
  double t_start, t_end, dt, t_rate;
  int method;      /* 0 = Runge-Kutta, 1 = Euler1 */
  int num_threads; /* OpenMP team size used for every pragma (>= 1) */
  /* sources: kind, params [x,y,z,size,amp,freq,phase,duration] */
  int n_src;
  const int* src_kind;
  const double* src_params; /* [n_src][8] */
  refcpu_src_fn src_fn;     /* value(t) for CALLBACK sources */
  void* src_user;
  const int64_t* src_table_offsets; /* [n_src+1] rows of (t,value) for TABLE sources */
  const double* src_table;          /* [rows][2] */
  /* observers [x,y,z,size] and Gaussian ICs [x,y,z,size,amp] */
  int n_obs;
  const double* obs;
  int n_ic;
  const double* ic;
  int64_t max_steps; /* stop after this many time steps (<0: full run) */
} refcpu_input;

typedef struct {
  /* filled when non-NULL; sizes from refcpu_count_steps */
  double* state;     /* [4][n_elems*nodes_per_elem], final state */
  double* residuals; /* [steps][5] res_p,res_rho,res_vx,res_vy,res_vz */
  double* times;     /* [steps] t at each step */
  double* obs_trace; /* [steps][n_obs][5] rho,p,vx,vy,vz */
  int64_t* snapshot_steps; /* [n_snap] */
  int64_t steps_done;
  int64_t n_snap;
  double setup_seconds;
  double loop_seconds;
  /* penalty-sign histogram of interior faces: [0] s_f=-1, [1] s_f=+1 */
  int64_t penalty_sign_hist[2];
  int64_t n_faces, n_boundary_faces;
} refcpu_output;

/* Number of time steps and snapshot steps of the reference time loop
 * (src/solver.cpp:413-423, floating accumulation of t and tDisplay). */
void refcpu_count_steps(double t_start, double t_end, double dt, double t_rate, int64_t* n_steps, int64_t* n_snap);

/* Full run. Returns 0 on success, non-zero on error (see refcpu_last_error). */
int refcpu_run(const refcpu_input* in, refcpu_output* out);

/* One numStep with beta=0 on state u (after the initial conditions are
 * ignored): k[eq] = dt * M^-1 (S - F) for all four equations
 * (src/solver.cpp:38-57 after Mesh::updateFlux). u, k: [4][E*Np]. */
int refcpu_stage(const refcpu_input* in, const double* u, double* k);

/* Per-face data of the setup: for each element local face, the unique face
 * id, the neighbour element (-1 on the boundary), the orientation sign, the
 * BC code (-1 interior) and the penalty sign (0 on the boundary).
 * Arrays of n_elems*faces_per_elem entries. */
int refcpu_faces(const refcpu_input* in, int64_t* face_id, int64_t* nbr, int* orient, int* bc, int* penalty);

/* Initial state from the Gaussian ICs (src/dgalerkin.cpp:51-70). u: [4][E*Np] */
int refcpu_initial_state(const refcpu_input* in, double* u);

/* The oracle's stand-in quadrature rules: kind 1 Gauss line with `degree`
 * points, 2 triangle rule, 3 tetrahedron rule of that degree. */
int refcpu_rule(int kind, int degree, int* n, double* x, double* w);

const char* refcpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
