/*
 * dgfem_host.h — host-side front end of the GB300 DG solver (no GPU needed).
 *
 * These entry points replace the parts of the reference that reach the mesh
 * and configuration through the Gmsh SDK and nlohmann-json:
 *   dgh_mesh_*    : gmsh::open + getElementsByType + getNodesForPhysicalGroup
 *                   (src/Mesh.cpp:40-48, src/Mesh.cpp:588, src/configParser.cpp:197-223)
 *   dgh_config_*  : config::parseConfig / config::parseJSON
 *                   (src/configParser.cpp:33-242, :243-451, include/configParser.h:69-115)
 *   dgh_formula_eval : EQ_EDIT::value (src/eqEdit.cpp:292-311)
 *   dgh_source_value : Sources::value / Sources::interpolate_value and the
 *                   per-step source rule of src/solver.cpp:455-483
 *   dgh_count_steps : the time-loop step and snapshot schedule (src/solver.cpp:413-423)
 *   dgh_write_*   : VTU/PVD, WAV and spectrum writers (src/Mesh.cpp:1136-1253,
 *                   src/utils.cpp:179-296, src/fft.cpp:146-271)
 * All functions return 0 on success and a non-zero code on error; the error
 * text is available from dgh_last_error(). Nothing here throws or exits.
 */
#ifndef DGFEM_HOST_H
#define DGFEM_HOST_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

const char* dgh_last_error(void);

/* ---- mesh ---------------------------------------------------------------- */
typedef struct dgh_mesh dgh_mesh;
int dgh_mesh_load(const char* path, dgh_mesh** out);
void dgh_mesh_free(dgh_mesh* m);
/* dim, order, nodes per element, node count, element count, boundary group count */
void dgh_mesh_info(const dgh_mesh* m, int* dim, int* order, int* nodes_per_elem, int64_t* n_nodes,
                   int64_t* n_elems, int* n_groups);
const double* dgh_mesh_xyz(const dgh_mesh* m);          /* [n_nodes][3] */
const int64_t* dgh_mesh_node_tags(const dgh_mesh* m);   /* [n_nodes] */
const int64_t* dgh_mesh_elem_nodes(const dgh_mesh* m);  /* [n_elems][nodes_per_elem], node indices */
/* boundary group g (ascending physical tag): tag, name, node indices */
int dgh_mesh_group(const dgh_mesh* m, int g, int* tag, const char** name, int64_t* n_nodes, const int64_t** nodes);
/* Writes a Gmsh 4.1 ASCII mesh (volume elements + one entity per boundary group). */
int dgh_mesh_write(const char* path, int dim, int order, int64_t n_nodes, const double* xyz, int64_t n_elems,
                   const int64_t* elem_nodes, int n_groups, const int* group_tags, const char* const* group_names,
                   const int64_t* group_face_offsets, const int64_t* group_face_nodes);

/* ---- configuration ------------------------------------------------------- */
typedef struct dgh_config dgh_config;
/* Parses a .conf or .json file (chosen by extension) and the mesh it names,
 * exactly like the reference: the mesh is opened to map physical names to
 * BC types. */
int dgh_config_load(const char* path, dgh_config** out);
void dgh_config_free(dgh_config* c);
const char* dgh_config_mesh_file(const dgh_config* c);
const char* dgh_config_time_method(const dgh_config* c);
const char* dgh_config_element_type(const dgh_config* c);
/* project extension: working precision "fp64" (default) or "fp32"
 * (.json: "gpu": {"precision": ...}; .conf: gpuPrecision = ...) */
const char* dgh_config_precision(const dgh_config* c);
/* t_start, t_end, dt, t_rate, v0[3], rho0, c0 */
void dgh_config_numbers(const dgh_config* c, double* t_start, double* t_end, double* dt, double* t_rate,
                        double* v0, double* rho0, double* c0);
int dgh_config_num_threads(const dgh_config* c); /* after the 1 -> 0 rewrite */
/* boundary conditions: count, then physical tag and type (0 Absorbing, 1 Reflecting) in ascending tag order */
int dgh_config_num_bc(const dgh_config* c);
void dgh_config_bc(const dgh_config* c, int i, int* tag, int* type);
/* sources after dipole/quadrupole expansion: kind 0 = sine, 1 = formula, 2 = data table;
 * params[8] = x, y, z, size, amp, freq, phase, duration (formula: duration in params[7]) */
int dgh_config_num_sources(const dgh_config* c);
void dgh_config_source(const dgh_config* c, int i, int* kind, double* params, const char** formula,
                       int64_t* table_rows, const double** table);
/* observers [x,y,z,size] and Gaussian ICs [x,y,z,size,amp] */
int dgh_config_num_observers(const dgh_config* c);
void dgh_config_observer(const dgh_config* c, int i, double* xyzr);
int dgh_config_num_ics(const dgh_config* c);
void dgh_config_ic(const dgh_config* c, int i, double* xyz_size_amp);
/* Value written by source i at time t, or NaN when the source writes nothing
 * at t (sine/formula sources past their duration). */
double dgh_source_value(const dgh_config* c, int i, double t);

/* ---- formula evaluator ---------------------------------------------------- */
/* Evaluates expr with variable t. Returns 0 and the value, or non-zero for a
 * malformed expression (the reference then yields -1, which *value is set to). */
int dgh_formula_eval(const char* expr, double t, double* value);

/* ---- time schedule --------------------------------------------------------- */
void dgh_count_steps(double t_start, double t_end, double dt, double t_rate, int64_t* n_steps, int64_t* n_snap);
/* times[n_steps] and snapshot flags[n_steps] (1 at snapshot steps) */
void dgh_schedule(double t_start, double t_end, double dt, double t_rate, double* times, unsigned char* snap);

/* ---- outputs --------------------------------------------------------------- */
/* results/result<step>.vtu: linear cells from the first dim+1 nodes of each
 * element, points = all mesh nodes indexed by tag-1, cell data = element means */
int dgh_write_vtu(const char* path, const dgh_mesh* m, const double* cell_p, const double* cell_rho,
                  const double* cell_v /* [E][3] */);
int dgh_write_pvd(const char* path, double t_start, double t_end, double dt, double t_rate);
/* 16-bit mono PCM, sample rate (uint32)(1/dt), value*32767 truncated */
int dgh_write_wav(const char* path, const float* samples, int64_t n, uint32_t sample_rate);
/* WAV reader (8/16/24/32-bit PCM): samples as float in [-1,1], sample rate */
int dgh_read_wav(const char* path, float** samples, int64_t* n, uint32_t* sample_rate);
void dgh_free(void* p);
/* <prefix>_fft.txt and <prefix>_psd.txt from a pressure trace (largest
 * power-of-two prefix, mean removed) */
int dgh_write_spectra(const char* prefix, const float* p, int64_t n, double dt);
/* Amplitude spectrum rows [nb/2][5] (freq, norm, real, imag, SPL) and one-sided
 * PSD rows [nb/2+1][3] (freq, PSD, dB) of a trace, as written to the files */
/* Quadrature rules of the curved-element path (stand-ins for Gmsh's
 * Gauss(2p) rules, src/Mesh.cpp:49-52,213-215): kind 1 Gauss-Legendre line
 * on [-1,1] with `degree` points, 2 triangle rule of that degree, 3
 * tetrahedron rule of that degree. *n receives the point count; x (n*dim
 * reference coordinates) and w (n weights) are filled when non-NULL. */
int dgh_quadrature(int kind, int degree, int* n, double* x, double* w);
int dgh_spectra(const float* p, int64_t n, double dt, int64_t* nb, double* fft_rows, double* psd_rows);

#ifdef __cplusplus
}
#endif
#endif
