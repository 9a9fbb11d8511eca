// Mesh and schedule entry points of the host front end (include/dgfem_host.h).
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../../include/dgfem_host.h"
#include "host_common.h"
#include "mshio.h"

namespace dghost {
thread_local std::string g_last_error;
void set_error(const std::string& s) { g_last_error = s; }
}  // namespace dghost

extern "C" {

const char* dgh_last_error(void) { return dghost::g_last_error.c_str(); }

int dgh_mesh_load(const char* path, dgh_mesh** out) {
  return dghost::guard([&] {
    auto* m = new dgh_mesh;
    try {
      m->m = dgmsh::load_volume_mesh(path ? path : "");
    } catch (...) {
      delete m;
      throw;
    }
    *out = m;
  });
}

void dgh_mesh_free(dgh_mesh* m) { delete m; }

void dgh_mesh_info(const dgh_mesh* m, int* dim, int* order, int* nodes_per_elem, int64_t* n_nodes,
                   int64_t* n_elems, int* n_groups) {
  if (dim) *dim = m->m.dim;
  if (order) *order = m->m.order;
  if (nodes_per_elem) *nodes_per_elem = m->m.nodes_per_elem;
  if (n_nodes) *n_nodes = (int64_t)m->m.node_tags.size();
  if (n_elems) *n_elems = (int64_t)m->m.elem_tags.size();
  if (n_groups) *n_groups = (int)m->m.bc_groups.size();
}

const double* dgh_mesh_xyz(const dgh_mesh* m) { return m->m.xyz.data(); }
const int64_t* dgh_mesh_node_tags(const dgh_mesh* m) { return m->m.node_tags.data(); }
const int64_t* dgh_mesh_elem_nodes(const dgh_mesh* m) { return m->m.elem_nodes.data(); }

int dgh_mesh_group(const dgh_mesh* m, int g, int* tag, const char** name, int64_t* n_nodes, const int64_t** nodes) {
  if (g < 0 || g >= (int)m->m.bc_groups.size()) {
    dghost::set_error("group index out of range");
    return 1;
  }
  if (tag) *tag = m->m.bc_groups[g].tag;
  if (name) *name = m->m.bc_groups[g].name.c_str();
  if (n_nodes) *n_nodes = (int64_t)m->m.bc_group_nodes[g].size();
  if (nodes) *nodes = m->m.bc_group_nodes[g].data();
  return 0;
}

int dgh_mesh_write(const char* path, int dim, int order, int64_t n_nodes, const double* xyz, int64_t n_elems,
                   const int64_t* elem_nodes, int n_groups, const int* group_tags, const char* const* group_names,
                   const int64_t* group_face_offsets, const int64_t* group_face_nodes) {
  return dghost::guard([&] {
    int vn = dgmsh::gmsh_type_nodes(dgmsh::gmsh_type_for(dim, order));
    int fn = dgmsh::gmsh_type_nodes(dgmsh::gmsh_type_for(dim - 1, order));
    if (vn == 0 || fn == 0) throw std::runtime_error("unsupported dim/order for writing");
    std::vector<double> X(xyz, xyz + 3 * n_nodes);
    std::vector<int64_t> EN(elem_nodes, elem_nodes + n_elems * vn);
    std::vector<dgmsh::WriteGroup> groups(n_groups);
    for (int g = 0; g < n_groups; ++g) {
      groups[g].tag = group_tags[g];
      groups[g].name = group_names[g] ? group_names[g] : "";
      groups[g].face_nodes.assign(group_face_nodes + group_face_offsets[g] * fn,
                                  group_face_nodes + group_face_offsets[g + 1] * fn);
    }
    dgmsh::write_msh41(path, dim, order, X, EN, groups);
  });
}

// src/solver.cpp:413-423: the loop runs while t <= t_end with t and tDisplay
// accumulated in double; a snapshot is taken when tDisplay >= rate or at step 0.
void dgh_count_steps(double t_start, double t_end, double dt, double t_rate, int64_t* n_steps, int64_t* n_snap) {
  int64_t ns = 0, nsn = 0;
  for (double t = t_start, step = 0, tDisplay = 0; t <= t_end; t += dt, tDisplay += dt, ++step) {
    if (tDisplay >= t_rate || step == 0) {
      tDisplay = 0;
      ++nsn;
    }
    ++ns;
    if (!(dt > 0)) break;
  }
  if (n_steps) *n_steps = ns;
  if (n_snap) *n_snap = nsn;
}

void dgh_schedule(double t_start, double t_end, double dt, double t_rate, double* times, unsigned char* snap) {
  int64_t i = 0;
  for (double t = t_start, step = 0, tDisplay = 0; t <= t_end; t += dt, tDisplay += dt, ++step) {
    unsigned char s = 0;
    if (tDisplay >= t_rate || step == 0) {
      tDisplay = 0;
      s = 1;
    }
    if (times) times[i] = t;
    if (snap) snap[i] = s;
    ++i;
    if (!(dt > 0)) break;
  }
}

void dgh_free(void* p) { std::free(p); }

}  // extern "C"
