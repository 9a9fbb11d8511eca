// Configuration, formula, source and output entry points of the host front
// end (include/dgfem_host.h).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "quadrature.h"
#include "../../include/dgfem_host.h"
#include "config.h"
#include "host_common.h"

struct dgh_config {
  dgcfg::Config c;
};

namespace dgout {
void write_wav(const std::string& path, const float* s, int64_t n, uint32_t rate);
void read_wav(const std::string& path, std::vector<float>& out, uint32_t& rate);
void spectra(const float* V, int64_t count, double dt, int64_t* nb_out, std::vector<double>& fftrows,
             std::vector<double>& psdrows);
void write_spectra(const std::string& prefix, const float* V, int64_t count, double dt);
void write_vtu(const std::string& path, int dim, const std::vector<int64_t>& node_tags, const std::vector<double>& xyz,
               int nodes_per_elem, const std::vector<int64_t>& elem_nodes, const double* cp, const double* crho,
               const double* cv);
void write_pvd(const std::string& path, double t_start, double t_end, double dt, double t_rate);
}  // namespace dgout

extern "C" {

int dgh_config_load(const char* path, dgh_config** out) {
  return dghost::guard([&] {
    auto* c = new dgh_config;
    try {
      c->c = dgcfg::load(path ? path : "");
    } catch (...) {
      delete c;
      throw;
    }
    *out = c;
  });
}
void dgh_config_free(dgh_config* c) { delete c; }
const char* dgh_config_mesh_file(const dgh_config* c) { return c->c.mesh_file.c_str(); }
const char* dgh_config_time_method(const dgh_config* c) { return c->c.time_method.c_str(); }
const char* dgh_config_element_type(const dgh_config* c) { return c->c.element_type.c_str(); }
const char* dgh_config_precision(const dgh_config* c) { return c->c.precision.c_str(); }
void dgh_config_numbers(const dgh_config* c, double* t_start, double* t_end, double* dt, double* t_rate, double* v0,
                        double* rho0, double* c0) {
  const auto& k = c->c;
  if (t_start) *t_start = k.t_start;
  if (t_end) *t_end = k.t_end;
  if (dt) *dt = k.dt;
  if (t_rate) *t_rate = k.t_rate;
  if (v0) v0[0] = k.v0[0], v0[1] = k.v0[1], v0[2] = k.v0[2];
  if (rho0) *rho0 = k.rho0;
  if (c0) *c0 = k.c0;
}
int dgh_config_num_threads(const dgh_config* c) { return c->c.num_threads; }
int dgh_config_num_bc(const dgh_config* c) { return (int)c->c.bcs.size(); }
void dgh_config_bc(const dgh_config* c, int i, int* tag, int* type) {
  if (tag) *tag = c->c.bcs[i].first;
  if (type) *type = c->c.bcs[i].second;
}
int dgh_config_num_sources(const dgh_config* c) { return (int)c->c.sources.size(); }
void dgh_config_source(const dgh_config* c, int i, int* kind, double* params, const char** formula,
                       int64_t* table_rows, const double** table) {
  const auto& s = c->c.sources[i];
  if (kind) *kind = s.kind;
  if (params) std::memcpy(params, s.params, sizeof(s.params));
  if (formula) *formula = s.formula.c_str();
  if (table_rows) *table_rows = (int64_t)s.table.size() / 2;
  if (table) *table = s.table.data();
}
int dgh_config_num_observers(const dgh_config* c) { return (int)c->c.observers.size(); }
void dgh_config_observer(const dgh_config* c, int i, double* xyzr) {
  for (int k = 0; k < 4; ++k) xyzr[k] = c->c.observers[i][k];
}
int dgh_config_num_ics(const dgh_config* c) { return (int)c->c.ics.size(); }
void dgh_config_ic(const dgh_config* c, int i, double* v) {
  for (int k = 0; k < 5; ++k) v[k] = c->c.ics[i][k];
}
double dgh_source_value(const dgh_config* c, int i, double t) { return dgcfg::source_value(c->c.sources[i], t); }

int dgh_formula_eval(const char* expr, double t, double* value) {
  double v = -1.0;
  bool ok = dgcfg::eval_formula(expr ? expr : "", t, &v);
  if (value) *value = v;
  if (!ok) dghost::set_error(std::string("malformed formula: '") + (expr ? expr : "") + "'");
  return ok ? 0 : 1;
}

int dgh_write_vtu(const char* path, const dgh_mesh* m, const double* cell_p, const double* cell_rho,
                  const double* cell_v) {
  return dghost::guard([&] {
    dgout::write_vtu(path, m->m.dim, m->m.node_tags, m->m.xyz, m->m.nodes_per_elem, m->m.elem_nodes, cell_p, cell_rho,
                     cell_v);
  });
}
int dgh_write_pvd(const char* path, double t_start, double t_end, double dt, double t_rate) {
  return dghost::guard([&] { dgout::write_pvd(path, t_start, t_end, dt, t_rate); });
}
int dgh_write_wav(const char* path, const float* samples, int64_t n, uint32_t sample_rate) {
  return dghost::guard([&] { dgout::write_wav(path, samples, n, sample_rate); });
}
int dgh_read_wav(const char* path, float** samples, int64_t* n, uint32_t* sample_rate) {
  return dghost::guard([&] {
    std::vector<float> v;
    uint32_t r = 0;
    dgout::read_wav(path, v, r);
    float* p = (float*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(float));
    if (!v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(float));
    *samples = p;
    *n = (int64_t)v.size();
    *sample_rate = r;
  });
}
int dgh_write_spectra(const char* prefix, const float* p, int64_t n, double dt) {
  return dghost::guard([&] { dgout::write_spectra(prefix, p, n, dt); });
}
int dgh_spectra(const float* p, int64_t n, double dt, int64_t* nb, double* fft_rows, double* psd_rows) {
  return dghost::guard([&] {
    std::vector<double> f, q;
    dgout::spectra(p, n, dt, nb, f, q);
    if (fft_rows) std::memcpy(fft_rows, f.data(), f.size() * sizeof(double));
    if (psd_rows) std::memcpy(psd_rows, q.data(), q.size() * sizeof(double));
  });
}

int dgh_quadrature(int kind, int degree, int* n, double* x, double* w) {
  return dghost::guard([&] {
    dgref::QRule r;
    if (kind == 1)
      r = dgref::gauss_legendre(degree);
    else if (kind == 2)
      r = dgref::triangle_rule(degree);
    else if (kind == 3)
      r = dgref::tetrahedron_rule(degree);
    else
      throw std::runtime_error("quadrature kind must be 1 (line), 2 (triangle) or 3 (tetrahedron)");
    *n = r.n;
    if (x) std::memcpy(x, r.x.data(), r.x.size() * sizeof(double));
    if (w) std::memcpy(w, r.w.data(), r.w.size() * sizeof(double));
  });
}

}  // extern "C"
