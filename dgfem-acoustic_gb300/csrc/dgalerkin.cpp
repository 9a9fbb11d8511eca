// dgalerkin — drop-in driver with the reference's command line and outputs
// (src/dgalerkin.cpp:14-85, src/solver.cpp:311-582), running the time loop on
// the GPU through the C ABI (include/dgfem_gb300.h).
//
//   dgalerkin <config.conf | config.json>
//
// Reads the configuration and the Gmsh mesh it names, applies the Gaussian
// initial conditions, runs Runge-Kutta (RK4) or Euler1 time stepping and
// writes, relative to the working directory:
//   residuals.csv, results/observers<i>.txt, results/result<step>.vtu,
//   results/observer_<i>.wav, results/observer_<i>_fft.txt / _psd.txt,
//   results.pvd.
// Exit status: 0 on success, E2BIG without exactly one argument (as the
// reference), 1 on any error (message on stderr).
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dgfem_gb300.h"
#include "../../include/dgfem_host.h"
#include "config.h"
#include "mshio.h"

namespace {

[[noreturn]] void fail(const std::string& m) { throw std::runtime_error(m); }

void ck(int rc, dg_ctx* c, const char* what) {
  if (rc != DG_OK) fail(std::string(what) + ": " + dg_last_error(c));
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 2) return E2BIG;
  dg_ctx* ctx = nullptr;
  dg_vtu_writer* vw = nullptr;
  try {
    auto wall0 = std::chrono::steady_clock::now();
    dgcfg::Config cfg = dgcfg::load(argv[1]);
    std::printf("Config loaded : %s\n", argv[1]);
    if (cfg.time_method != "Euler1" && cfg.time_method != "Runge-Kutta") fail("Time integration method error");
    dgmsh::VolumeMesh mesh = dgmsh::load_volume_mesh(cfg.mesh_file);
    const int dim = mesh.dim, np = mesh.nodes_per_elem;
    const int64_t E = (int64_t)mesh.elem_tags.size(), N = E * np;
    // boundary groups with a BC type, ascending physical tag
    std::vector<int> gbc;
    std::vector<int64_t> goff{0}, gnodes;
    for (size_t g = 0; g < mesh.bc_groups.size(); ++g)
      for (auto& bc : cfg.bcs)
        if (bc.first == mesh.bc_groups[g].tag) {
          gbc.push_back(bc.second);
          gnodes.insert(gnodes.end(), mesh.bc_group_nodes[g].begin(), mesh.bc_group_nodes[g].end());
          goff.push_back((int64_t)gnodes.size());
        }
    dg_mesh_desc md{};
    md.dim = dim, md.order = mesh.order, md.nodes_per_elem = np;
    md.n_nodes = (int64_t)mesh.node_tags.size(), md.xyz = mesh.xyz.data();
    md.n_elems = E, md.elem_nodes = mesh.elem_nodes.data();
    md.n_groups = (int)gbc.size(), md.group_bc = gbc.data(), md.group_offsets = goff.data();
    md.group_nodes = gnodes.data();
    dg_phys ph{};
    for (int d = 0; d < 3; ++d) ph.v0[d] = cfg.v0[d];
    ph.rho0 = cfg.rho0, ph.c0 = cfg.c0;
    int prec = cfg.precision == "fp32" ? DG_FP32 : DG_FP64;
    ck(dg_create(&md, &ph, prec, 0, &ctx), nullptr, "dg_create");
    dg_info_t info{};
    dg_get_info(ctx, &info);
    std::printf("Mesh: %lld elements, dim %d, order %d, %lld faces (%lld boundary), %s, setup %.1f ms\n",
                (long long)E, dim, mesh.order, (long long)info.n_faces, (long long)info.n_boundary_faces,
                prec == DG_FP32 ? "FP32" : "FP64", info.setup_ms);

    // DG node coordinates (element-major, mesh local order)
    auto X = [&](int64_t n, int d) { return mesh.xyz[3 * mesh.elem_nodes[n] + d]; };
    // Gaussian initial conditions (src/dgalerkin.cpp:51-70)
    std::vector<double> u(4 * N, 0.0);
    for (auto& ic : cfg.ics) {
      double x = ic[0], y = ic[1], z = ic[2], size = ic[3], amp = ic[4];
      for (int64_t n = 0; n < N; ++n)
        u[n] += amp * std::exp(-((X(n, 0) - x) * (X(n, 0) - x) + (X(n, 1) - y) * (X(n, 1) - y) +
                                 (X(n, 2) - z) * (X(n, 2) - z)) / size);
    }
    ck(dg_set_state(ctx, u.data()), ctx, "dg_set_state");
    // source node sets (src/solver.cpp:339-358)
    const int ns = (int)cfg.sources.size();
    std::vector<int64_t> soff{0}, sdofs;
    for (auto& s : cfg.sources) {
      for (int64_t n = 0; n < N; ++n)
        if (std::pow(X(n, 0) - s.params[0], 2) + std::pow(X(n, 1) - s.params[1], 2) +
                std::pow(X(n, 2) - s.params[2], 2) <
            std::pow(s.params[3], 2))
          sdofs.push_back(n);
      soff.push_back((int64_t)sdofs.size());
    }
    ck(dg_set_sources(ctx, ns, soff.data(), sdofs.data()), ctx, "dg_set_sources");
    // observer node sets and IDW weights (src/solver.cpp:360-383, :559)
    const int no = (int)cfg.observers.size();
    std::vector<int64_t> ooff{0}, odofs;
    std::vector<double> ow;
    for (auto& o : cfg.observers) {
      for (int64_t n = 0; n < N; ++n) {
        double d = std::sqrt(std::pow(X(n, 0) - o[0], 2) + std::pow(X(n, 1) - o[1], 2) + std::pow(X(n, 2) - o[2], 2));
        if (d < o[3]) odofs.push_back(n), ow.push_back(1.0 / (std::pow(d, 2) + 1.0e-12));
      }
      ooff.push_back((int64_t)odofs.size());
    }
    ck(dg_set_observers(ctx, no, ooff.data(), odofs.data(), ow.data()), ctx, "dg_set_observers");
    // time schedule (src/solver.cpp:413-423) and per-step source values
    int64_t nsteps = 0, nsnap = 0;
    dgh_count_steps(cfg.t_start, cfg.t_end, cfg.dt, cfg.t_rate, &nsteps, &nsnap);
    std::vector<double> times(nsteps);
    std::vector<unsigned char> snap(nsteps);
    dgh_schedule(cfg.t_start, cfg.t_end, cfg.dt, cfg.t_rate, times.data(), snap.data());
    if (ns > 0) {
      std::vector<double> vals(nsteps * ns);
      for (int64_t k = 0; k < nsteps; ++k)
        for (int s = 0; s < ns; ++s) vals[k * ns + s] = dgcfg::source_value(cfg.sources[s], times[k]);
      ck(dg_set_source_values(ctx, nsteps, vals.data()), ctx, "dg_set_source_values");
    }
    // outputs
    mkdir("results", 0755);
    FILE* fres = std::fopen("residuals.csv", "w");
    if (!fres) fail("cannot write residuals.csv");
    std::fprintf(fres, "time;res_p;res_rho;res_vx;res_vy;res_vz;elapsed_time\n");
    const bool rk4 = cfg.time_method == "Runge-Kutta";
    std::vector<FILE*> fobs(no, nullptr);
    for (int o = 0; o < no; ++o) {
      std::string fn = "results/observers" + std::to_string(o + 1) + ".txt";
      fobs[o] = std::fopen(fn.c_str(), "w");
      if (!fobs[o]) fail("cannot write " + fn);
      // the Euler1 path of the reference labels the columns differently (src/solver.cpp:150)
      std::fprintf(fobs[o], rk4 ? "time;density;pressure;velocity_x;velocity_y;velocity_z\n"
                                : "time;pressure;density;velocity_x;velocity_y;velocity_z\n");
    }
    std::vector<std::vector<float>> wave(no);
    // VTU snapshots (src/Mesh.cpp:1136-1230): the mesh part once, the cell
    // means of each output step computed on the GPU and written by the
    // writer's background thread while the time loop goes on.
    // DGFEM_VTU_COMPRESSION: 1 zlib (VTK's default), 0 none, unset: zlib when
    // the system library loads.
    {
      int64_t maxtag = 0;
      for (auto t : mesh.node_tags) maxtag = std::max<int64_t>(maxtag, t);
      std::vector<double> pts(3 * maxtag, 0.0);
      for (size_t k = 0; k < mesh.node_tags.size(); ++k)
        for (int d = 0; d < 3; ++d) pts[3 * (mesh.node_tags[k] - 1) + d] = mesh.xyz[3 * k + d];
      const int nc = dim + 1;
      std::vector<int64_t> cells(E * nc);
      for (int64_t e = 0; e < E; ++e)
        for (int k = 0; k < nc; ++k) cells[e * nc + k] = mesh.node_tags[mesh.elem_nodes[e * np + k]] - 1;
      const char* ev = std::getenv("DGFEM_VTU_COMPRESSION");
      const int comp = ev ? std::atoi(ev) : -1;
      if (dg_vtu_writer_create(ctx, maxtag, pts.data(), cells.data(), comp, 0, &vw) != DG_OK)
        fail("cannot create the VTU writer (compression " + std::to_string(comp) + ")");
    }
    const double c0sq = std::pow(cfg.c0, 2);
    double loop_s = 0.0;
    int64_t i = 0;
    while (i < nsteps) {
      int64_t j = i + 1;
      while (j < nsteps && !snap[j]) ++j;
      if (snap[i]) {
        ck(dg_snapshot(ctx), ctx, "dg_snapshot");
        std::string vtu = "results/result" + std::to_string((int)i) + ".vtu";
        if (dg_vtu_write_async(vw, vtu.c_str()) != DG_OK) fail(std::string("VTU: ") + dg_vtu_writer_last_error(vw));
        std::printf("[%g/%g s] Step number : %lld\n", times[i], cfg.t_end, (long long)i);
      }
      const int64_t n = j - i;
      std::vector<double> res(n * 5), obs(n * std::max(no, 1) * 4);
      auto t0 = std::chrono::steady_clock::now();
      int rc = rk4 ? dg_run(ctx, n, cfg.dt, res.data(), obs.data()) : dg_run_euler(ctx, n, cfg.dt, res.data(), obs.data());
      double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      loop_s += el;
      if (rc != DG_OK && rc != DG_ERR_NONFINITE) ck(rc, ctx, "dg_run");
      for (int64_t k = 0; k < n; ++k) {
        std::fprintf(fres, "%g;", times[i + k]);
        for (int q = 0; q < 5; ++q) std::fprintf(fres, "%g;", res[k * 5 + q]);
        std::fprintf(fres, "%g\n", el / n);
        for (int o = 0; o < no; ++o) {
          const double* ov = &obs[(k * no + o) * 4];
          double p = ov[0];
          std::fprintf(fobs[o], "%g;%g;%g;%g;%g;%g\n", times[i + k], p / c0sq, p, ov[1], ov[2], ov[3]);
          wave[o].push_back((float)p);
        }
      }
      if (rc == DG_ERR_NONFINITE) std::fprintf(stderr, "warning: %s\n", dg_last_error(ctx));
      i = j;
    }
    std::fclose(fres);
    for (FILE* f : fobs) std::fclose(f);
    for (int o = 0; o < no; ++o) {
      std::string base = "results/observer_" + std::to_string(o + 1);
      if (dgh_write_wav((base + ".wav").c_str(), wave[o].data(), (int64_t)wave[o].size(), (uint32_t)(1.0 / cfg.dt)) != 0)
        fail(dgh_last_error());
      if (wave[o].size() >= 2 && dgh_write_spectra(base.c_str(), wave[o].data(), (int64_t)wave[o].size(), cfg.dt) != 0)
        fail(dgh_last_error());
    }
    if (dgh_write_pvd("results.pvd", cfg.t_start, cfg.t_end, cfg.dt, cfg.t_rate) != 0) fail(dgh_last_error());
    if (dg_vtu_writer_flush(vw) != DG_OK) fail(std::string("VTU: ") + dg_vtu_writer_last_error(vw));
    dg_vtu_writer_destroy(vw);
    vw = nullptr;
    double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    double dofs = (double)E * np * (dim + 1);
    std::printf("Done: %lld steps, time loop %.3f s (%.3e DOF-updates/s), total %.3f s\n", (long long)nsteps, loop_s,
                nsteps > 0 && loop_s > 0 ? dofs * nsteps / loop_s : 0.0, total);
    dg_destroy(ctx);
    return 0;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "Error: %s\n", e.what());
    if (vw) dg_vtu_writer_destroy(vw);
    if (ctx) dg_destroy(ctx);
    return 1;
  }
}
