"""Benchmark: RK4 DOF-updates/s of the GB300 DG solver on the 3-D LEE
workload (cube [-1,1]^3, 32^3 x 6 = 196,608 jittered tetrahedra, p = 3,
quiescent medium rho0 = 1.225, c0 = 340, 50 Hz monopole at the centre,
Reflecting on x = +-1, Absorbing elsewhere, dt from CFL 0.5, 8 observers).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp32|fp64]
  python bench.py --impl reference ...   (the reference's CPU path, restated)

One step = one full RK4 time step of the reference's loop (source injection,
four RHS stages, the combine, the residual diagnostic and the observer
samples) over the whole mesh. Prints one JSON line (rank 0).

Multi-GPU runs are independent replicas (one solver per GPU, no collective
on the data path); value = DOF-updates of all ranks / max rank time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="3D LEE cube, 196,608 tets, p=3", counts=(32, 32, 32), order=3, jitter=0.2, seed=2,
                rho0=1.225, c0=340.0, v0=(0.0, 0.0, 0.0), freq=50.0, amp=0.1, size=0.1, cfl=0.5, n_obs=8)
BCS = {"xmin": "Reflecting", "xmax": "Reflecting", "ymin": "Absorbing", "ymax": "Absorbing", "zmin": "Absorbing",
       "zmax": "Absorbing"}
METRIC = "RK4 DOF-updates/s"
UNIT = "DOF-updates/s"
L2_FLUSH_BYTES = 256 << 20


def _pkg():
    import importlib
    return importlib.import_module("dgfem-acoustic_gb300")


def _oracle():
    import importlib.util
    spec = importlib.util.spec_from_file_location("refcpu", os.path.join(ROOT, "oracle", "refcpu.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def build_problem(counts=None):
    """Mesh, solver groups, dt, sources and observers of the workload."""
    pkg = _pkg()
    W = WORKLOAD
    m = pkg.meshgen.box(counts=counts or W["counts"], order=W["order"], jitter=W["jitter"], seed=W["seed"])
    mesh = dict(dim=3, order=W["order"], xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=pkg.meshgen.solver_groups(m, BCS))
    # dt = CFL * h_min / ((c0 + |v0|) (2p + 1)), h_min = smallest element altitude
    hmin = pkg.meshgen.min_altitude(mesh)
    dt = W["cfl"] * hmin / ((W["c0"] + np.linalg.norm(W["v0"])) * (2 * W["order"] + 1))
    rng = np.random.default_rng(W["seed"])
    obs = [tuple(rng.uniform(-0.8, 0.8, 3)) + (0.1,) for _ in range(W["n_obs"])]
    src = [0.0, 0.0, 0.0, W["size"], W["amp"], W["freq"], 0.0, 1e9]
    return mesh, dt, src, obs


def node_sets(mesh, src, obs):
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    d2 = (x[:, 0] - src[0]) ** 2 + (x[:, 1] - src[1]) ** 2 + (x[:, 2] - src[2]) ** 2
    sdofs = [np.nonzero(d2 < src[3] ** 2)[0]]
    odofs, ows = [], []
    for o in obs:
        d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2 + (x[:, 2] - o[2]) ** 2)
        idx = np.nonzero(d < o[3])[0]
        odofs.append(idx)
        ows.append(1.0 / (d[idx] ** 2 + 1e-12))
    return sdofs, odofs, ows


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler reports (nvidia-smi
            # takes a moment to start), so that its samples fall inside it
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) > 8 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def geometry_record_words(dim, w):
    """Words of one element's geometry record as the stage kernel reads it:
    metric (dim*dim), per face normal (dim) and scale, the element's mean flow
    (dim) and time-step scale, padded to 16 bytes."""
    raw = dim * dim + (dim + 1) * (dim + 1) + dim + 1
    vec = 16 // w
    return (raw + vec - 1) // vec * vec


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the stage kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")
    try:
        d = json.load(open(p))
        return d.get("bytes_per_launch_full_workload")
    except Exception:
        return None


def run_gpu(args, rank, world):
    pkg = _pkg()
    import ctypes
    device = int(os.environ.get("LOCAL_RANK", "0"))
    mesh, dt, src, obs = build_problem()
    prec = pkg.gpu.DG_FP32 if args.precision == "fp32" else pkg.gpu.DG_FP64
    W = WORKLOAD
    S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], precision=prec, device=device)
    if args.variant != -2:
        S.tune(args.variant)
    info = S.info()
    E, np_ = mesh["elem_nodes"].shape
    nv = 4
    dofs = E * np_ * nv
    sdofs, odofs, ows = node_sets(mesh, src, obs)
    S.set_sources(sdofs)
    nsteps_total = args.warmup + 3 * args.steps + 8
    times = np.arange(nsteps_total) * dt
    S.set_source_values((src[4] * np.sin(2 * np.pi * src[5] * times + src[6]))[:, None])
    S.set_observers(odofs, ows)
    u0 = np.zeros((4, E * np_))
    S.set_state(u0)
    S.snapshot()
    # warm-up (also builds the per-step graph)
    S.run(args.warmup, dt)
    barrier(world)
    # ---- timed device region: per-step CUDA events on the solver's stream ----
    with ClockSampler(device) as clk:
        step_ms, kern_ms = S.bench_steps(args.steps, dt, flush_bytes=L2_FLUSH_BYTES, kernel_time=True)
    total_ms = step_ms * args.steps
    total_ms = allmax(total_ms, world)
    # ---- end-to-end through the C ABI with host buffers (page-locked, as a
    # user of the library allocates them with dg_host_alloc) ----
    u_host = pkg.gpu.pinned_empty((4, E * np_))
    u_host[:] = 0.0
    u_out = pkg.gpu.pinned_empty((4, E * np_))
    barrier(world)
    t0 = time.perf_counter()
    S.set_state(u_host)
    res, tr = S.run(args.steps, dt)
    S.get_state(out=u_out)
    e2e_s = time.perf_counter() - t0
    e2e_s = allmax(e2e_s, world)
    state_bytes = 4 * E * np_ * 8
    h2d = state_bytes / args.steps + 8 * 1
    d2h = state_bytes / args.steps + 5 * 8 + len(obs) * 4 * 8
    # roofline of the stage kernel: algorithmic bytes of one RK4 step's four
    # launches (18 state words per DOF incl. the residual snapshot read, plus
    # the per-element geometry records read once per stage) / their time
    w = 4 if args.precision == "fp32" else 8
    recf = geometry_record_words(3, w)
    geo_bytes = 4 * E * (recf * w + 8 * 4)
    alg_bytes = 18 * dofs * w + geo_bytes
    peak, peak_kind = measured_peak_gbs()
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    traffic = ncu_traffic()
    value = world * dofs * args.steps / (total_ms * 1e-3)
    e2e_value = world * dofs * args.steps / e2e_s
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "f64", "data": "synthetic (seeded jittered mesh, monopole)",
        "config": {"workload": WORKLOAD["name"], "elements": int(E), "order": 3, "n_var": nv, "dofs": int(dofs),
                   "dt": dt, "precision": args.precision, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between timed steps (256 MiB write)",
                   "step": "source inject + 4 fused RK4 stages + residual + 8 observers (one CUDA graph)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "note": "dg_set_state + dg_run(K steps, host residual/observer arrays) + dg_get_state, state in pinned host memory"},
        # per step: source injection (when the source covers nodes), four
        # stage kernels, residual/observer finalize, step counter
        "gpu_launches": int(args.steps * (6 + (1 if len(sdofs[0]) > 0 else 0))),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind, "kernel": "stage_kernel (4 launches per step)",
                     "kernel_ms_per_step": kern_ms, "algorithmic_bytes_per_step": int(alg_bytes)},
        "clocks": clk.summary(),
        "setup_ms": info["setup_ms"],
        "kernel_variant": info["kernel_variant"], "kernel_grid": info["kernel_grid"],
        "kernel_variants": {str(v): S.kernel_info(v) for v in [-1] + list(range(8)) + [16, 17, 18] + list(range(32, 40)) if S.kernel_info(v)[0] > 0},
    }
    S.close()
    return line


SCALE = dict(name="3D LEE at scale: box [0,4]x[0,2]x[0,2], 1,996,500 tets, p=4", counts=(110, 55, 55),
             lo=(0.0, 0.0, 0.0), hi=(4.0, 2.0, 2.0), order=4, jitter=0.2, seed=3, v0=(34.0, 0.0, 0.0), rho0=1.225,
             c0=340.0, cfl=0.5, freq=200.0, amp=0.1, size=0.1, centre=(2.0, 1.0, 1.0), n_obs=4)


def scale_sources():
    """Superposed dipole and quadrupole at the centre, expanded into monopoles
    as the reference's configuration parser does (src/configParser.cpp:87-115):
    [x, y, z, size, amp, freq, phase, duration] each."""
    W = SCALE
    x, y, z = W["centre"]
    s, a, f = W["size"], W["amp"], W["freq"]
    mono = lambda px, py, ph: [px, py, z, s / 2.0, a, f, ph, 1e9]
    dipole = [mono(x - s, y, 0.0), mono(x + s, y, np.pi)]
    quad = [mono(x - s, y, 0.0), mono(x + s, y, 0.0), mono(x, y - s, np.pi), mono(x, y + s, np.pi)]
    return dipole + quad


def run_scale(args):
    """Config 3: one 280 M-DOF instance (FP32), the bandwidth roofline study.
    Reports the autotuned stage kernel's rate, its HBM fraction, the
    per-variant stage-kernel times on this mesh, and for the tensor-core
    kernel its MMA rate (3 TF32 products per operand pair)."""
    pkg = _pkg()
    W = SCALE
    t0 = time.perf_counter()
    m = pkg.meshgen.box(counts=W["counts"], lo=W["lo"], hi=W["hi"], order=W["order"], jitter=W["jitter"],
                        seed=W["seed"])
    bcs = {k: "Absorbing" for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")}
    mesh = dict(dim=3, order=W["order"], xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=pkg.meshgen.solver_groups(m, bcs))
    del m
    gen_s = time.perf_counter() - t0
    hmin = pkg.meshgen.min_altitude(mesh)
    dt = W["cfl"] * hmin / ((W["c0"] + np.linalg.norm(W["v0"])) * (2 * W["order"] + 1))
    srcs = scale_sources()
    rng = np.random.default_rng(W["seed"])
    obs = [(rng.uniform(0.4, 3.6), rng.uniform(0.2, 1.8), rng.uniform(0.2, 1.8), 0.05) for _ in range(W["n_obs"])]
    E, np_ = mesh["elem_nodes"].shape
    nv = 4
    dofs = E * np_ * nv
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    sdofs = [np.nonzero((x[:, 0] - c[0]) ** 2 + (x[:, 1] - c[1]) ** 2 + (x[:, 2] - c[2]) ** 2 < c[3] ** 2)[0]
             for c in srcs]
    odofs, ows = [], []
    for o in obs:
        d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2 + (x[:, 2] - o[2]) ** 2)
        idx = np.nonzero(d < o[3])[0]
        odofs.append(idx)
        ows.append(1.0 / (d[idx] ** 2 + 1e-12))
    del x
    S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], precision=pkg.gpu.DG_FP32)
    info = S.info()
    if args.variant != -2:
        S.tune(args.variant)
        info = S.info()
    S.set_sources(sdofs)
    n_total = args.warmup + 3 * args.steps + 64
    times = np.arange(n_total) * dt
    vals = np.stack([c[4] * np.sin(2 * np.pi * c[5] * times + c[6]) for c in srcs], axis=1)
    S.set_source_values(vals)
    S.set_observers(odofs, ows)
    S.snapshot()
    S.run(args.warmup, dt)
    with ClockSampler(0) as clk:
        step_ms, kern_ms = S.bench_steps(args.steps, dt, flush_bytes=L2_FLUSH_BYTES, kernel_time=True)
    chosen = info["kernel_variant"]
    # every offered stage-kernel variant on this mesh (stage kernels only, a few steps each)
    per_variant = {}
    for v in [-1] + list(range(8)) + [16, 17, 18] + list(range(32, 40)):
        if v >= 0 and S.kernel_info(v)[0] == 0:
            continue
        S.tune(v)
        S.run(2, dt)
        _, km = S.bench_steps(4, dt, flush_bytes=L2_FLUSH_BYTES, kernel_time=True)
        per_variant[str(v)] = round(km, 4)
    S.tune(chosen)
    recf = geometry_record_words(3, 4)
    alg_bytes = 18 * dofs * 4 + 4 * E * (recf * 4 + 8 * 4)
    peak, peak_kind = measured_peak_gbs()
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": dofs * args.steps / (step_ms * args.steps * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
        "dtype": "f32", "data": "synthetic (seeded jittered box mesh, dipole + quadrupole)",
        "config": {"workload": W["name"], "elements": int(E), "order": W["order"], "n_var": nv, "dofs": int(dofs),
                   "dt": dt, "mesh_generation_s": round(gen_s, 1), "setup_ms": info["setup_ms"],
                   "sources": "dipole + quadrupole at (2,1,1), 200 Hz (6 monopoles)", "observers": len(obs)},
        "kernel_variant": chosen,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "kernel_ms_per_step": kern_ms, "algorithmic_bytes_per_step": int(alg_bytes)},
        "stage_kernel_ms_per_step": per_variant,
        "clocks": clk.summary(),
    }
    if any(v in per_variant for v in ("16", "17", "18")):
        # MMA work of the tensor-core kernel per step: per tile of 32 elements
        # three kind::tf32 MMAs of M = 128, N = Np rounded to 16, K = the
        # padded volume and face columns
        NP, NK = 35, 4 * 15
        NN = (NP + 15) // 16 * 16
        NPP = (NP + 3) // 4 * 4
        KT = (3 * NPP + (NK + 3) // 4 * 4 + 7) // 8 * 8
        flops_step = 4 * (E // 32) * 3 * 2 * 128 * NN * KT
        tc = {}
        for v in ("16", "17", "18"):
            if v in per_variant:
                tc[v] = {"tflops": flops_step / (per_variant[v] * 1e-3) / 1e12, "mma_flops_per_step": flops_step}
        line["tensor_core"] = tc
    S.close()
    return line


ENSEMBLE_NAME = "batched ensemble: 256 2-D LEE instances, 1k-50k tris, p in {2,3,4}"


def run_ensemble(args):
    """Aggregate DOF-updates/s of the batched path over the ensemble, the
    plain single-instance path on a sample of the same instances, and the
    per-instance FP32 error against the FP64 batch."""
    pkg = _pkg()
    ens = pkg.ensemble
    t0 = time.perf_counter()
    insts = ens.draw_instances(256, seed=4)
    gen_s = time.perf_counter() - t0

    def make(prec, subset):
        return ens.make_batch(subset, prec, args.warmup + args.steps + 2)

    dofs = sum(i["mesh"]["elem_nodes"].size * 3 for i in insts)
    B = make(pkg.gpu.DG_FP32, insts)
    fused = B.fused
    B.run(args.warmup)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = B.bench(args.steps)
    batched = dofs / (ms * 1e-3)
    # the other way of running the same batch, for comparison
    alt = None
    try:
        B.set_fused(not fused)
        B.run(args.warmup)
        ms_alt = B.bench(args.steps)
        alt = {"mode": "one stage kernel per element order (parallel graph branches)" if fused else
               "one persistent launch per RK stage for all orders (work queue)", "ms_per_step": ms_alt,
               "dof_updates_per_s": dofs / (ms_alt * 1e-3)}
    except pkg.gpu.SolverError:
        pass
    B.close()
    peak, peak_kind = measured_peak_gbs()
    rec_bytes = geometry_record_words(2, 4) * 4 + 8 * 4

    def alg_bytes(subset):
        # 18 state words per DOF and 4 geometry records per element per step
        d = sum(i["mesh"]["elem_nodes"].size * 3 for i in subset)
        e = sum(i["mesh"]["elem_nodes"].shape[0] for i in subset)
        return d, 18 * d * 4 + 4 * e * rec_bytes

    # the same instances, one batch per element order, timed alone
    per_order = {}
    for p in (2, 3, 4):
        sub = [i for i in insts if i["p"] == p]
        Bp = make(pkg.gpu.DG_FP32, sub)
        Bp.run(args.warmup)
        msp = Bp.bench(args.steps)
        Bp.close()
        d, bts = alg_bytes(sub)
        per_order[str(p)] = {"instances": len(sub), "dofs": d, "ms_per_step": msp, "dof_updates_per_s": d / (msp * 1e-3),
                             "hbm_frac": bts / (msp * 1e-3) / 1e9 / peak}
    _, all_bytes = alg_bytes(insts)
    # plain path: every 32nd instance on its own, same steps
    sample = insts[::32]
    tot_dof, tot_ms = 0, 0.0
    for i in sample:
        S = pkg.gpu.Solver(i["mesh"], v0=i["v0"], rho0=ens.RHO0, c0=ens.C0, precision=pkg.gpu.DG_FP32)
        sd, od, ow = node_sets(i["mesh"], i["src"], i["obs"])
        S.set_sources(sd)
        t = np.arange(args.warmup + 3 * args.steps + 8) * i["dt"]
        S.set_source_values((i["src"][4] * np.sin(2 * np.pi * i["src"][5] * t))[:, None])
        S.set_observers(od, ow)
        S.snapshot()
        S.run(args.warmup, i["dt"])
        sm, _ = S.bench_steps(args.steps, i["dt"], flush_bytes=0, kernel_time=False)
        tot_dof += i["mesh"]["elem_nodes"].size * 3
        tot_ms += sm
        S.close()
    plain = tot_dof / (tot_ms * 1e-3)
    # accuracy: FP32 vs FP64 batch on every 8th instance
    sub = insts[::8]
    nerr = min(args.steps, 100)
    res = []
    for prec in (pkg.gpu.DG_FP64, pkg.gpu.DG_FP32):
        B = make(prec, sub)
        for k, i in enumerate(sub):
            x = i["mesh"]["xyz"][i["mesh"]["elem_nodes"].reshape(-1)]
            u = np.zeros((4, x.shape[0]))
            u[0] = np.exp(-((x[:, 0] - i["src"][0]) ** 2 + (x[:, 1] - i["src"][1]) ** 2) / 0.5)
            B.set_state(k, u)
        B.run(nerr)
        res.append([B.get_state(k) for k in range(len(sub))])
        B.close()
    errs = [float(np.linalg.norm(a[:3] - b[:3]) / np.linalg.norm(b[:3])) for a, b in zip(res[1], res[0])]
    return {"metric": "RK4 DOF-updates/s (batched ensemble)", "value": batched, "unit": UNIT,
            "ms_per_step": ms, "steps": args.steps, "warmup": args.warmup, "dtype": "f32",
            "config": {"workload": ENSEMBLE_NAME, "instances": len(insts), "dofs": int(dofs),
                       "elements": int(sum(i["mesh"]["elem_nodes"].shape[0] for i in insts)),
                       "orders": {str(p): sum(1 for i in insts if i["p"] == p) for p in (2, 3, 4)},
                       "generation_s": gen_s},
            "plain_single_instance": {"value": plain, "unit": UNIT, "sample": "%d instances run one by one"
                                      % len(sample)},
            "batched_over_plain": batched / plain,
            "launch": "one persistent launch per RK stage for all orders (work queue)" if fused else
                      "one stage kernel per element order (parallel graph branches)",
            "other_launch_mode": alt,
            "roofline": {"bound": "hbm", "achieved": all_bytes / (ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": all_bytes / (ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_step": int(all_bytes), "time": "whole step (graph)"},
            "per_order": per_order,
            "fp32_vs_fp64_rel_l2_max": max(errs), "error_steps": nerr, "error_instances": len(sub),
            "clocks": clk.summary()}


SURROGATE_PATH = os.path.join(ROOT, "dgfem-acoustic_gb300", "data", "surrogate.npz")


def run_surrogate(args, n_dg=256, bound_db=1.0):
    """The learned spectral surrogate against DG: query throughput of the
    surrogate (all its networks, host arrays in and out) on the 2,000 held-out
    parameter draws, the batched DG path's query throughput on the first
    n_dg of them (same mesh and step count the targets came from), and the
    surrogate's spectral error against those DG answers."""
    pkg = _pkg()
    S = pkg.surrogate
    if not os.path.exists(SURROGATE_PATH):
        return {"metric": "surrogate spectral queries/s", "unavailable": "no trained surrogate at %s" % SURROGATE_PATH}
    sur = S.Surrogate.load(SURROGATE_PATH)
    P = S.draw_params(2000, 6)
    Y, dg_s = S.dg_spectra(P[:n_dg], steps=sur.steps, grid=sur.grid)
    for _ in range(args.warmup):
        sur.predict(P)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sur.predict(P)
    q_s = len(P) * args.steps / (time.perf_counter() - t0)
    mean, est = sur.predict(P[:n_dg])
    err = S.rms_db(mean, Y)
    acc = est <= sur.threshold(bound_db)
    spec, from_dg, _ = sur.query(P[:n_dg], bound_db=bound_db)
    delivered = S.rms_db(spec, Y)
    return {"metric": "surrogate spectral queries/s", "value": q_s, "unit": "queries/s", "steps": args.steps,
            "warmup": args.warmup, "dtype": "bf16 weights, f32 accumulate",
            "config": {"workload": "learned surrogate: 6 -> 4x256 GELU -> 4x128 log-PSD, %d networks" % len(sur.nets),
                       "queries": len(P), "dg_grid": sur.grid, "dg_steps": sur.steps},
            "dg": {"value": n_dg / dg_s, "unit": "queries/s", "sample": "%d held-out draws, batched FP32 DG" % n_dg},
            "speedup_over_dg": q_s / (n_dg / dg_s),
            "heldout": {"queries": n_dg, "bound_db": bound_db, "rms_db_median": float(np.median(err)),
                        "rms_db_p95": float(np.quantile(err, 0.95)),
                        "within_bound_fraction": float(np.mean(err <= bound_db)), "accepted_fraction": float(acc.mean()),
                        "accepted_rms_db_max": float(err[acc].max()) if acc.any() else None,
                        "accepted_above_bound_fraction": float(np.mean(err[acc] > bound_db)) if acc.any() else None,
                        "delivered_rms_db_max": float(delivered.max()),
                        "rerun_through_dg": int(from_dg.sum())}}


def run_ensemble_profile(args):
    """Warm-up plus a few steps of the 256-instance ensemble (FP32 batch),
    nothing else (the command line of the ensemble ncu summaries)."""
    pkg = _pkg()
    keep = {int(o) for o in args.orders.split(",")}
    insts = [i for i in pkg.ensemble.draw_instances(256, seed=4) if i["p"] in keep]
    B = pkg.ensemble.make_batch(insts, pkg.gpu.DG_FP32, args.warmup + args.steps + 2)
    B.run(args.warmup)
    obs = B.run(args.steps)
    print(json.dumps({"profile": True, "workload": "ensemble", "steps": args.steps, "warmup": args.warmup,
                      "groups": B.info()["n_groups"], "p_obs0_last": float(obs[0][-1, 0, 0])}))
    B.close()


def run_profile(args):
    """Warm-up plus a few RK4 steps of the workload through the per-step graph,
    nothing else (the command line that the ncu summaries in profiles/ use)."""
    pkg = _pkg()
    mesh, dt, src, obs = build_problem()
    W = WORKLOAD
    prec = pkg.gpu.DG_FP32 if args.precision == "fp32" else pkg.gpu.DG_FP64
    S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], precision=prec, device=0)
    if args.variant != -2:
        S.tune(args.variant)
    sdofs, odofs, ows = node_sets(mesh, src, obs)
    S.set_sources(sdofs)
    n = args.warmup + args.steps
    times = np.arange(n) * dt
    S.set_source_values((src[4] * np.sin(2 * np.pi * src[5] * times + src[6]))[:, None])
    S.set_observers(odofs, ows)
    S.snapshot()
    S.run(args.warmup, dt)
    res, _ = S.run(args.steps, dt)
    print(json.dumps({"profile": True, "steps": args.steps, "warmup": args.warmup, "res_p_last": float(res[-1, 0])}))
    S.close()


def run_cpu_baseline(args, sample_counts=(12, 12, 12), steps=4):
    """The oracle in the reference's loop structure and pragmas, all host
    threads, on a bounded sample of the workload (same order and physics,
    a 12^3 x 6 = 10,368-tet box)."""
    oracle = _oracle()
    W = WORKLOAD
    mesh, dt, src, obs = build_problem(sample_counts)
    cores = os.cpu_count() or 1
    P = oracle.Problem(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], t_start=0.0, t_end=1.0, dt=dt, t_rate=1.0,
                       num_threads=cores, sources=[dict(kind=oracle.SRC_SINE, params=src)], observers=obs,
                       max_steps=steps)
    r = P.run()
    E, np_ = mesh["elem_nodes"].shape
    rate = E * np_ * 4 * r["steps"] / r["loop_seconds"]
    return {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d steps on a %dx%dx%d x 6 = %d-tet box of the same workload (p=3, same physics), "
                      "reference loop structure and OpenMP pragmas, setup %.1f s excluded"
                      % (r["steps"], *sample_counts, E, r["setup_seconds"])}


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(v, world):
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--variant", type=int, default=-2,
                    help="stage kernel variant (-2: autotuned at setup, -1: baseline kernel, k: pipelined variant k)")
    ap.add_argument("--workload", default="cube", choices=["cube", "scale", "ensemble", "surrogate"])
    ap.add_argument("--orders", default="2,3,4",
                    help="ensemble workload: element orders of the instances to keep (profiling subsets)")
    ap.add_argument("--profile", action="store_true",
                    help="only build the workload and run warmup + steps time steps (for ncu captures)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    if args.profile:
        if args.workload == "ensemble":
            run_ensemble_profile(args)
        else:
            run_profile(args)
        return
    if args.workload == "ensemble" and args.impl != "reference":
        if rank == 0:
            print(json.dumps(run_ensemble(args)), flush=True)
        return
    if args.workload == "scale" and args.impl != "reference":
        if rank == 0:
            print(json.dumps(run_scale(args)), flush=True)
        return
    if args.workload == "surrogate" and args.impl != "reference":
        if rank == 0:
            print(json.dumps(run_surrogate(args)), flush=True)
        return
    if args.impl == "reference":
        if rank == 0:
            # each "step" of this arm is one reference time step on the bounded sample
            t0 = time.perf_counter()
            base = run_cpu_baseline(args, steps=max(1, min(args.steps, 6)))
            line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                    "dtype": "f64", "data": "synthetic (seeded jittered mesh, monopole)", "impl": "reference",
                    "config": {"workload": WORKLOAD["name"], "parallelism": "host threads (OpenMP)"},
                    "cpu_baseline": base,
                    "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    "wall_s": time.perf_counter() - t0}
            print(json.dumps(line), flush=True)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return
    # the oracle is timed before any CUDA call (its OpenMP team must not be
    # forked after the GPU is initialised)
    base = None
    if rank == 0 and not args.no_cpu_baseline:
        base = run_cpu_baseline(args)
    line = run_gpu(args, rank, world)
    if rank == 0:
        line["cpu_baseline"] = base
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
