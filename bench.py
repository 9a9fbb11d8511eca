"""Benchmark: RK4 DOF-updates/s of the GB300 DG solver.

Default workload (the largest single-GPU configuration of the metric, the
bandwidth roofline study): 3-D LEE at scale, box [0,4]x[0,2]x[0,2] split into
110 x 55 x 55 cubes x 6 jittered tetrahedra (1,996,500 tets, seed 3),
Lagrange order p = 4 (35 nodes per element, 4 variables: 279.5 M DOF),
uniform mean flow (34, 0, 0), rho0 = 1.225, c0 = 340, a dipole and a
quadrupole at (2, 1, 1) (200 Hz, amplitude 0.1, size 0.1; six monopoles
after the reference's expansion), all faces Absorbing, dt from CFL 0.5,
4 observers; FP32.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp32|fp64]
  python bench.py --impl reference ...   (the reference's CPU path, restated)
  python bench.py --workload cube|ensemble|surrogate|precision ...

One step = one full RK4 time step of the reference's loop (source injection,
four RHS stages, the combine, the residual diagnostic and the observer
samples) over the whole mesh. Prints one JSON line (rank 0). At N = 1 the
line also carries the batched ensemble (256 uneven 2-D instances, one
persistent launch per RK stage) against the plain single-instance path on
the same instances, with the per-instance FP32-vs-FP64 error.

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

METRIC = "RK4 DOF-updates/s"
UNIT = "DOF-updates/s"
L2_FLUSH_BYTES = 256 << 20
ABSORBING = {k: "Absorbing" for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")}

# Config 3: the 280 M-DOF box (default). The CPU sample is a sub-box with the
# same element size, order and physics.
SCALE = dict(key="scale", name="3D LEE at scale: box [0,4]x[0,2]x[0,2], 1,996,500 tets, p=4", counts=(110, 55, 55),
             lo=(0.0, 0.0, 0.0), hi=(4.0, 2.0, 2.0), order=4, jitter=0.2, seed=3, v0=(34.0, 0.0, 0.0), rho0=1.225,
             c0=340.0, cfl=0.5, freq=200.0, amp=0.1, size=0.1, centre=(2.0, 1.0, 1.0), n_obs=4, obs_radius=0.05,
             bcs=ABSORBING, poles="dipole+quadrupole",
             sample=dict(counts=(16, 8, 8), lo=(0.0, 0.0, 0.0), hi=(16 * 4.0 / 110, 8 * 2.0 / 55, 8 * 2.0 / 55),
                         centre=(8 * 4.0 / 110, 4 * 2.0 / 55, 4 * 2.0 / 55)))
# Config 2: the 16 M-DOF cube.
CUBE = dict(key="cube", name="3D LEE cube, 196,608 tets, p=3", counts=(32, 32, 32), lo=(-1.0, -1.0, -1.0),
            hi=(1.0, 1.0, 1.0), order=3, jitter=0.2, seed=2, v0=(0.0, 0.0, 0.0), rho0=1.225, c0=340.0, cfl=0.5,
            freq=50.0, amp=0.1, size=0.1, centre=(0.0, 0.0, 0.0), n_obs=8, obs_radius=0.1,
            bcs={"xmin": "Reflecting", "xmax": "Reflecting", "ymin": "Absorbing", "ymax": "Absorbing",
                 "zmin": "Absorbing", "zmax": "Absorbing"}, poles="monopole",
            sample=None)
WORKLOADS = {"scale": SCALE, "cube": CUBE}


def _pkg():
    import importlib
    return importlib.import_module("dgfem-acoustic_gb300")


def _oracle():
    import importlib.util
    spec = importlib.util.spec_from_file_location("refcpu", os.path.join(ROOT, "oracle", "refcpu.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def pole_sources(W, centre=None):
    """The workload's sources as monopoles [x, y, z, size, amp, freq, phase,
    duration], dipoles and quadrupoles expanded as the reference's
    configuration parser does (src/configParser.cpp:87-115)."""
    x, y, z = centre or W["centre"]
    s, a, f = W["size"], W["amp"], W["freq"]
    if W["poles"] == "monopole":
        return [[x, y, z, s, a, f, 0.0, 1e9]]
    mono = lambda px, py, ph: [px, py, z, s / 2.0, a, f, ph, 1e9]
    dipole = [mono(x - s, y, 0.0), mono(x + s, y, np.pi)]
    quad = [mono(x - s, y, 0.0), mono(x + s, y, 0.0), mono(x, y - s, np.pi), mono(x, y + s, np.pi)]
    return dipole + quad


def build_problem(W, sample=False):
    """Mesh, dt, sources and observers of a workload (or of its CPU sample:
    a sub-box with the same element size, order and physics)."""
    pkg = _pkg()
    counts, lo, hi, centre = W["counts"], W["lo"], W["hi"], W["centre"]
    if sample and W["sample"]:
        S = W["sample"]
        counts, lo, hi, centre = S["counts"], S["lo"], S["hi"], S["centre"]
    elif sample:
        counts = (12, 12, 12)  # the cube's sample: the same cube at 12^3 x 6 tets
    m = pkg.meshgen.box(counts=counts, lo=lo, hi=hi, order=W["order"], jitter=W["jitter"], seed=W["seed"])
    mesh = dict(dim=3, order=W["order"], xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=pkg.meshgen.solver_groups(m, W["bcs"]))
    del m
    # dt = CFL * h_min / ((c0 + |v0|) (2p + 1)), h_min = smallest element altitude
    hmin = pkg.meshgen.min_altitude(mesh)
    dt = W["cfl"] * hmin / ((W["c0"] + np.linalg.norm(W["v0"])) * (2 * W["order"] + 1))
    rng = np.random.default_rng(W["seed"])
    lo_, hi_ = np.asarray(lo), np.asarray(hi)
    span = hi_ - lo_
    obs = [tuple(lo_ + span * (0.1 + 0.8 * rng.uniform(0, 1, 3))) + (W["obs_radius"],) for _ in range(W["n_obs"])]
    return mesh, dt, pole_sources(W, centre), obs


def node_sets(mesh, srcs, obs):
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    sdofs = [np.nonzero((x[:, 0] - c[0]) ** 2 + (x[:, 1] - c[1]) ** 2 + (x[:, 2] - c[2]) ** 2 < c[3] ** 2)[0]
             for c in srcs]
    odofs, ows = [], []
    for o in obs:
        d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2 + (x[:, 2] - o[2]) ** 2)
        idx = np.nonzero(d < o[3])[0]
        odofs.append(idx)
        ows.append(1.0 / (d[idx] ** 2 + 1e-12))
    return sdofs, odofs, ows


def source_values(srcs, n, dt):
    times = np.arange(n) * dt
    return np.stack([c[4] * np.sin(2 * np.pi * c[5] * times + c[6]) for c in srcs], axis=1)


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi (every 50 ms)
    while running; the window is opened before the timed region starts and
    closed after the last GPU measurement of the line."""

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
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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

    def summary(self, window):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0, "window": window}
        ok = [r for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        sm = [float(r[1]) for r in ok]
        mx = [float(r[2]) for r in ok if r[2].replace(".", "").isdigit()]
        pw = [float(r[3]) for r in ok if r[3].replace(".", "").isdigit()]
        # under load: samples drawing more than a third of the window's peak power
        load = [s for s, p in zip(sm, pw) if pw and p > max(pw) / 3] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in ok for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(load)) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(ok), "samples_under_load": len(load),
                "power_w_max": max(pw) if pw else None, "window": window}


def geometry_record_words(dim, w):
    """Words of one element's geometry record as the stage kernel reads it:
    metric (dim*dim), per face normal (dim) and scale, the element's mean flow
    (dim) and time-step scale, padded to 16 bytes."""
    raw = dim * dim + (dim + 1) * (dim + 1) + dim + 1
    vec = 16 // w
    return (raw + vec - 1) // vec * vec


def algorithmic_bytes_per_step(E, dofs, dim, w):
    """Algorithmic HBM bytes of one RK4 step's four stage launches: 18 state
    words per DOF (stage 1: u in, accumulator and next input out; stages
    2-3: input, u, accumulator in, accumulator and next input out; stage 4:
    input, u, accumulator and residual snapshot in, u out) plus the element's
    geometry record and integer face record read once per stage."""
    recf = geometry_record_words(dim, w)
    reci = ((2 * (dim + 1)) + 3) // 4 * 4
    return 18 * dofs * w + 4 * E * (recf * w + reci * 4)


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def recorded(name):
    """A measurement record committed under profiles/ (ncu DRAM traffic of
    the stage kernel, the FP32-vs-FP64 runs of the configurations)."""
    try:
        return json.load(open(os.path.join(ROOT, "profiles", name)))
    except Exception:
        return None


def tc_mma_flops_per_step(E, dim, order):
    """MMA work of the tensor-core stage kernel per RK4 step: per tile of 32
    elements three kind::tf32 products of the split operands (M = 128, N = Np
    rounded to 16, K = the padded volume and face columns) in each of the
    four stages."""
    from math import comb
    NP = comb(order + dim, dim)
    NK = (dim + 1) * comb(order + dim - 1, dim - 1)
    NN = (NP + 15) // 16 * 16
    NPP = (NP + 3) // 4 * 4
    KT = (dim * NPP + (NK + 3) // 4 * 4 + 7) // 8 * 8
    return 4 * ((E + 31) // 32) * 3 * 2 * 128 * NN * KT


def run_plain(args, W, rank, world):
    """One workload through the plain single-instance path: device-timed RK4
    steps (per-step graph, CUDA events on the solver's stream), the stage
    kernels' own time for the roofline, and the end-to-end rate through the
    C ABI with host buffers."""
    pkg = _pkg()
    device = int(os.environ.get("LOCAL_RANK", "0"))
    t0 = time.perf_counter()
    mesh, dt, srcs, obs = build_problem(W)
    gen_s = time.perf_counter() - t0
    prec = pkg.gpu.DG_FP32 if args.precision == "fp32" else pkg.gpu.DG_FP64
    S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], precision=prec, device=device)
    if args.variant != -2:
        S.tune(args.variant)
    info = S.info()
    E, np_ = mesh["elem_nodes"].shape
    nv = 4
    dofs = E * np_ * nv
    sdofs, odofs, ows = node_sets(mesh, srcs, obs)
    del mesh
    S.set_sources(sdofs)
    S.set_source_values(source_values(srcs, args.warmup + 3 * args.steps + 8, dt))
    S.set_observers(odofs, ows)
    # the host state of the end-to-end leg, page-locked (dg_host_alloc) as a
    # user of the library allocates it; one array serves as input and output
    u_host = pkg.gpu.pinned_empty((4, E * np_))
    u_host[:] = 0.0
    S.set_state(u_host)
    S.snapshot()
    S.run(args.warmup, dt)  # warm-up (also captures the per-step graph)
    state_large = 5 * dofs * (4 if args.precision == "fp32" else 8) > (129 << 20) * 4
    flush = 0 if state_large else L2_FLUSH_BYTES
    barrier(world)
    with ClockSampler(device) as clk:
        # ---- timed device region: K per-step graph launches bracketed by
        # CUDA events on the solver's stream; then a second pass of K steps
        # with events around each stage launch (the stage kernels' own time) ----
        step_ms, kern_ms = S.bench_steps(args.steps, dt, flush_bytes=flush, kernel_time=True)
        total_ms = allmax(step_ms * args.steps, world)
        # ---- end to end through the C ABI with host buffers ----
        barrier(world)
        t1 = time.perf_counter()
        S.set_state(u_host)
        S.run(args.steps, dt)
        S.get_state(out=u_host)
        e2e_s = allmax(time.perf_counter() - t1, world)
    state_bytes = 4 * E * np_ * 8
    h2d = state_bytes / args.steps
    d2h = state_bytes / args.steps + 5 * 8 + len(obs) * 4 * 8
    w = 4 if args.precision == "fp32" else 8
    alg_bytes = algorithmic_bytes_per_step(E, dofs, 3, w)
    bytes_16w = E * (16 * nv * np_ * w + 4 * (9 + 4 * 6) * w)  # 16 state words per DOF + geometry
    peak, peak_kind = measured_peak_gbs()
    achieved = alg_bytes / (kern_ms * 1e-3) / 1e9
    variant = info["kernel_variant"]
    traffic, traffic_src = None, None
    rec = recorded("stage_kernel_traffic.json")
    if rec and rec.get(W["key"], {}).get("variant") == variant:
        traffic = rec[W["key"]]["bytes_per_launch"]
        traffic_src = rec[W["key"]]["source"]
    value = world * dofs * args.steps / (total_ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "f64",
        "data": "synthetic (seeded jittered box mesh, %s)" % W["poles"],
        "config": workload_config(W, E, np_, dt, world),
        "e2e": {"value": world * dofs * args.steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h),
                "note": "dg_set_state + dg_run(K steps, host residual/observer arrays) + dg_get_state, "
                        "state in pinned host memory"},
        # per step: source injection, four stage kernels, residual/observer
        # finalize, step counter
        "gpu_launches": int(args.steps * (6 + (1 if sum(len(s) for s in sdofs) > 0 else 0))),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "traffic_source": traffic_src or "not captured for this kernel variant",
                     "peak_kind": peak_kind, "kernel": "stage kernel variant %d (4 launches per step)" % variant,
                     "kernel_ms_per_step": kern_ms, "algorithmic_bytes_per_step": int(alg_bytes),
                     "bytes_per_dof_update": alg_bytes / dofs,
                     "frac_16_word_count": bytes_16w / (kern_ms * 1e-3) / 1e9 / peak},
        "setup_ms": info["setup_ms"], "mesh_generation_s": round(gen_s, 1),
        "kernel_variant": variant, "kernel_grid": info["kernel_grid"],
    }
    if 16 <= variant < 32:  # tensor-core kernels
        f = tc_mma_flops_per_step(E, 3, W["order"])
        line["tensor_core"] = {"mma_tflops": f / (kern_ms * 1e-3) / 1e12, "mma_flops_per_step": f,
                               "note": "3 kind::tf32 products per operand pair (head x head and the two head x tail corrections)"}
    if args.variants:
        per_variant = {}
        for v in [-1] + list(range(8)) + [16, 17, 18, 19, 20, 21, 22] + list(range(32, 40)) + list(range(48, 64)):
            if v >= 0 and S.kernel_info(v)[0] == 0:
                continue
            S.tune(v)
            S.run(2, dt)
            _, km = S.bench_steps(4, dt, flush_bytes=flush, kernel_time=True)
            per_variant[str(v)] = round(km, 4)
        S.tune(variant)
        line["stage_kernel_ms_per_step"] = per_variant
    line["clocks"] = clk.summary("device-timed steps, stage-kernel-timed steps and the end-to-end run")
    S.close()
    return line


def workload_config(W, E, np_, dt, world):
    return {"workload": W["name"], "elements": int(E), "order": W["order"], "n_var": 4, "dofs": int(E * np_ * 4),
            "dt": dt, "sources": W["poles"], "observers": W["n_obs"],
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2 (state arrays 1.1 GB each)" if W["key"] == "scale" else
                  "flushed between timed steps (256 MiB write)",
            "step": "source inject + 4 fused RK4 stages + residual + observers (one CUDA graph)"}


ENSEMBLE_NAME = "batched ensemble: 256 2-D LEE instances, 1k-50k tris, p in {2,3,4}"


def ensemble_summary(args, full=False):
    """Aggregate DOF-updates/s of the batched path over the 256-instance
    ensemble (config 4: one persistent launch per RK stage for all orders,
    the batch default, and the per-order graph for comparison), the plain
    single-instance path on every 32nd instance run one by one, their ratio,
    and the largest per-instance FP32-vs-FP64 relative L2 on every 8th
    instance. With full, also one batch per element order."""
    pkg = _pkg()
    ens = pkg.ensemble
    t0 = time.perf_counter()
    insts = ens.draw_instances(256, seed=4)
    gen_s = time.perf_counter() - t0
    steps = args.ens_steps or args.steps

    def make(prec, subset):
        return ens.make_batch(subset, prec, args.warmup + 3 * steps + 2)

    dofs = sum(i["mesh"]["elem_nodes"].size * 3 for i in insts)
    elems = sum(i["mesh"]["elem_nodes"].shape[0] for i in insts)
    B = make(pkg.gpu.DG_FP32, insts)
    fused = B.fused
    B.run(args.warmup)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = B.bench(steps)
        alt = None
        try:
            B.set_fused(not fused)
            B.run(args.warmup)
            ms_alt = B.bench(steps)
            alt = {"mode": "one stage kernel per element order (parallel graph branches)" if fused else
                   "one persistent launch per RK stage for all orders (work queue)", "ms_per_step": ms_alt,
                   "dof_updates_per_s": dofs / (ms_alt * 1e-3)}
        except pkg.gpu.SolverError:
            pass
    B.close()
    batched = dofs / (ms * 1e-3)
    peak, _ = measured_peak_gbs()
    rec_bytes = geometry_record_words(2, 4) * 4 + 8 * 4

    def alg_bytes(subset):
        d = sum(i["mesh"]["elem_nodes"].size * 3 for i in subset)
        e = sum(i["mesh"]["elem_nodes"].shape[0] for i in subset)
        return d, 18 * d * 4 + 4 * e * rec_bytes

    _, all_bytes = alg_bytes(insts)
    # plain path: every 32nd instance on its own, same steps
    sample = insts[::32]
    tot_dof, tot_ms = 0, 0.0
    for i in sample:
        S = pkg.gpu.Solver(i["mesh"], v0=i["v0"], rho0=ens.RHO0, c0=ens.C0, precision=pkg.gpu.DG_FP32)
        sd, od, ow = node_sets(i["mesh"], [i["src"]], i["obs"])
        S.set_sources(sd)
        t = np.arange(args.warmup + 3 * steps + 8) * i["dt"]
        S.set_source_values((i["src"][4] * np.sin(2 * np.pi * i["src"][5] * t))[:, None])
        S.set_observers(od, ow)
        S.snapshot()
        S.run(args.warmup, i["dt"])
        sm, _ = S.bench_steps(steps, i["dt"], flush_bytes=0, kernel_time=False)
        tot_dof += i["mesh"]["elem_nodes"].size * 3
        tot_ms += sm
        S.close()
    plain = tot_dof / (tot_ms * 1e-3)
    # accuracy: FP32 vs FP64 batch on every 8th instance
    sub = insts[::8]
    nerr = max(steps, 100)
    res = []
    for prec in (pkg.gpu.DG_FP64, pkg.gpu.DG_FP32):
        Bp = ens.make_batch(sub, prec, nerr + 2)
        for k, i in enumerate(sub):
            x = i["mesh"]["xyz"][i["mesh"]["elem_nodes"].reshape(-1)]
            u = np.zeros((4, x.shape[0]))
            u[0] = np.exp(-((x[:, 0] - i["src"][0]) ** 2 + (x[:, 1] - i["src"][1]) ** 2) / 0.5)
            Bp.set_state(k, u)
        Bp.run(nerr)
        res.append([Bp.get_state(k) for k in range(len(sub))])
        Bp.close()
    errs = [float(np.linalg.norm(a[:3] - b[:3]) / np.linalg.norm(b[:3])) for a, b in zip(res[1], res[0])]
    out = {"workload": ENSEMBLE_NAME, "instances": len(insts), "dofs": int(dofs), "elements": int(elems),
           "orders": {str(p): sum(1 for i in insts if i["p"] == p) for p in (2, 3, 4)}, "generation_s": gen_s,
           "steps": steps, "value": batched, "unit": UNIT, "ms_per_step": ms,
           "launch": "one persistent launch per RK stage for all orders (work queue)" if fused else
                     "one stage kernel per element order (parallel graph branches)",
           "other_launch_mode": alt,
           "plain_single_instance": {"value": plain, "unit": UNIT,
                                     "sample": "%d instances (every 32nd) run one by one" % len(sample)},
           "batched_over_plain": batched / plain,
           "hbm_frac": all_bytes / (ms * 1e-3) / 1e9 / peak,
           "fp32_vs_fp64_rel_l2_max": max(errs), "error_steps": nerr, "error_instances": len(sub),
           "clocks": clk.summary("batched steps in both launch modes")}
    if full:
        per_order = {}
        for p in (2, 3, 4):
            subp = [i for i in insts if i["p"] == p]
            Bp = make(pkg.gpu.DG_FP32, subp)
            Bp.run(args.warmup)
            msp = Bp.bench(steps)
            Bp.close()
            d, bts = alg_bytes(subp)
            per_order[str(p)] = {"instances": len(subp), "dofs": d, "ms_per_step": msp,
                                 "dof_updates_per_s": d / (msp * 1e-3), "hbm_frac": bts / (msp * 1e-3) / 1e9 / peak}
        out["per_order"] = per_order
    return out


def oracle_bytes_full(W, E):
    """Host memory the reference's data layout needs for the whole workload
    (the oracle keeps it): per-element gradient tables E*Ng*Np*3 doubles
    (Ng = 125 points of the degree-8 rule at p = 4, 24 at p = 3), mass
    matrices E*Np^2 doubles, the nodal flux as heap 3-vectors (~64 B per node
    and variable) and five state copies."""
    from math import comb
    np_ = comb(W["order"] + 3, 3)
    ng = {1: 4, 2: 11, 3: 24, 4: 125}[W["order"]]
    grad = E * ng * np_ * 3 * 8
    mass = E * np_ * np_ * 8
    flux = 4 * E * np_ * 64
    state = 5 * 4 * E * np_ * 8
    return grad + mass + flux + state, grad, mass, flux


def run_cpu_baseline(W, steps):
    """The oracle in the reference's loop structure and OpenMP pragmas, all
    host threads, on a bounded sample of the workload (a sub-box with the
    same element size, order and physics)."""
    oracle = _oracle()
    mesh, dt, srcs, obs = build_problem(W, sample=True)
    cores = os.cpu_count() or 1
    P = oracle.Problem(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], t_start=0.0, t_end=1.0, dt=dt, t_rate=1.0,
                       num_threads=cores, sources=[dict(kind=oracle.SRC_SINE, params=s) for s in srcs],
                       observers=obs, max_steps=steps)
    r = P.run()
    E, np_ = mesh["elem_nodes"].shape
    rate = E * np_ * 4 * r["steps"] / r["loop_seconds"]
    counts = W["sample"]["counts"] if W["sample"] else (12, 12, 12)
    out = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": "%d time steps on a %dx%dx%d x 6 = %d-tet box of the same workload (same element size, "
                     "p=%d, mean flow, sources and boundary conditions), the reference's loop structure and OpenMP "
                     "pragmas, FP64, setup %.1f s excluded"
                     % (r["steps"], counts[0], counts[1], counts[2], E, W["order"], r["setup_seconds"])}
    Efull = 6 * W["counts"][0] * W["counts"][1] * W["counts"][2]
    if W["key"] == "scale":
        tot, grad, mass, flux = oracle_bytes_full(W, Efull)
        out["full_workload"] = ("infeasible: memory: the reference's layout needs about %.0f GB for the %d-tet mesh "
                                "(%.0f GB per-element gradient tables, %.0f GB mass matrices, %.0f GB nodal flux "
                                "3-vectors), and one step would take about %.0f s at the sampled rate"
                                % (tot / 1e9, Efull, grad / 1e9, mass / 1e9, flux / 1e9,
                                   Efull * np_ * 4 / rate))
    return out


def run_reference(args, W, world):
    """--impl reference: the reference's CPU path (restated: the reference
    itself cannot be built here) on the host cores, same metric and config
    as the GPU arm; each step is one reference time step on the bounded
    sample."""
    t0 = time.perf_counter()
    base = run_cpu_baseline(W, steps=max(1, min(args.steps, 5)))
    E = 6 * W["counts"][0] * W["counts"][1] * W["counts"][2]
    from math import comb
    np_ = comb(W["order"] + 3, 3)
    line = {"metric": METRIC, "value": base["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded jittered box mesh, %s)" % W["poles"], "impl": "reference",
            "config": workload_config(W, E, np_, reference_dt(W), world),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.perf_counter() - t0}
    return line


def reference_dt(W):
    """The workload's dt (CFL rule on the full mesh), as the GPU arm's config
    reports it; computed from the mesh without building the solver."""
    mesh, dt, _, _ = build_problem(W)
    return dt


PRECISION_RUNS = {"cube": 2000, "scale": 500}


def run_precision(args):
    """FP32 against FP64 on the GPU after the full run of each 3-D
    configuration (config 2: 2000 steps, config 3: 500 steps), from the same
    zero initial state driven by the workload's sources: relative L2 of the
    final pressure, the velocity and the whole state, and of the observer
    traces (pressure and velocity at every step). FP64 runs once with its
    autotuned kernel; FP32 runs with its autotuned kernel and with every
    stage-kernel variant listed in --fp32-variants."""
    pkg = _pkg()
    out = {}
    extra = [int(v) for v in args.fp32_variants.split(",") if v]
    for key in [k for k in args.configs.split(",") if k]:
        W = WORKLOADS[key]
        nsteps = args.steps if args.steps_override else PRECISION_RUNS[key]
        mesh, dt, srcs, obs = build_problem(W)
        E, np_ = mesh["elem_nodes"].shape
        sdofs, odofs, ows = node_sets(mesh, srcs, obs)

        def run(prec, variant):
            t0 = time.perf_counter()
            S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"],
                               precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32)
            if variant is not None:
                if variant >= 0 and S.kernel_info(variant)[0] == 0:
                    S.close()
                    return None
                S.tune(variant)
            S.set_sources(sdofs)
            S.set_source_values(source_values(srcs, nsteps + 2, dt))
            S.set_observers(odofs, ows)
            S.set_state(np.zeros((4, E * np_)))
            S.snapshot()
            tr, done = [], 0
            while done < nsteps:
                k = min(100, nsteps - done)
                _, o = S.run(k, dt)
                tr.append(o)
                done += k
            r = dict(state=S.get_state(), obs=np.concatenate(tr), s=time.perf_counter() - t0,
                     variant=S.info()["kernel_variant"])
            S.close()
            return r

        ref = run("fp64", None)
        rl = lambda x, y: float(np.linalg.norm(x - y) / np.linalg.norm(y))
        fp32 = {}
        for v in [None] + extra:
            a = run("fp32", v)
            if a is None:
                continue
            fp32[str(a["variant"]) if v is not None else "autotuned(%d)" % a["variant"]] = {
                "rel_l2_p": rl(a["state"][0], ref["state"][0]),
                "rel_l2_velocity": rl(a["state"][1:], ref["state"][1:]),
                "rel_l2_state": rl(a["state"], ref["state"]),
                "rel_l2_observer_p": rl(a["obs"][:, :, 0], ref["obs"][:, :, 0]),
                "rel_l2_observer_velocity": rl(a["obs"][:, :, 1:], ref["obs"][:, :, 1:]),
                "wall_s": round(a["s"], 1)}
        auto = [k for k in fp32 if k.startswith("autotuned")][0]
        out[key] = dict({"workload": W["name"], "steps": nsteps, "dt": dt, "variant_fp64": ref["variant"],
                         "wall_s_fp64": round(ref["s"], 1), "max_abs_p_fp64": float(np.abs(ref["state"][0]).max()),
                         "fp32_variant": int(auto.split("(")[1].rstrip(")")), "fp32_by_variant": fp32},
                        **fp32[auto])
        del ref, mesh
    return {"metric": "FP32 vs FP64 relative L2 after the full run", "runs": out}


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
    t1 = time.perf_counter()
    spec, from_dg, _ = sur.query(P[:n_dg], bound_db=bound_db)
    q_fb = n_dg / (time.perf_counter() - t1)
    delivered = S.rms_db(spec, Y)
    return {"metric": "surrogate spectral queries/s", "value": q_s, "unit": "queries/s", "steps": args.steps,
            "warmup": args.warmup, "dtype": "bf16 weights, f32 accumulate",
            "config": {"workload": "learned surrogate: 6 -> 4x256 GELU -> 4x128 log-PSD, %d networks" % len(sur.nets),
                       "queries": len(P), "dg_grid": sur.grid, "dg_steps": sur.steps},
            "dg": {"value": n_dg / dg_s, "unit": "queries/s", "sample": "%d held-out draws, batched FP32 DG" % n_dg},
            "speedup_over_dg": q_s / (n_dg / dg_s),
            "with_fallback": {"bound_db": bound_db, "queries_per_s": q_fb, "speedup_over_dg": q_fb / (n_dg / dg_s)},
            "heldout": {"queries": n_dg, "bound_db": bound_db, "rms_db_median": float(np.median(err)),
                        "rms_db_p95": float(np.quantile(err, 0.95)),
                        "within_bound_fraction": float(np.mean(err <= bound_db)), "accepted_fraction": float(acc.mean()),
                        "accepted_rms_db_max": float(err[acc].max()) if acc.any() else None,
                        "accepted_above_bound_fraction": float(np.mean(err[acc] > bound_db)) if acc.any() else None,
                        "delivered_rms_db_max": float(delivered.max()),
                        "rerun_through_dg": int(from_dg.sum())}}


def run_profile(args, W):
    """Warm-up plus a few RK4 steps of the workload through the per-step graph,
    nothing else (the command line of the ncu summaries in profiles/)."""
    pkg = _pkg()
    if args.workload == "ensemble":
        keep = {int(o) for o in args.orders.split(",")}
        insts = [i for i in pkg.ensemble.draw_instances(256, seed=4) if i["p"] in keep]
        B = pkg.ensemble.make_batch(insts, pkg.gpu.DG_FP32, args.warmup + args.steps + 2)
        B.run(args.warmup)
        obs = B.run(args.steps)
        print(json.dumps({"profile": True, "workload": "ensemble", "steps": args.steps, "warmup": args.warmup,
                          "groups": B.info()["n_groups"], "p_obs0_last": float(obs[0][-1, 0, 0])}))
        B.close()
        return
    if args.counts:
        W = dict(W, counts=tuple(int(c) for c in args.counts.split(",")))
        W["hi"] = tuple(W["lo"][k] + (W["hi"][k] - W["lo"][k]) * W["counts"][k] / WORKLOADS[W["key"]]["counts"][k]
                        for k in range(3))
    mesh, dt, srcs, obs = build_problem(W)
    prec = pkg.gpu.DG_FP32 if args.precision == "fp32" else pkg.gpu.DG_FP64
    S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], precision=prec, device=0)
    if args.variant != -2:
        S.tune(args.variant)
    sdofs, odofs, ows = node_sets(mesh, srcs, obs)
    S.set_sources(sdofs)
    S.set_source_values(source_values(srcs, args.warmup + args.steps + 2, dt))
    S.set_observers(odofs, ows)
    S.snapshot()
    S.run(args.warmup, dt)
    res, _ = S.run(args.steps, dt)
    print(json.dumps({"profile": True, "workload": W["key"], "elements": int(mesh["elem_nodes"].shape[0]),
                      "variant": S.info()["kernel_variant"], "steps": args.steps, "warmup": args.warmup,
                      "res_p_last": float(res[-1, 0])}))
    S.close()


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
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="leave the batched-ensemble keys out of the line")
    ap.add_argument("--ens-steps", type=int, default=0, help="steps of the ensemble keys (default: --steps)")
    ap.add_argument("--variants", action="store_true", help="also time every stage-kernel variant on the workload")
    ap.add_argument("--variant", type=int, default=-2,
                    help="stage kernel variant (-2: autotuned at setup, -1: baseline kernel, k: variant k)")
    ap.add_argument("--workload", default="scale", choices=["scale", "cube", "ensemble", "surrogate", "precision"])
    ap.add_argument("--configs", default="cube,scale", help="precision workload: the configurations to run")
    ap.add_argument("--steps-override", action="store_true", help="precision workload: run --steps steps")
    ap.add_argument("--fp32-variants", default="", help="precision workload: FP32 stage-kernel variants to run too")
    ap.add_argument("--orders", default="2,3,4",
                    help="ensemble workload: element orders of the instances to keep (profiling subsets)")
    ap.add_argument("--counts", default="", help="profile: cube counts of a smaller box of the same workload")
    ap.add_argument("--profile", action="store_true",
                    help="only build the workload and run warmup + steps time steps (for ncu captures)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    W = WORKLOADS.get(args.workload, SCALE)
    try:
        if args.profile:
            run_profile(args, W)
        elif args.impl == "reference":
            # rank 0 alone times the host path; the other ranks do no work
            if rank == 0:
                print(json.dumps(run_reference(args, W, world)), flush=True)
        elif args.workload == "ensemble":
            if rank == 0:
                line = ensemble_summary(args, full=True)
                line = dict({"metric": "RK4 DOF-updates/s (batched ensemble)", "dtype": "f32",
                             "warmup": args.warmup}, **line)
                print(json.dumps(line), flush=True)
        elif args.workload == "surrogate":
            if rank == 0:
                print(json.dumps(run_surrogate(args)), flush=True)
        elif args.workload == "precision":
            if rank == 0:
                print(json.dumps(run_precision(args)), flush=True)
        else:
            # the oracle is timed before any CUDA call (its OpenMP team must
            # not be forked after the GPU is initialised)
            base = None
            if rank == 0 and not args.no_cpu_baseline:
                base = run_cpu_baseline(W, steps=3)
            line = run_plain(args, W, rank, world)
            if rank == 0:
                line["cpu_baseline"] = base
                prec = recorded("fp32_vs_fp64.json")
                if prec and W["key"] in prec.get("runs", {}):
                    r = prec["runs"][W["key"]]
                    line["fp32_vs_fp64_rel_l2"] = {k: r[k] for k in ("rel_l2_p", "rel_l2_velocity", "rel_l2_state",
                                                                     "rel_l2_observer_p", "rel_l2_observer_velocity",
                                                                     "steps")}
                    line["fp32_vs_fp64_rel_l2"]["source"] = ("profiles/fp32_vs_fp64.json (python bench.py "
                                                             "--workload precision, the full run on a GB300)")
                if world == 1 and not args.no_ensemble:
                    line["batched"] = ensemble_summary(args)
                print(json.dumps(line), flush=True)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
