"""Every source kind of the reference on the GPU, against the oracle.

One .conf case holds a monopole, a dipole, a quadrupole, a formula source, a
CSV table source and a WAV table source (src/configParser.cpp:72-168), with
keys source10 and source2 on overlapping discs, so that the lexicographic key
order of the reference's std::map (source10 before source2: the dipole's
values win where both write) decides the result. The product parses the
case (dipole/quadrupole expansion, formula evaluation, CSV/WAV tables and
their interpolation: include/configParser.h:38-58) and the GPU runs it in
FP64. The oracle (oracle/refcpu.cpp, the injection rule of
src/solver.cpp:455-483) gets the same sources built independently here: the
expansions written out, the formula as a Python function, the tables parsed
from the files with the reference's conventions (CSV fields through stof,
WAV samples / INT16_MAX with accumulated 1/rate times, src/utils.cpp:138-258).

* through the library (dg_set_sources / dg_set_source_values / dg_run):
  final state and observer traces within 1e-12 relative L2 of the oracle;
* through the dgalerkin driver on the same files: its observer files within
  their printed precision (6 significant digits) of the oracle.
"""
import math
import os
import subprocess
import wave

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "dgfem-acoustic_gb300", "_build", "dgalerkin")
DT, STEPS, T_RATE = 5e-5, 200, 2.5e-3
PHYS = dict(v0=(20.0, -15.0, 0.0), rho0=1.225, c0=340.0)
OBS = [(-2.2, -2.0, 0.0, 0.8), (1.0, 1.5, 0.0, 1.2)]
FORMULA = "0.1 * sin(2 * pi * 50 * t) + 0.05 * cos(2 * pi * 120 * t)"
WAV_RATE = 8000


def _formula(t):
    return 0.1 * math.sin(2 * math.pi * 50 * t) + 0.05 * math.cos(2 * math.pi * 120 * t)


def _write_inputs(pkg, d):
    m = pkg.meshgen.square(n=8, order=3, seed=5)
    pkg.host.write_mesh(str(d / "sq.msh"), 2, 3, m["xyz"], m["elem_nodes"],
                        [(g[0], g[1], g[3]) for g in m["groups"]])
    # CSV table: header line, a comment line, irregular times up to 6 ms
    rng = np.random.default_rng(9)
    tt = np.concatenate([[0.0], np.sort(rng.uniform(0.0, 6e-3, 40)), [6e-3]])
    vv = 0.2 * np.sin(2 * np.pi * 300 * tt) + rng.normal(0, 0.01, len(tt))
    with open(d / "table.csv", "w") as f:
        f.write("time;value\n# measured signal\n")
        for a, b in zip(tt, vv):
            f.write("%.9g;%.9g\n" % (a, b))
    # WAV: 16-bit mono at 8 kHz, 60 samples (7.4 ms)
    samples = np.round(20000 * np.sin(2 * np.pi * 400 * np.arange(60) / WAV_RATE)).astype(np.int16)
    with wave.open(str(d / "tone.wav"), "wb") as w:
        w.setnchannels(1)
        w.setsampwidth(2)
        w.setframerate(WAV_RATE)
        w.writeframes(samples.tobytes())
    conf = """meshFileName = sq.msh
timeStart = 0
timeEnd = {t_end!r}
timeStep = {dt!r}
timeRate = {rate!r}
elementType = Lagrange
timeIntMethod = Runge-Kutta
numThreads = 1
v0_x = {v0[0]!r}
v0_y = {v0[1]!r}
v0_z = 0
rho0 = {rho0!r}
c0 = {c0!r}
gpuPrecision = fp64
Absorbing = Absorbing
source10 = monopole, -2.5, -2.5, 0, 1.5, 1.0, 200, 0.3, 1.0
source2 = dipole, -2.0, -2.0, 0, 1.0, 0.5, 150, 0.1, 1.0
source3 = formula, "{formula}", 2.5, 2.5, 0, 1.0, 0.005
source4 = quadrupole, 2.5, -2.5, 0, 1.0, 0.3, 180, 0.0, 1.0
source5 = file, "table.csv", -2.5, 2.5, 0, 1.0
source6 = file, "tone.wav", 0, 0, 0, 1.0
observer1 = {o0[0]!r}, {o0[1]!r}, 0, {o0[3]!r}
observer2 = {o1[0]!r}, {o1[1]!r}, 0, {o1[3]!r}
""".format(t_end=(STEPS - 0.5) * DT, dt=DT, rate=T_RATE, v0=PHYS["v0"], rho0=PHYS["rho0"], c0=PHYS["c0"],
           formula=FORMULA, o0=OBS[0], o1=OBS[1])
    (d / "case.conf").write_text(conf)
    return m, samples


def _oracle_sources(oracle, d, samples):
    """The case's sources in the reference's order after expansion, built
    here from the configuration's numbers and files."""
    S, C, T = oracle.SRC_SINE, oracle.SRC_CALLBACK, oracle.SRC_TABLE
    mono = lambda x, y, size, amp, f, ph, dur: dict(kind=S, params=[x, y, 0.0, size, amp, f, ph, dur])
    out = [mono(-2.5, -2.5, 1.5, 1.0, 200.0, 0.3, 1.0)]                       # source10
    out += [mono(-3.0, -2.0, 0.5, 0.5, 150.0, 0.1, 1.0),                      # source2 (dipole)
            mono(-1.0, -2.0, 0.5, 0.5, 150.0, 0.1 + math.pi, 1.0)]
    out += [dict(kind=C, params=[2.5, 2.5, 0.0, 1.0, 0, 0, 0, 0.005])]        # source3 (formula)
    out += [mono(1.5, -2.5, 0.5, 0.3, 180.0, 0.0, 1.0), mono(3.5, -2.5, 0.5, 0.3, 180.0, 0.0, 1.0),
            mono(2.5, -3.5, 0.5, 0.3, 180.0, math.pi, 1.0), mono(2.5, -1.5, 0.5, 0.3, 180.0, math.pi, 1.0)]
    rows = [r for r in (d / "table.csv").read_text().splitlines()[1:] if not r.startswith("#")]
    tab = np.array([[float(np.float32(c)) for c in r.split(";")] for r in rows])
    out += [dict(kind=T, params=[-2.5, 2.5, 0.0, 1.0], table=tab)]            # source5 (CSV)
    t, wt = 0.0, []
    for s in samples:
        wt.append([t, float(np.float32(s) / np.float32(32767))])
        t += 1.0 / WAV_RATE
    out += [dict(kind=T, params=[0.0, 0.0, 0.0, 1.0], table=np.array(wt))]    # source6 (WAV)
    return out


def _node_sets(mesh, centres):
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    return [np.nonzero((x[:, 0] - c[0]) ** 2 + (x[:, 1] - c[1]) ** 2 + (x[:, 2] - c[2]) ** 2 < c[3] ** 2)[0]
            for c in centres]


@pytest.fixture(scope="module")
def case(pkg, oracle, tmp_path_factory):
    d = tmp_path_factory.mktemp("sources")
    m, samples = _write_inputs(pkg, d)
    mesh = dict(dim=2, order=3, xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=pkg.meshgen.solver_groups(m, {"Absorbing": "Absorbing"}))
    srcs = _oracle_sources(oracle, d, samples)
    P = oracle.Problem(mesh, t_start=0.0, t_end=(STEPS - 0.5) * DT, dt=DT, t_rate=T_RATE, sources=srcs, observers=OBS,
                       src_fn=lambda i, t, u: _formula(t), **PHYS)
    ref = P.run()
    assert ref["steps"] == STEPS
    return dict(dir=d, mesh=mesh, srcs=srcs, ref=ref)


def test_source_discs_overlap_where_the_key_order_decides(case):
    s = _node_sets(case["mesh"], [c["params"][:4] for c in case["srcs"]])
    assert len(set(s[0]) & set(s[1])) > 0  # source10 and the dipole's first monopole share nodes
    assert all(len(k) > 0 for k in s)        # every source writes some nodes


def test_every_source_kind_through_the_library_matches_oracle(pkg, case, monkeypatch):
    d, mesh, ref = case["dir"], case["mesh"], case["ref"]
    monkeypatch.chdir(d)  # the configuration names its files relative to the working directory
    times, snap = pkg.host.schedule(0.0, (STEPS - 0.5) * DT, DT, T_RATE)
    cfg = pkg.host.load_config(str(d / "case.conf"), times=times)
    assert [s["kind"] for s in cfg["sources"]] == [0, 0, 0, 1, 0, 0, 0, 0, 2, 2]
    # the product's values against the independent restatement at every step
    vals = cfg["source_values"]
    exp = np.full_like(vals, np.nan)
    for k, c in enumerate(case["srcs"]):
        for i, t in enumerate(times):
            if c["kind"] == 0:
                if t < c["params"][7]:
                    exp[i, k] = c["params"][4] * math.sin(2 * math.pi * c["params"][5] * t + c["params"][6])
            elif c["kind"] == 1:
                if t < c["params"][7]:
                    exp[i, k] = _formula(t)
    tab_cols = [k for k, c in enumerate(case["srcs"]) if c["kind"] == 2]
    np.testing.assert_allclose(vals[:, :tab_cols[0]], exp[:, :tab_cols[0]], rtol=1e-13, atol=1e-15)
    S = pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64, **PHYS)
    S.set_sources(_node_sets(mesh, [s["params"][:4] for s in cfg["sources"]]))
    S.set_source_values(vals)
    od = _node_sets(mesh, OBS)
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    ow = [1.0 / ((x[i, 0] - o[0]) ** 2 + (x[i, 1] - o[1]) ** 2 + 1e-12) for i, o in zip(od, OBS)]
    S.set_observers(od, ow)
    S.set_state(np.zeros((4, mesh["elem_nodes"].size)))
    tr, i = [], 0
    while i < STEPS:
        j = i + 1
        while j < STEPS and not snap[j]:
            j += 1
        if snap[i]:
            S.snapshot()
        _, o = S.run(j - i, DT)
        tr.append(o)
        i = j
    tr = np.concatenate(tr)
    u = S.get_state()
    S.close()
    assert rel_l2(u[:3], ref["state"][:3]) <= 1e-12
    ob_ref = ref["obs"][:, :, [1, 2, 3]]
    assert rel_l2(tr[:, :, :3], ob_ref) <= 1e-12


def test_every_source_kind_through_dgalerkin_matches_oracle(case):
    d, ref = case["dir"], case["ref"]
    r = subprocess.run([EXE, "case.conf"], cwd=str(d), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout
    for k in range(2):
        obs = np.genfromtxt(d / "results" / ("observers%d.txt" % (k + 1)), delimiter=";", skip_header=1)
        assert obs.shape == (STEPS, 6)
        # columns: time; density; pressure; vx; vy; vz, printed with 6 digits
        np.testing.assert_allclose(obs[:, 2:5], ref["obs"][:, k, 1:4], rtol=2e-5,
                                   atol=2e-5 * np.abs(ref["obs"][:, k, 1:4]).max())
