"""The 2-D LEE workload at its full size and length on the GPU against the
oracle's FP64 answer (tests/golden/config1_fp64.npz, made by
tests/golden/make_config1.py, which also stores the mesh it ran on):

square [-5,5]^2 with 4050 jittered triangles (seed 1), p = 3, all sides
Absorbing, v0 = (-30, 30, 0), rho0 = 1.225, c0 = 100, Gaussian initial
pressure at the origin (size 1, amplitude 1; src/dgalerkin.cpp:51-70), RK4
with dt = 1e-5 for 5000 steps (src/solver.cpp:413-574), snapshots every
1e-3, observers at (+-2.1, 0, 0) with radius 0.1.

* FP64, every stage-kernel variant offered for the mesh: final pressure and
  velocity, and both observers' pressure and velocity traces, within 1e-12
  relative L2 of the oracle; residual trace within 1e-10.
* FP32 (FP32 accumulation), the autotuned kernel and every FP32 variant:
  the same quantities within 1e-5 relative L2 of the FP64 oracle.
"""
import os

import numpy as np
import pytest

from conftest import ROOT, rel_l2

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "config1_fp64.npz")


def _golden_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_config1", os.path.join(ROOT, "tests", "golden",
                                                                               "make_config1.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def config1(pkg):
    g = np.load(GOLDEN)
    M = _golden_module()
    mesh = M.mesh_from_golden(g)  # the mesh the oracle ran on
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    od, ow = [], []
    for o in M.OBS:
        d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2 + (x[:, 2] - o[2]) ** 2)
        idx = np.nonzero(d < o[3])[0]
        od.append(idx)
        ow.append(1.0 / (d[idx] ** 2 + 1e-12))
    return dict(g=g, M=M, mesh=mesh, od=od, ow=ow)


def _run(pkg, c, precision, variant):
    M = c["M"]
    S = pkg.gpu.Solver(c["mesh"], precision=precision, **M.PHYS)
    if variant is not None:
        if S.kernel_info(variant)[0] == 0 and variant != -1:
            S.close()
            return None
        S.tune(variant)
    v = S.info()["kernel_variant"]
    # the Gaussian IC of the reference (exp(-r^2/size) on the pressure)
    x = c["mesh"]["xyz"][c["mesh"]["elem_nodes"].reshape(-1)]
    u0 = np.zeros((4, x.shape[0]))
    ic = M.IC
    u0[0] = ic[4] * np.exp(-((x[:, 0] - ic[0]) ** 2 + (x[:, 1] - ic[1]) ** 2 + (x[:, 2] - ic[2]) ** 2) / ic[3])
    S.set_state(u0)
    S.set_observers(c["od"], c["ow"])
    times, snap = pkg.host.schedule(0.0, M.T_END, M.DT, M.T_RATE)
    assert len(times) == M.STEPS
    res, tr = [], []
    i = 0
    while i < M.STEPS:
        j = i + 1
        while j < M.STEPS and not snap[j]:
            j += 1
        if snap[i]:
            S.snapshot()
        r, o = S.run(j - i, M.DT)
        res.append(r), tr.append(o)
        i = j
    u = S.get_state()
    S.close()
    return dict(u=u, res=np.concatenate(res), obs=np.concatenate(tr), variant=v)


def _errors(out, g):
    return dict(p=rel_l2(out["u"][0], g["state"][0]), velocity=rel_l2(out["u"][1:3], g["state"][1:3]),
                obs_p=rel_l2(out["obs"][:, :, 0], g["obs"][:, :, 1]),
                obs_velocity=rel_l2(out["obs"][:, :, 1:3], g["obs"][:, :, 2:4]),
                residuals=rel_l2(out["res"][:, :4], g["residuals"]))


def test_golden_is_the_reference_schedule(pkg, config1):
    g, M = config1["g"], config1["M"]
    times, snap = pkg.host.schedule(0.0, M.T_END, M.DT, M.T_RATE)
    assert g["times"].shape == (5000,) and np.array_equal(g["times"], times)
    assert np.array_equal(g["snapshots"], np.nonzero(snap)[0])
    assert tuple(g["penalty_hist"])[0] == 0  # no anti-dissipative interior face
    assert np.all(np.isfinite(g["obs"])) and np.abs(g["state"][0]).max() > 1e-3


@pytest.mark.parametrize("variant", [None, -1, 0, 1, 2, 3])
def test_config1_fp64_full_run_matches_oracle(pkg, config1, variant):
    out = _run(pkg, config1, pkg.gpu.DG_FP64, variant)
    if out is None:
        pytest.skip("variant %s does not exist for 2-D p=3 FP64" % variant)
    e = _errors(out, config1["g"])
    for k in ("p", "velocity", "obs_p", "obs_velocity"):
        assert e[k] <= 1e-12, (out["variant"], e)
    assert e["residuals"] <= 1e-10, (out["variant"], e)


@pytest.mark.parametrize("variant", [None, 0, 1, 2, 32, 33, 34, 16, 19])
def test_config1_fp32_full_run_within_1e5_of_fp64_oracle(pkg, config1, variant):
    out = _run(pkg, config1, pkg.gpu.DG_FP32, variant)
    if out is None:
        pytest.skip("variant %s does not exist for 2-D p=3 FP32" % variant)
    e = _errors(out, config1["g"])
    for k in ("p", "velocity", "obs_p", "obs_velocity"):
        assert e[k] <= 1e-5, (out["variant"], e)
