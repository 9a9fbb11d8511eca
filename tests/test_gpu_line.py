"""1-D line meshes on the GPU against the CPU oracle: single right-hand
sides for orders 1..4 (jittered elements, some with their end points in
reverse order, a mean flow, a reflecting and an absorbing end), full RK4 runs
with a source and observers, and the dgalerkin driver on the reference's own
1-D example mesh (tests/golden/line_1d.msh)."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2, smooth_state
from test_gpu_tensor_core import _obs_err, _run

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
EXE = os.path.join(ROOT, "dgfem-acoustic_gb300", "_build", "dgalerkin")
PHYS1 = dict(v0=(25.0, 0.0, 0.0), rho0=1.2, c0=340.0)
# runs: the helper's time step 2e-4 s is stable on these meshes (h >= 0.3 m,
# p <= 3) for c0 + |v0| = 60 m/s
PHYS_RUN = dict(v0=(10.0, 0.0, 0.0), rho0=1.2, c0=50.0)


def _line_mesh(pkg, p, n=24, flip_nodes=True, reverse_half=True):
    """Jittered line mesh. flip_nodes: every third element lists its end
    points right to left (interior nodes reversed with them: a negative
    dx/du). reverse_half: the second half of the elements is numbered right to
    left, so that the lower-numbered neighbour of a face lies to its right and
    the reference's penalty sign (the orientation seen from that neighbour) is
    s_f = -1 there: an anti-dissipative face flux, which the reference
    applies as well; such a mesh is used for single right-hand sides only,
    its runs grow without bound."""
    mg = pkg.meshgen
    m = mg.line(n=n, order=p, jitter=0.25, seed=p)
    en = m["elem_nodes"].copy()
    if flip_nodes:
        for e in range(0, n, 3):
            en[e, 0], en[e, 1] = en[e, 1], en[e, 0]
            if p > 1:
                en[e, 2:] = en[e, 2:][::-1]
    if reverse_half:
        en = np.concatenate([en[:n // 2], en[n // 2:][::-1]])
    groups = mg.solver_groups(m, {"left": "Reflecting", "right": "Absorbing"})
    return dict(dim=1, order=p, xyz=m["xyz"], elem_nodes=en, groups=groups)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_line_rhs_matches_oracle(pkg, oracle, p, prec):
    mesh = _line_mesh(pkg, p)
    u = smooth_state(mesh, seed=40 + p)
    dt = 1e-4
    ref = oracle.Problem(mesh, dt=dt, **PHYS1).stage(u)
    S = pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **PHYS1)
    tol = 5e-11 if prec == "fp64" else 5e-4
    variants = [v for v in [-1, 0, 1, 16, 17, 18, 19, 20, 32] if v < 0 or S.kernel_info(v)[0] > 0]
    assert variants == [-1, 0]
    for v in variants:
        S.tune(v)
        k = S.rhs(u, dt)
        assert rel_l2(k[:2], ref[:2]) <= tol, (p, prec, v, rel_l2(k[:2], ref[:2]))
        assert np.all(k[2:] == 0.0)
    # penalty signs as the oracle's: s_f = -1 on the faces of the right-to-left numbered half
    pen = oracle.Problem(mesh, dt=dt, **PHYS1).faces()["penalty"]
    assert (pen < 0).any() and (pen > 0).any()
    assert np.array_equal(S.face_info()["penalty"], pen)
    S.close()


@pytest.mark.parametrize("p", [1, 3])
@pytest.mark.parametrize("prec,variant", [("fp64", -1), ("fp64", 0), ("fp32", 0)])
def test_line_run_matches_oracle(pkg, oracle, p, prec, variant):
    mesh = _line_mesh(pkg, p, reverse_half=False)
    # the helper's source and observers sit in the plane; the line is y = z = 0
    u, res, tr, ref = _run(pkg, oracle, mesh, PHYS_RUN, prec, variant, 40)
    assert np.abs(ref["state"][0]).max() < 10.0  # bounded: source and initial amplitudes are 1
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert rel_l2(u[:2], ref["state"][:2]) <= tol
    assert np.all(u[2:] == 0.0)
    if prec == "fp64":
        assert rel_l2(res[:, :3], ref["residuals"][:, :3]) <= 1e-9


def test_dgalerkin_on_reference_line_mesh(tmp_path, pkg, oracle):
    shutil.copy(os.path.join(GOLDEN, "line_1d.msh"), tmp_path / "line.msh")
    cfg = {
        "mesh": {"File": "line.msh", "BC": {"number": 1, "boundary1": {"name": "ends", "type": "Absorbing"}}},
        "solver": {"time": {"start": 0.0, "end": 0.01, "step": 1e-4, "rate": 0.005}, "elementType": "Lagrange",
                   "timeIntMethod": "Runge-Kutta", "numThreads": 4},
        "initialization": {"meanFlow": {"vx": 10.0, "vy": 0.0, "vz": 0.0, "rho": 1.225, "c": 340.0}, "number": 1,
                           "initialCondition1": {"type": "gaussian", "x": 0.0, "y": 0.0, "z": 0.0, "size": 0.5,
                                                 "amplitude": 1.0}},
        "observers": {"number": 1, "observer1": {"x": 1.0, "y": 0.0, "z": 0.0, "size": 0.15}},
        "sources": {"number": 0},
    }
    (tmp_path / "case.json").write_text(json.dumps(cfg))
    r = subprocess.run([EXE, "case.json"], cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    mine = np.genfromtxt(tmp_path / "residuals.csv", delimiter=";", skip_header=1)
    m = pkg.host.load_mesh(str(tmp_path / "line.msh"))
    mesh = dict(dim=1, order=1, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=[(0, m["groups"][0][2])])
    P = oracle.Problem(mesh, v0=(10.0, 0, 0), rho0=1.225, c0=340.0, t_end=0.01, dt=1e-4, t_rate=0.005,
                       observers=[(1.0, 0.0, 0.0, 0.15)], ics=[(0.0, 0.0, 0.0, 0.5, 1.0)])
    ref = P.run()
    assert ref["steps"] == mine.shape[0]
    np.testing.assert_allclose(mine[:, 1:4], ref["residuals"][:, :3], rtol=1e-5)
    obs = np.genfromtxt(tmp_path / "results" / "observers1.txt", delimiter=";", skip_header=1)
    np.testing.assert_allclose(obs[:, 2], ref["obs"][:, 0, 1], rtol=1e-5, atol=1e-12)
    assert (tmp_path / "results" / "result0.vtu").exists()
