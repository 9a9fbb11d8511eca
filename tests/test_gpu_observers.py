"""Observers with many node slots: the finalize kernel sums an observer whose
radius holds more than one block's share of slots over several blocks and
combines their partial sums in block order. Observer traces of such runs
(thousands of slots per observer, mixed with small observers and one that
holds no node) against the CPU oracle, FP64 and FP32, and identical traces
from two runs (the combine does not depend on the blocks' timing)."""
import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_parity import _phys, _sources_observers

pytestmark = pytest.mark.gpu


def _big_mesh(pkg):
    mg = pkg.meshgen
    m = mg.square(n=24, order=3, seed=7, half_width=1.0, side_names=["xmin", "xmax", "ymin", "ymax"])
    groups = mg.solver_groups(m, {"xmin": "Absorbing", "xmax": "Absorbing", "ymin": "Reflecting", "ymax": "Absorbing"})
    return dict(dim=2, order=3, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=groups)


def _run(pkg, oracle, prec, nsteps=12):
    mesh = _big_mesh(pkg)
    ph = _phys(2)
    dt = 1e-5  # CFL about 0.4: smallest altitude 0.027 m, p = 3, c0 + |v0| = 142 m/s
    src = [0.1, -0.2, 0.0, 0.3, 1.0, 60.0, 0.3, 1.0]
    # radius 0.9: thousands of slots; 0.15: tens; far outside: none (NaN)
    obs = [(0.0, 0.0, 0.0, 0.9), (0.4, 0.3, 0.0, 0.15), (-0.3, 0.2, 0.0, 0.7), (9.0, 9.0, 0.0, 0.1)]
    ics = [(0.2, 0.1, 0.0, 0.3, 1.0)]
    P = oracle.Problem(mesh, t_start=0.0, t_end=(nsteps - 0.5) * dt, dt=dt, t_rate=100 * dt,
                       sources=[dict(kind=oracle.SRC_SINE, params=src)], observers=obs, ics=ics, **ph)
    ref = P.run()
    S = pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **ph)
    S.set_state(P.initial_state())
    sdofs, odofs, ows = _sources_observers(mesh, [src], obs)
    assert max(len(o) for o in odofs) > 4096 and len(odofs[3]) == 0
    S.set_sources(sdofs)
    times, _ = pkg.host.schedule(0.0, (nsteps - 0.5) * dt, dt, 100 * dt)
    S.set_source_values(np.where(times < src[7], src[4] * np.sin(2 * np.pi * src[5] * times + src[6]), np.nan)[:, None])
    S.set_observers(odofs, ows)
    S.snapshot()
    _, tr = S.run(nsteps, dt)
    S.close()
    return tr, ref["obs"][:, :, [1, 2, 3, 4]]


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_large_observers_match_oracle(pkg, oracle, prec, tol):
    tr, ref = _run(pkg, oracle, prec)
    assert tr.shape == ref.shape
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(tr), ok)
    assert not ok[:, 3].any() and ok[:, :3].all()
    for o in range(3):
        assert rel_l2(tr[:, o][ok[:, o]], ref[:, o][ok[:, o]]) <= tol, o


def test_large_observers_are_deterministic(pkg, oracle):
    a, _ = _run(pkg, oracle, "fp32")
    b, _ = _run(pkg, oracle, "fp32")
    np.testing.assert_array_equal(np.nan_to_num(a, nan=-1.0), np.nan_to_num(b, nan=-1.0))
