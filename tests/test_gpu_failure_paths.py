"""Failure paths of the GPU solver, made without a GPU fault.

* Timeout: the bounded device waits of the stage kernels (mbarrier waits for
  their TMA copies and tensor-core work) are given a limit of 0 polling
  rounds through dg_set_wait_limit, so that every wait gives up. The kernel
  must then issue no further copy, drain the copies it already issued, set
  the context's error flag and return; dg_run reports DG_ERR_TIMEOUT, and the
  same context, with the limit restored, runs on correctly.
* Non-finite state: a NaN injected on the host through dg_set_state makes
  dg_run return DG_ERR_NONFINITE (the reference reports NaN observers,
  src/solver.cpp:566, and aborts on errors, include/err.h:5-9), and the
  context runs correctly from a finite state afterwards.
"""
import numpy as np
import pytest

from conftest import rel_l2, smooth_state

pytestmark = pytest.mark.gpu

PHYS = dict(v0=(20.0, -10.0, 5.0), rho0=1.225, c0=340.0)
DT = 2e-5


def _mesh(pkg, dim, p):
    mg = pkg.meshgen
    m = mg.square(n=6, order=p, seed=7) if dim == 2 else mg.box(counts=(3, 3, 3), order=p, seed=8)
    bcs = {"Absorbing": "Absorbing", "xmin": "Reflecting", "xmax": "Absorbing", "ymin": "Absorbing",
           "ymax": "Absorbing", "zmin": "Absorbing", "zmax": "Reflecting"}
    return dict(dim=dim, order=p, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=mg.solver_groups(m, bcs))


def _phys(dim):
    return dict(PHYS, v0=PHYS["v0"] if dim == 3 else (PHYS["v0"][0], PHYS["v0"][1], 0.0))


def _waiting_variants(S):
    """Stage-kernel variants that wait on mbarriers: pipelined (0..7),
    tensor-core (16-21), constant-operator (32..) and wide-chunk (48..)
    kernels."""
    return [v for v in list(range(8)) + [16, 17, 18, 19, 20, 21, 22] + list(range(32, 40)) + list(range(48, 64)) if S.kernel_info(v)[0] > 0]


@pytest.mark.parametrize("dim,p,prec", [(3, 3, "fp32"), (3, 4, "fp32"), (2, 3, "fp32"), (3, 2, "fp64"),
                                        (2, 4, "fp64")])
def test_timed_out_wait_reports_timeout_and_context_recovers(pkg, dim, p, prec):
    mesh = _mesh(pkg, dim, p)
    ph = _phys(dim)
    precision = pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32
    u0 = smooth_state(mesh, seed=3)
    nv = dim + 1
    ref = pkg.gpu.Solver(mesh, precision=precision, **ph)
    ref.tune(-1)  # the baseline kernel has no device waits
    ref.set_state(u0)
    ref.snapshot()
    ref.run(3, DT)
    u_ref = ref.get_state()
    ref.close()
    S = pkg.gpu.Solver(mesh, precision=precision, **ph)
    variants = _waiting_variants(S)
    assert variants
    for v in variants:
        S.tune(v)
        S.set_state(u0)
        S.snapshot()
        S.set_wait_limit(0)
        with pytest.raises(pkg.gpu.SolverError, match="DG_ERR_TIMEOUT"):
            S.run(1, DT)
        S.set_wait_limit(1 << 20)
        S.set_state(u0)
        S.snapshot()
        S.run(3, DT)  # no error left behind
        err = rel_l2(S.get_state()[:nv], u_ref[:nv])
        assert err <= (1e-12 if prec == "fp64" else 1e-5), (v, err)
    S.close()


@pytest.mark.parametrize("dim,prec", [(2, "fp64"), (3, "fp32")])
def test_nonfinite_state_reports_nonfinite_and_context_recovers(pkg, dim, prec):
    mesh = _mesh(pkg, dim, 3)
    ph = _phys(dim)
    precision = pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32
    S = pkg.gpu.Solver(mesh, precision=precision, **ph)
    u0 = smooth_state(mesh, seed=4)
    bad = u0.copy()
    bad[0, bad.shape[1] // 2] = np.nan
    S.set_state(bad)
    S.snapshot()
    with pytest.raises(pkg.gpu.SolverError, match="DG_ERR_NONFINITE"):
        S.run(2, DT)
    S.set_state(u0)
    S.snapshot()
    res, _ = S.run(2, DT)
    assert np.all(np.isfinite(res))
    assert np.all(np.isfinite(S.get_state()))
    S.close()
