"""The tensor-core stage kernel (tcgen05, 3xTF32 split, FP32 state) and the
Euler1 integrator against the CPU oracle, through the C ABI.

The tensor-core kernel is kernel variant 16, 17 or 18 (256, 512 or 1024
threads per block: each tile row's columns split 2, 4 or 8 ways) of an FP32
context. Its products
keep about 21 mantissa bits (x = tf32 head + fp32 tail, the tail-tail product
dropped), so it is held to the same bounds as the CUDA-core FP32 kernels: a
single right-hand side within the FP32 single-RHS bound of the oracle and
within a few times the CUDA-core kernel's own error; a full run within 1e-5
relative L2 of the FP64 oracle on the state and the observer traces."""
import numpy as np
import pytest

from conftest import rel_l2, smooth_state
from test_gpu_parity import _mesh, _phys, _sources_observers

pytestmark = pytest.mark.gpu

TC = 16
TC4 = 17
TC8 = 18


def _obs_err(tr, ref_obs):
    """Relative L2 over the observer samples; an observer with no DG node in
    its radius reports NaN (the reference's rule) in both."""
    ok = np.isfinite(ref_obs)
    assert np.array_equal(np.isfinite(tr), ok)
    return rel_l2(tr[ok], ref_obs[ok])


def _solver(pkg, mesh, ph, prec="fp32"):
    return pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **ph)


@pytest.mark.parametrize("tc", [TC, TC4, TC8])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tc_rhs_matches_oracle(pkg, oracle, dim, p, tc):
    mesh = _mesh(pkg, dim, p)
    ph = _phys(dim)
    u = smooth_state(mesh, seed=dim * 10 + p)
    dt = 1e-4
    ref = oracle.Problem(mesh, dt=dt, **ph).stage(u)
    S = _solver(pkg, mesh, ph)
    nv = dim + 1
    assert S.tune(0) == 0
    err_cc = rel_l2(S.rhs(u, dt)[:nv], ref[:nv])
    assert S.tune(tc) == tc
    k = S.rhs(u, dt)
    err_tc = rel_l2(k[:nv], ref[:nv])
    assert err_tc <= 5e-4, (dim, p, err_tc)
    assert err_tc <= 4 * err_cc + 1e-6, (dim, p, err_tc, err_cc)
    if dim == 2:
        assert np.all(k[3] == 0.0)


def test_tc_not_offered_in_fp64(pkg):
    mesh = _mesh(pkg, 2, 2)
    S = _solver(pkg, mesh, _phys(2), "fp64")
    for tc in (TC, TC4, TC8):
        with pytest.raises(pkg.gpu.SolverError):
            S.tune(tc)


def _run(pkg, oracle, mesh, ph, prec, variant, nsteps, euler=False):
    dim = mesh["dim"]
    dt = 2e-4
    src = [0.1, -0.2, 0.1 if dim == 3 else 0.0, 0.45, 1.0, 50.0, 0.3, 1.0]
    obs = [(0.5, 0.3, 0.2 if dim == 3 else 0.0, 0.4), (-0.4, -0.5, 0.0, 0.5)]
    ics = [(0.2, 0.1, 0.0, 0.3, 1.0)]
    P = oracle.Problem(mesh, t_start=0.0, t_end=(nsteps - 0.5) * dt, dt=dt, t_rate=10 * dt, method=1 if euler else 0,
                       sources=[dict(kind=oracle.SRC_SINE, params=src)], observers=obs, ics=ics, **ph)
    ref = P.run()
    assert ref["steps"] == nsteps
    S = _solver(pkg, mesh, ph, prec)
    assert S.tune(variant) == variant
    S.set_state(P.initial_state())
    sdofs, odofs, ows = _sources_observers(mesh, [src], obs)
    S.set_sources(sdofs)
    times, snap = pkg.host.schedule(0.0, (nsteps - 0.5) * dt, dt, 10 * dt)
    vals = np.where(times < src[7], src[4] * np.sin(2 * np.pi * src[5] * times + src[6]), np.nan)[:, None]
    S.set_source_values(vals)
    S.set_observers(odofs, ows)
    res, tr = [], []
    i = 0
    while i < nsteps:
        j = i + 1
        while j < nsteps and not snap[j]:
            j += 1
        if snap[i]:
            S.snapshot()
        r, o = S.run(j - i, dt, euler=euler)
        res.append(r), tr.append(o)
        i = j
    return S.get_state(), np.concatenate(res), np.concatenate(tr), ref


@pytest.mark.parametrize("dim,p,tc", [(2, 2, TC), (2, 3, TC), (2, 4, TC), (3, 2, TC), (3, 3, TC), (3, 4, TC),
                                      (2, 3, TC4), (3, 3, TC4), (3, 4, TC8)])
def test_tc_run_matches_oracle(pkg, oracle, dim, p, tc):
    mesh = _mesh(pkg, dim, p)
    u, res, tr, ref = _run(pkg, oracle, mesh, _phys(dim), "fp32", tc, 40)
    nv = dim + 1
    assert rel_l2(u[:nv], ref["state"][:nv]) <= 1e-5
    assert rel_l2(res[:, :4], ref["residuals"][:, :4]) <= 1e-3
    assert _obs_err(tr, ref["obs"][:, :, [1, 2, 3, 4]]) <= 1e-4


@pytest.mark.parametrize("prec,variant", [("fp64", -1), ("fp64", 0), ("fp32", 1), ("fp32", TC)])
@pytest.mark.parametrize("dim,p", [(2, 3), (3, 3)])
def test_euler_run_matches_oracle(pkg, oracle, dim, p, prec, variant):
    mesh = _mesh(pkg, dim, p)
    # Euler1 is unstable for the RK4 time step over many steps; 12 steps stay bounded
    u, res, tr, ref = _run(pkg, oracle, mesh, _phys(dim), prec, variant, 12, euler=True)
    nv = dim + 1
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert rel_l2(u[:nv], ref["state"][:nv]) <= tol
    assert _obs_err(tr, ref["obs"][:, :, [1, 2, 3, 4]]) <= tol * 10


@pytest.mark.parametrize("tc", [TC, TC4, TC8])
def test_tc_many_tiles_per_block(pkg, oracle, tc):
    """A mesh with more tiles than resident blocks, so that every block walks
    several tiles through both halves of its double buffer: one RHS against
    the oracle and 20 RK4 steps against the CUDA-core FP32 kernel."""
    mg = pkg.meshgen
    m = mg.box(counts=(14, 14, 14), order=3, seed=21)
    bcs = {"xmin": "Reflecting", "xmax": "Reflecting", "ymin": "Absorbing", "ymax": "Absorbing",
           "zmin": "Absorbing", "zmax": "Absorbing"}
    mesh = dict(dim=3, order=3, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=mg.solver_groups(m, bcs))
    ph = _phys(3)
    u0 = smooth_state(mesh, seed=77)
    dt = 2e-5
    ref = oracle.Problem(mesh, dt=dt, **ph).stage(u0)
    S = _solver(pkg, mesh, ph)
    assert S.tune(tc) == tc
    assert rel_l2(S.rhs(u0, dt)[:4], ref[:4]) <= 5e-4
    out = []
    for v in (1, tc):
        S.tune(v)
        S.set_state(u0)
        S.snapshot()
        r, _ = S.run(20, dt)
        out.append((S.get_state(), r))
    assert rel_l2(out[1][0][:4], out[0][0][:4]) <= 1e-6
    np.testing.assert_allclose(out[1][1][:, :4], out[0][1][:, :4], rtol=1e-3, atol=0)
