"""The tensor-core stage kernels (tcgen05 TF32 MMAs of head/tail-split
operands, FP32 state) and the Euler1 integrator against the CPU oracle,
through the C ABI.

The tensor-core kernels are kernel variants 16, 17 or 18 (one-chunk kernel,
256, 512 or 1024 threads per block: each tile row's columns split 2, 4 or 8
ways), 19 or 20 (two-chunk kernel, two blocks per SM: K applied in at most
two chunks, 256 or 512 threads per block) and 21 or 22 (warp-specialised kernel,
tetrahedra of orders 3 and 4: builder, MMA and epilogue warps handing K
chunks and double-buffered accumulators to each other; 8 or 16 builder
warps) of an FP32 context. Each operand is
a TF32 head plus a TF32 tail (the operator rounded to 22 significand bits so
that the pair is exact; the data within 2^-22), four products summed in
FP32, so they are held to the same bounds as the CUDA-core FP32 kernels: a
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
TC2 = 19
TC2_4 = 20
TC3 = 21
TC3_4 = 22


def _obs_err(tr, ref_obs):
    """Relative L2 over the observer samples; an observer with no DG node in
    its radius reports NaN (the reference's rule) in both."""
    ok = np.isfinite(ref_obs)
    assert np.array_equal(np.isfinite(tr), ok)
    return rel_l2(tr[ok], ref_obs[ok])


def _solver(pkg, mesh, ph, prec="fp32"):
    return pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **ph)


@pytest.mark.parametrize("tc", [TC, TC4, TC8, TC2, TC2_4, TC3, TC3_4])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tc_rhs_matches_oracle(pkg, oracle, dim, p, tc):
    mesh = _mesh(pkg, dim, p)
    ph = _phys(dim)
    u = smooth_state(mesh, seed=dim * 10 + p)
    dt = 1e-4
    ref = oracle.Problem(mesh, dt=dt, **ph).stage(u)
    S = _solver(pkg, mesh, ph)
    if S.kernel_info(tc)[0] == 0:
        pytest.skip("variant %d is not built for dim %d, p %d" % (tc, dim, p))
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
    for tc in (TC, TC4, TC8, TC2, TC2_4):
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
                                      (2, 3, TC4), (3, 3, TC4), (3, 4, TC8), (2, 2, TC2), (2, 4, TC2),
                                      (3, 2, TC2), (3, 3, TC2), (3, 4, TC2), (3, 4, TC2_4), (2, 3, TC2_4),
                                      (3, 3, TC3), (3, 4, TC3), (3, 3, TC3_4), (3, 4, TC3_4)])
def test_tc_run_matches_oracle(pkg, oracle, dim, p, tc):
    mesh = _mesh(pkg, dim, p)
    u, res, tr, ref = _run(pkg, oracle, mesh, _phys(dim), "fp32", tc, 40)
    nv = dim + 1
    assert rel_l2(u[:nv], ref["state"][:nv]) <= 1e-5
    assert rel_l2(res[:, :4], ref["residuals"][:, :4]) <= 1e-3
    assert _obs_err(tr, ref["obs"][:, :, [1, 2, 3, 4]]) <= 1e-4


@pytest.mark.parametrize("prec,variant", [("fp64", -1), ("fp64", 0), ("fp32", 1), ("fp32", TC), ("fp32", TC2)])
@pytest.mark.parametrize("dim,p", [(2, 3), (3, 3)])
def test_euler_run_matches_oracle(pkg, oracle, dim, p, prec, variant):
    mesh = _mesh(pkg, dim, p)
    # Euler1 is unstable for the RK4 time step over many steps; 12 steps stay bounded
    u, res, tr, ref = _run(pkg, oracle, mesh, _phys(dim), prec, variant, 12, euler=True)
    nv = dim + 1
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert rel_l2(u[:nv], ref["state"][:nv]) <= tol
    assert _obs_err(tr, ref["obs"][:, :, [1, 2, 3, 4]]) <= tol * 10


@pytest.mark.parametrize("tc,p", [(TC, 3), (TC4, 3), (TC8, 3), (TC2, 3), (TC2_4, 3), (TC, 4), (TC2, 4), (TC2_4, 4),
                                  (TC3, 3), (TC3, 4), (TC3_4, 3), (TC3_4, 4)])
def test_tc_many_tiles_per_block(pkg, oracle, tc, p):
    """A mesh with more tiles than resident blocks, so that every block walks
    several tiles through its tile buffers (at p = 4 the two-chunk kernel
    applies K in two chunks): one RHS against the oracle, and 20 RK4 steps of
    the tensor-core and the CUDA-core FP32 kernels against an FP64 run of the
    same steps (the tensor-core run within the FP32 bound and within a few
    times the CUDA-core kernel's own error)."""
    mg = pkg.meshgen
    m = mg.box(counts=(14, 14, 14) if p == 3 else (12, 12, 12), order=p, seed=21)
    bcs = {"xmin": "Reflecting", "xmax": "Reflecting", "ymin": "Absorbing", "ymax": "Absorbing",
           "zmin": "Absorbing", "zmax": "Absorbing"}
    mesh = dict(dim=3, order=p, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=mg.solver_groups(m, bcs))
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
    S64 = _solver(pkg, mesh, ph, "fp64")
    S64.set_state(u0)
    S64.snapshot()
    r64, _ = S64.run(20, dt)
    u64 = S64.get_state()
    S64.close()
    err_cc, err_tc = rel_l2(out[0][0][:4], u64[:4]), rel_l2(out[1][0][:4], u64[:4])
    assert err_tc <= 1e-5 and err_tc <= 4 * err_cc + 1e-6, (err_tc, err_cc)
    np.testing.assert_allclose(out[1][1][:, :4], r64[:, :4], rtol=1e-3, atol=0)
