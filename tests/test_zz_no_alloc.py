"""The allocation-free residual diagnostic (dg_residuals_noalloc).

Callers that cannot allocate device memory where they need the diagnostic
(a host framework that owns every allocation, loops that must not enter the
allocator, callers that pass their own device buffers) use this entry point
with device arrays they already own. This file checks it through the C ABI
against the residuals that dg_run reports for the same states, on two calls
in a row (the second call reuses the library's fixed scratch array), and that
it rejects inputs larger than that scratch allows. It is collected last so
that a failure here cannot hide the results of the other GPU tests.
"""
import numpy as np
import pytest

from conftest import smooth_state

pytestmark = pytest.mark.gpu


def _mesh(pkg, dim):
    mg = pkg.meshgen
    m = mg.square(n=4, order=3, seed=11) if dim == 2 else mg.box(counts=(2, 2, 2), order=2, seed=12)
    bcs = {"Absorbing": "Absorbing", "xmin": "Reflecting", "xmax": "Absorbing", "ymin": "Absorbing",
           "ymax": "Reflecting", "zmin": "Absorbing", "zmax": "Absorbing"}
    return dict(dim=dim, order=m["order"], xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=mg.solver_groups(m, bcs))


@pytest.mark.parametrize("dim", [3, 2])
def test_noalloc_residuals_match_dg_run_on_two_calls(pkg, dim):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    mesh = _mesh(pkg, dim)
    c0 = 340.0
    S = pkg.gpu.Solver(mesh, v0=(10.0, -5.0, 0.0), rho0=1.225, c0=c0, precision=pkg.gpu.DG_FP64)
    u0 = smooth_state(mesh, seed=5)
    S.set_state(u0)
    S.snapshot()
    dt = 2e-5
    res1, _ = S.run(1, dt)
    u1 = S.get_state()
    res2, _ = S.run(1, dt)
    u2 = S.get_state()
    S.close()
    n = u0.shape[1]
    nv = dim + 1
    dev = torch.device("cuda")
    d_u0 = torch.tensor(u0[:nv].reshape(-1), dtype=torch.float64, device=dev)
    d_u1 = torch.tensor(u1[:nv].reshape(-1), dtype=torch.float64, device=dev)
    d_u2 = torch.tensor(u2[:nv].reshape(-1), dtype=torch.float64, device=dev)
    d_out = torch.full((5,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for d_u, ref in ((d_u1, res1[0]), (d_u2, res2[0])):
        pkg.gpu.residuals_noalloc(d_u.data_ptr(), d_u0.data_ptr(), pkg.gpu.DG_FP64, nv, n, n, c0, d_out.data_ptr(),
                                  stream)
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        # same tolerance as the FP64 state parity of the other GPU tests
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0.0)
        if dim == 2:
            assert got[4] == 0.0
    assert res1[0][0] != res2[0][0]


def _residuals_f64(u, snap, n_var, n, c0):
    """The five residual means (src/solver.cpp:518-545) in float64 numpy."""
    out = np.zeros(5)
    c0sq = c0 * c0
    for q in range(n_var):
        s, v = snap[q, :n].astype(np.float64), u[q, :n].astype(np.float64)
        if q == 0:
            out[0] = np.sum((s - v) ** 2) / n
            out[1] = np.sum((s / c0sq - v / c0sq) ** 2) / n
        else:
            out[1 + q] = np.sum((s - v) ** 2) / n
    return out


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_noalloc_several_chunks_padded_planes_larger_call_first(pkg, prec):
    """Inputs spanning several of the kernel's fixed node chunks (a partial
    last chunk), variable planes longer than the node count, and a smaller
    call after a larger one: the smaller call must not read the scratch rows
    the larger call left behind."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(21)
    dt = np.float64 if prec == "fp64" else np.float32
    tdt = torch.float64 if prec == "fp64" else torch.float32
    flag = pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32
    c0 = 340.0
    d_out = torch.full((5,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    # (nodes per variable, plane stride, variables): 4 chunks then 2 chunks
    for n, stride, nv in ((50_000, 50_021, 4), (20_000, 20_013, 3)):
        u = rng.standard_normal((nv, stride)).astype(dt)
        snap = (u + 0.01 * rng.standard_normal((nv, stride))).astype(dt)
        # the padding past n holds large values that must not enter the sums
        u[:, n:] = 1e6
        snap[:, n:] = -1e6
        d_u = torch.tensor(u.reshape(-1), dtype=tdt, device="cuda")
        d_s = torch.tensor(snap.reshape(-1), dtype=tdt, device="cuda")
        for _ in range(2):
            pkg.gpu.residuals_noalloc(d_u.data_ptr(), d_s.data_ptr(), flag, nv, n, stride, c0, d_out.data_ptr(),
                                      stream)
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            ref = _residuals_f64(u, snap, nv, n, c0)
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=0.0)
        if nv == 3:
            assert got[4] == 0.0


def test_noalloc_rejects_inputs_beyond_its_scratch(pkg):
    torch = pytest.importorskip("torch")
    d = torch.zeros(8, dtype=torch.float64, device="cuda")
    too_many = 16384 * 4096 + 1
    with pytest.raises(pkg.gpu.SolverError, match="limit of its fixed scratch"):
        pkg.gpu.residuals_noalloc(d.data_ptr(), d.data_ptr(), pkg.gpu.DG_FP64, 4, too_many, too_many, 340.0,
                                  d.data_ptr(), None)
