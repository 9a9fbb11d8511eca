"""Curved (non-affine) elements against the CPU oracle, which integrates
every element with the reference's quadrature formulation.

Meshes: the parity meshes with every node moved by a smooth displacement
(meshgen.warp), either a global bend (every element curved, boundary faces
included) or a local bump (a mix of curved and straight-sided elements, so
that curved and affine neighbours meet). The stage kernels that have a
curved path (baseline and pipelined) must agree with the oracle at the same
bounds as on straight-sided meshes; the tensor-core and constant-operator
kernels are not offered on such meshes."""
import numpy as np
import pytest

from conftest import rel_l2, smooth_state
from test_gpu_parity import _mesh, _phys, kernel_variants
from test_gpu_tensor_core import _obs_err, _run

pytestmark = pytest.mark.gpu


def _curved_mesh(pkg, dim, p, kind):
    mesh = _mesh(pkg, dim, p)
    mg = pkg.meshgen
    if kind == "bend":
        amp = 0.01 if dim == 2 else 0.05
        return mg.warp(mesh, amp)
    if dim == 2:
        return mg.warp(mesh, 0.4, center=(1.0, 1.0), radius=3.0)
    return mg.warp(mesh, 0.12, center=(0.3, 0.2, 0.1), radius=0.9)


@pytest.mark.parametrize("kind", ["bend", "bump"])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("p", [2, 3, 4])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_curved_rhs_matches_oracle(pkg, oracle, dim, p, prec, kind):
    mesh = _curved_mesh(pkg, dim, p, kind)
    ph = _phys(dim)
    u = smooth_state(mesh, seed=dim * 10 + p)
    dt = 1e-4
    ref = oracle.Problem(mesh, dt=dt, **ph).stage(u)
    S = pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **ph)
    info = S.info()
    E = len(mesh["elem_nodes"])
    assert 0 < info["n_curved"] <= E
    if kind == "bend":
        assert info["n_curved"] == E
    else:
        assert info["n_curved"] < E
    tol = 5e-11 if prec == "fp64" else 5e-4
    nv = dim + 1
    variants = kernel_variants(pkg, S)
    assert variants and all(v < 16 for v in variants)
    for v in variants:
        S.tune(v)
        k = S.rhs(u, dt)
        err = rel_l2(k[:nv], ref[:nv])
        assert err <= tol, (dim, p, prec, kind, v, err)
        if dim == 2:
            assert np.all(k[3] == 0.0)
    # the straight-sided-only kernels are not offered
    for v in [16, 17, 18, 19, 20, 21, 22, 32]:
        assert S.kernel_info(v)[0] == 0
        with pytest.raises(pkg.gpu.SolverError):
            S.tune(v)
    S.close()


def test_straight_mesh_has_no_curved_elements(pkg):
    S = pkg.gpu.Solver(_mesh(pkg, 3, 3), **_phys(3))
    assert S.info()["n_curved"] == 0
    S.close()


@pytest.mark.parametrize("dim,p,kind", [(2, 3, "bend"), (2, 4, "bump"), (3, 2, "bend"), (3, 3, "bump")])
@pytest.mark.parametrize("prec,variant", [("fp64", -1), ("fp64", 0), ("fp32", 0)])
def test_curved_run_matches_oracle(pkg, oracle, dim, p, kind, prec, variant):
    mesh = _curved_mesh(pkg, dim, p, kind)
    u, res, tr, ref = _run(pkg, oracle, mesh, _phys(dim), prec, variant, 40)
    nv = dim + 1
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert rel_l2(u[:nv], ref["state"][:nv]) <= tol
    assert _obs_err(tr, ref["obs"][:, :, [1, 2, 3, 4]]) <= 10 * tol
    if prec == "fp64":
        assert rel_l2(res[:, :4], ref["residuals"][:, :4]) <= 1e-9
