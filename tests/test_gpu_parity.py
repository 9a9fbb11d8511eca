"""GPU parity against the CPU oracle through the C ABI.

Full runs: final state within 1e-12 (FP64) and 1e-5 (FP32) relative L2 of the
oracle. A single right-hand-side evaluation is compared with a looser bound:
L(u) = Vol - Surf is a difference of terms about (p+1)^2/(h |grad u|/|u|)
times larger than the result, so two FP64 implementations that order their
arithmetic differently agree only to about 1e-11 on L itself (the state they
produce after dt*L is added still agrees to 1e-12)."""
import numpy as np
import pytest

from conftest import rel_l2, smooth_state

pytestmark = pytest.mark.gpu

PHYS = dict(v0=(-30.0, 30.0, 10.0), rho0=1.225, c0=100.0)


def _mesh(pkg, dim, p, reflect=True):
    mg = pkg.meshgen
    if dim == 2:
        m = mg.square(n=5, order=p, seed=3, side_names=["xmin", "xmax", "ymin", "ymax"])
    else:
        m = mg.box(counts=(2, 2, 2), order=p, seed=4)
    bcs = {"xmin": "Reflecting" if reflect else "Absorbing", "xmax": "Absorbing", "ymin": "Reflecting",
           "ymax": "Absorbing", "zmin": "Absorbing", "zmax": "Reflecting"}
    groups = mg.solver_groups(m, bcs)
    return dict(dim=dim, order=p, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=groups)


def kernel_variants(pkg, S):
    """-1 (baseline kernel) and every other stage-kernel variant available
    for S: pipelined (0..), tensor-core (16-20), constant-operator (32..),
    flux-form (48..)."""
    out = [-1]
    for v in list(range(8)) + [16, 17, 18, 19, 20, 21, 22] + list(range(32, 40)) + list(range(48, 64)):
        if S.kernel_info(v)[0] > 0:
            out.append(v)
    return out


def _phys(dim):
    v0 = PHYS["v0"] if dim == 3 else (PHYS["v0"][0], PHYS["v0"][1], 0.0)
    return dict(v0=v0, rho0=PHYS["rho0"], c0=PHYS["c0"])


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("p", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_rhs_parity(pkg, oracle, dim, p, prec):
    mesh = _mesh(pkg, dim, p)
    ph = _phys(dim)
    u = smooth_state(mesh, seed=dim * 10 + p)
    dt = 1e-4
    ref = oracle.Problem(mesh, dt=dt, **ph).stage(u)
    S = pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **ph)
    tol = 5e-11 if prec == "fp64" else 5e-4
    nv = dim + 1
    for v in kernel_variants(pkg, S):
        S.tune(v)
        k = S.rhs(u, dt)
        err = rel_l2(k[:nv], ref[:nv])
        assert err <= tol, (dim, p, prec, v, err)
        if dim == 2:
            assert np.all(k[3] == 0.0)


@pytest.mark.parametrize("dim,p", [(2, 2), (3, 2), (3, 3)])
def test_face_info_matches_oracle(pkg, oracle, dim, p):
    mesh = _mesh(pkg, dim, p)
    f_ref = oracle.Problem(mesh, dt=1e-3, **_phys(dim)).faces()
    S = pkg.gpu.Solver(mesh, **_phys(dim))
    f = S.face_info()
    assert np.array_equal(f["nbr"], f_ref["nbr"])
    assert np.array_equal(f["penalty"], f_ref["penalty"])
    assert np.array_equal(f["bc"], f_ref["bc"])
    info = S.info()
    assert info["penalty_sign_hist"][0] == 0


def _sources_observers(mesh, srcs, obs):
    en = mesh["elem_nodes"]
    x = mesh["xyz"][en.reshape(-1)]
    sdofs = []
    for s in srcs:
        d2 = (x[:, 0] - s[0]) ** 2 + (x[:, 1] - s[1]) ** 2 + (x[:, 2] - s[2]) ** 2
        sdofs.append(np.nonzero(d2 < s[3] ** 2)[0])
    odofs, ows = [], []
    for o in obs:
        d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2 + (x[:, 2] - o[2]) ** 2)
        idx = np.nonzero(d < o[3])[0]
        odofs.append(idx)
        ows.append(1.0 / (d[idx] ** 2 + 1e-12))
    return sdofs, odofs, ows


@pytest.mark.parametrize("variant", [-1, 0, 1, 32, 33, 48, 49, 50, 51, 52, 53])
@pytest.mark.parametrize("dim,p,prec", [(2, 3, "fp64"), (3, 2, "fp64"), (3, 3, "fp64"), (2, 3, "fp32"), (3, 3, "fp32"),
                                        (2, 4, "fp32"), (2, 2, "fp32")])
def test_run_parity(pkg, oracle, dim, p, prec, variant):
    mesh = _mesh(pkg, dim, p)
    ph = _phys(dim)
    dt, nsteps = 2e-4, 40
    src = [0.1, -0.2, 0.1 if dim == 3 else 0.0, 0.45, 1.0, 50.0, 0.3, 1.0]  # x,y,z,size,amp,freq,phase,duration
    obs = [(0.5, 0.3, 0.2 if dim == 3 else 0.0, 0.4), (-0.4, -0.5, 0.0, 0.5)]
    ics = [(0.2, 0.1, 0.0, 0.3, 1.0)]
    P = oracle.Problem(mesh, t_start=0.0, t_end=(nsteps - 0.5) * dt, dt=dt, t_rate=10 * dt,
                       sources=[dict(kind=oracle.SRC_SINE, params=src)], observers=obs, ics=ics, **ph)
    ref = P.run()
    assert ref["steps"] == nsteps
    S = pkg.gpu.Solver(mesh, precision=pkg.gpu.DG_FP64 if prec == "fp64" else pkg.gpu.DG_FP32, **ph)
    if S.kernel_info(variant)[0] == 0:
        pytest.skip("variant %d does not exist for this element type and precision" % variant)
    S.tune(variant)
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
        r, o = S.run(j - i, dt)
        res.append(r), tr.append(o)
        i = j
    res, tr = np.concatenate(res), np.concatenate(tr)
    u = S.get_state()
    tol = 1e-12 if prec == "fp64" else 1e-5
    nv = dim + 1
    assert rel_l2(u[:nv], ref["state"][:nv]) <= tol
    assert rel_l2(res[:, :4], ref["residuals"][:, :4]) <= (1e-10 if prec == "fp64" else 1e-3)
    ob_ref = ref["obs"][:, :, [1, 2, 3, 4]]  # p, vx, vy, vz
    # an observer with no DG node in its radius reports NaN in both (the
    # reference's rule)
    ok = np.isfinite(ob_ref)
    assert np.array_equal(np.isfinite(tr), ok)
    assert rel_l2(tr[ok], ob_ref[ok]) <= tol * 10
