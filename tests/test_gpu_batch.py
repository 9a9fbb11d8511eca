"""Batched ensembles (dg_batch_*): a batch of instances with different element
types, mean flows, time steps, sources and observers must give each instance
the result of its own single-instance run, and the FP32 batch must stay within
1e-5 relative L2 of the FP64 batch."""
import numpy as np
import pytest

from conftest import rel_l2, smooth_state

pytestmark = pytest.mark.gpu


def _instances(pkg):
    mg = pkg.meshgen
    specs = [("sq", 4, 2, (-20.0, 10.0, 0.0), 3e-5, 1), ("sq", 5, 3, (15.0, 5.0, 0.0), 2e-5, 2),
             ("sq", 3, 3, (0.0, -30.0, 0.0), 2.5e-5, 3), ("box", 2, 2, (5.0, 0.0, -10.0), 1e-5, 4),
             ("sq", 3, 2, (0.0, 0.0, 0.0), 4e-5, 5)]
    out = []
    for kind, n, p, v0, dt, seed in specs:
        if kind == "sq":
            m = mg.square(n=n, order=p, seed=seed, half_width=1.0)
            groups = mg.solver_groups(m, {"Absorbing": "Absorbing"})
            src = [0.1, -0.1, 0.0, 0.3, 1.0, 40.0 + 10 * seed, 0.2, 1.0]
            obs = [(0.3, 0.2, 0.0, 0.3), (-0.4, -0.3, 0.0, 0.35)]
        else:
            m = mg.box(counts=(n, n, n), order=p, seed=seed)
            groups = mg.solver_groups(m, {"xmin": "Reflecting", "xmax": "Reflecting", "ymin": "Absorbing",
                                          "ymax": "Absorbing", "zmin": "Absorbing", "zmax": "Absorbing"})
            src = [0.0, 0.1, 0.0, 0.5, 1.0, 60.0, 0.0, 1.0]
            obs = [(0.3, 0.3, 0.3, 0.4)]
        mesh = dict(dim=m["dim"], order=p, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=groups)
        out.append(dict(mesh=mesh, v0=v0 if m["dim"] == 3 else (v0[0], v0[1], 0.0), dt=dt, src=src, obs=obs,
                        seed=seed))
    return out


def _sets(mesh, src, obs):
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    d2 = ((x - np.array(src[:3])) ** 2).sum(1)
    sd = [np.nonzero(d2 < src[3] ** 2)[0]]
    od, ow = [], []
    for o in obs:
        d = np.sqrt(((x - np.array(o[:3])) ** 2).sum(1))
        idx = np.nonzero(d < o[3])[0]
        od.append(idx)
        ow.append(1.0 / (d[idx] ** 2 + 1e-12))
    return sd, od, ow


def _values(inst, nsteps):
    t = np.arange(nsteps) * inst["dt"]
    s = inst["src"]
    return np.where(t < s[7], s[4] * np.sin(2 * np.pi * s[5] * t + s[6]), np.nan)[:, None]


def _run_batch(pkg, insts, nsteps, precision):
    B = pkg.gpu.Batch([dict(mesh=i["mesh"], v0=i["v0"], dt=i["dt"]) for i in insts], rho0=1.225, c0=100.0,
                      precision=precision)
    for k, i in enumerate(insts):
        B.set_state(k, smooth_state(i["mesh"], seed=i["seed"]))
        sd, od, ow = _sets(i["mesh"], i["src"], i["obs"])
        B.set_sources(k, sd, _values(i, nsteps))
        B.set_observers(k, od, ow)
    obs = B.run(nsteps)
    states = [B.get_state(k) for k in range(len(insts))]
    info = B.info()
    B.close()
    return states, obs, info


def test_batch_equals_single_instance_runs(pkg):
    insts = _instances(pkg)
    nsteps = 25
    states, obs, info = _run_batch(pkg, insts, nsteps, pkg.gpu.DG_FP64)
    assert info["n_groups"] == 3
    for k, i in enumerate(insts):
        S = pkg.gpu.Solver(i["mesh"], v0=i["v0"], rho0=1.225, c0=100.0, precision=pkg.gpu.DG_FP64)
        S.set_state(smooth_state(i["mesh"], seed=i["seed"]))
        sd, od, ow = _sets(i["mesh"], i["src"], i["obs"])
        S.set_sources(sd)
        S.set_source_values(_values(i, nsteps))
        S.set_observers(od, ow)
        S.snapshot()
        _, o = S.run(nsteps, i["dt"])
        u = S.get_state()
        S.close()
        nv = i["mesh"]["dim"] + 1
        assert rel_l2(states[k][:nv], u[:nv]) <= 1e-13, k
        assert rel_l2(obs[k], o) <= 1e-13, k


def test_batch_fp32_within_1e5_of_fp64(pkg):
    insts = _instances(pkg)
    nsteps = 200
    s64, o64, _ = _run_batch(pkg, insts, nsteps, pkg.gpu.DG_FP64)
    s32, o32, _ = _run_batch(pkg, insts, nsteps, pkg.gpu.DG_FP32)
    for k, i in enumerate(insts):
        nv = i["mesh"]["dim"] + 1
        assert rel_l2(s32[k][:nv], s64[k][:nv]) <= 1e-5, (k, rel_l2(s32[k][:nv], s64[k][:nv]))


def test_sources_covering_no_node(pkg):
    """A source whose radius holds no node overwrites nothing (as in the
    reference's node selection): a batch in which every instance of an
    element type has such a source runs, and each instance matches its
    single-instance run with the same empty source."""
    insts = _instances(pkg)[:2]  # 2-D squares of orders 2 and 3: one group each
    for i in insts:
        i["src"] = list(i["src"])
        i["src"][3] = 1e-9
    nsteps = 10
    states, obs, _ = _run_batch(pkg, insts, nsteps, pkg.gpu.DG_FP64)
    for k, i in enumerate(insts):
        sd, od, ow = _sets(i["mesh"], i["src"], i["obs"])
        assert sd[0].size == 0
        S = pkg.gpu.Solver(i["mesh"], v0=i["v0"], rho0=1.225, c0=100.0, precision=pkg.gpu.DG_FP64)
        S.set_state(smooth_state(i["mesh"], seed=i["seed"]))
        S.set_sources(sd)
        S.set_source_values(_values(i, nsteps))
        S.set_observers(od, ow)
        _, o = S.run(nsteps, i["dt"])
        u = S.get_state()
        S.close()
        assert rel_l2(states[k][:3], u[:3]) <= 1e-13, k
        assert rel_l2(obs[k], o) <= 1e-13, k
