"""One launch per RK stage for a batch of 2-D instances of mixed order (the
mixed-order stage kernel and its work queue, dg_batch_set_fused): the same
results as the batch's per-order graph and as the FP64 batch, with more tiles
than resident blocks so that blocks take several queue items of different
orders, and with an order missing from the batch."""
import numpy as np
import pytest

from conftest import rel_l2, smooth_state

pytestmark = pytest.mark.gpu


def _instances(pkg, orders, grids):
    mg = pkg.meshgen
    out = []
    for k, (p, n) in enumerate(zip(orders, grids)):
        m = mg.square(n=n, order=p, seed=100 + k, half_width=1.0)
        mesh = dict(dim=2, order=p, xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                    groups=mg.solver_groups(m, {"Absorbing": "Absorbing"}))
        ang = 0.7 * k
        out.append(dict(mesh=mesh, v0=(25.0 * np.cos(ang), 25.0 * np.sin(ang), 0.0), dt=(1.0 + 0.1 * k) * 4e-6 / p,
                        src=[0.1 * (k % 3) - 0.1, 0.05, 0.0, 0.2, 1.0, 300.0 + 40 * k, 0.0, 1.0],
                        obs=[(0.4, 0.3, 0.0, 0.2), (-0.5, -0.2, 0.0, 0.25)], seed=k + 1))
    return out


def _run(pkg, insts, nsteps, precision, fused):
    B = pkg.gpu.Batch([dict(mesh=i["mesh"], v0=i["v0"], dt=i["dt"]) for i in insts], rho0=1.225, c0=340.0,
                      precision=precision)
    if fused is not None:
        B.set_fused(fused)
    for k, i in enumerate(insts):
        B.set_state(k, smooth_state(i["mesh"], seed=i["seed"]))
        x = i["mesh"]["xyz"][i["mesh"]["elem_nodes"].reshape(-1)]
        s = i["src"]
        sd = [np.nonzero(((x[:, 0] - s[0]) ** 2 + (x[:, 1] - s[1]) ** 2) < s[3] ** 2)[0]]
        od, ow = [], []
        for o in i["obs"]:
            d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2)
            idx = np.nonzero(d < o[3])[0]
            od.append(idx)
            ow.append(1.0 / (d[idx] ** 2 + 1e-12))
        t = np.arange(nsteps + 1) * i["dt"]
        B.set_sources(k, sd, (s[4] * np.sin(2 * np.pi * s[5] * t))[:, None])
        B.set_observers(k, od, ow)
    used = B.fused
    obs = B.run(nsteps)
    states = [B.get_state(k) for k in range(len(insts))]
    B.close()
    return states, obs, used


@pytest.mark.parametrize("orders", [(2, 3, 4, 2, 3, 4, 4, 2), (3, 4, 4, 3)])
def test_fused_matches_per_order_graph_and_fp64(pkg, orders):
    grids = [60, 45, 40, 30, 50, 35, 45, 55][:len(orders)]
    insts = _instances(pkg, orders, grids)
    nsteps = 30
    s_f, o_f, used_f = _run(pkg, insts, nsteps, pkg.gpu.DG_FP32, True)
    s_g, o_g, used_g = _run(pkg, insts, nsteps, pkg.gpu.DG_FP32, False)
    s_64, o_64, _ = _run(pkg, insts, nsteps, pkg.gpu.DG_FP64, None)
    assert used_f and not used_g
    # both FP32 paths (different kernels, different rounding) within the FP32
    # bound of the FP64 batch and of each other
    for k in range(len(insts)):
        assert rel_l2(s_f[k][:3], s_g[k][:3]) <= 1e-5, (k, rel_l2(s_f[k][:3], s_g[k][:3]))
        assert rel_l2(s_f[k][:3], s_64[k][:3]) <= 1e-5, (k, rel_l2(s_f[k][:3], s_64[k][:3]))
        ok = np.isfinite(o_64[k])
        assert np.array_equal(np.isfinite(o_f[k]), ok)
        assert rel_l2(o_f[k][ok], o_64[k][ok]) <= 1e-4, k


def test_fused_needs_fp32_2d_orders_2_to_4(pkg):
    mg = pkg.meshgen
    m3 = mg.box(counts=(2, 2, 2), order=2, seed=1)
    mesh3 = dict(dim=3, order=2, xyz=m3["xyz"], elem_nodes=m3["elem_nodes"], groups=[])
    insts = _instances(pkg, (2, 3), (10, 10))
    B = pkg.gpu.Batch([dict(mesh=i["mesh"], v0=i["v0"], dt=i["dt"]) for i in insts] +
                      [dict(mesh=mesh3, v0=(0.0, 0.0, 0.0), dt=1e-6)], rho0=1.225, c0=340.0,
                      precision=pkg.gpu.DG_FP32)
    assert not B.fused
    with pytest.raises(pkg.gpu.SolverError, match="one launch per stage"):
        B.set_fused(True)
    B.close()
    B = pkg.gpu.Batch([dict(mesh=i["mesh"], v0=i["v0"], dt=i["dt"]) for i in insts], rho0=1.225, c0=340.0,
                      precision=pkg.gpu.DG_FP64)
    assert not B.fused
    B.close()
