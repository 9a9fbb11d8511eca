"""The project's time-step rule dt = CFL h_min / ((c0 + |v0|)(2p + 1)) with
CFL 0.5 and h_min the smallest element altitude keeps the benchmark
workloads stable over their full run lengths: the most restrictive ensemble
instance (p = 4, no mean flow: the largest dt) for 3000 steps, and the 3-D
cube (p = 3) for its 2000 steps. With h_min taken as the nominal edge length
instead, p = 4 ensemble instances at Mach < 0.02 grew without bound."""
import importlib.util
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ensemble_p4_without_mean_flow_stays_bounded(pkg):
    ens = pkg.ensemble
    mesh = ens.square_mesh(25, 4, 504)
    inst = ens.instance(mesh, 4, 0.5, -1.0, 350.0, 0.0, 0.0)
    B = ens.make_batch([inst], pkg.gpu.DG_FP32, 3000)
    peak = 0.0
    for _ in range(6):
        obs = B.run(500)[0]
        assert np.all(np.isfinite(obs))
        peak = max(peak, float(np.abs(obs[:, :, 0]).max()))
    B.close()
    assert 0.0 < peak < 10 * ens.SOURCE_AMP, peak


def test_cube_workload_stays_bounded(pkg):
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    W = bench.CUBE
    mesh, dt, srcs, obs = bench.build_problem(W)
    src = srcs[0]
    S = pkg.gpu.Solver(mesh, v0=W["v0"], rho0=W["rho0"], c0=W["c0"], precision=pkg.gpu.DG_FP32)
    sd, od, ow = bench.node_sets(mesh, srcs, obs)
    S.set_sources(sd)
    n = 2000
    S.set_source_values(bench.source_values(srcs, n + 1, dt))
    S.set_observers(od, ow)
    S.snapshot()
    peak = 0.0
    for _ in range(4):
        res, tr = S.run(n // 4, dt)
        assert np.all(np.isfinite(res)) and np.all(np.isfinite(tr))
        peak = max(peak, float(np.abs(tr[:, :, 0]).max()))
    S.close()
    assert 0.0 < peak < 10 * src[4], peak
