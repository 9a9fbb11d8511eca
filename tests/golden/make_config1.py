"""Generates the oracle's FP64 answer for the 2-D LEE workload of the
parity tests (tests/test_gpu_config_parity.py):

  square [-5,5]^2, 45 x 45 cells split into 4050 triangles, interior vertices
  jittered by up to 0.2 h (seed 1), Lagrange order p = 3, all four sides
  Absorbing, mean flow v0 = (-30, 30, 0), rho0 = 1.225, c0 = 100, Gaussian
  initial pressure at the origin (size 1, amplitude 1), RK4 with dt = 1e-5
  for exactly 5000 steps (the reference's accumulated-t loop, t_end chosen
  so that it runs 5000 steps), snapshots every 1e-3, observers at
  (+-2.1, 0, 0) with radius 0.1.

The oracle (oracle/refcpu.cpp, one thread: its multi-threaded faithful mode
keeps the reference's racy nested face loop) runs the reference loop of
src/solver.cpp:413-574 with the initial conditions of
src/dgalerkin.cpp:51-70. About 20 minutes on one x86 core.

Writes config1_fp64.npz next to this script: the mesh the oracle ran on
(node coordinates, element nodes, boundary-group nodes: numpy's arithmetic
on another CPU architecture can build the seeded mesh with last-bit
differences, so the test takes the mesh from the file), the final p, vx,
vy, the observer traces (rho, p, vx, vy per step), the residual trace and
the step times.

  python tests/golden/make_config1.py
"""
import importlib
import importlib.util
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "config1_fp64.npz")

DT = 1e-5
STEPS = 5000
PHYS = dict(v0=(-30.0, 30.0, 0.0), rho0=1.225, c0=100.0)
IC = (0.0, 0.0, 0.0, 1.0, 1.0)
OBS = [(2.1, 0.0, 0.0, 0.1), (-2.1, 0.0, 0.0, 0.1)]
T_RATE = 1e-3
T_END = (STEPS - 0.5) * DT


def mesh_config1(pkg):
    m = pkg.meshgen.square(n=45, half_width=5.0, order=3, jitter=0.2, seed=1)
    return dict(dim=2, order=3, xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=pkg.meshgen.solver_groups(m, {"Absorbing": "Absorbing"}))


def mesh_from_golden(g):
    """The mesh stored with the oracle's answer."""
    return dict(dim=2, order=3, xyz=g["xyz"], elem_nodes=g["elem_nodes"].astype(np.int64),
                groups=[(0, g["boundary_nodes"].astype(np.int64))])


def main():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    pkg = importlib.import_module("dgfem-acoustic_gb300")
    spec = importlib.util.spec_from_file_location("refcpu", os.path.join(ROOT, "oracle", "refcpu.py"))
    oracle = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(oracle)
    mesh = mesh_config1(pkg)
    P = oracle.Problem(mesh, t_start=0.0, t_end=T_END, dt=DT, t_rate=T_RATE, ics=[IC], observers=OBS,
                       num_threads=1, **PHYS)
    assert P.count_steps()[0] == STEPS, P.count_steps()
    t0 = time.time()
    r = P.run()
    assert r["steps"] == STEPS
    assert len(mesh["groups"]) == 1 and mesh["groups"][0][0] == 0  # one Absorbing group
    np.savez_compressed(OUT, state=r["state"][:3], obs=r["obs"][:, :, :4], residuals=r["residuals"][:, :4],
                        times=r["times"], snapshots=r["snapshots"], penalty_hist=np.array(r["penalty_hist"]),
                        xyz=mesh["xyz"], elem_nodes=mesh["elem_nodes"].astype(np.int32),
                        boundary_nodes=np.asarray(mesh["groups"][0][1]).astype(np.int32))
    print("wrote %s (%d steps, %.0f s)" % (OUT, STEPS, time.time() - t0))


if __name__ == "__main__":
    main()
