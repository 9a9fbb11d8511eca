"""Batched-ensemble workload: independent 2-D LEE instances on jittered square
meshes, each with its own order, monopole source, mean flow and time step,
advanced together by the batched GPU path (gpu.Batch).

The parameter distributions are the ensemble study's: element count
log-uniform in [1e3, 5e4] (structured grid of n x n squares split into
triangles, n = ceil(sqrt(E/2)), interior vertices jittered by up to 20 % of
the spacing), order uniform in {2, 3, 4}, monopole position uniform in
[-4, 4]^2, frequency uniform in [20, 400] Hz, Mach number uniform in
[0, 0.3] in a uniform direction (v0 = M c0 (cos th, sin th)), all sides
Absorbing, time step from CFL 0.5: dt = CFL h_min / ((c0 + |v0|)(2p + 1)),
h_min the smallest element altitude of the instance's mesh.
"""
import importlib
import math

import numpy as np

HALF_WIDTH = 5.0
RHO0, C0 = 1.225, 340.0
CFL, JITTER = 0.5, 0.2
SOURCE_SIZE, SOURCE_AMP = 0.2, 0.1
OBSERVERS = [(2.5, 2.5, 0.0, 0.3), (-2.5, 2.5, 0.0, 0.3), (-2.5, -2.5, 0.0, 0.3), (2.5, -2.5, 0.0, 0.3)]


def _pkg():
    return importlib.import_module(__name__.rsplit(".", 1)[0])


def square_mesh(grid, p, seed):
    """Jittered [-5,5]^2 triangle mesh of order p, all sides Absorbing."""
    mg = _pkg().meshgen
    m = mg.square(n=grid, order=p, half_width=HALF_WIDTH, jitter=JITTER, seed=seed)
    return dict(dim=2, order=p, xyz=m["xyz"], elem_nodes=m["elem_nodes"],
                groups=mg.solver_groups(m, {"Absorbing": "Absorbing"}))


def time_step(mesh, p, mach):
    """dt = CFL h_min / ((c0 + |v0|)(2p + 1)), h_min the mesh's smallest
    element altitude (cached on the mesh dict)."""
    if "h_min" not in mesh:
        mesh["h_min"] = _pkg().meshgen.min_altitude(mesh)
    return CFL * mesh["h_min"] / ((C0 + mach * C0) * (2 * p + 1))


def instance(mesh, p, sx, sy, f, mach, theta):
    v0 = (mach * C0 * math.cos(theta), mach * C0 * math.sin(theta), 0.0)
    src = [sx, sy, 0.0, SOURCE_SIZE, SOURCE_AMP, f, 0.0, 1e9]  # x,y,z,size,amp,freq,phase,duration
    return dict(mesh=mesh, v0=v0, dt=time_step(mesh, p, mach), src=src, obs=OBSERVERS, p=p,
                params=(sx, sy, f, mach, theta, p))


def draw_instances(n=256, seed=4):
    """Seeded draws with the distributions above (one mesh per instance)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        E = float(np.exp(rng.uniform(np.log(1e3), np.log(5e4))))
        grid = int(np.ceil(np.sqrt(E / 2)))
        p = int(rng.integers(2, 5))
        sx, sy = rng.uniform(-4, 4, 2)
        f = rng.uniform(20, 400)
        mach = rng.uniform(0, 0.3)
        th = rng.uniform(0, 2 * np.pi)
        mesh = square_mesh(grid, p, int(rng.integers(1 << 30)))
        out.append(instance(mesh, p, sx, sy, f, mach, th))
    return out


def node_sets(mesh, src, obs):
    """DG node slots of the source (strict radius) and of each observer with
    their inverse-distance weights 1/(d^2 + 1e-12), as the reference selects
    them (src/solver.cpp:339-383)."""
    x = mesh["xyz"][mesh["elem_nodes"].reshape(-1)]
    d2 = (x[:, 0] - src[0]) ** 2 + (x[:, 1] - src[1]) ** 2 + (x[:, 2] - src[2]) ** 2
    sdofs = [np.nonzero(d2 < src[3] ** 2)[0]]
    odofs, ows = [], []
    for o in obs:
        d = np.sqrt((x[:, 0] - o[0]) ** 2 + (x[:, 1] - o[1]) ** 2 + (x[:, 2] - o[2]) ** 2)
        idx = np.nonzero(d < o[3])[0]
        odofs.append(idx)
        ows.append(1.0 / (d[idx] ** 2 + 1e-12))
    return sdofs, odofs, ows


def make_batch(insts, precision, n_steps, device=0):
    """A gpu.Batch of the instances with sources (monopole values for n_steps
    steps) and observers set; the state starts at rest."""
    gpu = _pkg().gpu
    B = gpu.Batch([dict(mesh=i["mesh"], v0=i["v0"], dt=i["dt"]) for i in insts], rho0=RHO0, c0=C0,
                  precision=precision, device=device)
    cache = {}
    for k, i in enumerate(insts):
        key = id(i["mesh"])
        if key not in cache:
            cache[key] = node_sets(i["mesh"], i["src"], i["obs"])[1:]
        od, ow = cache[key]
        sd = node_sets(i["mesh"], i["src"], [])[0]
        t = np.arange(n_steps + 1) * i["dt"]
        B.set_sources(k, sd, (i["src"][4] * np.sin(2 * np.pi * i["src"][5] * t + i["src"][6]))[:, None])
        B.set_observers(k, od, ow)
    return B
