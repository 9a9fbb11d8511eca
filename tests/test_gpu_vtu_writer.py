"""Asynchronous VTU snapshots (dg_vtu_*): the files decode to the mesh the
writer was given and to the cell means (the reference's VTU formula) of the
state at the moment of each call, whether compressed (zlib blocks) or raw,
with several files in flight while the solver keeps stepping."""
import os

import numpy as np
import pytest

from test_gpu_parity import _mesh, _phys
from vtu_read import read_vtu

pytestmark = pytest.mark.gpu


def _setup(pkg, dim=2, p=3, prec=None):
    mesh = _mesh(pkg, dim, p)
    g = pkg.gpu
    S = g.Solver(mesh, precision=prec if prec is not None else g.DG_FP64, **_phys(dim))
    pts = np.asarray(mesh["xyz"], dtype=np.float64)
    cells = np.asarray(mesh["elem_nodes"], dtype=np.int64)[:, :dim + 1].copy()
    return mesh, S, pts, cells


def _state(S, mesh, seed):
    from conftest import smooth_state
    u = smooth_state(mesh, seed=seed)
    S.set_state(u)
    return u


@pytest.mark.parametrize("compression", [0, 1])
@pytest.mark.parametrize("dim", [2, 3])
def test_file_holds_mesh_and_cell_means(pkg, tmp_path, compression, dim):
    mesh, S, pts, cells = _setup(pkg, dim)
    _state(S, mesh, 5)
    W = pkg.gpu.VtuWriter(S, pts, cells, compression=compression)
    path = tmp_path / "a.vtu"
    W.write(path)
    W.flush()
    assert W.stats() == (1, bool(compression))
    W.close()
    v = read_vtu(str(path))
    assert v["compressed"] == bool(compression)
    E = len(cells)
    assert v["n_points"] == len(pts) and v["n_cells"] == E
    np.testing.assert_array_equal(v["points"], pts)
    np.testing.assert_array_equal(v["connectivity"], cells.reshape(-1))
    np.testing.assert_array_equal(v["offsets"], (np.arange(E) + 1) * (dim + 1))
    assert np.all(v["types"] == (10 if dim == 3 else 5))
    p, rho, vel = S.cell_means()
    np.testing.assert_array_equal(v["Pressure [Pa]"], p)
    np.testing.assert_array_equal(v["Density [kg/m³]"], rho)
    np.testing.assert_array_equal(v["Velocity [m/s]"], vel)
    S.close()


@pytest.mark.parametrize("prec_name", ["fp64", "fp32"])
def test_snapshots_in_flight_track_the_state(pkg, tmp_path, prec_name):
    """Three files written while stepping with a single slot (every call
    waits for the previous file): each holds the state of its own call, the
    same as the cell means of an identical solver stepped in lockstep."""
    g = pkg.gpu
    prec = g.DG_FP64 if prec_name == "fp64" else g.DG_FP32
    mesh, S, pts, cells = _setup(pkg, 2, 3, prec)
    _, T, _, _ = _setup(pkg, 2, 3, prec)
    for X in (S, T):
        _state(X, mesh, 9)
        X.snapshot()
    W = g.VtuWriter(S, pts, cells, compression=-1, slots=1)
    expect = []
    dt = 2e-4
    for k in range(3):
        W.write(tmp_path / ("s%d.vtu" % k))
        expect.append(T.cell_means())
        S.run(7, dt)
        T.run(7, dt)
    W.close()
    for k in range(3):
        v = read_vtu(str(tmp_path / ("s%d.vtu" % k)))
        np.testing.assert_array_equal(v["Pressure [Pa]"], expect[k][0])
        np.testing.assert_array_equal(v["Velocity [m/s]"], expect[k][2])
    assert not np.array_equal(expect[0][0], expect[2][0])
    S.close(), T.close()


def test_errors(pkg, tmp_path):
    mesh, S, pts, cells = _setup(pkg, 2, 2)
    bad = cells.copy()
    bad[0, 0] = len(pts)
    with pytest.raises(pkg.gpu.SolverError):
        pkg.gpu.VtuWriter(S, pts, bad)
    W = pkg.gpu.VtuWriter(S, pts, cells, compression=0)
    W.write(os.path.join(str(tmp_path), "no_such_dir", "x.vtu"))
    with pytest.raises(pkg.gpu.SolverError, match="cannot write"):
        W.flush()
    # the writer stays usable after a failed file
    W.write(tmp_path / "ok.vtu")
    W.flush()
    assert W.stats()[0] == 1
    W.close()
    S.close()
