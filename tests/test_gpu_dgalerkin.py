"""End-to-end runs of the dgalerkin driver on the GPU: the reference's
2d_hilltop case against its golden residual trace and against the oracle,
and the output files a user of the reference expects."""
import gzip
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from vtu_read import read_vtu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")
EXE = os.path.join(ROOT, "dgfem-acoustic_gb300", "_build", "dgalerkin")


def _case(tmp_path, t_end=None, extra=None):
    import json
    cfg = json.load(open(os.path.join(GOLDEN, "2d_hilltop.json")))
    if t_end is not None:
        cfg["solver"]["time"]["end"] = t_end
    if extra:
        cfg.update(extra)
    with gzip.open(os.path.join(GOLDEN, "2d_hilltop_fs.msh.gz"), "rb") as f:
        (tmp_path / "2d_hilltop_fs.msh").write_bytes(f.read())
    (tmp_path / "case.json").write_text(json.dumps(cfg))
    return tmp_path


def _run(cwd, cfg="case.json"):
    r = subprocess.run([EXE, cfg], cwd=str(cwd), stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout
    return r.stdout


def _residuals(path):
    return np.genfromtxt(path, delimiter=";", skip_header=1)


def test_hilltop_matches_golden_trace(tmp_path):
    d = _case(tmp_path)
    _run(d)
    mine = _residuals(d / "residuals.csv")
    gold = _residuals(os.path.join(GOLDEN, "hilltop_residuals.csv"))
    assert mine.shape[0] == gold.shape[0] == 1000
    np.testing.assert_allclose(mine[:, 0], gold[:, 0], rtol=0, atol=1e-9)  # step times
    # rows dominated by the physical change (last 40 steps of each 0.1 s
    # snapshot interval); the reference run's data race sets the floor
    for k in range(10):
        rows = np.arange(100 * k + 60, 100 * k + 100)
        rel = np.abs(mine[rows, 1:5] - gold[rows, 1:5]) / gold[rows, 1:5]
        assert rel.max() < (0.05 if k < 1 else 0.1), (k, rel.max(axis=0))
    assert np.all(mine[:, 5] == 0.0)  # res_vz in 2-D
    # outputs of the reference's interface
    res = d / "results"
    for step in range(0, 1000, 100):
        assert (res / ("result%d.vtu" % step)).exists()
    # snapshots written by the asynchronous writer decode to the mesh's
    # triangles and finite cell data; the state changes between snapshots
    v0, v9 = read_vtu(str(res / "result0.vtu")), read_vtu(str(res / "result900.vtu"))
    for v in (v0, v9):
        assert v["n_cells"] == len(v["types"]) and np.all(v["types"] == 5)
        assert v["connectivity"].shape == (3 * v["n_cells"],) and v["connectivity"].max() < v["n_points"]
        assert np.all(np.isfinite(v["Pressure [Pa]"])) and v["Velocity [m/s]"].shape == (v["n_cells"], 3)
        scale = np.abs(v["Pressure [Pa]"]).max() / 340.0 ** 2
        np.testing.assert_allclose(v["Density [kg/m³]"], v["Pressure [Pa]"] / 340.0 ** 2, rtol=0, atol=1e-13 * scale)
    assert not np.array_equal(v0["Pressure [Pa]"], v9["Pressure [Pa]"])
    pvd = (d / "results.pvd").read_text()
    assert pvd.count("<DataSet") == 10 and 'timestep="0.1" part="0" file="results/result100.vtu"' in pvd
    obs = np.genfromtxt(res / "observers1.txt", delimiter=";", skip_header=1)
    assert obs.shape == (1000, 6)
    assert (res / "observers1.txt").read_text().splitlines()[0] == "time;density;pressure;velocity_x;velocity_y;velocity_z"
    np.testing.assert_allclose(obs[:, 1], obs[:, 2] / 340.0 ** 2, rtol=1e-5)
    wav = (res / "observer_1.wav").read_bytes()
    assert wav[:4] == b"RIFF" and wav[8:12] == b"WAVE"
    rate, bits = struct.unpack("<I", wav[24:28])[0], struct.unpack("<H", wav[34:36])[0]
    assert rate == 1000 and bits == 16
    assert len(wav) == 44 + 2 * 1000
    fft = (res / "observer_1_fft.txt").read_text().splitlines()
    psd = (res / "observer_1_psd.txt").read_text().splitlines()
    assert fft[0] == "Frequency Norm Real Imag SPL" and len(fft) == 1 + 255  # rows 1..nb/2-1, nb = 512
    assert psd[0] == "Frequency Norm PSD" and len(psd) == 1 + 256  # rows 1..nb/2


def test_hilltop_short_run_matches_oracle(tmp_path, pkg, oracle):
    d = _case(tmp_path, t_end=0.0495)
    _run(d)
    mine = _residuals(d / "residuals.csv")
    m = pkg.host.load_mesh(str(d / "2d_hilltop_fs.msh"))
    groups = [(0, m["groups"][0][2]), (1, m["groups"][1][2])]
    mesh = dict(dim=2, order=1, xyz=m["xyz"], elem_nodes=m["elem_nodes"], groups=groups)
    P = oracle.Problem(mesh, rho0=1.225, c0=340.0, t_end=0.0495, dt=1e-3, t_rate=0.1,
                       observers=[(500, 2, 0, 10)], ics=[(0, 200, 0, 2000, 1.0)])
    ref = P.run()
    assert ref["steps"] == mine.shape[0] == 50
    # residuals are written with 6 significant digits
    np.testing.assert_allclose(mine[:, 1:5], ref["residuals"][:, :4], rtol=1e-5)
    obs = np.genfromtxt(d / "results" / "observers1.txt", delimiter=";", skip_header=1)
    np.testing.assert_allclose(obs[:, 2], ref["obs"][:, 0, 1], rtol=1e-5, atol=1e-12)


def test_bad_arguments_and_missing_files(tmp_path):
    r = subprocess.run([EXE], cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    assert r.returncode == 7  # E2BIG, as the reference
    r = subprocess.run([EXE, "missing.json"], cwd=str(tmp_path), stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    assert r.returncode == 1 and "not found" in r.stdout
