"""Host front end: mesh reading/writing, configuration parsing with the
reference's semantics, the formula evaluator, source values, WAV I/O,
spectra and the PVD schedule (src/configParser.cpp, src/eqEdit.cpp,
src/utils.cpp, src/fft.cpp, src/Mesh.cpp:1232-1253)."""
import gzip
import json
import math
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture
def hilltop_dir(tmp_path):
    with gzip.open(os.path.join(GOLDEN, "2d_hilltop_fs.msh.gz"), "rb") as f:
        (tmp_path / "2d_hilltop_fs.msh").write_bytes(f.read())
    return tmp_path


def test_read_hilltop_mesh(pkg, hilltop_dir):
    m = pkg.host.load_mesh(str(hilltop_dir / "2d_hilltop_fs.msh"))
    assert (m["dim"], m["order"]) == (2, 1)
    assert m["elem_nodes"].shape == (7199, 3)
    assert m["xyz"].shape == (3815, 3)
    assert [(g[0], g[1], len(g[2])) for g in m["groups"]] == [(1, "abs", 194), (2, "ref", 237)]


MSH40 = """$MeshFormat
4 0 8
$EndMeshFormat
$PhysicalNames
2
1 7 "wall"
2 1 "Domain"
$EndPhysicalNames
$Entities
4 1 1 0
1 0 0 0 0 0 0 0
2 1 0 0 1 0 0 0
3 1 1 0 1 1 0 0
4 0 1 0 0 1 0 0
1 0 0 0 1 0 0 1 7 2 1 -2
1 0 0 0 1 1 0 1 1 0
$EndEntities
$Nodes
2 4
1 2 0 3
1 0 0 0
2 1 0 0
3 1 1 0
1 1 0 1
4 0 1 0
$EndNodes
$Elements
2 3
1 1 1 1
1 1 2
1 2 2 2
2 1 2 3
3 1 3 4
$EndElements
"""


def test_read_msh40(pkg, tmp_path):
    p = tmp_path / "m.msh"
    p.write_text(MSH40)
    m = pkg.host.load_mesh(str(p))
    assert (m["dim"], m["order"]) == (2, 1)
    assert m["elem_nodes"].tolist() == [[0, 1, 2], [0, 2, 3]]
    assert [(g[0], g[1], sorted(g[2].tolist())) for g in m["groups"]] == [(7, "wall", [0, 1])]


@pytest.mark.parametrize("dim,p", [(2, 3), (3, 2), (3, 4)])
def test_mesh_write_read_roundtrip(pkg, tmp_path, dim, p):
    mg = pkg.meshgen
    m = mg.square(n=3, order=p, side_names=["a", "b", "c", "d"]) if dim == 2 else mg.box(counts=(2, 1, 1), order=p)
    path = str(tmp_path / "w.msh")
    pkg.host.write_mesh(path, dim, p, m["xyz"], m["elem_nodes"], [(g[0], g[1], g[3]) for g in m["groups"]])
    r = pkg.host.load_mesh(path)
    assert (r["dim"], r["order"]) == (dim, p)
    np.testing.assert_array_equal(r["elem_nodes"], m["elem_nodes"])
    np.testing.assert_allclose(r["xyz"], m["xyz"], rtol=0, atol=0)
    for g, h in zip(m["groups"], r["groups"]):
        assert g[0] == h[0] and g[1] == h[1]
        assert set(h[2].tolist()) <= set(g[2].tolist())  # nodes of the written boundary faces


FORMULAS = [
    ("0.1*sin(2*pi*50*t)", 0.003, 0.1 * math.sin(2 * math.pi * 50 * 0.003)),
    ("2^3^2", 0, 64.0),                  # left associative
    ("-2^2", 0, -4.0),                   # unary minus binds like '*'
    ("-2*3+1", 0, -5.0),
    ("(1+2)*3-4/2", 0, 7.0),
    ("exp(-t)*cos(t)", 0.5, math.exp(-0.5) * math.cos(0.5)),
    ("abs(-3)+int(2.7)+frac(2.25)+rond(2.5)+rond(2.4)", 0, 3 + 2 + 0.25 + 3 + 2),
    ("log(100)+ln(e)", 0, 3.0),
    ("sh(1)-ch(1)+th(0)", 0, math.sinh(1) - math.cosh(1)),
    ("ash(-1)+ach(2)+ath(0.5)", 0, -math.asinh(1) + math.acosh(2) + math.atanh(0.5)),
    ("(1+2", 0, 3.0),                    # one missing ')' is tolerated
    ("1e-3*t", 2.0, 2e-3),
    ("pi", 0, math.pi),
]


@pytest.mark.parametrize("expr,t,val", FORMULAS)
def test_formula_evaluator(pkg, expr, t, val):
    ok, v = pkg.host.formula(expr, t)
    assert ok
    assert v == pytest.approx(val, rel=1e-14, abs=1e-15)


@pytest.mark.parametrize("expr", ["2*-3", "--2", "foo(1)", "x+1", "2 + 3", "", "2(3)", "1+", "sin"])
def test_formula_errors_give_minus_one(pkg, expr):
    ok, v = pkg.host.formula(expr, 0.0)
    assert not ok and v == -1.0


def test_json_config_hilltop(pkg, hilltop_dir):
    cfg = json.load(open(os.path.join(GOLDEN, "2d_hilltop.json")))
    cfg["mesh"]["File"] = str(hilltop_dir / "2d_hilltop_fs.msh")
    p = hilltop_dir / "c.json"
    p.write_text(json.dumps(cfg))
    c = pkg.host.load_config(str(p))
    assert (c["t_start"], c["t_end"], c["dt"], c["t_rate"]) == (0.0, 1.0, 1e-3, 0.1)
    assert c["time_method"] == "Runge-Kutta" and c["num_threads"] == 20
    assert c["bcs"] == [(1, 0), (2, 1)]
    assert c["v0"] == (0.0, 0.0, 0.0) and c["rho0"] == 1.225 and c["c0"] == 340.0
    assert c["ics"] == [(0.0, 200.0, 0.0, 2000.0, 1.0)]
    assert c["observers"] == [(500.0, 2.0, 0.0, 10.0)]
    assert c["sources"] == []
    assert c["precision"] == "fp64"


def test_json_bc_matching_is_positional(pkg, hilltop_dir):
    cfg = json.load(open(os.path.join(GOLDEN, "2d_hilltop.json")))
    cfg["mesh"]["File"] = str(hilltop_dir / "2d_hilltop_fs.msh")
    cfg["mesh"]["BC"]["boundary1"], cfg["mesh"]["BC"]["boundary2"] = cfg["mesh"]["BC"]["boundary2"], cfg["mesh"]["BC"]["boundary1"]
    p = hilltop_dir / "c.json"
    p.write_text(json.dumps(cfg))
    assert pkg.host.load_config(str(p))["bcs"] == []  # names no longer match their positions


def test_conf_config_semantics(pkg, hilltop_dir):
    (hilltop_dir / "sig.csv").write_text("time;value\n0;0\n# comment\n0.5;1.0\n1.0;0.5\n")
    conf = """[Config]
meshFileName = {mesh}
timeStart=0
timeEnd = 0.01
timeStep=1e-3
timeRate=0.005
elementType=Lagrange
timeIntMethod=Runge-Kutta
abs = Absorbing
ref = Reflecting
numThreads=1
v0_x = 1
v0_y = 2
v0_z = 0
rho0 = 1.225
c0 = 340
source2 = dipole, 0,200,0, 10, 2, 5, 0.25, 5
source10 = monopole, 1,2,3, 4, 5, 6, 0.5, 7
source3 = formula, "0.1 * sin(2 * pi * 50 * t)", 0,200,0, 0.1, 0.05
source4 = quadrupole, 0,0,0, 2, 1, 10, 0, 1
source5 = file, "{csv}", 5,6,7, 8
observer1 = 500.0,2.0,0.0,10.0
initialCondtition1 = gaussian, 0, 200, 0, 2000, 1
""".format(mesh=hilltop_dir / "2d_hilltop_fs.msh", csv=hilltop_dir / "sig.csv")
    p = hilltop_dir / "c.conf"
    p.write_text(conf)
    c = pkg.host.load_config(str(p), times=[0.0, 0.25, 0.75, 2.0])
    assert c["num_threads"] == 0  # numThreads = 1 means all cores in the reference
    assert c["bcs"] == [(1, 0), (2, 1)]
    assert c["v0"] == (1.0, 2.0, 0.0)
    kinds = [s["kind"] for s in c["sources"]]
    # lexicographic key order: source10, source2, source3, source4, source5
    assert kinds == [0, 0, 0, 1, 0, 0, 0, 0, 2]
    s10 = c["sources"][0]["params"]
    assert s10 == [1, 2, 3, 4, 5, 6, 0.5, 7]
    d1, d2 = c["sources"][1]["params"], c["sources"][2]["params"]
    assert d1[:4] == [-10, 200, 0, 5] and d2[:4] == [10, 200, 0, 5]
    assert d2[6] == pytest.approx(0.25 + math.pi)
    assert c["sources"][3]["formula"] == "0.1*sin(2*pi*50*t)"  # whitespace removed
    q = [c["sources"][k]["params"] for k in range(4, 8)]
    assert [x[:2] for x in q] == [[-2, 0], [2, 0], [0, -2], [0, 2]]
    assert [x[6] for x in q] == [0, 0, pytest.approx(math.pi), pytest.approx(math.pi)]
    tab = c["sources"][8]["table"]
    assert tab.tolist() == [[0.0, 0.0], [0.5, 1.0], [1.0, 0.5]]
    sv = c["source_values"]
    assert sv[0, 0] == pytest.approx(5 * math.sin(0.5))            # t < duration
    assert sv[3, 0] == pytest.approx(5 * math.sin(2 * math.pi * 6 * 2.0 + 0.5))
    assert sv[0, 3] == pytest.approx(0.0, abs=1e-15)                # formula at t = 0
    assert math.isnan(sv[1, 3])                                    # formula past its duration
    assert math.isnan(sv[3, 4])                                    # quadrupole past its duration
    assert sv[1, 8] == pytest.approx(0.5) and sv[2, 8] == pytest.approx(0.75) and sv[3, 8] == 0.0


def test_missing_files_are_errors(pkg, tmp_path):
    with pytest.raises(RuntimeError, match="not found"):
        pkg.host.load_config(str(tmp_path / "nope.json"))
    (tmp_path / "c.json").write_text(json.dumps({"mesh": {"File": str(tmp_path / "none.msh"), "BC": {"number": 0}}}))
    with pytest.raises(RuntimeError, match="not found"):
        pkg.host.load_config(str(tmp_path / "c.json"))


def test_wav_roundtrip(pkg, tmp_path):
    x = np.sin(np.linspace(0, 20, 1000)).astype(np.float32) * 0.9
    p = str(tmp_path / "a.wav")
    pkg.host.write_wav(p, x, 1000)
    y, rate = pkg.host.read_wav(p)
    assert rate == 1000 and len(y) == 1000
    # int16(x * 32767) / 32767 (truncation toward zero)
    expect = np.trunc(x * np.float32(32767)).astype(np.int16).astype(np.float32) / np.float32(32767)
    np.testing.assert_array_equal(y, expect)


def test_spectra_match_numpy(pkg):
    dt = 1e-3
    t = np.arange(1000) * dt
    p = (0.3 * np.sin(2 * np.pi * 50 * t) + 0.1 * np.cos(2 * np.pi * 120 * t) + 0.05).astype(np.float32)
    fft, psd = pkg.host.spectra(p, dt)
    nb = 512
    x = p[:nb].astype(np.float64)
    x -= x.mean()
    X = np.fft.fft(x)
    periods = (nb - 1) * dt
    assert fft.shape == (nb // 2, 5) and psd.shape == (nb // 2 + 1, 3)
    np.testing.assert_allclose(fft[:, 0], np.arange(nb // 2) / periods)
    np.testing.assert_allclose(fft[:, 1], 2 * np.abs(X[:nb // 2]) / nb, rtol=1e-9, atol=1e-12)
    nf = periods / nb ** 2
    ref = 2 * np.abs(X[:nb // 2 + 1]) ** 2 * nf
    ref[0] /= 2
    ref[-1] /= 2
    np.testing.assert_allclose(psd[:, 1], ref, rtol=1e-9, atol=1e-18)


def test_pvd_replays_schedule(pkg, tmp_path):
    p = str(tmp_path / "r.pvd")
    pkg.host.write_pvd(p, 0.0, 1.0, 1e-3, 0.1)
    lines = [l for l in open(p).read().splitlines() if "DataSet" in l]
    assert len(lines) == 10
    assert lines[1] == '    <DataSet timestep="0.1" part="0" file="results/result100.vtu"/>'
    times, snap = pkg.host.schedule(0.0, 1.0, 1e-3, 0.1)
    assert len(times) == 1000 and np.nonzero(snap)[0].tolist() == list(range(0, 1000, 100))


def test_msh_parallel_parse_round_trip(pkg, tmp_path):
    """A mesh whose node and element sections span many parallel parse tasks
    (65,536 tokens each) reads back exactly as written; a malformed number in
    the bulk sections is reported."""
    m = pkg.meshgen.box(counts=(16, 16, 16), order=3, seed=5)
    path = str(tmp_path / "big.msh")
    pkg.host.write_mesh(path, 3, 3, m["xyz"], m["elem_nodes"], [(g[0], g[1], g[3]) for g in m["groups"]])
    r = pkg.host.load_mesh(path)
    assert len(m["xyz"]) * 3 > 4 * 65536
    np.testing.assert_array_equal(r["xyz"], m["xyz"])
    np.testing.assert_array_equal(r["elem_nodes"], m["elem_nodes"])
    txt = open(path).read()
    i = txt.index("$Nodes")
    j = txt.index("\n", txt.index("\n", txt.index("\n", i) + 1) + 1)  # past the section and first block headers
    bad = txt[:j + 1] + "x" + txt[j + 1:]
    p2 = str(tmp_path / "bad.msh")
    open(p2, "w").write(bad)
    with pytest.raises(RuntimeError, match="malformed"):
        pkg.host.load_mesh(p2)
