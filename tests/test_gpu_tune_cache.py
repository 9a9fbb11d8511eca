"""The autotuner's result cache: a second context of the same GPU model,
element type, precision and mesh size class takes the first one's kernel
variant without timing; an explicit re-tune times again; with
DGFEM_TUNE_CACHE set, results persist in a file that later processes read
(a planted entry there is obeyed)."""
import json
import os
import subprocess
import sys

import pytest

from test_gpu_parity import _mesh, _phys

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import importlib, json, os, sys
sys.path.insert(0, os.getcwd())
sys.path.insert(0, os.path.join(os.getcwd(), "tests"))
pkg = importlib.import_module("dgfem-acoustic_gb300")
from test_gpu_parity import _mesh, _phys
S = pkg.gpu.Solver(_mesh(pkg, 2, 3), precision=pkg.gpu.DG_FP32, **_phys(2))
print(json.dumps({"variant": S.info()["kernel_variant"], "stats": pkg.gpu.tune_cache_stats()}))
S.close()
"""


def test_second_context_takes_cached_variant(pkg, monkeypatch):
    # the in-process cache only: no cache file from the environment
    monkeypatch.delenv("DGFEM_TUNE_CACHE", raising=False)
    g = pkg.gpu
    g.tune_cache_clear()
    mesh = _mesh(pkg, 2, 3)
    A = g.Solver(mesh, precision=g.DG_FP32, **_phys(2))
    h0, m0, n0 = g.tune_cache_stats()
    assert (h0, m0) == (0, 1) and n0 == 1
    B = g.Solver(mesh, precision=g.DG_FP32, **_phys(2))
    h1, m1, n1 = g.tune_cache_stats()
    assert (h1, m1, n1) == (1, 1, 1)
    assert B.info()["kernel_variant"] == A.info()["kernel_variant"]
    # another precision is another key
    C64 = g.Solver(mesh, precision=g.DG_FP64, **_phys(2))
    assert g.tune_cache_stats() == (1, 2, 2)
    # an explicit re-tune times the variants again (no lookup) and stores
    B.tune(-2)
    assert g.tune_cache_stats()[:2] == (1, 2)
    # -3 looks up
    B.tune(-3)
    assert g.tune_cache_stats()[:2] == (2, 2)
    for s in (A, B, C64):
        s.close()


def _child(env):
    r = subprocess.run([sys.executable, "-c", CHILD], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])


def test_cache_file_persists_across_processes(tmp_path):
    path = tmp_path / "tune.txt"
    env = dict(os.environ, DGFEM_TUNE_CACHE=str(path))
    env.pop("DGFEM_STAGE_VARIANT", None)
    first = _child(env)
    assert first["stats"][:2] == [0, 1]
    lines = path.read_text().splitlines()
    assert len(lines) == 1
    key, v = lines[0].rsplit("\t", 1)
    assert int(v) == first["variant"]
    assert "|d2|p3|fp32|" in key
    second = _child(env)
    assert second["stats"][:2] == [1, 0] and second["variant"] == first["variant"]
    # a later line for the same key wins: plant the baseline kernel
    with open(path, "a") as f:
        f.write(key + "\t-1\n")
    third = _child(env)
    assert third["stats"][:2] == [1, 0] and third["variant"] == -1
