"""Shared fixtures: package modules, the oracle binding and small meshes."""
import importlib
import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("dgfem-acoustic_gb300")


@pytest.fixture(scope="session")
def oracle():
    return _load("refcpu", os.path.join(ROOT, "oracle", "refcpu.py"))


def smooth_state(mesh, seed=0, dim=None):
    """Smooth random-ish state [4][E*Np] on the mesh's DG nodes (vz = 0 in 2-D)."""
    rng = np.random.default_rng(seed)
    en = mesh["elem_nodes"]
    x = mesh["xyz"][en.reshape(-1)]
    dim = dim or mesh["dim"]
    u = np.zeros((4, en.size))
    for q in range(dim + 1):
        k = rng.uniform(0.5, 2.0, 3)
        ph = rng.uniform(0, 2 * np.pi, 3)
        u[q] = rng.uniform(0.5, 1.5) * (np.sin(k[0] * x[:, 0] + ph[0]) * np.cos(k[1] * x[:, 1] + ph[1])
                                        + 0.3 * np.sin(k[2] * x[:, 2] + ph[2]))
    return u


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
