"""The shared libraries load and export every entry point their headers
declare (no GPU calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dgh?_[a-z_0-9]+)\s*\(", text)))


@pytest.mark.parametrize("header,lib", [("dgfem_gb300.h", "libdgfem_gb300.so"), ("dgfem_host.h", "libdgfem_host.so")])
def test_library_exports_all_declared_symbols(header, lib):
    L = ctypes.CDLL(os.path.join(ROOT, "dgfem-acoustic_gb300", "_build", lib))
    names = _declared(header)
    assert len(names) > 10
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_lists_every_gpu_symbol(pkg):
    assert sorted(pkg.gpu.SYMBOLS) == _declared("dgfem_gb300.h")


def test_oracle_library_loads(oracle):
    L = oracle.lib()
    for n in ("refcpu_run", "refcpu_stage", "refcpu_faces", "refcpu_initial_state", "refcpu_count_steps"):
        assert hasattr(L, n)
