"""GB300-native DG solver core for linearized Euler acoustics.

A drop-in for the RK4 LEE hot path of DGFEM-Acoustic: host front end
(host.py, libdgfem_host.so), GPU solver behind a C ABI (gpu.py,
libdgfem_gb300.so), the dgalerkin driver executable, and mesh generators
(meshgen.py), the batched-ensemble workload (ensemble.py) and its learned spectral
surrogate (surrogate.py). Build with build.build() (or __graft_entry__.build()).
"""
import importlib.util as _ilu
import os as _os

_HERE = _os.path.dirname(_os.path.abspath(__file__))


def _load(name):
    spec = _ilu.spec_from_file_location(__name__ + "." + name, _os.path.join(_HERE, name + ".py"))
    mod = _ilu.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


build = _load("build")
host = _load("host")
gpu = _load("gpu")
meshgen = _load("meshgen")
ensemble = _load("ensemble")
surrogate = _load("surrogate")
