"""Pinned host buffers (dg_host_alloc / dg_host_free): a state round trip
through page-locked arrays equals the one through ordinary numpy arrays."""
import numpy as np
import pytest

from conftest import smooth_state
from test_gpu_parity import _mesh, _phys

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_pinned_state_round_trip(pkg, prec):
    g = pkg.gpu
    mesh = _mesh(pkg, 3, 2)
    S = g.Solver(mesh, precision=g.DG_FP64 if prec == "fp64" else g.DG_FP32, **_phys(3))
    u = smooth_state(mesh, seed=3)
    pin = g.pinned_empty(u.shape)
    pin[:] = u
    S.set_state(pin)
    S.snapshot()
    S.run(3, 1e-4)
    out = g.pinned_empty(u.shape)
    assert S.get_state(out=out) is out
    np.testing.assert_array_equal(out, S.get_state())
    with pytest.raises(ValueError):
        S.get_state(out=np.zeros(5))
    S.close()
