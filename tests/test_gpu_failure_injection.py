"""Error path of the host entry points under an injected workspace-allocation
failure (host side; no GPU fault): the status and message reach the caller,
the void drop-in fills its outputs with NaN, and the next call succeeds."""
import ctypes as C

import numpy as np
import pytest

from horayzon_extpar_gb300 import _lib, horizon_svf_comp_py, synthetic

pytestmark = pytest.mark.gpu

ARGS = (24, 1, 40000.0, 0.2, 1, 2)


def test_injected_allocation_failure_is_reported_and_recovers(monkeypatch):
    d = synthetic.make_domain(edge_km=2.5, box_km=60.0, seed=41)
    h0, s0 = horizon_svf_comp_py(*d.inputs(), *ARGS, device=0)
    L = _lib.load()
    assert L.hz_release_workspace(0) == 0  # the next call must grow the workspace
    monkeypatch.setenv("HZ_INJECT_ALLOC_FAILURE", "1")
    with pytest.raises(_lib.HorizonError) as e:
        horizon_svf_comp_py(*d.inputs(), *ARGS, device=0)
    assert e.value.status == _lib.HZ_ERR_CUDA and "injected" in str(e.value)
    # The void entry point (mo_lradtopo_horayzon.h:4-11) reports through NaN.
    inp = [np.ascontiguousarray(a) for a in d.inputs()]
    h = np.zeros((ARGS[0], d.ncell))
    s = np.zeros(d.ncell)
    D, I32 = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    L.horizon_svf_comp(*(a.ctypes.data_as(D) for a in inp[:5]), inp[5].ctypes.data_as(I32),
                       h.ctypes.data_as(D), s.ctypes.data_as(D), d.ncell, d.nvertex, *ARGS)
    assert np.isnan(h).all() and np.isnan(s).all()
    monkeypatch.delenv("HZ_INJECT_ALLOC_FAILURE")
    h1, s1 = horizon_svf_comp_py(*d.inputs(), *ARGS, device=0)
    np.testing.assert_array_equal(h1, h0)
    np.testing.assert_array_equal(s1, s0)
