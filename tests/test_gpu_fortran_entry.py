"""The Fortran-style entry point with the stdout-buffer contract of the
reference's dormant Fortran variant (mo_lradtopo_horayzon.cpp:561-574,
778-784): progress text copied into a caller buffer, truncated to its
capacity, byte count returned through buffer_len."""
import ctypes as C

import numpy as np
import pytest

from horayzon_extpar_gb300 import _lib, horizon_svf_comp_py, synthetic

pytestmark = pytest.mark.gpu

ARGS = (24, 1, 40000.0, 0.2, 1, 2)
D, I32 = C.POINTER(C.c_double), C.POINTER(C.c_int32)


def _call(dom, capacity, cov=None):
    L = _lib.load()
    inp = [np.ascontiguousarray(a) for a in dom.inputs()]
    if cov is not None:
        inp[5] = cov
    h = np.empty((ARGS[0], dom.ncell))
    s = np.empty(dom.ncell)
    buf = C.create_string_buffer(max(capacity, 1))
    n = C.c_int(capacity)
    L.horizon_svf_comp_buffer(*(a.ctypes.data_as(D) for a in inp[:5]), inp[5].ctypes.data_as(I32),
                              h.ctypes.data_as(D), s.ctypes.data_as(D), dom.ncell, dom.nvertex,
                              *ARGS, buf, C.byref(n))
    return h, s, buf.raw[:n.value].decode(), n.value


def test_buffer_entry_returns_results_and_progress_text():
    dom = synthetic.make_domain(edge_km=2.5, box_km=60.0, seed=5)
    h, s, text, n = _call(dom, 4096)
    h0, s0, st = horizon_svf_comp_py(*dom.inputs(), *ARGS, return_stats=True)
    np.testing.assert_array_equal(h, h0)
    np.testing.assert_array_equal(s, s0)
    assert n == len(text) < 4096
    lines = text.splitlines()
    assert lines[0] == lines[2] == lines[-1] == "-" * 79
    assert "Number of triangles in mesh: %d" % st["n_tri"] in lines
    assert "Number of rays shot: %d" % st["num_rays"] in lines
    assert "Sky View Factor computation algorithm: geometric scaled with sin(horizon)**2" in lines
    assert any(x.startswith("Average number of rays per cell and azimuth sector: ")
               for x in lines)


def test_buffer_entry_truncates_to_capacity():
    dom = synthetic.make_domain(edge_km=2.5, box_km=60.0, seed=5)
    _, _, full, n_full = _call(dom, 4096)
    _, _, part, n = _call(dom, 50)
    assert n == 50 and part == full[:50]
    _, _, none, n0 = _call(dom, 0)
    assert n0 == 0 and none == ""


def test_buffer_entry_reports_errors_in_text():
    dom = synthetic.make_domain(edge_km=2.5, box_km=60.0, seed=5)
    cov = np.ascontiguousarray(dom.inputs()[5]).copy()
    cov[0, 0] = dom.ncell + 7  # index out of range
    h, s, text, n = _call(dom, 4096, cov=cov)
    assert "horizon_svf_comp: " in text and "out of range" in text
    assert np.isnan(h).all() and np.isnan(s).all()


def test_verbose_prints_the_same_lines(capfd):
    dom = synthetic.make_domain(edge_km=2.5, box_km=60.0, seed=5)
    _, _, text, _ = _call(dom, 4096)
    horizon_svf_comp_py(*dom.inputs(), *ARGS, verbose=True)
    out = capfd.readouterr().out
    strip = lambda t: [x for x in t.splitlines() if not x.endswith(" s")]  # timings differ
    assert strip(out) == strip(text)
