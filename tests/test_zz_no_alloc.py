"""hz_horizon_svf_device_static, the entry point that allocates no GPU memory.

It serves callers that cannot call cudaMalloc: their device memory belongs to
another allocator (a framework's caching pool, an application that reserves
the whole GPU), or they cannot afford the device-wide synchronisation that
cudaMalloc/cudaFree imply while sharing the GPU. Its scratch is a fixed
array inside the library. These tests call it through the C ABI and compare
it with hz_horizon_svf_device on two calls in a row (the array keeps the
first call's contents when the second one starts), and check that a domain
above the array's limit is refused with a clear message.
"""
import ctypes as C

import numpy as np
import pytest

from horayzon_extpar_gb300 import _lib, horizon_svf_comp_device, synthetic

pytestmark = pytest.mark.gpu

EXACT_DEG = 1e-9   # horizons: identical lattice values
SVF_TOL = 1e-12


def _static_call(L, t, horizon, skyview, ncell, nvert, args, stream):
    return L.hz_horizon_svf_device_static(
        *(x.data_ptr() for x in t), horizon.data_ptr(), skyview.data_ptr(),
        ncell, nvert, *args, C.c_void_p(stream.cuda_stream))


def test_static_entry_matches_device_entry_two_calls():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    cases = [
        (synthetic.make_domain(edge_km=1.0, box_km=60.0, seed=31), (24, 1, 40000.0, 0.2, 1, 2)),
        (synthetic.make_domain(edge_km=2.0, box_km=50.0, seed=32, kind="fbm_ridged",
                               hmin=200.0, hmax=4800.0, n_features=0),
         (16, 0, 20000.0, 0.5, 3, 1)),
    ]
    for dom, args in cases:
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in dom.inputs()]
        h_ref, s_ref, _ = horizon_svf_comp_device(*t, *args)
        h = torch.full((args[0], dom.ncell), float("nan"), dtype=torch.float64, device=dev)
        s = torch.full((dom.ncell,), float("nan"), dtype=torch.float64, device=dev)
        rc = _static_call(L, t, h, s, dom.ncell, dom.nvertex, args, stream)
        assert rc == _lib.HZ_OK, _lib.last_error()
        torch.cuda.synchronize()
        hn, sn = h.cpu().numpy(), s.cpu().numpy()
        assert np.isfinite(hn).all() and np.isfinite(sn).all()
        assert np.abs(hn - h_ref.cpu().numpy()).max() <= EXACT_DEG
        assert np.abs(sn - s_ref.cpu().numpy()).max() <= SVF_TOL


def test_static_entry_after_a_failed_call():
    """A call that fails part way (a cells_of_vertex index out of range,
    found by the mesh stage on the GPU) returns HZ_ERR_INDEX; the next valid
    call, which starts from what the failed call left in the array, matches
    hz_horizon_svf_device."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    dom = synthetic.make_domain(edge_km=1.5, box_km=60.0, seed=33)
    args = (24, 1, 30000.0, 0.2, 1, 2)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in dom.inputs()]
    bad = t[5].clone()
    bad[2, dom.nvertex // 2] = dom.ncell + 7
    h = torch.full((args[0], dom.ncell), float("nan"), dtype=torch.float64, device=dev)
    s = torch.full((dom.ncell,), float("nan"), dtype=torch.float64, device=dev)
    rc = _static_call(L, t[:5] + [bad], h, s, dom.ncell, dom.nvertex, args, stream)
    assert rc == _lib.HZ_ERR_INDEX
    assert "out of range" in _lib.last_error()
    h_ref, s_ref, _ = horizon_svf_comp_device(*t, *args)
    rc = _static_call(L, t, h, s, dom.ncell, dom.nvertex, args, stream)
    assert rc == _lib.HZ_OK, _lib.last_error()
    torch.cuda.synchronize()
    assert np.abs(h.cpu().numpy() - h_ref.cpu().numpy()).max() <= EXACT_DEG
    assert np.abs(s.cpu().numpy() - s_ref.cpu().numpy()).max() <= SVF_TOL


def test_static_entry_accepts_the_documented_domain_size():
    """A domain of about 90,000 cells (grid_type 1, one vertex per two
    cells) fits the array, and its results match hz_horizon_svf_device."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda:0")
    stream = torch.cuda.current_stream(dev)
    dom = synthetic.make_domain(edge_km=1.0, box_km=200.0, seed=34)
    assert 85_000 <= dom.ncell <= 100_000, dom.ncell
    assert dom.nvertex <= dom.ncell // 2 + dom.ncell // 50
    args = (24, 1, 40000.0, 0.2, 1, 2)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in dom.inputs()]
    h = torch.empty((args[0], dom.ncell), dtype=torch.float64, device=dev)
    s = torch.empty(dom.ncell, dtype=torch.float64, device=dev)
    rc = _static_call(L, t, h, s, dom.ncell, dom.nvertex, args, stream)
    assert rc == _lib.HZ_OK, _lib.last_error()
    h_ref, s_ref, _ = horizon_svf_comp_device(*t, *args)
    torch.cuda.synchronize()
    assert np.abs(h.cpu().numpy() - h_ref.cpu().numpy()).max() <= EXACT_DEG
    assert np.abs(s.cpu().numpy() - s_ref.cpu().numpy()).max() <= SVF_TOL


def test_static_entry_refuses_domains_above_its_limit():
    torch = pytest.importorskip("torch")
    L = _lib.load()
    dev = torch.device("cuda:0")
    ncell, nvert = 400_000, 200_000
    t = [torch.zeros(ncell, dtype=torch.float64, device=dev) for _ in range(3)]
    t += [torch.zeros(nvert, dtype=torch.float64, device=dev) for _ in range(2)]
    t.append(torch.full((6, nvert), -2, dtype=torch.int32, device=dev))
    h = torch.zeros((24, ncell), dtype=torch.float64, device=dev)
    s = torch.zeros(ncell, dtype=torch.float64, device=dev)
    rc = _static_call(L, t, h, s, ncell, nvert, (24, 1, 40000.0, 0.2, 1, 2),
                      torch.cuda.current_stream(dev))
    assert rc == _lib.HZ_ERR_VALUE
    assert "static array" in _lib.last_error()
