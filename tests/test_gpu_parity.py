"""GPU path (through the C ABI) against the reference's golden outputs and
the CPU oracle. Bar: identical horizons on >= 99.9 % of (cell, azimuth) and
|dSVF| <= 1e-3; in practice the hit decisions are bit-identical, so the
tests also require exact agreement of horizons (1e-9 deg) on >= 99.9 %."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_cases, load_golden
from horayzon_extpar_gb300 import _lib, build_mesh, horizon_svf_comp_py, mesh_enu32
from horayzon_extpar_gb300 import synthetic
from oracle import api as oracle

pytestmark = pytest.mark.gpu

HORIZON_TOL_DEG = 0.25   # search accuracy of the bracketing method (cpp:577)
SVF_TOL = 1e-3
EXACT_DEG = 1e-9


def assert_parity(h, s, h_ref, s_ref, min_exact=0.999):
    d = np.abs(h - h_ref)
    assert np.mean(d <= HORIZON_TOL_DEG) >= 0.999, "horizon parity %.6f" % np.mean(
        d <= HORIZON_TOL_DEG)
    assert np.mean(d <= EXACT_DEG) >= min_exact, "exact fraction %.6f" % np.mean(
        d <= EXACT_DEG)
    # Where the searches agree the degrees agree bit for bit (the same sums,
    # and the epilogue's division-free rad -> deg is the IEEE quotient).
    same = d <= EXACT_DEG
    np.testing.assert_array_equal(h[same], h_ref[same])
    assert np.abs(s - s_ref).max() <= SVF_TOL
    # Cells whose horizons all agree have the same SVF to rounding.
    cells = same.all(axis=0)
    np.testing.assert_allclose(s[cells], s_ref[cells], rtol=0, atol=1e-12)


@pytest.fixture(scope="module", autouse=True)
def library():
    return _lib.load()


@pytest.mark.parametrize("name", golden_cases())
def test_gpu_matches_reference_golden(name):
    g = load_golden(name)
    h, s = horizon_svf_comp_py(*g["inputs"], *g["args"])
    assert h.shape == g["horizon"].shape and h.dtype == np.float64
    assert h.flags["C_CONTIGUOUS"] and s.shape == g["skyview"].shape
    assert_parity(h, s, g["horizon"], g["skyview"])
    np.testing.assert_allclose(s, g["skyview"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", golden_cases())
def test_gpu_mesh_matches_reference_mesh(name):
    g = load_golden(name)
    mlon, mlat, mh, vot = build_mesh(*g["inputs"], g["args"][1])
    np.testing.assert_array_equal(vot, g["mesh_vot"])
    np.testing.assert_array_equal(mlon, g["mesh_lon"])
    np.testing.assert_array_equal(mlat, g["mesh_lat"])
    np.testing.assert_array_equal(mh, g["mesh_h"])


@pytest.mark.parametrize("grid_type", [0, 1])
def test_gpu_mesh_order_near_ties(small_domain, grid_type):
    """The mesh kernel orders the cells around a vertex by FP32 angles and
    falls back to FP64 angles near ties: cells due north or south of a
    vertex (angle 0 / pi, at the wrap), cells on one line through the vertex
    (equal angles, stable order) and cells 1e-12 rad off that line give the
    oracle's triangles."""
    d = small_domain
    clon, clat = d.clon.copy(), d.clat.copy()
    cov = d.cells_of_vertex
    full = np.where((cov >= 0).all(0))[0]
    rng = np.random.default_rng(5)
    picks = rng.choice(full, 30, replace=False)
    for v in picks[:10]:
        clon[cov[0, v]] = d.vlon[v]
    for k, v in enumerate(picks[10:]):
        c1, c2 = cov[1, v], cov[3, v]
        clon[c2] = d.vlon[v] + 0.5 * (clon[c1] - d.vlon[v]) + (1e-12 if k % 2 else 0.0)
        clat[c2] = d.vlat[v] + 0.5 * (clat[c1] - d.vlat[v])
    inputs = (clon, clat, d.hsurf, d.vlon, d.vlat, cov)
    enu, vot = mesh_enu32(*inputs, grid_type)
    _, _, vot_o = oracle.mesh_enu(*inputs, grid_type)
    np.testing.assert_array_equal(vot, vot_o)


@pytest.mark.parametrize("grid_type", [0, 1])
def test_gpu_enu32_matches_oracle(small_domain, grid_type):
    enu, vot = mesh_enu32(*small_domain.inputs(), grid_type)
    e64, e32, vot_o = oracle.mesh_enu(*small_domain.inputs(), grid_type)
    np.testing.assert_array_equal(vot, vot_o)
    assert enu.shape == e32.shape
    assert np.mean(enu == e32) >= 0.9999
    ulp = np.spacing(np.abs(e32).astype(np.float32))
    assert (np.abs(enu - e32) <= ulp).all()


CONFIGS = [
    # (domain kwargs, (num_hori, grid_type, dist_search, ray_org_elev, refine, svf))
    (dict(edge_km=2.5, box_km=70.0, seed=21), (24, 1, 40000.0, 0.2, 1, 2)),
    (dict(edge_km=2.5, box_km=70.0, seed=21), (24, 0, 40000.0, 0.2, 1, 1)),
    (dict(edge_km=1.0, box_km=30.0, seed=22, kind="fbm_ridged", hmin=200.0, hmax=4800.0,
          hurst=0.7, n_features=0), (36, 1, 15000.0, 0.2, 3, 0)),
    (dict(edge_km=0.5, box_km=12.0, seed=23, kind="eroded", hmin=500.0, hmax=4200.0,
          n_features=0), (8, 1, 100000.0, 1.5, 7, 2)),
    (dict(edge_km=3.0, box_km=90.0, seed=24, lat0_deg=-33.0, lon0_deg=150.0,
          face_rotation_deg=40.0), (24, 1, 500000.0, 0.2, 1, 2)),
]


@pytest.mark.parametrize("dkw,args", CONFIGS)
def test_gpu_matches_oracle(dkw, args):
    d = synthetic.make_domain(**dkw)
    h, s, st = horizon_svf_comp_py(*d.inputs(), *args, return_stats=True)
    ho, so, sto = oracle.horizon_svf(*d.inputs(), *args)
    assert_parity(h, s, ho, so)
    # The SVF terms of lattice horizons come from a table of sin(j * 0.25 deg):
    # the same sums to rounding.
    np.testing.assert_allclose(s, so, rtol=0, atol=1e-12)
    assert st["n_tri"] == sto["n_tri"] and st["n_mesh_vert"] == sto["n_mesh_vert"]
    # identical hit decisions imply identical ray counts
    assert abs(st["num_rays"] - sto["num_rays"]) <= 0.001 * sto["num_rays"]


def test_gpu_shuffled_slots(small_domain):
    """-2 entries anywhere in a vertex's column (slot mapping, not position)."""
    d = small_domain
    rng = np.random.default_rng(3)
    cov = d.cells_of_vertex.copy()
    for v in range(cov.shape[1]):
        cov[:, v] = cov[rng.permutation(6), v]
    inputs = (d.clon, d.clat, d.hsurf, d.vlon, d.vlat, cov)
    for grid_type in (0, 1):
        args = (24, grid_type, 30000.0, 0.2, 1, 2)
        h, s = horizon_svf_comp_py(*inputs, *args)
        ho, so, _ = oracle.horizon_svf(*inputs, *args)
        assert_parity(h, s, ho, so)


def test_gpu_deterministic(small_domain):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    a = horizon_svf_comp_py(*small_domain.inputs(), *args)
    b = horizon_svf_comp_py(*small_domain.inputs(), *args)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_gpu_count_work(small_domain):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h, s, st = horizon_svf_comp_py(*small_domain.inputs(), *args, count_work=True,
                                   return_stats=True)
    assert st["node_visits"] > st["num_rays"] > 0
    assert st["tri_tests"] > 0


def test_gpu_device_api_equals_host_api(small_domain):
    torch = pytest.importorskip("torch")
    from horayzon_extpar_gb300 import horizon_svf_comp_device
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h, s = horizon_svf_comp_py(*small_domain.inputs(), *args)
    dev = torch.device("cuda:0")
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in small_domain.inputs()]
    hd, sd, st = horizon_svf_comp_device(*t, *args)
    np.testing.assert_array_equal(hd.cpu().numpy(), h)
    np.testing.assert_array_equal(sd.cpu().numpy(), s)


def test_gpu_tiny_and_empty_meshes():
    d = synthetic.make_domain(edge_km=2.5, box_km=6.0, seed=2)
    for grid_type in (0, 1):
        for keep in (1, 2, d.nvertex):
            cov = d.cells_of_vertex.copy()
            cov[:, keep:] = -2
            inputs = (d.clon, d.clat, d.hsurf, d.vlon, d.vlat, cov)
            args = (24, grid_type, 40000.0, 0.2, 1, 2)
            h, s = horizon_svf_comp_py(*inputs, *args)
            ho, so, st = oracle.horizon_svf(*inputs, *args)
            np.testing.assert_array_equal(h, ho)
            np.testing.assert_allclose(s, so, atol=1e-12)
    # no triangles at all: every ray misses, horizon 0, SVF 1
    cov = np.full_like(d.cells_of_vertex, -2)
    h, s = horizon_svf_comp_py(d.clon, d.clat, d.hsurf, d.vlon, d.vlat, cov,
                               24, 1, 40000.0, 0.2, 1, 2)
    assert (h == 0).all() and (s == 1).all()


def test_gpu_bad_index_status():
    L = _lib.load()
    d = synthetic.make_domain(edge_km=2.5, box_km=20.0, seed=1)
    cov = d.cells_of_vertex.copy()
    cov[2, 5] = d.ncell + 7
    h = np.empty((24, d.ncell))
    s = np.empty(d.ncell)
    D = C.POINTER(C.c_double)
    rc = L.hz_horizon_svf(d.clon.ctypes.data_as(D), d.clat.ctypes.data_as(D),
                          d.hsurf.ctypes.data_as(D), d.vlon.ctypes.data_as(D),
                          d.vlat.ctypes.data_as(D), cov.ctypes.data_as(C.POINTER(C.c_int32)),
                          h.ctypes.data_as(D), s.ctypes.data_as(D), d.ncell, d.nvertex, 24, 1,
                          40000.0, 0.2, 1, 2, None, None)
    assert rc == _lib.HZ_ERR_INDEX
    assert "out of range" in _lib.last_error()
    # the library stays usable afterwards
    h2, s2 = horizon_svf_comp_py(*d.inputs(), 24, 1, 40000.0, 0.2, 1, 2)
    assert np.isfinite(h2).all()


def test_gpu_dropin_c_symbol(small_domain):
    """horizon_svf_comp: the reference's own signature, C linkage."""
    L = _lib.load()
    d = small_domain
    h = np.empty((24, d.ncell))
    s = np.empty(d.ncell)
    D = C.POINTER(C.c_double)
    L.horizon_svf_comp(d.clon.ctypes.data_as(D), d.clat.ctypes.data_as(D),
                       d.hsurf.ctypes.data_as(D), d.vlon.ctypes.data_as(D),
                       d.vlat.ctypes.data_as(D),
                       d.cells_of_vertex.ctypes.data_as(C.POINTER(C.c_int32)),
                       h.ctypes.data_as(D), s.ctypes.data_as(D), d.ncell, d.nvertex, 24, 1,
                       40000.0, 0.2, 1, 2)
    ho, so = horizon_svf_comp_py(*d.inputs(), 24, 1, 40000.0, 0.2, 1, 2)
    np.testing.assert_array_equal(h, ho)
    np.testing.assert_array_equal(s, so)


@pytest.mark.parametrize("kernel,advance_min,leaf_min",
                         [(0, 1, 1), (0, 4, 32), (0, 16, 8), (0, 32, 16), (0, 0, 0),
                          (2, 1, 32), (2, 24, 4), (2, 0, 0)])
def test_gpu_persistent_equals_per_cell(small_domain, kernel, advance_min, leaf_min):
    """The persistent searches (closed-form lattice directions; any leaf
    order) cast the same rays as the per-cell search (the reference's
    incremental rotations)."""
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h1, s1, st1 = horizon_svf_comp_py(*small_domain.inputs(), *args, kernel=1,
                                      count_work=True, return_stats=True)
    h2, s2, st2 = horizon_svf_comp_py(*small_domain.inputs(), *args, kernel=kernel,
                                      advance_min=advance_min, leaf_min=leaf_min,
                                      count_work=True, return_stats=True)
    np.testing.assert_array_equal(h1, h2)
    # SVF: tabulated sin of the lattice angle vs sin of the accumulated angle
    np.testing.assert_allclose(s1, s2, rtol=0, atol=1e-12)
    assert st1["num_rays"] == st2["num_rays"]
    assert st1["tri_tests"] > 0 and st2["tri_tests"] > 0


@pytest.mark.parametrize("kernel", [0, 1])
def test_gpu_cell_range(small_domain, kernel):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h, s = horizon_svf_comp_py(*small_domain.inputs(), *args, kernel=kernel)
    b, e = 100, 700
    hr, sr = horizon_svf_comp_py(*small_domain.inputs(), *args, kernel=kernel, cells=(b, e))
    np.testing.assert_array_equal(hr[:, b:e], h[:, b:e])
    np.testing.assert_array_equal(sr[b:e], s[b:e])
    assert np.isnan(sr[:b]).all() and np.isnan(sr[e:]).all()


def test_gpu_batch_equals_single_calls():
    """One batch call (one persistent search over all domains) gives each
    domain the same result as its own call."""
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    batch = synthetic.make_batch(n_domains=5, seed=7, min_cells=300, max_cells=4000)
    batch[1] = (batch[1][0], (24, 0, 15000.0, 0.5, 3, 1))
    batch[3] = (batch[3][0], (8, 1, 30000.0, 0.2, 2, 0))
    outs, st = horizon_svf_comp_batch([(d.inputs(), a) for d, a in batch], return_stats=True)
    assert len(st["latency_ms"]) == 5 and all(x > 0 for x in st["latency_ms"])
    rays = 0
    for (d, a), (h, s) in zip(batch, outs):
        h1, s1, st1 = horizon_svf_comp_py(*d.inputs(), *a, return_stats=True)
        np.testing.assert_array_equal(h, h1)
        np.testing.assert_array_equal(s, s1)
        rays += st1["num_rays"]
    assert st["num_rays"] == rays


def test_gpu_batch_takes_small_domains_first():
    """The batch queues its domains by ascending work (cells x azimuths): a
    domain of more cells than the GPU has resident lanes, given first,
    completes after a small one given last (whose cells all start in the
    first wave), and every domain still gets its own call's result."""
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch
    big = synthetic.make_domain(edge_km=1.0, box_km=500.0, seed=41)
    small = synthetic.make_domain(edge_km=1.0, box_km=25.0, seed=43)
    assert big.ncell > 250_000
    # A domain completes with its slowest cell, and a cell at a border that
    # looks out over the void walks down towards -85 deg and, at its next
    # azimuth, back up, one ray per step: the early floor (-0.25 deg) ends
    # those walks at the clip. 4 azimuths: a small-domain cell is a few rays
    # (a cell of 24 azimuths takes several ms of a loaded GPU, a good part of
    # the big domain's 3.5 waves of cells).
    calls = [(big, (24, 1, 30000.0, 0.2, 1, 2)), (small, (4, 1, 3000.0, 0.2, 1, 2))]
    floor = -0.25
    outs, st = horizon_svf_comp_batch([(d.inputs(), a) for d, a in calls], return_stats=True,
                                      elev_floor_deg=floor)
    lat = st["latency_ms"]
    assert lat[1] < 0.5 * lat[0], lat
    for (d, args), (h, s) in zip(calls, outs):
        h1, s1 = horizon_svf_comp_py(*d.inputs(), *args, elev_floor_deg=floor)
        np.testing.assert_array_equal(h, h1)
        np.testing.assert_array_equal(s, s1)


@pytest.mark.parametrize("kernel,leaf_size", [(0, 1), (0, 2), (0, 8), (2, 3), (1, 8)])
def test_gpu_leaf_size_keeps_results(small_domain, kernel, leaf_size):
    """Triangles per BVH leaf change the tree, not the rays or hit decisions."""
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h0, s0, st0 = horizon_svf_comp_py(*small_domain.inputs(), *args, return_stats=True)
    h1, s1, st1 = horizon_svf_comp_py(*small_domain.inputs(), *args, kernel=kernel,
                                      leaf_size=leaf_size, return_stats=True)
    np.testing.assert_array_equal(h0, h1)
    np.testing.assert_allclose(s0, s1, rtol=0, atol=1e-12)
    assert st0["num_rays"] == st1["num_rays"]


@pytest.mark.parametrize("kernel,leaf_size,precision", [(0, 0, 0), (2, 0, 0), (0, 4, 1),
                                                       (0, 1, 0)])
def test_gpu_treelets_keep_results(small_domain, kernel, leaf_size, precision):
    """Treelet restructuring changes the tree's topology and boxes (every box
    still the union of the padded leaf boxes), not the rays or hit decisions:
    same horizons, SVF and ray counts as the plain LBVH, on both trees."""
    args = (24, 1, 40000.0, 0.2, 1, 2)
    kw = dict(kernel=kernel, leaf_size=leaf_size, precision=precision, return_stats=True,
              count_work=True)
    h0, s0, st0 = horizon_svf_comp_py(*small_domain.inputs(), *args, **kw)
    h1, s1, st1 = horizon_svf_comp_py(*small_domain.inputs(), *args, bvh_treelets=True, **kw)
    print("node visits per ray: %.2f plain, %.2f treelets" % (
        st0["node_visits"] / st0["num_rays"], st1["node_visits"] / st1["num_rays"]))
    np.testing.assert_array_equal(h0, h1)
    np.testing.assert_allclose(s0, s1, rtol=0, atol=1e-12)
    assert st0["num_rays"] == st1["num_rays"]


@pytest.mark.parametrize("name", ["g1_n24_r1_svf2", "g0_n24_r1_svf0"])
def test_gpu_treelets_match_reference_golden(name):
    g = load_golden(name)
    h, s = horizon_svf_comp_py(*g["inputs"], *g["args"], bvh_treelets=True)
    assert_parity(h, s, g["horizon"], g["skyview"])


def test_gpu_autotune_picks_a_grid_setting(small_domain, tmp_path, monkeypatch):
    torch = pytest.importorskip("torch")
    from horayzon_extpar_gb300 import autotune, horizon_svf_comp_device
    monkeypatch.setenv("HZ_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    args = (24, 1, 40000.0, 0.2, 1, 2)
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in small_domain.inputs()]
    grid = {"leaf_size": (4, 2), "advance_min": (16, 8), "leaf_min": (12, 6),
            "queue_chunk": (32, 1), "kernel": (0, 2)}
    res = autotune.tune(t, args, sample_cells=500, reps=1, rounds=1, grid=grid)
    assert not res["cached"] and res["trials"] >= 5
    for k, v in grid.items():
        assert res[k] in v
    again = autotune.tune(t, args, grid=grid)
    assert again["cached"] and autotune.knobs(again) == autotune.knobs(res)
    h0, s0, _ = horizon_svf_comp_device(*t, *args)
    h1, s1, _ = horizon_svf_comp_device(*t, *args, **autotune.knobs(res))
    assert torch.equal(h0, h1)


@pytest.mark.parametrize("queue_chunk", [1, 7, 64])
def test_gpu_queue_chunk_keeps_results(small_domain, queue_chunk):
    """How many cells a warp takes from the work queue at a time changes the
    schedule only."""
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h0, s0, st0 = horizon_svf_comp_py(*small_domain.inputs(), *args, return_stats=True)
    h1, s1, st1 = horizon_svf_comp_py(*small_domain.inputs(), *args, queue_chunk=queue_chunk,
                                      return_stats=True)
    np.testing.assert_array_equal(h0, h1)
    np.testing.assert_array_equal(s0, s1)
    assert st0["num_rays"] == st1["num_rays"]



def test_gpu_graph_replay_matches_direct_launch(small_domain):
    """The captured CUDA graph (replayed, updated in place for a call of the
    same shape, re-instantiated for another shape) gives the same results as
    launching every kernel directly, on the caller's stream of any kind."""
    torch = pytest.importorskip("torch")
    from horayzon_extpar_gb300.horizon_svf import horizon_svf_comp_batch, horizon_svf_comp_device
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h0, s0, st0 = horizon_svf_comp_py(*small_domain.inputs(), *args, direct_launch=True,
                                      return_stats=True)
    for _ in range(2):  # first call instantiates, the second updates
        h1, s1, st1 = horizon_svf_comp_py(*small_domain.inputs(), *args, return_stats=True)
        np.testing.assert_array_equal(h0, h1)
        np.testing.assert_array_equal(s0, s1)
        assert st0["num_rays"] == st1["num_rays"]
    # Another shape (refinement), then back.
    args2 = (24, 1, 40000.0, 0.2, 3, 1)
    h2, s2 = horizon_svf_comp_py(*small_domain.inputs(), *args2, direct_launch=True)
    h3, s3 = horizon_svf_comp_py(*small_domain.inputs(), *args2)
    np.testing.assert_array_equal(h2, h3)
    np.testing.assert_array_equal(s2, s3)
    # Device entry on torch's default stream and on a side stream.
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in small_domain.inputs()]
    hd, sd, _ = horizon_svf_comp_device(*t, *args)
    np.testing.assert_array_equal(hd.cpu().numpy(), h0)
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        he, se, _ = horizon_svf_comp_device(*t, *args, stream=side)
    side.synchronize()
    np.testing.assert_array_equal(he.cpu().numpy(), h0)
    np.testing.assert_array_equal(se.cpu().numpy(), s0)
    # Batch of two domains.
    other = synthetic.make_domain(edge_km=3.0, box_km=50.0, seed=11)
    doms = [(small_domain.inputs(), args), (other.inputs(), args2)]
    ref = horizon_svf_comp_batch(doms, direct_launch=True)
    got = horizon_svf_comp_batch(doms)
    for (ha, sa), (hb, sb) in zip(ref, got):
        np.testing.assert_array_equal(ha, hb)
        np.testing.assert_array_equal(sa, sb)


def test_gpu_phase_times_without_graph():
    """Phase times of calls launched without the graph (direct launch, the
    learned start) bracket their work like those of captured calls: the
    events are recorded on the stream that carries the work."""
    torch = pytest.importorskip("torch")
    from horayzon_extpar_gb300 import horizon_svf_comp_device, learned
    d = synthetic.make_config("c3", seed=0, box_km=120.0)
    t = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in d.inputs()]
    args = (24, 1, 40000.0, 0.2, 1, 2)
    for _ in range(2):
        _, _, cap = horizon_svf_comp_device(*t, *args)
        _, _, direct = horizon_svf_comp_device(*t, *args, direct_launch=True)
        _, _, lrn = horizon_svf_comp_device(*t, *args, mlp_params=learned.init_params(0))
    assert cap["ms_trace"] > 2.0
    for st in (direct, lrn):
        assert 0.7 * cap["ms_trace"] < st["ms_trace"] < 3.0 * cap["ms_trace"]
        assert 0.5 * cap["ms_bvh"] < st["ms_bvh"] < 3.0 * cap["ms_bvh"]


@pytest.mark.parametrize("value", ["ncell", -1, -3])
def test_gpu_bad_indices_raise_reference_error(small_domain, value):
    """With every other argument valid, the index check of cells_of_vertex
    (pyx:88-90) is the GPU mesh stage's: same exception and message."""
    c = small_domain.inputs()
    bad = c[5].copy()
    bad[3, 17] = small_domain.ncell if value == "ncell" else value
    with pytest.raises(ValueError, match="Indices of 'cells_of_vertex' out of range$"):
        horizon_svf_comp_py(*c[:5], bad, 24, 1, 40000.0, 0.2, 1, 2)
    h, s = horizon_svf_comp_py(*c, 24, 1, 40000.0, 0.2, 1, 2)
    assert np.isfinite(h).all()


def _subdomain(d, keep_cells):
    """Cells keep_cells of d with the vertices they use; cells_of_vertex
    remapped (entries of dropped cells become -2)."""
    keep_cells = np.asarray(keep_cells)
    verts = np.unique(d.vertex_of_cell[:, keep_cells])
    new_cell = np.full(d.ncell, -2, dtype=np.int64)
    new_cell[keep_cells] = np.arange(keep_cells.size)
    cov = d.cells_of_vertex[:, verts].astype(np.int64)
    cov = np.where(cov >= 0, new_cell[np.maximum(cov, 0)], -2).astype(np.int32)
    return (d.clon[keep_cells].copy(), d.clat[keep_cells].copy(), d.hsurf[keep_cells].copy(),
            d.vlon[verts].copy(), d.vlat[verts].copy(), np.ascontiguousarray(cov))


@pytest.mark.parametrize("ncell", [1, 2, 3, 17])
def test_gpu_few_cell_domains(ncell):
    d = synthetic.make_domain(edge_km=2.5, box_km=20.0, seed=6)
    rng = np.random.default_rng(ncell)
    first = int(rng.integers(0, d.ncell - ncell))
    inputs = _subdomain(d, np.arange(first, first + ncell))
    for grid_type in (0, 1):
        for kernel in (0, 1, 2):
            args = (16, grid_type, 20000.0, 0.5, 2, 1)
            h, s = horizon_svf_comp_py(*inputs, *args, kernel=kernel)
            ho, so, _ = oracle.horizon_svf(*inputs, *args)
            np.testing.assert_array_equal(h, ho)
            np.testing.assert_allclose(s, so, rtol=0, atol=1e-12)


def test_gpu_cell_ranges_at_the_ends(small_domain):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h, s = horizon_svf_comp_py(*small_domain.inputs(), *args)
    n = small_domain.ncell
    for b, e in ((0, 1), (n - 1, n), (0, n), (5, 6)):
        hr, sr = horizon_svf_comp_py(*small_domain.inputs(), *args, cells=(b, e))
        np.testing.assert_array_equal(hr[:, b:e], h[:, b:e])
        np.testing.assert_array_equal(sr[b:e], s[b:e])


def test_gpu_concurrent_calls_from_threads():
    """Calls from several host threads at once (the library serialises them
    per device) give the results of sequential calls."""
    from concurrent.futures import ThreadPoolExecutor
    doms = [synthetic.make_domain(edge_km=2.5, box_km=30.0 + 5 * k, seed=40 + k) for k in range(4)]
    argsets = [(24, 1, 40000.0, 0.2, 1, 2), (16, 0, 20000.0, 0.5, 2, 1),
               (36, 1, 30000.0, 0.2, 1, 0), (8, 1, 40000.0, 1.0, 3, 2)]
    ref = [horizon_svf_comp_py(*d.inputs(), *a) for d, a in zip(doms, argsets)]

    def run(k):
        return [horizon_svf_comp_py(*doms[k].inputs(), *argsets[k]) for _ in range(3)]

    with ThreadPoolExecutor(max_workers=4) as ex:
        outs = list(ex.map(run, range(4)))
    for k in range(4):
        for h, s in outs[k]:
            np.testing.assert_array_equal(h, ref[k][0])
            np.testing.assert_array_equal(s, ref[k][1])
