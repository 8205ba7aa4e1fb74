"""The CPU oracle pinned against the reference's own outputs (CPU only)."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import api


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_golden(name):
    g = load_golden(name)
    h, s, st = api.horizon_svf(*g["inputs"], *g["args"])
    assert st["overflow"] == 0
    np.testing.assert_array_equal(h, g["horizon"])
    np.testing.assert_array_equal(s, g["skyview"])


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_mesh_matches_reference_mesh(name):
    g = load_golden(name)
    mlon, mlat, mh, vot = api.build_mesh(*g["inputs"], g["args"][1])
    np.testing.assert_array_equal(vot, g["mesh_vot"])
    np.testing.assert_array_equal(mlon, g["mesh_lon"])
    np.testing.assert_array_equal(mlat, g["mesh_lat"])
    np.testing.assert_array_equal(mh, g["mesh_h"])


def test_bvh_equals_brute_force(small_domain):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h1, s1, st1 = api.horizon_svf(*small_domain.inputs(), *args)
    h2, s2, st2 = api.horizon_svf(*small_domain.inputs(), *args, brute_force=True)
    np.testing.assert_array_equal(h1, h2)
    np.testing.assert_array_equal(s1, s2)
    assert st1["num_rays"] == st2["num_rays"]
    assert st1["node_visits"] > 0 and st2["node_visits"] == 0


def test_cell_subset_equals_full(small_domain):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h, s, _ = api.horizon_svf(*small_domain.inputs(), *args)
    cells = np.random.default_rng(0).choice(small_domain.ncell, 200, replace=False)
    hs, ss, _ = api.horizon_svf(*small_domain.inputs(), *args, cells=cells, nthreads=2)
    np.testing.assert_array_equal(hs[:, cells], h[:, cells])
    np.testing.assert_array_equal(ss[cells], s[cells])
    others = np.setdiff1d(np.arange(small_domain.ncell), cells)
    assert np.isnan(ss[others]).all()


def test_fp64_oracle_close_to_fp32(small_domain):
    args = (24, 1, 40000.0, 0.2, 1, 2)
    h32, s32, _ = api.horizon_svf(*small_domain.inputs(), *args)
    h64, s64, _ = api.horizon_svf(*small_domain.inputs(), *args, precision=1)
    assert np.mean(np.abs(h64 - h32) <= 0.25) >= 0.999
    assert np.abs(s64 - s32).max() <= 1e-3


def test_outputs_on_half_degree_lattice(small_domain):
    """refine_factor 1: horizons are 0 or k*0.5 deg - 0.25 deg (cpp:525-547)."""
    h, _, _ = api.horizon_svf(*small_domain.inputs(), 24, 1, 40000.0, 0.2, 1, 2)
    pos = h[h > 0]
    k = (pos + 0.25) / 0.5
    np.testing.assert_allclose(k, np.round(k), atol=1e-9)


def test_occlusion_brute_force_random_rays():
    rng = np.random.default_rng(4)
    n = 300
    vert = rng.uniform(-100, 100, (n, 3)).astype(np.float32)
    vot = rng.integers(0, n, (400, 3)).astype(np.int32)
    org = rng.uniform(-120, 120, (2000, 3)).astype(np.float32)
    d = rng.normal(size=(2000, 3)).astype(np.float32)
    a = api.occluded32(vert, vot, org, d, 150.0)
    b = api.occluded32(vert, vot, org, d, 150.0, brute_force=True)
    np.testing.assert_array_equal(a, b)
    assert 0 < a.sum() < a.size
