"""Synthetic ICON-like grids: structural properties (CPU only)."""
import numpy as np

from horayzon_extpar_gb300 import synthetic


def test_grid_structure():
    d = synthetic.make_domain(edge_km=2.5, box_km=100.0, seed=0)
    cov = d.cells_of_vertex
    assert cov.dtype == np.int32 and cov.shape == (6, d.nvertex)
    valid = cov != -2
    assert ((cov[valid] >= 0) & (cov[valid] < d.ncell)).all()
    # valid entries first, -2 after them
    assert not (~valid[:-1] & valid[1:]).any()
    # every cell appears exactly three times (one per vertex)
    counts = np.bincount(cov[valid], minlength=d.ncell)
    assert (counts == 3).all()
    # interior vertices have six cells
    assert (valid.sum(0) == 6).mean() > 0.9
    assert d.clon.dtype == np.float64 and d.hsurf.shape == (d.ncell,)


def test_edge_length_and_count():
    d = synthetic.make_domain(edge_km=2.5, box_km=200.0, seed=0)
    voc = d.vertex_of_cell
    p = np.stack([np.cos(d.vlat) * np.cos(d.vlon), np.cos(d.vlat) * np.sin(d.vlon),
                  np.sin(d.vlat)], 1)
    e = np.linalg.norm(p[voc[0]] - p[voc[1]], axis=1) * synthetic.R_EARTH / 1e3
    assert 2.2 < e.mean() < 2.8
    expect = (200.0 ** 2) / (np.sqrt(3) / 4 * e.mean() ** 2)
    assert 0.8 * expect < d.ncell < 1.2 * expect


def test_circumcentres_equidistant():
    d = synthetic.make_domain(edge_km=5.0, box_km=100.0, seed=1)
    voc = d.vertex_of_cell
    c = np.stack([np.cos(d.clat) * np.cos(d.clon), np.cos(d.clat) * np.sin(d.clon),
                  np.sin(d.clat)], 1)
    p = np.stack([np.cos(d.vlat) * np.cos(d.vlon), np.cos(d.vlat) * np.sin(d.vlon),
                  np.sin(d.vlat)], 1)
    r = np.stack([np.linalg.norm(c - p[voc[k]], axis=1) for k in range(3)])
    np.testing.assert_allclose(r[1], r[0], rtol=1e-7)
    np.testing.assert_allclose(r[2], r[0], rtol=1e-7)


def test_terrain_ranges_and_seed():
    a = synthetic.make_domain(edge_km=2.5, box_km=100.0, seed=7, kind="fbm_ridged",
                              hmin=200.0, hmax=4800.0, n_features=0)
    b = synthetic.make_domain(edge_km=2.5, box_km=100.0, seed=7, kind="fbm_ridged",
                              hmin=200.0, hmax=4800.0, n_features=0)
    np.testing.assert_array_equal(a.hsurf, b.hsurf)
    assert a.hsurf.min() >= 200.0 - 1e-6 and a.hsurf.max() <= 4800.0 + 1e-6
