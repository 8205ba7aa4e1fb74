"""ICON grid / EXTPAR file access (verification.py:81-104): round trips of
the classic-netCDF writer and reader, the index conventions, errors, and the
oracle run from file inputs."""
import numpy as np
import pytest

from horayzon_extpar_gb300 import icon_grid, synthetic
from oracle import api as oracle


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = synthetic.make_domain(edge_km=3.0, box_km=40.0, seed=4)
    root = tmp_path_factory.mktemp("icon")
    grid = str(root / "grid.nc")
    extpar = str(root / "extpar.nc")
    icon_grid.write_icon_grid(grid, d.clon, d.clat, d.vlon, d.vlat, d.vertex_of_cell,
                              d.cells_of_vertex, grid_root=2, grid_level=10)
    icon_grid.write_extpar(extpar, d.hsurf)
    return d, grid, extpar


def test_grid_round_trip_keeps_the_reference_index_convention(files):
    d, grid, _ = files
    g = icon_grid.read_icon_grid(grid)
    for name in ("clon", "clat", "vlon", "vlat"):
        np.testing.assert_array_equal(getattr(g, name), getattr(d, name))
        assert getattr(g, name).dtype == np.float64
    np.testing.assert_array_equal(g.vertex_of_cell, d.vertex_of_cell)
    np.testing.assert_array_equal(g.cells_of_vertex, d.cells_of_vertex)
    assert g.cells_of_vertex.dtype == np.int32
    assert (g.cells_of_vertex == -2).any()  # border vertices: ICON -1, minus 1
    assert g.grid_root == 2 and g.grid_level == 10
    assert g.grid_res_m == pytest.approx(5050.0 / (2 * 2 ** 10) * 1000.0)


def test_extpar_round_trip_squeezes_singleton_axes(files, tmp_path):
    d, _, extpar = files
    e = icon_grid.read_extpar(extpar)
    np.testing.assert_array_equal(e["hsurf"], d.hsurf)
    assert e["horizon"] is None and e["skyview"] is None and e["num_hori"] == 0
    rng = np.random.default_rng(0)
    h = rng.uniform(0, 30, (24, d.ncell))
    s = rng.uniform(0.5, 1, d.ncell)
    path = str(tmp_path / "out.nc")
    icon_grid.write_extpar(path, d.hsurf, h, s)
    e = icon_grid.read_extpar(path)
    np.testing.assert_array_equal(e["horizon"], h)
    np.testing.assert_array_equal(e["skyview"], s)
    assert e["num_hori"] == 24


def test_inputs_from_files_feed_the_path(files):
    d, grid, extpar = files
    ins = icon_grid.inputs_from_files(grid, extpar)
    args = (8, 1, 15000.0, 0.2, 1, 2)
    h0, s0, _ = oracle.horizon_svf(*d.inputs(), *args)
    h1, s1, _ = oracle.horizon_svf(*ins, *args)
    np.testing.assert_array_equal(h0, h1)
    np.testing.assert_array_equal(s0, s1)


def test_inconsistent_cell_counts(files, tmp_path):
    d, grid, _ = files
    bad = str(tmp_path / "bad.nc")
    icon_grid.write_extpar(bad, d.hsurf[:-1])
    with pytest.raises(ValueError, match="Inconsistent number of cells"):
        icon_grid.inputs_from_files(grid, bad)


def test_hdf5_and_foreign_files_are_rejected(tmp_path):
    h5 = tmp_path / "grid4.nc"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    with pytest.raises(ValueError, match="nccopy -k classic"):
        icon_grid.read_icon_grid(str(h5))
    txt = tmp_path / "x.nc"
    txt.write_bytes(b"hello world")
    with pytest.raises(ValueError, match="not a netCDF file"):
        icon_grid.read_extpar(str(txt))


def test_missing_variable_is_named(files, tmp_path):
    d, _, extpar = files
    with pytest.raises(KeyError, match="clon"):
        icon_grid.read_icon_grid(extpar)
