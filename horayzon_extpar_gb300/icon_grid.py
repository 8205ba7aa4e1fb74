"""ICON grid and EXTPAR files: the inputs of the horizon / SVF path.

The reference reads them with xarray (verification.py:81-104,
development.py:188-202):

* grid file: ``clon, clat`` (cell circumcentres) and ``vlon, vlat``
  (vertices) in radians; ``vertex_of_cell`` (3, ncell) and
  ``cells_of_vertex`` (6, nvertex) as 1-based Fortran indices, turned
  0-based by subtracting 1, so ICON's -1 for a missing cell becomes the -2
  that ``horizon_svf_comp`` expects (horizon_svf.pyx:88-90); attributes
  ``grid_root`` (n) and ``grid_level`` (k), nominal resolution
  5050 km / (n 2^k) (verification.py:92-93);
* EXTPAR file: cell elevation ``topography_c``, and ``HORIZON`` (nhori,
  ncell) and ``SKYVIEW`` (ncell), each squeezed of singleton axes
  (verification.py:99-103).

xarray and netCDF4 are not installed; scipy reads and writes the classic
netCDF formats (CDF-1 and 64-bit offset CDF-2). A netCDF-4 (HDF5) file
raises an error that names the conversion to the classic format
(``nccopy -k classic``). The writers produce files in the same layout, for
fixtures and for handing results back.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

_HDF5_MAGIC = b"\x89HDF\r\n\x1a\n"


@dataclass
class IconGrid:
    clon: np.ndarray             # (ncell,) float64 [rad]
    clat: np.ndarray             # (ncell,) float64 [rad]
    vlon: np.ndarray             # (nvertex,) float64 [rad]
    vlat: np.ndarray             # (nvertex,) float64 [rad]
    vertex_of_cell: np.ndarray   # (3, ncell) int32, 0-based
    cells_of_vertex: np.ndarray  # (6, nvertex) int32, 0-based, -2 = no cell
    grid_root: int
    grid_level: int

    @property
    def ncell(self) -> int:
        return int(self.clon.size)

    @property
    def grid_res_m(self) -> float:
        """Nominal resolution [m] (verification.py:92)."""
        return (5050.0 / (self.grid_root * 2 ** self.grid_level)) * 1000.0


def _open(path: str):
    from scipy.io import netcdf_file
    with open(path, "rb") as f:
        head = f.read(8)
    if head == _HDF5_MAGIC:
        raise ValueError("%s is a netCDF-4 (HDF5) file; neither netCDF4 nor h5py is "
                         "installed. Convert it to the classic format first: "
                         "nccopy -k classic in.nc out.nc" % path)
    if head[:3] != b"CDF":
        raise ValueError("%s is not a netCDF file" % path)
    return netcdf_file(path, "r", mmap=False)


def _var(ds, name: str, dtype=None):
    if name not in ds.variables:
        raise KeyError("variable '%s' not found (have: %s)"
                       % (name, ", ".join(sorted(ds.variables))))
    a = np.array(ds.variables[name].data)
    return a if dtype is None else a.astype(dtype)


def _attr(ds, name: str) -> int:
    v = getattr(ds, name, None)
    if v is None:
        raise KeyError("global attribute '%s' not found" % name)
    return int(np.asarray(v).ravel()[0])


def read_icon_grid(path: str) -> IconGrid:
    """The grid fields horizon_svf_comp needs (verification.py:82-91)."""
    ds = _open(path)
    try:
        g = IconGrid(clon=_var(ds, "clon", np.float64), clat=_var(ds, "clat", np.float64),
                     vlon=_var(ds, "vlon", np.float64), vlat=_var(ds, "vlat", np.float64),
                     vertex_of_cell=(_var(ds, "vertex_of_cell", np.int64) - 1).astype(np.int32),
                     cells_of_vertex=(_var(ds, "cells_of_vertex", np.int64) - 1).astype(np.int32),
                     grid_root=_attr(ds, "grid_root"), grid_level=_attr(ds, "grid_level"))
    finally:
        ds.close()
    if g.cells_of_vertex.ndim != 2 or g.cells_of_vertex.shape != (6, g.vlon.size):
        raise ValueError("cells_of_vertex must have shape (6, nvertex), got %s"
                         % (g.cells_of_vertex.shape,))
    if g.vertex_of_cell.shape != (3, g.clon.size):
        raise ValueError("vertex_of_cell must have shape (3, ncell), got %s"
                         % (g.vertex_of_cell.shape,))
    return g


def read_extpar(path: str) -> dict:
    """Cell elevation and, when present, the horizon / SVF fields
    (verification.py:99-103): ``hsurf`` (ncell,), ``horizon`` (nhori, ncell)
    or None, ``skyview`` (ncell,) or None, ``num_hori`` (0 without HORIZON)."""
    ds = _open(path)
    try:
        out = {"hsurf": np.squeeze(_var(ds, "topography_c", np.float64))}
        horizon = skyview = None
        if "HORIZON" in ds.variables:
            horizon = np.squeeze(_var(ds, "HORIZON", np.float64))
        if "SKYVIEW" in ds.variables:
            skyview = np.squeeze(_var(ds, "SKYVIEW", np.float64))
    finally:
        ds.close()
    out["horizon"] = horizon
    out["skyview"] = skyview
    out["num_hori"] = 0 if horizon is None else int(horizon.shape[0])
    return out


def inputs_from_files(grid_path: str, extpar_path: str):
    """The six array arguments of horizon_svf_comp_py from an ICON grid file
    and an EXTPAR file (verification.py:106-108: their cell counts must
    agree)."""
    g = read_icon_grid(grid_path)
    e = read_extpar(extpar_path)
    if g.clon.size != e["hsurf"].size:
        raise ValueError("Inconsistent number of cells in grid and topography")
    return (g.clon, g.clat, e["hsurf"], g.vlon, g.vlat, g.cells_of_vertex)


def write_icon_grid(path: str, clon, clat, vlon, vlat, vertex_of_cell, cells_of_vertex,
                    grid_root: int, grid_level: int) -> None:
    """An ICON grid file in the layout read_icon_grid reads (1-based indices,
    -1 for a missing cell)."""
    from scipy.io import netcdf_file
    cov = np.asarray(cells_of_vertex, dtype=np.int64)
    voc = np.asarray(vertex_of_cell, dtype=np.int64)
    with netcdf_file(path, "w", version=2) as ds:
        ds.grid_root = np.int32(grid_root)
        ds.grid_level = np.int32(grid_level)
        ds.createDimension("cell", int(np.size(clon)))
        ds.createDimension("vertex", int(np.size(vlon)))
        ds.createDimension("nv", 3)
        ds.createDimension("ne", 6)
        for name, dim, a in (("clon", "cell", clon), ("clat", "cell", clat),
                             ("vlon", "vertex", vlon), ("vlat", "vertex", vlat)):
            v = ds.createVariable(name, "d", (dim,))
            v[:] = np.asarray(a, dtype=np.float64)
            v.units = "radian"
        v = ds.createVariable("vertex_of_cell", "i", ("nv", "cell"))
        v[:] = (voc + 1).astype(np.int32)
        v = ds.createVariable("cells_of_vertex", "i", ("ne", "vertex"))
        v[:] = np.where(cov < 0, -1, cov + 1).astype(np.int32)


def write_extpar(path: str, hsurf, horizon=None, skyview=None) -> None:
    """An EXTPAR-style file: ``topography_c`` (1, ncell) and, if given,
    ``HORIZON`` (nhori, 1, ncell) [deg] and ``SKYVIEW`` (1, ncell)."""
    from scipy.io import netcdf_file
    hsurf = np.asarray(hsurf, dtype=np.float64)
    with netcdf_file(path, "w", version=2) as ds:
        ds.createDimension("cell", hsurf.size)
        ds.createDimension("time", 1)
        v = ds.createVariable("topography_c", "d", ("time", "cell"))
        v[:] = hsurf[None, :]
        v.units = "m"
        if horizon is not None:
            h = np.asarray(horizon, dtype=np.float64)
            ds.createDimension("nhori", h.shape[0])
            v = ds.createVariable("HORIZON", "d", ("nhori", "time", "cell"))
            v[:] = h[:, None, :]
            v.units = "deg"
        if skyview is not None:
            v = ds.createVariable("SKYVIEW", "d", ("time", "cell"))
            v[:] = np.asarray(skyview, dtype=np.float64)[None, :]
