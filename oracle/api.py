"""ctypes front end of the CPU oracle and of the shim-compiled reference.

TEST INFRASTRUCTURE (see ``oracle/__init__.py``): imported only by tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_U8 = C.POINTER(C.c_uint8)


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("nthreads", C.c_int),
                ("cells", _I), ("n_cells", C.c_int),
                ("elev_floor_deg", C.c_double), ("brute_force", C.c_int),
                ("start_m", C.POINTER(C.c_int16)), ("groups", C.c_int),
                ("start_all", C.c_int), ("bisect_walk", C.c_int)]


class Result(C.Structure):
    _fields_ = [("num_rays", C.c_int64), ("node_visits", C.c_int64),
                ("tri_tests", C.c_int64), ("overflow", C.c_int64),
                ("n_tri", C.c_int), ("n_mesh_vert", C.c_int),
                ("t_mesh", C.c_double), ("t_bvh", C.c_double),
                ("t_rays", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_ref = None


def lib():
    """The oracle library (compiled on first use)."""
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build_oracle())
        L.hzo_horizon_svf.restype = C.c_int
        L.hzo_horizon_svf.argtypes = [_D, _D, _D, _D, _D, _I, _D, _D, C.c_int, C.c_int,
                                      C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                                      C.c_int, C.POINTER(Options), C.POINTER(Result)]
        L.hzo_build_mesh.restype = C.c_int
        L.hzo_build_mesh.argtypes = [_D, _D, _D, _D, _D, _I, C.c_int, C.c_int, C.c_int,
                                     _D, _D, _D, C.c_int, _I, C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.hzo_mesh_enu.restype = C.c_int
        L.hzo_mesh_enu.argtypes = [_D, _D, _D, _D, _D, _I, C.c_int, C.c_int, C.c_int,
                                   _D, _F, C.c_int, _I, C.c_int,
                                   C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.hzo_occluded32.restype = C.c_int
        L.hzo_occluded32.argtypes = [_F, _I, C.c_int, _F, _F, C.c_float, C.c_int,
                                     C.c_int, _U8]
        _lib = L
    return _lib


def reference_lib():
    """The unmodified reference compiled against the shim, or None."""
    global _ref
    if _ref is None:
        path = _build.REF_SO
        if not os.path.exists(path):
            path = _build.build_reference()
            if path is None:
                return None
        R = C.CDLL(path)
        R.hzref_horizon_svf_comp.restype = None
        R.hzref_horizon_svf_comp.argtypes = [_D, _D, _D, _D, _D, _I, _D, _D, C.c_int,
                                             C.c_int, C.c_int, C.c_int, C.c_double,
                                             C.c_double, C.c_int, C.c_int]
        R.hzref_build_triangle_mesh.restype = C.c_int
        R.hzref_build_triangle_mesh.argtypes = [_D, _D, _D, _D, _D, _I, C.c_int,
                                                C.c_int, C.c_int, _D, C.c_int, _I,
                                                C.c_int, C.POINTER(C.c_int)]
        _ref = R
    return _ref


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _p(a, t):
    return a.ctypes.data_as(t)


def horizon_svf(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori, grid_type,
                dist_search, ray_org_elev, refine_factor, svf_type, *, precision=0,
                nthreads=0, cells=None, elev_floor_deg=-85.0, brute_force=False,
                start_index=None, groups=1, start_all=False, bisect_walk=False):
    """Oracle horizon [nhori, ncell] (deg), skyview [ncell], stats dict.

    With ``cells`` only those columns/entries are computed (others are NaN).
    ``start_index`` (int16 [L, ncell], L = num_hori * refine_factor): warm
    start lattice indices; each cell's azimuths form ``groups`` runs whose
    first azimuth starts there (every azimuth with ``start_all``).
    ``bisect_walk``: the downward walk below the clip by doubling and
    bisection (the GPU library's HZ_WALK_BISECT).
    """
    clon, clat, hsurf, vlon, vlat = map(_f64, (clon, clat, hsurf, vlon, vlat))
    cov = _i32(cells_of_vertex)
    ncell, nvert = clon.size, vlon.size
    horizon = np.full((num_hori, ncell), np.nan)
    skyview = np.full(ncell, np.nan)
    opt = Options(precision=precision, nthreads=nthreads, cells=None, n_cells=0,
                  elev_floor_deg=elev_floor_deg, brute_force=int(brute_force),
                  bisect_walk=int(bool(bisect_walk)))
    if cells is not None:
        cells = _i32(cells)
        opt.cells = _p(cells, _I)
        opt.n_cells = cells.size
    if start_index is not None:
        start_index = np.ascontiguousarray(start_index, dtype=np.int16)
        if start_index.shape != (num_hori * refine_factor, ncell):
            raise ValueError("start_index must have shape (num_hori * refine_factor, ncell)")
        opt.start_m = start_index.ctypes.data_as(C.POINTER(C.c_int16))
        opt.groups = int(groups)
        opt.start_all = int(bool(start_all))
    res = Result()
    rc = lib().hzo_horizon_svf(_p(clon, _D), _p(clat, _D), _p(hsurf, _D), _p(vlon, _D),
                               _p(vlat, _D), _p(cov, _I), _p(horizon, _D),
                               _p(skyview, _D), ncell, nvert, num_hori, grid_type,
                               dist_search, ray_org_elev, refine_factor, svf_type,
                               C.byref(opt), C.byref(res))
    if rc != 0:
        raise RuntimeError("oracle failed with status %d" % rc)
    return horizon, skyview, res.as_dict()


def build_mesh(clon, clat, hsurf, vlon, vlat, cells_of_vertex, grid_type):
    """Oracle mesh: (lon, lat, h) per mesh vertex and vertex_of_triangle (ntri, 3)."""
    clon, clat, hsurf, vlon, vlat = map(_f64, (clon, clat, hsurf, vlon, vlat))
    cov = _i32(cells_of_vertex)
    ncell, nvert = clon.size, vlon.size
    cap_v, cap_t = ncell + nvert, 6 * nvert
    mlon, mlat, mh = (np.empty(cap_v) for _ in range(3))
    vot = np.empty((max(cap_t, 1), 3), dtype=np.int32)
    nmv, ntri = C.c_int(0), C.c_int(0)
    rc = lib().hzo_build_mesh(_p(clon, _D), _p(clat, _D), _p(hsurf, _D), _p(vlon, _D),
                              _p(vlat, _D), _p(cov, _I), ncell, nvert, grid_type,
                              _p(mlon, _D), _p(mlat, _D), _p(mh, _D), cap_v,
                              _p(vot, _I), cap_t, C.byref(nmv), C.byref(ntri))
    if rc != 0:
        raise RuntimeError("oracle mesh failed with status %d" % rc)
    n = nmv.value
    return mlon[:n], mlat[:n], mh[:n], vot[:ntri.value]


def mesh_enu(clon, clat, hsurf, vlon, vlat, cells_of_vertex, grid_type):
    """Oracle ENU vertices: (enu64 (n,3), enu32 (n,3), vertex_of_triangle (ntri,3))."""
    clon, clat, hsurf, vlon, vlat = map(_f64, (clon, clat, hsurf, vlon, vlat))
    cov = _i32(cells_of_vertex)
    ncell, nvert = clon.size, vlon.size
    cap_v, cap_t = ncell + nvert, 6 * nvert
    e64 = np.empty((cap_v, 3))
    e32 = np.empty((cap_v, 3), dtype=np.float32)
    vot = np.empty((max(cap_t, 1), 3), dtype=np.int32)
    nmv, ntri = C.c_int(0), C.c_int(0)
    rc = lib().hzo_mesh_enu(_p(clon, _D), _p(clat, _D), _p(hsurf, _D), _p(vlon, _D),
                            _p(vlat, _D), _p(cov, _I), ncell, nvert, grid_type,
                            _p(e64, _D), _p(e32, _F), cap_v, _p(vot, _I), cap_t,
                            C.byref(nmv), C.byref(ntri))
    if rc != 0:
        raise RuntimeError("oracle mesh failed with status %d" % rc)
    n = nmv.value
    return e64[:n], e32[:n], vot[:ntri.value]


def occluded32(vert, vot, org, dirs, tfar, brute_force=False):
    """Any-hit flags of FP32 rays against an FP32 mesh (oracle semantics)."""
    vert = np.ascontiguousarray(vert, dtype=np.float32)
    vot = _i32(vot)
    org = np.ascontiguousarray(org, dtype=np.float32)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32)
    hit = np.zeros(org.shape[0], dtype=np.uint8)
    rc = lib().hzo_occluded32(_p(vert, _F), _p(vot, _I), vot.shape[0], _p(org, _F),
                              _p(dirs, _F), tfar, org.shape[0], int(brute_force),
                              _p(hit, _U8))
    if rc != 0:
        raise RuntimeError("oracle occlusion failed with status %d" % rc)
    return hit.astype(bool)


def reference_horizon_svf(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori,
                          grid_type, dist_search, ray_org_elev, refine_factor,
                          svf_type):
    """The unmodified reference (shim build): horizon, skyview. None if absent."""
    R = reference_lib()
    if R is None:
        return None
    clon, clat, hsurf, vlon, vlat = map(_f64, (clon, clat, hsurf, vlon, vlat))
    cov = _i32(cells_of_vertex)
    horizon = np.empty((num_hori, clon.size))
    skyview = np.empty(clon.size)
    R.hzref_horizon_svf_comp(_p(clon, _D), _p(clat, _D), _p(hsurf, _D), _p(vlon, _D),
                             _p(vlat, _D), _p(cov, _I), _p(horizon, _D), _p(skyview, _D),
                             clon.size, vlon.size, num_hori, grid_type, dist_search,
                             ray_org_elev, refine_factor, svf_type)
    return horizon, skyview


def reference_build_mesh(clon, clat, hsurf, vlon, vlat, cells_of_vertex, grid_type):
    """Reference mesh: (lon, lat, h) per mesh vertex and vertex_of_triangle."""
    R = reference_lib()
    if R is None:
        return None
    clon, clat, hsurf, vlon, vlat = map(_f64, (clon, clat, hsurf, vlon, vlat))
    cov = _i32(cells_of_vertex)
    ncell, nvert = clon.size, vlon.size
    cap_v, cap_t = ncell + nvert, 6 * nvert
    xyz = np.empty((cap_v, 3))
    vot = np.empty((max(cap_t, 1), 3), dtype=np.int32)
    nmv = C.c_int(0)
    ntri = R.hzref_build_triangle_mesh(_p(clon, _D), _p(clat, _D), _p(hsurf, _D),
                                       _p(vlon, _D), _p(vlat, _D), _p(cov, _I), ncell,
                                       nvert, grid_type, _p(xyz, _D), cap_v, _p(vot, _I),
                                       cap_t, C.byref(nmv))
    n = nmv.value
    return xyz[:n, 0], xyz[:n, 1], xyz[:n, 2], vot[:ntri]
