"""ctypes binding of libhorayzon_gb300.so (include/horayzon_gb300.h).

The library is built in-tree (``horayzon_extpar_gb300/_lib/``) by
``horayzon_extpar_gb300._build.build_library()``. Loading fails loudly when
it is missing: there is no CPU fallback for the horizon computation.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)

HZ_OK, HZ_ERR_VALUE, HZ_ERR_TYPE, HZ_ERR_INDEX, HZ_ERR_CUDA, HZ_ERR_INTERNAL = range(6)

#: Every symbol include/horayzon_gb300.h declares.
EXPORTED_SYMBOLS = ("hz_default_options", "horizon_svf_comp", "horizon_svf_comp_buffer",
                    "hz_horizon_svf",
                    "hz_horizon_svf_device", "hz_build_mesh", "hz_mesh_enu32",
                    "hz_last_error", "hz_version", "hz_release_workspace",
                    "hz_horizon_svf_device_static", "hz_horizon_svf_batch",
                    "hz_mlp_num_params", "hz_mlp_train_step", "hz_mlp_forward",
                    "hz_distance_to_border", "hz_occluded32")


class Domain(C.Structure):
    """hz_domain: one regional domain of a batch call."""
    _fields_ = [("clon", C.c_void_p), ("clat", C.c_void_p), ("hsurf", C.c_void_p),
                ("vlon", C.c_void_p), ("vlat", C.c_void_p),
                ("cells_of_vertex", C.c_void_p), ("horizon", C.c_void_p),
                ("skyview", C.c_void_p), ("num_cell", C.c_int32),
                ("num_vertex", C.c_int32), ("num_hori", C.c_int32),
                ("grid_type", C.c_int32), ("dist_search", C.c_double),
                ("ray_org_elev", C.c_double), ("refine_factor", C.c_int32),
                ("svf_type", C.c_int32), ("latency_ms", C.c_double)]


class Options(C.Structure):
    _fields_ = [("size", C.c_int32), ("device", C.c_int32), ("count_work", C.c_int32),
                ("verbose", C.c_int32), ("elev_floor_deg", C.c_double),
                ("cell_begin", C.c_int32), ("cell_count", C.c_int32),
                ("kernel", C.c_int32), ("advance_min", C.c_int32),
                ("precision", C.c_int32), ("mlp_params", C.c_void_p),
                ("mlp_every_azimuth", C.c_int32), ("raw_index", C.c_void_p),
                ("features", C.c_void_p), ("leaf_min", C.c_int32),
                ("leaf_size", C.c_int32), ("queue_chunk", C.c_int32),
                ("direct_launch", C.c_int32), ("mlp_azimuth_groups", C.c_int32),
                ("start_index", C.c_void_p), ("bvh_treelets", C.c_int32),
                ("elev_walk", C.c_int32), ("occluder_cache", C.c_int32)]


HZ_KERNEL_PERSISTENT, HZ_KERNEL_PER_CELL, HZ_KERNEL_PERSISTENT_BVH2 = 0, 1, 2
HZ_PRECISION_REFERENCE, HZ_PRECISION_LOCAL = 0, 1
HZ_WALK_REFERENCE, HZ_WALK_BISECT = 0, 1


class Stats(C.Structure):
    _fields_ = [("num_rays", C.c_int64), ("node_visits", C.c_int64),
                ("tri_tests", C.c_int64), ("n_tri", C.c_int32),
                ("n_mesh_vert", C.c_int32), ("ms_h2d", C.c_double),
                ("ms_mesh", C.c_double), ("ms_bvh", C.c_double),
                ("ms_trace", C.c_double), ("ms_d2h", C.c_double),
                ("ms_total", C.c_double), ("kernel_launches", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class HorizonError(RuntimeError):
    """A non-value failure reported by the CUDA library (status, message)."""

    def __init__(self, status: int, message: str):
        super().__init__("horayzon_gb300 error %d: %s" % (status, message))
        self.status = status


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return os.environ.get("HZ_LIBRARY", _build.LIB_PATH)


def load(build_if_missing: bool = True):
    """The loaded CUDA library (built in-tree on first use if absent)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError("libhorayzon_gb300.so not found at %s; build it with "
                                   "horayzon_extpar_gb300._build.build_library()" % path)
            path = _build.build_library()
        L = C.CDLL(path)
        L.hz_default_options.restype = None
        L.hz_default_options.argtypes = [C.POINTER(Options)]
        L.hz_last_error.restype = C.c_char_p
        L.hz_last_error.argtypes = []
        L.hz_version.restype = C.c_int
        L.hz_release_workspace.restype = C.c_int
        L.hz_release_workspace.argtypes = [C.c_int]
        common = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int,
                  C.c_int]
        L.horizon_svf_comp.restype = None
        L.horizon_svf_comp.argtypes = [_D, _D, _D, _D, _D, _I, _D, _D] + common
        L.horizon_svf_comp_buffer.restype = None
        L.horizon_svf_comp_buffer.argtypes = ([_D, _D, _D, _D, _D, _I, _D, _D] + common +
                                              [C.c_char_p, C.POINTER(C.c_int)])
        L.hz_horizon_svf.restype = C.c_int
        L.hz_horizon_svf.argtypes = ([_D, _D, _D, _D, _D, _I, _D, _D] + common +
                                     [C.POINTER(Options), C.POINTER(Stats)])
        L.hz_horizon_svf_device.restype = C.c_int
        L.hz_horizon_svf_device.argtypes = ([C.c_void_p] * 8 + common +
                                            [C.c_void_p, C.POINTER(Options),
                                             C.POINTER(Stats)])
        L.hz_horizon_svf_device_static.restype = C.c_int
        L.hz_horizon_svf_device_static.argtypes = [C.c_void_p] * 8 + common + [C.c_void_p]
        L.hz_horizon_svf_batch.restype = C.c_int
        L.hz_horizon_svf_batch.argtypes = [C.POINTER(Domain), C.c_int, C.c_int, C.c_void_p,
                                           C.POINTER(Options), C.POINTER(Stats)]
        L.hz_occluded32.restype = C.c_int
        L.hz_occluded32.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                    C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_int,
                                    C.c_int, C.c_int]
        L.hz_distance_to_border.restype = C.c_int
        L.hz_distance_to_border.argtypes = [C.c_void_p] * 5 + [C.c_int, C.c_int, C.c_void_p,
                                                               C.c_int, C.c_void_p]
        L.hz_mlp_num_params.restype = C.c_int
        L.hz_mlp_num_params.argtypes = []
        L.hz_mlp_train_step.restype = C.c_int
        L.hz_mlp_train_step.argtypes = [C.c_void_p] * 5 + [C.c_int, C.c_int, C.c_float] + \
            [C.c_void_p] * 3
        L.hz_mlp_forward.restype = C.c_int
        L.hz_mlp_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.hz_build_mesh.restype = C.c_int
        L.hz_build_mesh.argtypes = [_D, _D, _D, _D, _D, _I, C.c_int, C.c_int, C.c_int,
                                    _D, _D, _D, C.c_int, _I, C.c_int,
                                    C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
        L.hz_mesh_enu32.restype = C.c_int
        L.hz_mesh_enu32.argtypes = [_D, _D, _D, _D, _D, _I, C.c_int, C.c_int, C.c_int,
                                    _F, C.c_int, _I, C.c_int,
                                    C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]
        _lib = L
        return _lib


def last_error() -> str:
    return load().hz_last_error().decode("utf-8", "replace")


def default_options(**kw) -> Options:
    o = Options()
    load().hz_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def check(status: int):
    """Raise the reference's exception type for a failed call."""
    if status == HZ_OK:
        return
    msg = last_error()
    if status in (HZ_ERR_VALUE, HZ_ERR_INDEX):
        raise ValueError(msg)
    if status == HZ_ERR_TYPE:
        raise TypeError(msg)
    raise HorizonError(status, msg)
