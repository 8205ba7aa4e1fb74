"""Drop-in replacement of the reference's Cython module ``horizon_svf``.

``horizon_svf_comp_py`` keeps the signature, argument checks (same exception
types and messages), array layouts and return values of
horizon_svf.pyx:15-124; the computation runs on the GPU through
libhorayzon_gb300.so. ``horizon_svf_comp_device`` is the same call on arrays
that already live in GPU memory (torch tensors).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

__all__ = ["horizon_svf_comp_py", "horizon_svf_comp_device", "build_mesh", "mesh_enu32",
           "occluded32"]

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)


def _typed(name, arr, dtype, ndim):
    """Mimics Cython's typed-buffer argument checks (pyx:15-20)."""
    if not isinstance(arr, np.ndarray):
        raise TypeError("Argument '%s' has incorrect type (expected numpy.ndarray, got %s)"
                        % (name, type(arr).__name__))
    if arr.ndim != ndim:
        raise ValueError("Buffer has wrong number of dimensions (expected %d, got %d)"
                         % (ndim, arr.ndim))
    if arr.dtype != dtype:
        raise ValueError("Buffer dtype mismatch, expected '%s' but got '%s'"
                         % ("float64_t" if dtype == np.float64 else "int32_t", arr.dtype))
    return arr


def _int_arg(v):
    if isinstance(v, (float, np.floating)):
        raise TypeError("'float' object cannot be interpreted as an integer")
    return int(v)


def _scalar_error(num_hori, grid_type, dist_search, ray_org_elev, refine_factor, svf_type):
    """The first failing range check of horizon_svf.pyx:91-103, or None."""
    if (num_hori < 4) or (num_hori > 1440):
        return ValueError("'num_hori' must be in the range [4, 1440]")
    if (grid_type < 0) or (grid_type > 1):
        return ValueError("'grid_type' must be in the range [0, 1]")
    if (dist_search < 1_000.0) or (dist_search > 500_000.0):
        return ValueError("'dist_search' must be in the range "
                          + "[1'000, 500'000] km")
    if ray_org_elev < 0.1:
        return TypeError("Minimal allowed value for 'ray_org_elev' is 0.1 m")
    if (refine_factor < 1) or (refine_factor > 50):
        return ValueError("'refine_factor' must be in the range [1, 50]")
    if (svf_type < 0) or (svf_type > 2):
        return ValueError("'svf_type' must be in the range [0, 2]")
    return None


def _check_args(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori, grid_type,
                dist_search, ray_org_elev, refine_factor, svf_type):
    """horizon_svf.pyx:78-103, same order, types and messages.

    The index check of cells_of_vertex (pyx:88-90) is also made by the GPU
    mesh stage, with the same condition, exception and message; it runs
    here only where its place in the order of checks shows (another
    argument is invalid, or an array is empty), and is otherwise left to the
    GPU (a numpy pass over 6 x nvertex entries costs ~10 ms per call on
    the benchmark domain)."""
    if (clon.size != clat.size) or (clat.size != hsurf.size):
        raise ValueError("Inconsistent lengths of input arrays 'clon', "
                         "'clat' and 'hsurf'")
    if (vlon.size != vlat.size):
        raise ValueError("Inconsistent lengths of input arrays 'vlon' and "
                         "'vlat'")
    if cells_of_vertex.shape[0] != 6:
        raise ValueError("First dimension of 'cells_of_vertex' must "
                         + "have length 6")
    err = _scalar_error(num_hori, grid_type, dist_search, ray_org_elev, refine_factor,
                        svf_type)
    if err is not None or clon.size == 0 or vlon.size == 0:
        if not np.all((cells_of_vertex >= 0) & (cells_of_vertex <= clon.size - 1)
                      | (cells_of_vertex == -2)):
            raise ValueError("Indices of 'cells_of_vertex' out of range")
    if err is not None:
        raise err


def _options(device, count_work, elev_floor_deg, verbose, cells=None, kernel=0,
             advance_min=0, precision=0, mlp_params=None, raw_index=None, features=None,
             mlp_every_azimuth=False, leaf_min=0, leaf_size=0, queue_chunk=0,
             direct_launch=False, mlp_azimuth_groups=0, start_index=None,
             bvh_treelets=False, elev_walk=0, occluder_cache=True):
    begin, count = (0, 0) if cells is None else (int(cells[0]), int(cells[1]) - int(cells[0]))
    opt = _lib.default_options(device=int(device), count_work=int(bool(count_work)),
                               elev_floor_deg=float(elev_floor_deg),
                               verbose=int(bool(verbose)), cell_begin=begin,
                               cell_count=count, kernel=int(kernel),
                               advance_min=int(advance_min), precision=int(precision),
                               leaf_min=int(leaf_min), leaf_size=int(leaf_size),
                               queue_chunk=int(queue_chunk),
                               direct_launch=int(bool(direct_launch)),
                               bvh_treelets=int(bool(bvh_treelets)),
                               elev_walk=int(elev_walk),
                               occluder_cache=int(bool(occluder_cache)))
    if mlp_params is not None:
        p = np.ascontiguousarray(mlp_params, dtype=np.float32)
        if p.size != _lib.load().hz_mlp_num_params():
            raise ValueError("mlp_params must hold %d values"
                             % _lib.load().hz_mlp_num_params())
        opt._keep = p  # alive for the duration of the call
        opt.mlp_params = p.ctypes.data
        opt.mlp_every_azimuth = int(bool(mlp_every_azimuth))
        opt.mlp_azimuth_groups = int(mlp_azimuth_groups)
    if start_index is not None:
        opt.start_index = start_index.data_ptr()
        opt.mlp_every_azimuth = int(bool(mlp_every_azimuth))
        opt.mlp_azimuth_groups = int(mlp_azimuth_groups)
    if raw_index is not None:
        opt.raw_index = raw_index.data_ptr()
    if features is not None:
        opt.features = features.data_ptr()
    return opt


def horizon_svf_comp_py(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori,
                        grid_type, dist_search, ray_org_elev, refine_factor, svf_type,
                        *, device=-1, count_work=False, elev_floor_deg=-85.0,
                        verbose=False, return_stats=False, cells=None, kernel=0,
                        advance_min=0, precision=0, mlp_params=None,
                        mlp_every_azimuth=False, leaf_min=0, leaf_size=0, queue_chunk=0,
                        direct_launch=False, mlp_azimuth_groups=0, bvh_treelets=False,
                        elev_walk=0, occluder_cache=True):
    """Compute the terrain horizon and sky view factor on the GPU.

    Arguments and returns as horizon_svf.pyx:15-76: FP64 1-D ``clon, clat``
    [rad], ``hsurf`` [m], ``vlon, vlat`` [rad]; int32 (6, nvertex)
    ``cells_of_vertex`` (-2 = no cell); returns ``horizon`` (num_hori, ncell)
    [deg] and ``skyview`` (ncell) as new C-order float64 arrays. Keyword-only
    extras: CUDA ``device``, work counters, the downward-walk bound, a cell
    range ``cells=(begin, end)`` to trace (entries outside it are NaN), the
    search ``kernel`` (0 persistent, 1 one thread per cell, 2 the
    persistent search on the binary BVH), its ``advance_min`` / ``leaf_min``
    knobs, the work-queue ``queue_chunk``, the BVH ``leaf_size``,
    ``direct_launch`` (launch each kernel directly instead of replaying the
    captured CUDA graph of the BVH build and search), ``bvh_treelets``
    (treelet restructuring of the BVH: same results), ``elev_walk`` (1:
    bisection for the downward walk below the clip, see hz_options),
    ``occluder_cache`` (False: traverse the tree for every ray; same
    results), the
    learned warm start
    (``mlp_params``; ``mlp_every_azimuth``; ``mlp_azimuth_groups``: search
    items per cell, -1 = chosen by the library, see hz_options) and, with
    ``return_stats``, a third return value with ray counts and phase times.
    """
    clon = _typed("clon", clon, np.float64, 1)
    clat = _typed("clat", clat, np.float64, 1)
    hsurf = _typed("hsurf", hsurf, np.float64, 1)
    vlon = _typed("vlon", vlon, np.float64, 1)
    vlat = _typed("vlat", vlat, np.float64, 1)
    cells_of_vertex = _typed("cells_of_vertex", cells_of_vertex, np.int32, 2)
    num_hori, grid_type = _int_arg(num_hori), _int_arg(grid_type)
    refine_factor, svf_type = _int_arg(refine_factor), _int_arg(svf_type)
    dist_search, ray_org_elev = float(dist_search), float(ray_org_elev)
    _check_args(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori, grid_type,
                dist_search, ray_org_elev, refine_factor, svf_type)
    if clon.size == 0 or vlon.size == 0:
        raise IndexError("Out of bounds on buffer access (axis 0)")

    horizon = np.empty((num_hori, clon.size), dtype=np.float64)
    skyview = np.empty(clon.size, dtype=np.float64)
    if cells is not None:
        horizon.fill(np.nan)
        skyview.fill(np.nan)
    clon, clat, hsurf, vlon, vlat = (np.ascontiguousarray(a) for a in
                                     (clon, clat, hsurf, vlon, vlat))
    cells_of_vertex = np.ascontiguousarray(cells_of_vertex)
    L = _lib.load()
    opt = _options(device, count_work, elev_floor_deg, verbose, cells, kernel, advance_min,
                   precision, mlp_params, mlp_every_azimuth=mlp_every_azimuth,
                   leaf_min=leaf_min, leaf_size=leaf_size, queue_chunk=queue_chunk,
                   direct_launch=direct_launch, mlp_azimuth_groups=mlp_azimuth_groups,
                   bvh_treelets=bvh_treelets, elev_walk=elev_walk,
                   occluder_cache=occluder_cache)
    st = _lib.Stats()
    rc = L.hz_horizon_svf(clon.ctypes.data_as(_D), clat.ctypes.data_as(_D),
                          hsurf.ctypes.data_as(_D), vlon.ctypes.data_as(_D),
                          vlat.ctypes.data_as(_D), cells_of_vertex.ctypes.data_as(_I),
                          horizon.ctypes.data_as(_D), skyview.ctypes.data_as(_D),
                          clon.size, vlon.size, num_hori, grid_type, dist_search,
                          ray_org_elev, refine_factor, svf_type, C.byref(opt),
                          C.byref(st))
    _lib.check(rc)
    if return_stats:
        return horizon, skyview, st.as_dict()
    return horizon, skyview


def horizon_svf_comp_device(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori,
                            grid_type, dist_search, ray_org_elev, refine_factor,
                            svf_type, horizon=None, skyview=None, *, stream=None,
                            count_work=False, elev_floor_deg=-85.0, cells=None, kernel=0,
                            advance_min=0, precision=0, mlp_params=None, raw_index=None,
                            features=None, mlp_every_azimuth=False, leaf_min=0,
                            leaf_size=0, queue_chunk=0, direct_launch=False,
                            mlp_azimuth_groups=0, start_index=None, bvh_treelets=False,
                            elev_walk=0, occluder_cache=True):
    """Same computation on CUDA tensors (torch) already resident on one GPU.

    Inputs: contiguous float64 / int32 tensors on the same device, layouts as
    in :func:`horizon_svf_comp_py`. ``horizon``/``skyview`` may be passed
    preallocated. ``cells=(begin, end)`` traces only that cell range (the
    mesh and BVH always cover the whole domain; other output entries are left
    untouched). ``start_index`` (int16 tensor [L, ncell] on the device):
    given warm-start lattice indices used like the MLP's proposals (see
    hz_options.start_index). Runs on ``stream`` (default: torch's current
    stream) and returns ``(horizon, skyview, stats)``.
    """
    import torch

    dev = clon.device
    if dev.type != "cuda":
        raise ValueError("horizon_svf_comp_device needs CUDA tensors")
    for name, t, dt in (("clon", clon, torch.float64), ("clat", clat, torch.float64),
                        ("hsurf", hsurf, torch.float64), ("vlon", vlon, torch.float64),
                        ("vlat", vlat, torch.float64),
                        ("cells_of_vertex", cells_of_vertex, torch.int32)):
        if t.dtype != dt or t.device != dev or not t.is_contiguous():
            raise ValueError("'%s' must be a contiguous %s tensor on %s" % (name, dt, dev))
    if cells_of_vertex.dim() != 2 or cells_of_vertex.shape[0] != 6:
        raise ValueError("First dimension of 'cells_of_vertex' must have length 6")
    ncell, nvert = clon.numel(), vlon.numel()
    if clat.numel() != ncell or hsurf.numel() != ncell:
        raise ValueError("Inconsistent lengths of input arrays 'clon', 'clat' and 'hsurf'")
    if vlat.numel() != nvert or cells_of_vertex.shape[1] != nvert:
        raise ValueError("Inconsistent lengths of input arrays 'vlon' and 'vlat'")
    if horizon is None:
        horizon = torch.empty((num_hori, ncell), dtype=torch.float64, device=dev)
    if skyview is None:
        skyview = torch.empty(ncell, dtype=torch.float64, device=dev)
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    if start_index is not None:
        Lz = int(num_hori) * int(refine_factor)
        if (start_index.dtype != torch.int16 or start_index.device != dev
                or not start_index.is_contiguous() or tuple(start_index.shape) != (Lz, ncell)):
            raise ValueError("'start_index' must be a contiguous int16 tensor of shape "
                             "(num_hori * refine_factor, ncell) on %s" % dev)
    L = _lib.load()
    opt = _options(dev.index if dev.index is not None else -1, count_work,
                   elev_floor_deg, False, cells, kernel, advance_min, precision, mlp_params,
                   raw_index, features, mlp_every_azimuth, leaf_min, leaf_size, queue_chunk,
                   direct_launch, mlp_azimuth_groups, start_index, bvh_treelets, elev_walk,
                   occluder_cache)
    st = _lib.Stats()
    rc = L.hz_horizon_svf_device(clon.data_ptr(), clat.data_ptr(), hsurf.data_ptr(),
                                 vlon.data_ptr(), vlat.data_ptr(),
                                 cells_of_vertex.data_ptr(), horizon.data_ptr(),
                                 skyview.data_ptr(), ncell, nvert, int(num_hori),
                                 int(grid_type), float(dist_search), float(ray_org_elev),
                                 int(refine_factor), int(svf_type),
                                 C.c_void_p(stream.cuda_stream), C.byref(opt),
                                 C.byref(st))
    _lib.check(rc)
    return horizon, skyview, st.as_dict()


def occluded32(vert, vertex_of_triangle, org, dirs, tfar, *, tree=0, leaf_size=0, device=-1):
    """Any-hit flags of FP32 rays against an FP32 triangle soup on the GPU
    (the search's own query, mo_lradtopo_horayzon.cpp:446-460): ray i hits
    when it meets a triangle at 0 < t <= tfar (t in units of |dirs[i]|).
    ``tree``: 0 the 4-wide BVH of the persistent search, 1 the binary BVH."""
    vert = np.ascontiguousarray(vert, dtype=np.float32).reshape(-1, 3)
    vot = np.ascontiguousarray(vertex_of_triangle, dtype=np.int32).reshape(-1, 3)
    org = np.ascontiguousarray(org, dtype=np.float32).reshape(-1, 3)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
    if org.shape != dirs.shape:
        raise ValueError("org and dirs must have the same shape")
    hit = np.zeros(org.shape[0], dtype=np.uint8)
    rc = _lib.load().hz_occluded32(vert.ctypes.data, vert.shape[0], vot.ctypes.data,
                                   vot.shape[0], org.ctypes.data, dirs.ctypes.data,
                                   org.shape[0], float(tfar), hit.ctypes.data, int(tree),
                                   int(leaf_size), int(device))
    _lib.check(rc)
    return hit.astype(bool)


def build_mesh(clon, clat, hsurf, vlon, vlat, cells_of_vertex, grid_type, device=-1):
    """GPU mesh assembly (mo_lradtopo_horayzon.cpp:228-317).

    Returns mesh-vertex (lon, lat, h) arrays and vertex_of_triangle (ntri, 3).
    """
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (clon, clat, hsurf, vlon, vlat)]
    cov = np.ascontiguousarray(cells_of_vertex, dtype=np.int32)
    ncell, nvert = a[0].size, a[3].size
    cap_v, cap_t = ncell + nvert, max(6 * nvert, 1)
    mlon, mlat, mh = (np.empty(cap_v) for _ in range(3))
    vot = np.empty((cap_t, 3), dtype=np.int32)
    nmv, ntri = C.c_int(0), C.c_int(0)
    rc = _lib.load().hz_build_mesh(*(x.ctypes.data_as(_D) for x in a), cov.ctypes.data_as(_I),
                                   ncell, nvert, int(grid_type), mlon.ctypes.data_as(_D),
                                   mlat.ctypes.data_as(_D), mh.ctypes.data_as(_D), cap_v,
                                   vot.ctypes.data_as(_I), cap_t, C.byref(nmv),
                                   C.byref(ntri), int(device))
    _lib.check(rc)
    n = nmv.value
    return mlon[:n], mlat[:n], mh[:n], vot[:ntri.value]


def mesh_enu32(clon, clat, hsurf, vlon, vlat, cells_of_vertex, grid_type, device=-1):
    """FP32 ENU mesh vertices (n, 3) and vertex_of_triangle (ntri, 3) from the GPU."""
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (clon, clat, hsurf, vlon, vlat)]
    cov = np.ascontiguousarray(cells_of_vertex, dtype=np.int32)
    ncell, nvert = a[0].size, a[3].size
    cap_v, cap_t = ncell + nvert, max(6 * nvert, 1)
    enu = np.empty((cap_v, 3), dtype=np.float32)
    vot = np.empty((cap_t, 3), dtype=np.int32)
    nmv, ntri = C.c_int(0), C.c_int(0)
    rc = _lib.load().hz_mesh_enu32(*(x.ctypes.data_as(_D) for x in a), cov.ctypes.data_as(_I),
                                   ncell, nvert, int(grid_type), enu.ctypes.data_as(_F),
                                   cap_v, vot.ctypes.data_as(_I), cap_t, C.byref(nmv),
                                   C.byref(ntri), int(device))
    _lib.check(rc)
    return enu[:nmv.value], vot[:ntri.value]


def horizon_svf_comp_batch(domains, *, device=-1, count_work=False, elev_floor_deg=-85.0,
                           advance_min=0, return_stats=False, precision=0, mlp_params=None,
                           mlp_every_azimuth=False, kernel=0, leaf_min=0, leaf_size=0,
                           queue_chunk=0, direct_launch=False, mlp_azimuth_groups=0,
                           bvh_treelets=False, elev_walk=0, occluder_cache=True):
    """Many independent domains in one call (one persistent search launch).

    ``domains``: sequence of ``(inputs, args)`` with ``inputs`` the six arrays
    of :func:`horizon_svf_comp_py` and ``args`` its six scalar arguments
    ``(num_hori, grid_type, dist_search, ray_org_elev, refine_factor,
    svf_type)``; each domain has its own. Returns a list of ``(horizon,
    skyview)`` and, with ``return_stats``, the call statistics plus the
    per-domain completion latency in ms (from the start of the search).
    """
    keep, structs, outs = [], [], []
    for inputs, args in domains:
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in inputs[:5]]
        cov = np.ascontiguousarray(inputs[5], dtype=np.int32)
        num_hori, grid_type, dist_search, ray_org_elev, refine, svf = args
        _check_args(*arrs, cov, int(num_hori), int(grid_type), float(dist_search),
                    float(ray_org_elev), int(refine), int(svf))
        h = np.empty((int(num_hori), arrs[0].size))
        s = np.empty(arrs[0].size)
        keep += arrs + [cov]
        outs.append((h, s))
        structs.append(_lib.Domain(
            *(a.ctypes.data for a in arrs), cov.ctypes.data, h.ctypes.data, s.ctypes.data,
            arrs[0].size, arrs[3].size, int(num_hori), int(grid_type), float(dist_search),
            float(ray_org_elev), int(refine), int(svf), 0.0))
    arr = (_lib.Domain * len(structs))(*structs)
    opt = _options(device, count_work, elev_floor_deg, False, None, kernel, advance_min,
                   precision, mlp_params, mlp_every_azimuth=mlp_every_azimuth,
                   leaf_min=leaf_min, leaf_size=leaf_size, queue_chunk=queue_chunk,
                   direct_launch=direct_launch, mlp_azimuth_groups=mlp_azimuth_groups,
                   bvh_treelets=bvh_treelets, elev_walk=elev_walk,
                   occluder_cache=occluder_cache)
    st = _lib.Stats()
    rc = _lib.load().hz_horizon_svf_batch(arr, len(structs), 0, None, C.byref(opt),
                                          C.byref(st))
    _lib.check(rc)
    if return_stats:
        stats = st.as_dict()
        stats["latency_ms"] = [arr[i].latency_ms for i in range(len(structs))]
        return outs, stats
    return outs
