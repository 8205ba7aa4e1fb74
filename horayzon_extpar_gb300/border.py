"""Distance of each cell to the mesh border (functions.py:58-97) on the GPU.

The reference's verification masks cells closer to the domain edge than the
search distance (verification.py:302-304): their horizons look through the
border into empty space, so they differ from a larger domain's for reasons
that have nothing to do with the horizon computation. This is the same
diagnostic, computed by ``hz_distance_to_border``.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def distance_to_border(clon, clat, vlon, vlat, cells_of_vertex) -> np.ndarray:
    """Chord distance [km] from each cell circumcentre to the nearest border
    vertex (an ICON vertex with a -2 entry in ``cells_of_vertex``), as
    functions.distance_to_border returns it; +inf if there is none."""
    clon = np.ascontiguousarray(clon, dtype=np.float64)
    clat = np.ascontiguousarray(clat, dtype=np.float64)
    vlon = np.ascontiguousarray(vlon, dtype=np.float64)
    vlat = np.ascontiguousarray(vlat, dtype=np.float64)
    cov = np.ascontiguousarray(cells_of_vertex, dtype=np.int32)
    if clon.shape != clat.shape or vlon.shape != vlat.shape:
        raise ValueError("Inconsistent lengths of input arrays")
    if cov.ndim != 2 or cov.shape[0] != 6 or cov.shape[1] != vlon.size:
        raise ValueError("'cells_of_vertex' must have shape (6, number of vertices)")
    dist = np.empty(clon.size, dtype=np.float64)
    rc = _lib.load().hz_distance_to_border(clon.ctypes.data, clat.ctypes.data,
                                           vlon.ctypes.data, vlat.ctypes.data, cov.ctypes.data,
                                           clon.size, vlon.size, dist.ctypes.data, 0, None)
    _lib.check(rc)
    return dist


def distance_to_border_device(clon, clat, vlon, vlat, cells_of_vertex, out=None, stream=None):
    """The same on CUDA tensors (float64 / int32, contiguous, one device)."""
    import torch
    dev = clon.device
    if out is None:
        out = torch.empty(clon.numel(), dtype=torch.float64, device=dev)
    s = stream or torch.cuda.current_stream(dev)
    rc = _lib.load().hz_distance_to_border(clon.data_ptr(), clat.data_ptr(), vlon.data_ptr(),
                                           vlat.data_ptr(), cells_of_vertex.data_ptr(),
                                           clon.numel(), vlon.numel(), out.data_ptr(), 1,
                                           s.cuda_stream)
    _lib.check(rc)
    return out
