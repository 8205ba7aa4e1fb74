"""Autotuner for the launch knobs of the persistent horizon search.

The knobs change speed, never results (the same rays are cast and every hit
decision is the watertight test's):

* ``leaf_size``: most triangles per BVH leaf (1..8);
* ``advance_min``: lanes of a warp that must be waiting before the search
  state of the waiting lanes advances, i.e. how many rays a warp starts
  together;
* ``leaf_min``: lanes of a warp that must hold a postponed leaf before a
  triangle pass runs;
* ``queue_chunk``: consecutive cells (curve order) a warp takes from the
  work queue at a time;
* ``kernel``: the 4-wide or the binary BVH.

:func:`tune` times the device entry point on a contiguous sample of the
domain's cells (the mesh and BVH always cover the whole domain, so every
sample ray sees the full scene) and improves one knob at a time (coordinate
descent over a small grid), keeping the fastest setting. Results are cached
per GPU name and workload shape in a JSON file.
"""
from __future__ import annotations

import json
import math
import os
import threading

from . import _lib
from .horizon_svf import horizon_svf_comp_device

#: Candidate values per knob, in the order the descent visits them.
GRID = {
    "leaf_size": (2, 1, 3, 4, 6),
    "advance_min": (16, 12, 20, 8, 24),
    "leaf_min": (1, 2, 4, 8, 12),
    "queue_chunk": (32, 16, 24, 48, 64),
    "kernel": (_lib.HZ_KERNEL_PERSISTENT, _lib.HZ_KERNEL_PERSISTENT_BVH2),
}
DEFAULTS = {"leaf_size": 2, "advance_min": 16, "leaf_min": 1, "queue_chunk": 32,
            "kernel": _lib.HZ_KERNEL_PERSISTENT}
_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("HZ_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache",
                                       "horayzon_gb300_autotune.json"))


def workload_key(ncell: int, args) -> str:
    """Cache key: GPU name, log2 bucket of the cell count and the arguments
    that change the search (num_hori, grid_type, dist_search, refine_factor)."""
    import torch
    num_hori, grid_type, dist_search, _, refine_factor, _ = args
    return "%s|2^%d|%d|%d|%g|%d" % (torch.cuda.get_device_name(), int(math.log2(max(ncell, 1))),
                                    int(num_hori), int(grid_type), float(dist_search),
                                    int(refine_factor))


def _load_cache(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time(inputs, args, cells, knobs, reps, stream):
    best = math.inf
    for _ in range(reps):
        _, _, st = horizon_svf_comp_device(*inputs, *args, cells=cells, stream=stream, **knobs)
        best = min(best, st["ms_trace"])
    return best


def tune(inputs, args, sample_cells: int = 250_000, reps: int = 2, rounds: int = 2,
         grid: dict | None = None, use_cache: bool = True, stream=None) -> dict:
    """Fastest knob setting for this workload.

    ``inputs``: the six device tensors of :func:`horizon_svf_comp_device`
    (clon, clat, hsurf, vlon, vlat, cells_of_vertex); ``args``: (num_hori,
    grid_type, dist_search, ray_org_elev, refine_factor, svf_type). Returns a
    dict of keyword arguments for the entry points plus ``"ms_sample"`` (the
    sample's search time with it) and ``"trials"``.
    """
    ncell = int(inputs[0].numel())
    key = workload_key(ncell, args)
    path = cache_path()
    if use_cache:
        with _lock:
            hit = _load_cache(path).get(key)
        if hit:
            return dict(hit, cached=True)
    grid = grid or GRID
    n = min(sample_cells, ncell)
    begin = (ncell - n) // 2
    cells = (begin, begin + n)
    # Start from the first value of each knob in the grid (the library
    # defaults head the built-in grid).
    cur = {k: (grid[k][0] if k in grid else v) for k, v in DEFAULTS.items()}
    _time(inputs, args, cells, cur, 1, stream)  # warm-up (allocations, first launch)
    best_ms = _time(inputs, args, cells, cur, reps, stream)
    trials = 1
    for _ in range(rounds):
        changed = False
        for knob, values in grid.items():
            for v in values:
                if v == cur[knob]:
                    continue
                cand = dict(cur, **{knob: v})
                ms = _time(inputs, args, cells, cand, reps, stream)
                trials += 1
                if ms < best_ms * 0.995:
                    best_ms, cur, changed = ms, cand, True
        if not changed:
            break
    result = dict(cur, ms_sample=best_ms, trials=trials, sample_cells=n)
    if use_cache:
        with _lock:
            data = _load_cache(path)
            data[key] = result
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + ".%d.tmp" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1)
            os.replace(tmp, path)
    return dict(result, cached=False)


def knobs(result: dict) -> dict:
    """The entry-point keyword arguments of a :func:`tune` result."""
    return {k: result[k] for k in DEFAULTS}
