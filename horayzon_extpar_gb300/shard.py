"""Multi-GPU partitioning of one domain's cells (one process per GPU).

Cells are independent given the mesh (the reference's parallel_reduce over
cells has no cross-cell dependency besides the ray count,
mo_lradtopo_horayzon.cpp:686-761), so a domain shards into contiguous cell
ranges: every rank builds the whole mesh and BVH (cheap, no exchange) and
traces only its range; the only collective is the final gather of the
horizon/skyview slices and the sum of the ray counts. Independent domains
(batches of regional grids) need no collective at all.

``horizon_svf_sharded`` is that path end to end: each rank of a
torch.distributed group calls the library's device entry point on its own
GPU for its cell range, then the ranks all-gather the slices.
"""
from __future__ import annotations

import numpy as np


def cell_ranges(ncell: int, world: int) -> list[tuple[int, int]]:
    """Balanced contiguous [begin, end) ranges, one per rank."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    edges = [(ncell * r) // world for r in range(world + 1)]
    return [(edges[r], edges[r + 1]) for r in range(world)]


def assemble(parts, ncell: int, num_hori: int):
    """Stitch per-rank (begin, end, horizon_slice, skyview_slice) into full arrays."""
    horizon = np.full((num_hori, ncell), np.nan)
    skyview = np.full(ncell, np.nan)
    covered = np.zeros(ncell, dtype=bool)
    for begin, end, h, s in parts:
        h = np.asarray(h).reshape(num_hori, end - begin)
        horizon[:, begin:end] = h
        skyview[begin:end] = np.asarray(s)
        if covered[begin:end].any():
            raise ValueError("overlapping cell ranges")
        covered[begin:end] = True
    if not covered.all():
        raise ValueError("cell ranges do not cover the domain")
    return horizon, skyview


def gather(horizon_local, skyview_local, rays_local: int, ncell: int, num_hori: int,
           group=None):
    """All-gather the rank slices over torch.distributed (NCCL or gloo).

    ``horizon_local`` is (num_hori, end - begin) for this rank's range.
    Returns the full horizon, skyview and the total ray count on every rank.
    """
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    ranges = cell_ranges(ncell, world)
    width = max(max(e - b for b, e in ranges), 1)
    dev = horizon_local.device if isinstance(horizon_local, torch.Tensor) else "cpu"
    buf = torch.full((num_hori + 1, width), float("nan"), dtype=torch.float64, device=dev)
    b, e = ranges[rank]
    buf[:num_hori, : e - b] = torch.as_tensor(horizon_local, dtype=torch.float64)
    buf[num_hori, : e - b] = torch.as_tensor(skyview_local, dtype=torch.float64)
    out = [torch.empty_like(buf) for _ in range(world)]
    dist.all_gather(out, buf, group=group)
    rays = torch.tensor([int(rays_local)], dtype=torch.int64, device=dev)
    dist.all_reduce(rays, group=group)
    parts = []
    for r, (rb, re_) in enumerate(ranges):
        o = out[r].cpu().numpy()
        parts.append((rb, re_, o[:num_hori, : re_ - rb], o[num_hori, : re_ - rb]))
    h, s = assemble(parts, ncell, num_hori)
    return h, s, int(rays.item())


def horizon_svf_sharded(clon, clat, hsurf, vlon, vlat, cells_of_vertex, num_hori, grid_type,
                        dist_search, ray_org_elev, refine_factor, svf_type, *, group=None,
                        device=None, return_stats=False, **options):
    """One domain over the ranks of a torch.distributed group.

    Every rank passes the whole domain (the reference's arrays, numpy or
    torch). Each rank copies it to its GPU (``device``, default
    ``cuda:<LOCAL_RANK>``), builds the mesh and BVH there, and traces its
    contiguous cell range (:func:`cell_ranges`) with
    ``horizon_svf_comp_device(..., cells=(begin, end))``; then the slices are
    all-gathered (on the GPU for an NCCL group, through host memory
    otherwise) and every rank returns the full ``horizon`` (num_hori, ncell)
    and ``skyview`` (ncell) as numpy arrays, bit-identical to a single call
    on one GPU. ``options`` go to the device entry point (kernel knobs,
    precision, learned start). With ``return_stats`` a third value holds the
    total ray count and this rank's phase times.
    """
    import os

    import torch
    import torch.distributed as dist

    from .horizon_svf import horizon_svf_comp_device

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    if device is None:
        device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device(device)

    def on_dev(a, dtype):
        t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))
        return t.to(device=dev, dtype=dtype).contiguous()

    f64 = [on_dev(a, torch.float64) for a in (clon, clat, hsurf, vlon, vlat)]
    cov = on_dev(cells_of_vertex, torch.int32)
    ncell = f64[0].numel()
    num_hori = int(num_hori)
    b, e = cell_ranges(ncell, world)[rank]
    horizon = torch.empty((num_hori, ncell), dtype=torch.float64, device=dev)
    skyview = torch.empty(ncell, dtype=torch.float64, device=dev)
    st = {"num_rays": 0}
    if e > b:
        _, _, st = horizon_svf_comp_device(*f64, cov, num_hori, grid_type, dist_search,
                                           ray_org_elev, refine_factor, svf_type,
                                           horizon=horizon, skyview=skyview, cells=(b, e),
                                           **options)
    h_loc, s_loc = horizon[:, b:e], skyview[b:e]
    if dist.get_backend(group) != "nccl":
        h_loc, s_loc = h_loc.cpu(), s_loc.cpu()
    h, s, rays = gather(h_loc, s_loc, st["num_rays"], ncell, num_hori, group=group)
    if return_stats:
        st = dict(st)
        st["num_rays_total"] = rays
        st["cell_range"] = (b, e)
        return h, s, st
    return h, s
