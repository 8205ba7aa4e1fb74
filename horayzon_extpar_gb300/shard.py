"""Multi-GPU partitioning of one domain's cells (one process per GPU).

Cells are independent given the mesh (the reference's parallel_reduce over
cells has no cross-cell dependency besides the ray count,
mo_lradtopo_horayzon.cpp:686-761), so a domain shards into contiguous cell
ranges: every rank builds the whole mesh and BVH (cheap, no exchange) and
traces only its range; the only collective is the final gather of the
horizon/skyview slices and the sum of the ray counts. Independent domains
(batches of regional grids) need no collective at all.
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
    width = max(e - b for b, e in ranges)
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
