"""Cell sharding across ranks: ranges, stitching and the torch.distributed
gather, exercised with world_size 2 over gloo on the CPU (each rank computes
its range with the CPU oracle standing in for its GPU)."""
import os
import socket

import numpy as np
import pytest

from horayzon_extpar_gb300 import shard

ARGS = (16, 1, 20000.0, 0.2, 1, 2)


def test_cell_ranges_cover():
    for n, w in [(10, 3), (7, 7), (1000, 4), (5, 8)]:
        r = shard.cell_ranges(n, w)
        assert r[0][0] == 0 and r[-1][1] == n and len(r) == w
        assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
        sizes = [e - b for b, e in r]
        assert max(sizes) - min(sizes) <= 1


def test_assemble_rejects_gaps_and_overlaps():
    h = np.zeros((2, 5))
    s = np.zeros(5)
    with pytest.raises(ValueError):
        shard.assemble([(0, 5, h, s), (4, 9, h, s)], 9, 2)
    with pytest.raises(ValueError):
        shard.assemble([(0, 5, h, s)], 9, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, result_path):
    import torch.distributed as dist

    from horayzon_extpar_gb300 import synthetic
    from oracle import api as oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = synthetic.make_domain(edge_km=2.5, box_km=40.0, seed=9)
    b, e = shard.cell_ranges(d.ncell, world)[rank]
    h, s, st = oracle.horizon_svf(*d.inputs(), *ARGS, cells=np.arange(b, e), nthreads=1)
    hf, sf, rays = shard.gather(h[:, b:e], s[b:e], st["num_rays"], d.ncell, ARGS[0])
    if rank == 0:
        np.savez(result_path, horizon=hf, skyview=sf, rays=rays)
    dist.barrier()
    dist.destroy_process_group()


def test_gather_two_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    from horayzon_extpar_gb300 import synthetic
    from oracle import api as oracle

    path = str(tmp_path / "out.npz")
    mp.start_processes(_worker, args=(2, _free_port(), path), nprocs=2, join=True,
                       start_method="spawn")
    z = np.load(path)
    d = synthetic.make_domain(edge_km=2.5, box_km=40.0, seed=9)
    h, s, st = oracle.horizon_svf(*d.inputs(), *ARGS)
    np.testing.assert_array_equal(z["horizon"], h)
    np.testing.assert_array_equal(z["skyview"], s)
    assert int(z["rays"]) == st["num_rays"]
