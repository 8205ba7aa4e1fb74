"""The sharded multi-GPU path with the library in the loop: two ranks (gloo
process group, both on the one GPU of the test machine, each with its own
CUDA context and stream) trace their cell ranges of one domain through
horizon_svf_comp_device and all-gather the slices (shard.horizon_svf_sharded).
The ranks' kernels are independent (no kernel waits on another rank), and the
gathered result must equal a single call on one GPU bit for bit."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ARGS = (24, 1, 30000.0, 0.2, 1, 2)
DOMAIN = dict(edge_km=1.5, box_km=90.0, seed=41)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, result_path, options):
    import torch.distributed as dist

    from horayzon_extpar_gb300 import shard, synthetic

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    d = synthetic.make_domain(**DOMAIN)
    h, s, st = shard.horizon_svf_sharded(*d.inputs(), *ARGS, device="cuda:0",
                                         return_stats=True, **options)
    if rank == 0:
        np.savez(result_path, horizon=h, skyview=s, rays=st["num_rays_total"])
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("options", [{}, {"precision": 1}])
def test_sharded_domain_equals_single_call(tmp_path, options):
    import torch.multiprocessing as mp

    from horayzon_extpar_gb300 import horizon_svf_comp_py, synthetic

    path = str(tmp_path / "sharded.npz")
    mp.start_processes(_worker, args=(2, _free_port(), path, options), nprocs=2, join=True,
                       start_method="spawn")
    z = np.load(path)
    d = synthetic.make_domain(**DOMAIN)
    h, s, st = horizon_svf_comp_py(*d.inputs(), *ARGS, return_stats=True, **options)
    np.testing.assert_array_equal(z["horizon"], h)
    np.testing.assert_array_equal(z["skyview"], s)
    assert int(z["rays"]) == st["num_rays"]
