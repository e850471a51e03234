"""Multi-process (gloo, world size 2) checks of the replica path: the job time is the slowest
rank's, the throughput counts every rank's units, and the C-tile split covers each tile once."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from hcorepp_gb300.replicas import partition_c_tiles


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    from hcorepp_gb300.replicas import job_throughput
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 * (rank + 1)  # rank 1 is the slow one
        value, ms = job_throughput(local_ms, 32768)
        out[rank] = (value, ms)
    finally:
        dist.destroy_process_group()


def test_job_throughput_is_max_over_ranks():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        value, ms = res[rank]
        assert ms == 200.0
        assert abs(value - world * 32768 / 0.2) < 1e-6


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_partition_covers_every_tile_once(world):
    mt, nt = 32, 32
    seen = []
    for r in range(world):
        seen += partition_c_tiles(mt, nt, world, r)
    assert sorted(seen) == sorted((i, j) for i in range(mt) for j in range(nt))
