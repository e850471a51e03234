"""Multi-GPU form of the TLR multiply: independent replicas (one process per GPU).

A tile-matrix multiply has no exchange step: every C tile's k-chain is independent of the
others, so N GPUs either run N independent multiplies (replicas, what the throughput
measurement does) or split the C tiles between them (`partition_c_tiles`) with each GPU
holding the A row-panels and B column-panels its tiles need.  Neither needs a collective on the
data path; the only cross-process step is reporting: the job's time is the slowest rank's time.
"""
from __future__ import annotations


def partition_c_tiles(mt: int, nt: int, world: int, rank: int):
    """C tiles (i, j) owned by `rank`: a 1-D cyclic split of the column-major tile index."""
    return [(idx % mt, idx // mt) for idx in range(mt * nt) if idx % world == rank]


def job_throughput(local_ms: float, units_per_rank: int, group=None, device=None):
    """Whole-job throughput over all ranks: (world * units_per_rank) / max over ranks of local_ms.

    Returns (units per second, max ms).  Without an initialised process group it is the local value.
    """
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return units_per_rank / (local_ms * 1e-3), local_ms
    world = dist.get_world_size(group)
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=device or "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    ms = float(t.item())
    return world * units_per_rank / (ms * 1e-3), ms
