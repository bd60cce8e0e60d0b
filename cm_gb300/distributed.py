"""Several GPUs: independent work on each rank, no collective on the data path.

The assembly of one equations set does not shard without an exchange of the
partition-interface rows (the reference's ghost update,
distributed_matrix_vector.f90:7974-8200); this library runs one equations set
per GPU.  What does spread over GPUs is independent problems: a batch of
meshes, or the members of a parameter study, each rank assembling its own
shard.  The only communication is on the host side of a measurement: the
slowest rank's time (the job's time) and the total work.
"""
from __future__ import annotations


def _reduce(value, dist, device, op_name):
    if dist is None or not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(value, dist=None, device="cpu"):
    """The largest value over all ranks (every rank gets it)."""
    return _reduce(value, dist, device, "MAX")


def sum_over_ranks(value, dist=None, device="cpu"):
    """The sum over all ranks (every rank gets it)."""
    return _reduce(value, dist, device, "SUM")


def rank_batch_meshes(n, rank, seed=0, **kwargs):
    """Rank `rank`'s shard of a multi-GPU batched job: n independent meshes
    drawn by mesh.batch_meshes with seed + rank, so rank 0 holds the
    single-GPU batch and the shards of different ranks are different problems."""
    from .mesh import batch_meshes
    return batch_meshes(n, seed=seed + rank, **kwargs)
