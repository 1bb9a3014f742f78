"""Shot sharding over ranks (one process per GPU) and the one exchange step of the
gradient path: the sum of grad/prec over every rank's shots.

The reference farms one shot per Mosaic worker and sums per-shot gradients on the
parameter's owner (stride/__init__.py:305-381, stride/core.py:565-633); here each rank
advances its shots in one batched plan and the per-rank sums are all-reduced.
"""

__all__ = ['shard_shots', 'allreduce_sum']


def shard_shots(shot_ids, rank, world):
    """Round-robin assignment of shots to ranks, as the reference's task farm assigns shots
    to workers (stride/__init__.py:133, 326)."""
    return [s for k, s in enumerate(shot_ids) if k % world == rank]


def allreduce_sum(*tensors):
    """In-place sum over ranks of torch tensors (no-op without an initialised group)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return tensors
    for t in tensors:
        dist.all_reduce(t)
    return tensors
