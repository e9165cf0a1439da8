"""Trajectory sharding across GPUs (one process per GPU).

Trajectories never interact, so an ensemble of N trajectories splits into
contiguous index ranges, one per rank; each rank solves its range on its own
GPU with no collective on the data path (weak scaling).  This replaces the
reference's multi-process ensemble algorithms EnsembleDistributed /
EnsembleSplitThreads (test/qa/qa.jl:49,53), which pmap trajectories over Julia
worker processes.  `gather` is an optional host-side collection for callers
that want the whole ensemble on one rank.
"""
import numpy as np


def shard_range(n, rank, world):
    """[begin, end) of rank's contiguous slice; sizes differ by at most 1."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(int(n), int(world))
    begin = rank * base + min(rank, extra)
    end = begin + base + (1 if rank < extra else 0)
    return begin, end


def solve_shard(solve_fn, arrays, rank, world):
    """Solve this rank's slice.  `arrays` maps names to per-trajectory arrays
    (leading dimension N) or shared arrays (key prefixed with 'shared_');
    `solve_fn(**slice)` runs the local solve and returns a dict of
    per-trajectory result arrays."""
    n = None
    for k, v in arrays.items():
        if not k.startswith("shared_"):
            n = v.shape[0] if n is None else n
            if v.shape[0] != n:
                raise ValueError("inconsistent leading dimensions")
    a, b = shard_range(n or 0, rank, world)
    local = {k: (v if k.startswith("shared_") else v[a:b]) for k, v in arrays.items()}
    return (a, b), solve_fn(**local)


def gather(result, span, group=None, dst=0):
    """Collect every rank's result slices on rank `dst` (host objects via
    torch.distributed.gather_object).  Returns the concatenated dict on dst,
    None elsewhere."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    payload = (span, {k: np.asarray(v) for k, v in result.items()})
    objs = [None] * world if rank == dst else None
    dist.gather_object(payload, objs, dst=dst, group=group)
    if rank != dst:
        return None
    objs.sort(key=lambda o: o[0][0])
    keys = objs[0][1].keys()
    return {k: np.concatenate([o[1][k] for o in objs]) for k in keys}
