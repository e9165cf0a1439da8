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


def solve_sharded(solver, devices, model, opts, p, u0, t0, tf, saveat, save_kind,
                  u_dtype="f64", reduce=False, events=None):
    """One call, several GPUs of this process: contiguous trajectory slices
    (shard_range), one per entry of `devices`, each solved by
    `solver(model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype=,
    device=, out=, reduce=)` (api.solve_arrays on host arrays) in its own
    thread -- the C calls release the interpreter lock, and each device has
    its own context, stream and staging buffers.  Every slice writes straight
    into its rows of the full output arrays (C order, trajectory-major), so
    nothing is copied to reassemble the ensemble; per-save-point reduction
    sums add up across slices; events=K keeps K saves at callback events per
    trajectory.  No collective: trajectories never interact.
    The replacement of EnsembleDistributed / EnsembleSplitThreads
    (test/qa/qa.jl:49,53) within one node."""
    import threading
    N = int(u0.shape[0])
    n_save = int(saveat.shape[-1]) if saveat is not None else 0
    res = {"u": np.empty((N, n_save, model.n_state), np.float32 if u_dtype == "f32" else
                         np.float64),
           "retcode": np.empty(N, np.int32)}
    for k in ("naccept", "nreject", "nf", "method"):
        res[k] = np.empty(N, np.int32)
    res["t_end"] = np.empty(N, np.float64)
    res["dt_first"] = np.empty(N, np.float64)
    if events is not None:  # saves at callback events, K per trajectory
        res["ev_t"] = np.empty((N, int(events)), np.float64)
        res["ev_u"] = np.empty((N, int(events), model.n_state), res["u"].dtype)
        res["ev_count"] = np.empty(N, np.int32)
    per_traj_save = saveat is not None and saveat.ndim == 2
    spans = [shard_range(N, r, len(devices)) for r in range(len(devices))]
    parts, errors = [None] * len(devices), [None] * len(devices)

    def run(r):
        a, b = spans[r]
        try:
            out = {k: v[a:b] for k, v in res.items()}
            parts[r] = solver(model, opts, p[a:b], u0[a:b], t0[a:b], tf[a:b],
                              saveat[a:b] if per_traj_save else saveat, save_kind,
                              u_dtype=u_dtype, device=devices[r], out=out, reduce=reduce,
                              events=events)
        except Exception as e:  # re-raised on the calling thread
            errors[r] = e

    threads = [threading.Thread(target=run, args=(r,)) for r in range(len(devices))
               if spans[r][1] > spans[r][0]]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for e in errors:
        if e is not None:
            raise e
    done = [x for x in parts if x is not None]
    res["device_ms"] = max((x["device_ms"] for x in done), default=0.0)
    res["total_ms"] = max((x["total_ms"] for x in done), default=0.0)
    res["spans"] = spans
    if reduce:
        res["reduce"] = sum(x["reduce"] for x in done)
        s1, s2 = res["reduce"][0], res["reduce"][1]
        res["mean"] = s1 / N
        res["var"] = (s2 - s1 * s1 / N) / (N - 1) if N > 1 else s1 * float("nan")
    return res


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
