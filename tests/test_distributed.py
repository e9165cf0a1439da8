"""World-size-2 gloo test of the sharded ensemble path on CPU: each rank
solves its contiguous slice (here with the CPU oracle standing in for the
per-rank GPU solve), no collective touches the data path, and the gathered
result equals a single-process solve."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _inputs(N):
    rng = np.random.default_rng(5)
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
    return p, u0


def _worker(rank, world, port, N, out_path):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist
    import __graft_entry__
    import oracle
    de = __graft_entry__.load_package()
    from differentialequations_gb300 import distributed
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    capi = de._capi
    grid = de.save_grid(0.0, 1.0, 0.1)
    opts = capi.opts_default(capi.ALG_TSIT5)
    opts.reltol = opts.abstol = 1e-8
    p, u0 = _inputs(N)

    def local_solve(p, u0, shared_grid):
        n = p.shape[0]
        r = oracle.solve(capi, de.models.lorenz, opts, p, u0, np.zeros(n), np.ones(n),
                         shared_grid, capi.SAVE_GRID)
        return {"u": r["u"], "retcode": r["retcode"]}

    span, res = distributed.solve_shard(local_solve, {"p": p, "u0": u0, "shared_grid": grid},
                                        rank, world)
    full = distributed.gather(res, span)
    if rank == 0:
        np.savez(out_path, **full)
    dist.destroy_process_group()


def test_two_rank_sharded_solve(tmp_path, oracle, de):
    N = 37
    out = str(tmp_path / "gathered.npz")
    mp.start_processes(_worker, args=(2, _free_port(), N, out), nprocs=2, join=True,
                       start_method="spawn")
    g = np.load(out)
    capi = de._capi
    opts = capi.opts_default(capi.ALG_TSIT5)
    opts.reltol = opts.abstol = 1e-8
    p, u0 = _inputs(N)
    ref = oracle.solve(capi, de.models.lorenz, opts, p, u0, np.zeros(N), np.ones(N),
                       de.save_grid(0.0, 1.0, 0.1), capi.SAVE_GRID)
    assert np.array_equal(g["u"], ref["u"])
    assert np.array_equal(g["retcode"], ref["retcode"])
