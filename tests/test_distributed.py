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


def _oracle_solver(oracle, calls):
    """Stand-in for api.solve_arrays on the CPU (same signature; writes into
    `out`), recording which device each slice was given."""
    def solver(model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype="f64", device=0, out=None,
               reduce=False, events=None):
        r = oracle.solve(None, model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype=u_dtype)
        for k in ("u", "retcode", "naccept", "nreject", "nf", "t_end"):
            out[k][...] = r[k]
        if events is not None:  # stand-in event saves: t_end and u0, naccept times over
            out["ev_count"][...] = r["naccept"]
            out["ev_t"][...] = r["t_end"][:, None]
            out["ev_u"][...] = u0[:, None, :]
        calls.append((device, len(p)))
        res = dict(out, device_ms=1.0, total_ms=2.0)
        if reduce:
            u = np.asarray(r["u"], np.float64)
            res["reduce"] = np.stack([u.sum(0), (u * u).sum(0)])
        return res
    return solver


@pytest.mark.parametrize("ndev", [1, 2, 3, 5])
def test_solve_sharded_reassembles_bitwise(oracle, de, ndev):
    """One-call sharding over several GPUs (EnsembleGB300(devices=...)):
    contiguous slices, each written into its rows of the full outputs, equal
    a single solve bitwise; per-trajectory save times are sliced with their
    trajectories; reduction sums add up across slices."""
    from differentialequations_gb300 import distributed
    rng = np.random.default_rng(8)
    N = 41
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
    t0, tf = np.zeros(N), 10 ** rng.uniform(1, 3, N)
    saveat = tf[:, None] * np.linspace(0.1, 1.0, 6)
    opts = oracle.opts_default(oracle.ALG_RODAS5)
    opts.reltol, opts.abstol = 1e-6, 1e-10
    M = oracle.ModelRef(oracle.MODEL_ROBERTSON)
    calls = []
    got = distributed.solve_sharded(_oracle_solver(oracle, calls), list(range(10, 10 + ndev)), M,
                                    opts, p, u0, t0, tf, saveat, oracle.SAVE_PER_TRAJ,
                                    reduce=True, events=3)
    ref = oracle.solve(None, M, opts, p, u0, t0, tf, saveat, oracle.SAVE_PER_TRAJ)
    for k in ("u", "retcode", "naccept", "nreject", "t_end"):
        assert np.array_equal(got[k], ref[k]), k
    # event saves (callback save_positions) land in their trajectories' rows
    assert np.array_equal(got["ev_count"], ref["naccept"])
    assert np.array_equal(got["ev_t"], np.repeat(ref["t_end"][:, None], 3, axis=1))
    assert np.array_equal(got["ev_u"], np.repeat(u0[:, None, :], 3, axis=1))
    assert sorted(d for d, _ in calls) == list(range(10, 10 + ndev))
    sizes = [b - a for a, b in got["spans"]]
    assert sum(sizes) == N and max(sizes) - min(sizes) <= 1
    assert [a for a, _ in got["spans"]] == [0] + list(np.cumsum(sizes)[:-1])
    np.testing.assert_allclose(got["mean"], ref["u"].mean(0), rtol=1e-12, atol=1e-15)
