"""CUDA-graph replay of a solve and the autotuner (GPU), plus the tuner's
cache keys (CPU)."""
import numpy as np
import pytest


def robertson(N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
    tf = 10 ** rng.uniform(1, 5, N)
    saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
    return p, u0, np.zeros(N), tf, np.ascontiguousarray(saveat)


def rodas_opts(capi, batching):
    o = capi.opts_default(capi.ALG_RODAS5)
    o.reltol, o.abstol = 1e-6, 1e-10
    o.batching = batching
    return o


def test_cache_key_and_apply(de, tmp_path):
    capi = de._capi
    o = capi.opts_default(capi.ALG_TSIT5)
    k1 = de.tuning.cache_key("GB300", de.models.lorenz, o, 10000)
    k2 = de.tuning.cache_key("GB300", de.models.lorenz, o, 16000)
    k3 = de.tuning.cache_key("GB300", de.models.lorenz, o, 20000)
    assert k1 == k2 != k3
    path = str(tmp_path / "tune.json")
    de.tuning.save_cache(path, {k1: {"batching": 1, "block_size": 64, "ctas_per_sm": 2,
                                     "chunk": 4, "threads_per_traj": 0}})
    t = de.tuning.load_cache(path)
    de.tuning.apply_tuned(o, t[k1])
    assert (o.batching, o.block_size, o.ctas_per_sm, o.chunk) == (1, 64, 2, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("batching", ["plain", "persistent"])
def test_graph_replay_matches_solve(de, batching):
    import torch
    capi = de._capi
    host = robertson(3000, 5)
    dev = [torch.from_numpy(a).cuda() for a in host]
    o = rodas_opts(capi, capi.BATCH_PERSISTENT if batching == "persistent" else capi.BATCH_PLAIN)
    ref = de.solve_arrays(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ)
    g = de.tuning.Graph(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ)
    for _ in range(2):
        g.launch()
        assert torch.equal(g.out["u"], ref["u"]) and torch.equal(g.out["retcode"], ref["retcode"])
    # refill the inputs in place: the replay solves the new problem
    dev[0].mul_(1.01)
    ref2 = de.solve_arrays(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ)
    g.launch()
    assert torch.equal(g.out["u"], ref2["u"])
    assert not torch.equal(ref2["u"], ref["u"])
    g.close()


@pytest.mark.gpu
def test_graph_rejects_auto_and_host_memory(de):
    import torch
    capi = de._capi
    host = robertson(64, 6)
    dev = [torch.from_numpy(a).cuda() for a in host]
    o = capi.opts_default(capi.ALG_AUTO)
    with pytest.raises(capi.GBDEError) as e:
        de.tuning.Graph(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ)
    assert e.value.code == capi.GBDE_ERR_UNSUPPORTED


@pytest.mark.gpu
def test_autotune_picks_a_valid_fastest_config(de, tmp_path):
    import torch
    capi = de._capi
    host = robertson(20000, 7)
    dev = [torch.from_numpy(a).cuda() for a in host]
    o = rodas_opts(capi, capi.BATCH_PLAIN)
    cache = str(tmp_path / "tune.json")
    best, rows, cached = de.tuning.autotune(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ,
                                            cache=cache)
    assert not cached and len(rows) >= 14
    fastest = min(r["device_ms"] for r in rows)
    assert fastest < 1e29
    # the chosen options solve to the same answer as the defaults
    a = de.solve_arrays(de.models.robertson, best, *dev, capi.SAVE_PER_TRAJ)
    b = de.solve_arrays(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ)
    assert torch.equal(a["u"], b["u"])
    again, _, cached = de.tuning.autotune(de.models.robertson, o, *dev, capi.SAVE_PER_TRAJ,
                                          cache=cache)
    assert cached and again.block_size == best.block_size and again.batching == best.batching
