"""In-kernel reduction (EnsembleProblem's reduction, test/qa/qa.jl:50): the
step kernels accumulate, per save point, the sum over trajectories of every
saved state and of its square, optionally without storing the ensemble.  A
reduction-only solve runs the same trajectories as a stored one (the noise
is keyed by trajectory), so its moments must equal numpy's moments of the
stored ensemble to FP64 rounding -- the additions run in no fixed order."""
import numpy as np
import pytest


def _moments(u):
    u = np.asarray(u, np.float64)
    return u.mean(0), u.var(0, ddof=1)


def _check(res, stored, rtol=1e-10):
    m, v = _moments(stored)
    scale = np.abs(m) + np.sqrt(v) + 1e-300
    assert np.max(np.abs(np.asarray(res["mean"]) - m) / scale) <= rtol
    assert np.max(np.abs(np.asarray(res["var"]) - v) / (v + 1e-300)) <= 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("device_mode", [False, True], ids=["host", "device"])
def test_reduce_sde_em(capi, de, device_mode):
    """Euler-Maruyama Lotka-Volterra paths (the SDE configuration's model):
    E[u(t)] and Var[u(t)] without storing the paths."""
    import torch
    rng = np.random.default_rng(11)
    N = 20000
    p = np.c_[np.array([1.5, 1.0, 3.0, 1.0]) * rng.uniform(0.8, 1.2, (N, 4)), np.full(N, 0.1)]
    arrs = [p, np.ones((N, 2)), np.zeros(N), np.full(N, 5.0), de.save_grid(0.0, 5.0, 0.5)]
    if device_mode:
        arrs = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrs]
    o = capi.opts_default(capi.ALG_EM)
    o.dt, o.adaptive = 1e-3, 0
    full = de.solve_arrays(de.models.lotka_volterra, o, *arrs, capi.SAVE_GRID)
    red = de.solve_arrays(de.models.lotka_volterra, o, *arrs, capi.SAVE_GRID, reduce=True,
                          store_u=False)
    assert red["u"] is None
    to_np = (lambda x: x.cpu().numpy()) if device_mode else (lambda x: x)
    assert np.array_equal(to_np(red["retcode"]), to_np(full["retcode"]))
    _check({k: to_np(red[k]) for k in ("mean", "var")}, to_np(full["u"]))


@pytest.mark.gpu
def test_reduce_ode_persistent_and_stored(capi, de):
    """Tsit5 on Lorenz with the persistent queue, reducing and storing at once."""
    rng = np.random.default_rng(12)
    N = 8000
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-8
    o.batching = capi.BATCH_PERSISTENT
    r = de.solve_arrays(de.models.lorenz, o, p, np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N),
                        np.ones(N), de.save_grid(0.0, 1.0, 0.1), capi.SAVE_GRID, reduce=True)
    _check(r, r["u"])
    np.testing.assert_allclose(r["reduce"][0], r["u"].sum(0), rtol=1e-12, atol=1e-9)


@pytest.mark.gpu
def test_reduce_team_kernel(capi, de):
    """The 16-lane team kernels (Rodas5 on the stiff Van der Pol ring)."""
    rng = np.random.default_rng(13)
    N = 512
    p = np.c_[10 ** rng.uniform(2, 3, N), np.full(N, 0.05)]
    u0 = rng.uniform(-2, 2, (N, 16))
    o = capi.opts_default(capi.ALG_RODAS5)
    o.reltol = o.abstol = 1e-5
    o.maxiters = 10 ** 6
    args = (p, u0, np.zeros(N), np.full(N, 5.0), de.save_grid(0.0, 5.0, 1.0), capi.SAVE_GRID)
    full = de.solve_arrays(de.models.vdp_ring8, o, *args)
    red = de.solve_arrays(de.models.vdp_ring8, o, *args, reduce=True, store_u=False)
    assert np.all(full["retcode"] == capi.RET_SUCCESS)
    _check(red, full["u"])
