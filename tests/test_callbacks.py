"""Callbacks (ContinuousCallback / DiscreteCallback, test/qa/qa.jl:24,36): the
reference's own callback test (test/core.jl:60-79, Lorenz with a continuous
callback on t - 0.5 and a discrete one on t >= 0.5, both with a no-op
affect!) and event location pinned to an analytic solution -- a bouncing
ball, whose piecewise-quadratic trajectory the Runge-Kutta stages and the
dense output reproduce exactly, so every event time and post-event state has
a closed form."""
import numpy as np
import pytest

BALL_F = "du[0] = u[1];\ndu[1] = -p[0];"  # x'' = -g; p = [g, e]
BOUNCE = "u[1] = -p[1] * u[1];"            # restitution e


def _skip_without_nvrtc(capi, fn):
    try:
        fn()
    except capi.GBDEError as e:
        if e.code == capi.GBDE_ERR_UNSUPPORTED:
            pytest.skip("NVRTC unavailable: %s" % e)
        raise


def test_callback_compile_builtin_and_user_models(capi, de):
    cc = de.ContinuousCallback("g = t - 0.5;")
    dc = de.DiscreteCallback("g = t >= 0.5;")
    ball = de.ODEFunction(BALL_F, 2, 2, name="ball_compile")
    bc = de.ContinuousCallback("g = u[0];", BOUNCE)
    L = capi.lib()
    for model, cb in ((capi.MODEL_LORENZ, cc), (capi.MODEL_LORENZ, dc), (ball.id, bc)):
        for alg in (capi.ALG_TSIT5, capi.ALG_RODAS5):
            _skip_without_nvrtc(capi, lambda: capi.check(
                L.gbde_callback_compile(model, alg, capi.PREC_FP64, cb.id)))
    _skip_without_nvrtc(capi, lambda: capi.check(
        L.gbde_callback_compile(ball.id, capi.ALG_RODAS5, capi.PREC_F32X2, bc.id)))


def test_callback_compile_error_and_validation(capi, de):
    bad = de.ContinuousCallback("g = no_such_variable;")
    with pytest.raises(capi.GBDEError) as e:
        _skip_without_nvrtc(capi, lambda: capi.check(capi.lib().gbde_callback_compile(
            capi.MODEL_LORENZ, capi.ALG_TSIT5, capi.PREC_FP64, bad.id)))
    assert e.value.code == capi.GBDE_ERR_INVALID and "no_such_variable" in str(e.value)
    with pytest.raises(capi.GBDEError):
        capi.check(capi.lib().gbde_callback_compile(capi.MODEL_LORENZ, capi.ALG_TSIT5,
                                                    capi.PREC_FP64, 10 ** 6))


# ------------------------------------------------------------------ GPU
def _lorenz_ens(de, N=64):
    prob = de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8.0 / 3.0])
    return de.EnsembleProblem(prob)


@pytest.mark.gpu
def test_reference_callbacks_lorenz(capi, de, oracle):
    """test/core.jl:60-79 on the GPU: both callbacks return Success.  The
    no-op discrete affect restarts Tsit5 at the same state, so the solution is
    bit-identical to the solve without callback; the continuous one cuts the
    step at t = 0.5 and stays within tolerance of the FP64 oracle."""
    prob = de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8.0 / 3.0])
    kw = dict(saveat=0.1, reltol=1e-8, abstol=1e-8)
    ref = de.solve(prob, de.Tsit5(), **kw)
    cc = de.solve(prob, de.Tsit5(), callback=de.ContinuousCallback("g = t - 0.5;"), **kw)
    dc = de.solve(prob, de.Tsit5(), callback=de.DiscreteCallback("g = t >= 0.5;"), **kw)
    assert cc.retcode == de.ReturnCode.Success and dc.retcode == de.ReturnCode.Success
    assert len(cc.t) == 11 and np.array_equal(np.asarray(cc.u[0]), [1.0, 0.0, 0.0])
    assert np.array_equal(np.asarray(dc.u), np.asarray(ref.u))
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-8
    orc = oracle.solve(capi, de.models.lorenz, o, np.array([[10.0, 28.0, 8.0 / 3.0]]),
                       np.array([[1.0, 0.0, 0.0]]), np.zeros(1), np.ones(1),
                       de.save_grid(0.0, 1.0, 0.1), capi.SAVE_GRID)
    assert oracle.weighted_error(np.asarray(cc.u)[None], orc["u"], 1e-8, 1e-8) <= 10.0


def _ball_truth(h0, g, e, ts):
    """Analytic bouncing ball from rest at height h0: (x, v) at times ts.
    The impacts accumulate at t1 (1 + 2e / (1 - e)) (t1 the first impact);
    ts must end before that."""
    x = np.empty_like(ts)
    v = np.empty_like(ts)
    t_hit = np.sqrt(2 * h0 / g)        # first impact
    if ts[-1] >= t_hit * (1 + 2 * e / (1 - e)):
        raise ValueError("the save times reach the accumulation point of the impacts")
    v_up = e * g * t_hit               # speed after it
    start, vstart, t_next = 0.0, 0.0, t_hit
    pos0 = h0
    for k, t in enumerate(ts):
        bounces = 0
        while t > t_next:              # advance through impacts before t
            start, pos0, vstart = t_next, 0.0, v_up
            t_next = start + 2 * v_up / g
            v_up *= e
            bounces += 1
            if bounces > 1000:
                raise ValueError("too many impacts")
        dt = t - start
        x[k] = pos0 + vstart * dt - 0.5 * g * dt * dt
        v[k] = vstart - g * dt
    return x, v


@pytest.mark.gpu
@pytest.mark.parametrize("alg", ["Tsit5", "Vern7"])
@pytest.mark.parametrize("precision", ["fp64", "f32x2"])
def test_bouncing_ball_events_exact(capi, de, alg, precision):
    """Impacts located on the dense output: the saved states follow the
    analytic piecewise-quadratic solution through several bounces (the span
    ends well before the impacts accumulate: t1 (1 + 2e/(1-e)) >= 2.3), with
    the FP64 steppers and with the compact FP32-pair ones (their dense output
    at arbitrary theta and their restart after each affect)."""
    rng = np.random.default_rng(3)
    N = 512
    g = rng.uniform(5.0, 15.0, N)
    e = rng.uniform(0.8, 0.9, N)
    h0 = rng.uniform(0.5, 2.0, N)
    ball = de.ODEFunction(BALL_F, 2, 2, name="ball_%s_%s" % (alg, precision))
    cb = de.ContinuousCallback("g = u[0];", BOUNCE)
    ens = de.EnsembleProblem(de.ODEProblem(ball, [1.0, 0.0], (0.0, 1.0), [9.8, 0.8]),
                             batch=lambda prob, n: {"p": np.c_[g, e], "u0": np.c_[h0, np.zeros(N)]})
    sol = de.solve(ens, getattr(de, alg)(),
                   de.EnsembleGB300(batching="persistent", precision=precision),
                   trajectories=N, saveat=0.05, reltol=1e-10, abstol=1e-10, callback=cb)
    assert sol.converged
    ts = de.save_grid(0.0, 1.0, 0.05)
    err = 0.0
    for i in range(N):
        x, v = _ball_truth(h0[i], g[i], e[i], ts)
        err = max(err, np.abs(sol.U[i, :, 0] - x).max(), np.abs(sol.U[i, :, 1] - v).max() / g[i])
    assert err <= 1e-8, err


@pytest.mark.gpu
def test_terminating_callback(capi, de):
    """terminate at the first impact: ReturnCode.Terminated, the end time is
    the analytic impact time, saves before it are exact and later slots NaN."""
    N = 256
    rng = np.random.default_rng(4)
    g = rng.uniform(5.0, 15.0, N)
    h0 = rng.uniform(0.5, 2.0, N)
    ball = de.ODEFunction(BALL_F, 2, 2, name="ball_term")
    cb = de.ContinuousCallback("g = u[0];", terminate=True)
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-10
    o.callback = cb.id
    grid = de.save_grid(0.0, 2.0, 0.01)
    r = de.solve_arrays(ball, o, np.c_[g, np.full(N, 0.8)], np.c_[h0, np.zeros(N)],
                        np.zeros(N), np.full(N, 2.0), grid, capi.SAVE_GRID)
    assert np.all(r["retcode"] == capi.RET_TERMINATED)
    t_hit = np.sqrt(2 * h0 / g)
    np.testing.assert_allclose(r["t_end"], t_hit, rtol=1e-12)
    for i in range(N):
        before = grid <= t_hit[i] * (1 - 1e-12)
        np.testing.assert_allclose(r["u"][i, before, 0], h0[i] - 0.5 * g[i] * grid[before] ** 2,
                                   atol=1e-10)
        assert np.all(np.isnan(r["u"][i, grid > t_hit[i] * (1 + 1e-12), 0]))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "f32x2"])
def test_rodas5_event_on_robertson(capi, de, prec):
    """A continuous callback with the stiff method (and its FP32-pair
    stepper): terminate when y1 falls to 0.8 (between t = 4 and 133 for these
    rates); the event time matches the root of a fine dense sampling of the
    solve without callback."""
    N = 128
    rng = np.random.default_rng(5)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-0.3, 0.3, (N, 3))
    u0, t0, tf = np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), np.full(N, 200.0)
    o = capi.opts_default(capi.ALG_RODAS5)
    o.reltol, o.abstol = 1e-8, 1e-12
    o.precision = capi.PREC_F32X2 if prec == "f32x2" else capi.PREC_FP64
    fine = np.linspace(0.0, 200.0, 40001)
    ref = de.solve_arrays(de.models.robertson, o, p, u0, t0, tf, fine, capi.SAVE_GRID)
    cb = de.ContinuousCallback("g = u[0] - 0.8;", terminate=True)
    o.callback = cb.id
    r = de.solve_arrays(de.models.robertson, o, p, u0, t0, tf, fine[:2], capi.SAVE_GRID)
    assert np.all(r["retcode"] == capi.RET_TERMINATED)
    y = ref["u"][:, :, 0]
    assert np.all((y < 0.8).any(axis=1))
    k = np.argmax(y < 0.8, axis=1)  # first sample below 0.8
    t_lin = fine[k - 1] + (y[np.arange(N), k - 1] - 0.8) / (
        y[np.arange(N), k - 1] - y[np.arange(N), k]) * (fine[k] - fine[k - 1])
    np.testing.assert_allclose(r["t_end"], t_lin, rtol=1e-5)
