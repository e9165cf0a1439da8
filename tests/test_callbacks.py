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
    no-op discrete affect restarts Tsit5 at the same state, so the saveat
    points are bit-identical to the solve without callback; the continuous
    one cuts the step at t = 0.5 and stays within tolerance of the FP64
    oracle.  With the default save_positions the discrete callback adds
    (t, u) before and after its affect at every step end from t = 0.5 on
    (before: not at tf, a saveat point), the continuous one (no affect) at
    most one save at its event, before it."""
    prob = de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8.0 / 3.0])
    kw = dict(saveat=0.1, reltol=1e-8, abstol=1e-8)
    grid = de.save_grid(0.0, 1.0, 0.1)
    ref = de.solve(prob, de.Tsit5(), **kw)
    quiet = dict(save_positions=(False, False))
    cc = de.solve(prob, de.Tsit5(), callback=de.ContinuousCallback("g = t - 0.5;", **quiet), **kw)
    dc = de.solve(prob, de.Tsit5(), callback=de.DiscreteCallback("g = t >= 0.5;", **quiet), **kw)
    assert cc.retcode == de.ReturnCode.Success and dc.retcode == de.ReturnCode.Success
    assert len(cc.t) == 11 and np.array_equal(np.asarray(cc.u[0]), [1.0, 0.0, 0.0])
    assert np.array_equal(np.asarray(dc.u), np.asarray(ref.u))
    # the reference's default save_positions = (true, true)
    cc2 = de.solve(prob, de.Tsit5(), callback=de.ContinuousCallback("g = t - 0.5;"), **kw)
    assert len(cc2.t) in (11, 12)
    extra = ~np.isin(cc2.t, grid)
    assert np.all(np.abs(cc2.t[extra] - 0.5) <= 1e-12)
    dc2 = de.solve(prob, de.Tsit5(), callback=de.DiscreteCallback("g = t >= 0.5;"), **kw)
    on_grid = np.isin(dc2.t, grid)
    ev_t, ev_u = dc2.t[~on_grid], np.asarray(dc2.u)[~on_grid]
    assert len(ev_t) % 2 == 0 and len(ev_t) >= 2 and np.all(ev_t >= 0.5)
    assert np.array_equal(ev_t[0::2], ev_t[1::2]) and np.array_equal(ev_u[0::2], ev_u[1::2])
    assert len(dc2.t) - len(ev_t) == 11 + 1  # the save after the affect at tf
    u_grid = np.asarray(dc2.u)[on_grid]
    assert np.array_equal(u_grid[:11], np.asarray(ref.u)) and np.array_equal(u_grid[11], u_grid[10])
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


# ------------------------------------------- vector callbacks and sets
BALLS_F = "du[0] = u[1]; du[1] = -p[0]; du[2] = u[3]; du[3] = -p[1];"  # p = [g1, g2, e1, e2]
BOUNCE_IDX = "u[2 * idx + 1] = -p[2 + idx] * u[2 * idx + 1];"


def test_vector_callback_and_set_compile(capi, de):
    """VectorContinuousCallback / CallbackSet (qa.jl:124,26) compile for the
    one-thread methods and both precisions; sets nest; a set over the
    condition limit, an unknown member and a bad length are refused."""
    balls = de.ODEFunction(BALLS_F, 4, 4, name="balls_compile")
    vc = de.VectorContinuousCallback("out[0] = u[0]; out[1] = u[2];", BOUNCE_IDX, 2)
    c0 = de.ContinuousCallback("g = u[0];", "u[1] = -p[2] * u[1];")
    c1 = de.ContinuousCallback("g = u[2];", "u[3] = -p[3] * u[3];")
    d = de.DiscreteCallback("g = t > 0.5;", "u[1] += 0.0;")
    nested = de.CallbackSet(de.CallbackSet(c0, d), c1, vc)
    L = capi.lib()
    for cb in (vc, de.CallbackSet(c0, c1, d), nested):
        for alg, prec in ((capi.ALG_TSIT5, capi.PREC_FP64), (capi.ALG_VERN7, capi.PREC_F32X2),
                          (capi.ALG_RODAS5, capi.PREC_FP64)):
            _skip_without_nvrtc(capi, lambda: capi.check(
                L.gbde_callback_compile(balls.id, alg, prec, cb.id)))
    with pytest.raises(capi.GBDEError):
        de.VectorContinuousCallback("out[0] = u[0];", None, 0)
    with pytest.raises(capi.GBDEError):
        de.VectorContinuousCallback("out[0] = u[0];", None, capi.MAX_CB_CONDITIONS + 1)
    import ctypes as C
    ids, sid = (C.c_int32 * 1)(10 ** 6), C.c_int32()
    with pytest.raises(capi.GBDEError):
        capi.check(L.gbde_callback_set_register(ids, 1, C.byref(sid)))
    big = de.VectorContinuousCallback("out[0] = u[0];", None, capi.MAX_CB_CONDITIONS)
    over = de.CallbackSet(big, c0)
    with pytest.raises(capi.GBDEError) as e:
        _skip_without_nvrtc(capi, lambda: capi.check(
            L.gbde_callback_compile(balls.id, capi.ALG_TSIT5, capi.PREC_FP64, over.id)))
    assert "continuous conditions" in str(e.value)
    with pytest.raises(TypeError):
        de.CallbackSet(c0, "g = t;")


def _two_balls(de, N, seed):
    rng = np.random.default_rng(seed)
    g = rng.uniform(5.0, 15.0, (N, 2))
    e = rng.uniform(0.8, 0.9, (N, 2))
    h0 = rng.uniform(0.5, 2.0, (N, 2))
    u0 = np.c_[h0[:, 0], np.zeros(N), h0[:, 1], np.zeros(N)]
    return g, e, h0, u0, np.c_[g, e]


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["vector", "set"])
@pytest.mark.parametrize("precision", ["fp64", "f32x2"])
def test_two_balls_vector_callback_exact(capi, de, form, precision):
    """Two independent balls in one state, their impacts as one
    VectorContinuousCallback (idx picks the ball) or as a CallbackSet of two
    ContinuousCallbacks plus a no-op DiscreteCallback: every save follows the
    analytic solution of each ball through its own bounces, so the earliest
    root of the two conditions is taken each time and the affect gets the
    right index."""
    N = 384
    g, e, h0, u0, p = _two_balls(de, N, 6)
    balls = de.ODEFunction(BALLS_F, 4, 4, name="balls_%s_%s" % (form, precision))
    if form == "vector":
        cb = de.VectorContinuousCallback("out[0] = u[0]; out[1] = u[2];", BOUNCE_IDX, 2)
    else:
        cb = de.CallbackSet(de.ContinuousCallback("g = u[0];", "u[1] = -p[2] * u[1];"),
                            de.DiscreteCallback("g = 1.0;"),
                            de.ContinuousCallback("g = u[2];", "u[3] = -p[3] * u[3];"))
    ens = de.EnsembleProblem(de.ODEProblem(balls, u0[0], (0.0, 1.0), p[0]),
                             batch=lambda prob, n: {"p": p, "u0": u0})
    sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(precision=precision), trajectories=N,
                   saveat=0.05, reltol=1e-10, abstol=1e-10, callback=cb)
    assert sol.converged
    ts = de.save_grid(0.0, 1.0, 0.05)
    err = 0.0
    for i in range(N):
        for b in range(2):
            x, v = _ball_truth(h0[i, b], g[i, b], e[i, b], ts)
            err = max(err, np.abs(sol.U[i, :, 2 * b] - x).max(),
                      np.abs(sol.U[i, :, 2 * b + 1] - v).max() / g[i, b])
    assert err <= 1e-8, err


@pytest.mark.gpu
def test_discrete_callbacks_in_order_after_events(capi, de):
    """Discrete members of a set run in order after every accepted step and
    after every event: the first counts (u[4] += 1), the second doubles the
    count's copy (u[5] = 2 u[4]), so u[5] == 2 u[4] at every save only if
    the order holds.  naccept counts accepted steps, event-truncated ones
    included, and the save at the final time holds the state before that
    step's discrete affects (as the reference's saveat with the callbacks'
    default save_positions), so the last saved count is naccept - 1."""
    N = 64
    g, e, h0, u0, p = _two_balls(de, N, 7)
    f = BALLS_F + " du[4] = 0.0; du[5] = 0.0;"
    balls = de.ODEFunction(f, 6, 4, name="balls_counted")
    cb = de.CallbackSet(de.ContinuousCallback("g = u[0];", "u[1] = -p[2] * u[1];"),
                        de.DiscreteCallback("g = 1.0;", "u[4] += 1.0;"),
                        de.DiscreteCallback("g = 1.0;", "u[5] = 2.0 * u[4];"))
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-9
    o.callback = cb.id
    grid = de.save_grid(0.0, 1.0, 0.1)
    r = de.solve_arrays(balls, o, p, np.c_[u0, np.zeros((N, 2))], np.zeros(N), np.ones(N),
                        grid, capi.SAVE_GRID)
    assert np.all(r["retcode"] == capi.RET_SUCCESS)
    np.testing.assert_array_equal(r["u"][:, :, 5], 2.0 * r["u"][:, :, 4])
    np.testing.assert_array_equal(r["u"][:, -1, 4], r["naccept"] - 1)


# ------------------------------------------- saves at events (save_positions)
def _impacts(h0, g, e, t_end):
    """Analytic impacts of a ball dropped from rest at h0 up to t_end: their
    times, speeds before (downward) and after (upward, e times it)."""
    t, v_in = np.sqrt(2 * h0 / g), np.sqrt(2 * h0 / g) * g
    out = []
    while t <= t_end:
        out.append((t, v_in))
        v_in *= e
        t += 2 * v_in / g
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "f32x2"])
def test_event_saves_bouncing_ball(capi, de, precision):
    """save_positions=(true, true), the reference's default: every impact adds
    (t, u) before the bounce (x = 0, v = -v_in) and after it (x = 0,
    v = e v_in) to the trajectory's solution, between the saveat points of
    their time; the analytic impacts pin times and states."""
    N = 256
    rng = np.random.default_rng(11)
    g = rng.uniform(5.0, 15.0, N)
    e = rng.uniform(0.8, 0.9, N)
    h0 = rng.uniform(0.5, 2.0, N)
    ball = de.ODEFunction(BALL_F, 2, 2, name="ball_evsave_%s" % precision)
    cb = de.ContinuousCallback("g = u[0];", BOUNCE)
    ens = de.EnsembleProblem(de.ODEProblem(ball, [1.0, 0.0], (0.0, 1.0), [9.8, 0.8]),
                             batch=lambda prob, n: {"p": np.c_[g, e], "u0": np.c_[h0, np.zeros(N)]})
    sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(precision=precision), trajectories=N,
                   saveat=0.05, reltol=1e-10, abstol=1e-10, callback=cb)
    assert sol.converged
    ts = de.save_grid(0.0, 1.0, 0.05)
    ev_t, ev_u, ev_n = sol.events
    for i in range(N):
        imp = _impacts(h0[i], g[i], e[i], 1.0)
        assert ev_n[i] == 2 * len(imp), (i, ev_n[i], len(imp))
        for k, (t_hit, v_in) in enumerate(imp):
            for j, v in ((2 * k, -v_in), (2 * k + 1, e[i] * v_in)):
                assert abs(ev_t[i, j] - t_hit) <= 1e-9 * t_hit, (i, k)
                assert abs(ev_u[i, j, 0]) <= 1e-9 and abs(ev_u[i, j, 1] - v) <= 1e-8 * g[i]
        s = sol[i]
        assert len(s.t) == len(ts) + 2 * len(imp)
        assert np.all(np.diff(s.t) >= 0)
        grid_rows = np.isin(s.t, ts)
        assert np.array_equal(np.asarray(s.u)[grid_rows], sol.U[i])


@pytest.mark.gpu
def test_event_save_positions_flags(capi, de):
    """(true, false) keeps the saves before the affects, (false, true) those
    after, (false, false) none (no event buffers at all); a continuous
    callback without an affect saves nothing after its event."""
    N = 64
    rng = np.random.default_rng(12)
    g, e, h0 = rng.uniform(5.0, 15.0, N), rng.uniform(0.8, 0.9, N), rng.uniform(0.5, 2.0, N)
    ball = de.ODEFunction(BALL_F, 2, 2, name="ball_evflags")
    ens = de.EnsembleProblem(de.ODEProblem(ball, [1.0, 0.0], (0.0, 1.0), [9.8, 0.8]),
                             batch=lambda prob, n: {"p": np.c_[g, e], "u0": np.c_[h0, np.zeros(N)]})
    kw = dict(trajectories=N, saveat=0.05, reltol=1e-10, abstol=1e-10)
    n_imp = np.array([len(_impacts(h0[i], g[i], e[i], 1.0)) for i in range(N)])
    for sp, sign in (((True, False), -1.0), ((False, True), 1.0)):
        cb = de.ContinuousCallback("g = u[0];", BOUNCE, save_positions=sp)
        sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(), callback=cb, **kw)
        ev_t, ev_u, ev_n = sol.events
        assert np.array_equal(ev_n, n_imp), sp
        assert all(np.all(np.sign(ev_u[i, :ev_n[i], 1]) == sign) for i in range(N))
    sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(),
                   callback=de.ContinuousCallback("g = u[0];", BOUNCE,
                                                  save_positions=(False, False)), **kw)
    assert sol.events is None and len(sol[0].t) == 21
    # no affect: u is not modified, only the save before the event is made
    # (the ball then falls through zero: one crossing per trajectory)
    sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(),
                   callback=de.ContinuousCallback("g = u[0];"), **kw)
    ev_t, ev_u, ev_n = sol.events
    assert np.all(ev_n == 1)
    np.testing.assert_allclose(ev_t[:, 0], np.sqrt(2 * h0 / g), rtol=1e-9)


def _counting_problem(de, N, seed, name):
    g, e, h0, u0, p = _two_balls(de, N, seed)
    f = BALLS_F + " du[4] = 0.0; du[5] = 0.0;"
    balls = de.ODEFunction(f, 6, 4, name=name)
    cb = de.CallbackSet(de.ContinuousCallback("g = u[0];", "u[1] = -p[2] * u[1];"),
                        de.DiscreteCallback("g = 1.0;", "u[4] += 1.0;"),
                        de.DiscreteCallback("g = 1.0;", "u[5] = 2.0 * u[4];"))
    return g, e, h0, np.c_[u0, np.zeros((N, 2))], p, balls, cb


@pytest.mark.gpu
def test_discrete_event_saves_count_and_order(capi, de):
    """Two discrete callbacks firing after every accepted step and an impact
    callback: each impact saves twice, each discrete firing twice, but the
    first discrete callback after the last step (which ends on the saveat
    point tf) saves nothing before its affect -- so a trajectory makes
    2 impacts + 4 naccept - 1 saves, in time order, and the save after the
    second affect always holds u[5] == 2 u[4].  A capacity below the count
    stores the first saves of the same sequence and counts them all."""
    N = 64
    g, e, h0, u0, p, balls, cb = _counting_problem(de, N, 13, "balls_evcount")
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-9
    o.callback = cb.id
    grid = de.save_grid(0.0, 1.0, 0.1)
    args = (balls, o, p, u0, np.zeros(N), np.ones(N), grid, capi.SAVE_GRID)
    n_imp = np.array([len(_impacts(h0[i, 0], g[i, 0], e[i, 0], 1.0)) for i in range(N)])
    first = de.solve_arrays(*args, events=0)
    count = first["ev_count"]
    assert np.all(first["retcode"] == capi.RET_SUCCESS)
    assert np.array_equal(count, 2 * n_imp + 4 * first["naccept"] - 1)
    cap = int(count.max())
    full = de.solve_arrays(*args, events=cap)
    assert np.array_equal(full["ev_count"], count)
    for i in range(N):
        c = count[i]
        t, u = full["ev_t"][i, :c], full["ev_u"][i, :c]
        assert np.all(np.diff(t) >= 0)
        # the last save is the second discrete affect's after the final step
        assert t[-1] == 1.0 and u[-1, 5] == 2.0 * u[-1, 4] == 2.0 * first["naccept"][i]
    small = de.solve_arrays(*args, events=5)
    assert np.array_equal(small["ev_count"], count)
    assert np.array_equal(small["ev_t"], full["ev_t"][:, :5])
    assert np.array_equal(small["ev_u"], full["ev_u"][:, :5])


@pytest.mark.gpu
def test_event_saves_device_memory_and_resolve(capi, de):
    """Device-memory solves write the same event saves as host-memory ones,
    and solve() solves again when the first guess of room was short: every
    save of every trajectory ends up in its solution."""
    torch = pytest.importorskip("torch")
    N = 32
    g, e, h0, u0, p, balls, cb = _counting_problem(de, N, 14, "balls_evdev")
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-9
    o.callback = cb.id
    grid = de.save_grid(0.0, 1.0, 0.1)
    host = de.solve_arrays(balls, o, p, u0, np.zeros(N), np.ones(N), grid, capi.SAVE_GRID,
                           events=16)
    dv = [torch.from_numpy(np.ascontiguousarray(a)).cuda()
          for a in (p, u0, np.zeros(N), np.ones(N), grid)]
    dev = de.solve_arrays(balls, o, *dv, capi.SAVE_GRID, events=16)
    torch.cuda.synchronize()
    for k in ("ev_t", "ev_u", "ev_count"):
        assert np.array_equal(dev[k].cpu().numpy(), host[k]), k
    ens = de.EnsembleProblem(de.ODEProblem(balls, u0[0], (0.0, 1.0), p[0]),
                             batch=lambda prob, n: {"p": p, "u0": u0})
    sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=N, saveat=0.1,
                   reltol=1e-9, abstol=1e-9, callback=cb)
    ev_t, ev_u, ev_n = sol.events
    assert np.array_equal(ev_n, host["ev_count"]) and ev_t.shape[1] == ev_n.max() > 16
    for i in range(N):
        assert len(sol[i].t) == len(grid) + ev_n[i]
        c = min(16, int(ev_n[i]))
        assert np.array_equal(ev_t[i, :c], host["ev_t"][i, :c])
