"""User right-hand sides compiled at run time (ODEFunction, the reference's
ODEFunction f!(du, u, p, t), test/qa/qa.jl:84): registration, NVRTC
compilation of every algorithm and precision without a GPU, compile errors
reported with the compiler's log, and -- on the GPU -- parity of a user
restatement of a built-in model with the CPU FP64 oracle, the dual-number
Jacobian against the user's analytic one, and a model the library does not
build in against an independent scipy solution."""
import numpy as np
import pytest

# the built-in models' formulas (test/core.jl:22-27, 39-45), restated as user source
LORENZ_F = """
du[0] = p[0] * (u[1] - u[0]);
du[1] = u[0] * (p[1] - u[2]) - u[1];
du[2] = u[0] * u[1] - p[2] * u[2];
"""
ROBERTSON_F = """
T r1 = p[0] * u[0];
T r2 = p[1] * u[1] * u[1];
T r3 = p[2] * u[1] * u[2];
du[0] = -r1 + r3;
du[1] = r1 - r2 - r3;
du[2] = r2;
"""
ROBERTSON_J = """
J[0][0] = -p[0]; J[0][1] = p[2] * u[2]; J[0][2] = p[2] * u[1];
J[1][0] = p[0]; J[1][1] = T(-2) * p[1] * u[1] - p[2] * u[2]; J[1][2] = -p[2] * u[1];
J[2][0] = T(0); J[2][1] = T(2) * p[1] * u[1]; J[2][2] = T(0);
"""
# damped pendulum, not a built-in model: theta' = omega,
# omega' = -(g/L) sin(theta) - c omega; p = [g/L, c]
PENDULUM_F = """
du[0] = u[1];
du[1] = -p[0] * sin(u[0]) - p[1] * u[1];
"""


def _compile_or_skip(de, capi, model, alg, precision):
    try:
        de.compile_model(model, alg, precision)
    except capi.GBDEError as e:
        if e.code == capi.GBDE_ERR_UNSUPPORTED:
            pytest.skip("NVRTC unavailable: %s" % e)
        raise


def test_register_and_model_info(capi, de):
    m = de.ODEFunction(LORENZ_F, 3, 3, name="lorenz_user")
    assert m.id >= capi.MODEL_USER_BASE
    assert capi.model_info(m.id) == (3, 3)
    m2 = de.ODEFunction(LORENZ_F, 3, 3)
    assert m2.id == m.id + 1


@pytest.mark.parametrize("n_state,n_param", [(0, 1), (9, 1), (2, 0), (2, 33)])
def test_register_rejects_sizes(capi, de, n_state, n_param):
    with pytest.raises(capi.GBDEError) as e:
        de.ODEFunction("du[0] = u[0];", n_state, n_param)
    assert e.value.code == capi.GBDE_ERR_INVALID


def test_compile_every_algorithm_and_precision(capi, de):
    """The library's step kernels build around a user f for every one-thread
    ODE method in FP64, FP32 and FP32 pairs; Rosenbrock methods take the
    Jacobian from dual numbers (no jac given)."""
    m = de.ODEFunction(LORENZ_F, 3, 3, name="lorenz_all")
    for alg in (de.Tsit5(), de.Vern7(), de.Rosenbrock23(), de.Rodas5(), de.Rodas5P()):
        for prec in ("fp64", "mixed", "f32x2"):
            _compile_or_skip(de, capi, m, alg, prec)


def test_compile_autoswitch_composites(capi, de):
    """AutoTsit5(Rosenbrock23()) / AutoTsit5(Rodas5()) build around a user f
    (dual-number Jacobian) in FP64 and mixed precision; FP32 pairs are
    refused with GBDE_ERR_UNSUPPORTED."""
    m = de.ODEFunction(LORENZ_F, 3, 3, name="lorenz_autoswitch")
    for stiff in (de.Rosenbrock23(), de.Rodas5()):
        for prec in ("fp64", "mixed"):
            _compile_or_skip(de, capi, m, de.AutoTsit5(stiff), prec)
        with pytest.raises(capi.GBDEError) as e:
            de.compile_model(m, de.AutoTsit5(stiff), "f32x2")
        assert e.value.code == capi.GBDE_ERR_UNSUPPORTED
    with pytest.raises(TypeError):
        de.AutoTsit5(de.Vern7())


def test_compile_error_carries_the_log(capi, de):
    m = de.ODEFunction("du[0] = undefined_rate * u[0];", 1, 1, name="broken")
    with pytest.raises(capi.GBDEError) as e:
        _compile_or_skip(de, capi, m, de.Tsit5(), "fp64")
    assert e.value.code == capi.GBDE_ERR_INVALID
    assert "undefined_rate" in str(e.value) and "broken" in str(e.value)


def test_pairs_need_the_pair_operations(capi, de):
    """sin has no FP32-pair form: the F32X2 build fails with the log, FP64
    builds (its dual Jacobian differentiates sin)."""
    m = de.ODEFunction(PENDULUM_F, 2, 2, name="pendulum_pairs")
    _compile_or_skip(de, capi, m, de.Rodas5(), "fp64")
    with pytest.raises(capi.GBDEError) as e:
        de.compile_model(m, de.Rodas5(), "f32x2")
    assert e.value.code == capi.GBDE_ERR_INVALID


# ------------------------------------------------------------------ GPU
def _robertson(N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    tf = 10 ** rng.uniform(1, 5, N)
    saveat = np.ascontiguousarray(tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19))
    return p, np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), tf, saveat


def _opts(capi, alg, rt, at, batching="persistent", precision=None):
    o = capi.opts_default(alg)
    o.reltol, o.abstol = rt, at
    o.batching = capi.BATCH_PERSISTENT if batching == "persistent" else capi.BATCH_PLAIN
    if precision is not None:
        o.precision = precision
    return o


@pytest.mark.gpu
@pytest.mark.parametrize("jac", [ROBERTSON_J, None], ids=["analytic_jac", "dual_jac"])
@pytest.mark.parametrize("prec", ["fp64", "f32x2"])
def test_user_robertson_rodas5_vs_oracle(capi, de, oracle, jac, prec):
    """A user restatement of the Robertson model, Rodas5 at 1e-6 / 1e-10,
    against the CPU FP64 oracle of the built-in model: the lockstep bar of
    the built-in kernels (weighted error <= 1)."""
    m = de.ODEFunction(ROBERTSON_F, 3, 3, jac=jac, name="robertson_user")
    p, u0, t0, tf, sv = _robertson(2000, 21)
    precision = capi.PREC_F32X2 if prec == "f32x2" else capi.PREC_FP64
    r = de.solve_arrays(m, _opts(capi, capi.ALG_RODAS5, 1e-6, 1e-10, precision=precision),
                        p, u0, t0, tf, sv, capi.SAVE_PER_TRAJ)
    assert np.all(r["retcode"] == capi.RET_SUCCESS)
    ref = oracle.solve(capi, de.models.robertson, _opts(capi, capi.ALG_RODAS5, 1e-6, 1e-10),
                       p, u0, t0, tf, sv, capi.SAVE_PER_TRAJ, nthreads=8)
    assert oracle.weighted_error(r["u"], ref["u"], 1e-10, 1e-6) <= 1.0
    assert np.mean(r["naccept"] == ref["naccept"]) >= 0.99


@pytest.mark.gpu
def test_user_lorenz_tsit5_matches_builtin(capi, de, oracle):
    """Tsit5 at 1e-8 on a user Lorenz, plain and persistent, against the
    oracle of the built-in Lorenz and the built-in GPU kernel."""
    m = de.ODEFunction(LORENZ_F, 3, 3, name="lorenz_user_tsit5")
    rng = np.random.default_rng(5)
    N = 3000
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    u0, t0, tf = np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), np.ones(N)
    grid = de.save_grid(0.0, 1.0, 0.1)
    ref = oracle.solve(capi, de.models.lorenz, _opts(capi, capi.ALG_TSIT5, 1e-8, 1e-8),
                       p, u0, t0, tf, grid, capi.SAVE_GRID, nthreads=8)
    for batching in ("plain", "persistent"):
        o = _opts(capi, capi.ALG_TSIT5, 1e-8, 1e-8, batching)
        r = de.solve_arrays(m, o, p, u0, t0, tf, grid, capi.SAVE_GRID)
        b = de.solve_arrays(de.models.lorenz, o, p, u0, t0, tf, grid, capi.SAVE_GRID)
        assert np.all(r["retcode"] == capi.RET_SUCCESS)
        assert oracle.weighted_error(r["u"], ref["u"], 1e-8, 1e-8) <= 1.0
        assert oracle.weighted_error(r["u"], b["u"], 1e-8, 1e-8) <= 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("alg", ["TSIT5", "VERN7", "ROSENBROCK23"])
def test_user_model_f32x2_steppers(capi, de, oracle, alg):
    """The compact FP32-pair steppers compiled at run time around a user f
    (Rosenbrock23 with the dual-number Jacobian) take the FP64 oracle's steps."""
    N = 2000
    if alg == "ROSENBROCK23":
        m = de.ODEFunction(ROBERTSON_F, 3, 3, name="robertson_user_ros23_ff")
        model, (p, u0, t0, tf, sv), kind = de.models.robertson, _robertson(N, 9), capi.SAVE_PER_TRAJ
        rt, at = 1e-6, 1e-10
    else:
        m = de.ODEFunction(LORENZ_F, 3, 3, name="lorenz_user_ff_" + alg.lower())
        rng = np.random.default_rng(6)
        p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
        u0, t0, tf = np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), np.ones(N)
        model, sv, kind = de.models.lorenz, de.save_grid(0.0, 1.0, 0.1), capi.SAVE_GRID
        rt, at = 1e-8, 1e-8
    a = getattr(capi, "ALG_" + alg)
    r = de.solve_arrays(m, _opts(capi, a, rt, at, precision=capi.PREC_F32X2), p, u0, t0, tf, sv,
                        kind)
    assert np.all(r["retcode"] == capi.RET_SUCCESS)
    ref = oracle.solve(capi, model, _opts(capi, a, rt, at), p, u0, t0, tf, sv, kind, nthreads=8)
    e = (np.abs(r["u"] - ref["u"]) / (at + rt * np.abs(ref["u"]))).max(axis=(1, 2))
    assert np.percentile(e, 99) <= 0.1 and e.max() <= 10.0, (np.percentile(e, 99), e.max())
    assert np.mean(r["naccept"] == ref["naccept"]) >= 0.99


@pytest.mark.gpu
def test_user_pendulum_vs_scipy(capi, de):
    """A model the library does not build in (damped pendulum with sin):
    Tsit5 and Rodas5 with the dual-number Jacobian (chain rule through sin),
    through the high-level solve(), against scipy's DOP853 at rtol 1e-12."""
    from scipy.integrate import solve_ivp
    m = de.ODEFunction(PENDULUM_F, 2, 2, name="pendulum")
    rng = np.random.default_rng(8)
    N = 256
    pars = np.c_[rng.uniform(1.0, 10.0, N), rng.uniform(0.0, 0.5, N)]
    th0 = rng.uniform(-2.5, 2.5, N)
    grid = de.save_grid(0.0, 10.0, 1.0)
    truth = np.empty((N, len(grid), 2))
    for i in range(N):
        g, c = pars[i]
        s = solve_ivp(lambda t, y: [y[1], -g * np.sin(y[0]) - c * y[1]], (0.0, 10.0),
                      [th0[i], 0.0], method="DOP853", rtol=1e-12, atol=1e-12, t_eval=grid)
        truth[i] = s.y.T
    for alg, tol, bound in ((de.Tsit5(), 1e-8, 1e-5), (de.Rodas5(), 1e-7, 1e-4)):
        ens = de.EnsembleProblem(
            de.ODEProblem(m, [0.0, 0.0], (0.0, 10.0), [1.0, 0.0]),
            batch=lambda prob, n: {"p": pars, "u0": np.c_[th0, np.zeros(N)]})
        sol = de.solve(ens, alg, de.EnsembleGB300(batching="persistent"), trajectories=N,
                       saveat=1.0, reltol=tol, abstol=tol)
        assert sol.converged
        err = np.abs(sol.U - truth).max()
        assert err <= bound, (alg, err)


@pytest.mark.gpu
def test_user_model_rejects_auto_and_learned(capi, de):
    m = de.ODEFunction(LORENZ_F, 3, 3, name="lorenz_reject")
    p, u0 = np.array([[10.0, 28.0, 8.0 / 3.0]]), np.array([[1.0, 0.0, 0.0]])
    for alg, learned in ((capi.ALG_AUTO, 0), (capi.ALG_TSIT5, capi.LEARN_ORDER)):
        o = _opts(capi, alg, 1e-6, 1e-6)
        o.learned = learned
        with pytest.raises(capi.GBDEError) as e:
            de.solve_arrays(m, o, p, u0, np.zeros(1), np.ones(1), np.array([1.0]),
                            capi.SAVE_GRID)
        assert e.value.code in (capi.GBDE_ERR_UNSUPPORTED, capi.GBDE_ERR_STATE)


# a linear system whose W = I/(gamma h) - A needs a row swap after the first
# elimination step once the fast modes have decayed and the steps grow
# (eigenvalues -1.09 and -20.6 +- 78.6i)
LIN3_A = np.array([[-1.1, 0.0, 0.2], [-9.9, 25.3, -77.0], [-54.7, 107.3, -66.4]])
LIN3_F = """
du[0] = p[0] * u[0] + p[1] * u[1] + p[2] * u[2];
du[1] = p[3] * u[0] + p[4] * u[1] + p[5] * u[2];
du[2] = p[6] * u[0] + p[7] * u[1] + p[8] * u[2];
"""
LIN3_J = """
J[0][0] = p[0]; J[0][1] = p[1]; J[0][2] = p[2];
J[1][0] = p[3]; J[1][1] = p[4]; J[1][2] = p[5];
J[2][0] = p[6]; J[2][1] = p[7]; J[2][2] = p[8];
"""


@pytest.mark.gpu
@pytest.mark.parametrize("alg", ["ROSENBROCK23", "RODAS5", "RODAS5P"])
@pytest.mark.parametrize("precision", ["fp64", "f32x2"])
def test_rosenbrock_w_solve_with_row_swaps(capi, de, alg, precision):
    """Rosenbrock steps whose W-matrix LU swaps rows after its first step
    (P W = L U with whole-row swaps: every swap must reach the right-hand side
    before the substitutions): the solution of u' = A u matches exp(A t) u0
    within the metric's bar, and every trajectory succeeds."""
    from scipy.linalg import expm
    a = getattr(capi, "ALG_" + alg)
    m = de.ODEFunction(LIN3_F, 3, 9, jac=LIN3_J, name="lin3")
    _compile_or_skip(de, capi, m, {"ROSENBROCK23": de.Rosenbrock23(), "RODAS5": de.Rodas5(),
                                   "RODAS5P": de.Rodas5P()}[alg], precision)
    N = 64
    rng = np.random.default_rng(9)
    p = np.tile(LIN3_A.ravel(), (N, 1))
    u0 = rng.uniform(-1, 1, (N, 3))
    grid = de.save_grid(0.0, 5.0, 0.5)
    o = capi.opts_default(a)
    o.reltol, o.abstol = 1e-6, 1e-8
    o.precision = capi.PREC_F32X2 if precision == "f32x2" else capi.PREC_FP64
    g = de.solve_arrays(m, o, p, u0, np.zeros(N), np.full(N, 5.0), grid, capi.SAVE_GRID)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    exact = np.stack([u0 @ expm(LIN3_A * t).T for t in grid], axis=1)
    err = np.abs(g["u"] - exact) / (1e-8 + 1e-6 * np.abs(exact))
    # Rosenbrock23 is order 2: its global error runs to tens of tolerances
    assert err.max() <= (100.0 if alg == "ROSENBROCK23" else 10.0), err.max()


# the built-in Lotka-Volterra SDE (drift and diagonal noise sigma u) restated
LV_F = """
du[0] = p[0] * u[0] - p[1] * u[0] * u[1];
du[1] = p[3] * u[0] * u[1] - p[2] * u[1];
"""
LV_G = """
g[0] = p[4] * u[0];
g[1] = p[4] * u[1];
"""


@pytest.mark.parametrize("alg", ["EM", "SOSRI", "SRIW1"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_user_sde_compiles(capi, de, alg, precision):
    """A user SDE (SDEFunction: drift and diagonal noise as source) compiles
    into the library's EM / SRI drivers without a GPU."""
    m = de.SDEFunction(LV_F, LV_G, 2, 5, name="lv_user")
    assert m.noise and capi.model_info(m.id) == (2, 5)
    _compile_or_skip(de, capi, m, getattr(de, alg)(), precision)


def test_user_sde_rejections(capi, de):
    m = de.SDEFunction(LV_F, LV_G, 2, 5, name="lv_user")
    with pytest.raises(capi.GBDEError) as e:  # no FP32-pair SDE kernels
        de.compile_model(m, de.EM(), "f32x2")
    assert e.value.code == capi.GBDE_ERR_UNSUPPORTED
    ode = de.ODEFunction(LV_F, 2, 5, name="lv_drift_only")
    with pytest.raises(capi.GBDEError) as e:  # an ODE model has no noise term
        de.compile_model(ode, de.EM(), "fp64")
    assert e.value.code == capi.GBDE_ERR_UNSUPPORTED
    with pytest.raises(TypeError):
        de.SDEProblem(ode, None, [1.0, 1.0], (0.0, 1.0), np.ones(5))
    import ctypes as C
    d = capi.UserModel(name=b"x", n_state=2, n_param=5, f_body=LV_F.encode(), jac_body=None)
    mid = C.c_int32()
    assert capi.lib().gbde_sde_model_register(C.byref(d), b"", C.byref(mid)) == \
        capi.GBDE_ERR_INVALID


@pytest.mark.gpu
@pytest.mark.parametrize("alg,precision", [("EM", "fp64"), ("EM", "mixed"), ("SOSRI", "fp64"),
                                           ("SOSRI", "mixed"), ("SRIW1", "fp64")])
def test_user_sde_matches_builtin_oracle(capi, de, oracle, alg, precision):
    """The user restatement of the Lotka-Volterra SDE, compiled at run time,
    against the CPU oracle's built-in model on the same counter-based noise:
    EM in FP64 within 1e-12 relative; with FP32 state within 1e-3 of the
    oracle driven by the same FP32 normals; adaptive SRI on the oracle's
    Brownian path for >= 95 % of trajectories (an FMA-contracted accept /
    reject flip continues a trajectory on another path) with weighted error
    <= 10 on those."""
    m = de.SDEFunction(LV_F, LV_G, 2, 5, name="lv_user")
    N = 1000
    rng = np.random.default_rng(12)
    p = np.c_[np.array([1.5, 1.0, 3.0, 1.0]) * rng.uniform(0.8, 1.2, (N, 4)), np.full(N, 0.1)]
    u0, t0, tf = np.ones((N, 2)), np.zeros(N), np.full(N, 5.0)
    grid = de.save_grid(0.0, 5.0, 0.5)
    o = capi.opts_default(getattr(capi, "ALG_" + alg))
    o.seed = 21
    if alg == "EM":
        o.dt = 1e-3
    else:
        o.reltol = o.abstol = 1e-3
    o.precision = capi.PREC_MIXED if precision == "mixed" else capi.PREC_FP64
    g = de.solve_arrays(m, o, p, u0, t0, tf, grid, capi.SAVE_GRID,
                        u_dtype="f32" if precision == "mixed" else "f64")
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    r = oracle.solve(capi, de.models.lotka_volterra, o, p, u0, t0, tf, grid, capi.SAVE_GRID,
                     nthreads=8, noise_f32=precision == "mixed")
    u = np.asarray(g["u"], np.float64)
    if alg == "EM":
        rel = np.max(np.abs(u - r["u"]) / np.abs(r["u"]))
        assert rel <= (1e-12 if precision == "fp64" else 1e-3), rel
    else:
        same = (g["naccept"] == r["naccept"]) & (g["nreject"] == r["nreject"])
        e = oracle.weighted_errors(u, r["u"], 1e-3, 1e-3).max(axis=(1, 2))
        assert same.mean() >= 0.95, same.mean()
        assert e[same].max() <= 10.0


@pytest.mark.gpu
def test_user_sde_gbm_strong_error(capi, de, oracle):
    """Geometric Brownian motion dX = mu X dt + s X dW as a user SDE: EM at
    dt = 1e-3 against the exact solution X0 exp((mu - s^2/2) t + s W_t) on
    the Brownian path regenerated on the host from the same counter-based
    stream (gbde_philox_normals): the mean strong error is of order sqrt(dt)."""
    m = de.SDEFunction("du[0] = p[0] * u[0];", "g[0] = p[1] * u[0];", 1, 2, name="gbm")
    N, dt, T = 256, 1e-3, 1.0
    p = np.tile([0.5, 0.4], (N, 1))
    o = capi.opts_default(capi.ALG_EM)
    o.dt, o.seed = dt, 77
    g = de.solve_arrays(m, o, p, np.ones((N, 1)), np.zeros(N), np.full(N, T), np.array([T]),
                        capi.SAVE_GRID)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    nsteps = int(round(T / dt))
    W = np.array([np.sqrt(dt) * oracle.normals(77, i, 0, nsteps).sum() for i in range(N)])
    exact = np.exp((0.5 - 0.08) * T + 0.4 * W)
    err = np.abs(g["u"][:, 0, 0] - exact)
    assert err.mean() < 5 * np.sqrt(dt) * 0.4 * exact.mean(), err.mean()
