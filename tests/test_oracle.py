"""Pins of the CPU oracle: the reference's own pinned behaviours
(test/core.jl), analytic solutions, scipy solve_ivp truths, convergence
orders of every method, and the Philox known-answer vectors."""
import numpy as np
import pytest
from scipy.integrate import solve_ivp

ODE_ALGS = ["TSIT5", "VERN7", "ROSENBROCK23", "RODAS5", "RODAS5P"]


def run(oracle, capi, model, alg, p, u0, tspan, saveat, save_kind=None, **kw):
    opts = capi.opts_default(getattr(capi, "ALG_" + alg))
    for k, v in kw.items():
        setattr(opts, k, v)
    p = np.atleast_2d(np.asarray(p, float))
    u0 = np.atleast_2d(np.asarray(u0, float))
    N = p.shape[0]
    t0 = np.full(N, float(tspan[0]))
    tf = np.full(N, float(tspan[1])) if np.isscalar(tspan[1]) else np.asarray(tspan[1], float)
    saveat = np.asarray(saveat, float)
    if save_kind is None:
        save_kind = capi.SAVE_GRID if saveat.ndim == 1 else capi.SAVE_PER_TRAJ
    return oracle.solve(capi, model, opts, p, u0, t0, tf, saveat, save_kind)


# ------------------------------------------- reference pinned behaviours
@pytest.mark.parametrize("alg", ODE_ALGS)
def test_core_basic_solve(oracle, capi, de, alg):
    """core.jl:9-19 / 90-96: u' = 1.01u, u0 = 0.5, (0, 1), saveat 0.1 ->
    Success, 11 points, first point == u0."""
    grid = de.save_grid(0.0, 1.0, 0.1)
    assert len(grid) == 11 and grid[0] == 0.0 and grid[-1] == 1.0
    r = run(oracle, capi, de.models.linear, alg, [1.01], [0.5], (0.0, 1.0), grid,
            reltol=1e-8, abstol=1e-8)
    assert r["retcode"][0] == capi.RET_SUCCESS
    assert r["u"][0, 0, 0] == 0.5
    exact = 0.5 * np.exp(1.01 * grid)
    tol = 3e-5 if alg == "ROSENBROCK23" else 1e-7
    assert np.max(np.abs(r["u"][0, :, 0] - exact) / exact) < tol
    assert r["u"][0, 5, 0] > 0.5  # interpolated value at 0.5 (core.jl:51-58)


def lorenz(t, u, p=(10.0, 28.0, 8.0 / 3.0)):
    return [p[0] * (u[1] - u[0]), u[0] * (p[1] - u[2]) - u[1], u[0] * u[1] - p[2] * u[2]]


@pytest.mark.parametrize("alg", ["TSIT5", "VERN7"])
def test_core_lorenz(oracle, capi, de, alg):
    """core.jl:21-36: Lorenz (10, 28, 8/3), u0 = [1,0,0], (0, 1): Success,
    u[1] == u0 exactly, 3-vector end state; accuracy vs DOP853 truth."""
    grid = de.save_grid(0.0, 1.0, 0.1)
    r = run(oracle, capi, de.models.lorenz, alg, [10.0, 28.0, 8.0 / 3.0], [1.0, 0.0, 0.0],
            (0.0, 1.0), grid, reltol=1e-8, abstol=1e-8)
    assert r["retcode"][0] == capi.RET_SUCCESS
    assert np.array_equal(r["u"][0, 0], [1.0, 0.0, 0.0])
    ref = solve_ivp(lorenz, (0, 1), [1, 0, 0], method="DOP853", rtol=1e-13, atol=1e-13,
                    t_eval=grid).y.T
    assert oracle.weighted_error(r["u"][0], ref, 1e-8, 1e-8) < 10


def rober(t, u, k=(0.04, 3e7, 1e4)):
    return [-k[0] * u[0] + k[2] * u[1] * u[2],
            k[0] * u[0] - k[1] * u[1] ** 2 - k[2] * u[1] * u[2], k[1] * u[1] ** 2]


@pytest.mark.parametrize("alg", ["ROSENBROCK23", "RODAS5", "RODAS5P"])
def test_core_robertson(oracle, capi, de, alg):
    """core.jl:38-49: Robertson to t = 1e5 returns Success; accuracy vs Radau."""
    tf = 1e5
    grid = tf * 10 ** (-5 + 5 * np.arange(20) / 19)
    r = run(oracle, capi, de.models.robertson, alg, [0.04, 3e7, 1e4], [1.0, 0.0, 0.0],
            (0.0, tf), grid, reltol=1e-6, abstol=1e-10)
    assert r["retcode"][0] == capi.RET_SUCCESS
    ref = solve_ivp(rober, (0, tf), [1, 0, 0], method="Radau", rtol=1e-12, atol=1e-16,
                    t_eval=grid).y.T
    bound = {"ROSENBROCK23": 100, "RODAS5": 20, "RODAS5P": 20}[alg]
    assert oracle.weighted_error(r["u"][0], ref, 1e-10, 1e-6) < bound
    assert abs(r["u"][0, -1].sum() - 1.0) < 1e-8  # mass conservation


# --------------------------------------------------- convergence orders
@pytest.mark.parametrize("alg,order", [("TSIT5", 5), ("VERN7", 7), ("ROSENBROCK23", 2),
                                       ("RODAS5", 5), ("RODAS5P", 5)])
def test_fixed_step_convergence(oracle, capi, de, alg, order):
    """Fixed steps on Lotka-Volterra drift (smooth, nonlinear): the observed
    global order matches the method order."""
    model = de.models.lotka_volterra
    p = [1.5, 1.0, 3.0, 1.0, 0.0]
    T = 2.0
    ref = solve_ivp(lambda t, u: [p[0] * u[0] - p[1] * u[0] * u[1],
                                  p[3] * u[0] * u[1] - p[2] * u[1]],
                    (0, T), [1.0, 1.0], method="DOP853", rtol=1e-14, atol=1e-14).y[:, -1]
    hs = {5: [0.1, 0.05, 0.025], 7: [0.1, 0.05, 0.025], 2: [0.02, 0.01, 0.005]}[order]
    errs = []
    for h in hs:
        r = run(oracle, capi, model, alg, p, [1.0, 1.0], (0.0, T), np.array([T]),
                adaptive=0, dt=h, maxiters=10 ** 6)
        assert r["retcode"][0] == capi.RET_SUCCESS
        errs.append(np.max(np.abs(r["u"][0, -1] - ref)))
    slopes = np.diff(np.log(errs)) / np.diff(np.log(hs))
    assert np.all(slopes > order - 0.6), (errs, slopes)


@pytest.mark.parametrize("alg,order", [("TSIT5", 4), ("VERN7", 5), ("RODAS5", 4),
                                       ("RODAS5P", 4)])
def test_dense_output_order(oracle, capi, de, alg, order):
    """Interpolated save points converge with the dense output's order + 1
    locally; checked on one step of varying size."""
    model = de.models.lotka_volterra
    p = [1.5, 1.0, 3.0, 1.0, 0.0]
    f = lambda t, u: [p[0] * u[0] - p[1] * u[0] * u[1], p[3] * u[0] * u[1] - p[2] * u[1]]
    errs = []
    hs = [0.2, 0.1, 0.05]
    for h in hs:
        ts = np.array([0.37 * h, h])
        ref = solve_ivp(f, (0, h), [1.0, 1.0], method="DOP853", rtol=1e-14, atol=1e-14,
                        t_eval=ts).y.T
        r = run(oracle, capi, model, alg, p, [1.0, 1.0], (0.0, h), ts, adaptive=0, dt=h)
        errs.append(np.max(np.abs(r["u"][0, 0] - ref[0])))
    slopes = np.diff(np.log(errs)) / np.diff(np.log(hs))
    assert np.all(slopes > order + 1 - 0.6), (errs, slopes)


# -------------------------------------------------------- failure codes
def test_retcodes(oracle, capi, de):
    m = de.models.lorenz
    grid = np.linspace(0, 1, 5)
    r = run(oracle, capi, m, "TSIT5", [10, 28, 8 / 3], [1, 0, 0], (0.0, 1.0), grid,
            reltol=1e-8, abstol=1e-8, maxiters=3)
    assert r["retcode"][0] == capi.RET_MAXITERS
    assert np.isnan(r["u"][0, -1]).all()
    r = run(oracle, capi, m, "TSIT5", [10, 28, 8 / 3], [np.nan, 0, 0], (0.0, 1.0), grid)
    assert r["retcode"][0] == capi.RET_INITIALFAILURE
    r = run(oracle, capi, m, "TSIT5", [10, 28, 8 / 3], [1, 0, 0], (0.0, -1.0),
            np.array([0.0]))
    assert r["retcode"][0] == capi.RET_INITIALFAILURE
    r = run(oracle, capi, m, "TSIT5", [10, 28, 8 / 3], [1, 0, 0], (0.0, 0.0), np.array([0.0]))
    assert r["retcode"][0] == capi.RET_SUCCESS and r["u"][0, 0, 0] == 1.0


# ------------------------------------------------------------- noise
KAT = [  # Random123 known-answer vectors for Philox4x32-10
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


@pytest.mark.parametrize("ctr,key,out", KAT)
def test_philox_kat(oracle, capi, ctr, key, out):
    assert list(oracle.philox4x32_10(ctr, key)) == out
    assert list(capi.philox4x32_10(ctr, key)) == out  # host path of libgbde.so


def test_normals_bit_identical_and_distributed(oracle, capi):
    z_lib = capi.philox_normals(20261204, 7, 0, 4096)
    z_orc = oracle.normals(20261204, 7, 0, 4096)
    assert np.array_equal(z_lib.view(np.uint64), z_orc.view(np.uint64))
    z = oracle.normals(1, 3, 0, 200000)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    from scipy import stats
    assert stats.kstest(z, "norm").pvalue > 1e-3
    z32 = oracle.normals(1, 3, 0, 200000, f32=True)
    assert abs(z32.mean()) < 0.01 and abs(z32.std() - 1.0) < 0.01
    assert stats.kstest(z32, "norm").pvalue > 1e-3
    # different trajectories give different streams
    assert not np.array_equal(oracle.normals(1, 4, 0, 8), oracle.normals(1, 3, 0, 8))


def test_normals_series_accuracy(oracle):
    """The series log / sin / cos of the transform are accurate: Box-Muller
    pairs recomputed with numpy's libm agree to ~1e-15."""
    seed, traj = 5, 11
    z = oracle.normals(seed, traj, 0, 2000)
    # regenerate the uniforms from the raw Philox blocks
    zz = []
    for b in range(1000):
        r = oracle.philox4x32_10([b, 0, traj, 0], [seed, 0]).astype(np.uint64)
        a = ((r[0] >> 5) << 26) | (r[1] >> 6)
        c = ((r[2] >> 5) << 26) | (r[3] >> 6)
        u1 = (float(a) + 0.5) * 2.0 ** -53
        u2 = float(c) * 2.0 ** -53
        rad = np.sqrt(-2 * np.log(u1))
        zz += [rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)]
    assert np.max(np.abs(z - np.array(zz))) < 1e-13


def test_em_uses_the_stream(oracle, capi, de):
    """EM with sigma > 0 is u_{n+1} = u_n + f h + sigma u_n sqrt(h) z_n with
    z the documented stream (normal n*2 + c of trajectory i)."""
    model = de.models.lotka_volterra
    p = np.array([[1.5, 1.0, 3.0, 1.0, 0.1]])
    h, nsteps = 1e-2, 7
    r = run(oracle, capi, model, "EM", p, [[1.0, 1.0]], (0.0, h * nsteps), np.array([h * nsteps]),
            dt=h, seed=99)
    z = oracle.normals(99, 0, 0, 2 * nsteps)
    u = np.array([1.0, 1.0])
    a, b, g, d, s = p[0]
    for k in range(nsteps):
        f = np.array([a * u[0] - b * u[0] * u[1], d * u[0] * u[1] - g * u[1]])
        u = u + f * h + s * u * (np.sqrt(h) * z[2 * k:2 * k + 2])
    assert np.allclose(r["u"][0, -1], u, rtol=1e-13, atol=0)


@pytest.mark.parametrize("alg", ["SOSRI", "SRIW1"])
def test_sri_reduces_to_rk2_without_noise(oracle, capi, de, alg):
    """SOSRI and SRIW1 with sigma = 0 are their deterministic parts (order 2):
    an adaptive solve at tight tolerance matches the ODE truth."""
    model = de.models.lotka_volterra
    p = [1.5, 1.0, 3.0, 1.0, 0.0]
    grid = np.linspace(0, 2, 5)
    r = run(oracle, capi, model, alg, p, [1.0, 1.0], (0.0, 2.0), grid, reltol=1e-7,
            abstol=1e-7, seed=1)
    assert r["retcode"][0] == capi.RET_SUCCESS
    ref = solve_ivp(lambda t, u: [p[0] * u[0] - p[1] * u[0] * u[1], p[3] * u[0] * u[1] - p[2] * u[1]],
                    (0, 2), [1.0, 1.0], method="DOP853", rtol=1e-13, atol=1e-13, t_eval=grid).y.T
    assert np.max(np.abs(r["u"][0] - ref)) < 1e-4


@pytest.mark.parametrize("alg", ["SOSRI", "SRIW1"])
def test_sri_adaptive_statistics(oracle, capi, de, alg):
    """Adaptive SRI with rejection sampling with memory keeps the Brownian
    path a Brownian path: on dX = sigma X dW (mean-zero drift) E[X_T] = X0,
    Var[log X_T] = sigma^2 T."""
    model = de.models.lotka_volterra
    N = 4000
    # alpha = beta = gamma = delta = 0: pure multiplicative noise
    p = np.tile([0.0, 0.0, 0.0, 0.0, 0.5], (N, 1))
    r = run(oracle, capi, model, alg, p, np.ones((N, 2)), (0.0, 1.0), np.array([1.0]),
            reltol=1e-2, abstol=1e-2, seed=3)
    assert np.all(r["retcode"] == capi.RET_SUCCESS)
    assert r["nreject"].sum() > 0  # the rejection path was exercised
    x = r["u"][:, 0, 0]
    assert abs(x.mean() - 1.0) < 4 * x.std() / np.sqrt(N)
    lx = np.log(x)
    assert abs(lx.var() - 0.25) < 0.05


@pytest.mark.parametrize("n", [2, 3, 5, 16])
def test_oracle_lu_solve_with_row_swaps(oracle, n):
    """The Rosenbrock steppers' partial-pivot LU solves W x = b to rounding
    when rows are swapped at every elimination step (the factorisation swaps
    whole rows, P W = L U, so the solve applies every swap before the
    substitutions).  Rows are ordered by increasing magnitude of their
    leading entries so that every step swaps."""
    rng = np.random.default_rng(n)
    for _ in range(200):
        A = rng.normal(size=(n, n))
        A[:, 0] = np.arange(1, n + 1) * rng.choice([-1.0, 1.0], n)
        b = rng.normal(size=n)
        x = oracle.lu_solve(A, b)
        assert np.max(np.abs(A @ x - b)) <= 1e-10 * (1 + np.abs(A).sum(1).max() * np.abs(x).max())


# ------------------------------------------------ AutoTsit5 composites
@pytest.mark.parametrize("stiff", ["ROSENBROCK23", "RODAS5"])
def test_autoswitch_nonstiff_is_tsit5(oracle, capi, de, stiff):
    """AutoTsit5(stiff) on a non-stiff problem (Lorenz at reltol 1e-8, where
    h * eig stays far inside Tsit5's stability region) never switches: the
    same steps and values as Tsit5 itself, bit for bit."""
    grid = de.save_grid(0.0, 2.0, 0.1)
    kw = dict(reltol=1e-8, abstol=1e-8)
    p, u0 = [10.0, 28.0, 8.0 / 3.0], [1.0, 0.0, 0.0]
    a = run(oracle, capi, de.models.lorenz, "AUTOTSIT5_" + stiff, p, u0, (0.0, 2.0), grid, **kw)
    t = run(oracle, capi, de.models.lorenz, "TSIT5", p, u0, (0.0, 2.0), grid, **kw)
    assert a["method"][0] == capi.ALG_TSIT5
    assert np.array_equal(a["u"], t["u"]) and a["naccept"][0] == t["naccept"][0]


@pytest.mark.parametrize("stiff", ["ROSENBROCK23", "RODAS5"])
def test_autoswitch_stiff_linear_switches(oracle, capi, de, stiff):
    """u' = a u with a = -1e4 on (0, 1): Tsit5's steps are held at its
    stability limit (h |a| ~ 3.5), every estimate is stiff, and after 11 of
    them the composite continues with the stiff method (the run ends in it)
    in a small fraction of Tsit5's step count; the solution stays within
    tolerance of exp(a t)."""
    grid = de.save_grid(0.0, 1.0, 0.1)
    kw = dict(reltol=1e-6, abstol=1e-8)
    a = run(oracle, capi, de.models.linear, "AUTOTSIT5_" + stiff, [-1e4], [1.0], (0.0, 1.0),
            grid, **kw)
    t = run(oracle, capi, de.models.linear, "TSIT5", [-1e4], [1.0], (0.0, 1.0), grid, **kw)
    assert a["retcode"][0] == capi.RET_SUCCESS
    assert a["method"][0] == getattr(capi, "ALG_" + stiff)
    assert a["naccept"][0] + a["nreject"][0] < 0.2 * (t["naccept"][0] + t["nreject"][0])
    exact = np.exp(-1e4 * grid)
    assert np.max(np.abs(a["u"][0, :, 0] - exact)) < 1e-6


def test_autoswitch_robertson(oracle, capi, de):
    """AutoTsit5(Rodas5()) on Robertson (core.jl:38-49's problem, to t = 1e5):
    Success, ends in Rodas5, and stays within 10x tolerance of Rodas5 at a
    tight tolerance."""
    grid = np.array([1e-3, 1e-1, 1.0, 1e2, 1e4, 1e5])
    kw = dict(reltol=1e-6, abstol=1e-10)
    k, u0 = [0.04, 3e7, 1e4], [1.0, 0.0, 0.0]
    a = run(oracle, capi, de.models.robertson, "AUTOTSIT5_RODAS5", k, u0, (0.0, 1e5), grid, **kw)
    ref = run(oracle, capi, de.models.robertson, "RODAS5", k, u0, (0.0, 1e5), grid,
              reltol=1e-10, abstol=1e-14)
    assert a["retcode"][0] == capi.RET_SUCCESS and a["method"][0] == capi.ALG_RODAS5
    assert oracle.weighted_error(a["u"][0], ref["u"][0], 1e-10, 1e-6) < 10
