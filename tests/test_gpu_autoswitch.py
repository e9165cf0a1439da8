"""AutoTsit5(Rosenbrock23()) / AutoTsit5(Rodas5()) (test/qa/qa.jl:15) on the
GPU: per-trajectory run-time stiffness switching against the FP64 oracle's
restatement of the same rule (oracle/gbde_oracle.cpp, solve_ode_traj with a
stiff method), plus an analytic problem that is stiff at first and
non-stiff later, so the composite switches to the stiff method and back."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(de, name, N, rng):
    if name == "robertson":  # stiff after the initial transient
        p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
        return de.models.robertson, p, np.tile([1.0, 0.0, 0.0], (N, 1)), 10 ** rng.uniform(1, 5, N)
    if name == "linear":  # u' = a u, a = -10^U(0, 5): non-stiff to very stiff
        p = -(10 ** rng.uniform(0, 5, (N, 1)))
        return de.models.linear, p, rng.uniform(0.5, 1.5, (N, 1)), np.ones(N)
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    return de.models.lorenz, p, np.tile([1.0, 0.0, 0.0], (N, 1)), np.ones(N)


CASES = [("robertson", 1e-6, 1e-10), ("linear", 1e-6, 1e-8), ("lorenz", 1e-8, 1e-8)]


@pytest.mark.parametrize("stiff", ["ROSENBROCK23", "RODAS5"])
@pytest.mark.parametrize("name,rt,at", CASES)
@pytest.mark.parametrize("batching", ["plain", "persistent"])
def test_autoswitch_fp64_lockstep(de, oracle, rng, stiff, name, rt, at, batching):
    """FP64: the GPU composite takes the oracle's decisions (same final method
    and the same accepted / rejected step counts on >= 95 % of trajectories;
    the two differ only by FMA contraction) and stays within 1x tolerance of
    it on every trajectory."""
    capi = de._capi
    N = 1500
    model, p, u0, tf = _inputs(de, name, N, rng)
    alg = getattr(capi, "ALG_AUTOTSIT5_" + stiff)
    saves = np.c_[tf * 0.25, tf * 0.5, tf]
    o = capi.opts_default(alg)
    o.reltol, o.abstol = rt, at
    g = de.solve_arrays(model, o, p, u0, np.zeros(N), tf, saves, capi.SAVE_PER_TRAJ)
    r = oracle.solve(capi, model, o, p, u0, np.zeros(N), tf, saves, capi.SAVE_PER_TRAJ, nthreads=8)
    assert np.all(g["retcode"] == capi.RET_SUCCESS) and np.all(r["retcode"] == capi.RET_SUCCESS)
    same = (g["naccept"] == r["naccept"]) & (g["nreject"] == r["nreject"])
    assert same.mean() >= 0.95, same.mean()
    assert (g["method"] == r["method"]).mean() >= 0.95
    if name == "robertson":
        assert np.all(r["method"] == getattr(capi, "ALG_" + stiff))
    if name == "lorenz":
        assert np.all(g["method"] == capi.ALG_TSIT5)
    err = oracle.weighted_errors(g["u"], r["u"], at, rt)
    assert np.max(err) <= 1.0, np.max(err)


def test_autoswitch_nonstiff_equals_tsit5(de, rng):
    """On Lorenz at reltol 1e-8 no trajectory switches, and the composite's
    Tsit5 is the Tsit5 kernel's: identical saves and step counts."""
    capi = de._capi
    N = 1024
    model, p, u0, tf = _inputs(de, "lorenz", N, rng)
    grid = de.save_grid(0.0, 1.0, 0.1)
    res = []
    for alg in (capi.ALG_AUTOTSIT5_ROSENBROCK23, capi.ALG_TSIT5):
        o = capi.opts_default(alg)
        o.reltol = o.abstol = 1e-8
        res.append(de.solve_arrays(model, o, p, u0, np.zeros(N), tf, grid, capi.SAVE_GRID))
    a, t = res
    assert np.all(a["method"] == capi.ALG_TSIT5)
    assert np.array_equal(a["naccept"], t["naccept"]) and np.array_equal(a["u"], t["u"])


# u' = -k s u, s' = -r s: the decay rate k s = k e^(-r t) fades from k = 100
# to below 1 by t = 25; u(t) = u0 exp(-(k / r) (1 - e^(-r t))) stays a normal
# FP64 number (k / r = 500).  Every component keeps changing between the
# last two stages, so Hairer's estimate (a ratio of stage differences) is
# defined; a component whose derivative is a constant (a clock, t' = 1) would
# give 0/0 there, which counts as non-stiff -- in the reference's formula as
# here.
FADING = "du[0] = -p[0] * u[1] * u[0];\ndu[1] = -p[1] * u[1];"
K_RATE, R_RATE = 100.0, 0.2


@pytest.mark.parametrize("stiff", ["Rosenbrock23", "Rodas5"])
def test_autoswitch_there_and_back(de, stiff):
    """A problem whose stiffness fades: u' = -k s u, s' = -r s on (0, T),
    T in [40, 60].  Once u is below abstol, Tsit5 alone is held at its
    stability limit until k s is small (about (k / r) / 3.5 steps); the
    composite switches to the stiff method and, once k s dt is small, back
    to Tsit5 (every run ends in Tsit5; a composite that never switched would
    take Tsit5's steps exactly), and follows the analytic solution: within
    50x tolerance with Rodas5, 200x with the second-order Rosenbrock23 (its
    global error at these tolerances is tens of times reltol; the oracle's
    on Robertson is 53x)."""
    N = 64
    fading = de.ODEFunction(FADING, 2, 2, name="fading_stiffness_%s" % stiff)
    p = np.tile([K_RATE, R_RATE], (N, 1))
    u0 = np.tile([0.5, 1.0], (N, 1))
    tf = np.linspace(40.0, 60.0, N)
    saves = np.c_[np.full(N, 0.01), np.full(N, 1.0), np.full(N, 10.0), tf]
    capi = de._capi
    out = {}
    for name, alg in (("auto", de.AutoTsit5(getattr(de, stiff)()).alg_id),
                      ("tsit5", capi.ALG_TSIT5)):
        o = capi.opts_default(alg)
        o.reltol, o.abstol = 1e-6, 1e-9
        o.maxiters = 10 ** 7
        out[name] = de.solve_arrays(fading, o, p, u0, np.zeros(N), tf, saves, capi.SAVE_PER_TRAJ)
    a, t = out["auto"], out["tsit5"]
    assert np.all(a["retcode"] == capi.RET_SUCCESS)
    assert np.all(a["method"] == capi.ALG_TSIT5)
    steps_a = a["naccept"] + a["nreject"]
    steps_t = t["naccept"] + t["nreject"]
    assert np.all(steps_a < 0.9 * steps_t), (steps_a[:4], steps_t[:4])
    s_exact = np.exp(-R_RATE * saves)
    u_exact = 0.5 * np.exp(-(K_RATE / R_RATE) * (1.0 - s_exact))
    bar = 200.0 if stiff == "Rosenbrock23" else 50.0
    for c, exact in ((0, u_exact), (1, s_exact)):
        err = np.abs(a["u"][:, :, c] - exact) / (1e-9 + 1e-6 * np.abs(exact))
        assert np.max(err) < bar, (c, np.max(err))


def test_autoswitch_rejections(de):
    """The composites run in FP64 and mixed precision on one-thread models:
    FP32 pairs, the 16-state ring and callbacks are refused."""
    capi = de._capi
    o = capi.opts_default(capi.ALG_AUTOTSIT5_RODAS5)
    o.precision = capi.PREC_F32X2
    p, u0 = np.array([[10.0, 28.0, 8.0 / 3.0]]), np.array([[1.0, 0.0, 0.0]])
    with pytest.raises(capi.GBDEError):
        de.solve_arrays(de.models.lorenz, o, p, u0, np.zeros(1), np.ones(1), np.array([1.0]),
                        capi.SAVE_GRID)
    o = capi.opts_default(capi.ALG_AUTOTSIT5_RODAS5)
    with pytest.raises(capi.GBDEError):
        de.solve_arrays(de.models.vdp_ring8, o, np.array([[10.0, 0.05]]), np.zeros((1, 16)),
                        np.zeros(1), np.ones(1), np.array([1.0]), capi.SAVE_GRID)
    o.callback = de.ContinuousCallback("g = t - 0.5;").id
    with pytest.raises(capi.GBDEError):
        de.solve_arrays(de.models.lorenz, o, p, u0, np.zeros(1), np.ones(1), np.array([1.0]),
                        capi.SAVE_GRID)
