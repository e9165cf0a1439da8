"""GPU parity: every kernel through the C ABI against the CPU FP64 oracle on
identical seeded inputs.

Tolerances: adaptive methods pass when the weighted error
max |u - u*| / (abstol + reltol |u*|) against the oracle (same algorithm,
same tolerances) is <= 10; FP64 runs are held to <= 1 (they differ from the
oracle only by FMA contraction).  Fixed-step EM in FP64 on identical noise is
held to 1e-12 relative."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_inputs(de, model, N, rng, tf=None):
    if model is de.models.lorenz:
        p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
        u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
        tf = np.ones(N) if tf is None else tf
    elif model is de.models.robertson:
        p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
        u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
        tf = 10 ** rng.uniform(1, 5, N) if tf is None else tf
    elif model is de.models.linear:
        p = rng.uniform(0.5, 1.5, (N, 1))
        u0 = rng.uniform(0.1, 1.0, (N, 1))
        tf = np.ones(N) if tf is None else tf
    elif model is de.models.lotka_volterra:
        p = np.array([1.5, 1.0, 3.0, 1.0, 0.1]) * np.c_[rng.uniform(0.8, 1.2, (N, 4)), np.ones(N)]
        u0 = np.ones((N, 2))
        tf = np.full(N, 10.0) if tf is None else tf
    elif model is de.models.vdp_ring8:
        p = np.c_[10 ** rng.uniform(-1, 3, N), np.full(N, 0.05)]
        u0 = rng.uniform(-2, 2, (N, 16))
        tf = np.full(N, 20.0) if tf is None else tf
    return p, u0, np.zeros(N), np.asarray(tf, float)


def run_both(de, oracle, model, alg_id, p, u0, t0, tf, saveat, save_kind, precision="fp64",
             batching="plain", noise_f32=False, u_dtype="f64", **kw):
    capi = de._capi
    opts = capi.opts_default(alg_id)
    for k, v in kw.items():
        setattr(opts, k, v)
    opts_gpu = capi.opts_default(alg_id)
    for k, v in kw.items():
        setattr(opts_gpu, k, v)
    opts_gpu.precision = capi.PREC_MIXED if precision == "mixed" else capi.PREC_FP64
    opts_gpu.batching = capi.BATCH_PERSISTENT if batching == "persistent" else capi.BATCH_PLAIN
    g = de.solve_arrays(model, opts_gpu, p, u0, t0, tf, saveat, save_kind, u_dtype=u_dtype)
    r = oracle.solve(capi, model, opts, p, u0, t0, tf, saveat, save_kind, nthreads=8,
                     noise_f32=noise_f32)
    return g, r, opts


ODE_CASES = [
    ("lorenz", "TSIT5", 1e-8, 1e-8), ("lorenz", "VERN7", 1e-8, 1e-8),
    ("linear", "TSIT5", 1e-8, 1e-8), ("linear", "VERN7", 1e-10, 1e-10),
    ("robertson", "ROSENBROCK23", 1e-6, 1e-10), ("robertson", "RODAS5", 1e-6, 1e-10),
    ("robertson", "RODAS5P", 1e-6, 1e-10), ("lorenz", "RODAS5", 1e-7, 1e-7),
    ("linear", "RODAS5P", 1e-8, 1e-8), ("lorenz", "VERN7", 1e-10, 1e-10),
]


@pytest.mark.parametrize("model_name,alg,rt,at", ODE_CASES)
def test_ode_fp64_parity(de, oracle, rng, model_name, alg, rt, at):
    capi = de._capi
    model = getattr(de.models, model_name)
    N = 777
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    if model_name == "robertson":
        saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
        kind = capi.SAVE_PER_TRAJ
    else:
        saveat = de.save_grid(0.0, 1.0, 0.1)
        kind = capi.SAVE_GRID
    g, r, _ = run_both(de, oracle, model, getattr(capi, "ALG_" + alg), p, u0, t0, tf, saveat,
                       kind, reltol=rt, abstol=at)
    assert np.array_equal(g["retcode"], r["retcode"])
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    err = oracle.weighted_error(g["u"], r["u"], at, rt)
    assert err <= 1.0, err
    # step statistics agree except for rare FMA-rounding-induced differences
    assert np.mean(g["naccept"] == r["naccept"]) > 0.95
    # first save point is u0 exactly
    assert np.array_equal(g["u"][:, 0, :], u0) or kind == capi.SAVE_PER_TRAJ


@pytest.mark.parametrize("alg", ["TSIT5", "RODAS5"])
def test_persistent_is_bitwise_plain(de, oracle, rng, alg):
    capi = de._capi
    model = de.models.robertson if alg == "RODAS5" else de.models.lorenz
    N = 5000
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    saveat = tf[:, None] * np.linspace(0.1, 1.0, 10)
    outs = []
    for b in ("plain", "persistent"):
        opts = capi.opts_default(getattr(capi, "ALG_" + alg))
        opts.reltol, opts.abstol = (1e-6, 1e-10) if alg == "RODAS5" else (1e-8, 1e-8)
        opts.batching = capi.BATCH_PERSISTENT if b == "persistent" else capi.BATCH_PLAIN
        outs.append(de.solve_arrays(model, opts, p, u0, t0, tf, saveat, capi.SAVE_PER_TRAJ))
    assert np.array_equal(outs[0]["u"], outs[1]["u"])
    assert np.array_equal(outs[0]["naccept"], outs[1]["naccept"])


# Mixed precision (FP32 state and stages) is checked where the tolerance
# allows it.  Robertson kinetics is left out on purpose: late in a solve
# du1 = -k1 y1 + k3 y2 y3 is the difference of two terms of ~2e-3 that agree
# to ~1e-4, so one FP32 right-hand side evaluation already carries ~5e-4
# relative error in du1 and the solution drifts by ~100x reltol at
# reltol=1e-6 / abstol=1e-10 (measured on GB300: Rodas5 139, Rosenbrock23 71).
# That workload runs in FP64.
@pytest.mark.parametrize("model_name,alg,rt,at", [
    ("lorenz", "TSIT5", 1e-5, 1e-5), ("lorenz", "VERN7", 1e-5, 1e-5),
    ("lorenz", "RODAS5", 1e-5, 1e-5), ("lorenz", "ROSENBROCK23", 1e-4, 1e-4),
    ("vdp_ring8", "TSIT5", 1e-5, 1e-5)])
def test_mixed_precision_vs_fp64_oracle(de, oracle, rng, model_name, alg, rt, at):
    capi = de._capi
    model = getattr(de.models, model_name)
    N = 512
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    if model_name == "vdp_ring8":
        p[:, 0] = 10 ** rng.uniform(-1, 0.5, N)  # non-stiff part of the distribution
        saveat = de.save_grid(0.0, 20.0, 1.0)
        kind = capi.SAVE_GRID
    elif model_name == "robertson":
        saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
        kind = capi.SAVE_PER_TRAJ
    else:
        saveat = de.save_grid(0.0, 1.0, 0.1)
        kind = capi.SAVE_GRID
    g, r, _ = run_both(de, oracle, model, getattr(capi, "ALG_" + alg), p, u0, t0, tf, saveat,
                       kind, precision="mixed", u_dtype="f32", reltol=rt, abstol=at,
                       maxiters=10 ** 6)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    if model_name != "vdp_ring8":
        err = oracle.weighted_error(g["u"], r["u"], at, rt)
        assert err <= 10.0, err
        return
    # On the ring of Van der Pol oscillators the global error of the method
    # itself is 50-80x reltol, and any change of the step sequence (even
    # gamma 0.9 -> 0.89 in the FP64 oracle) moves the solution by as much.
    # The mixed-precision kernel is therefore held to the accuracy of the
    # FP64 oracle: against a tight-tolerance truth, its per-trajectory error
    # quantiles stay within twice the FP64 oracle's.
    opts_t = capi.opts_default(capi.ALG_VERN7)
    opts_t.reltol = opts_t.abstol = 1e-12
    opts_t.maxiters = 10 ** 7
    truth = oracle.solve(capi, model, opts_t, p, u0, t0, tf, saveat, kind, nthreads=8)["u"]

    def per_traj(u):
        return (np.abs(u - truth) / (at + rt * np.abs(truth))).max(axis=(1, 2))

    e_mixed, e_fp64 = per_traj(g["u"].astype(np.float64)), per_traj(r["u"])
    for q in (50, 90, 99):
        assert np.percentile(e_mixed, q) <= 2.0 * np.percentile(e_fp64, q) + 1.0, q


def test_em_fp64_identical_noise(de, oracle, rng):
    capi = de._capi
    model = de.models.lotka_volterra
    N = 1000
    p, u0, t0, tf = make_inputs(de, model, N, rng, tf=np.full(N, 2.0))
    saveat = de.save_grid(0.0, 2.0, 0.25)
    g, r, _ = run_both(de, oracle, model, capi.ALG_EM, p, u0, t0, tf, saveat, capi.SAVE_GRID,
                       dt=1e-3, seed=20261204)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    rel = np.max(np.abs(g["u"] - r["u"]) / np.abs(r["u"]))
    assert rel <= 1e-12, rel


def test_em_fp32_on_fp32_stream(de, oracle, rng):
    capi = de._capi
    model = de.models.lotka_volterra
    N = 1000
    p, u0, t0, tf = make_inputs(de, model, N, rng, tf=np.full(N, 2.0))
    saveat = de.save_grid(0.0, 2.0, 0.25)
    g, r, _ = run_both(de, oracle, model, capi.ALG_EM, p, u0, t0, tf, saveat, capi.SAVE_GRID,
                       precision="mixed", noise_f32=True, u_dtype="f32", dt=1e-3, seed=7)
    rel = np.max(np.abs(g["u"] - r["u"]) / np.abs(r["u"]))
    assert rel <= 1e-4, rel


def test_em_fp32_step_bookkeeping(de, oracle, rng):
    """The FP32 EM loop counts steps instead of accumulating FP64 time: the
    step count, the partial last step, save points between step boundaries
    and the maxiters exit must be the FP64 loop's (the oracle's)."""
    capi = de._capi
    model = de.models.lotka_volterra
    N = 600
    p, u0, _, _ = make_inputs(de, model, N, rng)
    t0 = rng.uniform(-0.5, 0.5, N)
    tf = t0 + rng.uniform(0.05, 1.5, N)
    frac = np.sort(rng.uniform(0.0, 1.0, (N, 9)), axis=1)
    saveat = np.c_[t0, t0[:, None] + frac * (tf - t0)[:, None], tf]
    for maxiters in (10 ** 6, 60):
        g, r, _ = run_both(de, oracle, model, capi.ALG_EM, p, u0, t0, tf, saveat,
                           capi.SAVE_PER_TRAJ, precision="mixed", noise_f32=True, u_dtype="f32",
                           dt=1e-2, seed=5, maxiters=maxiters)
        assert np.array_equal(g["retcode"], r["retcode"])
        assert np.array_equal(g["naccept"], r["naccept"])
        np.testing.assert_allclose(g["t_end"], r["t_end"], rtol=1e-15, atol=0)
        ok = ~np.isnan(r["u"])
        assert np.array_equal(np.isnan(g["u"]), ~ok)
        rel = np.max(np.abs(g["u"][ok] - r["u"][ok]) / np.abs(r["u"][ok]))
        assert rel <= 1e-4, rel
    assert np.any(r["retcode"] == capi.RET_MAXITERS) and np.any(r["retcode"] == capi.RET_SUCCESS)


@pytest.mark.parametrize("alg", ["SOSRI", "SRIW1"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sosri_parity(de, oracle, rng, precision, alg):
    """SOSRI (and SRIW1) on the GPU against the oracle on identical noise."""
    capi = de._capi
    model = de.models.lotka_volterra
    N = 1000
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    saveat = de.save_grid(0.0, 10.0, 1.0)
    g, r, _ = run_both(de, oracle, model, getattr(capi, "ALG_" + alg), p, u0, t0, tf, saveat,
                       capi.SAVE_GRID,
                       precision=precision, noise_f32=(precision == "mixed"),
                       u_dtype="f64" if precision == "fp64" else "f32",
                       reltol=1e-3, abstol=1e-3, seed=11)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    assert g["nreject"].sum() > 0
    if precision == "fp64":
        # FMA contraction on the GPU (the oracle has none) moves EEst by a
        # few ulps; where that flips an accept/reject decision the rest of the
        # counter-based stream is consumed along another step sequence, i.e.
        # the trajectory continues on another Brownian path.  All others are
        # the same path to round-off.
        same = np.all(np.abs(g["u"] - r["u"]) <= 1e-9 * np.abs(r["u"]) + 1e-12, axis=(1, 2))
        assert same.mean() > 0.95, same.mean()
        # the flipped trajectories are draws from the same law: the ensemble
        # mean at every save time agrees within 3 standard errors
        se = r["u"].std(axis=0) / np.sqrt(N)
        assert np.all(np.abs(g["u"].mean(axis=0) - r["u"].mean(axis=0)) <= 3 * se + 1e-12)
    else:
        err = np.abs(g["u"] - r["u"]) / (1e-3 + 1e-3 * np.abs(r["u"]))
        assert np.median(err.max(axis=(1, 2))) <= 10.0


def test_failure_codes_gpu(de, oracle, rng):
    capi = de._capi
    model = de.models.lorenz
    p = np.tile([10.0, 28.0, 8.0 / 3.0], (4, 1))
    u0 = np.array([[1.0, 0, 0], [np.nan, 0, 0], [1.0, 0, 0], [1.0, 0, 0]])
    t0 = np.zeros(4)
    tf = np.array([1.0, 1.0, -1.0, 0.0])
    saveat = np.array([0.0])
    opts = capi.opts_default(capi.ALG_TSIT5)
    g = de.solve_arrays(model, opts, p, u0, t0, tf, saveat, capi.SAVE_GRID)
    assert list(g["retcode"]) == [capi.RET_SUCCESS, capi.RET_INITIALFAILURE,
                                  capi.RET_INITIALFAILURE, capi.RET_SUCCESS]
    opts.maxiters = 3
    opts.reltol = opts.abstol = 1e-10
    g = de.solve_arrays(model, opts, p[:1], u0[:1], t0[:1], np.ones(1),
                        np.array([0.0, 0.5, 1.0]), capi.SAVE_GRID)
    assert g["retcode"][0] == capi.RET_MAXITERS and np.isnan(g["u"][0, 2]).all()
    # empty ensemble and empty save list
    g = de.solve_arrays(model, opts, p[:0], u0[:0], t0[:0], tf[:0], saveat, capi.SAVE_GRID)
    assert g["u"].shape == (0, 1, 3)
    g = de.solve_arrays(model, capi.opts_default(capi.ALG_TSIT5), p[:1], u0[:1], t0[:1],
                        np.ones(1), np.zeros(0), capi.SAVE_GRID)
    assert g["retcode"][0] == capi.RET_SUCCESS and g["t_end"][0] == 1.0


def test_invalid_arguments_rejected(de):
    capi = de._capi
    model = de.models.lorenz
    p = np.tile([10.0, 28.0, 8.0 / 3.0], (2, 1))
    u0 = np.tile([1.0, 0, 0], (2, 1))
    opts = capi.opts_default(capi.ALG_TSIT5)
    opts.reltol = -1.0
    with pytest.raises(capi.GBDEError) as e:
        de.solve_arrays(model, opts, p, u0, np.zeros(2), np.ones(2), np.array([1.0]),
                        capi.SAVE_GRID)
    assert e.value.code == capi.GBDE_ERR_INVALID
    opts = capi.opts_default(capi.ALG_EM)
    opts.dt = 0.1
    with pytest.raises(capi.GBDEError) as e:
        de.solve_arrays(model, opts, p, u0, np.zeros(2), np.ones(2), np.array([1.0]),
                        capi.SAVE_GRID)
    assert e.value.code == capi.GBDE_ERR_UNSUPPORTED


def test_device_deadline_returns_status(de, rng):
    """A deadline that expires mid-solve ends the kernel with an error status
    the host reads (no fault, no hang); the context stays usable."""
    capi = de._capi
    model = de.models.robertson
    N = 20000
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    opts = capi.opts_default(capi.ALG_RODAS5)
    opts.reltol, opts.abstol = 1e-10, 1e-14
    opts.timeout_s = 1e-6
    with pytest.raises(capi.GBDEError) as e:
        g = de.solve_arrays(model, opts, p, u0, t0, tf, tf[:, None], capi.SAVE_PER_TRAJ)
    assert e.value.code == capi.GBDE_ERR_TIMEOUT
    opts.timeout_s = 0.0
    opts.reltol, opts.abstol = 1e-6, 1e-10
    g = de.solve_arrays(model, opts, p[:100], u0[:100], t0[:100], tf[:100], tf[:100, None],
                        capi.SAVE_PER_TRAJ)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)


@pytest.mark.parametrize("alg,precision", [("EM", "fp64"), ("EM", "mixed"), ("SOSRI", "mixed"),
                                           ("SRIW1", "fp64")])
def test_sde_device_deadline_returns_status(de, rng, alg, precision):
    """The SDE loops honour the device deadline as the ODE loops do: a solve
    whose deadline expires returns GBDE_ERR_TIMEOUT (no fault, no hang)."""
    capi = de._capi
    model = de.models.lotka_volterra
    N = 20000
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    opts = capi.opts_default(getattr(capi, "ALG_" + alg))
    opts.precision = capi.PREC_MIXED if precision == "mixed" else capi.PREC_FP64
    opts.seed = 3
    if alg == "EM":
        opts.dt = 1e-5
        opts.maxiters = 10 ** 8
    else:
        opts.reltol = opts.abstol = 1e-7
        opts.maxiters = 10 ** 8
    opts.timeout_s = 1e-6
    with pytest.raises(capi.GBDEError) as e:
        de.solve_arrays(model, opts, p, u0, t0, tf, de.save_grid(0.0, 10.0, 1.0), capi.SAVE_GRID,
                        u_dtype="f32" if precision == "mixed" else "f64")
    assert e.value.code == capi.GBDE_ERR_TIMEOUT


def test_device_mode_matches_host_mode(de, rng):
    import torch
    capi = de._capi
    model = de.models.lorenz
    N = 300
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    saveat = de.save_grid(0.0, 1.0, 0.1)
    opts = capi.opts_default(capi.ALG_TSIT5)
    h = de.solve_arrays(model, opts, p, u0, t0, tf, saveat, capi.SAVE_GRID)
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (p, u0, t0, tf, saveat)]
    d = de.solve_arrays(model, opts, *dev, capi.SAVE_GRID)
    torch.cuda.synchronize()
    assert np.array_equal(d["u"].cpu().numpy(), h["u"])
    assert np.array_equal(d["retcode"].cpu().numpy(), h["retcode"])


def test_public_api_core_pins(de):
    """The reference's pinned behaviours through solve(EnsembleProblem, ...,
    EnsembleGB300()) (test/core.jl:9-19, 21-36, 38-49, 81-96)."""
    prob = de.ODEProblem(de.models.linear, 0.5, (0.0, 1.0), [1.01])
    sol = de.solve(prob, de.Tsit5(), de.EnsembleGB300(), saveat=0.1, reltol=1e-8, abstol=1e-8)
    assert sol.retcode == de.ReturnCode.Success
    assert len(sol.t) == 11 and sol.u[0][0] == 0.5 and sol.u[5][0] > 0.5
    lor = de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0), [10.0, 28.0, 8.0 / 3.0])
    sol = de.solve(lor, de.Tsit5(), de.EnsembleGB300(), saveat=0.1)
    assert sol.retcode == de.ReturnCode.Success and list(sol.u[0]) == [1.0, 0.0, 0.0]
    assert len(sol.u[-1]) == 3
    rob = de.ODEProblem(de.models.robertson, [1.0, 0.0, 0.0], (0.0, 1e5), [0.04, 3e7, 1e4])
    sol = de.solve(rob, de.Rodas5P(), de.EnsembleGB300(), saveat=[1e5])
    assert sol.retcode == de.ReturnCode.Success
    prob2 = de.remake(prob, u0=1.0)
    sol = de.solve(prob2, de.Tsit5(), de.EnsembleGB300(), saveat=0.5)
    assert sol.retcode == de.ReturnCode.Success and sol.u[0][0] == 1.0
    # an ensemble through prob_func
    ens = de.EnsembleProblem(lor, prob_func=lambda pr, i, rep: de.remake(pr, p=pr.p * (1 + 0.01 * i)))
    es = de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=64, saveat=0.1)
    assert es.converged and len(es.u) == 64 and es.U.shape == (64, 11, 3)


def test_config1_full_size(de, oracle):
    """Lorenz ensemble, Float64, 10,000 trajectories (parameters scaled by
    U[0.9, 1.1]), Tsit5 at 1e-8, saveat 0.1: every trajectory vs the oracle."""
    capi = de._capi
    rng = np.random.default_rng(20261204)
    N = 10000
    p, u0, t0, tf = make_inputs(de, de.models.lorenz, N, rng)
    g, r, _ = run_both(de, oracle, de.models.lorenz, capi.ALG_TSIT5, p, u0, t0, tf,
                       de.save_grid(0.0, 1.0, 0.1), capi.SAVE_GRID, reltol=1e-8, abstol=1e-8)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    assert oracle.weighted_error(g["u"], r["u"], 1e-8, 1e-8) <= 1.0


def test_config2_full_size_properties(de, oracle):
    """Robertson ensemble, 100,000 trajectories, Rodas5 and Rosenbrock23:
    every trajectory succeeds and conserves mass; a 2,000-trajectory sample
    matches the oracle; plain and persistent launches agree bitwise."""
    capi = de._capi
    rng = np.random.default_rng(20261204)
    N = 100000
    p, u0, t0, tf = make_inputs(de, de.models.robertson, N, rng)
    saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
    for alg in (capi.ALG_RODAS5, capi.ALG_ROSENBROCK23):
        res = {}
        for b in (capi.BATCH_PLAIN, capi.BATCH_PERSISTENT):
            opts = capi.opts_default(alg)
            opts.reltol, opts.abstol, opts.batching = 1e-6, 1e-10, b
            res[b] = de.solve_arrays(de.models.robertson, opts, p, u0, t0, tf, saveat,
                                     capi.SAVE_PER_TRAJ)
        g = res[capi.BATCH_PLAIN]
        assert np.all(g["retcode"] == capi.RET_SUCCESS)
        assert np.max(np.abs(g["u"].sum(axis=2) - 1.0)) < 1e-8
        assert np.array_equal(g["u"], res[capi.BATCH_PERSISTENT]["u"])
        idx = rng.choice(N, 2000, replace=False)
        opts = capi.opts_default(alg)
        opts.reltol, opts.abstol = 1e-6, 1e-10
        r = oracle.solve(capi, de.models.robertson, opts, p[idx], u0[idx], t0[idx], tf[idx],
                         saveat[idx], capi.SAVE_PER_TRAJ, nthreads=8)
        assert oracle.weighted_error(g["u"][idx], r["u"], 1e-10, 1e-6) <= 1.0


def test_fma_peak_microbenchmark(de):
    ctx = de._capi.context(0)
    f64 = ctx.fma_peak(0)
    f32 = ctx.fma_peak(1)
    assert f64 > 0.1 and f32 > f64


def test_rcp64_accuracy(de):
    """The Newton-refined reciprocal of the hot loops (error norm, LU pivots,
    1/dt) agrees with the device's IEEE division to ~2^-40 relative (one
    Newton step from the ~2^-20 hardware estimate; measured 9.6e-13)."""
    err = de._capi.context(0).check_rcp64(1 << 22)
    assert err <= 2.0 ** -38, err


# F32X2: state, stages and right-hand sides as FP32 pairs (~48 bits), FP64 LU,
# norm and time.  Near-FP64 accuracy: the steps follow the FP64 oracle's and
# the saved states agree to well inside the tolerance.  The limit is the
# error estimate, a sum whose terms cancel to ~reltol: at reltol 1e-10 Vern7's
# cancels ~10 digits, leaving ~4 in 48-bit pairs (~5.5 in FP64), and about 1%
# of the linear model's trajectories then take another step sequence than the
# oracle (measured on GB300: 99th percentile 8x tolerance) -- so the lockstep
# cases stop at 1e-8 for Vern7.
@pytest.mark.parametrize("model_name,alg,rt,at", [
    ("robertson", "RODAS5", 1e-6, 1e-10), ("robertson", "RODAS5P", 1e-6, 1e-10),
    ("robertson", "ROSENBROCK23", 1e-6, 1e-10), ("lorenz", "TSIT5", 1e-8, 1e-8),
    ("lorenz", "VERN7", 1e-8, 1e-8), ("lorenz", "RODAS5", 1e-7, 1e-7),
    ("linear", "TSIT5", 1e-10, 1e-10), ("linear", "VERN7", 1e-8, 1e-8)])
def test_f32x2_vs_fp64_oracle(de, oracle, rng, model_name, alg, rt, at):
    capi = de._capi
    model = getattr(de.models, model_name)
    N = 2000
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    if model_name == "robertson":
        saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
        kind = capi.SAVE_PER_TRAJ
    else:
        saveat = de.save_grid(0.0, 1.0, 0.1)
        kind = capi.SAVE_GRID
    for batching in ("plain", "persistent"):
        g, r, _ = run_both(de, oracle, model, getattr(capi, "ALG_" + alg), p, u0, t0, tf, saveat,
                           kind, batching=batching, reltol=rt, abstol=at)
        g2 = de.solve_arrays(model, _f32x2(capi, alg, rt, at, batching), p, u0, t0, tf, saveat, kind)
        assert np.all(g2["retcode"] == capi.RET_SUCCESS)
        e = (np.abs(g2["u"] - r["u"]) / (at + rt * np.abs(r["u"]))).max(axis=(1, 2))
        assert np.percentile(e, 99) <= 0.1, np.percentile(e, 99)
        assert e.max() <= 10.0, e.max()
        assert np.mean(g2["naccept"] == r["naccept"]) >= 0.99


def _f32x2(capi, alg, rt, at, batching):
    o = capi.opts_default(getattr(capi, "ALG_" + alg))
    o.reltol, o.abstol = rt, at
    o.precision = capi.PREC_F32X2
    o.batching = capi.BATCH_PERSISTENT if batching == "persistent" else capi.BATCH_PLAIN
    return o


def test_f32x2_rejected_where_not_built(de, rng):
    capi = de._capi
    o = capi.opts_default(capi.ALG_EM)
    o.dt = 1e-2
    o.precision = capi.PREC_F32X2
    p, u0, t0, tf = make_inputs(de, de.models.lotka_volterra, 4, rng)
    with pytest.raises(capi.GBDEError) as e:
        de.solve_arrays(de.models.lotka_volterra, o, p, u0, t0, tf, np.array([0.0]), capi.SAVE_GRID)
    assert e.value.code == capi.GBDE_ERR_UNSUPPORTED


def test_one_call_sharding_matches_single_device(de):
    """EnsembleGB300(devices=[...]) splits the ensemble into contiguous
    slices solved concurrently (one host thread and context per entry; here
    both on GPU 0) and reassembles them in place: bitwise the single-device
    solve."""
    N = 5001
    rng = np.random.default_rng(31)
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    ens = de.EnsembleProblem(de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0),
                                           p[0]), batch=lambda prob, n: {"p": p})
    one = de.solve(ens, de.Tsit5(), de.EnsembleGB300(device=0), trajectories=N, saveat=0.1,
                   reltol=1e-8, abstol=1e-8)
    two = de.solve(ens, de.Tsit5(), de.EnsembleGB300(devices=[0, 0]), trajectories=N,
                   saveat=0.1, reltol=1e-8, abstol=1e-8)
    assert one.converged and two.converged
    assert np.array_equal(one.U, two.U)
    assert np.array_equal(one.retcode, two.retcode)


@pytest.mark.parametrize("precision", ["fp64", "f32x2"])
def test_vern7_dense_output_is_7th_order(de, precision):
    """Save points inside Vern7's steps carry the method's own accuracy: on
    u' = a u with saves at every 0.01 (most inside a step), the error against
    exp(a t) at reltol 1e-10 stays within the bar of the step endpoints (a
    lower-order interpolant would dominate the 7th-order steps here)."""
    capi = de._capi
    N = 256
    rng = np.random.default_rng(17)
    p = rng.uniform(0.5, 1.5, (N, 1))
    u0 = rng.uniform(0.1, 1.0, (N, 1))
    grid = np.linspace(0.0, 1.0, 101)
    o = capi.opts_default(capi.ALG_VERN7)
    o.reltol = o.abstol = 1e-10
    o.precision = capi.PREC_F32X2 if precision == "f32x2" else capi.PREC_FP64
    g = de.solve_arrays(de.models.linear, o, p, u0, np.zeros(N), np.ones(N), grid,
                        capi.SAVE_GRID)
    assert np.all(g["retcode"] == capi.RET_SUCCESS)
    exact = u0 * np.exp(p * grid[None, :])
    err = np.abs(g["u"][:, :, 0] - exact) / (1e-10 + 1e-10 * np.abs(exact))
    assert err.max() <= 2.0, err.max()
    # most save points fall inside steps: the steps are far longer than 0.01
    assert g["naccept"].mean() < 30


@pytest.mark.parametrize("alg", ["Tsit5", "Vern7", "Rodas5P"])
def test_dense_solution_evaluation(de, alg):
    """sol(t) on a dense solve (test/core.jl:51-58: u' = 1.01 u, u0 = 0.5,
    sol(0.5) is a number > 0.5) is the method's own dense output: exactly the
    value a saveat containing t stores (save points never change the steps),
    within the tolerance of the exact solution."""
    prob = de.ODEProblem(de.models.linear, 0.5, (0.0, 1.0), [1.01])
    a = getattr(de, alg)()
    sol = de.solve(prob, a, de.EnsembleGB300(), dense=True, reltol=1e-8, abstol=1e-8)
    assert sol.retcode == de.ReturnCode.Success
    assert list(sol.t) == [0.0, 1.0]  # the end points are stored
    v = sol(0.5)
    assert v.shape == (1,) and v[0] > 0.5
    ts = np.array([0.73, 0.1, 0.5])
    vs = sol(ts)
    ref = de.solve(prob, a, de.EnsembleGB300(), saveat=np.sort(ts), reltol=1e-8, abstol=1e-8)
    order = np.argsort(ts)
    assert np.array_equal(vs[order, 0], np.array([u[0] for u in ref.u]))
    assert np.allclose(vs[:, 0], 0.5 * np.exp(1.01 * ts), rtol=1e-6, atol=0)
    with pytest.raises(ValueError):
        sol(1.5)
    # an ensemble member's dense output
    ens = de.EnsembleProblem(prob, prob_func=lambda pr, i, rep: de.remake(pr, u0=0.5 + 0.1 * i))
    es = de.solve(ens, a, de.EnsembleGB300(), trajectories=4, dense=True, reltol=1e-8,
                  abstol=1e-8)
    assert np.allclose(es[3](0.25), 0.8 * np.exp(1.01 * 0.25), rtol=1e-6)


@pytest.mark.parametrize("model_name,alg", [("lorenz", "TSIT5"), ("vdp_ring8", "AUTO")])
def test_host_outputs_pinned_equal_staged(de, rng, model_name, alg):
    """GBDE_MEM_HOST with a page-locked output buffer: the kernels store the
    saves straight into it (no staging copy); the result is bitwise the staged
    path's (pageable output) and the device path's."""
    import torch
    capi = de._capi
    model = getattr(de.models, model_name)
    N = 3000
    p, u0, t0, tf = make_inputs(de, model, N, rng)
    grid = de.save_grid(0.0, float(tf[0]), float(tf[0]) / 10)
    o = capi.opts_default(getattr(capi, "ALG_" + alg))
    o.reltol = o.abstol = 1e-6
    o.maxiters = 10 ** 6
    if alg == "AUTO":
        o.stiff_threshold = 100.0
        o.precision = capi.PREC_F32X2
        o.batching = capi.BATCH_PERSISTENT
    shape = (N, len(grid), model.n_state)
    pinned = {"u": torch.empty(shape, dtype=torch.float32).pin_memory().numpy(),
              "retcode": torch.empty(N, dtype=torch.int32).pin_memory().numpy()}
    staged = {"u": np.empty(shape, np.float32), "retcode": np.empty(N, np.int32)}
    for out in (pinned, staged):
        out["u"][:] = -1.0
        de.solve_arrays(model, o, p, u0, t0, tf, grid, capi.SAVE_GRID, u_dtype="f32", out=out)
    d = de.solve_arrays(model, o, *[torch.from_numpy(np.ascontiguousarray(a)).cuda()
                                    for a in (p, u0, t0, tf, grid)], capi.SAVE_GRID,
                        u_dtype="f32")
    assert np.all(pinned["retcode"] == capi.RET_SUCCESS)
    assert np.array_equal(pinned["u"], staged["u"])
    assert np.array_equal(pinned["u"], d["u"].cpu().numpy())
