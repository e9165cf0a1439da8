"""The CPU oracle and the GPU kernels against the committed golden truths
(tests/golden/ode_truth.json, made by tests/golden/make_golden.py with scipy
solve_ivp at rtol <= 1e-12).

Each bound is the method's own global error at the given tolerance on that
problem (weighted: |u - u*| / (abstol + reltol |u*|)), as measured for the
oracle when the fixtures were made, times ~2.5: a pin on the accuracy of the
restated methods, not a lockstep check (that is test_gpu_parity.py).  Vern7's
bounds are those of its 7th-order dense output: the 5th-order extension it
replaced left Lorenz at 2 x tolerance, interpolation error dominating the
7th-order steps (now 0.02)."""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = json.load(open(os.path.join(HERE, "golden", "ode_truth.json")))["cases"]
BY_NAME = {c["name"]: c for c in CASES}

# (case, algorithm, reltol, abstol, bound)
RUNS = [
    ("linear_1.01", "TSIT5", 1e-8, 1e-8, 0.5), ("linear_1.01", "VERN7", 1e-8, 1e-8, 0.001),
    ("linear_1.01", "ROSENBROCK23", 1e-8, 1e-8, 330), ("linear_1.01", "RODAS5", 1e-8, 1e-8, 1.5),
    ("linear_1.01", "RODAS5P", 1e-8, 1e-8, 1.5),
    ("lorenz_core", "TSIT5", 1e-8, 1e-8, 6), ("lorenz_core", "VERN7", 1e-8, 1e-8, 0.05),
    ("lorenz_scaled", "TSIT5", 1e-8, 1e-8, 6), ("lorenz_scaled", "VERN7", 1e-8, 1e-8, 0.05),
    ("robertson_core", "ROSENBROCK23", 1e-6, 1e-10, 110), ("robertson_core", "RODAS5", 1e-6, 1e-10, 17),
    ("robertson_core", "RODAS5P", 1e-6, 1e-10, 31), ("robertson_scaled", "ROSENBROCK23", 1e-6, 1e-10, 70),
    ("robertson_scaled", "RODAS5", 1e-6, 1e-10, 20), ("robertson_scaled", "RODAS5P", 1e-6, 1e-10, 37),
    ("vdp_ring8_mu1", "TSIT5", 1e-6, 1e-6, 34), ("vdp_ring8_mu1", "VERN7", 1e-6, 1e-6, 4),
    ("vdp_ring8_mu1", "RODAS5", 1e-6, 1e-6, 32), ("vdp_ring8_mu1", "RODAS5P", 1e-6, 1e-6, 36),
    ("vdp_ring8_mu30", "RODAS5", 1e-6, 1e-6, 800), ("vdp_ring8_mu30", "RODAS5P", 1e-6, 1e-6, 1100),
    ("lotka_volterra_drift", "TSIT5", 1e-8, 1e-8, 10), ("lotka_volterra_drift", "VERN7", 1e-8, 1e-8, 2),
    ("lotka_volterra_drift", "RODAS5", 1e-8, 1e-8, 26), ("lotka_volterra_drift", "RODAS5P", 1e-8, 1e-8, 53),
]


def problem(de, c):
    m = getattr(de.models, c["model"])
    p = list(c["p"]) + ([0.0] if c["model"] == "lotka_volterra" else [])  # noise off
    t = np.array(c["t"])
    return (m, np.array(p)[None], np.array(c["u0"])[None], np.zeros(1), np.array([t[-1]]), t,
            np.array(c["u"]))


def opts(capi, alg, rt, at):
    o = capi.opts_default(getattr(capi, "ALG_" + alg))
    o.reltol, o.abstol, o.maxiters = rt, at, 10 ** 7
    return o


def test_fixtures_are_complete():
    assert {c["model"] for c in CASES} == {"linear", "lorenz", "robertson", "vdp_ring8",
                                          "lotka_volterra"}
    for c in CASES:
        assert np.array(c["u"]).shape == (len(c["t"]), len(c["u0"]))
        assert c["made_with"].startswith("scipy solve_ivp")


@pytest.mark.parametrize("name,alg,rt,at,bound", RUNS)
def test_oracle_vs_golden(de, oracle, name, alg, rt, at, bound):
    capi = de._capi
    m, p, u0, t0, tf, t, ref = problem(de, BY_NAME[name])
    r = oracle.solve(capi, m, opts(capi, alg, rt, at), p, u0, t0, tf, t, capi.SAVE_GRID)
    assert r["retcode"][0] == capi.RET_SUCCESS
    assert oracle.weighted_error(r["u"][0], ref, at, rt) <= bound
    if t[0] == 0.0:
        assert np.array_equal(r["u"][0, 0], u0[0])  # sol.u[1] == u0 (test/core.jl:34)


@pytest.mark.gpu
@pytest.mark.parametrize("name,alg,rt,at,bound", RUNS)
def test_gpu_vs_golden(de, oracle, name, alg, rt, at, bound):
    capi = de._capi
    m, p, u0, t0, tf, t, ref = problem(de, BY_NAME[name])
    g = de.solve_arrays(m, opts(capi, alg, rt, at), p, u0, t0, tf, t, capi.SAVE_GRID)
    assert g["retcode"][0] == capi.RET_SUCCESS
    assert oracle.weighted_error(g["u"][0], ref, at, rt) <= bound
    if t[0] == 0.0:
        assert np.array_equal(g["u"][0, 0], u0[0])
