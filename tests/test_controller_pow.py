"""How far the kernels' FP32-series step-size controller moves a solve away
from the textbook FP64 pow() controller (CPU only, oracle against oracle).

The kernels evaluate the PI controller's factor q = EEst^beta1 / qold^beta2 /
gamma with a FP32 log2 / exp2 series (controller.h) so that the oracle takes
their steps bit for bit; OrdinaryDiffEq evaluates the same factor in FP64 with
`^`.  The oracle runs either form (oracle.set_controller), so the deviation
is measured on samples of the Lorenz (Tsit5, reltol 1e-8), Robertson
(Rodas5 / Rosenbrock23, 1e-6 / 1e-10) and 16-state Van der Pol ring (Tsit5 /
Rodas5, 1e-5) ensembles.  Bars: at most 1 % of trajectories take a different
number of steps (3 % on the stiff ring), and where the step counts agree the
two solutions agree to a weighted error of <= 1 (on the relaxation-oscillation
ring, whose jump times move with any change of step size: <= 10 at the 99th
percentile).  Measured on 1,500-trajectory samples: no step count changed on
Lorenz, Robertson or the non-stiff ring (weighted max 9e-5, 0.27, 0.0014,
0.11); on the stiff ring 1.0 % changed (weighted max 66 among those, p99 5.2
over all)."""
import numpy as np
import pytest

SEED = 20261204


def _inputs(name, N, rng):
    if name == "lorenz":
        p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
        return p, np.tile([1.0, 0, 0], (N, 1)), np.zeros(N), np.ones(N), np.linspace(0, 1, 11)
    if name == "robertson":
        p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
        tf = 10 ** rng.uniform(1, 5, N)
        sv = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
        return p, np.tile([1.0, 0, 0], (N, 1)), np.zeros(N), tf, sv
    p = np.c_[10 ** rng.uniform(-1, 3, N), np.full(N, 0.05)]
    return p, rng.uniform(-2, 2, (N, 16)), np.zeros(N), np.full(N, 20.0), np.arange(21.0)


CASES = [  # (workload, model, algorithm, reltol, abstol, mu filter, weighted bar,
           #  bar on the fraction of trajectories whose step counts change)
    ("lorenz", "MODEL_LORENZ", "ALG_TSIT5", 1e-8, 1e-8, None, 1.0, 0.01),
    ("robertson", "MODEL_ROBERTSON", "ALG_RODAS5", 1e-6, 1e-10, None, 1.0, 0.01),
    ("robertson", "MODEL_ROBERTSON", "ALG_ROSENBROCK23", 1e-6, 1e-10, None, 1.0, 0.01),
    ("vdp", "MODEL_VDP_RING8", "ALG_TSIT5", 1e-5, 1e-5, "nonstiff", 1.0, 0.01),
    ("vdp", "MODEL_VDP_RING8", "ALG_RODAS5", 1e-5, 1e-5, "stiff", 10.0, 0.03),
]


@pytest.mark.parametrize("case", CASES, ids=["-".join(c[:3:2]) + "-" + (c[5] or "")
                                             for c in CASES])
def test_fp32_series_controller_vs_fp64_pow(oracle, case):
    name, mid, alg, rt, at, part, bar, moved_bar = case
    rng = np.random.default_rng(SEED)
    p, u0, t0, tf, sv = _inputs(name, 1500, rng)
    if part is not None:
        keep = p[:, 0] > 100.0 if part == "stiff" else p[:, 0] <= 100.0
        p, u0, t0, tf = p[keep], u0[keep], t0[keep], tf[keep]
    kind = oracle.SAVE_PER_TRAJ if sv.ndim == 2 else oracle.SAVE_GRID
    if sv.ndim == 2:
        sv = sv[keep] if part is not None else sv
    o = oracle.opts_default(getattr(oracle, alg))
    o.reltol, o.abstol, o.maxiters = rt, at, 10 ** 6
    M = oracle.ModelRef(getattr(oracle, mid))
    try:
        oracle.set_controller(0)
        a = oracle.solve(None, M, o, p, u0, t0, tf, sv, kind, nthreads=8)
        oracle.set_controller(1)
        b = oracle.solve(None, M, o, p, u0, t0, tf, sv, kind, nthreads=8)
    finally:
        oracle.set_controller(0)
    assert np.all(a["retcode"] == oracle.RET_SUCCESS)
    assert np.all(b["retcode"] == oracle.RET_SUCCESS)
    moved = (a["naccept"] != b["naccept"]) | (a["nreject"] != b["nreject"])
    e = oracle.weighted_errors(a["u"], b["u"], at, rt).max(axis=(1, 2))
    print("%s %s: steps changed on %.2f %% of %d; weighted max %.3g p99 %.3g"
          % (name, alg, 100 * moved.mean(), len(moved), e.max(), np.percentile(e, 99)))
    assert moved.mean() <= moved_bar
    # where the step counts agree the solutions agree inside the bar (on the
    # stiff ring, whose jump times move with any change of step size: the
    # 99th percentile)
    kept = e[~moved]
    assert (np.percentile(kept, 99) if part == "stiff" else kept.max()) <= bar
    # the mean step count is unchanged to 0.5 %
    sa, sb = (a["naccept"] + a["nreject"]).mean(), (b["naccept"] + b["nreject"]).mean()
    assert abs(sa / sb - 1.0) <= 0.005


def test_weighted_error_nan_is_a_failure(oracle):
    """A NaN on one side only is an infinite error; NaN on both sides (save
    slots neither solve reached) is agreement."""
    ref = np.array([[1.0, 2.0, np.nan]])
    assert oracle.weighted_error(np.array([[1.0, 2.0, np.nan]]), ref, 1e-6, 1e-6) == 0.0
    assert oracle.weighted_error(np.array([[1.0, np.nan, np.nan]]), ref, 1e-6, 1e-6) == np.inf
    assert oracle.weighted_error(np.array([[1.0, 2.0, 3.0]]), ref, 1e-6, 1e-6) == np.inf
    assert oracle.weighted_error(np.array([[np.inf, 2.0, np.nan]]), ref, 1e-6, 1e-6) == np.inf
    inf = np.array([[np.inf]])
    assert oracle.weighted_error(inf, inf, 1e-6, 1e-6) == 0.0
    assert oracle.weighted_error(-inf, inf, 1e-6, 1e-6) == np.inf


def test_d2f_rn_bits_matches_the_conversion(oracle):
    """The controller narrows its error norm (clamped to [2^-120, 2^120]) to
    FP32 on the integer pipe: the same float as an IEEE round-to-nearest-even
    conversion, for random doubles, exact ties and values that round up
    across a power of two."""
    rng = np.random.default_rng(21)
    x = np.ldexp(rng.uniform(0.5, 1.0, 200000), rng.integers(-119, 121, 200000))
    x *= rng.choice([-1.0, 1.0], x.size)
    f = x.astype(np.float32).astype(np.float64)
    ulp = np.spacing(np.abs(x).astype(np.float32)).astype(np.float64)
    ties = np.concatenate([f + 0.5 * ulp, f - 0.5 * np.spacing(np.abs(f).astype(np.float32) * 0.5).astype(np.float64)])
    below_two = np.nextafter(np.ldexp(1.0, np.arange(-110, 111)), 0.0)
    xs = np.concatenate([x, ties, below_two, -below_two])
    xs = xs[(np.abs(xs) >= 2.0 ** -120) & (np.abs(xs) <= 2.0 ** 120)]
    got = oracle.d2f_rn(xs)
    want = xs.astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_controller_helpers_exact(oracle):
    """The controller's series use exact integer-pipe helpers instead of
    frexpf, int -> float, rintf and ldexpf: the same values over every input
    the controller gives them."""
    assert oracle.ctl_selfcheck() == 0
