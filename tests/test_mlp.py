"""The learned predictor's network: the CPU oracle (oracle/mlp_oracle.py)
pinned by finite differences and by torch's BF16 rounding, the library's
initialiser, and (on the GPU) the library's forward / gradient kernels
against the oracle, training, and what the trained predictor gains inside a
solve over the method without it."""
import numpy as np
import pytest

import mlp_oracle as M


def random_net(capi, de, seed):
    net = de.learned.init(seed)
    rng = np.random.default_rng(seed)
    net[M.OFF_B1:M.OFF_W2] = rng.normal(0, 0.1, M.HID)
    net[M.OFF_B4:M.NPARAM] = rng.normal(0, 0.1, M.OUT)
    net[M.OFF_XMEAN:M.OFF_XSCALE] = rng.normal(0, 1, M.IN)
    net[M.OFF_XSCALE:M.OFF_YMEAN] = rng.uniform(0.5, 2, M.IN)
    net[M.OFF_YMEAN], net[M.OFF_YSCALE] = -2.0, 1.5
    net[M.OFF_CMEAN], net[M.OFF_CSCALE] = 6.0, 0.8
    return net


def batch(rng, n):
    x = rng.normal(0, 1.5, (n, M.IN)).astype(np.float32)
    y = np.c_[rng.normal(-2, 1.5, n), (rng.uniform(size=n) < 0.4),
              rng.normal(6, 1, n)].astype(np.float32)
    y[rng.uniform(size=n) < 0.1, 0] = np.nan  # unlabelled dt
    y[rng.uniform(size=n) < 0.2, 1] = np.nan  # unlabelled stiffness
    y[rng.uniform(size=n) < 0.15, 2] = np.nan  # unlogged cost
    return x, y


def test_init_layout(capi, de):
    a, b = de.learned.init(7), de.learned.init(7)
    assert a.shape == (capi.MLP_NET_FLOATS,) == (M.NET_FLOATS,) and capi.MLP_PARAMS == M.NPARAM
    assert np.array_equal(a, b) and not np.array_equal(a, de.learned.init(8))
    assert np.all(a[M.OFF_B1:M.OFF_W2] == 0) and np.all(a[M.OFF_XSCALE:M.OFF_YMEAN] == 1)
    lim = np.sqrt(6.0 / M.HID)
    assert np.abs(a[M.OFF_W2:M.OFF_B2]).max() <= lim


def test_oracle_bf16_matches_torch():
    import torch
    x = np.random.default_rng(0).normal(0, 10, 10000).astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(M.bf16(x), ref)


def test_oracle_gradient_finite_differences(capi, de):
    """FP64 oracle: analytic gradient == central differences."""
    rng = np.random.default_rng(3)
    net = random_net(capi, de, 3).astype(np.float64)
    x, y = batch(rng, 64)
    _, g = M.loss_and_grad(net, x, y, bf=False)
    idx = np.r_[rng.choice(M.NPARAM, 60, replace=False), M.OFF_B4, M.OFF_B4 + 1, M.OFF_B4 + 2]
    for i in idx:
        h = 1e-6 * max(1.0, abs(net[i]))
        a, b = net.copy(), net.copy()
        a[i] += h
        b[i] -= h
        fd = (M.loss_and_grad(a, x, y, bf=False)[0] - M.loss_and_grad(b, x, y, bf=False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])


@pytest.mark.gpu
def test_gpu_forward_vs_oracle(capi, de):
    rng = np.random.default_rng(4)
    net = random_net(capi, de, 4)
    x, _ = batch(rng, 1000)
    y = de.learned.forward(net, x)
    ref, _ = M.forward(net, x, bf=True)
    assert np.max(np.abs(y - ref)) <= 1e-2 * np.max(np.abs(ref)) + 1e-3


@pytest.mark.gpu
def test_gpu_gradient_vs_oracle(capi, de):
    """The library's backward kernel against the oracle at the same BF16
    rounding points: loss to 1e-4, every weight tensor's gradient to 2% (L2)."""
    rng = np.random.default_rng(5)
    net = random_net(capi, de, 5)
    x, y = batch(rng, 777)
    loss, g = de.learned.grad(net, x, y)
    lref, gref = M.loss_and_grad(net, x, y, bf=True)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    cuts = [M.OFF_W1, M.OFF_B1, M.OFF_W2, M.OFF_B2, M.OFF_W3, M.OFF_B3, M.OFF_W4, M.OFF_B4, M.NPARAM]
    for a, b in zip(cuts[:-1], cuts[1:]):
        err = np.linalg.norm(g[a:b] - gref[a:b]) / (np.linalg.norm(gref[a:b]) + 1e-30)
        assert err <= 2e-2, (a, b, err)


@pytest.mark.gpu
def test_gpu_training_fits(capi, de):
    """Training on the GPU fits two smooth synthetic targets and a label."""
    rng = np.random.default_rng(6)
    n = 40000

    def targets(x):
        return (np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2] - 3.0, (x[:, 3] + x[:, 4] > 0),
                5.0 + x[:, 5] - 0.5 * x[:, 6] ** 2)

    x = rng.uniform(-1, 1, (n, M.IN)).astype(np.float32)
    y = np.stack(targets(x), 1).astype(np.float32)
    net, hist = de.learned.train(x, y, epochs=30, batch=1024, lr=2e-3, seed=1)
    assert hist[-1] < 0.25 * hist[0], hist
    xt = rng.uniform(-1, 1, (5000, M.IN)).astype(np.float32)
    dt, st, cost = de.learned.predict(net, xt)
    t0, t1, t2 = targets(xt)
    assert np.median(np.abs(np.log10(dt) - t0)) < 0.1
    assert np.mean(st == t1) > 0.9
    assert np.median(np.abs(np.log2(cost) - t2)) < 0.1


def _lorenz(de, N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    return p, np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), np.ones(N)


@pytest.mark.gpu
def test_learned_first_dt_lorenz(capi, de, oracle):
    """Trained on the solver's own step logs, the predicted first step
    replaces the Hairer-Wanner starting step (one f evaluation and its
    norms): results stay within tolerance of the FP64 oracle, every step is
    still error-controlled, and the solve saves f evaluations."""
    model = de.models.lorenz
    grid = de.save_grid(0.0, 1.0, 0.1)
    o = capi.opts_default(capi.ALG_TSIT5)
    o.reltol = o.abstol = 1e-8
    p, u0, t0, tf = _lorenz(de, 20000, 1)
    r = de.solve_arrays(model, o, p, u0, t0, tf, grid, capi.SAVE_GRID)
    x = de.learned.features(model, p, u0, t0, tf)
    y = np.c_[np.log10(r["dt_first"]), np.zeros(len(p)),
              de.learned.cost_targets(r["naccept"], r["nreject"])].astype(np.float32)
    net, hist = de.learned.train(x, y, epochs=20, batch=1024, seed=2)
    de.learned.load(model, net)
    p, u0, t0, tf = _lorenz(de, 5000, 99)  # held out
    plain = de.solve_arrays(model, o, p, u0, t0, tf, grid, capi.SAVE_GRID)
    o.learned = 1
    lr = de.solve_arrays(model, o, p, u0, t0, tf, grid, capi.SAVE_GRID)
    assert np.all(lr["retcode"] == capi.RET_SUCCESS)
    ref = oracle.solve(capi, model, _o(capi, 1e-8),
                       p, u0, t0, tf, grid, capi.SAVE_GRID, nthreads=8)
    assert oracle.weighted_error(lr["u"], ref["u"], 1e-8, 1e-8) <= 10.0
    pred, _, _ = de.learned.predict(net, de.learned.features(model, p, u0, t0, tf))
    assert np.median(np.abs(np.log10(pred / plain["dt_first"]))) < 0.15
    assert lr["nf"].sum() < plain["nf"].sum()


def _o(capi, tol, alg=None):
    o = capi.opts_default(alg or capi.ALG_TSIT5)
    o.reltol = o.abstol = tol
    return o


@pytest.mark.gpu
def test_learned_stiffness_vdp(capi, de):
    """On the ring of Van der Pol oscillators (mu log-uniform in [0.1, 1000])
    the predictor learns from measured costs which trajectories Rodas5 solves
    more cheaply than Tsit5; learned AUTO then costs less than the default
    threshold rule, and every trajectory still succeeds."""
    model = de.models.vdp_ring8
    grid = de.save_grid(0.0, 20.0, 1.0)

    def inputs(N, seed):
        rng = np.random.default_rng(seed)
        return (np.c_[10 ** rng.uniform(-1, 3, N), np.full(N, 0.05)], rng.uniform(-2, 2, (N, 16)),
                np.zeros(N), np.full(N, 20.0))

    p, u0, t0, tf = inputs(16000, 3)
    lab, cost = de.learned.stiff_labels(de.solve_arrays, model, p, u0, t0, tf, grid,
                                        capi.SAVE_GRID, 1e-5, 1e-5)
    o = _o(capi, 1e-5, capi.ALG_AUTO)
    o.maxiters = 10 ** 6
    r = de.solve_arrays(model, o, p, u0, t0, tf, grid, capi.SAVE_GRID)
    x = de.learned.features(model, p, u0, t0, tf)
    y = np.c_[np.log10(r["dt_first"]), lab, np.full(len(p), np.nan)].astype(np.float32)
    net, _ = de.learned.train(x, y, epochs=40, batch=1024, seed=4)
    de.learned.load(model, net)
    p, u0, t0, tf = inputs(8000, 77)  # held out
    lab_t, _ = de.learned.stiff_labels(de.solve_arrays, model, p, u0, t0, tf, grid,
                                       capi.SAVE_GRID, 1e-5, 1e-5)
    runs = {}
    for name, learned in (("threshold", 0), ("learned", 1)):
        o.learned = learned
        o.precision = capi.PREC_MIXED
        runs[name] = de.solve_arrays(model, o, p, u0, t0, tf, grid, capi.SAVE_GRID, u_dtype="f32")
        assert np.all(runs[name]["retcode"] == capi.RET_SUCCESS)

    def units(rr):  # device cost: steps x measured time per step of the method used
        steps = rr["naccept"] + rr["nreject"]
        c = np.where(rr["method"] == capi.ALG_RODAS5, cost["rodas5_ms_per_step"],
                     cost["tsit5_ms_per_step"])
        return float((steps * c).sum())

    chosen = (runs["learned"]["method"] == capi.ALG_RODAS5).astype(np.float32)
    assert np.mean(chosen == lab_t) > 0.85
    assert units(runs["learned"]) < units(runs["threshold"])


def _robertson(N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    tf = 10 ** rng.uniform(1, 5, N)
    saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
    return p, np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), tf, np.ascontiguousarray(saveat)


@pytest.mark.gpu
def test_learned_queue_order_robertson(capi, de):
    """Trained on the attempted-step logs of a Rodas5 solve, the cost head
    predicts held-out step counts closely (R^2 > 0.9), and a persistent solve
    whose queue is ordered by the predicted cost (learned = LEARN_ORDER)
    gives bit-identical results to the span-ordered one: the order decides
    only which lane runs a trajectory when."""
    model = de.models.robertson
    o = capi.opts_default(capi.ALG_RODAS5)
    o.reltol, o.abstol = 1e-6, 1e-10
    o.batching = capi.BATCH_PERSISTENT
    o.precision = capi.PREC_F32X2
    p, u0, t0, tf, sv = _robertson(20000, 11)
    r = de.solve_arrays(model, o, p, u0, t0, tf, sv, capi.SAVE_PER_TRAJ)
    x = de.learned.features(model, p, u0, t0, tf)
    y = np.c_[np.full(len(p), np.nan), np.full(len(p), np.nan),
              de.learned.cost_targets(r["naccept"], r["nreject"])].astype(np.float32)
    net, _ = de.learned.train(x, y, epochs=20, batch=1024, seed=5)
    de.learned.load(model, net)
    p, u0, t0, tf, sv = _robertson(8000, 12)  # held out
    base = de.solve_arrays(model, o, p, u0, t0, tf, sv, capi.SAVE_PER_TRAJ)
    steps = (base["naccept"] + base["nreject"]).astype(np.float64)
    _, _, pred = de.learned.predict(net, de.learned.features(model, p, u0, t0, tf))
    r2 = 1 - np.sum((np.log2(steps) - np.log2(pred)) ** 2) / np.sum(
        (np.log2(steps) - np.log2(steps).mean()) ** 2)
    assert r2 > 0.9, r2
    o.learned = capi.LEARN_ORDER
    lo = de.solve_arrays(model, o, p, u0, t0, tf, sv, capi.SAVE_PER_TRAJ)
    for k in ("u", "retcode", "naccept", "nreject", "nf", "t_end"):
        assert np.array_equal(lo[k], base[k], equal_nan=(k == "u")), k
