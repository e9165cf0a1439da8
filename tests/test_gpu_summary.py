"""Ensemble statistics on the device (EnsembleSummary / EnsembleAnalysis,
test/qa/qa.jl:54,211): mean, variance and exact quantiles per save point and
component across trajectories, against numpy's mean, var(ddof=1) and
quantile(method="linear") -- the defaults of Julia's Statistics."""
import numpy as np
import pytest

QS = (0.0, 0.05, 0.333, 0.5, 0.95, 1.0)


def _check(de, u, qs=QS, device_mode=False, rtol_q=1e-12):
    import torch
    uu = torch.from_numpy(u).cuda() if device_mode else u
    mean, var, qv = de.ensemble_summary(uu, qs)
    if device_mode:
        mean, var, qv = mean.cpu().numpy(), var.cpu().numpy(), qv.cpu().numpy()
    ref = u.astype(np.float64)
    np.testing.assert_allclose(mean, ref.mean(0), rtol=1e-12, atol=1e-12)
    if u.shape[0] > 1:
        np.testing.assert_allclose(var, ref.var(0, ddof=1), rtol=1e-9, atol=1e-12)
    else:
        assert np.all(np.isnan(var))
    for j, q in enumerate(qs):
        np.testing.assert_allclose(qv[j], np.quantile(ref, q, axis=0, method="linear"),
                                   rtol=rtol_q, atol=0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("device_mode", [False, True], ids=["host", "device"])
def test_summary_vs_numpy(de, dtype, device_mode):
    rng = np.random.default_rng(1)
    u = rng.standard_normal((1001, 7, 3)) * np.array([1.0, 1e3, 1e-4]) + np.array([0.0, -5.0, 2.0])
    u[::17] *= 40.0  # outliers
    _check(de, u.astype(dtype), device_mode=device_mode)


@pytest.mark.gpu
def test_summary_ties_signs_even_n(de):
    rng = np.random.default_rng(2)
    u = np.round(rng.standard_normal((2000, 5, 2)) * 3.0) / 2.0  # many exact ties
    u[:, 0, 0] = 0.0
    u[::2, 0, 0] = -0.0
    _check(de, u)
    _check(de, u[:1999])


@pytest.mark.gpu
def test_summary_single_trajectory_and_nan_column(de):
    rng = np.random.default_rng(3)
    _check(de, rng.standard_normal((1, 4, 2)))
    u = rng.standard_normal((300, 4, 2))
    u[7, 2, 1] = np.nan  # an unreached save slot of a failed trajectory
    mean, var, qv = de.ensemble_summary(u, (0.05, 0.95))
    assert np.isnan(mean[2, 1]) and np.isnan(var[2, 1]) and np.all(np.isnan(qv[:, 2, 1]))
    ok = np.ones((4, 2), bool)
    ok[2, 1] = False
    np.testing.assert_allclose(mean[ok], u.mean(0)[ok], rtol=1e-12)
    np.testing.assert_allclose(qv[1][ok], np.quantile(u, 0.95, axis=0)[ok], rtol=1e-12)


@pytest.mark.gpu
def test_summary_large_ensemble_properties(de):
    """1M trajectories x 21 saves x 16 states in FP32 (the 16-state ring's
    output size): q=0 / q=1 are the column minima / maxima, the median
    brackets half the values, and the mean matches torch's."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(0)
    u = torch.randn((1_000_000, 21, 16), generator=g, device="cuda", dtype=torch.float32)
    u.mul_(torch.linspace(0.1, 3.0, 16, device="cuda"))
    mean, var, qv = de.ensemble_summary(u, (0.0, 0.5, 1.0))
    torch.testing.assert_close(qv[0], u.amin(0).double(), rtol=0, atol=0)
    torch.testing.assert_close(qv[2], u.amax(0).double(), rtol=0, atol=0)
    below = (u.double() < qv[1]).double().mean(0)
    assert float((below - 0.5).abs().max()) < 1e-5
    torch.testing.assert_close(mean, u.double().mean(0), rtol=1e-9, atol=1e-9)
    torch.testing.assert_close(var, u.double().var(0), rtol=1e-7, atol=1e-9)


@pytest.mark.gpu
def test_ensemble_summary_of_a_solve(de):
    """EnsembleSummary of a Lorenz ensemble solved on the GPU."""
    rng = np.random.default_rng(4)
    N = 5000
    p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
    ens = de.EnsembleProblem(de.ODEProblem(de.models.lorenz, [1.0, 0.0, 0.0], (0.0, 1.0),
                                           [10.0, 28.0, 8.0 / 3.0]),
                             batch=lambda prob, n: {"p": p})
    sol = de.solve(ens, de.Tsit5(), de.EnsembleGB300(), trajectories=N, saveat=0.1,
                   reltol=1e-8, abstol=1e-8)
    sm = de.EnsembleSummary(sol)
    assert sm.num_monte == N and sm.converged
    np.testing.assert_allclose(sm.u, sol.U.mean(0), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(sm.qlow, np.quantile(sol.U, 0.05, axis=0), rtol=1e-12)
    np.testing.assert_allclose(sm.med, np.median(sol.U, axis=0), rtol=1e-12)
