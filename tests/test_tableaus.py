"""Order-condition pins of every coefficient table (tableaus.h,
dense_coeffs.h).  The reference ships no golden vectors for its solvers
(its tests pin only return codes, lengths and u[1] == u0, test/core.jl), so
the coefficients are pinned by the rooted-tree order conditions of the
methods' published orders."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "differentialequations.jl_gb300", "csrc")

import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("derive_dense_output",
                                               os.path.join(CSRC, "derive_dense_output.py"))
dd = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(dd)

TB = dd.parse_tableaus()
DENSE = dd.parse_tableaus(os.path.join(CSRC, "dense_coeffs.h"))
TREES = dd.trees(8)


def rk_residual(A, w, order):
    """max over trees with rho <= order of |w . Phi(t) - 1/gamma(t)|"""
    out = 0.0
    for n in range(1, order + 1):
        for t in TREES[n]:
            out = max(out, abs(w @ dd.rk_phi(t, A) - 1.0 / dd.tree_gamma(t)))
    return out


def tsit5():
    v = TB["tsit5"]
    A = np.zeros((7, 7))
    for i in range(2, 8):
        for j in range(1, i):
            A[i - 1, j - 1] = v["a%d%d" % (i, j)]
    b = A[6].copy()
    bt = np.array([v["bt%d" % j] for j in range(1, 8)])
    return A, b, b - bt, v


def test_tsit5_orders():
    A, b, bh, v = tsit5()
    c = np.array([0, v["c2"], v["c3"], v["c4"], v["c5"], 1, 1])
    assert np.allclose(A.sum(1), c, atol=1e-14)
    assert rk_residual(A, b, 5) < 1e-13
    assert rk_residual(A, bh, 4) < 1e-13
    assert rk_residual(A, b, 6) > 1e-6  # exactly order 5
    assert rk_residual(A, bh, 5) > 1e-6


@pytest.mark.parametrize("theta", [0.1, 0.35, 0.8])
def test_tsit5_interpolant(theta):
    A, b, _, v = tsit5()
    th = theta
    t2 = th * th
    w = np.array([
        v["r11"] * th * (th - v["r12"]) * (t2 - v["r13"] * th + v["r14"]),
        v["r21"] * t2 * (t2 - v["r22"] * th + v["r23"]),
        v["r31"] * t2 * (t2 - v["r32"] * th + v["r33"]),
        v["r41"] * (th - v["r42"]) * (th - v["r43"]) * t2,
        v["r51"] * (th - v["r52"]) * (th - v["r53"]) * t2,
        v["r61"] * (th - v["r62"]) * (th - v["r63"]) * t2,
        v["r71"] * (th - v["r72"]) * (th - v["r73"]) * t2])
    for n in range(1, 5):
        for t in TREES[n]:
            assert abs(w @ dd.rk_phi(t, A) - th ** n / dd.tree_gamma(t)) < 1e-13


def test_vern7_orders():
    A, b, bh = dd.vern7_tableau(TB)
    assert rk_residual(A, b, 7) < 1e-13
    assert rk_residual(A, bh, 6) < 1e-13
    assert rk_residual(A, b, 8) > 1e-7


@pytest.mark.parametrize("theta", [0.2, 0.5, 0.9, 1.0])
def test_vern7_dense_output(theta):
    A, b, _ = dd.vern7_tableau(TB)
    A2 = np.zeros((11, 11))
    A2[:10, :10] = A
    A2[10, :10] = b
    v = DENSE["vern7d"]
    w = np.array([sum(v["B%d_%d" % (j, k)] * theta ** k for k in range(1, 6))
                  for j in range(1, 12)])
    for n in range(1, 6):
        for t in TREES[n]:
            assert abs(w @ dd.rk_phi(t, A2) - theta ** n / dd.tree_gamma(t)) < 1e-12
    if theta == 1.0:
        assert np.allclose(w, np.append(b, 0.0), atol=1e-12)


@pytest.mark.parametrize("name", ["rodas5", "rodas5p"])
def test_rodas_orders(name):
    R = dd.rodas_tableau(TB, name)
    alpha, beta = R["alpha"], R["beta"]
    assert np.allclose(np.diag(R["G"]), R["gamma"])
    for w, p in ((R["m"] @ R["G"], 5), (R["mh"] @ R["G"], 4)):
        for n in range(1, p + 1):
            for t in TREES[n]:
                assert abs(w @ dd.ros_phi(t, alpha, beta) - 1.0 / dd.tree_gamma(t)) < 1e-12
    # stiffly accurate: y1 = U_8 + u_8 -> R(inf) = 0
    a = R["a"]
    ut = np.zeros(8)
    for i in range(8):
        ut[i] = -1.0 - a[i, :i] @ ut[:i]
    assert abs(1.0 + R["m"] @ ut) < 1e-10


@pytest.mark.parametrize("name", ["rodas5", "rodas5p"])
@pytest.mark.parametrize("theta", [0.25, 0.5, 0.75])
def test_rodas_dense_output(name, theta):
    R = dd.rodas_tableau(TB, name)
    v = DENSE[name + "d"]
    H = [np.array([v["H%d_%d" % (q, j)] for j in range(1, 8)] + [0.0]) for q in (2, 3, 4)]
    th = theta
    # transformed weights: theta m + theta(1-theta)(H2 + theta H3 + theta^2 H4)
    wt = th * R["m"] + th * (1 - th) * (H[0] + th * H[1] + th * th * H[2])
    w = wt @ R["G"]
    for n in range(1, 5):
        for t in TREES[n]:
            got = w @ dd.ros_phi(t, R["alpha"], R["beta"])
            assert abs(got - th ** n / dd.tree_gamma(t)) < 1e-11
    # stiff limit (1-theta)^4
    a = R["a"]
    ut = np.zeros(8)
    for i in range(8):
        ut[i] = -1.0 - a[i, :i] @ ut[:i]
    assert abs(1.0 + wt @ ut - (1 - th) ** 4) < 1e-10


def test_ros23_constants():
    v = TB["ros23"]
    assert abs(v["d"] - 1.0 / (2.0 + np.sqrt(2.0))) < 1e-16
    assert abs(v["e32"] - (6.0 + np.sqrt(2.0))) < 1e-15


def test_sriw1_strong_order_gbm():
    """SRIW1 (tableaus.h) has strong order ~1.5 on geometric Brownian motion
    dX = mu X dt + s X dW, whose exact solution is known given W."""
    v = TB["sriw1"]
    rng = np.random.default_rng(1)
    mu, sig, T, M, nfine = 1.5, 1.0, 1.0, 2000, 2 ** 11
    dtf = T / nfine
    W = np.concatenate([np.zeros((M, 1)),
                        np.cumsum(rng.normal(0, np.sqrt(dtf), (M, nfine)), 1)], 1)
    exact = np.exp((mu - sig ** 2 / 2) * T + sig * W[:, -1])
    A0 = np.zeros((4, 4)); A0[1, 0] = v["A0_21"]
    B0 = np.zeros((4, 4)); B0[1, 0] = v["B0_21"]
    A1 = np.zeros((4, 4)); A1[1, 0] = v["A1_21"]; A1[2, 0] = v["A1_31"]; A1[3, 2] = v["A1_43"]
    B1 = np.zeros((4, 4))
    B1[1, 0], B1[2, 0], B1[3, 0], B1[3, 1], B1[3, 2] = (v["B1_21"], v["B1_31"], v["B1_41"],
                                                        v["B1_42"], v["B1_43"])
    al = [v["al1"], v["al2"], 0, 0]
    bb = [[v["b%d_%d" % (q, i)] for i in range(1, 5)] for q in range(1, 5)]

    def run(n):
        h, k, x = T / n, nfine // n, np.ones(M)
        for s in range(n):
            Wi = W[:, s * k:(s + 1) * k + 1] - W[:, [s * k]]
            I1 = Wi[:, -1]
            I10 = np.trapezoid(Wi, dx=dtf, axis=1)
            I11, I111 = (I1 ** 2 - h) / 2, (I1 ** 3 - 3 * h * I1) / 6
            F, G, H0, H1 = [None] * 4, [None] * 4, [None] * 4, [None] * 4
            for i in range(4):
                H0[i] = x + sum(A0[i, j] * F[j] * h + B0[i, j] * G[j] * I10 / h for j in range(i))
                H1[i] = x + sum(A1[i, j] * F[j] * h + B1[i, j] * G[j] * np.sqrt(h) for j in range(i))
                F[i], G[i] = mu * H0[i], sig * H1[i]
            x = x + sum(al[i] * F[i] * h for i in range(4)) + sum(
                (bb[0][i] * I1 + bb[1][i] * I11 / np.sqrt(h) + bb[2][i] * I10 / h +
                 bb[3][i] * I111 / h) * G[i] for i in range(4))
        return np.mean(np.abs(x - exact))

    ns = [16, 32, 64, 128]
    e = np.array([run(n) for n in ns])
    slope = np.polyfit(np.log(1.0 / np.array(ns)), np.log(e), 1)[0]
    assert 1.25 < slope < 1.75, slope


def test_dense_coeffs_regenerate(tmp_path):
    """dense_coeffs.h is exactly what derive_dense_output.py produces."""
    import subprocess
    import shutil
    import sys
    work = tmp_path / "csrc"
    shutil.copytree(CSRC, work, ignore=shutil.ignore_patterns("*.o"))
    subprocess.check_call([sys.executable, str(work / "derive_dense_output.py")])
    assert (work / "dense_coeffs.h").read_text() == open(os.path.join(CSRC, "dense_coeffs.h")).read()
