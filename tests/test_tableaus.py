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


def sri_table(name):
    """Full 4 x 4 arrays of an SRI table parsed from tableaus.h (entries not
    listed are zero)."""
    v = TB[name]
    M = {k: np.zeros((4, 4)) for k in ("A0", "B0", "A1", "B1")}
    for key, val in v.items():
        if key[:2] in M and "_" in key:
            i, j = int(key[3]) - 1, int(key[4]) - 1
            M[key[:2]][i, j] = val
    al = np.array([v.get("al%d" % i, 0.0) for i in range(1, 5)])
    b = np.array([[v["b%d_%d" % (q, i)] for i in range(1, 5)] for q in range(1, 5)])
    return M["A0"], M["B0"], M["A1"], M["B1"], al, b


def sri_conditions(A0, B0, A1, B1, al, b):
    """Roessler's conditions for strong order 1.5 of an SRI method with
    diagonal noise (SIAM J. Numer. Anal. 48 (2010)), as residuals."""
    e = np.ones(4)
    b1, b2, b3, b4 = b
    B1e, B0e, A1e = B1 @ e, B0 @ e, A1 @ e
    return {
        "a.e=1": al @ e - 1, "b1.e=1": b1 @ e - 1, "b2.e=0": b2 @ e, "b3.e=0": b3 @ e,
        "b4.e=0": b4 @ e,
        "b1.B1e=0": b1 @ B1e, "b2.B1e=1": b2 @ B1e - 1, "b3.B1e=0": b3 @ B1e, "b4.B1e=0": b4 @ B1e,
        "a.A0e=1/2": al @ A0 @ e - 0.5, "a.B0e=1": al @ B0e - 1, "a.(B0e)^2=3/2": al @ B0e ** 2 - 1.5,
        "b1.A1e=1": b1 @ A1e - 1, "b2.A1e=0": b2 @ A1e, "b3.A1e=-1": b3 @ A1e + 1, "b4.A1e=0": b4 @ A1e,
        "b1.(B1e)^2=1": b1 @ B1e ** 2 - 1, "b2.(B1e)^2=0": b2 @ B1e ** 2,
        "b3.(B1e)^2=-1": b3 @ B1e ** 2 + 1, "b4.(B1e)^2=2": b4 @ B1e ** 2 - 2,
        "b1.B1B1e=0": b1 @ B1 @ B1e, "b2.B1B1e=0": b2 @ B1 @ B1e, "b3.B1B1e=0": b3 @ B1 @ B1e,
        "b4.B1B1e=1": b4 @ B1 @ B1e - 1,
        "b1.A1B0e/2+b3.A1B0e/3=0": 0.5 * b1 @ A1 @ B0e + b3 @ A1 @ B0e / 3.0,
    }


@pytest.mark.parametrize("name", ["sriw1", "sosri"])
def test_sri_order_conditions(name):
    """SRIW1 (Roessler 2010) and SOSRI (Rackauckas & Nie 2018) satisfy the
    strong-order-1.5 conditions.  SOSRI's published coefficients come from a
    numerical optimisation: the two conditions on B0 hold to ~7e-11, the rest
    to rounding."""
    res = sri_conditions(*sri_table(name))
    for k, r in res.items():
        tol = 1e-9 if (name == "sosri" and "B0e" in k and "A1" not in k) else 1e-14
        assert abs(r) < tol, (name, k, r)


def test_sosri_is_not_sriw1():
    """The SOSRI slot holds the stability-optimised table (all stages used),
    not SRIW1's."""
    A0, B0, A1, B1, al, b = sri_table("sosri")
    assert np.all(al != 0) and np.count_nonzero(A0) == 6 and np.count_nonzero(B1) == 6
    assert not np.allclose(al, sri_table("sriw1")[4])


@pytest.mark.parametrize("name", ["sriw1", "sosri"])
def test_sri_strong_order_gbm(name):
    """SRIW1 and SOSRI (tableaus.h) have strong order ~1.5 on geometric
    Brownian motion dX = mu X dt + s X dW, whose exact solution is known
    given W."""
    A0, B0, A1, B1, al, bb = sri_table(name)
    rng = np.random.default_rng(1)
    mu, sig, T, M, nfine = 1.5, 1.0, 1.0, 2000, 2 ** 11
    dtf = T / nfine
    W = np.concatenate([np.zeros((M, 1)),
                        np.cumsum(rng.normal(0, np.sqrt(dtf), (M, nfine)), 1)], 1)
    exact = np.exp((mu - sig ** 2 / 2) * T + sig * W[:, -1])

    def run(n):
        h, k, x = T / n, nfine // n, np.ones(M)
        for s in range(n):
            Wi = W[:, s * k:(s + 1) * k + 1] - W[:, [s * k]]
            I1 = Wi[:, -1]
            I10 = np.trapezoid(Wi, dx=dtf, axis=1)
            I11, I111 = (I1 ** 2 - h) / 2, (I1 ** 3 - 3 * h * I1) / 6
            F, G = [None] * 4, [None] * 4
            for i in range(4):
                H0 = x + sum(A0[i, j] * F[j] * h + B0[i, j] * G[j] * I10 / h for j in range(i))
                H1 = x + sum(A1[i, j] * F[j] * h + B1[i, j] * G[j] * np.sqrt(h) for j in range(i))
                F[i], G[i] = mu * H0, sig * H1
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


@pytest.mark.parametrize("theta", [0.1, 0.37, 0.5, 0.9, 1.0])
def test_vern7_dense_output_order7(theta):
    """Vern7's dense output (dense_coeffs.h, vern7l) is a 7th-order continuous
    extension: over the 18 stages (Vern7's 10, f(t+h, y1), three lazy stages
    on the 5th-order extension, four on the degree-6 interpolant) its weights
    satisfy every order condition up to order 7 at each theta, and not all of
    order 8."""
    A, b, _ = dd.vern7_tableau(TB)
    v = DENSE["vern7l"]
    S = 18
    AA = np.zeros((S, S))
    AA[:10, :10] = A
    AA[10, :10] = b
    for i in range(3):
        AA[11 + i, :11] = [v["L1_%d_%d" % (i + 1, j + 1)] for j in range(11)]
    for i in range(4):
        AA[14 + i, :14] = [v["L2_%d_%d" % (i + 1, j + 1)] for j in range(14)]
    w = np.array([sum(v["D%d_%d" % (j + 1, m)] * theta ** m for m in range(1, 8))
                  for j in range(S)])
    for n in range(1, 8):
        for t in TREES[n]:
            assert abs(w @ dd.rk_phi(t, AA) - theta ** n / dd.tree_gamma(t)) < 1e-11, (n, t)
    assert max(abs(w @ dd.rk_phi(t, AA) - theta ** 8 / dd.tree_gamma(t)) for t in TREES[8]) > 1e-7
    # the extra stages sit where their abscissae say
    c = AA.sum(1)
    assert np.allclose(c[11:14], [v["TH1_%d" % i] for i in (1, 2, 3)], atol=1e-12)
    assert np.allclose(c[14:18], [v["TH2_%d" % i] for i in (1, 2, 3, 4)], atol=1e-12)
    if theta == 1.0:
        assert np.allclose(w[:10], b, atol=1e-12)  # the interpolant ends at y1
