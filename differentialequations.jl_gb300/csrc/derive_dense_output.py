"""Derive the dense-output coefficients that are this library's own.

Writes ``dense_coeffs.h`` beside this file.  Run: ``python derive_dense_output.py``.

1. Vern7 5th-order continuous extension.  Stages 1..10 of Verner's 7(6) pair
   plus stage 11 = f(t + h, y1) (the next step's first stage, so it costs no
   extra evaluation on accepted steps).  Weights b_j(theta) = sum_k B[j,k]
   theta^k, k = 1..5, solve the continuous order conditions
       sum_j b_j(theta) Phi_j(t) = theta^rho(t) / gamma(t)   (rho(t) <= 5)
   as polynomial identities, plus b_j(1) = b_j (the interpolant ends at y1);
   minimum-norm solution.

2. Vern7 7th-order continuous extension by bootstrapping (Enright, Jackson,
   Norsett, Thomsen, ACM TOMS 12 (1986)): three extra stages on the 5th-order
   extension, a degree-6 Hermite-Birkhoff interpolant through y0, y1, f0, f1
   and their values, four more stages on it and the degree-7 interpolant;
   checked here against the order-7 conditions over all 18 stages.

3. Rodas5 / Rodas5P 4th-order continuous extension in transformed variables
       y(theta) = (1-theta) y0 + theta y1
                  + theta (1-theta) sum_j (H2_j + theta H3_j + theta^2 H4_j) u_j
   over stages 1..7: the continuous order conditions up to order 4
   (Rosenbrock elementary weights, Hairer-Wanner IV.7) plus
   R_theta(inf) = (1-theta)^4 on y' = lambda y; a square full-rank system.

The tree machinery here is the same as in tests/test_tableaus.py.
"""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_tableaus(path=os.path.join(HERE, "tableaus.h")):
    """Return {namespace: {name: value}} from `constexpr double` lines."""
    out, ns = {}, None
    for line in open(path):
        m = re.match(r"\s*namespace (\w+) \{", line)
        if m and m.group(1) not in ("gbde", "tab"):
            ns = m.group(1)
            out[ns] = {}
        m = re.match(r"\s*constexpr double (\w+) = ([-+0-9.eE]+);", line)
        if m and ns:
            out[ns][m.group(1)] = float(m.group(2))
    return out


# ---------------------------------------------------------------- trees
def trees(order):
    """Rooted trees by order; a tree is a sorted tuple of subtrees."""
    T = {1: [()]}
    for n in range(2, order + 1):
        res = set()

        def gen(rem, maxkey):
            if rem == 0:
                yield ()
                return
            for k in range(rem, 0, -1):
                for st in T[k]:
                    key = (k, st)
                    if maxkey is not None and key > maxkey:
                        continue
                    for rest in gen(rem - k, key):
                        yield (st,) + rest

        for c in gen(n - 1, None):
            res.add(tuple(sorted(c)))
        T[n] = sorted(res)
    return T


def rho(t):
    return 1 + sum(rho(s) for s in t)


def tree_gamma(t):
    g = rho(t)
    for s in t:
        g *= tree_gamma(s)
    return g


def rk_phi(t, A):
    v = np.ones(A.shape[0])
    for st in t:
        v = v * (A @ rk_phi(st, A))
    return v


def ros_phi(t, alpha, beta):
    """Rosenbrock elementary weights: a single-subtree node uses
    beta = alpha + Gamma (diagonal included), a multi-subtree node alpha."""
    s = alpha.shape[0]
    if len(t) == 0:
        return np.ones(s)
    if len(t) == 1:
        return beta @ ros_phi(t[0], alpha, beta)
    v = np.ones(s)
    for st in t:
        v = v * (alpha @ ros_phi(st, alpha, beta))
    return v


# ---------------------------------------------------------------- tables
def vern7_tableau(tb):
    v = tb["vern7"]
    A = np.zeros((10, 10))
    for i in range(2, 11):
        for j in range(1, i):
            key = "a%d%d" % (i, j)
            if key in v:
                A[i - 1, j - 1] = v[key]
    b = np.zeros(10)
    bh = np.zeros(10)
    for j in range(1, 11):
        b[j - 1] = v.get("b%d" % j, 0.0)
        bh[j - 1] = v.get("bh%d" % j, 0.0)
    return A, b, bh


def rodas_tableau(tb, name):
    v = tb[name]
    s = 8
    a = np.zeros((s, s))
    C = np.zeros((s, s))
    for i in range(2, 7):
        for j in range(1, i):
            a[i - 1, j - 1] = v["a%d%d" % (i, j)]
    a[6, :5] = a[5, :5]
    a[6, 5] = 1.0
    a[7, :6] = a[6, :6]
    a[7, 6] = 1.0
    for i in range(2, 9):
        for j in range(1, i):
            C[i - 1, j - 1] = v["C%d%d" % (i, j)]
    g = v["gamma"]
    m = np.zeros(s)
    m[:7] = a[7, :7]
    m[7] = 1.0
    mh = m.copy()
    mh[7] = 0.0
    Ginv = np.diag(np.full(s, 1.0 / g)) - C
    G = np.linalg.inv(Ginv)
    alpha = a @ G
    return dict(a=a, C=C, gamma=g, m=m, mh=mh, G=G, alpha=alpha, beta=alpha + G)


# ---------------------------------------------------------------- Vern7
def derive_vern7(tb, q=5):
    A, b, _ = vern7_tableau(tb)
    s = 11
    A2 = np.zeros((s, s))
    A2[:10, :10] = A
    A2[10, :10] = b
    b2 = np.append(b, 0.0)
    T = trees(q)
    # stages 2 and 3 carry no weight in Vern7 (b2 = b3 = 0); keep them at 0
    use = [j for j in range(s) if j not in (1, 2)]
    nu = len(use)
    rows, rhs = [], []
    nun = nu * q  # unknown B[use[j],k] at index j*q + (k-1)
    for n in range(1, q + 1):
        for t in T[n]:
            phi = rk_phi(t, A2)[use]
            for k in range(1, q + 1):
                r = np.zeros(nun)
                r[np.arange(nu) * q + (k - 1)] = phi
                rows.append(r)
                rhs.append(1.0 / tree_gamma(t) if k == n else 0.0)
    for jj, j in enumerate(use):
        r = np.zeros(nun)
        r[jj * q:(jj + 1) * q] = 1.0
        rows.append(r)
        rhs.append(b2[j])
    M = np.array(rows)
    y = np.array(rhs)
    x = np.linalg.lstsq(M, y, rcond=None)[0]
    resid = np.abs(M @ x - y).max()
    assert resid < 1e-12, resid
    B = np.zeros((s, q))
    B[use] = x.reshape(nu, q)
    return B, resid


# -------------------------------------------- Vern7, 7th-order interpolant
# Level-1 and level-2 abscissae of the bootstrapped interpolant (chosen for a
# small order-8 defect and moderate coefficients; the Hermite-Birkhoff systems
# are nonsingular for them).
V7_THETA1 = (0.12, 0.25, 0.78)
V7_THETA2 = (0.11, 0.22, 0.55, 0.75)


def _hermite_birkhoff(nstage, nodes, node_stages, b, deg):
    """Coefficients of u(theta) = y0 + h sum_{m=1..deg} c_m theta^m with
    u(1) = y1 = y0 + h b.K, u'(0) = h K_1, u'(1) = h K_11 (= f(y1)) and
    u'(theta_i) = h K_{node_stages[i]}: returns C (deg x nstage) with
    c_m = sum_j C[m-1, j] K_j."""
    V, R = [], []
    V.append(np.ones(deg))
    r = np.zeros(nstage)
    r[:len(b)] = b
    R.append(r)
    v = np.zeros(deg)
    v[0] = 1.0
    V.append(v)
    r = np.zeros(nstage)
    r[0] = 1.0
    R.append(r)
    V.append(np.arange(1, deg + 1, dtype=float))
    r = np.zeros(nstage)
    r[10] = 1.0
    R.append(r)
    for th, j in zip(nodes, node_stages):
        V.append(np.arange(1, deg + 1) * th ** np.arange(0, deg))
        r = np.zeros(nstage)
        r[j] = 1.0
        R.append(r)
    V = np.array(V)
    assert V.shape == (deg, deg)
    return np.linalg.solve(V, np.array(R))


def derive_vern7_lazy(tb, B5):
    """7th-order continuous extension of Vern7 by bootstrapping (W.H. Enright,
    K.R. Jackson, S.P. Norsett, P.G. Thomsen, "Interpolants for Runge-Kutta
    formulas", ACM TOMS 12 (1986) 193-218): stages 1-10 of Vern7 and
    K11 = f(y1); three stages at theta in V7_THETA1 on the 5th-order
    extension (local error O(h^6)) feed a degree-6 Hermite-Birkhoff
    interpolant (y0, y1, f0, f1 and their derivatives: O(h^7)); four stages at
    theta in V7_THETA2 on that one feed the degree-7 interpolant (O(h^8),
    order 7).  The seven extra stages are evaluated only on steps that save.
    Returns (AA: 18 x 18 stage matrix, W1 3 x 11, W2 4 x 14, C7 7 x 18)."""
    A, b, _ = vern7_tableau(tb)
    S = 18
    AA = np.zeros((S, S))
    AA[:10, :10] = A
    AA[10, :10] = b
    W1 = np.array([B5 @ (th ** np.arange(1, 6)) for th in V7_THETA1])
    AA[11:14, :11] = W1
    C6 = _hermite_birkhoff(14, V7_THETA1, (11, 12, 13), b, 6)
    W2 = np.array([(th ** np.arange(1, 7)) @ C6 for th in V7_THETA2])
    AA[14:18, :14] = W2
    C7 = _hermite_birkhoff(S, V7_THETA2, (14, 15, 16, 17), b, 7)
    return AA, W1, W2, C7


# ---------------------------------------------------------------- Rodas
def derive_rodas(tb, name):
    """4th-order continuous extension over stages u_1..u_7:
    y(theta) = (1-theta) y0 + theta y1 + theta(1-theta)(K2 + theta K3 + theta^2 K4),
    K_q = sum_j H_q[j] u_j.  Conditions (as polynomials in theta):
      rho(t)=1: H2.Phi = H3.Phi = H4.Phi = 0
      rho(t)=2: H2.Phi = -1/2, H3.Phi = H4.Phi = 0
      rho(t)=3: H2.Phi = H3.Phi = -1/gamma(t), H4.Phi = 0
      rho(t)=4: H2.Phi = H3.Phi = H4.Phi = -1/gamma(t)
    (Phi = Gamma times the Rosenbrock elementary weights), plus the stiff
    limit R_theta(inf) = (1-theta)^4 on y' = lambda y.  The system is square
    and of full rank: the solution is unique."""
    R = rodas_tableau(tb, name)
    s = 8
    ns = 7
    G, alpha, beta, a = R["G"], R["alpha"], R["beta"], R["a"]
    T = trees(4)
    ut = np.zeros(s)
    for i in range(s):
        ut[i] = -1.0 - a[i, :i] @ ut[:i]
    minf = R["m"] @ ut
    assert abs(minf + 1.0) < 1e-10, minf  # L-stable step
    rows, rhs = [], []
    for n in range(1, 5):
        for t in T[n]:
            gp = (G @ ros_phi(t, alpha, beta))[:ns]
            g = tree_gamma(t)
            tgt = {1: (0.0, 0.0, 0.0), 2: (-0.5, 0.0, 0.0), 3: (-1.0 / g, -1.0 / g, 0.0),
                   4: (-1.0 / g, -1.0 / g, -1.0 / g)}[n]
            for q in range(3):
                r = np.zeros(3 * ns)
                r[q * ns:(q + 1) * ns] = gp
                rows.append(r)
                rhs.append(tgt[q])
    # (1-theta)[1 + theta (a + b theta + c theta^2)] = (1-theta)^4: a=-3, b=3, c=-1
    for q, v in enumerate((-3.0, 3.0, -1.0)):
        r = np.zeros(3 * ns)
        r[q * ns:(q + 1) * ns] = ut[:ns]
        rows.append(r)
        rhs.append(v)
    M = np.array(rows)
    y = np.array(rhs)
    assert np.linalg.matrix_rank(M, 1e-9) == 3 * ns
    x = np.linalg.lstsq(M, y, rcond=None)[0]
    resid = np.abs(M @ x - y).max()
    assert resid < 1e-10, resid
    return x[:ns], x[ns:2 * ns], x[2 * ns:], resid


def fmt(v):
    return repr(float(v))


def main():
    tb = parse_tableaus()
    B, r7 = derive_vern7(tb)
    lines = [
        "// dense_coeffs.h -- GENERATED by derive_dense_output.py; do not edit.",
        "#pragma once",
        "namespace gbde {",
        "namespace tab {",
        "// Vern7 5th-order continuous extension: b_j(theta) = sum_k B_j_k theta^k,",
        "// j = 1..10 the Vern7 stages, j = 11 the stage f(t+h, y1).",
        "// max residual of the defining equations: %.3e" % r7,
        "namespace vern7d {",
    ]
    for j in range(B.shape[0]):
        for k in range(B.shape[1]):
            lines.append("constexpr double B%d_%d = %s;" % (j + 1, k + 1, fmt(B[j, k])))
    lines.append("}  // namespace vern7d")
    AA, W1, W2, C7 = derive_vern7_lazy(tb, B)
    T7 = trees(7)
    r7l = max(abs(((th ** np.arange(1, 8)) @ C7) @ rk_phi(t, AA) - th ** rho(t) / tree_gamma(t))
              for th in (0.1, 0.5, 0.9) for n in range(1, 8) for t in T7[n])
    assert r7l < 1e-11, r7l
    lines += [
        "// Vern7 7th-order continuous extension by bootstrapping (derive_vern7_lazy):",
        "// stages K12..K14 at y0 + h sum_j L1_i_j K_j (i = 1..3, j = 1..11, the 5th-order",
        "// extension's weights at theta = %s), K15..K18 at y0 + h sum_j L2_i_j K_j"
        % ", ".join("%g" % t for t in V7_THETA1),
        "// (i = 1..4, j = 1..14, theta = %s); output"
        % ", ".join("%g" % t for t in V7_THETA2),
        "// u(theta) = y0 + h sum_j (sum_m D_j_m theta^m) K_j, j = 1..18, m = 1..7.",
        "// max residual of the order-7 conditions: %.3e" % r7l,
        "namespace vern7l {",
    ]
    for i in range(3):
        lines.append("constexpr double TH1_%d = %s;" % (i + 1, fmt(V7_THETA1[i])))
    for i in range(4):
        lines.append("constexpr double TH2_%d = %s;" % (i + 1, fmt(V7_THETA2[i])))
    for i in range(3):
        for j in range(11):
            lines.append("constexpr double L1_%d_%d = %s;" % (i + 1, j + 1, fmt(W1[i, j])))
    for i in range(4):
        for j in range(14):
            lines.append("constexpr double L2_%d_%d = %s;" % (i + 1, j + 1, fmt(W2[i, j])))
    for j in range(18):
        for m in range(7):
            lines.append("constexpr double D%d_%d = %s;" % (j + 1, m + 1, fmt(C7[m, j])))
    lines.append("}  // namespace vern7l")
    for name in ("rodas5", "rodas5p"):
        h2, h3, h4, rr = derive_rodas(tb, name)
        lines.append("// %s 4th-order continuous extension (transformed stages u_1..u_7),"
                     " max residual %.3e" % (name, rr))
        lines.append("namespace %sd {" % name)
        for nm, h in (("H2", h2), ("H3", h3), ("H4", h4)):
            for j in range(7):
                lines.append("constexpr double %s_%d = %s;" % (nm, j + 1, fmt(h[j])))
        lines.append("}  // namespace %sd" % name)
    lines += ["}  // namespace tab", "}  // namespace gbde", ""]
    with open(os.path.join(HERE, "dense_coeffs.h"), "w") as f:
        f.write("\n".join(lines))


if __name__ == "__main__":
    main()
