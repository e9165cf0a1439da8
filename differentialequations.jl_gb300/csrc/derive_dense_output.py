"""Derive the dense-output coefficients that are this library's own.

Writes ``dense_coeffs.h`` beside this file.  Run: ``python derive_dense_output.py``.

1. Vern7 5th-order continuous extension.  Stages 1..10 of Verner's 7(6) pair
   plus stage 11 = f(t + h, y1) (the next step's first stage, so it costs no
   extra evaluation on accepted steps).  Weights b_j(theta) = sum_k B[j,k]
   theta^k, k = 1..5, solve the continuous order conditions
       sum_j b_j(theta) Phi_j(t) = theta^rho(t) / gamma(t)   (rho(t) <= 5)
   as polynomial identities, plus b_j(1) = b_j (the interpolant ends at y1);
   minimum-norm solution.

2. Rodas5 / Rodas5P 4th-order continuous extension in transformed variables
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
