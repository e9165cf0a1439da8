"""Generate the golden truth fixtures in this folder (ode_truth.json).

The reference's own tests pin no numbers (test/core.jl checks return codes,
lengths and u[1] == u0 only), so these fixtures are independent truths from
scipy's solve_ivp at tight tolerances: DOP853 for the non-stiff problems,
Radau for the stiff ones.  Cases follow the reference's pinned problems
(test/core.jl:10 u' = 1.01u, :22-27 Lorenz, :39-45 Robertson to t = 1e5) and
the ensemble configurations' systems (ring of 8 Van der Pol oscillators,
Lotka-Volterra drift).

Run:  python tests/golden/make_golden.py   (writes ode_truth.json)
"""
import json
import os

import numpy as np
from scipy.integrate import solve_ivp

HERE = os.path.dirname(os.path.abspath(__file__))


def lorenz(t, u, s, r, b):
    return [s * (u[1] - u[0]), u[0] * (r - u[2]) - u[1], u[0] * u[1] - b * u[2]]


def robertson(t, u, k1, k2, k3):
    return [-k1 * u[0] + k3 * u[1] * u[2], k1 * u[0] - k2 * u[1] ** 2 - k3 * u[1] * u[2],
            k2 * u[1] ** 2]


def vdp_ring8(t, u, mu, ka):
    du = np.empty(16)
    for i in range(8):
        x, v = u[2 * i], u[2 * i + 1]
        xl, xr = u[2 * ((i + 7) % 8)], u[2 * ((i + 1) % 8)]
        du[2 * i] = v
        du[2 * i + 1] = mu * (1 - x * x) * v - x + ka * (xl - 2 * x + xr)
    return du


def lv(t, u, a, b, g, d):
    return [a * u[0] - b * u[0] * u[1], d * u[0] * u[1] - g * u[1]]


def case(name, model, f, p, u0, t_save, method, rtol, atol):
    sol = solve_ivp(f, (0.0, float(t_save[-1])), u0, method=method, rtol=rtol, atol=atol,
                    t_eval=t_save, args=tuple(p))
    assert sol.success, name
    return {"name": name, "model": model, "p": list(map(float, p)), "u0": list(map(float, u0)),
            "t": list(map(float, t_save)), "u": sol.y.T.tolist(),
            "made_with": "scipy solve_ivp %s rtol=%g atol=%g" % (method, rtol, atol)}


def main():
    grid01 = [k / 10 for k in range(11)]
    rober_t = list(1e5 * 10 ** (-5 + 5 * np.arange(20) / 19))
    rng = np.random.default_rng(20261204)
    cases = [
        case("linear_1.01", "linear", lambda t, u, a: [a * u[0]], [1.01], [0.5], grid01,
             "DOP853", 1e-14, 1e-14),
        case("lorenz_core", "lorenz", lorenz, [10.0, 28.0, 8.0 / 3.0], [1.0, 0.0, 0.0], grid01,
             "DOP853", 1e-13, 1e-13),
        case("lorenz_scaled", "lorenz", lorenz, list(np.array([10.0, 28.0, 8.0 / 3.0]) * [1.07, 0.93, 1.02]),
             [1.0, 0.0, 0.0], grid01, "DOP853", 1e-13, 1e-13),
        case("robertson_core", "robertson", robertson, [0.04, 3e7, 1e4], [1.0, 0.0, 0.0], rober_t,
             "Radau", 1e-12, 1e-16),
        case("robertson_scaled", "robertson", robertson, [0.04 * 2.5, 3e7 * 0.3, 1e4 * 4.0],
             [1.0, 0.0, 0.0], rober_t, "Radau", 1e-12, 1e-16),
        case("vdp_ring8_mu1", "vdp_ring8", vdp_ring8, [1.0, 0.05], list(rng.uniform(-2, 2, 16)),
             [float(k) for k in range(21)], "DOP853", 1e-13, 1e-13),
        case("vdp_ring8_mu30", "vdp_ring8", vdp_ring8, [30.0, 0.05], list(rng.uniform(-2, 2, 16)),
             [float(k) for k in range(21)], "Radau", 1e-12, 1e-12),
        case("lotka_volterra_drift", "lotka_volterra", lv, [1.5, 1.0, 3.0, 1.0], [1.0, 1.0],
             [float(k) for k in range(11)], "DOP853", 1e-13, 1e-13),
    ]
    with open(os.path.join(HERE, "ode_truth.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": cases}, fh, indent=0)


if __name__ == "__main__":
    main()
