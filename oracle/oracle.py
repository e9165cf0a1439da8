"""Python wrapper of the CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module: it is the checker, never the product path.  It calls
liboracle_gbde.so (gbde_oracle.cpp) with the C structs of include/gbde.h, so
oracle and GPU consume identical inputs.  The struct layouts, constants and
option defaults below are this module's own restatement of gbde.h; it never
loads the product library (tests/test_api.py checks that the two agree).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None

# ---- gbde.h constants the oracle needs
MODEL_LINEAR, MODEL_LORENZ, MODEL_ROBERTSON, MODEL_VDP_RING8, MODEL_LOTKA_VOLTERRA = 1, 2, 3, 4, 5
ALG_TSIT5, ALG_VERN7, ALG_ROSENBROCK23, ALG_RODAS5, ALG_RODAS5P = 1, 2, 3, 4, 5
ALG_EM, ALG_SOSRI, ALG_AUTO, ALG_SRIW1 = 6, 7, 8, 9
ALG_AUTOTSIT5_ROSENBROCK23, ALG_AUTOTSIT5_RODAS5 = 10, 11
SAVE_GRID, SAVE_PER_TRAJ = 0, 1
MEM_HOST = 0
F64, F32 = 0, 1
RET_SUCCESS = 1


class Problem(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("n_state", C.c_int32), ("n_param", C.c_int32),
        ("mem", C.c_int32), ("n_traj", C.c_int64),
        ("p", C.c_void_p), ("u0", C.c_void_p), ("t0", C.c_void_p), ("tf", C.c_void_p),
        ("save_kind", C.c_int32), ("n_save", C.c_int32), ("saveat", C.c_void_p),
    ]


class Opts(C.Structure):
    _fields_ = [
        ("alg", C.c_int32), ("precision", C.c_int32), ("batching", C.c_int32),
        ("adaptive", C.c_int32),
        ("reltol", C.c_double), ("abstol", C.c_double), ("dt", C.c_double),
        ("dtmin", C.c_double), ("dtmax", C.c_double), ("maxiters", C.c_int64),
        ("qmin", C.c_double), ("qmax", C.c_double), ("gamma", C.c_double),
        ("beta1", C.c_double), ("beta2", C.c_double), ("qsteady_min", C.c_double),
        ("qsteady_max", C.c_double), ("qoldinit", C.c_double),
        ("seed", C.c_uint64), ("learned", C.c_int32), ("block_size", C.c_int32),
        ("chunk", C.c_int32), ("ctas_per_sm", C.c_int32),
        ("stiff_threshold", C.c_double), ("timeout_s", C.c_double),
        ("threads_per_traj", C.c_int32), ("callback", C.c_int32),
    ]


class Outputs(C.Structure):
    _fields_ = [
        ("u", C.c_void_p), ("u_dtype", C.c_int32), ("retcode", C.c_void_p),
        ("naccept", C.c_void_p), ("nreject", C.c_void_p), ("nf", C.c_void_p),
        ("t_end", C.c_void_p), ("method", C.c_void_p),
        ("device_ms", C.c_float), ("total_ms", C.c_float), ("dt_first", C.c_void_p),
        ("reduce", C.c_void_p), ("ev_t", C.c_void_p), ("ev_u", C.c_void_p),
        ("ev_count", C.c_void_p), ("ev_capacity", C.c_int32),
    ]


# (state size, parameter count) of the built-in models
MODEL_SIZES = {MODEL_LINEAR: (1, 1), MODEL_LORENZ: (3, 3), MODEL_ROBERTSON: (3, 3),
               MODEL_VDP_RING8: (16, 2), MODEL_LOTKA_VOLTERRA: (2, 5)}


class ModelRef:
    """A built-in model by id (the oracle's stand-in for the package's Model)."""

    def __init__(self, model_id):
        self.id = model_id
        self.n_state, self.n_param = MODEL_SIZES[model_id]


def opts_default(alg):
    """The solver defaults of gbde_opts_default (PI-controller exponents per
    method, Hairer-Norsett-Wanner I, Sec. II.4), restated."""
    o = Opts()
    o.alg, o.adaptive = alg, 1
    o.reltol, o.abstol, o.maxiters = 1e-3, 1e-6, 100000
    o.qmin, o.qmax, o.gamma = 0.2, 10.0, 0.9
    o.qsteady_min, o.qsteady_max, o.qoldinit = 1.0, 1.0, 1e-4
    if alg in (ALG_TSIT5, ALG_AUTO, ALG_AUTOTSIT5_ROSENBROCK23, ALG_AUTOTSIT5_RODAS5):
        o.beta2 = 0.04
        o.beta1 = 0.2 - 0.75 * 0.04
        if alg == ALG_AUTO:
            o.stiff_threshold = 30.0
    elif alg == ALG_VERN7:
        o.beta2, o.beta1 = 2.0 / (5.0 * 7.0), 7.0 / (10.0 * 7.0)
    elif alg == ALG_ROSENBROCK23:
        o.beta1 = 1.0 / 3.0
    elif alg in (ALG_RODAS5, ALG_RODAS5P):
        o.beta1 = 1.0 / 5.0
    elif alg == ALG_EM:
        o.adaptive, o.beta1 = 0, 0.5
    elif alg in (ALG_SOSRI, ALG_SRIW1):
        o.beta1 = 0.5
        o.reltol = o.abstol = 1e-2
    else:
        raise ValueError("unknown algorithm id %d" % alg)
    return o


def _as_opts(opts):
    if isinstance(opts, Opts):
        return opts
    o = Opts()
    for name, _ in Opts._fields_:
        setattr(o, name, getattr(opts, name))
    return o


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.oracle_ensemble_solve.restype = C.c_int
        L.oracle_ensemble_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.oracle_philox4x32_10.restype = None
        L.oracle_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_normals.restype = None
        L.oracle_normals.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64, C.c_int,
                                     C.c_void_p]
        L.oracle_hardware_threads.restype = C.c_int
        L.oracle_lu_solve.restype = C.c_int
        L.oracle_lu_solve.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_set_controller.restype = None
        L.oracle_set_controller.argtypes = [C.c_int]
        L.oracle_ctl_selfcheck.restype = C.c_int64
        L.oracle_ctl_selfcheck.argtypes = []
        L.oracle_d2f_rn.restype = None
        L.oracle_d2f_rn.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _lib = L
    return _lib


def hardware_threads():
    return lib().oracle_hardware_threads()


def set_controller(mode):
    """0: the kernels' FP32-series step-size factor (identical steps; the
    default); 1: the FP64 pow() form of the same PI controller."""
    lib().oracle_set_controller(int(mode))


def ctl_selfcheck():
    """Mismatches of the controller's exact helpers against frexpf, (float),
    rintf and ldexpf (0 expected)."""
    return int(lib().oracle_ctl_selfcheck())


def d2f_rn(x):
    """The controller's integer-pipe double -> float rounding (d2f_rn_bits)."""
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty(x.shape, np.float32)
    lib().oracle_d2f_rn(x.ctypes.data, out.ctypes.data, x.size)
    return out


def lu_solve(A, b):
    """x = A^{-1} b with the oracle's partial-pivot LU (its Rosenbrock solve)."""
    A = np.ascontiguousarray(A, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.empty_like(b)
    if lib().oracle_lu_solve(len(b), A.ctypes.data, b.ctypes.data, x.ctypes.data) != 0:
        raise ValueError("lu_solve: n must be 1..16")
    return x


def solve(capi, model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype="f64", nthreads=1,
          noise_f32=False):
    """FP64 CPU solve of the ensemble.  `capi` is accepted for call-site
    compatibility and not used; `model` needs .id, .n_state and .n_param;
    `opts` is an Opts or any object with gbde_opts' fields.  Returns a dict
    of numpy arrays."""
    N = int(u0.shape[0])
    arrs = [np.ascontiguousarray(a, np.float64) for a in (p, u0, t0, tf, saveat)]
    n_save = int(arrs[4].shape[-1]) if arrs[4].size else 0
    prob = Problem()
    prob.model = model.id
    prob.n_state, prob.n_param = model.n_state, model.n_param
    prob.mem = MEM_HOST
    prob.n_traj = N
    prob.p, prob.u0, prob.t0, prob.tf, prob.saveat = [a.ctypes.data for a in arrs]
    prob.save_kind = save_kind
    prob.n_save = n_save
    res = {
        "u": np.empty((N, n_save, model.n_state), np.float32 if u_dtype == "f32" else np.float64),
        "retcode": np.empty(N, np.int32),
        "naccept": np.empty(N, np.int32),
        "nreject": np.empty(N, np.int32),
        "nf": np.empty(N, np.int32),
        "t_end": np.empty(N, np.float64),
        "method": np.empty(N, np.int32),
    }
    outs = Outputs()
    outs.u = res["u"].ctypes.data
    outs.u_dtype = F32 if u_dtype == "f32" else F64
    for k in ("retcode", "naccept", "nreject", "nf", "t_end", "method"):
        setattr(outs, k, res[k].ctypes.data)
    o = _as_opts(opts)
    rc = lib().oracle_ensemble_solve(C.addressof(prob), C.addressof(o), C.addressof(outs),
                                     int(nthreads), int(bool(noise_f32)))
    if rc != 0:
        raise RuntimeError("oracle_ensemble_solve failed with %d" % rc)
    return res


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.empty(4, np.uint32)
    lib().oracle_philox4x32_10(c.ctypes.data, k.ctypes.data, o.ctypes.data)
    return o


def normals(seed, traj, counter, n, f32=False):
    out = np.empty(n, np.float64)
    lib().oracle_normals(seed, traj, counter, n, int(bool(f32)), out.ctypes.data)
    return out


def weighted_errors(u, ref, abstol, reltol):
    """Elementwise |u - u*| / (abstol + reltol |u*|).  A NaN on exactly one
    side counts as an infinite error; NaN on both sides (save slots that
    neither solve reached) as zero."""
    u = np.asarray(u, np.float64)
    ref = np.asarray(ref, np.float64)
    with np.errstate(invalid="ignore", over="ignore"):
        e = np.abs(u - ref) / (abstol + reltol * np.abs(ref))
    nu, nr = np.isnan(u), np.isnan(ref)
    e = np.where(nu & nr, 0.0, e)
    e = np.where(nu ^ nr, np.inf, e)
    # infinities on both sides with the same sign agree; any other NaN left
    # (inf - inf of opposite signs, inf / inf) is a disagreement
    same_inf = np.isinf(u) & np.isinf(ref) & (np.sign(u) == np.sign(ref))
    e = np.where(same_inf, 0.0, e)
    return np.where(np.isnan(e), np.inf, e)


def weighted_error(u, ref, abstol, reltol):
    """max over trajectories, save points and components of
    |u - u*| / (abstol + reltol |u*|)  (the pass bar is <= 10); a NaN on one
    side only gives inf."""
    e = weighted_errors(u, ref, abstol, reltol)
    return float(e.max()) if e.size else 0.0
