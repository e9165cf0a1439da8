"""ctypes binding of libgbde.so (include/gbde.h).

This module is the Python-side twin of the `ccall` wrapper a Julia
`EnsembleGB300 <: SciMLBase.EnsembleAlgorithm` would use: the struct layouts
mirror gbde.h field for field.  Nothing here computes on the CPU: if the
library is missing or no GPU is present, calls fail loudly.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbde.so")

# ---- constants (gbde.h)
GBDE_OK = 0
GBDE_ERR_INVALID = -1
GBDE_ERR_CUDA = -2
GBDE_ERR_UNSUPPORTED = -3
GBDE_ERR_TIMEOUT = -4
GBDE_ERR_NOMEM = -5
GBDE_ERR_STATE = -6

RET_DEFAULT, RET_SUCCESS, RET_MAXITERS, RET_DTLESSTHANMIN, RET_UNSTABLE = 0, 1, 2, 3, 4
RET_INITIALFAILURE, RET_TIMEOUT, RET_TERMINATED = 5, 6, 7

MODEL_LINEAR, MODEL_LORENZ, MODEL_ROBERTSON, MODEL_VDP_RING8, MODEL_LOTKA_VOLTERRA = 1, 2, 3, 4, 5
MODEL_USER_BASE, USER_MAX_STATE, USER_MAX_PARAM = 1000, 8, 32

ALG_TSIT5, ALG_VERN7, ALG_ROSENBROCK23, ALG_RODAS5, ALG_RODAS5P = 1, 2, 3, 4, 5
ALG_EM, ALG_SOSRI, ALG_AUTO, ALG_SRIW1 = 6, 7, 8, 9
ALG_AUTOTSIT5_ROSENBROCK23, ALG_AUTOTSIT5_RODAS5 = 10, 11

PREC_FP64, PREC_MIXED, PREC_F32X2 = 0, 1, 2
BATCH_PLAIN, BATCH_PERSISTENT = 0, 1
SAVE_GRID, SAVE_PER_TRAJ = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1
F64, F32 = 0, 1


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


class MlpTrainOpts(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float),
                ("weight_decay", C.c_float), ("seed", C.c_uint64)]


MLP_IN, MLP_OUT, MLP_PARAMS, MLP_NET_FLOATS = 8, 3, 9091, 9111
LEARN_START, LEARN_ORDER, LEARN_STIFF = 1, 2, 4  # gbde_opts.learned flags


class TuneEntry(C.Structure):
    _fields_ = [("batching", C.c_int32), ("block_size", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("chunk", C.c_int32), ("threads_per_traj", C.c_int32), ("device_ms", C.c_float)]


SUMMARY_MAX_Q = 8


class Summary(C.Structure):
    _fields_ = [("n_quantiles", C.c_int32), ("quantiles", C.c_double * SUMMARY_MAX_Q),
                ("mean", C.c_void_p), ("var", C.c_void_p), ("qvals", C.c_void_p)]


CB_CONTINUOUS, CB_DISCRETE, CB_VECTOR = 1, 2, 3
SAVE_BEFORE, SAVE_AFTER = 1, 2
MAX_CB_CONDITIONS = 64


class Callback(C.Structure):
    _fields_ = [("kind", C.c_int32), ("condition", C.c_char_p), ("affect", C.c_char_p),
                ("terminate", C.c_int32), ("save_positions", C.c_int32)]


class UserModel(C.Structure):
    _fields_ = [("name", C.c_char_p), ("n_state", C.c_int32), ("n_param", C.c_int32),
                ("f_body", C.c_char_p), ("jac_body", C.c_char_p)]


# Every function gbde.h declares, with its ctypes signature.
SIGNATURES = {
    "gbde_version": (C.c_int, []),
    "gbde_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gbde_ctx_destroy": (C.c_int, [C.c_void_p]),
    "gbde_last_error": (C.c_char_p, [C.c_void_p]),
    "gbde_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "gbde_opts_default": (C.c_int, [C.c_int32, C.POINTER(Opts)]),
    "gbde_ensemble_solve": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(Opts),
                                      C.POINTER(Outputs)]),
    "gbde_model_info": (C.c_int, [C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "gbde_philox_normals": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64,
                                      C.c_void_p]),
    "gbde_philox4x32_10": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "gbde_measure_fma_peak": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double)]),
    "gbde_ensemble_solve_noalloc": (C.c_int, [C.POINTER(Problem), C.POINTER(Opts),
                                              C.POINTER(Outputs), C.c_void_p]),
    "gbde_check_rcp64": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double)]),
    "gbde_mlp_init": (C.c_int, [C.c_uint64, C.c_void_p]),
    "gbde_mlp_features": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.c_void_p]),
    "gbde_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                 C.POINTER(MlpTrainOpts), C.c_void_p, C.c_void_p]),
    "gbde_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "gbde_mlp_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                C.c_void_p, C.POINTER(C.c_float)]),
    "gbde_mlp_load": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "gbde_graph_create": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(Opts),
                                    C.POINTER(Outputs), C.POINTER(C.c_void_p)]),
    "gbde_graph_launch": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "gbde_graph_destroy": (C.c_int, [C.c_void_p]),
    "gbde_ensemble_summary": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int64,
                                        C.c_int32, C.c_int32, C.POINTER(Summary)]),
    "gbde_model_register": (C.c_int, [C.POINTER(UserModel), C.POINTER(C.c_int32)]),
    "gbde_sde_model_register": (C.c_int, [C.POINTER(UserModel), C.c_char_p, C.POINTER(C.c_int32)]),
    "gbde_model_compile": (C.c_int, [C.c_int32, C.c_int32, C.c_int32]),
    "gbde_callback_register": (C.c_int, [C.POINTER(Callback), C.POINTER(C.c_int32)]),
    "gbde_vector_callback_register": (C.c_int, [C.POINTER(Callback), C.c_int32,
                                                C.POINTER(C.c_int32)]),
    "gbde_callback_set_register": (C.c_int, [C.POINTER(C.c_int32), C.c_int32,
                                             C.POINTER(C.c_int32)]),
    "gbde_callback_compile": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "gbde_autotune": (C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(Opts),
                                C.POINTER(Outputs), C.c_int32, C.POINTER(Opts),
                                C.POINTER(TuneEntry), C.c_int32, C.POINTER(C.c_int32)]),
}

_lib = None


class GBDEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gbde error %d: %s" % (code, msg))
        self.code = code


def lib():
    """Load libgbde.so (building it first if the toolchain is present)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code, ctx=None):
    if code != GBDE_OK:
        msg = lib().gbde_last_error(ctx)
        raise GBDEError(code, msg.decode() if msg else "")


def model_info(model):
    ns, np_ = C.c_int32(), C.c_int32()
    check(lib().gbde_model_info(model, C.byref(ns), C.byref(np_)))
    return ns.value, np_.value


def opts_default(alg):
    o = Opts()
    check(lib().gbde_opts_default(alg, C.byref(o)))
    return o


class Context:
    """A libgbde context bound to one CUDA device."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().gbde_ctx_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            lib().gbde_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        check(lib().gbde_ctx_set_stream(self.handle, C.c_void_p(stream_ptr)), self.handle)

    def fma_peak(self, kind):
        v = C.c_double()
        check(lib().gbde_measure_fma_peak(self.handle, kind, C.byref(v)), self.handle)
        return v.value

    def check_rcp64(self, n):
        v = C.c_double()
        check(lib().gbde_check_rcp64(self.handle, int(n), C.byref(v)), self.handle)
        return v.value

    def solve(self, prob, opts, outs):
        check(lib().gbde_ensemble_solve(self.handle, C.byref(prob), C.byref(opts),
                                        C.byref(outs)), self.handle)
        return outs


_contexts = {}


def context(device=0):
    if device not in _contexts:
        _contexts[device] = Context(device)
    return _contexts[device]


def ptr(a):
    """Data pointer of a numpy array or a torch tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def philox_normals(seed, traj, counter, n):
    out = np.empty(n, np.float64)
    check(lib().gbde_philox_normals(seed, traj, counter, n, out.ctypes.data))
    return out


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.empty(4, np.uint32)
    check(lib().gbde_philox4x32_10(c.ctypes.data, k.ctypes.data, o.ctypes.data))
    return o
