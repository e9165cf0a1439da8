"""Python wrapper of the CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module: it is the checker, never the product path.  It calls
liboracle_gbde.so (gbde_oracle.cpp) with the same C structs as the product's
gbde_ensemble_solve, so oracle and GPU consume identical inputs.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None


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
        _lib = L
    return _lib


def hardware_threads():
    return lib().oracle_hardware_threads()


def solve(capi, model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype="f64", nthreads=1,
          noise_f32=False):
    """FP64 CPU solve of the ensemble; `capi` is the product's _capi module
    (for the struct layouts only).  Returns a dict of numpy arrays."""
    N = int(u0.shape[0])
    arrs = [np.ascontiguousarray(a, np.float64) for a in (p, u0, t0, tf, saveat)]
    n_save = int(arrs[4].shape[-1]) if arrs[4].size else 0
    prob = capi.Problem()
    prob.model = model.id
    prob.n_state, prob.n_param = model.n_state, model.n_param
    prob.mem = capi.MEM_HOST
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
    }
    outs = capi.Outputs()
    outs.u = res["u"].ctypes.data
    outs.u_dtype = capi.F32 if u_dtype == "f32" else capi.F64
    for k in ("retcode", "naccept", "nreject", "nf", "t_end"):
        setattr(outs, k, res[k].ctypes.data)
    rc = lib().oracle_ensemble_solve(C.addressof(prob), C.addressof(opts), C.addressof(outs),
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


def weighted_error(u, ref, abstol, reltol):
    """max over trajectories, save points and components of
    |u - u*| / (abstol + reltol |u*|)  (the pass bar is <= 10)."""
    u = np.asarray(u, np.float64)
    ref = np.asarray(ref, np.float64)
    e = np.abs(u - ref) / (abstol + reltol * np.abs(ref))
    return float(np.nanmax(e)) if e.size else 0.0
