"""Repeated and tuned ensemble solves: CUDA-graph replay and the autotuner.

graph(...)     captures one device-memory solve (gbde_graph_create) and
               replays it with .launch(); refill the input tensors in place
               between launches.
autotune(...)  times the launch configurations of gbde_autotune on the
               caller's problem and returns the fastest options; with
               `cache` (a JSON file path) the choice is stored per
               (device, model, algorithm, precision, trajectory-count bucket)
               and reused without re-timing.
"""
import ctypes as C
import json
import math
import os

import numpy as np

from . import _capi as capi

TUNED_FIELDS = ("batching", "block_size", "ctas_per_sm", "chunk", "threads_per_traj")


def _problem(model, arrs, save_kind):
    prob = capi.Problem()
    prob.model, prob.n_state, prob.n_param = model.id, model.n_state, model.n_param
    prob.mem = capi.MEM_DEVICE
    prob.n_traj = int(arrs[1].shape[0])
    prob.p, prob.u0, prob.t0, prob.tf, prob.saveat = [a.data_ptr() for a in arrs]
    prob.save_kind = save_kind
    prob.n_save = int(arrs[4].shape[-1])
    return prob


def _outputs(model, N, n_save, u_dtype, dev):
    import torch
    res = {"u": torch.empty((N, n_save, model.n_state),
                            dtype=torch.float32 if u_dtype == "f32" else torch.float64, device=dev),
           "retcode": torch.empty(N, dtype=torch.int32, device=dev),
           "naccept": torch.empty(N, dtype=torch.int32, device=dev),
           "nreject": torch.empty(N, dtype=torch.int32, device=dev)}
    outs = capi.Outputs()
    outs.u_dtype = capi.F32 if u_dtype == "f32" else capi.F64
    for k in ("u", "retcode", "naccept", "nreject"):
        setattr(outs, k, res[k].data_ptr())
    return res, outs


class Graph:
    """A captured solve; inputs and outputs are the tensors given at capture."""

    def __init__(self, model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype="f64", device=0):
        import torch
        self.ctx = capi.context(device)
        self.inputs = (p, u0, t0, tf, saveat)
        self._prob = _problem(model, self.inputs, save_kind)
        self.out, self._outs = _outputs(model, int(u0.shape[0]), int(saveat.shape[-1]), u_dtype,
                                        u0.device)
        self._opts = opts
        self.handle = C.c_void_p()
        self.ctx.set_stream(torch.cuda.current_stream(u0.device).cuda_stream)
        capi.check(capi.lib().gbde_graph_create(self.ctx.handle, C.byref(self._prob),
                                                C.byref(opts), C.byref(self._outs),
                                                C.byref(self.handle)), self.ctx.handle)

    def launch(self):
        ms = C.c_float()
        capi.check(capi.lib().gbde_graph_launch(self.handle, C.byref(ms)), self.ctx.handle)
        return ms.value

    def close(self):
        if self.handle:
            capi.lib().gbde_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cache_key(device_name, model, opts, n_traj):
    """(device, model, algorithm, precision, power-of-two bucket of N)."""
    bucket = 1 << max(0, int(math.ceil(math.log2(max(1, n_traj)))))
    return "%s|%s|alg%d|prec%d|N%d" % (device_name, model.name, opts.alg, opts.precision, bucket)


def apply_tuned(opts, entry):
    for k in TUNED_FIELDS:
        setattr(opts, k, int(entry[k]))
    return opts


def load_cache(path):
    if path and os.path.exists(path):
        with open(path) as fh:
            return json.load(fh)
    return {}


def save_cache(path, cache):
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(cache, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype="f64", reps=2, cache=None,
             device=0):
    """Fastest launch options for this problem (device tensors).  Returns
    (options, timing table as a list of dicts, from_cache)."""
    import torch
    name = torch.cuda.get_device_name(u0.device)
    key = cache_key(name, model, opts, int(u0.shape[0]))
    table = load_cache(cache)
    if key in table:
        best = capi.Opts()
        C.memmove(C.byref(best), C.byref(opts), C.sizeof(capi.Opts))
        return apply_tuned(best, table[key]), [], True
    ctx = capi.context(device)
    ctx.set_stream(torch.cuda.current_stream(u0.device).cuda_stream)
    prob = _problem(model, (p, u0, t0, tf, saveat), save_kind)
    _, outs = _outputs(model, int(u0.shape[0]), int(saveat.shape[-1]), u_dtype, u0.device)
    best = capi.Opts()
    entries = (capi.TuneEntry * 64)()
    n = C.c_int32()
    capi.check(capi.lib().gbde_autotune(ctx.handle, C.byref(prob), C.byref(opts), C.byref(outs),
                                        int(reps), C.byref(best), entries, 64, C.byref(n)),
               ctx.handle)
    rows = [{k: getattr(entries[i], k) for k in TUNED_FIELDS + ("device_ms",)}
            for i in range(n.value)]
    if cache:
        table[key] = {k: getattr(best, k) for k in TUNED_FIELDS}
        save_cache(cache, table)
    return best, rows, False
