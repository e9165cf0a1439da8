"""gbde_ensemble_solve_noalloc: the solve for callers that must not allocate
device memory (their device memory belongs to another allocator, or they run
where cudaMalloc's implicit synchronisation is not allowed).  It keeps its
scratch (work-queue counter, status word) in a static device array inside
libgbde.so instead of a cudaMalloc'd buffer.

Called through the C ABI with device pointers; its outputs must equal those
of gbde_ensemble_solve on the same inputs on two calls in a row (the second
call finds the first call's counter in the shared array and must clear it).
This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
    t0 = np.zeros(N)
    tf = 10 ** rng.uniform(1, 5, N)
    saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
    return p, u0, t0, tf, np.ascontiguousarray(saveat)


def _noalloc(capi, model, opts, dev, n_save, stream):
    import torch
    p, u0, t0, tf, saveat = dev
    N = u0.shape[0]
    prob = capi.Problem()
    prob.model, prob.n_state, prob.n_param = model.id, model.n_state, model.n_param
    prob.mem = capi.MEM_DEVICE
    prob.n_traj = N
    prob.p, prob.u0, prob.t0, prob.tf, prob.saveat = [a.data_ptr() for a in dev]
    prob.save_kind = capi.SAVE_PER_TRAJ
    prob.n_save = n_save
    res = {"u": torch.full((N, n_save, model.n_state), -1.0, dtype=torch.float64, device=u0.device),
           "retcode": torch.zeros(N, dtype=torch.int32, device=u0.device),
           "naccept": torch.zeros(N, dtype=torch.int32, device=u0.device)}
    outs = capi.Outputs()
    outs.u_dtype = capi.F64
    outs.u = res["u"].data_ptr()
    outs.retcode = res["retcode"].data_ptr()
    outs.naccept = res["naccept"].data_ptr()
    rc = capi.lib().gbde_ensemble_solve_noalloc(C.byref(prob), C.byref(opts), C.byref(outs),
                                                C.c_void_p(stream))
    if rc != capi.GBDE_OK:
        raise capi.GBDEError(rc, capi.lib().gbde_last_error(None).decode())
    return {k: v.cpu().numpy() for k, v in res.items()}


@pytest.mark.parametrize("batching", ["persistent", "plain"])
def test_noalloc_matches_ensemble_solve(de, batching):
    import torch
    capi = de._capi
    model = de.models.robertson
    N = 3000
    host = _inputs(N, 20261204)
    dev = [torch.from_numpy(a).cuda() for a in host]
    opts = capi.opts_default(capi.ALG_RODAS5)
    opts.reltol, opts.abstol = 1e-6, 1e-10
    opts.batching = capi.BATCH_PERSISTENT if batching == "persistent" else capi.BATCH_PLAIN
    ref = de.solve_arrays(model, opts, *dev, capi.SAVE_PER_TRAJ)
    torch.cuda.synchronize()
    ref = {k: ref[k].cpu().numpy() for k in ("u", "retcode", "naccept")}
    assert np.all(ref["retcode"] == capi.RET_SUCCESS)
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):  # two calls in a row share the static scratch
        got = _noalloc(capi, model, opts, dev, host[4].shape[1], stream)
        # same kernel, same inputs: the tolerance of the FP64 batching tests (bitwise)
        assert np.array_equal(got["retcode"], ref["retcode"])
        assert np.array_equal(got["naccept"], ref["naccept"])
        assert np.array_equal(got["u"], ref["u"])


def test_noalloc_rejects_host_memory(de):
    capi = de._capi
    model = de.models.robertson
    p, u0, t0, tf, saveat = _inputs(4, 1)
    prob = capi.Problem()
    prob.model, prob.n_state, prob.n_param = model.id, model.n_state, model.n_param
    prob.mem = capi.MEM_HOST
    prob.n_traj = 4
    prob.p, prob.u0, prob.t0, prob.tf, prob.saveat = [a.ctypes.data for a in (p, u0, t0, tf, saveat)]
    prob.save_kind, prob.n_save = capi.SAVE_PER_TRAJ, saveat.shape[1]
    u = np.empty((4, saveat.shape[1], 3))
    rc_arr = np.empty(4, np.int32)
    outs = capi.Outputs()
    outs.u, outs.retcode, outs.u_dtype = u.ctypes.data, rc_arr.ctypes.data, capi.F64
    opts = capi.opts_default(capi.ALG_RODAS5)
    rc = capi.lib().gbde_ensemble_solve_noalloc(C.byref(prob), C.byref(opts), C.byref(outs), None)
    assert rc == capi.GBDE_ERR_INVALID
    assert b"device pointers" in capi.lib().gbde_last_error(None)
