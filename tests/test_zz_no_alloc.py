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


def _noalloc(capi, model, opts, dev, n_save, stream, save_kind=None):
    import torch
    p, u0, t0, tf, saveat = dev
    N = u0.shape[0]
    prob = capi.Problem()
    prob.model, prob.n_state, prob.n_param = model.id, model.n_state, model.n_param
    prob.mem = capi.MEM_DEVICE
    prob.n_traj = N
    prob.p, prob.u0, prob.t0, prob.tf, prob.saveat = [a.data_ptr() for a in dev]
    prob.save_kind = capi.SAVE_PER_TRAJ if save_kind is None else save_kind
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


def _ring_inputs(N, seed):
    rng = np.random.default_rng(seed)
    p = np.c_[10 ** rng.uniform(-1, 3, N), np.full(N, 0.05)]
    return p, rng.uniform(-2, 2, (N, 16)), np.zeros(N), np.full(N, 20.0), np.arange(21.0)


def _lv_inputs(N, seed):
    rng = np.random.default_rng(seed)
    p = np.c_[np.array([1.5, 1.0, 3.0, 1.0]) * rng.uniform(0.8, 1.2, (N, 4)), np.full(N, 0.1)]
    return p, np.ones((N, 2)), np.zeros(N), np.full(N, 2.0), np.linspace(0.0, 2.0, 9)


def _robertson_inputs(N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    return p, np.tile([1.0, 0.0, 0.0], (N, 1)), np.zeros(N), np.full(N, 1e3), np.logspace(-3, 3, 7)


@pytest.mark.parametrize("case", ["em", "ring_rodas5", "autotsit5_rosenbrock23"])
def test_noalloc_matches_ensemble_solve_other_kernels(de, case):
    """The SDE kernel (Euler-Maruyama on the Lotka-Volterra ensemble), the
    ring's team kernel (Rodas5 on the 16-state ring) and the AutoTsit5
    composite (Robertson: Tsit5, then Rosenbrock23) through the
    no-allocation entry point: bitwise the outputs of gbde_ensemble_solve, on
    two calls in a row."""
    import torch
    capi = de._capi
    if case == "em":
        model, host = de.models.lotka_volterra, _lv_inputs(2000, 3)
        opts = capi.opts_default(capi.ALG_EM)
        opts.dt, opts.seed = 1e-3, 17
    elif case == "autotsit5_rosenbrock23":
        model, host = de.models.robertson, _robertson_inputs(1000, 5)
        opts = capi.opts_default(capi.ALG_AUTOTSIT5_ROSENBROCK23)
        opts.reltol, opts.abstol = 1e-6, 1e-10
    else:
        model, host = de.models.vdp_ring8, _ring_inputs(512, 4)
        opts = capi.opts_default(capi.ALG_RODAS5)
        opts.reltol = opts.abstol = 1e-5
        opts.maxiters = 10 ** 6
        opts.batching = capi.BATCH_PERSISTENT
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in host]
    ref = de.solve_arrays(model, opts, *dev, capi.SAVE_GRID)
    torch.cuda.synchronize()
    ref = {k: ref[k].cpu().numpy() for k in ("u", "retcode", "naccept")}
    assert np.all(ref["retcode"] == capi.RET_SUCCESS)
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        got = _noalloc(capi, model, opts, dev, len(host[4]), stream, save_kind=capi.SAVE_GRID)
        assert np.array_equal(got["retcode"], ref["retcode"])
        assert np.array_equal(got["naccept"], ref["naccept"])
        assert np.array_equal(got["u"], ref["u"])


def test_noalloc_deadline_status(de):
    """A device deadline that expires mid-solve is reported through the status
    word in the static array (GBDE_ERR_TIMEOUT, no fault); the next call
    clears that word and succeeds."""
    import torch
    capi = de._capi
    model = de.models.robertson
    host = _inputs(20000, 5)
    dev = [torch.from_numpy(a).cuda() for a in host]
    opts = capi.opts_default(capi.ALG_RODAS5)
    opts.reltol, opts.abstol = 1e-10, 1e-14
    opts.timeout_s = 1e-6
    stream = torch.cuda.current_stream().cuda_stream
    with pytest.raises(capi.GBDEError) as e:
        _noalloc(capi, model, opts, dev, host[4].shape[1], stream)
    assert e.value.code == capi.GBDE_ERR_TIMEOUT
    opts.timeout_s = 0.0
    opts.reltol, opts.abstol = 1e-6, 1e-10
    small = [a[:100].contiguous() for a in dev]
    got = _noalloc(capi, model, opts, small, host[4].shape[1], stream)
    assert np.all(got["retcode"] == capi.RET_SUCCESS)


def test_noalloc_rejects_user_models(de):
    """A user model's kernels are compiled and loaded by gbde_ensemble_solve;
    the no-allocation entry point says so instead of failing in the launch."""
    import torch
    capi = de._capi
    m = de.ODEFunction("du[0] = -p[0] * u[0];", 1, 1, name="decay_noalloc")
    dev = [torch.ones((4, 1), dtype=torch.float64, device="cuda"),
           torch.ones((4, 1), dtype=torch.float64, device="cuda"),
           torch.zeros(4, dtype=torch.float64, device="cuda"),
           torch.ones(4, dtype=torch.float64, device="cuda"),
           torch.ones(1, dtype=torch.float64, device="cuda")]
    opts = capi.opts_default(capi.ALG_TSIT5)
    with pytest.raises(capi.GBDEError) as e:
        _noalloc(capi, m, opts, dev, 1, torch.cuda.current_stream().cuda_stream,
                 save_kind=capi.SAVE_GRID)
    assert e.value.code == capi.GBDE_ERR_UNSUPPORTED
    assert "user model" in str(e.value)
