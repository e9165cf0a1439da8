"""The learned step-size / stiffness / cost predictor, host side.

The network (a 4-layer BF16 MLP, include/gbde.h "learned") is trained on the
GPU by the library's own kernels (gbde_mlp_train) on step logs that the
solver itself writes:
  * features: gbde_mlp_features -- 8 numbers per trajectory from its
    parameters, initial state and time span;
  * target 0: log10 of the first accepted step of a plain solve (the
    `dt_first` step log);
  * target 1: stiff label -- 1 where the Rosenbrock method (Rodas5, FP64) is
    cheaper than the explicit one (Tsit5) on that trajectory, measured as
    steps x the measured device time per step of each kernel; NaN where
    the model has no stiff regime worth predicting;
  * target 2: log2 of the attempted steps (naccept + nreject step logs) of
    the method the predictor will order the queue for; NaN where not logged.
A solve with EnsembleGB300(learned=True) (opts.learned = LEARN_START) then
starts every trajectory at the predicted dt and, for GBDE_ALG_AUTO, uses the
predicted label instead of the threshold; learned="order" (LEARN_ORDER) has
the persistent queue hand out trajectories by predicted cost.  The error
controller still accepts or rejects every step, and the plain method is the
fallback.
"""
import ctypes as C

import numpy as np

from . import _capi as capi


def _np(a):
    """numpy view of a result array (host arrays pass through, CUDA tensors copy)."""
    return a if isinstance(a, np.ndarray) else a.cpu().numpy()


def _dev_problem(model, arrs, save_kind=None, n_save=0):
    prob = capi.Problem()
    prob.model, prob.n_state, prob.n_param = model.id, model.n_state, model.n_param
    prob.mem = capi.MEM_DEVICE
    prob.n_traj = int(arrs[1].shape[0])
    prob.p, prob.u0, prob.t0, prob.tf = [a.data_ptr() for a in arrs[:4]]
    prob.save_kind = capi.SAVE_GRID if save_kind is None else save_kind
    prob.n_save = n_save
    return prob


def features(model, p, u0, t0, tf, device=0):
    """features[N][8] (numpy float32) of every trajectory, computed on the GPU."""
    import torch
    dev = torch.device("cuda", device)
    arrs = [torch.as_tensor(np.ascontiguousarray(a, np.float64), device=dev)
            for a in (p, u0, t0, tf)]
    out = torch.empty((arrs[1].shape[0], capi.MLP_IN), dtype=torch.float32, device=dev)
    ctx = capi.context(device)
    capi.check(capi.lib().gbde_mlp_features(ctx.handle, C.byref(_dev_problem(model, arrs)),
                                            C.c_void_p(out.data_ptr())), None)
    return out.cpu().numpy()


def init(seed=0):
    net = np.empty(capi.MLP_NET_FLOATS, np.float32)
    capi.check(capi.lib().gbde_mlp_init(int(seed), net.ctypes.data))
    return net


def train(x, y, epochs=20, batch=4096, lr=2e-3, weight_decay=1e-4, seed=0, device=0, net=None):
    """Train on the GPU; returns (net, loss per epoch)."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    net = init(seed) if net is None else np.array(net, np.float32)
    o = capi.MlpTrainOpts(epochs=int(epochs), batch=int(batch), lr=float(lr),
                          weight_decay=float(weight_decay), seed=int(seed))
    hist = np.empty(int(epochs), np.float32)
    ctx = capi.context(device)
    capi.check(capi.lib().gbde_mlp_train(ctx.handle, x.ctypes.data, y.ctypes.data, x.shape[0],
                                         C.byref(o), net.ctypes.data, hist.ctypes.data),
               ctx.handle)
    return net, hist


def forward(net, x, device=0):
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty((x.shape[0], capi.MLP_OUT), np.float32)
    ctx = capi.context(device)
    capi.check(capi.lib().gbde_mlp_forward(ctx.handle, np.ascontiguousarray(net, np.float32)
                                           .ctypes.data, x.ctypes.data, x.shape[0],
                                           y.ctypes.data), ctx.handle)
    return y


def grad(net, x, y, device=0):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    g = np.empty(capi.MLP_PARAMS, np.float32)
    loss = C.c_float()
    ctx = capi.context(device)
    capi.check(capi.lib().gbde_mlp_grad(ctx.handle, np.ascontiguousarray(net, np.float32)
                                        .ctypes.data, x.ctypes.data, y.ctypes.data, x.shape[0],
                                        g.ctypes.data, C.byref(loss)), ctx.handle)
    return float(loss.value), g


def load(model, net, device=0):
    """Make `net` the predictor of learned=True solves of `model`."""
    ctx = capi.context(device)
    capi.check(capi.lib().gbde_mlp_load(ctx.handle, model.id,
                                        np.ascontiguousarray(net, np.float32).ctypes.data),
               ctx.handle)


def predict(net, x, device=0):
    """(predicted first dt, stiff label, predicted attempted steps) from
    features, as the solve uses them."""
    y = forward(net, x, device)
    off = capi.MLP_PARAMS + 2 * capi.MLP_IN  # y_mean, y_scale, c_mean, c_scale
    ym, ys, cm, cs = (float(v) for v in net[off:off + 4])
    return (10.0 ** (y[:, 0] * ys + ym), (y[:, 1] > 0).astype(np.int8),
            2.0 ** (y[:, 2] * cs + cm))


def cost_targets(naccept, nreject):
    """Target 2 from a solve's step log: log2 of the attempted steps."""
    steps = np.asarray(_np(naccept), np.float64) + np.asarray(_np(nreject), np.float64)
    return np.log2(np.maximum(steps, 1.0)).astype(np.float32)


def stiff_labels(solve_arrays, model, p, u0, t0, tf, saveat, save_kind, reltol, abstol,
                 explicit_maxiters=20000, precision=None):
    """Label 1 where Rodas5 is cheaper than Tsit5 on a trajectory: steps x
    device time per step of each kernel, both measured on these inputs in the
    precision the learned solves will run (GBDE_ALG_AUTO's: Tsit5 in
    `precision`, Rodas5 in FP64 for an FP64 solve and in FP32 pairs
    otherwise; default FP32 pairs for both).  Tsit5 runs that hit
    explicit_maxiters count as stiff."""
    prec = capi.PREC_F32X2 if precision is None else precision
    stiff_prec = capi.PREC_FP64 if prec == capi.PREC_FP64 else capi.PREC_F32X2
    res = {}
    for name, alg, pr, mi in (("tsit5", capi.ALG_TSIT5, prec, explicit_maxiters),
                              ("rodas5", capi.ALG_RODAS5, stiff_prec, 10 ** 6)):
        o = capi.opts_default(alg)
        o.reltol, o.abstol, o.maxiters, o.precision = reltol, abstol, mi, pr
        o.batching = capi.BATCH_PERSISTENT
        r = solve_arrays(model, o, p, u0, t0, tf, saveat, save_kind,
                         u_dtype="f64" if pr == capi.PREC_FP64 else "f32")
        steps = (_np(r["naccept"]) + _np(r["nreject"])).astype(np.float64)
        res[name] = (steps, r["device_ms"] / max(steps.sum(), 1.0), _np(r["retcode"]))
    (st_t, c_t, rc_t), (st_r, c_r, _) = res["tsit5"], res["rodas5"]
    stiff = (st_r * c_r < st_t * c_t) | (rc_t != capi.RET_SUCCESS)
    return stiff.astype(np.float32), {"tsit5_ms_per_step": c_t, "rodas5_ms_per_step": c_r}
