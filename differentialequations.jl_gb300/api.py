"""SciMLBase-shaped host API over the C ABI.

Mirrors the surface the reference re-exports (src/DifferentialEquations.jl:8-9;
allow-list test/qa/qa.jl): ODEProblem (qa.jl:86), SDEProblem (qa.jl:103),
remake (qa.jl:183), EnsembleProblem (qa.jl:50), solve (qa.jl:192),
ReturnCode (qa.jl:213), EnsembleSolution (qa.jl:52), the algorithm types
Tsit5 / Vern7 / Rosenbrock23 / Rodas5P (qa.jl:119,126,98,97) plus Rodas5, EM
and SOSRI, and a new ensemble algorithm `EnsembleGB300` that routes the whole
ensemble through one `gbde_ensemble_solve` call.

Semantics kept from the reference's pinned tests (test/core.jl):
  * saveat=0.1 on (0, 1) stores 11 points, t0 and tf included (core.jl:90-96);
  * the first stored state equals u0 exactly (core.jl:34);
  * remake(prob; u0=...) changes u0 (core.jl:81-88);
  * a Robertson solve with Rodas5P to t=1e5 returns Success (core.jl:38-49).
Callbacks (ContinuousCallback / DiscreteCallback, core.jl:60-79, and
VectorContinuousCallback / CallbackSet, qa.jl:124,26) take their condition
and affect as CUDA C++ source compiled into the kernels.  dense=True gives
solutions callable at any t (sol(0.5), core.jl:51-58).  Unsupported solve
keywords (save_everystep=True, tstops, save_idxs) raise instead of silently
changing behaviour.
"""
import copy
import enum
from fractions import Fraction

import numpy as np

from . import _capi as capi


class ReturnCode(enum.IntEnum):
    """SciMLBase.ReturnCode subset (qa.jl:213)."""
    Default = capi.RET_DEFAULT
    Success = capi.RET_SUCCESS
    MaxIters = capi.RET_MAXITERS
    DtLessThanMin = capi.RET_DTLESSTHANMIN
    Unstable = capi.RET_UNSTABLE
    InitialFailure = capi.RET_INITIALFAILURE
    Timeout = capi.RET_TIMEOUT
    Terminated = capi.RET_TERMINATED


# ---------------------------------------------------------------- models
class Model:
    """A built-in right-hand side f!(du, u, p, t) (and noise g for SDEs)."""

    def __init__(self, name, model_id, n_state, n_param, noise=False, doc=""):
        self.name, self.id = name, model_id
        self.n_state, self.n_param, self.noise = n_state, n_param, noise
        self.__doc__ = doc

    def __repr__(self):
        return "Model(%s, n_state=%d, n_param=%d)" % (self.name, self.n_state, self.n_param)

    def __deepcopy__(self, memo):
        return self  # built-in models are immutable singletons


class models:
    linear = Model("linear", capi.MODEL_LINEAR, 1, 1, doc="du = a u (test/core.jl:10)")
    lorenz = Model("lorenz", capi.MODEL_LORENZ, 3, 3, doc="Lorenz (test/core.jl:22-27)")
    robertson = Model("robertson", capi.MODEL_ROBERTSON, 3, 3,
                      doc="Robertson kinetics (test/core.jl:39-45)")
    vdp_ring8 = Model("vdp_ring8", capi.MODEL_VDP_RING8, 16, 2,
                      doc="ring of 8 Van der Pol oscillators, p=[mu, kappa]")
    lotka_volterra = Model("lotka_volterra", capi.MODEL_LOTKA_VOLTERRA, 2, 5, noise=True,
                           doc="Lotka-Volterra drift, diagonal noise sigma*u; "
                               "p=[alpha, beta, gamma, delta, sigma]")


def ODEFunction(f, n_state, n_param, jac=None, name="user_model"):
    """A user right-hand side (the reference's ODEFunction, qa.jl:84), given
    as CUDA C++ source and compiled at run time for the GPU (NVRTC).

    f: statements that fill du[0..n_state) from u[0..n_state) and
    p[0..n_param) in a function template over the scalar type T, e.g.
        "du[0] = p[0] * (u[1] - u[0]);  du[1] = ..."
    jac: optional statements filling J[r][c] = d du_r / d u_c; without it the
    Rosenbrock methods differentiate f with forward-mode dual numbers.
    The system is autonomous (carry t as an extra state if f depends on it).
    Registration copies the source; the first solve with an algorithm and a
    precision compiles the kernels (under a second) and caches them.
    Returns a Model usable as ODEProblem's f.
    """
    import ctypes as C
    d = capi.UserModel(name=name.encode(), n_state=int(n_state), n_param=int(n_param),
                       f_body=f.encode(), jac_body=jac.encode() if jac else None)
    mid = C.c_int32()
    capi.check(capi.lib().gbde_model_register(C.byref(d), C.byref(mid)))
    m = Model(name, mid.value, int(n_state), int(n_param), doc="user model (runtime-compiled)")
    m.f_source, m.jac_source = f, jac
    return m


def SDEFunction(f, g, n_state, n_param, jac=None, name="user_sde"):
    """A user SDE with diagonal noise (the reference's SDEFunction(f, g),
    qa.jl:102): du_i = f_i(u, p) dt + g_i(u, p) dW_i, both given as CUDA C++
    statements over the scalar type T -- f fills du[0..n_state), g fills
    g[0..n_state).  Compiled at run time for EM, SOSRI and SRIW1 (and for the
    ODE methods on f alone); the noise is the library's counter-based stream,
    the same as for the built-in models.  Returns a Model usable as
    SDEProblem's f (pass g=None or the same model as g)."""
    import ctypes as C
    d = capi.UserModel(name=name.encode(), n_state=int(n_state), n_param=int(n_param),
                       f_body=f.encode(), jac_body=jac.encode() if jac else None)
    mid = C.c_int32()
    capi.check(capi.lib().gbde_sde_model_register(C.byref(d), g.encode(), C.byref(mid)))
    m = Model(name, mid.value, int(n_state), int(n_param), noise=True,
              doc="user SDE model (runtime-compiled)")
    m.f_source, m.g_source, m.jac_source = f, g, jac
    return m


def compile_model(model, alg, precision="fp64"):
    """Compile a user model's kernels for one algorithm and precision ahead of
    the first solve (no GPU needed); raises GBDEError with NVRTC's log."""
    prec = {"fp64": capi.PREC_FP64, "mixed": capi.PREC_MIXED, "f32x2": capi.PREC_F32X2}[precision]
    capi.check(capi.lib().gbde_model_compile(model.id, alg.alg_id, prec))


def _save_bits(save_positions):
    before, after = save_positions
    return (capi.SAVE_BEFORE if before else 0) | (capi.SAVE_AFTER if after else 0)


class _Callback:
    def __init__(self, kind, condition, affect, terminate, len=1, save_positions=(True, True)):
        import ctypes as C
        bits = _save_bits(save_positions)
        d = capi.Callback(kind=kind, condition=condition.encode(),
                          affect=affect.encode() if affect is not None else None,
                          terminate=int(bool(terminate)), save_positions=bits)
        cid = C.c_int32()
        if kind == capi.CB_VECTOR:
            capi.check(capi.lib().gbde_vector_callback_register(C.byref(d), int(len),
                                                                C.byref(cid)))
        else:
            capi.check(capi.lib().gbde_callback_register(C.byref(d), C.byref(cid)))
        self.id, self.kind, self.len = cid.value, kind, int(len)
        self.condition, self.affect, self.terminate = condition, affect, terminate
        self.save_positions = tuple(bool(x) for x in save_positions)
        # the saves the kernels make: a continuous callback without an affect
        # leaves u unmodified and saves nothing after it
        modifies = kind == capi.CB_DISCRETE or affect is not None or terminate
        self.save_bits = bits if modifies else bits & capi.SAVE_BEFORE


class ContinuousCallback(_Callback):
    """ContinuousCallback(condition, affect=None; terminate=False,
    save_positions=(True, True)) (qa.jl:24).

    condition: CUDA C++ statements setting `g` (double) from `u` (the state,
    const double*), `t` and `p`; an event is a sign change of g, located on
    the method's dense output, where the trajectory stops (left of the root),
    runs affect (statements modifying `u[i]`, may set `terminate = true`) and
    restarts.  Example: ContinuousCallback("g = t - 0.5;").

    save_positions: save (t, u) at the event before / after the affect (the
    reference's keyword and default).  These saves join the saveat points in
    each trajectory's solution (sol[i].t, sol[i].u; the ensemble's U array
    holds the saveat points only).  affect=None (the reference's `nothing`)
    leaves u unmodified and saves nothing after the event; affect="" is a
    no-op affect, like a Julia function that does nothing."""

    def __init__(self, condition, affect=None, terminate=False, save_positions=(True, True)):
        super().__init__(capi.CB_CONTINUOUS, condition, affect, terminate,
                         save_positions=save_positions)


class DiscreteCallback(_Callback):
    """DiscreteCallback(condition, affect=None; terminate=False,
    save_positions=(True, True)) (qa.jl:36): after every accepted step, g != 0
    runs affect, with saves of (t, u) before and after it as save_positions
    asks (the one before is skipped when a saveat point falls on t).
    Example: DiscreteCallback("g = t >= 0.5;")."""

    def __init__(self, condition, affect=None, terminate=False, save_positions=(True, True)):
        super().__init__(capi.CB_DISCRETE, condition, affect, terminate,
                         save_positions=save_positions)


class VectorContinuousCallback(_Callback):
    """VectorContinuousCallback(condition, affect, len; terminate=False,
    save_positions=(True, True)) (qa.jl:124): len continuous conditions in
    one callback, with the event saves of ContinuousCallback.

    condition: CUDA C++ statements setting `out[0..len-1]` (double*) from
    `u`, `t` and `p`; the earliest sign change among them is the event, and
    affect runs with `idx` (int, 0-based: the reference's event_index - 1)
    naming the condition that fired.  Example, two balls bouncing:
    VectorContinuousCallback("out[0] = u[0]; out[1] = u[2];",
                             "u[2 * idx + 1] = -0.9 * u[2 * idx + 1];", 2)."""

    def __init__(self, condition, affect=None, len=1, terminate=False,
                 save_positions=(True, True)):
        super().__init__(capi.CB_VECTOR, condition, affect, terminate, len, save_positions)


class CallbackSet:
    """CallbackSet(cb1, cb2, ...) (qa.jl:26): continuous conditions of every
    member compete for the earliest root of a step (the first member on a
    tie); after each accepted step or event the discrete members run in
    order.  Members may be sets."""

    def __init__(self, *callbacks):
        import ctypes as C
        if not callbacks:
            raise ValueError("CallbackSet needs at least one callback")
        for cb in callbacks:
            if not isinstance(cb, (_Callback, CallbackSet)):
                raise TypeError("CallbackSet members are callbacks or callback sets")
        ids = (C.c_int32 * len(callbacks))(*[cb.id for cb in callbacks])
        sid = C.c_int32()
        capi.check(capi.lib().gbde_callback_set_register(ids, len(callbacks), C.byref(sid)))
        self.id, self.callbacks = sid.value, tuple(callbacks)
        self.save_bits = 0
        for cb in callbacks:
            self.save_bits |= cb.save_bits


# -------------------------------------------------------------- problems
class ODEProblem:
    """ODEProblem(f, u0, tspan, p; kwargs...) with a built-in model or a
    user model (ODEFunction) as f."""

    is_sde = False

    def __init__(self, f, u0, tspan, p=None, **kwargs):
        if not isinstance(f, Model):
            raise TypeError("f must be a Model: a built-in one (models.lorenz, ...) or a "
                            "user right-hand side from ODEFunction(source, n_state, n_param)")
        self.f = f
        self.u0 = np.atleast_1d(np.asarray(u0, dtype=np.float64)).copy()
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.p = (np.zeros(f.n_param) if p is None
                  else np.atleast_1d(np.asarray(p, dtype=np.float64)).copy())
        self.kwargs = dict(kwargs)
        if self.u0.shape != (f.n_state,):
            raise ValueError("u0 must have %d entries for %s" % (f.n_state, f.name))
        if self.p.shape != (f.n_param,):
            raise ValueError("p must have %d entries for %s" % (f.n_param, f.name))


class SDEProblem(ODEProblem):
    """SDEProblem(f, g, u0, tspan, p): the model carries both drift and noise."""

    is_sde = True

    def __init__(self, f, g, u0, tspan, p=None, **kwargs):
        if not (isinstance(f, Model) and f.noise):
            raise TypeError("SDEProblem needs a model with a noise term (a built-in one, or "
                            "SDEFunction(f, g, ...))")
        if g is not None and g is not f:
            raise TypeError("the noise term is part of the model; pass g=None or g=f")
        super().__init__(f, u0, tspan, p, **kwargs)


def remake(prob, u0=None, tspan=None, p=None, **kwargs):
    """remake(prob; u0, tspan, p, kwargs...) (qa.jl:183, core.jl:81-88)."""
    q = copy.copy(prob)
    q.u0 = prob.u0.copy() if u0 is None else np.atleast_1d(np.asarray(u0, np.float64)).copy()
    q.p = prob.p.copy() if p is None else np.atleast_1d(np.asarray(p, np.float64)).copy()
    q.tspan = prob.tspan if tspan is None else (float(tspan[0]), float(tspan[1]))
    q.kwargs = dict(prob.kwargs)
    q.kwargs.update(kwargs)
    if q.u0.shape != (prob.f.n_state,) or q.p.shape != (prob.f.n_param,):
        raise ValueError("remake: u0 / p have the wrong size for %s" % prob.f.name)
    return q


class EnsembleProblem:
    """EnsembleProblem(prob; prob_func, output_func, reduction, safetycopy)
    (qa.jl:50).

    prob_func(prob, i, repeat) -> problem for trajectory i (0-based here).
    batch(prob, N) -> dict with any of "u0" (N, n_state), "p" (N, n_param),
    "tspan" (N, 2), "saveat" (N, n_save): a vectorised prob_func for large
    ensembles (an extension; SciMLBase evaluates prob_func per trajectory).
    """

    def __init__(self, prob, prob_func=None, output_func=None, reduction=None,
                 safetycopy=True, batch=None):
        self.prob = prob
        self.prob_func = prob_func
        self.output_func = output_func
        self.reduction = reduction
        self.safetycopy = safetycopy
        self.batch = batch


# ------------------------------------------------------------ algorithms
class _Alg:
    alg_id = 0
    sde = False

    def __repr__(self):
        return type(self).__name__ + "()"


class Tsit5(_Alg):
    alg_id = capi.ALG_TSIT5


class Vern7(_Alg):
    alg_id = capi.ALG_VERN7


class Rosenbrock23(_Alg):
    alg_id = capi.ALG_ROSENBROCK23


class Rodas5(_Alg):
    alg_id = capi.ALG_RODAS5


class Rodas5P(_Alg):
    alg_id = capi.ALG_RODAS5P


class AutoTsit5(_Alg):
    """AutoTsit5(stiff_alg) (qa.jl:15): per trajectory, Tsit5 with a run-time
    stiffness estimate that switches to stiff_alg (Rosenbrock23() or
    Rodas5()) and back, with OrdinaryDiffEq's AutoSwitch defaults (10
    successive stiff estimates to switch, 3 non-stiff ones to switch back,
    tolerance 9/10, dt doubled / halved at a switch).  FP64 or "mixed"."""

    def __init__(self, stiff_alg=None):
        stiff_alg = Rosenbrock23() if stiff_alg is None else stiff_alg
        if isinstance(stiff_alg, Rosenbrock23):
            self.alg_id = capi.ALG_AUTOTSIT5_ROSENBROCK23
        elif isinstance(stiff_alg, Rodas5) and not isinstance(stiff_alg, Rodas5P):
            self.alg_id = capi.ALG_AUTOTSIT5_RODAS5
        else:
            raise TypeError("AutoTsit5 takes Rosenbrock23() or Rodas5()")
        self.stiff_alg = stiff_alg

    def __repr__(self):
        return "AutoTsit5(%r)" % (self.stiff_alg,)


class EM(_Alg):
    alg_id = capi.ALG_EM
    sde = True


class SOSRI(_Alg):
    """Rackauckas & Nie's stability-optimised SRI (strong order 1.5), adaptive."""
    alg_id = capi.ALG_SOSRI
    sde = True


class SRIW1(_Alg):
    """Roessler's SRIW1 (strong order 1.5), adaptive."""
    alg_id = capi.ALG_SRIW1
    sde = True


class EnsembleGB300:
    """Ensemble algorithm that solves every trajectory on one GB300 GPU.

    precision: "fp64", "mixed" (FP32 state/stages; FP64 time, error norm and
    W-matrix LU) or "f32x2" (state, stages and right-hand sides as FP32 pairs
    of ~48 bits; FP64 Jacobian, LU, error norm and time).  batching: "plain" (one launch, a thread per trajectory) or
    "persistent" (threads refill from a device work queue).  learned: False;
    True or "start" (the loaded predictor's first dt and AUTO method choice);
    "order" (the persistent queue ordered by the predicted cost); "stiff" (the
    AUTO method choice only); or a tuple of names.  devices: a list of GPU
    indices to split the trajectories over in one call (contiguous slices, one
    host thread and context per GPU, no collective); default: `device` alone.
    """

    def __init__(self, device=0, precision="fp64", batching="plain", learned=False,
                 block_size=0, ctas_per_sm=0, chunk=0, out_dtype=None, timeout_s=0.0,
                 devices=None):
        if precision not in ("fp64", "mixed", "f32x2"):
            raise ValueError("precision must be 'fp64', 'mixed' or 'f32x2'")
        if batching not in ("plain", "persistent"):
            raise ValueError("batching must be 'plain' or 'persistent'")
        self.device, self.precision, self.batching = device, precision, batching
        self.learned, self.block_size, self.ctas_per_sm = learned, block_size, ctas_per_sm
        self.learned_flags = learned_flags(learned)
        self.chunk, self.timeout_s = chunk, timeout_s
        self.out_dtype = out_dtype or ("f32" if precision == "mixed" else "f64")
        self.devices = [int(d) for d in devices] if devices else [int(device)]
        if not self.devices:
            raise ValueError("devices must name at least one GPU")


def learned_flags(learned):
    """gbde_opts.learned from EnsembleGB300's `learned` argument."""
    if learned is False or learned is None:
        return 0
    if learned is True:
        return capi.LEARN_START
    names = (learned,) if isinstance(learned, str) else tuple(learned)
    flags = 0
    table = {"start": capi.LEARN_START, "order": capi.LEARN_ORDER, "stiff": capi.LEARN_STIFF}
    for n in names:
        if n not in table:
            raise ValueError("learned takes True/False, 'start', 'order', 'stiff' or a tuple "
                             "of them")
        flags |= table[n]
    return flags


class EnsembleThreads:
    """The reference's CPU ensemble algorithm (qa.jl:56).  This library does
    not solve on the CPU; pass EnsembleGB300() instead."""


class EnsembleSerial(EnsembleThreads):
    """(qa.jl:51) -- see EnsembleThreads."""


# ------------------------------------------------------------- solutions
class ODESolution:
    """One trajectory's solution: views into the ensemble arrays."""

    def __init__(self, t, u, retcode, prob=None, stats=None, dense=None):
        self.t = t
        self._u = u
        self.retcode = ReturnCode(int(retcode))
        self.prob = prob
        self.stats = stats or {}
        self._dense = dense  # callable(times) -> (len(times), n_state), or None

    @property
    def u(self):
        return [self._u[j] for j in range(self._u.shape[0])]

    def __getitem__(self, j):
        return self._u[j]

    def __len__(self):
        return self._u.shape[0]

    def __call__(self, t):
        """The solution at time(s) t.  A solve with dense=True evaluates the
        method's own dense output (the interpolant the kernels save with) at t:
        the trajectory is solved again on the GPU with t as its save times --
        save points never change a trajectory's steps, so the values are
        exactly those a saveat containing t would have stored.  Without
        dense=True: linear interpolation between the stored points."""
        scalar = np.ndim(t) == 0
        ts = np.atleast_1d(np.asarray(t, np.float64))
        if self._dense is not None:
            order = np.argsort(ts, kind="stable")
            vals = np.empty((len(ts), self._u.shape[1]))
            vals[order] = self._dense(ts[order])
        else:
            vals = np.stack([np.interp(ts, self.t, self._u[:, c])
                             for c in range(self._u.shape[1])], axis=1)
        return vals[0] if scalar else vals


class EnsembleSolution:
    """EnsembleSolution (qa.jl:52): `u` is the list of per-trajectory
    solutions; `U`, `t`, `retcode` expose the underlying arrays."""

    def __init__(self, U, t, retcode, lengths, stats, elapsed_ms, device_ms, output_func=None,
                 reduction=None, probs=None, dense=None, events=None):
        self.U = U                  # (N, n_save, n_state): the saveat points
        self.events = events        # (ev_t, ev_u, ev_count) of the callbacks' saves, or None
        self.t = t                  # (n_save,) or (N, n_save)
        self.retcode = retcode      # (N,) int32
        self.lengths = lengths      # (N,) stored points per trajectory
        self.stats = stats          # dict of (N,) arrays
        self.elapsedTime = elapsed_ms / 1e3
        self.device_ms = device_ms
        self._output_func = output_func
        self._probs = probs
        self._dense = dense  # callable(i, times), or None

    def __len__(self):
        return self.U.shape[0]

    def solution(self, i):
        n = int(self.lengths[i])
        t = self.t[:n] if self.t.ndim == 1 else self.t[i, :n]
        u = self.U[i, :n]
        if self.events is not None and int(self.events[2][i]) > 0:
            # the saveat points and the event saves in time order; at one
            # time the saveat points first, then the event saves as made
            ev_t, ev_u, ev_n = self.events
            c = int(ev_n[i])
            tt = np.concatenate([np.asarray(t, np.float64), np.asarray(ev_t[i, :c])])
            kind = np.r_[np.zeros(n, np.int8), np.ones(c, np.int8)]
            order = np.lexsort((np.arange(n + c), kind, tt))
            t = tt[order]
            u = np.concatenate([np.asarray(u), np.asarray(ev_u[i, :c])])[order]
        st = {k: v[i] for k, v in self.stats.items()}
        dense = None
        if self._dense is not None:
            dense = (lambda ts, i=i: self._dense(i, ts))
        return ODESolution(t, u, self.retcode[i],
                           None if self._probs is None else self._probs[i], st, dense)

    def __getitem__(self, i):
        return self.solution(i)

    @property
    def u(self):
        return [self.solution(i) for i in range(len(self))]

    @property
    def converged(self):
        return bool(np.all(self.retcode == capi.RET_SUCCESS))


# ------------------------------------------------------ ensemble statistics
def ensemble_summary(u, quantiles=(), device=0):
    """Mean, variance (N - 1) and quantiles across trajectories of
    u[N][n_save][n_state], computed on the GPU (gbde_ensemble_summary).
    u: a CUDA tensor (statistics stay on its device and come back as CUDA
    tensors) or a host array (staged).  Returns (mean, var, qvals) with
    qvals[j] for quantiles[j]."""
    import ctypes as C
    q = [float(x) for x in quantiles]
    if len(q) > capi.SUMMARY_MAX_Q:
        raise ValueError("at most %d quantiles" % capi.SUMMARY_MAX_Q)
    if u.ndim != 3:
        raise ValueError("u must be [N][n_save][n_state]")
    N, ns, nst = (int(x) for x in u.shape)
    sm = capi.Summary()
    sm.n_quantiles = len(q)
    for j, v in enumerate(q):
        sm.quantiles[j] = v
    on_device = not isinstance(u, np.ndarray)
    if on_device:
        import torch
        if u.dtype not in (torch.float32, torch.float64):
            raise TypeError("u must be float32 or float64")
        u = u.contiguous()
        mean = torch.empty((ns, nst), dtype=torch.float64, device=u.device)
        var = torch.empty_like(mean)
        qv = torch.empty((max(len(q), 1), ns, nst), dtype=torch.float64, device=u.device)
        ctx = capi.context(u.device.index or 0)
        ctx.set_stream(torch.cuda.current_stream(u.device).cuda_stream)
        dt = capi.F32 if u.dtype == torch.float32 else capi.F64
        mem = capi.MEM_DEVICE
    else:
        if u.dtype not in (np.float32, np.float64):
            u = u.astype(np.float64)
        u = np.ascontiguousarray(u)
        mean = np.empty((ns, nst))
        var = np.empty((ns, nst))
        qv = np.empty((max(len(q), 1), ns, nst))
        ctx = capi.context(device)
        ctx.set_stream(0)
        dt = capi.F32 if u.dtype == np.float32 else capi.F64
        mem = capi.MEM_HOST
    sm.mean, sm.var = capi.ptr(mean), capi.ptr(var)
    sm.qvals = capi.ptr(qv) if q else None
    capi.check(capi.lib().gbde_ensemble_summary(ctx.handle, capi.ptr(u), dt, mem, N, ns, nst,
                                                C.byref(sm)), ctx.handle)
    return mean, var, qv[:len(q)]


class EnsembleSummary:
    """EnsembleSummary (qa.jl:54) of an ensemble solution at its save times:
    `t`, `u` (mean), `v` (variance), `med`, `qlow`, `qhigh` as
    [n_save][n_state] arrays, computed on the GPU.  Like the reference, the
    statistics are taken per time point across trajectories; with per-
    trajectory save times they are per save index."""

    def __init__(self, sim, quantiles=(0.05, 0.95), device=0):
        U = sim.U if isinstance(sim, EnsembleSolution) else sim
        mean, var, qv = ensemble_summary(U, (0.5, float(quantiles[0]), float(quantiles[1])),
                                         device)
        self.t = sim.t if isinstance(sim, EnsembleSolution) else None
        self.u, self.v = mean, var
        self.med, self.qlow, self.qhigh = qv[0], qv[1], qv[2]
        self.num_monte = int(U.shape[0])
        self.converged = bool(sim.converged) if isinstance(sim, EnsembleSolution) else None


# ----------------------------------------------------------- save times
def _dec(x):
    """Exact rational of the shortest decimal that round-trips x (so that
    t0 + k*0.1 is the correctly rounded k/10, as a decimal step range)."""
    return Fraction(repr(float(x)))


def save_grid(t0, tf, saveat, save_start=None, save_end=None):
    """Save times for one trajectory with the reference's defaults:
    a number Δ gives t0, t0+Δ, ..., and tf (save_start/save_end default
    True); a vector keeps the times in [t0, tf], with t0 / tf stored only if
    listed (or requested)."""
    if np.isscalar(saveat):
        d = float(saveat)
        if not d > 0:
            raise ValueError("saveat step must be > 0")
        ts = []
        f0, fd, ff = _dec(t0), _dec(d), _dec(tf)
        k = 1
        while True:
            tk = f0 + k * fd
            if tk >= ff:
                break
            ts.append(float(tk))
            k += 1
        start = True if save_start is None else save_start
        end = True if save_end is None else save_end
        out = ([t0] if start else []) + ts + ([tf] if end else [])
        return np.asarray(out, np.float64)
    v = np.asarray(saveat, np.float64).ravel()
    inside = v[(v > t0) & (v < tf)]
    start = (t0 in v) if save_start is None else save_start
    end = (tf in v) if save_end is None else save_end
    out = np.concatenate([[t0] if start else [], np.sort(inside), [tf] if end else []])
    return out.astype(np.float64)


# ----------------------------------------------------------------- solve
_UNSUPPORTED = ("save_everystep", "tstops", "save_idxs")


def _gather_inputs(ens, N):
    prob = ens.prob
    ns, np_ = prob.f.n_state, prob.f.n_param
    u0 = np.broadcast_to(prob.u0, (N, ns)).copy()
    p = np.broadcast_to(prob.p, (N, np_)).copy()
    tspan = np.broadcast_to(np.asarray(prob.tspan), (N, 2)).copy()
    saves = None
    probs = None
    if ens.batch is not None:
        b = ens.batch(prob, N)
        if "u0" in b:
            u0 = np.ascontiguousarray(b["u0"], np.float64).reshape(N, ns)
        if "p" in b:
            p = np.ascontiguousarray(b["p"], np.float64).reshape(N, np_)
        if "tspan" in b:
            tspan = np.ascontiguousarray(b["tspan"], np.float64).reshape(N, 2)
        if "saveat" in b:
            saves = np.ascontiguousarray(b["saveat"], np.float64).reshape(N, -1)
    elif ens.prob_func is not None:
        probs = []
        per_save = []
        for i in range(N):
            base = copy.deepcopy(prob) if ens.safetycopy else prob
            pi = ens.prob_func(base, i, 1)
            if pi.f is not prob.f:
                raise ValueError("prob_func must keep the model of the ensemble's problem")
            u0[i], p[i], tspan[i] = pi.u0, pi.p, pi.tspan
            per_save.append(pi.kwargs.get("saveat"))
            probs.append(pi)
        if any(s is not None for s in per_save):
            saves = per_save
    return u0, p, tspan, saves, probs


_EVENT_SAVES_GUESS = 8  # event saves per trajectory room of a callback solve's first try


def solve(ens, alg, ensemblealg=None, trajectories=None, saveat=None, save_start=None,
          save_end=None, reltol=None, abstol=None, dt=None, adaptive=None, maxiters=None,
          dtmin=None, dtmax=None, seed=0, **kwargs):
    """solve(EnsembleProblem, alg, EnsembleGB300(); trajectories, saveat,
    reltol, abstol, ...) -> EnsembleSolution.  A plain ODEProblem /
    SDEProblem is solved as an ensemble of one trajectory."""
    for k in _UNSUPPORTED:
        if k in kwargs and kwargs[k] not in (None, False):
            raise NotImplementedError("solve keyword %r is not supported by EnsembleGB300" % k)
    extra = set(kwargs) - set(_UNSUPPORTED) - {"qmin", "qmax", "gamma", "beta1", "beta2",
                                               "qsteady_min", "qsteady_max", "qoldinit",
                                               "callback", "dense"}
    if extra:
        raise TypeError("unknown solve keywords: %s" % sorted(extra))
    single = not isinstance(ens, EnsembleProblem)
    if single:
        ens = EnsembleProblem(ens)
        trajectories = 1
    if ensemblealg is None:
        ensemblealg = EnsembleGB300()
    if not isinstance(ensemblealg, EnsembleGB300):
        raise NotImplementedError("this library solves ensembles on the GPU only: "
                                  "use EnsembleGB300()")
    if not isinstance(alg, _Alg):
        raise TypeError("alg must be one of Tsit5(), Vern7(), Rosenbrock23(), Rodas5(), "
                        "Rodas5P(), EM(), SOSRI(), SRIW1()")
    prob = ens.prob
    if alg.sde and not prob.is_sde:
        raise TypeError("%r needs an SDEProblem" % alg)
    if trajectories is None or int(trajectories) < 0:
        raise ValueError("trajectories must be a non-negative integer")
    N = int(trajectories)
    if saveat is None:
        saveat = prob.kwargs.get("saveat")
    u0, p, tspan, saves, probs = _gather_inputs(ens, N)
    t0 = np.ascontiguousarray(tspan[:, 0])
    tf = np.ascontiguousarray(tspan[:, 1])

    # ---- save layout
    if isinstance(saves, np.ndarray):
        save_kind, save_arr = capi.SAVE_PER_TRAJ, saves
        lengths = np.full(N, saves.shape[1], np.int64)
    else:
        per = None
        if isinstance(saves, list):
            per = [s if s is not None else saveat for s in saves]
        if per is None and saveat is None and kwargs.get("dense"):
            # dense=True without saveat: store the end points; sol(t) evaluates
            # the method's interpolant anywhere in between
            saveat = []
            save_start = True if save_start is None else save_start
            save_end = True if save_end is None else save_end
        if per is None and saveat is None:
            if save_end is False and save_start is False:
                raise ValueError("nothing to save")
            raise NotImplementedError(
                "EnsembleGB300 stores fixed save grids: pass saveat (a step or a vector), or "
                "dense=True (saving every step is not supported)")
        uniform = per is None and (N == 0 or (np.all(t0 == t0[0]) and np.all(tf == tf[0])))
        if uniform:
            grid = save_grid(t0[0] if N else prob.tspan[0], tf[0] if N else prob.tspan[1],
                             saveat, save_start, save_end)
            save_kind, save_arr = capi.SAVE_GRID, grid
            lengths = np.full(N, len(grid), np.int64)
        else:
            grids = [save_grid(t0[i], tf[i], per[i] if per else saveat, save_start, save_end)
                     for i in range(N)]
            lengths = np.array([len(g) for g in grids], np.int64)
            m = int(lengths.max()) if N else 0
            save_arr = np.empty((N, m), np.float64)
            for i, g in enumerate(grids):
                save_arr[i, :len(g)] = g
                save_arr[i, len(g):] = tf[i]  # padding: repeats of the final state
            save_kind = capi.SAVE_PER_TRAJ

    opts = capi.opts_default(alg.alg_id)
    opts.precision = {"mixed": capi.PREC_MIXED, "f32x2": capi.PREC_F32X2}.get(
        ensemblealg.precision, capi.PREC_FP64)
    opts.batching = (capi.BATCH_PERSISTENT if ensemblealg.batching == "persistent"
                     else capi.BATCH_PLAIN)
    if reltol is not None:
        opts.reltol = reltol
    if abstol is not None:
        opts.abstol = abstol
    if dt is not None:
        opts.dt = dt
    if adaptive is not None:
        opts.adaptive = int(bool(adaptive))
    if maxiters is not None:
        opts.maxiters = int(maxiters)
    if dtmin is not None:
        opts.dtmin = dtmin
    if dtmax is not None:
        opts.dtmax = dtmax
    for k in ("qmin", "qmax", "gamma", "beta1", "beta2", "qsteady_min", "qsteady_max",
              "qoldinit"):
        if k in kwargs:
            setattr(opts, k, float(kwargs[k]))
    opts.seed = int(seed)
    opts.learned = ensemblealg.learned_flags
    cb = kwargs.get("callback")
    if cb is not None:
        if not isinstance(cb, (_Callback, CallbackSet)):
            raise TypeError("callback must be a ContinuousCallback, DiscreteCallback, "
                            "VectorContinuousCallback or CallbackSet")
        opts.callback = cb.id
    opts.block_size = int(ensemblealg.block_size)
    opts.ctas_per_sm = int(ensemblealg.ctas_per_sm)
    opts.chunk = int(ensemblealg.chunk)
    opts.timeout_s = float(ensemblealg.timeout_s)

    def run(events):
        if len(ensemblealg.devices) > 1:
            from . import distributed
            return distributed.solve_sharded(solve_arrays, ensemblealg.devices, prob.f, opts, p,
                                             u0, t0, tf, save_arr, save_kind,
                                             u_dtype=ensemblealg.out_dtype, events=events)
        return solve_arrays(prob.f, opts, p, u0, t0, tf, save_arr, save_kind,
                            u_dtype=ensemblealg.out_dtype, device=ensemblealg.devices[0],
                            events=events)

    # saves at callback events: a first guess of their number per trajectory;
    # a trajectory that made more has them all counted, and the ensemble is
    # solved again with room for the largest count (same steps, same results)
    events = _EVENT_SAVES_GUESS if cb is not None and cb.save_bits else None
    res = run(events)
    if events is not None and N and int(res["ev_count"].max()) > events:
        events = int(res["ev_count"].max())
        res = run(events)
    t_out = save_arr
    term = res["retcode"] == capi.RET_TERMINATED
    if np.any(term):
        # a terminated trajectory ends at its event: keep the saves up to t_end
        ts = t_out if t_out.ndim == 2 else np.broadcast_to(t_out, (N, t_out.shape[-1]))
        lengths = np.where(term, np.sum(ts <= res["t_end"][:, None], axis=1), lengths)
    dense = None
    if kwargs.get("dense"):
        dev = ensemblealg.devices[0]

        def dense(i, ts, opts=opts, model=prob.f):
            ts = np.asarray(ts, np.float64)
            if np.any(ts < t0[i]) or np.any(ts > tf[i]):
                raise ValueError("dense output is defined on [t0, tf] = [%g, %g]" % (t0[i], tf[i]))
            r = solve_arrays(model, opts, p[i:i + 1], u0[i:i + 1], t0[i:i + 1], tf[i:i + 1], ts,
                             capi.SAVE_GRID, u_dtype=ensemblealg.out_dtype, device=dev)
            return np.asarray(r["u"][0], np.float64)

    ev = None if events is None else (res["ev_t"], res["ev_u"], res["ev_count"])
    sol = EnsembleSolution(res["u"], t_out, res["retcode"], lengths,
                           {k: res[k] for k in ("naccept", "nreject", "nf", "t_end")},
                           res["total_ms"], res["device_ms"], probs=probs, dense=dense,
                           events=ev)
    if ens.output_func is not None:
        outs = []
        for i in range(N):
            o, _rerun = ens.output_func(sol.solution(i), i)
            outs.append(o)
        sol.outputs = outs
    if single:
        return sol.solution(0)
    return sol


def solve_arrays(model, opts, p, u0, t0, tf, saveat, save_kind, u_dtype="f64", device=0,
                 out=None, stats=True, reduce=False, store_u=True, events=None):
    """Low-level entry: arrays in, arrays out, one gbde_ensemble_solve call.

    reduce=True accumulates, inside the step kernels, the sums over
    trajectories of every saved state and of its square (gbde_outputs.reduce),
    returned as res["reduce"] [2][n_save][n_state] with res["mean"] and
    res["var"] (N - 1); store_u=False then skips storing the ensemble.

    events=K (a solve with opts.callback) keeps up to K saves at callback
    events per trajectory (the callbacks' save_positions): res["ev_t"] [N][K],
    res["ev_u"] [N][K][n_state] and res["ev_count"] [N], which counts every
    save made, also those beyond K.

    Host numpy arrays -> GBDE_MEM_HOST (the call stages the copies).
    CUDA torch tensors -> GBDE_MEM_DEVICE on the tensors' device and the
    current torch stream; results are CUDA tensors.
    """
    N = int(u0.shape[0])
    n_save = int(saveat.shape[-1]) if saveat is not None else 0
    on_device = not isinstance(u0, np.ndarray)
    prob = capi.Problem()
    prob.model = model.id
    prob.n_state, prob.n_param = model.n_state, model.n_param
    prob.n_traj = N
    prob.save_kind = save_kind
    prob.n_save = n_save
    outs = capi.Outputs()
    outs.u_dtype = capi.F32 if u_dtype == "f32" else capi.F64
    ctx = capi.context(device)
    if on_device:
        import torch
        prob.mem = capi.MEM_DEVICE
        dev = u0.device
        tdt = torch.float32 if u_dtype == "f32" else torch.float64
        res = out or {
            "u": (torch.empty((N, n_save, model.n_state), dtype=tdt, device=dev)
                  if store_u else None),
            "retcode": torch.empty(N, dtype=torch.int32, device=dev),
        }
        if reduce:
            res["reduce"] = torch.empty((2, n_save, model.n_state), dtype=torch.float64,
                                        device=dev)
        if stats and out is None:
            for k in ("naccept", "nreject", "nf", "method"):
                res[k] = torch.empty(N, dtype=torch.int32, device=dev)
            res["t_end"] = torch.empty(N, dtype=torch.float64, device=dev)
            res["dt_first"] = torch.empty(N, dtype=torch.float64, device=dev)
        ctx.set_stream(torch.cuda.current_stream(dev).cuda_stream)
        arrs = (p, u0, t0, tf, saveat)
    else:
        prob.mem = capi.MEM_HOST
        arrs = tuple(np.ascontiguousarray(a, np.float64) if a is not None else None
                     for a in (p, u0, t0, tf, saveat))
        res = out or {
            "u": (np.empty((N, n_save, model.n_state),
                           np.float32 if u_dtype == "f32" else np.float64) if store_u else None),
            "retcode": np.empty(N, np.int32),
        }
        if reduce:
            res["reduce"] = np.empty((2, n_save, model.n_state))
        if stats and out is None:
            for k in ("naccept", "nreject", "nf", "method"):
                res[k] = np.empty(N, np.int32)
            res["t_end"] = np.empty(N, np.float64)
            res["dt_first"] = np.empty(N, np.float64)
        ctx.set_stream(0)
    if events is not None:
        cap = int(events)
        if on_device:
            res.setdefault("ev_t", torch.empty((N, cap), dtype=torch.float64, device=dev))
            res.setdefault("ev_u", torch.empty((N, cap, model.n_state), dtype=tdt, device=dev))
            res.setdefault("ev_count", torch.empty(N, dtype=torch.int32, device=dev))
        else:
            res.setdefault("ev_t", np.empty((N, cap), np.float64))
            res.setdefault("ev_u", np.empty((N, cap, model.n_state),
                                            np.float32 if u_dtype == "f32" else np.float64))
            res.setdefault("ev_count", np.empty(N, np.int32))
        outs.ev_t, outs.ev_u = capi.ptr(res["ev_t"]), capi.ptr(res["ev_u"])
        outs.ev_count, outs.ev_capacity = capi.ptr(res["ev_count"]), cap
    prob.p, prob.u0, prob.t0, prob.tf, prob.saveat = [capi.ptr(a) for a in arrs]
    outs.u = capi.ptr(res["u"])
    outs.retcode = capi.ptr(res["retcode"])
    if reduce:
        outs.reduce = capi.ptr(res["reduce"])
    for k in ("naccept", "nreject", "nf", "t_end", "method", "dt_first"):
        if k in res:
            setattr(outs, k, capi.ptr(res[k]))
    for k in ("naccept", "nreject", "nf", "t_end", "method", "dt_first"):
        res.setdefault(k, None)
    ctx.solve(prob, opts, outs)
    res["device_ms"] = outs.device_ms
    res["total_ms"] = outs.total_ms
    if reduce:
        s1, s2 = res["reduce"][0], res["reduce"][1]
        res["mean"] = s1 / N
        res["var"] = (s2 - s1 * s1 / N) / (N - 1) if N > 1 else s1 * float("nan")
    return res
