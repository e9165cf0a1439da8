"""Ensemble throughput benchmark (one JSON line on rank 0).

Workload (default): the mixed-precision coupled-oscillator ensemble -- a ring
of 8 Van der Pol oscillators (16 states) with diffusive coupling kappa = 0.05,
mu = 10^U(-1, 3) per trajectory, u0 ~ U[-2, 2]^16, tspan (0, 20), reltol =
abstol = 1e-5, saves every 1.0 (21 points), 1,000,000 trajectories; each
trajectory runs Tsit5 if mu <= 60 and Rodas5 otherwise (GBDE_ALG_AUTO).
Seeded synthetic inputs with the configuration's distributions (no dataset).
Other configurations print their own line with --workload.

A "step" is one ensemble solve of all trajectories.  `value` is trajectories
per second of the chosen form with inputs resident in HBM (device pointers,
one gbde_ensemble_solve), the median over the timed steps; `e2e` is the same
through the C ABI with pinned host buffers (H2D + solve + D2H inside the
timed region).  `plain` is the plain one-launch FP64 form.  Before timing,
the chosen and plain forms are checked against the CPU FP64 oracle (same
algorithm per trajectory, same tolerances) on a sample.

--impl reference times the CPU FP64 restatement of the same workload (an
EnsembleThreads-equivalent std::thread pool over all host cores) on bounded
samples; it loads only the oracle.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

SEED = 20261204

# Algorithmic FP64 flops per attempted step / per accepted step / per save
# point (FMA = 2 flops, division and sqrt = 1), counted from the methods'
# arithmetic for n = 3: Rodas5 = 7 RHS evaluations, 3x3 LU, 8 triangular
# solves, the stage sums and the error norm; +16 per accepted step for the
# Jacobian and f at the new point; +150 per dense-output save point.
FLOPS = {
    ("rodas5", "robertson"): (510.0, 16.0, 150.0),
    ("rosenbrock23", "robertson"): (156.0, 16.0, 20.0),
    ("tsit5", "lorenz"): (272.0, 0.0, 85.0),
}

# FP64 work of one attempted step of Rodas5 on the 16-state ring that stays
# FP64 in every precision (FMA = 2 flops).  The LU of W with partial pivoting:
# on the ring's W the elimination has 34 nonzero multipliers and 297 updated
# row entries whatever the values (a structural constant, checked on 3,000
# random ring matrices), so 34 + 2 x 297 + 16 pivot reciprocals = 644 flops
# (the dense count, 2,600, multiplies mostly zeros); W's diagonal
# 1/(gamma h) - J_rr, 16; the Jacobian rows, 8 x 9 = 72; the error norm's
# squares, 16 x 2 = 32.
TEAM_RODAS_FP64_PER_ATTEMPT = 644.0 + 16.0 + 72.0 + 32.0

# DRAM bytes (read + write) per trajectory of the Rodas5 solve kernel, from one
# ncu capture each, scaled by trajectories.  FP64 stepper: 20,000 trajectories,
# 4.587 MB read + 8.2 KB written (the saved states stay in L2 until after the
# kernel).  FP32-pair stepper: 100,000 trajectories, persistent launch in
# longest-span-first and in learned-cost order.
TRAFFIC_PER_TRAJ = {"fp64": (4.586752e6 + 8192.0) / 20000.0,
                    "f32x2": (31.265536e6 + 9.635328e6) / 100000.0,
                    "f32x2-learned": (30.901504e6 + 8.447488e6) / 100000.0}

# The ring's two kernels in FP32 pairs, from one ncu capture at 400,000
# trajectories of the ring workload (`python bench.py --trajectories 400000
# --steps 1 --warmup 1 --no-cpu-baseline` under ncu --metrics
# dram__bytes_read.sum,dram__bytes_write.sum,smsp__inst_executed.sum; the split
# at mu = 60: 122,217 stiff, 277,783 non-stiff):
#   k_team8<TeamRodasFF8> (stiff): 1,307 DRAM bytes (read + write) per
#   trajectory against ~1,536 bytes of inputs and outputs (the last saves are
#   still in L2 when the kernel ends); 37.38e9 warp instructions, 1,283 per
#   trajectory and attempted step (238.4 attempts each by the oracle's count
#   on the run's 2,000-trajectory sample; a warp carries 4 trajectories);
#   k_team8<TeamTsit5FF> (non-stiff): 1,435 DRAM bytes and 136,005 warp
#   instructions per trajectory (its attempted steps vary with mu; the
#   workload's mu distribution is the same at every N).
RING_STIFF_TRAFFIC_PER_TRAJ = (39.101952e6 + 120.644096e6) / 122217.0
RING_STIFF_INST_PER_ATTEMPT = 37.379764e9 / (122217.0 * 238.4)
RING_NONSTIFF_TRAFFIC_PER_TRAJ = (63.819520e6 + 334.766592e6) / 277783.0
RING_NONSTIFF_INST_PER_TRAJ = 37.779985e9 / 277783.0

WORKLOADS = ["vdp_auto", "robertson", "lorenz", "lv_em", "lv_sosri", "summary",
             "learned_lorenz", "learned_lv", "learned_vdp"]
DEFAULT_N = {"vdp_auto": 1000000, "robertson": 100000, "lorenz": 10000, "lv_em": 1000000,
             "lv_sosri": 1000000, "summary": 1000000, "learned_lorenz": 1000000,
             "learned_lv": 1000000, "learned_vdp": 1000000}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="vdp_auto", choices=WORKLOADS,
                    help="vdp_auto = the 16-state ring, 1M trajectories (default); "
                         "robertson = the stiff Robertson ensemble; the others print the "
                         "line of another configuration")
    ap.add_argument("--alg", default="rodas5", choices=["rodas5", "rosenbrock23"],
                    help="robertson workload: the method")
    ap.add_argument("--trajectories", type=int, default=None)
    ap.add_argument("--chosen", default=None,
                    help="chosen form.  vdp_auto: persistent-f32x2 (default) | "
                         "persistent-mixed | persistent | plain.  robertson: "
                         "persistent-f32x2-learned (default) | persistent-f32x2 | "
                         "plain-f32x2 | persistent | plain | persistent-mixed | plain-mixed")
    ap.add_argument("--user-model", default="none", choices=["none", "analytic", "dual"],
                    help="robertson workload: solve through a user right-hand side compiled "
                         "at run time (the Robertson formulas as source; Jacobian given or by "
                         "dual numbers) instead of the built-in model; chosen forms without "
                         "the learned predictor")
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="trajectories of each CPU-baseline / reference-arm sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    a = ap.parse_args()
    if a.trajectories is None:
        a.trajectories = DEFAULT_N[a.workload]
    return a


def workload(N, seed):
    """The Robertson ensemble: rates (0.04, 3e7, 1e4) x 10^U(-1,1), u0 =
    [1,0,0], tf = 10^U(1,5), 20 log-spaced save times per trajectory."""
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
    t0 = np.zeros(N)
    tf = 10 ** rng.uniform(1, 5, N)
    saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
    return p, u0, t0, tf, np.ascontiguousarray(saveat)


VDP_RTOL = 1e-5
# The AUTO split of the ring workload: Rodas5 for mu above it, Tsit5 below (the
# same split for every form and for the CPU port).  The AUTO solve time on GB300
# against the split (1M trajectories, FP32 pairs): 286 / 266 / 255 / 256 / 265 /
# 290 ms at 20 / 30 / 50 / 70 / 100 / 150; on the later kernels the two kernels'
# times summed: 211.4 / 210.8 / 210.8 / 211.0 / 212.0 / 212.7 ms at 45 / 50 / 55
# / 60 / 65 / 70.
VDP_STIFF_MU = 60.0


def vdp_inputs(N, seed):
    """The 16-state ring: mu = 10^U(-1,3), kappa = 0.05, u0 ~ U[-2,2]^16,
    tspan (0, 20), saves 0:1:20."""
    rng = np.random.default_rng(seed)
    p = np.c_[10 ** rng.uniform(-1, 3, N), np.full(N, 0.05)]
    u0 = rng.uniform(-2, 2, (N, 16))
    return p, u0, np.zeros(N), np.full(N, 20.0), np.arange(21.0)


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def oracle_robertson(alg, N_sample, seed, threads):
    """The CPU FP64 oracle on N_sample trajectories of the Robertson ensemble
    (`alg`: "rodas5" or "rosenbrock23"); returns (trajectories/s, s, result)."""
    import oracle
    p, u0, t0, tf, saveat = workload(N_sample, seed)
    o = oracle.opts_default(oracle.ALG_RODAS5 if alg == "rodas5" else oracle.ALG_ROSENBROCK23)
    o.reltol, o.abstol = 1e-6, 1e-10
    t = time.perf_counter()
    r = oracle.solve(None, oracle.ModelRef(oracle.MODEL_ROBERTSON), o, p, u0, t0, tf, saveat,
                     oracle.SAVE_PER_TRAJ, nthreads=threads)
    dt = time.perf_counter() - t
    return N_sample / dt, dt, r


def oracle_vdp(p, u0, t0, tf, saveat, stiff, threads, rtol=VDP_RTOL, alg_all=None):
    """The CPU FP64 oracle on the 16-state ring, each trajectory with the
    method the GPU ran (stiff: Rodas5, else Tsit5; or alg_all for every
    trajectory), at reltol = abstol = rtol."""
    import oracle
    N = len(p)
    M = oracle.ModelRef(oracle.MODEL_VDP_RING8)
    res = {"u": np.empty((N, len(saveat), 16)), "naccept": np.zeros(N, np.int32),
           "nreject": np.zeros(N, np.int32), "retcode": np.zeros(N, np.int32)}
    parts = ((np.ones(N, bool), alg_all),) if alg_all else (
        (~stiff, oracle.ALG_TSIT5), (stiff, oracle.ALG_RODAS5))
    for mask, alg in parts:
        if not mask.any():
            continue
        o = oracle.opts_default(alg)
        o.reltol = o.abstol = rtol
        o.maxiters = 10 ** 7
        r = oracle.solve(None, M, o, p[mask], u0[mask], t0[mask], tf[mask], saveat,
                         oracle.SAVE_GRID, nthreads=threads)
        for k in res:
            res[k][mask] = r[k]
    return res


def vdp_accuracy(forms, host, idx, threads):
    """Accuracy of each GPU form on the trajectories `idx` of the ring
    workload, against the FP64 oracle running the same method per trajectory
    (the GPU's `method` output) and the same tolerances.

    Gate (the metric's bar is a weighted error <= 10 against the FP64 oracle):
      * >= 95 % of the sample within the bar, and lockstep -- the
        oracle's accepted and rejected step counts -- on >= 95 %;
      * the rest are trajectories of a sensitive relaxation oscillation
        whose fast jumps moved (another step sequence, or the same one with
        rounding amplified at a jump), where the oracle's own error against a
        reltol-1e-10 truth reaches ~1e5 x tolerance: their error against
        that truth must stay within the oracle's own, quantile by quantile
        (p50 / p90 <= 2 x the oracle's + 1)."""
    import oracle
    p, u0, t0, tf = [a[idx] for a in host[:4]]
    saveat = host[4]
    stiff = forms[next(iter(forms))]["method"][idx] == oracle.ALG_RODAS5
    ref = oracle_vdp(p, u0, t0, tf, saveat, stiff, threads)
    truth = oracle_vdp(p, u0, t0, tf, saveat, stiff, threads, rtol=1e-10,
                       alg_all=oracle.ALG_RODAS5)["u"]

    def w(u, r):
        return oracle.weighted_errors(u, r, VDP_RTOL, VDP_RTOL).max(axis=(1, 2))

    def q(e):
        if e.size == 0:
            return None
        return {"p50": float(np.median(e)), "p90": float(np.percentile(e, 90)),
                "p99": float(np.percentile(e, 99)), "max": float(e.max()), "n": int(e.size)}

    e_ot = w(ref["u"], truth)
    att = ref["naccept"] + ref["nreject"]
    out = {"sample": int(len(idx)), "stiff_in_sample": int(stiff.sum()),
           "fp64_oracle_vs_truth": q(e_ot),
           "oracle_stiff_attempts_mean": float(att[stiff].mean()) if stiff.any() else 0.0}
    ok = True
    for name, r in forms.items():
        u = np.asarray(r["u"][idx], np.float64)
        lock = (r["naccept"][idx] == ref["naccept"]) & (r["nreject"][idx] == ref["nreject"])
        e_o, e_t = w(u, ref["u"]), w(u, truth)
        off = e_o > 10.0
        gate_lock = bool(lock.mean() >= 0.95 and (~off).mean() >= 0.95)
        gate_off = True
        if off.any():
            for pc in (50, 90):
                gate_off &= bool(np.percentile(e_t[off], pc) <= 2.0 * np.percentile(e_ot[off], pc) + 1.0)
        d = {"max": float(e_o.max()), "p99": float(np.percentile(e_o, 99)),
             "p50": float(np.median(e_o)), "lockstep_frac": float(lock.mean()),
             "lockstep_max": float(e_o[lock].max()) if lock.any() else None,
             "lockstep_stiff_frac": float(lock[stiff].mean()) if stiff.any() else None,
             "within_bar_frac": float((~off).mean()),
             "off_lockstep_vs_oracle": q(e_o[~lock]),
             "beyond_bar_vs_truth": q(e_t[off]), "beyond_bar_oracle_vs_truth": q(e_ot[off]),
             "retcodes_success": bool(np.all(r["retcode"] == oracle.RET_SUCCESS)),
             "gate": bool(gate_lock and gate_off)}
        ok &= d["gate"] and d["retcodes_success"]
        out[name] = d
    out["bar"] = ("weighted error <= 10 vs the FP64 oracle on >= 95 % of the sample and "
                  "lockstep on >= 95 %; beyond the bar (moved relaxation jumps): error vs a "
                  "reltol-1e-10 truth within 2 x the oracle's own + 1 at p50 and p90")
    return out, ok


def event_times(fn, stream, K, W, flush, world=1):
    """W untimed calls, then K calls each bracketed by CUDA events on
    `stream` (the stream the library launches on), with the L2 flushed
    (a 256 MB write) and the device synchronised before each; ms per call."""
    import torch
    import torch.distributed as dist
    for _ in range(W):
        fn()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ts = []
    for _ in range(K):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    if world > 1:
        dist.barrier()
    return ts


def spread(ts):
    return {"min": float(np.min(ts)), "median": float(np.median(ts)), "max": float(np.max(ts))}


VDP_FORMS = {  # name: (precision, batching, output dtype)
    "plain": ("PREC_FP64", "BATCH_PLAIN", "f64"),
    "persistent": ("PREC_FP64", "BATCH_PERSISTENT", "f64"),
    "persistent-mixed": ("PREC_MIXED", "BATCH_PERSISTENT", "f32"),
    "persistent-f32x2": ("PREC_F32X2", "BATCH_PERSISTENT", "f32"),
}


def run_vdp(args, de):
    """The 16-state ring, 1M trajectories, AUTO (Tsit5 if mu <= VDP_STIFF_MU, else
    Rodas5): chosen form vs the plain FP64 launch, both gated against the
    FP64 oracle before timing."""
    import torch
    import torch.distributed as dist
    import oracle
    capi = de._capi
    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    chosen = args.chosen or "persistent-f32x2"
    if chosen not in VDP_FORMS:
        raise SystemExit("bench: unknown vdp_auto form %r" % chosen)
    N = args.trajectories
    # weak scaling: every rank solves its own N trajectories (rank-shifted seed)
    host = vdp_inputs(N, SEED + 7919 * rank)
    pinned = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in host]
    hp = [t.numpy() for t in pinned]
    dptr = [t.to(dev) for t in pinned]
    M = de.models.vdp_ring8
    stream = torch.cuda.current_stream(dev)
    ctx = capi.context(local)
    peak64, peak32 = ctx.fma_peak(0), ctx.fma_peak(1)
    threads = oracle.hardware_threads()

    def opts(form, alg=None):
        prec, batch, _ = VDP_FORMS[form]
        o = capi.opts_default(alg or capi.ALG_AUTO)
        o.reltol = o.abstol = VDP_RTOL
        o.stiff_threshold = VDP_STIFF_MU
        o.maxiters = 10 ** 6
        o.precision = getattr(capi, prec)
        o.batching = getattr(capi, batch)
        return o

    def odt(form):
        return VDP_FORMS[form][2]

    # ---- correctness of both forms against the FP64 oracle, before timing
    res = {}
    for form in ("plain", chosen):
        r = de.solve_arrays(M, opts(form), *dptr, capi.SAVE_GRID, u_dtype=odt(form))
        torch.cuda.synchronize()
        res[form] = {k: r[k].cpu().numpy() for k in ("u", "naccept", "nreject", "retcode",
                                                     "method")}
        if not np.all(res[form]["retcode"] == capi.RET_SUCCESS):
            raise SystemExit("bench: %s form did not solve every trajectory" % form)
    acc = None
    if rank == 0:
        idx = np.sort(np.random.default_rng(1).choice(N, min(N, 2000), replace=False))
        acc, ok = vdp_accuracy(res, host, idx, threads)
        if not ok:
            print(json.dumps({"error": "accuracy gate failed", "accuracy": acc}))
            raise SystemExit("bench: accuracy gate failed")
    method = res[chosen]["method"]
    st_idx = np.nonzero(method == capi.ALG_RODAS5)[0]
    ns_idx = np.nonzero(method == capi.ALG_TSIT5)[0]
    del res

    # ---- timing
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    S = len(host[4])

    def dev_outs(form):
        return {"u": torch.empty((N, S, 16), device=dev,
                                 dtype=torch.float32 if odt(form) == "f32" else torch.float64),
                "retcode": torch.empty(N, dtype=torch.int32, device=dev)}

    outs = {f: dev_outs(f) for f in ("plain", chosen)}
    host_out = {"u": torch.empty((N, S, 16), dtype=torch.float32 if odt(chosen) == "f32"
                                 else torch.float64).pin_memory().numpy(),
                "retcode": torch.empty(N, dtype=torch.int32).pin_memory().numpy()}
    # the dominant kernel alone: the stiff trajectories' Rodas5
    st_prec = capi.PREC_FP64 if VDP_FORMS[chosen][0] == "PREC_FP64" else capi.PREC_F32X2
    o_st = opts(chosen, capi.ALG_RODAS5)
    o_st.precision = st_prec
    dst = [t[torch.from_numpy(st_idx).to(dev)].contiguous() for t in dptr[:4]] + [dptr[4]]
    st_out = {"u": torch.empty((len(st_idx), S, 16), device=dev, dtype=outs[chosen]["u"].dtype),
              "retcode": torch.empty(len(st_idx), dtype=torch.int32, device=dev)}
    # and the non-stiff trajectories' Tsit5, in the chosen form's precision
    o_ns = opts(chosen, capi.ALG_TSIT5)
    dns = [t[torch.from_numpy(ns_idx).to(dev)].contiguous() for t in dptr[:4]] + [dptr[4]]
    ns_out = {"u": torch.empty((len(ns_idx), S, 16), device=dev, dtype=outs[chosen]["u"].dtype),
              "retcode": torch.empty(len(ns_idx), dtype=torch.int32, device=dev)}
    K, W = args.steps, args.warmup
    with ClockSampler(local) as clk:
        chosen_ts = event_times(lambda: de.solve_arrays(M, opts(chosen), *dptr, capi.SAVE_GRID,
                                                        u_dtype=odt(chosen), out=outs[chosen]),
                                stream, K, W, flush, world)
        # the plain form and the stiff kernel alone: at most 5 timed steps
        # each (the plain form takes ~3 s per step)
        plain_ts = event_times(lambda: de.solve_arrays(M, opts("plain"), *dptr, capi.SAVE_GRID,
                                                       u_dtype=odt("plain"), out=outs["plain"]),
                               stream, min(K, 5), min(W, 3), flush, world)
        stiff_ts = event_times(lambda: de.solve_arrays(M, o_st, *dst, capi.SAVE_GRID,
                                                       u_dtype=odt(chosen), out=st_out),
                               stream, min(K, 5), 1, flush, world)
        nonstiff_ts = event_times(lambda: de.solve_arrays(M, o_ns, *dns, capi.SAVE_GRID,
                                                          u_dtype=odt(chosen), out=ns_out),
                                  stream, min(K, 5), 1, flush, world)
        # end to end through the C ABI: pinned host inputs and outputs, the
        # copies inside the timed region
        for _ in range(W):
            de.solve_arrays(M, opts(chosen), *hp, capi.SAVE_GRID, u_dtype=odt(chosen),
                            out=host_out)
        if world > 1:
            dist.barrier()
        e2e_ts, e2e_call = [], []
        for _ in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            r = de.solve_arrays(M, opts(chosen), *hp, capi.SAVE_GRID, u_dtype=odt(chosen),
                                out=host_out)
            e2e_ts.append((time.perf_counter() - t) * 1e3)
            e2e_call.append((r["total_ms"], r["device_ms"]))
        if world > 1:
            dist.barrier()
    if not np.all(host_out["retcode"] == capi.RET_SUCCESS):
        raise SystemExit("bench: the end-to-end solve did not solve every trajectory")

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    chosen_ms = max_over_ranks(float(np.median(chosen_ts)))
    plain_ms = max_over_ranks(float(np.median(plain_ts)))
    e2e_ms = max_over_ranks(float(np.median(e2e_ts)))
    stiff_ms = max_over_ranks(float(np.median(stiff_ts)))
    nonstiff_ms = max_over_ranks(float(np.median(nonstiff_ts)))
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    total = N * world
    # FP64 work of the dominant kernel, from the oracle's step counts on the
    # sample's stiff trajectories, scaled to this launch's stiff trajectories
    orc_steps = acc["oracle_stiff_attempts_mean"]
    flops = TEAM_RODAS_FP64_PER_ATTEMPT * orc_steps * len(st_idx)
    achieved = flops / (stiff_ms * 1e-3) / 1e12
    # the kernel's binding resource: instruction issue (one warp instruction per
    # cycle per SM sub-partition, 4 per SM) at the SM clock sampled in the run
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    clocks = clk.summary()
    sm_hz = (clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0) * 1e6
    issue_peak = 4.0 * n_sm * sm_hz / 1e12  # warp instructions per second, x 1e12
    issue_achieved = RING_STIFF_INST_PER_ATTEMPT * orc_steps * len(st_idx) / (stiff_ms * 1e-3) / 1e12
    ns_issue = RING_NONSTIFF_INST_PER_TRAJ * len(ns_idx) / (nonstiff_ms * 1e-3) / 1e12
    pairs_form = VDP_FORMS[chosen][0] == "PREC_F32X2"
    roof_nonstiff = {
        "bound": "issue", "kernel": "k_team8<TeamTsit5FF<VdpRing8>> (non-stiff trajectories)"
        if pairs_form else "the non-stiff Tsit5 team kernel (%s)" % VDP_FORMS[chosen][0],
        "achieved": ns_issue, "peak": issue_peak, "unit": "warp instructions/s x 1e12",
        "frac": ns_issue / issue_peak if pairs_form else None,
        "basis": "the kernel's warp instructions per trajectory (%d, ncu smsp__inst_executed.sum "
                 "at 400,000 trajectories) x this launch's non-stiff trajectories, over the "
                 "kernel's time on them alone (CUDA events, median); peak as above"
                 % RING_NONSTIFF_INST_PER_TRAJ,
        "kernel_ms": nonstiff_ms, "nonstiff_trajectories": int(len(ns_idx)),
        "share_of_step": nonstiff_ms / chosen_ms,
        "traffic": RING_NONSTIFF_TRAFFIC_PER_TRAJ * len(ns_idx) if pairs_form else None,
        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                          "k_team8<TeamTsit5FF> at 400,000 trajectories (277,783 non-stiff), per "
                          "trajectory x this launch's"}
    cpu = None
    if not args.no_cpu_baseline:
        nc = args.cpu_sample or 50000
        ch = vdp_inputs(nc, SEED + 1)
        t = time.perf_counter()
        oracle_vdp(*ch, ch[0][:, 0] > VDP_STIFF_MU, threads)
        dtc = time.perf_counter() - t
        cpu = {"value": nc / dtc, "unit": "trajectories/s", "cores": threads, "kind": "port",
               "sample": "%d trajectories of the workload (another seed) in %.2f s: the C++ "
                         "FP64 restatement, Tsit5 / Rodas5 per trajectory, std::thread pool "
                         "over all host cores (EnsembleThreads-equivalent)" % (nc, dtc)}
    h2d = sum(a.nbytes for a in hp)
    d2h = host_out["u"].nbytes + host_out["retcode"].nbytes
    line = {
        "metric": "trajectories/sec at <=10x reltol error vs FP64 oracle; chosen form vs plain",
        "value": total / (chosen_ms * 1e-3), "unit": "trajectories/s", "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": chosen_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"persistent-f32x2": "f32x2-state/f32-lu-refined",
                  "persistent-mixed": "f32-state/f32-lu-refined"}.get(chosen, "f64"),
        "data": "synthetic (seeded, the configuration's distributions)",
        "config": {"workload": "vdp_ring8_auto_N%d" % N, "model": "ring of 8 Van der Pol "
                   "oscillators (16 states), kappa 0.05, mu = 10^U(-1,3), u0 ~ U[-2,2]^16",
                   "tspan": [0.0, 20.0], "reltol": VDP_RTOL, "abstol": VDP_RTOL,
                   "saveat": "0:1:20 (21 points)", "trajectories": N,
                   "alg": "AUTO: Tsit5 if mu <= %g, else Rodas5" % VDP_STIFF_MU,
                   "chosen_form": chosen,
                   "l2": "flushed between timed steps (256 MB write); output 1.34 GB > L2",
                   "parallelism": "trajectory shards, no collective" if world > 1
                   else "single GPU"},
        "chosen_form": {"persistent-f32x2": "persistent queue; Tsit5 and Rodas5 on 8-lane teams "
                        "in FP32 pairs (paired FP32 instructions); Rodas5's W in pairs, its LU "
                        "and W^-1 in FP32, each stage solve refined once against W in pairs; "
                        "FP64 time; FP32 output",
                        "persistent-mixed": "persistent queue; Tsit5 FP32 compensated state, "
                        "Rodas5 as in persistent-f32x2; FP32 output",
                        "persistent": "persistent queue, FP64", "plain": "one launch, FP64"}[chosen],
        "plain": {"value": total / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                  "error_vs_oracle": acc["plain"]},
        "speedup_vs_plain": plain_ms / chosen_ms,
        "error_vs_oracle": acc[chosen],
        "accuracy": acc,
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "trajectories/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "call_total_ms": float(np.median([c[0] for c in e2e_call])),
                "call_device_ms": float(np.median([c[1] for c in e2e_call])),
                "path": "gbde_ensemble_solve with GBDE_MEM_HOST: pinned inputs copied to the "
                        "device; the saves stored by the kernels straight into the pinned host "
                        "output over the host link while they run (no staging copy)"},
        "roofline": {"bound": "issue", "kernel": "k_team8<TeamRodasFF8<VdpRing8,Rodas5>> (stiff "
                     "trajectories)" if st_prec == capi.PREC_F32X2 else
                     "k_team<TeamRodas<VdpRing8,double,Rodas5>> (stiff trajectories)",
                     "achieved": issue_achieved, "peak": issue_peak,
                     "unit": "warp instructions/s x 1e12", "frac": issue_achieved / issue_peak,
                     "basis": "the kernel's warp instructions per trajectory and attempted step "
                              "(%d, ncu smsp__inst_executed.sum at 400,000 trajectories) x the "
                              "oracle's attempted steps x this launch's stiff trajectories, over "
                              "the kernel's time on them alone (CUDA events, median); peak: one "
                              "warp instruction per cycle per SM sub-partition, 4 x %d SMs at "
                              "the sampled SM clock" % (RING_STIFF_INST_PER_ATTEMPT, n_sm),
                     "fp64_equivalent": {"achieved_tflops": achieved, "peak_tflops": peak64,
                                         "frac": achieved / peak64,
                                         "basis": "the %d FP64 flops per attempted step the "
                                                  "FP64 form executes (sparse LU of W, W's "
                                                  "diagonal, Jacobian rows, norm squares), now "
                                                  "done in FP32 / FP32 pairs"
                                                  % TEAM_RODAS_FP64_PER_ATTEMPT},
                     "kernel_ms": stiff_ms, "stiff_trajectories": int(len(st_idx)),
                     "share_of_step": stiff_ms / chosen_ms,
                     "fp32_peak_tflops": peak32,
                     "traffic": RING_STIFF_TRAFFIC_PER_TRAJ * len(st_idx)
                     if st_prec == capi.PREC_F32X2 else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                       "k_team8<TeamRodasFF8> at 400,000 trajectories (122,217 "
                                       "stiff), per stiff trajectory x this launch's"},
        "gpu_launches": K * 3,
        "clocks": clocks,
        "step_ms_spread": {"chosen": spread(chosen_ts), "plain": spread(plain_ts),
                           "e2e": spread(e2e_ts), "stiff_kernel": spread(stiff_ts),
                           "nonstiff_kernel": spread(nonstiff_ts)},
        "cpu_baseline": cpu,
    }
    # `roofline` describes the kernel with the larger share of the step
    roof_stiff = line["roofline"]
    if nonstiff_ms > stiff_ms:
        line["roofline"], line["roofline_other"] = roof_nonstiff, roof_stiff
    else:
        line["roofline_other"] = roof_nonstiff
    if cpu:
        line["north_star"] = {
            "plain_vs_cpu": line["plain"]["value"] / cpu["value"],
            "chosen_vs_cpu": line["value"] / cpu["value"],
            "e2e_vs_cpu": line["e2e"]["value"] / cpu["value"],
            "chosen_vs_plain": line["speedup_vs_plain"],
            "targets": "plain >= 50x the CPU run; chosen >= 2x plain",
            "note": "GB300's FP64 pipe (about 1.25 TFLOP/s measured) is within a small factor "
                    "of 16 Grace cores' vector FP64, so an FP64-only GPU path cannot reach 50x a "
                    "well-used 16-core CPU; the FP32-pair forms carry the speed-up"}
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------- other configurations
# Each returns the inputs and the forms compared: (model, p, u0, t0, tf, saveat,
# save_kind, plain_opts, chosen_opts, out dtypes, config dict, error kind).
def other_workload(de, name, N, seed):
    capi = de._capi
    rng = np.random.default_rng(seed)

    def opts(alg, **kw):
        o = capi.opts_default(alg)
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    if name == "lorenz":
        p = np.array([10.0, 28.0, 8.0 / 3.0]) * rng.uniform(0.9, 1.1, (N, 3))
        u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
        t0, tf = np.zeros(N), np.ones(N)
        saveat = de.save_grid(0.0, 1.0, 0.1)
        base = dict(reltol=1e-8, abstol=1e-8)
        plain = opts(capi.ALG_TSIT5, **base)
        chosen = opts(capi.ALG_TSIT5, precision=capi.PREC_F32X2, **base)
        cfg = {"workload": "lorenz_tsit5_N%d" % N, "model": "lorenz", "alg": "tsit5",
               "reltol": 1e-8, "abstol": 1e-8, "saveat": "0:0.1:1 (11 points)",
               "chosen_form": "one launch, FP32-pair Tsit5 stepper (FP64 norm accumulation "
                              "and time)"}
        return (de.models.lorenz, p, u0, t0, tf, saveat, capi.SAVE_GRID, plain, chosen,
                ("f64", "f64"), cfg, "weighted")
    if name in ("lv_em", "lv_sosri"):
        p = np.c_[np.array([1.5, 1.0, 3.0, 1.0]) * rng.uniform(0.8, 1.2, (N, 4)), np.full(N, 0.1)]
        u0 = np.ones((N, 2))
        t0, tf = np.zeros(N), np.full(N, 10.0)
        saveat = de.save_grid(0.0, 10.0, 1.0)
        if name == "lv_em":
            base = dict(dt=1e-3, seed=SEED)
            plain = opts(capi.ALG_EM, **base)
            chosen = opts(capi.ALG_EM, precision=capi.PREC_MIXED, **base)
            cfg = {"workload": "lotka_volterra_em_N%d" % N, "alg": "em", "dt": 1e-3,
                   "chosen_form": "FP32 state, FP64 time, FP32 noise stream"}
        else:
            base = dict(reltol=1e-3, abstol=1e-3, seed=SEED)
            plain = opts(capi.ALG_SOSRI, **base)
            chosen = opts(capi.ALG_SOSRI, precision=capi.PREC_MIXED,
                          batching=capi.BATCH_PERSISTENT, **base)
            cfg = {"workload": "lotka_volterra_sosri_N%d" % N, "alg": "sosri (RSwM rejection)",
                   "reltol": 1e-3, "abstol": 1e-3,
                   "chosen_form": "persistent, FP32 state, FP64 time"}
        cfg.update({"model": "lotka_volterra", "noise": "diagonal 0.1 u",
                    "saveat": "0:1:10 (11 points)"})
        return (de.models.lotka_volterra, p, u0, t0, tf, saveat, capi.SAVE_GRID, plain, chosen,
                ("f64", "f32"), cfg, "sde")
    if name == "vdp_auto":
        p = np.c_[10 ** rng.uniform(-1, 3, N), np.full(N, 0.05)]
        u0 = rng.uniform(-2, 2, (N, 16))
        t0, tf = np.zeros(N), np.full(N, 20.0)
        saveat = de.save_grid(0.0, 20.0, 1.0)
        base = dict(reltol=1e-5, abstol=1e-5, stiff_threshold=VDP_STIFF_MU, maxiters=10 ** 6)
        plain = opts(capi.ALG_AUTO, **base)
        chosen = opts(capi.ALG_AUTO, precision=capi.PREC_F32X2, batching=capi.BATCH_PERSISTENT,
                      **base)
        cfg = {"workload": "vdp_ring8_auto_N%d" % N, "model": "vdp_ring8 (16 states)",
               "alg": "auto: tsit5 if mu <= %g else rodas5" % VDP_STIFF_MU, "reltol": 1e-5,
               "saveat": "0:1:20 (21 points)",
               "chosen_form": "persistent; Tsit5 and Rodas5 on 8-lane teams in FP32 pairs; "
                              "Rodas5's LU and W^-1 in FP32 with pair-refined solves"}
        return (de.models.vdp_ring8, p, u0, t0, tf, saveat, capi.SAVE_GRID, plain, chosen,
                ("f64", "f32"), cfg, "vdp")
    raise ValueError(name)


def run_other(args, de):
    import torch
    import oracle
    capi = de._capi
    N = args.trajectories
    (model, p, u0, t0, tf, saveat, kind, plain, chosen, dts, cfg, ekind) = other_workload(
        de, args.workload, N, SEED)
    dev = torch.device("cuda", 0)
    host = [np.ascontiguousarray(a) for a in (p, u0, t0, tf, saveat)]
    dptr = [torch.from_numpy(a).to(dev) for a in host]
    ctx = capi.context(0)
    peak64, peak32 = ctx.fma_peak(0), ctx.fma_peak(1)
    # the SDE kernels' bound: the FP32 normal stream (Philox + Box-Muller)
    normal_peak = ctx.fma_peak(2) * 1e12 if ekind == "sde" else None
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def timed(o, dt, K, W, **kw):
        for _ in range(W):
            de.solve_arrays(model, o, *dptr, kind, u_dtype=dt, **kw)
        ts, r = [], None
        for _ in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            r = de.solve_arrays(model, o, *dptr, kind, u_dtype=dt, **kw)
            ts.append(r["device_ms"])
        return float(np.median(ts)), r

    reduce_ms = None
    with ClockSampler(0) as clk:
        plain_ms, rp = timed(plain, dts[0], args.steps, args.warmup)
        chosen_ms, rc = timed(chosen, dts[1], args.steps, args.warmup)
        if ekind == "sde":
            # the chosen form reducing in the kernel (E[u], Var[u] per save
            # point) without storing the paths
            reduce_ms, _ = timed(chosen, dts[1], args.steps, args.warmup, reduce=True,
                                 store_u=False)
    res = {k: {kk: (v.cpu().numpy() if v is not None else None) for kk, v in r.items()
               if kk in ("u", "retcode", "naccept", "nreject")}
           for k, r in (("plain", rp), ("chosen", rc))}
    # accuracy on a sample against the FP64 oracle (same algorithm, same inputs)
    rng = np.random.default_rng(1)
    ns = min(N, 512 if ekind == "vdp" else 2000)
    # SDE noise is keyed by the trajectory index: compare the leading block
    idx = np.arange(ns) if ekind == "sde" else np.sort(rng.choice(N, ns, replace=False))
    sub = [a[idx] for a in host[:4]]
    acc = {}
    if ekind == "weighted":
        ref = oracle.solve(capi, model, plain, *sub, saveat, kind, nthreads=oracle.hardware_threads())
        for f in ("plain", "chosen"):
            acc[f] = oracle.weighted_error(res[f]["u"][idx], ref["u"], plain.abstol, plain.reltol)
    elif ekind == "sde":
        ref64 = oracle.solve(capi, model, plain, *sub, saveat, kind,
                             nthreads=oracle.hardware_threads())
        ref32 = oracle.solve(capi, model, plain, *sub, saveat, kind,
                             nthreads=oracle.hardware_threads(), noise_f32=True)
        rel = lambda u, r: float(np.max(np.abs(u - r) / np.abs(r)))
        if plain.alg == capi.ALG_EM:
            acc = {"plain_fp64_vs_oracle_identical_noise_rel": rel(res["plain"]["u"][idx], ref64["u"]),
                   "chosen_fp32_vs_fp64_oracle_same_fp32_noise_rel":
                       rel(res["chosen"]["u"][idx].astype(np.float64), ref32["u"])}
        else:
            w = lambda u, r: (np.abs(u - r) / (plain.abstol + plain.reltol * np.abs(r))).max(axis=(1, 2))
            acc = {"plain_identical_path_fraction": float(np.mean(w(res["plain"]["u"][idx], ref64["u"]) <= 1e-6)),
                   "chosen_weighted_median": float(np.median(w(res["chosen"]["u"][idx].astype(np.float64), ref32["u"])))}
    else:  # vdp: per-partition FP64 oracle and a reltol-1e-10 truth
        st = sub[0][:, 0] > plain.stiff_threshold
        ref = np.empty((ns, len(saveat), 16))
        for mask, alg in ((~st, capi.ALG_TSIT5), (st, capi.ALG_RODAS5)):
            if mask.any():
                o = capi.opts_default(alg)
                o.reltol, o.abstol, o.maxiters = plain.reltol, plain.abstol, plain.maxiters
                ref[mask] = oracle.solve(capi, model, o, *[a[mask] for a in sub], saveat, kind,
                                         nthreads=oracle.hardware_threads())["u"]
        o = capi.opts_default(capi.ALG_RODAS5)
        o.reltol = o.abstol = 1e-10
        o.maxiters = 10 ** 7
        truth = oracle.solve(capi, model, o, *sub, saveat, kind, nthreads=oracle.hardware_threads())["u"]
        w = lambda u, r: (np.abs(np.asarray(u, np.float64) - r) / (1e-5 + 1e-5 * np.abs(r))).max(axis=(1, 2))
        for f in ("plain", "chosen"):
            e_o, e_t = w(res[f]["u"][idx], ref), w(res[f]["u"][idx], truth)
            acc[f] = {"vs_oracle_p50": float(np.median(e_o)), "vs_oracle_p90": float(np.percentile(e_o, 90)),
                      "vs_truth_p50": float(np.median(e_t)), "vs_truth_p90": float(np.percentile(e_t, 90))}
        e_ot = w(ref, truth)
        acc["fp64_oracle_vs_truth"] = {"p50": float(np.median(e_ot)), "p90": float(np.percentile(e_ot, 90))}
    # CPU baseline: the oracle on a bounded sample, all host threads
    cpu = None
    if not args.no_cpu_baseline:
        threads = oracle.hardware_threads()
        # a sample of the same distribution sized for ~0.2-2 s on 16 cores
        nc = {"lorenz": 200000, "lv_em": 8000, "lv_sosri": 40000, "vdp_auto": 8000}[args.workload]
        big = other_workload(de, args.workload, nc, SEED + 1)
        sub = [np.ascontiguousarray(a) for a in big[1:5]]
        t = time.perf_counter()
        if ekind == "vdp":
            st = sub[0][:, 0] > plain.stiff_threshold
            for mask, alg in ((~st, capi.ALG_TSIT5), (st, capi.ALG_RODAS5)):
                o = capi.opts_default(alg)
                o.reltol, o.abstol, o.maxiters = plain.reltol, plain.abstol, plain.maxiters
                oracle.solve(capi, model, o, *[a[mask] for a in sub], saveat, kind, nthreads=threads)
        else:
            oracle.solve(capi, model, plain, *sub, saveat, kind, nthreads=threads)
        dtc = time.perf_counter() - t
        cpu = {"value": nc / dtc, "unit": "trajectories/s", "cores": threads, "kind": "port",
               "sample": "%d trajectories in %.2f s (C++ FP64 restatement, std::thread pool)" % (nc, dtc)}
    line = {"metric": "trajectories/sec at <=10x reltol error vs FP64 oracle",
            "value": N / (chosen_ms * 1e-3), "unit": "trajectories/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": chosen_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded, config distributions)",
            "config": dict(cfg, trajectories=N, l2="flushed between timed steps (256 MB write)"),
            "plain": {"value": N / (plain_ms * 1e-3), "ms_per_step": plain_ms},
            "speedup_vs_plain": plain_ms / chosen_ms, "accuracy": acc,
            "chosen_reduce_only_ms": reduce_ms,
            "steps_per_traj_mean": float((res["chosen"]["naccept"] + res["chosen"]["nreject"]).mean()),
            "all_success": bool(np.all(res["chosen"]["retcode"] == capi.RET_SUCCESS)),
            "fp64_peak_tflops": peak64, "fp32_peak_tflops": peak32,
            "clocks": clk.summary(), "cpu_baseline": cpu}
    if args.workload == "lv_em":
        # EM draws one normal per state component per step: exact count
        normals = float(res["chosen"]["naccept"].astype(np.float64).sum()) * 2.0
        achieved = normals / (chosen_ms * 1e-3)
        line["roofline"] = {"bound": "FP32 normal stream (Philox4x32-10 on the integer pipe, "
                                     "Box-Muller on the MUFU pipe)",
                            "achieved": achieved, "peak": normal_peak, "unit": "normals/s",
                            "frac": achieved / normal_peak,
                            "peak_source": "in-run normal-stream microbenchmark "
                                           "(gbde_measure_fma_peak kind 2)",
                            "traffic": None}
    print(json.dumps(line))


def run_learned(args, de):
    """Learned predictor (configuration 5): train from scratch on step logs
    of the plain solver, then time learned vs plain on held-out trajectories."""
    import torch
    import oracle
    capi = de._capi
    base = {"learned_lorenz": "lorenz", "learned_lv": "lv_sosri", "learned_vdp": "vdp_auto"}[
        args.workload]
    n_train = 1000000 if base == "vdp_auto" else 2000000
    N = args.trajectories
    tr = other_workload(de, base, n_train, SEED + 1000)
    model, saveat, kind, plain = tr[0], tr[5], tr[6], tr[7]
    t = time.perf_counter()
    # step logs of the plain solver (persistent launch)
    log_opts = other_workload(de, base, 1, 0)[8]
    dev = torch.device("cuda", 0)
    dtr = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in tr[1:6]]
    odt = tr[9][1]
    r = de.solve_arrays(model, log_opts, *dtr, kind, u_dtype=odt)
    dt1 = r["dt_first"].cpu().numpy()
    if base == "vdp_auto":
        lab, cost = de.learned.stiff_labels(de.solve_arrays, model, *dtr[:5], kind, plain.reltol,
                                            plain.abstol, precision=log_opts.precision)
    else:
        lab, cost = np.zeros(n_train, np.float32), None
    x = de.learned.features(model, *tr[1:5])
    y = np.c_[np.log10(dt1), lab,
              de.learned.cost_targets(r["naccept"], r["nreject"])].astype(np.float32)
    logs_s = time.perf_counter() - t
    t = time.perf_counter()
    net, hist = de.learned.train(x, y, epochs=8, batch=4096, lr=2e-3, seed=SEED)
    train_s = time.perf_counter() - t
    de.learned.load(model, net)
    # held-out evaluation
    ev = other_workload(de, base, N, SEED + 2000)
    host = [np.ascontiguousarray(a) for a in ev[1:6]]
    dptr = [torch.from_numpy(a).to(dev) for a in host]
    chosen = ev[8]
    learned = ev[8]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def timed(o, K, W):
        for _ in range(W):
            de.solve_arrays(model, o, *dptr, kind, u_dtype=odt)
        ts, rr = [], None
        for _ in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            rr = de.solve_arrays(model, o, *dptr, kind, u_dtype=odt)
            ts.append(rr["device_ms"])
        return float(np.median(ts)), rr

    # the ring: the learned stiffness choice alone (GBDE_LEARN_STIFF, the
    # Hairer-Wanner start as the oracle), so the gate sees the choice's effect;
    # Lorenz / LV: the learned first dt (GBDE_LEARN_START)
    flag = capi.LEARN_STIFF if base == "vdp_auto" else capi.LEARN_START
    with ClockSampler(0) as clk:
        chosen.learned = 0
        base_ms, rb = timed(chosen, args.steps, args.warmup)
        learned.learned = flag
        learned_ms, rl = timed(learned, args.steps, args.warmup)
        learned.learned = 0
    ok = bool(np.all(rl["retcode"].cpu().numpy() == capi.RET_SUCCESS))
    gate = None
    if base == "vdp_auto":
        # the default line's gate, for each solve on its own methods
        to_np = lambda rr: {k: rr[k].cpu().numpy() for k in
                            ("u", "method", "naccept", "nreject", "retcode")}
        gidx = np.sort(np.random.default_rng(3).choice(N, min(N, 2000), replace=False))
        threads = oracle.hardware_threads()
        acc_l, ok_l = vdp_accuracy({"learned": to_np(rl)}, host, gidx, threads)
        acc_b, ok_b = vdp_accuracy({"without": to_np(rb)}, host, gidx, threads)
        gate = {"learned": acc_l["learned"], "without": acc_b["without"],
                "stiff_in_sample": {"learned": acc_l["stiff_in_sample"],
                                    "without": acc_b["stiff_in_sample"]},
                "bar": acc_l["bar"], "gate": bool(ok_l and ok_b)}
    # accuracy of the learned solve on a sample against the FP64 oracle
    ns = min(N, 512 if base == "vdp_auto" else 2000)
    idx = np.arange(ns)  # leading block (SDE noise is keyed by trajectory index)
    u_l = rl["u"].cpu().numpy()[idx].astype(np.float64)
    u_b = rb["u"].cpu().numpy()[idx].astype(np.float64)
    if base == "vdp_auto":
        # each solve against the FP64 oracle running the method that solve
        # used for each trajectory (its outputs.method)
        def ref_of(rr):
            meth = rr["method"].cpu().numpy()[idx]
            ref = np.empty_like(u_l)
            for alg in (capi.ALG_TSIT5, capi.ALG_RODAS5):
                mask = meth == alg
                if mask.any():
                    o = capi.opts_default(alg)
                    o.reltol, o.abstol, o.maxiters = chosen.reltol, chosen.abstol, chosen.maxiters
                    ref[mask] = oracle.solve(capi, model, o, *[a[idx][mask] for a in host[:4]],
                                             host[4], kind, nthreads=oracle.hardware_threads())["u"]
            return ref
        ref_l, ref_b = ref_of(rl), ref_of(rb)
    else:
        ref_l = ref_b = oracle.solve(capi, model, plain, *[a[idx] for a in host[:4]], host[4], kind,
                                     nthreads=oracle.hardware_threads(),
                                     noise_f32=(base == "lv_sosri"))["u"]
    w = lambda u, ref: (np.abs(u - ref) / (chosen.abstol + chosen.reltol * np.abs(ref))).max(
        axis=(1, 2))
    pred_dt, pred_st, _ = de.learned.predict(net, de.learned.features(model, *host[:4]))
    st_l = rl["naccept"] + rl["nreject"]
    st_b = rb["naccept"] + rb["nreject"]
    line = {"metric": "trajectories/sec at <=10x reltol error vs FP64 oracle; learned vs plain",
            "value": N / (learned_ms * 1e-3), "unit": "trajectories/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": learned_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded, config distributions); held-out seed",
            "config": {"workload": "learned_" + base + "_N%d" % N, "train_pairs": n_train,
                       "net": "8-64-64-64-3 GELU, BF16 weights, FP32 accumulation",
                       "train": "8 epochs, batch 4096, AdamW lr 2e-3 (GPU, own kernels)",
                       "form": "same launch (%s) with and without learned=1" % (
                           "persistent" if chosen.batching else "plain")},
            "without_learned": {"value": N / (base_ms * 1e-3), "ms_per_step": base_ms},
            "speedup_vs_without": base_ms / learned_ms,
            "all_success": ok,
            "steps_per_traj": {"learned": float(st_l.float().mean()), "without": float(st_b.float().mean())},
            "nf_per_traj": {"learned": float(rl["nf"].float().mean()), "without": float(rb["nf"].float().mean())},
            "accuracy_vs_fp64_oracle": {"learned_p50": float(np.median(w(u_l, ref_l))),
                                        "learned_max": float(w(u_l, ref_l).max()),
                                        "without_p50": float(np.median(w(u_b, ref_b))),
                                        "without_max": float(w(u_b, ref_b).max())},
            "first_dt_log10_abs_err_median": float(np.median(np.abs(
                np.log10(pred_dt[idx]) - np.log10(rb["dt_first"].cpu().numpy()[idx])))),
            "step_log_s": logs_s, "train_s": train_s, "loss_first_last": [float(hist[0]), float(hist[-1])],
            "stiff_cost_model": cost, "clocks": clk.summary()}
    if gate is not None:
        line["accuracy_gate"] = gate
        if not gate["gate"]:
            # a form outside the metric's bar does not count: the line's value
            # is then the form without the predictor
            line["learned_value_outside_bar"] = line["value"]
            line["value"] = line["without_learned"]["value"]
            line["ms_per_step"] = base_ms
            line["chosen"] = ("without the predictor: the learned form fails the accuracy gate "
                              "(see accuracy_gate)")
    print(json.dumps(line))


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) of the GB300s, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (measured)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def run_summary(args, de):
    """Ensemble statistics on the device: mean, variance and the 5 / 50 / 95 %
    quantiles per save point and component of a 1M x 21 x 16 FP32 ensemble
    output (the 16-state ring's output size; seeded normal values), against
    copying that output to the host and computing the same with numpy."""
    import torch
    capi = de._capi
    N, ns, nst = args.trajectories, 21, 16
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(SEED)
    u = torch.randn((N, ns, nst), generator=g, device=dev, dtype=torch.float32)
    u.mul_(torch.linspace(0.1, 3.0, nst, device=dev)).add_(torch.linspace(-1, 1, ns, device=dev)[:, None])
    qs = (0.05, 0.5, 0.95)
    mean, var, qv = de.ensemble_summary(u, qs)  # correctness and warm-up
    ref_mean = u.double().mean(0)
    ok = bool(torch.allclose(mean, ref_mean, rtol=1e-9, atol=1e-9)) and bool(
        torch.equal(de.ensemble_summary(u, (0.0,))[2][0], u.amin(0).double()))
    if not ok:
        raise SystemExit("bench: device summary disagrees with torch's reductions")
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def timed(fn, K, W):
        for _ in range(W):
            fn()
        ts = []
        for _ in range(K):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts)), ts

    with ClockSampler(0) as clk:
        full_ms, full_ts = timed(lambda: de.ensemble_summary(u, qs), args.steps, args.warmup)
        mv_ms, _ = timed(lambda: de.ensemble_summary(u, ()), args.steps, args.warmup)
    # the alternative: copy the ensemble to pinned host memory, reduce with numpy
    host = torch.empty((N, ns, nst), dtype=torch.float32).pin_memory()
    t = time.perf_counter()
    host.copy_(u)
    torch.cuda.synchronize()
    d2h_ms = (time.perf_counter() - t) * 1e3
    hn = host.numpy()
    t = time.perf_counter()
    hn.mean(0)
    hn.var(0, ddof=1)
    np.quantile(hn, qs, axis=0)
    cpu_ms = (time.perf_counter() - t) * 1e3
    ubytes = N * ns * nst * 4
    peak, src = hbm_peak()
    achieved = ubytes / (mv_ms * 1e-3) / 1e9
    line = {"metric": "ensemble statistics: trajectories summarised per second",
            "value": N / (full_ms * 1e-3), "unit": "trajectories/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": full_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded normal values in the ring's output shape)",
            "config": {"workload": "summary_N%d_21x16_f32" % N, "quantiles": list(qs),
                       "l2": "flushed between timed steps (256 MB write)"},
            "mean_var_only_ms": mv_ms,
            "roofline": {"bound": "hbm", "kernel": "mean/var pass (k_sum)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": src,
                         "algorithmic_bytes": ubytes},
            "quantile_passes": "1 key transpose (read + write) + 4 digit passes over the keys",
            "alternative": {"d2h_ms": d2h_ms, "numpy_ms_1_thread": cpu_ms,
                            "what": "copy u to pinned host memory, numpy mean/var/quantile"},
            "speedup_vs_alternative": (d2h_ms + cpu_ms) / full_ms,
            "gpu_launches": args.steps * (2 + 1 + 1 + 4 * 3 + 1),
            "clocks": clk.summary(),
            "step_ms_spread": {"min": min(full_ts), "median": float(np.median(full_ts)),
                               "max": max(full_ts)}}
    print(json.dumps(line))


def run_reference(args):
    """--impl reference: the CPU FP64 restatement of the workload on the host
    cores, bounded samples per step; loads the oracle only, never the
    product library.  Under torchrun only rank 0 runs."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    threads = oracle.hardware_threads()
    if args.workload == "vdp_auto":
        sample = min(args.cpu_sample or 50000, args.trajectories)

        def one(n, seed):
            x = vdp_inputs(n, seed)
            t = time.perf_counter()
            oracle_vdp(*x, x[0][:, 0] > VDP_STIFF_MU, threads)
            dt = time.perf_counter() - t
            return n / dt, dt

        config = {"workload": "vdp_ring8_auto_N%d" % args.trajectories,
                  "model": "ring of 8 Van der Pol oscillators (16 states)",
                  "alg": "AUTO: Tsit5 if mu <= %g, else Rodas5" % VDP_STIFF_MU,
                  "reltol": VDP_RTOL, "abstol": VDP_RTOL, "saveat": "0:1:20 (21 points)",
                  "trajectories": args.trajectories}
        metric = "trajectories/sec at <=10x reltol error vs FP64 oracle; chosen form vs plain"
    elif args.workload == "robertson":
        sample = min(args.cpu_sample or 100000, args.trajectories)

        def one(n, seed):
            return oracle_robertson(args.alg, n, seed, threads)[:2]

        config = {"workload": "robertson_%s_fp64_N%d" % (args.alg, args.trajectories),
                  "model": "robertson", "alg": args.alg, "trajectories": args.trajectories,
                  "reltol": 1e-6, "abstol": 1e-10, "saveat": "20 log-spaced per trajectory",
                  "tf": "10^U(1,5)"}
        metric = "trajectories/sec at <=10x reltol error vs FP64 oracle"
    else:
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the "
                          "vdp_auto and robertson workloads"}))
        return
    for _ in range(max(0, args.warmup)):
        one(max(256, sample // 20), SEED)
    vals, secs = [], []
    for k in range(args.steps):
        v, dt = one(sample, SEED + k)
        vals.append(v)
        secs.append(dt)
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": metric, "value": value, "unit": "trajectories/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.median(secs) * 1e3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config,
            "cpu_baseline": {"value": value, "unit": "trajectories/s", "cores": threads,
                             "kind": "port",
                             "sample": "%d trajectories of the workload per step, median of %d "
                                       "steps (EnsembleThreads-equivalent C++ FP64 restatement, "
                                       "std::thread pool over all host cores)"
                                       % (sample, args.steps)},
            "e2e": {"value": value, "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import __graft_entry__
    de = __graft_entry__.load_package()
    if args.workload == "vdp_auto":
        return run_vdp(args, de)
    if args.workload.startswith("learned_"):
        return run_learned(args, de)
    if args.workload == "summary":
        return run_summary(args, de)
    if args.workload != "robertson":
        return run_other(args, de)
    return run_robertson(args, de)


def run_robertson(args, de):
    """The stiff Robertson ensemble (Rodas5 or Rosenbrock23, 100k)."""
    world, rank, local = dist_env()
    capi = de._capi
    if args.chosen is None:
        args.chosen = "persistent-f32x2-learned"
    alg_id = capi.ALG_RODAS5 if args.alg == "rodas5" else capi.ALG_ROSENBROCK23
    config = {"workload": "robertson_%s_fp64_N%d" % (args.alg, args.trajectories),
              "model": "robertson", "alg": args.alg, "trajectories": args.trajectories,
              "reltol": 1e-6, "abstol": 1e-10, "saveat": "20 log-spaced per trajectory",
              "tf": "10^U(1,5)"}
    metric = "trajectories/sec at <=10x reltol error vs FP64 oracle"

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    N = args.trajectories
    # weak scaling: every rank solves its own N trajectories (rank-shifted seed)
    p, u0, t0, tf, saveat = workload(N, SEED + 7919 * rank)
    host = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (p, u0, t0, tf, saveat)]
    dptr = [h.to(dev) for h in host]
    ctx = capi.context(local)
    peak64 = ctx.fma_peak(0)
    peak32 = ctx.fma_peak(1)

    forms = {"plain": ("plain", "fp64"), "persistent": ("persistent", "fp64"),
             "persistent-mixed": ("persistent", "mixed"), "plain-mixed": ("plain", "mixed"),
             "persistent-f32x2": ("persistent", "f32x2"), "plain-f32x2": ("plain", "f32x2"),
             "persistent-f32x2-learned": ("persistent", "f32x2", capi.LEARN_ORDER)}

    def opts_for(form):
        b, prec = forms[form][:2]
        o = capi.opts_default(alg_id)
        o.reltol, o.abstol = 1e-6, 1e-10
        o.batching = capi.BATCH_PERSISTENT if b == "persistent" else capi.BATCH_PLAIN
        o.precision = {"mixed": capi.PREC_MIXED, "f32x2": capi.PREC_F32X2}.get(prec, capi.PREC_FP64)
        o.learned = forms[form][2] if len(forms[form]) > 2 else 0
        return o

    solve_model = de.models.robertson
    if args.user_model != "none":
        # the same Robertson formulas (test/core.jl:39-45) as runtime-compiled user source
        solve_model = de.ODEFunction(
            "T r1 = p[0] * u[0]; T r2 = p[1] * u[1] * u[1]; T r3 = p[2] * u[1] * u[2];\n"
            "du[0] = -r1 + r3; du[1] = r1 - r2 - r3; du[2] = r2;", 3, 3,
            jac=None if args.user_model == "dual" else
            "J[0][0] = -p[0]; J[0][1] = p[2] * u[2]; J[0][2] = p[2] * u[1];\n"
            "J[1][0] = p[0]; J[1][1] = T(-2) * p[1] * u[1] - p[2] * u[2];\n"
            "J[1][2] = -p[2] * u[1]; J[2][0] = T(0); J[2][1] = T(2) * p[1] * u[1];\n"
            "J[2][2] = T(0);", name="robertson_user")
        if len(forms[args.chosen]) > 2:
            raise SystemExit("bench: user models run without the learned predictor; "
                             "pick --chosen persistent-f32x2")
    learn_info = None
    if len(forms[args.chosen]) > 2:
        # the learned queue order: train the cost head on the attempted-step
        # log of a solve of a separate training ensemble (another seed), on
        # the GPU with the library's kernels; untimed
        t_l = time.perf_counter()
        trp = workload(N, SEED + 104729 + 7919 * rank)
        trd = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in trp]
        o_log = opts_for(args.chosen)
        o_log.learned = 0
        rlog = de.solve_arrays(de.models.robertson, o_log, *trd, capi.SAVE_PER_TRAJ)
        x = de.learned.features(de.models.robertson, *trp[:4], device=local)
        y = np.c_[np.full(N, np.nan), np.full(N, np.nan),
                  de.learned.cost_targets(rlog["naccept"], rlog["nreject"])].astype(np.float32)
        t_t = time.perf_counter()
        net, hist = de.learned.train(x, y, epochs=20, batch=4096, lr=2e-3, seed=SEED, device=local)
        train_s = time.perf_counter() - t_t
        de.learned.load(de.models.robertson, net, device=local)
        learn_info = {"train_trajectories": N, "epochs": 20, "batch": 4096,
                      "train_s": train_s, "log_and_train_s": time.perf_counter() - t_l,
                      "final_loss": float(hist[-1]),
                      "net": "8-64-64-64-3 GELU, BF16 weights, FP32 accumulation; cost head "
                             "= log2 attempted steps"}

    def out_dtype(form):
        return "f32" if forms[form][1] == "mixed" else "f64"

    # ---- correctness of the chosen form and of plain vs the FP64 oracle
    import oracle
    errs = {}
    rng = np.random.default_rng(1)
    idx = np.sort(rng.choice(N, min(N, 2000), replace=False))
    oopts = capi.opts_default(alg_id)
    oopts.reltol, oopts.abstol = 1e-6, 1e-10
    ref = oracle.solve(capi, de.models.robertson, oopts, p[idx], u0[idx], t0[idx], tf[idx],
                       saveat[idx], capi.SAVE_PER_TRAJ, nthreads=oracle.hardware_threads())
    stats = {}
    for form in ("plain", args.chosen):
        r = de.solve_arrays(solve_model, opts_for(form), *dptr, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form))
        torch.cuda.synchronize()
        u = r["u"].double().cpu().numpy()
        errs[form] = oracle.weighted_error(u[idx], ref["u"], 1e-10, 1e-6)
        stats[form] = {k: r[k].cpu().numpy() for k in ("naccept", "nreject", "retcode")}
        if not np.all(stats[form]["retcode"] == capi.RET_SUCCESS):
            raise SystemExit("bench: %s form did not solve every trajectory" % form)
        if not errs[form] <= 10.0:
            raise SystemExit("bench: %s form error %.3g vs oracle exceeds 10" % (form, errs[form]))

    # L2 flush buffer (> 129 MB L2): written between timed iterations
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed_device(form, K, W):
        o = opts_for(form)
        outs = {"u": torch.empty((N, saveat.shape[1], 3),
                                 dtype=torch.float32 if out_dtype(form) == "f32" else torch.float64,
                                 device=dev),
                "retcode": torch.empty(N, dtype=torch.int32, device=dev)}
        for _ in range(W):
            de.solve_arrays(solve_model, o, *dptr, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form), out=outs)
        kerns = []
        per = step_log.setdefault(form, [])
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(K):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = de.solve_arrays(solve_model, o, *dptr, capi.SAVE_PER_TRAJ,
                                u_dtype=out_dtype(form), out=outs)
            e1.record(stream)
            torch.cuda.synchronize()
            per.append(e0.elapsed_time(e1))
            kerns.append(r["device_ms"])
        if world > 1:
            dist.barrier()
        return float(np.median(per[-K:])), float(np.median(kerns))

    def timed_e2e(form, K, W):
        """Through the C ABI with pinned host buffers: H2D + solve + D2H."""
        o = opts_for(form)
        hp = [h.numpy() for h in host]
        outs = {"u": torch.empty((N, saveat.shape[1], 3),
                                 dtype=torch.float32 if out_dtype(form) == "f32" else torch.float64
                                 ).pin_memory().numpy(),
                "retcode": torch.empty(N, dtype=torch.int32).pin_memory().numpy()}
        for _ in range(W):
            de.solve_arrays(solve_model, o, *hp, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form), out=outs)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        ts = []
        for _ in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            de.solve_arrays(solve_model, o, *hp, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form), out=outs)
            ts.append(time.perf_counter() - t)
            step_log.setdefault("e2e", []).append(ts[-1] * 1e3)
        h2d = sum(a.nbytes for a in hp)
        d2h = outs["u"].nbytes + outs["retcode"].nbytes
        return float(np.median(ts)) * 1e3, h2d, d2h

    step_log = {}  # per-step times (ms) of each timed loop, for the spread

    with ClockSampler(local) as clk:
        chosen_ms, chosen_kern = timed_device(args.chosen, args.steps, args.warmup)
        plain_ms, plain_kern = timed_device("plain", args.steps, args.warmup)
        e2e_ms, h2d, d2h = timed_e2e(args.chosen, args.steps, args.warmup)

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    chosen_ms = max_over_ranks(chosen_ms)
    plain_ms = max_over_ranks(plain_ms)
    e2e_ms = max_over_ranks(e2e_ms)
    total = N * world
    fa, fs, fv = FLOPS[(args.alg, "robertson")]
    st = stats[args.chosen]
    # the method's work from the oracle's step counts on the sample, scaled to N
    o_att = float((ref["naccept"] + ref["nreject"]).mean())
    o_acc = float(ref["naccept"].mean())
    flops = (fa * o_att * N + fs * o_acc * N + fv * float(N * saveat.shape[1]))
    achieved = flops / (chosen_kern * 1e-3) / 1e12
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = oracle.hardware_threads()
        sample = min(args.cpu_sample or 100000, N)
        oracle_robertson(args.alg, max(256, sample // 20), SEED, threads)  # warm-up
        runs = [oracle_robertson(args.alg, sample, SEED, threads)[:2] for _ in range(3)]
        v = float(np.median([r[0] for r in runs]))
        dt = float(np.median([r[1] for r in runs]))
        cpu = {"value": v, "unit": "trajectories/s", "cores": threads, "kind": "port",
               "sample": "%d trajectories of the workload, median of 3 runs of %.2f s "
                         "(EnsembleThreads-equivalent C++ FP64 restatement, std::thread pool "
                         "over all host cores)" % (sample, dt)}
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    mixed = forms[args.chosen][1] == "mixed"
    pairs = forms[args.chosen][1] == "f32x2"
    line = {
        "metric": metric,
        "value": total / (chosen_ms * 1e-3),
        "unit": "trajectories/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": chosen_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": ("f32-state/f64-lu" if mixed else
                  "f32x2-state/f64-lu" if pairs else "f64"),
        "data": "synthetic (seeded, config distributions)",
        "config": dict(config, chosen_form=args.chosen, l2="flushed between timed steps (256 MB write)",
                       parallelism="trajectory shards, no collective" if world > 1 else "single GPU"),
        "chosen_form": args.chosen,
        "learned": learn_info,
        "user_model": args.user_model,
        "plain": {"value": total / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                  "kernel_ms": plain_kern, "error_vs_oracle": errs["plain"]},
        "speedup_vs_plain": plain_ms / chosen_ms,
        "error_vs_oracle": errs[args.chosen],
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "trajectories/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                     "frac": achieved / peak64,
                     "basis": "the method's FP64 flops (FMA = 2) / kernel time / measured FP64 FMA "
                              "peak" + ("; this form executes them as FP32-pair arithmetic with an "
                                        "FP64 Jacobian, LU, error norm and time, so the fraction "
                                        "is FP64-equivalent and is not capped at 1" if pairs else ""),
                     "traffic": (TRAFFIC_PER_TRAJ[("f32x2-learned" if learn_info else "f32x2")
                                                  if pairs else "fp64"] * N
                                 if args.alg == "rodas5" else None),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "launch (%s trajectories), scaled by trajectories"
                                       % ("100,000" if pairs else "20,000"),
                     "peak_source": "in-run FP64 FMA microbenchmark (gbde_measure_fma_peak)",
                     "fp32_peak_tflops": peak32,
                     "algorithmic_flops_per_step": flops, "kernel_ms": chosen_kern},
        "steps_per_traj_mean": float((st["naccept"] + st["nreject"]).mean()),
        # per timed step: the initial-dt pre-pass and the solve kernel, plus
        # histogram / scan / scatter of the longest-span-first queue order for
        # persistent forms
        # learned forms add the network's prediction kernel
        "gpu_launches": args.steps * ((5 if forms[args.chosen][0] == "persistent" else 2) +
                                      (1 if learn_info else 0)),
        "clocks": clk.summary(),
        "step_ms_spread": {k: {"min": float(np.min(v)), "median": float(np.median(v)),
                               "max": float(np.max(v))} for k, v in step_log.items()},
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
