"""Ensemble throughput benchmark (one JSON line on rank 0).

Workload (default): stiff Robertson kinetics ensemble, Float64 -- 100,000
trajectories, rates (0.04, 3e7, 1e4) each scaled by 10^U(-1,1), u0=[1,0,0],
tspan (0, 10^U(1,5)), Rodas5 at reltol=1e-6 / abstol=1e-10, 20 log-spaced save
times t_j = tf * 10^(-5 + 5 j/19).  Seeded synthetic inputs (no dataset).

A "step" is one ensemble solve of all trajectories.  `value` is trajectories
per second of the chosen form with inputs resident in HBM (device pointers,
one gbde_ensemble_solve); `e2e` is the same through the C ABI with pinned
host buffers (H2D + solve + D2H inside the timed region).  `plain` is the
plain one-thread-per-trajectory launch for comparison.  The chosen form's
result is checked against the CPU FP64 oracle on a sample before timing.

--impl reference times the CPU FP64 restatement (EnsembleThreads-equivalent
std::thread pool over all host cores) on the same workload.
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

# DRAM bytes (read + write) per trajectory of the Rodas5 solve kernel, from one
# ncu capture (20,000 trajectories: 4.587 MB read + 8.2 KB written; the saved
# states stay in L2 until after the kernel), scaled by trajectories.
TRAFFIC_PER_TRAJ = (4.586752e6 + 8192.0) / 20000.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--alg", default="rodas5", choices=["rodas5", "rosenbrock23"])
    ap.add_argument("--trajectories", type=int, default=100000)
    ap.add_argument("--chosen", default="persistent",
                    help="chosen form: plain | persistent | persistent-mixed")
    ap.add_argument("--cpu-sample", type=int, default=100000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def workload(N, seed):
    rng = np.random.default_rng(seed)
    p = np.array([0.04, 3e7, 1e4]) * 10 ** rng.uniform(-1, 1, (N, 3))
    u0 = np.tile([1.0, 0.0, 0.0], (N, 1))
    t0 = np.zeros(N)
    tf = 10 ** rng.uniform(1, 5, N)
    saveat = tf[:, None] * 10 ** (-5 + 5 * np.arange(20) / 19)
    return p, u0, t0, tf, np.ascontiguousarray(saveat)


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


def cpu_reference(de, alg_id, args, N_sample, seed, threads):
    import oracle
    capi = de._capi
    p, u0, t0, tf, saveat = workload(N_sample, seed)
    opts = capi.opts_default(alg_id)
    opts.reltol, opts.abstol = 1e-6, 1e-10
    t = time.perf_counter()
    r = oracle.solve(capi, de.models.robertson, opts, p, u0, t0, tf, saveat, capi.SAVE_PER_TRAJ,
                     nthreads=threads)
    dt = time.perf_counter() - t
    return N_sample / dt, dt, r


def main():
    args = parse()
    world, rank, local = dist_env()
    import __graft_entry__
    de = __graft_entry__.load_package()
    capi = de._capi
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    alg_id = capi.ALG_RODAS5 if args.alg == "rodas5" else capi.ALG_ROSENBROCK23
    config = {"workload": "robertson_%s_fp64_N%d" % (args.alg, args.trajectories),
              "model": "robertson", "alg": args.alg, "trajectories": args.trajectories,
              "reltol": 1e-6, "abstol": 1e-10, "saveat": "20 log-spaced per trajectory",
              "tf": "10^U(1,5)"}
    metric = "trajectories/sec at <=10x reltol error vs FP64 oracle"

    if args.impl == "reference":
        if rank != 0:
            return
        import oracle
        threads = oracle.hardware_threads()
        sample = min(args.cpu_sample, args.trajectories)
        for _ in range(max(0, args.warmup)):
            cpu_reference(de, alg_id, args, max(256, sample // 20), SEED, threads)
        vals, secs = [], []
        for k in range(args.steps):
            v, dt, _ = cpu_reference(de, alg_id, args, sample, SEED + k, threads)
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
                                 "sample": "%d trajectories of the workload per step "
                                           "(EnsembleThreads-equivalent C++ FP64 restatement)"
                                           % sample},
                "e2e": {"value": value, "unit": "trajectories/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

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
             "persistent-mixed": ("persistent", "mixed"), "plain-mixed": ("plain", "mixed")}

    def opts_for(form):
        b, prec = forms[form]
        o = capi.opts_default(alg_id)
        o.reltol, o.abstol = 1e-6, 1e-10
        o.batching = capi.BATCH_PERSISTENT if b == "persistent" else capi.BATCH_PLAIN
        o.precision = capi.PREC_MIXED if prec == "mixed" else capi.PREC_FP64
        return o

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
        r = de.solve_arrays(de.models.robertson, opts_for(form), *dptr, capi.SAVE_PER_TRAJ,
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
            de.solve_arrays(de.models.robertson, o, *dptr, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form), out=outs)
        tot, kern = 0.0, 0.0
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(K):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = de.solve_arrays(de.models.robertson, o, *dptr, capi.SAVE_PER_TRAJ,
                                u_dtype=out_dtype(form), out=outs)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
            kern += r["device_ms"]
        if world > 1:
            dist.barrier()
        return tot / K, kern / K

    def timed_e2e(form, K, W):
        """Through the C ABI with pinned host buffers: H2D + solve + D2H."""
        o = opts_for(form)
        hp = [h.numpy() for h in host]
        outs = {"u": torch.empty((N, saveat.shape[1], 3),
                                 dtype=torch.float32 if out_dtype(form) == "f32" else torch.float64
                                 ).pin_memory().numpy(),
                "retcode": torch.empty(N, dtype=torch.int32).pin_memory().numpy()}
        for _ in range(W):
            de.solve_arrays(de.models.robertson, o, *hp, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form), out=outs)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        ts = []
        for _ in range(K):
            flush.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            de.solve_arrays(de.models.robertson, o, *hp, capi.SAVE_PER_TRAJ,
                            u_dtype=out_dtype(form), out=outs)
            ts.append(time.perf_counter() - t)
        h2d = sum(a.nbytes for a in hp)
        d2h = outs["u"].nbytes + outs["retcode"].nbytes
        return float(np.mean(ts)) * 1e3, h2d, d2h

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
    flops = (fa * float(st["naccept"].sum() + st["nreject"].sum()) + fs * float(st["naccept"].sum())
             + fv * float(N * saveat.shape[1]))
    achieved = flops / (chosen_kern * 1e-3) / 1e12
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = oracle.hardware_threads()
        sample = min(args.cpu_sample, N)
        cpu_reference(de, alg_id, args, max(256, sample // 20), SEED, threads)  # warm-up
        runs = [cpu_reference(de, alg_id, args, sample, SEED, threads)[:2] for _ in range(3)]
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
        "dtype": "f32-state/f64-lu" if mixed else "f64",
        "data": "synthetic (seeded, config distributions)",
        "config": dict(config, chosen_form=args.chosen, l2="flushed between timed steps (256 MB write)",
                       parallelism="trajectory shards, no collective" if world > 1 else "single GPU"),
        "chosen_form": args.chosen,
        "plain": {"value": total / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                  "kernel_ms": plain_kern, "error_vs_oracle": errs["plain"]},
        "speedup_vs_plain": plain_ms / chosen_ms,
        "error_vs_oracle": errs[args.chosen],
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "trajectories/s",
                "ms_per_step": e2e_ms, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                     "frac": achieved / peak64,
                     "traffic": TRAFFIC_PER_TRAJ * N if args.alg == "rodas5" else None,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                       "20,000-trajectory launch, scaled by trajectories",
                     "peak_source": "in-run FP64 FMA microbenchmark (gbde_measure_fma_peak)",
                     "fp32_peak_tflops": peak32,
                     "algorithmic_flops_per_step": flops, "kernel_ms": chosen_kern},
        "steps_per_traj_mean": float((st["naccept"] + st["nreject"]).mean()),
        # per timed step: the solve kernel, plus histogram / scan / scatter of
        # the longest-span-first queue order for persistent forms
        "gpu_launches": args.steps * (4 if forms[args.chosen][0] == "persistent" else 1),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
