#!/usr/bin/env python3
"""Benchmark: ensemble trajectories/s of adaptive GPUSimpleATsit5 (FP64) on
1,048,576 Lorenz trajectories (sigma=10, beta=8/3, rho ~ U[0,30],
u0 ~ U[-1,1]^3 + (0,0,20), tspan (0,10), abstol 1e-8, reltol 1e-6, dt 0.1,
100 uniform saveat times), one solve of the whole ensemble per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value      trajectories/s with inputs and outputs resident in HBM, device time
           of each step from CUDA events on the launching stream, L2 flushed
           (512 MB write) between steps;
e2e        the same metric through the C ABI with pinned host buffers: host to
           device copy of u0/p and device to host copy of every output inside
           the timed region;
plain      the plain one-thread-per-trajectory kernel on the same inputs (the
           metric compares the measured schedule against it at matched error);
roofline   FP64 pipe: algorithmic FLOPs per launch (263 per step attempt, 101 per
           saveat point) over the kernel's event time, against the FP64 FMA
           peak this run measures with the probe library;
cpu_baseline  the oracle's SimpleATsit5 (CPU restatement, reference rounding)
           on all host cores over a bounded sample of the same workload.
With --impl reference only the CPU restatement runs (rank 0).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ensemble trajectories/s at matched error: learned-binned vs plain GPU ATsit5"
UNIT = "trajectories/s"
N_TRAJ = 1 << 20
TSPAN = (0.0, 10.0)
ABSTOL, RELTOL, DT0 = 1e-8, 1e-6, 0.1
NSAVE = 100
FLOPS_PER_ATTEMPT = 263  # 67*D + 6*8 + 14 for D = 3 (stage combinations, 6 Lorenz RHS, controller)
FLOPS_PER_SAVE = 101     # 56 + 15*D dense-output flops per saveat point
WORKLOAD = ("adaptive GPUSimpleATsit5 FP64, 1,048,576 Lorenz trajectories, rho~U[0,30], u0~U[-1,1]^3+(0,0,20), "
            "tspan (0,10), abstol 1e-8, reltol 1e-6, saveat 100 uniform times")


def inputs(n, seed=2024):
    rng = np.random.default_rng(seed)
    u0 = rng.uniform(-1, 1, (3, n))
    u0[2] += 20
    p = np.stack([np.full(n, 10.0), rng.uniform(0, 30, n), np.full(n, 8 / 3)])
    return np.ascontiguousarray(u0), np.ascontiguousarray(p)


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(n_sample=65536, threads=None):
    """SimpleATsit5 restated in C++ (reference rounding) over a bounded sample."""
    import __graft_entry__ as g
    po = g.oracle()
    threads = threads or os.cpu_count()
    u0, p = inputs(N_TRAJ)
    u0, p = np.ascontiguousarray(u0[:, :n_sample]), np.ascontiguousarray(p[:, :n_sample])
    sv = np.linspace(*TSPAN, NSAVE)
    t = time.perf_counter()
    po.solve("SimpleATsit5", "lorenz", u0, p, TSPAN, DT0, rounding="ref", abstol=ABSTOL, reltol=RELTOL, saveat=sv,
             nthreads=threads)
    dt = time.perf_counter() - t
    return {"value": n_sample / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "first %d trajectories of the 1,048,576-trajectory workload, SimpleATsit5 C++ restatement "
                      "(reference rounding, libm pow), one std::thread per core, static chunks" % n_sample,
            "seconds": dt}


def run_reference(args, rank):
    if rank != 0:
        return
    import __graft_entry__ as g
    po = g.oracle()
    threads = os.cpu_count()
    n_sample = 65536
    u0, p = inputs(N_TRAJ)
    u0, p = np.ascontiguousarray(u0[:, :n_sample]), np.ascontiguousarray(p[:, :n_sample])
    sv = np.linspace(*TSPAN, NSAVE)
    run = lambda: po.solve("SimpleATsit5", "lorenz", u0, p, TSPAN, DT0, rounding="ref", abstol=ABSTOL,
                           reltol=RELTOL, saveat=sv, nthreads=threads)
    for _ in range(args.warmup):
        run()
    t = time.perf_counter()
    for _ in range(args.steps):
        run()
    el = time.perf_counter() - t
    v = n_sample * args.steps / el
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_trajectories": n_sample},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "first %d trajectories per step; Julia SimpleDiffEq.jl cannot run on this box, "
                                   "the C++ restatement of SimpleATsit5 stands in" % n_sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def load_traffic():
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(path):
        try:
            return json.load(open(path))
        except ValueError:
            return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--schedule", default=os.environ.get("GBODE_BENCH_SCHEDULE", "learned"))
    ap.add_argument("--n", type=int, default=N_TRAJ)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import __graft_entry__ as g
    pkg = g.package()
    L = pkg._lib
    h = L.Handle(local)

    n = args.n
    u0, p = inputs(n, seed=2024 + rank)
    sv = np.linspace(*TSPAN, NSAVE)
    dev = torch.device("cuda", local)
    du0 = torch.from_numpy(u0).to(dev)
    dp = torch.from_numpy(p).to(dev)
    outs = {"us": torch.empty((NSAVE, 3, n), dtype=torch.float64, device=dev),
            "u_final": torch.empty((3, n), dtype=torch.float64, device=dev),
            "t_final": torch.empty(n, dtype=torch.float64, device=dev),
            "retcode": torch.empty(n, dtype=torch.int8, device=dev),
            "naccept": torch.empty(n, dtype=torch.int32, device=dev),
            "nreject": torch.empty(n, dtype=torch.int32, device=dev)}
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def args_for(schedule, memory, u0p, pp):
        a = pkg.make_args(pkg.GPUSimpleATsit5(), L.RHS["lorenz"], u0, p, TSPAN, DT0, ABSTOL, RELTOL, sv, False,
                          "fp64", schedule, 0, memory=memory)
        a.u0, a.p = u0p, pp
        return a

    def out_dev():
        o = L.SolveOut()
        for k, v in outs.items():
            setattr(o, k, v.data_ptr())
        return o

    schedule = args.schedule
    fit_report = None
    if schedule == "learned":
        # fit the cost model on a separate 65,536-trajectory training ensemble solved by the plain kernel
        tu0, tp = inputs(65536, seed=777 + rank)
        ta = pkg.make_args(pkg.GPUSimpleATsit5(), L.RHS["lorenz"], tu0, tp, TSPAN, DT0, ABSTOL, RELTOL, sv, False,
                           "fp64", "plain", 0)
        try:
            rep = h.learn_fit(ta)
            fit_report = {"loss_first": rep.loss_first, "loss_last": rep.loss_last, "r2_log_attempts": rep.r2_attempts,
                          "train_solve_ms": rep.train_solve_ms, "train_fit_ms": rep.train_fit_ms}
        except L.GB300ODEError as e:
            fit_report = {"unavailable": str(e)}
            schedule = "persistent"

    # pick the launch shape of the solver kernel on a 65,536-trajectory sample (excluded from timing)
    tune = None
    if not args.no_tune:
        try:
            rep = h.autotune(args_for(schedule if schedule != "learned" else "persistent", L.MEM_DEVICE,
                                      du0.data_ptr(), dp.data_ptr()), 65536)
            tune = {"block": rep.block, "max_registers": rep.max_registers, "stage_bytes": rep.stage_bytes,
                    "variants": rep.variants, "sample_ms_default": rep.default_ms, "sample_ms_best": rep.best_ms,
                    "tune_ms": rep.tune_ms}
        except L.GB300ODEError as e:
            tune = {"unavailable": str(e)}

    def device_step(sched):
        a = args_for(sched, L.MEM_DEVICE, du0.data_ptr(), dp.data_ptr())
        st = L.SolveStats()
        h.check(h.solve_raw(a, out_dev(), st))
        return st

    def timed(sched, steps, warmup):
        for _ in range(warmup):
            device_step(sched)
        kms, att, sav, launches = [], 0, 0, 0
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            st = device_step(sched)
            kms.append(st.kernel_ms)
            att, sav, launches = att + st.attempts, sav + st.saves, launches + st.launches
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return kms, att, sav, launches

    with ClockSampler(local) as clk:
        kms, att, sav, launches = timed(schedule, args.steps, args.warmup)
    clocks = clk.summary()
    step_ms = sum(kms) / len(kms)
    if dist:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    uf_measured = outs["u_final"].cpu().numpy()
    value = n * world / (step_ms * 1e-3)

    # plain one-thread-per-trajectory kernel on the same inputs, same timing rules
    pk, patt, psav, _ = timed("plain", max(1, min(args.steps, 3)), 1)
    plain_ms = sum(pk) / len(pk)
    uf_plain = outs["u_final"].cpu().numpy()
    scale = ABSTOL + RELTOL * np.abs(uf_plain).max(0)
    dev_err = np.abs(uf_measured - uf_plain).max(0) / scale

    # end to end through the C ABI with pinned host buffers
    hu0 = torch.from_numpy(u0).pin_memory()
    hp = torch.from_numpy(p).pin_memory()
    hout = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in outs.items()}
    ho = L.SolveOut()
    for k, v in hout.items():
        setattr(ho, k, v.data_ptr())
    ha = args_for(schedule, L.MEM_HOST, hu0.data_ptr(), hp.data_ptr())
    for _ in range(1):
        h.check(h.solve_raw(ha, ho, L.SolveStats()))
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        h.check(h.solve_raw(ha, ho, L.SolveStats()))
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = sum(e2e_t) / len(e2e_t)
    h2d = u0.nbytes + p.nbytes + sv.nbytes
    d2h = sum(v.numel() * v.element_size() for v in hout.values())

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # FP64 pipe peak, measured live
    peak = L.probe_rates(local, 2000)["dfma"][0] * 2 / 1e12
    flops = (att / args.steps) * FLOPS_PER_ATTEMPT + (sav / args.steps) * FLOPS_PER_SAVE
    achieved = flops / (step_ms * 1e-3) / 1e12
    traffic = load_traffic()
    tr = None
    if traffic and "atsit5_lorenz" in traffic:
        tr = traffic["atsit5_lorenz"]["bytes_per_trajectory"] * n
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; no public dataset involved)",
        "config": {"workload": WORKLOAD, "trajectories_per_gpu": n, "schedule": schedule,
                   "l2": "flushed between steps by a 512 MB device write; outputs (2.5 GB) exceed L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "plain": {"value": n * world / (plain_ms * 1e-3), "ms_per_step": plain_ms},
        "speedup_vs_plain": plain_ms / step_ms,
        "matched_error": {"max_err_vs_plain_in_error_scale": float(dev_err.max()),
                          "frac_within_10x": float(np.mean(dev_err <= 10)),
                          "error_scale": "abstol + reltol*max|u_final|"},
        "attempts_per_step": att / args.steps, "saves_per_step": sav / args.steps,
        "rhs_evals_per_s": (att / args.steps) * 6 / (step_ms * 1e-3),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": tr,
                     "peak_source": "FP64 FMA lane rate measured by this run's probe (libgb300ode_probe.so); "
                                    "MEASURED_PEAKS.json carries no FP64 figure"},
        "e2e": {"value": n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if fit_report is not None:
        line["learned_fit"] = fit_report
    if tune is not None:
        line["autotune"] = tune
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
