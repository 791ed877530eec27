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
           on all host cores over a bounded sample of the same workload;
persistent_unsorted  the learned schedule's kernel in identity order (what
           the trained network's ordering adds), amortized  the learned
           schedule's one-off cost (training solve + fit) against plain;
parity_vs_ref  the GPU's results on the first 4,096 trajectories against the
           oracle in the reference's rounding.
With --impl reference only the CPU restatement runs (rank 0), over the whole
1,048,576-trajectory workload every step.

--config N measures another ensemble workload of the same solver family
(1: fixed-step Tsit5; 3: AVern7 Van der Pol; 4: AVern9 restricted three-body
in FP32 with Kahan-compensated state, with its full-FP64 variant on a sample;
5: ATsit5 Kuramoto-12 with the order parameter reduced in the kernel;
6: SimpleEM stochastic Lorenz).  The default is the 1M adaptive Lorenz
workload above (config 2).

workloads  (default run on one GPU without --n) each other workload measured by a
           child process `bench.py --config N --brief` after the headline
           line's own measurements, its line condensed into this key;
           `--workloads none` skips them, `--workloads 3,5` picks some.
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


def inputs_fixed_lorenz(n, seed):
    rng = np.random.default_rng(seed)
    u0 = np.tile(np.array([[1.0], [0.0], [0.0]]), (1, n))
    p = np.stack([np.full(n, 10.0), rng.uniform(0, 21, n), np.full(n, 8 / 3)])
    return np.ascontiguousarray(u0), np.ascontiguousarray(p)


def inputs_vdp(n, seed):
    rng = np.random.default_rng(seed)
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))[None, :]
    return np.ascontiguousarray(rng.uniform(-2, 2, (2, n))), np.ascontiguousarray(mu)


def inputs_r3bp(n, seed):
    rng = np.random.default_rng(seed)
    u0 = np.array([0.994, 0.0, 0.0, -2.00158510637908])[:, None] + rng.normal(0, 1e-4, (4, n))
    return np.ascontiguousarray(u0), np.full((1, n), 0.012277471)


def inputs_kuramoto(n, seed, D=12):
    rng = np.random.default_rng(seed)
    th = rng.uniform(0, 2 * np.pi, (D, n))
    p = np.vstack([rng.normal(0, 1, (D, n)), rng.uniform(0, 4, (1, n))])
    return np.ascontiguousarray(th), np.ascontiguousarray(p)


def inputs_sde_lorenz(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1, 1, (3, n))
    u[2] += 20
    p = np.stack([np.full(n, 10.0), rng.uniform(0, 30, n), np.full(n, 8 / 3), np.full(n, 0.5)])
    return np.ascontiguousarray(u), np.ascontiguousarray(p)


T_ARENSTORF = 17.0652165601579625588917206249
# Per-unit algorithmic work (FMA = 2 flops): per step attempt and per saveat point.
CONFIGS = {
    1: dict(workload="fixed-step GPUSimpleTsit5 FP64, 8192 Lorenz trajectories, u0=(1,0,0), rho~U[0,21], "
                     "tspan (0,1), dt 0.01, final state only",
            alg="Tsit5", rhs="lorenz", n=8192, tspan=(0.0, 1.0), dt=0.01, abstol=1e-6, reltol=1e-3, nsave=0,
            precision="fp64", output="state", inputs=inputs_fixed_lorenz, flops_attempt=192, flops_save=0,
            rhs_per_attempt=6, oracle_alg="SimpleTsit5", dtype="f64"),
    2: dict(workload=WORKLOAD, alg="ATsit5", rhs="lorenz", n=N_TRAJ, tspan=TSPAN, dt=DT0, abstol=ABSTOL,
            reltol=RELTOL, nsave=NSAVE, precision="fp64", output="state", inputs=inputs,
            flops_attempt=FLOPS_PER_ATTEMPT, flops_save=FLOPS_PER_SAVE, rhs_per_attempt=6,
            oracle_alg="SimpleATsit5", dtype="f64"),
    3: dict(workload="adaptive GPUSimpleAVern7 FP64, 524,288 Van der Pol trajectories, mu~LogUniform[0.1,10], "
                     "(x,v)(0)~U[-2,2]^2, tspan (0,20), abstol 1e-10, reltol 1e-8, saveat 200 uniform times",
            alg="AVern7", rhs="vanderpol", n=524288, tspan=(0.0, 20.0), dt=0.1, abstol=1e-10, reltol=1e-8,
            nsave=200, precision="fp64", output="state", inputs=inputs_vdp, flops_attempt=298, flops_save=494,
            rhs_per_attempt=10, oracle_alg="AVern7", dtype="f64"),
    4: dict(workload="adaptive GPUSimpleAVern9, FP32 stages with Kahan-compensated state and FP64 t, 262,144 "
                     "planar restricted three-body trajectories (mu=0.012277471, Arenstorf u0 + N(0,1e-4)), "
                     "one Arenstorf period, abstol = reltol = 1e-7, final state",
            alg="AVern9", rhs="r3bp", n=262144, tspan=(0.0, T_ARENSTORF), dt=0.1, abstol=1e-7, reltol=1e-7,
            nsave=0, precision="fp32_kahan", output="state", inputs=inputs_r3bp, flops_attempt=1290,
            flops_save=0, rhs_per_attempt=16, oracle_alg="AVern9", dtype="f32 (Kahan state, f64 t)"),
    5: dict(workload="adaptive GPUSimpleATsit5 FP64, 4,194,304 Kuramoto-12 trajectories, omega~N(0,1), "
                     "K~U[0,4], theta(0)~U[0,2pi)^12, tspan (0,50), abstol 1e-8, reltol 1e-6, final state + "
                     "order parameter at 50 saveat times (reduced in the kernel)",
            alg="ATsit5", rhs="kuramoto", n=4194304, tspan=(0.0, 50.0), dt=0.1, abstol=1e-8, reltol=1e-6,
            nsave=50, precision="fp64", output="kuramoto_r", inputs=inputs_kuramoto,
            # 1310 stage/RHS/controller flops + 6 RHS x 12 sin/cos pairs x 33 flops of the kernel's
            # sincos_cw (15 FMA + 2 multiplies + 1 add); per save 266 + 12 pairs x 33
            flops_attempt=1310 + 6 * 12 * 33, flops_save=266 + 12 * 33, rhs_per_attempt=6, oracle_alg="ATsit5",
            dtype="f64"),
    6: dict(kind="sde", workload="SimpleEM (Euler-Maruyama) FP64, 1,048,576 stochastic Lorenz trajectories "
                                 "(drift sigma=10, rho~U[0,30], beta=8/3; additive noise 0.5 per component), "
                                 "u0~U[-1,1]^3+(0,0,20), tspan (0,1), dt 1e-3, final state; Philox4x32-10 normals",
            sde="lorenz", n=1048576, tspan=(0.0, 1.0), dt=1e-3, inputs=inputs_sde_lorenz, dtype="f64",
            # FP64 work per step: drift 8, update 3 x 5, grid time 2, and 1.5 Box-Muller pairs (3 normals a
            # step from a stream of pairs) x 2 double additions that turn a pair's double-single normals into
            # doubles; the normals' log, square root, sine and cosine run in double-single on the
            # single-precision pipe and are not FP64 work
            flops_step=8 + 15 + 2 + 1.5 * 2),
}


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


CPU_SECONDS = 10.0  # target length of the timed CPU-baseline sample


def sized_sample(solve_first, n_max, seconds, pilot=2048):
    """Time solve_first(m) (a solve of the first m trajectories) on a sample
    sized to take about `seconds`: a pilot of `pilot` trajectories measures the
    rate, then the timed run covers rate * seconds trajectories; when that is
    more than the whole workload (n_max), the whole workload is solved as many
    times as fill the time.  Returns (trajectories solved, elapsed seconds,
    trajectories per solve)."""
    m0 = min(pilot, n_max)
    t = time.perf_counter()
    solve_first(m0)
    rate = m0 / max(time.perf_counter() - t, 1e-6)
    m = int(min(n_max, max(m0, rate * seconds)))
    reps = max(1, int(rate * seconds / m))
    t = time.perf_counter()
    for _ in range(reps):
        solve_first(m)
    return m * reps, time.perf_counter() - t, m


def cpu_baseline(cfg, seconds=CPU_SECONDS, threads=None):
    """The oracle's CPU restatement of the reference solver (reference rounding)
    over a bounded sample of the same workload (the first trajectories, about
    `seconds` of work), on all host cores."""
    import __graft_entry__ as g
    po = g.oracle()
    threads = threads or os.cpu_count()
    u0_all, p_all = cfg["inputs"](cfg["n"], 2024)
    sv = np.linspace(*cfg["tspan"], cfg["nsave"]) if cfg["nsave"] else None
    prec = "fp32" if cfg["precision"] == "fp32_kahan" else cfg["precision"]

    def solve_first(m):
        po.solve(cfg["oracle_alg"], cfg["rhs"], np.ascontiguousarray(u0_all[:, :m]),
                 np.ascontiguousarray(p_all[:, :m]), cfg["tspan"], cfg["dt"], rounding="ref",
                 abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv, nthreads=threads, precision=prec,
                 output=cfg["output"])
    solved, dt, m = sized_sample(solve_first, cfg["n"], seconds)
    return {"value": solved / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "the first %d trajectories of the workload%s, %s restated in C++ (reference rounding, "
                      "libm pow%s), one std::thread per core, static chunks"
                      % (m, "" if solved == m else " (all of it, solved %d times)" % (solved // m),
                         cfg["oracle_alg"], ", FP32 as the reference with Float32 state" if prec == "fp32" else ""),
            "seconds": dt}


def run_reference(args, rank):
    """The CPU restatement of SimpleATsit5 (reference rounding) on every host
    core, over the whole workload each step (all 1,048,576 trajectories)."""
    if rank != 0:
        return
    import __graft_entry__ as g
    po = g.oracle()
    threads = os.cpu_count()
    u0, p = inputs(N_TRAJ)
    sv = np.linspace(*TSPAN, NSAVE)

    def run():
        po.solve("SimpleATsit5", "lorenz", u0, p, TSPAN, DT0, rounding="ref", abstol=ABSTOL, reltol=RELTOL,
                 saveat=sv, nthreads=threads)
    for _ in range(args.warmup):
        run()
    t = time.perf_counter()
    for _ in range(args.steps):
        run()
    el = time.perf_counter() - t
    v = N_TRAJ * args.steps / el
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "trajectories_per_step": N_TRAJ},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "all %d trajectories of the workload per step; Julia SimpleDiffEq.jl cannot run "
                                   "on this box, the C++ restatement of SimpleATsit5 stands in" % N_TRAJ},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def parity_vs_ref(cfg, u0, p, sv, res, m=4096):
    """The GPU's results on the first m trajectories against the oracle's
    restatement of the reference's own rounding (unfused SVector arithmetic,
    libm pow): fraction of final states and of saveat series within 10x the
    error scale abstol + reltol*max|u| of each trajectory, the largest
    deviation in that unit, and the accepted-step count differences.  Fixed
    step: the largest normwise relative deviation of the final state."""
    import __graft_entry__ as g
    po = g.oracle()
    m = min(m, u0.shape[1])
    ref = po.solve(cfg["alg"], cfg["rhs"], np.ascontiguousarray(u0[:, :m]), np.ascontiguousarray(p[:, :m]),
                   cfg["tspan"], cfg["dt"], rounding="ref", abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv,
                   nthreads=os.cpu_count(), output=cfg["output"])
    uf = res["u_final"][:, :m]
    if cfg["alg"] in ("Tsit5", "Vern7", "Vern9", "RK4"):
        rel = np.abs(uf - ref["u_final"]).max(0) / np.maximum(np.abs(ref["u_final"]).max(0), 1e-300)
        return {"trajectories": m, "max_rel_err_final": float(rel.max()), "bar": "1e-12 relative"}
    scale = cfg["abstol"] + cfg["reltol"] * np.abs(ref["u_final"]).max(0)
    e = np.abs(uf - ref["u_final"]).max(0) / scale
    dn = np.abs(res["naccept"][:m].astype(np.int64) - ref["naccept"])
    out = {"trajectories": m, "final_frac_within_10x": float(np.mean(e <= 10)), "final_max_in_error_scale": float(e.max()),
           "naccept_max_abs_diff": int(dn.max()), "naccept_frac_within_1": float(np.mean(dn <= 1)),
           "error_scale": "abstol + reltol*max|u_final| per trajectory (saveat: max|us|)"}
    if sv is not None and res.get("us") is not None:
        us = res["us"][:, :, :m]
        us_scale = cfg["abstol"] + cfg["reltol"] * np.nanmax(np.abs(ref["us"]), axis=(0, 1))
        eu = np.nanmax(np.abs(us - ref["us"]), axis=(0, 1)) / us_scale
        out.update(saveat_frac_within_10x=float(np.mean(eu <= 10)), saveat_max_in_error_scale=float(eu.max()))
    return out


def bitexact_vs_oracle(cfg, u0, p, sv, res, m=4096):
    """Fraction of the first m trajectories whose every output (final state,
    accepted and rejected steps, saveat values) is bit-identical to the
    oracle's REF rounding with correctly rounded powers (controller "ref"),
    the restatement of the reference-arithmetic mode."""
    import __graft_entry__ as g
    po = g.oracle()
    m = min(m, u0.shape[1])
    ref = po.solve(cfg["alg"], cfg["rhs"], np.ascontiguousarray(u0[:, :m]), np.ascontiguousarray(p[:, :m]),
                   cfg["tspan"], cfg["dt"], rounding="ref", controller="ref", abstol=cfg["abstol"],
                   reltol=cfg["reltol"], saveat=sv, nthreads=os.cpu_count(), output=cfg["output"])
    def eq(a, b):
        return (a == b) | (np.isnan(a) & np.isnan(b))
    same = np.all(eq(res["u_final"][:, :m], ref["u_final"]), axis=0)
    same &= (res["naccept"][:m] == ref["naccept"]) & (res["nreject"][:m] == ref["nreject"])
    if sv is not None and res.get("us") is not None:
        same &= np.all(eq(res["us"][:, :, :m], ref["us"]), axis=(0, 1))
    return {"trajectories": m, "frac_bit_identical": float(same.mean()),
            "oracle": "REF rounding with correctly rounded powers"}


WORKLOAD_TIMEOUT_S = 420


def condense(sub):
    """A workload's line without what the headline line already says (metric,
    unit, step counts) and without the autotuner's per-variant table."""
    drop = {"metric", "unit", "n_gpus", "higher_is_better", "scaling", "vs_baseline", "data"}
    out = {k: v for k, v in sub.items() if k not in drop}
    if isinstance(out.get("autotune"), dict):
        out["autotune"] = {k: v for k, v in out["autotune"].items() if k != "table"}
    return out


def run_workloads(args):
    """Each other workload measured by a child process (`bench.py --config N
    --brief`, the same timing rules: warm-up, L2 flush, CUDA events, clock
    samples) one after another on this GPU; this process's own solves have
    ended.  A failed or timed-out child is recorded as such."""
    which = sorted(c for c in CONFIGS if c != 2) if args.workloads == "auto" else \
        [int(x) for x in args.workloads.split(",") if x.strip()]
    out = {}
    for c in which:
        cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--config", str(c), "--steps", str(min(args.steps, 3)),
               "--warmup", "3", "--brief", "--workloads", "none",
               "--cpu-seconds", "3"]
        t0 = time.perf_counter()
        try:
            r = subprocess.run(cmd, capture_output=True, text=True, timeout=WORKLOAD_TIMEOUT_S)
            lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
            if r.returncode == 0 and lines:
                out[str(c)] = condense(json.loads(lines[-1]))
            else:
                out[str(c)] = {"error": "exit %d: %s" % (r.returncode, (r.stderr or r.stdout)[-400:])}
        except subprocess.TimeoutExpired:
            out[str(c)] = {"error": "timed out after %d s" % WORKLOAD_TIMEOUT_S}
        out[str(c)]["wall_s"] = time.perf_counter() - t0
    return out


def probe_rates(device=0, iters=2000):
    """Measured lane-operation rates of the arithmetic pipes (bench_probe.cu,
    built by __graft_entry__.build() into _build/libbench_probe.so)."""
    import ctypes
    lib = ctypes.CDLL(os.path.join(ROOT, "_build", "libbench_probe.so"))
    lib.probe_op_rates.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    r = np.zeros(7)
    ms = np.zeros(7)
    rc = lib.probe_op_rates(int(device), int(iters), r.ctypes.data, ms.ctypes.data, 7)
    if rc != 0:
        raise RuntimeError("probe failed (%d)" % rc)
    names = ["dfma", "dadd", "ffma", "ddiv", "dsqrt_add", "dmax_add", "fdiv"]
    return {k: (float(r[i]), float(ms[i])) for i, k in enumerate(names)}


def load_traffic():
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if os.path.exists(path):
        try:
            return json.load(open(path))
        except ValueError:
            return None
    return None


def max_over_ranks(value, dist, device):
    """The slowest replica's step time: with one process per GPU (replicas of
    the workload, no collective on the data path) the job takes as long as its
    slowest rank, and whole-job throughput = trajectories of all ranks / that."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_seed(rank):
    """Each rank solves its own replica of the workload (weak scaling)."""
    return 2024 + rank


def run_sde(args, cfg, rank, world, local):
    """SimpleEM workload: device-timed solves (L2 flushed between steps), the
    C ABI end to end with pinned host buffers, the FP64 roofline and the
    oracle's CPU restatement on a sample."""
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
    n = args.n or cfg["n"]
    u0, p = cfg["inputs"](n, replica_seed(rank))
    dim, nparams = u0.shape[0], p.shape[0]
    nsteps = int(round((cfg["tspan"][1] - cfg["tspan"][0]) / cfg["dt"]))
    dev = torch.device("cuda", local)
    du0, dp = torch.from_numpy(u0).to(dev), torch.from_numpy(p).to(dev)
    uf = torch.empty((dim, n), dtype=torch.float64, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def sargs(memory, u0p, pp):
        a = L.SdeArgs()
        a.sde, a.n, a.dim, a.nparams = L.SDE[cfg["sde"]], n, dim, nparams
        a.t0, a.tf, a.dt, a.seed = cfg["tspan"][0], cfg["tspan"][1], cfg["dt"], 1234 + rank
        a.save_everystep, a.memory, a.u0, a.p = 0, memory, u0p, pp
        return a

    a = sargs(L.MEM_DEVICE, du0.data_ptr(), dp.data_ptr())
    o = L.SdeOut()
    o.u_final = uf.data_ptr()
    for _ in range(args.warmup):
        h.check(h.sde_solve(a, o, L.SolveStats()))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    kms, launches = [], 0
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            st = L.SolveStats()
            h.check(h.sde_solve(a, o, st))
            kms.append(st.kernel_ms)
            launches += st.launches
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    step_ms = max_over_ranks(sum(kms) / len(kms), dist, dev)
    hu0, hp = torch.from_numpy(u0).pin_memory(), torch.from_numpy(p).pin_memory()
    huf = torch.empty((dim, n), dtype=torch.float64).pin_memory()
    ha = sargs(L.MEM_HOST, hu0.data_ptr(), hp.data_ptr())
    ho = L.SdeOut()
    ho.u_final = huf.data_ptr()
    h.check(h.sde_solve(ha, ho))
    e2e_t = []
    for _ in range(max(3, args.steps)):  # the median of at least three: host copies vary
        t0 = time.perf_counter()
        h.check(h.sde_solve(ha, ho))
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    rates = probe_rates(local, 2000)
    peak = rates["dfma"][0] * 2 / 1e12
    achieved = n * nsteps * cfg["flops_step"] / (step_ms * 1e-3) / 1e12
    line = {
        "metric": "ensemble trajectories/s (workload 6, SimpleEM)", "value": n * world / (step_ms * 1e-3),
        "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": cfg["dtype"],
        "data": "synthetic (seeded; no public dataset involved)",
        "config": {"workload": cfg["workload"], "trajectories_per_gpu": n, "steps_per_trajectory": nsteps,
                   "l2": "flushed between steps by a 512 MB device write",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "trajectory_steps_per_s": n * world * nsteps / (step_ms * 1e-3),
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": None,
                     "peak_source": "FP64 FMA lane rate measured by this run's probe (bench_probe.cu)",
                     "counted": "the FP64 flops the kernel executes a step (drift, update, grid time, the "
                                "normals' conversion to double); the normals themselves are double-single "
                                "work on the single-precision pipe"},
        "e2e": {"value": n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": u0.nbytes + p.nbytes,
                "d2h_bytes_per_step": huf.numel() * 8},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        po = g.oracle()
        threads = os.cpu_count()

        def solve_first(m):
            po.sde_solve(cfg["sde"], np.ascontiguousarray(u0[:, :m]), np.ascontiguousarray(p[:, :m]),
                         cfg["tspan"], cfg["dt"], seed=1234, rounding="ref", save_everystep=False, nthreads=threads)
        solved, el, m = sized_sample(solve_first, n, args.cpu_seconds)
        line["cpu_baseline"] = {"value": solved / el, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": "the first %d trajectories%s, SimpleEM restated in C++ with the same "
                                          "counter-based normals, one std::thread per core"
                                          % (m, "" if solved == m else " (solved %d times)" % (solved // m)),
                                "seconds": el}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=sorted(CONFIGS))
    ap.add_argument("--schedule", default=os.environ.get("GBODE_BENCH_SCHEDULE", "learned"))
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--tune-sample", type=int, default=262144, help="trajectories the autotuner times each variant on")
    ap.add_argument("--layout", default="traj", choices=["soa", "traj"],
                    help="saveat output layout: [npoints][dim][n] (soa) or [n][npoints][dim] (traj)")
    ap.add_argument("--cpu-seconds", type=float, default=CPU_SECONDS,
                    help="length of the timed CPU-baseline sample")
    ap.add_argument("--brief", action="store_true",
                    help="skip the dt0-seeding leg, and the identity-order and single-precision-controller legs of "
                         "workloads whose solve takes over a second")
    ap.add_argument("--workloads", default="auto",
                    help="other workloads measured after the default one on a single GPU: 'auto' (all), "
                         "'none', or a comma list of config numbers")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)
    cfg = CONFIGS[args.config]
    if cfg.get("kind") == "sde":
        return run_sde(args, cfg, rank, world, local)
    fixed = cfg["alg"] in ("Tsit5", "Vern7", "Vern9", "RK4")

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
    alg = getattr(pkg, "GPUSimple" + cfg["alg"])()

    n = args.n or cfg["n"]
    u0, p = cfg["inputs"](n, replica_seed(rank))
    dim, nparams = u0.shape[0], p.shape[0]
    nsave = cfg["nsave"]
    sv = np.linspace(*cfg["tspan"], nsave) if nsave else None
    width = 1 if cfg["output"] == "kuramoto_r" else dim
    dev = torch.device("cuda", local)
    du0 = torch.from_numpy(u0).to(dev)
    dp = torch.from_numpy(p).to(dev)
    outs = {"u_final": torch.empty((dim, n), dtype=torch.float64, device=dev),
            "t_final": torch.empty(n, dtype=torch.float64, device=dev),
            "retcode": torch.empty(n, dtype=torch.int8, device=dev),
            "naccept": torch.empty(n, dtype=torch.int32, device=dev),
            "nreject": torch.empty(n, dtype=torch.int32, device=dev)}
    if nsave:
        outs["us"] = torch.empty((n, nsave, width) if args.layout == "traj" else (nsave, width, n),
                                 dtype=torch.float64, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)

    def args_for(schedule, memory, u0p, pp, uu=u0, ppp=p, controller="ds"):
        a = pkg.make_args(alg, L.RHS[cfg["rhs"]], uu, ppp, cfg["tspan"], cfg["dt"], cfg["abstol"], cfg["reltol"],
                          sv, False, cfg["precision"], schedule, 0, memory=memory, output=cfg["output"],
                          controller=controller, layout=args.layout)
        a.u0, a.p = u0p, pp
        return a

    def out_dev():
        o = L.SolveOut()
        for k, v in outs.items():
            setattr(o, k, v.data_ptr())
        return o

    schedule = "plain" if fixed else args.schedule
    fit_report = None
    if schedule == "learned":
        # fit the cost model on a separate 65,536-trajectory training ensemble solved by the plain kernel
        tu0, tp = cfg["inputs"](65536, 777 + rank)
        ta = pkg.make_args(alg, L.RHS[cfg["rhs"]], tu0, tp, cfg["tspan"], cfg["dt"], cfg["abstol"], cfg["reltol"],
                           None, False, cfg["precision"], "plain", 0)
        try:
            rep = h.learn_fit(ta)
            fit_report = {"loss_first": rep.loss_first, "loss_last": rep.loss_last, "r2_log_attempts": rep.r2_attempts,
                          "train_solve_ms": rep.train_solve_ms, "train_fit_ms": rep.train_fit_ms,
                          "train_kernel_ms": rep.train_kernel_ms, "train_cluster_ctas": rep.train_ctas}
        except L.GB300ODEError as e:
            fit_report = {"unavailable": str(e)}
            schedule = "persistent"

    # pick the launch shape of the solver kernel on a sample (default 262,144 trajectories: smaller samples
    # are dominated by the end-of-kernel tail and mislead), timed in the order the
    # schedule uses (excluded from timing)
    tune = None
    if not args.no_tune and not fixed:
        try:
            rep = h.autotune(args_for(schedule, L.MEM_DEVICE, du0.data_ptr(), dp.data_ptr()), args.tune_sample)
            tune = {"block": rep.block, "max_registers": rep.max_registers, "stage_bytes": rep.stage_bytes,
                    "variants": rep.variants, "sample": rep.sample, "sample_ms_default": rep.default_ms,
                    "sample_ms_best": rep.best_ms, "tune_ms": rep.tune_ms,
                    "table": [[b, r, s, round(ms, 3)] for b, r, s, ms in rep.rows()]}
        except L.GB300ODEError as e:
            tune = {"unavailable": str(e)}

    def device_step(sched, controller="ds"):
        a = args_for(sched, L.MEM_DEVICE, du0.data_ptr(), dp.data_ptr(), controller=controller)
        st = L.SolveStats()
        h.check(h.solve_raw(a, out_dev(), st), allow=(L.ETRAJ,))
        return st

    def timed(sched, steps, warmup, controller="ds"):
        for _ in range(warmup):
            device_step(sched, controller)
        kms, att, sav, launches = [], 0, 0, 0
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            st = device_step(sched, controller)
            kms.append(st.kernel_ms)
            att, sav, launches = att + st.attempts, sav + st.saves, launches + st.launches
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        return kms, att, sav, launches

    with ClockSampler(local) as clk:
        kms, att, sav, launches = timed(schedule, args.steps, args.warmup)
    clocks = clk.summary()
    step_ms = max_over_ranks(sum(kms) / len(kms), dist, dev)
    uf_measured = outs["u_final"].cpu().numpy()
    m_par = min(n, 4096)
    def us_sample():
        if not nsave:
            return None
        if args.layout == "traj":
            return outs["us"][:m_par].permute(1, 2, 0).cpu().numpy()
        return outs["us"][:, :, :m_par].cpu().numpy()
    res_sample = {"u_final": uf_measured[:, :m_par], "naccept": outs["naccept"][:m_par].cpu().numpy(),
                  "us": us_sample()}
    value = n * world / (step_ms * 1e-3)

    # the same persistent staged kernel in identity order: what the trained network's ordering adds
    long_solve = args.brief and step_ms > 1000.0
    unsorted_ms = None
    if schedule == "learned" and not long_solve:
        uk, _, _, _ = timed("persistent", max(1, min(args.steps, 3)), 1)
        unsorted_ms = sum(uk) / len(uk)

    # plain one-thread-per-trajectory kernel on the same inputs, same timing rules
    if schedule != "plain":
        pk, _, _, _ = timed("plain", max(1, min(args.steps, 3)), 1)
        plain_ms = sum(pk) / len(pk)
    else:
        plain_ms = step_ms
    uf_plain = outs["u_final"].cpu().numpy()

    # the same schedule with the single-precision error norm and controller (kernel compiled at run time and
    # autotuned like the default's): what the default double-single arithmetic costs, and the parity it buys
    ctl32 = None
    if not fixed and cfg["precision"] == "fp64" and not long_solve:  # every rank: timed() holds barriers
        if tune is not None and "unavailable" not in tune:
            # the same launch-shape search as the default's, so the two legs compare arithmetic only
            h.autotune(args_for(schedule, L.MEM_DEVICE, du0.data_ptr(), dp.data_ptr(), controller="fp32"),
                       args.tune_sample)
        ck, _, _, _ = timed(schedule, max(1, min(args.steps, 3)), 1, controller="fp32")
        ctl32 = {"ms_per_step": sum(ck) / len(ck), "value": n / (sum(ck) / len(ck) * 1e-3),
                 "default_cost": step_ms / (sum(ck) / len(ck))}
        ctl32_sample = {"u_final": outs["u_final"][:, :m_par].cpu().numpy(),
                        "naccept": outs["naccept"][:m_par].cpu().numpy(),
                        "us": us_sample()}

    # the reference's own arithmetic throughout (ODE_CTRL_REF: unfused vector multiply-adds, the right-hand
    # side as written, IEEE division and square root, the PI controller with correctly rounded powers), same
    # schedule, tuned alike: what following the reference operation for operation costs, its parity with the
    # reference's rounding, and its bit-identity with the oracle's restatement of that arithmetic
    refa = None
    if not fixed and cfg["precision"] == "fp64" and not long_solve:  # every rank: timed() holds barriers
        if tune is not None and "unavailable" not in tune:
            h.autotune(args_for(schedule, L.MEM_DEVICE, du0.data_ptr(), dp.data_ptr(), controller="ref"),
                       args.tune_sample)
        rk, _, _, _ = timed(schedule, max(1, min(args.steps, 3)), 1, controller="ref")
        refa = {"ms_per_step": sum(rk) / len(rk), "value": n / (sum(rk) / len(rk) * 1e-3),
                "cost_vs_default": (sum(rk) / len(rk)) / step_ms}
        refa_sample = {"u_final": outs["u_final"][:, :m_par].cpu().numpy(),
                       "naccept": outs["naccept"][:m_par].cpu().numpy(),
                       "nreject": outs["nreject"][:m_par].cpu().numpy(),
                       "us": us_sample()}
    scale = cfg["abstol"] + cfg["reltol"] * np.abs(uf_plain).max(0)
    dev_err = np.abs(uf_measured - uf_plain).max(0) / scale
    dev_err = dev_err[np.isfinite(dev_err)] if np.isfinite(dev_err).any() else np.zeros(1)

    # the cost model's second use: seeding each trajectory's first dt with its prediction (opt-in, changes the
    # step sequences): time, attempts and deviation from the plain kernel's results, then back to ordering only
    seeded = None
    if schedule == "learned" and fit_report and "train_fit_ms" in fit_report and not args.brief:
        try:
            h.learn_fit(ta, {"seed_dt0": 1})
            sk, s_att, _, _ = timed("learned", max(1, min(args.steps, 3)), 1)
            s_steps = max(1, min(args.steps, 3))
            uf_seeded = outs["u_final"].cpu().numpy()
            s_err = np.abs(uf_seeded - uf_plain).max(0) / scale
            s_err = s_err[np.isfinite(s_err)]
            seeded = {"ms_per_step": sum(sk) / len(sk), "speedup_vs_ordering_only": step_ms / (sum(sk) / len(sk)),
                      "attempts_per_step": s_att / s_steps, "attempts_ordering_only": att / args.steps,
                      "vs_plain_frac_within_10x": float(np.mean(s_err <= 10)),
                      "note": "results change (other step sequences); chaotic trajectories move beyond the "
                              "error scale in both roundings"}
        finally:
            h.learn_fit(ta)

    # end to end through the C ABI with pinned host buffers
    hu0 = torch.from_numpy(u0).pin_memory()
    hp = torch.from_numpy(p).pin_memory()
    hout = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in outs.items()}
    ho = L.SolveOut()
    for k, v in hout.items():
        setattr(ho, k, v.data_ptr())
    ha = args_for(schedule, L.MEM_HOST, hu0.data_ptr(), hp.data_ptr())
    h.check(h.solve_raw(ha, ho, L.SolveStats()), allow=(L.ETRAJ,))
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(max(3, args.steps)):  # the median of at least three: host copies vary
        t0 = time.perf_counter()
        h.check(h.solve_raw(ha, ho, L.SolveStats()), allow=(L.ETRAJ,))
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e_t)  # host-side copies vary from call to call: the median of the steps
    h2d = u0.nbytes + p.nbytes + (sv.nbytes if sv is not None else 0)
    d2h = sum(v.numel() * v.element_size() for v in hout.values())

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    # pipe peak, measured live: FP64 FMA (or FP32 FMA for the single-precision mode)
    rates = probe_rates(local, 2000)
    fp32 = cfg["precision"] != "fp64"
    peak = (rates["ffma"][0] if fp32 else rates["dfma"][0]) * 2 / 1e12
    flops = (att / args.steps) * cfg["flops_attempt"] + (sav / args.steps) * cfg["flops_save"]
    achieved = flops / (step_ms * 1e-3) / 1e12
    traffic = load_traffic()
    tr = None
    tkey = "atsit5_lorenz" + ("_traj" if args.layout == "traj" else "")
    if args.config == 2 and traffic and tkey in traffic:
        tr = traffic[tkey]["bytes_per_trajectory"] * n
    line = {
        "metric": METRIC if args.config == 2 else "ensemble trajectories/s (workload %d)" % args.config,
        "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": cfg["dtype"], "data": "synthetic (seeded; no public dataset involved)",
        "config": {"workload": cfg["workload"], "trajectories_per_gpu": n, "schedule": schedule,
                   "output_layout": "[n][nsave][dim]" if args.layout == "traj" else "[nsave][dim][n]",
                   "l2": "flushed between steps by a 512 MB device write",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "plain": {"value": n * world / (plain_ms * 1e-3), "ms_per_step": plain_ms},
        "speedup_vs_plain": plain_ms / step_ms,
        "matched_error": {"max_err_vs_plain_in_error_scale": float(dev_err.max()),
                          "frac_within_10x": float(np.mean(dev_err <= 10)),
                          "error_scale": "abstol + reltol*max|u_final|"},
        "attempts_per_step": att / args.steps, "saves_per_step": sav / args.steps,
        "rhs_evals_per_s": (att / args.steps) * cfg["rhs_per_attempt"] / (step_ms * 1e-3),
        "roofline": {"bound": "fp32" if fp32 else "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": tr,
                     "peak_source": "%s FMA lane rate measured by this run's probe (bench_probe.cu); "
                                    "MEASURED_PEAKS.json carries no FP64/FP32-pipe figure" % ("FP32" if fp32 else "FP64")},
        "e2e": {"value": n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if unsorted_ms is not None:
        line["persistent_unsorted"] = {"value": n * world / (unsorted_ms * 1e-3), "ms_per_step": unsorted_ms}
        line["speedup_vs_unsorted"] = unsorted_ms / step_ms
    if fit_report is not None:
        line["learned_fit"] = fit_report
        if "train_fit_ms" in fit_report:
            # the learned schedule's one-off cost (training solve + fit) against what each solve saves
            once = fit_report["train_solve_ms"] + fit_report["train_fit_ms"]
            line["amortized"] = {
                "fit_cost_ms": once, "first_solve_ms_incl_fit": once + step_ms,
                "speedup_vs_plain_first_solve": plain_ms / (once + step_ms),
                "break_even_solves_vs_plain": once / (plain_ms - step_ms) if plain_ms > step_ms else None,
                "break_even_solves_vs_unsorted": (once / (unsorted_ms - step_ms)
                                                  if unsorted_ms and unsorted_ms > step_ms else None),
                "fit_over_solve": fit_report["train_fit_ms"] / step_ms}
    if args.config != 4:
        line["parity_vs_ref"] = parity_vs_ref(cfg, u0, p, sv, res_sample)
    if seeded is not None:
        line["dt0_seeded"] = seeded
    if ctl32 is not None:
        if args.config != 4:
            ctl32["parity_vs_ref"] = parity_vs_ref(cfg, u0, p, sv, ctl32_sample)
        line["fp32_controller"] = ctl32
    if refa is not None:
        refa["parity_vs_ref"] = parity_vs_ref(cfg, u0, p, sv, refa_sample)
        refa["bitexact_vs_oracle"] = bitexact_vs_oracle(cfg, u0, p, sv, refa_sample)
        line["ref_arithmetic"] = refa
    if tune is not None:
        line["autotune"] = tune
    if args.config == 4:
        # accuracy of the single-precision result against the FP64 oracle at abstol = reltol = 1e-14
        po = g.oracle()
        m = 2048
        ref = po.solve("AVern9", "r3bp", np.ascontiguousarray(u0[:, :m]), np.ascontiguousarray(p[:, :m]),
                       cfg["tspan"], cfg["dt"], rounding="ref", abstol=1e-14, reltol=1e-14, nthreads=os.cpu_count())
        ok = ref["retcode"] == 0
        err = np.abs(uf_measured[:, :m][:, ok] - ref["u_final"][:, ok]).max(0)
        line["error_vs_fp64_oracle_1e-14"] = {"max": float(err.max()), "median": float(np.median(err)),
                                              "trajectories": int(ok.sum())}
        # the full-FP64 variant of the same ensemble (abstol = reltol = 1e-12, persistent schedule)
        k = n
        a64 = pkg.make_args(alg, L.RHS[cfg["rhs"]], u0, p, cfg["tspan"], cfg["dt"], 1e-12, 1e-12, None, False,
                            "fp64", "persistent", 0, memory=L.MEM_DEVICE)
        a64.u0, a64.p = du0.data_ptr(), dp.data_ptr()
        uf64 = torch.empty((u0.shape[0], k), dtype=torch.float64, device=dev)
        o64 = L.SolveOut()
        o64.u_final = uf64.data_ptr()
        ms64 = []
        for _ in range(2):  # warm-up (and kernel load), then the timed solve
            st64 = L.SolveStats()
            h.check(h.solve_raw(a64, o64, st64), allow=(L.ETRAJ,))
            ms64.append(st64.kernel_ms)
        e64 = np.abs(uf64.cpu().numpy()[:, :m][:, ok] - ref["u_final"][:, ok]).max(0)
        line["fp64_variant"] = {"trajectories": k, "abstol": 1e-12, "reltol": 1e-12, "schedule": "persistent",
                                "ms": ms64[-1], "value": k / (ms64[-1] * 1e-3), "attempts": int(st64.attempts),
                                "error_vs_fp64_oracle_1e-14": {"max": float(e64.max()),
                                                               "median": float(np.median(e64))}}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg, args.cpu_seconds)
    if args.config == 2 and world == 1 and not args.n and args.workloads != "none":
        line["workloads"] = run_workloads(args)
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
