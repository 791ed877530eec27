"""GPU checks of the remaining ensemble workloads: Kuramoto-12 (bit-identical
to the oracle's device canon, whose double sine and cosine are the kernels'
own Cody-Waite/Taylor routine, and within tolerance of the reference
rounding with libm), the single-precision modes' accuracy against the FP64
oracle at abstol = reltol = 1e-14, the staged saveat path in the compensated
single-precision mode, and every committed device-canon golden fixture."""
import os
import sys

import numpy as np
import pytest

from test_gpu_parity import T_ARENSTORF, assert_bitexact, gpu, r3bp_inputs

pytestmark = pytest.mark.gpu
sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402  (input generators shared with the golden fixtures)


@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_kuramoto12_bitexact_and_within_reference_tolerance(pkg, po, schedule):
    u0, p = make_golden.kuramoto(2048, 9)
    sv = np.linspace(0, 50, 50)
    kw = dict(abstol=1e-8, reltol=1e-6)
    sol = gpu(pkg, pkg.GPUSimpleATsit5(), "kuramoto", u0, p, (0.0, 50.0), 0.1, saveat=sv, schedule=schedule, **kw)
    dev = po.solve("ATsit5", "kuramoto", u0, p, (0, 50), 0.1, rounding="device", saveat=sv, nthreads=8, **kw)
    assert_bitexact(sol, dev)
    # against the reference rounding (libm sin/cos, unfused products): the adaptive tolerance
    ref = po.solve("ATsit5", "kuramoto", u0, p, (0, 50), 0.1, rounding="ref", saveat=sv, nthreads=8, **kw)
    scale = 1e-8 + 1e-6 * np.abs(ref["u_final"]).max(0)
    err = np.abs(sol.u_final - ref["u_final"]).max(0) / scale
    assert np.mean(err <= 10) >= 0.999
    assert np.mean(sol.naccept == ref["naccept"]) >= 0.99
    assert np.abs(sol.naccept - ref["naccept"]).max() <= 2
    es = np.abs(sol.us - ref["us"]).max(axis=(0, 1)) / scale
    assert np.mean(es <= 10) >= 0.999


@pytest.mark.parametrize("name", [k for k, c in make_golden.CASES.items() if c["rounding"] == "device"])
def test_committed_device_golden_fixtures(pkg, name):
    """Each committed device-canon fixture, reproduced bit for bit by the GPU
    (plain and persistent schedules) from the same seeded inputs."""
    case = dict(make_golden.CASES[name])
    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz"))
    case.pop("inputs")
    u0, p = fx["u0"], fx["p"]  # stored: regenerating them here could round differently
    alg, rhs, tspan, dt = case.pop("alg"), case.pop("rhs"), case.pop("tspan"), case.pop("dt")
    case.pop("rounding")
    scheds = ["plain"] if alg in ("Tsit5", "Vern7", "Vern9", "RK4") else ["plain", "persistent"]
    for sched in scheds:
        sol = gpu(pkg, getattr(pkg, "GPUSimple" + alg)(), rhs, u0, p, (float(tspan[0]), float(tspan[1])), dt,
                  schedule=sched, throw=False, **case)
        assert np.array_equal(sol.u_final, fx["u_final"], equal_nan=True), (name, sched)
        assert np.array_equal(sol.naccept, fx["naccept"]) and np.array_equal(sol.nreject, fx["nreject"])
        assert np.array_equal(sol.retcode, fx["retcode"])
        if "us" in fx.files:
            assert np.array_equal(sol.us, fx["us"], equal_nan=True), (name, sched)


def test_fp32_modes_error_against_fp64_oracle(pkg, po):
    """Arenstorf ensemble: FP32 and FP32-Kahan (tol 1e-7) against the FP64
    oracle at abstol = reltol = 1e-14 (trajectories the oracle finishes;
    Vern9's 1f-7 dtmin stops a few, as in the reference)."""
    u0, mu = r3bp_inputs(1024, seed=21)
    ref = po.solve("AVern9", "r3bp", u0, mu, (0, T_ARENSTORF), 0.1, rounding="ref", abstol=1e-14, reltol=1e-14,
                   nthreads=8)
    out = {}
    for prec in ("fp32", "fp32_kahan"):
        sol = gpu(pkg, pkg.GPUSimpleAVern9(), "r3bp", u0, mu, (0.0, T_ARENSTORF), 0.1, abstol=1e-7, reltol=1e-7,
                  precision=prec, throw=False)
        ok = (ref["retcode"] == 0) & (sol.retcode == 0)
        assert ok.mean() > 0.97
        err = np.abs(sol.u_final[:, ok] - ref["u_final"][:, ok]).max(0)
        out[prec] = (np.median(err), err.max())
        print("%s: max error vs FP64 oracle at 1e-14: %.3e (median %.3e) over %d trajectories"
              % (prec, err.max(), np.median(err), ok.sum()))
    assert out["fp32_kahan"][0] < 1e-3
    assert out["fp32"][0] > 2 * out["fp32_kahan"][0]  # the compensated update is what buys the accuracy


def test_staged_saveat_fp32_kahan_bitexact(pkg, po):
    rng = np.random.default_rng(12)
    n = 2048
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10), n))[None, :]
    u0 = rng.uniform(-2, 2, (2, n))
    sv = np.linspace(0, 20, 200)
    sol = gpu(pkg, pkg.GPUSimpleAVern7(), "vanderpol", u0, mu, (0.0, 20.0), 0.1, abstol=1e-6, reltol=1e-6,
              saveat=sv, precision="fp32_kahan", schedule="persistent")
    ref = po.solve("AVern7", "vanderpol", u0, mu, (0, 20), 0.1, rounding="device", precision="fp32_kahan",
                   abstol=1e-6, reltol=1e-6, saveat=sv, nthreads=8)
    assert_bitexact(sol, ref)


def test_learned_default_is_ordering_only(pkg):
    """With the default options the learned schedule only reorders: every
    trajectory's result equals the plain schedule's."""
    from conftest import lorenz_inputs
    kw = dict(dt=0.1, abstol=1e-8, reltol=1e-6)
    tr = lorenz_inputs(8192, seed=111)
    ens = lambda u0, p: pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p)
    pkg.learn_fit(ens(*tr), pkg.GPUSimpleATsit5(), 8192, **kw)
    u0, p = lorenz_inputs(8192, seed=112)
    sv = np.linspace(0, 10, 100)
    a = pkg.solve(ens(u0, p), pkg.GPUSimpleATsit5(), trajectories=8192, schedule="learned", saveat=sv, **kw)
    b = pkg.solve(ens(u0, p), pkg.GPUSimpleATsit5(), trajectories=8192, schedule="plain", saveat=sv, **kw)
    assert a.stats.schedule_used == 2
    assert np.array_equal(a.u_final, b.u_final) and np.array_equal(a.us, b.us, equal_nan=True)


@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_kuramoto_order_parameter_output(pkg, po, schedule):
    """4,194,304-trajectory workload shape, small n: final state plus the order
    parameter r(t) at 50 saveat times, reduced inside the kernel."""
    u0, p = make_golden.kuramoto(1024, 19)
    sv = np.linspace(0, 50, 50)
    kw = dict(abstol=1e-8, reltol=1e-6)
    sol = gpu(pkg, pkg.GPUSimpleATsit5(), "kuramoto", u0, p, (0.0, 50.0), 0.1, saveat=sv, schedule=schedule,
              output="kuramoto_r", **kw)
    full = gpu(pkg, pkg.GPUSimpleATsit5(), "kuramoto", u0, p, (0.0, 50.0), 0.1, saveat=sv, schedule=schedule, **kw)
    ref = po.solve("ATsit5", "kuramoto", u0, p, (0, 50), 0.1, rounding="device", saveat=sv, nthreads=8,
                   output="kuramoto_r", **kw)
    assert sol.us.shape == (50, 1, 1024)
    # the kernel's reduction equals the order parameter of its own full-state output
    r_full = np.abs(np.exp(1j * full.us).mean(1))
    assert np.abs(sol.us[:, 0, :] - r_full).max() < 1e-12
    assert np.array_equal(sol.u_final, full.u_final)
    # and is the oracle's, bit for bit
    assert np.array_equal(sol.us, ref["us"])


def test_repeated_solve_replays_the_captured_graph(pkg):
    from conftest import lorenz_inputs
    u0, p = lorenz_inputs(4096, seed=31)
    sv = np.linspace(0, 10, 20)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p)
    kw = dict(dt=0.1, abstol=1e-8, reltol=1e-6, saveat=sv, schedule="persistent")
    a = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=4096, **kw)
    b = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=4096, **kw)
    assert b.stats.graph_replayed == 1
    assert np.array_equal(a.u_final, b.u_final) and np.array_equal(a.us, b.us)
    assert a.stats.attempts == b.stats.attempts


def test_autotuner_keeps_results(pkg):
    """The tuned kernel differs only in launch shape: results are unchanged."""
    from conftest import lorenz_inputs
    n = 32768
    u0, p = lorenz_inputs(n, seed=41)
    sv = np.linspace(0, 10, 100)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p)
    kw = dict(dt=0.1, abstol=1e-8, reltol=1e-6, saveat=sv, schedule="persistent")
    before = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, **kw)
    h = pkg._handle(0)
    args = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 10.0), 0.1, 1e-8, 1e-6, sv, False, "fp64",
                         "persistent", 0)
    rep = h.autotune(args, sample=16384)
    assert rep.variants >= 4 and rep.sample == 16384
    assert rep.best_ms <= rep.default_ms
    print("autotune: block %d, regs %d, stage %d B: %.2f ms vs default %.2f ms (%d variants, %.0f ms)"
          % (rep.block, rep.max_registers, rep.stage_bytes, rep.best_ms, rep.default_ms, rep.variants, rep.tune_ms))
    after = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, **kw)
    assert np.array_equal(before.u_final, after.u_final) and np.array_equal(before.us, after.us)


@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_user_output_function_fused_into_the_solve(pkg, schedule):
    """An ensemble output function compiled with NVRTC (ode_output_compile):
    at every saved point the kernel stores (|u|^2, sigma*u0*u1 + t) instead of
    the state.  It equals the same arithmetic applied to the kernel's own
    full-state output, bit for bit (the body has no fusable multiply-add pairs
    that the host evaluates differently), for adaptive saveat and for the
    fixed-step save-every-step grid."""
    from conftest import lorenz_inputs
    u0, p = lorenz_inputs(3000, seed=51)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p)
    out = pkg.UserOutput("double s = u[0] * u[0];\n s = s + u[1] * u[1];\n out[0] = s + u[2] * u[2];\n"
                         " double q = p[0] * u[0];\n out[1] = q * u[1] + t;", width=2)
    sv = np.linspace(0, 10, 37)
    kw = dict(dt=0.1, abstol=1e-8, reltol=1e-6, saveat=sv, schedule=schedule)
    a = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=3000, output=out, **kw)
    b = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=3000, **kw)
    assert a.us.shape == (37, 2, 3000)
    s = b.us[:, 0, :] * b.us[:, 0, :]
    s = s + b.us[:, 1, :] * b.us[:, 1, :]
    assert np.array_equal(a.us[:, 0, :], s + b.us[:, 2, :] * b.us[:, 2, :])
    q = p[0][None, :] * b.us[:, 0, :]
    assert np.array_equal(a.us[:, 1, :], q * b.us[:, 1, :] + sv[:, None])
    assert np.array_equal(a.u_final, b.u_final)
    # fixed step, every grid point
    c = pkg.solve(e, pkg.GPUSimpleTsit5(), trajectories=3000, dt=0.05, save_everystep=True, output=out)
    d = pkg.solve(e, pkg.GPUSimpleTsit5(), trajectories=3000, dt=0.05, save_everystep=True)
    assert c.us.shape == (201, 2, 3000)
    q = p[0][None, :] * d.us[:, 0, :]
    assert np.array_equal(c.us[:, 1, :], q * d.us[:, 1, :] + pkg.fixed_grid(0.0, 0.05, 10.0)[:, None])


def test_user_output_compile_errors_are_reported(pkg):
    h = pkg._handle(0)
    with pytest.raises(pkg.GB300ODEError) as e:
        h.compile_output("out[0] = u[0] +;", 3, 3, 1)
    assert e.value.code == -5  # ODE_ENVRTC


@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_every_step_output_bitexact(pkg, po, schedule):
    """Ragged every-step output of the adaptive solvers (two passes: count, then
    fill) against the oracle's rows, through the Python API (host buffers) and
    the C ABI with device buffers, including the ODE_ESMALL size protocol."""
    from conftest import lorenz_inputs
    import torch
    u0, p = lorenz_inputs(1500, seed=61)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 5.0), p[:, 0]), u0s=u0, ps=p)
    kw = dict(abstol=1e-8, reltol=1e-6)
    sol = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=1500, dt=0.1, save_everystep=True, schedule=schedule,
                    **kw)
    ref = po.solve("ATsit5", "lorenz", u0, p, (0, 5), 0.1, rounding="device", save_everystep=True, nthreads=8, **kw)
    assert np.array_equal(sol.offsets, ref["offsets"])
    assert np.array_equal(sol.ts_rows, ref["ts_rows"]) and np.array_equal(sol.us_rows, ref["us_rows"])
    assert np.array_equal(sol.u_final, ref["u_final"]) and np.array_equal(sol.naccept, ref["naccept"])
    tr = sol[7]
    assert tr.t[0] == 0.0 and tr.t[-1] == 5.0 and len(tr.u) == sol.naccept[7] + 1
    # the C ABI with device buffers: first call reports the size, second fills
    L = pkg._lib
    h = pkg._handle(0)
    du0 = torch.tensor(u0, device="cuda")
    dp = torch.tensor(p, device="cuda")
    a = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 5.0), 0.1, 1e-8, 1e-6, None, False, "fp64", schedule,
                      0, memory=L.MEM_DEVICE)
    a.u0, a.p = du0.data_ptr(), dp.data_ptr()
    off = torch.empty(1501, dtype=torch.int64, device="cuda")
    o = L.EverystepOut()
    o.offsets = off.data_ptr()
    assert h.solve_everystep(a, o) == L.ESMALL
    assert o.total == ref["offsets"][-1]
    ts = torch.empty(o.total, dtype=torch.float64, device="cuda")
    us = torch.empty((o.total, 3), dtype=torch.float64, device="cuda")
    o.ts, o.us, o.capacity = ts.data_ptr(), us.data_ptr(), o.total
    h.check(h.solve_everystep(a, o))
    assert np.array_equal(off.cpu().numpy(), ref["offsets"])
    assert np.array_equal(ts.cpu().numpy(), ref["ts_rows"]) and np.array_equal(us.cpu().numpy(), ref["us_rows"])


def test_every_step_output_verner_fp32_kahan(pkg, po):
    u0, mu = make_golden.r3bp(256, 5)
    sol = pkg.solve(pkg.EnsembleProblem(pkg.ODEProblem("r3bp", u0[:, 0], (0.0, 2.0), mu[:, 0]), u0s=u0, ps=mu),
                    pkg.GPUSimpleAVern9(), trajectories=256, dt=0.1, save_everystep=True, precision="fp32_kahan",
                    abstol=1e-7, reltol=1e-7, throw=False)
    ref = po.solve("AVern9", "r3bp", u0, mu, (0, 2), 0.1, rounding="device", precision="fp32_kahan",
                   save_everystep=True, abstol=1e-7, reltol=1e-7, nthreads=8)
    assert np.array_equal(sol.offsets, ref["offsets"])
    assert np.array_equal(sol.ts_rows, ref["ts_rows"]) and np.array_equal(sol.us_rows, ref["us_rows"])


def test_chunked_host_path_equals_device_path(pkg):
    """Host buffers and at least 2 x 262,144 trajectories: the solve runs in
    chunks whose output copies overlap the next chunk's kernel.  Every output
    equals the unchunked device-buffer solve's."""
    import torch
    from conftest import lorenz_inputs
    n = 540000
    u0, p = lorenz_inputs(n, seed=71)
    sv = np.linspace(0, 2, 11)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 2.0), p[:, 0]), u0s=u0, ps=p)
    kw = dict(dt=0.1, abstol=1e-8, reltol=1e-6, saveat=sv, schedule="persistent")
    a = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, **kw)
    assert a.stats.launches >= 3  # three chunks
    L = pkg._lib
    h = pkg._handle(0)
    args = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 2.0), 0.1, 1e-8, 1e-6, sv, False, "fp64",
                         "persistent", 0, memory=L.MEM_DEVICE)
    du0, dp = torch.tensor(u0, device="cuda"), torch.tensor(p, device="cuda")
    args.u0, args.p = du0.data_ptr(), dp.data_ptr()
    outs = {"us": torch.empty((11, 3, n), dtype=torch.float64, device="cuda"),
            "u_final": torch.empty((3, n), dtype=torch.float64, device="cuda"),
            "naccept": torch.empty(n, dtype=torch.int32, device="cuda"),
            "retcode": torch.empty(n, dtype=torch.int8, device="cuda")}
    o = L.SolveOut()
    for k, v in outs.items():
        setattr(o, k, v.data_ptr())
    st = L.SolveStats()
    h.check(h.solve_raw(args, o, st), allow=(L.ETRAJ,))
    assert st.launches == 1
    assert np.array_equal(a.us, outs["us"].cpu().numpy())
    assert np.array_equal(a.u_final, outs["u_final"].cpu().numpy())
    assert np.array_equal(a.naccept, outs["naccept"].cpu().numpy())
    assert np.array_equal(a.retcode, outs["retcode"].cpu().numpy())


def test_asynchronous_device_solve_on_a_caller_stream(pkg):
    """Device buffers + the caller's stream + no stats: the call returns once
    the solve is enqueued; after a stream synchronize the results equal a
    synchronous solve's."""
    import torch
    from conftest import lorenz_inputs
    L = pkg._lib
    h = pkg._handle(0)
    n = 20000
    u0, p = lorenz_inputs(n, seed=81)
    sv = np.linspace(0, 5, 26)
    stream = torch.cuda.Stream()
    du0, dp = torch.tensor(u0, device="cuda"), torch.tensor(p, device="cuda")
    res = []
    for asynchronous in (True, False):
        a = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 5.0), 0.1, 1e-8, 1e-6, sv, False, "fp64",
                          "persistent", 0, memory=L.MEM_DEVICE)
        a.u0, a.p = du0.data_ptr(), dp.data_ptr()
        a.stream = stream.cuda_stream if asynchronous else None
        us = torch.empty((26, 3, n), dtype=torch.float64, device="cuda")
        uf = torch.empty((3, n), dtype=torch.float64, device="cuda")
        o = L.SolveOut()
        o.us, o.u_final = us.data_ptr(), uf.data_ptr()
        rc = h.solve_raw(a, o, None if asynchronous else L.SolveStats())
        assert rc == L.OK
        stream.synchronize()
        torch.cuda.synchronize()
        res.append((us.cpu(), uf.cpu()))
    assert torch.equal(res[0][0], res[1][0]) and torch.equal(res[0][1], res[1][1])


def test_user_output_unreached_points_are_nan_in_its_width(pkg):
    """Save points after tf are never reached: their rows are NaN in the
    output function's own width (2 here, not the state's 3), and every reached
    row equals the function of the full-state solve."""
    from conftest import lorenz_inputs
    u0, p = lorenz_inputs(500, seed=91)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 1.0), p[:, 0]), u0s=u0, ps=p)
    out = pkg.UserOutput("out[0] = u[0] + u[1];\n out[1] = u[2];", width=2)
    sv = np.array([0.0, 0.5, 1.0, 1.5, 2.0])
    for sched in ("plain", "persistent"):
        a = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=500, dt=0.1, saveat=sv, schedule=sched, output=out)
        b = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=500, dt=0.1, saveat=sv, schedule=sched)
        assert a.us.shape == (5, 2, 500)
        assert np.isnan(a.us[3:]).all()
        assert np.array_equal(a.us[:3, 0], b.us[:3, 0] + b.us[:3, 1]) and np.array_equal(a.us[:3, 1], b.us[:3, 2])


def test_tuning_cache_round_trip(pkg, tmp_path):
    """ode_autotune's choice saved to a file and loaded by a fresh handle: the
    fresh handle solves with the tuned variant (run-time compiled) without
    tuning, and the results are unchanged; malformed files are refused."""
    from conftest import lorenz_inputs
    L = pkg._lib
    n = 20000
    u0, p = lorenz_inputs(n, seed=111)
    sv = np.linspace(0, 5, 11)
    args = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 5.0), 0.1, 1e-8, 1e-6, sv, False, "fp64",
                         "persistent", 0)
    h1 = L.Handle(0)
    rep = h1.autotune(args, sample=8192)
    # a kernel built for another controller has its own key, and its choice travels too
    args32 = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 5.0), 0.1, 1e-8, 1e-6, sv, False, "fp64",
                           "persistent", 0, controller="fp32")
    h1.autotune(args32, sample=8192)
    path = tmp_path / "tune.txt"
    h1.tune_save(path)
    text = path.read_text().splitlines()
    assert text[0].startswith("gb300ode-tune 1 ") and len(text) == 3
    assert sum(line.split()[0].endswith("|c32") for line in text[1:]) == 1
    h2 = L.Handle(0)
    assert h2.tune_load(path) == L.OK
    outs = []
    for h in (h1, h2):
        us, uf = np.empty((11, 3, n)), np.empty((3, n))
        o = L.SolveOut()
        o.us, o.u_final = us.ctypes.data, uf.ctypes.data
        st = L.SolveStats()
        h.check(h.solve_raw(args, o, st), allow=(L.ETRAJ,))
        outs.append((us, uf, st.jit))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    if rep.block and rep.best_ms < rep.default_ms:
        assert outs[1][2] == 1  # the loaded shape was compiled at run time
    bad = tmp_path / "bad.txt"
    bad.write_text("gb300ode-tune 1 %s\natsit5|staged|0|3|fp64|0 33 0 12288\n" % text[0].split()[2])
    assert h2.tune_load(bad) == L.EINVAL
    other = tmp_path / "other.txt"
    other.write_text("gb300ode-tune 1 Some_Other_GPU/99\n")
    assert h2.tune_load(other) == L.ENOTSUP
    h1.close()
    h2.close()


@pytest.mark.parametrize("nsave", [151, 401, 2001])
def test_two_queue_staging_dense_saveat_bitexact(pkg, po, nsave):
    """The Verner two-queue staged kernel when steps hold several save points
    (about 62 steps per trajectory here): with 151 points (2.4 a step) the
    point queue fills and the warp makes room with partial rounds; with 401
    and 2001 points (6 and 32 a step) one iteration can bring more save points
    than the queue holds and the lanes interpolate those in place.  Every
    path gives the oracle's values."""
    rng = np.random.default_rng(nsave)
    n = 1024
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10), n))[None, :]
    u0 = rng.uniform(-2, 2, (2, n))
    sv = np.linspace(0, 20, nsave)
    sol = gpu(pkg, pkg.GPUSimpleAVern7(), "vanderpol", u0, mu, (0.0, 20.0), 0.1, abstol=1e-5, reltol=1e-4,
              saveat=sv, schedule="persistent")
    ref = po.solve("AVern7", "vanderpol", u0, mu, (0, 20), 0.1, rounding="device", abstol=1e-5, reltol=1e-4,
                   saveat=sv, nthreads=8)
    assert_bitexact(sol, ref)
    assert sol.stats.saves == n * (nsave - 1)  # interpolated points; saveat[0] = t0 is the initial state
