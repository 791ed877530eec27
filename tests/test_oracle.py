"""The CPU oracle against known answers and the reference's own tests.

The reference (Julia) cannot run here, so the oracle is pinned by:
  * analytic solutions: f(u) = -u (test/gpu_ode_regression.jl:2-9) and the
    2x2 linear system [2 3; 4 5] (test/simpleatsit5_tests.jl:87-93);
  * the reference's relational tests, restated: SimpleATsit5 == GPUSimpleATsit5
    (test/gpusimpleatsit5_tests.jl:35-39,49), SimpleTsit5 == GPUSimpleTsit5 on
    a chaotic Lorenz run to t = 100 (:59-67), the last fixed step landing on tf
    (test/simpletsit5_tests.jl:84-90), saveat lengths (test/gpu_ode_regression.jl:60-61,84-85),
    fixed vs adaptive agreement within the reference's tolerances (:35-36,57-58,81-82);
  * the committed golden fixtures (tests/golden/), regenerated by make_golden.py.
"""
import os
import sys

import numpy as np
import pytest

from conftest import decay_inputs, lorenz_inputs

ALGS = ["RK4", "Tsit5", "ATsit5", "Vern7", "AVern7", "Vern9", "AVern9"]


@pytest.mark.parametrize("alg", ALGS)
@pytest.mark.parametrize("rounding", ["ref", "device"])
def test_decay_known_answer(po, alg, rounding):
    u0, A = decay_inputs(2)
    kw = {} if alg == "RK4" else {"saveat": [0.0, 0.4, 1.0]}
    o = po.solve(alg, "linear", u0, A, (0, 1), 0.01, rounding=rounding, abstol=1e-10, reltol=1e-10, **kw)
    assert np.abs(o["u_final"] - np.exp(-1)).max() < (1e-10 if alg != "RK4" else 1e-9)
    assert (o["retcode"] == 0).all()
    if alg != "RK4":
        assert o["us"].shape[0] == 3  # length(sol.u) == length(saveat)
        assert np.array_equal(o["us"][0], u0)  # saveat[1] == t0 copies u0
        tol = 1e-4 if alg == "Vern9" else 1e-9  # fixed-step Vern9 keeps the reference's unrelabelled dense stages
        assert np.abs(o["us"][1] - np.exp(-0.4)).max() < tol


@pytest.mark.parametrize("adaptive,fixed", [("ATsit5", "Tsit5"), ("AVern7", "Vern7"), ("AVern9", "Vern9")])
def test_fp32_regression_pairs(po, adaptive, fixed):
    """test/gpu_ode_regression.jl in Float32: fixed dt=0.01 vs adaptive at 1f-7,
    against the exact solution in place of OrdinaryDiffEq's Vern9."""
    u0, A = decay_inputs(1)
    exact = np.exp(-1.0)
    s = po.solve(fixed, "linear", u0, A, (0, 1), 0.01, precision="fp32")
    a = po.solve(adaptive, "linear", u0, A, (0, 1), 0.01, precision="fp32", abstol=1e-7, reltol=1e-7)
    assert np.linalg.norm(s["u_final"][:, 0] - exact) < 5e-3
    assert np.linalg.norm(a["u_final"][:, 0] - exact) < 5e-4
    sv = np.array([0.0, 0.4], dtype=np.float32).astype(np.float64)
    s = po.solve(fixed, "linear", u0, A, (0, 1), 0.01, precision="fp32", saveat=sv)
    a = po.solve(adaptive, "linear", u0, A, (0, 1), 0.01, precision="fp32", abstol=1e-7, reltol=1e-7, saveat=sv)
    ex = np.exp(-sv)[:, None, None] * np.ones((2, 3, 1))
    assert np.linalg.norm(a["us"] - ex) < 2e-4
    assert np.linalg.norm(s["us"] - ex) < (2e-4 if fixed != "Vern9" else 2e-3)


def test_linear_2x2_interpolation(po):
    """test/simpleatsit5_tests.jl:86-112: du = [2 3; 4 5] u, u0 = (1, 1),
    abstol = reltol = 1e-6, dt = 0.1; here against the matrix exponential."""
    from scipy.linalg import expm
    M = np.array([[2.0, 3.0], [4.0, 5.0]])
    u0 = np.ones((2, 1))
    A = M.reshape(4, 1)
    sv = np.linspace(0, 1, 21)
    for alg in ("ATsit5", "SimpleATsit5"):
        o = po.solve(alg, "linear", u0, A, (0, 1), 0.1, abstol=1e-6, reltol=1e-6, saveat=sv)
        ex = np.stack([expm(M * t) @ u0[:, 0] for t in sv])
        rel = np.abs(o["us"][:, :, 0] - ex) / np.abs(ex)
        assert rel.max() < 2e-5


def test_simple_vs_gpu_atsit5_identical(po):
    """GPUSimpleATsit5 and SimpleATsit5 are the same algorithm (test/gpusimpleatsit5_tests.jl:35-39,49)."""
    u0 = np.full((3, 1), 10.0)
    p = np.array([[10.0], [28.0], [8 / 3]])
    for sv in (None, np.arange(0, 1001) * 0.1):
        a = po.solve("ATsit5", "lorenz", u0, p, (0, 100), 0.01, abstol=1e-6, reltol=1e-3, saveat=sv)
        b = po.solve("SimpleATsit5", "lorenz", u0, p, (0, 100), 0.01, abstol=1e-6, reltol=1e-3, saveat=sv)
        assert np.array_equal(a["u_final"], b["u_final"])
        assert np.array_equal(a["naccept"], b["naccept"])
        if sv is not None:
            assert np.array_equal(a["us"], b["us"], equal_nan=True)


def test_simple_vs_gpu_tsit5_identical_chaotic(po):
    """test/gpusimpleatsit5_tests.jl:54-67: SimpleTsit5 and GPUSimpleTsit5 agree
    on Lorenz over (0, 100) with dt = 0.1 although their update is grouped
    differently; with left-to-right @muladd accumulation they are identical."""
    u0 = np.full((3, 1), 10.0)
    p = np.array([[10.0], [28.0], [8 / 3]])
    a = po.solve("Tsit5", "lorenz", u0, p, (0, 100), 0.1)
    b = po.solve("SimpleTsit5", "lorenz", u0, p, (0, 100), 0.1)
    assert np.array_equal(a["u_final"], b["u_final"])
    c = po.solve("Tsit5", "lorenz", u0, p, (0, 100), 0.1, saveat=[5.0, 100.0])
    assert np.allclose(c["us"][1], a["u_final"], rtol=1e-12)  # sol.u[end] ≈ sol4.u[end] (:64-66)


def test_last_step_lands_on_tf(po):
    """test/simpletsit5_tests.jl:84-90: dt = 0.05/11 on (0, 0.05).  Julia's range
    0:dt:0.05 takes the literal path (Float64(1/220) != 0.05/11) and has 11
    points ending at 10*dt; SimpleTsit5 then adds a last partial step and its
    solution ends exactly at 0.05."""
    g = po.julia_range(0.0, 0.05 / 11, 0.05)
    assert len(g) == 11 and g[-1] == 10 * (0.05 / 11)
    u0 = np.ones((1, 1))
    o = po.solve("SimpleTsit5", "linear", u0, np.ones((1, 1)), (0, 0.05), 0.05 / 11)
    assert o["t_final"][0] == 0.05
    assert o["naccept"][0] == 12


def test_julia_ranges(po):
    assert len(po.julia_range(0, 0.01, 1)) == 101
    assert po.julia_range(0, 0.1, 1)[3] == 0.3          # the rational path rounds i/10 exactly
    assert list(po.julia_range(0, 0.3, 1)) == [0.0, 0.3, 0.6, 0.9]
    assert len(po.julia_range(0, 0.01, 1, "fp32")) == 101
    g = po.julia_range(0.0, 0.1, 100.0)
    assert len(g) == 1001 and g[-1] == 100.0


def test_rounding_modes_agree_within_parity_tolerance(po):
    """The device rounding canon (fused multiply-adds, double-single error norm
    and step-size factor) against the reference's rounding: identical
    accepted-step counts and every final state within the error scale abstol
    + reltol*|u|.  With the optional single-precision norm and controller
    (ODE_CTRL_FP32) the factor q carries 2^-24 relative rounding into every
    step size, which chaotic trajectories amplify: there the bar is steps
    within +/-1 and 10x the error scale for 99.9% of trajectories."""
    u0, p = lorenz_inputs(3000, seed=21)
    kw = dict(abstol=1e-8, reltol=1e-6, nthreads=8)
    a = po.solve("ATsit5", "lorenz", u0, p, (0, 10), 0.1, rounding="ref", **kw)
    scale = 1e-8 + 1e-6 * np.abs(a["u_final"]).max(0)
    b = po.solve("ATsit5", "lorenz", u0, p, (0, 10), 0.1, rounding="device", **kw)
    assert np.array_equal(a["naccept"], b["naccept"])
    err = np.abs(a["u_final"] - b["u_final"]).max(0) / scale
    assert err.max() <= 1, err.max()
    c = po.solve("ATsit5", "lorenz", u0, p, (0, 10), 0.1, rounding="device", controller="fp32", **kw)
    assert np.abs(a["naccept"] - c["naccept"]).max() <= 1
    err = np.abs(a["u_final"] - c["u_final"]).max(0) / scale
    assert np.mean(err <= 10) >= 0.999


def test_fixed_step_rounding_modes_1e12(po):
    """Fixed-step FP64 final states: device canon within 1e-12 relative of the
    reference rounding on the 8192-trajectory fixed Tsit5 Lorenz workload."""
    n = 8192
    rng = np.random.default_rng(11)
    u0 = np.tile(np.array([[1.0], [0.0], [0.0]]), (1, n))
    p = np.stack([np.full(n, 10.0), rng.uniform(0, 21, n), np.full(n, 8 / 3)])
    a = po.solve("Tsit5", "lorenz", u0, p, (0, 1), 0.01, rounding="ref", nthreads=8)
    b = po.solve("Tsit5", "lorenz", u0, p, (0, 1), 0.01, rounding="device", nthreads=8)
    rel = np.abs(a["u_final"] - b["u_final"]).max(0) / np.abs(a["u_final"]).max(0)
    assert rel.max() <= 1e-12


def test_ctrl_pow_accuracy(po):
    xs = np.concatenate([np.logspace(-40, 38, 400), [1.0, 0.5, 2.0, 1e-4, 3.0]]).astype(np.float32)
    for b in (0.14, 0.08):
        got = np.array([po.ctrl_pow(float(x), np.float32(b)) for x in xs])
        ref = xs.astype(np.float64) ** np.float64(np.float32(b))
        assert np.max(np.abs(got / ref - 1)) < 2e-6  # about 10 ulp across the whole float range
    assert po.ctrl_pow(0.0, 0.14) == 0.0
    assert np.isnan(po.ctrl_pow(float("nan"), 0.14))
    assert po.ctrl_pow(float("inf"), 0.14) == float("inf")


def test_dtmin_and_maxiters(po):
    u0, p = lorenz_inputs(4, seed=2)
    o = po.solve("ATsit5", "lorenz", u0, p, (0, 1), 0.1, abstol=0.0, reltol=1e-30)
    assert (o["retcode"] == 1).all()
    o = po.solve("ATsit5", "lorenz", u0, p, (0, 10), 0.1, abstol=1e-8, reltol=1e-6, maxiters=10)
    assert (o["retcode"] == 2).all() and ((o["naccept"] + o["nreject"]) == 10).all()


def test_nan_is_accepted_like_reference(po):
    """A NaN error estimate is not > 1, so the reference accepts the step and
    carries on; the trajectory finishes (flagged with retcode 3)."""
    u0 = np.array([[np.nan], [1.0], [1.0]])
    p = np.array([[10.0], [28.0], [8 / 3]])
    o = po.solve("ATsit5", "lorenz", u0, p, (0, 1), 0.1)
    assert o["retcode"][0] == 3 and o["t_final"][0] == 1.0
    assert np.isnan(o["u_final"]).all()
    for ctrl in ("ds", "fp64", "fp32"):  # the device canon ends the same way with every controller
        o = po.solve("ATsit5", "lorenz", u0, p, (0, 1), 0.1, rounding="device", controller=ctrl)
        assert o["retcode"][0] == 3 and o["t_final"][0] == 1.0, ctrl


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)


def test_golden_fixtures(po):
    import make_golden
    for name, case in make_golden.CASES.items():
        path = os.path.join(GOLDEN, name + ".npz")
        ref = np.load(path)
        out = make_golden.run_case(po, case, (ref["u0"], ref["p"]))
        for k in ("u_final", "naccept", "nreject", "retcode"):
            assert np.array_equal(out[k], ref[k], equal_nan=True), (name, k)
        if "us" in ref.files:
            assert np.array_equal(out["us"], ref["us"], equal_nan=True), name


def test_device_canon_sincos_accuracy(po):
    """The device canon's double sine and cosine (Cody-Waite reduction modulo
    pi/2, near-minimax polynomials on [-pi/4, pi/4]) against libm: within
    2 ulp below 2^19 (1.5 ulp of the exact value, measured with mpmath), an
    absolute error below 1e-30 where the result is tiny, and libm itself
    beyond 2^19 and for NaN."""
    rng = np.random.default_rng(1)
    for lo, hi, bound in ((0, np.pi, 2), (0, 1000, 2), (0, 5e5, 2)):
        x = rng.uniform(-hi, hi, 4000)
        got = np.array([po.sincos(v) for v in x])
        for col, fn in ((0, np.sin), (1, np.cos)):
            want = fn(x)
            ulp = np.abs(got[:, col] - want) / np.spacing(np.abs(want))
            assert ulp.max() <= bound, (hi, col, ulp.max())
    # near the zeros (x within 1e-15 of a multiple of pi/2) the two-part reduction keeps an absolute
    # error below 1e-30 rather than a relative one
    k = np.arange(-200, 200) * (np.pi / 2)
    got = np.array([po.sincos(v) for v in k])
    for col, fn in ((0, np.sin), (1, np.cos)):
        want = fn(k)
        err = np.abs(got[:, col] - want)
        assert ((err <= 2 * np.spacing(np.abs(want))) | (err <= 1e-30)).all()
    assert po.sincos(1e6) == (np.sin(1e6), np.cos(1e6))
    assert all(np.isnan(po.sincos(float("nan"))))


@pytest.mark.parametrize("rounding", ["ref", "device"])
def test_euler_known_answer_and_lorenz_stability(po, rounding):
    """GPUSimpleEuler (src/euler/gpueuler.jl): on f(u) = -u the discrete solution
    is (1 - dt)^k at every grid point; and the stability test of
    test/simpleeuler_tests.jl:40-60 (Lorenz from u0 = 10 ones, dt = 0.01,
    10,000 steps, no NaN)."""
    u0, A = decay_inputs(2)
    o = po.solve("Euler", "linear", u0, A, (0, 1), 0.01, rounding=rounding, save_everystep=True)
    k = np.arange(101)
    assert np.abs(o["us"][:, 0, 0] - 0.99 ** k).max() < 1e-14
    assert o["naccept"][0] == 100
    u0 = np.full((3, 1), 10.0)
    p = np.array([[10.0], [28.0], [8 / 3]])
    o = po.solve("Euler", "lorenz", u0, p, (0, 100.0), 0.01, rounding=rounding)
    assert np.isfinite(o["u_final"]).all() and o["naccept"][0] == 10000


def test_every_step_output_rows(po):
    """GPUSimpleATsit5's default save_everystep = true without saveat
    (src/tsit5/gpuatsit5.jl:225-229, :301-303): t0/u0, then the time and state
    after each accepted step.  Restated from test/gpusimpleatsit5_tests.jl:28-39:
    the last time equals the save_everystep = false solve's final time."""
    u0 = np.full((3, 1), 10.0)
    p = np.array([[10.0], [28.0], [8 / 3]])
    kw = dict(abstol=1e-6, reltol=1e-3)
    ev = po.solve("ATsit5", "lorenz", u0, p, (0, 100), 1e-2, save_everystep=True, **kw)
    fin = po.solve("ATsit5", "lorenz", u0, p, (0, 100), 1e-2, **kw)
    off, ts, us = ev["offsets"], ev["ts_rows"], ev["us_rows"]
    assert off[1] == ev["naccept"][0] + 1
    assert ts[0] == 0.0 and np.array_equal(us[0], u0[:, 0])
    assert ts[-1] == fin["t_final"][0] == 100.0
    assert np.array_equal(us[-1], fin["u_final"][:, 0])
    assert (np.diff(ts) > 0).all()
    # the Verner solvers too (gpuvern7.jl:428-430, gpuvern9.jl:597-599), in both rounding modes:
    # one row per accepted step plus u0, the last row the final state
    for alg, rhs, u, pp, tsp in (("AVern7", "vanderpol", np.array([[2.0], [0.0]]), np.array([[1.5]]), (0, 5)),
                                 ("AVern9", "r3bp", np.array([[0.994], [0.0], [0.0], [-2.00158510637908]]),
                                  np.array([[0.012277471]]), (0, 1))):
        for rounding in ("ref", "device"):
            e = po.solve(alg, rhs, u, pp, tsp, 0.1, rounding=rounding, save_everystep=True, abstol=1e-9, reltol=1e-9)
            f = po.solve(alg, rhs, u, pp, tsp, 0.1, rounding=rounding, abstol=1e-9, reltol=1e-9)
            assert len(e["ts_rows"]) == f["naccept"][0] + 1
            assert np.array_equal(e["us_rows"][-1], f["u_final"][:, 0])


# ---------------------------------------------------------------- SimpleEM
def test_philox_known_answers(po):
    """Philox4x32-10 against the known-answer vectors published with the
    Random123 library (Salmon et al., SC'11): zero, all-ones and pi-digit
    counter/key pairs."""
    assert po.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert po.philox([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert po.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_device_canon_log_accuracy(po):
    """The table-driven logarithm of the normal generator: within 2 ulp, except
    in the table's last interval below 1, [1 - 2^-8, 1), where its result
    (below 2^-8 in size) is the sum of two terms of that size and the error is
    bounded absolutely, by 2^-60 (log x for x = 1 - 2^-53 is -1.1e-16)."""
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(2.0 ** -53, 1.0, 4000), np.exp(rng.uniform(-700, 700, 2000)),
                        1.0 - rng.uniform(0, 2.0 ** -8, 1000), 1.0 + rng.uniform(0, 2.0 ** -7, 1000),
                        [2.0 ** -53, 0.5, 1.0 - 2.0 ** -53, np.sqrt(2.0), 2.0 ** -1022, 1.4140625, 2.0 - 2.0 ** -52]])
    got = np.array([po.log_dev(v) for v in x])
    want = np.log(x)
    assert po.log_dev(1.0) == 0.0
    nz = want != 0
    err = np.abs(got[nz] - want[nz])
    last = (x[nz] >= 1.0 - 2.0 ** -8) & (x[nz] < 1.0)
    assert (err[~last] / np.spacing(np.abs(want[nz][~last]))).max() <= 2
    assert err[last].max() <= 2.0 ** -60


def test_log_table_is_the_generator_output():
    """csrc/log_table.h is what csrc/gen_logtab.py writes (60-digit mpmath)."""
    pytest.importorskip("mpmath")
    import importlib.util
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "simplediffeq.jl_gb300", "csrc")
    spec = importlib.util.spec_from_file_location("gen_logtab", os.path.join(here, "gen_logtab.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    assert open(os.path.join(here, "log_table.h")).read() == mod.header()


def test_counter_based_normals(po):
    """Box-Muller pairs from Philox: standard normal moments, uncorrelated
    components, and a stream that depends only on (seed, pair, trajectory)."""
    z = np.array([po.normal_pair(7, P, i) for P in range(200) for i in range(250)])
    for col in (z[:, 0], z[:, 1]):
        assert abs(col.mean()) < 0.02 and abs(col.var() - 1) < 0.03
        assert abs(((col - col.mean()) ** 4).mean() / col.var() ** 2 - 3) < 0.15
    assert abs(np.corrcoef(z[:, 0], z[:, 1])[0, 1]) < 0.02
    assert po.normal_pair(7, 3, 9) == po.normal_pair(7, 3, 9) != po.normal_pair(8, 3, 9)
    assert po.normal_pair(7, 3, 9) != po.normal_pair(7, 3 + (1 << 32), 9)  # the pair index's high word counts


def test_normals_are_box_muller_of_the_philox_uniforms(po):
    """The double-single normals against the exact Box-Muller transform of the
    same 53-bit uniforms (40-digit values): within 2^-42 of max(1, r)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    seed = 7
    worst = 0
    for P in range(0, 400, 3):
        for i in (0, 1, 12345, (1 << 33) + 5):
            r = po.philox([P & 0xffffffff, P >> 32, i & 0xffffffff, i >> 32], [seed, 0])
            a = ((r[0] >> 5) << 26) | (r[1] >> 6)
            c = ((r[2] >> 5) << 26) | (r[3] >> 6)
            rad = mp.sqrt(-2 * mp.log(mp.mpf(a + 1) / 2 ** 53))
            ang = 2 * mp.pi * mp.mpf(c) / 2 ** 53
            g0, g1 = po.normal_pair(seed, P, i)
            err = max(abs(mp.mpf(g0) - rad * mp.cos(ang)), abs(mp.mpf(g1) - rad * mp.sin(ang))) / max(1, rad)
            worst = max(worst, err)
    assert worst < mp.mpf(2) ** -42, float(worst)


@pytest.mark.parametrize("dim", [1, 2, 3, 5])
def test_simple_em_consumes_the_normal_stream_in_order(po, dim):
    """Step k of a dim-D SDE takes normals z_{kD} .. z_{kD+D-1} of its
    trajectory's stream; for odd D a pair straddles two steps and is drawn once.
    With dW-only Ornstein-Uhlenbeck noise (theta = 0, sigma = 1, dt = 1) each
    increment is the normal itself."""
    n, steps = 3, 6
    o = po.sde_solve("ou", np.zeros((dim, n)), np.tile([[0.0], [0.0], [1.0]], (1, n)), (0.0, float(steps)), 1.0,
                     seed=11, save_everystep=True)
    inc = np.diff(o["us"], axis=0)  # (steps, dim, n)
    for i in range(n):
        stream = [z for P in range((steps * dim + 1) // 2) for z in po.normal_pair(11, P, i)]
        want = np.array(stream[:steps * dim]).reshape(steps, dim)
        assert np.allclose(inc[:, :, i], want, rtol=0, atol=1e-12)


def test_simple_em_weak_moments(po):
    """The reference's example SDE du = 0.1u dt + 0.2u dW, u0 = 1 on (0, 1),
    dt = 0.01 (src/euler_maruyama.jl docstring): Euler-Maruyama's exact mean
    is (1 + 0.1 dt)^100; and an Ornstein-Uhlenbeck ensemble's variance against
    the EM recursion's exact value sigma^2 dt sum (1 - theta dt)^(2k)."""
    n = 20000
    o = po.sde_solve("gbm", np.ones((1, n)), np.tile([[0.1], [0.2]], (1, n)), (0.0, 1.0), 0.01, seed=1,
                     save_everystep=False, nthreads=8)
    m = o["u_final"].mean()
    sd = np.sqrt(np.exp(0.2) * (np.exp(0.04) - 1) / n)
    assert abs(m - 1.001 ** 100) < 4 * sd
    th, sig, dt = 1.0, 0.5, 0.01
    o = po.sde_solve("ou", np.zeros((1, n)), np.tile([[th], [0.0], [sig]], (1, n)), (0.0, 10.0), dt, seed=2,
                     save_everystep=True, nthreads=8)
    exact = sig ** 2 * dt * sum((1 - th * dt) ** (2 * k) for k in range(1000))
    v = o["u_final"].var()
    assert abs(v - exact) < 5 * exact * np.sqrt(2.0 / n)
    assert o["us"].shape == (1001, 1, n) and np.array_equal(o["us"][0], np.zeros((1, n)))
    assert o["t"][-1] == 10.0


def test_simple_em_non_diagonal_noise(po):
    """Non-diagonal noise (src/euler_maruyama.jl:126-134): the reference's test
    SDE (test/simpleem_tests.jl) f = 1.01u, G = [0.3 0.6 0.9 0.12; 1.2 0.2 0.3 1.8] .* u,
    a 2 x 4 noise matrix, u0 = ones(2), dt = 0.25 on (0, 1): five points per
    trajectory, EM's exact mean (1 + 1.01 dt)^4 (the noise has mean zero), and
    with one noise dimension the same path as diagonal GBM up to rounding."""
    n = 40000
    c = np.array([[0.3, 0.6, 0.9, 0.12], [1.2, 0.2, 0.3, 1.8]])
    p = np.tile(np.concatenate([[1.01], c.ravel()])[:, None], (1, n))
    o = po.sde_solve("mult", np.ones((2, n)), p, (0.0, 1.0), 0.25, seed=5, noise_dim=4, nthreads=8)
    assert o["us"].shape == (5, 2, n) and len(o["t"]) == 5
    # per component the EM factor is prod_k (1 + 1.01 dt + sqrt(dt) c_d . xi_k): mean (1 + 1.01 dt)^4
    var1 = (1 + 1.01 * 0.25) ** 2 + 0.25 * (c ** 2).sum(axis=1)
    sd = np.sqrt(var1 ** 4 - (1 + 1.01 * 0.25) ** 8) / np.sqrt(n)
    assert np.all(np.abs(o["u_final"].mean(axis=1) - (1 + 1.01 * 0.25) ** 4) < 5 * sd)
    # the two components share the four normals of a step: their increments correlate as c0 . c1 says
    inc = np.diff(o["us"][:2], axis=0)[0]
    rho = (c[0] @ c[1]) / np.sqrt((c[0] @ c[0]) * (c[1] @ c[1]))
    assert abs(np.corrcoef(inc[0], inc[1])[0, 1] - rho) < 0.02
    # one noise dimension: the diagonal GBM path, up to the rounding of sqdt (g xi) against (sqdt g) xi
    m = 2000
    a = po.sde_solve("mult", np.ones((1, m)), np.tile([[0.1], [0.2]], (1, m)), (0.0, 1.0), 0.01, seed=9,
                     noise_dim=1, save_everystep=False)
    b = po.sde_solve("gbm", np.ones((1, m)), np.tile([[0.1], [0.2]], (1, m)), (0.0, 1.0), 0.01, seed=9,
                     save_everystep=False)
    assert np.allclose(a["u_final"], b["u_final"], rtol=1e-13, atol=0)
    with pytest.raises(ValueError):
        po.sde_solve("mult", np.ones((2, 4)), np.ones((9, 4)), (0.0, 1.0), 0.25, seed=1, noise_dim=3)


def test_simple_em_rounding_modes_and_grid(po):
    u0 = np.array([[1.0], [1.0], [1.0]])
    p = np.array([[10.0], [28.0], [8 / 3], [0.1]])
    a = po.sde_solve("lorenz", u0, p, (0.0, 0.5), 0.001, seed=3, rounding="ref", save_everystep=False)
    b = po.sde_solve("lorenz", u0, p, (0.0, 0.5), 0.001, seed=3, rounding="device", save_everystep=False)
    assert np.abs(a["u_final"] - b["u_final"]).max() < 1e-9
    with pytest.raises(ValueError):
        po.sde_grid_steps(0.0, 1.0, 0.3)  # Int((tf - t0)/dt) throws InexactError in the reference


@pytest.mark.parametrize("alg,rhs,tol,tspan", [("AVern7", "vanderpol", 1e-8, (0, 20)),
                                               ("ATsit5", "kuramoto", 1e-6, (0, 50))])
def test_device_canon_within_parity_tolerance_of_reference_rounding(po, alg, rhs, tol, tspan):
    """The adaptive workloads: the device canon (which the GPU reproduces bit
    for bit) against the reference's rounding, every final state within 10x
    the error scale abstol + reltol*|u| and accepted steps within +/-1 for
    >= 99.9% of trajectories (Van der Pol's step sequences sit at its
    stability boundary, where last-bit differences of the fused stage sums
    flip accept/reject: 9 of 524,288 trajectories differ by 2-3 steps)."""
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    if rhs == "vanderpol":
        u0, p = make_golden.vdp(1000, 31)
        abstol = 1e-10
    else:
        u0, p = make_golden.kuramoto(400, 33)
        abstol = 1e-8
    kw = dict(abstol=abstol, reltol=tol, nthreads=8)
    a = po.solve(alg, rhs, u0, p, tspan, 0.1, rounding="ref", **kw)
    b = po.solve(alg, rhs, u0, p, tspan, 0.1, rounding="device", **kw)
    ok = (a["retcode"] == 0) & (b["retcode"] == 0)
    assert ok.mean() > 0.98
    scale = abstol + tol * np.abs(a["u_final"][:, ok]).max(0)
    err = np.abs(a["u_final"][:, ok] - b["u_final"][:, ok]).max(0) / scale
    assert err.max() <= 10, err.max()
    assert np.mean(np.abs(a["naccept"][ok] - b["naccept"][ok]) <= 1) >= 0.999


def test_arenstorf_fp64_matched_accuracy_of_both_roundings(po):
    """AVern9 on the Arenstorf orbit at abstol = reltol = 1e-12: the orbit's
    close approaches amplify last-bit rounding differences so much that even
    two 1e-15 solves in the two roundings differ by ~3e-10, so trajectory-wise
    agreement within 10x the tolerance is out of reach for any two correct
    implementations.  What must match is the accuracy: both roundings' errors
    against a 1e-15 solution have the same median and maximum (within 1.5x)."""
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    u0, p = make_golden.r3bp(500, 32)
    span = (0, make_golden.T_ARENSTORF)
    a = po.solve("AVern9", "r3bp", u0, p, span, 0.1, rounding="ref", abstol=1e-12, reltol=1e-12, nthreads=8)
    b = po.solve("AVern9", "r3bp", u0, p, span, 0.1, rounding="device", abstol=1e-12, reltol=1e-12, nthreads=8)
    t = po.solve("AVern9", "r3bp", u0, p, span, 0.1, rounding="ref", abstol=1e-15, reltol=1e-15, nthreads=8)
    ea = np.abs(a["u_final"] - t["u_final"]).max(0)
    eb = np.abs(b["u_final"] - t["u_final"]).max(0)
    for f in (np.median, np.max):
        assert f(eb) < 1.5 * f(ea) and f(ea) < 1.5 * f(eb)
    assert np.mean(np.abs(a["naccept"] - b["naccept"]) <= 2) >= 0.99


ARENSTORF_MU = 0.012277471
ARENSTORF_U0 = [0.994, 0.0, 0.0, -2.00158510637908252240537862224]
ARENSTORF_T = 17.0652165601579625588917206249


@pytest.mark.parametrize("alg,loose,tight,bound,est_order", [("AVern9", 1e-10, 1e-13, 1e-9, 9),
                                                            ("ATsit5", 1e-10, 1e-12, 2e-9, 5),
                                                            ("AVern7", 1e-10, 1e-13, 5e-10, 7)])
def test_arenstorf_orbit_closes_after_one_period(po, alg, loose, tight, bound, est_order):
    """A published known answer, independent of the oracle's own fixtures: the
    Arenstorf orbit of the restricted three-body problem (Hairer, Norsett and
    Wanner, Solving ODEs I, section II.0: mu = 0.012277471, u0 = (0.994, 0, 0,
    -2.00158510637908252240537862224)) is periodic with period
    T = 17.0652165601579625588917206249, so the state at T returns to u0.  In
    the reference's rounding the solvers close the orbit to the bound, and the
    accepted-step counts at two tolerances scale as tol^(-1/q) for the order q
    of the error estimate (Tsit5 5(4): q = 5, Vern7 7(6): 7, Vern9 9(8): 9), as
    they do only with correct coefficients and stage order."""
    u0 = np.array(ARENSTORF_U0)[:, None]
    p = np.array([[ARENSTORF_MU]])
    r = {}
    for tol in (loose, tight):
        r[tol] = po.solve(alg, "r3bp", u0, p, (0.0, ARENSTORF_T), 0.01, rounding="ref", abstol=tol, reltol=tol)
        assert r[tol]["retcode"][0] == 0
    err = np.abs(r[tight]["u_final"][:, 0] - u0[:, 0]).max()
    assert err < bound, err
    assert err < np.abs(r[loose]["u_final"][:, 0] - u0[:, 0]).max()
    ratio = r[tight]["naccept"][0] / r[loose]["naccept"][0]
    expected = (loose / tight) ** (1.0 / est_order)
    assert abs(ratio / expected - 1) < 0.15, (ratio, expected)


def test_device_canon_exp_accuracy(po):
    """The table-driven exponential of the FP64 step-size controller: within
    1 ulp over the controller's range and beyond (|x| < 700), against values
    computed in 40-digit arithmetic."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.uniform(-3, 3, 3000), rng.uniform(-700, 700, 1000), [0.0, -0.0, 1e-300, 0.5, -2.3025]])
    got = np.array([po.exp_dev(v) for v in x])
    want = np.array([float(mp.exp(mp.mpf(float(v)))) for v in x])
    assert po.exp_dev(0.0) == 1.0
    assert (np.abs(got - want) / np.spacing(want)).max() <= 1


def test_exp_table_is_the_generator_output():
    """csrc/exp_table.h is what csrc/gen_exptab.py writes (60-digit mpmath)."""
    pytest.importorskip("mpmath")
    import importlib.util
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "simplediffeq.jl_gb300", "csrc")
    spec = importlib.util.spec_from_file_location("gen_exptab", os.path.join(here, "gen_exptab.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    assert gen.header() == open(os.path.join(here, "exp_table.h")).read()


@pytest.mark.parametrize("controller", ["ds", "fp64"])
@pytest.mark.parametrize("alg,rhs", [("ATsit5", "lorenz"), ("AVern7", "vanderpol")])
def test_controllers_follow_reference_step_sizes(po, alg, rhs, controller):
    """With the double-single norm and controller (the default) or the FP64
    controller the device canon's step sequence follows the reference
    rounding's: on the benchmark ensembles' first 8,192 trajectories
    (adaptive Lorenz, Van der Pol) every accepted-step count is within +/-1
    (the default: Lorenz identical) and every final state within the error
    scale (10x for the FP64 controller, whose single-precision norm still
    rounds to 2^-24), where the single-precision controller's factor q
    carries 2^-24 relative rounding into every step size (chaotic Lorenz
    trajectories then drift beyond the bar: 21 of 1,048,576 at up to 559x).
    The Arenstorf orbit at 1e-12 is excluded: there fused and unfused stage
    sums alone separate the solutions (see the matched-accuracy test)."""
    import bench
    cid = {"lorenz": 2, "vanderpol": 3}[rhs]
    cfg = bench.CONFIGS[cid]
    m = 8192
    u0, p = cfg["inputs"](cfg["n"], 2024)
    u0, p = np.ascontiguousarray(u0[:, :m]), np.ascontiguousarray(p[:, :m])
    tol = (cfg["abstol"], cfg["reltol"])
    kw = dict(abstol=tol[0], reltol=tol[1], nthreads=8)
    ref = po.solve(alg, rhs, u0, p, cfg["tspan"], cfg["dt"], rounding="ref", **kw)
    dev = po.solve(alg, rhs, u0, p, cfg["tspan"], cfg["dt"], rounding="device", controller=controller, **kw)
    ok = (ref["retcode"] == 0) & (dev["retcode"] == 0)
    assert ok.mean() > 0.99
    dn = np.abs(dev["naccept"].astype(np.int64) - ref["naccept"])[ok]
    assert dn.max() <= (0 if (controller == "ds" and rhs == "lorenz") else 1)
    scale = tol[0] + tol[1] * np.abs(ref["u_final"]).max(0)
    e = (np.abs(dev["u_final"] - ref["u_final"]).max(0) / scale)[ok]
    assert e.max() <= (1 if controller == "ds" else 10), e.max()


def test_double_single_functions(po):
    """The double-single norm's and controller's building blocks against
    40-digit values: ds_split holds a double to 2^-47 relative (2^-74 <= |x|
    < 2^128), ds_log is within 2^-45 absolute where |ln a| < 2 and 2^-40 over
    the whole range 2^-120 .. 2^126, ds_exp within 2^-45 relative on the
    controller's arguments (|x| < 2.4)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(6)

    def val(pair):
        return mp.mpf(float(pair[0])) + mp.mpf(float(pair[1]))

    def pair(x):
        h = np.float32(x)
        return h, np.float32(x - float(h))
    for x in np.concatenate([rng.uniform(-1e3, 1e3, 500), 10 ** rng.uniform(-22, 38, 1000),
                             -(10 ** rng.uniform(-20, 20, 200))]):
        assert abs(val(po.ds("split", x)) - mp.mpf(x)) <= abs(mp.mpf(x)) * mp.mpf(2) ** -47, x
    assert po.ds("split", 0.0) == (0.0, 0.0) and np.isinf(po.ds("split", 4e38)[0])
    assert np.isnan(po.ds("split", float("nan"))[0])
    for e in np.concatenate([rng.uniform(-120, 126, 800), rng.uniform(-2.8, 2.8, 800), [0.0]]):
        h, l = pair(2.0 ** e)
        exact = mp.log(val((h, l)))
        bound = mp.mpf(2) ** (-45 if abs(exact) < 2 else -40)
        assert abs(val(po.ds("log", h, l)) - exact) <= bound, e
    for x in np.concatenate([rng.uniform(-2.4, 2.4, 1500), rng.uniform(-1e-3, 1e-3, 200), [0.0]]):
        h, l = pair(x)
        exact = mp.exp(val((h, l)))
        assert abs(val(po.ds("exp", h, l)) - exact) <= exact * mp.mpf(2) ** -45, x
    assert np.isnan(po.ds("exp", float("nan"))[0])


@pytest.mark.parametrize("abstol,reltol", [(1e-25, 1e-10), (1e-32, 1e-10), (1e-3, 1e-3), (1e-12, 1e-12)])
def test_double_single_norm_across_tolerances(po, abstol, reltol):
    """The double-single norm keeps the reference's step sequence from loose to
    very tight tolerances: abstol 1e-25 (the norm's terms near the single
    exponent range's edge), 1e-32 (below 1e-30, where the norm is computed
    in double), 1e-3 and 1e-12 -- identical accepted-step counts and final
    states within a tenth of the error scale on 200 Lorenz trajectories."""
    u0, p = lorenz_inputs(200, seed=5)
    kw = dict(abstol=abstol, reltol=reltol, nthreads=8)
    a = po.solve("ATsit5", "lorenz", u0, p, (0, 1), 0.1, rounding="ref", **kw)
    b = po.solve("ATsit5", "lorenz", u0, p, (0, 1), 0.1, rounding="device", **kw)
    assert np.array_equal(a["naccept"], b["naccept"])
    scale = abstol + reltol * np.abs(a["u_final"]).max(0)
    assert (np.abs(a["u_final"] - b["u_final"]).max(0) / scale).max() < 0.1


def test_ds_table_is_the_generator_output():
    """csrc/ds_table.h is what csrc/gen_dstab.py writes (60-digit mpmath)."""
    pytest.importorskip("mpmath")
    import importlib.util
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "simplediffeq.jl_gb300", "csrc")
    spec = importlib.util.spec_from_file_location("gen_dstab", os.path.join(here, "gen_dstab.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    assert gen.header() == open(os.path.join(here, "ds_table.h")).read()


def test_single_precision_r3bp_pull_accuracy(po):
    """The single-precision R3BP right-hand side takes mu / r^(3/2) as mu * y^3
    with y = 1/sqrt(r) from Lomont's bit-level seed and three Newton steps:
    within 8 float ulps of the exact value (measured: 6) over the squared
    radii an Arenstorf orbit visits (1e-6 .. 10) and beyond (1e-12 .. 1e12)."""
    rng = np.random.default_rng(8)
    r = np.concatenate([10.0 ** rng.uniform(-6, 1, 4000), 10.0 ** rng.uniform(-12, 12, 1000)]).astype(np.float32)
    mu = np.float32(0.987722529)
    got = np.array([po.r3bp_pull_f(mu, float(v)) for v in r], dtype=np.float32)
    want = float(mu) / r.astype(np.float64) ** 1.5
    ulp = np.spacing(want.astype(np.float32)).astype(np.float64)
    assert (np.abs(got.astype(np.float64) - want) / ulp).max() <= 8


def test_single_precision_controller_functions(po):
    """The division-free reciprocal, log2 and exp2 of the single-precision
    modes' error norm and controller: 1/d within 2 ulp, log2 within 3e-7
    absolute plus one ulp of the result (an error d in log2 EEst moves the
    factor EEst^beta by beta d ln 2 relative, so absolute accuracy is what
    counts), 2^y within 3 ulp on the controller's range; log2 of 0 and of
    subnormals finite and below -120."""
    rng = np.random.default_rng(9)
    d = (10.0 ** rng.uniform(-30, 30, 3000)).astype(np.float32)
    got = np.array([po.fp32_ctrl("rcp_nr", v) for v in d], dtype=np.float32).astype(np.float64)
    want = 1.0 / d.astype(np.float64)
    assert (np.abs(got - want) / np.spacing(want.astype(np.float32))).max() <= 2
    x = np.concatenate([(10.0 ** rng.uniform(-37, 37, 3000)), rng.uniform(0.5, 2.0, 2000)]).astype(np.float32)
    got = np.array([po.fp32_ctrl("log2_nr", v) for v in x], dtype=np.float64)
    want = np.log2(x.astype(np.float64))
    assert (np.abs(got - want) <= 3e-7 + np.spacing(np.abs(want).astype(np.float32))).all()
    assert -130 < po.fp32_ctrl("log2_nr", 0.0) < -120 and -150 < po.fp32_ctrl("log2_nr", 1e-40) < -120
    y = rng.uniform(-20, 20, 3000).astype(np.float32)
    got = np.array([po.fp32_ctrl("exp2_nr", v) for v in y], dtype=np.float64)
    want = 2.0 ** y.astype(np.float64)
    assert (np.abs(got - want) / np.spacing(want.astype(np.float32))).max() <= 3


def test_bench_parity_block_against_reference_rounding(po):
    """bench.py's parity_vs_ref on a small sample: the oracle's device canon
    stands in for the GPU (the GPU reproduces it bit for bit), and the block
    reports the fractions and extremes it promises."""
    import bench
    cfg = dict(bench.CONFIGS[2])
    u0, p = cfg["inputs"](300, 5)
    sv = np.linspace(*cfg["tspan"], cfg["nsave"])
    dev = po.solve("ATsit5", "lorenz", u0, p, cfg["tspan"], cfg["dt"], rounding="device", abstol=cfg["abstol"],
                   reltol=cfg["reltol"], saveat=sv, nthreads=4)
    out = bench.parity_vs_ref(cfg, u0, p, sv, {"u_final": dev["u_final"], "naccept": dev["naccept"],
                                                "us": dev["us"]}, m=300)
    assert out["trajectories"] == 300
    assert out["final_frac_within_10x"] == 1.0 and out["saveat_frac_within_10x"] == 1.0
    assert out["naccept_max_abs_diff"] <= 1 and 0 <= out["final_max_in_error_scale"] < 10
