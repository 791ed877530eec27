"""Learned schedule and run-time compiled right-hand sides, on the GPU.

The plain one-thread-per-trajectory schedule is both the fallback and the
judge: ordering trajectories by predicted cost must not change any
trajectory's result (bit-identical), seeding dt0 must keep the adaptive
tolerance where the dynamics allow it and the accuracy everywhere, and the
trained network must beat the method without it on the cost it is meant to
reduce."""
import numpy as np
import pytest

from conftest import lorenz_inputs

pytestmark = pytest.mark.gpu

KW = dict(dt=0.1, abstol=1e-8, reltol=1e-6)


def ens(pkg, u0, p):
    return pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p)


@pytest.fixture(scope="module")
def fitted(pkg):
    u0, p = lorenz_inputs(65536, seed=101)
    rep = pkg.learn_fit(ens(pkg, u0, p), pkg.GPUSimpleATsit5(), 65536, **KW)
    return rep


def test_fit_quality(fitted):
    assert fitted.loss_last < 0.5 * fitted.loss_first
    assert fitted.r2_attempts > 0.8
    assert fitted.train_ctas in (8, 16) and 0 < fitted.train_kernel_ms < fitted.train_fit_ms


def test_training_is_deterministic_and_narrow_models_train(pkg):
    """The training cluster reduces every gradient in a fixed order, so two fits
    with the same seed give bit-identical predictions; a model narrower than
    the kernels' 64 units (zero-padded inside the kernel) trains as well."""
    u0, p = lorenz_inputs(8192, seed=111)
    h = pkg._handle(0)
    args = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 10.0), 0.1, 1e-8, 1e-6, None, False, "fp64",
                         "plain", 0)
    preds = []
    for _ in range(2):
        h.learn_fit(args, {"epochs": 10})
        preds.append(h.learn_predict(args, 8192))
    assert np.array_equal(preds[0][0], preds[1][0]) and np.array_equal(preds[0][1], preds[1][1])
    u1, p1 = lorenz_inputs(65536, seed=112)
    args1 = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u1, p1, (0.0, 10.0), 0.1, 1e-8, 1e-6, None, False, "fp64",
                          "plain", 0)
    rep = h.learn_fit(args1, {"hidden": 24})
    assert rep.r2_attempts > 0.8, rep.r2_attempts
    tr = lorenz_inputs(65536, seed=101)
    pkg.learn_fit(ens(pkg, *tr), pkg.GPUSimpleATsit5(), 65536, **KW)  # the module's model back for later tests


def warp_cost(att, order):
    a = att[order][: len(order) // 32 * 32].reshape(-1, 32)
    return a.max(1).sum()


def test_ordering_keeps_results_and_gains(pkg, fitted):
    n = 65536
    u0, p = lorenz_inputs(n, seed=202)
    e = ens(pkg, u0, p)
    plain = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, schedule="plain", **KW)
    # a caller-given dt0 disables seeding: only the order changes
    ordered = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, schedule="learned", dt0=np.full(n, 0.1), **KW)
    assert ordered.stats.schedule_used == 2
    assert np.array_equal(ordered.u_final, plain.u_final)
    assert np.array_equal(ordered.naccept, plain.naccept) and np.array_equal(ordered.nreject, plain.nreject)
    # what the ordering buys: warps of similar predicted cost waste fewer lane-attempts
    att = (plain.naccept + plain.nreject).astype(np.int64)
    h = pkg._handle(0)
    args = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 10.0), 0.1, 1e-8, 1e-6, None, False, "fp64",
                         "plain", 0)
    la, _ = h.learn_predict(args, n)
    learned_order = np.argsort(-la, kind="stable")
    identity = np.arange(n)
    ideal = np.argsort(-att, kind="stable")
    c_plain, c_learned, c_ideal = warp_cost(att, identity), warp_cost(att, learned_order), warp_cost(att, ideal)
    assert c_learned < 0.8 * c_plain, (c_plain, c_learned, c_ideal)
    assert np.corrcoef(la, np.log(att))[0, 1] > 0.9


def test_dt0_seeding_matches_accuracy_and_cuts_rejects(pkg, fitted):
    """Seeding dt0 changes each trajectory's step sequence.  Where the dynamics
    do not amplify perturbations (rho < 13.9: no chaos) the results stay within
    10x the error scale of the plain schedule's; everywhere the accuracy
    against a tight-tolerance solution is the same as the plain schedule's
    (chaotic trajectories carry global errors far above reltol in both)."""
    n = 65536
    u0, p = lorenz_inputs(n, seed=303)
    e = ens(pkg, u0, p)
    tr = lorenz_inputs(65536, seed=101)
    pkg.learn_fit(ens(pkg, *tr), pkg.GPUSimpleATsit5(), 65536, opts={"seed_dt0": 1}, **KW)
    try:
        plain = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, schedule="plain", **KW)
        seeded = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=n, schedule="learned", **KW)
        truth = pkg.solve(e, pkg.GPUSimpleAVern9(), trajectories=n, dt=0.01, abstol=1e-13, reltol=1e-13,
                          schedule="persistent")
    finally:
        pkg.learn_fit(ens(pkg, *tr), pkg.GPUSimpleATsit5(), 65536, **KW)
    scale = 1e-8 + 1e-6 * np.abs(truth.u_final).max(0)
    rho = p[1]
    calm = rho < 13.9
    d = np.abs(seeded.u_final - plain.u_final).max(0) / scale
    assert np.mean(d[calm] <= 10) >= 0.999
    ep = np.abs(plain.u_final - truth.u_final).max(0) / scale
    es = np.abs(seeded.u_final - truth.u_final).max(0) / scale
    for lo, hi in ((0, 13.9), (13.9, 24.7), (24.7, 30.0)):
        m = (rho >= lo) & (rho < hi)
        for q in (50, 90):
            a, b = np.percentile(ep[m], q), np.percentile(es[m], q)
            assert 0.75 * a <= b <= 1.33 * a, (lo, q, a, b)
    assert seeded.nreject.sum() < 0.5 * plain.nreject.sum()
    assert (seeded.naccept + seeded.nreject).sum() < (plain.naccept + plain.nreject).sum()


USER_LORENZ = """
du[0] = p[0] * (u[1] - u[0]);
du[1] = fma(u[0], p[1] - u[2], -u[1]);
du[2] = fma(u[0], u[1], -(p[2] * u[2]));
"""


@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_user_rhs_matches_builtin(pkg, schedule):
    n = 4096
    u0, p = lorenz_inputs(n, seed=404)
    sv = np.linspace(0, 10, 11)
    user = pkg.UserRHS(USER_LORENZ, 3, 3)
    a = pkg.solve(pkg.EnsembleProblem(pkg.ODEProblem(user, u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p),
                  pkg.GPUSimpleATsit5(), trajectories=n, saveat=sv, schedule=schedule, **KW)
    b = pkg.solve(ens(pkg, u0, p), pkg.GPUSimpleATsit5(), trajectories=n, saveat=sv, schedule=schedule, **KW)
    assert a.stats.jit == 1
    assert np.array_equal(a.u_final, b.u_final) and np.array_equal(a.us, b.us)


def test_user_rhs_compile_error_is_reported(pkg):
    bad = pkg.UserRHS("du[0] = undefined_symbol(u[0]);", 1, 0)
    with pytest.raises(pkg.GB300ODEError) as ei:
        pkg.solve(pkg.ODEProblem(bad, [1.0], (0.0, 1.0)), pkg.GPUSimpleATsit5())
    assert ei.value.code == -5
    assert "undefined_symbol" in str(ei.value)
