"""Bounds-check mode (ode_set_bounds_check): the kernels recompiled with an
index check before every access to a caller array and a per-trajectory start
counter.  Every schedule and path reports no violation, every trajectory is
started exactly once (the persistent work counter hands each out once), and
the results equal those of the unchecked kernels."""
import numpy as np
import pytest

from conftest import lorenz_inputs

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked(pkg):
    h = pkg._lib.Handle(0)
    h.set_bounds_check(True)
    yield h
    h.close()


def _solve(pkg, h, alg, sched, u0, p, tspan, sv, every=False, output="state"):
    L = pkg._lib
    n = u0.shape[1]
    oid = pkg._output_id(h, output, 3, 3)
    a = pkg.make_args(alg, 0, u0, p, tspan, 0.1 if alg.adaptive else 0.01, 1e-8, 1e-6, sv, every, "fp64", sched, 0,
                      output=oid)
    width = output.width if isinstance(output, pkg.UserOutput) else 3
    npts = len(sv) if sv is not None else (len(pkg.fixed_grid(tspan[0], 0.01, tspan[1])) if every else 0)
    outs = {"u_final": np.empty((3, n)), "naccept": np.empty(n, dtype=np.int32),
            "retcode": np.empty(n, dtype=np.int8)}
    if npts:
        outs["us"] = np.empty((npts, width, n))
    o = L.SolveOut()
    for k, v in outs.items():
        setattr(o, k, v.ctypes.data)
    rc = h.solve_raw(a, o, L.SolveStats())
    return rc, outs


@pytest.mark.parametrize("alg,sched", [("ATsit5", "plain"), ("ATsit5", "persistent"), ("AVern7", "persistent"),
                                       ("AVern9", "persistent"), ("Tsit5", "plain"), ("RK4", "plain"),
                                       ("Euler", "plain")])
def test_no_violation_and_same_results(pkg, checked, alg, sched):
    L = pkg._lib
    u0, p = lorenz_inputs(3000, seed=101)
    algo = getattr(pkg, "GPUSimple" + alg)()
    fixed = alg in ("Tsit5", "RK4", "Euler")
    sv = None if alg in ("RK4", "Euler") else np.linspace(0, 2, 17)
    every = alg in ("RK4", "Euler")
    rc, a = _solve(pkg, checked, algo, sched, u0, p, (0.0, 2.0), sv, every)
    assert rc in (L.OK, L.ETRAJ), checked.error()
    rc2, b = _solve(pkg, pkg._handle(0), algo, sched, u0, p, (0.0, 2.0), sv, every)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    assert not fixed or (a["naccept"] == 200).all()


@pytest.mark.parametrize("n", [1000, 3000])
def test_no_violation_component_split_kernel(pkg, checked, n):
    """Fixed-step Tsit5 with every-step output on a small FP64 ensemble runs the
    component-split kernel in bounds-check mode too: no violation, every
    trajectory started once (counted by the block's first warp), results
    equal to the unchecked kernel's."""
    L = pkg._lib
    u0, p = lorenz_inputs(n, seed=103)
    rc, a = _solve(pkg, checked, pkg.GPUSimpleTsit5(), "plain", u0, p, (0.0, 1.0), None, every=True)
    assert rc == L.OK, checked.error()
    rc2, b = _solve(pkg, pkg._handle(0), pkg.GPUSimpleTsit5(), "plain", u0, p, (0.0, 1.0), None, every=True)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
    a2 = pkg.make_args(pkg.GPUSimpleTsit5(), 0, u0, p, (0.0, 1.0), 0.01, 1e-8, 1e-6, None, True, "fp64", "plain", 0)
    us = np.empty((101, 3, n))
    o = L.SolveOut()
    o.us = us.ctypes.data
    st = L.SolveStats()
    assert checked.solve_raw(a2, o, st) == L.OK, checked.error()
    assert L.KERNEL[st.kernel] == "fixedsplit"


def test_no_violation_every_step_and_user_output(pkg, checked):
    L = pkg._lib
    u0, p = lorenz_inputs(2000, seed=102)
    out = pkg.UserOutput("out[0] = u[0] * u[1];", width=1)
    sv = np.array([0.0, 1.0, 3.0])  # the last point is never reached: NaN rows in width 1
    rc, a = _solve(pkg, checked, pkg.GPUSimpleATsit5(), "persistent", u0, p, (0.0, 2.0), sv, output=out)
    assert rc == L.OK, checked.error()
    assert np.isnan(a["us"][2]).all()
    args = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 2.0), 0.1, 1e-8, 1e-6, None, False, "fp64",
                         "persistent", 0)
    off = np.empty(2001, dtype=np.int64)
    o = L.EverystepOut()
    o.offsets = off.ctypes.data
    assert checked.solve_everystep(args, o) == L.ESMALL
    ts, us = np.empty(o.total), np.empty((o.total, 3))
    o.ts, o.us, o.capacity = ts.ctypes.data, us.ctypes.data, o.total
    assert checked.solve_everystep(args, o) == L.OK, checked.error()


@pytest.mark.parametrize("alg", ["ATsit5", "AVern7"])
def test_no_violation_trajectory_major_layout_and_fp64_controller(pkg, checked, alg):
    """The trajectory-major output layout and the FP64 step-size controller in
    bounds-check mode (staged and two-queue staged kernels): no violation,
    every trajectory started once, results equal to the unchecked kernels'."""
    L = pkg._lib
    n = 3000
    u0, p = lorenz_inputs(n, seed=104)
    sv = np.linspace(0, 2, 17)
    algo = getattr(pkg, "GPUSimple" + alg)()
    res = []
    for h in (checked, pkg._handle(0)):
        a = pkg.make_args(algo, 0, u0, p, (0.0, 2.0), 0.1, 1e-8, 1e-6, sv, False, "fp64", "persistent", 0,
                          layout="traj", controller="fp64")
        out = {"us": np.empty((n, len(sv), 3)), "u_final": np.empty((3, n)), "naccept": np.empty(n, dtype=np.int32)}
        o = L.SolveOut()
        for k, v in out.items():
            setattr(o, k, v.ctypes.data)
        rc = h.solve_raw(a, o, L.SolveStats())
        assert rc in (L.OK, L.ETRAJ), h.error()
        res.append(out)
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k], equal_nan=True), k
