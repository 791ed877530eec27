"""Edge cases at the boundary, on the GPU: empty ensembles on every path,
single trajectories, zero-length and backward spans, save points outside the
span, and n = 1 every-step output, each against the oracle where it applies."""
import numpy as np
import pytest

from conftest import lorenz_inputs
from test_gpu_parity import assert_bitexact, gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("alg", ["ATsit5", "AVern9", "Tsit5", "RK4", "Euler"])
@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_empty_ensemble(pkg, alg, schedule):
    L = pkg._lib
    h = pkg._handle(0)
    u0 = np.zeros((3, 0))
    p = np.zeros((3, 0))
    sv = None if alg in ("RK4", "Euler") else np.linspace(0, 1, 5)
    a = pkg.make_args(getattr(pkg, "GPUSimple" + alg)(), 0, u0, p, (0.0, 1.0), 0.1, 1e-6, 1e-3, sv, False, "fp64",
                      schedule, 0)
    st = L.SolveStats()
    assert h.solve_raw(a, L.SolveOut(), st) == L.OK
    assert st.attempts == 0


def test_empty_every_step_and_sde(pkg):
    L = pkg._lib
    h = pkg._handle(0)
    a = pkg.make_args(pkg.GPUSimpleATsit5(), 0, np.zeros((3, 0)), np.zeros((3, 0)), (0.0, 1.0), 0.1, 1e-6, 1e-3,
                      None, False, "fp64", "persistent", 0)
    off = np.zeros(1, dtype=np.int64)
    o = L.EverystepOut()
    o.offsets = off.ctypes.data
    assert h.solve_everystep(a, o) == L.ESMALL and o.total == 0
    s = L.SdeArgs()
    s.sde, s.n, s.dim, s.nparams, s.t0, s.tf, s.dt = L.SDE["gbm"], 0, 1, 2, 0.0, 1.0, 0.1
    assert h.sde_solve(s, L.SdeOut()) == L.OK


@pytest.mark.parametrize("alg", ["ATsit5", "AVern7", "AVern9"])
def test_single_trajectory_and_degenerate_spans(pkg, po, alg):
    u0, p = lorenz_inputs(1, seed=5)
    algo = getattr(pkg, "GPUSimple" + alg)()
    kw = dict(abstol=1e-8, reltol=1e-6)
    # a point before the span is extrapolated from the first step's interpolant (theta < 0), as the
    # reference's `while ts[cur_t] <= t` loop does; a point after the span is never reached (NaN)
    sv = np.array([-1.0, 0.0, 0.5, 1.0, 2.0])
    sol = gpu(pkg, algo, "lorenz", u0, p, (0.0, 1.0), 0.1, saveat=sv, **kw)
    ref = po.solve(alg, "lorenz", u0, p, (0, 1), 0.1, rounding="device", saveat=sv, **kw)
    assert_bitexact(sol, ref)
    assert np.isfinite(sol.us[0]).all() and np.isnan(sol.us[4]).all() and np.array_equal(sol.us[1], u0)
    # zero-length and backward spans: the reference's `while t < tf` never runs
    for tspan in ((1.0, 1.0), (1.0, 0.0)):
        z = gpu(pkg, algo, "lorenz", u0, p, tspan, 0.1, **kw)
        assert np.array_equal(z.u_final, u0) and z.naccept[0] == 0 and z.t_final[0] == tspan[0]
        zr = po.solve(alg, "lorenz", u0, p, tspan, 0.1, rounding="device", **kw)
        assert np.array_equal(zr["u_final"], u0)


def test_single_trajectory_every_step(pkg, po):
    u0, p = lorenz_inputs(1, seed=6)
    e = pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 1.0), p[:, 0]), u0s=u0, ps=p)
    sol = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=1, dt=0.1, save_everystep=True)
    ref = po.solve("ATsit5", "lorenz", u0, p, (0, 1), 0.1, rounding="device", save_everystep=True)
    assert np.array_equal(sol.ts_rows, ref["ts_rows"]) and np.array_equal(sol.us_rows, ref["us_rows"])
    one = pkg.solve(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 1.0), p[:, 0]), pkg.GPUSimpleATsit5(), dt=0.1,
                    save_everystep=True)
    assert np.array_equal(one.t, ref["ts_rows"]) and len(one.u) == len(ref["ts_rows"])


def test_rhs_builtin_selects_by_dimension(pkg):
    """ode_rhs_builtin: the id and parameter count of a built-in right-hand
    side for a dimension, EINVAL where it has no form of that dimension."""
    h = pkg._handle(0)
    assert h.rhs_builtin("lorenz", 3) == (0, 3)
    assert h.rhs_builtin("kuramoto", 12) == (3, 13)
    assert h.rhs_builtin("linear", 4) == (4, 16)
    for name, dim in (("lorenz", 2), ("vanderpol", 3), ("r3bp", 2), ("linear", 9), ("kuramoto", 0)):
        with pytest.raises(pkg.GB300ODEError):
            h.rhs_builtin(name, dim)
    with pytest.raises(pkg.GB300ODEError):
        h.rhs_builtin(999, 3)
