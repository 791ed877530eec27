"""The trajectory-major output layout (ODE_LAYOUT_TRAJ, us[n][npoints][width]):
every kernel that writes saveat or every-step output gives the same values in
it as in the default [npoints][width][n] layout, bit for bit, on every
schedule and path (staged and two-queue rings, fixed-step and
component-split kernels, order-parameter and user outputs, chunked host
pipeline, bounds-check mode)."""
import numpy as np
import pytest

from conftest import lorenz_inputs

pytestmark = pytest.mark.gpu


def ens(pkg, rhs, u0, p, tspan):
    return pkg.EnsembleProblem(pkg.ODEProblem(rhs, u0[:, 0], tspan, p[:, 0]), u0s=u0, ps=p)


def both(pkg, e, alg, n, **kw):
    a = pkg.solve(e, alg, trajectories=n, throw=False, **kw)
    b = pkg.solve(e, alg, trajectories=n, layout="traj", throw=False, **kw)
    assert np.array_equal(a.retcode, b.retcode)
    assert b.us_traj is not None and b.us_traj.shape == (n, a.us.shape[0], a.us.shape[1])
    assert np.array_equal(np.ascontiguousarray(b.us_traj.transpose(1, 2, 0)), a.us, equal_nan=True)
    assert np.array_equal(a.u_final, b.u_final) and np.array_equal(a.naccept, b.naccept)
    return a, b


@pytest.mark.parametrize("schedule", ["plain", "persistent"])
def test_atsit5_saveat(pkg, schedule):
    u0, p = lorenz_inputs(5000, seed=901)
    sv = np.linspace(0, 10, 100)
    both(pkg, ens(pkg, "lorenz", u0, p, (0.0, 10.0)), pkg.GPUSimpleATsit5(), 5000, dt=0.1, abstol=1e-8,
         reltol=1e-6, saveat=sv, schedule=schedule)


def test_atsit5_unreached_points_nan(pkg):
    u0, p = lorenz_inputs(500, seed=902)
    sv = np.array([0.0, 0.5, 1.0, 5.0, 7.0])  # beyond tspan: NaN rows
    _, b = both(pkg, ens(pkg, "lorenz", u0, p, (0.0, 2.0)), pkg.GPUSimpleATsit5(), 500, dt=0.1, abstol=1e-8,
                reltol=1e-6, saveat=sv, schedule="persistent")
    assert np.isnan(b.us_traj[:, 3:, :]).all() and not np.isnan(b.us_traj[:, :3, :]).any()


def test_avern7_two_queue_staging(pkg):
    rng = np.random.default_rng(903)
    n = 4000
    mu = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n))[None, :]
    u0 = rng.uniform(-2, 2, (2, n))
    both(pkg, ens(pkg, "vanderpol", u0, mu, (0.0, 20.0)), pkg.GPUSimpleAVern7(), n, dt=0.1, abstol=1e-10,
         reltol=1e-8, saveat=np.linspace(0, 20, 200), schedule="persistent")


def test_avern9_fp32_kahan(pkg):
    rng = np.random.default_rng(904)
    n = 2000
    u0 = np.array([0.994, 0.0, 0.0, -2.00158510637908])[:, None] + rng.normal(0, 1e-4, (4, n))
    mu = np.full((1, n), 0.012277471)
    both(pkg, ens(pkg, "r3bp", u0, mu, (0.0, 17.0652165601579625588917206249)), pkg.GPUSimpleAVern9(), n, dt=0.1,
         abstol=1e-7, reltol=1e-7, saveat=np.linspace(0, 17, 9), precision="fp32_kahan", schedule="persistent")


@pytest.mark.parametrize("n", [3000, 20000])
def test_fixed_step_every_grid_point(pkg, n):
    """n = 3000 runs the component-split kernel (small FP64 ensemble), 20000 the
    thread-per-trajectory fixed-step kernel."""
    u0, p = lorenz_inputs(n, seed=905)
    both(pkg, ens(pkg, "lorenz", u0, p, (0.0, 1.0)), pkg.GPUSimpleTsit5(), n, dt=0.01, save_everystep=True)


def test_rk4_every_step(pkg):
    u0, p = lorenz_inputs(3000, seed=906)
    both(pkg, ens(pkg, "lorenz", u0, p, (0.0, 1.0)), pkg.GPUSimpleRK4(), 3000, dt=0.01, save_everystep=True)


def test_kuramoto_order_parameter_and_user_output(pkg):
    rng = np.random.default_rng(907)
    n, D = 3000, 12
    th = rng.uniform(0, 2 * np.pi, (D, n))
    p = np.vstack([rng.normal(0, 1, (D, n)), rng.uniform(0, 4, (1, n))])
    e = ens(pkg, "kuramoto", th, p, (0.0, 5.0))
    both(pkg, e, pkg.GPUSimpleATsit5(), n, dt=0.1, abstol=1e-8, reltol=1e-6, saveat=np.linspace(0, 5, 11),
         schedule="persistent", output="kuramoto_r")
    u0, pl = lorenz_inputs(3000, seed=908)
    out = pkg.UserOutput("out[0] = u[0] * u[1];\n out[1] = u[2] + t;", width=2)
    both(pkg, ens(pkg, "lorenz", u0, pl, (0.0, 3.0)), pkg.GPUSimpleATsit5(), 3000, dt=0.1, abstol=1e-8,
         reltol=1e-6, saveat=np.linspace(0, 3, 7), schedule="persistent", output=out)


def test_chunked_host_path(pkg):
    """Host buffers, 540,000 trajectories: three chunks, each chunk's series one
    contiguous block of the host array."""
    n = 540000
    u0, p = lorenz_inputs(n, seed=909)
    a, b = both(pkg, ens(pkg, "lorenz", u0, p, (0.0, 2.0)), pkg.GPUSimpleATsit5(), n, dt=0.1, abstol=1e-8,
                reltol=1e-6, saveat=np.linspace(0, 2, 11), schedule="persistent")
    assert b.stats.launches >= 3


def test_bounds_check_mode(pkg):
    L = pkg._lib
    h = L.Handle(0)
    try:
        h.set_bounds_check(True)
        n = 3000
        u0, p = lorenz_inputs(n, seed=910)
        sv = np.linspace(0, 2, 17)
        ref = pkg.solve(ens(pkg, "lorenz", u0, p, (0.0, 2.0)), pkg.GPUSimpleATsit5(), trajectories=n, dt=0.1,
                        abstol=1e-8, reltol=1e-6, saveat=sv, schedule="persistent")
        a = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 2.0), 0.1, 1e-8, 1e-6, sv, False, "fp64",
                          "persistent", 0, layout="traj")
        us = np.empty((n, len(sv), 3))
        o = L.SolveOut()
        o.us = us.ctypes.data
        rc = h.solve_raw(a, o, L.SolveStats())
        assert rc == L.OK, h.error()
        assert np.array_equal(us.transpose(1, 2, 0), ref.us)
    finally:
        h.close()


def test_unknown_layout_rejected(pkg):
    L = pkg._lib
    u0, p = lorenz_inputs(8, seed=1)
    a = pkg.make_args(pkg.GPUSimpleATsit5(), 0, u0, p, (0.0, 1.0), 0.1, 1e-6, 1e-3, None, False, "fp64",
                      "persistent", 0)
    a.layout = 7
    h = pkg._handle(0)
    assert h.solve_raw(a, L.SolveOut(), L.SolveStats()) == L.EINVAL
