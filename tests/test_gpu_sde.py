"""GPU SimpleEM (src/euler_maruyama.jl:48-142) against the oracle: every
trajectory's path bit-identical to the CPU restatement with the same
counter-based normals (Philox4x32-10 + Box-Muller), for the built-in SDEs
compiled ahead of time and at run time, a user SDE compiled with NVRTC, host
and device buffers."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def sde(pkg, kind, u0, p, tspan, dt, seed, every=True, n=None):
    ep = pkg.EnsembleProblem(pkg.SDEProblem(kind, u0[:, 0], tspan, p[:, 0]), u0s=u0, ps=p)
    return pkg.solve(ep, pkg.SimpleEM(), trajectories=u0.shape[1], dt=dt, seed=seed, save_everystep=every)


@pytest.mark.parametrize("kind,dim", [("gbm", 1), ("gbm", 3), ("ou", 1), ("ou", 5), ("lorenz", 3)])
def test_simple_em_bitexact(pkg, po, kind, dim):
    rng = np.random.default_rng(dim)
    n = 3000
    if kind == "gbm":
        u0 = rng.uniform(0.5, 2.0, (dim, n))
        p = np.stack([rng.uniform(-0.5, 0.5, n), rng.uniform(0.05, 0.5, n)])
    elif kind == "ou":
        u0 = rng.normal(0, 1, (dim, n))
        p = np.stack([rng.uniform(0.5, 2, n), rng.normal(0, 1, n), rng.uniform(0.1, 1, n)])
    else:
        u0 = rng.uniform(-1, 1, (3, n)) + np.array([[0], [0], [20]])
        p = np.stack([np.full(n, 10.0), rng.uniform(0, 30, n), np.full(n, 8 / 3), rng.uniform(0, 1, n)])
    sol = sde(pkg, kind, u0, p, (0.0, 1.0), 0.01, seed=11)
    ref = po.sde_solve(kind, u0, p, (0.0, 1.0), 0.01, seed=11, nthreads=8)
    assert sol.us.shape == (101, dim, n)
    assert np.array_equal(sol.us, ref["us"]) and np.array_equal(sol.u_final, ref["u_final"])
    assert np.array_equal(sol.t, ref["t"])
    other = sde(pkg, kind, u0, p, (0.0, 1.0), 0.01, seed=12, every=False)
    assert not np.array_equal(other.u_final, sol.u_final)


def test_user_sde_equals_builtin(pkg):
    rng = np.random.default_rng(4)
    n = 2000
    u0 = rng.uniform(0.5, 2.0, (2, n))
    p = np.stack([rng.uniform(-0.5, 0.5, n), rng.uniform(0.05, 0.5, n)])
    user = pkg.UserSDE("for (int d = 0; d < 2; ++d) f[d] = p[0] * u[d];",
                       "for (int d = 0; d < 2; ++d) g[d] = p[1] * u[d];", dim=2, nparams=2)
    a = sde(pkg, user, u0, p, (0.0, 2.0), 0.02, seed=5)
    b = sde(pkg, "gbm", u0, p, (0.0, 2.0), 0.02, seed=5)
    assert np.array_equal(a.us, b.us)


def test_simple_em_device_buffers_and_bad_grid(pkg, po):
    import torch
    L = pkg._lib
    h = pkg._handle(0)
    n = 1000
    u0 = np.ones((1, n))
    p = np.tile([[0.1], [0.2]], (1, n))
    a = L.SdeArgs()
    a.sde, a.n, a.dim, a.nparams = L.SDE["gbm"], n, 1, 2
    a.t0, a.tf, a.dt, a.seed = 0.0, 1.0, 0.01, 99
    a.save_everystep, a.memory = 0, L.MEM_DEVICE
    du0, dp = torch.tensor(u0, device="cuda"), torch.tensor(p, device="cuda")
    uf = torch.empty((1, n), dtype=torch.float64, device="cuda")
    a.u0, a.p = du0.data_ptr(), dp.data_ptr()
    o = L.SdeOut()
    o.u_final = uf.data_ptr()
    h.check(h.sde_solve(a, o))
    ref = po.sde_solve("gbm", u0, p, (0.0, 1.0), 0.01, seed=99, save_everystep=False)
    assert np.array_equal(uf.cpu().numpy(), ref["u_final"])
    a.dt = 0.3  # (tf - t0)/dt not an integer: the reference's Int(...) throws
    assert h.sde_solve(a, o) == L.EINVAL


def sde_nd(pkg, kind, u0, p, M, tspan, dt, seed, every=True):
    proto = np.zeros((u0.shape[0], M))
    ep = pkg.EnsembleProblem(pkg.SDEProblem(kind, u0[:, 0], tspan, p[:, 0], noise_rate_prototype=proto),
                             u0s=u0, ps=p)
    return pkg.solve(ep, pkg.SimpleEM(), trajectories=u0.shape[1], dt=dt, seed=seed, save_everystep=every)


@pytest.mark.parametrize("dim,M", [(2, 4), (3, 3), (1, 1), (4, 5)])
def test_simple_em_non_diagonal_bitexact(pkg, po, dim, M):
    """Non-diagonal noise (src/euler_maruyama.jl:126-134), the reference's test
    SDE generalised (test/simpleem_tests.jl: f = 1.01u, G = c .* u, 2 x 4):
    bit-identical to the oracle, for even and odd noise dimensions (odd M
    shares a Box-Muller pair between steps)."""
    rng = np.random.default_rng(10 * dim + M)
    n = 2500
    u0 = rng.uniform(0.5, 2.0, (dim, n))
    c = rng.uniform(0.05, 1.8, (dim * M, n))
    p = np.vstack([np.full((1, n), 1.01), c])
    sol = sde_nd(pkg, "mult", u0, p, M, (0.0, 1.0), 0.25 if (dim, M) == (2, 4) else 0.01, seed=21)
    ref = po.sde_solve("mult", u0, p, (0.0, 1.0), 0.25 if (dim, M) == (2, 4) else 0.01, seed=21, nthreads=8,
                       noise_dim=M)
    assert sol.us.shape == ref["us"].shape
    assert np.array_equal(sol.us, ref["us"]) and np.array_equal(sol.u_final, ref["u_final"])


def test_user_sde_non_diagonal_equals_builtin(pkg):
    rng = np.random.default_rng(8)
    n, M = 2000, 3
    u0 = rng.uniform(0.5, 2.0, (2, n))
    p = np.vstack([np.full((1, n), 0.3), rng.uniform(0.1, 1.0, (2 * M, n))])
    user = pkg.UserSDE("for (int d = 0; d < 2; ++d) f[d] = p[0] * u[d];",
                       "for (int d = 0; d < 2; ++d) for (int m = 0; m < 3; ++m) g[d * 3 + m] = p[1 + d * 3 + m] * u[d];",
                       dim=2, nparams=1 + 2 * M, noise_dim=M)
    a = sde_nd(pkg, user, u0, p, M, (0.0, 1.0), 0.01, seed=6)
    b = sde_nd(pkg, "mult", u0, p, M, (0.0, 1.0), 0.01, seed=6)
    assert np.array_equal(a.us, b.us)
    with pytest.raises(ValueError):
        sde_nd(pkg, user, u0, p, M + 1, (0.0, 1.0), 0.01, seed=6)  # declared noise_dim differs


def test_non_diagonal_argument_checks(pkg):
    L = pkg._lib
    h = pkg._handle(0)
    n = 10
    u0 = np.ones((2, n))
    p = np.ones((9, n))
    a = L.SdeArgs()
    a.sde, a.n, a.dim, a.nparams, a.noise_dim = L.SDE["mult"], n, 2, 9, 4
    a.t0, a.tf, a.dt, a.seed = 0.0, 1.0, 0.25, 1
    a.memory = L.MEM_HOST
    a.u0, a.p = u0.ctypes.data, p.ctypes.data
    uf = np.zeros((2, n))
    o = L.SdeOut()
    o.u_final = uf.ctypes.data
    h.check(h.sde_solve(a, o))
    assert np.all(np.isfinite(uf))
    a.nparams = 8  # needs 1 + dim x noise_dim
    assert h.sde_solve(a, o) == L.EINVAL
    a.nparams, a.noise_dim = 9, 0  # the multiplicative SDE is non-diagonal only
    assert h.sde_solve(a, o) == L.EINVAL
    a.sde, a.nparams, a.noise_dim = L.SDE["gbm"], 2, 2  # a diagonal built-in takes no noise matrix
    assert h.sde_solve(a, o) == L.EINVAL


def test_readme_non_diagonal_example(pkg):
    """The README's SimpleEM example (the reference test's non-diagonal SDE)."""
    c = [0.3, 0.6, 0.9, 0.12, 1.2, 0.2, 0.3, 1.8]
    n = 5000
    sde = pkg.SDEProblem("mult", [1.0, 1.0], (0.0, 1.0), [1.01] + c, noise_rate_prototype=np.zeros((2, 4)))
    ens = pkg.EnsembleProblem(sde, u0s=np.ones((2, n)), ps=np.tile(np.array([1.01] + c)[:, None], (1, n)))
    paths = pkg.solve(ens, pkg.SimpleEM(), trajectories=n, dt=0.01, seed=1)
    assert paths.us.shape == (101, 2, n)
    assert np.all(np.isfinite(paths.us)) and np.array_equal(paths.us[0], np.ones((2, n)))
