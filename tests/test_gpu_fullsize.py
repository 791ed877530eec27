"""Parity at the full sizes of the benchmark workloads (1,048,576 adaptive
Lorenz, 524,288 AVern7 Van der Pol, 4,194,304 Kuramoto-12), through
properties that do not need the oracle to solve the whole ensemble: every
trajectory succeeds, the learned or persistent schedule gives every
trajectory bit-for-bit the plain kernel's result (the matched-error claim of
the benchmark), and a random sample of trajectories taken from the full
solve equals the oracle bit for bit."""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu


def ens(pkg, rhs, u0, p, tspan):
    return pkg.EnsembleProblem(pkg.ODEProblem(rhs, u0[:, 0], tspan, p[:, 0]), u0s=u0, ps=p)


def check_sample(po, sol, cfg, alg, u0, p, sv, output, k=384, seed=0):
    idx = np.sort(np.random.default_rng(seed).choice(u0.shape[1], k, replace=False))
    ref = po.solve(alg, cfg["rhs"], np.ascontiguousarray(u0[:, idx]), np.ascontiguousarray(p[:, idx]), cfg["tspan"],
                   cfg["dt"], rounding="device", abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv, nthreads=8,
                   output=output)
    assert np.array_equal(sol.u_final[:, idx], ref["u_final"])
    assert np.array_equal(sol.us[:, :, idx], ref["us"], equal_nan=True)
    assert np.array_equal(sol.naccept[idx], ref["naccept"]) and np.array_equal(sol.nreject[idx], ref["nreject"])


def test_full_size_lorenz_learned(pkg, po):
    cfg = bench.CONFIGS[2]
    u0, p = cfg["inputs"](cfg["n"], 2024)
    sv = np.linspace(*cfg["tspan"], cfg["nsave"])
    kw = dict(dt=cfg["dt"], abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv)
    tu0, tp = cfg["inputs"](65536, 777)
    pkg.learn_fit(ens(pkg, "lorenz", tu0, tp, cfg["tspan"]), pkg.GPUSimpleATsit5(), 65536, **kw)
    e = ens(pkg, "lorenz", u0, p, cfg["tspan"])
    a = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=cfg["n"], schedule="learned", **kw)
    assert np.all(a.retcode == 0)
    b = pkg.solve(e, pkg.GPUSimpleATsit5(), trajectories=cfg["n"], schedule="plain", **kw)
    assert np.array_equal(a.us, b.us) and np.array_equal(a.u_final, b.u_final)
    assert np.array_equal(a.naccept, b.naccept) and np.array_equal(a.nreject, b.nreject)
    check_sample(po, a, cfg, "ATsit5", u0, p, sv, "state")


def test_full_size_vanderpol_avern7(pkg, po):
    cfg = bench.CONFIGS[3]
    u0, p = cfg["inputs"](cfg["n"], 2024)
    sv = np.linspace(*cfg["tspan"], cfg["nsave"])
    kw = dict(dt=cfg["dt"], abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv)
    e = ens(pkg, "vanderpol", u0, p, cfg["tspan"])
    a = pkg.solve(e, pkg.GPUSimpleAVern7(), trajectories=cfg["n"], schedule="persistent", **kw)
    assert np.all(a.retcode == 0)
    b = pkg.solve(e, pkg.GPUSimpleAVern7(), trajectories=cfg["n"], schedule="plain", **kw)
    assert np.array_equal(a.us, b.us) and np.array_equal(a.u_final, b.u_final)
    check_sample(po, a, cfg, "AVern7", u0, p, sv, "state")


def test_full_size_kuramoto_order_parameter(pkg, po):
    cfg = bench.CONFIGS[5]
    u0, p = cfg["inputs"](cfg["n"], 2024)
    sv = np.linspace(*cfg["tspan"], cfg["nsave"])
    kw = dict(dt=cfg["dt"], abstol=cfg["abstol"], reltol=cfg["reltol"], saveat=sv, output="kuramoto_r")
    a = pkg.solve(ens(pkg, "kuramoto", u0, p, cfg["tspan"]), pkg.GPUSimpleATsit5(), trajectories=cfg["n"],
                  schedule="persistent", **kw)
    assert np.all(a.retcode == 0)
    assert a.us.shape == (cfg["nsave"], 1, cfg["n"])
    assert np.all((a.us >= 0) & (a.us <= 1 + 1e-12))  # |mean of unit phasors| is in [0, 1]
    check_sample(po, a, cfg, "ATsit5", u0, p, sv, "kuramoto_r", k=256)
