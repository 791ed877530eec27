"""Shared fixtures.  Tests marked `gpu` need a CUDA device; everything else
runs on the CPU (oracle, host logic, library loading and exports)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the C ABI on cuda:0)")


@pytest.fixture(scope="session")
def po():
    import __graft_entry__ as g
    return g.oracle()


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    lib = os.path.join(ROOT, "simplediffeq.jl_gb300", "lib", "libgb300ode.so")
    if not os.path.exists(lib):
        g.build()
    return g.package()


def lorenz_inputs(n, seed=1, rho_hi=30.0):
    """Adaptive-Lorenz ensemble: sigma=10, beta=8/3, rho ~ U[0, rho_hi],
    u0 ~ U[-1,1]^3 + (0,0,20), as the 1M-trajectory workload."""
    rng = np.random.default_rng(seed)
    u0 = rng.uniform(-1, 1, (3, n))
    u0[2] += 20
    p = np.stack([np.full(n, 10.0), rng.uniform(0, rho_hi, n), np.full(n, 8 / 3)])
    return u0, p


def decay_inputs(n, dim=3):
    """f(u) = -u with u0 = ones, as test/gpu_ode_regression.jl:2-9."""
    u0 = np.ones((dim, n))
    A = (-np.eye(dim)).reshape(dim * dim, 1).repeat(n, 1)
    return u0, A
