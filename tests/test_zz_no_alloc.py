"""The allocation-free entry point ode_ensemble_solve_noalloc.

It exists for callers that cannot allocate GPU memory (applications that own
the device memory budget, real-time loops that cannot afford cudaMalloc's
synchronisation): they pass device buffers and the solver uses a fixed scratch
array in the library's device image.  This file is collected last so that a
run stopping at the first failure has run everything else first; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from conftest import lorenz_inputs

pytestmark = pytest.mark.gpu

KW = dict(dt=0.1, abstol=1e-8, reltol=1e-6)


def test_noalloc_matches_the_allocating_solve_twice(pkg):
    torch = pytest.importorskip("torch")
    L = pkg._lib
    lib = L.load()
    n = 20000
    u0, p = lorenz_inputs(n, seed=606)
    sv = np.linspace(0, 10, 50)
    # the existing entry point (allocating, host buffers) gives the expected results
    ref = pkg.solve(pkg.EnsembleProblem(pkg.ODEProblem("lorenz", u0[:, 0], (0.0, 10.0), p[:, 0]), u0s=u0, ps=p),
                    pkg.GPUSimpleATsit5(), trajectories=n, saveat=sv, schedule="persistent", **KW)
    dev = torch.device("cuda", 0)
    du0 = torch.from_numpy(u0).to(dev)
    dp = torch.from_numpy(p).to(dev)
    out = {"us": torch.empty((len(sv), 3, n), dtype=torch.float64, device=dev),
           "u_final": torch.empty((3, n), dtype=torch.float64, device=dev),
           "t_final": torch.empty(n, dtype=torch.float64, device=dev),
           "retcode": torch.empty(n, dtype=torch.int8, device=dev),
           "naccept": torch.empty(n, dtype=torch.int32, device=dev),
           "nreject": torch.empty(n, dtype=torch.int32, device=dev)}
    a = pkg.make_args(pkg.GPUSimpleATsit5(), L.RHS["lorenz"], u0, p, (0.0, 10.0), KW["dt"], KW["abstol"],
                      KW["reltol"], sv, False, "fp64", "persistent", 0, memory=L.MEM_DEVICE)
    a.u0, a.p = du0.data_ptr(), dp.data_ptr()
    o = L.SolveOut()
    for k, v in out.items():
        setattr(o, k, v.data_ptr())
    err = ctypes.create_string_buffer(256)
    dsv = torch.from_numpy(sv).to(dev)
    for call in range(2):
        for v in out.values():  # stale values must not survive
            v.fill_(-1 if v.dtype.is_floating_point else 7)
        if call == 1:
            a.saveat = dsv.data_ptr()  # saveat may also be a device array
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(0)[0]
        rc = lib.ode_ensemble_solve_noalloc(ctypes.byref(a), ctypes.byref(o), err, 256)
        assert rc == 0, (call, rc, err.value)
        if call == 1:
            # after the first call's one-off set-up (kernel loading), a call takes no device memory
            assert torch.cuda.mem_get_info(0)[0] == free_before
        assert np.array_equal(out["u_final"].cpu().numpy(), ref.u_final), call
        assert np.array_equal(out["us"].cpu().numpy(), ref.us, equal_nan=True), call
        assert np.array_equal(out["t_final"].cpu().numpy(), ref.t_final), call
        assert np.array_equal(out["retcode"].cpu().numpy(), ref.retcode), call
        assert np.array_equal(out["naccept"].cpu().numpy(), ref.naccept), call
        assert np.array_equal(out["nreject"].cpu().numpy(), ref.nreject), call


def test_noalloc_rejects_what_it_cannot_hold(pkg):
    L = pkg._lib
    lib = L.load()
    n = 8
    u0, p = lorenz_inputs(n, seed=1)
    sv = np.linspace(0, 1, 5000)  # more than ODE_NOALLOC_MAX_SAVE
    a = pkg.make_args(pkg.GPUSimpleATsit5(), L.RHS["lorenz"], u0, p, (0.0, 1.0), 0.1, 1e-6, 1e-3, sv, False,
                      "fp64", "persistent", 0, memory=L.MEM_DEVICE)
    o = L.SolveOut()
    err = ctypes.create_string_buffer(256)
    assert lib.ode_ensemble_solve_noalloc(ctypes.byref(a), ctypes.byref(o), err, 256) == L.EINVAL
    assert b"4096" in err.value
    a = pkg.make_args(pkg.GPUSimpleAVern7(), L.RHS["lorenz"], u0, p, (0.0, 1.0), 0.1, 1e-6, 1e-3, None, False,
                      "fp64", "persistent", 0, memory=L.MEM_DEVICE)
    assert lib.ode_ensemble_solve_noalloc(ctypes.byref(a), ctypes.byref(o), err, 256) == L.ENOTSUP
    a = pkg.make_args(pkg.GPUSimpleATsit5(), L.RHS["lorenz"], u0, p, (0.0, 1.0), 0.1, 1e-6, 1e-3, None, False,
                      "fp64", "persistent", 0, memory=L.MEM_DEVICE)  # host pointers
    assert lib.ode_ensemble_solve_noalloc(ctypes.byref(a), ctypes.byref(o), err, 256) == L.EINVAL
    assert b"device pointer" in err.value


def test_noalloc_reports_trajectories_stopped_early(pkg):
    """An attempt cap of 2 stops every trajectory: ODE_ETRAJ, retcode MAXITERS,
    as ode_ensemble_solve reports it."""
    torch = pytest.importorskip("torch")
    L = pkg._lib
    lib = L.load()
    n = 1000
    u0, p = lorenz_inputs(n, seed=7)
    dev = torch.device("cuda", 0)
    du0, dp = torch.from_numpy(u0).to(dev), torch.from_numpy(p).to(dev)
    ret = torch.full((n,), 9, dtype=torch.int8, device=dev)
    uf = torch.empty((3, n), dtype=torch.float64, device=dev)
    a = pkg.make_args(pkg.GPUSimpleATsit5(), L.RHS["lorenz"], u0, p, (0.0, 10.0), KW["dt"], KW["abstol"],
                      KW["reltol"], None, False, "fp64", "persistent", 2, memory=L.MEM_DEVICE)
    a.u0, a.p = du0.data_ptr(), dp.data_ptr()
    o = L.SolveOut()
    o.retcode, o.u_final = ret.data_ptr(), uf.data_ptr()
    err = ctypes.create_string_buffer(256)
    rc = lib.ode_ensemble_solve_noalloc(ctypes.byref(a), ctypes.byref(o), err, 256)
    assert rc == L.ETRAJ, (rc, err.value)
    assert (ret.cpu().numpy() == 2).all()
