"""The correctly rounded power function of the reference-arithmetic mode
(simplediffeq.jl_gb300/csrc/crpow.h), compiled on the host with g++: equal to
the double nearest x^y (mpmath at 220 bits) on the controller's exponents
and on random ones, over the whole normal range, near 1 and at the edges;
its tables are the generator's output; and the oracle's REF rounding with
these powers (controller "ref") against libm's pow."""
import ctypes
import importlib.util
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "simplediffeq.jl_gb300", "csrc")

SHIM = r'''
#include "crpow.h"
extern "C" long vsincos(const double* x, double* s, double* c, long n) {
  long handled = 0;
  for (long i = 0; i < n; ++i) handled += gbode::cr_sincos(x[i], s + i, c + i);
  return handled;
}
extern "C" void vpow(const double* x, const double* y, double* o, long n) {
  for (long i = 0; i < n; ++i) o[i] = gbode::cr_pow(x[i], y[i]);
}
/* first phase against the double-double path: returns how many differ, *fell = how many fell through */
extern "C" long vphases(const double* x, const double* y, long n, long* fell) {
  long bad = 0;
  *fell = 0;
  for (long i = 0; i < n; ++i) {
    double f;
    if (!gbode::cr_pow_fast(x[i], y[i], &f)) { ++*fell; continue; }
    if (f != gbode::cr_exp(gbode::cr_mul_d(gbode::cr_log(x[i]), y[i])).h) ++bad;
  }
  return bad;
}
'''


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("crpow")
    src, so = d / "shim.cpp", d / "libshim.so"
    src.write_text(SHIM)
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC, str(src), "-o",
                    str(so)], check=True)
    L = ctypes.CDLL(str(so))
    L.vpow.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long]
    L.vphases.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_long, ctypes.POINTER(ctypes.c_long)]
    L.vphases.restype = ctypes.c_long
    L.vsincos.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_long]
    L.vsincos.restype = ctypes.c_long
    return L


def cr_pow(lib, x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.broadcast_to(y, x.shape), dtype=np.float64)
    o = np.empty_like(x)
    lib.vpow(x.ctypes.data, y.ctypes.data, o.ctypes.data, x.size)
    return o


def test_correctly_rounded(lib):
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 220
    rng = np.random.default_rng(5)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 3000), 10.0 ** rng.uniform(-12, 3, 3000),
                        1 + rng.uniform(-1e-6, 1e-6, 500), 1 + rng.uniform(-0.3, 0.3, 500),
                        np.array([2.2250738585072014e-308, 1.7976931348623157e308, 0.5, 2.0, 1 - 2.0 ** -53,
                                  1 + 2.0 ** -52, 1e-4, 3.0])])
    lo, hi = mp.mpf(2.2250738585072014e-308), mp.mpf(1.7976931348623157e308)
    checked = 0
    for y in (np.full(x.size, 7.0 / 50.0), np.full(x.size, 2.0 / 25.0), rng.uniform(-3, 3, x.size)):
        got = cr_pow(lib, x, y)
        for xi, yi, g in zip(x, y, got):
            ex = mp.mpf(xi) ** mp.mpf(yi)
            if not lo <= ex <= hi:
                continue
            assert g == float(ex), (xi.hex(), yi, g.hex(), float(ex).hex())
            checked += 1
    assert checked > 20000


def test_first_phase_agrees_with_double_double_path(lib):
    """Ziv's first phase (double polynomials, a rounding test with a 2^-63
    margin; its largest error measured about 2^-68) returns what the double-double
    path returns, and falls through in about 0.15% of calls."""
    rng = np.random.default_rng(6)
    x = np.concatenate([10.0 ** rng.uniform(-12, 3, 300000), 10.0 ** rng.uniform(-300, 300, 100000),
                        1 + rng.uniform(-1e-3, 1e-3, 100000)])
    for y in (np.full(x.size, 7.0 / 50.0), np.full(x.size, 2.0 / 25.0), rng.uniform(-1, 1, x.size)):
        fell = ctypes.c_long(0)
        assert lib.vphases(x.ctypes.data, np.ascontiguousarray(y).ctypes.data, x.size, ctypes.byref(fell)) == 0
        assert fell.value < 0.005 * x.size


def test_sincos_correctly_rounded(lib):
    """cr_sincos: both results the doubles nearest sin x and cos x (mpmath at
    300 bits) for |x| < 2^19, near multiples of pi/2 (the reduction's
    cancellation) and for tiny x; beyond 2^19 and for non-finite x it
    declines (the caller's math library takes over)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 300
    rng = np.random.default_rng(7)
    k = np.arange(-400, 400) * (np.pi / 2)
    x = np.concatenate([rng.uniform(-7, 7, 4000), rng.uniform(-1000, 1000, 4000),
                        10.0 ** rng.uniform(-30, 5.7, 2000) * rng.choice([-1.0, 1.0], 2000), k,
                        np.nextafter(k, np.inf), np.nextafter(k, -np.inf), np.array([0.0, -0.0, 5e-324, 2.0 ** -27])])
    s, c = np.empty_like(x), np.empty_like(x)
    assert lib.vsincos(x.ctypes.data, s.ctypes.data, c.ctypes.data, x.size) == x.size
    for xi, si, ci in zip(x, s, c):
        assert si == float(mp.sin(mp.mpf(xi))) and ci == float(mp.cos(mp.mpf(xi))), xi.hex()
    assert np.signbit(s[-3]) and not np.signbit(s[-4])
    big = np.array([2.0 ** 19, -1e6, np.inf, np.nan])
    sb, cb = np.empty_like(big), np.empty_like(big)
    assert lib.vsincos(big.ctypes.data, sb.ctypes.data, cb.ctypes.data, big.size) == 0


def test_special_values(lib):
    inf, nan = np.inf, np.nan
    x = np.array([0.0, 0.0, inf, inf, 1.0, 1.0, nan, 2.0, -1.0, 4.0, 2.0, 1e300, 1e-300])
    y = np.array([0.14, -0.5, 0.14, -0.5, 123.0, nan, 0.14, nan, 0.5, 0.5, 0.0, 3.0, 3.0])
    want = np.array([0.0, inf, inf, 0.0, 1.0, nan, nan, nan, nan, 2.0, 1.0, inf, 0.0])
    assert np.array_equal(cr_pow(lib, x, y), want, equal_nan=True)


def test_crpow_table_is_the_generator_output():
    """csrc/crpow_table.h is what csrc/gen_crpow.py writes (60-digit mpmath)."""
    pytest.importorskip("mpmath")
    spec = importlib.util.spec_from_file_location("gen_crpow", os.path.join(CSRC, "gen_crpow.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    assert gen.header() == open(os.path.join(CSRC, "crpow_table.h")).read()


def test_oracle_ref_with_correctly_rounded_powers(po):
    """The oracle's REF rounding with the correctly rounded powers (controller
    "ref", what the kernels' ODE_CTRL_REF mode computes) against its REF
    rounding with libm's pow: the same step counts and final states within a
    small fraction of the error scale; fixed-step solves, which take no
    power, identical."""
    rng = np.random.default_rng(3)
    n = 400
    u0 = rng.uniform(-1, 1, (3, n))
    u0[2] += 20
    p = np.stack([np.full(n, 10.0), rng.uniform(0, 30, n), np.full(n, 8 / 3)])
    kw = dict(rounding="ref", abstol=1e-8, reltol=1e-6, nthreads=4)
    a = po.solve("ATsit5", "lorenz", u0, p, (0.0, 5.0), 0.1, controller="ref", **kw)
    b = po.solve("ATsit5", "lorenz", u0, p, (0.0, 5.0), 0.1, **kw)
    assert np.array_equal(a["naccept"], b["naccept"])
    scale = 1e-8 + 1e-6 * np.abs(b["u_final"]).max(0)
    assert (np.abs(a["u_final"] - b["u_final"]).max(0) / scale).max() < 0.1
    f1 = po.solve("Tsit5", "lorenz", u0, p, (0.0, 1.0), 0.01, rounding="ref", controller="ref")
    f2 = po.solve("Tsit5", "lorenz", u0, p, (0.0, 1.0), 0.01, rounding="ref")
    assert np.array_equal(f1["u_final"], f2["u_final"])


def test_oracle_ref_with_correctly_rounded_sines(po):
    """Kuramoto-12 in the oracle's REF rounding with correctly rounded sines
    and cosines (controller "ref") against libm's: the same accepted steps
    and final phases within a small fraction of the error scale."""
    rng = np.random.default_rng(4)
    n = 200
    th = rng.uniform(0, 2 * np.pi, (12, n))
    p = np.vstack([rng.normal(0, 1, (12, n)), rng.uniform(0, 4, (1, n))])
    kw = dict(rounding="ref", abstol=1e-8, reltol=1e-6, nthreads=4)
    a = po.solve("ATsit5", "kuramoto", th, p, (0.0, 10.0), 0.1, controller="ref", **kw)
    b = po.solve("ATsit5", "kuramoto", th, p, (0.0, 10.0), 0.1, **kw)
    assert np.abs(a["naccept"].astype(int) - b["naccept"]).max() <= 1
    scale = 1e-8 + 1e-6 * np.abs(b["u_final"]).max(0)
    assert (np.abs(a["u_final"] - b["u_final"]).max(0) / scale).max() < 1.0
