"""The FP64 kernels' integer forms of double comparisons
(simplediffeq.jl_gb300/csrc/bitops.h) against the IEEE comparisons they
stand for: the header compiled on the host with g++ and run on a few million
input pairs (every exponent range, neighbours one ulp apart, zeros of both
signs, infinities and NaN)."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "simplediffeq.jl_gb300", "csrc")

SHIM = r'''
#include "bitops.h"
extern "C" {
void cmp(const double* x, const double* y, unsigned char* lt, unsigned char* le, long n) {
  for (long i = 0; i < n; ++i) { lt[i] = gbode::bo_lt(x[i], y[i]); le[i] = gbode::bo_le(x[i], y[i]); }
}
}
'''


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("bitops")
    src, so = d / "shim.cpp", d / "libshim.so"
    src.write_text(SHIM)
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", CSRC, str(src), "-o",
                    str(so)], check=True)
    L = ctypes.CDLL(str(so))
    L.cmp.argtypes = [ctypes.c_void_p] * 4 + [ctypes.c_long]
    return L


def doubles(rng, n):
    """Doubles of many magnitudes: random bit patterns over a wide exponent
    range, midpoints between neighbouring singles and one double ulp either
    side of them, and specials."""
    e = rng.integers(1023 - 160, 1023 + 140, n).astype(np.uint64)
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    s = rng.integers(0, 2, n).astype(np.uint64)
    x = ((s << np.uint64(63)) | (e << np.uint64(52)) | m).view(np.float64)
    f = rng.standard_normal(n // 4).astype(np.float32) * np.float32(1e3)
    nxt = np.nextafter(f, np.float32(np.inf))
    mid = (f.astype(np.float64) + nxt.astype(np.float64)) / 2
    ties = np.concatenate([mid, np.nextafter(mid, np.inf), np.nextafter(mid, -np.inf)])
    fmax = np.float64(np.finfo(np.float32).max)
    tiny = np.float64(np.finfo(np.float32).tiny)
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, fmax, -fmax, np.nextafter(fmax, np.inf),
                      fmax + 2.0 ** 103, fmax + 2.0 ** 104, 2.0 ** 128, tiny, -tiny, np.nextafter(tiny, 0),
                      tiny * (1 - 2.0 ** -25), tiny * (1 - 2.0 ** -24), 2.0 ** -149, 2.0 ** -150, 2.0 ** -151,
                      1 - 2.0 ** -25, 1 - 2.0 ** -26, 2 - 2.0 ** -24, 1.0, 3.0e-39, 1e-45, 1e300, -1e-300])
    return np.concatenate([x, ties, edges, edges * 1.0000001])


def test_comparisons_match_ieee(lib):
    rng = np.random.default_rng(13)
    a = doubles(rng, 500_000)
    b = np.concatenate([rng.permutation(a), a, -a, np.nextafter(a, np.inf)])
    a = np.concatenate([a, a, a, a])
    lt = np.empty(a.size, np.uint8)
    le = np.empty(a.size, np.uint8)
    lib.cmp(a.ctypes.data, b.ctypes.data, lt.ctypes.data, le.ctypes.data, a.size)
    with np.errstate(invalid="ignore"):
        assert np.array_equal(lt.astype(bool), a < b)
        assert np.array_equal(le.astype(bool), a <= b)
    # signed zeros compare equal
    z = np.array([0.0, -0.0, 0.0, -0.0])
    w = np.array([-0.0, 0.0, 0.0, -0.0])
    lib.cmp(z.ctypes.data, w.ctypes.data, lt.ctypes.data, le.ctypes.data, 4)
    assert not lt[:4].any() and le[:4].all()
