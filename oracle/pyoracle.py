"""Python access to the CPU oracle (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It loads ``oracle/_build/liboracle.so`` (a
C++ restatement of SimpleDiffEq.jl's solvers, see oracle.cpp) and provides
``julia_range``, an independent Python statement of how Julia builds the
fixed-step time grid ``tspan[1]:dt:tspan[2]`` that the GPUSimple fixed-step
solvers iterate over (src/tsit5/gpuatsit5.jl:92, src/verner/gpuvern7.jl:101,
src/verner/gpuvern9.jl:99, src/rk4/gpurk4.jl:66).
"""
import ctypes
import math
import os
import subprocess
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

ALG = {"RK4": 0, "Tsit5": 1, "ATsit5": 2, "Vern7": 3, "AVern7": 4, "Vern9": 5, "AVern9": 6,
       "SimpleATsit5": 7, "SimpleTsit5": 8, "Euler": 9}
FIXED = {"RK4", "Tsit5", "Vern7", "Vern9", "SimpleTsit5", "Euler"}
RHS = {"lorenz": 0, "vanderpol": 1, "r3bp": 2, "kuramoto": 3, "linear": 4}
PREC = {"fp64": 0, "fp32": 1, "fp32_kahan": 2}
ROUND = {"ref": 0, "device": 1}
# error norm and step-size controller of the FP64 adaptive solves (DEVICE rounding), as ODE_CTRL_*; with
# REF rounding "ref" takes the controller's powers correctly rounded (the kernels' ODE_CTRL_REF mode)
CTRL = {"ds": 0, "fp64": 1, "fp32": 2, "ref": 3}


class _Args(ctypes.Structure):
    _fields_ = [("alg", ctypes.c_int), ("rhs", ctypes.c_int), ("precision", ctypes.c_int),
                ("rounding", ctypes.c_int), ("n", ctypes.c_int64), ("dim", ctypes.c_int),
                ("nparams", ctypes.c_int), ("t0", ctypes.c_double), ("tf", ctypes.c_double),
                ("dt", ctypes.c_double), ("abstol", ctypes.c_double), ("reltol", ctypes.c_double),
                ("saveat", ctypes.c_void_p), ("nsave", ctypes.c_int64), ("save_everystep", ctypes.c_int),
                ("grid", ctypes.c_void_p), ("ngrid", ctypes.c_int64), ("maxiters", ctypes.c_int64),
                ("u0", ctypes.c_void_p), ("p", ctypes.c_void_p), ("dt0", ctypes.c_void_p),
                ("nthreads", ctypes.c_int), ("output", ctypes.c_int), ("ctrl", ctypes.c_int)]


class _Out(ctypes.Structure):
    _fields_ = [("us", ctypes.c_void_p), ("u_final", ctypes.c_void_p), ("t_final", ctypes.c_void_p),
                ("retcode", ctypes.c_void_p), ("naccept", ctypes.c_void_p), ("nreject", ctypes.c_void_p),
                ("dt_first", ctypes.c_void_p), ("ev_off", ctypes.c_void_p), ("ev_t", ctypes.c_void_p),
                ("ev_u", ctypes.c_void_p)]


class _SdeArgs(ctypes.Structure):
    _fields_ = [("sde", ctypes.c_int), ("rounding", ctypes.c_int), ("n", ctypes.c_int64), ("dim", ctypes.c_int),
                ("nparams", ctypes.c_int), ("t0", ctypes.c_double), ("dt", ctypes.c_double),
                ("nsteps", ctypes.c_int64), ("seed", ctypes.c_uint64), ("u0", ctypes.c_void_p),
                ("p", ctypes.c_void_p), ("us", ctypes.c_void_p), ("u_final", ctypes.c_void_p),
                ("nthreads", ctypes.c_int), ("noise_dim", ctypes.c_int)]


SDE = {"gbm": 0, "ou": 1, "lorenz": 2, "mult": 3}

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.oracle_solve.argtypes = [ctypes.POINTER(_Args), ctypes.POINTER(_Out)]
        _lib.oracle_solve.restype = ctypes.c_int
        _lib.oracle_ctrl_pow.argtypes = [ctypes.c_float, ctypes.c_float]
        _lib.oracle_ctrl_pow.restype = ctypes.c_float
        _lib.oracle_sincos.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        _lib.oracle_sincos.restype = None
        _lib.oracle_sde_solve.argtypes = [ctypes.POINTER(_SdeArgs)]
        _lib.oracle_philox.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib.oracle_philox.restype = None
        _lib.oracle_log.argtypes = [ctypes.c_double]
        _lib.oracle_log.restype = ctypes.c_double
        _lib.oracle_exp.argtypes = [ctypes.c_double]
        _lib.oracle_exp.restype = ctypes.c_double
        _lib.oracle_r3bp_pull_f.argtypes = [ctypes.c_float, ctypes.c_float]
        _lib.oracle_r3bp_pull_f.restype = ctypes.c_float
        for nm in ("oracle_ds_log", "oracle_ds_exp"):
            getattr(_lib, nm).argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_void_p]
            getattr(_lib, nm).restype = None
        _lib.oracle_ds_split.argtypes = [ctypes.c_double, ctypes.c_void_p]
        _lib.oracle_ds_split.restype = None
        for nm in ("oracle_rcp_nr", "oracle_log2_nr", "oracle_exp2_nr"):
            getattr(_lib, nm).argtypes = [ctypes.c_float]
            getattr(_lib, nm).restype = ctypes.c_float
        _lib.oracle_normal_pair.argtypes = [ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        _lib.oracle_normal_pair.restype = None
        _lib.oracle_mlp_forward_backward.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64] + [ctypes.c_void_p] * 5
        _lib.oracle_mlp_forward_backward_dev.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64] + [ctypes.c_void_p] * 5
    return _lib


def ctrl_pow(x, b):
    return lib().oracle_ctrl_pow(x, b)


def sincos(x):
    """The device canon's double (sin x, cos x)."""
    s, c = ctypes.c_double(), ctypes.c_double()
    lib().oracle_sincos(float(x), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def mlp_forward_backward(nin, nh, params, x, y, rounding="exact"):
    """Gradient and loss of the learned-schedule MLP: "exact" in double
    precision, "device" in the device training kernel's rounding (bf16
    operands of every product, fp32 accumulation)."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    grad = np.zeros_like(params)
    loss = np.zeros(1, dtype=np.float32)
    fn = lib().oracle_mlp_forward_backward_dev if rounding == "device" else lib().oracle_mlp_forward_backward
    rc = fn(nin, nh, x.shape[0], params.ctypes.data, x.ctypes.data, y.ctypes.data, grad.ctypes.data,
            loss.ctypes.data)
    assert rc == 0
    return grad, float(loss[0])


def bf16_round(a):
    """Round float32 values to bfloat16 (nearest, ties to even), returned as float32."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


# --------------------------------------------------------------------------- Julia ranges
def _t(T, x):
    return float(np.float32(x)) if T == "fp32" else float(x)


def _narrow_maxint(T):
    # maxintfloat(narrow(T), Int): narrow(Float64) = Float32, narrow(Float32) = Float16
    return 2 ** 24 if T == "fp64" else 2 ** 11


def _maxint(T):
    return 2 ** 53 if T == "fp64" else 2 ** 24


def _rat(x, T):
    """Base.rat: continued-fraction rational approximation, in T arithmetic."""
    y = x
    a = d = 1
    b = c = 0
    m = _narrow_maxint(T)
    while abs(y) <= m:
        f = math.trunc(y)
        y = _t(T, y - f)
        a, c = f * a + c, a
        b, d = f * b + d, b
        if max(abs(a), abs(b)) > m:
            return c, d
        if _t(T, _t(T, a) / _t(T, b)) == x:
            break
        y = _t(T, 1.0 / y) if y != 0 else math.inf
    return a, b


def _jdiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _isbetween(a, x, b):
    return (a <= x <= b) or (b <= x <= a)


def _to_T(fr, T):
    v = float(fr)  # correctly rounded to double
    return _t(T, v)


def julia_range(start, step, stop, T="fp64"):
    """Elements of Julia's ``start:step:stop`` for IEEE floats
    (Base.(:)(start::T, step::T, stop::T), base/twiceprecision.jl)."""
    start, step, stop = _t(T, start), _t(T, step), _t(T, stop)
    if step == 0:
        raise ValueError("range step cannot be zero")
    step_n, step_d = _rat(step, T)
    if step_d != 0 and _t(T, step_n / step_d) == step:
        start_n, start_d = _rat(start, T)
        stop_n, stop_d = _rat(stop, T)
        if start_d != 0 and stop_d != 0 and _t(T, start_n / start_d) == start and _t(T, stop_n / stop_d) == stop:
            den = start_d * step_d // math.gcd(start_d, step_d)
            m = _maxint(T)
            if den != 0 and abs(_t(T, start * den)) <= m and abs(_t(T, step * den)) <= m and \
                    den % start_d == 0 and den % step_d == 0:
                start_n = round(_t(T, start * den))
                step_n = round(_t(T, step * den))
                ln = max(0, _jdiv(den * stop_n - stop_d * start_n + step_n * stop_d, step_n * stop_d))
                if _isbetween(start, _t(T, start + _t(T, (ln - 1) * step)), _t(T, stop + _t(T, step / 2))) and \
                        not _isbetween(start, _t(T, start + _t(T, ln * step)), stop):
                    return np.array([_to_T(Fraction(start_n + i * step_n, den), T) for i in range(ln)])
    lf = _t(T, _t(T, stop - start) / step)
    if lf < 0:
        ln = 0
    elif lf == 0:
        ln = 1
    else:
        ln = round(lf) + 1
        stop2 = _t(T, start + _t(T, (ln - 1) * step))
        ln -= int(start < stop < stop2) + int(start > stop > stop2)
    # literal StepRangeLen: start + (i*step), each rounded once in Float64 (Float32 ranges too), then to T
    return np.array([_to_T(Fraction(float(start) + float(i) * float(step)), T) for i in range(ln)])


# --------------------------------------------------------------------------- solve
def _ptr(a):
    return None if a is None else a.ctypes.data


def solve(alg, rhs, u0, p, tspan, dt, precision="fp64", rounding="ref", abstol=1e-6, reltol=1e-3,
          saveat=None, save_everystep=False, maxiters=0, dt0=None, nthreads=1, grid=None, output="state",
          controller="ds"):
    """Solve n trajectories.  u0: (dim, n) float64, p: (nparams, n) float64.
    Returns a dict of numpy arrays (us is (npoints, dim, n))."""
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    dim, n = u0.shape
    nparams = p.shape[0]
    t0, tf = float(tspan[0]), float(tspan[1])
    if alg in FIXED and grid is None:
        grid = julia_range(t0, dt, tf, "fp32" if precision == "fp32" else "fp64")
    if grid is not None:
        grid = np.ascontiguousarray(grid, dtype=np.float64)
    sv = None if saveat is None else np.ascontiguousarray(saveat, dtype=np.float64)
    if sv is not None:
        npts = len(sv)
    elif (alg in FIXED and save_everystep):
        npts = len(grid)
    else:
        npts = 0
    width = 1 if output == "kuramoto_r" else dim
    out = {
        "us": np.full((npts, width, n), np.nan) if npts else None,
        "u_final": np.zeros((dim, n)),
        "t_final": np.zeros(n),
        "retcode": np.zeros(n, dtype=np.int8),
        "naccept": np.zeros(n, dtype=np.int32),
        "nreject": np.zeros(n, dtype=np.int32),
        "dt_first": np.zeros(n),
    }
    d0 = None if dt0 is None else np.ascontiguousarray(dt0, dtype=np.float64)
    args = _Args(ALG[alg], RHS[rhs], PREC[precision], ROUND[rounding], n, dim, nparams, t0, tf, float(dt),
                 float(abstol), float(reltol), _ptr(sv), 0 if sv is None else len(sv), int(bool(save_everystep)),
                 _ptr(grid), 0 if grid is None else len(grid), int(maxiters), _ptr(u0), _ptr(p), _ptr(d0),
                 int(nthreads), 1 if output == "kuramoto_r" else 0, CTRL[controller])
    o = _Out(_ptr(out["us"]), _ptr(out["u_final"]), _ptr(out["t_final"]), _ptr(out["retcode"]),
             _ptr(out["naccept"]), _ptr(out["nreject"]), _ptr(out["dt_first"]), None, None, None)
    rc = lib().oracle_solve(ctypes.byref(args), ctypes.byref(o))
    if rc != 0:
        raise ValueError("oracle_solve rejected the arguments (rc=%d)" % rc)
    if save_everystep and sv is None and alg not in FIXED:
        # every-step output (ragged): count accepted steps, then solve again writing the rows
        off = np.zeros(n + 1, dtype=np.int64)
        off[1:] = np.cumsum(out["naccept"].astype(np.int64) + 1)
        ts = np.full(off[-1], np.nan)
        us = np.full((off[-1], dim), np.nan)
        o.ev_off, o.ev_t, o.ev_u = _ptr(off), _ptr(ts), _ptr(us)
        rc = lib().oracle_solve(ctypes.byref(args), ctypes.byref(o))
        if rc != 0:
            raise ValueError("oracle_solve rejected the arguments (rc=%d)" % rc)
        out.update(offsets=off, ts_rows=ts, us_rows=us)
    return out


def sde_grid_steps(t0, tf, dt):
    """n - 1 of SimpleEM's n = Int((tf - t0)/dt) + 1; ValueError where Julia's Int() throws."""
    q = (float(tf) - float(t0)) / float(dt)
    if q != np.floor(q) or q < 0:
        raise ValueError("InexactError: (tf - t0)/dt = %r is not an integer" % q)
    return int(q)


def sde_solve(sde, u0, p, tspan, dt, seed, rounding="device", save_everystep=True, nthreads=1, noise_dim=0):
    """SimpleEM (src/euler_maruyama.jl:48-142) for n trajectories with the device
    canon's counter-based normals; noise_dim > 0 for the non-diagonal "mult"
    SDE (dim x noise_dim noise matrix).  Returns u_final (dim, n) and, with
    save_everystep, us (npoints, dim, n) and the grid t."""
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    dim, n = u0.shape
    nsteps = sde_grid_steps(tspan[0], tspan[1], dt)
    us = np.full((nsteps + 1, dim, n), np.nan) if save_everystep else None
    uf = np.zeros((dim, n))
    a = _SdeArgs(SDE[sde], ROUND[rounding], n, dim, p.shape[0], float(tspan[0]), float(dt), nsteps, int(seed),
                 _ptr(u0), _ptr(p), _ptr(us), _ptr(uf), int(nthreads), int(noise_dim))
    if lib().oracle_sde_solve(ctypes.byref(a)) != 0:
        raise ValueError("oracle_sde_solve rejected the arguments")
    # t_k = fma(k, dt, t0): one rounding of the exact value
    t = np.array([float(Fraction(k) * Fraction(float(dt)) + Fraction(float(tspan[0]))) for k in range(nsteps + 1)])
    return {"u_final": uf, "us": us, "t": t}


def philox(counter, key):
    c = (ctypes.c_uint32 * 4)(*counter)
    k = (ctypes.c_uint32 * 2)(*key)
    out = (ctypes.c_uint32 * 4)()
    lib().oracle_philox(c, k, out)
    return list(out)


def log_dev(x):
    return lib().oracle_log(float(x))


def exp_dev(x):
    """The device canon's double exponential (table-driven, |x| < 700)."""
    return lib().oracle_exp(float(x))


def fp32_ctrl(fn, x):
    """The single-precision modes' rcp_nr / log2_nr / exp2_nr of the device canon."""
    return getattr(lib(), "oracle_" + fn)(float(x))


def ds(fn, h, l=0.0):
    """The double-single norm's and controller's ds_log / ds_exp of the device
    canon on the pair (h, l) (singles), or ds_split of the double h; returns
    the result pair as two float32 values."""
    out = np.zeros(2, dtype=np.float32)
    if fn == "split":
        lib().oracle_ds_split(float(h), out.ctypes.data)
    else:
        getattr(lib(), "oracle_ds_" + fn)(float(h), float(l), out.ctypes.data)
    return out[0], out[1]


def r3bp_pull_f(mu, r):
    """The device canon's single-precision mu / r^(3/2) (Newton-refined reciprocal square root)."""
    return lib().oracle_r3bp_pull_f(float(mu), float(r))


def normal_pair(seed, pair, idx):
    """Normals z_{2 pair} and z_{2 pair + 1} of trajectory idx's stream (step k
    of a dim-D SDE takes z_{kD} .. z_{kD+D-1})."""
    z0, z1 = ctypes.c_double(), ctypes.c_double()
    lib().oracle_normal_pair(int(seed), int(pair), int(idx), ctypes.byref(z0), ctypes.byref(z1))
    return z0.value, z1.value
