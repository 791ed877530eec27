"""GB300 ensemble solves behind SimpleDiffEq.jl's GPU-solver API.

Host-side mirror of the reference interface, for Python callers and tests:

    prob = ODEProblem("lorenz", u0, (0.0, 10.0), p)          # SciMLBase ODEProblem
    eprob = EnsembleProblem(prob, u0s=U0, ps=P)               # or prob_func=...
    sol = solve(eprob, GPUSimpleATsit5(), trajectories=n, dt=0.1,
                abstol=1e-8, reltol=1e-6, saveat=ts)

The algorithm types and keyword arguments are those of the reference's
GPU-crutch solvers (src/tsit5/gpuatsit5.jl:52,200 and :55-61,205-212;
src/verner/gpuvern7.jl:52,295; src/verner/gpuvern9.jl:52,406;
src/rk4/gpurk4.jl:50) with the same defaults (dt = 0.1, abstol = 1e-6,
reltol = 1e-3).  Every trajectory runs the reference's solver loop on the GPU
through libgb300ode.so; there is no CPU path.  Errors behave like the
reference's: a trajectory that hits dt < dtmin raises ``DtLessThanMin``
(``error("dt<dtmin")`` in the reference), in-place problems are rejected
(``@assert !isinplace(prob)``).
"""
import importlib.util as _ilu
import os as _os
import sys as _sys

import numpy as np

_spec = _ilu.spec_from_file_location(__name__ + "._lib", _os.path.join(_os.path.dirname(__file__), "_lib.py"))
_lib = _ilu.module_from_spec(_spec)
_sys.modules[__name__ + "._lib"] = _lib
_spec.loader.exec_module(_lib)

GB300ODEError = _lib.GB300ODEError
Handle = _lib.Handle
fixed_grid = _lib.fixed_grid


class DtLessThanMin(RuntimeError):
    """Raised where the reference throws ``error("dt<dtmin")``."""


# --------------------------------------------------------------------------- algorithms
class _Alg:
    name = ""
    adaptive = False

    def __repr__(self):
        return "%s()" % type(self).__name__


class GPUSimpleRK4(_Alg):
    """Fixed-step classic RK4 (src/rk4/gpurk4.jl:50). Saves every step."""
    name = "RK4"


class GPUSimpleEuler(_Alg):
    """Fixed-step forward Euler (src/euler/gpueuler.jl:50). Saves every step."""
    name = "Euler"


class GPUSimpleTsit5(_Alg):
    """Fixed-step Tsitouras 5(4) (src/tsit5/gpuatsit5.jl:52)."""
    name = "Tsit5"


class GPUSimpleATsit5(_Alg):
    """Adaptive Tsitouras 5(4) with PI control (src/tsit5/gpuatsit5.jl:200)."""
    name = "ATsit5"
    adaptive = True


class GPUSimpleVern7(_Alg):
    """Fixed-step Verner 7(6) (src/verner/gpuvern7.jl:52)."""
    name = "Vern7"


class GPUSimpleAVern7(_Alg):
    """Adaptive Verner 7(6) (src/verner/gpuvern7.jl:295)."""
    name = "AVern7"
    adaptive = True


class GPUSimpleVern9(_Alg):
    """Fixed-step Verner 9(8) (src/verner/gpuvern9.jl:52)."""
    name = "Vern9"


class GPUSimpleAVern9(_Alg):
    """Adaptive Verner 9(8) (src/verner/gpuvern9.jl:406)."""
    name = "AVern9"
    adaptive = True


def isadaptive(alg):
    """SciMLBase.isadaptive (src/tsit5/gpuatsit5.jl:203 and the Verner files)."""
    return alg.adaptive


# --------------------------------------------------------------------------- problems
class UserRHS:
    """A right-hand side given as the C++ body of
    ``template <class R> __device__ void rhs(R* du, const R* u, const R* p, R t)``,
    compiled for the GPU with NVRTC the first time it is solved."""

    def __init__(self, body, dim, nparams):
        self.body, self.dim, self.nparams = body, int(dim), int(nparams)


class UserOutput:
    """An ensemble output function fused into the solve: the C++ body of
    ``__device__ void output(double* out, const double* u, const double* p, double t)``
    writing ``width`` values per saved point, compiled with NVRTC on first use.
    SciMLBase's ``output_func`` would run on the host for every trajectory."""

    def __init__(self, body, width):
        self.body, self.width = body, int(width)


_BUILTIN_DIMS = {"lorenz": (3, 3), "vanderpol": (2, 1), "r3bp": (4, 1)}


class ODEProblem:
    """Out-of-place ODE problem du = f(u, p, t) on tspan.

    ``f`` is a built-in right-hand side name ("lorenz", "vanderpol", "r3bp",
    "kuramoto", "linear") or a ``UserRHS``.  ``inplace=True`` mirrors an
    in-place Julia problem and is rejected by every GPU solver, as the
    reference asserts ``!isinplace(prob)``."""

    def __init__(self, f, u0, tspan, p=(), inplace=False):
        self.f = f
        self.u0 = np.atleast_1d(np.asarray(u0, dtype=np.float64))
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.p = np.atleast_1d(np.asarray(p, dtype=np.float64)) if np.size(p) else np.zeros(0)
        self.inplace = bool(inplace)

    def remake(self, u0=None, p=None, tspan=None):
        return ODEProblem(self.f, self.u0 if u0 is None else u0, self.tspan if tspan is None else tspan,
                          self.p if p is None else p, self.inplace)


class SimpleEM(_Alg):
    """Fixed-step Euler-Maruyama for SDEProblems (src/euler_maruyama.jl:48).
    The noise comes from a counter-based generator keyed by ``seed``."""
    name = "EM"


class UserSDE:
    """A user SDE: the C++ bodies of
    ``__device__ void drift(double* f, const double* u, const double* p, double t)`` and
    ``__device__ void diffusion(double* g, const double* u, const double* p, double t)``,
    compiled with NVRTC on first use.  With ``noise_dim = M > 0`` the noise is
    non-diagonal and ``diffusion`` writes the dim x M matrix row-major,
    ``g[d * M + m]``."""

    def __init__(self, drift, diffusion, dim, nparams, noise_dim=0):
        self.drift, self.diffusion, self.dim, self.nparams = drift, diffusion, int(dim), int(nparams)
        self.noise_dim = int(noise_dim)


class SDEProblem:
    """Out-of-place SDE du = f(u, p, t) dt + g(u, p, t) dW.  ``sde`` is "gbm"
    (f = mu u, g = sigma u; p = (mu, sigma)), "ou" (f = theta (mu - u),
    g = sigma; p = (theta, mu, sigma)), "lorenz" (Lorenz drift, additive noise;
    p = (sigma, rho, beta, noise)), "mult" (non-diagonal multiplicative noise
    f = mu u, G[d, m] = c[d, m] u[d]; p = (mu, c row-major)) or a UserSDE.
    ``noise_rate_prototype`` (a dim x M array, as in the reference) makes the
    noise non-diagonal with M Wiener processes; without it the noise is
    diagonal (g .* dW)."""

    def __init__(self, sde, u0, tspan, p=(), inplace=False, noise_rate_prototype=None):
        self.f = sde
        self.u0 = np.atleast_1d(np.asarray(u0, dtype=np.float64))
        self.tspan = (float(tspan[0]), float(tspan[1]))
        self.p = np.atleast_1d(np.asarray(p, dtype=np.float64)) if np.size(p) else np.zeros(0)
        self.inplace = bool(inplace)
        self.noise_rate_prototype = None if noise_rate_prototype is None else np.asarray(noise_rate_prototype)
        if self.noise_rate_prototype is not None and (
                self.noise_rate_prototype.ndim != 2 or self.noise_rate_prototype.shape[0] != self.u0.size):
            raise ValueError("noise_rate_prototype must be a (dim, M) array")

    @property
    def noise_dim(self):
        """M of a non-diagonal problem, 0 for diagonal noise."""
        return 0 if self.noise_rate_prototype is None else int(self.noise_rate_prototype.shape[1])


class EnsembleProblem:
    """SciMLBase.EnsembleProblem: ``prob_func(prob, i, repeat)`` returns the
    problem of trajectory i (1-based, as in Julia), or pass the stacked initial
    states ``u0s`` (dim x n) and parameters ``ps`` (nparams x n) directly."""

    def __init__(self, prob, prob_func=None, u0s=None, ps=None):
        self.prob = prob
        self.prob_func = prob_func
        self.u0s = None if u0s is None else np.ascontiguousarray(u0s, dtype=np.float64)
        self.ps = None if ps is None else np.ascontiguousarray(ps, dtype=np.float64)


class ODESolution:
    """Per-trajectory solution: ``t`` and ``u`` (list of state vectors), ``retcode``."""

    def __init__(self, t, u, retcode, naccept=0, nreject=0):
        self.t, self.u, self.retcode = t, u, retcode
        self.naccept, self.nreject = naccept, nreject

    def __len__(self):
        return len(self.u)


_RETNAMES = {0: "Default", 1: "DtLessThanMin", 2: "MaxIters", 3: "Default"}


class EnsembleSolution:
    """Results of an ensemble solve, kept as structure-of-arrays:
    ``us`` (npoints, dim, n), ``u_final`` (dim, n), ``t_final`` (n,),
    ``retcode``, ``naccept``, ``nreject`` (n,), ``t`` (the save times).
    With every-step output of an adaptive solver the points are ragged:
    trajectory i's times and states are rows ``offsets[i]:offsets[i+1]`` of
    ``ts_rows`` (rows,) and ``us_rows`` (rows, dim).
    ``sol[i]`` builds the ODESolution of trajectory i (0-based)."""

    def __init__(self, t, us, u_final, t_final, retcode, naccept, nreject, dt_first, stats, offsets=None,
                 ts_rows=None, us_rows=None):
        self.t, self.us, self.u_final, self.t_final = t, us, u_final, t_final
        self.retcode, self.naccept, self.nreject, self.dt_first = retcode, naccept, nreject, dt_first
        self.stats = stats
        self.offsets, self.ts_rows, self.us_rows = offsets, ts_rows, us_rows
        self.us_traj = None

    def __len__(self):
        return self.u_final.shape[1]

    def __getitem__(self, i):
        if self.offsets is not None:
            a, b = int(self.offsets[i]), int(self.offsets[i + 1])
            return ODESolution(self.ts_rows[a:b].copy(), [self.us_rows[r].copy() for r in range(a, b)],
                               _RETNAMES.get(int(self.retcode[i]), "Failure"), int(self.naccept[i]),
                               int(self.nreject[i]))
        if self.us is not None:
            u = [self.us[j, :, i].copy() for j in range(self.us.shape[0])]
            t = self.t
        else:
            u = [self.u_final[:, i].copy()]
            t = np.array([self.t_final[i]])
        return ODESolution(t, u, _RETNAMES.get(int(self.retcode[i]), "Failure"), int(self.naccept[i]),
                           int(self.nreject[i]))


# --------------------------------------------------------------------------- solve
_handles = {}


def _handle(device=0):
    h = _handles.get(device)
    if h is None:
        h = _handles[device] = Handle(device)
    return h


def _rhs_id(h, f):
    if isinstance(f, str):
        if f not in _lib.RHS:
            raise ValueError("unknown built-in right-hand side %r" % f)
        return _lib.RHS[f]
    if isinstance(f, UserRHS):
        cache = h.__dict__.setdefault("_user_ids", {})
        key = (f.body, f.dim, f.nparams)
        if key not in cache:
            cache[key] = h.compile_rhs(f.body, f.dim, f.nparams)
        return cache[key]
    raise TypeError("f must be a built-in name or a UserRHS (Python callables cannot run on the GPU)")


def _output_id(h, output, dim, nparams):
    if isinstance(output, UserOutput):
        cache = h.__dict__.setdefault("_output_ids", {})
        key = (output.body, output.width, dim, nparams)
        if key not in cache:
            cache[key] = h.compile_output(output.body, dim, nparams, output.width)
        return cache[key]
    if output not in _lib.OUTPUT:
        raise ValueError("output must be 'state', 'kuramoto_r' or a UserOutput")
    return _lib.OUTPUT[output]


def _stack(eprob, trajectories):
    prob = eprob.prob
    if eprob.u0s is not None or eprob.ps is not None:
        u0s = eprob.u0s if eprob.u0s is not None else np.repeat(prob.u0[:, None], trajectories, 1)
        ps = eprob.ps if eprob.ps is not None else np.repeat(prob.p[:, None], trajectories, 1)
        if u0s.shape[1] != trajectories or ps.shape[1] != trajectories:
            raise ValueError("u0s/ps must have `trajectories` columns")
        return u0s, ps
    if eprob.prob_func is None:
        return np.repeat(prob.u0[:, None], trajectories, 1), np.repeat(prob.p[:, None], trajectories, 1)
    u0s = np.zeros((prob.u0.size, trajectories))
    ps = np.zeros((prob.p.size, trajectories))
    for i in range(trajectories):
        pi = eprob.prob_func(prob, i + 1, 1)
        u0s[:, i] = pi.u0
        ps[:, i] = pi.p
    return u0s, ps


def make_args(alg, f_id, u0s, ps, tspan, dt, abstol, reltol, saveat, save_everystep, precision, schedule,
              maxiters, memory=_lib.MEM_HOST, dt0=None, output="state", layout="soa", controller="ds"):
    a = _lib.SolveArgs()
    a.alg = _lib.ALG[alg.name]
    a.rhs = f_id
    a.precision = _lib.PREC[precision]
    a.schedule = _lib.SCHED[schedule]
    a.dim, a.n = u0s.shape
    a.nparams = ps.shape[0]
    a.t0, a.tf = float(tspan[0]), float(tspan[1])
    a.dt, a.abstol, a.reltol = float(dt), float(abstol), float(reltol)
    if saveat is not None:
        a.saveat, a.nsave = saveat.ctypes.data, len(saveat)
    a.save_everystep = int(bool(save_everystep))
    a.memory = memory
    a.maxiters = int(maxiters)
    a.u0, a.p = u0s.ctypes.data, ps.ctypes.data
    a.dt0 = None if dt0 is None else dt0.ctypes.data
    a.output = output if isinstance(output, int) else _lib.OUTPUT[output]
    a.layout = _lib.LAYOUT[layout]
    a.controller = _lib.CTRL[controller]
    return a


def solve(prob, alg, trajectories=None, dt=0.1, abstol=1e-6, reltol=1e-3, saveat=None, save_everystep=None,
          precision="fp64", schedule="persistent", maxiters=0, device=0, dt0=None, throw=True, output="state",
          layout="soa", controller="ds", **kwargs):
    """Solve an EnsembleProblem (or a single ODEProblem as an ensemble of one).

    Unknown keyword arguments are accepted and ignored, as the reference's
    ``kwargs...`` swallows them.  ``save_everystep`` defaults to False for
    ensembles; with ``save_everystep=True`` and no ``saveat`` an adaptive
    solver returns every accepted step, a different number per trajectory
    (ragged output, as the reference's default for one trajectory); for the
    fixed-step algorithms it saves every grid point.  GPUSimpleRK4 and
    GPUSimpleEuler ignore ``saveat`` as the reference does.  ``layout="traj"``
    has the library write each trajectory's saved series contiguously
    (ODE_LAYOUT_TRAJ); ``sol.us`` is then a (npoints, width, n) view of that
    (n, npoints, width) array, ``sol.us_traj``.  ``controller`` picks the error
    norm and step-size controller arithmetic of adaptive FP64 solves: "ds"
    (default, double-single: step sizes follow the reference's to about
    2^-44), "fp64" (double factors on a single-precision norm) or "fp32"
    (single precision throughout), ODE_CTRL_DS / _FP64 / _FP32; or "ref"
    (ODE_CTRL_REF, FP64 only), the reference's arithmetic throughout the
    solve, fixed-step ones included: no fused vector multiply-adds, the
    right-hand sides as written, IEEE division and square root, pow in the
    controller (slower)."""
    single = isinstance(prob, (ODEProblem, SDEProblem))
    eprob = EnsembleProblem(prob) if single else prob
    if isinstance(eprob.prob, SDEProblem) or isinstance(alg, SimpleEM):
        return _solve_sde(eprob, alg, 1 if single else trajectories, dt, save_everystep, device, single,
                          kwargs.get("seed", 0))
    base = eprob.prob
    if base.inplace:
        raise AssertionError("!isinplace(prob)")  # @assert !isinplace(prob) in every GPUSimple solve
    n = 1 if single else trajectories
    if n is None:
        n = eprob.u0s.shape[1] if eprob.u0s is not None else 1
    h = _handle(device)
    fid = _rhs_id(h, base.f)
    u0s, ps = _stack(eprob, n)
    if ps.shape[0] == 0:
        ps = np.zeros((0, n))
    if alg.name in ("RK4", "Euler"):
        # GPUSimpleRK4 and GPUSimpleEuler have no saveat keyword (gpurk4.jl:53-58, gpueuler.jl:53-58);
        # they save every step
        saveat = None
        if save_everystep is None:
            save_everystep = True
    if save_everystep is None:
        save_everystep = False
    ragged = bool(save_everystep) and saveat is None and alg.adaptive
    sv = None if saveat is None else np.ascontiguousarray(np.asarray(saveat, dtype=np.float64))
    if not alg.adaptive:
        schedule = "plain"
    dim = u0s.shape[0]
    args = make_args(alg, fid, u0s, ps, base.tspan, dt, abstol, reltol, sv, save_everystep, precision, schedule,
                     maxiters, dt0=None if dt0 is None else np.ascontiguousarray(dt0, dtype=np.float64),
                     output=_output_id(h, output, dim, ps.shape[0]), layout=layout, controller=controller)
    width = output.width if isinstance(output, UserOutput) else (1 if output == "kuramoto_r" else dim)
    if sv is not None:
        npts = len(sv)
        tpts = sv
    elif not alg.adaptive and save_everystep:
        tpts = fixed_grid(base.tspan[0], dt, base.tspan[1], "fp32" if precision == "fp32" else "fp64")
        npts = len(tpts)
    else:
        npts, tpts = 0, None
    out = {"u_final": np.empty((dim, n)), "t_final": np.empty(n), "retcode": np.empty(n, dtype=np.int8),
           "naccept": np.empty(n, dtype=np.int32), "nreject": np.empty(n, dtype=np.int32),
           "dt_first": np.empty(n)}
    if ragged:
        return _solve_everystep(h, args, out, n, dim, throw, single)
    us_traj = None
    if npts and layout == "traj":
        us_traj = np.empty((n, npts, width))
        us = us_traj.transpose(1, 2, 0)
    else:
        us = np.empty((npts, width, n)) if npts else None
    o = _lib.SolveOut()
    o.us = None if us is None else (us_traj if us_traj is not None else us).ctypes.data
    for k, v in out.items():
        setattr(o, k, v.ctypes.data)
    st = _lib.SolveStats()
    rc = h.solve_raw(args, o, st)
    h.check(rc, allow=(_lib.ETRAJ,))
    sol = EnsembleSolution(tpts, us, out["u_final"], out["t_final"], out["retcode"], out["naccept"],
                           out["nreject"], out["dt_first"], st)
    sol.us_traj = us_traj
    if rc == _lib.ETRAJ and throw:
        if (out["retcode"] == _lib.RET_DTMIN).any():
            raise DtLessThanMin("dt<dtmin")
        raise RuntimeError("maxiters reached")
    return sol[0] if single else sol


def _solve_everystep(h, args, out, n, dim, throw, single):
    """save_everystep = true without saveat for an adaptive solver: ragged
    output through ode_ensemble_solve_everystep (count, then fill)."""
    args.save_everystep = 0
    offsets = np.empty(n + 1, dtype=np.int64)
    eo = _lib.EverystepOut()
    eo.offsets = offsets.ctypes.data
    for k in ("u_final", "t_final", "retcode", "naccept", "nreject"):
        setattr(eo, k, out[k].ctypes.data)
    st = _lib.SolveStats()
    rc = h.solve_everystep(args, eo, st)
    if rc != _lib.ESMALL:
        h.check(rc, allow=(_lib.ETRAJ,))
    ts = np.empty(eo.total)
    us = np.empty((eo.total, dim))
    eo.ts, eo.us, eo.capacity = ts.ctypes.data, us.ctypes.data, eo.total
    rc = h.solve_everystep(args, eo, st)
    h.check(rc, allow=(_lib.ETRAJ,))
    out["dt_first"][:] = np.nan
    sol = EnsembleSolution(None, None, out["u_final"], out["t_final"], out["retcode"], out["naccept"],
                           out["nreject"], out["dt_first"], st, offsets=offsets, ts_rows=ts, us_rows=us)
    if rc == _lib.ETRAJ and throw:
        if (out["retcode"] == _lib.RET_DTMIN).any():
            raise DtLessThanMin("dt<dtmin")
        raise RuntimeError("maxiters reached")
    return sol[0] if single else sol


def _solve_sde(eprob, alg, n, dt, save_everystep, device, single, seed):
    """SimpleEM over the ensemble (ode_sde_solve); saves every grid point by
    default, as the reference does."""
    base = eprob.prob
    if not isinstance(base, SDEProblem) or not isinstance(alg, SimpleEM):
        raise TypeError("SimpleEM solves SDEProblems, and SDEProblems need SimpleEM")
    if base.inplace:
        raise NotImplementedError("in-place SDE functions: give the out-of-place form")
    if n is None:
        n = eprob.u0s.shape[1] if eprob.u0s is not None else 1
    h = _handle(device)
    u0s, ps = _stack(eprob, n)
    dim, nparams = u0s.shape[0], ps.shape[0]
    if ps.shape[0] == 0:
        ps = np.zeros((0, n))
    M = base.noise_dim
    if isinstance(base.f, UserSDE):
        if base.f.noise_dim != M:
            raise ValueError("the UserSDE was declared with noise_dim %d, the problem's noise_rate_prototype has %d "
                             "columns" % (base.f.noise_dim, M))
        cache = h.__dict__.setdefault("_sde_ids", {})
        key = (base.f.drift, base.f.diffusion, base.f.dim, base.f.nparams, M)
        if key not in cache:
            cache[key] = h.compile_sde(base.f.drift, base.f.diffusion, base.f.dim, base.f.nparams, M)
        sid = cache[key]
    else:
        sid = _lib.SDE[base.f]
    every = True if save_everystep is None else bool(save_everystep)
    t0, tf = base.tspan
    q = (tf - t0) / float(dt)
    if q != np.floor(q) or q < 0:
        raise ValueError("InexactError: (tf - t0)/dt = %r is not an integer" % q)
    nsteps = int(q)
    a = _lib.SdeArgs()
    a.sde, a.n, a.dim, a.nparams, a.noise_dim = sid, n, dim, nparams, M
    a.t0, a.tf, a.dt, a.seed = t0, tf, float(dt), int(seed)
    a.save_everystep, a.memory = int(every), _lib.MEM_HOST
    a.u0, a.p = u0s.ctypes.data, ps.ctypes.data
    us = np.empty((nsteps + 1, dim, n)) if every else None
    uf = np.empty((dim, n))
    o = _lib.SdeOut()
    o.us = None if us is None else us.ctypes.data
    o.u_final = uf.ctypes.data
    st = _lib.SolveStats()
    h.check(h.sde_solve(a, o, st))
    from fractions import Fraction
    t = np.array([float(Fraction(k) * Fraction(float(dt)) + Fraction(t0)) for k in range(nsteps + 1)])
    zeros = np.zeros(n, dtype=np.int32)
    sol = EnsembleSolution(t if every else None, us, uf, np.full(n, t[-1]), np.zeros(n, dtype=np.int8),
                           np.full(n, nsteps, dtype=np.int32), zeros, np.full(n, float(dt)), st)
    return sol[0] if single else sol


def learn_fit(prob, alg, trajectories, device=0, opts=None, **kw):
    """Fit the learned-schedule model of the device handle on a training
    ensemble (solved with the plain schedule) — see ode_learn_fit."""
    h = _handle(device)
    u0s, ps = _stack(prob, trajectories)
    sv = kw.get("saveat")
    sv = None if sv is None else np.ascontiguousarray(np.asarray(sv, dtype=np.float64))
    args = make_args(alg, _rhs_id(h, prob.prob.f), u0s, ps, prob.prob.tspan, kw.get("dt", 0.1),
                     kw.get("abstol", 1e-6), kw.get("reltol", 1e-3), sv, False, kw.get("precision", "fp64"),
                     "plain", kw.get("maxiters", 0))
    return h.learn_fit(args, opts)


__all__ = ["ODEProblem", "SDEProblem", "EnsembleProblem", "EnsembleSolution", "ODESolution", "UserRHS", "UserOutput",
           "UserSDE", "SimpleEM", "solve", "learn_fit", "GPUSimpleRK4", "GPUSimpleEuler", "GPUSimpleTsit5", "GPUSimpleATsit5", "GPUSimpleVern7", "GPUSimpleAVern7",
           "GPUSimpleVern9", "GPUSimpleAVern9", "isadaptive", "DtLessThanMin", "GB300ODEError", "Handle",
           "fixed_grid"]
