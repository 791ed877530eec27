"""ctypes binding of libgb300ode.so (include/gb300ode.h).

The library is built in-tree by ``csrc/build.py`` into ``lib/``.  There is no
fallback: if the shared library is missing or cannot be loaded, every entry
point raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgb300ode.so")

OK, EINVAL, ECUDA, ENOMEM, ENOTSUP, ENVRTC, ETRAJ, ENOMODEL, ESMALL, ECHECK = 0, -1, -2, -3, -4, -5, -6, -7, -8, -9
ALG = {"RK4": 0, "Tsit5": 1, "ATsit5": 2, "Vern7": 3, "AVern7": 4, "Vern9": 5, "AVern9": 6, "Euler": 7}
RHS = {"lorenz": 0, "vanderpol": 1, "r3bp": 2, "kuramoto": 3, "linear": 4}
PREC = {"fp64": 0, "fp32": 1, "fp32_kahan": 2}
KERNEL = {0: "plain", 1: "persistent", 2: "staged", 3: "fixed", 4: "fixedsplit", 5: "onestep"}
CTRL = {"ds": 0, "fp64": 1, "fp32": 2, "ref": 3}
LAYOUT = {"soa": 0, "traj": 1}
SCHED = {"plain": 0, "persistent": 1, "learned": 2}
MEM_HOST, MEM_DEVICE = 0, 1
OUTPUT = {"state": 0, "kuramoto_r": 1}
RET_DEFAULT, RET_DTMIN, RET_MAXITERS, RET_NAN = 0, 1, 2, 3

# Every symbol include/gb300ode.h declares.
EXPORTS = ["ode_abi_version", "ode_create", "ode_destroy", "ode_last_error", "ode_ensemble_solve",
           "ode_fixed_grid", "ode_rhs_compile", "ode_output_compile", "ode_learn_default_opts", "ode_learn_fit",
           "ode_learn_predict", "ode_learn_gradcheck", "ode_ensemble_solve_noalloc", "ode_autotune",
           "ode_ensemble_solve_everystep", "ode_sde_solve", "ode_sde_compile", "ode_sde_compile_noise",
           "ode_set_bounds_check", "ode_tune_save", "ode_tune_load", "ode_rhs_builtin"]
SDE = {"gbm": 0, "ou": 1, "lorenz": 2, "mult": 3}


class SolveArgs(ctypes.Structure):
    _fields_ = [("alg", ctypes.c_int32), ("rhs", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("schedule", ctypes.c_int32), ("n", ctypes.c_int64), ("dim", ctypes.c_int32),
                ("nparams", ctypes.c_int32), ("t0", ctypes.c_double), ("tf", ctypes.c_double),
                ("dt", ctypes.c_double), ("abstol", ctypes.c_double), ("reltol", ctypes.c_double),
                ("saveat", ctypes.c_void_p), ("nsave", ctypes.c_int64), ("save_everystep", ctypes.c_int32),
                ("memory", ctypes.c_int32), ("maxiters", ctypes.c_int64), ("u0", ctypes.c_void_p),
                ("p", ctypes.c_void_p), ("dt0", ctypes.c_void_p), ("stream", ctypes.c_void_p),
                ("output", ctypes.c_int32), ("layout", ctypes.c_int32), ("controller", ctypes.c_int32)]


class SolveOut(ctypes.Structure):
    _fields_ = [("us", ctypes.c_void_p), ("u_final", ctypes.c_void_p), ("t_final", ctypes.c_void_p),
                ("retcode", ctypes.c_void_p), ("naccept", ctypes.c_void_p), ("nreject", ctypes.c_void_p),
                ("dt_first", ctypes.c_void_p)]


class EverystepOut(ctypes.Structure):
    _fields_ = [("offsets", ctypes.c_void_p), ("ts", ctypes.c_void_p), ("us", ctypes.c_void_p),
                ("capacity", ctypes.c_int64), ("total", ctypes.c_int64), ("u_final", ctypes.c_void_p),
                ("t_final", ctypes.c_void_p), ("retcode", ctypes.c_void_p), ("naccept", ctypes.c_void_p),
                ("nreject", ctypes.c_void_p)]


class SdeArgs(ctypes.Structure):
    _fields_ = [("sde", ctypes.c_int32), ("n", ctypes.c_int64), ("dim", ctypes.c_int32), ("nparams", ctypes.c_int32),
                ("t0", ctypes.c_double), ("tf", ctypes.c_double), ("dt", ctypes.c_double), ("seed", ctypes.c_uint64),
                ("save_everystep", ctypes.c_int32), ("memory", ctypes.c_int32), ("u0", ctypes.c_void_p),
                ("p", ctypes.c_void_p), ("stream", ctypes.c_void_p), ("noise_dim", ctypes.c_int32)]


class SdeOut(ctypes.Structure):
    _fields_ = [("us", ctypes.c_void_p), ("u_final", ctypes.c_void_p)]


class SolveStats(ctypes.Structure):
    _fields_ = [("kernel_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("attempts", ctypes.c_int64),
                ("saves", ctypes.c_int64), ("launches", ctypes.c_int32), ("schedule_used", ctypes.c_int32),
                ("graph_replayed", ctypes.c_int32), ("jit", ctypes.c_int32), ("kernel", ctypes.c_int32)]


class LearnOpts(ctypes.Structure):
    _fields_ = [("hidden", ctypes.c_int32), ("epochs", ctypes.c_int32), ("batch", ctypes.c_int32),
                ("lr", ctypes.c_float), ("seed", ctypes.c_uint64), ("seed_dt0", ctypes.c_int32),
                ("dt0_safety", ctypes.c_float)]


class LearnReport(ctypes.Structure):
    _fields_ = [("loss_first", ctypes.c_float), ("loss_last", ctypes.c_float), ("r2_attempts", ctypes.c_float),
                ("train_solve_ms", ctypes.c_double), ("train_fit_ms", ctypes.c_double),
                ("train_kernel_ms", ctypes.c_double), ("train_ctas", ctypes.c_int32)]


TUNE_MAX_VARIANTS = 64


class TuneVariant(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("max_registers", ctypes.c_int32), ("stage_bytes", ctypes.c_int32),
                ("ms", ctypes.c_float)]


class TuneReport(ctypes.Structure):
    _fields_ = [("variants", ctypes.c_int32), ("block", ctypes.c_int32), ("max_registers", ctypes.c_int32),
                ("stage_bytes", ctypes.c_int32), ("default_ms", ctypes.c_double), ("best_ms", ctypes.c_double),
                ("sample", ctypes.c_int64), ("tune_ms", ctypes.c_double), ("ntable", ctypes.c_int32),
                ("table", TuneVariant * TUNE_MAX_VARIANTS)]

    def rows(self):
        """(block, max_registers, stage_bytes, ms) of every variant tried; ms < 0: not compiled."""
        return [(v.block, v.max_registers, v.stage_bytes, v.ms) for v in self.table[:self.ntable]]


class GB300ODEError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gb300ode error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load():
    """Load libgb300ode.so (raises if it is missing: there is no CPU path)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise GB300ODEError(ECUDA, "libgb300ode.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    lib.ode_abi_version.restype = ctypes.c_int
    lib.ode_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    lib.ode_destroy.argtypes = [ctypes.c_void_p]
    lib.ode_destroy.restype = None
    lib.ode_last_error.argtypes = [ctypes.c_void_p]
    lib.ode_last_error.restype = ctypes.c_char_p
    lib.ode_ensemble_solve.argtypes = [ctypes.c_void_p, ctypes.POINTER(SolveArgs), ctypes.POINTER(SolveOut),
                                       ctypes.POINTER(SolveStats)]
    lib.ode_ensemble_solve_everystep.argtypes = [ctypes.c_void_p, ctypes.POINTER(SolveArgs),
                                                 ctypes.POINTER(EverystepOut), ctypes.POINTER(SolveStats)]
    lib.ode_sde_solve.argtypes = [ctypes.c_void_p, ctypes.POINTER(SdeArgs), ctypes.POINTER(SdeOut),
                                  ctypes.POINTER(SolveStats)]
    lib.ode_sde_compile.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, ctypes.c_size_t]
    lib.ode_sde_compile_noise.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_char_p,
                                          ctypes.c_size_t]
    lib.ode_fixed_grid.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    lib.ode_rhs_builtin.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_int)]
    lib.ode_rhs_compile.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, ctypes.c_size_t]
    lib.ode_output_compile.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int), ctypes.c_char_p, ctypes.c_size_t]
    lib.ode_learn_default_opts.argtypes = [ctypes.POINTER(LearnOpts)]
    lib.ode_learn_default_opts.restype = None
    lib.ode_learn_fit.argtypes = [ctypes.c_void_p, ctypes.POINTER(SolveArgs), ctypes.POINTER(LearnOpts),
                                  ctypes.POINTER(LearnReport)]
    lib.ode_learn_predict.argtypes = [ctypes.c_void_p, ctypes.POINTER(SolveArgs), ctypes.c_void_p, ctypes.c_void_p]
    lib.ode_learn_gradcheck.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.ode_autotune.argtypes = [ctypes.c_void_p, ctypes.POINTER(SolveArgs), ctypes.c_int64, ctypes.POINTER(TuneReport)]
    lib.ode_tune_save.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.ode_tune_load.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    lib.ode_set_bounds_check.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.ode_ensemble_solve_noalloc.argtypes = [ctypes.POINTER(SolveArgs), ctypes.POINTER(SolveOut), ctypes.c_char_p,
                                               ctypes.c_size_t]
    _lib = lib
    return lib


def fixed_grid(t0, dt, tf, precision="fp64"):
    """Julia's t0:dt:tf as the library computes it."""
    lib = load()
    n = ctypes.c_int64(0)
    rc = lib.ode_fixed_grid(float(t0), float(dt), float(tf), PREC[precision], None, 0, ctypes.byref(n))
    if rc != OK:
        raise GB300ODEError(rc, "invalid range")
    out = np.zeros(n.value)
    rc = lib.ode_fixed_grid(float(t0), float(dt), float(tf), PREC[precision], out.ctypes.data, n.value,
                            ctypes.byref(n))
    return out


class Handle:
    """One library handle (device workspace, compiled kernels, learned model)."""

    def __init__(self, device=0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.ode_create(ctypes.byref(h), int(device))
        if rc != OK:
            raise GB300ODEError(rc, "ode_create failed (is a CUDA device visible?)")
        self.h = h

    def close(self):
        if self.h:
            self.lib.ode_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self):
        return self.lib.ode_last_error(self.h).decode()

    def check(self, rc, allow=()):
        if rc != OK and rc not in allow:
            raise GB300ODEError(rc, self.error())
        return rc

    def solve_raw(self, args, out, stats=None):
        return self.lib.ode_ensemble_solve(self.h, ctypes.byref(args), ctypes.byref(out),
                                           ctypes.byref(stats) if stats is not None else None)

    def tune_save(self, path):
        self.check(self.lib.ode_tune_save(self.h, str(path).encode()))

    def tune_load(self, path):
        return self.lib.ode_tune_load(self.h, str(path).encode())

    def set_bounds_check(self, enable=True):
        self.check(self.lib.ode_set_bounds_check(self.h, int(bool(enable))))

    def solve_everystep(self, args, out, stats=None):
        return self.lib.ode_ensemble_solve_everystep(self.h, ctypes.byref(args), ctypes.byref(out),
                                                     ctypes.byref(stats) if stats is not None else None)

    def sde_solve(self, args, out, stats=None):
        return self.lib.ode_sde_solve(self.h, ctypes.byref(args), ctypes.byref(out),
                                      ctypes.byref(stats) if stats is not None else None)

    def rhs_builtin(self, name, dim):
        """(rhs id, number of parameters) of a built-in right-hand side of dimension dim."""
        rid, np_ = ctypes.c_int(-1), ctypes.c_int(-1)
        self.check(self.lib.ode_rhs_builtin(self.h, RHS[name] if isinstance(name, str) else int(name), int(dim),
                                            ctypes.byref(rid), ctypes.byref(np_)))
        return rid.value, np_.value

    def compile_sde(self, drift, diffusion, dim, nparams, noise_dim=0):
        sid = ctypes.c_int(0)
        log = ctypes.create_string_buffer(8192)
        rc = self.lib.ode_sde_compile_noise(self.h, drift.encode(), diffusion.encode(), int(dim), int(noise_dim),
                                            int(nparams), ctypes.byref(sid), log, 8192)
        if rc != OK:
            raise GB300ODEError(rc, self.error() + "\n" + log.value.decode(errors="replace"))
        return sid.value

    def compile_rhs(self, body, dim, nparams):
        rid = ctypes.c_int(0)
        log = ctypes.create_string_buffer(8192)
        rc = self.lib.ode_rhs_compile(self.h, body.encode(), int(dim), int(nparams), ctypes.byref(rid), log, 8192)
        if rc != OK:
            raise GB300ODEError(rc, self.error())
        return rid.value

    def compile_output(self, body, dim, nparams, width):
        oid = ctypes.c_int(0)
        log = ctypes.create_string_buffer(8192)
        rc = self.lib.ode_output_compile(self.h, body.encode(), int(dim), int(nparams), int(width), ctypes.byref(oid),
                                         log, 8192)
        if rc != OK:
            raise GB300ODEError(rc, self.error() + "\n" + log.value.decode(errors="replace"))
        return oid.value

    def learn_fit(self, args, opts=None):
        o = LearnOpts()
        self.lib.ode_learn_default_opts(ctypes.byref(o))
        for k, v in (opts or {}).items():
            setattr(o, k, v)
        rep = LearnReport()
        self.check(self.lib.ode_learn_fit(self.h, ctypes.byref(args), ctypes.byref(o), ctypes.byref(rep)))
        return rep

    def autotune(self, args, sample=0):
        rep = TuneReport()
        self.check(self.lib.ode_autotune(self.h, ctypes.byref(args), int(sample), ctypes.byref(rep)))
        return rep

    def learn_gradcheck(self, nin, nh, params, x, y):
        params = np.ascontiguousarray(params, dtype=np.float32)
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        grad = np.zeros_like(params)
        loss = np.zeros(1, dtype=np.float32)
        self.check(self.lib.ode_learn_gradcheck(self.h, nin, nh, x.shape[0], params.ctypes.data, x.ctypes.data,
                                                y.ctypes.data, grad.ctypes.data, loss.ctypes.data))
        return grad, float(loss[0])

    def learn_predict(self, args, n):
        la = np.zeros(n, dtype=np.float32)
        ld = np.zeros(n, dtype=np.float32)
        self.check(self.lib.ode_learn_predict(self.h, ctypes.byref(args), la.ctypes.data, ld.ctypes.data))
        return la, ld


