"""The C ABI library: loads without a GPU, exports every entry point that
include/gb300ode.h declares, and its host-side logic (Julia-range time grid,
argument checking) behaves as specified.  No device computation here."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gb300ode.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|const char\*)\s+(ode_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_expected_entry_points(pkg):
    names = declared_functions()
    assert set(names) == set(pkg._lib.EXPORTS)


def test_library_exports_every_declared_symbol(pkg):
    lib = pkg._lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", pkg._lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (ode_\w+)", out))
    for name in declared_functions():
        assert name in exported, name
        assert getattr(lib, name) is not None
    assert lib.ode_abi_version() == 6


def test_library_needs_no_driver_at_load_time(pkg):
    out = subprocess.run(["ldd", pkg._lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "libcuda" not in out and "libnvrtc" not in out


GRID_CASES = [(0, 0.01, 1), (0, 0.1, 1), (0, 0.3, 1), (0, 0.05 / 11, 0.05), (0.0, 0.1, 100.0), (1.5, 0.25, 4.0),
              (0, 1 / 3, 2), (0, 0.013, 0.5), (-1, 0.07, 1), (0, 1e-3, 0.1), (2.0, 0.1, 1.0), (0, 0.7, 0.7),
              (0.1, 0.2, 0.9), (0, 0.001, 1.0), (0, np.pi / 10, np.pi)]


@pytest.mark.parametrize("t0,dt,tf", GRID_CASES)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fixed_grid_matches_julia_range(pkg, po, t0, dt, tf, precision):
    """The library's C++ restatement of Julia's t0:dt:tf equals the oracle's
    independent Python restatement (element by element)."""
    a = pkg.fixed_grid(t0, dt, tf, precision)
    b = po.julia_range(t0, dt, tf, precision)
    assert len(a) == len(b)
    assert np.array_equal(a, b)


def test_create_without_gpu_fails_cleanly(pkg):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    lib = pkg._lib.load()
    h = ctypes.c_void_p()
    rc = lib.ode_create(ctypes.byref(h), 0)
    assert rc in (pkg._lib.ECUDA, pkg._lib.EINVAL)
    assert not h.value


def test_null_handle_and_bad_arguments(pkg):
    lib = pkg._lib.load()
    assert lib.ode_ensemble_solve(None, None, None, None) == pkg._lib.EINVAL
    n = ctypes.c_int64()
    assert lib.ode_fixed_grid(0.0, 0.0, 1.0, 0, None, 0, ctypes.byref(n)) == pkg._lib.EINVAL
    assert lib.ode_fixed_grid(0.0, float("nan"), 1.0, 0, None, 0, ctypes.byref(n)) == pkg._lib.EINVAL
    assert lib.ode_last_error(None) == b"null handle"


STRUCTS = [("SolveArgs", "ode_solve_args"), ("SolveOut", "ode_solve_out"), ("SolveStats", "ode_solve_stats"),
           ("LearnOpts", "ode_learn_opts"), ("LearnReport", "ode_learn_report"), ("TuneVariant", "ode_tune_variant"),
           ("TuneReport", "ode_tune_report"), ("SdeArgs", "ode_sde_args"), ("SdeOut", "ode_sde_out"),
           ("EverystepOut", "ode_everystep_out")]


def test_ctypes_structs_match_the_c_layout(pkg, tmp_path):
    """Every struct of the Python binding has the size and field offsets that
    a C compiler gives the header's struct."""
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gb300ode.h"', "int main(void) {"]
    expect = []
    for py, c in STRUCTS:
        cls = getattr(pkg._lib, py)
        lines.append('printf("%%zu\\n", sizeof(%s));' % c)
        expect.append(ctypes.sizeof(cls))
        for f in cls._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (c, f[0]))
            expect.append(getattr(cls, f[0]).offset)
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == expect


def test_fixed_grid_property_random_ranges(pkg, po):
    """Property check of the library's Julia-range restatement against the
    oracle's independent one on random (t0, dt, tf), including steps that do
    not divide the span and spans of one point."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @hyp.settings(max_examples=300, deadline=None)
    @hyp.given(st.floats(-100, 100), st.floats(1e-3, 10), st.floats(0, 200))
    def check(t0, dt, span):
        tf = t0 + span
        if span / dt > 1e5:
            return
        a = pkg.fixed_grid(t0, dt, tf, "fp64")
        b = po.julia_range(t0, dt, tf, "fp64")
        assert len(a) == len(b) and np.array_equal(a, b)

    check()


def test_tuning_cache_rejects_bad_files_without_a_gpu(pkg, tmp_path):
    lib = pkg._lib.load()
    assert lib.ode_tune_load(None, b"x") == pkg._lib.EINVAL
    assert lib.ode_tune_save(None, b"x") == pkg._lib.EINVAL


def test_rhs_builtin_without_handle(pkg):
    lib = pkg._lib.load()
    rid = ctypes.c_int(-1)
    assert lib.ode_rhs_builtin(None, 0, 3, ctypes.byref(rid), None) == pkg._lib.EINVAL


def test_python_symbol_tables_match_header_enums(pkg, tmp_path):
    """The package's id tables (_lib.ALG, RHS, PREC, SCHED, CTRL, LAYOUT,
    OUTPUT, KERNEL, SDE) hold the header's enum values, as the C compiler
    gives them."""
    L = pkg._lib
    tables = {
        "ALG": {k: "ODE_ALG_" + k.upper() for k in L.ALG},
        "RHS": {k: "ODE_RHS_" + k.upper() for k in L.RHS},
        "PREC": {"fp64": "ODE_FP64", "fp32": "ODE_FP32", "fp32_kahan": "ODE_FP32_KAHAN"},
        "SCHED": {k: "ODE_SCHED_" + k.upper() for k in L.SCHED},
        "CTRL": {k: "ODE_CTRL_" + k.upper() for k in L.CTRL},
        "LAYOUT": {k: "ODE_LAYOUT_" + k.upper() for k in L.LAYOUT},
        "OUTPUT": {"state": "ODE_OUTPUT_STATE", "kuramoto_r": "ODE_OUTPUT_KURAMOTO_R"},
        "SDE": {k: "ODE_SDE_" + k.upper() for k in L.SDE},
    }
    kernels = {v: "ODE_KERNEL_" + v.upper() for v in L.KERNEL.values()}
    names = sorted({c for t in tables.values() for c in t.values()} | set(kernels.values()))
    src = tmp_path / "enums.c"
    src.write_text('#include <stdio.h>\n#include "%s"\nint main(void) {\n%s  return 0;\n}\n' % (
        HEADER, "".join('  printf("%s %%d\\n", (int)%s);\n' % (n, n) for n in names)))
    exe = tmp_path / "enums"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True, capture_output=True)
    value = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                          check=True).stdout.splitlines())
    for table, mapping in tables.items():
        assert getattr(L, table) == {k: int(value[c]) for k, c in mapping.items()}, table
    assert L.KERNEL == {int(value[c]): k for k, c in kernels.items()}
