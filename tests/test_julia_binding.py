"""The Julia binding's struct definitions (julia/GB300SimpleDiffEq.jl) against
the C header (include/gb300ode.h): the same fields in the same order, and
Julia's C-compatible layout of them (natural alignment, as for isbits
structs passed by Ref to ccall) at the offsets and total size the C compiler
gives.  A field added to one side only fails here."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JL = os.path.join(ROOT, "julia", "GB300SimpleDiffEq.jl")
HDR = os.path.join(ROOT, "include", "gb300ode.h")

PAIRS = {"SolveArgs": "ode_solve_args", "SolveOut": "ode_solve_out", "SolveStats": "ode_solve_stats",
         "EverystepOut": "ode_everystep_out", "SdeArgs": "ode_sde_args", "SdeOut": "ode_sde_out",
         "TuneVariant": "ode_tune_variant", "TuneReport": "ode_tune_report", "LearnOpts": "ode_learn_opts",
         "LearnReport": "ode_learn_report"}
SCALAR = {"Int8": 1, "UInt8": 1, "Int32": 4, "UInt32": 4, "Cint": 4, "Float32": 4, "Int64": 8, "UInt64": 8,
          "Float64": 8, "Csize_t": 8}


def julia_structs():
    text = open(JL).read()
    out = {}
    for m in re.finditer(r"^struct (\w+)\n(.*?)^end", text, re.S | re.M):
        fields = re.findall(r"^\s+(\w+)::(.+?)\s*$", m.group(2), re.M)
        out[m.group(1)] = fields
    return out


def c_structs():
    text = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct \{(.*?)\}\s*(\w+);", text, re.S):
        names = []
        for decl in m.group(1).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            # "type a, b" or "type* a" or "type a[N]"
            decl = re.sub(r"\[.*?\]", "", decl)
            head, *rest = decl.split(",")
            names.append(re.findall(r"(\w+)\s*$", head)[0])
            names += [r.strip().lstrip("*").strip() for r in rest]
        out[m.group(2)] = names
    return out


def julia_layout(structs, name):
    """(offsets, size, align) of a Julia isbits struct laid out C-style."""
    off, pos, align = [], 0, 1
    for _, ty in structs[name]:
        size, a = type_size(structs, ty)
        pos = (pos + a - 1) // a * a
        off.append(pos)
        pos += size
        align = max(align, a)
    return off, (pos + align - 1) // align * align, align


def type_size(structs, ty):
    if ty in SCALAR:
        return SCALAR[ty], SCALAR[ty]
    if ty.startswith("Ptr{"):
        return 8, 8
    m = re.match(r"NTuple\{(\d+), (\w+)\}", ty)
    if m:
        s, a = type_size(structs, m.group(2))
        return int(m.group(1)) * s, a
    if ty in structs:
        _, size, align = julia_layout(structs, ty)
        return size, align
    raise AssertionError("unknown Julia field type " + ty)


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    js = julia_structs()
    d = tmp_path_factory.mktemp("jl")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "%s"' % HDR, "int main(void) {"]
    for jname, cname in PAIRS.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in js[jname]:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = d / "layout.c"
    src.write_text("\n".join(lines))
    exe = d / "layout"
    r = subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = line.split()
        out[(s, f)] = int(v)
    return out


def test_every_c_struct_has_a_julia_twin():
    js, cs = julia_structs(), c_structs()
    assert set(PAIRS.values()) == set(cs), "structs of the header without a Julia binding"
    for jname, cname in PAIRS.items():
        assert [f for f, _ in js[jname]] == cs[cname], jname


@pytest.mark.parametrize("jname", sorted(PAIRS))
def test_field_offsets_and_size(c_layout, jname):
    js = julia_structs()
    cname = PAIRS[jname]
    off, size, _ = julia_layout(js, jname)
    for (f, _), o in zip(js[jname], off):
        assert c_layout[(cname, f)] == o, (jname, f)
    assert c_layout[(cname, "sizeof")] == size, jname


def test_abi_version_matches_header():
    text = open(JL).read()
    v = re.search(r"const ABI_VERSION = (\d+)", text).group(1)
    assert re.search(r"#define ODE_ABI_VERSION %s\b" % v, open(HDR).read())


# the Julia module's symbol tables against the header's enums (names as the header spells them)
ENUM_MAPS = {
    "RHS_BUILTIN": {"lorenz": "ODE_RHS_LORENZ", "vanderpol": "ODE_RHS_VANDERPOL", "r3bp": "ODE_RHS_R3BP",
                    "kuramoto": "ODE_RHS_KURAMOTO", "linear": "ODE_RHS_LINEAR"},
    "PRECISION": {"fp64": "ODE_FP64", "fp32": "ODE_FP32", "fp32_kahan": "ODE_FP32_KAHAN"},
    "SCHEDULE": {"plain": "ODE_SCHED_PLAIN", "persistent": "ODE_SCHED_PERSISTENT", "learned": "ODE_SCHED_LEARNED"},
    "CONTROLLER": {"ds": "ODE_CTRL_DS", "fp64": "ODE_CTRL_FP64", "fp32": "ODE_CTRL_FP32", "ref": "ODE_CTRL_REF"},
    "SDE_BUILTIN": {"gbm": "ODE_SDE_GBM", "ou": "ODE_SDE_OU", "lorenz": "ODE_SDE_LORENZ", "mult": "ODE_SDE_MULT"},
}


def test_symbol_tables_match_header_enums(tmp_path):
    """Every `const X = Dict(:name => id, ...)` table of the Julia module
    names exactly the header's enumerators, with the values the C compiler
    gives them (so a renumbered enum fails here)."""
    text = open(JL).read()
    names = sorted({c for m in ENUM_MAPS.values() for c in m.values()})
    src = tmp_path / "enums.c"
    src.write_text('#include <stdio.h>\n#include "%s"\nint main(void) {\n%s  return 0;\n}\n' % (
        HDR, "".join('  printf("%s %%d\\n", (int)%s);\n' % (n, n) for n in names)))
    exe = tmp_path / "enums"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True, capture_output=True)
    value = {k: int(v) for k, v in (line.split() for line in
                                     subprocess.run([str(exe)], capture_output=True, text=True,
                                                    check=True).stdout.splitlines())}
    for table, mapping in ENUM_MAPS.items():
        m = re.search(r"^const %s = Dict\((.*?)\)\s*$" % table, text, re.M)
        assert m, table
        got = {k: int(v) for k, v in re.findall(r":(\w+) => (\d+)", m.group(1))}
        assert got == {k: value[c] for k, c in mapping.items()}, table
