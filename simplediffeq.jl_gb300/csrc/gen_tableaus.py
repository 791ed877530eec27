#!/usr/bin/env python3
"""Extract the Runge-Kutta coefficient tables of SimpleDiffEq.jl into a C header.

The numbers in ``tableaus.h`` must be exactly the numbers the reference uses,
so they are read from the reference's own source files rather than typed in:

* Tsitouras 5(4): ``src/tsit5/atsit5_cache.jl:1-105`` (``cs``, ``as``,
  ``btildes`` and the dense-output ``rs``), the positional names being those of
  ``src/tsit5/gpuatsit5.jl:244-247`` and ``src/tsit5/tsit5.jl:387-388``.
* Verner 7(6) and 9(8): ``src/verner/verner_tableaus.jl`` — every
  ``name = convert(T, literal)`` / ``convert(T2, literal)`` assignment inside
  the constructors ``Vern7ExtraStages`` (:65-135), ``Vern7InterpolationCoefficients``
  (:219-311), ``Vern7Tableau`` (:376-452), ``Vern9ExtraStages`` (:595-751),
  ``Vern9InterpolationCoefficients`` (:909-1083) and ``Vern9Tableau``
  (:1201-1335).  Commented-out assignments (the unused ``bhat`` row) are skipped.

Each literal is written back with ``repr(float(literal))`` — the shortest
string that round-trips to the same IEEE double — so C's ``strtod`` yields the
bit pattern Julia's parser gives the same literal.  Float32 variants are made
by the consumer with ``(float)value``, which is what ``convert(Float32, x)``
does to a Float64 literal.

Usage: ``python gen_tableaus.py <reference root> <output header>``.
"""
import re
import sys
from pathlib import Path

ASSIGN = re.compile(r"^\s*([A-Za-z_][A-Za-z0-9_]*)\s*=\s*convert\(\s*(T2?)\s*,\s*([-+0-9.eE]+)\s*\)\s*$")

TSIT5_C = ["c1", "c2", "c3", "c4", "c5", "c6"]
TSIT5_A = ["a21", "a31", "a32", "a41", "a42", "a43", "a51", "a52", "a53", "a54",
           "a61", "a62", "a63", "a64", "a65", "a71", "a72", "a73", "a74", "a75", "a76"]
TSIT5_BT = ["btilde1", "btilde2", "btilde3", "btilde4", "btilde5", "btilde6", "btilde7"]
TSIT5_R = ["r11", "r12", "r13", "r14", "r22", "r23", "r24", "r32", "r33", "r34", "r42",
           "r43", "r44", "r52", "r53", "r54", "r62", "r63", "r64", "r72", "r73", "r74"]


def _literal(text):
    return repr(float(text))


def _svector_literals(body):
    """All numeric literals of an ``SVector{N, T}(...)`` constructor body, in order."""
    body = re.sub(r"#=.*?=#", "", body)
    vals = []
    for m in re.finditer(r"convert\(\s*T\s*,\s*([-+0-9.eE]+)\s*\)|(?<![A-Za-z_0-9])([-+]?[0-9]+\.[0-9]*(?:[eE][-+]?[0-9]+)?)", body):
        vals.append(m.group(1) or m.group(2))
    return vals


def parse_tsit5(path):
    src = Path(path).read_text()
    out = {}
    for name, names in (("cs", TSIT5_C), ("as", TSIT5_A), ("btildes", TSIT5_BT), ("rs", TSIT5_R)):
        m = re.search(r"\b%s\s*=\s*SVector\{(\d+),\s*T\}\(" % name, src)
        n = int(m.group(1))
        depth, i = 1, m.end()
        while depth:  # scan to the parenthesis that closes the constructor call
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        vals = _svector_literals(src[m.end():i - 1])
        if len(vals) != n or n != len(names):
            raise SystemExit("tsit5 %s: expected %d literals, found %d" % (name, n, len(vals)))
        for k, v in zip(names, vals):
            out[k] = _literal(v)
    return out


def parse_constructor(src_lines, fname):
    """Ordered (name, literal) pairs of one Julia constructor ``function fname(...)``."""
    start = None
    for i, line in enumerate(src_lines):
        if re.match(r"^(@inline\s+)?function\s+%s\(" % fname, line):
            start = i
            break
    if start is None:
        raise SystemExit("constructor %s not found" % fname)
    pairs = []
    for line in src_lines[start + 1:]:
        if re.match(r"^end\b", line):
            break
        m = ASSIGN.match(line)
        if m:
            pairs.append((m.group(1), _literal(m.group(3))))
    return pairs


def emit(ref_root, out_path):
    ref = Path(ref_root)
    tsit5 = parse_tsit5(ref / "src/tsit5/atsit5_cache.jl")
    vlines = (ref / "src/verner/verner_tableaus.jl").read_text().splitlines()
    groups = [
        ("tsit5", list(tsit5.items()), "src/tsit5/atsit5_cache.jl:1-105"),
        ("vern7", parse_constructor(vlines, "Vern7Tableau"), "src/verner/verner_tableaus.jl:376-452"),
        ("vern7x", parse_constructor(vlines, "Vern7ExtraStages"), "src/verner/verner_tableaus.jl:65-135"),
        ("vern7r", parse_constructor(vlines, "Vern7InterpolationCoefficients"), "src/verner/verner_tableaus.jl:219-311"),
        ("vern9", parse_constructor(vlines, "Vern9Tableau"), "src/verner/verner_tableaus.jl:1201-1335"),
        ("vern9x", parse_constructor(vlines, "Vern9ExtraStages"), "src/verner/verner_tableaus.jl:595-751"),
        ("vern9r", parse_constructor(vlines, "Vern9InterpolationCoefficients"), "src/verner/verner_tableaus.jl:909-1083"),
    ]
    expected = {"tsit5": 56, "vern7": 58, "vern7x": 60, "vern7r": 79,
                "vern9": 108, "vern9x": 135, "vern9r": 153}
    lines = [
        "/* Runge-Kutta coefficient tables of SimpleDiffEq.jl, extracted verbatim.",
        " *",
        " * Generated by gen_tableaus.py from the reference's coefficient files; do",
        " * not edit by hand.  Each group is a namespace of constexpr doubles named",
        " * as in the reference, an enum of positions (<group>_<name>) and an",
        " * initializer list (GBTAB_<GROUP>_INIT) holding the values in that order,",
        " * so device code can place a group in __constant__ memory and index it",
        " * with compile-time positions.",
        " */",
        "#pragma once",
        "",
    ]
    for g, pairs, cite in groups:
        if len(pairs) != expected[g]:
            raise SystemExit("%s: expected %d coefficients, found %d" % (g, expected[g], len(pairs)))
        names = [n for n, _ in pairs]
        if len(set(names)) != len(names):
            raise SystemExit("%s: duplicate names" % g)
        lines.append("/* %s: %s (%d values) */" % (g, cite, len(pairs)))
        lines.append("namespace gbtab { namespace %s {" % g)
        for n, v in pairs:
            lines.append("constexpr double %s = %s;" % (n, v))
        lines.append("} }")
        lines.append("enum gbtab_%s_pos {" % g)
        for i, (n, _) in enumerate(pairs):
            lines.append("  %s_%s = %d," % (g, n, i))
        lines.append("  %s_COUNT = %d" % (g, len(pairs)))
        lines.append("};")
        lines.append("#define GBTAB_%s_INIT { \\" % g.upper())
        for i, (_, v) in enumerate(pairs):
            sep = "," if i + 1 < len(pairs) else ""
            lines.append("  %s%s \\" % (v, sep))
        lines.append("}")
        lines.append("")
    Path(out_path).write_text("\n".join(lines) + "\n")


if __name__ == "__main__":
    if len(sys.argv) != 3:
        raise SystemExit(__doc__)
    emit(sys.argv[1], sys.argv[2])
