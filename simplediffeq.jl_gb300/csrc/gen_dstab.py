"""Tables and constants of the double-single arithmetic: the error norm and
step-size controller of the FP64 solves (ODE_CTRL_DS) and the Box-Muller
normals of the SDE solver, with values held as unevaluated sums hi + lo of two
IEEE single-precision numbers (about 48 significant bits), so that their
logarithm, exponential, square root, sine and cosine run on the
single-precision pipe.

Logarithm (after P. T. P. Tang, ACM TOMS 16(4), 1990, with single-precision
parts): a = 2^E m, m in [1, 2); the top 7 bits of m's fraction pick row j;
c_j is a multiple of 2^-8 near 1/m on the row's interval, so that
r = m c_j - 1 (|r| <= 2^-7, a multiple of 2^-31) is exact in one fma, and

    ln a = E ln2 + (-ln c_j) + ln(1 + r),

with -ln c_j = hi + lo from this table.  Exponential (after Tang, ACM TOMS
15(2), 1989): k = round(x 64/ln2), x = k ln2/64 + r, exp x = 2^(k>>6) *
2^((k&63)/64) * exp(r), with 2^(j/64) = hi + lo from this table.  ln2 and
ln2/64 are split in three singles, the first with 16 significant bits so that
its product with an integer below 2^8 in magnitude is exact.  The
controller's constants (src/SimpleDiffEq.jl: beta1 = 7/50, beta2 = 2/25,
qmax = 10, qmin = 1/5, gamma = 9/10, qoldinit = 1e-4, each first rounded to
double as the reference's Float64 cache holds it) are written as hi + lo
singles, their logarithms as hi + lo of the logarithm of that double.

Sine and cosine (the normals' angle, reduced to |r| <= pi/4 exactly): the
Taylor series of sin r / r and cos r in r^2, the terms above 2^-24 in
double-single, the rest in single precision (truncation below 2^-50); pi/2 as
a double-single pair.

All values in 60-digit arithmetic (mpmath).  Writes ds_table.h next to this
script; ode_solver.cuh and the oracle include it.

Usage: python gen_dstab.py
"""
import os

import mpmath as mp
import numpy as np

mp.mp.dps = 60
NLOG = 128
NEXP = 64


def f32(x):
    return float(np.float32(float(x)))


def split2(v):
    """v = hi + lo, hi the nearest single, lo the nearest single to the rest."""
    hi = f32(v)
    lo = f32(mp.mpf(v) - mp.mpf(hi))
    return hi, lo


def split3(v, lead_bits=16):
    """v = a + b + c: a with lead_bits significant bits, b and c singles."""
    v = mp.mpf(v)
    e = int(mp.floor(mp.log(abs(v), 2)))
    q = mp.mpf(2) ** (e - lead_bits + 1)
    a = float(mp.nint(v / q) * q)
    assert f32(a) == a
    b, c = split2(v - mp.mpf(a))
    return a, b, c


def log_rows():
    rows = []
    for j in range(NLOG):
        mid = 1 + (mp.mpf(j) + mp.mpf("0.5")) / NLOG
        c = float(mp.nint(256 / mid)) / 256
        lo_m, hi_m = 1 + mp.mpf(j) / NLOG, 1 + mp.mpf(j + 1) / NLOG - mp.mpf(2) ** -23
        assert abs(lo_m * c - 1) <= mp.mpf(2) ** -7 and abs(hi_m * c - 1) <= mp.mpf(2) ** -7, j
        h, l = split2(-mp.log(mp.mpf(c)))
        rows.append((c, h, l))
    return rows


def exp_rows():
    return [split2(mp.mpf(2) ** (mp.mpf(j) / NEXP)) for j in range(NEXP)]


def hexf(x):
    return "%sf" % float(x).hex() if x != 0 else "0.0f"


def header():
    ln2 = mp.log(2)
    a, b, c = split3(ln2)
    ea, eb, ec = split3(ln2 / NEXP)
    consts = {
        "LN2_A": a, "LN2_B": b, "LN2_C": c,
        "EXP_L_A": ea, "EXP_L_B": eb, "EXP_L_C": ec,
        "EXP_INV_L": f32(NEXP / ln2),
    }
    fact = mp.factorial
    # sin r / r = 1 + r2 (S1 + r2 (S2 + r2 (S3 + r2 (S4 + r2 T(r2))))), T in single precision; cos alike
    trig_ds = {"SIN_C%d" % i: (-1) ** i / fact(2 * i + 1) for i in range(1, 5)}
    trig_ds.update({"COS_C%d" % i: (-1) ** i / fact(2 * i) for i in range(1, 5)})
    trig_ds["PIO2"] = mp.pi / 2
    consts.update({"SIN_T%d" % i: f32((-1) ** i / fact(2 * i + 1)) for i in range(5, 8)})
    consts.update({"COS_T%d" % i: f32((-1) ** i / fact(2 * i)) for i in range(5, 9)})
    dbl = {"B1": 7.0 / 50.0, "B2": 2.0 / 25.0}
    logs = {"LN_QMAXI": 1.0 / 10.0, "LN_QMINI": 5.0, "LN_GAMMA": 9.0 / 10.0, "LN_QOLDINIT": 1.0e-4}
    out = ["/* generated by gen_dstab.py: tables and constants of the double-single error norm,\n",
           " * step-size controller and normals (values as hi + lo single-precision pairs) */\n",
           "#pragma once\n",
           "#ifndef GBODE_DSTAB_SPACE\n#define GBODE_DSTAB_SPACE static const\n#endif\n"]
    for k, v in consts.items():
        out.append("#define GBODE_DS_%s %s\n" % (k, hexf(v)))
    for k, v in dbl.items():
        h, l = split2(mp.mpf(v))
        out.append("#define GBODE_DS_%s_H %s\n#define GBODE_DS_%s_L %s\n" % (k, hexf(h), k, hexf(l)))
    for k, v in logs.items():
        h, l = split2(mp.log(mp.mpf(v)))
        out.append("#define GBODE_DS_%s_H %s\n#define GBODE_DS_%s_L %s\n" % (k, hexf(h), k, hexf(l)))
    for k, v in trig_ds.items():
        h, l = split2(mp.mpf(v))
        out.append("#define GBODE_DS_%s_H %s\n#define GBODE_DS_%s_L %s\n" % (k, hexf(h), k, hexf(l)))
    out.append("/* row j: c_j (a multiple of 2^-8), -ln c_j = hi + lo */\n")
    out.append("GBODE_DSTAB_SPACE float kDsLogTab[%d][3] = {\n" % NLOG)
    for c, h, l in log_rows():
        out.append("    {%s, %s, %s},\n" % (hexf(c), hexf(h), hexf(l)))
    out.append("};\n/* row j: 2^(j/64) = hi + lo */\n")
    out.append("GBODE_DSTAB_SPACE float kDsExpTab[%d][2] = {\n" % NEXP)
    for h, l in exp_rows():
        out.append("    {%s, %s},\n" % (hexf(h), hexf(l)))
    out.append("};\n")
    return "".join(out)


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ds_table.h")
    with open(path, "w") as f:
        f.write(header())
    print("wrote", path)
