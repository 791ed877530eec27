"""Table of the double exponential used by the FP64 step-size controller.

Table-driven exponential after P. T. P. Tang, "Table-driven implementation
of the exponential function in IEEE floating-point arithmetic", ACM TOMS
15(2), 1989: with n = round(x * 32/ln 2), j = n mod 32, m = (n - j)/32 and
r = x - n ln2/32 (ln2/32 in two parts, so |r| <= ln2/64 + tiny),

    exp(x) = 2^m * 2^(j/32) * exp(r),

where 2^(j/32) comes from the table split into lead + trail doubles and
exp(r) - 1 is the Taylor polynomial of degree 6 (truncation below 2^-59
relative to exp(r)).

Each entry holds 2^(j/32) as lead (rounded to double) + trail (the rest),
computed in 60-digit arithmetic (mpmath).  Writes exp_table.h next to this
script; ode_solver.cuh and the oracle include it.

Usage: python gen_exptab.py
"""
import os

import mpmath as mp

mp.mp.dps = 60
N = 32


def table():
    rows = []
    for j in range(N):
        v = mp.mpf(2) ** (mp.mpf(j) / N)
        lead = float(v)
        trail = float(v - mp.mpf(lead))
        rows.append((lead, trail))
    return rows


def header():
    l1 = mp.log(2) / N
    # ln2/32 in two parts: the lead with 42 significant bits, so n * lead is exact for |n| < 2^11
    lead = float(mp.nint(l1 * 2 ** 47)) / 2 ** 47
    trail = float(l1 - mp.mpf(lead))
    out = ["/* generated by gen_exptab.py: 2^(j/32) = lead + trail for j = 0..31, the exponential table of the\n",
           " * FP64 step-size controller, and ln2/32 in two parts */\n",
           "#pragma once\n",
           "#ifndef GBODE_EXPTAB_SPACE\n#define GBODE_EXPTAB_SPACE static const\n#endif\n",
           "#define GBODE_EXP_INV_L %s /* 32/ln 2 */\n" % float(N / mp.log(2)).hex(),
           "#define GBODE_EXP_L_LEAD %s /* ln2/32, 42 significant bits */\n" % lead.hex(),
           "#define GBODE_EXP_L_TRAIL %s\n" % trail.hex(),
           "GBODE_EXPTAB_SPACE double kExpTab[%d][2] = {\n" % N]
    for a, b in table():
        out.append("    {%s, %s},\n" % (a.hex(), b.hex()))
    out.append("};\n")
    return "".join(out)


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "exp_table.h")
    with open(path, "w") as f:
        f.write(header())
    print("wrote", path)
