"""Table of the double logarithm used by the FP64 step-size controller
(ODE_CTRL_FP64).

Table-driven logarithm after P. T. P. Tang, "Table-driven implementation of
the logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4),
1990: for x = 2^e m, m in [1, 2), the top 7 bits of m's fraction pick
F_j = 1 + j/128 and

    log x = e ln 2 - log(inv_j) + log1p(r),   r = m inv_j - 1 (one fma),

with inv_j = 1/F_j rounded to double (the identity holds exactly for any
inv_j, so inv_j need not be exact) and |r| < 2^-7, where a degree-8 Taylor
polynomial of log1p has truncation error below 2^-66.  Entries with
F_j >= 1.4140625 (j >= 53) fold one ln 2 into the table
(T_j = -log(inv_j) - ln 2, with e + 1 in place of e), so that for x just
below 1 the sum does not cancel two numbers of size ln 2.

Each entry holds inv_j and T_j split into hi + lo doubles, computed in
60-digit arithmetic (mpmath).  Writes log_table.h next to this script;
sde_solver.cuh and the oracle include it.

Usage: python gen_logtab.py
"""
import os

import mpmath as mp

mp.mp.dps = 60
N = 128
SHIFT_FROM = 53  # F_j >= 1.4140625: the entry is taken with e + 1


def table():
    rows = []
    for j in range(N):
        F = mp.mpf(1) + mp.mpf(j) / N
        inv = float(1 / F)  # round to nearest double
        T = -mp.log(mp.mpf(inv))
        if j >= SHIFT_FROM:
            T -= mp.log(2)
        hi = float(T)
        lo = float(T - mp.mpf(hi))
        rows.append((inv, hi, lo))
    return rows


def header():
    out = ["/* generated by gen_logtab.py: {1/F_j, T_j hi, T_j lo} for F_j = 1 + j/128, the logarithm table of\n",
           " * the FP64 step-size controller (T_j = -log(1/F_j rounded), minus ln 2 for j >= %d) */\n" % SHIFT_FROM,
           "#pragma once\n",
           "#ifndef GBODE_LOGTAB_SPACE\n#define GBODE_LOGTAB_SPACE static const\n#endif\n",
           "#define GBODE_LOGTAB_SHIFT_FROM %d\n" % SHIFT_FROM,
           "GBODE_LOGTAB_SPACE double kLogTab[%d][3] = {\n" % N]
    for inv, hi, lo in table():
        out.append("    {%s, %s, %s},\n" % (inv.hex(), hi.hex(), lo.hex()))
    out.append("};\n")
    return "".join(out)


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "log_table.h")
    with open(path, "w") as f:
        f.write(header())
    print("wrote", path)
