"""Tables and constants of the correctly rounded power function, sine and
cosine of the reference-arithmetic mode (crpow.h): x^y = exp(y log x) for x > 0 with log x
and the exponential carried in double-double arithmetic (unevaluated sums
hi + lo of two doubles), about 100 significant bits, so that rounding the
result to double gives the correctly rounded x^y except when x^y lies within
about 2^-97 relative of a midpoint between two doubles.

Logarithm (after P. T. P. Tang, ACM TOMS 16(4), 1990, in double-double): for
x = 2^e m, m in [1, 2), the top 8 bits of m's fraction pick row j; c_j is a
multiple of 2^-9 near 1/m on the row's interval, so that r = m c_j - 1 is
exact in one fma (|r| < 2^-8: m c_j - 1 is a multiple of 2^-61 below 2^-8
in magnitude, 53 bits), and

    log x = e ln2 + T_j + log1p(r),   T_j = -log c_j.

Rows with c_j < 1/sqrt(2) fold one ln 2 into T_j (T_j = -log c_j - ln 2,
taken with e + 1), so that for x just below 1 the sum does not cancel two
numbers of size ln 2.  log1p(r) = r - r^2/2 + ... + r^13/13: the terms to
r^6 in double-double, the rest in double (their rounding is below 2^-106).

Exponential (after Tang, ACM TOMS 15(2), 1989, in double-double): k =
round(z 64/ln2), z = k ln2/64 + r, exp z = 2^(k>>6) 2^((k&63)/64) exp(r),
|r| < 2^-7.4, exp(r) = 1 + r + ... + r^11/11!: the terms to r^5 in
double-double, the rest in double.  ln 2 and ln2/64 are split in three
doubles, the first with 40 and 36 significant bits, so that e ln2_a
(|e| < 2^11) and k (ln2/64)_a (|k| < 2^17) are exact.

Sine and cosine (cr_sincos, the same two-phase method): x = k pi/2 + r with
pi/2 split in four doubles (the first with 33 significant bits, so that
k (pi/2)_a is exact for |k| < 2^20), r in double-double; r = a_j + s with
a_j = j/64 (|s| <= 1/128) and

    sin r = sin a_j (1 + C(s)) + cos a_j (s + S(s)),
    cos r = cos a_j (1 + C(s)) - sin a_j (s + S(s)),

C(s) = cos s - 1, S(s) = sin s - s, with sin a_j and cos a_j (j = 0..50)
from this table in double-double and the series coefficients 1/n! in
double-double.

All values in 60-digit arithmetic (mpmath).  Writes crpow_table.h next to
this script; crpow.h includes it.

Usage: python gen_crpow.py
"""
import os

import mpmath as mp

mp.mp.dps = 60
NLOG = 256
NEXP = 64
NTRIG = 51  # a_j = j/64 covers |r| <= pi/4 + 1/128


def dbl(x):
    return float(mp.mpf(x))


def split2(v):
    hi = dbl(v)
    lo = dbl(mp.mpf(v) - mp.mpf(hi))
    return hi, lo


def split3(v, lead_bits):
    v = mp.mpf(v)
    e = int(mp.floor(mp.log(abs(v), 2)))
    q = mp.mpf(2) ** (e - lead_bits + 1)
    a = float(mp.nint(v / q) * q)
    b, c = split2(v - mp.mpf(a))
    return a, b, c


def log_rows():
    rows = []
    ln2 = mp.log(2)
    for j in range(NLOG):
        lo_m = 1 + mp.mpf(j) / NLOG
        hi_m = 1 + mp.mpf(j + 1) / NLOG - mp.mpf(2) ** -52
        mid = (lo_m + hi_m) / 2
        c = mp.nint(512 / mid) / 512
        assert abs(lo_m * c - 1) < mp.mpf(2) ** -8 and abs(hi_m * c - 1) < mp.mpf(2) ** -8, j
        t = -mp.log(c)
        fold = c < 1 / mp.sqrt(2)
        if fold:
            t -= ln2
        h, l = split2(t)
        rows.append((float(c), h, l, 1 if fold else 0))
    return rows


def sincos_rows():
    return [split2(mp.sin(mp.mpf(j) / 64)) + split2(mp.cos(mp.mpf(j) / 64)) for j in range(NTRIG)]


def exp_rows():
    return [split2(mp.mpf(2) ** (mp.mpf(j) / NEXP)) for j in range(NEXP)]


def hexd(x):
    return float(x).hex() if x != 0 else "0.0"


def header():
    ln2 = mp.log(2)
    consts = {}
    consts["LN2_A"], consts["LN2_B"], consts["LN2_C"] = split3(ln2, 40)
    consts["L64_A"], consts["L64_B"], consts["L64_C"] = split3(ln2 / NEXP, 36)
    consts["INV_L64"] = dbl(NEXP / ln2)
    pio2 = mp.pi / 2
    a = split3(pio2, 33)[0]
    b = dbl(pio2 - mp.mpf(a))
    c = dbl(pio2 - mp.mpf(a) - mp.mpf(b))
    d = dbl(pio2 - mp.mpf(a) - mp.mpf(b) - mp.mpf(c))
    consts["PIO2_A"], consts["PIO2_B"], consts["PIO2_C"], consts["PIO2_D"] = a, b, c, d
    consts["TWO_OVER_PI"] = dbl(2 / mp.pi)
    out = ["/* generated by gen_crpow.py: tables and constants of the correctly rounded power, sine and cosine */\n",
           "#pragma once\n",
           "#ifndef GBODE_CRPOW_SPACE\n#define GBODE_CRPOW_SPACE static const\n#endif\n"]
    for k, v in consts.items():
        out.append("#define GBODE_CR_%s %s\n" % (k, hexd(v)))
    # log1p coefficients (-1)^(k+1)/k: k = 2..6 double-double, 7..13 double
    for k in range(2, 7):
        h, l = split2(mp.mpf((-1) ** (k + 1)) / k)
        out.append("#define GBODE_CR_LG%d_H %s\n#define GBODE_CR_LG%d_L %s\n" % (k, hexd(h), k, hexd(l)))
    for k in range(7, 14):
        out.append("#define GBODE_CR_LG%d %s\n" % (k, hexd(dbl(mp.mpf((-1) ** (k + 1)) / k))))
    # exp coefficients 1/n!: n = 2..5 double-double, 6..11 double
    for n in range(2, 6):
        h, l = split2(1 / mp.factorial(n))
        out.append("#define GBODE_CR_EX%d_H %s\n#define GBODE_CR_EX%d_L %s\n" % (n, hexd(h), n, hexd(l)))
    for n in range(6, 12):
        out.append("#define GBODE_CR_EX%d %s\n" % (n, hexd(dbl(1 / mp.factorial(n)))))
    # (-1)^n / (2n)! for cos s - 1 and (-1)^n / (2n+1)! for sin s - s, n = 1..6, double-double
    for n in range(1, 7):
        h, l = split2(mp.mpf(-1) ** n / mp.factorial(2 * n))
        out.append("#define GBODE_CR_COS%d_H %s\n#define GBODE_CR_COS%d_L %s\n" % (n, hexd(h), n, hexd(l)))
        h, l = split2(mp.mpf(-1) ** n / mp.factorial(2 * n + 1))
        out.append("#define GBODE_CR_SIN%d_H %s\n#define GBODE_CR_SIN%d_L %s\n" % (n, hexd(h), n, hexd(l)))
    out.append("/* row j: sin(j/64) = hi + lo, cos(j/64) = hi + lo */\n")
    out.append("GBODE_CRPOW_SPACE double kCrTrigTab[%d][4] = {\n" % NTRIG)
    for sh, sl, ch, cl in sincos_rows():
        out.append("    {%s, %s, %s, %s},\n" % (hexd(sh), hexd(sl), hexd(ch), hexd(cl)))
    out.append("};\n")
    out.append("/* row j: c_j (a multiple of 2^-9), T_j = hi + lo, and 1 where T_j holds -ln 2 */\n")
    out.append("GBODE_CRPOW_SPACE double kCrLogTab[%d][3] = {\n" % NLOG)
    rows = log_rows()
    for c, h, l, f in rows:
        out.append("    {%s, %s, %s},\n" % (hexd(c), hexd(h), hexd(l)))
    out.append("};\n")
    first_fold = min(j for j, r in enumerate(rows) if r[3])
    assert all(r[3] for r in rows[first_fold:])
    out.append("#define GBODE_CR_FOLD_FROM %d /* rows from here hold -log c_j - ln 2 */\n" % first_fold)
    out.append("/* row j: 2^(j/64) = hi + lo */\n")
    out.append("GBODE_CRPOW_SPACE double kCrExpTab[%d][2] = {\n" % NEXP)
    for h, l in exp_rows():
        out.append("    {%s, %s},\n" % (hexd(h), hexd(l)))
    out.append("};\n")
    return "".join(out)


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "crpow_table.h")
    with open(path, "w") as f:
        f.write(header())
    print("wrote", path)
