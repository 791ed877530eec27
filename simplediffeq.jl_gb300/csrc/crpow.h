/* Correctly rounded power function x^y, sine and cosine (cr_sincos, at the
 * end of this file) of the reference-arithmetic mode (ODE_CTRL_REF).
 * x^y = exp(y log x) with the logarithm, the product and the
 * exponential carried in double-double arithmetic (unevaluated sums hi + lo
 * of two doubles, about 100 significant bits; T. J. Dekker, "A
 * floating-point technique for extending the available precision", Numer.
 * Math. 18, 1971), so that the double nearest the double-double result is
 * the correctly rounded x^y unless x^y lies within about 2^-97 relative of a
 * midpoint between two doubles.  Table-driven logarithm and exponential
 * after P. T. P. Tang (ACM TOMS 16(4), 1990 and 15(2), 1989); the tables and
 * the method's details are in gen_crpow.py.
 *
 * Every step is an IEEE double operation or an explicit fused multiply-add,
 * so the kernels (nvcc / NVRTC, --fmad=false) and the CPU oracle (host C++,
 * -ffp-contract=off) compute the same bits.  Domain: x >= 0 or NaN, any
 * finite y (the controller's EEst^beta1 and qold^beta2); x < 0 gives NaN.
 * Results that overflow give +Inf; results below 2^-1022 (subnormal) are
 * not correctly rounded, and below about 2^-1021.9 are flushed to 0. */
#pragma once

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define GBODE_CR __device__ __forceinline__
/* the second phases, taken in about one call in 500: out of line on the
 * device, so that each inlined call site stays small */
#define GBODE_CR_COLD __device__ __noinline__
#define GBODE_CRPOW_SPACE __device__ const
namespace gbode {
GBODE_CR double cr_fma(double a, double b, double c) { return __fma_rn(a, b, c); }
GBODE_CR long long cr_bits(double x) { return __double_as_longlong(x); }
GBODE_CR double cr_from_bits(long long b) { return __longlong_as_double(b); }
}  // namespace gbode
#else
#include <cmath>
#include <cstring>
#define GBODE_CR static inline
#define GBODE_CR_COLD static inline
namespace gbode {
GBODE_CR double cr_fma(double a, double b, double c) { return std::fma(a, b, c); }
GBODE_CR long long cr_bits(double x) { long long b; std::memcpy(&b, &x, 8); return b; }
GBODE_CR double cr_from_bits(long long b) { double x; std::memcpy(&x, &b, 8); return x; }
}  // namespace gbode
#endif
#include "crpow_table.h"
#include "bitops.h"

namespace gbode {

struct ddr { double h, l; };

/* a + b = s + e exactly (Knuth's two-sum) */
GBODE_CR ddr cr_two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
/* a + b = s + e exactly when |a| >= |b| or a == 0 (Dekker's fast two-sum) */
GBODE_CR ddr cr_fast(double a, double b) {
  const double s = a + b;
  return {s, b - (s - a)};
}
/* a * b = p + e exactly */
GBODE_CR ddr cr_two_prod(double a, double b) {
  const double p = a * b;
  return {p, cr_fma(a, b, -p)};
}
GBODE_CR ddr cr_add(ddr x, ddr y) {
  const ddr s = cr_two_sum(x.h, y.h);
  return cr_fast(s.h, s.l + (x.l + y.l));
}
/* double-double times double */
GBODE_CR ddr cr_mul_d(ddr x, double d) {
  const ddr p = cr_two_prod(x.h, d);
  return cr_fast(p.h, cr_fma(x.l, d, p.l));
}
GBODE_CR ddr cr_mul(ddr x, ddr y) {
  const ddr p = cr_two_prod(x.h, y.h);
  return cr_fast(p.h, p.l + cr_fma(x.h, y.l, x.l * y.h));
}

/* log x in double-double for a positive normal or subnormal x */
GBODE_CR ddr cr_log(double x) {
  long long b = cr_bits(x);
  int e = 0;
  if (b < 0x0010000000000000LL) {  /* subnormal: scale by 2^54 */
    b = cr_bits(x * 0x1p54);
    e = -54;
  }
  e += (int)(b >> 52) - 1023;
  const int j = (int)((b >> 44) & 0xff);
  const double m = cr_from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  if (j >= GBODE_CR_FOLD_FROM) e += 1;
  const double r = cr_fma(m, kCrLogTab[j][0], -1.0);  /* exact */
  /* log1p(r): r + r^2 (c2 + r (c3 + ... + r c6)) in double-double, plus r^7 q(r) in double */
  double q = GBODE_CR_LG13;
  q = cr_fma(q, r, GBODE_CR_LG12);
  q = cr_fma(q, r, GBODE_CR_LG11);
  q = cr_fma(q, r, GBODE_CR_LG10);
  q = cr_fma(q, r, GBODE_CR_LG9);
  q = cr_fma(q, r, GBODE_CR_LG8);
  q = cr_fma(q, r, GBODE_CR_LG7);
  ddr a = cr_add({GBODE_CR_LG6_H, GBODE_CR_LG6_L}, cr_fast(0.0, q * r));
  a = cr_add({GBODE_CR_LG5_H, GBODE_CR_LG5_L}, cr_mul_d(a, r));
  a = cr_add({GBODE_CR_LG4_H, GBODE_CR_LG4_L}, cr_mul_d(a, r));
  a = cr_add({GBODE_CR_LG3_H, GBODE_CR_LG3_L}, cr_mul_d(a, r));
  a = cr_add({GBODE_CR_LG2_H, GBODE_CR_LG2_L}, cr_mul_d(a, r));
  const ddr l1p = cr_add(cr_fast(r, 0.0), cr_mul(a, cr_two_prod(r, r)));
  /* e ln2 + T_j: e ln2_a exact, e ln2_b exact as a product pair, e ln2_c in double */
  const double ed = (double)e;
  ddr s = cr_add(cr_two_prod(ed, GBODE_CR_LN2_B), cr_fast(ed * GBODE_CR_LN2_A, ed * GBODE_CR_LN2_C));
  s = cr_add(s, {kCrLogTab[j][1], kCrLogTab[j][2]});
  return cr_add(s, l1p);
}

/* exp z for a double-double z with |z.h| <= 709.7 (2^-1022 <= result <= DBL_MAX) */
GBODE_CR ddr cr_exp(ddr z) {
  const double kb = cr_fma(z.h, GBODE_CR_INV_L64, 0x1.8p52);
  const double kd = kb - 0x1.8p52;
  const int k = (int)(cr_bits(kb) & 0xffffffffLL);  /* kd as a two's-complement integer */
  /* r = z - k ln2/64: k L64_a exact, z.h - k L64_a exact (Sterbenz, or k == 0) */
  const double t1 = cr_fma(-kd, GBODE_CR_L64_A, z.h);
  ddr r = cr_add(cr_two_sum(t1, z.l), cr_two_prod(-kd, GBODE_CR_L64_B));
  r = cr_add(r, cr_fast(-kd * GBODE_CR_L64_C, 0.0));
  /* exp(r.h) (1 + r.l): 1 + r + r^2 (1/2 + r (1/6 + r (1/24 + r (1/120 + r q(r))))) */
  const double x = r.h;
  double q = GBODE_CR_EX11;
  q = cr_fma(q, x, GBODE_CR_EX10);
  q = cr_fma(q, x, GBODE_CR_EX9);
  q = cr_fma(q, x, GBODE_CR_EX8);
  q = cr_fma(q, x, GBODE_CR_EX7);
  q = cr_fma(q, x, GBODE_CR_EX6);
  ddr a = cr_add({GBODE_CR_EX5_H, GBODE_CR_EX5_L}, cr_fast(0.0, q * x));
  a = cr_add({GBODE_CR_EX4_H, GBODE_CR_EX4_L}, cr_mul_d(a, x));
  a = cr_add({GBODE_CR_EX3_H, GBODE_CR_EX3_L}, cr_mul_d(a, x));
  a = cr_add({GBODE_CR_EX2_H, GBODE_CR_EX2_L}, cr_mul_d(a, x));
  ddr er = cr_add(cr_fast(1.0, x), cr_mul(a, cr_two_prod(x, x)));
  er = cr_add(er, cr_mul_d(er, r.l));
  const int jj = k & 63;
  const ddr res = cr_mul({kCrExpTab[jj][0], kCrExpTab[jj][1]}, er);
  /* times 2^(k >> 6): split in two factors so that each is a normal double */
  const int n = k >> 6;
  const int n1 = n / 2, n2 = n - n1;
  const double s1 = cr_from_bits((long long)(n1 + 1023) << 52), s2 = cr_from_bits((long long)(n2 + 1023) << 52);
  return {(res.h * s1) * s2, (res.l * s1) * s2};
}

/* First phase (A. Ziv, "Fast evaluation of elementary mathematical functions
 * with correctly rounded last bit", ACM TOMS 17(3), 1991): the same
 * reductions with the polynomials in double, x^y as hi + lo within 2^-65.5
 * relative for |y| <= 1 (log x to 2^-68 absolute, exp's polynomial and sums
 * to 2^-67); returns true with *out = the double nearest x^y when every value
 * within 2^-63 |hi| of hi + lo rounds to the same double, false otherwise (in
 * about one call in 500), and then cr_pow takes the double-double path. */
GBODE_CR bool cr_pow_fast(double x, double y, double* out) {
  long long b = cr_bits(x);
  int e = 0;
  if (b < 0x0010000000000000LL) {
    b = cr_bits(x * 0x1p54);
    e = -54;
  }
  e += (int)(b >> 52) - 1023;
  const int j = (int)((b >> 44) & 0xff);
  const double m = cr_from_bits((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  if (j >= GBODE_CR_FOLD_FROM) e += 1;
  const double r = cr_fma(m, kCrLogTab[j][0], -1.0);  /* exact */
  /* log1p(r) - r = r^2 (-1/2 + r/3 - ... + r^7/9), in double */
  double q = GBODE_CR_LG9;
  q = cr_fma(q, r, GBODE_CR_LG8);
  q = cr_fma(q, r, GBODE_CR_LG7);
  q = cr_fma(q, r, GBODE_CR_LG6_H);
  q = cr_fma(q, r, GBODE_CR_LG5_H);
  q = cr_fma(q, r, GBODE_CR_LG4_H);
  q = cr_fma(q, r, GBODE_CR_LG3_H);
  q = cr_fma(q, r, GBODE_CR_LG2_H);
  const double pl = (r * r) * q;
  const double ed = (double)e;
  const ddr a = cr_two_sum(ed * GBODE_CR_LN2_A, kCrLogTab[j][1]);
  const ddr s = cr_two_sum(a.h, r);
  const double lo = ((a.l + s.l) + (pl + kCrLogTab[j][2])) + cr_fma(ed, GBODE_CR_LN2_B, ed * GBODE_CR_LN2_C);
  const ddr z = cr_mul_d(cr_fast(s.h, lo), y);
  if (!(bo_le(z.h, 709.0) && bo_le(-708.0, z.h))) return false;
  /* exp(z) = 2^(k>>6) 2^((k&63)/64) exp(r), r = rh + rl */
  const double kb = cr_fma(z.h, GBODE_CR_INV_L64, 0x1.8p52);
  const double kd = kb - 0x1.8p52;
  const int k = (int)(cr_bits(kb) & 0xffffffffLL);
  const double t1 = cr_fma(-kd, GBODE_CR_L64_A, z.h);  /* exact */
  const ddr rr = cr_two_sum(t1, cr_fma(-kd, GBODE_CR_L64_B, z.l));
  const double rh = rr.h, rl = cr_fma(-kd, GBODE_CR_L64_C, rr.l);
  /* exp(r) - 1 = rh + (rl + rh^2 (1/2 + rh/6 + ... + rh^5/5040)) */
  double p = GBODE_CR_EX7;
  p = cr_fma(p, rh, GBODE_CR_EX6);
  p = cr_fma(p, rh, GBODE_CR_EX5_H);
  p = cr_fma(p, rh, GBODE_CR_EX4_H);
  p = cr_fma(p, rh, GBODE_CR_EX3_H);
  p = cr_fma(p, rh, GBODE_CR_EX2_H);
  const double pl2 = cr_fma(rh * rh, p, rl);
  const int jj = k & 63;
  const double th = kCrExpTab[jj][0], tl = kCrExpTab[jj][1];
  /* T (1 + rh + pl2), T = th + tl */
  const ddr tp = cr_two_prod(th, rh);
  const double lo2 = cr_fma(th, pl2, tp.l) + cr_fma(tl, rh, tl);
  const ddr u = cr_two_sum(th, tp.h);
  const ddr v = cr_fast(u.h, u.l + lo2);
  const double d = 0x1p-63 * v.h;  /* v.h > 0 */
  const double up = v.h + (v.l + d), dn = v.h + (v.l - d);
  if (cr_bits(up) != cr_bits(dn)) return false;  /* both positive */
  const int n = k >> 6;
  const int n1 = n / 2, n2 = n - n1;
  *out = (up * cr_from_bits((long long)(n1 + 1023) << 52)) * cr_from_bits((long long)(n2 + 1023) << 52);
  return true;
}

/* x^y in double-double, rounded: the second phase */
GBODE_CR_COLD double cr_pow_dd(double x, double y) {
  const ddr lx = cr_log(x);
  const ddr z = cr_mul_d(lx, y);
  if (z.h > 709.7) return cr_from_bits(0x7ff0000000000000LL);
  if (z.h < -708.3) return 0.0;
  /* v is normalized (v.h is the double nearest v.h + v.l) and the scaling
   * by 2^n in cr_exp is exact for normal results */
  return cr_exp(z).h;
}

/* x^y, correctly rounded (see the header comment) */
GBODE_CR double cr_pow(double x, double y) {
  /* the special cases by integer tests of the bits (a double compare would
   * take an FP64-pipe slot) */
  const long long bx = cr_bits(x), by = cr_bits(y);
  const long long ax = bx & 0x7fffffffffffffffLL, ay = by & 0x7fffffffffffffffLL;
  if (ax > 0x7ff0000000000000LL || ay > 0x7ff0000000000000LL) return x + y;  /* NaN */
  if (ay == 0) return 1.0;
  const bool ypos = by > 0;                                                     /* y > 0 */
  if (ax == 0) return ypos ? 0.0 : cr_from_bits(0x7ff0000000000000LL);          /* x = +-0 */
  if (bx < 0) return cr_from_bits(0x7ff8000000000000LL);                        /* x < 0 */
  if (bx == 0x7ff0000000000000LL) return ypos ? x : 0.0;                        /* x = +Inf */
  if (bx == 0x3ff0000000000000LL) return 1.0;                                   /* x = 1 */
  double f;
  if (ay <= 0x3ff0000000000000LL && cr_pow_fast(x, y, &f)) return f;            /* |y| <= 1 */
  return cr_pow_dd(x, y);
}

/* The second phase of cr_sincos: sin r and cos r from s = r - a_j (sd) and
 * the table's sin a_j, cos a_j, with C(s) and S(s) in double-double */
GBODE_CR_COLD void cr_sincos_dd(ddr sd, double sa_h, double sa_l, double ca_h, double ca_l, double* sr,
                                double* cr) {
  const ddr zz = cr_add(cr_two_prod(sd.h, sd.h), cr_fast(0.0, 2.0 * sd.h * sd.l));
  ddr ac = {GBODE_CR_COS6_H, GBODE_CR_COS6_L};
  ac = cr_add({GBODE_CR_COS5_H, GBODE_CR_COS5_L}, cr_mul(ac, zz));
  ac = cr_add({GBODE_CR_COS4_H, GBODE_CR_COS4_L}, cr_mul(ac, zz));
  ac = cr_add({GBODE_CR_COS3_H, GBODE_CR_COS3_L}, cr_mul(ac, zz));
  ac = cr_add({GBODE_CR_COS2_H, GBODE_CR_COS2_L}, cr_mul(ac, zz));
  ac = cr_add({GBODE_CR_COS1_H, GBODE_CR_COS1_L}, cr_mul(ac, zz));
  const ddr cmd = cr_mul(ac, zz);                          /* cos s - 1 */
  ddr as = {GBODE_CR_SIN6_H, GBODE_CR_SIN6_L};
  as = cr_add({GBODE_CR_SIN5_H, GBODE_CR_SIN5_L}, cr_mul(as, zz));
  as = cr_add({GBODE_CR_SIN4_H, GBODE_CR_SIN4_L}, cr_mul(as, zz));
  as = cr_add({GBODE_CR_SIN3_H, GBODE_CR_SIN3_L}, cr_mul(as, zz));
  as = cr_add({GBODE_CR_SIN2_H, GBODE_CR_SIN2_L}, cr_mul(as, zz));
  as = cr_add({GBODE_CR_SIN1_H, GBODE_CR_SIN1_L}, cr_mul(as, zz));
  const ddr ssd = cr_add(sd, cr_mul(cr_mul(as, zz), sd));  /* sin s */
  const ddr sa = {sa_h, sa_l}, ca = {ca_h, ca_l};
  const ddr one_c = cr_add(cr_fast(1.0, 0.0), cmd);       /* cos s */
  *sr = cr_add(cr_mul(sa, one_c), cr_mul(ca, ssd)).h;
  const ddr nsa = {-sa_h, -sa_l};
  *cr = cr_add(cr_mul(ca, one_c), cr_mul(nsa, ssd)).h;
}

/* Sine and cosine of x, correctly rounded (the two phases of cr_pow): x =
 * k pi/2 + r, |r| <= pi/4, with pi/2 in four parts (the reduction's error is
 * below 2^-105 |r| for |x| < 2^19), r = a_j + s with a_j = j/64, and
 * sin r = sin a_j (1 + C(s)) + cos a_j (s + S(s)), cos r = cos a_j (1 + C(s))
 * - sin a_j (s + S(s)), C(s) = cos s - 1, S(s) = sin s - s.  The first phase
 * takes C and S in double (within 2^-66 relative), the second in
 * double-double.  Returns false for |x| >= 2^19 and non-finite x, which the
 * caller hands to its math library. */
GBODE_CR bool cr_sincos(double x, double* sn, double* cs) {
  const long long ax = cr_bits(x) & 0x7fffffffffffffffLL;
  if (!(ax < 0x4120000000000000LL)) return false;  /* |x| < 2^19, not NaN */
  if (ax < 0x3e40000000000000LL) {                 /* |x| < 2^-27: sin x = x, cos x = 1 rounded */
    *sn = x;
    *cs = 1.0;
    return true;
  }
  const double kb = cr_fma(x, GBODE_CR_TWO_OVER_PI, 0x1.8p52);
  const double kd = kb - 0x1.8p52;
  const int q = (int)(cr_bits(kb) & 3);
  const double t = cr_fma(-kd, GBODE_CR_PIO2_A, x);  /* exact */
  const ddr p2 = cr_two_prod(kd, GBODE_CR_PIO2_B), p3 = cr_two_prod(kd, GBODE_CR_PIO2_C);
  const ddr r0 = cr_two_sum(t, -p2.h);
  const ddr r = cr_two_sum(r0.h, ((r0.l - p2.l) - p3.h) - (p3.l + kd * GBODE_CR_PIO2_D));
  /* signs, magnitudes and the row index by integer operations (a double
   * compare, negation or conversion would take an FP64-pipe slot): j =
   * |rh| * 64 rounded to nearest by the 1.5 * 2^52 shifter, a_j = +-j/64 */
  const double rh = r.h;
  const long long sgn = cr_bits(rh) & (long long)0x8000000000000000ULL;
  const double rabs = cr_from_bits(cr_bits(rh) ^ sgn);
  const double jb = cr_fma(rabs, 64.0, 0x1.8p52);
  const int j = (int)(cr_bits(jb) & 0xff);
  const double aj = cr_from_bits(cr_bits((jb - 0x1.8p52) * 0x1p-6) | sgn);
  const ddr sd = cr_two_sum(rh - aj, r.l);  /* rh - aj exact */
  const double sa_h = cr_from_bits(cr_bits(kCrTrigTab[j][0]) ^ sgn);
  const double sa_l = cr_from_bits(cr_bits(kCrTrigTab[j][1]) ^ sgn);
  const double ca_h = kCrTrigTab[j][2], ca_l = kCrTrigTab[j][3];
  double sr, cr;
  {
    /* first phase */
    const double z = sd.h * sd.h;
    double c = GBODE_CR_COS4_H;
    c = cr_fma(c, z, GBODE_CR_COS3_H);
    c = cr_fma(c, z, GBODE_CR_COS2_H);
    c = cr_fma(c, z, GBODE_CR_COS1_H);
    const double cm = z * c;                                   /* cos s - 1 */
    double sv = GBODE_CR_SIN3_H;
    sv = cr_fma(sv, z, GBODE_CR_SIN2_H);
    sv = cr_fma(sv, z, GBODE_CR_SIN1_H);
    const double sm = (z * sd.h) * sv;                          /* sin s - s */
    const double tail = sd.l + sm;
    /* sin r = sa + ca sh + (sa cm + ca tail + ca_l sh + sa_l) */
    const ddr m1 = cr_two_prod(ca_h, sd.h);
    const ddr u1 = cr_two_sum(sa_h, m1.h);
    const double lo1 = u1.l + (m1.l + (cr_fma(sa_h, cm, sa_l) + cr_fma(ca_h, tail, ca_l * sd.h)));
    const ddr vs = cr_fast(u1.h, lo1);
    /* cos r = ca - sa sh + (ca cm - sa tail - sa_l sh + ca_l) */
    const ddr m2 = cr_two_prod(-sa_h, sd.h);
    const ddr u2 = cr_two_sum(ca_h, m2.h);
    const double lo2 = u2.l + (m2.l + (cr_fma(ca_h, cm, ca_l) - cr_fma(sa_h, tail, sa_l * sd.h)));
    const ddr vc = cr_fast(u2.h, lo2);
    const double ds = 0x1p-62 * cr_from_bits(cr_bits(vs.h) & 0x7fffffffffffffffLL), dc = 0x1p-62 * vc.h;
    /* the rounding tests compare bits (neither side is zero or NaN here) */
    const bool oks = cr_bits(vs.h + (vs.l + ds)) == cr_bits(vs.h + (vs.l - ds));
    const bool okc = cr_bits(vc.h + (vc.l + dc)) == cr_bits(vc.h + (vc.l - dc));
    sr = vs.h + vs.l;
    cr = vc.h + vc.l;
    if (!(oks && okc)) cr_sincos_dd(sd, sa_h, sa_l, ca_h, ca_l, &sr, &cr);
  }
  /* quadrant q: (sin, cos) = (sr, cr), (cr, -sr), (-sr, -cr), (-cr, sr), the
   * negations as sign-bit flips */
  const long long fs = (long long)((unsigned long long)(q & 2) << 62);
  const long long fc = (long long)((unsigned long long)((q + 1) & 2) << 62);
  *sn = cr_from_bits(cr_bits((q & 1) ? cr : sr) ^ fs);
  *cs = cr_from_bits(cr_bits((q & 1) ? sr : cr) ^ fc);
  return true;
}

}  // namespace gbode
