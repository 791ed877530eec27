/* Device side of the ensemble solver: one trajectory per thread.
 *
 * Compiled ahead of time by nvcc (kern_*.cu) and at run time by NVRTC for
 * combinations that are not prebuilt, so it includes nothing but project
 * headers (launch parameters, tables, bitops.h) and uses only CUDA built-ins.
 *
 * The solver loop is the reference's (SimpleDiffEq.jl):
 *   adaptive:  src/tsit5/gpuatsit5.jl:250-320, src/verner/gpuvern7.jl:353-520,
 *              src/verner/gpuvern9.jl:461-763 — stages, embedded error, RMS
 *              norm, PI controller with reject/retry, saveat interpolation;
 *   fixed:     src/tsit5/gpuatsit5.jl:95-129, src/verner/gpuvern7.jl:104-224,
 *              src/verner/gpuvern9.jl:102-335, src/rk4/gpurk4.jl:73-85.
 * It is written as a flat loop of attempts (one iteration = one stage
 * evaluation of a step attempt plus its accept/reject decision), which runs
 * the same sequence of operations as the reference's nested
 * `while t < tf; while EEst > 1` loops and lets the persistent kernel hand a
 * finished lane a new trajectory between two attempts.
 *
 * Rounding canon (matched bit for bit by the oracle's DEVICE mode):
 *   - each multiply-add of the reference's expressions is one fused
 *     multiply-add; linear combinations sum_j c_j k_j accumulate left to right
 *     (the nesting @muladd produces); no other operation is fused (the files
 *     are compiled with --fmad=false);
 *   - stage times t + c*dt and Horner steps of the dense-output polynomials
 *     are fused, as Julia fuses scalar muladd;
 *   - FP64 solves (default, GBODE_CTRL_DS): the error norm EEst and the
 *     step-size factor q (EEst^beta1 / qold^beta2 and its clamps, taken on
 *     logarithms) are computed in double-single arithmetic, pairs of singles
 *     split from the doubles by integer operations (ds_* below), the error
 *     estimate's sum multiplied by dt inside the norm, and dt times the
 *     factor as fma(dt, l, dt * h); the norm is double when abstol < 1e-30.
 *     With GBODE_CTRL64 q is double on logarithms (log_dev, exp_dev) on a
 *     single-precision norm; without either, norm and q are single precision
 *     (q with the deterministic ctrl_pow below).  dt, t and the state keep
 *     the solver precision;
 *   - the dense-output abscissa theta multiplies by recip(dt) (a float
 *     reciprocal refined by one Newton step) and the polynomials that start at
 *     theta^2 multiply by one shared theta^2;
 *   - in single precision the restricted three-body pull mu / r^(3/2) is
 *     mu * y^3 with y from rsqrt_nr (no IEEE division or square root);
 *   - in the single-precision modes the error norm and the controller use
 *     rcp_nr, log2_nr and exp2_nr (no IEEE division, square root or branch;
 *     the PI factors on log2 EEst).
 * GBODE_REF (ODE_CTRL_REF, FP64 only) compiles the reference's arithmetic
 * instead: a*b + c of the vector expressions rounded twice (Julia's generic
 * muladd on SVector does not fuse), the right-hand sides and the RK4 update
 * as their plain Julia expressions, theta = (t_save - told) / dt, the
 * polynomials from theta^2 multiplied by theta twice, the error norm in IEEE
 * double with division and square root, and the PI controller with a
 * correctly rounded pow (cr_pow, crpow.h; src/SimpleDiffEq.jl:67-77,
 * src/tsit5/gpuatsit5.jl:272-299); sine and cosine are correctly rounded
 * too (cr_sincos) below 2^19, CUDA's beyond.  Scalar muladds (stage times,
 * Horner steps) stay fused, as Julia fuses them.
 */
#pragma once
#include "ode_kparams.h"
#include "bitops.h"
#ifdef GBODE_REF
#include "crpow.h"
#endif
#include "tableaus.h"
#define GBODE_LOGTAB_SPACE __device__ const
#include "log_table.h"
#define GBODE_EXPTAB_SPACE __device__ const
#include "exp_table.h"

namespace gbode {

/* Bounds-check build (-DGBODE_BOUNDS_CHECK, compiled at run time when a
 * handle asks for it): every index into a caller array is checked against
 * its extent before the access; a violation sets a bit in P.check_flags and
 * the access is skipped (or clamped to a valid index).  Each trajectory start
 * is counted in P.visited, so the host can verify that the schedule handed
 * every trajectory out exactly once.  Without the flag the checks vanish. */
enum { CHK_TRAJ = 1, CHK_SAVE = 2, CHK_STEP = 4, CHK_RING = 8, CHK_ORDER = 16 };
#ifdef GBODE_BOUNDS_CHECK
#define GBODE_CHECK(P, cond, bit) ((cond) ? true : (atomicOr((P).check_flags, (unsigned)(bit)), false))
#else
#define GBODE_CHECK(P, cond, bit) true
#endif

/* ------------------------------------------------------------------ math */
__device__ __forceinline__ double fmaR(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmaR(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double sqrtR(double x) { return __dsqrt_rn(x); }
__device__ __forceinline__ float sqrtR(float x) { return __fsqrt_rn(x); }
__device__ __forceinline__ double absR(double x) { return fabs(x); }
__device__ __forceinline__ float absR(float x) { return fabsf(x); }
/* Sine and cosine of a double with one argument reduction, in 18 double
 * operations.  Method: Cody and Waite's reduction modulo pi/2 (W. J. Cody and
 * W. Waite, Software Manual for the Elementary Functions, 1980) in its fused
 * form: k = x * 2/pi rounded to the nearest integer (one fused multiply-add
 * with 1.5 * 2^52, whose low bits then hold k), r = (x - k*C1) - k*C2 with
 * C1 = pi/2 rounded to double and C2 the rounded remainder, each term one
 * fused multiply-add; then sin r = r + r^3 P(r^2) and cos r = 1 + r^2 Q(r^2)
 * with near-minimax P and Q of degree 5 from csrc/gen_sincos.py, in Horner
 * form.  Within 1.5 ulp (1.7e-16 absolute) of the exact values below 2^19
 * (checked against 40-digit values), except that results below 1e-15 in
 * magnitude (x within 1e-15 of a multiple of pi/2) keep an absolute error
 * below 1e-30 instead of a relative one.  Every step is one IEEE double operation, so the oracle reproduces it
 * bit for bit.  |x| >= 2^19 and non-finite x go to CUDA's sincos. */
__device__ __forceinline__ void sincos_cw(double x, double* s, double* c) {
  /* |x| < 2^19 as an integer compare of the magnitude bits (a double compare
   * would issue on the FP64 pipe; NaN's bits lie above 2^19's, as its IEEE
   * compare is false) */
  if (!(((unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL) < 0x4120000000000000ULL)) {
    sincos(x, s, c);
    return;
  }
  const double kb = __fma_rn(x, 0x1.45f306dc9c883p-1, 0x1.8p52);  /* 2/pi; 1.5 * 2^52 */
  const double k = kb - 0x1.8p52;
  const int q = __double2loint(kb) & 3;
  double r = __fma_rn(-k, 0x1.921fb54442d18p+0, x);
  r = __fma_rn(-k, 0x1.1a62633145c07p-54, r);
  const double z = r * r;
  double ps = 0x1.5d8fd0a40698ep-33;
  ps = __fma_rn(ps, z, -0x1.ae5e5a8d61ce7p-26);
  ps = __fma_rn(ps, z, 0x1.71de3567ccfe8p-19);
  ps = __fma_rn(ps, z, -0x1.a01a019bfde60p-13);
  ps = __fma_rn(ps, z, 0x1.111111110f7d0p-7);
  ps = __fma_rn(ps, z, -0x1.5555555555548p-3);
  const double sr = __fma_rn(z * r, ps, r);
  double pc = 0x1.1b8b9800ee7dap-29;
  pc = __fma_rn(pc, z, -0x1.27df4604d6713p-22);
  pc = __fma_rn(pc, z, 0x1.a019f81ca810ap-16);
  pc = __fma_rn(pc, z, -0x1.6c16c1640a98bp-10);
  pc = __fma_rn(pc, z, 0x1.555555554f0a9p-5);
  pc = __fma_rn(pc, z, -0x1.fffffffffff96p-2);
  const double cr = __fma_rn(z, pc, 1.0);
  /* quadrant q: (sin, cos) = (sr, cr), (cr, -sr), (-sr, -cr), (-cr, sr); the
   * negations flip the sign bit of the high word, off the FP64 pipe */
  const double so = (q & 1) ? cr : sr, co = (q & 1) ? sr : cr;
  *s = __hiloint2double(__double2hiint(so) ^ (int)((unsigned)(q & 2) << 30), __double2loint(so));
  *c = __hiloint2double(__double2hiint(co) ^ (int)((unsigned)((q + 1) & 2) << 30), __double2loint(co));
}
/* sine and cosine of one argument with a single argument reduction */
__device__ __forceinline__ void sincosR(double x, double* s, double* c) {
#ifdef GBODE_REF
  if (!cr_sincos(x, s, c)) sincos(x, s, c);  /* correctly rounded below 2^19 */
#else
  sincos_cw(x, s, c);
#endif
}
__device__ __forceinline__ void sincosR(float x, float* s, float* c) { sincosf(x, s, c); }

/* Julia's min/max propagate NaN; @fastmath min/max are compare-and-select. */
template <class X> __device__ __forceinline__ X jmin(X a, X b) { return (a != a || b != b) ? a + b : (b < a ? b : a); }
template <class X> __device__ __forceinline__ X jmax(X a, X b) { return (a != a || b != b) ? a + b : (b > a ? b : a); }
template <class X> __device__ __forceinline__ X fm_min(X x, X y) { return (y > x) ? x : y; }
template <class X> __device__ __forceinline__ X fm_max(X x, X y) { return (y > x) ? y : x; }

/* min(|a|, |b|) with Julia's NaN propagation.  For doubles it compares the
 * bit patterns as integers (for non-negative IEEE values integer order is
 * numeric order and NaNs sort above +Inf), keeping the work off the FP64 pipe. */
__device__ __forceinline__ double absmin(double a, double b) {
  const unsigned long long MASK = 0x7fffffffffffffffULL, INF = 0x7ff0000000000000ULL;
  const unsigned long long ua = (unsigned long long)__double_as_longlong(a) & MASK;
  const unsigned long long ub = (unsigned long long)__double_as_longlong(b) & MASK;
  const unsigned long long r = (ua > INF) ? ua : ((ub > INF) ? ub : (ua < ub ? ua : ub));
  return __longlong_as_double((long long)r);
}
__device__ __forceinline__ float absmin(float a, float b) { return jmin(fabsf(a), fabsf(b)); }

/* The time comparisons of the solver loops: (T)s <= t for a saveat time s,
 * t < (T)tf, and x < dtmin.  The FP64 kernels, bound by their FP64 pipe,
 * compare doubles with the exact integer forms of bitops.h (a double
 * comparison issues on the FP64 pipe); the single-precision modes, whose
 * long trajectories are bound by one lane's dependency chain, keep the IEEE
 * comparisons and casts, which are shorter on that chain. */
template <class PR> __device__ __forceinline__ bool t_le(double s, typename PR::T t) {
  if (sizeof(typename PR::R) == sizeof(double)) return bo_le(s, (double)t);
  return (typename PR::T)s <= t;
}
template <class PR> __device__ __forceinline__ bool t_lt(typename PR::T t, double tf) {
  if (sizeof(typename PR::R) == sizeof(double)) return bo_lt((double)t, tf);
  return t < (typename PR::T)tf;
}
template <class PR> __device__ __forceinline__ bool d_lt(double x, double y) {
  if (sizeof(typename PR::R) == sizeof(double)) return bo_lt(x, y);
  return x < y;
}

/* 1/x for the dense-output abscissa theta = (t_save - told) / dt: a single
 * precision reciprocal refined by one Newton step in double (relative error
 * below 1e-14, four FP64 operations instead of a full division). */
__device__ __forceinline__ double recip(double x) {
  const double r0 = (double)__frcp_rn((float)x);
  const double e = __fma_rn(-x, r0, 1.0);
  return __fma_rn(r0, e, r0);
}
__device__ __forceinline__ float recip(float x) { return __frcp_rn(x); }

/* a*b + c of a vector expression (linear combinations, state updates): one
 * fused multiply-add, or with GBODE_REF two roundings as the reference's
 * SVector arithmetic does it (the files are compiled with --fmad=false). */
template <class X> __device__ __forceinline__ X vmaddR(X a, X b, X c) {
#ifdef GBODE_REF
  return a * b + c;
#else
  return fmaR(a, b, c);
#endif
}

/* The dense-output abscissa (t_save - told) / dtold: times recip(dtold), or
 * with GBODE_REF the IEEE division. */
template <class T> __device__ __forceinline__ T theta_of(T ts, T told, T dtold, T inv) {
#ifdef GBODE_REF
  return (ts - told) / dtold;
#else
  return (ts - told) * inv;
#endif
}

/* b = theta^2 * ex of a dense-output polynomial that starts at theta^2:
 * one shared theta^2, or with GBODE_REF theta * (theta * ex) as @evalpoly
 * with two leading zero coefficients evaluates it. */
template <class R> __device__ __forceinline__ R th2_times(R th, R th2, R ex) {
#ifdef GBODE_REF
  return th * (th * ex);
#else
  return th2 * ex;
#endif
}

/* Small integers as singles without a conversion instruction (integer-to-
 * float conversions issue on this GPU's FP64 pipe): the bits of 2^23 + i
 * for 0 <= i < 2^23, minus 2^23, exact; small_int_f(i + 127) - 127 for an
 * exponent i >= -127. */
__device__ __forceinline__ float small_int_f(int i) { return __int_as_float(0x4b000000 | i) - 8388608.0f; }

/* Single-precision x^b for the step-size controller (x >= 0 or NaN).
 * log2 from the atanh series of the reduced mantissa, 2^y from the Taylor
 * series of exp on [-ln2/2, ln2/2]; every step is one IEEE single operation,
 * so the result is identical on any IEEE-754 machine. */
__device__ __forceinline__ float ctrl_log2(float x) {
  int e = 0;
  if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; }
  unsigned u = __float_as_uint(x);
  e += (int)((u >> 23) & 0xffu) - 127;
  float m = __uint_as_float((u & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421354f) { m = m * 0.5f; e += 1; }
  float s = __fdiv_rn(m - 1.0f, m + 1.0f);
  float s2 = s * s;
  float poly = __fmaf_rn(s2, 0.0909090936f, 0.111111112f);
  poly = __fmaf_rn(s2, poly, 0.142857149f);
  poly = __fmaf_rn(s2, poly, 0.200000003f);
  poly = __fmaf_rn(s2, poly, 0.333333343f);
  poly = __fmaf_rn(s2, poly, 1.0f);
  float atanh_s = s * poly;
  return __fmaf_rn(atanh_s, 2.88539004f, small_int_f(e + 151) - 151.0f); /* e >= -151 */
}
__device__ __forceinline__ float ctrl_exp2(float y) {
  if (y > 128.0f) return __int_as_float(0x7f800000);
  if (y < -150.0f) return 0.0f;
  float n = rintf(y);
  float f = y - n;
  float z = f * 0.693147182f;
  float p = __fmaf_rn(z, 2.48015876e-05f, 1.98412701e-04f);
  p = __fmaf_rn(z, p, 1.38888892e-03f);
  p = __fmaf_rn(z, p, 8.33333377e-03f);
  p = __fmaf_rn(z, p, 4.16666679e-02f);
  p = __fmaf_rn(z, p, 0.166666672f);
  p = __fmaf_rn(z, p, 0.5f);
  p = __fmaf_rn(z, p, 1.0f);
  p = __fmaf_rn(z, p, 1.0f);
  int ni = (int)n;
  int h = ni / 2;
  float s1 = __uint_as_float((unsigned)(h + 127) << 23);
  float s2 = __uint_as_float((unsigned)(ni - h + 127) << 23);
  return (p * s1) * s2;
}
__device__ __forceinline__ float ctrl_pow(float x, float b) {
  if (x != x) return x;
  if (x == 0.0f) return 0.0f;
  if (x == __int_as_float(0x7f800000)) return x;
  return ctrl_exp2(b * ctrl_log2(x));
}

/* Natural logarithm of a positive normal double, table-driven (P. T. P.
 * Tang, ACM TOMS 16(4), 1990): x = 2^e m with m in [1, 2); the top 7 bits of
 * m's fraction pick row j of log_table.h (gen_logtab.py), and
 *   log x = e' ln 2 + T_j + log1p(r),  r = fma(m, 1/F_j, -1),  |r| < 2^-7,
 * e' = e + 1 for j >= 53, whose T_j carries the -ln 2 (no cancellation of two
 * terms of size ln 2 just below 1); log1p(r) = r + r^2 q(r) with q the Taylor
 * coefficients -1/2, 1/3, ..., -1/8 (truncation below 2^-66), and e' ln 2 in
 * two parts (LN2_HI of 42 significant bits, so e' LN2_HI is exact).  Every
 * step is one IEEE double operation; no division. */
__device__ __forceinline__ double log_dev(double x) {
  const long long b = __double_as_longlong(x);
  const int j = (int)((b >> 45) & 127);
  const int e = (int)((b >> 52) & 0x7ff) - 1023 + (j >= GBODE_LOGTAB_SHIFT_FROM ? 1 : 0);
  const double m = __longlong_as_double((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  const double inv = __ldg(&kLogTab[j][0]), thi = __ldg(&kLogTab[j][1]), tlo = __ldg(&kLogTab[j][2]);
  const double r = __fma_rn(m, inv, -1.0);
  double q = -0.125;
  q = __fma_rn(q, r, 0x1.2492492492492p-3);   /* 1/7 */
  q = __fma_rn(q, r, -0x1.5555555555555p-3);  /* -1/6 */
  q = __fma_rn(q, r, 0x1.999999999999ap-3);   /* 1/5 */
  q = __fma_rn(q, r, -0.25);
  q = __fma_rn(q, r, 0x1.5555555555555p-2);   /* 1/3 */
  q = __fma_rn(q, r, -0.5);
  const double l1p = __fma_rn(r * r, q, r);
  const double de = (double)e;
  return __fma_rn(de, 0x1.62e42fefa38p-1, thi) + (__fma_rn(de, 0x1.ef35793c7673p-45, tlo) + l1p);
}

/* Exponential of a double x with |x| < 700, table-driven (P. T. P. Tang,
 * ACM TOMS 15(2), 1989): n = round(x 32/ln 2) (added to 1.5 * 2^52, so that
 * the sum's low bits hold n), r = x - n ln2/32 with ln2/32 in two parts
 * (exp_table.h: a lead of 42 significant bits makes n * lead exact),
 * |r| <= ln2/64 + tiny; exp(r) - 1 = r + r^2 q(r), q the Taylor coefficients
 * 1/2 .. 1/720 (degree 6, truncation below 2^-59); with j = n mod 32,
 * m = (n - j)/32 and 2^(j/32) = lead_j + trail_j from the table,
 *   exp(x) = 2^m (lead_j + (lead_j p + trail_j (1 + p))).
 * Every step is one IEEE double operation; within 1 ulp (checked against
 * 60-digit values by the CPU tests). */
__device__ __forceinline__ double exp_dev(double x) {
  const double t = __fma_rn(x, GBODE_EXP_INV_L, 0x1.8p52);
  const int n = (int)(__double_as_longlong(t) - 0x4338000000000000LL);
  const double nd = t - 0x1.8p52;
  const double r = __fma_rn(-nd, GBODE_EXP_L_TRAIL, __fma_rn(-nd, GBODE_EXP_L_LEAD, x));
  double q = __fma_rn(r, 0x1.6c16c16c16c17p-10, 0x1.1111111111111p-7); /* 1/720, 1/120 */
  q = __fma_rn(q, r, 0x1.5555555555555p-5);                           /* 1/24 */
  q = __fma_rn(q, r, 0x1.5555555555555p-3);                           /* 1/6 */
  q = __fma_rn(q, r, 0.5);
  const double p = __fma_rn(r * r, q, r);
  const int j = n & 31, m = n >> 5;
  const double lead = __ldg(&kExpTab[j][0]), trail = __ldg(&kExpTab[j][1]);
  const double v = lead + __fma_rn(lead, p, __fma_rn(trail, p, trail));
  return v * __longlong_as_double((long long)(m + 1023) << 52);
}

/* Logarithms of the controller constants (src/SimpleDiffEq.jl:67-77) for the
 * FP64 controller, rounded to double: ln(1/qmax) = ln 0.1, ln(1/qmin) = ln 5,
 * ln gamma = ln 0.9, ln qoldinit = ln 1e-4. */
#define CTRL64_LN_QMAXI (-0x1.26bb1bbb55516p+1)
#define CTRL64_LN_QMINI 0x1.9c041f7ed8d33p+0
#define CTRL64_LN_GAMMA (-0x1.af8e8210a415dp-4)
#define CTRL64_LN_QOLDINIT (-0x1.26bb1bbb55516p+3)

/* Error norm and step-size controller of the single-precision modes, free of
 * IEEE division, square root and branches (a lone lane's long trajectory
 * waits on their slow-path checks).  rcp_nr: 1/d for a positive normal float
 * from the bit-level seed 0x7ef311c7 (relative error below 1.3e-1) and three
 * Newton steps y (2 - d y) (1.6e-2, 2.7e-4, then rounding).  log2_nr: the
 * atanh series of ctrl_log2 with the quotient (m-1)/(m+1) taken by rcp_nr and
 * the sqrt(2) fold by selects; finite for every non-NaN input (0 and
 * subnormals come out near -127, which the controller's clamps absorb).
 * exp2_nr: y = n + f by the 1.5 * 2^23 shifter, 2^f from the Taylor series of
 * exp(f ln 2) to degree 7, scaled by 2^n through the exponent bits; for
 * |y| < 126.  Every step an IEEE single operation or an explicit fma, so
 * the oracle reproduces them bit for bit. */
__device__ __forceinline__ float rcp_nr(float d) {
  float y = __int_as_float(0x7ef311c7 - __float_as_int(d));
  y = y * __fmaf_rn(-d, y, 2.0f);
  y = y * __fmaf_rn(-d, y, 2.0f);
  y = y * __fmaf_rn(-d, y, 2.0f);
  return y;
}
__device__ __forceinline__ float log2_nr(float x) {
  const int b = __float_as_int(x);
  const int e0 = ((b >> 23) & 0xff) - 127;
  const float m0 = __int_as_float((b & 0x007fffff) | 0x3f800000);
  const bool fold = m0 > 1.41421354f;
  const float m = fold ? 0.5f * m0 : m0;
  const int e = fold ? e0 + 1 : e0;
  const float s = (m - 1.0f) * rcp_nr(m + 1.0f);
  const float s2 = s * s;
  float poly = __fmaf_rn(s2, 0.0909090936f, 0.111111112f);
  poly = __fmaf_rn(s2, poly, 0.142857149f);
  poly = __fmaf_rn(s2, poly, 0.200000003f);
  poly = __fmaf_rn(s2, poly, 0.333333343f);
  poly = __fmaf_rn(s2, poly, 1.0f);
  return __fmaf_rn(s * poly, 2.88539004f, small_int_f(e + 127) - 127.0f);
}
__device__ __forceinline__ float exp2_nr(float y) {
  const float t = y + 12582912.0f;
  const int n = __float_as_int(t) - 0x4b400000;
  const float f = y - (t - 12582912.0f);
  const float z = f * 0.693147182f;
  float p = __fmaf_rn(z, 1.98412701e-04f, 1.38888892e-03f); /* 1/7!, 1/6! */
  p = __fmaf_rn(z, p, 8.33333377e-03f);
  p = __fmaf_rn(z, p, 4.16666679e-02f);
  p = __fmaf_rn(z, p, 0.166666672f);
  p = __fmaf_rn(z, p, 0.5f);
  p = __fmaf_rn(z, p, 1.0f);
  p = __fmaf_rn(z, p, 1.0f);
  return p * __int_as_float((n + 127) << 23);
}
/* log2 of the controller constants: 1/qmin = 5, 1/qmax = 0.1, gamma = 0.9, qoldinit = 1e-4 */
#define CTRL32_L2_QMINI 2.32192809f
#define CTRL32_L2_QMAXI (-3.32192809f)
#define CTRL32_L2_GAMMA (-0.152003093f)
#define CTRL32_L2_QOLDINIT (-13.2877124f)

/* Double-single arithmetic for the error norm and step-size controller of
 * the FP64 solves (ODE_CTRL_DS).  A value is an unevaluated sum h + l of two
 * IEEE singles (|l| <= ulp(h)/2: about 48 significant bits), computed with
 * the error-free transformations of Knuth (two_sum), Dekker (fast two_sum)
 * and the fma product error, so that the norm and the controller's
 * logarithm and exponential run on the single-precision pipe, which on this
 * GPU issues 62 lane operations for each double one.  Every step is one IEEE
 * single operation, an fma, an integer operation or an exact conversion, so
 * the oracle reproduces each result bit for bit.  Tables and constants:
 * ds_table.h (gen_dstab.py). */
#define GBODE_DSTAB_SPACE __device__ const
#include "ds_table.h"

struct dsf { float h, l; };

__device__ __forceinline__ dsf ds_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
/* |a| >= |b| (or a == 0) */
__device__ __forceinline__ dsf ds_fast(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dsf ds_add(dsf x, dsf y) {
  const dsf s = ds_two_sum(x.h, y.h);
  return ds_fast(s.h, s.l + (x.l + y.l));
}
__device__ __forceinline__ dsf ds_neg(dsf x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dsf ds_mul(dsf x, dsf y) {
  const float p = x.h * y.h;
  const float e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, __fmaf_rn(x.h, y.h, -p)));
  return ds_fast(p, e);
}
__device__ __forceinline__ dsf ds_sqr(dsf x) {
  const float p = x.h * x.h;
  return ds_fast(p, __fmaf_rn(x.h + x.h, x.l, __fmaf_rn(x.h, x.h, -p)));
}
/* x / y for y > 0: q1 = x.h / y.h by rcp_nr, then one correction from the
 * remainder x - q1 y (x.h - q1 y.h is exact by Sterbenz); y == 0 gives the
 * IEEE quotient of x.h (an infinity, or NaN for 0/0) */
__device__ __forceinline__ dsf ds_div(dsf x, dsf y) {
  if (y.h == 0.0f) return {x.h * __int_as_float(0x7f800000), 0.0f};
  const float ry = rcp_nr(y.h);
  const float q1 = x.h * ry;
  const float p = q1 * y.h, pe = __fmaf_rn(q1, y.h, -p);
  const float rem = (((x.h - p) - pe) + x.l) - q1 * y.l;
  return ds_fast(q1, rem * ry);
}
/* x > y in the order of the represented values; false when either is NaN */
__device__ __forceinline__ bool ds_gt(dsf x, dsf y) { return x.h > y.h || (x.h == y.h && x.l > y.l); }
/* the clamps of the controller, with fm_min / fm_max's NaN behaviour */
__device__ __forceinline__ dsf ds_min(dsf x, dsf y) { return ds_gt(y, x) ? x : y; }
__device__ __forceinline__ dsf ds_max(dsf x, dsf y) { return ds_gt(y, x) ? y : x; }

/* A double as h + l with integer operations only (a conversion between
 * double and single issues on this GPU's FP64 pipe, as a double operation
 * does): h is x's sign, exponent and top 23 fraction bits repacked as a
 * single (x truncated to 24 significant bits) for 2^-126 <= |x| < 2^128,
 * +-0 below that range, +-infinity above it and NaN for NaN; l is x's 29 low
 * fraction bits as an integer rounded to a single (one fma of its exact top 6
 * and low 23 bits) and scaled by 2^(e - 52) through the exponent field
 * (|l| < 2^-23 |h|; 0 when |x| < 2^-74, where the norm needs no more than h,
 * or x is not finite). */
__device__ __forceinline__ dsf ds_split(double x) {
  const long long b = __double_as_longlong(x);
  const int eb = (int)((b >> 52) & 0x7ff);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned frac = (unsigned)((b >> 29) & 0x7fffff);
  const unsigned hb = eb >= 897 && eb <= 1150 ? sign | ((unsigned)(eb - 896) << 23) | frac
                      : eb < 897 ? sign
                      : (eb == 2047 && (b & 0xfffffffffffffLL)) ? 0x7fc00000u | sign
                                                                : 0x7f800000u | sign;
  const float h = __uint_as_float(hb);
  float l = 0.0f;
  if (eb >= 949 && eb <= 1150) {
    const int low = (int)(b & 0x1fffffff);
    const float lf = __fmaf_rn(small_int_f(low >> 23), 8388608.0f, small_int_f(low & 0x7fffff));
    const float mag = lf * __int_as_float((eb - 948) << 23);
    l = b < 0 ? -mag : mag;
  }
  return {h, l};
}
/* max(|u|, |v|) of two doubles by an integer comparison of their magnitudes'
 * bit patterns (the order of non-negative doubles; a NaN compares above
 * infinity, so it propagates as Julia's max does) */
__device__ __forceinline__ double ds_absmax(double u, double v) {
  const long long au = __double_as_longlong(u) & 0x7fffffffffffffffLL;
  const long long av = __double_as_longlong(v) & 0x7fffffffffffffffLL;
  return __longlong_as_double(au >= av ? au : av);
}

/* ln(a) for a = h + l with h a positive normal single, 2^-120 <= h <= 2^126:
 * h = 2^E m, r = fma(m, c_j, -1) exact, ln(1 + r) = r - r^2/2 + r^3 (1/3 -
 * r/4 + r^2/5 - r^3/6 + r^4/7) with r^2 an exact product pair (truncation
 * below 2^-59), E ln2 from the three-part ln2 (E A exact, E B an exact
 * product pair), and ln(h + l) = ln(h) + l/h.  Absolute error about 2^-46
 * for |ln a| < 1, 2^-41 at the ends of the range. */
__device__ __forceinline__ dsf ds_log(dsf a) {
  const int b = __float_as_int(a.h);
  const int j = (b >> 16) & 127;
  const float m = __int_as_float((b & 0x007fffff) | 0x3f800000);
  const float c = __ldg(&kDsLogTab[j][0]), th = __ldg(&kDsLogTab[j][1]), tl = __ldg(&kDsLogTab[j][2]);
  const float r = __fmaf_rn(m, c, -1.0f);
  const float p = r * r, pe = __fmaf_rn(r, r, -p);
  float t = __fmaf_rn(r, 0x1.24924ap-3f, -0x1.555556p-3f); /* 1/7, -1/6 */
  t = __fmaf_rn(r, t, 0x1.99999ap-3f);                     /* 1/5 */
  t = __fmaf_rn(r, t, -0.25f);
  t = __fmaf_rn(r, t, 0x1.555556p-2f);                     /* 1/3 */
  const float tail = t * (r * p);
  const dsf l1 = ds_fast(r, -0.5f * p);
  const dsf lp = {l1.h, l1.l + (tail - 0.5f * pe)};
  const float fE = small_int_f((b >> 23) & 0xff) - 127.0f; /* the exponent E, exact */
  const float eb = fE * GBODE_DS_LN2_B, ebe = __fmaf_rn(fE, GBODE_DS_LN2_B, -eb);
  const dsf e0 = ds_fast(fE * GBODE_DS_LN2_A, eb);
  const dsf eln2 = ds_fast(e0.h, e0.l + (ebe + fE * GBODE_DS_LN2_C));
  const dsf s = ds_add(ds_add(eln2, {th, tl}), lp);
  return ds_fast(s.h, s.l + a.l * rcp_nr(a.h));
}

/* exp(x) for |x| < 2.7 (|k| < 256 keeps k A exact; the controller's
 * arguments lie in [ln 0.2, ln 10]): k = rint(x 64/ln2), r = x - k ln2/64 (x.h - k A exact by
 * Sterbenz, k B an exact product pair), exp(r) - 1 = r + r^2/2 + r^3 (1/6 +
 * r/24 + r^2/120) (|r| <= ln2/128 + tiny, truncation below 2^-54), and
 * exp(x) = 2^(k >> 6) 2^((k & 63)/64) (1 + (exp(r) - 1)).  Relative error
 * about 2^-46; NaN in, NaN out. */
__device__ __forceinline__ dsf ds_exp(dsf x) {
  if (x.h != x.h) return x;
  /* k = rint(x.h 64/ln2) by the 1.5 * 2^23 shifter: the sum's low bits hold k */
  const float sh = x.h * GBODE_DS_EXP_INV_L + 12582912.0f;
  const int k = __float_as_int(sh) - 0x4b400000;
  const float kf = sh - 12582912.0f;
  const float r0 = __fmaf_rn(-kf, GBODE_DS_EXP_L_A, x.h);
  const float pb = kf * GBODE_DS_EXP_L_B, pbe = __fmaf_rn(kf, GBODE_DS_EXP_L_B, -pb);
  const dsf rr = ds_two_sum(r0, -pb);
  const dsf r = ds_fast(rr.h, rr.l + ((x.l - pbe) - kf * GBODE_DS_EXP_L_C));
  const float p = r.h * r.h, pe = __fmaf_rn(r.h, r.h, -p);
  float t = __fmaf_rn(r.h, 0x1.111112p-7f, 0x1.555556p-5f); /* 1/120, 1/24 */
  t = __fmaf_rn(r.h, t, 0x1.555556p-3f);                      /* 1/6 */
  const float tail = t * (r.h * p);
  const dsf e1 = ds_fast(r.h, 0.5f * p);
  const dsf em1 = ds_fast(e1.h, e1.l + ((r.l + 0.5f * pe) + (r.h * r.l + tail)));
  const int j = k & 63;
  const float th = __ldg(&kDsExpTab[j][0]), tl = __ldg(&kDsExpTab[j][1]);
  const float pp = th * em1.h, ppe = __fmaf_rn(th, em1.h, -pp);
  const dsf v0 = ds_fast(th, pp);
  const dsf v = ds_fast(v0.h, v0.l + (tl + (ppe + __fmaf_rn(th, em1.l, tl * em1.h))));
  const float sc = __int_as_float(((k >> 6) + 127) << 23);
  return {v.h * sc, v.l * sc};
}
/* a single as a double with integer operations: exact for normal singles,
 * +-0 for zeros and subnormals, infinities and NaN kept */
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xff;
  const unsigned long long s = (unsigned long long)(u & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)s);
  const unsigned long long de = e == 255 ? 0x7ffULL : (unsigned long long)(e + 896);
  return __longlong_as_double((long long)(s | (de << 52) | ((unsigned long long)(u & 0x7fffff) << 29)));
}
/* d * (x.h + x.l) as fma(d, x.l, d * x.h): two double operations */
__device__ __forceinline__ double ds_scale(double d, dsf x) { return __fma_rn(d, f2d_bits(x.l), d * f2d_bits(x.h)); }
/* h + l as a double: both parts moved into doubles by their bits, one double addition */
__device__ __forceinline__ double ds_to_double(dsf x) { return f2d_bits(x.h) + f2d_bits(x.l); }

/* With the double-single norm the FP64 kernels hand the error estimate over
 * unscaled: sum(btilde_i k_i), which the norm multiplies by dt in
 * double-single (one double multiplication per component less an attempt). */
#ifdef GBODE_CTRL_DS
template <class R> struct ErrUnscaled { enum { value = sizeof(R) == sizeof(double) }; };
#else
template <class R> struct ErrUnscaled { enum { value = 0 }; };
#endif

/* ------------------------------------------------------------------ precisions */
struct PFP64 { typedef double R; typedef double T; enum { KAHAN = 0 }; };
struct PFP32 { typedef float R; typedef float T; enum { KAHAN = 0 }; };
struct PFP32K { typedef float R; typedef double T; enum { KAHAN = 1 }; };

/* ------------------------------------------------------------------ tableaus in constant memory */
__constant__ double c_tsit5_d[tsit5_COUNT] = GBTAB_TSIT5_INIT;
__constant__ float c_tsit5_f[tsit5_COUNT] = GBTAB_TSIT5_INIT;
__constant__ double c_vern7_d[vern7_COUNT] = GBTAB_VERN7_INIT;
__constant__ float c_vern7_f[vern7_COUNT] = GBTAB_VERN7_INIT;
__constant__ double c_vern7x_d[vern7x_COUNT] = GBTAB_VERN7X_INIT;
__constant__ float c_vern7x_f[vern7x_COUNT] = GBTAB_VERN7X_INIT;
__constant__ double c_vern7r_d[vern7r_COUNT] = GBTAB_VERN7R_INIT;
__constant__ float c_vern7r_f[vern7r_COUNT] = GBTAB_VERN7R_INIT;
__constant__ double c_vern9_d[vern9_COUNT] = GBTAB_VERN9_INIT;
__constant__ float c_vern9_f[vern9_COUNT] = GBTAB_VERN9_INIT;
__constant__ double c_vern9x_d[vern9x_COUNT] = GBTAB_VERN9X_INIT;
__constant__ float c_vern9x_f[vern9x_COUNT] = GBTAB_VERN9X_INIT;
__constant__ double c_vern9r_d[vern9r_COUNT] = GBTAB_VERN9R_INIT;
__constant__ float c_vern9r_f[vern9r_COUNT] = GBTAB_VERN9R_INIT;

template <class X> struct CB;
template <> struct CB<double> {
  __device__ static __forceinline__ double t5(int i) { return c_tsit5_d[i]; }
  __device__ static __forceinline__ double v7(int i) { return c_vern7_d[i]; }
  __device__ static __forceinline__ double v7x(int i) { return c_vern7x_d[i]; }
  __device__ static __forceinline__ double v7r(int i) { return c_vern7r_d[i]; }
  __device__ static __forceinline__ double v9(int i) { return c_vern9_d[i]; }
  __device__ static __forceinline__ double v9x(int i) { return c_vern9x_d[i]; }
  __device__ static __forceinline__ double v9r(int i) { return c_vern9r_d[i]; }
};
template <> struct CB<float> {
  __device__ static __forceinline__ float t5(int i) { return c_tsit5_f[i]; }
  __device__ static __forceinline__ float v7(int i) { return c_vern7_f[i]; }
  __device__ static __forceinline__ float v7x(int i) { return c_vern7x_f[i]; }
  __device__ static __forceinline__ float v7r(int i) { return c_vern7r_f[i]; }
  __device__ static __forceinline__ float v9(int i) { return c_vern9_f[i]; }
  __device__ static __forceinline__ float v9x(int i) { return c_vern9x_f[i]; }
  __device__ static __forceinline__ float v9r(int i) { return c_vern9r_f[i]; }
};

/* ------------------------------------------------------------------ vector algebra (D compile-time) */
/* s = c1 k1 + c2 k2 + ... + cn kn, accumulated left to right:
 * s = c1 k1, then s = fma(ci, ki, s) for i = 2..n (the order @muladd nests
 * a sum of products in) */
template <int D, class R>
__device__ __forceinline__ void lc_acc(R (&s)[D]) {}
template <int D, class R, class K, class... Rest>
__device__ __forceinline__ void lc_acc(R (&s)[D], R c, const K& k, const Rest&... rest) {
#pragma unroll
  for (int d = 0; d < D; ++d) s[d] = vmaddR(c, k[d], s[d]);
  lc_acc(s, rest...);
}
/* k: any row indexable by d (a register array, or a RingRow of staged stage values) */
template <int D, class R, class K, class... Rest>
__device__ __forceinline__ void lc(R (&s)[D], R c, const K& k, const Rest&... rest) {
#pragma unroll
  for (int d = 0; d < D; ++d) s[d] = c * k[d];
  lc_acc(s, rest...);
}
/* out = base + h * s */
template <int D, class R>
__device__ __forceinline__ void axpy(R (&out)[D], const R (&base)[D], R h, const R (&s)[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) out[d] = vmaddR(h, s[d], base[d]);
}
/* stage time t + c*dt */
template <class T>
__device__ __forceinline__ T stime(T t, T c, T dt) { return fmaR(c, dt, t); }

/* new state = old + h*s; in Kahan mode a compensated sum with value hi - c */
template <class PR, int D>
__device__ __forceinline__ void state_update(const typename PR::R (&uh)[D], const typename PR::R (&uc)[D],
                                             typename PR::R h, const typename PR::R (&s)[D],
                                             typename PR::R (&nh)[D], typename PR::R (&nc)[D]) {
  typedef typename PR::R R;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    if (PR::KAHAN) {
      R delta = h * s[d];
      R y = delta - uc[d];
      R sum = uh[d] + y;
      nc[d] = (sum - uh[d]) - y;
      nh[d] = sum;
    } else {
      nh[d] = vmaddR(h, s[d], uh[d]);
      nc[d] = (R)0;
    }
  }
}

/* dense-output value uprev + h*s, written as double */
template <class PR, int D>
__device__ __forceinline__ void finish_dense(const typename PR::R (&uh)[D], const typename PR::R (&uc)[D],
                                             typename PR::R h, const typename PR::R (&s)[D], double (&out)[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    if (PR::KAHAN) out[d] = ((double)uh[d] - (double)uc[d]) + (double)(h * s[d]);
    else out[d] = (double)vmaddR(h, s[d], uh[d]);
  }
}

/* ------------------------------------------------------------------ right-hand sides */
/* Each functor holds its parameters in registers and evaluates du = f(u, p, t).
 * The forms match the oracle's DEVICE forms term for term, and with GBODE_REF
 * its REF forms (the plain Julia expressions). */
template <class R, class T>
struct RhsLorenz {
  enum { D = 3, NP = 3 };
  R p[3];
  __device__ __forceinline__ void operator()(const R (&u)[3], T t, R (&du)[3]) const {
    du[0] = p[0] * (u[1] - u[0]);
#ifdef GBODE_REF
    du[1] = u[0] * (p[1] - u[2]) - u[1];
    du[2] = u[0] * u[1] - p[2] * u[2];
#else
    du[1] = fmaR(u[0], p[1] - u[2], -u[1]);
    du[2] = fmaR(u[0], u[1], -(p[2] * u[2]));
#endif
  }
};

template <class R, class T>
struct RhsVanDerPol {
  enum { D = 2, NP = 1 };
  R p[1];
  __device__ __forceinline__ void operator()(const R (&u)[2], T t, R (&du)[2]) const {
    du[0] = u[1];
#ifdef GBODE_REF
    du[1] = p[0] * ((R)1 - u[0] * u[0]) * u[1] - u[0];
#else
    R w = fmaR(-u[0], u[0], (R)1);
    du[1] = fmaR(p[0] * w, u[1], -u[0]);
#endif
  }
};

/* 1/sqrt(x) for a positive normal float: the bit-level seed of C. Lomont,
 * "Fast inverse square root" (2003; magic constant 0x5f375a86, relative error
 * below 3.5e-2) refined by three Newton steps y <- y (3/2 - (x/2) y^2), each
 * an explicit fma and IEEE single products (errors 1.8e-3, 4.6e-6, then
 * rounding), so the oracle reproduces it bit for bit.  No division and no
 * square root: the IEEE single division and square root take a slow-path
 * branch that dominates a lone lane's step time (the single-precision R3BP
 * step of the longest trajectory ran 1.9x faster with this). */
__device__ __forceinline__ float rsqrt_nr(float x) {
  float y = __int_as_float(0x5f375a86 - (__float_as_int(x) >> 1));
  const float hx = 0.5f * x;
  y = y * __fmaf_rn(-(hx * y), y, 1.5f);
  y = y * __fmaf_rn(-(hx * y), y, 1.5f);
  y = y * __fmaf_rn(-(hx * y), y, 1.5f);
  return y;
}

/* mu / r^(3/2): in double the reference's r * sqrt(r) and division; in single
 * precision mu * y^3 with y = rsqrt_nr(r), within 6 ulp */
__device__ __forceinline__ double r3bp_pull(double mu, double r) { return mu / (r * sqrtR(r)); }
__device__ __forceinline__ float r3bp_pull(float mu, float r) {
  const float y = rsqrt_nr(r);
  return mu * ((y * y) * y);
}

template <class R, class T>
struct RhsR3BP {
  enum { D = 4, NP = 1 };
  R p[1];
  __device__ __forceinline__ void operator()(const R (&u)[4], T t, R (&du)[4]) const {
    const R mu = p[0], mu1 = (R)1 - mu;
    const R x = u[0], y = u[1], vx = u[2], vy = u[3];
    const R a = x + mu, b = x - mu1;
    du[0] = vx;
    du[1] = vy;
#ifdef GBODE_REF
    const R r1 = a * a + y * y, r2 = b * b + y * y;
    const R d1 = r1 * sqrtR(r1), d2 = r2 * sqrtR(r2);
    du[2] = x + (R)2 * vy - mu1 * a / d1 - mu * b / d2;
    du[3] = y - (R)2 * vx - mu1 * y / d1 - mu * y / d2;
#else
    const R r1 = fmaR(a, a, y * y), r2 = fmaR(b, b, y * y);
    const R g1 = r3bp_pull(mu1, r1), g2 = r3bp_pull(mu, r2);
    du[2] = fmaR(-g2, b, fmaR(-g1, a, fmaR((R)2, vy, x)));
    du[3] = fmaR(-g2, y, fmaR(-g1, y, fmaR((R)-2, vx, y)));
#endif
  }
};

/* The phases' sine/cosine loop is kept rolled: unrolled, the seven right-hand
 * side evaluations of a Tsit5 step put 7 x 12 sine/cosine bodies in the step
 * loop, more code than the instruction cache holds once the warps of an SM
 * are at different points of their steps (measured on the persistent
 * kernel: about ten warps waiting for instruction fetch per instruction
 * issued, and 1.56x the time of a rolled loop).  Indexed by the loop
 * counter, the phases and the sines and cosines live in local memory (L1),
 * whose traffic costs far less than the FP64 work it sits between. */
template <class R, class T, int DD>
struct RhsKuramoto {
  enum { D = DD, NP = DD + 1 };
  R p[DD + 1];  /* omega_1..omega_D, then K / D (rhs_loaded divides the loaded K once) */
  __device__ __forceinline__ void operator()(const R (&u)[DD], T t, R (&du)[DD]) const {
    R sn[DD], cs[DD], S = 0, C = 0;
#pragma unroll 1
    for (int j = 0; j < DD; ++j) {
      sincosR(u[j], &sn[j], &cs[j]);
      S = S + sn[j];
      C = C + cs[j];
    }
    const R kd = p[DD];
#pragma unroll
    for (int i = 0; i < DD; ++i) {
#ifdef GBODE_REF
      du[i] = p[i] + kd * (cs[i] * S - sn[i] * C);
#else
      du[i] = fmaR(kd, fmaR(cs[i], S, -(sn[i] * C)), p[i]);
#endif
    }
  }
};

/* Called once after a trajectory's parameters are loaded from the caller's
 * array: the Kuramoto coupling K / D is divided there, not in every
 * right-hand-side evaluation (a double division is about nine FP64
 * instructions); the same IEEE operation on the same operands. */
template <class F> __device__ __forceinline__ void rhs_loaded(F&) {}
template <class R, class T, int DD> __device__ __forceinline__ void rhs_loaded(RhsKuramoto<R, T, DD>& f) {
  f.p[DD] = f.p[DD] / (R)DD;
}

template <class R, class T, int DD>
struct RhsLinear {
  enum { D = DD, NP = DD * DD };
  R p[DD * DD];
  __device__ __forceinline__ void operator()(const R (&u)[DD], T t, R (&du)[DD]) const {
#pragma unroll
    for (int i = 0; i < DD; ++i) {
      R s = p[i * DD] * u[0];
#pragma unroll
      for (int j = 1; j < DD; ++j) s = vmaddR(p[i * DD + j], u[j], s);
      du[i] = s;
    }
  }
};

/* ------------------------------------------------------------------ Tsitouras 5(4) */
/* src/tsit5/gpuatsit5.jl:258-275 (stages, FSAL k7), :306-314 and
 * src/tsit5/tsit5.jl:385-399 (dense output). */
template <class PR, int D, class F>
struct MTsit5 {
  typedef typename PR::R R;
  typedef typename PR::T T;
  enum { NK = 7, FSAL = 1, DTMIN_1F7 = 0, DENSE_F = 0 };  /* DENSE_F: dense output evaluates f */

  __device__ static __forceinline__ void attempt(const F& f, const R (&uh)[D], const R (&uc)[D], T t, T dt,
                                                 R (&k)[NK][D], R (&nh)[D], R (&nc)[D], R (&e)[D], bool want_err) {
#define C5(x) CB<R>::t5(tsit5_##x)
#define C5T(x) CB<T>::t5(tsit5_##x)
    R tmp[D], s[D];
    const R h = (R)dt;
#ifdef GBODE_REF
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = h * (C5(a21) * k[0][d]) + uh[d];
#else
    const R a = (R)(dt * C5T(a21));
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = fmaR(a, k[0][d], uh[d]);
#endif
    f(tmp, stime(t, C5T(c1), dt), k[1]);
    lc(s, C5(a31), k[0], C5(a32), k[1]);
    axpy(tmp, uh, h, s);
    f(tmp, stime(t, C5T(c2), dt), k[2]);
    lc(s, C5(a41), k[0], C5(a42), k[1], C5(a43), k[2]);
    axpy(tmp, uh, h, s);
    f(tmp, stime(t, C5T(c3), dt), k[3]);
    lc(s, C5(a51), k[0], C5(a52), k[1], C5(a53), k[2], C5(a54), k[3]);
    axpy(tmp, uh, h, s);
    f(tmp, stime(t, C5T(c4), dt), k[4]);
    lc(s, C5(a61), k[0], C5(a62), k[1], C5(a63), k[2], C5(a64), k[3], C5(a65), k[4]);
    axpy(tmp, uh, h, s);
    f(tmp, t + dt, k[5]);
    lc(s, C5(a71), k[0], C5(a72), k[1], C5(a73), k[2], C5(a74), k[3], C5(a75), k[4], C5(a76), k[5]);
    state_update<PR, D>(uh, uc, h, s, nh, nc);
    f(nh, t + dt, k[6]);
    if (want_err) {
      lc(s, C5(btilde1), k[0], C5(btilde2), k[1], C5(btilde3), k[2], C5(btilde4), k[3], C5(btilde5), k[4],
         C5(btilde6), k[5], C5(btilde7), k[6]);
#pragma unroll
      for (int d = 0; d < D; ++d) e[d] = ErrUnscaled<R>::value ? s[d] : h * s[d];
    }
  }

  template <class KK>
  __device__ static __forceinline__ void dense(const F& f, const R (&uh)[D], const R (&uc)[D], T told, T tnew,
                                               T dtold, T theta, const KK& k, double (&out)[D]) {
    const R th = (R)theta;
    const R th2 = th * th;
    R ex, b1, b2, b3, b4, b5, b6, b7;
    ex = C5(r14); ex = fmaR(th, ex, C5(r13)); ex = fmaR(th, ex, C5(r12)); ex = fmaR(th, ex, C5(r11)); b1 = th * ex;
#define TSIT5_B(i, out_)                                                        \
  ex = C5(r##i##4); ex = fmaR(th, ex, C5(r##i##3)); ex = fmaR(th, ex, C5(r##i##2)); \
  out_ = th2_times(th, th2, ex);
    TSIT5_B(2, b2) TSIT5_B(3, b3) TSIT5_B(4, b4) TSIT5_B(5, b5) TSIT5_B(6, b6) TSIT5_B(7, b7)
#undef TSIT5_B
    R s[D];
    lc(s, b1, k[0], b2, k[1], b3, k[2], b4, k[3], b5, k[4], b6, k[5], b7, k[6]);
    finish_dense<PR, D>(uh, uc, (R)dtold, s, out);
#undef C5
#undef C5T
  }
};

/* ------------------------------------------------------------------ Verner 7(6) */
/* src/verner/gpuvern7.jl:360-404 (adaptive attempt), :107-136 (fixed step),
 * :441-513 dense output with six extra stages at t + c*dtold (t already
 * advanced), bθs at src/verner/verner_tableaus.jl:1337-1360. */
template <class PR, int D, class F>
struct MVern7 {
  typedef typename PR::R R;
  typedef typename PR::T T;
  enum { NK = 10, FSAL = 0, DTMIN_1F7 = 0, DENSE_F = 1 };

  __device__ static __forceinline__ void attempt(const F& f, const R (&uh)[D], const R (&uc)[D], T t, T dt,
                                                 R (&k)[NK][D], R (&nh)[D], R (&nc)[D], R (&e)[D], bool want_err) {
#define C7(x) CB<R>::v7(vern7_##x)
#define C7T(x) CB<T>::v7(vern7_##x)
    R tmp[D], s[D];
    const R h = (R)dt;
    f(uh, t, k[0]);
    const R a = (R)(dt * C7T(a021));
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = vmaddR(a, k[0][d], uh[d]);
    f(tmp, stime(t, C7T(c2), dt), k[1]);
    lc(s, C7(a031), k[0], C7(a032), k[1]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C7T(c3), dt), k[2]);
    lc(s, C7(a041), k[0], C7(a043), k[2]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C7T(c4), dt), k[3]);
    lc(s, C7(a051), k[0], C7(a053), k[2], C7(a054), k[3]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C7T(c5), dt), k[4]);
    lc(s, C7(a061), k[0], C7(a063), k[2], C7(a064), k[3], C7(a065), k[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C7T(c6), dt), k[5]);
    lc(s, C7(a071), k[0], C7(a073), k[2], C7(a074), k[3], C7(a075), k[4], C7(a076), k[5]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C7T(c7), dt), k[6]);
    lc(s, C7(a081), k[0], C7(a083), k[2], C7(a084), k[3], C7(a085), k[4], C7(a086), k[5], C7(a087), k[6]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C7T(c8), dt), k[7]);
    R g10[D];
    lc(s, C7(a091), k[0], C7(a093), k[2], C7(a094), k[3], C7(a095), k[4], C7(a096), k[5], C7(a097), k[6],
       C7(a098), k[7]);
    axpy(tmp, uh, h, s);
    lc(s, C7(a101), k[0], C7(a103), k[2], C7(a104), k[3], C7(a105), k[4], C7(a106), k[5], C7(a107), k[6]);
    axpy(g10, uh, h, s);
    f(tmp, t + dt, k[8]);
    f(g10, t + dt, k[9]);
    lc(s, C7(b1), k[0], C7(b4), k[3], C7(b5), k[4], C7(b6), k[5], C7(b7), k[6], C7(b8), k[7], C7(b9), k[8]);
    state_update<PR, D>(uh, uc, h, s, nh, nc);
    if (want_err) {
      lc(s, C7(btilde1), k[0], C7(btilde4), k[3], C7(btilde5), k[4], C7(btilde6), k[5], C7(btilde7), k[6],
         C7(btilde8), k[7], C7(btilde9), k[8], C7(btilde10), k[9]);
#pragma unroll
      for (int d = 0; d < D; ++d) e[d] = ErrUnscaled<R>::value ? s[d] : h * s[d];
    }
#undef C7
#undef C7T
  }

  enum { NX = 6 };  /* extra stages of the dense output */

  /* The six extra stages of the dense output (they depend on the step, not
   * on theta); dense = dense_stages + dense_eval, so that several save
   * points of one step can share them. */
  template <class KK>
  __device__ static __forceinline__ void dense_stages(const F& f, const R (&uh)[D], const R (&uc)[D], T told,
                                                      T tnew, T dtold, const KK& k, R (&x)[NX][D]) {
#define X7(x) CB<R>::v7x(vern7x_##x)
#define X7T(x) CB<T>::v7x(vern7x_##x)
    const R h = (R)dtold;
    R s[D], tmp[D];
    lc(s, X7(a1101), k[0], X7(a1104), k[3], X7(a1105), k[4], X7(a1106), k[5], X7(a1107), k[6], X7(a1108), k[7],
       X7(a1109), k[8]);
    axpy(tmp, uh, h, s); f(tmp, stime(tnew, X7T(c11), dtold), x[0]);
    lc(s, X7(a1201), k[0], X7(a1204), k[3], X7(a1205), k[4], X7(a1206), k[5], X7(a1207), k[6], X7(a1208), k[7],
       X7(a1209), k[8], X7(a1211), x[0]);
    axpy(tmp, uh, h, s); f(tmp, stime(tnew, X7T(c12), dtold), x[1]);
    lc(s, X7(a1301), k[0], X7(a1304), k[3], X7(a1305), k[4], X7(a1306), k[5], X7(a1307), k[6], X7(a1308), k[7],
       X7(a1309), k[8], X7(a1311), x[0], X7(a1312), x[1]);
    axpy(tmp, uh, h, s); f(tmp, stime(tnew, X7T(c13), dtold), x[2]);
    lc(s, X7(a1401), k[0], X7(a1404), k[3], X7(a1405), k[4], X7(a1406), k[5], X7(a1407), k[6], X7(a1408), k[7],
       X7(a1409), k[8], X7(a1411), x[0], X7(a1412), x[1], X7(a1413), x[2]);
    axpy(tmp, uh, h, s); f(tmp, stime(tnew, X7T(c14), dtold), x[3]);
    lc(s, X7(a1501), k[0], X7(a1504), k[3], X7(a1505), k[4], X7(a1506), k[5], X7(a1507), k[6], X7(a1508), k[7],
       X7(a1509), k[8], X7(a1511), x[0], X7(a1512), x[1], X7(a1513), x[2]);
    axpy(tmp, uh, h, s); f(tmp, stime(tnew, X7T(c15), dtold), x[4]);
    lc(s, X7(a1601), k[0], X7(a1604), k[3], X7(a1605), k[4], X7(a1606), k[5], X7(a1607), k[6], X7(a1608), k[7],
       X7(a1609), k[8], X7(a1611), x[0], X7(a1612), x[1], X7(a1613), x[2]);
    axpy(tmp, uh, h, s); f(tmp, stime(tnew, X7T(c16), dtold), x[5]);
#undef X7
#undef X7T
  }

  /* The dense output at theta from the step's stages and extra stages. */
  template <class KK, class XX>
  __device__ static __forceinline__ void dense_eval(const R (&uh)[D], const R (&uc)[D], T dtold, T theta,
                                                    const KK& k, const XX& x, double (&out)[D]) {
#define R7(x) CB<R>::v7r(vern7r_##x)
    const R h = (R)dtold;
    R s[D];
    const R th = (R)theta;
    const R th2 = th * th;
    R b[13], ex;
    ex = R7(r017); ex = fmaR(th, ex, R7(r016)); ex = fmaR(th, ex, R7(r015)); ex = fmaR(th, ex, R7(r014));
    ex = fmaR(th, ex, R7(r013)); ex = fmaR(th, ex, R7(r012)); ex = fmaR(th, ex, R7(r011)); b[0] = th * ex;
#define V7B(i, j)                                                                      \
  ex = R7(r##i##7); ex = fmaR(th, ex, R7(r##i##6)); ex = fmaR(th, ex, R7(r##i##5));        \
  ex = fmaR(th, ex, R7(r##i##4)); ex = fmaR(th, ex, R7(r##i##3)); ex = fmaR(th, ex, R7(r##i##2)); \
  b[j] = th2_times(th, th2, ex);
    V7B(04, 1) V7B(05, 2) V7B(06, 3) V7B(07, 4) V7B(08, 5) V7B(09, 6)
    V7B(11, 7) V7B(12, 8) V7B(13, 9) V7B(14, 10) V7B(15, 11) V7B(16, 12)
#undef V7B
    lc(s, b[0], k[0], b[1], k[3], b[2], k[4], b[3], k[5], b[4], k[6], b[5], k[7], b[6], k[8], b[7], x[0],
       b[8], x[1], b[9], x[2], b[10], x[3], b[11], x[4], b[12], x[5]);
    finish_dense<PR, D>(uh, uc, h, s, out);
#undef R7
  }

  template <class KK>
  __device__ static __forceinline__ void dense(const F& f, const R (&uh)[D], const R (&uc)[D], T told, T tnew,
                                               T dtold, T theta, const KK& k, double (&out)[D]) {
    R x[NX][D];
    dense_stages(f, uh, uc, told, tnew, dtold, k, x);
    dense_eval(uh, uc, dtold, theta, k, x, out);
  }
};

/* ------------------------------------------------------------------ Verner 9(8) */
/* src/verner/gpuvern9.jl:468-573 (adaptive attempt, dtmin and end snap 1f-7),
 * :105-183 (fixed step, no k16), dense output :631-757 (adaptive: relabelled
 * k2..k9 := k8..k15, stage times told + c*dtold) and :216-331 (fixed step:
 * stages 2..9 as they are, times t + c*dt with t advanced). */
template <class PR, int D, class F, bool ADAPTIVE>
struct MVern9Impl {
  typedef typename PR::R R;
  typedef typename PR::T T;
  enum { NK = 16, FSAL = 0, DTMIN_1F7 = 1, DENSE_F = 1 };

  __device__ static __forceinline__ void attempt(const F& f, const R (&uh)[D], const R (&uc)[D], T t, T dt,
                                                 R (&k)[NK][D], R (&nh)[D], R (&nc)[D], R (&e)[D], bool want_err) {
#define C9(x) CB<R>::v9(vern9_##x)
#define C9T(x) CB<T>::v9(vern9_##x)
    R tmp[D], s[D];
    const R h = (R)dt;
    f(uh, t, k[0]);
    const R a = (R)(dt * C9T(a0201));
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = vmaddR(a, k[0][d], uh[d]);
    f(tmp, stime(t, C9T(c1), dt), k[1]);
    lc(s, C9(a0301), k[0], C9(a0302), k[1]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c2), dt), k[2]);
    lc(s, C9(a0401), k[0], C9(a0403), k[2]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c3), dt), k[3]);
    lc(s, C9(a0501), k[0], C9(a0503), k[2], C9(a0504), k[3]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c4), dt), k[4]);
    lc(s, C9(a0601), k[0], C9(a0604), k[3], C9(a0605), k[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c5), dt), k[5]);
    lc(s, C9(a0701), k[0], C9(a0704), k[3], C9(a0705), k[4], C9(a0706), k[5]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c6), dt), k[6]);
    lc(s, C9(a0801), k[0], C9(a0806), k[5], C9(a0807), k[6]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c7), dt), k[7]);
    lc(s, C9(a0901), k[0], C9(a0906), k[5], C9(a0907), k[6], C9(a0908), k[7]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c8), dt), k[8]);
    lc(s, C9(a1001), k[0], C9(a1006), k[5], C9(a1007), k[6], C9(a1008), k[7], C9(a1009), k[8]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c9), dt), k[9]);
    lc(s, C9(a1101), k[0], C9(a1106), k[5], C9(a1107), k[6], C9(a1108), k[7], C9(a1109), k[8], C9(a1110), k[9]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c10), dt), k[10]);
    lc(s, C9(a1201), k[0], C9(a1206), k[5], C9(a1207), k[6], C9(a1208), k[7], C9(a1209), k[8], C9(a1210), k[9],
       C9(a1211), k[10]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c11), dt), k[11]);
    lc(s, C9(a1301), k[0], C9(a1306), k[5], C9(a1307), k[6], C9(a1308), k[7], C9(a1309), k[8], C9(a1310), k[9],
       C9(a1311), k[10], C9(a1312), k[11]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c12), dt), k[12]);
    lc(s, C9(a1401), k[0], C9(a1406), k[5], C9(a1407), k[6], C9(a1408), k[7], C9(a1409), k[8], C9(a1410), k[9],
       C9(a1411), k[10], C9(a1412), k[11], C9(a1413), k[12]);
    axpy(tmp, uh, h, s); f(tmp, stime(t, C9T(c13), dt), k[13]);
    lc(s, C9(a1501), k[0], C9(a1506), k[5], C9(a1507), k[6], C9(a1508), k[7], C9(a1509), k[8], C9(a1510), k[9],
       C9(a1511), k[10], C9(a1512), k[11], C9(a1513), k[12], C9(a1514), k[13]);
    axpy(tmp, uh, h, s);
    if (ADAPTIVE) {
      R g16[D];
      lc(s, C9(a1601), k[0], C9(a1606), k[5], C9(a1607), k[6], C9(a1608), k[7], C9(a1609), k[8], C9(a1610), k[9],
         C9(a1611), k[10], C9(a1612), k[11], C9(a1613), k[12]);
      axpy(g16, uh, h, s);
      f(tmp, t + dt, k[14]);
      f(g16, t + dt, k[15]);
    } else {
      f(tmp, t + dt, k[14]);
    }
    lc(s, C9(b1), k[0], C9(b8), k[7], C9(b9), k[8], C9(b10), k[9], C9(b11), k[10], C9(b12), k[11], C9(b13), k[12],
       C9(b14), k[13], C9(b15), k[14]);
    state_update<PR, D>(uh, uc, h, s, nh, nc);
    if (want_err) {
      lc(s, C9(btilde1), k[0], C9(btilde8), k[7], C9(btilde9), k[8], C9(btilde10), k[9], C9(btilde11), k[10],
         C9(btilde12), k[11], C9(btilde13), k[12], C9(btilde14), k[13], C9(btilde15), k[14], C9(btilde16), k[15]);
#pragma unroll
      for (int d = 0; d < D; ++d) e[d] = ErrUnscaled<R>::value ? s[d] : h * s[d];
    }
#undef C9
#undef C9T
  }

  enum { NX = 10 };  /* extra stages of the dense output */

  /* The ten extra stages of the dense output (they depend on the step, not on
   * theta); dense = dense_stages + dense_eval. */
  template <class KK>
  __device__ static __forceinline__ void dense_stages(const F& f, const R (&uh)[D], const R (&uc)[D], T told,
                                                      T tnew, T dtold, const KK& k, R (&x)[NX][D]) {
#define X9(x) CB<R>::v9x(vern9x_##x)
#define X9T(x) CB<T>::v9x(vern9x_##x)
    /* K1..K9: the nine stages the dense formulas call k1..k9 */
    const auto& K1 = k[0];
    const auto& K2 = k[ADAPTIVE ? 7 : 1];
    const auto& K3 = k[ADAPTIVE ? 8 : 2];
    const auto& K4 = k[ADAPTIVE ? 9 : 3];
    const auto& K5 = k[ADAPTIVE ? 10 : 4];
    const auto& K6 = k[ADAPTIVE ? 11 : 5];
    const auto& K7 = k[ADAPTIVE ? 12 : 6];
    const auto& K8 = k[ADAPTIVE ? 13 : 7];
    const auto& K9 = k[ADAPTIVE ? 14 : 8];
    const T tb = ADAPTIVE ? told : tnew;
    const R h = (R)dtold;
    R s[D], tmp[D];
    lc(s, X9(a1701), K1, X9(a1708), K2, X9(a1709), K3, X9(a1710), K4, X9(a1711), K5, X9(a1712), K6, X9(a1713), K7,
       X9(a1714), K8, X9(a1715), K9);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c17), dtold), x[0]);
    lc(s, X9(a1801), K1, X9(a1808), K2, X9(a1809), K3, X9(a1810), K4, X9(a1811), K5, X9(a1812), K6, X9(a1813), K7,
       X9(a1814), K8, X9(a1815), K9, X9(a1817), x[0]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c18), dtold), x[1]);
    lc(s, X9(a1901), K1, X9(a1908), K2, X9(a1909), K3, X9(a1910), K4, X9(a1911), K5, X9(a1912), K6, X9(a1913), K7,
       X9(a1914), K8, X9(a1915), K9, X9(a1917), x[0], X9(a1918), x[1]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c19), dtold), x[2]);
    lc(s, X9(a2001), K1, X9(a2008), K2, X9(a2009), K3, X9(a2010), K4, X9(a2011), K5, X9(a2012), K6, X9(a2013), K7,
       X9(a2014), K8, X9(a2015), K9, X9(a2017), x[0], X9(a2018), x[1], X9(a2019), x[2]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c20), dtold), x[3]);
    lc(s, X9(a2101), K1, X9(a2108), K2, X9(a2109), K3, X9(a2110), K4, X9(a2111), K5, X9(a2112), K6, X9(a2113), K7,
       X9(a2114), K8, X9(a2115), K9, X9(a2117), x[0], X9(a2118), x[1], X9(a2119), x[2], X9(a2120), x[3]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c21), dtold), x[4]);
    lc(s, X9(a2201), K1, X9(a2208), K2, X9(a2209), K3, X9(a2210), K4, X9(a2211), K5, X9(a2212), K6, X9(a2213), K7,
       X9(a2214), K8, X9(a2215), K9, X9(a2217), x[0], X9(a2218), x[1], X9(a2219), x[2], X9(a2220), x[3],
       X9(a2221), x[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c22), dtold), x[5]);
    lc(s, X9(a2301), K1, X9(a2308), K2, X9(a2309), K3, X9(a2310), K4, X9(a2311), K5, X9(a2312), K6, X9(a2313), K7,
       X9(a2314), K8, X9(a2315), K9, X9(a2317), x[0], X9(a2318), x[1], X9(a2319), x[2], X9(a2320), x[3],
       X9(a2321), x[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c23), dtold), x[6]);
    lc(s, X9(a2401), K1, X9(a2408), K2, X9(a2409), K3, X9(a2410), K4, X9(a2411), K5, X9(a2412), K6, X9(a2413), K7,
       X9(a2414), K8, X9(a2415), K9, X9(a2417), x[0], X9(a2418), x[1], X9(a2419), x[2], X9(a2420), x[3],
       X9(a2421), x[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c24), dtold), x[7]);
    lc(s, X9(a2501), K1, X9(a2508), K2, X9(a2509), K3, X9(a2510), K4, X9(a2511), K5, X9(a2512), K6, X9(a2513), K7,
       X9(a2514), K8, X9(a2515), K9, X9(a2517), x[0], X9(a2518), x[1], X9(a2519), x[2], X9(a2520), x[3],
       X9(a2521), x[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c25), dtold), x[8]);
    lc(s, X9(a2601), K1, X9(a2608), K2, X9(a2609), K3, X9(a2610), K4, X9(a2611), K5, X9(a2612), K6, X9(a2613), K7,
       X9(a2614), K8, X9(a2615), K9, X9(a2617), x[0], X9(a2618), x[1], X9(a2619), x[2], X9(a2620), x[3],
       X9(a2621), x[4]);
    axpy(tmp, uh, h, s); f(tmp, stime(tb, X9T(c26), dtold), x[9]);
#undef X9
#undef X9T
  }

  /* The dense output at theta from the step's stages and extra stages. */
  template <class KK, class XX>
  __device__ static __forceinline__ void dense_eval(const R (&uh)[D], const R (&uc)[D], T dtold, T theta,
                                                    const KK& k, const XX& x, double (&out)[D]) {
#define R9(x) CB<R>::v9r(vern9r_##x)
    const auto& K1 = k[0];
    const auto& K2 = k[ADAPTIVE ? 7 : 1];
    const auto& K3 = k[ADAPTIVE ? 8 : 2];
    const auto& K4 = k[ADAPTIVE ? 9 : 3];
    const auto& K5 = k[ADAPTIVE ? 10 : 4];
    const auto& K6 = k[ADAPTIVE ? 11 : 5];
    const auto& K7 = k[ADAPTIVE ? 12 : 6];
    const auto& K8 = k[ADAPTIVE ? 13 : 7];
    const auto& K9 = k[ADAPTIVE ? 14 : 8];
    const R h = (R)dtold;
    R s[D];
    const R th = (R)theta;
    const R th2 = th * th;
    R b[19], ex;
    ex = R9(r019); ex = fmaR(th, ex, R9(r018)); ex = fmaR(th, ex, R9(r017)); ex = fmaR(th, ex, R9(r016));
    ex = fmaR(th, ex, R9(r015)); ex = fmaR(th, ex, R9(r014)); ex = fmaR(th, ex, R9(r013));
    ex = fmaR(th, ex, R9(r012)); ex = fmaR(th, ex, R9(r011)); b[0] = th * ex;
#define V9B(i, j)                                                                             \
  ex = R9(r##i##9); ex = fmaR(th, ex, R9(r##i##8)); ex = fmaR(th, ex, R9(r##i##7));               \
  ex = fmaR(th, ex, R9(r##i##6)); ex = fmaR(th, ex, R9(r##i##5)); ex = fmaR(th, ex, R9(r##i##4)); \
  ex = fmaR(th, ex, R9(r##i##3)); ex = fmaR(th, ex, R9(r##i##2)); b[j] = th2_times(th, th2, ex);
    V9B(08, 1) V9B(09, 2) V9B(10, 3) V9B(11, 4) V9B(12, 5) V9B(13, 6) V9B(14, 7) V9B(15, 8)
    V9B(17, 9) V9B(18, 10) V9B(19, 11) V9B(20, 12) V9B(21, 13) V9B(22, 14) V9B(23, 15) V9B(24, 16)
    V9B(25, 17) V9B(26, 18)
#undef V9B
    lc(s, b[0], K1, b[1], K2, b[2], K3, b[3], K4, b[4], K5, b[5], K6, b[6], K7, b[7], K8, b[8], K9, b[9], x[0],
       b[10], x[1], b[11], x[2], b[12], x[3], b[13], x[4], b[14], x[5], b[15], x[6], b[16], x[7], b[17], x[8],
       b[18], x[9]);
    finish_dense<PR, D>(uh, uc, h, s, out);
#undef R9
  }

  template <class KK>
  __device__ static __forceinline__ void dense(const F& f, const R (&uh)[D], const R (&uc)[D], T told, T tnew,
                                               T dtold, T theta, const KK& k, double (&out)[D]) {
    R x[NX][D];
    dense_stages(f, uh, uc, told, tnew, dtold, k, x);
    dense_eval(uh, uc, dtold, theta, k, x, out);
  }
};
template <class PR, int D, class F> struct MAVern9 : MVern9Impl<PR, D, F, true> {};
template <class PR, int D, class F> struct MVern9 : MVern9Impl<PR, D, F, false> {};

/* ------------------------------------------------------------------ classic RK4 (fixed step) */
/* uprev + (dt/2) k of RK4's middle stages: one fused multiply-add with the
 * halved step, or with GBODE_REF the reference's dt * (1/2 * k) + uprev */
template <class R> __device__ __forceinline__ R half_step(R h, R hh, R k, R u) {
#ifdef GBODE_REF
  return h * ((R)0.5 * k) + u;
#else
  return fmaR(hh, k, u);
#endif
}
/* src/rk4/gpurk4.jl:73-84; the stage time t is the END of the step (ts[i]). */
template <class PR, int D, class F>
struct MRK4 {
  typedef typename PR::R R;
  typedef typename PR::T T;
  __device__ static __forceinline__ void step(const F& f, const R (&uh)[D], const R (&uc)[D], T t, T dt,
                                              R (&nh)[D], R (&nc)[D]) {
    R k1[D], k2[D], k3[D], k4[D], tmp[D], s[D];
    const R h = (R)dt;
    const R hh = h * (R)0.5;
    f(uh, t, k1);
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = half_step(h, hh, k1[d], uh[d]);
    f(tmp, fmaR((T)0.5, dt, t), k2);
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = half_step(h, hh, k2[d], uh[d]);
    f(tmp, fmaR((T)0.5, dt, t), k3);
#pragma unroll
    for (int d = 0; d < D; ++d) tmp[d] = vmaddR(h, k3[d], uh[d]);
    f(tmp, t + dt, k4);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      R sum = k1[d] + k4[d];
      sum = vmaddR((R)2, k2[d], sum);
      s[d] = vmaddR((R)2, k3[d], sum);
    }
#ifdef GBODE_REF
    /* u = uprev + dt * (1/6 * (k1 + 2k2 + 2k3 + k4)) */
#pragma unroll
    for (int d = 0; d < D; ++d) s[d] = (R)(1.0 / 6.0) * s[d];
    state_update<PR, D>(uh, uc, h, s, nh, nc);
#else
    state_update<PR, D>(uh, uc, h * (R)(1.0 / 6.0), s, nh, nc);
#endif
  }
};

/* Forward Euler, src/euler/gpueuler.jl:67-76: k1 = f(u, p, t) with t the END
 * of the step (t = ts[i], the same quirk as GPUSimpleRK4), u = uprev + dt*k1
 * (one fused multiply-add; the compensated sum in the Kahan mode). */
template <class PR, int D, class F>
struct MEuler {
  typedef typename PR::R R;
  typedef typename PR::T T;
  __device__ static __forceinline__ void step(const F& f, const R (&uh)[D], const R (&uc)[D], T t, T dt,
                                              R (&nh)[D], R (&nc)[D]) {
    R k1[D];
    f(uh, t, k1);
    state_update<PR, D>(uh, uc, (R)dt, k1, nh, nc);
  }
};

/* ------------------------------------------------------------------ per-lane trajectory state */
template <class PR, int D, class F, int NK>
struct Lane {
  typedef typename PR::R R;
  typedef typename PR::T T;
  R uh[D], uc[D];
  R k[NK][D];
  F f;
  T t, dt;
  float qoldp;
#ifdef GBODE_CTRL64
  double lqold; /* beta2 * log(qold) of the FP64 controller */
#endif
#ifdef GBODE_CTRL_DS
  dsf lqds; /* beta2 * log(qold) of the double-single controller */
#endif
#ifdef GBODE_REF
  double qold; /* the reference controller's qold */
#endif
  long long idx, att, cur, ninterp;
  int nacc, nrej;
  double dt_first;
  bool nan_seen;
};

/* Address of value w of output point j of trajectory idx (either layout). */
__device__ __forceinline__ double* us_at(const KParams& P, long long j, long long w, long long idx) {
  return P.us + j * P.us_sj + w * P.us_sw + idx * P.us_si;
}

/* Write saveat point j of trajectory idx: the state, or (P.output == 1) the
 * Kuramoto order parameter r = |(1/D) sum_k exp(i v_k)| = sqrt(C^2 + S^2) / D
 * of it, so a phase ensemble keeps one number per save point. */
template <class PR, int D>
__device__ __forceinline__ void store_point(const KParams& P, long long idx, long long j, const double (&v)[D]) {
  if (!P.us) return;
  if (!GBODE_CHECK(P, idx >= 0 && idx < P.n && j >= 0 && j < (P.nsave > 0 ? P.nsave : P.ngrid), CHK_SAVE)) return;
#ifdef GBODE_USER_OUTPUT
  /* a user output function (ode_output_compile), defined before this header by
   * the run-time compiled translation unit together with GBODE_OUTPUT_WIDTH and
   * GBODE_OUTPUT_NP */
  if (P.output >= 1000) {
    double pv[GBODE_OUTPUT_NP > 0 ? GBODE_OUTPUT_NP : 1];
#pragma unroll
    for (int q = 0; q < GBODE_OUTPUT_NP; ++q) pv[q] = P.p[(long long)q * P.n + idx];
    const double t = P.saveat ? P.saveat[j] : P.grid[j];
    double o[GBODE_OUTPUT_WIDTH];
    gbode_user_output(o, v, pv, t);
#pragma unroll
    for (int w = 0; w < GBODE_OUTPUT_WIDTH; ++w) *us_at(P, j, w, idx) = o[w];
    return;
  }
#endif
  if (P.output == 1) {
    double C = 0.0, S = 0.0;
#pragma unroll 1
    for (int d = 0; d < D; ++d) {
      double sn, cs;
      sincosR(v[d], &sn, &cs);
      C = C + cs;
      S = S + sn;
    }
#ifdef GBODE_REF
    *us_at(P, j, 0, idx) = __dsqrt_rn(C * C + S * S) / (double)D;
#else
    *us_at(P, j, 0, idx) = __dsqrt_rn(__fma_rn(C, C, S * S)) / (double)D;
#endif
    return;
  }
#pragma unroll
  for (int d = 0; d < D; ++d) *us_at(P, j, d, idx) = v[d];
}

template <class PR, int D, class L>
__device__ __forceinline__ void state_value(const L& l, double (&v)[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) v[d] = PR::KAHAN ? (double)l.uh[d] - (double)l.uc[d] : (double)l.uh[d];
}

/* Every-step output (save_everystep = true without saveat, the reference's
 * push!(us, u); push!(ts, t) after each accepted step, gpuatsit5.jl:301-303):
 * row k of trajectory l.idx is the state after its k-th accepted step. */
template <class PR, int D, class L>
__device__ __forceinline__ void store_step(const KParams& P, const L& l, long long k) {
  if (!P.ev_t) return;
  const long long r = P.ev_off[l.idx] + k;
  if (!GBODE_CHECK(P, r >= P.ev_off[l.idx] && r < P.ev_off[l.idx + 1], CHK_STEP)) return;
  double v[D];
  state_value<PR, D>(l, v);
  P.ev_t[r] = (double)l.t;
#pragma unroll
  for (int d = 0; d < D; ++d) P.ev_u[r * D + d] = v[d];
}

/* Load trajectory idx: parameters, u0, t0, dt; first saveat point if it is t0. */
template <class PR, int D, class F, int NK>
__device__ __forceinline__ void lane_load(const KParams& P, long long idx, Lane<PR, D, F, NK>& l) {
  if (!GBODE_CHECK(P, idx >= 0 && idx < P.n, CHK_TRAJ)) idx = 0;
#ifdef GBODE_BOUNDS_CHECK
  atomicAdd(&P.visited[idx], 1u);
#endif
  typedef typename PR::R R;
  typedef typename PR::T T;
  l.idx = idx;
#pragma unroll
  for (int j = 0; j < F::NP; ++j) l.f.p[j] = (R)P.p[(long long)j * P.n + idx];
  rhs_loaded(l.f);
#pragma unroll
  for (int d = 0; d < D; ++d) {
    l.uh[d] = (R)P.u0[(long long)d * P.n + idx];
    l.uc[d] = (R)0;
  }
  l.t = (T)P.t0;
  l.dt = (T)(P.dt0 ? P.dt0[idx] : P.dt);
  /* qold^beta2, or in the single-precision modes beta2 * log2(qold) */
  l.qoldp = sizeof(R) == sizeof(float) ? (float)(2.0 / 25.0) * CTRL32_L2_QOLDINIT
                                       : ctrl_pow((float)1.0e-4, (float)(2.0 / 25.0));
#ifdef GBODE_CTRL64
  l.lqold = (2.0 / 25.0) * CTRL64_LN_QOLDINIT;
#endif
#ifdef GBODE_CTRL_DS
  l.lqds = ds_mul({GBODE_DS_B2_H, GBODE_DS_B2_L}, {GBODE_DS_LN_QOLDINIT_H, GBODE_DS_LN_QOLDINIT_L});
#endif
#ifdef GBODE_REF
  l.qold = 1.0e-4;
#endif
  l.att = 0;
  l.cur = 0;
  l.ninterp = 0;
  l.nacc = 0;
  l.nrej = 0;
  l.dt_first = __longlong_as_double(0x7ff8000000000000LL);
  l.nan_seen = false;
  if (P.nsave > 0 && (T)P.saveat[0] == (T)P.t0) {
    double v[D];
    state_value<PR, D>(l, v);
    store_point<PR, D>(P, idx, 0, v);
    l.cur = 1;
  }
  store_step<PR, D>(P, l, 0);
}

/* Attempts, dense-output points and early stops summed over the trajectories
 * a thread finished; reduced across the warp once, at kernel exit. */
struct Totals {
  unsigned long long att, sav, fail;
};

__device__ __forceinline__ void flush_totals(const KParams& P, Totals t) {
  const unsigned FULL = 0xffffffffu;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    t.att += __shfl_xor_sync(FULL, t.att, o);
    t.sav += __shfl_xor_sync(FULL, t.sav, o);
    t.fail += __shfl_xor_sync(FULL, t.fail, o);
  }
  if ((threadIdx.x & 31) == 0 && P.stats) {
    atomicAdd(P.stats, t.att);
    atomicAdd(P.stats + 1, t.sav);
    atomicAdd(P.stats + 2, t.fail);
  }
}

template <class PR, int D, class F, int NK>
__device__ __forceinline__ void lane_finish(const KParams& P, Lane<PR, D, F, NK>& l, int ret, Totals& tot) {
  const long long idx = l.idx;
  double v[D];
  state_value<PR, D>(l, v);
  if (P.u_final) {
#pragma unroll
    for (int d = 0; d < D; ++d) P.u_final[(long long)d * P.n + idx] = v[d];
  }
  if (ret == RET_DTMIN || ret == RET_MAXITERS) tot.fail += 1;
  if (ret == RET_DEFAULT && l.nan_seen) ret = RET_NAN;
  if (P.t_final) P.t_final[idx] = (double)l.t;
  if (P.retcode) P.retcode[idx] = (signed char)ret;
  if (P.naccept) P.naccept[idx] = l.nacc;
  if (P.nreject) P.nreject[idx] = l.nrej;
  if (P.dt_first) P.dt_first[idx] = l.dt_first;
  if (P.us) {
    /* save points never reached: NaN, in the layout of the output kind */
    const double qnan = __longlong_as_double(0x7ff8000000000000LL);
#ifdef GBODE_USER_OUTPUT
    const int width = P.output == 1 ? 1 : (P.output >= 1000 ? GBODE_OUTPUT_WIDTH : D);
#else
    const int width = P.output == 1 ? 1 : D;
#endif
    for (long long j = l.cur; j < P.nsave; ++j)
      for (int d = 0; d < width; ++d) *us_at(P, j, d, idx) = qnan;
  }
  tot.att += (unsigned long long)l.att;
  tot.sav += (unsigned long long)l.ninterp;
}

enum { TRY_REJECTED = 0, TRY_ACCEPTED = 1, TRY_STOPPED = 2 };

/* What an accepted step leaves for its dense output and commit. */
template <class T>
struct Accepted {
  T told, dtold;
};

/* One attempt of an adaptive method and its accept/reject decision: the
 * stages, the error norm and the controller; on acceptance t, dt and the
 * counters advance, while the saveat points of the step and the commit of the
 * new state are left to the caller (the state before the step, the stage
 * values and the proposal nh/nc are still intact).  TRY_STOPPED: dt fell
 * below dtmin or the attempt cap was reached; the outputs are written. */
template <class M, class PR, int D, class F, int NK>
__device__ __forceinline__ int adaptive_try(const KParams& P, Lane<PR, D, F, NK>& l, Totals& tot,
                                            typename PR::R (&nh)[D], typename PR::R (&nc)[D],
                                            Accepted<typename PR::T>& acc_out) {
  typedef typename PR::R R;
  typedef typename PR::T T;
  const double dtmin = M::DTMIN_1F7 ? (double)1.0e-7f : 1.0e-14;
  if (d_lt<PR>((double)l.dt, dtmin)) { lane_finish(P, l, RET_DTMIN, tot); return TRY_STOPPED; }
  if (P.maxiters > 0 && l.att >= P.maxiters) { lane_finish(P, l, RET_MAXITERS, tot); return TRY_STOPPED; }
  /* The end-of-span bookkeeping of an accepted step depends only on t and dt,
   * both known now: computed before the stages (the same operations, so the
   * same values), it overlaps them instead of lengthening every attempt's
   * dependency chain after the error estimate. */
  const T tf = (T)P.tf;
  const T rest = tf - l.t - l.dt;
  const T tnext = d_lt<PR>((double)rest, dtmin) ? tf : l.t + l.dt;
  R e[D];
  M::attempt(l.f, l.uh, l.uc, l.t, l.dt, l.k, nh, nc, e, true);
  l.att += 1;
#ifdef GBODE_REF
  if (sizeof(R) == sizeof(double)) {
    /* The reference's norm and PI controller in IEEE double (ODE_CTRL_REF):
     * EEst = sqrt(sum((e ./ (abstol .+ max.(|uprev|, |u|) .* reltol)).^2) / D),
     * q11 = EEst^beta1; reject: dt /= min(1/qmin, q11/gamma); accept:
     * q = q11 / qold^beta2 (1/qmax when EEst == 0), dt /= max(1/qmax,
     * min(1/qmin, q/gamma)), qold = max(EEst, qoldinit) -- with
     * (beta1, beta2, qmax, qmin, gamma, qoldinit) = (7/50, 2/25, 10, 1/5,
     * 9/10, 1e-4), src/SimpleDiffEq.jl:67-77, src/tsit5/gpuatsit5.jl:276-299;
     * 1/qmax and 1/qmin are 0.1 and 5.0 in double; the powers correctly
     * rounded (cr_pow, crpow.h). */
    /* The comparisons, maxima and minima are the integer forms of bitops.h
     * and ds_absmax (the same results; a double compare would take an
     * FP64-pipe slot), with Julia's NaN propagation for min and max and the
     * @fastmath clamps' compare-and-select. */
    const double abstol = P.abstol, reltol = P.reltol;
    double acc = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const double m = ds_absmax((double)l.uh[d], (double)nh[d]);
      const double r = (double)e[d] / (abstol + m * reltol);
      acc = (d == 0) ? r * r : acc + r * r;
    }
    const double EEst = sqrtR(acc / (double)D);
    const bool enan = bo_isnan(EEst);
    if (enan) l.nan_seen = true;
    const double q11 = cr_pow(EEst, 7.0 / 50.0);
    if (bo_lt(1.0, EEst)) {
      const double f = q11 / (9.0 / 10.0);  /* min(1/qmin, q11/gamma), q11 >= 0 */
      l.dt = l.dt / (T)(bo_isnan(f) || bo_lt(f, 5.0) ? f : 5.0);
      l.nrej += 1;
      return TRY_REJECTED;
    }
    const bool ezero = (__double_as_longlong(EEst) & 0x7fffffffffffffffLL) == 0;
    double q = ezero ? 0.1 : q11 / cr_pow(l.qold, 2.0 / 25.0);
    const double g = q / (9.0 / 10.0);
    const double gm = bo_lt(5.0, g) ? 5.0 : g;  /* fm_min(1/qmin, q/gamma) */
    q = bo_lt(0.1, gm) ? gm : 0.1;              /* fm_max(1/qmax, .) */
    l.qold = enan ? EEst : (bo_lt(EEst, 1.0e-4) ? 1.0e-4 : EEst);  /* max(EEst, qoldinit), EEst >= 0 */
    const T dtold = l.dt;
    const T dtn = l.dt / (T)q;
    l.dt = absmin(dtn, rest);
    const T told = l.t;
    l.t = tnext;
    if (l.nacc == 0) l.dt_first = (double)dtold;
    l.nacc += 1;
    acc_out.told = told;
    acc_out.dtold = dtold;
    return TRY_ACCEPTED;
  }
#endif
#ifdef GBODE_CTRL_DS
  if (sizeof(R) == sizeof(double)) {
    /* Double-single norm and controller: a = EEst^2 = mean((e ./ (abstol .+
     * max.(|uprev|, |u|) .* reltol)).^2) with every term split into single
     * pairs (ds_split, integer operations only), le = ln(a)/2 (ds_log), and
     * the reference's factors on logarithms as in the FP64 controller below,
     * with one ds_exp for the factor: dt follows the reference's step sizes
     * to about 2^-44, and the attempt's only double operations here are the
     * two of ds_scale.  With abstol below 1e-30 the norm is the double one
     * (the single exponent range cannot hold its scale); the tolerances come
     * split on the host (KParams::tol_ds). */
    const dsf one = {1.0f, 0.0f};
    dsf le;
    bool reject, is_zero = true;
    if (!P.norm_fp64) {
      const dsf abstol = {P.tol_ds[0], P.tol_ds[1]}, reltol = {P.tol_ds[2], P.tol_ds[3]};
      /* e holds the unscaled sum: e_d = dt e[d], formed before the division
       * so that the quotient stays in the single range for any tolerance */
      const dsf hds = ds_split((double)l.dt);
      dsf acc = {0.0f, 0.0f};
      bool nan_in = bo_isnan((double)l.dt);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const long long eb = __double_as_longlong((double)e[d]) & 0x7fffffffffffffffLL;
        const double mx = ds_absmax((double)l.uh[d], (double)nh[d]);
        is_zero = is_zero && eb == 0;
        nan_in = nan_in || eb > 0x7ff0000000000000LL || __double_as_longlong(mx) > 0x7ff0000000000000LL;
        const dsf r = ds_div(ds_mul(ds_split((double)e[d]), hds), ds_add(ds_mul(ds_split(mx), reltol), abstol));
        acc = d == 0 ? ds_sqr(r) : ds_add(acc, ds_sqr(r));
      }
      const dsf a = ds_mul(acc, {(float)(1.0 / D), (float)(1.0 / D - (double)(float)(1.0 / D))});
      if (nan_in) {
        l.nan_seen = true;
        reject = false;
        le = {__int_as_float(0x7fffffff), 0.0f};
      } else {
        /* beyond the single range (an overflow leaves NaN or infinity) the
         * step is rejected with the largest shrink, as the reference's factor
         * min(1/qmin, EEst^beta1/gamma) is for every EEst above 5e4 */
        const bool huge = !(a.h <= 0x1p126f);
        reject = huge || ds_gt(a, one);
        const dsf ac = huge ? dsf{0x1p126f, 0.0f} : a.h < 0x1p-120f ? dsf{0x1p-120f, 0.0f} : a;
        const dsf lg = ds_log(ac);
        le = {0.5f * lg.h, 0.5f * lg.l};
      }
    } else {
      const double abstol = P.abstol, reltol = P.reltol;
      double acc = 0.0;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        const double m = jmax(fabs((double)l.uh[d]), fabs((double)nh[d]));
        const double r = ((double)e[d] * (double)l.dt) / __fma_rn(m, reltol, abstol);
        acc = (d == 0) ? r * r : __fma_rn(r, r, acc);
      }
      const double EEst = __dsqrt_rn(acc / (double)D);
      is_zero = EEst == 0.0;
      reject = EEst > 1.0;
      if (EEst != EEst) {
        l.nan_seen = true;
        le = {(float)EEst, 0.0f};
      } else {
        const dsf es = ds_split(fmin(fmax(EEst, 0x1p-60), 0x1p63));  /* a normal single pair */
        le = ds_log(es);
      }
    }
    const dsf B1 = {GBODE_DS_B1_H, GBODE_DS_B1_L}, B2 = {GBODE_DS_B2_H, GBODE_DS_B2_L};
    const dsf LQMAXI = {GBODE_DS_LN_QMAXI_H, GBODE_DS_LN_QMAXI_L};
    const dsf LQMINI = {GBODE_DS_LN_QMINI_H, GBODE_DS_LN_QMINI_L};
    const dsf MLGAMMA = {-GBODE_DS_LN_GAMMA_H, -GBODE_DS_LN_GAMMA_L};
    const dsf LQOLDINIT = {GBODE_DS_LN_QOLDINIT_H, GBODE_DS_LN_QOLDINIT_L};
    /* the log of the factor dt is divided by: rejected, min(ln(1/qmin),
     * beta1 le - ln gamma); accepted, the clamped beta1 le - beta2 ln qold -
     * ln gamma (ln(1/qmax) when EEst == 0); one ds_exp for both */
    dsf lfac;
    if (reject) {
      lfac = ds_min(LQMINI, ds_add(ds_mul(B1, le), MLGAMMA));
    } else {
      const dsf lq0 = is_zero ? LQMAXI : ds_add(ds_mul(B1, le), ds_neg(l.lqds));
      lfac = ds_max(LQMAXI, ds_min(LQMINI, ds_add(lq0, MLGAMMA)));
      l.lqds = ds_mul(B2, ds_max(le, LQOLDINIT));
    }
    const dsf fac = ds_exp(ds_neg(lfac));
    if (reject) {
      l.dt = (T)ds_scale((double)l.dt, fac);
      l.nrej += 1;
      return TRY_REJECTED;
    }
    const T dtold = l.dt;
    const T dtn = (T)ds_scale((double)l.dt, fac);
    l.dt = absmin(dtn, rest);
    const T told = l.t;
    l.t = tnext;
    if (l.nacc == 0) l.dt_first = (double)dtold;
    l.nacc += 1;
    acc_out.told = told;
    acc_out.dtold = dtold;
    return TRY_ACCEPTED;
  }
#endif
  /* EEst = sqrt(mean((e ./ (abstol .+ max.(|uprev|, |u|) .* reltol)).^2)), in
   * single precision (ODE_CTRL_FP32 and the single-precision modes; each
   * conversion of a double term costs one FP64-pipe instruction, the FP64
   * division and square root it avoids about nine each); double when abstol
   * is so small that the scale could leave the float range (P.norm_fp64). */
  float Ef;
  double EEst64 = 0.0; /* the double norm, when computed */
  bool reject, is_zero;
  if (sizeof(R) == sizeof(float)) {
    /* single-precision modes: the mean square a = EEst^2 without division or
     * square root (rcp_nr; the controller below works on log2 EEst =
     * log2(a) / 2, and a > 1 exactly when EEst > 1) */
    const float abstol = (float)P.abstol, reltol = (float)P.reltol;
    float acc = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float m = jmax(fabsf((float)l.uh[d]), fabsf((float)nh[d]));
      const float r = (float)e[d] * rcp_nr(__fmaf_rn(m, reltol, abstol));
      acc = (d == 0) ? r * r : __fmaf_rn(r, r, acc);
    }
    Ef = acc * (float)(1.0 / D);
    reject = Ef > 1.0f;
    is_zero = Ef == 0.0f;
  } else if (!P.norm_fp64) {
    const float abstol = (float)P.abstol, reltol = (float)P.reltol;
    float acc = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float m = jmax(fabsf((float)l.uh[d]), fabsf((float)nh[d]));
      const float r = __fdiv_rn((float)e[d], __fmaf_rn(m, reltol, abstol));
      acc = (d == 0) ? r * r : __fmaf_rn(r, r, acc);
    }
    Ef = __fsqrt_rn(__fdiv_rn(acc, (float)D));
    reject = Ef > 1.0f;
    is_zero = Ef == 0.0f;
  } else {
    const R abstol = (R)P.abstol, reltol = (R)P.reltol;
    R acc = (R)0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const R m = jmax(absR(l.uh[d]), absR(nh[d]));
      const R r = e[d] / fmaR(m, reltol, abstol);
      acc = (d == 0) ? r * r : fmaR(r, r, acc);
    }
    const R EEst = sqrtR(acc / (R)D);
    EEst64 = (double)EEst;
    Ef = (float)EEst;
    reject = EEst > (R)1;
    is_zero = EEst == (R)0;
  }
  if (Ef != Ef) l.nan_seen = true;
#ifdef GBODE_CTRL64
  if (sizeof(R) == sizeof(double)) {
    /* FP64 controller: the factors of the reference's controller in double,
     * in the log domain.  le = log(EEst); reject: dt /= min(1/qmin,
     * EEst^beta1/gamma); accept: q = EEst^beta1 / qold^beta2 (1/qmax when
     * EEst == 0), dt /= max(1/qmax, min(1/qmin, q/gamma)), qold = max(EEst,
     * qoldinit) -- with every power, quotient and clamp taken on logarithms
     * (log_dev, exp_dev: within 2 ulp) and one exp_dev for the factor, so
     * that dt follows the reference's step sizes to a few ulps instead of the
     * single-precision controller's 2^-24. */
    const double E = (sizeof(R) == sizeof(float) || !P.norm_fp64) ? (double)Ef : (double)EEst64;
    const double le = (E != E) ? E : log_dev(fmin(fmax(E, 0x1p-1022), 0x1.fffffffffffffp+1023));
    if (reject) {
      const double lf = jmin(CTRL64_LN_QMINI, __fma_rn(7.0 / 50.0, le, -CTRL64_LN_GAMMA));
      l.dt = l.dt * (T)exp_dev(-lf);
      l.nrej += 1;
      return TRY_REJECTED;
    }
    const double lq0 = is_zero ? CTRL64_LN_QMAXI : __fma_rn(7.0 / 50.0, le, -l.lqold);
    const double lq = fm_max(CTRL64_LN_QMAXI, fm_min(CTRL64_LN_QMINI, lq0 - CTRL64_LN_GAMMA));
    l.lqold = (2.0 / 25.0) * jmax(le, CTRL64_LN_QOLDINIT);
    const T dtold = l.dt;
    const T dtn = l.dt * (T)exp_dev(-lq);
    l.dt = absmin(dtn, rest);
    const T told = l.t;
    l.t = tnext;
    if (l.nacc == 0) l.dt_first = (double)dtold;
    l.nacc += 1;
    acc_out.told = told;
    acc_out.dtold = dtold;
    return TRY_ACCEPTED;
  }
#endif
  if (sizeof(R) == sizeof(float)) {
    /* single-precision modes: the PI factors on log2 EEst, one exp2_nr per
     * attempt; l.qoldp holds beta2 * log2(qold).  The clamps are those of
     * the double controller below, in the log domain. */
    const float B1F = (float)(7.0 / 50.0), B2F = (float)(2.0 / 25.0);
    const float l2E = (Ef != Ef) ? Ef : 0.5f * log2_nr(Ef);
    if (reject) {
      const float lf = jmin(CTRL32_L2_QMINI, __fmaf_rn(B1F, l2E, -CTRL32_L2_GAMMA));
      l.dt = l.dt * (T)exp2_nr(-lf);
      l.nrej += 1;
      return TRY_REJECTED;
    }
    const float lq0 = is_zero ? CTRL32_L2_QMAXI : __fmaf_rn(B1F, l2E, -l.qoldp);
    const float lq = fm_max(CTRL32_L2_QMAXI, fm_min(CTRL32_L2_QMINI, lq0 - CTRL32_L2_GAMMA));
    l.qoldp = B2F * jmax(l2E, CTRL32_L2_QOLDINIT);
    const T dtold = l.dt;
    const T dtn = l.dt * (T)exp2_nr(-lq);
    l.dt = absmin(dtn, rest);
    const T told = l.t;
    l.t = tnext;
    if (l.nacc == 0) l.dt_first = (double)dtold;
    l.nacc += 1;
    acc_out.told = told;
    acc_out.dtold = dtold;
    return TRY_ACCEPTED;
  }
  const float B1 = (float)(7.0 / 50.0), B2 = (float)(2.0 / 25.0), GAM = (float)(9.0 / 10.0);
  const float QMAXI = 0.1f, QMINI = 5.0f, QOLDINIT = (float)1.0e-4;
  const float q11 = ctrl_pow(Ef, B1);
  if (reject) {
    const float fac = jmin(QMINI, __fdiv_rn(q11, GAM));
    l.dt = l.dt * (T)__fdiv_rn(1.0f, fac);
    l.nrej += 1;
    return TRY_REJECTED;
  }
  float q = is_zero ? QMAXI : __fdiv_rn(q11, l.qoldp);
  q = fm_max(QMAXI, fm_min(QMINI, __fdiv_rn(q, GAM)));
  l.qoldp = ctrl_pow(jmax(Ef, QOLDINIT), B2);
  const T dtold = l.dt;
  const T dtn = l.dt * (T)__fdiv_rn(1.0f, q);
  l.dt = absmin(dtn, rest);
  const T told = l.t;
  l.t = tnext;
  if (l.nacc == 0) l.dt_first = (double)dtold;
  l.nacc += 1;
  acc_out.told = told;
  acc_out.dtold = dtold;
  return TRY_ACCEPTED;
}

/* Replace the state by the accepted proposal (and the FSAL stage). */
template <class M, class PR, int D, class F, int NK>
__device__ __forceinline__ void adaptive_commit(Lane<PR, D, F, NK>& l, const typename PR::R (&nh)[D],
                                                const typename PR::R (&nc)[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    l.uh[d] = nh[d];
    l.uc[d] = nc[d];
  }
  if (M::FSAL) {
#pragma unroll
    for (int d = 0; d < D; ++d) l.k[0][d] = l.k[NK - 1][d];
  }
}

/* One attempt with the saveat points of an accepted step interpolated at once
 * by this lane.  Returns true when the trajectory has finished (outputs written). */
template <class M, class PR, int D, class F, int NK>
__device__ __forceinline__ bool adaptive_iter(const KParams& P, Lane<PR, D, F, NK>& l, Totals& tot) {
  typedef typename PR::R R;
  typedef typename PR::T T;
  R nh[D], nc[D];
  Accepted<T> st;
  const int r = adaptive_try<M>(P, l, tot, nh, nc, st);
  if (r == TRY_STOPPED) return true;
  if (r == TRY_REJECTED) return false;
  const T told = st.told, dtold = st.dtold;
  T inv_dt = (T)0;
  if (l.cur < P.nsave && t_le<PR>(P.saveat[l.cur], l.t)) inv_dt = recip(dtold);
  while (l.cur < P.nsave && t_le<PR>(P.saveat[l.cur], l.t)) {
    const T theta = theta_of((T)P.saveat[l.cur], told, dtold, inv_dt);
    double v[D];
    M::dense(l.f, l.uh, l.uc, told, l.t, dtold, theta, l.k, v);
    store_point<PR, D>(P, l.idx, l.cur, v);
    l.cur += 1;
    l.ninterp += 1;
  }
  adaptive_commit<M>(l, nh, nc);
  store_step<PR, D>(P, l, l.nacc);
  if (!t_lt<PR>(l.t, P.tf)) { lane_finish(P, l, RET_DEFAULT, tot); return true; }
  return false;
}

/* Start trajectory idx; returns true if it is already finished (t0 >= tf). */
template <class M, class PR, int D, class F, int NK>
__device__ __forceinline__ bool adaptive_start(const KParams& P, long long idx, Lane<PR, D, F, NK>& l, Totals& tot) {
  lane_load(P, idx, l);
  if (!(l.t < (typename PR::T)P.tf)) { lane_finish(P, l, RET_DEFAULT, tot); return true; }
  if (M::FSAL) l.f(l.uh, l.t, l.k[0]);
  return false;
}

/* Plain schedule: thread i solves trajectory i from start to end. */
template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_adaptive_plain(const KParams& P) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Totals tot = {0, 0, 0};
  if (i < P.n) {
    Lane<PR, D, F, M::NK> l;
    if (!adaptive_start<M>(P, i, l, tot)) {
      while (!adaptive_iter<M>(P, l, tot)) {
      }
    }
  }
  flush_totals(P, tot);
}

/* Persistent schedule: resident warps loop over attempts; a lane whose
 * trajectory finished takes the next position from a device counter
 * (one atomicAdd per warp for all lanes that need work) and the position is
 * mapped through P.order.  Every lane of a warp runs the loop until the whole
 * warp has no work left, so the warp-wide ballots stay convergent. */
template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_adaptive_persistent(const KParams& P) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Lane<PR, D, F, M::NK> l;
  Totals tot = {0, 0, 0};
  bool active = false, exhausted = false;
  for (;;) {
    const bool want = !active && !exhausted;
    const unsigned need = __ballot_sync(FULL, want);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(P.counter, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (want) {
        const unsigned long long w = base + (unsigned long long)__popc(need & ((1u << lane) - 1u));
        if (w < (unsigned long long)P.n) {
          long long idx = P.order ? (long long)P.order[w] : (long long)w;
          if (!GBODE_CHECK(P, idx >= 0 && idx < P.n, CHK_ORDER)) idx = 0;
          active = !adaptive_start<M>(P, idx, l, tot);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (!__any_sync(FULL, !exhausted)) break;
      continue;
    }
    if (active && adaptive_iter<M>(P, l, tot)) active = false;
  }
  flush_totals(P, tot);
}

/* ------------------------------------------------------------------ staged dense output */
/* Persistent schedule with the saveat interpolation staged through shared
 * memory.  In the plain and persistent drivers a lane interpolates its saveat
 * points as soon as its step is accepted, and the other lanes of the warp
 * idle meanwhile (about one step in three has a save point, so nearly every
 * warp iteration pays for a full interpolation on a few lanes).  Here an
 * accepted step only appends a job per saveat point to a per-warp ring in
 * shared memory (a snapshot of what the interpolation reads: the state before
 * the step, the stage values, for Verner the parameters, t and dt); whenever 32
 * jobs are waiting the whole warp interpolates 32 points at once, one per
 * lane.  Each point is computed by the same M::dense call on the same values,
 * so the results are bit-identical to the other drivers. */
/* Launch shape: threads per block and the bytes of each warp's staging ring.
 * Both can be set at compile time (the autotuner compiles variants); the
 * defaults give 4 warps x 12 KB = 48 KB of static shared memory per block. */
#ifndef GBODE_BLOCK
#define GBODE_BLOCK 128
#endif
#ifndef GBODE_STAGE_BYTES
#define GBODE_STAGE_BYTES 12288
#endif
constexpr int kStageBytesPerWarp = GBODE_STAGE_BYTES;
constexpr int kWarpsPerBlock = GBODE_BLOCK / 32;

template <class M, class PR, int D, class F>
struct StageLayout {
  typedef typename PR::R R;
  typedef typename PR::T T;
  /* the parameters ride along only when the dense output evaluates f (Verner's extra stages) */
  enum { NREC = D * (PR::KAHAN ? 2 : 1) + M::NK * D + (M::DENSE_F ? F::NP : 0) };
  enum { JOB = 3 * (int)sizeof(T) + 8 + NREC * (int)sizeof(R) + 4 };
  enum { CAP = (kStageBytesPerWarp / JOB) & ~7 };
};

/* The stage values of one staged job as the dense formulas index them,
 * k[q][d], read where they are used from the ring's [row][CAP] layout (rows
 * STRIDE elements apart) instead of into registers first: a round then holds
 * one accumulator per component rather than every stage value of its job,
 * which for large states (Kuramoto-12: 84 stage values) is the difference
 * between spilling the lane's own state and not. */
template <class R, int STRIDE>
struct RingRow {
  const R* p;
  __device__ __forceinline__ R operator[](int d) const { return p[d * STRIDE]; }
};
template <class R, int D, int STRIDE>
struct RingStages {
  const R* p;
  __device__ __forceinline__ RingRow<R, STRIDE> operator[](int q) const {
    return RingRow<R, STRIDE>{p + q * D * STRIDE};
  }
};

template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_adaptive_staged(const KParams& P) {
  typedef typename PR::R R;
  typedef typename PR::T T;
  typedef StageLayout<M, PR, D, F> SL;
  enum { CAP = SL::CAP, NK = M::NK, KOFF = D * (PR::KAHAN ? 2 : 1), POFF = KOFF + NK * D };
  __shared__ __align__(16) unsigned char qmem[kWarpsPerBlock][kStageBytesPerWarp];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  unsigned char* qb = qmem[threadIdx.x >> 5];
  T* tv = (T*)qb;                                            /* told, tnew, dtold: [3][CAP] */
  long long* iv = (long long*)(qb + 3 * CAP * sizeof(T));    /* trajectory: [CAP] */
  R* rv = (R*)(qb + 3 * CAP * sizeof(T) + 8 * CAP);          /* record values: [NREC][CAP] */
  int* jv = (int*)(qb + 3 * CAP * sizeof(T) + 8 * CAP + SL::NREC * CAP * sizeof(R)); /* saveat index */
  int qhead = 0, qcount = 0; /* warp-uniform */

  Lane<PR, D, F, NK> l;
  Totals tot = {0, 0, 0};
  bool active = false, exhausted = false;

  /* interpolate the m oldest jobs, one per lane */
  auto round = [&](int m) {
    __syncwarp();
    if (lane < m) {
      const int slot = (qhead + lane) % CAP;
      R uh[D], uc[D];
      F f2;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        uh[d] = rv[d * CAP + slot];
        uc[d] = PR::KAHAN ? rv[(D + d) * CAP + slot] : (R)0;
      }
      const RingStages<R, D, CAP> kk{rv + KOFF * CAP + slot};
      if (M::DENSE_F) {
#pragma unroll
        for (int q = 0; q < F::NP; ++q) f2.p[q] = rv[(POFF + q) * CAP + slot];
      }
      double v[D];
      /* the abscissa is computed here, by all lanes of the round at once, rather
       * than by the few lanes that crossed a save point in their step */
      const T told = tv[slot], dtold = tv[2 * CAP + slot];
      const T theta = theta_of((T)P.saveat[jv[slot]], told, dtold, recip(dtold));
      M::dense(f2, uh, uc, told, tv[CAP + slot], dtold, theta, kk, v);
      store_point<PR, D>(P, iv[slot], jv[slot], v);
    }
    __syncwarp();
    qhead = (qhead + m) % CAP;
    qcount -= m;
  };

  for (;;) {
    const bool want = !active && !exhausted;
    const unsigned need = __ballot_sync(FULL, want);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(P.counter, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (want) {
        const unsigned long long w = base + (unsigned long long)__popc(need & ((1u << lane) - 1u));
        if (w < (unsigned long long)P.n) {
          long long idx = P.order ? (long long)P.order[w] : (long long)w;
          if (!GBODE_CHECK(P, idx >= 0 && idx < P.n, CHK_ORDER)) idx = 0;
          active = !adaptive_start<M>(P, idx, l, tot);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (!__any_sync(FULL, !exhausted)) break;
      continue;
    }
    R nh[D], nc[D];
    Accepted<T> st;
    int r = TRY_REJECTED, njobs = 0;
    if (active) {
      r = adaptive_try<M>(P, l, tot, nh, nc, st);
      if (r == TRY_STOPPED) active = false;
      if (r == TRY_ACCEPTED)
        while (l.cur + njobs < P.nsave && t_le<PR>(P.saveat[l.cur + njobs], l.t)) ++njobs;
    }
    /* slots for this iteration's jobs: exclusive prefix sum over the warp */
    int incl = njobs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int excl = incl - njobs;
    int space = CAP - qcount;
    if (total > space && qcount > 0) {
      /* this iteration's jobs do not all fit: interpolate the waiting ones
       * (fewer than 32) now, so that the new jobs go to the ring instead of
       * being interpolated in place by their lanes one after another */
      round(qcount < 32 ? qcount : 32);
      space = CAP - qcount;
    }
    if (njobs) {
      for (int q = 0; q < njobs; ++q) {
        const long long j = l.cur + q;
        if (excl + q < space) {
          const int slot = (qhead + qcount + excl + q) % CAP;
          tv[slot] = st.told;
          tv[CAP + slot] = l.t;
          tv[2 * CAP + slot] = st.dtold;
          iv[slot] = l.idx;
          jv[slot] = (int)j;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            rv[d * CAP + slot] = l.uh[d];
            if (PR::KAHAN) rv[(D + d) * CAP + slot] = l.uc[d];
          }
#pragma unroll
          for (int k = 0; k < NK; ++k)
#pragma unroll
            for (int d = 0; d < D; ++d) rv[(KOFF + k * D + d) * CAP + slot] = l.k[k][d];
          if (M::DENSE_F) {
#pragma unroll
            for (int k = 0; k < F::NP; ++k) rv[(POFF + k) * CAP + slot] = l.f.p[k];
          }
        } else {
          /* the ring is full: interpolate here */
          const T theta = theta_of((T)P.saveat[j], st.told, st.dtold, recip(st.dtold));
          double v[D];
          M::dense(l.f, l.uh, l.uc, st.told, l.t, st.dtold, theta, l.k, v);
          store_point<PR, D>(P, l.idx, j, v);
        }
      }
      l.cur += njobs;
      l.ninterp += njobs;
    }
    qcount += total < space ? total : space;
    (void)GBODE_CHECK(P, qcount >= 0 && qcount <= CAP, CHK_RING);
    if (r == TRY_ACCEPTED) {
      adaptive_commit<M>(l, nh, nc);
      store_step<PR, D>(P, l, l.nacc);
      if (!t_lt<PR>(l.t, P.tf)) {
        lane_finish(P, l, RET_DEFAULT, tot);
        active = false;
      }
    }
    while (qcount >= 32) round(32);
  }
  while (qcount > 0) round(qcount < 32 ? qcount : 32);
  flush_totals(P, tot);
}

/* ------------------------------------------------------------------ staged dense output, two queues */
/* For the methods whose dense output first evaluates extra stages (Verner 7
 * and 9, M::NX of them), those stages depend on the step and not on the save
 * point, and a step often holds two or three save points.  This driver keeps
 * two per-warp queues in shared memory: step records (what the extra stages
 * and the interpolation read, and room for the extra stages) and save points
 * (a record slot and a saveat index).  The warp computes the extra stages of
 * 32 records at a time, one per lane, then interpolates 32 save points at a
 * time from their records, so each step's extra stages are computed once
 * however many save points it holds.  The operations and their operands are
 * those of M::dense: results are bit-identical to the other drivers. */
template <class M, class PR, int D, class F>
struct StageLayout2 {
  typedef typename PR::R R;
  typedef typename PR::T T;
  enum { KOFF = D * (PR::KAHAN ? 2 : 1), POFF = KOFF + M::NK * D, XOFF = POFF + F::NP, NREC = XOFF + M::NX * D };
  /* bytes of a record (3 times, trajectory, point count, values) and of a point (record slot, saveat index) */
  enum { REC = 3 * (int)sizeof(T) + 8 + 4 + NREC * (int)sizeof(R), PT = 8 };
  /* room for twice as many points as records */
  enum { CR = (kStageBytesPerWarp / (REC + 2 * PT)) & ~7, CP = 2 * CR };
};

template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_adaptive_staged2(const KParams& P) {
  typedef typename PR::R R;
  typedef typename PR::T T;
  typedef StageLayout2<M, PR, D, F> SL;
  enum { CR = SL::CR, CP = SL::CP, NK = M::NK, NX = M::NX, KOFF = SL::KOFF, POFF = SL::POFF, XOFF = SL::XOFF,
         NREC = SL::NREC };
  __shared__ __align__(16) unsigned char qmem[kWarpsPerBlock][kStageBytesPerWarp];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  unsigned char* qb = qmem[threadIdx.x >> 5];
  T* tv = (T*)qb;                                                      /* told, tnew, dtold: [3][CR] */
  long long* iv = (long long*)(qb + 3 * CR * sizeof(T));               /* trajectory: [CR] */
  R* rv = (R*)(qb + 3 * CR * sizeof(T) + 8 * CR);                      /* record values: [NREC][CR] */
  int* nv = (int*)(qb + 3 * CR * sizeof(T) + 8 * CR + NREC * CR * sizeof(R)); /* save points of a record: [CR] */
  int* pv = nv + CR;                                                   /* record slot, saveat index: [2][CP] */
  /* warp-uniform queue state: records [rh, rh + rc), of which the first rs
   * have their extra stages; points [ph, ph + pc), of which the first pr
   * belong to such records; hd points of the head record done */
  int rh = 0, rc = 0, rs = 0, ph = 0, pc = 0, pr = 0, hd = 0;

  /* extra stages of the m oldest records without them, one per lane */
  auto stage_round = [&](int m) {
    __syncwarp();
    int np = 0;
    if (lane < m) {
      const int slot = (rh + rs + lane) % CR;
      R uh[D], uc[D];
      F f2;
#pragma unroll
      for (int d = 0; d < D; ++d) {
        uh[d] = rv[d * CR + slot];
        uc[d] = PR::KAHAN ? rv[(D + d) * CR + slot] : (R)0;
      }
#pragma unroll
      for (int q = 0; q < F::NP; ++q) f2.p[q] = rv[(POFF + q) * CR + slot];
      const RingStages<R, D, CR> kk{rv + KOFF * CR + slot};
      R x[NX][D];
      M::dense_stages(f2, uh, uc, tv[slot], tv[CR + slot], tv[2 * CR + slot], kk, x);
#pragma unroll
      for (int q = 0; q < NX; ++q)
#pragma unroll
        for (int d = 0; d < D; ++d) rv[(XOFF + q * D + d) * CR + slot] = x[q][d];
      np = nv[slot];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) np += __shfl_xor_sync(FULL, np, o);
    __syncwarp();
    rs += m;
    pr += np;
  };

  /* interpolate the m oldest points (their records have the extra stages), one per lane */
  auto point_round = [&](int m) {
    __syncwarp();
    if (lane < m) {
      const int ps = (ph + lane) % CP;
      int slot = pv[ps];
      const int j = pv[CP + ps];
      if (!GBODE_CHECK(P, slot >= 0 && slot < CR, CHK_RING)) slot = 0;
      R uh[D], uc[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        uh[d] = rv[d * CR + slot];
        uc[d] = PR::KAHAN ? rv[(D + d) * CR + slot] : (R)0;
      }
      const T told = tv[slot], dtold = tv[2 * CR + slot];
      const T theta = theta_of((T)P.saveat[j], told, dtold, recip(dtold));
      const RingStages<R, D, CR> kk{rv + KOFF * CR + slot};
      const RingStages<R, D, CR> xx{rv + XOFF * CR + slot};
      double v[D];
      M::dense_eval(uh, uc, dtold, theta, kk, xx, v);
      store_point<PR, D>(P, iv[slot], j, v);
    }
    __syncwarp();
    ph = (ph + m) % CP;
    pc -= m;
    pr -= m;
    hd += m;
    /* records whose points are all done leave the queue, oldest first */
    while (rs > 0 && hd >= nv[rh]) {
      hd -= nv[rh];
      rh = (rh + 1) % CR;
      --rc;
      --rs;
    }
  };

  Lane<PR, D, F, NK> l;
  Totals tot = {0, 0, 0};
  bool active = false, exhausted = false;
  for (;;) {
    const bool want = !active && !exhausted;
    const unsigned need = __ballot_sync(FULL, want);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(P.counter, (unsigned long long)__popc(need));
      base = __shfl_sync(FULL, base, leader);
      if (want) {
        const unsigned long long w = base + (unsigned long long)__popc(need & ((1u << lane) - 1u));
        if (w < (unsigned long long)P.n) {
          long long idx = P.order ? (long long)P.order[w] : (long long)w;
          if (!GBODE_CHECK(P, idx >= 0 && idx < P.n, CHK_ORDER)) idx = 0;
          active = !adaptive_start<M>(P, idx, l, tot);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, active)) {
      if (!__any_sync(FULL, !exhausted)) break;
      continue;
    }
    R nh[D], nc[D];
    Accepted<T> st;
    int r = TRY_REJECTED, njobs = 0;
    if (active) {
      r = adaptive_try<M>(P, l, tot, nh, nc, st);
      if (r == TRY_STOPPED) active = false;
      if (r == TRY_ACCEPTED)
        while (l.cur + njobs < P.nsave && t_le<PR>(P.saveat[l.cur + njobs], l.t)) ++njobs;
    }
    /* a record per lane with save points, and its points: ranks over the warp */
    const unsigned hb = __ballot_sync(FULL, njobs > 0);
    const int nrec = __popc(hb), rrank = __popc(hb & ((1u << lane) - 1u));
    int incl = njobs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += v;
    }
    const int total = __shfl_sync(FULL, incl, 31);
    const int excl = incl - njobs;
    if (nrec > 0) {
      /* make room: extra stages for the records waiting for them, then every
       * ready point, until this iteration's records and points fit */
      while ((rc + nrec > CR || pc + total > CP) && rc > 0) {
        if (rc - rs > 0) stage_round(rc - rs < 32 ? rc - rs : 32);
        while (pr > 0) point_round(pr < 32 ? pr : 32);
      }
      if (total <= CP) {
        if (njobs) {
          const int slot = (rh + rc + rrank) % CR;
          tv[slot] = st.told;
          tv[CR + slot] = l.t;
          tv[2 * CR + slot] = st.dtold;
          iv[slot] = l.idx;
          nv[slot] = njobs;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            rv[d * CR + slot] = l.uh[d];
            if (PR::KAHAN) rv[(D + d) * CR + slot] = l.uc[d];
          }
#pragma unroll
          for (int k = 0; k < NK; ++k)
#pragma unroll
            for (int d = 0; d < D; ++d) rv[(KOFF + k * D + d) * CR + slot] = l.k[k][d];
#pragma unroll
          for (int k = 0; k < F::NP; ++k) rv[(POFF + k) * CR + slot] = l.f.p[k];
          for (int q = 0; q < njobs; ++q) {
            const int ps = (ph + pc + excl + q) % CP;
            pv[ps] = slot;
            pv[CP + ps] = l.cur + q;
          }
        }
        rc += nrec;
        pc += total;
      } else if (njobs) {
        /* more save points in one iteration than the point queue holds: interpolate here */
        for (int q = 0; q < njobs; ++q) {
          const long long j = l.cur + q;
          const T theta = theta_of((T)P.saveat[j], st.told, st.dtold, recip(st.dtold));
          double v[D];
          M::dense(l.f, l.uh, l.uc, st.told, l.t, st.dtold, theta, l.k, v);
          store_point<PR, D>(P, l.idx, j, v);
        }
      }
      if (njobs) {
        l.cur += njobs;
        l.ninterp += njobs;
      }
    }
    (void)GBODE_CHECK(P, rc >= 0 && rc <= CR && pc >= 0 && pc <= CP && rs <= rc && pr <= pc, CHK_RING);
    if (r == TRY_ACCEPTED) {
      adaptive_commit<M>(l, nh, nc);
      store_step<PR, D>(P, l, l.nacc);
      if (!t_lt<PR>(l.t, P.tf)) {
        lane_finish(P, l, RET_DEFAULT, tot);
        active = false;
      }
    }
    while (rc - rs >= 32) stage_round(32);
    while (pr >= 32) point_round(32);
  }
  while (rc - rs > 0) stage_round(rc - rs < 32 ? rc - rs : 32);
  while (pr > 0) point_round(pr < 32 ? pr : 32);
  flush_totals(P, tot);
}

/* Staged when a full round of jobs fits the ring, the unstaged persistent
 * driver otherwise (large states: Verner 9 with dim 4, Kuramoto-12). */
template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_adaptive_staged_or_persistent(const KParams& P) {
  if constexpr (M::DENSE_F) {
    /* dense output with extra stages: the two-queue form shares them between a step's save points */
    if constexpr (StageLayout2<M, PR, D, F>::CR >= 32) {
      if (P.nsave > 0) {
        run_adaptive_staged2<M, PR, D, F>(P);
        return;
      }
    }
  }
  if constexpr (StageLayout<M, PR, D, F>::CAP >= 32) {
    if (P.nsave > 0) {
      run_adaptive_staged<M, PR, D, F>(P);
      return;
    }
  }
  run_adaptive_persistent<M, PR, D, F>(P);
}

/* ------------------------------------------------------------------ fixed-step Tsit5, components over warps */
/* Small fixed-step ensembles.  Every SM sub-partition issues one FP64 warp
 * instruction per 64 cycles whatever the number of active lanes, so an
 * ensemble of fewer warps than the GPU has sub-partitions leaves most of them
 * idle (8,192 trajectories are 256 warps for 608 sub-partitions).  Here a
 * block of D warps solves 32 trajectories: lane l of warp c holds component c
 * of trajectory 32 * blockIdx.x + l and computes that component's stage
 * combinations and right-hand side; the stage inputs are exchanged through
 * shared memory (double-buffered, one barrier per exchange).  The right-hand
 * side functor is inlined with the component fixed at compile time, so the
 * other components' arithmetic is dead code.  Per component these are the
 * operations of MTsit5::attempt (without the error estimate) and run_fixed,
 * in the same order: results are bit-identical.  Final states and
 * save_everystep output only (no saveat dense output). */
template <class PR, int D, class F>
struct FixedSplitTsit5 {
  typedef typename PR::R R;
  typedef typename PR::T T;

  /* all D components of the stage input of the 32 trajectories: each warp
   * writes its own, then reads all of them.  The warps run different
   * instantiations of run<C>, so they meet at the barrier from different
   * instructions: the non-aligned barrier.sync over the block's 32 * D
   * threads (every lane of every warp arrives, the same number of times). */
  __device__ static __forceinline__ void exchange(R (*xb)[D][32], int& b, int c, int lane, R mine, R (&full)[D]) {
    xb[b][c][lane] = mine;
    asm volatile("barrier.sync 1, %0;" ::"r"(32 * D) : "memory");
#pragma unroll
    for (int d = 0; d < D; ++d) full[d] = xb[b][d][lane];
    b ^= 1;
  }

  template <int C>
  __device__ static __forceinline__ R rhs(const F& f, const R (&u)[D], T t) {
    R du[D];
    f(u, t, du);
    return du[C];
  }

  template <int C>
  __device__ static __forceinline__ void run(const KParams& P, R (*xb)[D][32]) {
#define C5(x) CB<R>::t5(tsit5_##x)
#define C5T(x) CB<T>::t5(tsit5_##x)
    const int lane = threadIdx.x & 31;
    const long long i = (long long)blockIdx.x * 32 + lane;
    const bool valid = i < P.n;
    long long idx = valid ? i : 0;  /* lanes past n compute on trajectory 0 and store nothing */
    if (!GBODE_CHECK(P, idx >= 0 && idx < P.n, CHK_TRAJ)) idx = 0;
#ifdef GBODE_BOUNDS_CHECK
    if (C == 0 && valid) atomicAdd(&P.visited[idx], 1u);  /* one start per trajectory, counted by warp 0 */
#endif
    F f;
#pragma unroll
    for (int j = 0; j < F::NP; ++j) f.p[j] = (R)P.p[(long long)j * P.n + idx];
    rhs_loaded(f);
    R uh[1] = {(R)P.u0[(long long)C * P.n + idx]}, uc[1] = {(R)0};
    T t = (T)P.t0;
    const T dt = (T)P.dt;
    const bool every = P.nsave == 0 && P.save_everystep && P.us;
    auto value = [&]() { return PR::KAHAN ? (double)uh[0] - (double)uc[0] : (double)uh[0]; };
    if (every && valid && GBODE_CHECK(P, i < P.n && P.ngrid > 0, CHK_SAVE)) *us_at(P, 0, C, i) = value();
    int b = 0;
    R full[D], k[7][1];
    exchange(xb, b, C, lane, uh[0], full);
    k[0][0] = rhs<C>(f, full, t);
    const R h0 = (R)dt;
    for (long long g = 1; g < P.ngrid; ++g) {
      t = (T)P.grid[g - 1];
      const R h = h0;
      const R a = (R)(dt * C5T(a21));
      R tmp[1], sv[1], nh[1], nc[1];
      tmp[0] = fmaR(a, k[0][0], uh[0]);
      exchange(xb, b, C, lane, tmp[0], full);
      k[1][0] = rhs<C>(f, full, stime(t, C5T(c1), dt));
      lc(sv, C5(a31), k[0], C5(a32), k[1]);
      axpy(tmp, uh, h, sv);
      exchange(xb, b, C, lane, tmp[0], full);
      k[2][0] = rhs<C>(f, full, stime(t, C5T(c2), dt));
      lc(sv, C5(a41), k[0], C5(a42), k[1], C5(a43), k[2]);
      axpy(tmp, uh, h, sv);
      exchange(xb, b, C, lane, tmp[0], full);
      k[3][0] = rhs<C>(f, full, stime(t, C5T(c3), dt));
      lc(sv, C5(a51), k[0], C5(a52), k[1], C5(a53), k[2], C5(a54), k[3]);
      axpy(tmp, uh, h, sv);
      exchange(xb, b, C, lane, tmp[0], full);
      k[4][0] = rhs<C>(f, full, stime(t, C5T(c4), dt));
      lc(sv, C5(a61), k[0], C5(a62), k[1], C5(a63), k[2], C5(a64), k[3], C5(a65), k[4]);
      axpy(tmp, uh, h, sv);
      exchange(xb, b, C, lane, tmp[0], full);
      k[5][0] = rhs<C>(f, full, t + dt);
      lc(sv, C5(a71), k[0], C5(a72), k[1], C5(a73), k[2], C5(a74), k[3], C5(a75), k[4], C5(a76), k[5]);
      state_update<PR, 1>(uh, uc, h, sv, nh, nc);
      exchange(xb, b, C, lane, nh[0], full);
      k[6][0] = rhs<C>(f, full, t + dt);
      t = t + dt;
      uh[0] = nh[0];
      uc[0] = nc[0];
      if (every && valid && GBODE_CHECK(P, i < P.n && g < P.ngrid, CHK_SAVE)) *us_at(P, g, C, i) = value();
      k[0][0] = k[6][0];
    }
#undef C5
#undef C5T
    const int nacc = P.ngrid > 0 ? (int)(P.ngrid - 1) : 0;
    if (valid && P.u_final && GBODE_CHECK(P, i < P.n, CHK_TRAJ)) P.u_final[(long long)C * P.n + i] = value();
    if (C == 0) {
      Totals tot = {0, 0, 0};
      if (valid && GBODE_CHECK(P, i < P.n, CHK_TRAJ)) {
        if (P.t_final) P.t_final[i] = (double)t;
        if (P.retcode) P.retcode[i] = (signed char)RET_DEFAULT;
        if (P.naccept) P.naccept[i] = nacc;
        if (P.nreject) P.nreject[i] = 0;
        if (P.dt_first) P.dt_first[i] = nacc > 0 ? (double)dt : __longlong_as_double(0x7ff8000000000000LL);
        tot.att = (unsigned long long)nacc;
      }
      flush_totals(P, tot);
    }
  }

  /* the warp's component as a compile-time constant */
  template <int C>
  __device__ static __forceinline__ void dispatch(const KParams& P, R (*xb)[D][32], int w) {
    if constexpr (C < D) {
      if (w == C) run<C>(P, xb);
      else dispatch<C + 1>(P, xb, w);
    }
  }
};

template <class PR, int D, class F>
__device__ __forceinline__ void run_fixed_split(const KParams& P) {
  typedef typename PR::R R;
  __shared__ R xb[2][D][32];
  FixedSplitTsit5<PR, D, F>::template dispatch<0>(P, xb, (int)(threadIdx.x >> 5));
}

/* Fixed-step methods: thread i, the grid of Julia's t0:dt:tf shared by all. */
template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_fixed(const KParams& P) {
  typedef typename PR::R R;
  typedef typename PR::T T;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Totals tot = {0, 0, 0};
  if (i < P.n) {
  Lane<PR, D, F, M::NK> l;
  lane_load(P, i, l);
  const T dt = (T)P.dt;
  const bool every = P.nsave == 0 && P.save_everystep;
  if (every) {
    double v[D];
    state_value<PR, D>(l, v);
    store_point<PR, D>(P, i, 0, v);
  }
  if (M::FSAL) l.f(l.uh, l.t, l.k[0]);
  R nh[D], nc[D], e[D];
  for (long long g = 1; g < P.ngrid; ++g) {
    l.t = (T)P.grid[g - 1];
    M::attempt(l.f, l.uh, l.uc, l.t, dt, l.k, nh, nc, e, false);
    l.t = l.t + dt;
    while (l.cur < P.nsave && t_le<PR>(P.saveat[l.cur], l.t)) {
      const T theta = ((T)P.saveat[l.cur] - (l.t - dt)) / dt;
      double v[D];
      M::dense(l.f, l.uh, l.uc, l.t - dt, l.t, dt, theta, l.k, v);
      store_point<PR, D>(P, i, l.cur, v);
      l.cur += 1;
      l.ninterp += 1;
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      l.uh[d] = nh[d];
      l.uc[d] = nc[d];
    }
    if (every) {
      double v[D];
      state_value<PR, D>(l, v);
      store_point<PR, D>(P, i, g, v);
    }
    if (M::FSAL) {
#pragma unroll
      for (int d = 0; d < D; ++d) l.k[0][d] = l.k[M::NK - 1][d];
    }
  }
  l.nacc = P.ngrid > 0 ? (int)(P.ngrid - 1) : 0;
  l.att = l.nacc;
  if (l.nacc > 0) l.dt_first = (double)dt;
  lane_finish(P, l, RET_DEFAULT, tot);
  }
  flush_totals(P, tot);
}

/* GPUSimpleRK4 and GPUSimpleEuler (M = MRK4 or MEuler): one step per grid
 * point, every grid point saved when asked (us[1] = u0). */
template <class M, class PR, int D, class F>
__device__ __forceinline__ void run_onestep(const KParams& P) {
  typedef typename PR::R R;
  typedef typename PR::T T;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  Totals tot = {0, 0, 0};
  if (i < P.n) {
  Lane<PR, D, F, 1> l;
  lane_load(P, i, l);
  l.cur = 0;
  const T dt = (T)P.dt;
  const bool every = P.save_everystep != 0;
  if (every) {
    double v[D];
    state_value<PR, D>(l, v);
    store_point<PR, D>(P, i, 0, v);
  }
  R nh[D], nc[D];
  for (long long g = 1; g < P.ngrid; ++g) {
    l.t = (T)P.grid[g];
    M::step(l.f, l.uh, l.uc, l.t, dt, nh, nc);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      l.uh[d] = nh[d];
      l.uc[d] = nc[d];
    }
    if (every) {
      double v[D];
      state_value<PR, D>(l, v);
      store_point<PR, D>(P, i, g, v);
    }
  }
  l.nacc = P.ngrid > 0 ? (int)(P.ngrid - 1) : 0;
  l.att = l.nacc;
  if (l.nacc > 0) l.dt_first = (double)dt;
  lane_finish(P, l, RET_DEFAULT, tot);
  }
  flush_totals(P, tot);
}

}  // namespace gbode

/* Entry-point generator: GBODE_ENTRY(name, kind, Method, Prec, Rhs) defines
 * extern "C" __global__ name(KParams).  kind: plain | persistent | staged | fixed | onestep. */
#define GBODE_ENTRY_plain(NAME, M, PR, RHS)                                                  \
  extern "C" __global__ void __launch_bounds__(GBODE_BLOCK) NAME(gbode::KParams P) {                \
    gbode::run_adaptive_plain<M<PR, RHS::D, RHS>, PR, RHS::D, RHS>(P);                      \
  }
#define GBODE_ENTRY_persistent(NAME, M, PR, RHS)                                             \
  extern "C" __global__ void __launch_bounds__(GBODE_BLOCK) NAME(gbode::KParams P) {                \
    gbode::run_adaptive_persistent<M<PR, RHS::D, RHS>, PR, RHS::D, RHS>(P);                 \
  }
#define GBODE_ENTRY_staged(NAME, M, PR, RHS)                                                 \
  extern "C" __global__ void __launch_bounds__(GBODE_BLOCK) NAME(gbode::KParams P) {                \
    gbode::run_adaptive_staged_or_persistent<M<PR, RHS::D, RHS>, PR, RHS::D, RHS>(P);       \
  }
#define GBODE_ENTRY_fixed(NAME, M, PR, RHS)                                                  \
  extern "C" __global__ void __launch_bounds__(GBODE_BLOCK) NAME(gbode::KParams P) {                \
    gbode::run_fixed<M<PR, RHS::D, RHS>, PR, RHS::D, RHS>(P);                               \
  }
/* fixed-step Tsit5 with a trajectory's components over the warps of a block (32 * D threads) */
#define GBODE_ENTRY_fixedsplit(NAME, M, PR, RHS)                                             \
  extern "C" __global__ void __launch_bounds__(32 * RHS::D) NAME(gbode::KParams P) {              \
    gbode::run_fixed_split<PR, RHS::D, RHS>(P);                                             \
  }
#define GBODE_ENTRY_onestep(NAME, M, PR, RHS)                                                \
  extern "C" __global__ void __launch_bounds__(GBODE_BLOCK) NAME(gbode::KParams P) {                \
    gbode::run_onestep<M<PR, RHS::D, RHS>, PR, RHS::D, RHS>(P);                              \
  }
#define GBODE_ENTRY(NAME, KIND, M, PR, RHS) GBODE_ENTRY_##KIND(NAME, M, PR, RHS)
