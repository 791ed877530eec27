/* Deterministic single-precision power x^b for the step-size controller.
 *
 * TEST INFRASTRUCTURE COPY: the oracle's own implementation of the controller
 * power used by the device rounding canon.  It is written independently of
 * the kernels' copy (ctrl_pow in simplediffeq.jl_gb300/csrc/ode_solver.cuh); the two must
 * agree bit for bit, which the parity tests check through whole solves.
 *
 * Method (textbook, no vendor code): x = m * 2^e with m in [sqrt(1/2), sqrt(2));
 * log2(m) = (2/ln 2) * atanh(s), s = (m-1)/(m+1), from the odd series
 * s + s^3/3 + ... + s^11/11 (|s| <= 0.1716, truncation < 1e-10);
 * 2^y = 2^n * exp(f ln 2), n = round(y), |f| <= 1/2, from the Taylor series of
 * exp to degree 8 (truncation < 3e-10).  Every step is an IEEE single
 * operation or an explicit fmaf, so any IEEE-754 machine gives the same bits.
 * Relative error below 2e-6 over the whole float range, far more accuracy
 * than a step-size factor needs.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace oracle_pow {

static inline uint32_t f2u(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
static inline float u2f(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }

/* log2(x) for finite x > 0, including subnormals. */
static inline float log2_pos(float x) {
  int e = 0;
  if (x < 1.17549435e-38f) { x = x * 16777216.0f; e = -24; }  /* scale subnormals by 2^24 */
  uint32_t u = f2u(x);
  e += (int)((u >> 23) & 0xff) - 127;
  float m = u2f((u & 0x007fffffu) | 0x3f800000u);            /* m in [1, 2) */
  if (m > 1.41421354f) { m = m * 0.5f; e += 1; }              /* m in (0.7071, 1.4142] */
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float poly = std::fmaf(s2, 0.0909090936f, 0.111111112f);    /* 1/11, 1/9 */
  poly = std::fmaf(s2, poly, 0.142857149f);                    /* 1/7 */
  poly = std::fmaf(s2, poly, 0.200000003f);                    /* 1/5 */
  poly = std::fmaf(s2, poly, 0.333333343f);                    /* 1/3 */
  poly = std::fmaf(s2, poly, 1.0f);
  float atanh_s = s * poly;
  return std::fmaf(atanh_s, 2.88539004f, (float)e);            /* 2/ln 2 */
}

/* 2^y for finite y. */
static inline float exp2_fin(float y) {
  if (y > 128.0f) return INFINITY;
  if (y < -150.0f) return 0.0f;
  float n = std::nearbyintf(y);
  float f = y - n;                                             /* exact, |f| <= 1/2 */
  float z = f * 0.693147182f;                                  /* ln 2 */
  float p = std::fmaf(z, 2.48015876e-05f, 1.98412701e-04f);   /* 1/8!, 1/7! */
  p = std::fmaf(z, p, 1.38888892e-03f);                        /* 1/6! */
  p = std::fmaf(z, p, 8.33333377e-03f);                        /* 1/5! */
  p = std::fmaf(z, p, 4.16666679e-02f);                        /* 1/4! */
  p = std::fmaf(z, p, 0.166666672f);                           /* 1/3! */
  p = std::fmaf(z, p, 0.5f);
  p = std::fmaf(z, p, 1.0f);
  p = std::fmaf(z, p, 1.0f);
  int ni = (int)n;
  /* scale by 2^ni in two halves so that neither factor overflows or underflows */
  int h = ni / 2;
  float s1 = u2f((uint32_t)(h + 127) << 23);
  float s2 = u2f((uint32_t)(ni - h + 127) << 23);
  return (p * s1) * s2;
}

/* x^b for x >= 0 (or NaN); b is a small positive exponent. */
static inline float ctrl_pow(float x, float b) {
  if (x != x) return x;
  if (x == 0.0f) return 0.0f;
  if (x == INFINITY) return INFINITY;
  return exp2_fin(b * log2_pos(x));
}

}  // namespace oracle_pow
