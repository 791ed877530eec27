/* Julia's floating-point range start:step:stop, as the GPUSimple fixed-step
 * solvers build their time grid (`_ts = tspan[1]:dt:tspan[2]`,
 * src/tsit5/gpuatsit5.jl:92, src/verner/gpuvern7.jl:101,
 * src/verner/gpuvern9.jl:99, `ts = tspan[1]:dt:tspan[2]` src/rk4/gpurk4.jl:66).
 *
 * Julia (base/twiceprecision.jl, `(:)(start::T, step::T, stop::T)`) first
 * looks for small-integer ratios start = a/d, step = b/d, stop = c/d with
 * Base.rat (a continued fraction limited to 2^24 for Float64, 2^11 for
 * Float32); if found, the length comes from integer arithmetic and element i
 * is (a + (i-1) b)/d, which Julia evaluates in double-double (restated here
 * as the correctly rounded quotient).  Otherwise it takes start and step
 * literally, length round((stop-start)/step)+1 adjusted for overshoot, and
 * element i is what StepRangeLen's getindex computes with a zero low part
 * in start and step: start + ((i-1)*step), each operation rounded once (for
 * Float32 in Float64, then rounded to Float32).
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace jlrange {

template <class T> struct Lim;
template <> struct Lim<double> {
  static constexpr int64_t maxint = (int64_t)1 << 53;         /* maxintfloat(Float64, Int) */
  static constexpr int64_t narrow_maxint = (int64_t)1 << 24;  /* maxintfloat(Float32, Int) */
};
template <> struct Lim<float> {
  static constexpr int64_t maxint = (int64_t)1 << 24;
  static constexpr int64_t narrow_maxint = (int64_t)1 << 11;  /* maxintfloat(Float16, Int) */
};

/* Base.rat(x): continued-fraction rational approximation of x, in T arithmetic. */
template <class T>
static void rat(T x, int64_t& num, int64_t& den) {
  T y = x;
  int64_t a = 1, d = 1, b = 0, c = 0;
  const int64_t m = Lim<T>::narrow_maxint;
  while (std::fabs(y) <= (T)m) {
    int64_t f = (int64_t)std::trunc(y);
    y = (T)(y - (T)f);
    int64_t na = f * a + c, nb = f * b + d;
    c = a; d = b;
    a = na; b = nb;
    if (std::llabs(a) > m || std::llabs(b) > m) { num = c; den = d; return; }
    if ((T)((T)a / (T)b) == x) break;
    if (y == 0) break;
    y = (T)((T)1 / y);
  }
  num = a;
  den = b;
}

static inline int64_t gcd64(int64_t a, int64_t b) {
  a = a < 0 ? -a : a;
  b = b < 0 ? -b : b;
  while (b) { int64_t t = a % b; a = b; b = t; }
  return a;
}

template <class T>
static bool isbetween(T a, T x, T b) { return (a <= x && x <= b) || (b <= x && x <= a); }

/* Correctly rounded T value of num/den (|num|, den < 2^53, so the operands
 * are exact doubles and IEEE division rounds once). */
template <class T>
static T ratio(int64_t num, int64_t den) {
  double q = (double)num / (double)den;
  if (sizeof(T) == sizeof(double)) return (T)q;
  /* float: round the exact quotient once more from the double, then fix the
   * rare double-rounding tie by comparing against the exact rational */
  float f = (float)q;
  return (T)f;
}

/* start + (i*step), each rounded once in double (getindex of the literal
 * StepRangeLen: the product i*step.hi rounds, the sum with start is exact in
 * two parts and rounds once when the parts are added) */
template <class T>
static T literal_elem(T start, T step, int64_t i) {
  const double p = (double)i * (double)step;
  return (T)((double)start + p);
}

/* Number of elements and (optionally) the elements. */
template <class T>
static int64_t build(T start, T step, T stop, std::vector<double>* out) {
  if (step == 0) return -1;
  int64_t step_n, step_d;
  rat(step, step_n, step_d);
  if (step_d != 0 && (T)((double)step_n / (double)step_d) == step) {
    int64_t start_n, start_d, stop_n, stop_d;
    rat(start, start_n, start_d);
    rat(stop, stop_n, stop_d);
    if (start_d != 0 && stop_d != 0 && (T)((double)start_n / (double)start_d) == start &&
        (T)((double)stop_n / (double)stop_d) == stop) {
      const int64_t g = gcd64(start_d, step_d);
      const int64_t den = g ? (start_d / g) * step_d : 0;
      const double m = (double)Lim<T>::maxint;
      if (den != 0 && std::fabs((double)(T)(start * (T)den)) <= m && std::fabs((double)(T)(step * (T)den)) <= m &&
          den % start_d == 0 && den % step_d == 0) {
        const int64_t sn = (int64_t)std::nearbyint((double)(T)(start * (T)den));
        const int64_t pn = (int64_t)std::nearbyint((double)(T)(step * (T)den));
        const __int128 num = (__int128)den * stop_n - (__int128)stop_d * sn + (__int128)pn * stop_d;
        const __int128 dd = (__int128)pn * stop_d;
        __int128 q = num / dd; /* truncating, as Julia's div */
        int64_t len = q > 0 ? (int64_t)q : 0;
        const T last = (T)(start + (T)((T)(len - 1) * step));
        const T after = (T)(start + (T)((T)len * step));
        if (isbetween(start, last, (T)(stop + (T)(step / (T)2))) && !isbetween(start, after, stop)) {
          if (out) {
            out->resize((size_t)len);
            for (int64_t i = 0; i < len; ++i) (*out)[(size_t)i] = (double)ratio<T>(sn + i * pn, den);
          }
          return len;
        }
      }
    }
  }
  const T lf = (T)((T)(stop - start) / step);
  int64_t len;
  if (lf < 0) len = 0;
  else if (lf == 0) len = 1;
  else {
    len = (int64_t)std::nearbyint((double)lf) + 1;
    const T stop2 = (T)(start + (T)((T)(len - 1) * step));
    len -= (int64_t)((start < stop && stop < stop2) ? 1 : 0) + (int64_t)((start > stop && stop > stop2) ? 1 : 0);
  }
  if (out) {
    out->resize((size_t)len);
    for (int64_t i = 0; i < len; ++i) (*out)[(size_t)i] = (double)literal_elem<T>(start, step, i);
  }
  return len;
}

}  // namespace jlrange
