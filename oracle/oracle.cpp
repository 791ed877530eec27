/* CPU oracle: a plain C++ restatement of the reference's per-trajectory solvers.
 *
 * TEST INFRASTRUCTURE — used only by tests/ and by the CPU-baseline leg of
 * bench.py.  The product library never links or calls this file.
 *
 * What is restated (paths inside SimpleDiffEq.jl):
 *   GPUSimpleTsit5 / GPUSimpleATsit5   src/tsit5/gpuatsit5.jl:55-147, :205-336
 *   GPUSimpleVern7 / GPUSimpleAVern7   src/verner/gpuvern7.jl:55-242, :300-536
 *   GPUSimpleVern9 / GPUSimpleAVern9   src/verner/gpuvern9.jl:55-353, :411-779
 *   GPUSimpleRK4                       src/rk4/gpurk4.jl:53-98
 *   GPUSimpleEuler                     src/euler/gpueuler.jl:53-90
 *   SimpleEM (SDE, diagonal noise)     src/euler_maruyama.jl:48-98
 *   SimpleATsit5 (integrator form)     src/tsit5/atsit5.jl:117-179, :322-413, :705-732
 *   SimpleTsit5 (integrator form)      src/tsit5/tsit5.jl:84-122, :303-352, :358-399
 *   PI controller constants            src/SimpleDiffEq.jl:67-77, src/tsit5/atsit5.jl:57-62
 *   error norm ODE_DEFAULT_NORM        DiffEqBase (not vendored): sqrt(sum(abs2, e) / length(e))
 * Coefficients come from tableaus.h, extracted verbatim from
 * src/tsit5/atsit5_cache.jl and src/verner/verner_tableaus.jl.
 *
 * Two rounding modes (oracle_round):
 *   REF     what the Julia code rounds: @muladd on SVector arithmetic falls back
 *           to a separate multiply and add, scalar muladd (stage times, Horner
 *           steps of @evalpoly) fuses, the controller uses libm pow and the
 *           Kuramoto functions libm sin/cos, or with ctrl == 3 the correctly
 *           rounded cr_pow and cr_sincos of the kernels' reference-arithmetic
 *           mode (ODE_CTRL_REF).
 *   DEVICE  the device rounding canon the CUDA kernels implement: every
 *           multiply-add of the reference's expressions is one fused
 *           multiply-add (linear combinations accumulate left to right in
 *           both modes, see Alg::lc); the error norm (when abstol >= 1e-30)
 *           and the step-size factor q are computed in single precision, q
 *           with ctrl_pow.h; the dense-output abscissa uses recip_dev and a
 *           shared theta^2 (horner).
 * Build with -ffp-contract=off so that no other multiply-add is fused.
 *
 * Documented deviations from the reference, shared with the device path:
 *   * "dt<dtmin" ends the trajectory with retcode 1 instead of throwing;
 *   * an optional attempt cap (maxiters) ends it with retcode 2;
 *   * a NaN error estimate is accepted exactly as the reference does
 *     (NaN > 1 is false) and the trajectory finishes; retcode 3 flags it;
 *   * saveat points never reached are NaN instead of uninitialised memory.
 */
#include "oracle.h"
#include "ctrl_pow.h"
#include "../simplediffeq.jl_gb300/csrc/tableaus.h"
#include "../simplediffeq.jl_gb300/csrc/log_table.h"
#include "../simplediffeq.jl_gb300/csrc/exp_table.h"
#include "../simplediffeq.jl_gb300/csrc/ds_table.h"
#include "../simplediffeq.jl_gb300/csrc/crpow.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr int MAXD = 16;
constexpr int MAXP = 32;
constexpr int MAXK = 26;

enum { RET_DEFAULT = 0, RET_DTMIN = 1, RET_MAXITERS = 2, RET_NAN = 3 };

/* ---------------------------------------------------------------- policy */
/* R: type of stage arithmetic and state; T: type of t and dt; KAHAN: the state
 * update is a compensated sum (u = hi - c); DEV: device rounding canon. */
template <class R_, class T_, bool KAHAN_, bool DEV_>
struct Pol {
  typedef R_ R;
  typedef T_ T;
  static constexpr bool KAHAN = KAHAN_;
  static constexpr bool DEV = DEV_;
};

template <class X>
static inline X fmaX(X a, X b, X c) { return std::fma(a, b, c); }

/* a*b+c of a vector expression: fused in the device canon, two roundings in
 * the reference (the generic muladd fallback for SVector). */
template <bool DEV, class X>
static inline X vmadd(X a, X b, X c) {
  if (DEV) return fmaX(a, b, c);
  return a * b + c;
}

/* Julia's non-fastmath min/max propagate NaN. */
template <class X> static inline X jmin(X a, X b) {
  if (a != a || b != b) return (X)NAN;
  return b < a ? b : a;
}
template <class X> static inline X jmax(X a, X b) {
  if (a != a || b != b) return (X)NAN;
  return b > a ? b : a;
}
/* @fastmath min/max: plain compare-and-select (Base.FastMath min_fast/max_fast). */
template <class X> static inline X fmin_(X x, X y) { return (y > x) ? x : y; }
template <class X> static inline X fmax_(X x, X y) { return (y > x) ? y : x; }

/* Sine and cosine in the device canon (double precision): Cody-Waite
 * reduction modulo pi/2 (Cody & Waite, Software Manual for the Elementary
 * Functions, 1980) in fused form, r = fma(-k, C2, fma(-k, C1, x)) with C1 the
 * double nearest pi/2 and C2 the double nearest pi/2 - C1; k is x * 2/pi
 * rounded to the nearest integer by adding 1.5 * 2^52 in one fused
 * multiply-add (the quadrant k mod 4 is then the low bits of that sum);
 * sin r = r + r^3 P(r^2), cos r = 1 + r^2 Q(r^2) with the near-minimax
 * coefficients printed by simplediffeq.jl_gb300/csrc/gen_sincos.py, Horner
 * form, one rounding per operation.  Outside |x| < 2^19 (and for NaN/Inf)
 * libm is used. */
static void sincos_dev(double x, double* s, double* c) {
  if (!(std::fabs(x) < 524288.0)) {
    *s = std::sin(x);
    *c = std::cos(x);
    return;
  }
  static const double P[6] = {-0x1.5555555555548p-3, 0x1.111111110f7d0p-7, -0x1.a01a019bfde60p-13,
                              0x1.71de3567ccfe8p-19, -0x1.ae5e5a8d61ce7p-26, 0x1.5d8fd0a40698ep-33};
  static const double Q[6] = {-0x1.fffffffffff96p-2, 0x1.555555554f0a9p-5, -0x1.6c16c1640a98bp-10,
                              0x1.a019f81ca810ap-16, -0x1.27df4604d6713p-22, 0x1.1b8b9800ee7dap-29};
  const double shifter = 6755399441055744.0;  /* 1.5 * 2^52 */
  const double kb = std::fma(x, 0x1.45f306dc9c883p-1, shifter);
  const double k = kb - shifter;
  uint64_t bits;
  std::memcpy(&bits, &kb, 8);
  const unsigned quadrant = (unsigned)(bits & 3u);
  double r = std::fma(-k, 0x1.921fb54442d18p+0, x);
  r = std::fma(-k, 0x1.1a62633145c07p-54, r);
  const double z = r * r;
  double ps = P[5], pc = Q[5];
  for (int m = 4; m >= 0; --m) {
    ps = std::fma(ps, z, P[m]);
    pc = std::fma(pc, z, Q[m]);
  }
  const double sr = std::fma(z * r, ps, r);
  const double cr = std::fma(z, pc, 1.0);
  switch (quadrant) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}

/* REF rounding with ctrl == 3 (the kernels' reference-arithmetic mode): the
 * correctly rounded sine and cosine of crpow.h below 2^19; set per worker
 * thread by oracle_solve */
static thread_local bool g_cr_trig = false;

template <class R, bool DEV>
static inline void sincos_of(R x, R* s, R* c) {
  if (!DEV && g_cr_trig && sizeof(R) == sizeof(double)) {
    double sd, cd;
    if (gbode::cr_sincos((double)x, &sd, &cd)) {
      *s = (R)sd;
      *c = (R)cd;
      return;
    }
  }
  if (DEV && sizeof(R) == sizeof(double)) {
    double sd, cd;
    sincos_dev((double)x, &sd, &cd);
    *s = (R)sd;
    *c = (R)cd;
  } else {
    *s = std::sin(x);
    *c = std::cos(x);
  }
}

/* mu / r^(3/2) in the device canon: double r * sqrt(r) and a division; single
 * precision mu * y^3, y = 1/sqrt(r) from Lomont's bit-level seed (magic
 * constant 0x5f375a86) and three Newton steps y (3/2 - (r/2) y^2) */
static inline double r3bp_pull_dev(double mu, double r) { return mu / (r * std::sqrt(r)); }
/* 1/sqrt(x) for a positive normal single (kernels: rsqrt_nr) */
static inline float rsqrt_nr_f(float x) {
  int32_t xi;
  std::memcpy(&xi, &x, 4);
  const int32_t yi = 0x5f375a86 - (xi >> 1);
  float y;
  std::memcpy(&y, &yi, 4);
  const float hx = 0.5f * x;
  y = y * std::fma(-(hx * y), y, 1.5f);
  y = y * std::fma(-(hx * y), y, 1.5f);
  y = y * std::fma(-(hx * y), y, 1.5f);
  return y;
}
static inline float r3bp_pull_dev(float mu, float r) {
  const float y = rsqrt_nr_f(r);
  return mu * ((y * y) * y);
}

/* ---------------------------------------------------------------- problems */
/* Built-in right-hand sides.  The REF form is the plain Julia expression; the
 * DEV form fuses the products the device functors fuse. */
template <class R, bool DEV>
static void rhs_eval(int id, int D, const R* u, const R* p, double t, R* du) {
  (void)t;
  switch (id) {
    case ORACLE_LORENZ: {  /* p = (sigma, rho, beta) */
      R s = p[0], r = p[1], b = p[2];
      du[0] = s * (u[1] - u[0]);
      if (DEV) {
        du[1] = fmaX(u[0], r - u[2], -u[1]);
        du[2] = fmaX(u[0], u[1], -(b * u[2]));
      } else {
        du[1] = u[0] * (r - u[2]) - u[1];
        du[2] = u[0] * u[1] - b * u[2];
      }
      break;
    }
    case ORACLE_VDP: {  /* x' = v, v' = mu (1 - x^2) v - x; p = (mu) */
      R mu = p[0];
      du[0] = u[1];
      if (DEV) {
        R w = fmaX(-u[0], u[0], (R)1);
        du[1] = fmaX(mu * w, u[1], -u[0]);
      } else {
        du[1] = mu * ((R)1 - u[0] * u[0]) * u[1] - u[0];
      }
      break;
    }
    case ORACLE_R3BP: {  /* planar restricted three-body; u = (x, y, vx, vy); p = (mu) */
      R mu = p[0];
      R mu1 = (R)1 - mu;
      R x = u[0], y = u[1], vx = u[2], vy = u[3];
      R a = x + mu, b = x - mu1;
      if (DEV) {
        R r1 = fmaX(a, a, y * y), r2 = fmaX(b, b, y * y);
        R g1 = r3bp_pull_dev(mu1, r1), g2 = r3bp_pull_dev(mu, r2);
        du[0] = vx;
        du[1] = vy;
        du[2] = fmaX(-g2, b, fmaX(-g1, a, fmaX((R)2, vy, x)));
        du[3] = fmaX(-g2, y, fmaX(-g1, y, fmaX((R)-2, vx, y)));
      } else {
        R r1 = a * a + y * y, r2 = b * b + y * y;
        R d1 = r1 * std::sqrt(r1), d2 = r2 * std::sqrt(r2);
        du[0] = vx;
        du[1] = vy;
        du[2] = x + (R)2 * vy - mu1 * a / d1 - mu * b / d2;
        du[3] = y - (R)2 * vx - mu1 * y / d1 - mu * y / d2;
      }
      break;
    }
    case ORACLE_KURAMOTO: {  /* theta_i' = w_i + (K/D) sum_j sin(theta_j - theta_i); p = (w_1..w_D, K) */
      R S = 0, C = 0, sn[MAXD], cs[MAXD];
      for (int j = 0; j < D; ++j) {
        sincos_of<R, DEV>(u[j], &sn[j], &cs[j]);
        S += sn[j];
        C += cs[j];
      }
      R kd = p[D] / (R)D;
      for (int i = 0; i < D; ++i) {
        if (DEV) du[i] = fmaX(kd, fmaX(cs[i], S, -(sn[i] * C)), p[i]);
        else du[i] = p[i] + kd * (cs[i] * S - sn[i] * C);
      }
      break;
    }
    case ORACLE_LINEAR: {  /* du = A u, A row-major in p */
      for (int i = 0; i < D; ++i) {
        R s = p[i * D] * u[0];
        for (int j = 1; j < D; ++j) s = DEV ? fmaX(p[i * D + j], u[j], s) : s + p[i * D + j] * u[j];
        du[i] = s;
      }
      break;
    }
    default:
      for (int i = 0; i < D; ++i) du[i] = (R)NAN;
  }
}

/* ---------------------------------------------------------------- stage algebra */
struct Term { double c; int k; };

template <class P>
struct Alg {
  typedef typename P::R R;
  typedef typename P::T T;
  int D, rhs;
  R p[MAXP];

  void f(const R* u, double t, R* du) const { rhs_eval<R, P::DEV>(rhs, D, u, p, t, du); }

  /* s = sum_j c_j k_j accumulated left to right, the nesting @muladd gives a
   * sum of products (s = c_1 k_1, then s = muladd(c_j, k_j, s)).  This order is
   * pinned by the reference's own test/gpusimpleatsit5_tests.jl:59-60, which
   * requires SimpleTsit5 and GPUSimpleTsit5 to agree over a chaotic Lorenz
   * run although they group the update differently (src/tsit5/tsit5.jl:335
   * vs src/tsit5/gpuatsit5.jl:109): only left-to-right accumulation makes
   * both groupings round identically. */
  void lc(const Term* tm, int nt, R (*k)[MAXD], R* s) const {
    for (int d = 0; d < D; ++d) s[d] = (R)tm[0].c * k[tm[0].k][d];
    for (int j = 1; j < nt; ++j)
      for (int d = 0; d < D; ++d) s[d] = vmadd<P::DEV>((R)tm[j].c, k[tm[j].k][d], s[d]);
  }
  /* out = base + h * s */
  void axpy(const R* base, R h, const R* s, R* out) const {
    for (int d = 0; d < D; ++d) out[d] = vmadd<P::DEV>(h, s[d], base[d]);
  }
  /* stage time t + c*dt (a scalar muladd, fused in Julia too) */
  static T st(T t, double c, T dt) { return fmaX((T)c, dt, t); }
};

/* Compensated state: value = hi - c in KAHAN mode, hi otherwise. */
template <class R>
struct State { R hi[MAXD]; R c[MAXD]; };

template <class P>
static void state_update(int D, const State<typename P::R>& a, typename P::R h,
                         const typename P::R* s, State<typename P::R>& out) {
  typedef typename P::R R;
  for (int d = 0; d < D; ++d) {
    if (P::KAHAN) {
      R delta = h * s[d];
      R y = delta - a.c[d];
      R sum = a.hi[d] + y;
      out.c[d] = (sum - a.hi[d]) - y;
      out.hi[d] = sum;
    } else {
      out.hi[d] = vmadd<P::DEV>(h, s[d], a.hi[d]);
      out.c[d] = 0;
    }
  }
}

/* Horner evaluation of c0 + c1 x + ... with leading zero coefficients, as
 * @evalpoly does it (scalar muladd, fused). nz = number of leading zeros.
 * The device canon multiplies the polynomials that start at x^2 by one shared
 * x*x instead of by x twice. */
template <bool DEV, class R>
static R horner(R x, const double* c, int n, int nz) {
  R ex = (R)c[n - 1];
  for (int i = n - 2; i >= 0; --i) ex = fmaX(x, ex, (R)c[i]);
  if (DEV && nz == 2) return (x * x) * ex;
  for (int i = 0; i < nz; ++i) ex = x * ex;
  return ex;
}

/* 1/x of the device canon for the dense-output abscissa: a correctly rounded
 * single-precision reciprocal refined by one Newton step in double. */
static inline double recip_dev(double x) {
  const double r0 = (double)(1.0f / (float)x);
  const double e = std::fma(-x, r0, 1.0);
  return std::fma(r0, e, r0);
}
static inline float recip_dev(float x) { return 1.0f / x; }

/* ---------------------------------------------------------------- tableaus */
namespace t5 = gbtab::tsit5;
namespace v7 = gbtab::vern7;
namespace v7x = gbtab::vern7x;
namespace v7r = gbtab::vern7r;
namespace v9 = gbtab::vern9;
namespace v9x = gbtab::vern9x;
namespace v9r = gbtab::vern9r;

/* ---- Tsitouras 5(4), src/tsit5/gpuatsit5.jl:258-275 (k slots 0..6 = k1..k7) */
const Term T5_S3[] = {{t5::a31, 0}, {t5::a32, 1}};
const Term T5_S4[] = {{t5::a41, 0}, {t5::a42, 1}, {t5::a43, 2}};
const Term T5_S5[] = {{t5::a51, 0}, {t5::a52, 1}, {t5::a53, 2}, {t5::a54, 3}};
const Term T5_S6[] = {{t5::a61, 0}, {t5::a62, 1}, {t5::a63, 2}, {t5::a64, 3}, {t5::a65, 4}};
const Term T5_U[] = {{t5::a71, 0}, {t5::a72, 1}, {t5::a73, 2}, {t5::a74, 3}, {t5::a75, 4}, {t5::a76, 5}};
const Term T5_E[] = {{t5::btilde1, 0}, {t5::btilde2, 1}, {t5::btilde3, 2}, {t5::btilde4, 3},
                     {t5::btilde5, 4}, {t5::btilde6, 5}, {t5::btilde7, 6}};
/* SimpleTsit5 groups the update as ((a71 k1 + .. + a74 k4) + a75 k5 + a76 k6), src/tsit5/tsit5.jl:335-336 */
const Term T5_U_IN[] = {{t5::a71, 0}, {t5::a72, 1}, {t5::a73, 2}, {t5::a74, 3}};

/* bθs of src/tsit5/tsit5.jl:385-399: b1θ = poly(0, r11..r14), b_iθ = poly(0, 0, r_i2..r_i4) */
template <bool DEV, class R>
static void tsit5_btheta(R th, R* b) {
  const double c1[] = {t5::r11, t5::r12, t5::r13, t5::r14};
  const double c2[] = {t5::r22, t5::r23, t5::r24};
  const double c3[] = {t5::r32, t5::r33, t5::r34};
  const double c4[] = {t5::r42, t5::r43, t5::r44};
  const double c5[] = {t5::r52, t5::r53, t5::r54};
  const double c6[] = {t5::r62, t5::r63, t5::r64};
  const double c7[] = {t5::r72, t5::r73, t5::r74};
  b[0] = horner<DEV>(th, c1, 4, 1);
  b[1] = horner<DEV>(th, c2, 3, 2);
  b[2] = horner<DEV>(th, c3, 3, 2);
  b[3] = horner<DEV>(th, c4, 3, 2);
  b[4] = horner<DEV>(th, c5, 3, 2);
  b[5] = horner<DEV>(th, c6, 3, 2);
  b[6] = horner<DEV>(th, c7, 3, 2);
}

/* ---- Verner 7(6), src/verner/gpuvern7.jl:360-404 (slots 0..9 = k1..k10) */
const Term V7_S3[] = {{v7::a031, 0}, {v7::a032, 1}};
const Term V7_S4[] = {{v7::a041, 0}, {v7::a043, 2}};
const Term V7_S5[] = {{v7::a051, 0}, {v7::a053, 2}, {v7::a054, 3}};
const Term V7_S6[] = {{v7::a061, 0}, {v7::a063, 2}, {v7::a064, 3}, {v7::a065, 4}};
const Term V7_S7[] = {{v7::a071, 0}, {v7::a073, 2}, {v7::a074, 3}, {v7::a075, 4}, {v7::a076, 5}};
const Term V7_S8[] = {{v7::a081, 0}, {v7::a083, 2}, {v7::a084, 3}, {v7::a085, 4}, {v7::a086, 5}, {v7::a087, 6}};
const Term V7_G9[] = {{v7::a091, 0}, {v7::a093, 2}, {v7::a094, 3}, {v7::a095, 4}, {v7::a096, 5},
                      {v7::a097, 6}, {v7::a098, 7}};
const Term V7_G10[] = {{v7::a101, 0}, {v7::a103, 2}, {v7::a104, 3}, {v7::a105, 4}, {v7::a106, 5}, {v7::a107, 6}};
const Term V7_U[] = {{v7::b1, 0}, {v7::b4, 3}, {v7::b5, 4}, {v7::b6, 5}, {v7::b7, 6}, {v7::b8, 7}, {v7::b9, 8}};
const Term V7_E[] = {{v7::btilde1, 0}, {v7::btilde4, 3}, {v7::btilde5, 4}, {v7::btilde6, 5},
                     {v7::btilde7, 6}, {v7::btilde8, 7}, {v7::btilde9, 8}, {v7::btilde10, 9}};
/* extra stages for dense output, gpuvern7.jl:441-504 (slots 10..15 = k11..k16) */
const Term V7_X11[] = {{v7x::a1101, 0}, {v7x::a1104, 3}, {v7x::a1105, 4}, {v7x::a1106, 5},
                       {v7x::a1107, 6}, {v7x::a1108, 7}, {v7x::a1109, 8}};
const Term V7_X12[] = {{v7x::a1201, 0}, {v7x::a1204, 3}, {v7x::a1205, 4}, {v7x::a1206, 5},
                       {v7x::a1207, 6}, {v7x::a1208, 7}, {v7x::a1209, 8}, {v7x::a1211, 10}};
const Term V7_X13[] = {{v7x::a1301, 0}, {v7x::a1304, 3}, {v7x::a1305, 4}, {v7x::a1306, 5}, {v7x::a1307, 6},
                       {v7x::a1308, 7}, {v7x::a1309, 8}, {v7x::a1311, 10}, {v7x::a1312, 11}};
const Term V7_X14[] = {{v7x::a1401, 0}, {v7x::a1404, 3}, {v7x::a1405, 4}, {v7x::a1406, 5}, {v7x::a1407, 6},
                       {v7x::a1408, 7}, {v7x::a1409, 8}, {v7x::a1411, 10}, {v7x::a1412, 11}, {v7x::a1413, 12}};
const Term V7_X15[] = {{v7x::a1501, 0}, {v7x::a1504, 3}, {v7x::a1505, 4}, {v7x::a1506, 5}, {v7x::a1507, 6},
                       {v7x::a1508, 7}, {v7x::a1509, 8}, {v7x::a1511, 10}, {v7x::a1512, 11}, {v7x::a1513, 12}};
const Term V7_X16[] = {{v7x::a1601, 0}, {v7x::a1604, 3}, {v7x::a1605, 4}, {v7x::a1606, 5}, {v7x::a1607, 6},
                       {v7x::a1608, 7}, {v7x::a1609, 8}, {v7x::a1611, 10}, {v7x::a1612, 11}, {v7x::a1613, 12}};
const double V7_XC[] = {v7x::c11, v7x::c12, v7x::c13, v7x::c14, v7x::c15, v7x::c16};

/* bθs of src/verner/verner_tableaus.jl:1337-1360; order b1,b4..b9,b11..b16 */
template <bool DEV, class R>
static void vern7_btheta(R th, R* b) {
  const double r1[] = {v7r::r011, v7r::r012, v7r::r013, v7r::r014, v7r::r015, v7r::r016, v7r::r017};
  const double r4[] = {v7r::r042, v7r::r043, v7r::r044, v7r::r045, v7r::r046, v7r::r047};
  const double r5[] = {v7r::r052, v7r::r053, v7r::r054, v7r::r055, v7r::r056, v7r::r057};
  const double r6[] = {v7r::r062, v7r::r063, v7r::r064, v7r::r065, v7r::r066, v7r::r067};
  const double r7[] = {v7r::r072, v7r::r073, v7r::r074, v7r::r075, v7r::r076, v7r::r077};
  const double r8[] = {v7r::r082, v7r::r083, v7r::r084, v7r::r085, v7r::r086, v7r::r087};
  const double r9[] = {v7r::r092, v7r::r093, v7r::r094, v7r::r095, v7r::r096, v7r::r097};
  const double r11[] = {v7r::r112, v7r::r113, v7r::r114, v7r::r115, v7r::r116, v7r::r117};
  const double r12[] = {v7r::r122, v7r::r123, v7r::r124, v7r::r125, v7r::r126, v7r::r127};
  const double r13[] = {v7r::r132, v7r::r133, v7r::r134, v7r::r135, v7r::r136, v7r::r137};
  const double r14[] = {v7r::r142, v7r::r143, v7r::r144, v7r::r145, v7r::r146, v7r::r147};
  const double r15[] = {v7r::r152, v7r::r153, v7r::r154, v7r::r155, v7r::r156, v7r::r157};
  const double r16[] = {v7r::r162, v7r::r163, v7r::r164, v7r::r165, v7r::r166, v7r::r167};
  b[0] = horner<DEV>(th, r1, 7, 1);
  const double* rs[] = {r4, r5, r6, r7, r8, r9, r11, r12, r13, r14, r15, r16};
  for (int i = 0; i < 12; ++i) b[i + 1] = horner<DEV>(th, rs[i], 6, 2);
}

/* ---- Verner 9(8), src/verner/gpuvern9.jl:468-573 (slots 0..15 = k1..k16) */
const Term V9_S3[] = {{v9::a0301, 0}, {v9::a0302, 1}};
const Term V9_S4[] = {{v9::a0401, 0}, {v9::a0403, 2}};
const Term V9_S5[] = {{v9::a0501, 0}, {v9::a0503, 2}, {v9::a0504, 3}};
const Term V9_S6[] = {{v9::a0601, 0}, {v9::a0604, 3}, {v9::a0605, 4}};
const Term V9_S7[] = {{v9::a0701, 0}, {v9::a0704, 3}, {v9::a0705, 4}, {v9::a0706, 5}};
const Term V9_S8[] = {{v9::a0801, 0}, {v9::a0806, 5}, {v9::a0807, 6}};
const Term V9_S9[] = {{v9::a0901, 0}, {v9::a0906, 5}, {v9::a0907, 6}, {v9::a0908, 7}};
const Term V9_S10[] = {{v9::a1001, 0}, {v9::a1006, 5}, {v9::a1007, 6}, {v9::a1008, 7}, {v9::a1009, 8}};
const Term V9_S11[] = {{v9::a1101, 0}, {v9::a1106, 5}, {v9::a1107, 6}, {v9::a1108, 7}, {v9::a1109, 8}, {v9::a1110, 9}};
const Term V9_S12[] = {{v9::a1201, 0}, {v9::a1206, 5}, {v9::a1207, 6}, {v9::a1208, 7}, {v9::a1209, 8},
                       {v9::a1210, 9}, {v9::a1211, 10}};
const Term V9_S13[] = {{v9::a1301, 0}, {v9::a1306, 5}, {v9::a1307, 6}, {v9::a1308, 7}, {v9::a1309, 8},
                       {v9::a1310, 9}, {v9::a1311, 10}, {v9::a1312, 11}};
const Term V9_S14[] = {{v9::a1401, 0}, {v9::a1406, 5}, {v9::a1407, 6}, {v9::a1408, 7}, {v9::a1409, 8},
                       {v9::a1410, 9}, {v9::a1411, 10}, {v9::a1412, 11}, {v9::a1413, 12}};
const Term V9_G15[] = {{v9::a1501, 0}, {v9::a1506, 5}, {v9::a1507, 6}, {v9::a1508, 7}, {v9::a1509, 8},
                       {v9::a1510, 9}, {v9::a1511, 10}, {v9::a1512, 11}, {v9::a1513, 12}, {v9::a1514, 13}};
const Term V9_G16[] = {{v9::a1601, 0}, {v9::a1606, 5}, {v9::a1607, 6}, {v9::a1608, 7}, {v9::a1609, 8},
                       {v9::a1610, 9}, {v9::a1611, 10}, {v9::a1612, 11}, {v9::a1613, 12}};
const Term V9_U[] = {{v9::b1, 0}, {v9::b8, 7}, {v9::b9, 8}, {v9::b10, 9}, {v9::b11, 10}, {v9::b12, 11},
                     {v9::b13, 12}, {v9::b14, 13}, {v9::b15, 14}};
const Term V9_E[] = {{v9::btilde1, 0}, {v9::btilde8, 7}, {v9::btilde9, 8}, {v9::btilde10, 9},
                     {v9::btilde11, 10}, {v9::btilde12, 11}, {v9::btilde13, 12}, {v9::btilde14, 13},
                     {v9::btilde15, 14}, {v9::btilde16, 15}};
/* Dense-output stages, gpuvern9.jl:631-745 (adaptive) and :216-319 (fixed step).
 * Slots: 0..8 hold the nine stages the formulas call k1..k9 and 16..25 hold the
 * new stages k11..k20.  Which original stages sit in slots 1..8 depends on the
 * caller: the adaptive solver relabels k2..k9 := k8..k15 first (:564-573), the
 * fixed-step solver does not. */
const Term V9_X17[] = {{v9x::a1701, 0}, {v9x::a1708, 1}, {v9x::a1709, 2}, {v9x::a1710, 3}, {v9x::a1711, 4},
                       {v9x::a1712, 5}, {v9x::a1713, 6}, {v9x::a1714, 7}, {v9x::a1715, 8}};
const Term V9_X18[] = {{v9x::a1801, 0}, {v9x::a1808, 1}, {v9x::a1809, 2}, {v9x::a1810, 3}, {v9x::a1811, 4},
                       {v9x::a1812, 5}, {v9x::a1813, 6}, {v9x::a1814, 7}, {v9x::a1815, 8}, {v9x::a1817, 16}};
const Term V9_X19[] = {{v9x::a1901, 0}, {v9x::a1908, 1}, {v9x::a1909, 2}, {v9x::a1910, 3}, {v9x::a1911, 4},
                       {v9x::a1912, 5}, {v9x::a1913, 6}, {v9x::a1914, 7}, {v9x::a1915, 8}, {v9x::a1917, 16},
                       {v9x::a1918, 17}};
const Term V9_X20[] = {{v9x::a2001, 0}, {v9x::a2008, 1}, {v9x::a2009, 2}, {v9x::a2010, 3}, {v9x::a2011, 4},
                       {v9x::a2012, 5}, {v9x::a2013, 6}, {v9x::a2014, 7}, {v9x::a2015, 8}, {v9x::a2017, 16},
                       {v9x::a2018, 17}, {v9x::a2019, 18}};
const Term V9_X21[] = {{v9x::a2101, 0}, {v9x::a2108, 1}, {v9x::a2109, 2}, {v9x::a2110, 3}, {v9x::a2111, 4},
                       {v9x::a2112, 5}, {v9x::a2113, 6}, {v9x::a2114, 7}, {v9x::a2115, 8}, {v9x::a2117, 16},
                       {v9x::a2118, 17}, {v9x::a2119, 18}, {v9x::a2120, 19}};
const Term V9_X22[] = {{v9x::a2201, 0}, {v9x::a2208, 1}, {v9x::a2209, 2}, {v9x::a2210, 3}, {v9x::a2211, 4},
                       {v9x::a2212, 5}, {v9x::a2213, 6}, {v9x::a2214, 7}, {v9x::a2215, 8}, {v9x::a2217, 16},
                       {v9x::a2218, 17}, {v9x::a2219, 18}, {v9x::a2220, 19}, {v9x::a2221, 20}};
const Term V9_X23[] = {{v9x::a2301, 0}, {v9x::a2308, 1}, {v9x::a2309, 2}, {v9x::a2310, 3}, {v9x::a2311, 4},
                       {v9x::a2312, 5}, {v9x::a2313, 6}, {v9x::a2314, 7}, {v9x::a2315, 8}, {v9x::a2317, 16},
                       {v9x::a2318, 17}, {v9x::a2319, 18}, {v9x::a2320, 19}, {v9x::a2321, 20}};
const Term V9_X24[] = {{v9x::a2401, 0}, {v9x::a2408, 1}, {v9x::a2409, 2}, {v9x::a2410, 3}, {v9x::a2411, 4},
                       {v9x::a2412, 5}, {v9x::a2413, 6}, {v9x::a2414, 7}, {v9x::a2415, 8}, {v9x::a2417, 16},
                       {v9x::a2418, 17}, {v9x::a2419, 18}, {v9x::a2420, 19}, {v9x::a2421, 20}};
const Term V9_X25[] = {{v9x::a2501, 0}, {v9x::a2508, 1}, {v9x::a2509, 2}, {v9x::a2510, 3}, {v9x::a2511, 4},
                       {v9x::a2512, 5}, {v9x::a2513, 6}, {v9x::a2514, 7}, {v9x::a2515, 8}, {v9x::a2517, 16},
                       {v9x::a2518, 17}, {v9x::a2519, 18}, {v9x::a2520, 19}, {v9x::a2521, 20}};
const Term V9_X26[] = {{v9x::a2601, 0}, {v9x::a2608, 1}, {v9x::a2609, 2}, {v9x::a2610, 3}, {v9x::a2611, 4},
                       {v9x::a2612, 5}, {v9x::a2613, 6}, {v9x::a2614, 7}, {v9x::a2615, 8}, {v9x::a2617, 16},
                       {v9x::a2618, 17}, {v9x::a2619, 18}, {v9x::a2620, 19}, {v9x::a2621, 20}};
const double V9_XC[] = {v9x::c17, v9x::c18, v9x::c19, v9x::c20, v9x::c21, v9x::c22, v9x::c23, v9x::c24,
                        v9x::c25, v9x::c26};

/* bθs of src/verner/verner_tableaus.jl:1362-1398; order b1,b8..b15,b17..b26 */
template <bool DEV, class R>
static void vern9_btheta(R th, R* b) {
  const double r1[] = {v9r::r011, v9r::r012, v9r::r013, v9r::r014, v9r::r015, v9r::r016, v9r::r017, v9r::r018, v9r::r019};
#define V9ROW(i) const double r##i[] = {v9r::r##i##2, v9r::r##i##3, v9r::r##i##4, v9r::r##i##5, \
                                         v9r::r##i##6, v9r::r##i##7, v9r::r##i##8, v9r::r##i##9}
  const double r8[] = {v9r::r082, v9r::r083, v9r::r084, v9r::r085, v9r::r086, v9r::r087, v9r::r088, v9r::r089};
  const double r9[] = {v9r::r092, v9r::r093, v9r::r094, v9r::r095, v9r::r096, v9r::r097, v9r::r098, v9r::r099};
  V9ROW(10); V9ROW(11); V9ROW(12); V9ROW(13); V9ROW(14); V9ROW(15);
  V9ROW(17); V9ROW(18); V9ROW(19); V9ROW(20); V9ROW(21); V9ROW(22); V9ROW(23); V9ROW(24); V9ROW(25); V9ROW(26);
#undef V9ROW
  b[0] = horner<DEV>(th, r1, 9, 1);
  const double* rs[] = {r8, r9, r10, r11, r12, r13, r14, r15, r17, r18, r19, r20, r21, r22, r23, r24, r25, r26};
  for (int i = 0; i < 18; ++i) b[i + 1] = horner<DEV>(th, rs[i], 8, 2);
}

/* ---------------------------------------------------------------- methods */
/* Each method provides:
 *   NK, FSAL, DTMIN_1F7 (Vern9 uses 1f-7 for dtmin and the end snap)
 *   attempt(): stages given k[0] (FSAL) or computing k[0]; the solution
 *              update, and (adaptive) the error estimate.
 *   dense():   one saveat point. */
template <class P>
struct Tsit5 {
  typedef typename P::R R;
  typedef typename P::T T;
  static constexpr int NK = 7;
  static constexpr bool FSAL = true;
  static constexpr bool DTMIN_1F7 = false;

  static void attempt(const Alg<P>& A, const State<R>& up, T t, T dt, R (*k)[MAXD], State<R>& u, R* e,
                      int want_err) {
    R tmp[MAXD], s[MAXD];
    const R h = (R)dt;
    const R* uprev = up.hi;
    const R a = (R)(dt * (T)t5::a21);  /* dt * a21, the scalar factor of the stage-2 update */
    for (int d = 0; d < A.D; ++d) {
      if (P::DEV) tmp[d] = fmaX(a, k[0][d], uprev[d]);
      else tmp[d] = h * ((R)t5::a21 * k[0][d]) + uprev[d];
    }
    A.f(tmp, (double)A.st(t, t5::c1, dt), k[1]);
    A.lc(T5_S3, 2, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, t5::c2, dt), k[2]);
    A.lc(T5_S4, 3, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, t5::c3, dt), k[3]);
    A.lc(T5_S5, 4, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, t5::c4, dt), k[4]);
    A.lc(T5_S6, 5, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)(t + dt), k[5]);
    A.lc(T5_U, 6, k, s);
    state_update<P>(A.D, up, h, s, u);
    A.f(u.hi, (double)(t + dt), k[6]);
    if (want_err) {
      A.lc(T5_E, 7, k, s);
      for (int d = 0; d < A.D; ++d) e[d] = want_err == 2 ? s[d] : h * s[d];
    }
  }

  /* src/tsit5/gpuatsit5.jl:306-314 */
  static void dense(const Alg<P>& A, const State<R>& up, T told, T tnew, T dtold, T theta, R (*k)[MAXD],
                    double* out) {
    (void)told; (void)tnew;
    R b[7], s[MAXD];
    tsit5_btheta<P::DEV, R>((R)theta, b);
    for (int d = 0; d < A.D; ++d) s[d] = b[0] * k[0][d];
    for (int j = 1; j < 7; ++j)
      for (int d = 0; d < A.D; ++d) s[d] = vmadd<P::DEV>(b[j], k[j][d], s[d]);
    finish_dense(A, up, (R)dtold, s, out);
  }

  static void finish_dense(const Alg<P>& A, const State<R>& up, R h, const R* s, double* out) {
    for (int d = 0; d < A.D; ++d) {
      if (P::KAHAN) out[d] = ((double)up.hi[d] - (double)up.c[d]) + (double)(h * s[d]);
      else out[d] = (double)vmadd<P::DEV>(h, s[d], up.hi[d]);
    }
  }
};

template <class P>
static void dense_sum(const Alg<P>& A, const typename P::R* b, const int* slot, int n,
                      typename P::R (*k)[MAXD], typename P::R* s) {
  for (int d = 0; d < A.D; ++d) s[d] = b[0] * k[slot[0]][d];
  for (int j = 1; j < n; ++j)
    for (int d = 0; d < A.D; ++d) s[d] = vmadd<P::DEV>(b[j], k[slot[j]][d], s[d]);
}

template <class P>
struct Vern7 {
  typedef typename P::R R;
  typedef typename P::T T;
  static constexpr int NK = 16;
  static constexpr bool FSAL = false;
  static constexpr bool DTMIN_1F7 = false;

  static void attempt(const Alg<P>& A, const State<R>& up, T t, T dt, R (*k)[MAXD], State<R>& u, R* e,
                      int want_err) {
    R tmp[MAXD], s[MAXD];
    const R h = (R)dt;
    const R* uprev = up.hi;
    A.f(uprev, (double)t, k[0]);
    const R a = (R)(dt * (T)v7::a021);
    for (int d = 0; d < A.D; ++d) tmp[d] = vmadd<P::DEV>(a, k[0][d], uprev[d]);
    A.f(tmp, (double)A.st(t, v7::c2, dt), k[1]);
    A.lc(V7_S3, 2, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, v7::c3, dt), k[2]);
    A.lc(V7_S4, 2, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, v7::c4, dt), k[3]);
    A.lc(V7_S5, 3, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, v7::c5, dt), k[4]);
    A.lc(V7_S6, 4, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, v7::c6, dt), k[5]);
    A.lc(V7_S7, 5, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, v7::c7, dt), k[6]);
    A.lc(V7_S8, 6, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, v7::c8, dt), k[7]);
    R g10[MAXD];
    A.lc(V7_G9, 7, k, s); A.axpy(uprev, h, s, tmp);
    A.lc(V7_G10, 6, k, s); A.axpy(uprev, h, s, g10);
    A.f(tmp, (double)(t + dt), k[8]);
    A.f(g10, (double)(t + dt), k[9]);
    A.lc(V7_U, 7, k, s);
    state_update<P>(A.D, up, h, s, u);
    if (want_err) {
      A.lc(V7_E, 8, k, s);
      for (int d = 0; d < A.D; ++d) e[d] = want_err == 2 ? s[d] : h * s[d];
    }
  }

  /* gpuvern7.jl:441-513 (adaptive; stage times use the advanced t) and
   * :153-219 (fixed step, same expressions with dt). */
  static void dense(const Alg<P>& A, const State<R>& up, T told, T tnew, T dtold, T theta, R (*k)[MAXD],
                    double* out) {
    (void)told;
    const R h = (R)dtold;
    R b[13], s[MAXD], tmp[MAXD];
    vern7_btheta<P::DEV, R>((R)theta, b);
    const Term* xs[] = {V7_X11, V7_X12, V7_X13, V7_X14, V7_X15, V7_X16};
    const int nx[] = {7, 8, 9, 10, 10, 10};
    for (int i = 0; i < 6; ++i) {
      A.lc(xs[i], nx[i], k, s);
      A.axpy(up.hi, h, s, tmp);
      A.f(tmp, (double)A.st(tnew, V7_XC[i], dtold), k[10 + i]);
    }
    static const int slot[13] = {0, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 14, 15};
    dense_sum<P>(A, b, slot, 13, k, s);
    Tsit5<P>::finish_dense(A, up, h, s, out);
  }
};

template <class P, bool ADAPTIVE>
struct Vern9 {
  typedef typename P::R R;
  typedef typename P::T T;
  static constexpr int NK = 26;
  static constexpr bool FSAL = false;
  static constexpr bool DTMIN_1F7 = true;

  static void attempt(const Alg<P>& A, const State<R>& up, T t, T dt, R (*k)[MAXD], State<R>& u, R* e,
                      int want_err) {
    R tmp[MAXD], s[MAXD];
    const R h = (R)dt;
    const R* uprev = up.hi;
    A.f(uprev, (double)t, k[0]);
    const R a = (R)(dt * (T)v9::a0201);
    for (int d = 0; d < A.D; ++d) tmp[d] = vmadd<P::DEV>(a, k[0][d], uprev[d]);
    A.f(tmp, (double)A.st(t, v9::c1, dt), k[1]);
    const Term* ss[] = {V9_S3, V9_S4, V9_S5, V9_S6, V9_S7, V9_S8, V9_S9, V9_S10, V9_S11, V9_S12, V9_S13, V9_S14};
    const int ns[] = {2, 2, 3, 3, 4, 3, 4, 5, 6, 7, 8, 9};
    const double cs[] = {v9::c2, v9::c3, v9::c4, v9::c5, v9::c6, v9::c7, v9::c8, v9::c9, v9::c10, v9::c11,
                         v9::c12, v9::c13};
    for (int i = 0; i < 12; ++i) {
      A.lc(ss[i], ns[i], k, s);
      A.axpy(uprev, h, s, tmp);
      A.f(tmp, (double)A.st(t, cs[i], dt), k[2 + i]);
    }
    R g16[MAXD];
    A.lc(V9_G15, 10, k, s); A.axpy(uprev, h, s, tmp);
    if (ADAPTIVE) { A.lc(V9_G16, 9, k, s); A.axpy(uprev, h, s, g16); }
    A.f(tmp, (double)(t + dt), k[14]);
    if (ADAPTIVE) A.f(g16, (double)(t + dt), k[15]);
    A.lc(V9_U, 9, k, s);
    state_update<P>(A.D, up, h, s, u);
    if (want_err) {
      A.lc(V9_E, 10, k, s);
      for (int d = 0; d < A.D; ++d) e[d] = want_err == 2 ? s[d] : h * s[d];
    }
  }

  /* Adaptive: gpuvern9.jl:564-573 relabels k2..k9 := k8..k15 and the dense
   * stages run at told + c*dtold (:631-757).  Fixed step: no relabel, stage
   * times t + c*dt with the advanced t (:216-331). */
  static void dense(const Alg<P>& A, const State<R>& up, T told, T tnew, T dtold, T theta, R (*k)[MAXD],
                    double* out) {
    const R h = (R)dtold;
    R kk[MAXK][MAXD];
    for (int d = 0; d < A.D; ++d) kk[0][d] = k[0][d];
    for (int j = 1; j <= 8; ++j)
      for (int d = 0; d < A.D; ++d) kk[j][d] = ADAPTIVE ? k[j + 6][d] : k[j][d];
    R b[19], s[MAXD], tmp[MAXD];
    vern9_btheta<P::DEV, R>((R)theta, b);
    const Term* xs[] = {V9_X17, V9_X18, V9_X19, V9_X20, V9_X21, V9_X22, V9_X23, V9_X24, V9_X25, V9_X26};
    const int nx[] = {9, 10, 11, 12, 13, 14, 14, 14, 14, 14};
    const T tb = ADAPTIVE ? told : tnew;
    for (int i = 0; i < 10; ++i) {
      A.lc(xs[i], nx[i], kk, s);
      A.axpy(up.hi, h, s, tmp);
      A.f(tmp, (double)A.st(tb, V9_XC[i], dtold), kk[16 + i]);
    }
    static const int slot[19] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25};
    dense_sum<P>(A, b, slot, 19, kk, s);
    Tsit5<P>::finish_dense(A, up, h, s, out);
  }
};

template <class P>
struct RK4 {
  typedef typename P::R R;
  typedef typename P::T T;
  /* src/rk4/gpurk4.jl:73-84; t is the END of the step (ts[i]) */
  static void step(const Alg<P>& A, const State<R>& up, T t, T dt, State<R>& u) {
    R k1[MAXD], k2[MAXD], k3[MAXD], k4[MAXD], tmp[MAXD], s[MAXD];
    const R h = (R)dt;
    const R half = (R)0.5, sixth = (R)(1.0 / 6.0);
    const R* uprev = up.hi;
    A.f(uprev, (double)t, k1);
    const R hh = h * half;
    for (int d = 0; d < A.D; ++d) tmp[d] = P::DEV ? fmaX(hh, k1[d], uprev[d]) : h * (half * k1[d]) + uprev[d];
    A.f(tmp, (double)fmaX((T)0.5, dt, t), k2);
    for (int d = 0; d < A.D; ++d) tmp[d] = P::DEV ? fmaX(hh, k2[d], uprev[d]) : h * (half * k2[d]) + uprev[d];
    A.f(tmp, (double)fmaX((T)0.5, dt, t), k3);
    for (int d = 0; d < A.D; ++d) tmp[d] = vmadd<P::DEV>(h, k3[d], uprev[d]);
    A.f(tmp, (double)(t + dt), k4);
    for (int d = 0; d < A.D; ++d) {
      /* k1 + 2k2 + 2k3 + k4 = muladd(2, k3, muladd(2, k2, k1 + k4)); the
       * doublings are exact, so fused and unfused forms round alike */
      R sum = k1[d] + k4[d];
      sum = vmadd<P::DEV>((R)2, k2[d], sum);
      sum = vmadd<P::DEV>((R)2, k3[d], sum);
      s[d] = P::DEV ? sum : sixth * sum;
    }
    if (P::DEV) {
      State<R> tmpu;
      state_update<P>(A.D, up, h * sixth, s, tmpu);
      u = tmpu;
    } else {
      for (int d = 0; d < A.D; ++d) { u.hi[d] = h * s[d] + uprev[d]; u.c[d] = 0; }
    }
  }
};

/* ---------------------------------------------------------------- drivers */
struct Job {
  const oracle_args* a;
  oracle_out* o;
};

template <class P>
static void load_traj(const oracle_args* a, int64_t i, Alg<P>& A, State<typename P::R>& st) {
  typedef typename P::R R;
  A.D = a->dim;
  A.rhs = a->rhs;
  for (int j = 0; j < a->nparams; ++j) A.p[j] = (R)a->p[(int64_t)j * a->n + i];
  for (int d = 0; d < a->dim; ++d) {
    st.hi[d] = (R)a->u0[(int64_t)d * a->n + i];
    st.c[d] = 0;
  }
}

/* Saveat point j of trajectory i: the state, or the Kuramoto order parameter
 * r = |(1/D) sum_k exp(i v_k)| (an ensemble output function: SciMLBase would
 * apply it to each solution on the host). */
static inline void put_us(const oracle_args* a, oracle_out* o, int64_t i, int64_t j, const double* v) {
  if (!o->us) return;
  if (a->output == 1) {
    /* device canon: sincos_dev and a fused C*C + S*S; reference rounding: libm and two roundings */
    const bool dev = a->rounding == ORACLE_ROUND_DEVICE;
    double C = 0, S = 0;
    for (int d = 0; d < a->dim; ++d) {
      double sn, cs;
      if (dev) {
        sincos_dev(v[d], &sn, &cs);
      } else if (!(g_cr_trig && gbode::cr_sincos(v[d], &sn, &cs))) {
        sn = std::sin(v[d]);
        cs = std::cos(v[d]);
      }
      C = C + cs;
      S = S + sn;
    }
    o->us[j * a->n + i] = std::sqrt(dev ? std::fma(C, C, S * S) : C * C + S * S) / a->dim;
    return;
  }
  for (int d = 0; d < a->dim; ++d) o->us[(j * a->dim + d) * a->n + i] = v[d];
}

template <class R>
static void value_of(const State<R>& s, int D, bool kahan, double* v) {
  for (int d = 0; d < D; ++d) v[d] = kahan ? (double)s.hi[d] - (double)s.c[d] : (double)s.hi[d];
}

template <class P>
static void finish(const oracle_args* a, oracle_out* o, int64_t i, const State<typename P::R>& st,
                   typename P::T t, int ret, int32_t nacc, int32_t nrej, double dtf) {
  double v[MAXD];
  value_of(st, a->dim, P::KAHAN, v);
  if (o->u_final)
    for (int d = 0; d < a->dim; ++d) o->u_final[(int64_t)d * a->n + i] = v[d];
  if (o->t_final) o->t_final[i] = (double)t;
  if (o->retcode) o->retcode[i] = (int8_t)ret;
  if (o->naccept) o->naccept[i] = nacc;
  if (o->nreject) o->nreject[i] = nrej;
  if (o->dt_first) o->dt_first[i] = dtf;
}

/* Adaptive driver: the loop of gpuatsit5.jl:250-320 / gpuvern7.jl:353-520 /
 * gpuvern9.jl:461-763 with the controller of :279-299. */
/* Row k of trajectory i's every-step output (gpuatsit5.jl:225-229, :301-303:
 * push!(us, u); push!(ts, t) after each accepted step, u0 first). */
template <class R>
static void put_step(const oracle_args* a, oracle_out* o, int64_t i, int64_t k, double t, const State<R>& st,
                     bool kahan) {
  if (!o->ev_t) return;
  double v[MAXD];
  value_of(st, a->dim, kahan, v);
  const int64_t r = o->ev_off[i] + k;
  o->ev_t[r] = t;
  for (int d = 0; d < a->dim; ++d) o->ev_u[r * a->dim + d] = v[d];
}

double log_dev(double x);
double exp_dev(double x);

/* Single-precision modes of the device canon: error norm and controller free
 * of IEEE division and square root (kernels: rcp_nr, log2_nr, exp2_nr in
 * ode_solver.cuh).  rcp: seed 0x7ef311c7 - bits(d), three Newton steps
 * y (2 - d y); log2: the atanh series with (m-1)/(m+1) by rcp and the
 * sqrt(2) fold; exp2: y = n + f by the 1.5 * 2^23 shifter, Taylor degree 7 in
 * f ln 2, scaled by 2^n through the exponent bits. */
static inline float bits_f(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline int32_t fbits(float f) { int32_t i; std::memcpy(&i, &f, 4); return i; }
static inline float rcp_nr(float d) {
  float y = bits_f(0x7ef311c7 - fbits(d));
  y = y * std::fma(-d, y, 2.0f);
  y = y * std::fma(-d, y, 2.0f);
  y = y * std::fma(-d, y, 2.0f);
  return y;
}
static inline float log2_nr(float x) {
  const int32_t b = fbits(x);
  const int e0 = ((b >> 23) & 0xff) - 127;
  const float m0 = bits_f((b & 0x007fffff) | 0x3f800000);
  const bool fold = m0 > 1.41421354f;
  const float m = fold ? 0.5f * m0 : m0;
  const int e = fold ? e0 + 1 : e0;
  const float s = (m - 1.0f) * rcp_nr(m + 1.0f);
  const float s2 = s * s;
  float poly = std::fma(s2, 0.0909090936f, 0.111111112f);
  poly = std::fma(s2, poly, 0.142857149f);
  poly = std::fma(s2, poly, 0.200000003f);
  poly = std::fma(s2, poly, 0.333333343f);
  poly = std::fma(s2, poly, 1.0f);
  return std::fma(s * poly, 2.88539004f, (float)e);
}
static inline float exp2_nr(float y) {
  const float t = y + 12582912.0f;
  const int n = fbits(t) - 0x4b400000;
  const float f = y - (t - 12582912.0f);
  const float z = f * 0.693147182f;
  float p = std::fma(z, 1.98412701e-04f, 1.38888892e-03f);
  p = std::fma(z, p, 8.33333377e-03f);
  p = std::fma(z, p, 4.16666679e-02f);
  p = std::fma(z, p, 0.166666672f);
  p = std::fma(z, p, 0.5f);
  p = std::fma(z, p, 1.0f);
  p = std::fma(z, p, 1.0f);
  return p * bits_f((n + 127) << 23);
}
static const float L2_QMINI = 2.32192809f, L2_QMAXI = -3.32192809f, L2_GAMMA = -0.152003093f,
                   L2_QOLDINIT = -13.2877124f;

/* Double-single error norm and controller of the FP64 solves (kernels:
 * ds_* in ode_solver.cuh, tables from ds_table.h).  A pair (h, l) stands for
 * h + l; the operations are Knuth's two-sum, Dekker's fast two-sum and the
 * fma product error, each step one IEEE single operation. */
struct DS { float h, l; };
static inline DS ds_two_sum(float a, float b) {
  const float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
static inline DS ds_fast(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
static inline DS ds_add(DS x, DS y) {
  const DS s = ds_two_sum(x.h, y.h);
  return ds_fast(s.h, s.l + (x.l + y.l));
}
static inline DS ds_neg(DS x) { return {-x.h, -x.l}; }
static inline DS ds_mul(DS x, DS y) {
  const float p = x.h * y.h;
  return ds_fast(p, std::fma(x.h, y.l, std::fma(x.l, y.h, std::fma(x.h, y.h, -p))));
}
static inline DS ds_sqr(DS x) {
  const float p = x.h * x.h;
  return ds_fast(p, std::fma(x.h + x.h, x.l, std::fma(x.h, x.h, -p)));
}
static inline DS ds_div(DS x, DS y) {
  if (y.h == 0.0f) return {x.h * INFINITY, 0.0f};
  const float ry = rcp_nr(y.h);
  const float q1 = x.h * ry;
  const float p = q1 * y.h, pe = std::fma(q1, y.h, -p);
  const float rem = (((x.h - p) - pe) + x.l) - q1 * y.l;
  return ds_fast(q1, rem * ry);
}
static inline bool ds_gt(DS x, DS y) { return x.h > y.h || (x.h == y.h && x.l > y.l); }
static inline DS ds_min(DS x, DS y) { return ds_gt(y, x) ? x : y; }
static inline DS ds_max(DS x, DS y) { return ds_gt(y, x) ? y : x; }
/* h: x with the 29 low fraction bits cleared; l: those bits as an integer
 * rounded to single, times 2^(e-52) (0 outside 2^-74 <= |x| < 2^128) */
/* an integer 0 <= i < 2^23 as a single: bits of 2^23 + i, minus 2^23 */
static inline float ds_small_int(int32_t i) { return bits_f(0x4b000000 | i) - 8388608.0f; }
/* h: x's sign, exponent and top 23 fraction bits repacked as a single
 * (2^-126 <= |x| < 2^128; +-0 below, +-inf above, NaN for NaN) */
static inline DS ds_split(double x) {
  int64_t b;
  std::memcpy(&b, &x, 8);
  const int eb = (int)((b >> 52) & 0x7ff);
  const uint32_t sign = (uint32_t)((uint64_t)b >> 32) & 0x80000000u;
  const uint32_t frac = (uint32_t)((b >> 29) & 0x7fffff);
  const uint32_t hb = eb >= 897 && eb <= 1150 ? sign | ((uint32_t)(eb - 896) << 23) | frac
                      : eb < 897 ? sign
                      : (eb == 2047 && (b & 0xfffffffffffffLL)) ? 0x7fc00000u | sign
                                                                : 0x7f800000u | sign;
  float hf;
  std::memcpy(&hf, &hb, 4);
  float l = 0.0f;
  if (eb >= 949 && eb <= 1150) {
    const int32_t low = (int32_t)(b & 0x1fffffff);
    const float lf = std::fma(ds_small_int(low >> 23), 8388608.0f, ds_small_int(low & 0x7fffff));
    const float mag = lf * bits_f((eb - 948) << 23);
    l = b < 0 ? -mag : mag;
  }
  return {hf, l};
}
static inline int64_t dbits_abs(double x) {
  int64_t b;
  std::memcpy(&b, &x, 8);
  return b & 0x7fffffffffffffffLL;
}
static inline double ds_absmax(double u, double v) {
  const int64_t au = dbits_abs(u), av = dbits_abs(v);
  const int64_t m = au >= av ? au : av;
  double r;
  std::memcpy(&r, &m, 8);
  return r;
}
/* ln(h + l), 2^-120 <= h <= 2^126: h = 2^E m, r = fma(m, c_j, -1) (exact),
 * ln(1+r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - r^3/6 + r^4/7), E ln2 in
 * three parts, + l/h */
static DS ds_log(DS a) {
  const int32_t b = fbits(a.h);
  const int j = (b >> 16) & 127;
  const float m = bits_f((b & 0x007fffff) | 0x3f800000);
  const float r = std::fma(m, kDsLogTab[j][0], -1.0f);
  const float p = r * r, pe = std::fma(r, r, -p);
  float t = std::fma(r, 0x1.24924ap-3f, -0x1.555556p-3f);
  t = std::fma(r, t, 0x1.99999ap-3f);
  t = std::fma(r, t, -0.25f);
  t = std::fma(r, t, 0x1.555556p-2f);
  const float tail = t * (r * p);
  const DS l1 = ds_fast(r, -0.5f * p);
  const DS lp = {l1.h, l1.l + (tail - 0.5f * pe)};
  const float fE = ds_small_int((b >> 23) & 0xff) - 127.0f;
  const float eb = fE * GBODE_DS_LN2_B, ebe = std::fma(fE, GBODE_DS_LN2_B, -eb);
  const DS e0 = ds_fast(fE * GBODE_DS_LN2_A, eb);
  const DS eln2 = ds_fast(e0.h, e0.l + (ebe + fE * GBODE_DS_LN2_C));
  const DS s = ds_add(ds_add(eln2, DS{kDsLogTab[j][1], kDsLogTab[j][2]}), lp);
  return ds_fast(s.h, s.l + a.l * rcp_nr(a.h));
}
/* exp(h + l), |x| < 2.7: k = rint(x 64/ln2), r = x - k ln2/64 (three parts),
 * exp(r) - 1 to degree 5, times 2^((k&63)/64) from the table and 2^(k>>6) */
static DS ds_exp(DS x) {
  if (x.h != x.h) return x;
  const float sh = x.h * GBODE_DS_EXP_INV_L + 12582912.0f;
  const int k = fbits(sh) - 0x4b400000;
  const float kf = sh - 12582912.0f;
  const float r0 = std::fma(-kf, GBODE_DS_EXP_L_A, x.h);
  const float pb = kf * GBODE_DS_EXP_L_B, pbe = std::fma(kf, GBODE_DS_EXP_L_B, -pb);
  const DS rr = ds_two_sum(r0, -pb);
  const DS r = ds_fast(rr.h, rr.l + ((x.l - pbe) - kf * GBODE_DS_EXP_L_C));
  const float p = r.h * r.h, pe = std::fma(r.h, r.h, -p);
  float t = std::fma(r.h, 0x1.111112p-7f, 0x1.555556p-5f);
  t = std::fma(r.h, t, 0x1.555556p-3f);
  const float tail = t * (r.h * p);
  const DS e1 = ds_fast(r.h, 0.5f * p);
  const DS em1 = ds_fast(e1.h, e1.l + ((r.l + 0.5f * pe) + (r.h * r.l + tail)));
  const int j = k & 63;
  const float th = kDsExpTab[j][0], tl = kDsExpTab[j][1];
  const float pp = th * em1.h, ppe = std::fma(th, em1.h, -pp);
  const DS v0 = ds_fast(th, pp);
  const DS v = ds_fast(v0.h, v0.l + (tl + (ppe + std::fma(th, em1.l, tl * em1.h))));
  const float sc = bits_f(((k >> 6) + 127) << 23);
  return {v.h * sc, v.l * sc};
}
/* a single as a double by its bits: exact for normal singles, +-0 for
 * zeros and subnormals */
static inline double f2d_bits(float f) {
  const uint32_t u = (uint32_t)fbits(f);
  const uint32_t e = (u >> 23) & 0xff;
  const uint64_t s = (uint64_t)(u & 0x80000000u) << 32;
  uint64_t r = s;
  if (e != 0) r = s | ((e == 255 ? 0x7ffULL : (uint64_t)(e + 896)) << 52) | ((uint64_t)(u & 0x7fffff) << 29);
  double d;
  std::memcpy(&d, &r, 8);
  return d;
}
/* d (h + l) as fma(d, l, d h) */
static inline double ds_scale(double d, DS x) { return std::fma(d, f2d_bits(x.l), d * f2d_bits(x.h)); }

/* logarithms of the controller constants for the FP64 controller (rounded to double):
 * ln(1/qmax) = ln 0.1, ln(1/qmin) = ln 5, ln gamma = ln 0.9, ln qoldinit = ln 1e-4 */
static const double LN_QMAXI = -0x1.26bb1bbb55516p+1, LN_QMINI = 0x1.9c041f7ed8d33p+0,
                    LN_GAMMA = -0x1.af8e8210a415dp-4, LN_QOLDINIT = -0x1.26bb1bbb55516p+3;

template <class P, class M>
static void solve_adaptive(const oracle_args* a, oracle_out* o, int64_t i) {
  typedef typename P::R R;
  typedef typename P::T T;
  Alg<P> A;
  State<R> st, un;
  load_traj<P>(a, i, A, st);
  const int D = a->dim;
  T t = (T)a->t0;
  const T tf = (T)a->tf;
  T dt = (T)(a->dt0 ? a->dt0[i] : a->dt);
  const R abstol = (R)a->abstol, reltol = (R)a->reltol;
  /* controller constants, build_adaptive_controller_cache(eltype(u0)) */
  const R beta1 = (R)(7.0 / 50.0), beta2 = (R)(2.0 / 25.0), qmax = (R)10.0, qmin = (R)(1.0 / 5.0),
          gamma = (R)(9.0 / 10.0), qoldinit = (R)1.0e-4;
  /* single-precision controller of the device canon */
  const float B1 = (float)(7.0 / 50.0), B2 = (float)(2.0 / 25.0), QMAXI = 0.1f, QMINI = 5.0f,
              GAM = (float)(9.0 / 10.0), QOLDINIT = (float)1.0e-4;
  R qold = qoldinit;
  /* qold^beta2, or in the single-precision modes beta2 * log2(qold) */
  float qoldp = sizeof(R) == sizeof(float) ? B2 * L2_QOLDINIT : oracle_pow::ctrl_pow(QOLDINIT, B2);
  /* FP64 controller of the device canon (a->ctrl == 1): beta2 * log(qold) */
  double lqold = (2.0 / 25.0) * LN_QOLDINIT;
  /* double-single norm and controller (a->ctrl == 0, FP64 solves): beta2 * log(qold) */
  const bool f32 = sizeof(R) == sizeof(float);
  const bool c64 = !f32 && a->ctrl == 1, cds = !f32 && a->ctrl == 0;
  const DS DB1 = {GBODE_DS_B1_H, GBODE_DS_B1_L}, DB2 = {GBODE_DS_B2_H, GBODE_DS_B2_L};
  const DS LQMAXI = {GBODE_DS_LN_QMAXI_H, GBODE_DS_LN_QMAXI_L}, LQMINI = {GBODE_DS_LN_QMINI_H, GBODE_DS_LN_QMINI_L};
  const DS MLGAMMA = {-GBODE_DS_LN_GAMMA_H, -GBODE_DS_LN_GAMMA_L};
  const DS LQOLDINIT = {GBODE_DS_LN_QOLDINIT_H, GBODE_DS_LN_QOLDINIT_L};
  DS lqds = ds_mul(DB2, LQOLDINIT);
  const double dtmin = M::DTMIN_1F7 ? (double)1.0e-7f : 1.0e-14;

  int64_t cur = 0;
  const int64_t P_ = a->saveat ? a->nsave : 0;
  double tmpv[MAXD];
  if (P_ > 0 && (T)a->saveat[0] == (T)a->t0) {
    value_of(st, D, P::KAHAN, tmpv);
    put_us(a, o, i, 0, tmpv);
    cur = 1;
  }
  R k[MAXK][MAXD], e[MAXD];
  if (M::FSAL) A.f(st.hi, (double)t, k[0]);
  int ret = RET_DEFAULT;
  int32_t nacc = 0, nrej = 0;
  put_step(a, o, i, 0, (double)t, st, P::KAHAN);
  int64_t attempts = 0;
  double dt_first = NAN;
  bool saw_nan = false;

  while (t < tf) {
    const State<R> up = st;
    R EEst = (R)INFINITY;
    while (EEst > (R)1) {
      if ((double)dt < dtmin) { ret = RET_DTMIN; goto done; }
      if (a->maxiters > 0 && attempts >= a->maxiters) { ret = RET_MAXITERS; goto done; }
      /* the double-single norm takes the unscaled sum and multiplies by dt itself */
      M::attempt(A, up, t, dt, k, un, e, (P::DEV && cds) ? 2 : 1);
      ++attempts;
      /* error norm: RMS of e ./ (abstol .+ max.(|uprev|, |u|) * reltol); the
       * device canon evaluates it in single precision unless abstol < 1e-30 */
      DS le_ds = {0.0f, 0.0f};
      bool ds_zero = false;
      if (P::DEV && cds) {
        /* double-single: the norm's terms split into single pairs (the
         * double one when abstol < 1e-30), le = ln(EEst); EEst here only
         * drives the attempt loop (2: reject, 0: accept) */
        bool reject;
        if (a->abstol >= 1e-30) {
          const DS dabs = ds_split(a->abstol), drel = ds_split(a->reltol);
          const DS hds = ds_split((double)dt);
          DS acc = {0.0f, 0.0f};
          bool nan_in = dbits_abs((double)dt) > 0x7ff0000000000000LL;
          ds_zero = true;
          for (int d = 0; d < D; ++d) {
            const int64_t eb = dbits_abs((double)e[d]);
            const double mx = ds_absmax((double)up.hi[d], (double)un.hi[d]);
            ds_zero = ds_zero && eb == 0;
            nan_in = nan_in || eb > 0x7ff0000000000000LL || dbits_abs(mx) > 0x7ff0000000000000LL;
            const DS r = ds_div(ds_mul(ds_split((double)e[d]), hds), ds_add(ds_mul(ds_split(mx), drel), dabs));
            acc = d == 0 ? ds_sqr(r) : ds_add(acc, ds_sqr(r));
          }
          const DS av = ds_mul(acc, DS{(float)(1.0 / D), (float)(1.0 / D - (double)(float)(1.0 / D))});
          if (nan_in) {
            saw_nan = true;
            reject = false;
            le_ds = {NAN, 0.0f};
          } else {
            const bool huge = !(av.h <= 0x1p126f);
            reject = huge || ds_gt(av, DS{1.0f, 0.0f});
            const DS ac = huge ? DS{0x1p126f, 0.0f} : av.h < 0x1p-120f ? DS{0x1p-120f, 0.0f} : av;
            const DS lg = ds_log(ac);
            le_ds = {0.5f * lg.h, 0.5f * lg.l};
          }
        } else {
          double acc = 0;
          for (int d = 0; d < D; ++d) {
            const double m = jmax(std::fabs((double)up.hi[d]), std::fabs((double)un.hi[d]));
            const double r = ((double)e[d] * (double)dt) / std::fma(m, a->reltol, a->abstol);
            acc = (d == 0) ? r * r : std::fma(r, r, acc);
          }
          const double E64 = std::sqrt(acc / (double)D);
          ds_zero = E64 == 0.0;
          reject = E64 > 1.0;
          if (E64 != E64) {
            saw_nan = true;
            le_ds = {(float)E64, 0.0f};
          } else {
            le_ds = ds_log(ds_split(std::fmin(std::fmax(E64, 0x1p-60), 0x1p63)));
          }
        }
        EEst = reject ? (R)2 : (R)0;
      } else if (P::DEV && sizeof(R) == sizeof(float)) {
        /* single-precision modes: EEst here holds the mean square a = EEst^2 */
        const float fa = (float)a->abstol, fr = (float)a->reltol;
        float acc = 0;
        for (int d = 0; d < D; ++d) {
          float m = jmax(std::fabs((float)up.hi[d]), std::fabs((float)un.hi[d]));
          float r = (float)e[d] * rcp_nr(std::fma(m, fr, fa));
          acc = (d == 0) ? r * r : std::fma(r, r, acc);
        }
        EEst = (R)(acc * (float)(1.0 / D));
      } else if (P::DEV && a->abstol >= 1e-30) {
        const float fa = (float)a->abstol, fr = (float)a->reltol;
        float acc = 0;
        for (int d = 0; d < D; ++d) {
          float m = jmax(std::fabs((float)up.hi[d]), std::fabs((float)un.hi[d]));
          float r = (float)e[d] / std::fma(m, fr, fa);
          acc = (d == 0) ? r * r : std::fma(r, r, acc);
        }
        EEst = (R)std::sqrt(acc / (float)D);
      } else {
        R acc = 0;
        for (int d = 0; d < D; ++d) {
          R m = jmax(std::fabs(up.hi[d]), std::fabs(un.hi[d]));
          R sc = P::DEV ? fmaX(m, reltol, abstol) : abstol + m * reltol;
          R r = e[d] / sc;
          if (d == 0) acc = r * r;
          else acc = P::DEV ? fmaX(r, r, acc) : acc + r * r;
        }
        EEst = std::sqrt(acc / (R)D);
      }
      if (EEst != EEst) saw_nan = true;

      if (!P::DEV) {
        const bool crp = a->ctrl == 3 && sizeof(R) == sizeof(double);
        R q11 = crp ? (R)gbode::cr_pow((double)EEst, (double)beta1) : std::pow(EEst, beta1);
        R q = (EEst == (R)0) ? (R)1 / qmax
                             : q11 / (crp ? (R)gbode::cr_pow((double)qold, (double)beta2) : std::pow(qold, beta2));
        if (EEst > (R)1) {
          dt = dt / (T)jmin((R)1 / qmin, q11 / gamma);
          ++nrej;
        } else {
          q = fmax_((R)1 / qmax, fmin_((R)1 / qmin, q / gamma));
          qold = jmax(EEst, qoldinit);
          const T dtold = dt;
          dt = dt / (T)q;
          dt = jmin((T)std::fabs(dt), (T)std::fabs(tf - t - dtold));
          const T told = t;
          if ((double)(tf - t - dtold) < dtmin) t = tf;
          else t += dtold;
          if (nacc == 0) dt_first = (double)dtold;
          ++nacc;
          while (cur < P_ && (T)a->saveat[cur] <= t) {
            const T savet = (T)a->saveat[cur];
            const T theta = (savet - told) / dtold;
            M::dense(A, up, told, t, dtold, theta, k, tmpv);
            put_us(a, o, i, cur, tmpv);
            ++cur;
          }
          st = un;
          put_step(a, o, i, nacc, (double)t, st, P::KAHAN);
          if (M::FSAL)
            for (int d = 0; d < D; ++d) k[0][d] = k[6][d];
        }
      } else {
        const float Ef = (float)EEst;
        /* FP64 controller: the reference's factors in double, on logarithms
         * (log_dev, exp_dev), in the kernels' order of operations */
        const double E = (double)EEst;
        const double lE = !c64 ? 0.0
                          : (E != E) ? E
                                     : log_dev(std::fmin(std::fmax(E, 0x1p-1022), 0x1.fffffffffffffp+1023));
        const float l2E = !f32 ? 0.0f : (Ef != Ef) ? Ef : 0.5f * log2_nr(Ef);
        const float q11 = (c64 || cds || f32) ? 0.0f : oracle_pow::ctrl_pow(Ef, B1);
        if (EEst > (R)1) {
          if (f32) {
            const float lf = jmin(L2_QMINI, std::fma(B1, l2E, -L2_GAMMA));
            dt = dt * (T)exp2_nr(-lf);
          } else if (cds) {
            const DS lf = ds_min(LQMINI, ds_add(ds_mul(DB1, le_ds), MLGAMMA));
            dt = (T)ds_scale((double)dt, ds_exp(ds_neg(lf)));
          } else if (c64) {
            const double lf = jmin(LN_QMINI, std::fma(7.0 / 50.0, lE, -LN_GAMMA));
            dt = dt * (T)exp_dev(-lf);
          } else {
            const float fac = jmin(QMINI, q11 / GAM);
            dt = dt * (T)(1.0f / fac);
          }
          ++nrej;
        } else {
          T dtn;
          if (f32) {
            const float lq0 = (EEst == (R)0) ? L2_QMAXI : std::fma(B1, l2E, -qoldp);
            const float lq = fmax_(L2_QMAXI, fmin_(L2_QMINI, lq0 - L2_GAMMA));
            qoldp = B2 * jmax(l2E, L2_QOLDINIT);
            dtn = dt * (T)exp2_nr(-lq);
          } else if (cds) {
            const DS lq0 = ds_zero ? LQMAXI : ds_add(ds_mul(DB1, le_ds), ds_neg(lqds));
            const DS lq = ds_max(LQMAXI, ds_min(LQMINI, ds_add(lq0, MLGAMMA)));
            lqds = ds_mul(DB2, ds_max(le_ds, LQOLDINIT));
            dtn = (T)ds_scale((double)dt, ds_exp(ds_neg(lq)));
          } else if (c64) {
            const double lq0 = (EEst == (R)0) ? LN_QMAXI : std::fma(7.0 / 50.0, lE, -lqold);
            const double lq = fmax_(LN_QMAXI, fmin_(LN_QMINI, lq0 - LN_GAMMA));
            lqold = (2.0 / 25.0) * jmax(lE, LN_QOLDINIT);
            dtn = dt * (T)exp_dev(-lq);
          } else {
            float q = (EEst == (R)0) ? QMAXI : q11 / qoldp;
            q = fmax_(QMAXI, fmin_(QMINI, q / GAM));
            const float qoldf = jmax(Ef, QOLDINIT);
            qoldp = oracle_pow::ctrl_pow(qoldf, B2);
            dtn = dt * (T)(1.0f / q);
          }
          const T dtold = dt;
          dt = jmin((T)std::fabs(dtn), (T)std::fabs(tf - t - dtold));
          const T told = t;
          if ((double)(tf - t - dtold) < dtmin) t = tf;
          else t += dtold;
          if (nacc == 0) dt_first = (double)dtold;
          ++nacc;
          const T inv_dt = recip_dev(dtold);
          while (cur < P_ && (T)a->saveat[cur] <= t) {
            const T savet = (T)a->saveat[cur];
            const T theta = (savet - told) * inv_dt;
            M::dense(A, up, told, t, dtold, theta, k, tmpv);
            put_us(a, o, i, cur, tmpv);
            ++cur;
          }
          st = un;
          put_step(a, o, i, nacc, (double)t, st, P::KAHAN);
          if (M::FSAL)
            for (int d = 0; d < D; ++d) k[0][d] = k[6][d];
        }
      }
    }
  }
done:
  if (ret == RET_DEFAULT && saw_nan) ret = RET_NAN;
  for (; cur < P_; ++cur) {
    for (int d = 0; d < D; ++d) tmpv[d] = NAN;
    put_us(a, o, i, cur, tmpv);
  }
  finish<P>(a, o, i, st, t, ret, nacc, nrej, dt_first);
}

/* Fixed-step driver: gpuatsit5.jl:92-129 / gpuvern7.jl:101-224 / gpuvern9.jl:99-335. */
template <class P, class M>
static void solve_fixed(const oracle_args* a, oracle_out* o, int64_t i) {
  typedef typename P::R R;
  typedef typename P::T T;
  Alg<P> A;
  State<R> st, un;
  load_traj<P>(a, i, A, st);
  const int D = a->dim;
  const T dt = (T)a->dt;
  T t = (T)a->t0;
  int64_t cur = 0;
  const int64_t P_ = a->saveat ? a->nsave : 0;
  double tmpv[MAXD];
  if (P_ > 0 && (T)a->saveat[0] == (T)a->t0) {
    value_of(st, D, P::KAHAN, tmpv);
    put_us(a, o, i, 0, tmpv);
    cur = 1;
  }
  const bool every = (P_ == 0) && a->save_everystep;
  if (every) { value_of(st, D, P::KAHAN, tmpv); put_us(a, o, i, 0, tmpv); }
  R k[MAXK][MAXD], e[MAXD];
  if (M::FSAL) A.f(st.hi, (double)t, k[0]);
  for (int64_t g = 1; g < a->ngrid; ++g) {
    const State<R> up = st;
    t = (T)a->grid[g - 1];
    M::attempt(A, up, t, dt, k, un, e, false);
    t += dt;
    st = un;
    if (every) { value_of(st, D, P::KAHAN, tmpv); put_us(a, o, i, g, tmpv); }
    while (cur < P_ && (T)a->saveat[cur] <= t) {
      const T savet = (T)a->saveat[cur];
      const T theta = (savet - (t - dt)) / dt;
      M::dense(A, up, t - dt, t, dt, theta, k, tmpv);
      put_us(a, o, i, cur, tmpv);
      ++cur;
    }
    if (M::FSAL)
      for (int d = 0; d < D; ++d) k[0][d] = k[6][d];
  }
  for (; cur < P_; ++cur) {
    for (int d = 0; d < D; ++d) tmpv[d] = NAN;
    put_us(a, o, i, cur, tmpv);
  }
  const int32_t steps = a->ngrid > 0 ? (int32_t)(a->ngrid - 1) : 0;
  finish<P>(a, o, i, st, t, RET_DEFAULT, steps, 0, steps > 0 ? (double)dt : NAN);
}

/* GPUSimpleEuler, src/euler/gpueuler.jl:67-76: k1 = f(u, p, ts[i]) (the END
 * of the step, as in GPUSimpleRK4) and u = uprev + dt*k1, @muladd of a
 * vector: fused in the device canon, a multiply and an add in the reference. */
template <class P>
struct Euler {
  typedef typename P::R R;
  typedef typename P::T T;
  static void step(const Alg<P>& A, const State<R>& up, T t, T dt, State<R>& u) {
    R k1[MAXD];
    const R h = (R)dt;
    A.f(up.hi, (double)t, k1);
    if (P::DEV) {
      State<R> tmpu;
      state_update<P>(A.D, up, h, k1, tmpu);
      u = tmpu;
    } else {
      for (int d = 0; d < A.D; ++d) { u.hi[d] = h * k1[d] + up.hi[d]; u.c[d] = 0; }
    }
  }
};

/* GPUSimpleRK4, gpurk4.jl:53-98, and GPUSimpleEuler, gpueuler.jl:53-90 (S =
 * RK4 or Euler): one step per grid point, every grid point saved (us[1] = u0). */
template <class P, class S>
static void solve_onestep(const oracle_args* a, oracle_out* o, int64_t i) {
  typedef typename P::R R;
  typedef typename P::T T;
  Alg<P> A;
  State<R> st, un;
  load_traj<P>(a, i, A, st);
  const T dt = (T)a->dt;
  double tmpv[MAXD];
  const bool every = a->save_everystep != 0;
  if (every) { value_of(st, a->dim, P::KAHAN, tmpv); put_us(a, o, i, 0, tmpv); }
  T t = (T)a->t0;
  for (int64_t g = 1; g < a->ngrid; ++g) {
    t = (T)a->grid[g];
    S::step(A, st, t, dt, un);
    st = un;
    if (every) { value_of(st, a->dim, P::KAHAN, tmpv); put_us(a, o, i, g, tmpv); }
  }
  const int32_t steps = a->ngrid > 0 ? (int32_t)(a->ngrid - 1) : 0;
  finish<P>(a, o, i, st, t, RET_DEFAULT, steps, 0, steps > 0 ? (double)dt : NAN);
}

/* SimpleATsit5 in integrator form (src/tsit5/atsit5.jl), double precision:
 * simpleatsit5_init :181-196, OOP step! :322-413, interpolation :705-732 and
 * the saveat loop of __solve :140-161. */
struct SAT5I {
  double uprev[MAXD], u[MAXD], tprev, t, tf, dt, dtnew, qold, abstol, reltol;
  double ks[7][MAXD];
  bool u_modified;
};

template <class P>
static int simple_atsit5_step(const Alg<P>& A, SAT5I& it, int64_t& attempts, int64_t maxiters,
                              int32_t& nacc, int32_t& nrej, double& dt_first, bool& saw_nan) {
  const int D = A.D;
  const double beta1 = 7.0 / 50.0, beta2 = 2.0 / 25.0, qmax = 10.0, qmin = 1.0 / 5.0, gamma = 9.0 / 10.0,
               qoldinit = 1.0e-4;
  double dt = it.dtnew;
  const double t = it.t;
  for (int d = 0; d < D; ++d) it.uprev[d] = it.u[d];
  double k[MAXK][MAXD];
  if (it.u_modified) {
    A.f(it.uprev, t, k[0]);
    it.u_modified = false;
  } else {
    for (int d = 0; d < D; ++d) k[0][d] = it.ks[6][d];
  }
  State<double> up, un;
  for (int d = 0; d < D; ++d) { up.hi[d] = it.uprev[d]; up.c[d] = 0; }
  double e[MAXD];
  double EEst = INFINITY;
  double qold = it.qold;
  while (EEst > 1) {
    if (dt < 1.0e-14) return RET_DTMIN;
    if (maxiters > 0 && attempts >= maxiters) return RET_MAXITERS;
    Tsit5<P>::attempt(A, up, t, dt, k, un, e, true);
    ++attempts;
    double acc = 0;
    for (int d = 0; d < D; ++d) {
      double m = jmax(std::fabs(it.uprev[d]), std::fabs(un.hi[d]));
      double sc = P::DEV ? std::fma(m, it.reltol, it.abstol) : it.abstol + m * it.reltol;
      double r = e[d] / sc;
      acc = (d == 0) ? r * r : (P::DEV ? std::fma(r, r, acc) : acc + r * r);
    }
    EEst = std::sqrt(acc / (double)D);
    if (EEst != EEst) saw_nan = true;
    double q11 = std::pow(EEst, beta1);
    double q = (EEst == 0) ? 1.0 / qmax : q11 / std::pow(qold, beta2);
    if (EEst > 1) {
      dt = dt / jmin(1.0 / qmin, q11 / gamma);
      ++nrej;
    } else {
      q = fmax_(1.0 / qmax, fmin_(1.0 / qmin, q / gamma));
      qold = jmax(EEst, qoldinit);
      double dtnew = dt / q;
      dtnew = jmin(std::fabs(dtnew), std::fabs(it.tf - t - dt));
      for (int j = 0; j < 7; ++j)
        for (int d = 0; d < D; ++d) it.ks[j][d] = k[j][d];
      it.dt = dt;
      it.dtnew = dtnew;
      it.qold = qold;
      it.tprev = t;
      for (int d = 0; d < D; ++d) it.u[d] = un.hi[d];
      if ((it.tf - t - dt) < 1.0e-14) it.t = it.tf;
      else it.t += dt;
      if (nacc == 0) dt_first = dt;
      ++nacc;
    }
  }
  return RET_DEFAULT;
}

template <class P>
static void solve_simple_atsit5(const oracle_args* a, oracle_out* o, int64_t i) {
  Alg<P> A;
  State<double> st;
  load_traj<P>(a, i, A, st);
  const int D = a->dim;
  SAT5I it;
  for (int d = 0; d < D; ++d) { it.u[d] = st.hi[d]; it.uprev[d] = st.hi[d]; }
  it.t = it.tprev = a->t0;
  it.tf = a->tf;
  it.dt = it.dtnew = a->dt0 ? a->dt0[i] : a->dt;
  it.qold = 1.0e-4;
  it.abstol = a->abstol;
  it.reltol = a->reltol;
  it.u_modified = true;
  int64_t cur = 0, attempts = 0;
  const int64_t P_ = a->saveat ? a->nsave : 0;
  double tmpv[MAXD];
  if (P_ > 0 && a->saveat[0] == a->t0) { put_us(a, o, i, 0, it.u); cur = 1; }
  int ret = RET_DEFAULT;
  int32_t nacc = 0, nrej = 0;
  double dt_first = NAN;
  bool saw_nan = false;
  while (it.t < a->tf) {
    ret = simple_atsit5_step<P>(A, it, attempts, a->maxiters, nacc, nrej, dt_first, saw_nan);
    if (ret != RET_DEFAULT) break;
    while (cur < P_ && a->saveat[cur] <= it.t) {
      /* integ(t): θ = (t - tprev)/dt, u = uprev + dt * Σ bθ_i ks_i */
      const double theta = (a->saveat[cur] - it.tprev) / it.dt;
      double b[7], s[MAXD];
      tsit5_btheta<P::DEV, double>(theta, b);
      for (int d = 0; d < D; ++d) s[d] = b[0] * it.ks[0][d];
      for (int j = 1; j < 7; ++j)
        for (int d = 0; d < D; ++d) s[d] = vmadd<P::DEV>(b[j], it.ks[j][d], s[d]);
      for (int d = 0; d < D; ++d) tmpv[d] = vmadd<P::DEV>(it.dt, s[d], it.uprev[d]);
      put_us(a, o, i, cur, tmpv);
      ++cur;
    }
  }
  if (ret == RET_DEFAULT && saw_nan) ret = RET_NAN;
  for (; cur < P_; ++cur) {
    for (int d = 0; d < D; ++d) tmpv[d] = NAN;
    put_us(a, o, i, cur, tmpv);
  }
  for (int d = 0; d < D; ++d) st.hi[d] = it.u[d];
  finish<P>(a, o, i, st, it.t, ret, nacc, nrej, dt_first);
}

/* SimpleTsit5 __solve (src/tsit5/tsit5.jl:84-122) with the OOP step! of :303-352;
 * t accumulates with integ.t += dt.  Only the final state is reported. */
template <class P>
static void solve_simple_tsit5(const oracle_args* a, oracle_out* o, int64_t i) {
  typedef typename P::R R;
  typedef typename P::T T;
  Alg<P> A;
  State<R> st;
  load_traj<P>(a, i, A, st);
  const int D = a->dim;
  const int64_t L = a->ngrid;
  const bool ends_at_tf = L > 0 && a->grid[L - 1] == a->tf;
  const int64_t n = ends_at_tf ? L : L + 1;
  T t = (T)a->t0, dt = (T)a->dt;
  R k[MAXK][MAXD], tmp[MAXD], s[MAXD];
  bool u_modified = true;
  auto step = [&](T h_) {
    const R h = (R)h_;
    R uprev[MAXD];
    for (int d = 0; d < D; ++d) uprev[d] = st.hi[d];
    if (u_modified) { A.f(uprev, (double)t, k[0]); u_modified = false; }
    else for (int d = 0; d < D; ++d) k[0][d] = k[6][d];
    const R a21 = (R)(h_ * (T)t5::a21);
    for (int d = 0; d < D; ++d)
      tmp[d] = P::DEV ? fmaX(a21, k[0][d], uprev[d]) : h * ((R)t5::a21 * k[0][d]) + uprev[d];
    A.f(tmp, (double)A.st(t, t5::c1, h_), k[1]);
    A.lc(T5_S3, 2, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, t5::c2, h_), k[2]);
    A.lc(T5_S4, 3, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, t5::c3, h_), k[3]);
    A.lc(T5_S5, 4, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)A.st(t, t5::c4, h_), k[4]);
    A.lc(T5_S6, 5, k, s); A.axpy(uprev, h, s, tmp); A.f(tmp, (double)(t + h_), k[5]);
    /* ((a71 k1 + .. + a74 k4) + a75 k5 + a76 k6) */
    A.lc(T5_U_IN, 4, k, s);
    for (int d = 0; d < D; ++d) {
      R acc = vmadd<P::DEV>((R)t5::a75, k[4][d], s[d]);
      s[d] = vmadd<P::DEV>((R)t5::a76, k[5][d], acc);
      st.hi[d] = vmadd<P::DEV>(h, s[d], uprev[d]);
    }
    A.f(st.hi, (double)(t + h_), k[6]);
    t += h_;
  };
  for (int64_t g = 1; g <= n - 1; ++g) step(dt);
  if (!ends_at_tf) {
    step((T)a->tf - t);
    t = (T)a->tf;  /* push!(ts, tspan[2]) */
  }
  const int32_t steps = (int32_t)(ends_at_tf ? n - 1 : n);
  finish<P>(a, o, i, st, t, RET_DEFAULT, steps, 0, (double)dt);
}

/* ---------------------------------------------------------------- dispatch */
template <class P>
static void solve_range(const oracle_args* a, oracle_out* o, int64_t i0, int64_t i1) {
  for (int64_t i = i0; i < i1; ++i) {
    switch (a->alg) {
      case ORACLE_RK4: solve_onestep<P, RK4<P>>(a, o, i); break;
      case ORACLE_EULER: solve_onestep<P, Euler<P>>(a, o, i); break;
      case ORACLE_TSIT5: solve_fixed<P, Tsit5<P>>(a, o, i); break;
      case ORACLE_ATSIT5: solve_adaptive<P, Tsit5<P>>(a, o, i); break;
      case ORACLE_VERN7: solve_fixed<P, Vern7<P>>(a, o, i); break;
      case ORACLE_AVERN7: solve_adaptive<P, Vern7<P>>(a, o, i); break;
      case ORACLE_VERN9: solve_fixed<P, Vern9<P, false>>(a, o, i); break;
      case ORACLE_AVERN9: solve_adaptive<P, Vern9<P, true>>(a, o, i); break;
      case ORACLE_SIMPLE_TSIT5: solve_simple_tsit5<P>(a, o, i); break;
      default: break;
    }
  }
}

template <bool DEV>
static void solve_range_prec(const oracle_args* a, oracle_out* o, int64_t i0, int64_t i1) {
  if (a->alg == ORACLE_SIMPLE_ATSIT5) {
    for (int64_t i = i0; i < i1; ++i) solve_simple_atsit5<Pol<double, double, false, DEV>>(a, o, i);
    return;
  }
  switch (a->precision) {
    case ORACLE_FP64: solve_range<Pol<double, double, false, DEV>>(a, o, i0, i1); break;
    case ORACLE_FP32: solve_range<Pol<float, float, false, DEV>>(a, o, i0, i1); break;
    case ORACLE_FP32_KAHAN: solve_range<Pol<float, double, true, DEV>>(a, o, i0, i1); break;
    default: break;
  }
}

}  // namespace

extern "C" int oracle_solve(const oracle_args* a, oracle_out* o) {
  if (!a || !o || a->n < 0 || a->dim < 1 || a->dim > MAXD || a->nparams < 0 || a->nparams > MAXP) return -1;
  if (a->alg < 0 || a->alg > ORACLE_EULER) return -1;
  if (a->alg == ORACLE_SIMPLE_ATSIT5 && a->precision != ORACLE_FP64) return -1;
  if (a->precision == ORACLE_FP32_KAHAN && a->rounding != ORACLE_ROUND_DEVICE) return -1;
  const bool fixed = a->alg == ORACLE_RK4 || a->alg == ORACLE_TSIT5 || a->alg == ORACLE_VERN7 ||
                     a->alg == ORACLE_VERN9 || a->alg == ORACLE_SIMPLE_TSIT5 || a->alg == ORACLE_EULER;
  if (fixed && (!a->grid || a->ngrid < 1)) return -1;
  if (a->rhs == ORACLE_R3BP && a->dim != 4) return -1;
  if (a->rhs == ORACLE_LORENZ && a->dim != 3) return -1;
  if (a->rhs == ORACLE_VDP && a->dim != 2) return -1;
  int nt = a->nthreads > 0 ? a->nthreads : 1;
  if ((int64_t)nt > a->n) nt = (int)std::max<int64_t>(1, a->n);
  auto run = [&](int64_t i0, int64_t i1) {
    g_cr_trig = a->rounding != ORACLE_ROUND_DEVICE && a->ctrl == 3;
    if (a->rounding == ORACLE_ROUND_DEVICE) solve_range_prec<true>(a, o, i0, i1);
    else solve_range_prec<false>(a, o, i0, i1);
  };
  if (nt == 1) {
    run(0, a->n);
    return 0;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (a->n + nt - 1) / nt;
  for (int w = 0; w < nt; ++w) {
    int64_t i0 = w * chunk, i1 = std::min<int64_t>(a->n, i0 + chunk);
    if (i0 >= i1) break;
    th.emplace_back(run, i0, i1);
  }
  for (auto& x : th) x.join();
  return 0;
}

/* ---------------------------------------------------------------- SimpleEM */
namespace {

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11): 10 rounds of two 32x32->64 multiplies and a key bump. */
void philox(const uint32_t* cin, const uint32_t* kin, uint32_t* out) {
  uint32_t c0 = cin[0], c1 = cin[1], c2 = cin[2], c3 = cin[3], k0 = kin[0], k1 = kin[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* log of a positive normal double, device canon (table-driven, Tang 1990):
 * x = 2^e m, m in [1, 2), row j = top 7 fraction bits of log_table.h;
 * log x = e' ln2 + T_j + log1p(r), r = fma(m, 1/F_j, -1), e' = e + [j >= 53],
 * log1p(r) = r + r^2 q(r) with the Taylor coefficients -1/2 .. -1/8. */
double log_dev(double x) {
  uint64_t b;
  std::memcpy(&b, &x, 8);
  const int j = (int)((b >> 45) & 127);
  const int e = (int)((b >> 52) & 0x7ff) - 1023 + (j >= GBODE_LOGTAB_SHIFT_FROM ? 1 : 0);
  const uint64_t mb = (b & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
  double m;
  std::memcpy(&m, &mb, 8);
  const double r = std::fma(m, kLogTab[j][0], -1.0);
  double q = -1.0 / 8.0;
  for (int k = 7; k >= 2; --k) q = std::fma(q, r, (k & 1 ? 1.0 : -1.0) / (double)k);
  const double l1p = std::fma(r * r, q, r);
  const double de = (double)e;
  return std::fma(de, 0x1.62e42fefa38p-1, kLogTab[j][1]) + (std::fma(de, 0x1.ef35793c7673p-45, kLogTab[j][2]) + l1p);
}

/* exp of a double with |x| < 700, device canon (table-driven, Tang 1989):
 * n = round(x 32/ln2) via the 1.5*2^52 shifter, r = x - n ln2/32 (two parts),
 * exp(r) - 1 = r + r^2 q(r) with the Taylor coefficients 1/2 .. 1/720,
 * 2^(j/32) = lead + trail from exp_table.h, scaled by 2^m. */
double exp_dev(double x) {
  const double t = std::fma(x, GBODE_EXP_INV_L, 0x1.8p52);
  int64_t tb;
  std::memcpy(&tb, &t, 8);
  const int n = (int)(tb - 0x4338000000000000LL);
  const double nd = t - 0x1.8p52;
  const double r = std::fma(-nd, GBODE_EXP_L_TRAIL, std::fma(-nd, GBODE_EXP_L_LEAD, x));
  double q = std::fma(r, 1.0 / 720.0, 1.0 / 120.0);
  q = std::fma(q, r, 1.0 / 24.0);
  q = std::fma(q, r, 1.0 / 6.0);
  q = std::fma(q, r, 0.5);
  const double p = std::fma(r * r, q, r);
  const int j = n & 31, m = n >> 5;
  const double lead = kExpTab[j][0], trail = kExpTab[j][1];
  const double v = lead + std::fma(lead, p, std::fma(trail, p, trail));
  const int64_t sb = (int64_t)(m + 1023) << 52;
  double sc;
  std::memcpy(&sc, &sb, 8);
  return v * sc;
}

/* normals z_{2P}, z_{2P+1} of trajectory idx's stream: Philox counter
 * (P low, P high, idx low, idx high), key = seed, then Box-Muller */
/* the SDE normals in double-single arithmetic (kernels: sde_solver.cuh's
 * normal_pair): v 2^-e from an integer's top 24 and next 24 bits; sqrt by
 * rsqrt_nr and one correction; sin and cos of |r| <= pi/4 by Taylor series */
static DS ds_from_u64(uint64_t v, int e) {
  const int z = __builtin_clzll(v);
  const uint64_t m = v << z;
  const float hi = (float)(uint32_t)(m >> 40) * bits_f((40 - z - e + 127) << 23);
  const float lo = (float)(uint32_t)((m >> 16) & 0xffffff) * bits_f((16 - z - e + 127) << 23);
  return {hi, lo};
}
static DS ds_sqrt(DS y) {
  if (!(y.h > 0.0f)) return {0.0f, 0.0f};
  const float r = rsqrt_nr_f(y.h);
  const float sq = y.h * r;
  const float p = sq * sq, pe = std::fma(sq, sq, -p);
  return ds_fast(sq, (((y.h - p) - pe) + y.l) * (0.5f * r));
}
static void ds_sincos_reduced(DS r, DS* sn, DS* cs) {
  const DS r2 = ds_sqr(r);
  float ts = std::fma(r2.h, GBODE_DS_SIN_T7, GBODE_DS_SIN_T6);
  ts = std::fma(r2.h, ts, GBODE_DS_SIN_T5);
  DS ps = {ts, 0.0f};
  ps = ds_add(ds_mul(ps, r2), DS{GBODE_DS_SIN_C4_H, GBODE_DS_SIN_C4_L});
  ps = ds_add(ds_mul(ps, r2), DS{GBODE_DS_SIN_C3_H, GBODE_DS_SIN_C3_L});
  ps = ds_add(ds_mul(ps, r2), DS{GBODE_DS_SIN_C2_H, GBODE_DS_SIN_C2_L});
  ps = ds_add(ds_mul(ps, r2), DS{GBODE_DS_SIN_C1_H, GBODE_DS_SIN_C1_L});
  ps = ds_add(ds_mul(ps, r2), DS{1.0f, 0.0f});
  *sn = ds_mul(r, ps);
  float tc = std::fma(r2.h, GBODE_DS_COS_T8, GBODE_DS_COS_T7);
  tc = std::fma(r2.h, tc, GBODE_DS_COS_T6);
  tc = std::fma(r2.h, tc, GBODE_DS_COS_T5);
  DS pc = {tc, 0.0f};
  pc = ds_add(ds_mul(pc, r2), DS{GBODE_DS_COS_C4_H, GBODE_DS_COS_C4_L});
  pc = ds_add(ds_mul(pc, r2), DS{GBODE_DS_COS_C3_H, GBODE_DS_COS_C3_L});
  pc = ds_add(ds_mul(pc, r2), DS{GBODE_DS_COS_C2_H, GBODE_DS_COS_C2_L});
  pc = ds_add(ds_mul(pc, r2), DS{GBODE_DS_COS_C1_H, GBODE_DS_COS_C1_L});
  *cs = ds_add(ds_mul(pc, r2), DS{1.0f, 0.0f});
}
static inline double ds_to_double(DS x) { return f2d_bits(x.h) + f2d_bits(x.l); }

/* normals z_{2P}, z_{2P+1} of trajectory idx's stream: Philox counter
 * (P low, P high, idx low, idx high), key = seed; u1 = (a + 1) 2^-53, u2 =
 * c 2^-53; r = sqrt(-2 ln u1); angle 2 pi u2 = (k + f) pi/2 with k =
 * round(4 u2) (half up) and f exact in integers; (r cos, r sin) */
void normal_pair(uint64_t seed, int64_t P, int64_t idx, double* z0, double* z1) {
  const uint32_t c[4] = {(uint32_t)P, (uint32_t)((uint64_t)P >> 32), (uint32_t)idx, (uint32_t)((uint64_t)idx >> 32)};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t r[4];
  philox(c, key, r);
  const uint64_t a = ((uint64_t)(r[0] >> 5) << 26) | (r[1] >> 6);
  const uint64_t cc = ((uint64_t)(r[2] >> 5) << 26) | (r[3] >> 6);
  const DS lg = ds_log(ds_from_u64(a + 1, 53));
  const DS rad = ds_sqrt(DS{-2.0f * lg.h, -2.0f * lg.l});
  const uint64_t k = (cc + (1ULL << 50)) >> 51;
  const int64_t fi = (int64_t)cc - (int64_t)(k << 51);
  DS f = {0.0f, 0.0f};
  if (fi != 0) {
    f = ds_from_u64((uint64_t)(fi < 0 ? -fi : fi), 51);
    if (fi < 0) f = ds_neg(f);
  }
  DS sr, cr;
  ds_sincos_reduced(ds_mul(f, DS{GBODE_DS_PIO2_H, GBODE_DS_PIO2_L}), &sr, &cr);
  const int q = (int)(k & 3);
  const DS sn = q == 0 ? sr : q == 1 ? cr : q == 2 ? ds_neg(sr) : ds_neg(cr);
  const DS cs = q == 0 ? cr : q == 1 ? ds_neg(sr) : q == 2 ? ds_neg(cr) : sr;
  *z0 = ds_to_double(ds_mul(rad, cs));
  *z1 = ds_to_double(ds_mul(rad, sn));
}

/* the same pair in the reference's rounding: the 53-bit uniforms as doubles
 * and the Box-Muller transform with libm's log, sqrt, sin and cos (as a
 * Float64 randn built from these uniforms would compute it) */
void normal_pair_ref(uint64_t seed, int64_t P, int64_t idx, double* z0, double* z1) {
  const uint32_t c[4] = {(uint32_t)P, (uint32_t)((uint64_t)P >> 32), (uint32_t)idx, (uint32_t)((uint64_t)idx >> 32)};
  const uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t r[4];
  philox(c, key, r);
  const uint64_t a = ((uint64_t)(r[0] >> 5) << 26) | (r[1] >> 6);
  const uint64_t cc = ((uint64_t)(r[2] >> 5) << 26) | (r[3] >> 6);
  const double u1 = (double)(a + 1) * 0x1.0p-53;
  const double u2 = (double)cc * 0x1.0p-53;
  const double rad = std::sqrt(-2.0 * std::log(u1));
  const double ang = 2.0 * M_PI * u2;
  *z0 = rad * std::cos(ang);
  *z1 = rad * std::sin(ang);
}

constexpr int MAXM = 16;  /* noise dimensions of a non-diagonal SDE */

/* drift and diffusion of the built-in SDEs (g: dim values for diagonal noise,
 * the row-major dim x noise_dim matrix otherwise); the Lorenz drift in the
 * REF/DEV forms of rhs_eval */
void sde_fg(const oracle_sde_args* a, bool dev, const double* u, const double* p, double* f, double* g) {
  const int D = a->dim, M = a->noise_dim;
  switch (a->sde) {
    case ORACLE_SDE_MULT:
      for (int d = 0; d < D; ++d) {
        f[d] = p[0] * u[d];
        for (int m = 0; m < M; ++m) g[d * M + m] = p[1 + d * M + m] * u[d];
      }
      break;
    case ORACLE_SDE_GBM:
      for (int d = 0; d < D; ++d) { f[d] = p[0] * u[d]; g[d] = p[1] * u[d]; }
      break;
    case ORACLE_SDE_OU:
      for (int d = 0; d < D; ++d) { f[d] = p[0] * (p[1] - u[d]); g[d] = p[2]; }
      break;
    default:
      f[0] = p[0] * (u[1] - u[0]);
      if (dev) {
        f[1] = std::fma(u[0], p[1] - u[2], -u[1]);
        f[2] = std::fma(u[0], u[1], -(p[2] * u[2]));
      } else {
        f[1] = u[0] * (p[1] - u[2]) - u[1];
        f[2] = u[0] * u[1] - p[2] * u[2];
      }
      for (int d = 0; d < 3; ++d) g[d] = p[3];
  }
}

/* xi[0..N) = z_{kN} .. z_{kN+N-1} of trajectory i's normal stream; a pair
 * that straddles two steps is drawn once, its second normal kept in carry;
 * device rounding: the kernels' double-single normals, reference rounding:
 * libm's */
void step_normals(uint64_t seed, int64_t k, int N, int64_t i, double* xi, double* carry, bool dev) {
  for (int d = 0; d < N; ++d) {
    const int64_t gi = k * N + d;
    if (d == 0 && (gi & 1)) {
      xi[0] = *carry;
      continue;
    }
    if (gi & 1) continue;  /* filled with its pair */
    double z1;
    if (dev) normal_pair(seed, gi / 2, i, &xi[d], &z1);
    else normal_pair_ref(seed, gi / 2, i, &xi[d], &z1);
    if (d + 1 < N) xi[d + 1] = z1;
    else *carry = z1;
  }
}

/* src/euler_maruyama.jl:66-91 (diagonal) and :126-134 (non-diagonal) for
 * trajectory i: t_k = t0 + k dt (scalar muladd).  Diagonal noise:
 * u += f dt + sqrt(dt) g .* xi, REF rounding (u + f dt) + (sqdt g) xi with a
 * separate multiply and add each, DEV fma(sqdt g, xi, fma(f, dt, u)).
 * Non-diagonal noise (M normals a step): s = G xi (left to right; DEV with
 * fmas), u += f dt + sqrt(dt) s, REF (u + f dt) + sqdt s, DEV
 * fma(sqdt, s, fma(f, dt, u)). */
void solve_em(const oracle_sde_args* a, int64_t i) {
  const int D = a->dim, M = a->noise_dim;
  const bool dev = a->rounding == ORACLE_ROUND_DEVICE;
  double u[MAXD], p[MAXP], f[MAXD], g[MAXD * MAXM], xi[MAXM + MAXD + 1];
  for (int q = 0; q < a->nparams; ++q) p[q] = a->p[q * a->n + i];
  for (int d = 0; d < D; ++d) u[d] = a->u0[d * a->n + i];
  if (a->us)
    for (int d = 0; d < D; ++d) a->us[d * a->n + i] = u[d];
  const double sqdt = std::sqrt(a->dt);
  double carry = 0.0;
  for (int64_t k = 0; k < a->nsteps; ++k) {
    const double t = std::fma((double)k, a->dt, a->t0);
    (void)t;  /* the built-in SDEs are autonomous */
    sde_fg(a, dev, u, p, f, g);
    /* step k takes the next D (diagonal) or M normals of the stream */
    step_normals(a->seed, k, M > 0 ? M : D, i, xi, &carry, dev);
    for (int d = 0; d < D; ++d) {
      if (M > 0) {
        double s = g[d * M] * xi[0];
        for (int m = 1; m < M; ++m) s = dev ? std::fma(g[d * M + m], xi[m], s) : s + g[d * M + m] * xi[m];
        u[d] = dev ? std::fma(sqdt, s, std::fma(f[d], a->dt, u[d])) : (u[d] + f[d] * a->dt) + sqdt * s;
      } else {
        const double sg = sqdt * g[d];
        u[d] = dev ? std::fma(sg, xi[d], std::fma(f[d], a->dt, u[d])) : (u[d] + f[d] * a->dt) + sg * xi[d];
      }
    }
    if (a->us)
      for (int d = 0; d < D; ++d) a->us[((k + 1) * D + d) * a->n + i] = u[d];
  }
  if (a->u_final)
    for (int d = 0; d < D; ++d) a->u_final[d * a->n + i] = u[d];
}

}  // namespace

extern "C" int oracle_sde_solve(const oracle_sde_args* a) {
  if (!a || a->n < 0 || a->dim < 1 || a->dim > MAXD || a->nparams < 0 || a->nparams > MAXP || a->nsteps < 0)
    return -1;
  if (a->sde == ORACLE_SDE_GBM && a->nparams != 2) return -1;
  if (a->sde == ORACLE_SDE_OU && a->nparams != 3) return -1;
  if (a->sde == ORACLE_SDE_LORENZ && (a->dim != 3 || a->nparams != 4)) return -1;
  if (a->sde < 0 || a->sde > ORACLE_SDE_MULT) return -1;
  if (a->noise_dim < 0 || a->noise_dim > MAXM || (a->noise_dim > 0) != (a->sde == ORACLE_SDE_MULT)) return -1;
  if (a->sde == ORACLE_SDE_MULT && a->nparams != 1 + a->dim * a->noise_dim) return -1;
  int nt = a->nthreads > 0 ? a->nthreads : 1;
  if ((int64_t)nt > a->n) nt = (int)std::max<int64_t>(1, a->n);
  auto run = [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) solve_em(a, i);
  };
  std::vector<std::thread> th;
  const int64_t chunk = (a->n + nt - 1) / nt;
  for (int w = 0; w < nt; ++w) {
    const int64_t i0 = w * chunk, i1 = std::min<int64_t>(a->n, i0 + chunk);
    if (i0 >= i1) break;
    th.emplace_back(run, i0, i1);
  }
  for (auto& x : th) x.join();
  return 0;
}

extern "C" void oracle_philox(const uint32_t* c, const uint32_t* k, uint32_t* out) { philox(c, k, out); }
extern "C" double oracle_log(double x) { return log_dev(x); }
extern "C" double oracle_exp(double x) { return exp_dev(x); }
/* the single-precision modes' reciprocal, log2 and exp2 of the device canon */
extern "C" float oracle_rcp_nr(float x) { return rcp_nr(x); }
extern "C" void oracle_ds_log(float h, float l, float* out) {
  const DS r = ds_log(DS{h, l});
  out[0] = r.h; out[1] = r.l;
}
extern "C" void oracle_ds_exp(float h, float l, float* out) {
  const DS r = ds_exp(DS{h, l});
  out[0] = r.h; out[1] = r.l;
}
extern "C" void oracle_ds_split(double x, float* out) {
  const DS r = ds_split(x);
  out[0] = r.h; out[1] = r.l;
}
extern "C" float oracle_log2_nr(float x) { return log2_nr(x); }
extern "C" float oracle_exp2_nr(float x) { return exp2_nr(x); }
/* the single-precision R3BP pull mu / r^(3/2) of the device canon */
extern "C" float oracle_r3bp_pull_f(float mu, float r) { return r3bp_pull_dev(mu, r); }
extern "C" void oracle_normal_pair(uint64_t seed, int64_t pair, int64_t idx, double* z0, double* z1) {
  normal_pair(seed, pair, idx, z0, z1);
}

extern "C" float oracle_ctrl_pow(float x, float b) { return oracle_pow::ctrl_pow(x, b); }
extern "C" void oracle_sincos(double x, double* s, double* c) { sincos_dev(x, s, c); }

/* Reference forward and backward pass of the learned-schedule MLP, in double
 * precision, for checking the device training kernel's gradients.
 * Layout W1[nh][nin] b1[nh] W2[nh][nh] b2[nh] W3[2][nh] b3[2];
 * loss = (1/batch) sum_b sum_o (out_bo - y_bo)^2. */
extern "C" int oracle_mlp_forward_backward(int nin, int nh, int64_t batch, const float* prm, const float* x,
                                           const float* y, float* grad, float* loss) {
  if (nin < 1 || nh < 1 || batch < 1) return -1;
  const int w1 = 0, b1 = nh * nin, w2 = b1 + nh, b2 = w2 + nh * nh, w3 = b2 + nh, b3 = w3 + 2 * nh;
  const int np = b3 + 2;
  std::vector<double> g(np, 0.0), a1(nh), a2(nh), d1(nh), d2(nh);
  double L = 0;
  for (int64_t s = 0; s < batch; ++s) {
    const float* xs = x + s * nin;
    for (int j = 0; j < nh; ++j) {
      double acc = prm[b1 + j];
      for (int f = 0; f < nin; ++f) acc += (double)prm[w1 + j * nin + f] * xs[f];
      a1[j] = acc > 0 ? acc : 0;
    }
    for (int j = 0; j < nh; ++j) {
      double acc = prm[b2 + j];
      for (int k = 0; k < nh; ++k) acc += (double)prm[w2 + j * nh + k] * a1[k];
      a2[j] = acc > 0 ? acc : 0;
    }
    double dout[2];
    for (int q = 0; q < 2; ++q) {
      double acc = prm[b3 + q];
      for (int k = 0; k < nh; ++k) acc += (double)prm[w3 + q * nh + k] * a2[k];
      const double e = acc - y[s * 2 + q];
      L += e * e / batch;
      dout[q] = 2 * e / batch;
      g[b3 + q] += dout[q];
      for (int k = 0; k < nh; ++k) g[w3 + q * nh + k] += dout[q] * a2[k];
    }
    for (int j = 0; j < nh; ++j) {
      double acc = 0;
      for (int q = 0; q < 2; ++q) acc += (double)prm[w3 + q * nh + j] * dout[q];
      d2[j] = a2[j] > 0 ? acc : 0;
      g[b2 + j] += d2[j];
      for (int k = 0; k < nh; ++k) g[w2 + j * nh + k] += d2[j] * a1[k];
    }
    for (int k = 0; k < nh; ++k) {
      double acc = 0;
      for (int j = 0; j < nh; ++j) acc += (double)prm[w2 + j * nh + k] * d2[j];
      d1[k] = a1[k] > 0 ? acc : 0;
      g[b1 + k] += d1[k];
      for (int f = 0; f < nin; ++f) g[w1 + k * nin + f] += d1[k] * xs[f];
    }
  }
  for (int i = 0; i < np; ++i) grad[i] = (float)g[i];
  *loss = (float)L;
  return 0;
}

/* The same forward and backward pass in the rounding of the device training
 * kernel (simplediffeq.jl_gb300/csrc/learn.cu): every matrix product takes
 * bfloat16 operands -- parameters, features, activations, output deltas --
 * and accumulates in fp32 (here: in double, rounded to float once, which the
 * fp32 tensor-core accumulation approaches within a few float ulps); the ReLU
 * masks come from the fp32 pre-activations; the output deltas are
 * 2 (out - y) / batch in float, rounded to bfloat16; the layer-2 deltas are
 * W3[0][j] d0 + W3[1][j] d1 (exact products, one rounding). */
static inline float bf16_rn(float v) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  if ((u & 0x7f800000u) == 0x7f800000u) return v;
  u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
  std::memcpy(&v, &u, 4);
  return v;
}

extern "C" int oracle_mlp_forward_backward_dev(int nin, int nh, int64_t batch, const float* prm_in, const float* x,
                                               const float* y, float* grad, float* loss) {
  if (nin < 1 || nh < 1 || batch < 1) return -1;
  const int w1 = 0, b1 = nh * nin, w2 = b1 + nh, b2 = w2 + nh * nh, w3 = b2 + nh, b3 = w3 + 2 * nh;
  const int np = b3 + 2;
  std::vector<float> prm(np);
  for (int i = 0; i < np; ++i) prm[i] = bf16_rn(prm_in[i]);
  std::vector<double> g(np, 0.0);
  std::vector<float> xb(nin), z1(nh), h1b(nh), z2(nh), h2b(nh), d2b(nh), d1b(nh);
  const float inv_b = 1.f / (float)batch;
  float L = 0.f;
  for (int64_t s = 0; s < batch; ++s) {
    for (int f = 0; f < nin; ++f) xb[f] = bf16_rn(x[s * nin + f]);
    for (int j = 0; j < nh; ++j) {
      double acc = prm[b1 + j];
      for (int f = 0; f < nin; ++f) acc += (double)prm[w1 + j * nin + f] * xb[f];
      z1[j] = (float)acc;
      h1b[j] = bf16_rn(z1[j] > 0.f ? z1[j] : 0.f);
    }
    for (int j = 0; j < nh; ++j) {
      double acc = prm[b2 + j];
      for (int k = 0; k < nh; ++k) acc += (double)prm[w2 + j * nh + k] * h1b[k];
      z2[j] = (float)acc;
      h2b[j] = bf16_rn(z2[j] > 0.f ? z2[j] : 0.f);
    }
    float db[2];
    for (int q = 0; q < 2; ++q) {
      double acc = prm[b3 + q];
      for (int k = 0; k < nh; ++k) acc += (double)prm[w3 + q * nh + k] * h2b[k];
      const float e = (float)acc - y[s * 2 + q];
      L += e * e * inv_b;
      db[q] = bf16_rn(2.f * e * inv_b);
      g[b3 + q] += db[q];
      for (int k = 0; k < nh; ++k) g[w3 + q * nh + k] += (double)db[q] * h2b[k];
    }
    for (int j = 0; j < nh; ++j) {
      const float d = z2[j] > 0.f ? std::fma(prm[w3 + j], db[0], prm[w3 + nh + j] * db[1]) : 0.f;
      d2b[j] = bf16_rn(d);
      g[b2 + j] += d2b[j];
      for (int k = 0; k < nh; ++k) g[w2 + j * nh + k] += (double)d2b[j] * h1b[k];
    }
    for (int k = 0; k < nh; ++k) {
      double acc = 0;
      for (int j = 0; j < nh; ++j) acc += (double)prm[w2 + j * nh + k] * d2b[j];
      d1b[k] = bf16_rn(z1[k] > 0.f ? (float)acc : 0.f);
      g[b1 + k] += d1b[k];
      for (int f = 0; f < nin; ++f) g[w1 + k * nin + f] += (double)d1b[k] * xb[f];
    }
  }
  for (int i = 0; i < np; ++i) grad[i] = (float)g[i];
  *loss = L;
  return 0;
}
