/* Device side of the SimpleEM ensemble solver (src/euler_maruyama.jl:48-142):
 * fixed-step Euler-Maruyama, one trajectory per thread.
 *
 *   n = Int((tf - t0) / dt) + 1 points, t_k = t0 + k*dt (a scalar muladd),
 *   diagonal noise:      u_{k+1} = u_k + f(u_k, p, t_k)*dt + sqrt(dt)*g(u_k, p, t_k) .* xi_k
 *   non-diagonal noise:  u_{k+1} = u_k + f(u_k, p, t_k)*dt + sqrt(dt)*(G(u_k, p, t_k) * xi_k)
 * with G a dim x M matrix (the reference's noise_rate_prototype) and xi_k M
 * normals.
 *
 * The reference draws xi_k with Julia's randn; this solver draws them from a
 * counter-based generator so that every trajectory's noise is reproducible
 * from (seed, trajectory) alone, on any thread and on the CPU.  Trajectory i
 * has the stream of standard normals z_0, z_1, z_2, ..., of which step k
 * takes z_{kD}, ..., z_{kD+D-1} (no normal is drawn and dropped, also for odd
 * D):
 *   - Philox4x32-10 (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw,
 *     "Parallel random numbers: as easy as 1, 2, 3", SC'11), counter
 *     (pair P low word, pair P high word, trajectory low word, trajectory
 *     high word), key = seed, gives z_{2P} and z_{2P+1}:
 *   - two 53-bit uniforms u1 in (0, 1], u2 in [0, 1) and the Box-Muller pair
 *     (G. E. P. Box, M. E. Muller, 1958) r = sqrt(-2 log u1),
 *     (r cos 2 pi u2, r sin 2 pi u2), evaluated in double-single arithmetic
 *     on the single-precision pipe (normal_pair below: within about 2^-44 of
 *     the exact values; two double operations a pair), so that the oracle
 *     reproduces every normal bit for bit.
 * Non-diagonal noise takes M normals a step from the same stream.
 * Update rounding (device canon): diagonal u = fma(sqdt*g, xi, fma(f, dt, u));
 * non-diagonal s = G[d][0] xi_0, s = fma(G[d][m], xi_m, s) for m = 1..M-1,
 * u = fma(sqdt, s, fma(f, dt, u)) (the reference's mul!(gtmp2, gtmp, dW) and
 * uprev + ftmp*dt + sqdt*gtmp2 under @muladd). */
#pragma once
#include "ode_solver.cuh"


namespace gbode {

struct SParams {
  long long n;           /* trajectories */
  long long nsteps;      /* steps (points - 1) */
  double t0, dt;
  unsigned long long seed;
  int dim, nparams;
  int noise_dim;         /* 0: diagonal noise; M: dim x M noise matrix */
  int save_everystep;
  const double* u0;      /* [dim][n] */
  const double* p;       /* [nparams][n] */
  double* us;            /* [nsteps + 1][dim][n], or 0 */
  double* u_final;       /* [dim][n], or 0 */
};

/* ------------------------------------------------------------------ Philox4x32-10 */
struct U4 {
  unsigned x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, unsigned k0, unsigned k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    const unsigned hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

/* Normals z_{2P} and z_{2P+1} of trajectory idx's stream. */
/* v 2^-e for 0 < v < 2^64 as a double-single pair, with integer operations:
 * v is shifted left by its leading zeros, h = its top 24 bits and l = the next
 * 24 (both exact singles) scaled through the exponent field; bits below those
 * 48 are dropped (v 2^-e must leave both scales in the normal single range). */
__device__ __forceinline__ dsf ds_from_u64(unsigned long long v, int e) {
  const int z = __clzll((long long)v);
  const unsigned long long m = v << z;
  const float hi = (float)(unsigned)(m >> 40) * __int_as_float((40 - z - e + 127) << 23);
  const float lo = (float)(unsigned)((m >> 16) & 0xffffff) * __int_as_float((16 - z - e + 127) << 23);
  return {hi, lo};
}

/* sqrt(y) for y >= 0: s = y.h rsqrt_nr(y.h), then one correction (y - s^2) /
 * (2 s) with s^2 an exact product pair (y.h - s^2 is exact by Sterbenz) */
__device__ __forceinline__ dsf ds_sqrt(dsf y) {
  if (!(y.h > 0.0f)) return {0.0f, 0.0f};
  const float r = rsqrt_nr(y.h);
  const float sq = y.h * r;
  const float p = sq * sq, pe = __fmaf_rn(sq, sq, -p);
  return ds_fast(sq, (((y.h - p) - pe) + y.l) * (0.5f * r));
}

/* sin r and cos r for |r| <= pi/4 + tiny: Taylor series of sin r / r and
 * cos r in r^2, the terms above 2^-24 in double-single and the rest in single
 * precision (truncation below 2^-50) */
__device__ __forceinline__ void ds_sincos_reduced(dsf r, dsf* sn, dsf* cs) {
  const dsf r2 = ds_sqr(r);
  float ts = __fmaf_rn(r2.h, GBODE_DS_SIN_T7, GBODE_DS_SIN_T6);
  ts = __fmaf_rn(r2.h, ts, GBODE_DS_SIN_T5);
  dsf ps = {ts, 0.0f};
  ps = ds_add(ds_mul(ps, r2), dsf{GBODE_DS_SIN_C4_H, GBODE_DS_SIN_C4_L});
  ps = ds_add(ds_mul(ps, r2), dsf{GBODE_DS_SIN_C3_H, GBODE_DS_SIN_C3_L});
  ps = ds_add(ds_mul(ps, r2), dsf{GBODE_DS_SIN_C2_H, GBODE_DS_SIN_C2_L});
  ps = ds_add(ds_mul(ps, r2), dsf{GBODE_DS_SIN_C1_H, GBODE_DS_SIN_C1_L});
  ps = ds_add(ds_mul(ps, r2), dsf{1.0f, 0.0f});
  *sn = ds_mul(r, ps);
  float tc = __fmaf_rn(r2.h, GBODE_DS_COS_T8, GBODE_DS_COS_T7);
  tc = __fmaf_rn(r2.h, tc, GBODE_DS_COS_T6);
  tc = __fmaf_rn(r2.h, tc, GBODE_DS_COS_T5);
  dsf pc = {tc, 0.0f};
  pc = ds_add(ds_mul(pc, r2), dsf{GBODE_DS_COS_C4_H, GBODE_DS_COS_C4_L});
  pc = ds_add(ds_mul(pc, r2), dsf{GBODE_DS_COS_C3_H, GBODE_DS_COS_C3_L});
  pc = ds_add(ds_mul(pc, r2), dsf{GBODE_DS_COS_C2_H, GBODE_DS_COS_C2_L});
  pc = ds_add(ds_mul(pc, r2), dsf{GBODE_DS_COS_C1_H, GBODE_DS_COS_C1_L});
  *cs = ds_add(ds_mul(pc, r2), dsf{1.0f, 0.0f});
}

/* The normals z_{2P}, z_{2P+1} of trajectory idx: Philox gives two 53-bit
 * integers a, c; u1 = (a + 1) 2^-53 and u2 = c 2^-53 are taken as
 * double-single pairs straight from the integers (ds_from_u64); r =
 * sqrt(-2 ln u1) (ds_log, ds_sqrt); the angle 2 pi u2 = k pi/2 + f pi/2 with
 * 4 u2 = k + f, k = round(4 u2) (half up) and f = (c - k 2^51) 2^-51 in
 * [-1/2, 1/2], both exact in integers, then sin and cos of f pi/2 and the
 * quadrant k mod 4; z0 = r cos, z1 = r sin, each a double from its pair (one
 * double addition). */
__device__ __forceinline__ void normal_pair(unsigned long long seed, long long P, long long idx, double* z0,
                                            double* z1) {
  const U4 r = philox4x32_10(U4{(unsigned)P, (unsigned)((unsigned long long)P >> 32), (unsigned)idx,
                                (unsigned)((unsigned long long)idx >> 32)},
                             (unsigned)seed, (unsigned)(seed >> 32));
  const unsigned long long a = ((unsigned long long)(r.x >> 5) << 26) | (r.y >> 6);
  const unsigned long long c = ((unsigned long long)(r.z >> 5) << 26) | (r.w >> 6);
  const dsf lg = ds_log(ds_from_u64(a + 1, 53));
  const dsf rad = ds_sqrt(dsf{-2.0f * lg.h, -2.0f * lg.l});
  const unsigned long long k = (c + (1ULL << 50)) >> 51;
  const long long fi = (long long)c - (long long)(k << 51);
  dsf f = {0.0f, 0.0f};
  if (fi != 0) {
    f = ds_from_u64((unsigned long long)(fi < 0 ? -fi : fi), 51);
    if (fi < 0) f = ds_neg(f);
  }
  dsf sr, cr;
  ds_sincos_reduced(ds_mul(f, dsf{GBODE_DS_PIO2_H, GBODE_DS_PIO2_L}), &sr, &cr);
  const int q = (int)(k & 3);
  const dsf sn = q == 0 ? sr : q == 1 ? cr : q == 2 ? ds_neg(sr) : ds_neg(cr);
  const dsf cs = q == 0 ? cr : q == 1 ? ds_neg(sr) : q == 2 ? ds_neg(cr) : sr;
  *z0 = ds_to_double(ds_mul(rad, cs));
  *z1 = ds_to_double(ds_mul(rad, sn));
}

/* ------------------------------------------------------------------ built-in SDEs (diagonal noise) */
/* geometric Brownian motion: f = mu u, g = sigma u; p = (mu, sigma) */
template <int DD>
struct SdeGBM {
  enum { D = DD, M = 0, GN = DD, NP = 2 };
  double p[2];
  __device__ __forceinline__ void drift(const double (&u)[DD], double t, double (&f)[DD]) const {
#pragma unroll
    for (int d = 0; d < DD; ++d) f[d] = p[0] * u[d];
  }
  __device__ __forceinline__ void diffusion(const double (&u)[DD], double t, double (&g)[DD]) const {
#pragma unroll
    for (int d = 0; d < DD; ++d) g[d] = p[1] * u[d];
  }
};

/* Ornstein-Uhlenbeck: f = theta (mu - u), g = sigma; p = (theta, mu, sigma) */
template <int DD>
struct SdeOU {
  enum { D = DD, M = 0, GN = DD, NP = 3 };
  double p[3];
  __device__ __forceinline__ void drift(const double (&u)[DD], double t, double (&f)[DD]) const {
#pragma unroll
    for (int d = 0; d < DD; ++d) f[d] = p[0] * (p[1] - u[d]);
  }
  __device__ __forceinline__ void diffusion(const double (&u)[DD], double t, double (&g)[DD]) const {
#pragma unroll
    for (int d = 0; d < DD; ++d) g[d] = p[2];
  }
};

/* Lorenz drift with additive noise of strength p[3]; p = (sigma, rho, beta, noise) */
struct SdeLorenz {
  enum { D = 3, M = 0, GN = 3, NP = 4 };
  double p[4];
  __device__ __forceinline__ void drift(const double (&u)[3], double t, double (&f)[3]) const {
    f[0] = p[0] * (u[1] - u[0]);
    f[1] = fmaR(u[0], p[1] - u[2], -u[1]);
    f[2] = fmaR(u[0], u[1], -(p[2] * u[2]));
  }
  __device__ __forceinline__ void diffusion(const double (&u)[3], double t, double (&g)[3]) const {
    g[0] = p[3];
    g[1] = p[3];
    g[2] = p[3];
  }
};

/* xi[0..N) = z_{kN}, ..., z_{kN+N-1} (N = dim for diagonal noise, M
 * otherwise).  For odd N a pair straddles two steps: an even step draws
 * (N+1)/2 pairs and keeps the last normal in `carry` for the next step, which
 * starts with it and draws (N-1)/2 pairs. */
template <int N>
__device__ __forceinline__ void step_normals(unsigned long long seed, long long k, long long idx, double (&xi)[N + 1],
                                             double& carry) {
  const long long g0 = k * N;
  if ((N & 1) && (g0 & 1)) {
    xi[0] = carry;
#pragma unroll
    for (int j = 0; j < (N - 1) / 2; ++j) normal_pair(seed, (g0 + 1) / 2 + j, idx, &xi[1 + 2 * j], &xi[2 + 2 * j]);
  } else {
#pragma unroll
    for (int j = 0; j < (N + 1) / 2; ++j) normal_pair(seed, g0 / 2 + j, idx, &xi[2 * j], &xi[2 * j + 1]);
    if (N & 1) carry = xi[N];
  }
}

/* Non-diagonal multiplicative noise, the reference's test SDE
 * (test/simpleem_tests.jl): f = mu u, G[d][m] = c[d][m] u[d];
 * p = (mu, c row-major DD x MM) */
template <int DD, int MM>
struct SdeMult {
  enum { D = DD, M = MM, GN = DD * MM, NP = 1 + DD * MM };
  double p[NP];
  __device__ __forceinline__ void drift(const double (&u)[DD], double t, double (&f)[DD]) const {
#pragma unroll
    for (int d = 0; d < DD; ++d) f[d] = p[0] * u[d];
  }
  __device__ __forceinline__ void diffusion(const double (&u)[DD], double t, double (&g)[GN]) const {
#pragma unroll
    for (int d = 0; d < DD; ++d)
#pragma unroll
      for (int m = 0; m < MM; ++m) g[d * MM + m] = p[1 + d * MM + m] * u[d];
  }
};

/* ------------------------------------------------------------------ the Euler-Maruyama loop */
template <class S>
__device__ __forceinline__ void run_em(const SParams& P) {
  enum { D = S::D };
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= P.n) return;
  S sde;
#pragma unroll
  for (int q = 0; q < S::NP; ++q) sde.p[q] = P.p[(long long)q * P.n + i];
  double u[D];
#pragma unroll
  for (int d = 0; d < D; ++d) u[d] = P.u0[(long long)d * P.n + i];
  if (P.save_everystep && P.us)
#pragma unroll
    for (int d = 0; d < D; ++d) P.us[(long long)d * P.n + i] = u[d];
  const double dt = P.dt, sqdt = __dsqrt_rn(P.dt);
  enum { N = S::M > 0 ? S::M : D };  /* normals a step */
  double carry = 0.0;
  for (long long k = 0; k < P.nsteps; ++k) {
    const double t = __fma_rn((double)k, dt, P.t0);
    double f[D], g[S::GN], xi[N + 1];
    sde.drift(u, t, f);
    sde.diffusion(u, t, g);
    step_normals<N>(P.seed, k, i, xi, carry);
    if constexpr (S::M > 0) {
#pragma unroll
      for (int d = 0; d < D; ++d) {
        double s = g[d * N] * xi[0];
#pragma unroll
        for (int m = 1; m < N; ++m) s = __fma_rn(g[d * N + m], xi[m], s);
        u[d] = __fma_rn(sqdt, s, __fma_rn(f[d], dt, u[d]));
      }
    } else {
#pragma unroll
      for (int d = 0; d < D; ++d) u[d] = __fma_rn(sqdt * g[d], xi[d], __fma_rn(f[d], dt, u[d]));
    }
    if (P.save_everystep && P.us)
#pragma unroll
      for (int d = 0; d < D; ++d) P.us[((k + 1) * D + d) * P.n + i] = u[d];
  }
  if (P.u_final)
#pragma unroll
    for (int d = 0; d < D; ++d) P.u_final[(long long)d * P.n + i] = u[d];
}

}  // namespace gbode

#define GBODE_SDE_ENTRY(NAME, S) \
  extern "C" __global__ void __launch_bounds__(128) NAME(gbode::SParams P) { gbode::run_em<S>(P); }
