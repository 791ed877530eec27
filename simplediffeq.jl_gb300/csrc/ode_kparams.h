/* Launch parameters of the solver kernels.  Shared verbatim by the host
 * library (g++/nvcc) and by kernels compiled at run time with NVRTC, so it
 * uses only built-in types. */
#pragma once
#if !defined(__CUDACC_RTC__)
#include <cstring>
#endif

namespace gbode {

enum { RET_DEFAULT = 0, RET_DTMIN = 1, RET_MAXITERS = 2, RET_NAN = 3 };

struct KParams {
  long long n;             /* trajectories */
  double t0, tf, dt, abstol, reltol;
  const double* u0;        /* [dim][n] */
  const double* p;         /* [nparams][n] */
  const double* dt0;       /* [n] per-trajectory initial dt, or 0 */
  const double* saveat;    /* [nsave] on the device, or 0 */
  long long nsave;
  const double* grid;      /* fixed-step time grid [ngrid] on the device, or 0 */
  long long ngrid;
  int save_everystep;
  int dim, nparams;
  long long maxiters;      /* <= 0: no cap */
  int norm_fp64;           /* 1: error norm in double (abstol below 1e-30) */
  float tol_ds[4];         /* abstol and reltol as double-single pairs (h, l, h, l): ds_split_host */
  int output;              /* 0: store the state at saveat points; 1: store the Kuramoto order parameter */
  double* us;              /* saveat / every-step output, or 0; element (point j, value w, trajectory i)
                              at us[j * us_sj + w * us_sw + i * us_si] */
  long long us_sj, us_sw, us_si; /* [npoints][width][n]: (width*n, n, 1); [n][npoints][width]: (width, 1, npoints*width) */
  double* u_final;         /* [dim][n] or 0 */
  double* t_final;         /* [n] or 0 */
  signed char* retcode;    /* [n] or 0 */
  int* naccept;            /* [n] or 0 */
  int* nreject;            /* [n] or 0 */
  double* dt_first;        /* [n] or 0 */
  const long long* ev_off; /* every-step output: trajectory i's points are rows ev_off[i].., or 0 */
  double* ev_t;            /* [rows] time of each accepted step (t0 first) */
  double* ev_u;            /* [rows][dim] state after each accepted step (u0 first) */
  const int* order;        /* persistent: position -> trajectory, or 0 for identity */
  unsigned long long* counter;   /* persistent: next position to hand out (zeroed before launch) */
  unsigned long long* stats;     /* [2] attempts and saves summed over trajectories, or 0 */
  unsigned* check_flags;   /* bounds-check builds: violation bits (CHK_*), or 0 */
  unsigned* visited;       /* bounds-check builds: [n] starts of each trajectory, or 0 */
};


#if !defined(__CUDACC_RTC__)
/* A double as a double-single pair h + l (the kernels' ds_split, on the
 * host): h is x's sign, exponent and top 23 fraction bits repacked as a
 * single (+-0 below 2^-126, +-infinity from 2^128, NaN for NaN), l the 29
 * low fraction bits as an integer rounded to a single and scaled by
 * 2^(e - 52) (0 outside 2^-74 <= |x| < 2^128). */
inline void ds_split_host(double x, float* hl) {
  long long b;
  std::memcpy(&b, &x, 8);
  const int eb = (int)((b >> 52) & 0x7ff);
  const unsigned sign = (unsigned)((unsigned long long)b >> 32) & 0x80000000u;
  const unsigned frac = (unsigned)((b >> 29) & 0x7fffff);
  const unsigned hb = eb >= 897 && eb <= 1150 ? sign | ((unsigned)(eb - 896) << 23) | frac
                      : eb < 897 ? sign
                      : (eb == 2047 && (b & 0xfffffffffffffLL)) ? 0x7fc00000u | sign
                                                                : 0x7f800000u | sign;
  float l = 0.0f;
  if (eb >= 949 && eb <= 1150) {
    const int sb = (eb - 948) << 23;
    float sc;
    std::memcpy(&sc, &sb, 4);
    const float mag = (float)(int)(b & 0x1fffffff) * sc;
    l = b < 0 ? -mag : mag;
  }
  std::memcpy(&hl[0], &hb, 4);
  hl[1] = l;
}
#endif
}  // namespace gbode
