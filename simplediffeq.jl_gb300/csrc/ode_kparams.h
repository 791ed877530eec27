/* Launch parameters of the solver kernels.  Shared verbatim by the host
 * library (g++/nvcc) and by kernels compiled at run time with NVRTC, so it
 * uses only built-in types. */
#pragma once

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

}  // namespace gbode
