/* CPU oracle for the ensemble solve: C ABI used by the tests and by the
 * bench's CPU-baseline leg only.
 *
 * TEST INFRASTRUCTURE.  This is a plain C++ restatement of the reference's
 * solver loops (SimpleDiffEq.jl, files cited in oracle.cpp).  The product
 * library never links, loads or calls it.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum oracle_alg {
  ORACLE_RK4 = 0,          /* GPUSimpleRK4           src/rk4/gpurk4.jl:53-98 */
  ORACLE_TSIT5 = 1,        /* GPUSimpleTsit5         src/tsit5/gpuatsit5.jl:55-147 */
  ORACLE_ATSIT5 = 2,       /* GPUSimpleATsit5        src/tsit5/gpuatsit5.jl:205-336 */
  ORACLE_VERN7 = 3,        /* GPUSimpleVern7         src/verner/gpuvern7.jl:55-242 */
  ORACLE_AVERN7 = 4,       /* GPUSimpleAVern7        src/verner/gpuvern7.jl:300-536 */
  ORACLE_VERN9 = 5,        /* GPUSimpleVern9         src/verner/gpuvern9.jl:55-353 */
  ORACLE_AVERN9 = 6,       /* GPUSimpleAVern9        src/verner/gpuvern9.jl:411-779 */
  ORACLE_SIMPLE_ATSIT5 = 7,/* SimpleATsit5 integrator src/tsit5/atsit5.jl:117-179,322-413,705-732 */
  ORACLE_SIMPLE_TSIT5 = 8, /* SimpleTsit5 integrator  src/tsit5/tsit5.jl:84-122,303-352 */
  ORACLE_EULER = 9         /* GPUSimpleEuler         src/euler/gpueuler.jl:53-90 */
};

enum oracle_rhs { ORACLE_LORENZ = 0, ORACLE_VDP = 1, ORACLE_R3BP = 2, ORACLE_KURAMOTO = 3, ORACLE_LINEAR = 4 };
enum oracle_prec { ORACLE_FP64 = 0, ORACLE_FP32 = 1, ORACLE_FP32_KAHAN = 2 };
/* ORACLE_ROUND_REF: the rounding the reference's Julia code performs
 * (@muladd on SVector falls back to separate multiply and add; libm pow).
 * ORACLE_ROUND_DEVICE: the documented device rounding canon (explicit fused
 * multiply-add chains, single-precision controller power). */
enum oracle_round { ORACLE_ROUND_REF = 0, ORACLE_ROUND_DEVICE = 1 };

typedef struct {
  int alg, rhs, precision, rounding;
  int64_t n;
  int dim, nparams;
  double t0, tf, dt, abstol, reltol;
  const double* saveat;  /* [nsave] or NULL */
  int64_t nsave;
  int save_everystep;    /* fixed-step algorithms only: save every grid point */
  const double* grid;    /* fixed-step time grid (elements of t0:dt:tf), [ngrid] */
  int64_t ngrid;
  int64_t maxiters;      /* attempts per trajectory; <= 0 means unlimited */
  const double* u0;      /* SoA [dim][n] */
  const double* p;       /* SoA [nparams][n] */
  const double* dt0;     /* optional per-trajectory initial dt [n] */
  int nthreads;
  int output;            /* 0: state at saveat points; 1: Kuramoto order parameter r(t) of it */
  int ctrl;              /* DEVICE rounding, FP64 adaptive solves: error norm and step-size controller, as
                            ODE_CTRL_*: 0 double-single, 1 FP64 factors (single norm), 2 single precision.
                            REF rounding: 3 (ODE_CTRL_REF) takes the controller's powers and the sines
                            and cosines correctly rounded (crpow.h, the kernels' reference-arithmetic
                            mode), any other value libm's */
} oracle_args;

typedef struct {
  double* us;        /* SoA [npoints][dim][n], npoints = nsave or ngrid; may be NULL */
  double* u_final;   /* SoA [dim][n]; may be NULL */
  double* t_final;   /* [n]; may be NULL */
  int8_t* retcode;   /* [n]; may be NULL */
  int32_t* naccept;  /* [n]; may be NULL */
  int32_t* nreject;  /* [n]; may be NULL */
  double* dt_first;  /* [n] dt of the first accepted step; may be NULL */
  /* every-step output of the adaptive solvers (save_everystep without saveat):
   * trajectory i's rows start at ev_off[i]; row k holds the time and state
   * after its k-th accepted step (k = 0: t0, u0).  NULL to skip. */
  const int64_t* ev_off;
  double* ev_t;      /* [rows] */
  double* ev_u;      /* [rows][dim] */
} oracle_out;

int oracle_solve(const oracle_args* a, oracle_out* o);

/* SimpleEM (src/euler_maruyama.jl:48-142), diagonal and non-diagonal noise,
 * with the counter-based normals of the device canon (Philox4x32-10 +
 * Box-Muller).  ORACLE_SDE_MULT is the non-diagonal multiplicative noise of the
 * reference's test (test/simpleem_tests.jl): f = mu u, G[d][m] = c[d][m] u[d],
 * p = (mu, c row-major dim x noise_dim). */
enum oracle_sde { ORACLE_SDE_GBM = 0, ORACLE_SDE_OU = 1, ORACLE_SDE_LORENZ = 2, ORACLE_SDE_MULT = 3 };
typedef struct {
  int sde, rounding;
  int64_t n;
  int dim, nparams;
  double t0, dt;
  int64_t nsteps;
  uint64_t seed;
  const double* u0;  /* [dim][n] */
  const double* p;   /* [nparams][n] */
  double* us;        /* [nsteps+1][dim][n] or NULL */
  double* u_final;   /* [dim][n] or NULL */
  int nthreads;
  int noise_dim;     /* 0: diagonal noise; M > 0: dim x M noise matrix, M normals a step */
} oracle_sde_args;
int oracle_sde_solve(const oracle_sde_args* a);
/* Philox4x32-10 of counter c[4] under key k[2] into out[4] */
void oracle_philox(const uint32_t* c, const uint32_t* k, uint32_t* out);
/* the device canon's double logarithm */
double oracle_log(double x);
/* normals z_{2 pair}, z_{2 pair + 1} of trajectory idx's stream */
void oracle_normal_pair(uint64_t seed, int64_t pair, int64_t idx, double* z0, double* z1);
float oracle_ctrl_pow(float x, float b);
/* the device canon's double sine and cosine (Cody-Waite reduction, Taylor polynomials) */
void oracle_sincos(double x, double* s, double* c);
int oracle_mlp_forward_backward(int nin, int nh, int64_t batch, const float* params, const float* x,
                                const float* y, float* grad, float* loss);
/* the same in the device training kernel's rounding (bf16 operands, fp32 accumulation) */
int oracle_mlp_forward_backward_dev(int nin, int nh, int64_t batch, const float* params, const float* x,
                                    const float* y, float* grad, float* loss);

#ifdef __cplusplus
}
#endif
