/* gb300ode — ensemble explicit Runge-Kutta solves on one NVIDIA GB300 GPU.
 *
 * C ABI of libgb300ode.so.  It replaces, for a whole ensemble at once, the
 * per-trajectory solve methods of SimpleDiffEq.jl's GPU-crutch solvers:
 *
 *   DiffEqBase.solve(prob, GPUSimpleRK4(); dt)                 src/rk4/gpurk4.jl:53-98
 *   DiffEqBase.solve(prob, GPUSimpleEuler(); dt)               src/euler/gpueuler.jl:53-90
 *   DiffEqBase.solve(prob, GPUSimpleTsit5(); dt, saveat, ...)  src/tsit5/gpuatsit5.jl:55-147
 *   DiffEqBase.solve(prob, GPUSimpleATsit5(); dt, abstol, reltol, saveat, ...)
 *                                                              src/tsit5/gpuatsit5.jl:205-336
 *   DiffEqBase.solve(prob, GPUSimpleVern7(); ...)              src/verner/gpuvern7.jl:55-242
 *   DiffEqBase.solve(prob, GPUSimpleAVern7(); ...)             src/verner/gpuvern7.jl:300-536
 *   DiffEqBase.solve(prob, GPUSimpleVern9(); ...)              src/verner/gpuvern9.jl:55-353
 *   DiffEqBase.solve(prob, GPUSimpleAVern9(); ...)             src/verner/gpuvern9.jl:411-779
 *
 * applied to every trajectory of an ensemble (the prob_func loop that
 * SciMLBase's EnsembleProblem would run on the host).  The keyword arguments
 * keep their meaning and defaults (dt = 0.1, abstol = 1e-6, reltol = 1e-3,
 * saveat = nothing) and the solver loop is the reference's: same stages,
 * error norm, PI controller (src/SimpleDiffEq.jl:67-77) and saveat
 * interpolation.
 *
 * Conventions
 *   - Every function returns ODE_OK (0) or a negative ODE_E* code and never
 *     throws, aborts or traps.  ode_last_error() describes the last failure.
 *   - The caller owns every input and output buffer.  The handle owns the
 *     device workspace, compiled kernels, captured CUDA graphs and the
 *     learned-schedule model.  One handle is used by one host thread at a time.
 *   - Arrays are structure-of-arrays over trajectories: element (d, i) of a
 *     [dim][n] array is at d*n + i.  All floating-point buffers are double;
 *     in the single-precision modes the kernels convert on load and store.
 *   - The reference throws ErrorException("dt<dtmin"); here the trajectory
 *     stops with retcode ODE_RET_DTMIN and the call returns ODE_ETRAJ, so a
 *     host layer can raise the same exception.
 */
#ifndef GB300ODE_H
#define GB300ODE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ODE_ABI_VERSION 6

/* status codes */
enum {
  ODE_OK = 0,
  ODE_EINVAL = -1,   /* invalid argument */
  ODE_ECUDA = -2,    /* CUDA runtime or driver error */
  ODE_ENOMEM = -3,   /* device or host allocation failed */
  ODE_ENOTSUP = -4,  /* valid but unsupported combination */
  ODE_ENVRTC = -5,   /* run-time compilation of a kernel failed (log in ode_last_error) */
  ODE_ETRAJ = -6,    /* the solve completed but some trajectory ended with retcode DTMIN or MAXITERS */
  ODE_ENOMODEL = -7, /* learned schedule requested without a fitted model */
  ODE_ESMALL = -8,   /* output buffers too small: the size needed is reported (ode_ensemble_solve_everystep) */
  ODE_ECHECK = -9    /* bounds-check mode found an out-of-range index or a trajectory not solved exactly once */
};

/* algorithms: the GPUSimple* solver types */
enum {
  ODE_ALG_RK4 = 0,     /* GPUSimpleRK4    (fixed step) */
  ODE_ALG_TSIT5 = 1,   /* GPUSimpleTsit5  (fixed step) */
  ODE_ALG_ATSIT5 = 2,  /* GPUSimpleATsit5 (adaptive)   */
  ODE_ALG_VERN7 = 3,   /* GPUSimpleVern7  (fixed step) */
  ODE_ALG_AVERN7 = 4,  /* GPUSimpleAVern7 (adaptive)   */
  ODE_ALG_VERN9 = 5,   /* GPUSimpleVern9  (fixed step) */
  ODE_ALG_AVERN9 = 6,  /* GPUSimpleAVern9 (adaptive)   */
  ODE_ALG_EULER = 7    /* GPUSimpleEuler  (fixed step) */
};

/* built-in right-hand sides f(u, p, t); ids >= ODE_RHS_USER come from ode_rhs_compile */
enum {
  ODE_RHS_LORENZ = 0,    /* dim 3, p = (sigma, rho, beta) */
  ODE_RHS_VANDERPOL = 1, /* dim 2, x' = v, v' = mu (1 - x^2) v - x, p = (mu) */
  ODE_RHS_R3BP = 2,      /* dim 4, planar restricted three-body (x, y, vx, vy), p = (mu) */
  ODE_RHS_KURAMOTO = 3,  /* dim D, theta_i' = w_i + (K/D) sum_j sin(theta_j - theta_i), p = (w_1..w_D, K) */
  ODE_RHS_LINEAR = 4,    /* dim D, du = A u, p = A row-major (D*D values) */
  ODE_RHS_USER = 1000
};

enum {
  ODE_FP64 = 0,       /* everything in double, as the reference with Float64 state */
  ODE_FP32 = 1,       /* everything in float, as the reference with Float32 state */
  ODE_FP32_KAHAN = 2  /* float stages, Kahan-compensated float state, double t and dt */
};

enum {
  ODE_SCHED_PLAIN = 0,      /* one thread per trajectory */
  ODE_SCHED_PERSISTENT = 1, /* resident warps refill lanes from a device work counter */
  ODE_SCHED_LEARNED = 2     /* persistent, trajectories ordered by predicted cost, dt0 seeded */
};

enum { ODE_MEM_HOST = 0, ODE_MEM_DEVICE = 1 };

/* what the saveat outputs hold */
enum {
  ODE_OUTPUT_STATE = 0,      /* us[nsave][dim][n]: the interpolated state (the reference's sol.u) */
  ODE_OUTPUT_KURAMOTO_R = 1, /* us[nsave][1][n]: r(t) = |(1/dim) sum_k exp(i u_k(t))|, the Kuramoto order
                                parameter of the interpolated state, reduced in the kernel (an ensemble
                                output_func fused into the solve) */
  ODE_OUTPUT_USER = 1000     /* ids >= ODE_OUTPUT_USER come from ode_output_compile: us[npoints][width][n] */
};

/* layout of the saveat / every-step output us */
enum {
  ODE_LAYOUT_SOA = 0,  /* us[npoints][width][n]: one row of n trajectories per point and value */
  ODE_LAYOUT_TRAJ = 1  /* us[n][npoints][width]: each trajectory's series contiguous, the layout of the
                          reference's per-trajectory sol.u (a Vector of SVectors).  A trajectory's
                          consecutive points fill whole memory sectors, where the [n]-inner layout
                          puts one 8-byte value of each sector per trajectory (neighbours in a
                          sector are solved at different times under the persistent schedules) */
};

/* arithmetic of the error norm and step-size controller of adaptive FP64 solves
 * (ode_solve_args.controller); single-precision solves always use their own
 * single-precision norm and controller.  ODE_CTRL_REF changes the arithmetic
 * of the whole solve, fixed-step ones included. */
enum {
  ODE_CTRL_DS = 0,   /* default: the norm EEst and the factor q = EEst^beta1 / qold^beta2 with its
                        clamps in double-single arithmetic (pairs of floats, about 48 bits, on the
                        single-precision pipe; table-driven log and exp; doubles split into pairs by
                        integer operations): step sizes follow the reference's to about 2^-44
                        relative, and an attempt takes two double operations (dt times the factor)
                        where the single-precision norm converts each of its terms to single, a
                        conversion that occupies the double-precision pipe on this GPU */
  ODE_CTRL_FP64 = 1, /* the factor q in double precision (table-driven log and exp) on a
                        single-precision norm, whose 2^-24 rounding (times beta1) bounds how closely
                        step sizes follow the reference's; FP64 precision only */
  ODE_CTRL_FP32 = 2, /* the norm and the factor q in single precision (deterministic power
                        function): step sizes follow the reference's to about 2^-24 relative */
  ODE_CTRL_REF = 3   /* the reference's arithmetic throughout, FP64 only: the vector expressions'
                        products and sums rounded separately (the reference's SVector muladd does
                        not fuse), its right-hand-side and RK4 expressions as written, the dense
                        abscissa by division, the norm in IEEE double, the PI controller with pow,
                        and pow, sin and cos correctly rounded (the double nearest the exact value,
                        where libm implementations can differ in the last bit; sin and cos for
                        |x| < 2^19); slower, for results that follow the reference operation for
                        operation */
};

/* per-trajectory return codes */
enum {
  ODE_RET_DEFAULT = 0,  /* finished at tf (ReturnCode.Default in the reference) */
  ODE_RET_DTMIN = 1,    /* dt fell below dtmin (the reference throws "dt<dtmin") */
  ODE_RET_MAXITERS = 2, /* attempt cap reached (no counterpart; the reference has no cap) */
  ODE_RET_NAN = 3       /* finished at tf, but a NaN error estimate was accepted on the way,
                           as the reference accepts it (NaN > 1 is false) */
};

typedef struct ode_handle ode_handle;

typedef struct {
  int32_t alg;          /* ODE_ALG_* */
  int32_t rhs;          /* ODE_RHS_* or an id from ode_rhs_compile */
  int32_t precision;    /* ODE_FP64 / ODE_FP32 / ODE_FP32_KAHAN */
  int32_t schedule;     /* ODE_SCHED_* (adaptive algorithms; fixed-step ones always run plain) */
  int64_t n;            /* trajectories */
  int32_t dim;          /* state dimension */
  int32_t nparams;      /* parameters per trajectory */
  double t0, tf;        /* tspan */
  double dt;            /* initial (adaptive) or fixed step; reference default 0.1 */
  double abstol, reltol;/* reference defaults 1e-6, 1e-3 */
  const double* saveat; /* [nsave] save times (always a host pointer), or NULL */
  int64_t nsave;
  int32_t save_everystep; /* fixed-step algorithms without saveat: save every grid point */
  int32_t memory;       /* ODE_MEM_HOST or ODE_MEM_DEVICE for u0, p, dt0 and all outputs */
  int64_t maxiters;     /* attempt cap per trajectory; <= 0: the default cap of 10^6 */
  const double* u0;     /* [dim][n] */
  const double* p;      /* [nparams][n] */
  const double* dt0;    /* optional [n] per-trajectory initial dt (adaptive), or NULL */
  void* stream;         /* cudaStream_t, or NULL for the handle's stream.  With device buffers, a
                           stream and stats == NULL, ode_ensemble_solve is asynchronous: it
                           returns once the work is enqueued (per-trajectory retcodes tell of
                           early stops; ODE_ETRAJ is not reported) and later calls on the same
                           stream are ordered after it */
  int32_t output;       /* ODE_OUTPUT_* (0: the state) */
  int32_t layout;       /* ODE_LAYOUT_* of us (0: [npoints][width][n]) */
  int32_t controller;   /* ODE_CTRL_* step-size controller arithmetic (adaptive FP64 solves) */
} ode_solve_args;

typedef struct {
  double* us;           /* [npoints][dim][n] (ODE_OUTPUT_STATE) or [npoints][1][n]
                           (ODE_OUTPUT_KURAMOTO_R), or [n][npoints][width] with ODE_LAYOUT_TRAJ:
                           npoints = nsave, or the grid length when save_everystep applies;
                           NULL to skip */
  double* u_final;      /* [dim][n] state at the end, or NULL */
  double* t_final;      /* [n], or NULL */
  int8_t* retcode;      /* [n] ODE_RET_*, or NULL */
  int32_t* naccept;     /* [n] accepted steps, or NULL */
  int32_t* nreject;     /* [n] rejected attempts, or NULL */
  double* dt_first;     /* [n] size of the first accepted step, or NULL */
} ode_solve_out;

typedef struct {
  double kernel_ms;       /* device time of the solve kernels (CUDA events) */
  double total_ms;        /* wall time of the call */
  int64_t attempts;       /* sum over trajectories of accepted + rejected attempts */
  int64_t saves;          /* saveat points written */
  int32_t launches;       /* kernels launched by the call */
  int32_t schedule_used;  /* ODE_SCHED_* actually run */
  int32_t graph_replayed; /* 1 if a captured CUDA graph was replayed */
  int32_t jit;            /* 1 if the solver kernel was compiled at run time */
  int32_t kernel;         /* ODE_KERNEL_* that ran */
} ode_solve_stats;

/* solver kernels (ode_solve_stats.kernel) */
enum {
  ODE_KERNEL_PLAIN = 0,      /* adaptive, one thread per trajectory */
  ODE_KERNEL_PERSISTENT = 1, /* adaptive, resident warps refilled from a work counter */
  ODE_KERNEL_STAGED = 2,     /* persistent with saveat interpolation batched per warp in shared memory */
  ODE_KERNEL_FIXED = 3,      /* fixed step, one thread per trajectory */
  ODE_KERNEL_FIXEDSPLIT = 4, /* fixed-step Tsit5 with a trajectory's components over the warps of a block
                                (FP64 ensembles of at most 2 x SMs warps, separable right-hand side) */
  ODE_KERNEL_ONESTEP = 5     /* RK4 / Euler, one thread per trajectory */
};

/* Bounds-check mode (debugging; compute-sanitizer stands in for nothing
 * here): with enable = 1 every later solve on this handle runs kernels
 * compiled at run time with an index check before every access to a caller
 * array and a per-trajectory start counter; a solve that saw an out-of-range
 * index, or a trajectory started other than exactly once, returns ODE_ECHECK
 * (the message says which).  Slower; results are unchanged. */
int ode_set_bounds_check(ode_handle* h, int enable);

/* Library version (ODE_ABI_VERSION). */
int ode_abi_version(void);

/* Create a handle bound to CUDA device `device`. */
int ode_create(ode_handle** h, int device);
/* Release the handle and everything it owns. */
void ode_destroy(ode_handle* h);
/* Text of the last error on this handle ("" if none). */
const char* ode_last_error(const ode_handle* h);

/* Solve an ensemble.  Replaces the per-trajectory solve calls listed above;
 * `stats` may be NULL.  Returns ODE_ETRAJ when the solve ran but some
 * trajectory ended with ODE_RET_DTMIN or ODE_RET_MAXITERS (see `retcode`). */
int ode_ensemble_solve(ode_handle* h, const ode_solve_args* a, ode_solve_out* o, ode_solve_stats* stats);

/* Elements of Julia's range t0:dt:tf (the fixed-step grid of the GPUSimple
 * fixed-step solvers, e.g. src/tsit5/gpuatsit5.jl:92) in double or float
 * semantics (precision ODE_FP32 for float).  Writes up to `cap` elements to
 * `out` (may be NULL) and the full length to *len. */
int ode_fixed_grid(double t0, double dt, double tf, int precision, double* out, int64_t cap, int64_t* len);

/* Select a built-in right-hand side (ODE_RHS_LORENZ .. ODE_RHS_LINEAR) for a
 * state of `dim` components: on success *rhs_out receives the id to put in
 * ode_solve_args.rhs and *nparams_out (may be NULL) the number of parameters
 * it takes; ODE_EINVAL if that right-hand side has no form of that dimension. */
int ode_rhs_builtin(ode_handle* h, int rhs_id, int dim, int* rhs_out, int* nparams_out);

/* Compile a user right-hand side with NVRTC.  `body` is the body of
 *   template <class R> __device__ void rhs(R* du, const R* u, const R* p, R t)
 * for a state of `dim` components and `nparams` parameters; R is double or
 * float.  On success *rhs_id receives an id usable in ode_solve_args.rhs.
 * Compiler diagnostics go to `log` (may be NULL). */
int ode_rhs_compile(ode_handle* h, const char* body, int dim, int nparams, int* rhs_id, char* log, size_t loglen);

/* ---- every-step output of the adaptive solvers ---------------------------
 * The reference's default for GPUSimpleATsit5 / AVern7 / AVern9 without
 * saveat is save_everystep = true: sol.t and sol.u hold t0, u0 and the time
 * and state after every accepted step (src/tsit5/gpuatsit5.jl:225-229,
 * :301-303; gpuvern7.jl:320-324, :428-430; gpuvern9.jl:431-435, :597-599),
 * a different length for every trajectory.  This call returns that ragged output for the whole ensemble in
 * two passes: the first counts each trajectory's accepted steps, the second
 * (same solve, bit-identical) writes the points.  Trajectory i's points are
 * rows offsets[i] .. offsets[i+1]-1 of ts[rows] and us[rows][dim].
 * Buffers are host or device memory as a->memory says; `a` must name an
 * adaptive algorithm, no saveat and the state output.  If ts or us is NULL or
 * capacity < total, only offsets and total are written and ODE_ESMALL is
 * returned: allocate total rows and call again.  No counterpart in the
 * reference beyond the per-trajectory push! it replaces. */
typedef struct {
  int64_t* offsets;   /* [n+1] first row of each trajectory; offsets[n] = total */
  double* ts;         /* [capacity] */
  double* us;         /* [capacity][dim] */
  int64_t capacity;   /* rows the ts / us buffers hold */
  int64_t total;      /* out: rows needed (sum over trajectories of accepted steps + 1) */
  double* u_final;    /* [dim][n], or NULL */
  double* t_final;    /* [n], or NULL */
  int8_t* retcode;    /* [n], or NULL */
  int32_t* naccept;   /* [n], or NULL */
  int32_t* nreject;   /* [n], or NULL */
} ode_everystep_out;

int ode_ensemble_solve_everystep(ode_handle* h, const ode_solve_args* a, ode_everystep_out* o,
                                 ode_solve_stats* stats);

/* Compile a saveat output function with NVRTC: an ensemble output_func fused
 * into the solve, applied to every saved point on the device instead of on the
 * host afterwards.  `body` is the body of
 *   __device__ void output(double* out, const double* u, const double* p, double t)
 * which writes `width` values from the saved state u (dim values), the
 * trajectory's parameters p (nparams values) and the save time t.  With
 * ode_solve_args.output = *output_id, us holds [npoints][width][n].  Compiler
 * diagnostics go to `log` (may be NULL).  No counterpart in the reference:
 * SciMLBase's EnsembleProblem applies output_func on the host, per trajectory. */
int ode_output_compile(ode_handle* h, const char* body, int dim, int nparams, int width, int* output_id, char* log,
                       size_t loglen);

/* ---- SimpleEM: Euler-Maruyama SDE ensembles ---------------------------------
 * DiffEqBase.solve(prob::SDEProblem, SimpleEM(); dt), src/euler_maruyama.jl:48-142,
 * for a whole ensemble:
 *   n = Int((tf - t0)/dt) + 1 points t_k = t0 + k*dt,
 *   diagonal noise:      u_{k+1} = u_k + f(u_k, p, t_k)*dt + sqrt(dt)*g(u_k, p, t_k) .* xi_k,
 *   non-diagonal noise:  u_{k+1} = u_k + f(u_k, p, t_k)*dt + sqrt(dt)*(G(u_k, p, t_k) * xi_k),
 * G a dim x noise_dim matrix (the reference's noise_rate_prototype) and xi_k
 * noise_dim normals.  The reference draws xi_k with Julia's randn; here each
 * trajectory has one stream of normals from a counter-based generator
 * (Philox4x32-10 keyed by `seed`, counter = pair index, trajectory;
 * Box-Muller of the two 53-bit uniforms in double-single arithmetic, within
 * about 2^-43 of the exact transform) that its steps consume in order, so
 * results depend only on (seed, trajectory index) and are reproducible on
 * the CPU. */
enum {
  ODE_SDE_GBM = 0,     /* geometric Brownian motion: f = mu u, g = sigma u (any dim), p = (mu, sigma) */
  ODE_SDE_OU = 1,      /* Ornstein-Uhlenbeck: f = theta (mu - u), g = sigma (any dim), p = (theta, mu, sigma) */
  ODE_SDE_LORENZ = 2,  /* Lorenz drift, additive noise: dim 3, p = (sigma, rho, beta, noise) */
  ODE_SDE_MULT = 3,    /* non-diagonal multiplicative noise: f = mu u, G[d][m] = c[d][m] u[d] (noise_dim >= 1),
                          p = (mu, c row-major dim x noise_dim); the reference's test SDE, test/simpleem_tests.jl */
  ODE_SDE_USER = 1000
};

typedef struct {
  int32_t sde;            /* ODE_SDE_* or an id from ode_sde_compile */
  int64_t n;              /* trajectories */
  int32_t dim, nparams;
  double t0, tf, dt;      /* (tf - t0)/dt must be an integer (the reference's Int(...) throws otherwise) */
  uint64_t seed;
  int32_t save_everystep; /* 1: every grid point (what the reference returns); 0: final state only */
  int32_t memory;         /* ODE_MEM_HOST or ODE_MEM_DEVICE */
  const double* u0;       /* [dim][n] */
  const double* p;        /* [nparams][n] */
  void* stream;           /* cudaStream_t, or NULL */
  int32_t noise_dim;      /* 0: diagonal noise; M >= 1: dim x M noise matrix (ODE_SDE_MULT, user SDEs compiled so) */
} ode_sde_args;

typedef struct {
  double* us;             /* [npoints][dim][n] (save_everystep), or NULL */
  double* u_final;        /* [dim][n], or NULL */
} ode_sde_out;

int ode_sde_solve(ode_handle* h, const ode_sde_args* a, ode_sde_out* o, ode_solve_stats* stats);

/* Compile a user SDE with NVRTC: `drift` and `diffusion` are the bodies of
 *   __device__ void drift(double* f, const double* u, const double* p, double t)
 *   __device__ void diffusion(double* g, const double* u, const double* p, double t)
 * (diagonal noise: g has dim components). */
int ode_sde_compile(ode_handle* h, const char* drift, const char* diffusion, int dim, int nparams, int* sde_id,
                    char* log, size_t loglen);
/* The same for non-diagonal noise: `diffusion` writes the dim x noise_dim
 * matrix row-major, g[d * noise_dim + m] (noise_dim 0: diagonal, as above).
 * Solve it with ode_sde_args.noise_dim = noise_dim. */
int ode_sde_compile_noise(ode_handle* h, const char* drift, const char* diffusion, int dim, int noise_dim,
                          int nparams, int* sde_id, char* log, size_t loglen);

/* ---- autotuner ----------------------------------------------------------
 * Times launch-shape variants of the solver kernel (threads per block,
 * register cap, bytes of the per-warp saveat staging ring) on the first
 * `sample` trajectories of `a` (<= 0: 65,536) and keeps the fastest for later
 * solves of the same algorithm / rhs / precision / dim / schedule kind on this
 * handle.  Variants differ only in launch shape: results are unchanged.  The
 * persistent kernel hands trajectories to lanes dynamically, so there is no
 * fixed trajectories-per-thread parameter to tune.  With ODE_SCHED_LEARNED
 * and a fitted model the sample is timed in the learned order.  The search
 * covers threads per block {128, 64, 32} x register caps {none, 128, 112,
 * 96, 80} x staging-ring bytes that hold at least 32 saveat jobs and fit the
 * 48 KB of static shared memory a block may have. */
#define ODE_TUNE_MAX_VARIANTS 64
typedef struct {
  int32_t block, max_registers, stage_bytes;
  float ms;               /* best kernel time on the sample; < 0: did not compile or load */
} ode_tune_variant;

typedef struct {
  int32_t variants;       /* variants timed */
  int32_t block;          /* chosen threads per block */
  int32_t max_registers;  /* chosen register cap (0: the compiler's choice) */
  int32_t stage_bytes;    /* chosen staging-ring bytes per warp */
  double default_ms;      /* kernel time of the default kernel on the sample */
  double best_ms;         /* kernel time of the chosen kernel on the sample */
  int64_t sample;         /* trajectories timed */
  double tune_ms;         /* wall time of the tuning */
  int32_t ntable;         /* rows of `table` filled */
  ode_tune_variant table[ODE_TUNE_MAX_VARIANTS];  /* every variant tried, in search order */
} ode_tune_report;

int ode_autotune(ode_handle* h, const ode_solve_args* a, int64_t sample, ode_tune_report* rep);

/* Autotuning cache: ode_tune_save writes the launch shapes this handle has
 * chosen (built-in right-hand sides and outputs only) to a text file tagged
 * with the GPU's name and SM count; ode_tune_load reads such a file and, if
 * it was written on the same kind of GPU, makes later solves use those shapes
 * without tuning again (the kernels are compiled on first use).  A file from
 * another GPU is ignored (ODE_ENOTSUP). */
int ode_tune_save(ode_handle* h, const char* path);
int ode_tune_load(ode_handle* h, const char* path);

/* ---- learned schedule ---------------------------------------------------
 * A 2-hidden-layer ReLU MLP (bf16 weights, fp32 accumulation) maps each
 * trajectory's (p, u0) to (log attempts, log dt of the first accepted step).
 * It is trained on the GPU on counts the plain solver records for a training
 * ensemble, then used by ODE_SCHED_LEARNED to order trajectories by predicted
 * cost (longest first) and, if asked, to seed each trajectory's initial dt. */
typedef struct {
  int32_t hidden;      /* hidden width (default 64) */
  int32_t epochs;      /* passes over the training set (default 30) */
  int32_t batch;       /* minibatch size (default 1024) */
  float lr;            /* Adam learning rate (default 5e-3) */
  uint64_t seed;       /* initialisation and shuffling seed */
  int32_t seed_dt0;    /* 1: seed each trajectory's initial dt with the prediction in
                          ODE_SCHED_LEARNED (default 0: ordering only, results
                          bit-identical to the plain schedule) */
  float dt0_safety;    /* predicted dt0 is multiplied by this (default 1.0) */
} ode_learn_opts;

typedef struct {
  float loss_first, loss_last;  /* training loss of the first and last epoch */
  float r2_attempts;            /* R^2 of log attempts on the training set */
  double train_solve_ms;        /* wall time of the training ensemble's solve (step counts recorded) */
  double train_fit_ms;          /* wall time of the fit: targets, standardisation, upload, training kernel */
  double train_kernel_ms;       /* device time of the training kernel (CUDA events), all epochs */
  int32_t train_ctas;           /* CTAs of the thread-block cluster that trained (16 or 8) */
} ode_learn_report;

/* Fill `o` with defaults. */
void ode_learn_default_opts(ode_learn_opts* o);
/* Solve the training ensemble `a` with the plain schedule, record its step
 * counts and fit the model held by the handle.  `a` follows ode_ensemble_solve. */
int ode_learn_fit(ode_handle* h, const ode_solve_args* a, const ode_learn_opts* opts, ode_learn_report* rep);
/* Predicted (log attempts, log dt_first) per trajectory into host arrays (either may be NULL). */
int ode_learn_predict(ode_handle* h, const ode_solve_args* a, float* log_attempts, float* log_dt_first);
/* One forward and backward pass of the training kernel on a batch, for
 * verification: params in the flat layout W1[nh][nin] b1[nh] W2[nh][nh]
 * b2[nh] W3[2][nh] b3[2] (rounded to bf16 as training uses them), x
 * [batch][nin], y [batch][2]; writes the fp32 gradient of the loss
 * mean_b sum_o (out - y)^2 and the loss. */
int ode_learn_gradcheck(ode_handle* h, int nin, int nh, int64_t batch, const float* params, const float* x,
                        const float* y, float* grad, float* loss);

/* ---- allocation-free solve ------------------------------------------------
 * No counterpart in the reference: an entry point for callers that cannot
 * allocate GPU memory, such as applications that own the whole device memory
 * budget (pools sized at start-up) or real-time loops that cannot afford
 * cudaMalloc/cudaFree synchronising the device.  The caller passes device
 * buffers of the current device for every input and output (memory =
 * ODE_MEM_DEVICE; managed memory is accepted too); `saveat` may be host or
 * device memory (it is copied into the scratch array); the solver's
 * own scratch (work counter, statistics, saveat times) lives in a fixed
 * 33,024-byte array inside the library's device image, which every GPU that
 * loads the library keeps until the process exits.
 *
 * Runs GPUSimpleATsit5, FP64, built-in Lorenz, persistent schedule (the
 * kernel of ode_ensemble_solve with ODE_SCHED_PERSISTENT, identical results);
 * other combinations return ODE_ENOTSUP, more than ODE_NOALLOC_MAX_SAVE saveat
 * points ODE_EINVAL.  No handle: diagnostics go to `err` (may be NULL).
 * The first call on a device (with that device current) looks the scratch
 * array up; make it before any stream capture.  All calls share the array:
 * calls that overlap on the GPU race, so serialise them.  Runs on
 * a->stream (NULL: the default stream) and returns after the solve finished. */
#define ODE_NOALLOC_MAX_SAVE 4096
int ode_ensemble_solve_noalloc(const ode_solve_args* a, ode_solve_out* o, char* err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* GB300ODE_H */
