/* C ABI of the SimpleEM (Euler-Maruyama) ensemble solver: ode_sde_solve and
 * ode_sde_compile.  The kernels are in sde_solver.cuh; the built-in SDEs of
 * low dimension are compiled ahead of time here, every other (SDE, dim) pair
 * and every user SDE at run time with NVRTC. */
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gb300ode.h"
#include "ode_host.h"
#include "sde_solver.cuh"

GBODE_SDE_ENTRY(gbode_sde_gbm1, gbode::SdeGBM<1>)
GBODE_SDE_ENTRY(gbode_sde_gbm3, gbode::SdeGBM<3>)
GBODE_SDE_ENTRY(gbode_sde_ou1, gbode::SdeOU<1>)
GBODE_SDE_ENTRY(gbode_sde_lorenz3, gbode::SdeLorenz)

using namespace gbode;

namespace {

#define SCK(call, what)                                  \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
  } while (0)

constexpr int kBlock = 128;

int check_sde(ode_handle* h, const ode_sde_args* a) {
  if (a->noise_dim < 0 || a->noise_dim > 32) return fail(h, ODE_EINVAL, "noise_dim must be in [0, 32]");
  if (a->sde == ODE_SDE_MULT) {
    if (a->dim < 1 || a->dim > 32 || a->noise_dim < 1 || a->dim * a->noise_dim > 64 ||
        a->nparams != 1 + a->dim * a->noise_dim)
      return fail(h, ODE_EINVAL, "non-diagonal multiplicative noise needs noise_dim >= 1, dim x noise_dim <= 64, "
                                 "1 + dim x noise_dim parameters");
    return ODE_OK;
  }
  if (a->noise_dim != 0 && a->sde < ODE_SDE_USER)
    return fail(h, ODE_EINVAL, "this built-in SDE has diagonal noise (noise_dim 0)");
  switch (a->sde) {
    case ODE_SDE_GBM:
      if (a->dim < 1 || a->dim > 32 || a->nparams != 2) return fail(h, ODE_EINVAL, "GBM needs 1 <= dim <= 32, 2 parameters");
      return ODE_OK;
    case ODE_SDE_OU:
      if (a->dim < 1 || a->dim > 32 || a->nparams != 3) return fail(h, ODE_EINVAL, "OU needs 1 <= dim <= 32, 3 parameters");
      return ODE_OK;
    case ODE_SDE_LORENZ:
      if (a->dim != 3 || a->nparams != 4) return fail(h, ODE_EINVAL, "stochastic Lorenz needs dim 3, 4 parameters");
      return ODE_OK;
  }
  if (a->sde >= ODE_SDE_USER && a->sde < ODE_SDE_USER + (int)h->sdes.size()) {
    const UserSde& u = h->sdes[a->sde - ODE_SDE_USER];
    if (u.dim != a->dim || u.nparams != a->nparams || u.noise_dim != a->noise_dim)
      return fail(h, ODE_EINVAL, "the SDE was compiled for another dim / nparams / noise_dim");
    return ODE_OK;
  }
  return fail(h, ODE_EINVAL, "unknown SDE");
}

/* Translation unit for NVRTC: the SDE type and one entry point gbode_jit. */
std::string sde_source(ode_handle* h, const ode_sde_args* a) {
  std::string src = "#include \"sde_solver.cuh\"\n";
  char buf[256];
  if (a->sde >= ODE_SDE_USER) {
    const UserSde& u = h->sdes[a->sde - ODE_SDE_USER];
    snprintf(buf, sizeof buf, "struct UserSde {\n  enum { D = %d, M = %d, GN = %d, NP = %d };\n  double p[%d];\n",
             u.dim, u.noise_dim, u.noise_dim > 0 ? u.dim * u.noise_dim : u.dim, u.nparams,
             u.nparams > 0 ? u.nparams : 1);
    src += buf;
    src += "  __device__ static __forceinline__ void user_drift(double* f, const double* u, const double* p, "
           "double t) {\n";
    src += u.drift;
    src += "\n  }\n  __device__ static __forceinline__ void user_diffusion(double* g, const double* u, "
           "const double* p, double t) {\n";
    src += u.diffusion;
    src += "\n  }\n"
           "  __device__ __forceinline__ void drift(const double (&u)[D], double t, double (&f)[D]) const {\n"
           "    user_drift(f, u, p, t);\n  }\n"
           "  __device__ __forceinline__ void diffusion(const double (&u)[D], double t, double (&g)[GN]) const {\n"
           "    user_diffusion(g, u, p, t);\n  }\n};\n";
    src += "GBODE_SDE_ENTRY(gbode_jit, UserSde)\n";
    return src;
  }
  if (a->sde == ODE_SDE_MULT)  /* a typedef: the macro argument may not hold the template's comma */
    snprintf(buf, sizeof buf, "typedef gbode::SdeMult<%d, %d> SdeT;\nGBODE_SDE_ENTRY(gbode_jit, SdeT)\n", a->dim,
             a->noise_dim);
  else if (a->sde == ODE_SDE_GBM) snprintf(buf, sizeof buf, "GBODE_SDE_ENTRY(gbode_jit, gbode::SdeGBM<%d>)\n", a->dim);
  else if (a->sde == ODE_SDE_OU) snprintf(buf, sizeof buf, "GBODE_SDE_ENTRY(gbode_jit, gbode::SdeOU<%d>)\n", a->dim);
  else snprintf(buf, sizeof buf, "GBODE_SDE_ENTRY(gbode_jit, gbode::SdeLorenz)\n");
  return src + buf;
}

int sde_kernel(ode_handle* h, const ode_sde_args* a, CUfunction* fn) {
  char key[64];
  snprintf(key, sizeof key, "%d|%d|%d", a->sde, a->dim, a->noise_dim);
  auto it = h->sde_kernels.find(key);
  if (it != h->sde_kernels.end()) {
    *fn = it->second;
    return ODE_OK;
  }
  const void* aot = nullptr;
  if (a->sde == ODE_SDE_GBM && a->dim == 1) aot = (const void*)gbode_sde_gbm1;
  if (a->sde == ODE_SDE_GBM && a->dim == 3) aot = (const void*)gbode_sde_gbm3;
  if (a->sde == ODE_SDE_OU && a->dim == 1) aot = (const void*)gbode_sde_ou1;
  if (a->sde == ODE_SDE_LORENZ) aot = (const void*)gbode_sde_lorenz3;
  if (aot) {
    cudaFunction_t f;
    SCK(cudaGetFuncBySymbol(&f, aot), "cudaGetFuncBySymbol");
    *fn = (CUfunction)f;
  } else {
    std::string log;
    const int rc = jit_function(h, sde_source(h, a), kBlock, fn, &log);
    if (rc != ODE_OK) return rc;
  }
  h->sde_kernels[key] = *fn;
  return ODE_OK;
}

}  // namespace

extern "C" {

int ode_sde_compile(ode_handle* h, const char* drift, const char* diffusion, int dim, int nparams, int* sde_id,
                    char* log, size_t loglen) {
  return ode_sde_compile_noise(h, drift, diffusion, dim, 0, nparams, sde_id, log, loglen);
}

int ode_sde_compile_noise(ode_handle* h, const char* drift, const char* diffusion, int dim, int noise_dim,
                          int nparams, int* sde_id, char* log, size_t loglen) {
  if (!h) return ODE_EINVAL;
  if (!drift || !diffusion || !sde_id || dim < 1 || dim > 32 || nparams < 0 || nparams > 256 || noise_dim < 0 ||
      noise_dim > 32 || dim * noise_dim > 256)
    return fail(h, ODE_EINVAL, "ode_sde_compile: bad arguments");
  SCK(cudaSetDevice(h->device), "cudaSetDevice");
  UserSde u;
  u.drift = drift;
  u.diffusion = diffusion;
  u.dim = dim;
  u.nparams = nparams;
  u.noise_dim = noise_dim;
  h->sdes.push_back(u);
  ode_sde_args a;
  std::memset(&a, 0, sizeof a);
  a.sde = ODE_SDE_USER + (int)h->sdes.size() - 1;
  a.dim = dim;
  a.nparams = nparams;
  a.noise_dim = noise_dim;
  CUfunction fn;
  std::string lg;
  const int rc = jit_function(h, sde_source(h, &a), kBlock, &fn, &lg);
  if (log && loglen) {
    std::strncpy(log, lg.c_str(), loglen - 1);
    log[loglen - 1] = '\0';
  }
  if (rc != ODE_OK) {
    h->sdes.pop_back();
    return rc;
  }
  char key[64];
  snprintf(key, sizeof key, "%d|%d|%d", a.sde, a.dim, a.noise_dim);
  h->sde_kernels[key] = fn;
  *sde_id = a.sde;
  return ODE_OK;
}

int ode_sde_solve(ode_handle* h, const ode_sde_args* a, ode_sde_out* o, ode_solve_stats* st) {
  const auto wall0 = std::chrono::steady_clock::now();
  if (!h) return ODE_EINVAL;
  if (!a || !o) return fail(h, ODE_EINVAL, "null argument");
  if (a->n < 0 || a->n > 0x7fffffffLL) return fail(h, ODE_EINVAL, "n must be in [0, 2^31)");
  if (a->memory != ODE_MEM_HOST && a->memory != ODE_MEM_DEVICE) return fail(h, ODE_EINVAL, "unknown memory kind");
  if (a->n > 0 && (!a->u0 || (a->nparams > 0 && !a->p))) return fail(h, ODE_EINVAL, "u0/p missing");
  int rc = check_sde(h, a);
  if (rc != ODE_OK) return rc;
  /* n = Int((tf - t0)/dt) + 1: Julia's Int(x) accepts only integral x */
  const double q = (a->tf - a->t0) / a->dt;
  if (!(a->dt > 0) || !(q >= 0) || q != std::floor(q) || q > 4294967295.0)
    return fail(h, ODE_EINVAL, "(tf - t0)/dt must be a non-negative integer below 2^32 (InexactError in the reference)");
  const long long nsteps = (long long)q;
  SCK(cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t s = a->stream ? (cudaStream_t)a->stream : h->stream;
  const long long n = a->n;
  const int D = a->dim, NP = a->nparams;
  CUfunction fn;
  rc = sde_kernel(h, a, &fn);
  if (rc != ODE_OK) return rc;

  SParams sp;
  std::memset(&sp, 0, sizeof sp);
  sp.n = n;
  sp.nsteps = nsteps;
  sp.t0 = a->t0;
  sp.dt = a->dt;
  sp.seed = a->seed;
  sp.dim = D;
  sp.nparams = NP;
  sp.noise_dim = a->noise_dim;
  sp.save_everystep = a->save_everystep ? 1 : 0;
  const bool host = a->memory == ODE_MEM_HOST;
  const size_t nd = (size_t)n * sizeof(double);
  const size_t us_bytes = a->save_everystep && o->us ? (size_t)(nsteps + 1) * D * nd : 0;
  if (host) {
    double* du0 = (double*)buf(h, "sde_u0", nd * D, &rc);
    if (!du0) return rc;
    double* dp = (double*)buf(h, "sde_p", nd * (NP > 0 ? NP : 1), &rc);
    if (!dp) return rc;
    if (n > 0) {
      SCK(cudaMemcpyAsync(du0, a->u0, nd * D, cudaMemcpyHostToDevice, s), "copy u0");
      if (NP > 0) SCK(cudaMemcpyAsync(dp, a->p, nd * NP, cudaMemcpyHostToDevice, s), "copy p");
    }
    sp.u0 = du0;
    sp.p = dp;
    if (us_bytes && !(sp.us = (double*)buf(h, "sde_us", us_bytes, &rc))) return rc;
    if (o->u_final && !(sp.u_final = (double*)buf(h, "sde_uf", nd * D, &rc))) return rc;
  } else {
    sp.u0 = a->u0;
    sp.p = a->p;
    sp.us = us_bytes ? o->us : nullptr;
    sp.u_final = o->u_final;
  }
  SCK(cudaEventRecord(h->ev0, s), "event");
  if (n > 0) {
    rc = launch_params(h, fn, (unsigned)((n + kBlock - 1) / kBlock), kBlock, &sp, s);
    if (rc != ODE_OK) return rc;
  }
  SCK(cudaEventRecord(h->ev1, s), "event");
  if (host) {
    if (us_bytes) SCK(cudaMemcpyAsync(o->us, sp.us, us_bytes, cudaMemcpyDeviceToHost, s), "copy us");
    if (o->u_final) SCK(cudaMemcpyAsync(o->u_final, sp.u_final, nd * D, cudaMemcpyDeviceToHost, s), "copy u_final");
  }
  SCK(cudaStreamSynchronize(s), "SDE solve");
  if (st) {
    float ms = 0;
    SCK(cudaEventElapsedTime(&ms, h->ev0, h->ev1), "event time");
    std::memset(st, 0, sizeof *st);
    st->kernel_ms = ms;
    st->attempts = n * nsteps;
    st->launches = n > 0 ? 1 : 0;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  }
  return ODE_OK;
}

}  // extern "C"
