/* ode_ensemble_solve_noalloc: an ensemble solve that allocates no GPU memory.
 *
 * Who needs it: callers that cannot call cudaMalloc.  A host application
 * that owns the whole device memory budget (pools sized at start-up, every
 * byte accounted) does not let a library take device memory of its own, and
 * real-time loops cannot afford cudaMalloc/cudaFree, which may synchronise the
 * device.  Such callers already hold device buffers for their inputs and
 * outputs; what they cannot provide is the solver's scratch memory.
 *
 * What it runs: the persistent adaptive Tsitouras 5(4) kernel (GPUSimpleATsit5,
 * FP64) for the built-in Lorenz right-hand side — the same kernel template as
 * ode_ensemble_solve with ODE_SCHED_PERSISTENT, so the results are identical.
 * Its scratch (the work counter the persistent warps draw trajectories from,
 * the statistics counters and a device copy of the saveat times) lives in
 * g_noalloc_scratch below, a fixed-size array in the library's device image:
 * every GPU that loads the library holds these 33,024 bytes until the process
 * exits.  At most ODE_NOALLOC_MAX_SAVE saveat points fit.
 *
 * Set-up: the first call on a device, with that device current, looks up the
 * array's device address with cudaGetSymbolAddress (the array's name in host
 * code is only a host-side stand-in, not a device address) and keeps it for
 * later calls on that device.  Make that first call before any stream capture.
 *
 * Arguments: every input and output array is device memory of the current
 * device (or managed memory); the saveat times may be host or device memory
 * (they are copied into the scratch array).
 *
 * Sharing: every call uses the same array and the array keeps the last call's
 * contents; each call clears the counters it needs at its start.  Calls that
 * overlap on the GPU (other host threads, or other streams before the
 * previous call finished) race on the array: serialise them.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gb300ode.h"
#define GBODE_CTRL_DS 1 /* the library's default error norm and controller */
#include "ode_solver.cuh"

namespace {

/* scratch layout: [0, 32) statistics (attempts, saves, early stops) and the
 * work counter; [256, 256 + 8*ODE_NOALLOC_MAX_SAVE) the saveat times */
constexpr size_t kStatsOffset = 0;
constexpr size_t kSaveatOffset = 256;
constexpr size_t kScratchBytes = kSaveatOffset + 8 * (size_t)ODE_NOALLOC_MAX_SAVE;
static_assert(kScratchBytes == 33024, "scratch size stated in the header comment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

typedef gbode::RhsLorenz<double, double> LorenzFP64;
GBODE_ENTRY(gbode_noalloc_atsit5_persistent_lorenz3_fp64, persistent, gbode::MTsit5, gbode::PFP64, LorenzFP64)

/* the attempt cap used when the caller gives none (the same as ode_ensemble_solve) */
constexpr long long kDefaultMaxIters = 1000000;

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_dev[kMaxDevices];
int g_resident_blocks[kMaxDevices];

int say(char* err, size_t errlen, int code, const char* msg) {
  if (err && errlen) {
    std::strncpy(err, msg, errlen - 1);
    err[errlen - 1] = '\0';
  }
  return code;
}

int say_cuda(char* err, size_t errlen, cudaError_t e, const char* what) {
  if (err && errlen) std::snprintf(err, errlen, "%s: %s", what, cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? ODE_ENOMEM : ODE_ECUDA;
}

/* p is NULL, or memory the current device `dev` can use in a kernel: its own
 * device memory, or managed memory */
bool on_device(const void* p, int dev) {
  if (!p) return true;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == dev;
}

}  // namespace

extern "C" int ode_ensemble_solve_noalloc(const ode_solve_args* a, ode_solve_out* o, char* err, size_t errlen) {
  if (!a || !o) return say(err, errlen, ODE_EINVAL, "null argument");
  if (a->alg != ODE_ALG_ATSIT5 || a->rhs != ODE_RHS_LORENZ || a->dim != 3 || a->nparams != 3 ||
      a->precision != ODE_FP64)
    return say(err, errlen, ODE_ENOTSUP,
               "the allocation-free solve runs GPUSimpleATsit5, FP64, built-in Lorenz (dim 3, 3 parameters) only");
  if (a->output != ODE_OUTPUT_STATE)
    return say(err, errlen, ODE_ENOTSUP, "the allocation-free solve stores the state at saveat points only");
  if (a->schedule != ODE_SCHED_PERSISTENT)
    return say(err, errlen, ODE_ENOTSUP, "the allocation-free solve runs the persistent schedule only");
  if (a->controller != ODE_CTRL_DS)
    return say(err, errlen, ODE_ENOTSUP, "the allocation-free solve runs the default (double-single) error norm "
                                         "and step-size controller");
  if (a->layout != ODE_LAYOUT_SOA && a->layout != ODE_LAYOUT_TRAJ)
    return say(err, errlen, ODE_EINVAL, "unknown output layout");
  if (a->memory != ODE_MEM_DEVICE)
    return say(err, errlen, ODE_EINVAL, "the allocation-free solve takes device buffers (memory = ODE_MEM_DEVICE)");
  if (a->n < 0 || a->n > 0x7fffffffLL) return say(err, errlen, ODE_EINVAL, "n must be in [0, 2^31)");
  if (a->nsave < 0 || a->nsave > ODE_NOALLOC_MAX_SAVE || (a->nsave > 0 && !a->saveat))
    return say(err, errlen, ODE_EINVAL, "nsave must be in [0, ODE_NOALLOC_MAX_SAVE] (4096) with saveat given");
  if (!(a->t0 == a->t0) || !(a->tf == a->tf) || !(a->dt == a->dt))
    return say(err, errlen, ODE_EINVAL, "t0, tf and dt must not be NaN");
  if (a->n > 0 && (!a->u0 || !a->p)) return say(err, errlen, ODE_EINVAL, "u0/p missing");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return say_cuda(err, errlen, e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return say(err, errlen, ODE_ENOTSUP, "device index out of range");
  const void* dev_ptrs[] = {a->u0, a->p, a->dt0, o->us, o->u_final, o->t_final, o->retcode, o->naccept,
                            o->nreject, o->dt_first};
  for (const void* q : dev_ptrs)
    if (!on_device(q, dev))
      return say(err, errlen, ODE_EINVAL, "every array must be a device pointer of the current device");
  {
    /* once per device: the scratch array's device address and the grid size */
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_dev[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) return say_cuda(err, errlen, e, "cudaGetSymbolAddress");
      int nsm = 0, nb = 0;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return say_cuda(err, errlen, e, "cudaDeviceGetAttribute");
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, gbode_noalloc_atsit5_persistent_lorenz3_fp64, 128, 0);
      if (e != cudaSuccess) return say_cuda(err, errlen, e, "occupancy");
      g_resident_blocks[dev] = (nb < 1 ? 1 : nb) * nsm;
      g_scratch_dev[dev] = (unsigned char*)ptr;
    }
  }
  unsigned char* scratch = g_scratch_dev[dev];
  cudaStream_t s = (cudaStream_t)a->stream;

  gbode::KParams kp;
  std::memset(&kp, 0, sizeof kp);
  kp.n = a->n;
  kp.t0 = a->t0;
  kp.tf = a->tf;
  kp.dt = a->dt;
  kp.abstol = a->abstol;
  kp.reltol = a->reltol;
  kp.u0 = a->u0;
  kp.p = a->p;
  kp.dt0 = a->dt0;
  kp.nsave = a->nsave;
  kp.dim = 3;
  kp.nparams = 3;
  kp.maxiters = a->maxiters > 0 ? a->maxiters : kDefaultMaxIters;
  kp.norm_fp64 = a->abstol < 1e-30 ? 1 : 0;  /* the same rule as ode_ensemble_solve */
  gbode::ds_split_host(a->abstol, kp.tol_ds);
  gbode::ds_split_host(a->reltol, kp.tol_ds + 2);
  kp.us = o->us;
  if (a->layout == ODE_LAYOUT_TRAJ) {
    kp.us_sj = 3;
    kp.us_sw = 1;
    kp.us_si = 3 * a->nsave;
  } else {
    kp.us_sj = 3 * a->n;
    kp.us_sw = a->n;
    kp.us_si = 1;
  }
  kp.u_final = o->u_final;
  kp.t_final = o->t_final;
  kp.retcode = (signed char*)o->retcode;
  kp.naccept = o->naccept;
  kp.nreject = o->nreject;
  kp.dt_first = o->dt_first;
  kp.stats = (unsigned long long*)(scratch + kStatsOffset);
  kp.counter = kp.stats + 3;
  kp.saveat = a->nsave > 0 ? (const double*)(scratch + kSaveatOffset) : nullptr;

  /* the previous call left its counters behind: clear them */
  e = cudaMemsetAsync(scratch + kStatsOffset, 0, 4 * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return say_cuda(err, errlen, e, "clear scratch");
  if (a->nsave > 0) {
    /* saveat may be host or device memory: the copy direction follows the pointer */
    e = cudaMemcpyAsync(scratch + kSaveatOffset, a->saveat, (size_t)a->nsave * sizeof(double), cudaMemcpyDefault,
                        s);
    if (e != cudaSuccess) return say_cuda(err, errlen, e, "copy saveat");
  }
  if (a->n > 0) {
    const long long blocks_needed = (a->n + 127) / 128;
    const unsigned grid = (unsigned)(blocks_needed < g_resident_blocks[dev] ? blocks_needed : g_resident_blocks[dev]);
    gbode_noalloc_atsit5_persistent_lorenz3_fp64<<<grid, 128, 0, s>>>(kp);
    e = cudaGetLastError();
    if (e != cudaSuccess) return say_cuda(err, errlen, e, "launch");
  }
  unsigned long long stats[3] = {0, 0, 0};
  e = cudaMemcpyAsync(stats, scratch + kStatsOffset, sizeof stats, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return say_cuda(err, errlen, e, "solve");
  if (stats[2] > 0) return say(err, errlen, ODE_ETRAJ, "some trajectories stopped early (dt<dtmin or maxiters)");
  return say(err, errlen, ODE_OK, "");
}
