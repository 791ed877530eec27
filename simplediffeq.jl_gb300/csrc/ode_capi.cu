/* C ABI of libgb300ode.so: handles, argument checking, device workspace,
 * kernel selection (prebuilt or compiled at run time with NVRTC), the plain /
 * persistent / learned schedules and CUDA-graph replay of repeated solves.
 *
 * ode_ensemble_solve replaces the per-trajectory solve methods of
 * SimpleDiffEq.jl's GPUSimple* solvers (see include/gb300ode.h for the list
 * with file:line citations) for a whole ensemble at once.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "jlrange.h"
#include "ode_host.h"

/* kernels compiled ahead of time, and the sources for run-time compilation */
#include "aot_registry.inc"
#include "embedded_src.inc"

namespace gbode {

/* Driver-API and NVRTC entry points, resolved at run time so that the library
 * loads on machines without a GPU driver (only the runtime is linked). */
struct DriverApi {
  bool ok = false;
  CUresult (*cuLaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned, unsigned,
                             CUstream, void**, void**) = nullptr;
  CUresult (*cuModuleLoadData)(CUmodule*, const void*) = nullptr;
  CUresult (*cuModuleGetFunction)(CUfunction*, CUmodule, const char*) = nullptr;
  CUresult (*cuModuleUnload)(CUmodule) = nullptr;
  CUresult (*cuOccupancyMaxActiveBlocksPerMultiprocessor)(int*, CUfunction, int, size_t) = nullptr;
  CUresult (*cuGetErrorName)(CUresult, const char**) = nullptr;
  CUresult (*cuGetErrorString)(CUresult, const char**) = nullptr;
  CUresult (*cuFuncGetAttribute)(int*, CUfunction_attribute, CUfunction) = nullptr;
};
struct NvrtcApi {
  bool ok = false;
  nvrtcResult (*create)(nvrtcProgram*, const char*, const char*, int, const char* const*, const char* const*);
  nvrtcResult (*compile)(nvrtcProgram, int, const char* const*);
  nvrtcResult (*logsize)(nvrtcProgram, size_t*);
  nvrtcResult (*log)(nvrtcProgram, char*);
  nvrtcResult (*cubinsize)(nvrtcProgram, size_t*);
  nvrtcResult (*cubin)(nvrtcProgram, char*);
  nvrtcResult (*destroy)(nvrtcProgram*);
  const char* (*errstr)(nvrtcResult);
};
static DriverApi g_drv;
static NvrtcApi g_nvrtc;

template <class F>
static bool drv_sym(const char* name, F* fp) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !p)
    return false;
  *fp = (F)p;
  return true;
}

static bool load_driver_api() {
  if (g_drv.ok) return true;
  DriverApi d;
  bool ok = drv_sym("cuLaunchKernel", &d.cuLaunchKernel) && drv_sym("cuModuleLoadData", &d.cuModuleLoadData) &&
            drv_sym("cuModuleGetFunction", &d.cuModuleGetFunction) && drv_sym("cuModuleUnload", &d.cuModuleUnload) &&
            drv_sym("cuOccupancyMaxActiveBlocksPerMultiprocessor", &d.cuOccupancyMaxActiveBlocksPerMultiprocessor) &&
            drv_sym("cuGetErrorName", &d.cuGetErrorName) && drv_sym("cuGetErrorString", &d.cuGetErrorString) &&
            drv_sym("cuFuncGetAttribute", &d.cuFuncGetAttribute);
  d.ok = ok;
  if (ok) g_drv = d;
  return ok;
}

static std::once_flag g_nvrtc_once;

static void load_nvrtc_once() {
  const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13"};
  void* h = nullptr;
  for (const char* n : names)
    if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL))) break;
  if (!h) return;
#define NV(field, sym) g_nvrtc.field = (decltype(g_nvrtc.field))dlsym(h, sym)
  NV(create, "nvrtcCreateProgram");
  NV(compile, "nvrtcCompileProgram");
  NV(logsize, "nvrtcGetProgramLogSize");
  NV(log, "nvrtcGetProgramLog");
  NV(cubinsize, "nvrtcGetCUBINSize");
  NV(cubin, "nvrtcGetCUBIN");
  NV(destroy, "nvrtcDestroyProgram");
  NV(errstr, "nvrtcGetErrorString");
#undef NV
  g_nvrtc.ok = g_nvrtc.create && g_nvrtc.compile && g_nvrtc.logsize && g_nvrtc.log && g_nvrtc.cubinsize &&
               g_nvrtc.cubin && g_nvrtc.destroy && g_nvrtc.errstr;
}

/* NVRTC is loaded on first use, once, safely from several threads. */
static bool load_nvrtc() {
  std::call_once(g_nvrtc_once, load_nvrtc_once);
  return g_nvrtc.ok;
}

int fail(ode_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}
int cuda_fail(ode_handle* h, cudaError_t e, const char* what) {
  /* the error is reported here: reset the runtime's per-thread last error so
   * that a later cudaGetLastError() check does not see it again (errors that
   * leave the context unusable stay sticky regardless) */
  cudaGetLastError();
  return fail(h, e == cudaErrorMemoryAllocation ? ODE_ENOMEM : ODE_ECUDA,
              std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}
int cu_fail(ode_handle* h, CUresult r, const char* what) {
  const char* name = nullptr;
  const char* str = nullptr;
  if (g_drv.ok) {
    g_drv.cuGetErrorName(r, &name);
    g_drv.cuGetErrorString(r, &str);
  }
  return fail(h, r == CUDA_ERROR_OUT_OF_MEMORY ? ODE_ENOMEM : ODE_ECUDA,
              std::string(what) + ": " + (name ? name : "?") + " (" + (str ? str : "?") + ")");
}

void* buf(ode_handle* h, const std::string& name, size_t bytes, int* rc) {
  DevBuf& b = h->bufs[name];
  if (bytes == 0) bytes = 16;
  if (b.cap < bytes) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.cap = 0;
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) {
      b.ptr = nullptr;
      *rc = cuda_fail(h, e, ("cudaMalloc " + name).c_str());
      return nullptr;
    }
    b.cap = bytes;
  }
  *rc = ODE_OK;
  return b.ptr;
}

}  // namespace gbode

using namespace gbode;

namespace {

#define CK(call, what)                                   \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
  } while (0)

/* Attempt cap used when the caller gives none: every trajectory loop on the
 * device must end, and the reference's loop has no cap of its own. */
const int64_t kDefaultMaxIters = 1000000;

bool is_fixed(int alg) {
  return alg == ODE_ALG_RK4 || alg == ODE_ALG_TSIT5 || alg == ODE_ALG_VERN7 || alg == ODE_ALG_VERN9 ||
         alg == ODE_ALG_EULER;
}
/* the one-step methods without saveat (they save every grid point) */
bool is_onestep(int alg) { return alg == ODE_ALG_RK4 || alg == ODE_ALG_EULER; }

const char* alg_name(int alg) {
  static const char* n[] = {"rk4", "tsit5", "atsit5", "vern7", "avern7", "vern9", "avern9", "euler"};
  return (alg >= 0 && alg <= 7) ? n[alg] : "?";
}
const char* prec_name(int p) {
  static const char* n[] = {"fp64", "fp32", "fp32k"};
  return (p >= 0 && p <= 2) ? n[p] : "?";
}

/* C++ names used to assemble a kernel for NVRTC */
const char* method_type(int alg) {
  switch (alg) {
    case ODE_ALG_RK4: return "gbode::MRK4";
    case ODE_ALG_EULER: return "gbode::MEuler";
    case ODE_ALG_TSIT5:
    case ODE_ALG_ATSIT5: return "gbode::MTsit5";
    case ODE_ALG_VERN7:
    case ODE_ALG_AVERN7: return "gbode::MVern7";
    case ODE_ALG_VERN9: return "gbode::MVern9";
    case ODE_ALG_AVERN9: return "gbode::MAVern9";
  }
  return "?";
}
const char* prec_type(int p) {
  switch (p) {
    case ODE_FP64: return "gbode::PFP64";
    case ODE_FP32: return "gbode::PFP32";
    case ODE_FP32_KAHAN: return "gbode::PFP32K";
  }
  return "?";
}
void rt_types(int p, const char** R, const char** T) {
  *R = (p == ODE_FP64) ? "double" : "float";
  *T = (p == ODE_FP32) ? "float" : "double";
}

/* Validate the (rhs, dim, nparams) triple; returns ODE_OK or an error. */
int check_rhs(ode_handle* h, const ode_solve_args* a) {
  switch (a->rhs) {
    case ODE_RHS_LORENZ:
      if (a->dim != 3 || a->nparams != 3) return fail(h, ODE_EINVAL, "Lorenz needs dim 3 and 3 parameters");
      return ODE_OK;
    case ODE_RHS_VANDERPOL:
      if (a->dim != 2 || a->nparams != 1) return fail(h, ODE_EINVAL, "Van der Pol needs dim 2 and 1 parameter");
      return ODE_OK;
    case ODE_RHS_R3BP:
      if (a->dim != 4 || a->nparams != 1) return fail(h, ODE_EINVAL, "R3BP needs dim 4 and 1 parameter");
      return ODE_OK;
    case ODE_RHS_KURAMOTO:
      if (a->dim < 1 || a->dim > 32 || a->nparams != a->dim + 1)
        return fail(h, ODE_EINVAL, "Kuramoto needs 1 <= dim <= 32 and dim+1 parameters");
      return ODE_OK;
    case ODE_RHS_LINEAR:
      if (a->dim < 1 || a->dim > 8 || a->nparams != a->dim * a->dim)
        return fail(h, ODE_EINVAL, "linear needs 1 <= dim <= 8 and dim*dim parameters");
      return ODE_OK;
  }
  if (a->rhs >= ODE_RHS_USER && a->rhs < ODE_RHS_USER + (int)h->users.size()) {
    const UserRhs& u = h->users[a->rhs - ODE_RHS_USER];
    if (a->dim != u.dim || a->nparams != u.nparams)
      return fail(h, ODE_EINVAL, "dim/nparams differ from the compiled user right-hand side");
    return ODE_OK;
  }
  return fail(h, ODE_EINVAL, "unknown right-hand side id");
}

std::string rhs_type_expr(ode_handle* /*h*/, const ode_solve_args* a) {
  const char *R, *T;
  rt_types(a->precision, &R, &T);
  char b[256];
  switch (a->rhs) {
    case ODE_RHS_LORENZ: snprintf(b, sizeof b, "gbode::RhsLorenz<%s, %s>", R, T); break;
    case ODE_RHS_VANDERPOL: snprintf(b, sizeof b, "gbode::RhsVanDerPol<%s, %s>", R, T); break;
    case ODE_RHS_R3BP: snprintf(b, sizeof b, "gbode::RhsR3BP<%s, %s>", R, T); break;
    case ODE_RHS_KURAMOTO: snprintf(b, sizeof b, "gbode::RhsKuramoto<%s, %s, %d>", R, T, a->dim); break;
    case ODE_RHS_LINEAR: snprintf(b, sizeof b, "gbode::RhsLinear<%s, %s, %d>", R, T, a->dim); break;
    default: snprintf(b, sizeof b, "RhsUser<%s, %s>", R, T); break;
  }
  return b;
}

/* kind of entry point: plain | persistent | staged | fixed | rk4.  The
 * persistent schedules use the staged driver (saveat interpolation batched
 * per warp through shared memory) when there are saveat points. */
const char* entry_kind(int alg, int sched, int64_t nsave) {
  if (is_onestep(alg)) return "onestep";
  if (is_fixed(alg)) return "fixed";
  if (sched == ODE_SCHED_PLAIN) return "plain";
  return nsave > 0 ? "staged" : "persistent";
}

/* Fixed-step Tsit5 on an ensemble of fewer warps than half the GPU's SM
 * sub-partitions (FP64, final states or every-step output, state output):
 * the kernel that spreads a trajectory's components over the warps of a
 * block (run_fixed_split), one block of 32 * dim threads per 32 trajectories.
 * Only for right-hand sides whose components are separate expressions (each
 * warp computes its own); one with shared work, like Kuramoto's sums of
 * sines, would repeat that work in every warp. */
bool use_fixed_split(const ode_handle* h, const ode_solve_args* a) {
  const bool separable = a->rhs == ODE_RHS_LORENZ || a->rhs == ODE_RHS_VANDERPOL || a->rhs == ODE_RHS_LINEAR;
  return a->alg == ODE_ALG_TSIT5 && separable && a->nsave == 0 && a->output == ODE_OUTPUT_STATE &&
         a->precision == ODE_FP64 && a->controller != ODE_CTRL_REF && a->dim >= 2 && a->dim <= 8 &&
         (a->n + 31) / 32 <= (int64_t)h->nsm * 2;
}

/* entry_kind, with the component-split fixed-step kernel where it applies */
const char* kernel_kind(const ode_handle* h, const ode_solve_args* a, int sched) {
  return use_fixed_split(h, a) ? "fixedsplit" : entry_kind(a->alg, sched, a->nsave);
}

int kernel_kind_id(const char* k) {
  if (!std::strcmp(k, "persistent")) return ODE_KERNEL_PERSISTENT;
  if (!std::strcmp(k, "staged")) return ODE_KERNEL_STAGED;
  if (!std::strcmp(k, "fixed")) return ODE_KERNEL_FIXED;
  if (!std::strcmp(k, "fixedsplit")) return ODE_KERNEL_FIXEDSPLIT;
  if (!std::strcmp(k, "onestep")) return ODE_KERNEL_ONESTEP;
  return ODE_KERNEL_PLAIN;
}

/* Bytes of one saveat job in the staged kernel's ring: the host-side copy of
 * StageLayout<M, PR, D, F>::JOB in ode_solver.cuh (3 times of type T, the
 * trajectory index, the saveat index, and D (x2 with Kahan) state values,
 * NK x D stage values and, for the Verner methods, the parameters, of type R). */
int stage_job_bytes(const ode_solve_args* a) {
  const int nk = a->alg == ODE_ALG_AVERN9 ? 16 : a->alg == ODE_ALG_AVERN7 ? 10 : 7;
  const int r = a->precision == ODE_FP64 ? 8 : 4, t = a->precision == ODE_FP32 ? 4 : 8;
  const bool dense_f = a->alg != ODE_ALG_ATSIT5;  /* Verner dense output evaluates f: parameters ride along */
  const int nrec = a->dim * (a->precision == ODE_FP32_KAHAN ? 2 : 1) + nk * a->dim + (dense_f ? a->nparams : 0);
  return 3 * t + 8 + nrec * r + 4;
}

/* Bytes per step record of the two-queue staged kernel of the Verner methods,
 * with room for two save points: the host-side copy of StageLayout2<...>::REC
 * + 2 * PT in ode_solver.cuh (3 times, trajectory, point count, state, stage
 * values, parameters and the extra dense-output stages; 8 bytes a point).
 * 0 for the methods without extra dense-output stages. */
int stage_record_bytes(const ode_solve_args* a) {
  const int nx = a->alg == ODE_ALG_AVERN9 ? 10 : a->alg == ODE_ALG_AVERN7 ? 6 : 0;
  if (!nx) return 0;
  const int nk = a->alg == ODE_ALG_AVERN9 ? 16 : 10;
  const int r = a->precision == ODE_FP64 ? 8 : 4, t = a->precision == ODE_FP32 ? 4 : 8;
  const int nrec = a->dim * (a->precision == ODE_FP32_KAHAN ? 2 : 1) + nk * a->dim + a->nparams + nx * a->dim;
  return 3 * t + 8 + 4 + nrec * r + 2 * 8;
}

/* Bytes a ring spends per queued unit: a step record for the Verner methods,
 * a save-point job otherwise. */
int stage_unit_bytes(const ode_solve_args* a) {
  const int rec = stage_record_bytes(a);
  return rec ? rec : stage_job_bytes(a);
}

/* Launch shape of an untuned run-time compiled kernel: 128 threads and 12 KB
 * staging rings, unless those rings cannot hold a round of 32 (a staged kernel
 * with large records): then one-warp blocks with the smallest ring that can,
 * up to 48 KB (measured on AVern9, restricted three-body problem, 65,536
 * trajectories, 100 save points: 161.7 ms unstaged, 116.4 ms staged in
 * one-warp blocks with 29 KB rings, 121.3 with 36 KB, 128.8 with 48 KB). */
void default_shape(const ode_solve_args* a, int sched, int* block, int* stage) {
  *block = 128;
  *stage = 12288;
  if (std::strcmp(entry_kind(a->alg, sched, a->nsave), "staged") != 0) return;
  const int unit = stage_unit_bytes(a);
  if (((12288 / unit) & ~7) >= 32) return;
  const int fit = (32 * unit + 511) / 512 * 512;
  if (fit > 49152) return;  /* no ring holds a round: the kernel runs unstaged */
  *block = 32;
  *stage = fit;
}

/* values stored per saveat point and trajectory */
int output_width(ode_handle* h, const ode_solve_args* a) {
  if (a->output == ODE_OUTPUT_KURAMOTO_R) return 1;
  if (a->output >= ODE_OUTPUT_USER) return h->outputs[a->output - ODE_OUTPUT_USER].width;
  return a->dim;
}

/* The norm/controller variant a kernel is compiled with: the controller
 * choice applies to adaptive FP64 kernels, every other kernel is the same
 * whichever is asked (and is built as the default, ODE_CTRL_DS), except that
 * ODE_CTRL_REF (FP64 only) sets the arithmetic of every kernel. */
int ctrl_variant(const ode_solve_args* a) {
  if (a->controller == ODE_CTRL_REF) return ODE_CTRL_REF;
  if (is_fixed(a->alg) || a->precision != ODE_FP64) return ODE_CTRL_DS;
  return a->controller;
}

/* kernel-key suffix of a controller variant */
const char* ctrl_suffix(int v) {
  return v == ODE_CTRL_FP64 ? "|c64" : v == ODE_CTRL_FP32 ? "|c32" : v == ODE_CTRL_REF ? "|ref" : "";
}

std::string kernel_key(ode_handle* h, const ode_solve_args* a, int sched) {
  char b[160];
  snprintf(b, sizeof b, "%s|%s|%d|%d|%s|%d%s%s", alg_name(a->alg), kernel_kind(h, a, sched), a->rhs, a->dim,
           prec_name(a->precision), a->output >= ODE_OUTPUT_USER ? a->output : 0, h->bounds_check ? "|chk" : "",
           ctrl_suffix(ctrl_variant(a)));
  return b;
}

/* Source of the one-kernel translation unit for (algorithm, rhs, precision,
 * dim, schedule kind). */
std::string jit_source(ode_handle* h, const ode_solve_args* a, int sched) {
  std::string src;
  if (ctrl_variant(a) == ODE_CTRL_FP64) src += "#define GBODE_CTRL64 1\n";
  if (ctrl_variant(a) == ODE_CTRL_DS) src += "#define GBODE_CTRL_DS 1\n";
  if (ctrl_variant(a) == ODE_CTRL_REF) src += "#define GBODE_REF 1\n";
  if (a->output >= ODE_OUTPUT_USER) {
    /* the output function goes before the solver header, whose store_point calls it */
    const UserOutput& u = h->outputs[a->output - ODE_OUTPUT_USER];
    char hdr[256];
    snprintf(hdr, sizeof hdr, "#define GBODE_USER_OUTPUT 1\n#define GBODE_OUTPUT_WIDTH %d\n#define GBODE_OUTPUT_NP %d\n",
             u.width, u.nparams);
    src += hdr;
    src += "__device__ __forceinline__ void gbode_user_output(double* out, const double* u, const double* p, "
           "double t) {\n";
    src += u.body;
    src += "\n}\n";
  }
  src += "#include \"ode_solver.cuh\"\n";
  if (a->rhs >= ODE_RHS_USER) {
    const UserRhs& u = h->users[a->rhs - ODE_RHS_USER];
    char hdr[256];
    snprintf(hdr, sizeof hdr,
             "template <class R> __device__ __forceinline__ void user_rhs(R* du, const R* u, const R* p, R t) {\n");
    src += hdr;
    src += u.body;
    src += "\n}\n";
    snprintf(hdr, sizeof hdr,
             "template <class R, class T> struct RhsUser {\n  enum { D = %d, NP = %d };\n  R p[%d];\n", u.dim,
             u.nparams, u.nparams > 0 ? u.nparams : 1);
    src += hdr;
    src += "  __device__ __forceinline__ void operator()(const R (&u)[D], T t, R (&du)[D]) const {\n"
           "    user_rhs<R>(du, u, p, (R)t);\n  }\n};\n";
  }
  src += "typedef " + rhs_type_expr(h, a) + " RHS_T;\n";
  src += std::string("GBODE_ENTRY(gbode_jit, ") + kernel_kind(h, a, sched) + ", " + method_type(a->alg) +
         ", " + prec_type(a->precision) + ", RHS_T)\n";
  return src;
}

/* NVRTC: source -> CUBIN for sm_103a.  Thread-safe (no handle state);
 * extra_opts carries the launch-shape variants of the autotuner. */
int nvrtc_cubin(const std::string& src, const std::vector<std::string>& extra_opts, std::vector<char>* cubin,
                std::string* log, std::string* err) {
  if (!load_nvrtc()) {
    *err = "libnvrtc.so.13 could not be loaded";
    return ODE_ENVRTC;
  }
  nvrtcProgram prog;
  const char* hdrs[] = {kSrc_ode_solver_cuh, kSrc_ode_kparams_h, kSrc_tableaus_h, kSrc_sde_solver_cuh, kSrc_log_table_h,
                        kSrc_exp_table_h, kSrc_ds_table_h, kSrc_bitops_h, kSrc_crpow_h, kSrc_crpow_table_h};
  const char* names[] = {"ode_solver.cuh", "ode_kparams.h", "tableaus.h", "sde_solver.cuh", "log_table.h",
                         "exp_table.h", "ds_table.h", "bitops.h", "crpow.h", "crpow_table.h"};
  nvrtcResult r = g_nvrtc.create(&prog, src.c_str(), "gbode_jit.cu", 10, hdrs, names);
  if (r != NVRTC_SUCCESS) {
    *err = std::string("nvrtcCreateProgram: ") + g_nvrtc.errstr(r);
    return ODE_ENVRTC;
  }
  std::vector<const char*> opts = {"--gpu-architecture=sm_103a", "--fmad=false", "-std=c++17", "-lineinfo",
                                   "-default-device"};
  for (const std::string& o : extra_opts) opts.push_back(o.c_str());
  r = g_nvrtc.compile(prog, (int)opts.size(), opts.data());
  size_t loglen = 0;
  g_nvrtc.logsize(prog, &loglen);
  std::string lg(loglen, '\0');
  if (loglen) g_nvrtc.log(prog, &lg[0]);
  if (log) *log = lg;
  if (r != NVRTC_SUCCESS) {
    g_nvrtc.destroy(&prog);
    *err = "run-time compilation failed:\n" + lg;
    return ODE_ENVRTC;
  }
  size_t n = 0;
  g_nvrtc.cubinsize(prog, &n);
  cubin->resize(n);
  g_nvrtc.cubin(prog, cubin->data());
  g_nvrtc.destroy(&prog);
  return ODE_OK;
}

int load_cubin(ode_handle* h, const std::vector<char>& cubin, int block, int stage, CUfunction* fn) {
  CUmodule mod;
  CUresult cr = g_drv.cuModuleLoadData(&mod, cubin.data());
  if (cr != CUDA_SUCCESS) return cu_fail(h, cr, "cuModuleLoadData");
  h->modules.push_back(mod);
  cr = g_drv.cuModuleGetFunction(fn, mod, "gbode_jit");
  if (cr != CUDA_SUCCESS) return cu_fail(h, cr, "cuModuleGetFunction");
  h->fblock[*fn] = block;
  h->fstage[*fn] = stage;
  return ODE_OK;
}

int compile_jit(ode_handle* h, const ode_solve_args* a, int sched, CUfunction* fn, std::string* log_out) {
  std::vector<char> cubin;
  std::string err;
  int block = 128, stage = 12288;
  default_shape(a, sched, &block, &stage);
  std::vector<std::string> opts = {"-DGBODE_BLOCK=" + std::to_string(block),
                                   "-DGBODE_STAGE_BYTES=" + std::to_string(stage)};
  if (h->bounds_check) opts.push_back("-DGBODE_BOUNDS_CHECK");
  const int rc = nvrtc_cubin(jit_source(h, a, sched), opts, &cubin, log_out, &err);
  if (rc != ODE_OK) return fail(h, rc, err);
  return load_cubin(h, cubin, block, stage, fn);
}

/* Find (or build) the kernel for this solve. */
int get_kernel(ode_handle* h, const ode_solve_args* a, int sched, CUfunction* fn, int* jit) {
  const std::string key = kernel_key(h, a, sched);
  auto tt = h->tuned.find(key);
  if (!h->bounds_check && tt != h->tuned.end()) {
    *fn = tt->second;
    *jit = 1;
    return ODE_OK;
  }
  auto ch = h->tune_choice.find(key);
  if (!h->bounds_check && ch != h->tune_choice.end() && ch->second.size() == 3 && ch->second[0] > 0) {
    /* a launch shape from ode_tune_load: compile that variant once */
    const std::vector<int>& c = ch->second;
    std::vector<std::string> o = {"-DGBODE_BLOCK=" + std::to_string(c[0]), "-DGBODE_STAGE_BYTES=" + std::to_string(c[2])};
    if (c[1]) o.push_back("--maxrregcount=" + std::to_string(c[1]));
    std::vector<char> cubin;
    std::string lg, err;
    int rc = nvrtc_cubin(jit_source(h, a, sched), o, &cubin, &lg, &err);
    if (rc != ODE_OK) return fail(h, rc, err);
    rc = load_cubin(h, cubin, c[0], c[2], fn);
    if (rc != ODE_OK) return rc;
    h->tuned[key] = *fn;
    *jit = 1;
    return ODE_OK;
  }
  auto it = h->kcache.find(key);
  if (it != h->kcache.end()) {
    *fn = it->second;
    *jit = h->kjit[key];
    return ODE_OK;
  }
  const char* kind = kernel_kind(h, a, sched);
  for (const AotEntry& e : kAotEntries) {
    if (!h->bounds_check && ctrl_variant(a) == ODE_CTRL_DS && a->output < ODE_OUTPUT_USER && e.alg == a->alg &&
        e.rhs == a->rhs &&
        e.dim == a->dim &&
        e.precision == a->precision && std::strcmp(e.kind, kind) == 0) {
      cudaFunction_t f;
      cudaError_t ce = cudaGetFuncBySymbol(&f, e.fn);
      if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaGetFuncBySymbol");
      *fn = (CUfunction)f;
      h->kcache[key] = *fn;
      h->kjit[key] = 0;
      h->fblock[*fn] = e.block;
      h->fstage[*fn] = e.stage;
      *jit = 0;
      return ODE_OK;
    }
  }
  int rc = compile_jit(h, a, sched, fn, nullptr);
  if (rc != ODE_OK) return rc;
  h->kcache[key] = *fn;
  h->kjit[key] = 1;
  *jit = 1;
  return ODE_OK;
}

int stage_of(ode_handle* h, CUfunction fn) {
  auto it = h->fstage.find(fn);
  return it == h->fstage.end() ? 12288 : it->second;
}

int block_of(ode_handle* h, CUfunction fn) {
  auto it = h->fblock.find(fn);
  return it == h->fblock.end() ? 128 : it->second;
}

/* Threads per block of a one-thread-per-trajectory launch: of the compiled
 * block size and its halves down to one warp, the one that puts the fewest
 * warps on the busiest SM (ties go to the larger block).  A small ensemble
 * then spreads over every SM: 8,192 trajectories in blocks of 128 would fill
 * 64 of 152 SMs with 4 warps each, in blocks of 64 they give 128 SMs 2 warps. */
int plain_block(int64_t n, int nsm, int maxb) {
  int best = maxb;
  int64_t best_w = INT64_MAX;
  for (int b = maxb; b >= 32; b /= 2) {
    const int64_t blocks = (n + b - 1) / b;
    const int64_t w = (blocks + nsm - 1) / nsm * (b / 32);
    if (w < best_w) {
      best_w = w;
      best = b;
    }
  }
  return best;
}

int launch(ode_handle* h, CUfunction fn, unsigned grid, int block, KParams* kp, cudaStream_t s) {
  void* params[] = {kp};
  CUresult r = g_drv.cuLaunchKernel(fn, grid, 1, 1, (unsigned)block, 1, 1, 0, (CUstream)s, params, nullptr);
  if (r != CUDA_SUCCESS) return cu_fail(h, r, "cuLaunchKernel");
  return ODE_OK;
}

template <class T>
int grid_for(double t0, double dt, double tf, std::vector<double>* out, int64_t* len) {
  int64_t n = jlrange::build<T>((T)t0, (T)dt, (T)tf, out);
  if (n < 0) return ODE_EINVAL;
  *len = n;
  return ODE_OK;
}

}  // namespace

namespace gbode {

int jit_function(ode_handle* h, const std::string& src, int block, CUfunction* fn, std::string* log) {
  std::vector<char> cubin;
  std::string err;
  const int rc = nvrtc_cubin(src, {}, &cubin, log, &err);
  if (rc != ODE_OK) return fail(h, rc, err);
  return load_cubin(h, cubin, block, 0, fn);
}

int launch_params(ode_handle* h, CUfunction fn, unsigned grid, unsigned block, void* params, cudaStream_t s) {
  void* args[] = {params};
  const CUresult r = g_drv.cuLaunchKernel(fn, grid, 1, 1, block, 1, 1, 0, (CUstream)s, args, nullptr);
  if (r != CUDA_SUCCESS) return cu_fail(h, r, "cuLaunchKernel");
  return ODE_OK;
}

}  // namespace gbode

extern "C" {

int ode_abi_version(void) { return ODE_ABI_VERSION; }

int ode_set_bounds_check(ode_handle* h, int enable) {
  if (!h) return ODE_EINVAL;
  h->bounds_check = enable != 0;
  return ODE_OK;
}

/* GPU tag of a tuning file: name and SM count */
static std::string gpu_tag(ode_handle* h) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) {
    cudaGetLastError();
    return "unknown";
  }
  std::string name = prop.name;
  for (char& c : name)
    if (c == ' ' || c == '\t') c = '_';
  return name + "/" + std::to_string(prop.multiProcessorCount);
}

/* kernel keys are alg|kind|rhs|dim|prec|output[|chk][|c64, |c32 or |ref]; only built-in ids travel,
 * and no bounds-check build */
static bool portable_key(const std::string& key) {
  std::vector<std::string> f;
  size_t a = 0;
  for (size_t b; (b = key.find('|', a)) != std::string::npos; a = b + 1) f.push_back(key.substr(a, b - a));
  f.push_back(key.substr(a));
  const bool has_ctrl = f.size() == 7 && (f[6] == "c64" || f[6] == "c32" || f[6] == "ref");
  return (f.size() == 6 || has_ctrl) && std::atoi(f[2].c_str()) < ODE_RHS_USER &&
         std::atoi(f[5].c_str()) < ODE_OUTPUT_USER;
}

int ode_tune_save(ode_handle* h, const char* path) {
  if (!h) return ODE_EINVAL;
  if (!path) return fail(h, ODE_EINVAL, "null path");
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(h, ODE_EINVAL, std::string("cannot write ") + path);
  std::fprintf(f, "gb300ode-tune 1 %s\n", gpu_tag(h).c_str());
  for (const auto& kv : h->tune_choice)
    if (portable_key(kv.first) && kv.second.size() == 3)
      std::fprintf(f, "%s %d %d %d\n", kv.first.c_str(), kv.second[0], kv.second[1], kv.second[2]);
  const bool ok = std::fclose(f) == 0;
  return ok ? ODE_OK : fail(h, ODE_EINVAL, std::string("cannot write ") + path);
}

int ode_tune_load(ode_handle* h, const char* path) {
  if (!h) return ODE_EINVAL;
  if (!path) return fail(h, ODE_EINVAL, "null path");
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(h, ODE_EINVAL, std::string("cannot read ") + path);
  char magic[32] = {0}, tag[256] = {0};
  int version = 0;
  if (std::fscanf(f, "%31s %d %255s", magic, &version, tag) != 3 || std::strcmp(magic, "gb300ode-tune") != 0 ||
      version != 1) {
    std::fclose(f);
    return fail(h, ODE_EINVAL, "not a tuning file");
  }
  if (gpu_tag(h) != tag) {
    std::fclose(f);
    return fail(h, ODE_ENOTSUP, std::string("tuning file written on another GPU (") + tag + ")");
  }
  std::map<std::string, std::vector<int>> read;
  char key[160];
  int b = 0, r = 0, st = 0;
  int rc = ODE_OK;
  while (true) {
    const int got = std::fscanf(f, "%159s %d %d %d", key, &b, &r, &st);
    if (got == EOF) break;
    if (got != 4 || b < 0 || b > 1024 || b % 32 || r < 0 || r > 255 || st < 0 || st > 49152 ||
        !portable_key(key)) {
      rc = fail(h, ODE_EINVAL, "malformed tuning entry");
      break;
    }
    read[key] = {b, r, st};
  }
  std::fclose(f);
  if (rc != ODE_OK) return rc;
  for (auto& kv : read) {
    h->tune_choice[kv.first] = kv.second;
    h->tuned.erase(kv.first);
  }
  return ODE_OK;
}

int ode_create(ode_handle** out, int device) {
  if (!out) return ODE_EINVAL;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess) return ODE_ECUDA;
  if (device < 0 || device >= ndev) return ODE_EINVAL;
  ode_handle* h = new ode_handle();
  h->device = device;
  e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaFree(0);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->chunk_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
  if (e != cudaSuccess) {
    ode_destroy(h);
    return ODE_ECUDA;
  }
  if (!load_driver_api()) {
    ode_destroy(h);
    return ODE_ECUDA;
  }
  *out = h;
  return ODE_OK;
}

void ode_destroy(ode_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->chunk_stream) cudaStreamSynchronize(h->chunk_stream);
  for (GraphEntry& g : h->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.graph) cudaGraphDestroy(g.graph);
  }
  for (auto& kv : h->bufs)
    if (kv.second.ptr) cudaFree(kv.second.ptr);
  for (CUmodule m : h->modules) g_drv.cuModuleUnload(m);
  if (h->model) model_free(h->model);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
  if (h->chunk_stream) cudaStreamDestroy(h->chunk_stream);
  if (h->chunk_stats) cudaFreeHost(h->chunk_stats);
  delete h;
}

const char* ode_last_error(const ode_handle* h) { return h ? h->err.c_str() : "null handle"; }

int ode_fixed_grid(double t0, double dt, double tf, int precision, double* out, int64_t cap, int64_t* len) {
  if (!len || !(dt == dt) || dt == 0.0) return ODE_EINVAL;
  std::vector<double> v;
  int rc = (precision == ODE_FP32) ? grid_for<float>(t0, dt, tf, &v, len) : grid_for<double>(t0, dt, tf, &v, len);
  if (rc != ODE_OK) return rc;
  if (out)
    for (int64_t i = 0; i < std::min<int64_t>(cap, *len); ++i) out[i] = v[(size_t)i];
  return ODE_OK;
}

int ode_rhs_compile(ode_handle* h, const char* body, int dim, int nparams, int* rhs_id, char* log, size_t loglen) {
  if (!h || !body || !rhs_id || dim < 1 || dim > 32 || nparams < 0 || nparams > 256)
    return fail(h, ODE_EINVAL, "ode_rhs_compile: bad arguments");
  cudaSetDevice(h->device);
  UserRhs u;
  u.body = body;
  u.dim = dim;
  u.nparams = nparams;
  h->users.push_back(u);
  const int id = ODE_RHS_USER + (int)h->users.size() - 1;
  /* compile one probe kernel now so that syntax errors surface here */
  ode_solve_args a;
  std::memset(&a, 0, sizeof a);
  a.alg = ODE_ALG_ATSIT5;
  a.rhs = id;
  a.precision = ODE_FP64;
  a.dim = dim;
  a.nparams = nparams;
  CUfunction fn;
  std::string lg;
  int rc = compile_jit(h, &a, ODE_SCHED_PLAIN, &fn, &lg);
  if (log && loglen) {
    std::strncpy(log, lg.c_str(), loglen - 1);
    log[loglen - 1] = '\0';
  }
  if (rc != ODE_OK) {
    h->users.pop_back();
    return rc;
  }
  h->kcache[kernel_key(h, &a, ODE_SCHED_PLAIN)] = fn;
  h->kjit[kernel_key(h, &a, ODE_SCHED_PLAIN)] = 1;
  *rhs_id = id;
  return ODE_OK;
}

int ode_output_compile(ode_handle* h, const char* body, int dim, int nparams, int width, int* output_id, char* log,
                       size_t loglen) {
  if (!h) return ODE_EINVAL;
  if (!body || !output_id || dim < 1 || dim > 32 || nparams < 0 || nparams > 256 || width < 1 || width > 64)
    return fail(h, ODE_EINVAL, "ode_output_compile: bad arguments");
  /* compile the function alone now so that syntax errors surface here; the
   * solver kernels that use it are compiled on first use */
  char hdr[160];
  snprintf(hdr, sizeof hdr, "#define GBODE_OUTPUT_WIDTH %d\n#define GBODE_OUTPUT_NP %d\n", width, nparams);
  std::string src = hdr;
  src += "__device__ __forceinline__ void gbode_user_output(double* out, const double* u, const double* p, double t) {\n";
  src += body;
  src += "\n}\nextern \"C\" __global__ void gbode_output_probe(double* out, const double* u, const double* p, "
         "double t) {\n  gbode_user_output(out, u, p, t);\n}\n";
  std::vector<char> cubin;
  std::string lg, err;
  const int rc = nvrtc_cubin(src, {}, &cubin, &lg, &err);
  if (log && loglen) {
    std::strncpy(log, lg.c_str(), loglen - 1);
    log[loglen - 1] = '\0';
  }
  if (rc != ODE_OK) return fail(h, rc, err.empty() ? "output function did not compile (see log)" : err);
  UserOutput u;
  u.body = body;
  u.dim = dim;
  u.nparams = nparams;
  u.width = width;
  h->outputs.push_back(u);
  *output_id = ODE_OUTPUT_USER + (int)h->outputs.size() - 1;
  return ODE_OK;
}

}  // extern "C"

namespace {

/* Device pointers of the every-step output (ode_ensemble_solve_everystep). */
struct EveryStep {
  const long long* off;
  double* t;
  double* u;
};

/* One chunk of the host-buffer pipeline, enqueued without waiting: its
 * scratch buffers carry the slot's tag (two chunks run at once), its timing
 * events and a pinned array for its statistics words come from the caller,
 * which reads them after synchronizing. */
struct ChunkSlot {
  const char* tag;
  cudaEvent_t ev0, ev1;
  unsigned long long* host_stats; /* 4 words: attempts, saves, early stops, work counter */
  int launches, replayed, jit, sched, kernel;
};

int solve_impl(ode_handle* h, const ode_solve_args* a, ode_solve_out* o, ode_solve_stats* st, const EveryStep* ev,
               ChunkSlot* slot = nullptr) {
  NvtxRange nvtx("gbode solve");
  const auto wall0 = std::chrono::steady_clock::now();
  if (!h) return ODE_EINVAL;
  if (!a || !o) return fail(h, ODE_EINVAL, "null argument");
  h->err.clear();
  if (a->alg < ODE_ALG_RK4 || a->alg > ODE_ALG_EULER) return fail(h, ODE_EINVAL, "unknown algorithm");
  if (a->precision < ODE_FP64 || a->precision > ODE_FP32_KAHAN) return fail(h, ODE_EINVAL, "unknown precision");
  if (a->schedule < ODE_SCHED_PLAIN || a->schedule > ODE_SCHED_LEARNED) return fail(h, ODE_EINVAL, "unknown schedule");
  if (a->memory != ODE_MEM_HOST && a->memory != ODE_MEM_DEVICE) return fail(h, ODE_EINVAL, "unknown memory kind");
  if (a->layout != ODE_LAYOUT_SOA && a->layout != ODE_LAYOUT_TRAJ) return fail(h, ODE_EINVAL, "unknown output layout");
  if (a->controller != ODE_CTRL_DS && a->controller != ODE_CTRL_FP64 && a->controller != ODE_CTRL_FP32 &&
      a->controller != ODE_CTRL_REF)
    return fail(h, ODE_EINVAL, "unknown step-size controller");
  if ((a->controller == ODE_CTRL_FP64 || a->controller == ODE_CTRL_REF) && a->precision != ODE_FP64)
    return fail(h, ODE_ENOTSUP, "the FP64 and reference-arithmetic controllers apply to FP64 solves");
  if (a->n < 0 || a->n > 0x7fffffffLL) return fail(h, ODE_EINVAL, "n must be in [0, 2^31)");
  if (a->n > 0 && (!a->u0 || (a->nparams > 0 && !a->p))) return fail(h, ODE_EINVAL, "u0/p missing");
  if (!(a->t0 == a->t0) || !(a->tf == a->tf) || !(a->dt == a->dt))
    return fail(h, ODE_EINVAL, "t0, tf and dt must not be NaN");
  if (a->nsave < 0 || (a->nsave > 0 && !a->saveat)) return fail(h, ODE_EINVAL, "saveat missing");
  if (a->output >= ODE_OUTPUT_USER) {
    if (a->output >= ODE_OUTPUT_USER + (int)h->outputs.size()) return fail(h, ODE_EINVAL, "unknown output function");
    const UserOutput& u = h->outputs[a->output - ODE_OUTPUT_USER];
    if (u.dim != a->dim || u.nparams != a->nparams)
      return fail(h, ODE_EINVAL, "the output function was compiled for another dim / nparams");
  } else if (a->output != ODE_OUTPUT_STATE && a->output != ODE_OUTPUT_KURAMOTO_R) {
    return fail(h, ODE_EINVAL, "unknown output kind");
  }
  if (a->output == ODE_OUTPUT_KURAMOTO_R && (a->save_everystep || is_onestep(a->alg)))
    return fail(h, ODE_EINVAL, "the order-parameter output applies to saveat points");
  if (is_onestep(a->alg) && a->nsave > 0)
    return fail(h, ODE_EINVAL, "GPUSimpleRK4 and GPUSimpleEuler have no saveat (they save every step; use save_everystep)");
  int rc = check_rhs(h, a);
  if (rc != ODE_OK) return rc;
  const bool fixed = is_fixed(a->alg);
  if (fixed && a->dt == 0.0) return fail(h, ODE_EINVAL, "dt is required for fixed-step algorithms");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t s = a->stream ? (cudaStream_t)a->stream : h->stream;
  const int64_t n = a->n;
  const int D = a->dim, NP = a->nparams;
  /* scratch buffer names, per chunk slot when two chunks are in flight */
  auto nm = [&](const char* base) { return slot ? std::string(base) + slot->tag : std::string(base); };
  cudaEvent_t ev0 = slot ? slot->ev0 : h->ev0, ev1 = slot ? slot->ev1 : h->ev1;

  int sched = fixed ? ODE_SCHED_PLAIN : a->schedule;
  if (sched == ODE_SCHED_LEARNED && !model_ready(h->model, a)) {
    return fail(h, ODE_ENOMODEL, "learned schedule requested but no model fitted for this problem shape");
  }

  /* time grid of the fixed-step solvers */
  std::vector<double> grid;
  int64_t ngrid = 0;
  if (fixed) {
    rc = (a->precision == ODE_FP32) ? grid_for<float>(a->t0, a->dt, a->tf, &grid, &ngrid)
                                    : grid_for<double>(a->t0, a->dt, a->tf, &grid, &ngrid);
    if (rc != ODE_OK) return fail(h, rc, "invalid fixed-step grid");
  }
  int64_t npoints = a->nsave;
  if (fixed && a->nsave == 0 && a->save_everystep) npoints = ngrid;

  CUfunction fn;
  int jit = 0;
  rc = get_kernel(h, a, sched, &fn, &jit);
  if (rc != ODE_OK) return rc;

  KParams kp;
  std::memset(&kp, 0, sizeof kp);
  kp.n = n;
  kp.t0 = a->t0;
  kp.tf = a->tf;
  kp.dt = a->dt;
  kp.abstol = a->abstol;
  kp.reltol = a->reltol;
  kp.nsave = a->nsave;
  kp.ngrid = ngrid;
  kp.save_everystep = a->save_everystep ? 1 : 0;
  kp.dim = D;
  kp.nparams = NP;
  kp.maxiters = a->maxiters > 0 ? a->maxiters : kDefaultMaxIters;
  kp.norm_fp64 = a->abstol < 1e-30 ? 1 : 0;
  ds_split_host(a->abstol, kp.tol_ds);
  ds_split_host(a->reltol, kp.tol_ds + 2);
  kp.output = a->output;
  {
    const long long W = output_width(h, a);
    if (a->layout == ODE_LAYOUT_TRAJ) {
      kp.us_sj = W;
      kp.us_sw = 1;
      kp.us_si = (long long)npoints * W;
    } else {
      kp.us_sj = W * (long long)n;
      kp.us_sw = n;
      kp.us_si = 1;
    }
  }

  const bool host = a->memory == ODE_MEM_HOST;
  const size_t nd = (size_t)n * sizeof(double);
  /* inputs */
  if (host) {
    double* du0 = (double*)buf(h, "u0", nd * D, &rc);
    if (!du0) return rc;
    double* dp = (double*)buf(h, "p", nd * (NP > 0 ? NP : 1), &rc);
    if (!dp) return rc;
    if (n > 0) {
      CK(cudaMemcpyAsync(du0, a->u0, nd * D, cudaMemcpyHostToDevice, s), "copy u0");
      if (NP > 0) CK(cudaMemcpyAsync(dp, a->p, nd * NP, cudaMemcpyHostToDevice, s), "copy p");
    }
    kp.u0 = du0;
    kp.p = dp;
    if (a->dt0) {
      double* dd = (double*)buf(h, "dt0", nd, &rc);
      if (!dd) return rc;
      CK(cudaMemcpyAsync(dd, a->dt0, nd, cudaMemcpyHostToDevice, s), "copy dt0");
      kp.dt0 = dd;
    }
  } else {
    kp.u0 = a->u0;
    kp.p = a->p;
    kp.dt0 = a->dt0;
  }
  if (a->nsave > 0) {
    double* ds = (double*)buf(h, nm("saveat"), (size_t)a->nsave * sizeof(double), &rc);
    if (!ds) return rc;
    CK(cudaMemcpyAsync(ds, a->saveat, (size_t)a->nsave * sizeof(double), cudaMemcpyHostToDevice, s), "copy saveat");
    kp.saveat = ds;
  }
  if (fixed && ngrid > 0) {
    double* dg = (double*)buf(h, nm("grid"), (size_t)ngrid * sizeof(double), &rc);
    if (!dg) return rc;
    CK(cudaMemcpyAsync(dg, grid.data(), (size_t)ngrid * sizeof(double), cudaMemcpyHostToDevice, s), "copy grid");
    kp.grid = dg;
  }
  /* outputs */
  struct OutMap { void* host; const char* name; size_t bytes; void** dev; };
  OutMap outs[] = {
      {o->us, "us", (size_t)npoints * output_width(h, a) * nd, (void**)&kp.us},
      {o->u_final, "u_final", nd * D, (void**)&kp.u_final},
      {o->t_final, "t_final", nd, (void**)&kp.t_final},
      {o->retcode, "retcode", (size_t)n, (void**)&kp.retcode},
      {o->naccept, "naccept", (size_t)n * 4, (void**)&kp.naccept},
      {o->nreject, "nreject", (size_t)n * 4, (void**)&kp.nreject},
      {o->dt_first, "dt_first", nd, (void**)&kp.dt_first},
  };
  for (OutMap& m : outs) {
    if (!m.host || m.bytes == 0) continue;
    if (host) {
      void* d = buf(h, m.name, m.bytes, &rc);
      if (!d) return rc;
      *m.dev = d;
    } else {
      *m.dev = m.host;
    }
  }
  if (ev) {
    kp.ev_off = ev->off;
    kp.ev_t = ev->t;
    kp.ev_u = ev->u;
  }
  unsigned long long* stats = (unsigned long long*)buf(h, nm("stats"), 4 * sizeof(unsigned long long), &rc);
  if (!stats) return rc;
  kp.stats = stats;
  kp.counter = stats + 3;
  unsigned* chk = nullptr;
  if (h->bounds_check) {
    /* [0] violation bits, [16..16+n) per-trajectory start counts */
    if (!(chk = (unsigned*)buf(h, "check", ((size_t)n + 16) * sizeof(unsigned), &rc))) return rc;
    kp.check_flags = chk;
    kp.visited = chk + 16;
  }

  /* schedule */
  int launches = 0;
  unsigned gridx;
  int block = block_of(h, fn);
  if (use_fixed_split(h, a)) {
    block = 32 * D;  /* D warps per 32 trajectories */
    gridx = (unsigned)((n + 31) / 32);
  } else if (sched == ODE_SCHED_PLAIN) {
    block = plain_block(n, h->nsm, block);
    gridx = (unsigned)((n + block - 1) / block);
  } else {
    int nb = 0;
    CUresult cr = g_drv.cuOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, 0);
    if (cr != CUDA_SUCCESS) return cu_fail(h, cr, "occupancy");
    if (nb < 1) nb = 1;
    const int64_t resident = (int64_t)nb * h->nsm;
    gridx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(resident, (n + block - 1) / block));
  }

  /* device buffers of the learned schedule, allocated before any capture */
  float *latt = nullptr, *ldt = nullptr;
  int* order = nullptr;
  unsigned* bins = nullptr;
  double* dseed = nullptr;
  const bool seeding = sched == ODE_SCHED_LEARNED && !a->dt0 && model_seed_dt0(h->model);
  if (sched == ODE_SCHED_LEARNED) {
    if (!(latt = (float*)buf(h, nm("pred_att"), (size_t)n * 4, &rc))) return rc;
    if (!(ldt = (float*)buf(h, nm("pred_dt"), (size_t)n * 4, &rc))) return rc;
    if (!(order = (int*)buf(h, nm("order"), (size_t)n * 4 + 16, &rc))) return rc;
    if (!(bins = (unsigned*)buf(h, nm("bins"), kCostBins * sizeof(unsigned), &rc))) return rc;
    if (seeding && !(dseed = (double*)buf(h, nm("dt0_seed"), nd, &rc))) return rc;
    kp.order = order;
    if (seeding) kp.dt0 = dseed;
  }

  /* The device-side sequence of a solve (statistics reset, cost prediction,
   * binning, dt0 seeding, the solver kernel) is captured once into a CUDA
   * graph and replayed while the launch parameters stay the same. */
  auto enqueue = [&](int* nl) -> int {
    CK(cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), s), "memset stats");
    if (chk) CK(cudaMemsetAsync(chk, 0, ((size_t)n + 16) * sizeof(unsigned), s), "memset check");
    if (sched == ODE_SCHED_LEARNED && n > 0) {
      int r = model_predict_device(h, a, kp, latt, ldt, s, nl);
      if (r == ODE_OK) r = order_by_cost(h, latt, n, order, bins, s, nl);
      if (r == ODE_OK && seeding) r = seed_dt0(h, ldt, n, model_dt0_safety(h->model), dseed, s, nl);
      if (r != ODE_OK) return r;
    }
    if (n > 0) {
      const int r = launch(h, fn, gridx, block, &kp, s);
      if (r != ODE_OK) return r;
      ++*nl;
    }
    return ODE_OK;
  };
  std::string key((const char*)&kp, sizeof kp);
  {
    char extra[256];
    snprintf(extra, sizeof extra, "|%p|%u|%d|%d|%d|", (void*)fn, gridx, block, sched, (int)seeding);
    key += extra;
    if (sched == ODE_SCHED_LEARNED) key += model_key(h->model);
  }
  const bool use_graph = s != 0;  /* the legacy default stream cannot be captured */
  int replayed = 0;
  CK(cudaEventRecord(ev0, s), "event");
  GraphEntry* cached = nullptr;
  for (GraphEntry& g : h->graphs)
    if (g.exec && g.key == key) cached = &g;
  if (use_graph && cached) {
    cached->last_use = ++h->graph_tick;
    CK(cudaGraphLaunch(cached->exec, s), "cudaGraphLaunch");
    launches = cached->launches;
    replayed = 1;
  } else if (use_graph) {
    if ((int)h->graphs.size() >= kGraphCache) {
      /* evict the least recently used captured solve */
      size_t lru = 0;
      for (size_t i = 1; i < h->graphs.size(); ++i)
        if (h->graphs[i].last_use < h->graphs[lru].last_use) lru = i;
      if (h->graphs[lru].exec) cudaGraphExecDestroy(h->graphs[lru].exec);
      if (h->graphs[lru].graph) cudaGraphDestroy(h->graphs[lru].graph);
      h->graphs.erase(h->graphs.begin() + (long)lru);
    }
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    int nl = 0;
    const int r = enqueue(&nl);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (r != ODE_OK) {
      if (g) cudaGraphDestroy(g);
      return r;
    }
    if (ce != cudaSuccess) return cuda_fail(h, ce, "cudaStreamEndCapture");
    cudaGraphExec_t ex = nullptr;
    cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
    if (ie != cudaSuccess) {
      cudaGraphDestroy(g);
      return cuda_fail(h, ie, "cudaGraphInstantiate");
    }
    GraphEntry ge;
    ge.graph = g;
    ge.exec = ex;
    ge.key = key;
    ge.launches = nl;
    ge.last_use = ++h->graph_tick;
    h->graphs.push_back(ge);
    CK(cudaGraphLaunch(ex, s), "cudaGraphLaunch");
    launches = nl;
  } else {
    rc = enqueue(&launches);
    if (rc != ODE_OK) return rc;
  }
  if (slot) {
    /* chunk of the host pipeline: statistics to pinned memory before the end
     * event, which the caller's copies and final synchronization wait on */
    CK(cudaMemcpyAsync(slot->host_stats, stats, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s),
       "copy stats");
    CK(cudaEventRecord(ev1, s), "event");
    slot->launches = launches;
    slot->replayed = replayed;
    slot->jit = jit;
    slot->sched = sched;
    slot->kernel = kernel_kind_id(kernel_kind(h, a, sched));
    return ODE_OK;
  }
  CK(cudaEventRecord(ev1, s), "event");

  /* asynchronous call: device buffers, the caller's stream, no statistics asked */
  if (!host && a->stream && !st && !chk) return ODE_OK;
  /* outputs back to the host */
  if (host) {
    for (OutMap& m : outs)
      if (m.host && m.bytes) CK(cudaMemcpyAsync(m.host, *m.dev, m.bytes, cudaMemcpyDeviceToHost, s), "copy out");
  }
  unsigned long long hs[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(hs, stats, sizeof hs, cudaMemcpyDeviceToHost, s), "copy stats");
  std::vector<unsigned> hchk;
  if (chk) {
    hchk.resize((size_t)n + 16);
    CK(cudaMemcpyAsync(hchk.data(), chk, hchk.size() * sizeof(unsigned), cudaMemcpyDeviceToHost, s), "copy check");
  }
  CK(cudaStreamSynchronize(s), "solve");
  if (chk) {
    int64_t bad = -1;
    for (int64_t i = 0; i < n && bad < 0; ++i)
      if (hchk[16 + (size_t)i] != 1) bad = i;
    if (hchk[0] || bad >= 0) {
      char m[256];
      snprintf(m, sizeof m, "bounds check: violation bits 0x%x (1 trajectory, 2 save point, 4 every-step row, "
               "8 staging ring, 16 order); trajectory %lld started %u times",
               hchk[0], (long long)bad, bad >= 0 ? hchk[16 + (size_t)bad] : 1u);
      return fail(h, ODE_ECHECK, m);
    }
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  if (st) {
    st->kernel_ms = ms;
    st->attempts = (int64_t)hs[0];
    st->saves = (int64_t)hs[1];
    st->launches = launches;
    st->schedule_used = sched;
    st->graph_replayed = replayed;
    st->jit = jit;
    st->kernel = kernel_kind_id(kernel_kind(h, a, sched));
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  }
  if (hs[2] > 0) {
    char m[128];
    snprintf(m, sizeof m, "%llu trajectories stopped early (dt<dtmin or maxiters); see retcode", hs[2]);
    return fail(h, ODE_ETRAJ, m);
  }
  return ODE_OK;
}

/* Host buffers, large adaptive ensembles: the solve runs in chunks of
 * trajectories so that copying one chunk's outputs to the host (copy stream)
 * overlaps the next chunk's kernel (compute stream).  Chunks are contiguous
 * trajectory ranges, each a complete solve of its own (learned order, graph
 * capture) on double-buffered device slots; rows of the [rows][n] host arrays
 * move with 2D copies.  Results are those of the unchunked solve: every
 * trajectory is solved by the same kernel from the same inputs. */
constexpr int64_t kChunk = 262144;
constexpr int64_t kMaxChunks = 4;

int solve_chunked(ode_handle* h, const ode_solve_args* a, ode_solve_out* o, ode_solve_stats* st) {
  NvtxRange nvtx("gbode chunked solve");
  const auto wall0 = std::chrono::steady_clock::now();
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const int64_t n = a->n;
  const int D = a->dim, NP = a->nparams;
  /* at most kMaxChunks chunks (each chunk boundary costs a partly filled GPU
   * while the chunk's last trajectories finish: 16 chunks of the 4,194,304-trajectory Kuramoto-12 ensemble cost
   * 7.5%, 4 chunks 1.4%); the last chunk half the size of the others, so that
   * the output copy nothing overlaps is short */
  const int64_t nchunks = std::min<int64_t>(kMaxChunks, (n + kChunk - 1) / kChunk);
  const int64_t m = (2 * n + 2 * nchunks - 2) / (2 * nchunks - 1);
  cudaStream_t s = a->stream ? (cudaStream_t)a->stream : h->stream;
  cudaStream_t cs = h->copy_stream;
  int rc = ODE_OK;
  if (a->output >= ODE_OUTPUT_USER && a->output >= ODE_OUTPUT_USER + (int)h->outputs.size())
    return fail(h, ODE_EINVAL, "unknown output function");
  const int W = output_width(h, a);
  struct Rows {
    const void* host_in;
    void* host_out;
    int64_t rows;
    size_t elem;
    const char* name;
  };
  const Rows ins[] = {{a->u0, nullptr, D, 8, "ck_u0"}, {a->p, nullptr, NP, 8, "ck_p"}, {a->dt0, nullptr, 1, 8, "ck_dt0"}};
  /* a chunk of the [n][nsave][W] layout is one contiguous block: one row of nsave*W doubles per trajectory */
  const bool traj = a->layout == ODE_LAYOUT_TRAJ;
  const Rows outs[] = {{nullptr, o->us, traj ? 1 : a->nsave * W, traj ? (size_t)(8 * a->nsave * W) : 8, "ck_us"},
                       {nullptr, o->u_final, D, 8, "ck_uf"},
                       {nullptr, o->t_final, 1, 8, "ck_tf"},       {nullptr, o->retcode, 1, 1, "ck_ret"},
                       {nullptr, o->naccept, 1, 4, "ck_nacc"},     {nullptr, o->nreject, 1, 4, "ck_nrej"},
                       {nullptr, o->dt_first, 1, 8, "ck_dtf"}};
  void* din[2][3] = {};
  void* dout[2][7] = {};
  for (int b = 0; b < 2; ++b) {
    for (int k = 0; k < 3; ++k) {
      if (!ins[k].host_in || ins[k].rows == 0) continue;
      if (!(din[b][k] = buf(h, std::string(ins[k].name) + (b ? "1" : "0"), (size_t)(m * ins[k].rows) * ins[k].elem,
                            &rc)))
        return rc;
    }
    for (int k = 0; k < 7; ++k) {
      if (!outs[k].host_out || outs[k].rows == 0) continue;
      if (!(dout[b][k] = buf(h, std::string(outs[k].name) + (b ? "1" : "0"),
                             (size_t)(m * outs[k].rows) * outs[k].elem, &rc)))
        return rc;
    }
  }
  if (h->chunk_stats_cap < nchunks) {
    if (h->chunk_stats) cudaFreeHost(h->chunk_stats);
    h->chunk_stats = nullptr;
    h->chunk_stats_cap = 0;
    CK(cudaMallocHost((void**)&h->chunk_stats, (size_t)nchunks * 4 * sizeof(unsigned long long)), "pinned stats");
    h->chunk_stats_cap = nchunks;
  }
  /* events: inputs of a slot uploaded; start and end of every chunk's solve */
  std::vector<cudaEvent_t> evs;
  auto release = [&]() {
    for (cudaEvent_t e : evs)
      if (e) cudaEventDestroy(e);
  };
  auto make_event = [&](unsigned flags, cudaEvent_t* e) -> int {
    const cudaError_t r = cudaEventCreateWithFlags(e, flags);
    if (r != cudaSuccess) return cuda_fail(h, r, "event");
    evs.push_back(*e);
    return ODE_OK;
  };
  cudaEvent_t ready[2];
  std::vector<cudaEvent_t> ev_start((size_t)nchunks), ev_end((size_t)nchunks);
  for (int b = 0; b < 2 && rc == ODE_OK; ++b) rc = make_event(cudaEventDisableTiming, &ready[b]);
  for (int64_t c = 0; c < nchunks && rc == ODE_OK; ++c) {
    rc = make_event(cudaEventDefault, &ev_start[(size_t)c]);
    if (rc == ODE_OK) rc = make_event(cudaEventDefault, &ev_end[(size_t)c]);
  }
  if (rc != ODE_OK) {
    release();
    return rc;
  }
  /* chunk c's inputs to slot c % 2 (copy stream), then the slot's ready event */
  auto upload = [&](int64_t c) -> int {
    const int b = (int)(c & 1);
    const int64_t i0 = c * m, mc = std::min(m, n - i0);
    for (int k = 0; k < 3; ++k) {
      if (!din[b][k]) continue;
      const size_t e = ins[k].elem;
      CK(cudaMemcpy2DAsync(din[b][k], mc * e, (const char*)ins[k].host_in + i0 * e, n * e, mc * e, ins[k].rows,
                           cudaMemcpyHostToDevice, cs),
         "copy chunk inputs");
    }
    CK(cudaEventRecord(ready[b], cs), "event");
    return ODE_OK;
  };
  /* chunk c's outputs from slot c % 2 to the host, after its solve (copy stream) */
  auto download = [&](int64_t c) -> int {
    const int b = (int)(c & 1);
    const int64_t i0 = c * m, mc = std::min(m, n - i0);
    CK(cudaStreamWaitEvent(cs, ev_end[(size_t)c], 0), "wait chunk solve");
    for (int k = 0; k < 7; ++k) {
      if (!dout[b][k]) continue;
      const size_t el = outs[k].elem;
      CK(cudaMemcpy2DAsync((char*)outs[k].host_out + i0 * el, n * el, dout[b][k], mc * el, mc * el, outs[k].rows,
                           cudaMemcpyDeviceToHost, cs),
         "copy chunk outputs");
    }
    return ODE_OK;
  };
  /* Even chunks solve on the caller's stream, odd ones on the handle's second
   * compute stream, so that a chunk's kernel starts on the SMs that the
   * previous chunk's finished warps leave, during that chunk's tail.  On the
   * copy stream: wait for chunk c-1's solve, copy its outputs out, then copy
   * chunk c+1's inputs into the slot chunk c-1 used; chunk c+1's solve waits
   * for those copies (its slot is free then) and overlaps chunk c. */
  ode_solve_stats total;
  std::memset(&total, 0, sizeof total);
  int replayed = 0;
  rc = upload(0);
  for (int64_t c = 0; c < nchunks && rc == ODE_OK; ++c) {
    const int b = (int)(c & 1);
    cudaStream_t sc = b ? h->chunk_stream : s;
    const int64_t i0 = c * m, mc = std::min(m, n - i0);
    ode_solve_args sa = *a;
    sa.n = mc;
    sa.memory = ODE_MEM_DEVICE;
    sa.stream = sc;
    sa.u0 = (const double*)din[b][0];
    sa.p = (const double*)din[b][1];
    sa.dt0 = (const double*)din[b][2];
    ode_solve_out so;
    so.us = (double*)dout[b][0];
    so.u_final = (double*)dout[b][1];
    so.t_final = (double*)dout[b][2];
    so.retcode = (int8_t*)dout[b][3];
    so.naccept = (int32_t*)dout[b][4];
    so.nreject = (int32_t*)dout[b][5];
    so.dt_first = (double*)dout[b][6];
    const cudaError_t e = cudaStreamWaitEvent(sc, ready[b], 0);
    if (e != cudaSuccess) {
      rc = cuda_fail(h, e, "wait chunk inputs");
      break;
    }
    ChunkSlot slot = {b ? "#1" : "#0", ev_start[(size_t)c], ev_end[(size_t)c], h->chunk_stats + 4 * c, 0, 0, 0, 0, 0};
    rc = solve_impl(h, &sa, &so, nullptr, nullptr, &slot);
    if (rc != ODE_OK) break;
    total.launches += slot.launches;
    total.schedule_used = slot.sched;
    total.jit = slot.jit;
    total.kernel = slot.kernel;
    replayed += slot.replayed;
    if (c >= 1) rc = download(c - 1);
    if (rc == ODE_OK && c + 1 < nchunks) rc = upload(c + 1);
  }
  if (rc == ODE_OK) rc = download(nchunks - 1);
  /* everything enqueued is waited for, also after a failure, before the slots are reused */
  const cudaError_t e1 = cudaStreamSynchronize(cs);
  const cudaError_t e2 = cudaStreamSynchronize(s);
  const cudaError_t e3 = cudaStreamSynchronize(h->chunk_stream);
  if (rc != ODE_OK) {
    release();
    return rc;
  }
  const cudaError_t e = e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : e3;
  if (e != cudaSuccess) {
    release();
    return cuda_fail(h, e, "chunked solve");
  }
  /* from the first chunk's start to the latest end (a short last chunk can end before the one before it) */
  float span = 0.f;
  for (int64_t c = 0; c < nchunks; ++c) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev_start[0], ev_end[(size_t)c]) == cudaSuccess) span = std::max(span, ms);
  }
  release();
  unsigned long long early = 0;
  for (int64_t c = 0; c < nchunks; ++c) {
    total.attempts += (int64_t)h->chunk_stats[4 * c];
    total.saves += (int64_t)h->chunk_stats[4 * c + 1];
    early += h->chunk_stats[4 * c + 2];
  }
  if (st) {
    *st = total;
    st->kernel_ms = span;  /* first chunk's start to last chunk's end: the chunks' solves overlap */
    st->graph_replayed = replayed == nchunks ? 1 : 0;
    st->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  }
  if (early) {
    char msg[128];
    snprintf(msg, sizeof msg, "%llu trajectories stopped early (dt<dtmin or maxiters); see retcode", early);
    return fail(h, ODE_ETRAJ, msg);
  }
  return ODE_OK;
}

}  // namespace

extern "C" {

int ode_rhs_builtin(ode_handle* h, int rhs_id, int dim, int* rhs_out, int* nparams_out) {
  if (!h) return ODE_EINVAL;
  if (!rhs_out) return fail(h, ODE_EINVAL, "null rhs_out");
  int np = -1;
  switch (rhs_id) {
    case ODE_RHS_LORENZ: np = 3; break;
    case ODE_RHS_VANDERPOL: np = 1; break;
    case ODE_RHS_R3BP: np = 1; break;
    case ODE_RHS_KURAMOTO: np = dim + 1; break;
    case ODE_RHS_LINEAR: np = dim * dim; break;
    default: return fail(h, ODE_EINVAL, "not a built-in right-hand side id");
  }
  ode_solve_args a;
  std::memset(&a, 0, sizeof a);
  a.rhs = rhs_id;
  a.dim = dim;
  a.nparams = np;
  const int rc = check_rhs(h, &a);  /* the dimension rules the solver applies */
  if (rc != ODE_OK) return rc;
  *rhs_out = rhs_id;
  if (nparams_out) *nparams_out = np;
  return ODE_OK;
}

int ode_ensemble_solve(ode_handle* h, const ode_solve_args* a, ode_solve_out* o, ode_solve_stats* st) {
  if (h && a && o && a->memory == ODE_MEM_HOST && a->n >= 2 * kChunk && !is_fixed(a->alg) && !h->bounds_check &&
      a->alg >= ODE_ALG_RK4 && a->alg <= ODE_ALG_EULER && a->dim >= 1 && a->nparams >= 0 &&
      (a->nparams == 0 || a->p) && a->u0 && (a->nsave == 0 || a->saveat))
    return solve_chunked(h, a, o, st);
  return solve_impl(h, a, o, st, nullptr);
}

/* Ragged every-step output in two passes: count, prefix-sum on the host,
 * solve again writing each accepted step at its row. */
int ode_ensemble_solve_everystep(ode_handle* h, const ode_solve_args* a, ode_everystep_out* o,
                                 ode_solve_stats* st) {
  if (!h) return ODE_EINVAL;
  if (!a || !o || !o->offsets) return fail(h, ODE_EINVAL, "null argument");
  if (is_fixed(a->alg)) return fail(h, ODE_EINVAL, "every-step output is for the adaptive algorithms");
  if (a->nsave != 0 || a->output != ODE_OUTPUT_STATE)
    return fail(h, ODE_EINVAL, "every-step output takes no saveat and the state output");
  if (a->memory != ODE_MEM_HOST && a->memory != ODE_MEM_DEVICE) return fail(h, ODE_EINVAL, "unknown memory kind");
  if (a->layout != ODE_LAYOUT_SOA && a->layout != ODE_LAYOUT_TRAJ) return fail(h, ODE_EINVAL, "unknown output layout");
  if (a->controller != ODE_CTRL_DS && a->controller != ODE_CTRL_FP64 && a->controller != ODE_CTRL_FP32 &&
      a->controller != ODE_CTRL_REF)
    return fail(h, ODE_EINVAL, "unknown step-size controller");
  if ((a->controller == ODE_CTRL_FP64 || a->controller == ODE_CTRL_REF) && a->precision != ODE_FP64)
    return fail(h, ODE_ENOTSUP, "the FP64 and reference-arithmetic controllers apply to FP64 solves");
  if (a->n < 0 || a->n > 0x7fffffffLL) return fail(h, ODE_EINVAL, "n must be in [0, 2^31)");
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const int64_t n = a->n;
  const int D = a->dim;
  const bool host = a->memory == ODE_MEM_HOST;
  cudaStream_t s = a->stream ? (cudaStream_t)a->stream : h->stream;
  int rc = ODE_OK;

  /* pass 1: accepted steps per trajectory */
  std::vector<int32_t> counts((size_t)n);
  {
    ode_solve_args a1 = *a;
    a1.save_everystep = 0;
    ode_solve_out o1;
    std::memset(&o1, 0, sizeof o1);
    int32_t* dcount = nullptr;
    if (host) {
      o1.naccept = counts.data();
    } else {
      if (!(dcount = (int32_t*)buf(h, "ev_count", (size_t)n * 4, &rc))) return rc;
      o1.naccept = dcount;
    }
    rc = solve_impl(h, &a1, &o1, nullptr, nullptr);
    if (rc != ODE_OK && rc != ODE_ETRAJ) return rc;
    if (!host && n > 0) {
      CK(cudaMemcpyAsync(counts.data(), dcount, (size_t)n * 4, cudaMemcpyDeviceToHost, s), "copy counts");
      CK(cudaStreamSynchronize(s), "sync counts");
    }
  }
  std::vector<long long> off((size_t)n + 1);
  off[0] = 0;
  for (int64_t i = 0; i < n; ++i) off[(size_t)i + 1] = off[(size_t)i] + (long long)counts[(size_t)i] + 1;
  const int64_t total = off[(size_t)n];
  o->total = total;
  const size_t offbytes = ((size_t)n + 1) * sizeof(long long);
  if (host) {
    std::memcpy(o->offsets, off.data(), offbytes);
  } else {
    CK(cudaMemcpyAsync(o->offsets, off.data(), offbytes, cudaMemcpyHostToDevice, s), "copy offsets");
    CK(cudaStreamSynchronize(s), "sync offsets");
  }
  if (!o->ts || !o->us || o->capacity < total)
    return fail(h, ODE_ESMALL, "every-step buffers too small: total rows needed are in ode_everystep_out.total");

  /* pass 2: the same solve, writing each accepted step */
  EveryStep ev;
  if (host) {
    long long* doff = (long long*)buf(h, "ev_off", offbytes, &rc);
    if (!doff) return rc;
    double* dt = (double*)buf(h, "ev_t", (size_t)total * sizeof(double), &rc);
    if (!dt) return rc;
    double* du = (double*)buf(h, "ev_u", (size_t)total * D * sizeof(double), &rc);
    if (!du) return rc;
    CK(cudaMemcpyAsync(doff, off.data(), offbytes, cudaMemcpyHostToDevice, s), "copy offsets");
    ev = EveryStep{doff, dt, du};
  } else {
    ev = EveryStep{(const long long*)o->offsets, o->ts, o->us};
  }
  ode_solve_args a2 = *a;
  a2.save_everystep = 0;
  ode_solve_out o2;
  std::memset(&o2, 0, sizeof o2);
  o2.u_final = o->u_final;
  o2.t_final = o->t_final;
  o2.retcode = o->retcode;
  o2.naccept = o->naccept;
  o2.nreject = o->nreject;
  rc = solve_impl(h, &a2, &o2, st, &ev);
  if (rc != ODE_OK && rc != ODE_ETRAJ) return rc;
  if (host && total > 0) {
    CK(cudaMemcpyAsync(o->ts, ev.t, (size_t)total * sizeof(double), cudaMemcpyDeviceToHost, s), "copy ts");
    CK(cudaMemcpyAsync(o->us, ev.u, (size_t)total * D * sizeof(double), cudaMemcpyDeviceToHost, s), "copy us");
    CK(cudaStreamSynchronize(s), "sync every-step output");
  }
  return rc;
}

/* Autotuner: time launch-shape variants of the solver kernel on a sample of
 * the caller's ensemble and keep the fastest for this handle.  Variants are
 * compiled with NVRTC in parallel; they differ in threads per block, register
 * cap (which sets how many warps an SM holds) and the bytes of each warp's
 * saveat staging ring, never in arithmetic, so results do not change. */
int ode_autotune(ode_handle* h, const ode_solve_args* a, int64_t sample, ode_tune_report* rep) {
  if (!h) return ODE_EINVAL;
  NvtxRange nvtx("gbode autotune");
  if (h->bounds_check) return fail(h, ODE_ENOTSUP, "autotuning is off in bounds-check mode");
  if (!a) return fail(h, ODE_EINVAL, "null arguments");
  if (is_fixed(a->alg)) return fail(h, ODE_EINVAL, "autotuning applies to the adaptive algorithms");
  if (a->n < 1 || (a->memory != ODE_MEM_HOST && a->memory != ODE_MEM_DEVICE))
    return fail(h, ODE_EINVAL, "bad ensemble");
  int rc = check_rhs(h, a);
  if (rc != ODE_OK) return rc;
  CK(cudaSetDevice(h->device), "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t n = a->n;
  const int64_t m = std::min<int64_t>(n, sample > 0 ? std::max<int64_t>(sample, 1024) : 65536);
  const int D = a->dim, NP = a->nparams;
  cudaStream_t s = h->stream;
  const cudaMemcpyKind kind = a->memory == ODE_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  /* the first m trajectories, gathered from the [rows][n] arrays by strided copies */
  double* du0 = (double*)buf(h, "tune_u0", (size_t)m * D * 8, &rc);
  if (!du0) return rc;
  double* dp = (double*)buf(h, "tune_p", (size_t)m * (NP > 0 ? NP : 1) * 8, &rc);
  if (!dp) return rc;
  CK(cudaMemcpy2DAsync(du0, m * 8, a->u0, n * 8, m * 8, D, kind, s), "copy sample u0");
  if (NP > 0) CK(cudaMemcpy2DAsync(dp, m * 8, a->p, n * 8, m * 8, NP, kind, s), "copy sample p");
  double* ddt0 = nullptr;
  if (a->dt0) {
    if (!(ddt0 = (double*)buf(h, "tune_dt0", (size_t)m * 8, &rc))) return rc;
    CK(cudaMemcpyAsync(ddt0, a->dt0, m * 8, kind, s), "copy sample dt0");
  }
  const int width = output_width(h, a);
  double* dus = nullptr;
  if (a->nsave > 0 && !(dus = (double*)buf(h, "tune_us", (size_t)a->nsave * width * m * 8, &rc))) return rc;
  double* duf = (double*)buf(h, "tune_uf", (size_t)m * D * 8, &rc);
  if (!duf) return rc;
  CK(cudaStreamSynchronize(s), "sample copies");
  ode_solve_args ta = *a;
  ta.n = m;
  ta.memory = ODE_MEM_DEVICE;
  ta.u0 = du0;
  ta.p = dp;
  ta.dt0 = ddt0;
  ta.stream = nullptr;
  /* time in the order the solves will use: learned when a model fits these arguments */
  ta.schedule = a->schedule == ODE_SCHED_PLAIN                                      ? ODE_SCHED_PLAIN
                : (a->schedule == ODE_SCHED_LEARNED && model_ready(h->model, &ta)) ? ODE_SCHED_LEARNED
                                                                                    : ODE_SCHED_PERSISTENT;
  ode_solve_out to;
  std::memset(&to, 0, sizeof to);
  to.us = dus;
  to.u_final = duf;
  const std::string key = kernel_key(h, &ta, ta.schedule);
  /* the baseline is the kernel an untuned handle would run */
  h->tuned.erase(key);
  h->tune_choice.erase(key);
  CUfunction fn0;
  int jit0 = 0;
  rc = get_kernel(h, &ta, ta.schedule, &fn0, &jit0);
  if (rc != ODE_OK) return rc;
  auto time_solve = [&](double* ms) -> int {
    double best = 1e300;
    for (int r = 0; r < 3; ++r) {
      ode_solve_stats st;
      const int rr = ode_ensemble_solve(h, &ta, &to, &st);
      if (rr != ODE_OK && rr != ODE_ETRAJ) return rr;
      best = std::min(best, st.kernel_ms);
    }
    *ms = best;
    return ODE_OK;
  };
  double base_ms = 0;
  rc = time_solve(&base_ms);
  if (rc != ODE_OK) return rc;

  /* Search space.  The staging ring only exists in the staged kernel (saveat
   * with a persistent schedule) and only when it holds a full round of 32
   * jobs; a block's rings share its 48 KB of static shared memory. */
  struct Variant {
    int block, regs, stage;
  };
  const bool staged = std::strcmp(entry_kind(ta.alg, ta.schedule, ta.nsave), "staged") == 0;
  const int job = stage_unit_bytes(&ta);
  std::vector<Variant> vars;
  /* large jobs (Kuramoto-12: 804 bytes) also try the smallest ring that holds
   * one round, which leaves room for the most warps per SM */
  const int fit = (32 * job + 511) / 512 * 512;
  for (int block : {128, 64, 32}) {
    std::vector<int> rings;
    if (staged) {
      if (fit > 12288 && fit / 32 * block <= 49152) rings.push_back(fit);
      for (int ring : {12288, 16384, 24576, 36864, 49152})
        if (ring / 32 * block <= 49152 && (ring / job & ~7) >= 32) rings.push_back(ring);
    }
    if (rings.empty()) rings.push_back(12288);
    for (int regs : {0, 128, 112, 96, 80})
      for (int ring : rings) vars.push_back({block, regs, ring});
  }
  if ((int)vars.size() > ODE_TUNE_MAX_VARIANTS) vars.resize(ODE_TUNE_MAX_VARIANTS);
  const int nv = (int)vars.size();
  const std::string src = jit_source(h, &ta, ta.schedule);
  std::vector<std::vector<char>> cubins(nv);
  std::vector<int> ok(nv, 0);
  {
    /* compile on the host's cores, one variant per worker at a time */
    std::atomic<int> next(0);
    const int nworkers = std::max(1, std::min<int>(nv, (int)std::thread::hardware_concurrency()));
    std::vector<std::thread> th;
    for (int w = 0; w < nworkers; ++w) {
      th.emplace_back([&]() {
        for (int v = next++; v < nv; v = next++) {
          std::vector<std::string> o = {"-DGBODE_BLOCK=" + std::to_string(vars[v].block),
                                        "-DGBODE_STAGE_BYTES=" + std::to_string(vars[v].stage)};
          if (vars[v].regs) o.push_back("--maxrregcount=" + std::to_string(vars[v].regs));
          std::string lg, err;
          ok[v] = nvrtc_cubin(src, o, &cubins[v], &lg, &err) == ODE_OK;
        }
      });
    }
    for (auto& t : th) t.join();
  }
  double best_ms = base_ms;
  int best = -1, tried = 0;
  CUfunction best_fn = nullptr;
  std::vector<double> ms_of(nv, -1.0);
  for (int v = 0; v < nv; ++v) {
    if (!ok[v]) continue;
    CUfunction fn;
    rc = load_cubin(h, cubins[v], vars[v].block, vars[v].stage, &fn);
    if (rc != ODE_OK) return rc;
    h->tuned[key] = fn;
    double ms = 0;
    rc = time_solve(&ms);
    h->tuned.erase(key);
    if (rc != ODE_OK) return rc;
    ++tried;
    ms_of[v] = ms;
    if (ms < 0.99 * best_ms) {
      best_ms = ms;
      best = v;
      best_fn = fn;
    }
  }
  if (best >= 0) h->tuned[key] = best_fn;
  h->tune_choice[key] = best >= 0 ? std::vector<int>{vars[best].block, vars[best].regs, vars[best].stage}
                                   : std::vector<int>{0, 0, 0};  /* 0: the default kernel won */
  if (rep) {
    rep->variants = tried;
    rep->block = best >= 0 ? vars[best].block : block_of(h, fn0);
    rep->max_registers = best >= 0 ? vars[best].regs : 0;
    rep->stage_bytes = best >= 0 ? vars[best].stage : stage_of(h, fn0);
    rep->default_ms = base_ms;
    rep->best_ms = best_ms;
    rep->sample = m;
    rep->tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    rep->ntable = nv;
    for (int v = 0; v < nv; ++v)
      rep->table[v] = ode_tune_variant{vars[v].block, vars[v].regs, vars[v].stage, (float)ms_of[v]};
  }
  return ODE_OK;
}

}  // extern "C"
