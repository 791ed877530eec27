/* Internal host-side declarations shared by the library's translation units. */
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/gb300ode.h"
#include "ode_kparams.h"

namespace gbode {

/* Growable device buffer owned by a handle. */
struct DevBuf {
  void* ptr = nullptr;
  size_t cap = 0;
};

struct UserRhs {
  std::string body;
  int dim = 0, nparams = 0;
};

/* a saveat output function compiled into the solver kernel */
struct UserOutput {
  std::string body;
  int dim = 0, nparams = 0, width = 0;
};

/* a user SDE: drift and diffusion bodies compiled into the Euler-Maruyama kernel */
struct UserSde {
  std::string drift, diffusion;
  int dim = 0, nparams = 0;
  int noise_dim = 0;  /* 0: diagonal noise */
};

struct Model;  /* learned-schedule model, defined in learn.cu */

struct GraphEntry {
  std::string key;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
  unsigned long long last_use = 0;
};

constexpr int kGraphCache = 6;  /* captured solves kept per handle (least recently used evicted) */

constexpr int kCostBins = 1024;  /* bins of the learned schedule's counting sort */

}  // namespace gbode

struct ode_handle {
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  /* host<->device copies of the chunked host-buffer path */
  cudaStream_t chunk_stream = nullptr; /* second compute stream of the chunked path (odd chunks) */
  unsigned long long* chunk_stats = nullptr;  /* pinned: 4 statistics words per chunk */
  int64_t chunk_stats_cap = 0;                /* chunks that chunk_stats holds */
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  std::map<std::string, gbode::DevBuf> bufs;
  std::map<std::string, CUfunction> kcache;
  std::map<std::string, int> kjit;  /* 1 if the cached function was compiled at run time */
  std::map<std::string, CUfunction> tuned;  /* autotuned variant per kernel key */
  /* launch shape chosen per kernel key (block, register cap, ring bytes), by
   * ode_autotune or read by ode_tune_load; compiled on first use */
  std::map<std::string, std::vector<int>> tune_choice;
  std::map<CUfunction, int> fblock;         /* threads per block of run-time compiled functions */
  std::map<CUfunction, int> fstage;         /* staging-ring bytes per warp they were compiled with */
  std::vector<CUmodule> modules;
  std::vector<gbode::UserRhs> users;
  std::vector<gbode::UserOutput> outputs;
  std::vector<gbode::UserSde> sdes;
  std::map<std::string, CUfunction> sde_kernels;
  std::vector<gbode::GraphEntry> graphs;
  unsigned long long graph_tick = 0;
  gbode::Model* model = nullptr;
  bool bounds_check = false;  /* ode_set_bounds_check */
};

namespace gbode {

/* NVTX range for the lifetime of a scope (visible in Nsight Systems / ncu --nvtx) */
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

/* error helpers: record a message on the handle and return the code */
int fail(ode_handle* h, int code, const std::string& msg);
int cuda_fail(ode_handle* h, cudaError_t e, const char* what);
int cu_fail(ode_handle* h, CUresult r, const char* what);

/* device buffer of at least `bytes` bytes under `name` (contents not kept on growth) */
void* buf(ode_handle* h, const std::string& name, size_t bytes, int* rc);

/* run-time compilation of a translation unit whose kernel is named gbode_jit
 * (NVRTC with the solver headers), loaded into the handle's modules */
int jit_function(ode_handle* h, const std::string& src, int block, CUfunction* fn, std::string* log);
/* launch fn(params) on s through the driver API */
int launch_params(ode_handle* h, CUfunction fn, unsigned grid, unsigned block, void* params, cudaStream_t s);

/* learned schedule hooks (learn.cu) */
void model_free(Model* m);
/* Predict per-trajectory (log attempts, log dt_first) on the device for the
 * inputs in `kp` (device pointers); writes keys for ordering and, if
 * dt0_out is non-null, the seeded initial dt.  Enqueued on `s`. */
int model_predict_device(ode_handle* h, const ode_solve_args* a, const KParams& kp, float* log_att,
                         float* log_dt, cudaStream_t s, int* launches);
/* Order trajectories by predicted cost, longest first: order[n] on the device;
 * bins: kCostBins counters of device scratch. */
int order_by_cost(ode_handle* h, const float* log_att, int64_t n, int* order, unsigned* bins, cudaStream_t s,
                  int* launches);
/* Everything about the model that a captured launch sequence depends on. */
std::string model_key(const Model* m);
/* dt0[i] = safety * exp(log_dt[i]) */
int seed_dt0(ode_handle* h, const float* log_dt, int64_t n, float safety, double* dt0, cudaStream_t s,
             int* launches);
bool model_ready(const Model* m, const ode_solve_args* a);
float model_dt0_safety(const Model* m);
bool model_seed_dt0(const Model* m);

}  // namespace gbode
