/* Learned schedule: a small MLP predicts each trajectory's cost and first step.
 *
 * Model: x = standardised (p, u0) -> ReLU(W1 x + b1) -> ReLU(W2 h1 + b2) ->
 * W3 h2 + b3 = standardised (log attempts, log dt of the first accepted step).
 * Weights are kept in bfloat16 for the forward and backward passes (fp32
 * activations and accumulation) with fp32 master weights for the Adam update.
 * Training data: the attempt counts and first accepted dt that the plain
 * solver records for a training ensemble (ode_learn_fit).
 *
 * Schedule (ODE_SCHED_LEARNED): predict on the device, bin trajectories by
 * predicted log attempts (counting sort into 1024 bins, longest first) so the
 * persistent kernel hands out long trajectories first and similar costs share
 * warps.  Ordering changes no trajectory's arithmetic, so the results are
 * bit-identical to the plain schedule's.  Optionally (seed_dt0) each
 * trajectory's initial dt is seeded with the prediction, which removes most
 * rejected first attempts but changes the step sequence: results then agree
 * with the plain schedule's within the adaptive tolerance where the dynamics
 * do not amplify perturbations, and with the same accuracy against the exact
 * solution everywhere.  The solver's controller still accepts or rejects
 * every step.
 *
 * Kernels: mlp_fwd_bwd (one tile of 32 samples per block, activations in
 * shared memory, gradients accumulated with fp32 atomics), adam_update,
 * mlp_predict (one trajectory per thread, weights in shared memory),
 * bin_histogram / bin_scan / bin_scatter, dt0_from_log.
 */
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "ode_host.h"

namespace gbode {

constexpr int MAXIN = 40;   /* nparams + dim */
constexpr int HMAX = 64;
constexpr int NOUT = 2;
constexpr int TILE = 32;    /* samples per block in training */
constexpr int NBINS = kCostBins;

struct Model {
  int nin = 0, nh = 0, rhs = -1, alg = -1, dim = 0, nparams = 0;
  int seed_dt0 = 0;
  float dt0_safety = 1.0f;
  std::vector<float> xmean, xstd, ymean, ystd;  /* standardisation */
  float lo = 0.f, hi = 1.f;                      /* binning range of log attempts */
  float* d_master = nullptr;                     /* fp32 master weights */
  __nv_bfloat16* d_w = nullptr;                  /* bf16 weights */
  float* d_norm = nullptr;                       /* xmean, xstd, ymean, ystd on the device */
  size_t nparam = 0;
};

void model_free(Model* m) {
  if (!m) return;
  if (m->d_master) cudaFree(m->d_master);
  if (m->d_w) cudaFree(m->d_w);
  if (m->d_norm) cudaFree(m->d_norm);
  delete m;
}

__host__ __device__ static inline size_t param_count(int nin, int nh) { return (size_t)nh * nin + nh + (size_t)nh * nh + nh + NOUT * nh + NOUT; }

/* parameter offsets in the flat layout W1[nh][nin] b1[nh] W2[nh][nh] b2[nh] W3[2][nh] b3[2] */
struct Off {
  int w1, b1, w2, b2, w3, b3;
  __host__ __device__ Off(int nin, int nh) {
    w1 = 0;
    b1 = nh * nin;
    w2 = b1 + nh;
    b2 = w2 + nh * nh;
    w3 = b2 + nh;
    b3 = w3 + NOUT * nh;
  }
};

/* ------------------------------------------------------------------ training kernels */
/* One block = TILE samples (indices idx[tile*TILE + s]); forward with bf16
 * weights, loss = mean over the minibatch of the squared error summed over
 * both outputs, backward, and fp32 atomic accumulation of the gradient. */
__global__ void __launch_bounds__(128) mlp_fwd_bwd(int nin, int nh, const float* __restrict__ X,
                                                   const float* __restrict__ Y, const int* __restrict__ idx, int nb,
                                                   float inv_batch, const __nv_bfloat16* __restrict__ W,
                                                   float* __restrict__ grad, float* __restrict__ loss) {
  __shared__ float sx[TILE][MAXIN];
  __shared__ float a1[TILE][HMAX], a2[TILE][HMAX], d1[TILE][HMAX], d2[TILE][HMAX];
  __shared__ float dout[TILE][NOUT];
  const Off o(nin, nh);
  const int np = (int)param_count(nin, nh);
  const int tid = threadIdx.x, nt = blockDim.x;
  /* weights are read through the read-only cache (under 10 KB in bf16) */
#define sw(i) __bfloat162float(W[(i)])
  const int base = blockIdx.x * TILE;
  for (int i = tid; i < TILE * nin; i += nt) {
    const int s = i / nin, f = i % nin;
    const int r = base + s;
    sx[s][f] = (r < nb) ? X[(size_t)idx[r] * nin + f] : 0.f;
  }
  __syncthreads();
  /* h1 = relu(W1 x + b1) */
  for (int i = tid; i < TILE * nh; i += nt) {
    const int s = i / nh, j = i % nh;
    float acc = sw(o.b1 + j);
    for (int f = 0; f < nin; ++f) acc = fmaf(sw(o.w1 + j * nin + f), sx[s][f], acc);
    a1[s][j] = fmaxf(acc, 0.f);
  }
  __syncthreads();
  for (int i = tid; i < TILE * nh; i += nt) {
    const int s = i / nh, j = i % nh;
    float acc = sw(o.b2 + j);
    for (int k = 0; k < nh; ++k) acc = fmaf(sw(o.w2 + j * nh + k), a1[s][k], acc);
    a2[s][j] = fmaxf(acc, 0.f);
  }
  __syncthreads();
  if (tid < TILE * NOUT) {
    const int s = tid / NOUT, q = tid % NOUT;
    const int r = base + s;
    float acc = sw(o.b3 + q);
    for (int k = 0; k < nh; ++k) acc = fmaf(sw(o.w3 + q * nh + k), a2[s][k], acc);
    float g = 0.f;
    if (r < nb) {
      const float e = acc - Y[(size_t)idx[r] * NOUT + q];
      atomicAdd(loss, e * e * inv_batch);
      g = 2.f * e * inv_batch;
    }
    dout[s][q] = g;
  }
  __syncthreads();
  /* d2 = (W3^T dout) * [a2 > 0] */
  for (int i = tid; i < TILE * nh; i += nt) {
    const int s = i / nh, j = i % nh;
    float acc = 0.f;
    for (int q = 0; q < NOUT; ++q) acc = fmaf(sw(o.w3 + q * nh + j), dout[s][q], acc);
    d2[s][j] = a2[s][j] > 0.f ? acc : 0.f;
  }
  __syncthreads();
  for (int i = tid; i < TILE * nh; i += nt) {
    const int s = i / nh, k = i % nh;
    float acc = 0.f;
    for (int j = 0; j < nh; ++j) acc = fmaf(sw(o.w2 + j * nh + k), d2[s][j], acc);
    d1[s][k] = a1[s][k] > 0.f ? acc : 0.f;
  }
  __syncthreads();
  /* parameter gradients: sums over the tile's samples */
  for (int i = tid; i < np; i += nt) {
    float acc = 0.f;
    if (i < o.b1) {
      const int j = i / nin, f = i % nin;
      for (int s = 0; s < TILE; ++s) acc = fmaf(d1[s][j], sx[s][f], acc);
    } else if (i < o.w2) {
      const int j = i - o.b1;
      for (int s = 0; s < TILE; ++s) acc += d1[s][j];
    } else if (i < o.b2) {
      const int j = (i - o.w2) / nh, k = (i - o.w2) % nh;
      for (int s = 0; s < TILE; ++s) acc = fmaf(d2[s][j], a1[s][k], acc);
    } else if (i < o.w3) {
      const int j = i - o.b2;
      for (int s = 0; s < TILE; ++s) acc += d2[s][j];
    } else if (i < o.b3) {
      const int q = (i - o.w3) / nh, k = (i - o.w3) % nh;
      for (int s = 0; s < TILE; ++s) acc = fmaf(dout[s][q], a2[s][k], acc);
    } else {
      const int q = i - o.b3;
      for (int s = 0; s < TILE; ++s) acc += dout[s][q];
    }
    atomicAdd(&grad[i], acc);
  }
#undef sw
}

__global__ void adam_update(int np, float* __restrict__ w, float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                            float c1, float c2, float eps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  w[i] = wi;
  wb[i] = __float2bfloat16(wi);
  g[i] = 0.f;
}

/* ------------------------------------------------------------------ inference */
/* One trajectory per thread: features gathered from the SoA inputs
 * (p rows then u0 rows), standardised, forward pass with bf16 weights from
 * shared memory, outputs de-standardised. */
__global__ void __launch_bounds__(128) mlp_predict(long long n, int nin, int nh, int nparams, int dim,
                                                   const double* __restrict__ p, const double* __restrict__ u0,
                                                   const __nv_bfloat16* __restrict__ W, const float* __restrict__ nrm,
                                                   float* __restrict__ log_att, float* __restrict__ log_dt) {
  __shared__ float sw[HMAX * HMAX + HMAX * MAXIN + NOUT * HMAX + 2 * HMAX + NOUT];
  const Off o(nin, nh);
  const int np = (int)param_count(nin, nh);
  for (int i = threadIdx.x; i < np; i += blockDim.x) sw[i] = __bfloat162float(W[i]);
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  float x[MAXIN];
  for (int f = 0; f < nin; ++f) {
    const double v = f < nparams ? p[(long long)f * n + t] : u0[(long long)(f - nparams) * n + t];
    x[f] = ((float)v - nrm[f]) / nrm[MAXIN + f];
  }
  float h1[HMAX];
  for (int j = 0; j < nh; ++j) {
    float acc = sw[o.b1 + j];
    for (int f = 0; f < nin; ++f) acc = fmaf(sw[o.w1 + j * nin + f], x[f], acc);
    h1[j] = fmaxf(acc, 0.f);
  }
  float out0 = sw[o.b3], out1 = sw[o.b3 + 1];
  for (int j = 0; j < nh; ++j) {
    float acc = sw[o.b2 + j];
    for (int k = 0; k < nh; ++k) acc = fmaf(sw[o.w2 + j * nh + k], h1[k], acc);
    const float h2 = fmaxf(acc, 0.f);
    out0 = fmaf(sw[o.w3 + j], h2, out0);
    out1 = fmaf(sw[o.w3 + nh + j], h2, out1);
  }
  log_att[t] = out0 * nrm[2 * MAXIN + 2] + nrm[2 * MAXIN];
  log_dt[t] = out1 * nrm[2 * MAXIN + 3] + nrm[2 * MAXIN + 1];
}

/* ------------------------------------------------------------------ binning (counting sort, longest first) */
__device__ __forceinline__ int cost_bin(float v, float lo, float inv_w) {
  int b = (int)((v - lo) * inv_w);
  b = b < 0 ? 0 : (b >= NBINS ? NBINS - 1 : b);
  return NBINS - 1 - b; /* descending cost */
}

__global__ void bin_histogram(long long n, const float* __restrict__ key, float lo, float inv_w,
                              unsigned* __restrict__ count) {
  __shared__ unsigned h[NBINS];
  for (int i = threadIdx.x; i < NBINS; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    atomicAdd(&h[cost_bin(key[i], lo, inv_w)], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < NBINS; i += blockDim.x)
    if (h[i]) atomicAdd(&count[i], h[i]);
}

/* exclusive prefix sum of NBINS counts, one block of NBINS threads */
__global__ void bin_scan(unsigned* __restrict__ count) {
  __shared__ unsigned s[NBINS];
  const int i = threadIdx.x;
  s[i] = count[i];
  __syncthreads();
  for (int off = 1; off < NBINS; off <<= 1) {
    const unsigned v = i >= off ? s[i - off] : 0u;
    __syncthreads();
    s[i] += v;
    __syncthreads();
  }
  count[i] = i ? s[i - 1] : 0u;
}

__global__ void bin_scatter(long long n, const float* __restrict__ key, float lo, float inv_w,
                            unsigned* __restrict__ offset, int* __restrict__ order) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned pos = atomicAdd(&offset[cost_bin(key[i], lo, inv_w)], 1u);
    order[pos] = (int)i;
  }
}

__global__ void dt0_from_log(long long n, const float* __restrict__ log_dt, float safety, double* __restrict__ dt0) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dt0[i] = (double)safety * exp((double)log_dt[i]);
}

/* ------------------------------------------------------------------ host hooks */
bool model_ready(const Model* m, const ode_solve_args* a) {
  return m && m->d_w && m->dim == a->dim && m->nparams == a->nparams && m->rhs == a->rhs;
}
float model_dt0_safety(const Model* m) { return m ? m->dt0_safety : 1.0f; }
bool model_seed_dt0(const Model* m) { return m && m->seed_dt0; }

int model_predict_device(ode_handle* h, const ode_solve_args* a, const KParams& kp, float* log_att, float* log_dt,
                         cudaStream_t s, int* launches) {
  Model* m = h->model;
  const long long n = a->n;
  if (n == 0) return ODE_OK;
  const unsigned grid = (unsigned)((n + 127) / 128);
  mlp_predict<<<grid, 128, 0, s>>>(n, m->nin, m->nh, m->nparams, m->dim, kp.p, kp.u0, m->d_w, m->d_norm, log_att,
                                   log_dt);
  ++*launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ODE_OK : cuda_fail(h, e, "mlp_predict");
}

std::string model_key(const Model* m) {
  if (!m) return "nomodel";
  char b[256];
  snprintf(b, sizeof b, "%p|%p|%a|%a|%a|%d|%d|%d", (void*)m->d_w, (void*)m->d_norm, m->lo, m->hi, m->dt0_safety,
           m->seed_dt0, m->nin, m->nh);
  return b;
}

int order_by_cost(ode_handle* h, const float* log_att, int64_t n, int* order, unsigned* cnt, cudaStream_t s,
                  int* launches) {
  Model* m = h->model;
  cudaError_t e = cudaMemsetAsync(cnt, 0, NBINS * sizeof(unsigned), s);
  if (e != cudaSuccess) return cuda_fail(h, e, "memset bins");
  const float inv_w = (float)NBINS / std::max(1e-6f, m->hi - m->lo);
  const unsigned grid = (unsigned)std::min<int64_t>(4 * h->nsm, (n + 255) / 256 + 1);
  bin_histogram<<<grid, 256, 0, s>>>(n, log_att, m->lo, inv_w, cnt);
  bin_scan<<<1, NBINS, 0, s>>>(cnt);
  bin_scatter<<<grid, 256, 0, s>>>(n, log_att, m->lo, inv_w, cnt, order);
  *launches += 3;
  e = cudaGetLastError();
  return e == cudaSuccess ? ODE_OK : cuda_fail(h, e, "binning");
}

int seed_dt0(ode_handle* h, const float* log_dt, int64_t n, float safety, double* dt0, cudaStream_t s,
             int* launches) {
  dt0_from_log<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, log_dt, safety, dt0);
  ++*launches;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ODE_OK : cuda_fail(h, e, "dt0");
}

/* Fit on host-resident features/targets (already standardised). */
static int train(ode_handle* h, Model* m, const std::vector<float>& X, const std::vector<float>& Y, int nb,
                 const ode_learn_opts& o, float* loss_first, float* loss_last) {
  int rc;
  const size_t np = param_count(m->nin, m->nh);
  m->nparam = np;
  float* dX = (float*)buf(h, "learn_X", X.size() * 4, &rc);
  if (!dX) return rc;
  float* dY = (float*)buf(h, "learn_Y", Y.size() * 4, &rc);
  if (!dY) return rc;
  int* didx = (int*)buf(h, "learn_idx", (size_t)nb * 4, &rc);
  if (!didx) return rc;
  float* dG = (float*)buf(h, "learn_grad", np * 4, &rc);
  if (!dG) return rc;
  float* dM = (float*)buf(h, "learn_m", np * 4, &rc);
  if (!dM) return rc;
  float* dV = (float*)buf(h, "learn_v", np * 4, &rc);
  if (!dV) return rc;
  float* dL = (float*)buf(h, "learn_loss", 4, &rc);
  if (!dL) return rc;
  cudaStream_t s = h->stream;
  cudaError_t ae;
  if (!m->d_master && (ae = cudaMalloc(&m->d_master, np * 4)) != cudaSuccess) return cuda_fail(h, ae, "model alloc");
  if (!m->d_w && (ae = cudaMalloc(&m->d_w, np * 2)) != cudaSuccess) return cuda_fail(h, ae, "model alloc");
  /* He initialisation, seeded */
  std::mt19937_64 rng(o.seed);
  std::vector<float> w(np, 0.f);
  const Off off(m->nin, m->nh);
  std::normal_distribution<float> nd(0.f, 1.f);
  for (int i = off.w1; i < off.b1; ++i) w[i] = nd(rng) * std::sqrt(2.f / m->nin);
  for (int i = off.w2; i < off.b2; ++i) w[i] = nd(rng) * std::sqrt(2.f / m->nh);
  for (int i = off.w3; i < off.b3; ++i) w[i] = nd(rng) * std::sqrt(1.f / m->nh);
  std::vector<__nv_bfloat16> wb(np);
  for (size_t i = 0; i < np; ++i) wb[i] = __float2bfloat16(w[i]);
  cudaMemcpyAsync(m->d_master, w.data(), np * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(m->d_w, wb.data(), np * 2, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dG, 0, np * 4, s);
  cudaMemsetAsync(dM, 0, np * 4, s);
  cudaMemsetAsync(dV, 0, np * 4, s);
  cudaMemcpyAsync(dX, X.data(), X.size() * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dY, Y.data(), Y.size() * 4, cudaMemcpyHostToDevice, s);
  std::vector<int> idx(nb);
  for (int i = 0; i < nb; ++i) idx[i] = i;
  const int batch = std::max(TILE, std::min(o.batch, nb));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  int t = 0;
  for (int ep = 0; ep < o.epochs; ++ep) {
    std::shuffle(idx.begin(), idx.end(), rng);
    cudaMemcpyAsync(didx, idx.data(), (size_t)nb * 4, cudaMemcpyHostToDevice, s);
    cudaMemsetAsync(dL, 0, 4, s);
    int nsteps = 0;
    for (int start = 0; start + batch <= nb; start += batch) {
      ++t;
      ++nsteps;
      const unsigned blocks = (unsigned)((batch + TILE - 1) / TILE);
      mlp_fwd_bwd<<<blocks, 128, 0, s>>>(m->nin, m->nh, dX, dY, didx + start, batch, 1.f / batch, m->d_w, dG, dL);
      const float lr = o.lr * (ep < o.epochs / 2 ? 1.f : 0.1f + 0.9f * (float)(o.epochs - ep) / (o.epochs / 2 + 1));
      adam_update<<<(unsigned)((np + 255) / 256), 256, 0, s>>>((int)np, m->d_master, dG, dM, dV, m->d_w, lr, b1, b2,
                                                               1.f - std::pow(b1, (float)t),
                                                               1.f - std::pow(b2, (float)t), eps);
    }
    if (ep == 0 || ep == o.epochs - 1) {
      float l = 0;
      cudaMemcpyAsync(&l, dL, 4, cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      l /= std::max(1, nsteps);
      if (ep == 0) *loss_first = l;
      *loss_last = l;
    }
  }
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? ODE_OK : cuda_fail(h, e, "training");
}

}  // namespace gbode

using namespace gbode;

extern "C" {

void ode_learn_default_opts(ode_learn_opts* o) {
  if (!o) return;
  o->hidden = 64;
  o->epochs = 60;
  o->batch = 1024;
  o->lr = 3e-3f;
  o->seed = 1;
  o->seed_dt0 = 0;
  o->dt0_safety = 1.0f;
}

int ode_learn_fit(ode_handle* h, const ode_solve_args* a, const ode_learn_opts* opts, ode_learn_report* rep) {
  if (!h) return ODE_EINVAL;
  if (!a) return fail(h, ODE_EINVAL, "null arguments");
  ode_learn_opts o;
  ode_learn_default_opts(&o);
  if (opts) o = *opts;
  if (o.hidden < 1 || o.hidden > HMAX) return fail(h, ODE_EINVAL, "hidden width must be in [1, 64]");
  if (a->nparams + a->dim > MAXIN) return fail(h, ODE_EINVAL, "too many features (nparams + dim > 40)");
  if (a->alg != ODE_ALG_ATSIT5 && a->alg != ODE_ALG_AVERN7 && a->alg != ODE_ALG_AVERN9)
    return fail(h, ODE_EINVAL, "the learned schedule needs an adaptive algorithm");
  if (a->memory != ODE_MEM_HOST) return fail(h, ODE_EINVAL, "ode_learn_fit takes host arrays");
  if (a->n < 2 * TILE) return fail(h, ODE_EINVAL, "training ensemble too small");
  cudaSetDevice(h->device);
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t n = a->n;
  std::vector<int32_t> nacc(n), nrej(n);
  std::vector<double> dtf(n);
  std::vector<int8_t> ret(n);
  ode_solve_args ta = *a;
  ta.schedule = ODE_SCHED_PLAIN;
  ta.saveat = nullptr;
  ta.nsave = 0;
  ode_solve_out out;
  std::memset(&out, 0, sizeof out);
  out.naccept = nacc.data();
  out.nreject = nrej.data();
  out.dt_first = dtf.data();
  out.retcode = ret.data();
  int rc = ode_ensemble_solve(h, &ta, &out, nullptr);
  if (rc != ODE_OK && rc != ODE_ETRAJ) return rc;
  const auto t1 = std::chrono::steady_clock::now();

  Model* m = h->model ? h->model : new Model();
  h->model = m;
  const int nin = a->nparams + a->dim;
  if (m->nin != nin || m->nh != o.hidden) {
    if (m->d_master) cudaFree(m->d_master);
    if (m->d_w) cudaFree(m->d_w);
    m->d_master = nullptr;
    m->d_w = nullptr;
  }
  m->nin = nin;
  m->nh = o.hidden;
  m->rhs = a->rhs;
  m->alg = a->alg;
  m->dim = a->dim;
  m->nparams = a->nparams;
  m->seed_dt0 = o.seed_dt0;
  m->dt0_safety = o.dt0_safety;
  /* features (p then u0) and targets of the trajectories that finished */
  std::vector<float> X, Y;
  X.reserve((size_t)n * nin);
  Y.reserve((size_t)n * NOUT);
  int nb = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (ret[i] != ODE_RET_DEFAULT || !(dtf[i] > 0)) continue;
    for (int f = 0; f < a->nparams; ++f) X.push_back((float)a->p[(int64_t)f * n + i]);
    for (int d = 0; d < a->dim; ++d) X.push_back((float)a->u0[(int64_t)d * n + i]);
    Y.push_back(std::log((float)(nacc[i] + nrej[i])));
    Y.push_back(std::log((float)dtf[i]));
    ++nb;
  }
  if (nb < 2 * TILE) return fail(h, ODE_EINVAL, "too few finished training trajectories");
  m->xmean.assign(nin, 0.f);
  m->xstd.assign(nin, 0.f);
  m->ymean.assign(NOUT, 0.f);
  m->ystd.assign(NOUT, 0.f);
  for (int f = 0; f < nin; ++f) {
    double s = 0, s2 = 0;
    for (int i = 0; i < nb; ++i) s += X[(size_t)i * nin + f];
    const double mu = s / nb;
    for (int i = 0; i < nb; ++i) s2 += (X[(size_t)i * nin + f] - mu) * (X[(size_t)i * nin + f] - mu);
    const double sd = std::sqrt(s2 / nb);
    m->xmean[f] = (float)mu;
    m->xstd[f] = sd > 1e-12 ? (float)sd : 1.f;
  }
  float ylo = 1e30f, yhi = -1e30f;
  for (int q = 0; q < NOUT; ++q) {
    double s = 0, s2 = 0;
    for (int i = 0; i < nb; ++i) s += Y[(size_t)i * NOUT + q];
    const double mu = s / nb;
    for (int i = 0; i < nb; ++i) s2 += (Y[(size_t)i * NOUT + q] - mu) * (Y[(size_t)i * NOUT + q] - mu);
    const double sd = std::sqrt(s2 / nb);
    m->ymean[q] = (float)mu;
    m->ystd[q] = sd > 1e-12 ? (float)sd : 1.f;
  }
  for (int i = 0; i < nb; ++i) {
    ylo = std::min(ylo, Y[(size_t)i * NOUT]);
    yhi = std::max(yhi, Y[(size_t)i * NOUT]);
  }
  const float margin = 0.05f * (yhi - ylo) + 1e-3f;
  m->lo = ylo - margin;
  m->hi = yhi + margin;
  std::vector<float> Xs(X.size()), Ys(Y.size());
  for (int i = 0; i < nb; ++i) {
    for (int f = 0; f < nin; ++f) Xs[(size_t)i * nin + f] = (X[(size_t)i * nin + f] - m->xmean[f]) / m->xstd[f];
    for (int q = 0; q < NOUT; ++q) Ys[(size_t)i * NOUT + q] = (Y[(size_t)i * NOUT + q] - m->ymean[q]) / m->ystd[q];
  }
  /* device copy of the standardisation: xmean[MAXIN], xstd[MAXIN], ymean[2], ystd[2] */
  std::vector<float> nrm(2 * MAXIN + 4, 0.f);
  for (int f = 0; f < nin; ++f) {
    nrm[f] = m->xmean[f];
    nrm[MAXIN + f] = m->xstd[f];
  }
  nrm[2 * MAXIN] = m->ymean[0];
  nrm[2 * MAXIN + 1] = m->ymean[1];
  nrm[2 * MAXIN + 2] = m->ystd[0];
  nrm[2 * MAXIN + 3] = m->ystd[1];
  cudaError_t ae = cudaSuccess;
  if (!m->d_norm && (ae = cudaMalloc(&m->d_norm, nrm.size() * 4)) != cudaSuccess) return cuda_fail(h, ae, "model alloc");
  cudaMemcpy(m->d_norm, nrm.data(), nrm.size() * 4, cudaMemcpyHostToDevice);
  float lf = 0, ll = 0;
  rc = train(h, m, Xs, Ys, nb, o, &lf, &ll);
  if (rc != ODE_OK) return rc;
  const auto t2 = std::chrono::steady_clock::now();
  if (rep) {
    rep->loss_first = lf;
    rep->loss_last = ll;
    rep->train_solve_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    rep->train_fit_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    /* R^2 of log attempts on the training set */
    std::vector<float> la(n), ld(n);
    ode_solve_args pa = *a;
    rc = ode_learn_predict(h, &pa, la.data(), ld.data());
    if (rc != ODE_OK) return rc;
    double sse = 0, sst = 0;
    for (int64_t i = 0, k = 0; i < n; ++i) {
      if (ret[i] != ODE_RET_DEFAULT || !(dtf[i] > 0)) continue;
      const double y = Y[(size_t)k * NOUT];
      sse += (la[i] - y) * (la[i] - y);
      sst += (y - m->ymean[0]) * (y - m->ymean[0]);
      ++k;
    }
    rep->r2_attempts = (float)(1.0 - sse / std::max(sst, 1e-30));
  }
  return ODE_OK;
}

int ode_learn_predict(ode_handle* h, const ode_solve_args* a, float* log_attempts, float* log_dt_first) {
  if (!h) return ODE_EINVAL;
  if (!a) return fail(h, ODE_EINVAL, "null arguments");
  if (!model_ready(h->model, a)) return fail(h, ODE_ENOMODEL, "no model fitted for this problem shape");
  cudaSetDevice(h->device);
  const int64_t n = a->n;
  int rc;
  cudaStream_t s = h->stream;
  KParams kp;
  std::memset(&kp, 0, sizeof kp);
  if (a->memory == ODE_MEM_HOST) {
    double* du0 = (double*)buf(h, "u0", (size_t)n * a->dim * 8, &rc);
    if (!du0) return rc;
    double* dp = (double*)buf(h, "p", (size_t)n * (a->nparams > 0 ? a->nparams : 1) * 8, &rc);
    if (!dp) return rc;
    cudaMemcpyAsync(du0, a->u0, (size_t)n * a->dim * 8, cudaMemcpyHostToDevice, s);
    if (a->nparams) cudaMemcpyAsync(dp, a->p, (size_t)n * a->nparams * 8, cudaMemcpyHostToDevice, s);
    kp.u0 = du0;
    kp.p = dp;
  } else {
    kp.u0 = a->u0;
    kp.p = a->p;
  }
  float* la = (float*)buf(h, "pred_att", (size_t)n * 4, &rc);
  if (!la) return rc;
  float* ld = (float*)buf(h, "pred_dt", (size_t)n * 4, &rc);
  if (!ld) return rc;
  int launches = 0;
  rc = model_predict_device(h, a, kp, la, ld, s, &launches);
  if (rc != ODE_OK) return rc;
  if (log_attempts) cudaMemcpyAsync(log_attempts, la, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
  if (log_dt_first) cudaMemcpyAsync(log_dt_first, ld, (size_t)n * 4, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? ODE_OK : cuda_fail(h, e, "predict");
}

/* The training kernels' forward and backward pass on one batch, for
 * verification against a CPU implementation: params in the flat layout
 * (rounded to bf16 on upload, as training uses them), x [batch][nin],
 * y [batch][2]; writes the fp32 gradient and the loss. */
int ode_learn_gradcheck(ode_handle* h, int nin, int nh, int64_t batch, const float* params, const float* x,
                        const float* y, float* grad, float* loss) {
  if (!h || !params || !x || !y || !grad || !loss || nin < 1 || nin > MAXIN || nh < 1 || nh > HMAX || batch < 1 ||
      batch > (1 << 20))
    return fail(h, ODE_EINVAL, "ode_learn_gradcheck: bad arguments");
  cudaSetDevice(h->device);
  const size_t np = param_count(nin, nh);
  int rc;
  float* dX = (float*)buf(h, "gc_X", (size_t)batch * nin * 4, &rc);
  if (!dX) return rc;
  float* dY = (float*)buf(h, "gc_Y", (size_t)batch * NOUT * 4, &rc);
  if (!dY) return rc;
  int* di = (int*)buf(h, "gc_idx", (size_t)batch * 4, &rc);
  if (!di) return rc;
  float* dG = (float*)buf(h, "gc_G", np * 4, &rc);
  if (!dG) return rc;
  __nv_bfloat16* dW = (__nv_bfloat16*)buf(h, "gc_W", np * 2, &rc);
  if (!dW) return rc;
  float* dL = (float*)buf(h, "gc_L", 4, &rc);
  if (!dL) return rc;
  std::vector<__nv_bfloat16> wb(np);
  for (size_t i = 0; i < np; ++i) wb[i] = __float2bfloat16(params[i]);
  std::vector<int> idx(batch);
  for (int64_t i = 0; i < batch; ++i) idx[i] = (int)i;
  cudaStream_t s = h->stream;
  cudaMemcpyAsync(dX, x, (size_t)batch * nin * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dY, y, (size_t)batch * NOUT * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(di, idx.data(), (size_t)batch * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dW, wb.data(), np * 2, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dG, 0, np * 4, s);
  cudaMemsetAsync(dL, 0, 4, s);
  mlp_fwd_bwd<<<(unsigned)((batch + TILE - 1) / TILE), 128, 0, s>>>(nin, nh, dX, dY, di, (int)batch,
                                                                    1.f / (float)batch, dW, dG, dL);
  cudaMemcpyAsync(grad, dG, np * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(loss, dL, 4, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? ODE_OK : cuda_fail(h, e, "gradcheck");
}

}  // extern "C"
