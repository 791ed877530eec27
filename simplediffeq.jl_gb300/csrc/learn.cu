/* Learned schedule: a small MLP predicts each trajectory's cost and first step.
 *
 * Model: x = standardised (p, u0) -> ReLU(W1 x + b1) -> ReLU(W2 h1 + b2) ->
 * W3 h2 + b3 = standardised (log attempts, log dt of the first accepted step).
 * Training data: the attempt counts and first accepted dt that the solver
 * records for a training ensemble (ode_learn_fit).
 *
 * Arithmetic (the same in training and inference): every matrix product --
 * forward, backward and weight gradient -- takes bfloat16 operands (weights,
 * biases, features, activations, output deltas) and accumulates in fp32 on
 * the tensor cores (mma.sync m16n8k16 bf16); ReLU masks come from the fp32
 * pre-activations; the Adam update keeps fp32 master weights.  The CPU
 * restatement of one forward/backward pass in the same rounding is
 * oracle_mlp_forward_backward (mode 1).
 *
 * Training (mlp_train): ONE launch of one thread-block cluster runs every
 * epoch.  A minibatch is split over the cluster's CTAs, each CTA takes its
 * share in tiles of 128 samples (16 per warp): forward and backward of the two
 * 64-wide layers on the tensor cores with the activations kept in registers
 * from one layer to the next and written to shared memory once (bf16) for the
 * weight-gradient products, which run CTA-wide over the tile's samples.
 * Each CTA's partial gradient sits in its shared memory; CTA r owns a slice
 * of the parameters, sums that slice over the cluster through distributed
 * shared memory (fixed order: every run gives the same bits), applies Adam to
 * its fp32 master copy and writes the bf16 weights into every CTA's network.
 * Two cluster barriers a step, no global-memory round trip, no host work
 * between steps.  Samples are drawn per epoch through a keyed Feistel
 * permutation of the training set computed on the device.
 *
 * Schedule (ODE_SCHED_LEARNED): predict on the device (mlp_predict: the
 * training kernel's forward pass, 16 trajectories per warp), bin trajectories
 * by predicted log attempts (counting sort into 1024 bins, longest first) so
 * the persistent kernel hands out long trajectories first and similar costs
 * share warps.  Ordering changes no trajectory's arithmetic, so the results
 * are bit-identical to the plain schedule's.  Optionally (seed_dt0) each
 * trajectory's initial dt is seeded with the prediction, which removes most
 * rejected first attempts but changes the step sequence: results then agree
 * with the plain schedule's within the adaptive tolerance where the dynamics
 * do not amplify perturbations, and with the same accuracy against the exact
 * solution everywhere.  The solver's controller still accepts or rejects
 * every step.
 */
#include <cooperative_groups.h>
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

namespace cg = cooperative_groups;

namespace gbode {

constexpr int MAXIN = 40;   /* nparams + dim */
constexpr int HMAX = 64;
constexpr int NOUT = 2;
constexpr int NBINS = kCostBins;

/* the network inside the kernels */
constexpr int NH = 64;          /* hidden units; narrower models are zero-padded (padded units stay zero) */
constexpr int LDH = NH + 8;     /* bf16 row stride of hidden-width tiles: 144 B, ldmatrix rows on distinct banks */
constexpr int W3ROWS = 8;       /* output rows padded to one n8 tile */
constexpr int TW = 8;           /* warps per training CTA */
constexpr int TROWS = 16 * TW;  /* samples per training tile */
constexpr int PW = 8;           /* warps per prediction block */

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

/* k-steps of 16 features the first layer takes for `nin` inputs */
__host__ __device__ static inline int kin_steps(int nin) { return (nin + 15) / 16; }

/* ------------------------------------------------------------------ tensor-core helpers */
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p))
               : "memory");
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p))
               : "memory");
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_u32(p))
               : "memory");
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], const void* p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(smem_u32(p))
               : "memory");
}
/* d += a (16x16, row) * b (16x8, col), bf16 operands, fp32 accumulation */
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16(x)); }
constexpr uint32_t kOnesBf16x2 = 0x3F803F80u; /* two bf16 ones */

/* The network in shared memory, padded for the tensor cores:
 *   w1 [NH][ldx]      W1[j][f], zero for f >= nin
 *   w2 [NH][LDH]      W2[j][k]
 *   w3 [W3ROWS][LDH]  rows 0, 1 = W3, zero below
 *   b1 [NH], b2 [NH], b3 [W3ROWS] biases (bf16 values held in fp32)
 * Units beyond the model's width are zero throughout. */
struct Net {
  __nv_bfloat16 *w1, *w2, *w3;
  float *b1, *b2, *b3;
  int ldx;
};

/* Fill `net` from a flat parameter array (external layout, width nh); reader(i) returns parameter i. */
template <class Reader>
__device__ void load_net(const Net& net, int nin, int nh, Reader reader) {
  const Off o(nin, nh);
  const int nt = blockDim.x;
  for (int i = threadIdx.x; i < NH * net.ldx; i += nt) {
    const int j = i / net.ldx, f = i % net.ldx;
    net.w1[i] = __float2bfloat16((j < nh && f < nin) ? reader(o.w1 + j * nin + f) : 0.f);
  }
  for (int i = threadIdx.x; i < NH * LDH; i += nt) {
    const int j = i / LDH, k = i % LDH;
    net.w2[i] = __float2bfloat16((j < nh && k < nh) ? reader(o.w2 + j * nh + k) : 0.f);
  }
  for (int i = threadIdx.x; i < W3ROWS * LDH; i += nt) {
    const int q = i / LDH, k = i % LDH;
    net.w3[i] = __float2bfloat16((q < NOUT && k < nh) ? reader(o.w3 + q * nh + k) : 0.f);
  }
  for (int i = threadIdx.x; i < NH; i += nt) {
    net.b1[i] = bf16r(i < nh ? reader(o.b1 + i) : 0.f);
    net.b2[i] = bf16r(i < nh ? reader(o.b2 + i) : 0.f);
  }
  for (int i = threadIdx.x; i < W3ROWS; i += nt) net.b3[i] = bf16r(i < NOUT ? reader(o.b3 + i) : 0.f);
}

/* Forward pass of the 16 samples in rows [r0, r0 + 16) of the bf16 feature
 * tile xs (row stride net.ldx, KIN k-steps of 16 features).  out[] is the
 * output-layer fragment: lanes with lane % 4 == 0 hold outputs (0, 1) of row
 * r0 + lane/4 in out[0], out[1] and of row r0 + lane/4 + 8 in out[2], out[3].
 * With TRAIN the bf16 activations go to rows r0.. of h1s / h2s and the ReLU
 * masks come back (bit 4 nt + i: element i of the lane's fragment of n-tile
 * nt is positive). */
template <int KIN, bool TRAIN>
__device__ __forceinline__ void warp_forward(const Net& net, const __nv_bfloat16* xs, int r0, float (&out)[4],
                                             __nv_bfloat16* h1s, __nv_bfloat16* h2s, uint32_t& mask1,
                                             uint32_t& mask2) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3, mi = lane >> 3, ri = lane & 7;
  float acc[8][4];
  uint32_t a[4][4];
  /* layer 1 */
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float c0 = net.b1[nt * 8 + 2 * t], c1 = net.b1[nt * 8 + 2 * t + 1];
    acc[nt][0] = c0;
    acc[nt][1] = c1;
    acc[nt][2] = c0;
    acc[nt][3] = c1;
  }
#pragma unroll
  for (int ks = 0; ks < KIN; ++ks) {
    uint32_t ax[4];
    ldsm_x4(ax, xs + (r0 + (mi & 1) * 8 + ri) * net.ldx + ks * 16 + (mi >> 1) * 8);
#pragma unroll
    for (int np = 0; np < 4; ++np) {
      uint32_t b[4];
      ldsm_x4(b, net.w1 + (np * 16 + (mi >> 1) * 8 + ri) * net.ldx + ks * 16 + (mi & 1) * 8);
      mma_bf16(acc[2 * np], ax, b[0], b[1]);
      mma_bf16(acc[2 * np + 1], ax, b[2], b[3]);
    }
  }
  uint32_t m = 0;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (acc[nt][i] > 0.f) m |= 1u << (nt * 4 + i);
      else acc[nt][i] = 0.f;
    }
  mask1 = m;
  /* the accumulator fragments of n-tiles 2kk, 2kk+1 are the A fragment of k-step kk */
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    a[kk][0] = pack_bf16(acc[2 * kk][0], acc[2 * kk][1]);
    a[kk][1] = pack_bf16(acc[2 * kk][2], acc[2 * kk][3]);
    a[kk][2] = pack_bf16(acc[2 * kk + 1][0], acc[2 * kk + 1][1]);
    a[kk][3] = pack_bf16(acc[2 * kk + 1][2], acc[2 * kk + 1][3]);
    if (TRAIN) {
      *reinterpret_cast<uint32_t*>(h1s + (r0 + g) * LDH + kk * 16 + 2 * t) = a[kk][0];
      *reinterpret_cast<uint32_t*>(h1s + (r0 + g + 8) * LDH + kk * 16 + 2 * t) = a[kk][1];
      *reinterpret_cast<uint32_t*>(h1s + (r0 + g) * LDH + kk * 16 + 8 + 2 * t) = a[kk][2];
      *reinterpret_cast<uint32_t*>(h1s + (r0 + g + 8) * LDH + kk * 16 + 8 + 2 * t) = a[kk][3];
    }
  }
  /* layer 2 */
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const float c0 = net.b2[nt * 8 + 2 * t], c1 = net.b2[nt * 8 + 2 * t + 1];
    acc[nt][0] = c0;
    acc[nt][1] = c1;
    acc[nt][2] = c0;
    acc[nt][3] = c1;
  }
#pragma unroll
  for (int kk = 0; kk < 4; ++kk)
#pragma unroll
    for (int np = 0; np < 4; ++np) {
      uint32_t b[4];
      ldsm_x4(b, net.w2 + (np * 16 + (mi >> 1) * 8 + ri) * LDH + kk * 16 + (mi & 1) * 8);
      mma_bf16(acc[2 * np], a[kk], b[0], b[1]);
      mma_bf16(acc[2 * np + 1], a[kk], b[2], b[3]);
    }
  m = 0;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (acc[nt][i] > 0.f) m |= 1u << (nt * 4 + i);
      else acc[nt][i] = 0.f;
    }
  mask2 = m;
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    a[kk][0] = pack_bf16(acc[2 * kk][0], acc[2 * kk][1]);
    a[kk][1] = pack_bf16(acc[2 * kk][2], acc[2 * kk][3]);
    a[kk][2] = pack_bf16(acc[2 * kk + 1][0], acc[2 * kk + 1][1]);
    a[kk][3] = pack_bf16(acc[2 * kk + 1][2], acc[2 * kk + 1][3]);
    if (TRAIN) {
      *reinterpret_cast<uint32_t*>(h2s + (r0 + g) * LDH + kk * 16 + 2 * t) = a[kk][0];
      *reinterpret_cast<uint32_t*>(h2s + (r0 + g + 8) * LDH + kk * 16 + 2 * t) = a[kk][1];
      *reinterpret_cast<uint32_t*>(h2s + (r0 + g) * LDH + kk * 16 + 8 + 2 * t) = a[kk][2];
      *reinterpret_cast<uint32_t*>(h2s + (r0 + g + 8) * LDH + kk * 16 + 8 + 2 * t) = a[kk][3];
    }
  }
  /* output layer: one n8 tile (outputs 0, 1 and zero padding) */
  out[0] = net.b3[2 * t];
  out[1] = net.b3[2 * t + 1];
  out[2] = out[0];
  out[3] = out[1];
#pragma unroll
  for (int kk = 0; kk < 4; ++kk) {
    uint32_t b[2];
    ldsm_x2(b, net.w3 + ri * LDH + kk * 16 + (mi & 1) * 8);
    mma_bf16(out, a[kk], b[0], b[1]);
  }
}

/* ------------------------------------------------------------------ training */
struct TrainParams {
  const float* X;      /* [nb][nin] standardised features */
  const float* Y;      /* [nb][2] standardised targets */
  int nb, nin, nh;
  int batch;           /* samples per step */
  int epochs;
  int steps_per_epoch;
  float lr;
  uint32_t seed_lo, seed_hi;
  int grad_only;       /* 1: one step over samples 0..batch-1 in order, the summed gradient to `grad`, no update */
  float* master;       /* in: initial fp32 parameters; out (training): trained fp32 parameters (flat layout) */
  __nv_bfloat16* wbf;  /* out (training): bf16 parameters */
  float* grad;         /* out (grad_only): fp32 gradient (flat layout) */
  float* loss;         /* [2]: summed minibatch losses of the first and the last epoch (atomic adds) */
};

/* Shared-memory layout of a training CTA (host and device agree on it). */
struct TrainLayout {
  int ldx, P, S;
  size_t w1, w2, w3, b1, b2, b3, xs, h1, h2, d1, d2, dout, ys, gp, om, ov, ow, misc, total;
  __host__ __device__ TrainLayout(int nin, int csize) {
    ldx = kin_steps(nin) * 16 + 8;
    P = NH * nin + NH + NH * NH + NH + NOUT * NH + NOUT;
    S = (P + csize - 1) / csize;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 15) & ~(size_t)15;
      return at;
    };
    w1 = take((size_t)NH * ldx * 2);
    w2 = take((size_t)NH * LDH * 2);
    w3 = take((size_t)W3ROWS * LDH * 2);
    b1 = take(NH * 4);
    b2 = take(NH * 4);
    b3 = take(W3ROWS * 4);
    xs = take((size_t)TROWS * ldx * 2);
    h1 = take((size_t)TROWS * LDH * 2);
    h2 = take((size_t)TROWS * LDH * 2);
    d1 = take((size_t)TROWS * LDH * 2);
    d2 = take((size_t)TROWS * LDH * 2);
    dout = take((size_t)TROWS * 8 * 2);
    ys = take((size_t)TROWS * 2 * 4);
    gp = take((size_t)P * 4);
    om = take((size_t)S * 4);
    ov = take((size_t)S * 4);
    ow = take((size_t)S * 4);
    misc = take(64);
    total = o;
  }
};

/* Internal parameter order (hidden width NH): W1[NH][nin] b1[NH] W2[NH][NH] b2[NH] W3[2][NH] b3[2].
 * For internal index i: the flat external index for width nh (-1 for a padded
 * unit) and the shared-memory element of the network it lives in. */
struct ParamSlot {
  int ext;          /* index in the external layout, or -1 */
  int kind;         /* 0: bf16 weight (w points into w1/w2/w3), 1: fp32 bias (b) */
  int off;          /* element offset within the array named by `arr` */
  int arr;          /* 0 w1, 1 w2, 2 w3, 3 b1, 4 b2, 5 b3 */
};

__device__ __forceinline__ ParamSlot param_slot(int i, int nin, int nh, int ldx) {
  const Off o(nin, nh);
  ParamSlot s;
  const int a1 = NH * nin, a2 = a1 + NH, a3 = a2 + NH * NH, a4 = a3 + NH, a5 = a4 + NOUT * NH;
  if (i < a1) {
    const int j = i / nin, f = i % nin;
    s = {j < nh ? o.w1 + j * nin + f : -1, 0, j * ldx + f, 0};
  } else if (i < a2) {
    const int j = i - a1;
    s = {j < nh ? o.b1 + j : -1, 1, j, 3};
  } else if (i < a3) {
    const int j = (i - a2) / NH, k = (i - a2) % NH;
    s = {(j < nh && k < nh) ? o.w2 + j * nh + k : -1, 0, j * LDH + k, 1};
  } else if (i < a4) {
    const int j = i - a3;
    s = {j < nh ? o.b2 + j : -1, 1, j, 4};
  } else if (i < a5) {
    const int q = (i - a4) / NH, k = (i - a4) % NH;
    s = {k < nh ? o.w3 + q * nh + k : -1, 0, q * LDH + k, 2};
  } else {
    const int q = i - a5;
    s = {o.b3 + q, 1, q, 5};
  }
  return s;
}

/* Keyed permutation of [0, n): a 4-round Feistel network on the smallest
 * even-width power-of-two domain that holds n, cycle-walked into [0, n). */
struct Perm {
  uint32_t n, half, mask;
  uint32_t key[4];
};

__device__ __forceinline__ uint32_t mix32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

__device__ __forceinline__ Perm make_perm(uint32_t n, uint32_t seed_lo, uint32_t seed_hi, uint32_t epoch) {
  Perm p;
  p.n = n;
  uint32_t bits = 2;
  while (bits < 32 && (1u << bits) < n) ++bits;
  p.half = (bits + 1) / 2;
  p.mask = (1u << p.half) - 1u;
  for (int r = 0; r < 4; ++r) p.key[r] = mix32(seed_lo ^ mix32(seed_hi + 0x9e3779b9U * (epoch * 4u + r + 1u)));
  return p;
}

__device__ __forceinline__ uint32_t permute(uint32_t i, const Perm& p) {
  uint32_t x = i;
  /* the walk returns to [0, n) after a few rounds on average (the domain is
   * under 4n); the bound only keeps the loop finite */
  for (int it = 0; it < 4096; ++it) {
    uint32_t L = x >> p.half, R = x & p.mask;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint32_t F = mix32(R ^ p.key[r]) & p.mask;
      const uint32_t nl = R;
      R = L ^ F;
      L = nl;
    }
    x = (L << p.half) | R;
    if (x < p.n) return x;
  }
  return i;
}

/* One thread-block cluster trains the network for every epoch (see the file
 * comment).  Grid = the cluster: CSIZE CTAs of TW warps. */
template <int KIN, int CSIZE>
__global__ void __launch_bounds__(TW * 32, 1) mlp_train(TrainParams tp) {
  constexpr int csize = CSIZE;
  extern __shared__ __align__(16) unsigned char smem[];
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3, mi = lane >> 3, ri = lane & 7;
  const int nin = tp.nin;
  const TrainLayout L(nin, csize);
  Net net;
  net.w1 = (__nv_bfloat16*)(smem + L.w1);
  net.w2 = (__nv_bfloat16*)(smem + L.w2);
  net.w3 = (__nv_bfloat16*)(smem + L.w3);
  net.b1 = (float*)(smem + L.b1);
  net.b2 = (float*)(smem + L.b2);
  net.b3 = (float*)(smem + L.b3);
  net.ldx = L.ldx;
  __nv_bfloat16* xs = (__nv_bfloat16*)(smem + L.xs);
  __nv_bfloat16* h1s = (__nv_bfloat16*)(smem + L.h1);
  __nv_bfloat16* h2s = (__nv_bfloat16*)(smem + L.h2);
  __nv_bfloat16* d1s = (__nv_bfloat16*)(smem + L.d1);
  __nv_bfloat16* d2s = (__nv_bfloat16*)(smem + L.d2);
  __nv_bfloat16* douts = (__nv_bfloat16*)(smem + L.dout);
  float* ys = (float*)(smem + L.ys);
  float* gp = (float*)(smem + L.gp);
  float* om = (float*)(smem + L.om);
  float* ov = (float*)(smem + L.ov);
  float* ow = (float*)(smem + L.ow);
  float* sloss = (float*)(smem + L.misc);
  const int nh = tp.nh;
  const int lo = rank * L.S, hi = min(L.P, lo + L.S);
  const int ldx = L.ldx;

  /* initial network, owner slice, zeroed output-delta padding */
  load_net(net, nin, nh, [&](int i) { return tp.master[i]; });
  for (int i = lo + tid; i < hi; i += blockDim.x) {
    const ParamSlot s = param_slot(i, nin, nh, ldx);
    ow[i - lo] = s.ext >= 0 ? tp.master[s.ext] : 0.f;
    om[i - lo] = 0.f;
    ov[i - lo] = 0.f;
  }
  for (int i = tid; i < TROWS * 8; i += blockDim.x) douts[i] = __float2bfloat16(0.f);
  if (tid == 0) *sloss = 0.f;
  cluster.sync();

  const float inv_b = 1.f / (float)tp.batch;
  const int chunk = (tp.batch + csize - 1) / csize;
  const int my0 = min(tp.batch, rank * chunk), my1 = min(tp.batch, my0 + chunk);
  const int total_steps = tp.grad_only ? 1 : tp.epochs * tp.steps_per_epoch;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;

  /* the tile of step `st` starting at batch row r0: features to bf16, targets,
   * zero rows beyond the batch */
  auto gather = [&](int st, int r0) {
    const int valid = min(TROWS, my1 - r0);
    const int sie = tp.grad_only ? 0 : st % tp.steps_per_epoch;
    const Perm perm = make_perm((uint32_t)tp.nb, tp.seed_lo, tp.seed_hi,
                                (uint32_t)(tp.grad_only ? 0 : st / tp.steps_per_epoch));
    for (int i = tid; i < TROWS * 2; i += blockDim.x) {
      const int s = i >> 1, half = i & 1;
      int idx = -1;
      if (s < valid) {
        const uint32_t pos = (uint32_t)(sie * tp.batch + r0 + s);
        idx = tp.grad_only ? (int)pos : (int)permute(pos, perm);
      }
      for (int f = half; f < ldx - 8; f += 2)
        xs[s * ldx + f] = __float2bfloat16((idx >= 0 && f < nin) ? tp.X[(size_t)idx * nin + f] : 0.f);
      ys[s * 2 + half] = idx >= 0 ? tp.Y[(size_t)idx * NOUT + half] : 0.f;
    }
  };
  bool prefetched = false; /* the step's first tile was gathered during the previous step's reduction */

  for (int step = 0; step < total_steps; ++step) {
    const int epoch = tp.grad_only ? 0 : step / tp.steps_per_epoch;
    const int sie = tp.grad_only ? 0 : step % tp.steps_per_epoch;
    for (int i = tid; i < L.P; i += blockDim.x) gp[i] = 0.f;

    for (int r0 = my0; r0 < my1; r0 += TROWS) {
      const int valid = min(TROWS, my1 - r0);
      const int kmax = (valid + 15) >> 4;
      if (!(prefetched && r0 == my0)) gather(step, r0);
      __syncthreads();
      /* per warp: forward, output deltas, backward through both hidden layers */
      const int wr = warp * 16;
      if (wr < valid) {
        float out[4];
        uint32_t mask1, mask2;
        warp_forward<KIN, true>(net, xs, wr, out, h1s, h2s, mask1, mask2);
        float dg0 = 0.f, dg1 = 0.f, dh0 = 0.f, dh1 = 0.f, lsum = 0.f;
        if (t == 0) {
          if (wr + g < valid) {
            const float e0 = out[0] - ys[(wr + g) * 2], e1 = out[1] - ys[(wr + g) * 2 + 1];
            lsum = e0 * e0 * inv_b + e1 * e1 * inv_b;
            dg0 = bf16r(2.f * e0 * inv_b);
            dg1 = bf16r(2.f * e1 * inv_b);
          }
          if (wr + g + 8 < valid) {
            const float e0 = out[2] - ys[(wr + g + 8) * 2], e1 = out[3] - ys[(wr + g + 8) * 2 + 1];
            lsum += e0 * e0 * inv_b + e1 * e1 * inv_b;
            dh0 = bf16r(2.f * e0 * inv_b);
            dh1 = bf16r(2.f * e1 * inv_b);
          }
          *reinterpret_cast<uint32_t*>(douts + (wr + g) * 8) = pack_bf16(dg0, dg1);
          *reinterpret_cast<uint32_t*>(douts + (wr + g + 8) * 8) = pack_bf16(dh0, dh1);
        }
        lsum += __shfl_xor_sync(0xffffffffu, lsum, 4);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, 8);
        lsum += __shfl_xor_sync(0xffffffffu, lsum, 16);
        if (lane == 0) atomicAdd(sloss, lsum);
        const int src = lane & ~3;
        dg0 = __shfl_sync(0xffffffffu, dg0, src);
        dg1 = __shfl_sync(0xffffffffu, dg1, src);
        dh0 = __shfl_sync(0xffffffffu, dh0, src);
        dh1 = __shfl_sync(0xffffffffu, dh1, src);
        /* d2 = W3^T dout (bf16 operands, both products exact in fp32), masked by layer 2's ReLU */
        uint32_t ad[4][4];
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const int j = nt * 8 + 2 * t;
          const float w0a = __bfloat162float(net.w3[j]), w0b = __bfloat162float(net.w3[j + 1]);
          const float w1a = __bfloat162float(net.w3[LDH + j]), w1b = __bfloat162float(net.w3[LDH + j + 1]);
          acc[nt][0] = (mask2 >> (nt * 4 + 0) & 1u) ? fmaf(w0a, dg0, w1a * dg1) : 0.f;
          acc[nt][1] = (mask2 >> (nt * 4 + 1) & 1u) ? fmaf(w0b, dg0, w1b * dg1) : 0.f;
          acc[nt][2] = (mask2 >> (nt * 4 + 2) & 1u) ? fmaf(w0a, dh0, w1a * dh1) : 0.f;
          acc[nt][3] = (mask2 >> (nt * 4 + 3) & 1u) ? fmaf(w0b, dh0, w1b * dh1) : 0.f;
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
          ad[kk][0] = pack_bf16(acc[2 * kk][0], acc[2 * kk][1]);
          ad[kk][1] = pack_bf16(acc[2 * kk][2], acc[2 * kk][3]);
          ad[kk][2] = pack_bf16(acc[2 * kk + 1][0], acc[2 * kk + 1][1]);
          ad[kk][3] = pack_bf16(acc[2 * kk + 1][2], acc[2 * kk + 1][3]);
          *reinterpret_cast<uint32_t*>(d2s + (wr + g) * LDH + kk * 16 + 2 * t) = ad[kk][0];
          *reinterpret_cast<uint32_t*>(d2s + (wr + g + 8) * LDH + kk * 16 + 2 * t) = ad[kk][1];
          *reinterpret_cast<uint32_t*>(d2s + (wr + g) * LDH + kk * 16 + 8 + 2 * t) = ad[kk][2];
          *reinterpret_cast<uint32_t*>(d2s + (wr + g + 8) * LDH + kk * 16 + 8 + 2 * t) = ad[kk][3];
        }
        /* d1 = W2^T d2, masked by layer 1's ReLU */
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
#pragma unroll
          for (int np = 0; np < 4; ++np) {
            uint32_t b[4];
            ldsm_x4_t(b, net.w2 + (kk * 16 + (mi & 1) * 8 + ri) * LDH + np * 16 + (mi >> 1) * 8);
            mma_bf16(acc[2 * np], ad[kk], b[0], b[1]);
            mma_bf16(acc[2 * np + 1], ad[kk], b[2], b[3]);
          }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const float v0 = (mask1 >> (nt * 4 + 0) & 1u) ? acc[nt][0] : 0.f;
          const float v1 = (mask1 >> (nt * 4 + 1) & 1u) ? acc[nt][1] : 0.f;
          const float v2 = (mask1 >> (nt * 4 + 2) & 1u) ? acc[nt][2] : 0.f;
          const float v3 = (mask1 >> (nt * 4 + 3) & 1u) ? acc[nt][3] : 0.f;
          *reinterpret_cast<uint32_t*>(d1s + (wr + g) * LDH + nt * 8 + 2 * t) = pack_bf16(v0, v1);
          *reinterpret_cast<uint32_t*>(d1s + (wr + g + 8) * LDH + nt * 8 + 2 * t) = pack_bf16(v2, v3);
        }
      }
      __syncthreads();
      /* weight gradients over the tile's samples (K = samples, operands read transposed) */
      {
        /* gW2[j][k] = sum_s d2[s][j] h1[s][k]; gb2[j] = sum_s d2[s][j] (ones operand) */
        const int mt = warp >> 1, nb0 = (warp & 1) * 32;
        float acc[4][4] = {};
        float accb[4] = {};
        const bool bias = (warp & 1) == 0;
        const uint32_t ones = g == 0 ? kOnesBf16x2 : 0u;
        for (int ks = 0; ks < kmax; ++ks) {
          uint32_t a[4];
          ldsm_x4_t(a, d2s + (ks * 16 + (mi >> 1) * 8 + ri) * LDH + mt * 16 + (mi & 1) * 8);
#pragma unroll
          for (int np = 0; np < 2; ++np) {
            uint32_t b[4];
            ldsm_x4_t(b, h1s + (ks * 16 + (mi & 1) * 8 + ri) * LDH + nb0 + np * 16 + (mi >> 1) * 8);
            mma_bf16(acc[2 * np], a, b[0], b[1]);
            mma_bf16(acc[2 * np + 1], a, b[2], b[3]);
          }
          if (bias) mma_bf16(accb, a, ones, ones);
        }
        const int gw2 = NH * nin + NH, gb2 = gw2 + NH * NH;
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) {
          const int j = mt * 16 + g, k = nb0 + nt * 8 + 2 * t;
          gp[gw2 + j * NH + k] += acc[nt][0];
          gp[gw2 + j * NH + k + 1] += acc[nt][1];
          gp[gw2 + (j + 8) * NH + k] += acc[nt][2];
          gp[gw2 + (j + 8) * NH + k + 1] += acc[nt][3];
        }
        if (bias && t == 0) {
          gp[gb2 + mt * 16 + g] += accb[0];
          gp[gb2 + mt * 16 + g + 8] += accb[2];
        }
      }
      {
        /* gW1[j][f] = sum_s d1[s][j] x[s][f]; gb1[j] = sum_s d1[s][j] */
        const int gw1 = 0, gb1 = NH * nin;
        const uint32_t ones = g == 0 ? kOnesBf16x2 : 0u;
        for (int id = warp; id < 8 * KIN; id += TW) {
          const int mt = id & 3, nt = id >> 2;
          float acc[4] = {};
          float accb[4] = {};
          const bool bias = nt == 0;
          for (int ks = 0; ks < kmax; ++ks) {
            uint32_t a[4], b[2];
            ldsm_x4_t(a, d1s + (ks * 16 + (mi >> 1) * 8 + ri) * LDH + mt * 16 + (mi & 1) * 8);
            ldsm_x2_t(b, xs + (ks * 16 + (mi & 1) * 8 + ri) * ldx + nt * 8);
            mma_bf16(acc, a, b[0], b[1]);
            if (bias) mma_bf16(accb, a, ones, ones);
          }
          const int j = mt * 16 + g, f = nt * 8 + 2 * t;
          if (f < nin) {
            gp[gw1 + j * nin + f] += acc[0];
            gp[gw1 + (j + 8) * nin + f] += acc[2];
          }
          if (f + 1 < nin) {
            gp[gw1 + j * nin + f + 1] += acc[1];
            gp[gw1 + (j + 8) * nin + f + 1] += acc[3];
          }
          if (bias && t == 0) {
            gp[gb1 + mt * 16 + g] += accb[0];
            gp[gb1 + mt * 16 + g + 8] += accb[2];
          }
        }
      }
      if (warp < 4) {
        /* gW3[q][k] = sum_s dout[s][q] h2[s][k] as (h2^T dout)[k][q]; warp 0 also gb3[q] = sum_s dout[s][q] */
        const int mt = warp;
        float acc[4] = {};
        float accb[4] = {};
        uint32_t onesa[4] = {g == 0 ? kOnesBf16x2 : 0u, 0u, g == 0 ? kOnesBf16x2 : 0u, 0u};
        for (int ks = 0; ks < kmax; ++ks) {
          uint32_t a[4], b[2];
          ldsm_x4_t(a, h2s + (ks * 16 + (mi >> 1) * 8 + ri) * LDH + mt * 16 + (mi & 1) * 8);
          ldsm_x2_t(b, douts + (ks * 16 + (mi & 1) * 8 + ri) * 8);
          mma_bf16(acc, a, b[0], b[1]);
          if (warp == 0) mma_bf16(accb, onesa, b[0], b[1]);
        }
        const int gw3 = NH * nin + 2 * NH + NH * NH, gb3 = gw3 + NOUT * NH;
        if (t == 0) {
          const int k = mt * 16 + g;
          gp[gw3 + k] += acc[0];
          gp[gw3 + NH + k] += acc[1];
          gp[gw3 + k + 8] += acc[2];
          gp[gw3 + NH + k + 8] += acc[3];
          if (warp == 0 && g == 0) {
            gp[gb3] += accb[0];
            gp[gb3 + 1] += accb[1];
          }
        }
      }
      __syncthreads();
    }

    /* every CTA's partial gradient is complete and visible cluster-wide */
    cluster.sync();
    /* the next step's first tile: its global loads overlap the reduction's remote loads */
    prefetched = step + 1 < total_steps && my0 < my1;
    if (prefetched) gather(step + 1, my0);
    const int tstep = step + 1;
    const float lr = tp.lr * (epoch < tp.epochs / 2 ? 1.f
                                                     : 0.1f + 0.9f * (float)(tp.epochs - epoch) / (tp.epochs / 2 + 1));
    const float c1 = 1.f - powf(b1, (float)tstep), c2 = 1.f - powf(b2, (float)tstep);
    for (int i = lo + tid; i < hi; i += blockDim.x) {
      float part[CSIZE];
#pragma unroll
      for (int q = 0; q < CSIZE; ++q) part[q] = cluster.map_shared_rank(gp, q)[i]; /* all loads in flight */
      float gs = 0.f;
#pragma unroll
      for (int q = 0; q < CSIZE; ++q) gs += part[q];
      const ParamSlot s = param_slot(i, nin, nh, ldx);
      if (tp.grad_only) {
        if (s.ext >= 0) tp.grad[s.ext] = gs;
        continue;
      }
      if (s.ext < 0) continue; /* padded unit: stays zero */
      const int k = i - lo;
      const float mv = b1 * om[k] + (1.f - b1) * gs;
      const float vv = b2 * ov[k] + (1.f - b2) * gs * gs;
      om[k] = mv;
      ov[k] = vv;
      const float w = ow[k] - lr * (mv / c1) / (sqrtf(vv / c2) + eps);
      ow[k] = w;
      const __nv_bfloat16 wb = __float2bfloat16(w);
      void* base = s.arr == 0 ? (void*)net.w1 : s.arr == 1 ? (void*)net.w2 : s.arr == 2 ? (void*)net.w3
                 : s.arr == 3 ? (void*)net.b1 : s.arr == 4 ? (void*)net.b2 : (void*)net.b3;
      if (s.kind == 0) {
#pragma unroll
        for (int q = 0; q < CSIZE; ++q) cluster.map_shared_rank((__nv_bfloat16*)base, q)[s.off] = wb;
      } else {
#pragma unroll
        for (int q = 0; q < CSIZE; ++q) cluster.map_shared_rank((float*)base, q)[s.off] = __bfloat162float(wb);
      }
    }
    /* loss of the first and the last epoch */
    if (tid == 0 && (tp.grad_only || sie == tp.steps_per_epoch - 1)) {
      if (epoch == 0) atomicAdd(&tp.loss[0], *sloss);
      if (epoch == tp.epochs - 1 || tp.grad_only) atomicAdd(&tp.loss[1], *sloss);
    }
    if (tid == 0 && (tp.grad_only || sie == tp.steps_per_epoch - 1)) *sloss = 0.f;
    /* the new weights are in place everywhere; the partial gradients may be overwritten */
    cluster.sync();
  }
  if (!tp.grad_only) {
    for (int i = lo + tid; i < hi; i += blockDim.x) {
      const ParamSlot s = param_slot(i, nin, nh, ldx);
      if (s.ext < 0) continue;
      tp.master[s.ext] = ow[i - lo];
      tp.wbf[s.ext] = __float2bfloat16(ow[i - lo]);
    }
  }
}

/* Launch the training cluster: 16 CTAs where the device allows clusters of
 * that size, else 8. */
template <int CSIZE>
static void (*train_fn(int kin))(TrainParams) {
  return kin == 1 ? mlp_train<1, CSIZE> : kin == 2 ? mlp_train<2, CSIZE> : mlp_train<3, CSIZE>;
}

static int launch_train(ode_handle* h, const TrainParams& tp, cudaStream_t s, int* csize_out) {
  const int kin = kin_steps(tp.nin);
  cudaError_t e = cudaSuccess;
  for (int csize : {16, 8}) {
    void (*fn)(TrainParams) = csize == 16 ? train_fn<16>(kin) : train_fn<8>(kin);
    const TrainLayout L(tp.nin, csize);
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total);
    if (e != cudaSuccess) return cuda_fail(h, e, "training kernel attributes");
    if (csize > 8) {
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      if (e != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
    }
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = csize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(csize, 1, 1);
    cfg.blockDim = dim3(TW * 32, 1, 1);
    cfg.dynamicSmemBytes = L.total;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    e = cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg);
    if (e != cudaSuccess || clusters < 1) {
      cudaGetLastError();
      continue;
    }
    e = cudaLaunchKernelEx(&cfg, fn, tp);
    if (e != cudaSuccess) return cuda_fail(h, e, "training kernel launch");
    if (csize_out) *csize_out = csize;
    return ODE_OK;
  }
  return fail(h, ODE_ECUDA, "no thread-block cluster of 8 CTAs fits the training kernel on this device");
}

/* ------------------------------------------------------------------ inference */
/* 16 trajectories per warp and pass: features gathered from the SoA inputs
 * (p rows then u0 rows), standardised, rounded to bf16 into the warp's tile,
 * then the training kernel's forward pass; outputs de-standardised. */
template <int KIN>
__global__ void __launch_bounds__(PW * 32) mlp_predict(long long n, int nin, int nh, int nparams,
                                                       const double* __restrict__ p,
                                                       const double* __restrict__ u0,
                                                       const __nv_bfloat16* __restrict__ W,
                                                       const float* __restrict__ nrm, float* __restrict__ log_att,
                                                       float* __restrict__ log_dt) {
  constexpr int LDX = KIN * 16 + 8;
  __shared__ __align__(16) __nv_bfloat16 w1[NH * LDX];
  __shared__ __align__(16) __nv_bfloat16 w2[NH * LDH];
  __shared__ __align__(16) __nv_bfloat16 w3[W3ROWS * LDH];
  __shared__ float b1[NH], b2[NH], b3[W3ROWS];
  __shared__ __align__(16) __nv_bfloat16 xs[PW][16 * LDX];
  const Net net{w1, w2, w3, b1, b2, b3, LDX};
  load_net(net, nin, nh, [&](int i) { return __bfloat162float(W[i]); });
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  __nv_bfloat16* x = xs[warp];
  const long long tiles = (n + 15) / 16;
  for (long long tile = (long long)blockIdx.x * PW + warp; tile < tiles; tile += (long long)gridDim.x * PW) {
    const long long base = tile * 16;
    for (int i = lane; i < 16 * (LDX - 8); i += 32) {
      const int s = i / (LDX - 8), f = i % (LDX - 8);
      const long long tr = base + s;
      float v = 0.f;
      if (tr < n && f < nin) {
        const double raw = f < nparams ? p[(long long)f * n + tr] : u0[(long long)(f - nparams) * n + tr];
        v = ((float)raw - nrm[f]) / nrm[MAXIN + f];
      }
      x[s * LDX + f] = __float2bfloat16(v);
    }
    __syncwarp();
    float out[4];
    uint32_t m1, m2;
    warp_forward<KIN, false>(net, x, 0, out, nullptr, nullptr, m1, m2);
    if (t == 0) {
      if (base + g < n) {
        log_att[base + g] = out[0] * nrm[2 * MAXIN + 2] + nrm[2 * MAXIN];
        log_dt[base + g] = out[1] * nrm[2 * MAXIN + 3] + nrm[2 * MAXIN + 1];
      }
      if (base + g + 8 < n) {
        log_att[base + g + 8] = out[2] * nrm[2 * MAXIN + 2] + nrm[2 * MAXIN];
        log_dt[base + g + 8] = out[3] * nrm[2 * MAXIN + 3] + nrm[2 * MAXIN + 1];
      }
    }
    __syncwarp();
  }
}

/* ------------------------------------------------------------------ binning (counting sort, longest first) */
__device__ __forceinline__ int cost_bin(float v, float lo, float inv_w) {
  int b = (int)((v - lo) * inv_w);
  b = b < 0 ? 0 : (b >= NBINS ? NBINS - 1 : b);
  return NBINS - 1 - b; /* descending cost */
}

__global__ void bin_histogram(long long n, const float* __restrict__ key, float lo, float inv_w,
                              unsigned* __restrict__ count) {
  __shared__ unsigned hcount[NBINS];
  for (int i = threadIdx.x; i < NBINS; i += blockDim.x) hcount[i] = 0;
  __syncthreads();
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    atomicAdd(&hcount[cost_bin(key[i], lo, inv_w)], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < NBINS; i += blockDim.x)
    if (hcount[i]) atomicAdd(&count[i], hcount[i]);
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
  const long long tiles = (n + 15) / 16;
  const unsigned grid = (unsigned)std::min<long long>(4LL * h->nsm, (tiles + PW - 1) / PW);
  const int kin = kin_steps(m->nin);
  if (kin == 1)
    mlp_predict<1><<<grid, PW * 32, 0, s>>>(n, m->nin, m->nh, m->nparams, kp.p, kp.u0, m->d_w, m->d_norm, log_att,
                                            log_dt);
  else if (kin == 2)
    mlp_predict<2><<<grid, PW * 32, 0, s>>>(n, m->nin, m->nh, m->nparams, kp.p, kp.u0, m->d_w, m->d_norm, log_att,
                                            log_dt);
  else
    mlp_predict<3><<<grid, PW * 32, 0, s>>>(n, m->nin, m->nh, m->nparams, kp.p, kp.u0, m->d_w, m->d_norm, log_att,
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

/* Fit on host-resident features/targets (already standardised): one launch
 * of the training cluster for all epochs. */
static int train(ode_handle* h, Model* m, const std::vector<float>& X, const std::vector<float>& Y, int nb,
                 const ode_learn_opts& o, float* loss_first, float* loss_last, double* kernel_ms, int* ctas) {
  int rc;
  const size_t np = param_count(m->nin, m->nh);
  m->nparam = np;
  float* dX = (float*)buf(h, "learn_X", X.size() * 4, &rc);
  if (!dX) return rc;
  float* dY = (float*)buf(h, "learn_Y", Y.size() * 4, &rc);
  if (!dY) return rc;
  float* dL = (float*)buf(h, "learn_loss", 2 * 4, &rc);
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
  cudaMemcpyAsync(m->d_master, w.data(), np * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dX, X.data(), X.size() * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dY, Y.data(), Y.size() * 4, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dL, 0, 2 * 4, s);
  TrainParams tp;
  tp.X = dX;
  tp.Y = dY;
  tp.nb = nb;
  tp.nin = m->nin;
  tp.nh = m->nh;
  tp.batch = std::max(32, std::min(o.batch, nb));
  tp.epochs = std::max(1, o.epochs);
  tp.steps_per_epoch = std::max(1, nb / tp.batch);
  tp.lr = o.lr;
  const uint64_t sk = o.seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  tp.seed_lo = (uint32_t)sk;
  tp.seed_hi = (uint32_t)(sk >> 32);
  tp.grad_only = 0;
  tp.master = m->d_master;
  tp.wbf = m->d_w;
  tp.grad = nullptr;
  tp.loss = dL;
  int csize = 0;
  cudaError_t ee = cudaEventRecord(h->ev0, s);
  if (ee != cudaSuccess) return cuda_fail(h, ee, "event");
  rc = launch_train(h, tp, s, &csize);
  if (rc != ODE_OK) return rc;
  ee = cudaEventRecord(h->ev1, s);
  if (ee != cudaSuccess) return cuda_fail(h, ee, "event");
  float l[2] = {0.f, 0.f};
  cudaMemcpyAsync(l, dL, sizeof l, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "training");
  *loss_first = l[0] / tp.steps_per_epoch;
  *loss_last = l[1] / tp.steps_per_epoch;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  *kernel_ms = ms;
  *ctas = csize;
  return ODE_OK;
}

}  // namespace gbode

using namespace gbode;

extern "C" {

void ode_learn_default_opts(ode_learn_opts* o) {
  if (!o) return;
  o->hidden = 64;
  o->epochs = 30;
  o->batch = 1024;
  o->lr = 5e-3f;
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
  if (a->n < 64) return fail(h, ODE_EINVAL, "training ensemble too small");
  cudaSetDevice(h->device);
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t n = a->n;
  std::vector<int32_t> nacc(n), nrej(n);
  std::vector<double> dtf(n);
  std::vector<int8_t> ret(n);
  /* the training solve records counts only: the persistent schedule runs the
   * plain kernel's arithmetic (identical counts) with idle lanes refilled */
  ode_solve_args ta = *a;
  ta.schedule = ODE_SCHED_PERSISTENT;
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
  if (nb < 64) return fail(h, ODE_EINVAL, "too few finished training trajectories");
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
  double kms = 0;
  int ctas = 0;
  rc = train(h, m, Xs, Ys, nb, o, &lf, &ll, &kms, &ctas);
  if (rc != ODE_OK) return rc;
  const auto t2 = std::chrono::steady_clock::now();
  if (rep) {
    rep->loss_first = lf;
    rep->loss_last = ll;
    rep->train_solve_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    rep->train_fit_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
    rep->train_kernel_ms = kms;
    rep->train_ctas = ctas;
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

/* The training kernel's forward and backward pass on one batch (the
 * training cluster with a single step over the samples in order and no
 * update), for verification against the CPU restatement: params in the flat
 * layout (rounded to bf16 on use, as training uses them), x [batch][nin],
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
  float* dG = (float*)buf(h, "gc_G", np * 4, &rc);
  if (!dG) return rc;
  float* dP = (float*)buf(h, "gc_P", np * 4, &rc);
  if (!dP) return rc;
  float* dL = (float*)buf(h, "gc_L", 2 * 4, &rc);
  if (!dL) return rc;
  cudaStream_t s = h->stream;
  cudaMemcpyAsync(dX, x, (size_t)batch * nin * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dY, y, (size_t)batch * NOUT * 4, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dP, params, np * 4, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dG, 0, np * 4, s);
  cudaMemsetAsync(dL, 0, 2 * 4, s);
  TrainParams tp;
  std::memset(&tp, 0, sizeof tp);
  tp.X = dX;
  tp.Y = dY;
  tp.nb = (int)batch;
  tp.nin = nin;
  tp.nh = nh;
  tp.batch = (int)batch;
  tp.epochs = 1;
  tp.steps_per_epoch = 1;
  tp.grad_only = 1;
  tp.master = dP;
  tp.grad = dG;
  tp.loss = dL;
  rc = launch_train(h, tp, s, nullptr);
  if (rc != ODE_OK) return rc;
  float l[2];
  cudaMemcpyAsync(grad, dG, np * 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(l, dL, sizeof l, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(h, e, "gradcheck");
  *loss = l[0];
  return ODE_OK;
}

}  // extern "C"
