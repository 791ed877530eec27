/* Throughput probes for the arithmetic pipes the solver kernels use: the
 * benchmark's roofline denominators (an FP64-bound solver is measured against
 * the FP64 pipe peak, which the measured-peaks file does not carry).
 *
 * Measurement aid of bench.py, built by __graft_entry__.build() into
 * _build/libbench_probe.so; not part of the solver library.  Each probe runs
 * a grid of 8 independent dependency chains per thread, two full waves of
 * resident blocks per SM, and times it with CUDA events after a warm-up
 * launch.
 */
#include <cuda_runtime.h>

#include <cstdio>

namespace {

enum {
  OP_DFMA = 0,    /* d = fma(d, a, b)                 2 flops */
  OP_DADD = 1,    /* d = d + a                        1 flop */
  OP_FFMA = 2,    /* f = fmaf(f, a, b)                2 flops */
  OP_DDIV = 3,    /* d = a / d                        IEEE double division */
  OP_DSQRT = 4,   /* d = sqrt(d) + b                  IEEE double square root + add */
  OP_DMAX = 5,    /* d = fmax(d, a) - b               double max + add */
  OP_FDIV = 6,    /* f = fa / f                       IEEE float division */
  OP_NOPS
};

template <int OP>
__global__ void __launch_bounds__(256) probe_kernel(double* out, int iters, double a, double b) {
  double d[8];
  float f[8];
  const float fa = (float)a, fb = (float)b;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    d[j] = 1.0 + 1e-3 * (threadIdx.x + j);
    f[j] = 1.0f + 1e-3f * (threadIdx.x + j);
  }
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if (OP == OP_DFMA) d[j] = __fma_rn(d[j], a, b);
        if (OP == OP_DADD) d[j] = __dadd_rn(d[j], a);
        if (OP == OP_FFMA) f[j] = __fmaf_rn(f[j], fa, fb);
        if (OP == OP_DDIV) d[j] = __ddiv_rn(a, d[j]);
        if (OP == OP_DSQRT) d[j] = __dadd_rn(__dsqrt_rn(d[j]), b);
        if (OP == OP_DMAX) d[j] = __dadd_rn(fmax(d[j], a), b);
        if (OP == OP_FDIV) f[j] = __fdiv_rn(fa, f[j]);
      }
    }
  }
  double s = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += d[j] + (double)f[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <int OP>
float time_op(double* out, int blocks, int iters) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  /* a, b chosen so chains neither overflow nor denormalise */
  const double a = (OP == OP_DFMA || OP == OP_FFMA) ? 0.999999 : (OP == OP_DADD ? 1e-9 : 1.0);
  const double b = (OP == OP_DFMA || OP == OP_FFMA) ? 1e-6 : (OP == OP_DSQRT ? 0.5 : (OP == OP_DMAX ? 0.0 : 0.0));
  probe_kernel<OP><<<blocks, 256>>>(out, iters / 8 + 1, a, b);
  cudaEventRecord(e0);
  probe_kernel<OP><<<blocks, 256>>>(out, iters, a, b);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

}  // namespace

extern "C" {

/* Lane operations per second for each probe (index = OP_*), and the device
 * time of each timed launch in ms.  `iters` sets the loop length (each
 * iteration issues 32 operations per thread).  Returns 0 on success. */
int probe_op_rates(int device, int iters, double* ops_per_s, double* ms_out, int nops) {
  if (cudaSetDevice(device) != cudaSuccess) return -2;
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, probe_kernel<OP_DFMA>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  const int blocks = 2 * nsm * per_sm;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * 256 * sizeof(double)) != cudaSuccess) return -3;
  float ms[OP_NOPS];
  ms[OP_DFMA] = time_op<OP_DFMA>(out, blocks, iters);
  ms[OP_DADD] = time_op<OP_DADD>(out, blocks, iters);
  ms[OP_FFMA] = time_op<OP_FFMA>(out, blocks, iters * 16);
  ms[OP_DDIV] = time_op<OP_DDIV>(out, blocks, iters / 4);
  ms[OP_DSQRT] = time_op<OP_DSQRT>(out, blocks, iters / 4);
  ms[OP_DMAX] = time_op<OP_DMAX>(out, blocks, iters);
  ms[OP_FDIV] = time_op<OP_FDIV>(out, blocks, iters);
  const double lanes = (double)blocks * 256.0 * 32.0;
  const int it[OP_NOPS] = {iters, iters, iters * 16, iters / 4, iters / 4, iters, iters};
  for (int k = 0; k < nops && k < OP_NOPS; ++k) {
    ops_per_s[k] = lanes * it[k] / (ms[k] * 1e-3);
    if (ms_out) ms_out[k] = ms[k];
  }
  cudaFree(out);
  return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* FP64 fused multiply-add peak in TFLOP/s (2 flops per lane FMA). */
int probe_fp64_peak(int device, int iters, double* tflops) {
  double r[1], ms[1];
  int rc = probe_op_rates(device, iters, r, ms, 1);
  if (rc) return rc;
  *tflops = r[0] * 2.0 / 1e12;
  return 0;
}
}
