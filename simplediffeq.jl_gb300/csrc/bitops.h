/* Exact double-precision comparisons with integer operations.  On this GPU
 * a double comparison issues on the FP64 pipe (one warp instruction per 64
 * cycles per SM sub-partition), the pipe the FP64 solver kernels are bound
 * by; integer operations issue elsewhere.  Every function returns exactly
 * what the IEEE comparison it replaces returns (false with a NaN operand,
 * -0 == +0).
 *
 * Compiled by nvcc / NVRTC for the kernels and by a host C++ compiler for
 * the CPU test that checks them against the IEEE operations. */
#pragma once

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define GBODE_BO __device__ __forceinline__
namespace gbode {
GBODE_BO long long bo_bits(double x) { return __double_as_longlong(x); }
}  // namespace gbode
#else
#include <cstring>
#define GBODE_BO static inline
namespace gbode {
GBODE_BO long long bo_bits(double x) { long long b; std::memcpy(&b, &x, 8); return b; }
}  // namespace gbode
#endif

namespace gbode {

/* the magnitude bits are above those of infinity */
GBODE_BO bool bo_isnan(double x) { return (bo_bits(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }

/* order key of a non-NaN double: the bits for x >= 0, minus the magnitude
 * bits for x < 0, so that -0 and +0 share the key 0 */
GBODE_BO long long bo_key(double x) {
  const long long b = bo_bits(x);
  return b >= 0 ? b : -(b & 0x7fffffffffffffffLL);
}

/* x < y and x <= y, as IEEE */
GBODE_BO bool bo_lt(double x, double y) { return !bo_isnan(x) && !bo_isnan(y) && bo_key(x) < bo_key(y); }
GBODE_BO bool bo_le(double x, double y) { return !bo_isnan(x) && !bo_isnan(y) && bo_key(x) <= bo_key(y); }

}  // namespace gbode
