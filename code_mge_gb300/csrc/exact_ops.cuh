// exact_ops.cuh -- exact binary64 operations moved off the FP64 pipe.
//
// GB300 issues FP64 at 2 thread-operations per SM per cycle, and the stage
// kernels are bound by that rate.  Some of their operations have results
// that integer instructions produce bit for bit: scaling by 2 or 1/2 is an
// exponent increment or decrement for normal numbers, and the order of
// non-negative doubles is the order of their bit patterns.  The functions
// below return exactly what the IEEE-754 operation they name returns (round
// to nearest even), and fall back to that operation, out of line, for the
// operands the integer form does not cover (subnormal, overflow, inf, NaN).
// For float they are the plain operations: the FP32 pipe is not the limit.
#pragma once
#include <cuda_runtime.h>

namespace mge {

__device__ __noinline__ inline double mul2_fp64(double x) { return x * 2.0; }
__device__ __noinline__ inline double mulhalf_fp64(double x) { return x * 0.5; }

// x * 2
__device__ __forceinline__ double mul2(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const unsigned e = (unsigned)hi & 0x7ff00000u;
  // biased exponent 1..0x7fd: 2x is normal and finite
  if (e - 0x00100000u < 0x7fd00000u) return __hiloint2double(hi + 0x00100000, lo);
  if ((((unsigned)hi & 0x7fffffffu) | (unsigned)lo) == 0u) return x;  // +-0
  return mul2_fp64(x);
}
__device__ __forceinline__ float mul2(float x) { return x * 2.0f; }

// x * 0.5
__device__ __forceinline__ double mulhalf(double x) {
  const int hi = __double2hiint(x), lo = __double2loint(x);
  const unsigned e = (unsigned)hi & 0x7ff00000u;
  // biased exponent 2..0x7fe: x/2 is normal
  if (e - 0x00200000u < 0x7fd00000u) return __hiloint2double(hi - 0x00100000, lo);
  if ((((unsigned)hi & 0x7fffffffu) | (unsigned)lo) == 0u) return x;  // +-0
  return mulhalf_fp64(x);
}
__device__ __forceinline__ float mulhalf(float x) { return x * 0.5f; }

// a > b ? a : b for a, b >= +0 (not NaN, not -0): the bit patterns order
// like the values
__device__ __forceinline__ double max_nonneg(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return x > y ? a : b;
}
__device__ __forceinline__ float max_nonneg(float a, float b) { return a > b ? a : b; }

// a > b for a, b >= +0 (not NaN, not -0)
__device__ __forceinline__ bool gt_nonneg(double a, double b) {
  return __double_as_longlong(a) > __double_as_longlong(b);
}
__device__ __forceinline__ bool gt_nonneg(float a, float b) { return a > b; }

}  // namespace mge
