// fast_pow.cuh -- the two powers of the far-field boundary for gamma = 1.4,
// with short dependency chains.
//
// bc_far.f90 forms rho = (s*c^2/gamma)**(1/(gamma-1)) and s = rho**gamma / p
// for every far-field ghost cell.  A general FP64 pow is a long chain of
// dependent operations (about 6,000 cycles on GB300), and these chains are the
// latency of the boundary passes on the coarse multigrid levels.  For
// gamma = 1.4 the exponents are 5/2 and 7/5:
//   x^(5/2) = x^2 * sqrt(x)                       (three roundings)
//   x^(7/5) = x * z,  z = (x^2)^(1/5)             (Newton's method for the
//             fifth root, z <- (4z + x^2/z^4)/5, two steps from an FP32 seed)
// Both stay within 2 ulp of the correctly rounded x^(5/2) and x^(7/5).  The
// double exponents of the reference, gamma = 1.4 - 8.9e-17 and
// 1/(gamma-1) = 2.5 + 5.6e-16, move the power by a relative e*|ln x|,
// under 2 ulp for x in [1/3, 3]; in the far field x stays near 1 (s*c^2/gamma
// is 1 in the free stream).  tests/test_gpu_exact_ops.py compares both with
// CUDA's pow at those exponents.  Outside [1e-30, 1e30] they return pow itself.
#pragma once
#include <cuda_runtime.h>

namespace mge {

__device__ __forceinline__ double pow_5_2(double x) {
  if (!(x > 1e-30 && x < 1e30)) return pow(x, 2.5);
  return (x * x) * sqrt(x);
}

__device__ __forceinline__ double pow_7_5(double x) {
  if (!(x > 1e-30 && x < 1e30)) return pow(x, 1.4);
  const double a = x * x;
  double z = (double)powf((float)x, 0.4f);  // x^(2/5) to single precision
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const double z2 = z * z;
    z = (4.0 * z + a / (z2 * z2)) / 5.0;
  }
  return x * z;
}

}  // namespace mge
