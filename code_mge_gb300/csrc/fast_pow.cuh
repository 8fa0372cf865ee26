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
// The exponents the reference actually uses are doubles: gamma = 7/5 + dg and
// 1/(gamma-1) = 5/2 + dm with dg = -8.9e-17 and dm = 4.4e-16.  x^(e+d) =
// x^e * (1 + d*ln x + ...), and d*ln x is a few 1e-16 at most, so the factor
// is applied as y + y*(d*ln x) with ln x to single precision.  Over
// x in [1/10, 10] the result stays within 3 ulp of the correctly rounded
// pow(x, e+d); tests/test_gpu_exact_ops.py allows 4 against CUDA's pow.
// Outside [1e-30, 1e30] the functions return pow itself.
#pragma once
#include <cuda_runtime.h>

namespace mge {

// x^(5/2 + d)
__device__ __forceinline__ double pow_5_2(double x, double d) {
  if (!(x > 1e-30 && x < 1e30)) return pow(x, 2.5 + d);
  const double y = (x * x) * sqrt(x);
  return y + y * (d * (double)logf((float)x));
}

// x^(7/5 + d)
__device__ __forceinline__ double pow_7_5(double x, double d) {
  if (!(x > 1e-30 && x < 1e30)) return pow(x, 1.4 + d);
  const double a = x * x;
  double z = (double)powf((float)x, 0.4f);  // x^(2/5) to single precision
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const double z2 = z * z;
    z = (4.0 * z + a / (z2 * z2)) / 5.0;
  }
  const double y = x * z;
  return y + y * (d * (double)logf((float)x));
}

}  // namespace mge
