// Checks the short powers of fast_pow.cuh against CUDA's pow at the
// exponents the far-field boundary uses for gamma = 1.4: the largest
// difference in units in the last place over x log-uniform in [1/10, 10].
// Prints "maxulp <p52> <p75> checked <n>"; exit status 0 when both are <= 4.
#include <cstdio>
#include "../code_mge_gb300/csrc/fast_pow.cuh"

using namespace mge;

__device__ double ulps(double a, double b) {
  const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
  return (double)(x > y ? x - y : y - x);
}

__global__ void check(long long n, unsigned long long* worst) {
  const double gamma = 1.4, gm = 1.0 / (gamma - 1.0);
  const double dg = fma(gamma, 5.0, -7.0) / 5.0, dm = gm - 2.5;
  double m1 = 0.0, m2 = 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    const double u = ((double)t + 0.5) / (double)n;   // [0, 1)
    const double x = exp((u - 0.5) * 2.0 * log(10.0));  // [1/10, 10)
    m1 = fmax(m1, ulps(pow_5_2(x, dm), pow(x, gm)));
    m2 = fmax(m2, ulps(pow_7_5(x, dg), pow(x, gamma)));
  }
  atomicMax(&worst[0], (unsigned long long)m1);
  atomicMax(&worst[1], (unsigned long long)m2);
}

int main() {
  unsigned long long* w;
  cudaMallocManaged(&w, 2 * sizeof(unsigned long long));
  w[0] = w[1] = 0;
  const long long n = 1LL << 24;
  check<<<1216, 256>>>(n, w);
  if (cudaDeviceSynchronize() != cudaSuccess) {
    printf("cuda error\n");
    return 2;
  }
  printf("maxulp %llu %llu checked %lld\n", w[0], w[1], n);
  return (w[0] <= 4 && w[1] <= 4) ? 0 : 1;
}
