// Checks the integer-pipe binary64 operations of exact_ops.cuh against the
// FP64 operations they replace, bit for bit, on random bit patterns and on
// the special operands (zeros, subnormals, binade edges, inf, NaN).
// Prints "mismatches <n> checked <m>"; exit status 0 when n == 0.
#include <cstdio>
#include <cstdint>
#include "../code_mge_gb300/csrc/exact_ops.cuh"

using namespace mge;

__device__ unsigned long long mix(unsigned long long x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ bool same(double a, double b) {
  if (a != a && b != b) return true;  // both NaN
  return __double_as_longlong(a) == __double_as_longlong(b);
}

__global__ void check(long long n, unsigned long long* bad, unsigned long long* first) {
  const unsigned long long specials[] = {
      0x0000000000000000ull, 0x8000000000000000ull, 0x0000000000000001ull, 0x8000000000000001ull,
      0x000fffffffffffffull, 0x0010000000000000ull, 0x0010000000000001ull, 0x001fffffffffffffull,
      0x0020000000000000ull, 0x0008000000000001ull, 0x0000000000000003ull, 0x7fdfffffffffffffull,
      0x7fe0000000000000ull, 0x7fefffffffffffffull, 0x7ff0000000000000ull, 0xfff0000000000000ull,
      0x7ff8000000000000ull, 0x3ff0000000000000ull, 0xbff0000000000000ull, 0x0017ffffffffffffull};
  const int ns = sizeof(specials) / sizeof(specials[0]);
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    unsigned long long r = mix((unsigned long long)t);
    unsigned long long bits;
    if (t < ns) {
      bits = specials[t];
    } else {
      // bias towards the edges: small, large and normal exponents
      const int kind = (int)(r & 3);
      unsigned long long m = mix(r) & 0x800fffffffffffffull;
      unsigned long long e = (r >> 8) & 0x7ff;
      if (kind == 0) e = (r >> 8) & 3;
      if (kind == 1) e = 0x7fc + ((r >> 8) & 3);
      bits = m | (e << 52);
    }
    const double x = __longlong_as_double((long long)bits);
    int fail = 0;
    if (!same(mul2(x), x * 2.0)) fail |= 1;
    if (!same(mulhalf(x), x * 0.5)) fail |= 2;
    const double a = fabs(x), b = fabs(__longlong_as_double((long long)(mix(r + 1) & 0x7fefffffffffffffull)));
    if (a == a && bits != 0x8000000000000000ull) {
      if (!same(max_nonneg(a, b), a > b ? a : b)) fail |= 4;
      if (gt_nonneg(a, b) != (a > b)) fail |= 8;
      if (!same(max_nonneg(a, a), a)) fail |= 16;
    }
    if (fail) {
      if (atomicAdd(bad, 1ull) == 0ull) *first = bits | ((unsigned long long)fail << 0);
    }
  }
}

int main() {
  unsigned long long *bad, *first;
  cudaMallocManaged(&bad, 8);
  cudaMallocManaged(&first, 8);
  *bad = 0;
  *first = 0;
  const long long n = 1LL << 26;
  check<<<1216, 256>>>(n, bad, first);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    printf("cuda error %s\n", cudaGetErrorString(e));
    return 2;
  }
  printf("mismatches %llu checked %lld first %016llx\n", *bad, n, *first);
  return *bad == 0 ? 0 : 1;
}
