// Checks the device build of mge::soft::mul, add, sub and div
// (code_mge_gb300/csrc/soft_fp64.cuh) bit for bit against the FP64
// hardware (__dmul_rn, __dadd_rn, __dsub_rn, __ddiv_rn) on 2^26 operand pairs
// of each of eight distributions: any bit patterns, moderate exponents with
// gaps up to 70, near cancellation, short significands (exact products,
// ties), operands near underflow and overflow, the magnitudes of a flow
// solver, divisors with a significand at or next to 1 or 2, and quotients
// that are exact or a few ulps from exact.  Prints
// "mismatches <n> " and exits 1 on any mismatch.
#include <cstdio>
#include <cstdint>

#include "soft_fp64.cuh"

using namespace mge::soft;

__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64 finaliser
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ double with_exp(uint64_t r, uint64_t e) { return from_bits((r & (kFrac | kSign)) | (e << 52)); }

__device__ void operands(int kind, uint64_t i, double& a, double& b) {
  const uint64_t r1 = mix(2 * i + 1), r2 = mix(2 * i + 2), r3 = mix(i ^ 0x5bd1e995ull);
  switch (kind) {
    case 0: a = from_bits(r1); b = from_bits(r2); break;
    case 1: a = with_exp(r1, 900 + r3 % 200); b = from_bits(bits(with_exp(r2, 900 + (r3 >> 8) % 200)) - ((r3 >> 20) % 71 << 52)); break;
    case 2: a = with_exp(r1, 1 + r3 % 2046); b = from_bits((bits(a) ^ kSign) + (r2 % 17) - 8); break;
    case 3: a = from_bits(bits(with_exp(r1, 1000 + r3 % 50)) & ~0xFFFFFFFFFFull); b = from_bits(bits(with_exp(r2, 1000 + (r3 >> 9) % 50)) & ~0xFFFFFFFull); break;
    case 4: a = with_exp(r1, 1 + r3 % 600); b = with_exp(r2, 1 + (r3 >> 12) % 600); if (r3 & 1) { a = with_exp(r1, 1500 + r3 % 547); b = with_exp(r2, 1000 + (r3 >> 12) % 100); } break;
    case 5: a = with_exp(r1, 1013 + r3 % 21); b = with_exp(r2, 1003 + (r3 >> 7) % 31); break;
    case 6: a = with_exp(r1, 1000 + r3 % 40); b = from_bits(((1000 + (r3 >> 9) % 40) << 52) | ((r2 & 1) ? (r2 >> 1) % 4096 : kFrac - (r2 >> 1) % 4096)); break;
    default: b = with_exp(r1, 1000 + r3 % 40); a = from_bits(bits(__dmul_rn(b, from_bits(bits(with_exp(r2, 1015 + (r3 >> 9) % 16)) & ~0xFFFFFFFFFull))) + (r3 >> 20) % 5 - 2); break;
  }
}

__device__ bool same(double x, double y) { return (isnan(x) && isnan(y)) || bits(x) == bits(y); }

__global__ void k_check(int kind, uint64_t n, unsigned long long* bad, unsigned long long* first) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double a, b;
    operands(kind, i, a, b);
    const bool ok = same(mul(a, b), __dmul_rn(a, b)) && same(add(a, b), __dadd_rn(a, b)) &&
                    same(sub(a, b), __dsub_rn(a, b)) && same(div(a, b), __ddiv_rn(a, b));
    if (!ok) {
      atomicAdd(bad, 1ull);
      if (atomicCAS(first + 2, 0ull, 1ull) == 0ull) {
        first[0] = bits(a);
        first[1] = bits(b);
      }
    }
  }
}

int main() {
  unsigned long long *bad, *first;
  cudaMalloc(&bad, 8);
  cudaMalloc(&first, 24);
  unsigned long long total = 0;
  for (int kind = 0; kind < 8; kind++) {
    cudaMemset(bad, 0, 8);
    cudaMemset(first, 0, 24);
    k_check<<<152 * 8, 256>>>(kind, 1ull << 26, bad, first);
    unsigned long long h = 0, f[3] = {0, 0, 0};
    cudaMemcpy(&h, bad, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(f, first, 24, cudaMemcpyDeviceToHost);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      printf("cuda error %s\n", cudaGetErrorString(e));
      return 2;
    }
    if (h) printf("kind %d: %llu mismatches, first a=%016llx b=%016llx\n", kind, h, f[0], f[1]);
    total += h;
  }
  printf("pairs %llu mismatches %llu \n", 8ull << 26, total);
  return total ? 1 : 0;
}
