// Checks mge::soft::mul, add, sub and div (code_mge_gb300/csrc/soft_fp64.cuh)
// bit for bit against the host's binary64 arithmetic (round to nearest
// even, no contraction): edge values, then random operands drawn so that
// every path of the algorithms is taken (all exponent gaps, cancellation,
// carries, ties, under- and overflow).  Prints the number of cases and of
// mismatches; exit status 1 on any mismatch.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "soft_fp64.cuh"

using namespace mge::soft;

static uint64_t rng = 0x9E3779B97F4A7C15ull;
static uint64_t next() {  // xorshift64*
  rng ^= rng >> 12;
  rng ^= rng << 25;
  rng ^= rng >> 27;
  return rng * 0x2545F4914F6CDD1Dull;
}

static long long cases = 0, bad = 0;

static bool same(double x, double y) {
  if (isnan(x) || isnan(y)) return isnan(x) && isnan(y);
  return bits(x) == bits(y);
}

static void check(double a, double b) {
  volatile double va = a, vb = b;
  const double pm = va * vb, pa = va + vb, ps = va - vb, pd = va / vb;
  const double qm = mul(a, b), qa = add(a, b), qs = sub(a, b), qd = div(a, b);
  cases += 4;
  if (!same(pm, qm) || !same(pa, qa) || !same(ps, qs) || !same(pd, qd)) {
    if (bad < 10)
      printf("mismatch a=%a b=%a  mul %a/%a  add %a/%a  sub %a/%a  div %a/%a\n", a, b, pm, qm, pa, qa, ps, qs, pd, qd);
    bad++;
  }
}

static double rnd_exp(int lo, int hi) {  // random significand, biased exponent in [lo, hi]
  const uint64_t e = (uint64_t)(lo + (int)(next() % (uint64_t)(hi - lo + 1)));
  return from_bits((next() & (kFrac | kSign)) | (e << 52));
}

int main(int argc, char** argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 2000000;
  const double edge[] = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 3.0, 1.5, INFINITY, -INFINITY, NAN,
                         4.9406564584124654e-324, 2.2250738585072014e-308, 2.2250738585072009e-308,
                         1.7976931348623157e308, -1.7976931348623157e308, 1.0000000000000002, 0.99999999999999989,
                         1e-300, 1e300, 3.0e-154, 1.5e154, 6.0e-309};
  for (double a : edge)
    for (double b : edge) check(a, b);
  for (long long q = 0; q < n; q++) {
    const int kind = (int)(q % 10);
    double a, b;
    if (kind == 0) {  // any bit patterns
      a = from_bits(next());
      b = from_bits(next());
    } else if (kind == 1) {  // moderate exponents, any gap up to 70
      a = rnd_exp(900, 1100);
      b = from_bits(bits(rnd_exp(900, 1100)) - ((next() % 71) << 52));
    } else if (kind == 2) {  // near cancellation: b = -a perturbed in its low bits
      a = rnd_exp(1, 2046);
      b = from_bits((bits(a) ^ kSign) + (next() % 17) - 8);
    } else if (kind == 3) {  // exponent gaps 0..3 with few significand bits (carries, ties)
      a = from_bits((bits(rnd_exp(1000, 1040)) & ~0x3FFFFFFFFFFull));
      b = from_bits((bits(rnd_exp(1000, 1040)) & ~0x3FFFFFFFFFFull) - ((next() % 4) << 52));
    } else if (kind == 4) {  // products near underflow and overflow
      a = rnd_exp(1, 600);
      b = rnd_exp(1, 600);
      if (next() & 1) {
        a = rnd_exp(1500, 2046);
        b = rnd_exp(1000, 1100);
      }
    } else if (kind == 5) {  // sums near the smallest normal
      a = rnd_exp(1, 60);
      b = rnd_exp(1, 60);
    } else if (kind == 6) {  // short significands: exact products, ties in sums
      a = from_bits(bits(rnd_exp(1000, 1050)) & ~0xFFFFFFFFFFull);
      b = from_bits(bits(rnd_exp(1000, 1050)) & ~0xFFFFFFFull);
    } else if (kind == 7) {  // the magnitudes a flow solver sees
      a = rnd_exp(1013, 1033);
      b = rnd_exp(1003, 1033);
    } else if (kind == 8) {  // divisors with a significand at or just above 1 (or just below 2)
      a = rnd_exp(1000, 1040);
      const uint64_t low = next() % 4096;
      b = from_bits(((uint64_t)(1000 + next() % 40) << 52) | ((next() & 1) ? low : kFrac - low));
    } else {  // quotients that are exact, or a few ulps from exact
      b = rnd_exp(1000, 1040);
      const double qq = from_bits(bits(rnd_exp(1015, 1031)) & ~0xFFFFFFFFFull);
      volatile double prod = b * qq;
      a = from_bits(bits(prod) + (next() % 5) - 2);
    }
    check(a, b);
  }
  printf("cases %lld mismatches %lld\n", cases, bad);
  return bad ? 1 : 0;
}
