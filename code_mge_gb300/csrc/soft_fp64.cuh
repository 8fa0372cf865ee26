// soft_fp64.cuh -- IEEE-754 binary64 multiply, add and divide, round to
// nearest even, in 32- and 64-bit integer arithmetic.
//
// GB300 issues FP64 at 2 thread-operations per SM per cycle: one FP64 warp
// instruction holds a scheduler's FP64 pipe for 64 cycles, while its issue
// slots and its integer pipes stay mostly idle in the stage kernels.  The
// functions below compute the correctly rounded product, sum and quotient on
// the integer pipes, so that a kernel can run part of its FP64 operations there,
// beside the native ones, with bit-identical results.
//
// The algorithm is the textbook one for binary floating point (unpack the
// exponents and 53-bit significands, form the exact product or the aligned
// sum with guard and sticky bits, normalise, round to nearest even, pack;
// as in J. R. Hauser's SoftFloat and J.-M. Muller et al., Handbook of
// Floating-Point Arithmetic, ch. 7-8).  Only the common case is done here:
// normal operands and a normal result.  Every other case (a zero,
// subnormal, infinite or NaN operand, an overflow or an underflow) returns
// the native operation, so the functions return exactly what IEEE-754
// multiplication, addition and division return for all inputs.
//
// The header compiles for the host as well, where the tests check it against
// the host's own binary64 arithmetic.
#pragma once
#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define MGE_SF_HD __host__ __device__ __forceinline__
#define MGE_SF_NOINLINE __host__ __device__ __noinline__
#else
#define MGE_SF_HD inline
#define MGE_SF_NOINLINE inline
#endif

namespace mge {
namespace soft {

constexpr uint64_t kFrac = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kOne = 0x0010000000000000ull;   // the implicit significand bit
constexpr uint64_t kSign = 0x8000000000000000ull;

MGE_SF_HD uint64_t bits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, 8);
  return u;
#endif
}

MGE_SF_HD double from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, 8);
  return x;
#endif
}

MGE_SF_HD int clz64(uint64_t x) {  // x != 0
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

// the high 64 bits of the 128-bit product of two 64-bit integers
MGE_SF_HD uint64_t mulhi64(uint64_t x, uint64_t y) {
#ifdef __CUDA_ARCH__
  return __umul64hi(x, y);
#else
  return (uint64_t)(((unsigned __int128)x * y) >> 64);
#endif
}

// the native operations, out of line, for the cases the integer forms leave
MGE_SF_NOINLINE double native_mul(double a, double b) { return a * b; }
MGE_SF_NOINLINE double native_add(double a, double b) { return a + b; }
MGE_SF_NOINLINE double native_div(double a, double b) { return a / b; }

// a * b
MGE_SF_HD double mul(double a, double b) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t ea = (uint32_t)(A >> 52) & 0x7ffu, eb = (uint32_t)(B >> 52) & 0x7ffu;
  // biased exponent of the product when the significands multiply into [1, 2)
  const int32_t e0 = (int32_t)(ea + eb) - 1023;
  // normal operands (ea, eb in 1..2046), and a product whose exponent e0 or
  // e0 + 1, after a rounding carry one more, stays in 1..2046
  if (ea - 1u >= 2046u || eb - 1u >= 2046u || (uint32_t)(e0 - 1) >= 2044u) return native_mul(a, b);
  const uint64_t ma = (A & kFrac) | kOne, mb = (B & kFrac) | kOne;  // [2^52, 2^53)
  // the exact 106-bit product hi * 2^64 + lo from 32-bit halves (ah, bh < 2^21)
  const uint32_t al = (uint32_t)ma, ah = (uint32_t)(ma >> 32), bl = (uint32_t)mb, bh = (uint32_t)(mb >> 32);
  const uint64_t t0 = (uint64_t)al * bl;
  const uint64_t mid = (uint64_t)ah * bl + ((uint64_t)al * bh + (t0 >> 32));  // < 2^54 + 2^32
  const uint64_t hi = (uint64_t)ah * bh + (mid >> 32);                         // [2^40, 2^42)
  const uint64_t lo = (mid << 32) | (t0 & 0xffffffffull);
  // the product's leading bit is bit 105 (top = 1) or 104 (top = 0); the
  // significand is the product shifted right by 52 + top, and the bits below
  // it, left-aligned in rest, give the round bit (its top bit) and the sticky
  const uint32_t top = (uint32_t)(hi >> 41);
  const uint32_t s = 12u - top;
  uint64_t m = (hi << s) | (lo >> (64u - s));
  const uint64_t rest = lo << s;
  m += (rest >> 63) & ((uint64_t)((rest << 1) != 0) | (m & 1u));
  // packing: a significand rounded up to 2^53 carries into the exponent
  return from_bits(((A ^ B) & kSign) | (((uint64_t)(e0 + (int32_t)top - 1) << 52) + m));
}

// a + b
MGE_SF_HD double add(double a, double b) {
  uint64_t A = bits(a), B = bits(b);
  uint64_t xa = A & ~kSign, xb = B & ~kSign;
  if (xa < xb) {  // |a| >= |b| from here on
    const uint64_t t = A;
    A = B;
    B = t;
    const uint64_t u = xa;
    xa = xb;
    xb = u;
  }
  const uint32_t ea = (uint32_t)(xa >> 52), eb = (uint32_t)(xb >> 52);
  if (ea - 1u >= 2046u || eb - 1u >= 2046u) return native_add(a, b);
  const uint32_t d = ea - eb;
  // significands with 10 guard bits: [2^62, 2^63)
  const uint64_t ma = ((xa & kFrac) | kOne) << 10, mb = ((xb & kFrac) | kOne) << 10;
  // mb aligned to ma's exponent; the bits shifted out set the sticky bit 0
  uint64_t mbs;
  if (d >= 64u) {
    mbs = 1u;
  } else {
    mbs = mb >> d;
    mbs |= (uint64_t)((mbs << d) != mb);
  }
  int32_t e = (int32_t)ea;
  uint64_t m;
  if (((A ^ B) >> 63) == 0) {
    m = ma + mbs;  // < 2^64
    const uint64_t c = m >> 63;
    m = (m >> c) | (m & c);  // a carry: one bit right, keeping the sticky
    e += (int32_t)c;
  } else {
    m = ma - mbs;
    if (m == 0) return 0.0;  // exact cancellation gives +0 in round to nearest
    // normalise the leading bit to bit 62; a shift of more than one happens
    // only when d <= 1, where the difference is exact
    const int z = clz64(m) - 1;
    m <<= z;
    e -= z;
  }
  // m in [2^62, 2^63): keep bits 62..10, round on bit 9, sticky bits 8..0
  if ((uint32_t)(e - 1) >= 2045u) return native_add(a, b);  // underflow, or overflow after rounding
  uint64_t r = m >> 10;
  r += ((m >> 9) & 1u) & ((uint64_t)((m & 0x1ffu) != 0) | (r & 1u));
  return from_bits((A & kSign) | (((uint64_t)(e - 1) << 52) + r));
}

MGE_SF_HD double sub(double a, double b) { return add(a, from_bits(bits(b) ^ kSign)); }

// a / b.  The significands' quotient comes from a reciprocal of the divisor
// in 64-bit fixed point: an FP32 reciprocal of its leading 24 bits (about 23
// correct bits), then two Newton steps x <- x + x(1 - d x) (about 60 bits).
// The quotient estimate c, with one bit below the last significand bit, is
// then within one unit of the true floor, and the exact remainder r = a - c b
// (which fits in a signed 64-bit integer) corrects it and gives the sticky
// bit for rounding to nearest even.
MGE_SF_HD double div(double a, double b) {
  const uint64_t A = bits(a), B = bits(b);
  const uint32_t ea = (uint32_t)(A >> 52) & 0x7ffu, eb = (uint32_t)(B >> 52) & 0x7ffu;
  const uint64_t ma = (A & kFrac) | kOne, mb = (B & kFrac) | kOne;  // [2^52, 2^53)
  const bool ge = ma >= mb;                                          // quotient in [1, 2), else (1/2, 1)
  // biased exponent of the result; 1..2045 leaves room for a rounding carry
  const int32_t e = (int32_t)ea - (int32_t)eb + (ge ? 1023 : 1022);
  if (ea - 1u >= 2046u || eb - 1u >= 2046u || (uint32_t)(e - 1) >= 2045u) return native_div(a, b);
  // divisor d = mb 2^11 in [2^63, 2^64) stands for D = d / 2^64 in [1/2, 1);
  // X stands for x = X / 2^62, an approximation of 1/D in (1, 2]
  const uint64_t d = mb << 11;
#ifdef __CUDA_ARCH__
  const float x0 = __frcp_rn((float)(uint32_t)(d >> 40) * 5.9604644775390625e-8f);  // 1 / (d_hi / 2^24)
  const uint32_t xb = __float_as_uint(x0);
#else
  const float x0 = 1.0f / ((float)(uint32_t)(d >> 40) * 5.9604644775390625e-8f);
  uint32_t xb;
  memcpy(&xb, &x0, 4);
#endif
  // x0 in (1, 2]: its significand (with the implicit bit) times 2^(39 + exponent)
  uint64_t X = (uint64_t)((xb & 0x7fffffu) | 0x800000u) << (39 + ((xb >> 23) & 0xffu) - 127);
  for (int it = 0; it < 2; it++) {
    // x (1 - D x) 2^62 = X e / 2^62 with e = (1 - D x) 2^62, |e| < 2^41
    const uint64_t p = mulhi64(d, X);  // D x 2^62
    if (p <= (1ull << 62)) {
      X += mulhi64(X, ((1ull << 62) - p) << 2);
    } else {
      X -= mulhi64(X, (p - (1ull << 62)) << 2);
    }
  }
  // the quotient ma/mb times 2^62, within a few units
  const uint64_t q = mulhi64(ma << 11, X);
  // c: the quotient with the significand's 53 bits and one more, as an
  // integer; its true floor is c - 1, c or c + 1
  const uint32_t sh = ge ? 9u : 8u;
  uint64_t c = q >> sh;
  // r = ma 2^(53 or 54) - c mb, exactly, in the low 64 bits (|r| < 2^55)
  int64_t r = (int64_t)((ma << (64u - 11u + (ge ? 0u : 1u))) - c * mb);
  if (r < 0) {
    c -= 1;
    r += (int64_t)mb;
  } else if (r >= (int64_t)mb) {
    c += 1;
    r -= (int64_t)mb;
  }
  uint64_t m = c >> 1;
  m += (c & 1u) & ((uint64_t)(r != 0) | (m & 1u));
  return from_bits(((A ^ B) & kSign) | (((uint64_t)(e - 1) << 52) + m));
}

}  // namespace soft
}  // namespace mge
