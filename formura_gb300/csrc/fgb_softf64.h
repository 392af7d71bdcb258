// Correctly rounded binary64 arithmetic on the integer pipes.
//
// On this part the FP64 pipe executes about one warp instruction per 67
// cycles per SM sub-partition, while the integer and FP32 pipes sit idle in
// the FP64 stencil kernels (issue slots are over 90 % free).  Every
// operation below returns exactly the IEEE 754 round-to-nearest-even result
// of the hardware instruction it stands for, computed with 64-bit integer
// significand arithmetic (the method of Berkeley SoftFloat: align with a
// sticky bit, add or subtract, normalise, round to nearest even).  Each one
// has a fast path for the common case and reports whether it applied; the
// callers fall back to the hardware instruction otherwise, so subnormal
// results, infinities, NaNs and exponents near the ends of the range are
// always rounded by the hardware.  Mixing the two pipes within a kernel is
// what raises the FP64 throughput; the results are bit-identical either way.
//
// The same code compiles for the host, where it is tested against the host's
// IEEE arithmetic.
#pragma once
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define FGB_SOFT_HD __host__ __device__ __forceinline__
#else
#define FGB_SOFT_HD static inline
#endif

namespace fgb {
namespace soft {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kAbs = 0x7fffffffffffffffull;
constexpr uint64_t kMant = 0x000fffffffffffffull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

FGB_SOFT_HD uint64_t to_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

FGB_SOFT_HD double from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

FGB_SOFT_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}

FGB_SOFT_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Round a significand whose leading one is at bit 63 (bits 62..11 are the
// fraction, bit 10 the round bit, bits 9..0 sticky; a sticky bit that stands
// for discarded low-order bits is always odd, so it never forms a tie) and
// pack it with sign and biased exponent field e (1 <= e, e + 1 <= 2046).  A
// carry out of the rounding increments the exponent through the addition.
FGB_SOFT_HD uint64_t round_pack(uint64_t sign, int e, uint64_t m) {
  uint64_t q = m >> 11;
  const uint32_t rem = (uint32_t)m & 0x7ffu;
  q += (rem > 0x400u || (rem == 0x400u && (q & 1u))) ? 1u : 0u;
  return sign | (((uint64_t)(e - 1) << 52) + q);
}

// a + b.  Fast path: both operands are zeros, or the operand of larger
// magnitude has an exponent field in [64, 2044]; then the result is a finite
// normal number or an exact zero, and the smaller operand may be anything
// finite (zero and subnormal included).
FGB_SOFT_HD bool add_bits(uint64_t A, uint64_t B, uint64_t& R) {
  const uint64_t a = A & kAbs, b = B & kAbs;
  const bool swap = b > a;
  const uint64_t big = swap ? B : A, sml = swap ? A : B;
  const uint64_t abig = swap ? b : a, asml = swap ? a : b;
  if (abig == 0) {  // both zero: -0 only if both are -0
    R = A & B;
    return true;
  }
  const int eb = (int)(abig >> 52);
  if ((unsigned)(eb - 64) > (unsigned)(2044 - 64)) return false;
  const int es = (int)(asml >> 52);
  const uint64_t mb = ((abig & kMant) | kHidden) << 10;             // leading one at bit 62
  const uint64_t ms = ((asml & kMant) | (es ? kHidden : 0)) << 10;  // subnormals: field 0 ~ 1
  int d = eb - (es ? es : 1);
  d = d > 63 ? 63 : d;
  const uint64_t lost = ms & ((1ull << d) - 1);
  const uint64_t al = (ms >> d) | (lost ? 1u : 0u);
  const uint64_t m = ((big ^ sml) & kSign) ? mb - al : mb + al;
  if (m == 0) {  // x + (-x) is +0 under round to nearest
    R = 0;
    return true;
  }
  const int lz = clz64(m);
  R = round_pack(big & kSign, eb + 1 - lz, m << lz);
  return true;
}

// a * b.  Fast path: both operands finite, and either one is zero (the
// result is a signed zero) or both are normal with a product exponent that
// stays normal after rounding.
FGB_SOFT_HD bool mul_bits(uint64_t A, uint64_t B, uint64_t& R) {
  const uint64_t sign = (A ^ B) & kSign;
  const int ea = (int)((A >> 52) & 0x7ff), eb = (int)((B >> 52) & 0x7ff);
  const int e = ea + eb - 1023;
  if (ea == 0 || eb == 0 || ea == 2047 || eb == 2047 || (unsigned)(e - 1) > 2043u) {
    if (ea != 2047 && eb != 2047 && ((A & kAbs) == 0 || (B & kAbs) == 0)) {
      R = sign;
      return true;
    }
    return false;
  }
  const uint64_t ma = ((A & kMant) | kHidden) << 11, mb = ((B & kMant) | kHidden) << 11;
  const uint64_t hi = mulhi64(ma, mb);   // leading one at bit 63 or 62
  const uint64_t lo = ma * mb;
  const uint64_t m = hi | (lo ? 1u : 0u);
  const int lz = (int)(~hi >> 63);       // 1 if the leading one is at bit 62
  R = round_pack(sign, e + 1 - lz, m << lz);
  return true;
}

// c * h for c = +-2^k (the exact power-of-two factors of the merged
// multiply-adds): exponent arithmetic when h is zero, or normal and stays
// normal.
FGB_SOFT_HD bool scale_bits(uint64_t H, int k, bool negate, uint64_t& R) {
  if ((H & kAbs) == 0) {
    R = H ^ (negate ? kSign : 0);
    return true;
  }
  const int eh = (int)((H >> 52) & 0x7ff);
  if (eh == 0 || eh == 2047 || (unsigned)(eh + k - 1) > 2045u) return false;
  R = (H + ((uint64_t)(int64_t)k << 52)) ^ (negate ? kSign : 0);
  return true;
}

// c*h + t for a power of two c, as the hardware's fused multiply-add gives it
// (the product is exact, so this is one rounding of the sum).
FGB_SOFT_HD bool scaled_add_bits(uint64_t C, uint64_t H, uint64_t T, uint64_t& R) {
  uint64_t S;
  const int k = (int)((C >> 52) & 0x7ff) - 1023;
  return scale_bits(H, k, (C >> 63) != 0, S) && add_bits(T, S, R);
}

}  // namespace soft
}  // namespace fgb
