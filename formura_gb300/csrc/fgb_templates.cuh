// Hand-written sm_103a kernel templates.  Each program's step function is
// emitted as one functor per stage (see formura_gb300/generator/cuda.py);
// these templates supply the arithmetic policy, the storage format, the
// periodic in-kernel wrap that replaces the reference's halo exchange
// (Functions.hs:265-307, Templates.hs:336-346) and the launch geometry.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>
#include <type_traits>
#include "fgb_internal.h"

namespace fgb {

// ---------------------------------------------------------------------------
// arithmetic policies
// ---------------------------------------------------------------------------
struct F64Fast;
struct F64Ieee;

// FP64, rounding exactly like the reference's C: one IEEE rounding per SSA
// operation, no contraction (the __d*_rn intrinsics are never fused).
//
// Three operations take shortened forms that equal the reference's only
// while no intermediate leaves the normal range: a multiply-add by a power
// of two, a division by a grid-independent value through its host
// reciprocal and a division through a shared reciprocal.  Each checks on the
// integer pipe whether its operands lie in its window.  The divisions take a
// warp-uniform branch when a lane's operands do not: the division by a
// grid-independent value to its forms for numerators below the window
// (divu_outside), else, like the other division, to the IEEE division;
// the multiply-add, whose window is left only near overflow or underflow,
// records it in the `ok` flag of the stage functor (which run() returns),
// and a warp in which any lane's flag dropped evaluates the functor again
// with F64Ieee, the plain separately rounded operations (eval() below).
// Inside the windows both forms give the same bits, so the result never
// depends on which lanes share a warp.  Comparisons, |x| and 1 - x (for x
// in [0.5, 2), else the FP64 subtraction) run on the integer pipe, exactly.
struct F64Exact {
  using T = double;
  using U = double;   // element type of the uniform table
  using Ieee = F64Ieee;
  static constexpr bool kChecked = true;
  // Arithmetic of the generated adjoint kernels: contracted FP64.  The
  // forward steps of a gradient keep this exact policy, but the arrays an
  // adjoint step recomputes (with the F64Fast stage kernels), the forward
  // values a partial-sum kernel differentiates and its derivative terms are
  // contracted, and a quotient there is a product with the reciprocal that
  // the derivative needs anyway.  A gradient is checked against finite
  // differences and the dot-product identity, not bit patterns; a fused
  // multiply-add is one FP64 instruction instead of two.
  using Deriv = F64Fast;
  static __device__ __forceinline__ T add(T a, T b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ T sub(T a, T b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ T mul(T a, T b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ T div(T a, T b) { return __ddiv_rn(a, b); }

  // The range checks read the two 32-bit halves through an opaque move, so
  // that the compiler keeps them on the integer pipe instead of turning a
  // bit test into an FP64 comparison on the (busy) FP64 pipe.
  static __device__ __forceinline__ void halves(T x, unsigned& lo, unsigned& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(x));
  }
  static __device__ __forceinline__ T join(unsigned lo, unsigned hi) {
    T r;
    asm("mov.b64 %0, {%1, %2};" : "=d"(r) : "r"(lo), "r"(hi));
    return r;
  }
  static __device__ __forceinline__ unsigned expo(T x) {
    unsigned lo, hi;
    halves(x, lo, hi);
    return (hi >> 20) & 0x7ffu;
  }
  static __device__ __forceinline__ bool is_zero(T x) {
    unsigned lo, hi;
    halves(x, lo, hi);
    return ((hi << 1) | lo) == 0u;
  }
  // biased exponent field within [1023 - w, 1023 + w]
  static __device__ __forceinline__ bool within(T x, unsigned w) { return expo(x) - (1023u - w) <= 2u * w; }

  // IEEE comparisons on the integer pipe (an FP64 compare costs the FP64
  // pipe as much as an FMA): an order key per operand, its magnitude bits
  // negated when the sign is set, so that -0 and +0 share the key 0; any
  // comparison with a NaN is false, except !=.
  static __device__ __forceinline__ long long okey(T x, bool& nan) {
    unsigned lo, hi;
    halves(x, lo, hi);
    const unsigned mhi = hi & 0x7fffffffu;
    nan = mhi > 0x7ff00000u || (mhi == 0x7ff00000u && lo != 0u);
    const long long mag = (long long)(((unsigned long long)mhi << 32) | lo);
    return (hi >> 31) ? -mag : mag;
  }
  static __device__ __forceinline__ bool lt(T a, T b) {
    bool na, nb;
    const long long ka = okey(a, na), kb = okey(b, nb);
    return !(na || nb) && ka < kb;
  }
  static __device__ __forceinline__ bool gt(T a, T b) { return lt(b, a); }
  static __device__ __forceinline__ bool le(T a, T b) {
    bool na, nb;
    const long long ka = okey(a, na), kb = okey(b, nb);
    return !(na || nb) && ka <= kb;
  }
  static __device__ __forceinline__ bool ge(T a, T b) { return le(b, a); }
  static __device__ __forceinline__ bool eq(T a, T b) {
    bool na, nb;
    const long long ka = okey(a, na), kb = okey(b, nb);
    return !(na || nb) && ka == kb;
  }
  static __device__ __forceinline__ bool ne(T a, T b) { return !eq(a, b); }

  // a*h + t for a = +-2^k (a literal): one rounding of the exact sum, which
  // is the reference's RN(RN(a*h) + t) as long as a*h is exact, that is h
  // is zero or a*h stays normal.
  static __device__ __forceinline__ T fma(T a, T h, T t, bool& ok) {
    const int k = (int)(((unsigned long long)__double_as_longlong(a) >> 52) & 0x7ffu) - 1023;   // a literal
    ok &= is_zero(h) || (unsigned)((int)expo(h) + k - 1) <= 2045u;
    return __fma_rn(a, h, t);
  }
  // q = RN(x / c) from y = RN(1 / c): Markstein's correction of RN(x * y),
  // exact when x - q*c is representable and q normal.  Zero numerators take
  // RN(x * y) itself, which carries the quotient's sign.
  static __device__ __forceinline__ T markstein(T x, T c, T y) {
    const T q = __dmul_rn(x, y);
    const T e = __fma_rn(-q, c, x);
    return is_zero(x) ? q : __fma_rn(e, y, q);
  }
  // The last rounding step of that quotient on the integer pipe, in place of
  // Markstein's second FMA.  With q0 = RN(x * y) and the exact remainder
  // r = x - q0*c: x*y is within |x/c| * 2^-53 of x/c, so where q0 lies at
  // least two ulps inside its binade, x/c lies in the same binade within
  // 1.5 ulp of q0, and RN(x/c) is q0 or the neighbour towards x/c (the sign
  // of r/c).  It is the neighbour when |r| > |c| * ulp(q0) / 2 (a quotient of
  // two doubles is never exactly a midpoint; the even one is taken if it
  // were).  |c| * ulp(q0) / 2 is |c| with its exponent field moved, and two
  // non-negative doubles compare like their bit patterns.  A neighbour is
  // the bit pattern plus or minus one inside the binade.  Where |r| is below
  // the threshold it is exact or, under 2^-1022, smaller than the threshold
  // whatever its rounding (the threshold is kept at least 2^-1021).
  // `fits` reports whether the step applies; zero numerators keep RN(x*y).
  static __device__ __forceinline__ T round_quotient(T x, T c, T q0, T r, bool& fits) {
    unsigned qlo, qhi, rlo, rhi, clo, chi;
    halves(q0, qlo, qhi);
    halves(r, rlo, rhi);
    halves(c, clo, chi);
    const unsigned eq = (qhi >> 20) & 0x7ffu, ec = (chi >> 20) & 0x7ffu;
    const unsigned long long m = ((unsigned long long)(qhi & 0xfffffu) << 32) | qlo;
    const int et = (int)ec + (int)eq - 1076;   // exponent field of |c| * ulp(q0) / 2
    const bool zero = is_zero(x);
    fits = zero || (m - 2ull <= (1ull << 52) - 5ull && (unsigned)(et - 2) <= 2044u);
    const unsigned long long t = ((unsigned long long)((chi & 0xfffffu) | ((unsigned)et << 20)) << 32) | clo;
    const unsigned long long a = ((unsigned long long)(rhi & 0x7fffffffu) << 32) | rlo;
    const bool step = a > t || (a == t && (qlo & 1u));
    const bool up = ((rhi ^ chi ^ qhi) >> 31) == 0;   // towards x/c the magnitude grows
    const unsigned long long qb = ((unsigned long long)qhi << 32) | qlo;
    const unsigned long long res = qb + (step ? (up ? 1ull : ~0ull) : 0ull);
    return zero ? q0 : join((unsigned)res, (unsigned)(res >> 32));
  }
  // RN(x / c) inside Markstein's window: two FP64 instructions and the
  // integer step where it applies to every lane of the warp, else
  // Markstein's second FMA (the same bits).
  static __device__ __forceinline__ T quotient(T x, T c, T y) {
    const T q0 = __dmul_rn(x, y);
    const T r = __fma_rn(-q0, c, x);
    bool fits;
    const T q = round_quotient(x, c, q0, r, fits);
    if (warp_all(fits)) return q;
    return markstein_last(x, q0, r, y);
  }
  // out of line, so that the compiler does not compute it ahead of the test
  static __device__ __noinline__ T markstein_last(T x, T q0, T r, T y) {
    return is_zero(x) ? q0 : __fma_rn(r, y, q0);
  }
  // The divisions decide per operation instead of raising the flag: a field
  // that decays through the subnormal range (Gray-Scott's v far from the
  // pattern) keeps whole warps out of the window for many steps, and there
  // one IEEE division costs less than evaluating the stage twice.
  static __device__ __forceinline__ bool warp_all(bool ok) { return __all_sync(__activemask(), ok); }
  // x / c for a grid-independent c with rc = RN(1/c) from the host: c in
  // [2^-100, 2^100]; x zero, or of exponent in [-960, 960] with the
  // quotient's exponent in [-1000, 1000] (then x - q*c is representable and
  // q normal)
  static __device__ __forceinline__ bool divu_window(T x, T c) {
    const unsigned ex = expo(x);
    return within(c, 100) && (is_zero(x) || (ex - 63u <= 1920u && ex - expo(c) + 1000u <= 2000u));
  }
  static __device__ __forceinline__ T divu(T x, T c, T rc, bool&) {
#ifdef FGB_DIVU_IEEE
    (void)rc;
    return __ddiv_rn(x, c);
#else
    if (warp_all(divu_window(x, c))) return quotient(x, c, rc);
    return divu_outside(x, c, rc);
#endif
  }
  // Numerators below the window (a field decaying through tiny values).
  // Where x/c is at least 2^-1022, x * 2^256 lies in the window and the
  // quotient comes back by 2^-256 exactly, both on the integer pipe, so such
  // a quotient costs what one inside the window costs.  That holds when x's
  // exponent (a subnormal's counted from its leading bit) is at least c's
  // minus 1021.  Quotients below 2^-1021 are rounded on the integer grid of
  // the subnormals (divu_sub, divu_mixed below), with the same two FP64
  // instructions; a warp with a lane in none of the forms (an operand out of
  // range) takes the IEEE division.
  // Out of line, so that the compiler cannot fold this path into the common
  // one.
  //
  // x * 2^k on the integer pipe for a nonzero x whose exponent field stays
  // within range: the field moves up by k; a subnormal's significand is
  // first shifted to its leading bit.
  template <int K>
  static __device__ __forceinline__ T scale_up(T x) {
    unsigned lo, hi;
    halves(x, lo, hi);
    const unsigned ex = (hi >> 20) & 0x7ffu;
    unsigned long long b = ((unsigned long long)hi << 32) | lo;
    if (ex != 0u) {
      b += (unsigned long long)K << 52;
    } else {
      const unsigned long long m = b & 0x000fffffffffffffull;
      const int sh = __clzll((long long)m) - 11;
      b = (b & 0x8000000000000000ull) | ((unsigned long long)(K + 1 - sh) << 52) |
          ((m << sh) & 0x000fffffffffffffull);
    }
    return join((unsigned)b, (unsigned)(b >> 32));
  }
  // q * 2^-256 for a q whose exponent field exceeds 256: exact
  static __device__ __forceinline__ T scale_down(T q) {
    unsigned lo, hi;
    halves(q, lo, hi);
    return join(lo, hi - (256u << 20));
  }
  static __device__ __forceinline__ bool divu_tiny(T x, T c) {
    unsigned lo, hi;
    halves(x, lo, hi);
    const unsigned ex = (hi >> 20) & 0x7ffu;
    const unsigned long long m = ((unsigned long long)(hi & 0xfffffu) << 32) | lo;
    const int eff = ex != 0u ? (int)ex : 12 - __clzll((long long)m);   // a subnormal's leading bit
    return within(c, 100) && ex < 63u && m + ex != 0ull && eff + 1021 >= (int)expo(c);
  }
  // Quotients below 2^-1021 (subnormal ones and the lowest normal binade):
  // RN(x/c) is N * 2^-1074 for the integer N nearest X/c, ties to even, with
  // X = |x| * 2^1074 an integer (exact on the integer pipe), since the
  // doubles below 2^-1021 lie on that grid; the bit pattern of N * 2^-1074
  // is N.  With q0 = RN(X * |RN(1/c)|):
  // - below 2^51, q0 lies within 0.5 + 2^-52 of X/c, so n0, q0 rounded to an
  //   integer, lies within 1 + 2^-52 of it; the remainder X - n0 * |c| is
  //   then exact (one FMA), and its size against |c|/2 picks N among
  //   n0 - 1, n0, n0 + 1;
  // - from 2^51 (ulp 1/2 or 1), q0 lies within one ulp of X/c, so
  //   X - q0 * |c| is exact; with q0's own fraction (0 or 1/2) it decides N
  //   in the same way.
  // Applies to a nonzero x whose exponent (a subnormal's counted from its
  // leading bit) is at most c's minus 1022.
  static __device__ __forceinline__ bool divu_sub(T x, T c) {
    unsigned lo, hi;
    halves(x, lo, hi);
    const unsigned ex = (hi >> 20) & 0x7ffu;
    const unsigned long long m = ((unsigned long long)(hi & 0xfffffu) << 32) | lo;
    const int eff = ex != 0u ? (int)ex : 12 - __clzll((long long)m);
    return within(c, 100) && m + ex != 0ull && eff - (int)expo(c) <= -1022;
  }
  // A warp whose lanes each lie in the window, among the tiny numerators or
  // among the quotients below 2^-1021: the same two FP64 instructions on
  // every lane's own operands, then the lane's integer steps.
  static __device__ __forceinline__ T divu_mixed(T x, T c, T rc, bool tiny, bool sub) {
    unsigned xl, xh, cl, ch, yl, yh;
    halves(x, xl, xh);
    halves(c, cl, ch);
    halves(rc, yl, yh);
    const T a = sub ? scale_up<1074>(join(xl, xh & 0x7fffffffu)) : (tiny ? scale_up<256>(x) : x);
    const T cc = sub ? join(cl, ch & 0x7fffffffu) : c;
    const T q0 = __dmul_rn(a, sub ? join(yl, yh & 0x7fffffffu) : rc);
    // below 2^51: q0 rounded to an integer (half up), and that integer as a
    // double; from 2^51: q0's integer part and whether q0 ends in a half
    unsigned ql, qh;
    halves(q0, ql, qh);
    const int e = (int)((qh >> 20) & 0x7ffu) - 1023;
    const unsigned long long qm = ((unsigned long long)((qh & 0xfffffu) | 0x100000u) << 32) | ql;
    const int sh = min(max(52 - e, 1), 53);
    const unsigned long long n0 = e < -1 ? 0ull : (qm + (1ull << (sh - 1))) >> sh;
    const int lead = 63 - __clzll((long long)(n0 | 1ull));
    const unsigned long long nb =
        n0 == 0ull ? 0ull : (((unsigned long long)(lead + 1023) << 52) | ((n0 << (52 - lead)) & 0x000fffffffffffffull));
    const bool upper = e >= 51;
    const unsigned long long base = upper ? (e >= 52 ? qm << min(e - 52, 11) : qm >> 1) : n0;
    const bool halfq = e == 51 && (qm & 1ull);
    const T r = __fma_rn(-((sub && !upper) ? join((unsigned)nb, (unsigned)(nb >> 32)) : q0), cc, a);
    // window and tiny lanes: the integer rounding step (or Markstein's FMA)
    bool fits;
    T q = round_quotient(a, c, q0, r, fits);
    if (!warp_all(fits || sub)) {
      if (!sub) q = markstein_last(a, q0, r, rc);
    }
    // lanes below 2^-1021: the remainder against |c|/2, or its sign where
    // q0 ends in a half
    unsigned rl, rh;
    halves(r, rl, rh);
    const unsigned long long ar = ((unsigned long long)(rh & 0x7fffffffu) << 32) | rl;
    const unsigned long long half = (((unsigned long long)(ch & 0x7fffffffu) << 32) | cl) - (1ull << 52);
    const bool rneg = (rh >> 31) != 0u;
    const bool step = halfq ? ((!rneg && ar != 0ull) || (ar == 0ull && (base & 1ull)))
                            : (ar > half || (ar == half && (base & 1ull)));
    const unsigned long long n = base + (step ? ((rneg && !halfq) ? ~0ull : 1ull) : 0ull);
    const unsigned long long sb = n | ((unsigned long long)((xh ^ ch) & 0x80000000u) << 32);
    return sub ? join((unsigned)sb, (unsigned)(sb >> 32)) : (tiny ? scale_down(q) : q);
  }
  static __device__ __noinline__ T divu_outside(T x, T c, T rc) {
    const bool win = divu_window(x, c), tiny = divu_tiny(x, c);
    if (warp_all(win || tiny)) {
      const T q = quotient(tiny ? scale_up<256>(x) : x, c, rc);
      return tiny ? scale_down(q) : q;
    }
    const bool sub = divu_sub(x, c);
    if (warp_all(win || tiny || sub)) return divu_mixed(x, c, rc, tiny, sub);
    return __ddiv_rn(x, c);
  }
  // RN(1/b) for a grid value b that several quotients divide by
  static __device__ __forceinline__ T rcp(T b) { return __drcp_rn(b); }
  // a / b with y = rcp(b): operands in [2^-400, 2^400] (a may be zero)
  static __device__ __forceinline__ bool divr_window(T a, T b) {
    return within(b, 400) && (is_zero(a) || within(a, 400));
  }
  static __device__ __forceinline__ T divr(T a, T b, T y, bool&) {
    if (warp_all(divr_window(a, b))) return quotient(a, b, y);
    return __ddiv_rn(a, b);
  }
  static __device__ __forceinline__ T neg(T a) { return -a; }
  // RN(1 - x) for the literal 1 (Gray-Scott's feed term F*(1 - u)).  For x
  // in [0.5, 2) the difference is exact (Sterbenz's lemma): with
  // x = X * 2^-53, X an integer below 2^54, 1 - x = (2^53 - X) * 2^-53, and
  // that integer is normalised by its leading bit on the integer pipe; 1 - 1
  // is +0 as in round-to-nearest.  A warp with a lane outside the range
  // subtracts on the FP64 pipe (the same bits).
  static __device__ __forceinline__ bool one_minus_window(T x) {
    unsigned lo, hi;
    halves(x, lo, hi);
    return (hi >> 21) == 511u;   // sign 0, exponent field 1022 or 1023
  }
  static __device__ __forceinline__ T one_minus_exact(T x) {
    unsigned lo, hi;
    halves(x, lo, hi);
    const unsigned long long X = ((((unsigned long long)((hi & 0xfffffu) | 0x100000u)) << 32) | lo) << ((hi >> 20) & 1u);
    const long long d = (long long)(1ull << 53) - (long long)X;
    const unsigned long long a = d < 0 ? (unsigned long long)(-d) : (unsigned long long)d;
    const int n = __clzll((long long)a);   // 10 <= n <= 64
    // leading bit to position 52; it carries into the exponent field
    const unsigned long long b = ((unsigned long long)(1032 - n) << 52) + (a << ((n - 11) & 63));
    const unsigned long long r = a == 0ull ? 0ull : (b | (d < 0 ? 0x8000000000000000ull : 0ull));
    return join((unsigned)r, (unsigned)(r >> 32));
  }
  static __device__ __forceinline__ T one_minus(T x) {
    if (warp_all(one_minus_window(x))) return one_minus_exact(x);
    return one_minus_ieee(x);
  }
  // out of line, so that the compiler does not compute it ahead of the test
  static __device__ __noinline__ T one_minus_ieee(T x) { return __dsub_rn(1.0, x); }
  static __device__ __forceinline__ T sqrt(T a) { return __dsqrt_rn(a); }
  // |a| by clearing the sign bit on the integer pipe (exact, NaN included)
  static __device__ __forceinline__ T fabs(T a) {
    unsigned lo, hi;
    halves(a, lo, hi);
    return join(lo, hi & 0x7fffffffu);
  }
  static __device__ __forceinline__ T exp(T a) { return ::exp(a); }
  static __device__ __forceinline__ T log(T a) { return ::log(a); }
  static __device__ __forceinline__ T sin(T a) { return ::sin(a); }
  static __device__ __forceinline__ T cos(T a) { return ::cos(a); }
  static __device__ __forceinline__ T pow(T a, T b) { return ::pow(a, b); }
};

// The reference's separately rounded IEEE operations, without shortened
// forms: what a warp of F64Exact falls back to.
struct F64Ieee {
  using T = double;
  using U = double;
  using Deriv = F64Fast;
  using Ieee = F64Ieee;
  static constexpr bool kChecked = false;
  static __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
  static __device__ __forceinline__ bool gt(T a, T b) { return a > b; }
  static __device__ __forceinline__ bool le(T a, T b) { return a <= b; }
  static __device__ __forceinline__ bool ge(T a, T b) { return a >= b; }
  static __device__ __forceinline__ bool eq(T a, T b) { return a == b; }
  static __device__ __forceinline__ bool ne(T a, T b) { return a != b; }
  static __device__ __forceinline__ T add(T a, T b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ T sub(T a, T b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ T mul(T a, T b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ T div(T a, T b) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ T fma(T a, T h, T t, bool&) { return __dadd_rn(__dmul_rn(a, h), t); }
  static __device__ __forceinline__ T divu(T x, T c, T, bool&) { return __ddiv_rn(x, c); }
  static __device__ __forceinline__ T rcp(T b) { return __drcp_rn(b); }
  static __device__ __forceinline__ T divr(T a, T b, T, bool&) { return __ddiv_rn(a, b); }
  static __device__ __forceinline__ T neg(T a) { return -a; }
  static __device__ __forceinline__ T one_minus(T x) { return __dsub_rn(1.0, x); }
  static __device__ __forceinline__ T sqrt(T a) { return __dsqrt_rn(a); }
  static __device__ __forceinline__ T fabs(T a) { return ::fabs(a); }
  static __device__ __forceinline__ T exp(T a) { return ::exp(a); }
  static __device__ __forceinline__ T log(T a) { return ::log(a); }
  static __device__ __forceinline__ T sin(T a) { return ::sin(a); }
  static __device__ __forceinline__ T cos(T a) { return ::cos(a); }
  static __device__ __forceinline__ T pow(T a, T b) { return ::pow(a, b); }
};

// F64Exact for a grid whose grid-independent divisors are all normal powers
// of two (the host checks the uniform table at fgb_open): x / c is then
// x * RN(1/c) exactly, one rounding for every x (subnormal, zero and
// non-finite included), so the division is that one product.  A run-time
// test of c inside the kernel instead cost Gray-Scott, whose divisor is not
// a power of two, 11 % (16.0 -> 14.3 GLUP/s).
struct F64ExactP2 : F64Exact {
  static __device__ __forceinline__ T divu(T x, T, T rc, bool&) { return __dmul_rn(x, rc); }
};

// FP64 with contraction and reciprocal multiplication (not bit-faithful).
struct F64Fast {
  using T = double;
  using U = double;
  using Deriv = F64Fast;
  using Ieee = F64Fast;
  static constexpr bool kChecked = false;
  static __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
  static __device__ __forceinline__ bool gt(T a, T b) { return a > b; }
  static __device__ __forceinline__ bool le(T a, T b) { return a <= b; }
  static __device__ __forceinline__ bool ge(T a, T b) { return a >= b; }
  static __device__ __forceinline__ bool eq(T a, T b) { return a == b; }
  static __device__ __forceinline__ bool ne(T a, T b) { return a != b; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T div(T a, T b) { return a / b; }
  static __device__ __forceinline__ T fma(T a, T b, T c, bool&) { return ::fma(a, b, c); }
  static __device__ __forceinline__ T divu(T x, T, T rc, bool&) { return x * rc; }
  static __device__ __forceinline__ T rcp(T b) { return __drcp_rn(b); }
  static __device__ __forceinline__ T divr(T a, T, T y, bool&) { return a * y; }
  static __device__ __forceinline__ T neg(T a) { return -a; }
  static __device__ __forceinline__ T one_minus(T x) { return 1.0 - x; }
  static __device__ __forceinline__ T sqrt(T a) { return ::sqrt(a); }
  static __device__ __forceinline__ T fabs(T a) { return ::fabs(a); }
  static __device__ __forceinline__ T exp(T a) { return ::exp(a); }
  static __device__ __forceinline__ T log(T a) { return ::log(a); }
  static __device__ __forceinline__ T sin(T a) { return ::sin(a); }
  static __device__ __forceinline__ T cos(T a) { return ::cos(a); }
  static __device__ __forceinline__ T pow(T a, T b) { return ::pow(a, b); }
};

// FP32 arithmetic (used with float or half storage).  The compiler may
// contract a product and a sum into one FFMA here: FP32 results are checked
// by their distance to the FP64 form, and every FP32 kernel evaluates the
// same stage code, so the one-step and the tile kernels still agree bit for
// bit.
struct F32 {
  using T = float;
  using U = float;
  using Deriv = F32;
  using Ieee = F32;
  static constexpr bool kChecked = false;
  static __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
  static __device__ __forceinline__ bool gt(T a, T b) { return a > b; }
  static __device__ __forceinline__ bool le(T a, T b) { return a <= b; }
  static __device__ __forceinline__ bool ge(T a, T b) { return a >= b; }
  static __device__ __forceinline__ bool eq(T a, T b) { return a == b; }
  static __device__ __forceinline__ bool ne(T a, T b) { return a != b; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  // reciprocal-based quotient (2 ulp): the FP32 form trades the IEEE
  // division sequence for two instructions; its distance to FP64 is reported
  static __device__ __forceinline__ T div(T a, T b) { return __fdividef(a, b); }
  static __device__ __forceinline__ T fma(T a, T b, T c, bool&) { return fmaf(a, b, c); }
  static __device__ __forceinline__ T divu(T x, T, T rc, bool&) { return x * rc; }
  static __device__ __forceinline__ T rcp(T b) { return __fdividef(1.0f, b); }
  static __device__ __forceinline__ T divr(T a, T, T y, bool&) { return a * y; }
  static __device__ __forceinline__ T neg(T a) { return -a; }
  static __device__ __forceinline__ T one_minus(T x) { return 1.0f - x; }
  static __device__ __forceinline__ T sqrt(T a) { return sqrtf(a); }
  static __device__ __forceinline__ T fabs(T a) { return fabsf(a); }
  static __device__ __forceinline__ T exp(T a) { return expf(a); }
  static __device__ __forceinline__ T log(T a) { return logf(a); }
  static __device__ __forceinline__ T sin(T a) { return sinf(a); }
  static __device__ __forceinline__ T cos(T a) { return cosf(a); }
  static __device__ __forceinline__ T pow(T a, T b) { return powf(a, b); }
};

// ---------------------------------------------------------------------------
// storage formats of the state
// ---------------------------------------------------------------------------
template <class S, class T> struct Storage;
template <> struct Storage<double, double> {
  static __device__ __forceinline__ double load(double s, float) { return s; }
  static __device__ __forceinline__ double store(double v, float) { return v; }
};
template <> struct Storage<float, float> {
  static __device__ __forceinline__ float load(float s, float) { return s; }
  static __device__ __forceinline__ float store(float v, float) { return v; }
};
// half storage with a per-field scale: value = half * scale
template <> struct Storage<__half, float> {
  static __device__ __forceinline__ float load(__half s, float scale) { return __half2float(s) * scale; }
  static __device__ __forceinline__ __half store(float v, float inv_scale) {
    return __float2half_rn(v * inv_scale);
  }
};

// precision index -> (policy, storage)
template <int P> struct Precision;
template <> struct Precision<0> { using M = F64Exact; using S = double; };
template <> struct Precision<1> { using M = F64Fast; using S = double; };
template <> struct Precision<2> { using M = F32; using S = float; };
template <> struct Precision<3> { using M = F32; using S = __half; };

// ---------------------------------------------------------------------------
// periodic index arithmetic (in-kernel wrap instead of halo buffers)
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ int wrap(int p, int n) {
  if constexpr (D == 0) {
    return p;
  } else if constexpr (D > 0) {
    const int i = p + D;
    return i >= n ? i - n : i;
  } else {
    const int i = p + D;
    return i < 0 ? i + n : i;
  }
}

// periodic wrap for offsets up to twice the axis length (adjoint cursors
// combine the stencil reach with the roll)
template <int D>
__device__ __forceinline__ int wrap2(int p, int n) {
  if constexpr (D >= -1 && D <= 1) {
    return wrap<D>(p, n);
  } else if constexpr (D > 0) {
    int i = p + D;
    i = i >= n ? i - n : i;
    return i >= n ? i - n : i;
  } else {
    int i = p + D;
    i = i < 0 ? i + n : i;
    return i < 0 ? i + n : i;
  }
}

// Every buffer a kernel reads is read-only for that launch (the stages of a
// step write only arrays that later launches read), so loads go through the
// non-coherent path and may be scheduled ahead of the launch's stores.
template <class X>
__device__ __forceinline__ X ro_load(const X* p) { return __ldg(p); }

// Accessor of the generic stage kernel: global loads at p + D, stores of the
// new state at p + shift (the reference's per-step roll, Templates.hs:346).
template <class S, class T, int DIM, int SHIFT>
struct GlobalAccess {
  const FgbLaunch& L;
  int p0, p1, p2;

  __device__ __forceinline__ uint32_t lin(int i0, int i1, int i2) const {
    return ((uint32_t)i0 * (uint32_t)L.n[1] + (uint32_t)i1) * (uint32_t)L.n[2] + (uint32_t)i2;
  }
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    const S* a = static_cast<const S*>(L.in[F]);
    const uint32_t k = lin(wrap<D0>(p0, L.n[0]), wrap<D1>(p1, L.n[1]), wrap<D2>(p2, L.n[2]));
    return Storage<S, T>::load(ro_load(a + k), L.scale[F]);
  }
  template <int K, int D0, int D1, int D2>
  __device__ __forceinline__ T ldm() const {
    const T* a = static_cast<const T*>(L.mid[K]);
    return ro_load(a + lin(wrap<D0>(p0, L.n[0]), wrap<D1>(p1, L.n[1]), wrap<D2>(p2, L.n[2])));
  }
  template <int F>
  __device__ __forceinline__ void st(T v) const {
    S* a = static_cast<S*>(L.out[F]);
    const int i0 = DIM >= 3 ? wrap<SHIFT>(p0, L.n[0]) : p0;
    const int i1 = DIM >= 2 ? wrap<SHIFT>(p1, L.n[1]) : p1;
    const int i2 = wrap<SHIFT>(p2, L.n[2]);
    a[lin(i0, i1, i2)] = Storage<S, T>::store(v, L.inv_scale[F]);
  }
  template <int K>
  __device__ __forceinline__ void stm(T v) const {
    static_cast<T*>(L.mid[K])[lin(p0, p1, p2)] = v;
  }
};

// Accessor of the adjoint kernel: the forward state u_n at q + D (in),
// the adjoint state lambda_{n+1} at q + D (mid[f]) and the new adjoint
// lambda_n at q (out).  No roll: the roll is folded into the cursors of the
// lambda loads by the generator.
template <class S, class T>
struct AdjointAccess {
  const FgbLaunch& L;
  int p0, p1, p2;

  __device__ __forceinline__ uint32_t lin(int i0, int i1, int i2) const {
    return ((uint32_t)i0 * (uint32_t)L.n[1] + (uint32_t)i1) * (uint32_t)L.n[2] + (uint32_t)i2;
  }
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    const S* a = static_cast<const S*>(L.in[F]);
    return Storage<S, T>::load(
        ro_load(a + lin(wrap2<D0>(p0, L.n[0]), wrap2<D1>(p1, L.n[1]), wrap2<D2>(p2, L.n[2]))), L.scale[F]);
  }
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ldl() const {
    const S* a = static_cast<const S*>(L.mid[F]);
    return Storage<S, T>::load(
        ro_load(a + lin(wrap2<D0>(p0, L.n[0]), wrap2<D1>(p1, L.n[1]), wrap2<D2>(p2, L.n[2]))), 1.0f);
  }
  template <int F>
  __device__ __forceinline__ void stl(T v) const {
    static_cast<S*>(L.out[F])[lin(p0, p1, p2)] = Storage<S, T>::store(v, 1.0f);
  }
};

constexpr int kBlockX = 128;

// One evaluation of a stage functor at the access's point.  In the
// bit-faithful FP64 policy a warp in which any lane met an operand outside a
// shortened form's window evaluates the functor again with the plain IEEE
// operations: it reads the same inputs and overwrites the same outputs.
template <class M, class F, class A>
__device__ __forceinline__ void eval(const A& a, const typename M::U* __restrict__ U) {
  const bool ok = F::template run<M>(a, U);
  if constexpr (M::kChecked) {
    if (__any_sync(__activemask(), !ok)) F::template run<typename M::Ieee>(a, U);
  } else {
    (void)ok;
  }
}

// One thread per grid point of RPT consecutive rows (the middle axis); x
// covers the contiguous (last) axis.  With RPT > 1 a thread has the loads of
// several points in flight at once, which is what a memory-bound FP32/FP16
// step needs to cover the HBM latency.
// (Capping the FP64 stages' registers for more resident blocks was measured
// and lost: HLLD FP64 0.212 GLUP/s uncapped, 0.203 at 128 registers, 0.193
// at 102; Gray-Scott FP64 16.64 at 38 registers (12 blocks per SM), 16.60 at
// 32 (16 blocks, 12 bytes spilled).)
template <class M, class S, int DIM, int SHIFT, class Stage, int RPT>
__global__ void __launch_bounds__(kBlockX) stage_kernel(const __grid_constant__ FgbLaunch L) {
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (p2 >= L.n[2]) return;
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int p1 = (int)blockIdx.y * RPT + r;
    if (RPT > 1 && p1 >= L.n[1]) break;
    GlobalAccess<S, typename M::T, DIM, SHIFT> a{L, (int)blockIdx.z, p1, p2};
    eval<M, Stage>(a, static_cast<const typename M::U*>(L.uniforms));
  }
}

template <class M, class S, class Adj, int RPT>
__global__ void __launch_bounds__(kBlockX) adjoint_kernel(const __grid_constant__ FgbLaunch L) {
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (p2 >= L.n[2]) return;
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int p1 = (int)blockIdx.y * RPT + r;
    if (RPT > 1 && p1 >= L.n[1]) break;
    AdjointAccess<S, typename M::T> a{L, (int)blockIdx.z, p1, p2};
    eval<M, Adj>(a, static_cast<const typename M::U*>(L.uniforms));
  }
}

// rows per thread: several for the memory-bound FP32/FP16 forms (four for
// single-kernel steps, two for the larger stages of multi-stage programs),
// one for FP64, which is bound by the FP64 pipe (two or four rows gave
// Gray-Scott the same 17.2 GLUP/s)
template <int P, bool Light>
constexpr int rows_per_thread() { return P >= 2 ? (Light ? 4 : 2) : 1; }

template <int P, class Adj>
cudaError_t launch_adjoint(const FgbLaunch* L, cudaStream_t stream) {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  constexpr int R = rows_per_thread<P, true>();
  const int bx = L->n[2] >= kBlockX ? kBlockX : ((L->n[2] + 31) / 32) * 32;
  dim3 grid((L->n[2] + bx - 1) / bx, (L->n[1] + R - 1) / R, L->n[0]);
  adjoint_kernel<M, S, Adj, R><<<grid, bx, 0, stream>>>(*L);
  return cudaGetLastError();
}

template <class Prog, int P, class Stage, class M = typename Precision<P>::M>
cudaError_t launch_stage(const FgbLaunch* L, cudaStream_t stream) {
  using S = typename Precision<P>::S;
  constexpr int R = rows_per_thread<P, Prog::kStages == 1 && Prog::kMids == 0>();
  const int bx = L->n[2] >= kBlockX ? kBlockX : ((L->n[2] + 31) / 32) * 32;
  dim3 grid((L->n[2] + bx - 1) / bx, (L->n[1] + R - 1) / R, L->n[0]);
  stage_kernel<M, S, Prog::kDim, Prog::kShift, Stage, R><<<grid, bx, 0, stream>>>(*L);
  return cudaGetLastError();
}

template <class Prog, class... Stages>
struct ProgramBuilder;
}  // namespace fgb
#include "fgb_fused.cuh"
namespace fgb {

template <class Prog, class Stage0, class... Rest>
struct FusedFill {
  template <int P>
  static void fill(FgbProgramDesc& d) {
    if constexpr (Prog::kDim == 2 && Prog::kStages == 1 && Prog::kMids == 0) {
      // (tile x, tile y, steps, rows per thread, thread rows).  The
      // warp-aligned shapes keep the first step's region (tile + 2(K-1)R)
      // within one pass of the CTA's rows and within whole 32-lane passes.
      constexpr int R = Prog::kReach;
      const FgbFusedVariant v[] = {
          Tb2dVariant<Prog, P, Stage0, 64, 32, 2>::describe(),
          Tb2dVariant<Prog, P, Stage0, 64, 32, 4>::describe(),
          Tb2dVariant<Prog, P, Stage0, 64 - 6 * R, 32 - 6 * R, 4, 4>::describe(),
          Tb2dVariant<Prog, P, Stage0, 64 - 6 * R, 64 - 6 * R, 4, 4, 16>::describe(),
          Tb2dVariant<Prog, P, Stage0, 64, 32, 4, 4>::describe(),
          Tb2dVariant<Prog, P, Stage0, 64 - 2 * R, 64 - 2 * R, 2, 4, 16>::describe(),
          Tb2dVariant<Prog, P, Stage0, 64 - 14 * R, 64 - 14 * R, 8, 4, 16>::describe(),
          // tiles whose halo is inside the grid arrive by TMA (64 x 64 boxes)
          Tb2dVariant<Prog, P, Stage0, 64 - 8 * R, 64 - 8 * R, 4, 4, 16, R == 1 && P <= 2>::describe(),
      };
      d.nfused[P] = (int)(sizeof v / sizeof v[0]);
      for (int i = 0; i < d.nfused[P]; ++i) d.fused[P][i] = v[i];
      if constexpr (P == 0 || P == 2) {
        const FgbBatchVariant b[] = {
            Tb2dBatchVariant<Prog, P, Stage0, 64, 32, 1>::describe(),
            Tb2dBatchVariant<Prog, P, Stage0, 64, 32, 4>::describe(),
            Tb2dBatchVariant<Prog, P, Stage0, 64 - 2 * R, 32 - 2 * R, 2, 4>::describe(),
            Tb2dBatchVariant<Prog, P, Stage0, 64 - 6 * R, 32 - 6 * R, 4, 4>::describe(),
            Tb2dBatchVariant<Prog, P, Stage0, 64 - 6 * R, 64 - 6 * R, 4, 4, 16>::describe(),
            Tb2dBatchVariant<Prog, P, Stage0, 64 - 14 * R, 64 - 14 * R, 8, 4, 16>::describe(),
        };
        d.nbatch[P] = (int)(sizeof b / sizeof b[0]);
        for (int i = 0; i < d.nbatch[P]; ++i) d.batch[P][i] = b[i];
      } else {
        d.nbatch[P] = 0;
      }
    } else if constexpr (Prog::kDim == 3 && Prog::kStages == 1 && Prog::kMids == 0) {
      // tile widths with tile + 2 * halo a multiple of the warp width, so
      // that the 32-lane rows of the CTA cover each level without idle lanes
      constexpr int R = Prog::kReach;
      const FgbFusedVariant v[] = {
          Tb3dVariant<Prog, P, Stage0, 64 - 4 * R, 16, 2>::describe(),
          Tb3dVariant<Prog, P, Stage0, 64 - 8 * R, 24, 4>::describe(),
          Tb3dVariant<Prog, P, Stage0, 64 - 8 * R, 16, 4>::describe(),
          // planes arrive by TMA where the tile's halo is inside the grid
          // (K = 2 with a 4-point halo in x and y, so boxes start aligned)
          Tb3dVariant<Prog, P, Stage0, 56, 24, 2, R == 1 && P <= 2, R == 1 ? 4 : 2 * R>::describe(),
          Tb3dVariant<Prog, P, Stage0, 64 - 4 * R, 24, 2>::describe(),
          Tb3dVariant<Prog, P, Stage0, 64 - 16 * R, 16, 8>::describe(),
      };
      int count = (int)(sizeof v / sizeof v[0]);
      for (int i = 0; i < count; ++i) d.fused[P][i] = v[i];
      // one step per launch on four-point row vectors (FP32 and FP16 storage,
      // star stencils of reach 1 rolled by one point)
      if constexpr ((P == 2 || P == 3) && Prog::kStar && Prog::kReach == 1 && Prog::kShift == 1) {
        d.fused[P][count++] = Quad3dVariant<Prog, P, Stage0, 2, 4>::describe();
        d.fused[P][count++] = Quad3dVariant<Prog, P, Stage0, 4, 2>::describe();
        // the same vectors, a chunk of planes per CTA through a shared-memory ring
        d.fused[P][count++] = Zring3dVariant<Prog, P, Stage0, 2, 4, 3>::describe();
        d.fused[P][count++] = Zring3dVariant<Prog, P, Stage0, 2, 8, 3>::describe();
        d.fused[P][count++] = Zring3dVariant<Prog, P, Stage0, 1, 8, 4>::describe();
        d.fused[P][count++] = Zring3dVariant<Prog, P, Stage0, 4, 4, 2>::describe();
      }
      d.nfused[P] = count;
      d.nbatch[P] = 0;
    } else if constexpr (Prog::kDim == 3 && Prog::kStages > 1 && (P == 2 || P == 3)) {
      // multi-stage steps in one launch, the stages' arrays in shared memory
      const FgbFusedVariant v[] = {
          Ms3dVariant<Prog, P, 16, 16, Stage0, Rest...>::describe(),
          Ms3dVariant<Prog, P, 12, 12, Stage0, Rest...>::describe(),
          Ms3dVariant<Prog, P, 8, 16, Stage0, Rest...>::describe(),
          Ms3dVariant<Prog, P, 8, 8, Stage0, Rest...>::describe(),
      };
      d.nfused[P] = (int)(sizeof v / sizeof v[0]);
      for (int i = 0; i < d.nfused[P]; ++i) d.fused[P][i] = v[i];
      d.nbatch[P] = 0;
    } else {
      d.nfused[P] = 0;
      d.nbatch[P] = 0;
    }
  }
};

template <class Adj>
struct AdjointFill {
  static void fill(FgbProgramDesc& d) {
    if constexpr (std::is_same<Adj, void>::value) {
      for (int p = 0; p < FGB_NUM_PRECISIONS; ++p) d.adjoint[p] = nullptr;
    } else {
      d.adjoint[0] = &launch_adjoint<0, Adj>;
      d.adjoint[1] = &launch_adjoint<1, Adj>;
      d.adjoint[2] = &launch_adjoint<2, Adj>;
      d.adjoint[3] = nullptr;   // FP16 storage has no adjoint
    }
  }
};

// ---------------------------------------------------------------------------
// adjoint of multi-stage steps
// ---------------------------------------------------------------------------
// Partial-sum pass: the stage's forward at p (its stores are dropped), the
// adjoints of its outputs at p, and one partial sum per (input, cursor).
template <class S, class T, int DIM, int SHIFT>
struct AdjPartialAccess {
  const FgbAdjLaunch& L;
  int p0, p1, p2;
  __device__ __forceinline__ uint32_t lin(int i0, int i1, int i2) const {
    return ((uint32_t)i0 * (uint32_t)L.n[1] + (uint32_t)i1) * (uint32_t)L.n[2] + (uint32_t)i2;
  }
  template <int D0, int D1, int D2>
  __device__ __forceinline__ uint32_t at() const {
    return lin(wrap2<D0>(p0, L.n[0]), wrap2<D1>(p1, L.n[1]), wrap2<D2>(p2, L.n[2]));
  }
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ld() const {
    return Storage<S, T>::load(ro_load(static_cast<const S*>(L.u[F]) + at<D0, D1, D2>()), L.scale[F]);
  }
  template <int K, int D0, int D1, int D2>
  __device__ __forceinline__ T ldm() const {
    return ro_load(static_cast<const T*>(L.mid[K]) + at<D0, D1, D2>());
  }
  template <int F>
  __device__ __forceinline__ void st(T) const {}
  template <int K>
  __device__ __forceinline__ void stm(T) const {}
  template <int F, int D0, int D1, int D2>
  __device__ __forceinline__ T ldl() const {
    return Storage<S, T>::load(ro_load(static_cast<const S*>(L.lnext[F]) + at<D0, D1, D2>()), 1.0f);
  }
  template <int K>
  __device__ __forceinline__ T ldlm() const {
    return ro_load(static_cast<const T*>(L.lmid[K]) + lin(p0, p1, p2));
  }
  // partial sum J of this kernel: every partial-sum kernel of a stage owns
  // its sums, so nothing here reads a sum back (the gather adds the kernels'
  // sums of the same array and cursor)
  template <int J>
  __device__ __forceinline__ void stp(T v) const {
    static_cast<T*>(L.pair[J])[lin(p0, p1, p2)] = v;
  }
};

// Gather pass: lambda of each input array at q from the partial sums at q - c.
template <class S, class T>
struct AdjGatherAccess {
  const FgbAdjLaunch& L;
  int p0, p1, p2;
  __device__ __forceinline__ uint32_t lin(int i0, int i1, int i2) const {
    return ((uint32_t)i0 * (uint32_t)L.n[1] + (uint32_t)i1) * (uint32_t)L.n[2] + (uint32_t)i2;
  }
  template <int J, int D0, int D1, int D2>
  __device__ __forceinline__ T ldp() const {
    return ro_load(static_cast<const T*>(L.pair[J]) +
                   lin(wrap2<D0>(p0, L.n[0]), wrap2<D1>(p1, L.n[1]), wrap2<D2>(p2, L.n[2])));
  }
  template <int G, bool FIRST>
  __device__ __forceinline__ void accs(T v) const {
    S* a = static_cast<S*>(L.lprev[G]) + lin(p0, p1, p2);
    if (!FIRST) v = v + Storage<S, T>::load(*a, 1.0f);
    *a = Storage<S, T>::store(v, 1.0f);
  }
  template <int K, bool FIRST>
  __device__ __forceinline__ void accm(T v) const {
    T* a = static_cast<T*>(L.lmid[K]) + lin(p0, p1, p2);
    if (!FIRST) v = v + *a;
    *a = v;
  }
};

// the partial-sum kernels of one stage, launched in order
template <class... Parts>
struct AdjParts {};

// A partial-sum functor evaluated at its point for sum J alone: the other
// sums are dropped, so only J's part of the functor survives compilation.
template <class S, class T, int DIM, int SHIFT, int J>
struct AdjCaptureAccess : AdjPartialAccess<S, T, DIM, SHIFT> {
  T* out;
  template <int J2>
  __device__ __forceinline__ void stp(T v) const {
    if constexpr (J2 == J) *out = v;
  }
};

// Gather pass of a stage whose partial sums are its outputs' adjoints times
// constants (a linear stage): instead of reading the stored sum J at q + D
// it evaluates the stage's partial-sum functors there.
template <class M, class S, class T, int DIM, int SHIFT, class Parts>
struct AdjDirectAccess;
template <class M, class S, class T, int DIM, int SHIFT, class... Parts>
struct AdjDirectAccess<M, S, T, DIM, SHIFT, AdjParts<Parts...>> : AdjGatherAccess<S, T> {
  template <int J, int D0, int D1, int D2>
  __device__ __forceinline__ T ldp() const {
    const FgbAdjLaunch& L = this->L;
    T v = T(0);
    const AdjCaptureAccess<S, T, DIM, SHIFT, J> c{
        {L, wrap2<D0>(this->p0, L.n[0]), wrap2<D1>(this->p1, L.n[1]), wrap2<D2>(this->p2, L.n[2])}, &v};
    const typename M::U* U = static_cast<const typename M::U*>(L.uniforms);
    (Parts::template run<M>(c, U), ...);
    return v;
  }
};

// One thread per point of RPT consecutive rows, as in stage_kernel.
template <class M, class Acc, class F, int RPT>
__global__ void __launch_bounds__(kBlockX) adj_stage_kernel(const __grid_constant__ FgbAdjLaunch L) {
  const int p2 = blockIdx.x * blockDim.x + threadIdx.x;
  if (p2 >= L.n[2]) return;
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int p1 = (int)blockIdx.y * RPT + r;
    if (RPT > 1 && p1 >= L.n[1]) break;
    Acc a{L, (int)blockIdx.z, p1, p2};
    eval<M, F>(a, static_cast<const typename M::U*>(L.uniforms));
  }
}

template <class M, class Acc, class F, int P>
cudaError_t launch_adj_rows(const FgbAdjLaunch* L, cudaStream_t stream) {
  constexpr int R = rows_per_thread<P, false>();
  const int bx = L->n[2] >= kBlockX ? kBlockX : ((L->n[2] + 31) / 32) * 32;
  dim3 grid((L->n[2] + bx - 1) / bx, (L->n[1] + R - 1) / R, L->n[0]);
  adj_stage_kernel<M, Acc, F, R><<<grid, bx, 0, stream>>>(*L);
  return cudaGetLastError();
}

template <class Prog, int P, class F, bool Gather>
cudaError_t launch_adj_stage(const FgbAdjLaunch* L, cudaStream_t stream) {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using T = typename M::T;
  using Acc = typename std::conditional<Gather, AdjGatherAccess<S, T>,
                                        AdjPartialAccess<S, T, Prog::kDim, Prog::kShift>>::type;
  return launch_adj_rows<M, Acc, F, P>(L, stream);
}

template <class Prog, int P, class Parts, class F>
cudaError_t launch_adj_direct(const FgbAdjLaunch* L, cudaStream_t stream) {
  using M = typename Precision<P>::M;
  using S = typename Precision<P>::S;
  using T = typename M::T;
  return launch_adj_rows<M, AdjDirectAccess<M, S, T, Prog::kDim, Prog::kShift, Parts>, F, P>(L, stream);
}

template <class Partial, class Gather>
struct AdjointStagePair {
  using P1 = Partial;
  using P2 = Gather;
};
// Rec::kStage[s]: the adjoint step recomputes stage s's forward arrays
template <class Rec, class... Pairs>
struct AdjointStages {};
template <class Prog, int P, class List>
struct PartialLauncher;
template <class Prog, int P, class... Parts>
struct PartialLauncher<Prog, P, AdjParts<Parts...>> {
  static constexpr int kCount = sizeof...(Parts);
  static cudaError_t launch(const FgbAdjLaunch* L, cudaStream_t stream) {
    cudaError_t e = cudaSuccess;
    ((e = (e == cudaSuccess ? launch_adj_stage<Prog, P, Parts, false>(L, stream) : e)), ...);
    return e;
  }
};
// the two passes of one stage's adjoint: partial sums and gather, or for a
// linear stage the gather alone, forming its partial sums itself.  Only the
// FP32 forms do the latter: there the stage's adjoint is bound by HBM and
// the direct gather moves a quarter of the bytes (HLLC's update stage:
// 0.94 -> 0.32 ms at 256^3), while the FP64 form is bound by the FP64 pipe
// and forming the sums once per cursor costs more than storing them
// (2.17 -> 2.41 ms).
template <class Prog, int P, class Pair>
struct StagePassLaunchers {
  using P1 = typename Pair::P1;
  static constexpr bool kDirect = P1::kDirect && std::is_same<typename Precision<P>::M::T, float>::value;
  static constexpr int kPartials = kDirect ? 0 : PartialLauncher<Prog, P, typename P1::Parts>::kCount;
  static cudaError_t none(const FgbAdjLaunch*, cudaStream_t) { return cudaSuccess; }
  static FgbAdjLaunchFn partial() {
    if constexpr (kDirect) return &none;
    else return &PartialLauncher<Prog, P, typename P1::Parts>::launch;
  }
  static FgbAdjLaunchFn gather() {
    if constexpr (kDirect) return &launch_adj_direct<Prog, P, typename P1::Parts, typename Pair::P2>;
    else return &launch_adj_stage<Prog, P, typename Pair::P2, true>;
  }
};

template <class Prog, class A>
struct StageAdjointFill {
  static void fill(FgbProgramDesc& d) {
    for (int p = 0; p < FGB_NUM_PRECISIONS; ++p)
      for (int s = 0; s < FGB_MAX_STAGES; ++s) d.adj_partial[p][s] = d.adj_gather[p][s] = nullptr;
  }
};
// FP64 (exact rounding) and FP32 forms; the others have no adjoint
template <class Prog, class Rec, class... Pairs>
struct StageAdjointFill<Prog, AdjointStages<Rec, Pairs...>> {
  static void fill(FgbProgramDesc& d) {
    static_assert(sizeof...(Pairs) == Prog::kStages, "one adjoint pair per stage");
    const int pairs[] = {Pairs::P1::kPairs...};
    const int parts[] = {StagePassLaunchers<Prog, 0, Pairs>::kPartials...};
    const FgbAdjLaunchFn p0[] = {StagePassLaunchers<Prog, 0, Pairs>::partial()...};
    const FgbAdjLaunchFn g0[] = {StagePassLaunchers<Prog, 0, Pairs>::gather()...};
    const FgbAdjLaunchFn p2[] = {StagePassLaunchers<Prog, 2, Pairs>::partial()...};
    const FgbAdjLaunchFn g2[] = {StagePassLaunchers<Prog, 2, Pairs>::gather()...};
    for (int p = 0; p < FGB_NUM_PRECISIONS; ++p)
      for (int s = 0; s < FGB_MAX_STAGES; ++s) d.adj_partial[p][s] = d.adj_gather[p][s] = nullptr;
    static_assert(((Pairs::P1::kPairs <= FGB_MAX_PAIRS) && ...), "too many (array, cursor) pairs in a stage");
    for (int s = 0; s < (int)sizeof...(Pairs); ++s) {
      d.adj_pairs[s] = pairs[s];
      d.adj_parts[s] = parts[s];
      d.adj_recompute[s] = Rec::kStage[s] ? 1 : 0;
      d.adj_partial[0][s] = p0[s];
      d.adj_gather[0][s] = g0[s];
      d.adj_partial[2][s] = p2[s];
      d.adj_gather[2][s] = g2[s];
    }
  }
};

// Programs whose forward step stores other arrays than the program's own
// (see the generator's store_shared_operands) carry the program's own
// forward stages for the adjoint: Prog::AdjProg and Prog::AdjStages.
template <class... S>
struct StageTypes {};
template <class P, class = void>
struct AdjStagesOf {
  using type = void;
};
template <class P>
struct AdjStagesOf<P, std::void_t<typename P::AdjStages>> {
  using type = typename P::AdjStages;
};
template <class Prog, class List>
struct AdjStagesFill {
  static void fill(FgbProgramDesc&) {}
};
template <class Prog, class... S>
struct AdjStagesFill<Prog, StageTypes<S...>> {
  using AP = typename Prog::AdjProg;
  static_assert(sizeof...(S) == Prog::kStages && AP::kStages == Prog::kStages, "the adjoint's stages are the step's");
  static_assert(AP::kMids <= FGB_MAX_MIDS, "too many intermediate arrays");
  template <int P>
  static void fill_p(FgbProgramDesc& d) {
    FgbStageLaunch l[] = {&launch_stage<AP, P, S>...};
    for (int i = 0; i < (int)sizeof...(S); ++i) d.adj_launch[P][i] = l[i];
  }
  static void fill(FgbProgramDesc& d) {
    fill_p<0>(d);
    fill_p<1>(d);
    fill_p<2>(d);
    fill_p<3>(d);
    d.nmids_adj = AP::kMids;
  }
};

template <class Prog, class... Stages>
struct ProgramBuilder {
  template <int P>
  static void fill(FgbProgramDesc& d) {
    FgbStageLaunch l[] = {&launch_stage<Prog, P, Stages>...};
    for (int i = 0; i < (int)sizeof...(Stages); ++i) {
      d.launch[P][i] = l[i];
      d.adj_launch[P][i] = l[i];
    }
  }
  static FgbProgramDesc make(const char* name, const char* const* fields) {
    static_assert(sizeof...(Stages) == Prog::kStages, "stage count");
    static_assert(Prog::kStages <= FGB_MAX_STAGES, "too many stages");
    static_assert(Prog::kFields <= FGB_MAX_FIELDS, "too many fields");
    static_assert(Prog::kMids <= FGB_MAX_MIDS, "too many intermediate arrays");
    FgbProgramDesc d = {};
    d.name = name;
    d.dim = Prog::kDim;
    d.nfields = Prog::kFields;
    d.nmids = Prog::kMids;
    d.nmids_adj = Prog::kMids;
    d.nstages = Prog::kStages;
    d.sleeve = Prog::kSleeve;
    d.shift = Prog::kShift;
    d.reach = Prog::kReach;
    d.nuniforms = Prog::kUniforms;
    d.field_names = fields;
    fill<0>(d);
    fill<1>(d);
    fill<2>(d);
    fill<3>(d);
    {
      FgbStageLaunch l[] = {&launch_stage<Prog, 0, Stages, F64ExactP2>...};
      for (int i = 0; i < (int)sizeof...(Stages); ++i) d.launch_p2[i] = l[i];
      static_assert(sizeof(Prog::kDivisors) / sizeof(int) <= FGB_MAX_DIVISORS, "too many divisors");
      d.ndivisors = Prog::kNumDivisors;
      for (int i = 0; i < Prog::kNumDivisors; ++i) d.divisors[i] = Prog::kDivisors[i];
    }
    FusedFill<Prog, Stages...>::template fill<0>(d);
    FusedFill<Prog, Stages...>::template fill<1>(d);
    FusedFill<Prog, Stages...>::template fill<2>(d);
    FusedFill<Prog, Stages...>::template fill<3>(d);
    AdjointFill<typename Prog::Adjoint>::fill(d);
    StageAdjointFill<Prog, typename Prog::StageAdjoint>::fill(d);
    AdjStagesFill<Prog, typename AdjStagesOf<Prog>::type>::fill(d);
    return d;
  }
};

}  // namespace fgb

#define FGB_DEFINE_PROGRAM(NAME, PROG, FIELDS, ...)                                   \
  extern "C" const FgbProgramDesc* fgb_program_##NAME(void) {                         \
    static const FgbProgramDesc d = fgb::ProgramBuilder<PROG, __VA_ARGS__>::make(#NAME, FIELDS); \
    return &d;                                                                         \
  }
