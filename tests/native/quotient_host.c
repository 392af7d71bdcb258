/* Host check of the bit-faithful FP64 policy's quotient with its last
 * rounding step on the integer pipe (fgb::F64Exact::round_quotient):
 * y = RN(1/c), q0 = RN(x*y), r = x - q0*c (one fma, exact), and then, where
 * q0 lies at least two ulps inside its binade, RN(x/c) is q0 or the
 * neighbour towards x/c: the neighbour when |r| > |c| * ulp(q0) / 2, the
 * even one of the two when |r| equals it.  The same integer steps as the
 * device code, on the host's correctly rounded fma; compared with the
 * host's IEEE division wherever the form applies.
 * Cases: random operands over the division windows, numerators built so
 * that x/c lies next to the midpoint between two doubles (an exact midpoint
 * is not a quotient of two doubles), exact quotients, and quotients within
 * a few ulps of a power of two, where the form does not apply (there the
 * neighbours below are half as far apart).
 * Numerators below the window (subnormal ones included) whose quotient is
 * normal are scaled by 2^256 on the integer pipe first and the quotient
 * scaled back, as on the device.
 * Prints "mismatches applied not_applied tiny_mismatches tiny_cases". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s = 0x243f6a8885a308d3ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double from(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

/* the device's round_quotient, step for step */
static double round_quotient(double x, double c, double q0, double r, int* fits) {
  const uint64_t qb = bits(q0), rb = bits(r), cb = bits(c);
  const unsigned qhi = (unsigned)(qb >> 32), qlo = (unsigned)qb;
  const unsigned rhi = (unsigned)(rb >> 32), rlo = (unsigned)rb;
  const unsigned chi = (unsigned)(cb >> 32), clo = (unsigned)cb;
  const unsigned eq = (qhi >> 20) & 0x7ffu, ec = (chi >> 20) & 0x7ffu;
  const uint64_t m = ((uint64_t)(qhi & 0xfffffu) << 32) | qlo;
  const int et = (int)ec + (int)eq - 1076;
  const int zero = ((bits(x) << 1) == 0);
  *fits = zero || ((m - 2u <= (1ull << 52) - 5u) && (unsigned)(et - 2) <= 2044u);
  const uint64_t t = ((uint64_t)((chi & 0xfffffu) | ((unsigned)et << 20)) << 32) | clo;
  const uint64_t a = ((uint64_t)(rhi & 0x7fffffffu) << 32) | rlo;
  const int step = a > t || (a == t && (qlo & 1u));
  const int up = ((rhi ^ chi ^ qhi) >> 31) == 0;
  const uint64_t res = qb + (step ? (up ? 1ull : ~0ull) : 0ull);
  return zero ? q0 : from(res);
}

/* the device's path for numerators below the window (F64Exact::divu_outside),
   step for step: where x/c is at least 2^-1022, x * 2^256 on the integer
   pipe, the quotient, and the quotient scaled back.  Returns 0 where the
   device would take the IEEE division instead. */
static double scale_up(double x, int k) {
  uint64_t b = bits(x);
  const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
  if (ex != 0u) {
    b += (uint64_t)k << 52;
  } else {
    const uint64_t m = b & 0x000fffffffffffffull;
    const int sh = __builtin_clzll(m) - 11;
    b = (b & 0x8000000000000000ull) | ((uint64_t)(k + 1 - sh) << 52) | ((m << sh) & 0x000fffffffffffffull);
  }
  return from(b);
}
static int outside(double x, double c, double* out) {
  const uint64_t xb = bits(x), cb = bits(c);
  const unsigned ex = (unsigned)(xb >> 52) & 0x7ffu, ec = (unsigned)(cb >> 52) & 0x7ffu;
  const uint64_t mx = xb & 0x000fffffffffffffull;
  const int eff = ex != 0u ? (int)ex : 12 - __builtin_clzll(mx ? mx : 1);
  if (!(ec - 923u <= 200u && ex < 63u && mx + ex != 0ull && eff + 1021 >= (int)ec)) return 0;
  const double xs = scale_up(x, 256);
  if (bits(xs) != bits(ldexp(x, 256))) return -1;   /* the scaling itself is wrong */
  const double y = 1.0 / c, q0 = xs * y, r = fma(-q0, c, xs);
  int fits;
  double q = round_quotient(xs, c, q0, r, &fits);
  if (!fits) q = fma(r, y, q0);
  *out = from(bits(q) - (256ull << 52));
  return 1;
}

static long tiny_bad = 0, tiny_done = 0;

static void check_outside(double x, double c) {
  double q;
  const int k = outside(x, c, &q);
  if (k < 0) {
    ++tiny_bad;
    return;
  }
  if (k == 0) return;
  ++tiny_done;
  tiny_bad += bits(q) != bits(x / c);
}

static double operand(int lo, int hi) {
  const int e = lo + (int)(rnd() % (uint64_t)(hi - lo + 1));
  return from(((rnd() & 1) << 63) | ((uint64_t)e << 52) | (rnd() & 0x000fffffffffffffull));
}

static long bad = 0, applied = 0, skipped = 0;

static void check(double x, double c) {
  const double y = 1.0 / c, q0 = x * y, r = fma(-q0, c, x);
  int fits;
  const double q = round_quotient(x, c, q0, r, &fits);
  if (!fits) {
    ++skipped;
    return;
  }
  ++applied;
  bad += bits(q) != bits(x / c);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 10000000;
  for (long i = 0; i < n; ++i) {
    /* constants in [2^-100, 2^100], numerators with the quotient's exponent
       in [-1000, 1000] */
    const double c = operand(1023 - 100, 1023 + 100);
    const int ec = (int)((bits(c) >> 52) & 0x7ff) - 1023;
    const int lo = -960 > ec - 1000 ? -960 : ec - 1000, hi = 960 < ec + 1000 ? 960 : ec + 1000;
    check(operand(1023 + lo, 1023 + hi), c);
    /* a shared reciprocal: both operands in [2^-400, 2^400] */
    check(operand(1023 - 400, 1023 + 400), operand(1023 - 400, 1023 + 400));
    /* x/c at or near a midpoint: x = RN((q + ulp(q)/2) * c) and neighbours */
    {
      const double q = operand(1023 - 200, 1023 + 200), cc = operand(1023 - 60, 1023 + 60);
      const double mid = q + 0.5 * (nextafter(q, INFINITY) - q);
      double x = mid * cc;
      for (int k = 0; k < 3; ++k) {
        check(x, cc);
        x = nextafter(x, k ? -INFINITY : INFINITY);
      }
      check(nextafter(mid * cc, -INFINITY), cc);
      /* exact quotients: x = q * c when that product is exact (short mantissas) */
      const double qs = from(bits(q) & 0xfffffff000000000ull), cs = from(bits(cc) & 0xfffffff000000000ull);
      check(qs * cs, cs);
    }
    /* quotients at the edges of a binade: x/c within a few ulps of 2^e,
       from x = RN((2^e + d) * c) with d a random fraction of those ulps */
    {
      const double cc = operand(1023 - 60, 1023 + 60);
      const int e = -100 + (int)(rnd() % 201);
      const double d = ldexp((double)(int64_t)(rnd() % 4096) - 2048.0, e - 52 - 9);   /* |d| < 4 ulp(2^e) */
      const double q = (rnd() & 1) ? -(ldexp(1.0, e) + d) : ldexp(1.0, e) + d;
      check(q * cc, cc);
      check(nextafter(q * cc, INFINITY), cc);
      check(nextafter(q * cc, -INFINITY), cc);
    }
    /* numerators below the window: subnormal and the lowest binades */
    {
      const double cc = operand(1023 - 100, 1023 + 100);
      const uint64_t sb = (rnd() & 1) << 63;
      check_outside(from(sb | ((rnd() & 0x000fffffffffffffull) >> (rnd() % 52))), cc);
      check_outside(from(sb | ((rnd() % 63) << 52) | (rnd() & 0x000fffffffffffffull)), cc);
    }
    /* signed zero numerators */
    if (i % 64 == 0) check(from((rnd() & 1) << 63), operand(1023 - 100, 1023 + 100));
  }
  printf("%ld %ld %ld %ld %ld\n", bad, applied, skipped, tiny_bad, tiny_done);
  return 0;
}
