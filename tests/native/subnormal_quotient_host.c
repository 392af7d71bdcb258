/* Host check of the bit-faithful FP64 policy's quotient below 2^-1021
 * (fgb::F64Exact::divu_mixed on its integer-grid lanes): RN(x/c) is
 * N * 2^-1074 for the integer N nearest X/c (ties to even),
 * X = |x| * 2^1074, since the doubles below 2^-1021 lie on that grid.
 * q0 = RN(X * |RN(1/c)|).  Below 2^51, q0 rounded to an integer gives n0
 * within 1 + 2^-52 of X/c, the remainder X - n0*|c| is exact (one fma) and
 * picks N among n0 - 1, n0, n0 + 1.  From 2^51, q0 is within one of its
 * ulps (1/2 or 1) of X/c, so X - q0*|c| is exact and, with q0's own
 * fraction (0 or 1/2), decides N.  The same integer steps as the device
 * code, compared with the host's IEEE division.  Cases: random subnormal
 * and tiny normal numerators against constants in [2^-100, 2^100]
 * wherever the path applies, numerators at the top of its range (q0 from
 * 2^51 to 2^53 - 1), exact quotients, and exact ties (X/c = k + 1/2
 * with c = 3 * 2^j, and with c = 2^j at the top of the range).
 * Prints "mismatches cases upper_cases". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s = 0x452821e638d01377ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double from(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

static int clz64(uint64_t v) { return v ? __builtin_clzll(v) : 64; }

/* the device's divu_sub: nonzero x, c in [2^-100, 2^100], |x/c| < 2^-1021 */
static int applies(double x, double c) {
  const uint64_t xb = bits(x), cb = bits(c);
  const unsigned ex = (unsigned)(xb >> 52) & 0x7ffu, ec = (unsigned)(cb >> 52) & 0x7ffu;
  const uint64_t m = xb & 0x000fffffffffffffull;
  const int eff = ex != 0u ? (int)ex : 12 - clz64(m);
  return ec - 923u <= 200u && ex < 2047u && (m | ex) != 0 && eff - (int)ec <= -1022;
}

/* the device's scale_up<K> of a non-negative x */
static double scale_up(double x, int k) {
  uint64_t b = bits(x);
  const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
  if (ex != 0u) {
    b += (uint64_t)k << 52;
  } else {
    const uint64_t m = b & 0x000fffffffffffffull;
    const int sh = clz64(m) - 11;
    b = ((uint64_t)(k + 1 - sh) << 52) | ((m << sh) & 0x000fffffffffffffull);
  }
  return from(b);
}

static long upper_cases = 0;

/* the device's integer-grid lanes, step for step */
static double sub_quotient(double x, double c, double rc) {
  const uint64_t xb = bits(x), cb = bits(c);
  const double X = scale_up(from(xb & 0x7fffffffffffffffull), 1074);
  const double ac = from(cb & 0x7fffffffffffffffull), ay = from(bits(rc) & 0x7fffffffffffffffull);
  const double q0 = X * ay;
  const uint64_t qb = bits(q0);
  const int e = (int)((qb >> 52) & 0x7ff) - 1023;
  const uint64_t qm = (qb & 0x000fffffffffffffull) | (1ull << 52);
  int sh = 52 - e;
  sh = sh < 1 ? 1 : (sh > 53 ? 53 : sh);
  const uint64_t n0 = e < -1 ? 0ull : (qm + (1ull << (sh - 1))) >> sh;
  const int lead = 63 - clz64(n0 | 1);
  const double nd = n0 == 0 ? 0.0 : from(((uint64_t)(lead + 1023) << 52) | ((n0 << (52 - lead)) & 0x000fffffffffffffull));
  const int upper = e >= 51;
  const int ush = e - 52 < 11 ? e - 52 : 11;
  const uint64_t iq = e >= 52 ? qm << ush : qm >> 1;
  const int halfq = e == 51 && (qm & 1);
  const uint64_t base = upper ? iq : n0;
  upper_cases += upper;
  const double r = fma(-(upper ? q0 : nd), ac, X);
  const uint64_t rb = bits(r), ar = rb & 0x7fffffffffffffffull, half = bits(ac) - (1ull << 52);
  const int rneg = (int)(rb >> 63);
  uint64_t n;
  if (halfq) {
    n = base + (((!rneg && ar != 0) || (ar == 0 && (base & 1))) ? 1ull : 0ull);
  } else {
    const int step = ar > half || (ar == half && (base & 1));
    n = base + (step ? (rneg ? ~0ull : 1ull) : 0ull);
  }
  return from(n | ((xb ^ cb) & 0x8000000000000000ull));
}

static long bad = 0, cases = 0;

static void check(double x, double c) {
  if (!applies(x, c)) return;
  ++cases;
  const double q = sub_quotient(x, c, 1.0 / c);
  if (bits(q) != bits(x / c)) {
    if (bad < 5) printf("# x=%a c=%a got %a want %a\n", x, c, q, x / c);
    ++bad;
  }
}

static double constant(void) {
  const int e = 1023 - 100 + (int)(rnd() % 201);
  return from(((rnd() & 1) << 63) | ((uint64_t)e << 52) | (rnd() & 0x000fffffffffffffull));
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  for (long i = 0; i < n; ++i) {
    const double c = constant();
    const int ec = (int)((bits(c) >> 52) & 0x7ff);
    const uint64_t sg = (rnd() & 1) << 63;
    /* subnormal numerators of every length */
    check(from(sg | ((rnd() & 0x000fffffffffffffull) >> (rnd() % 53))), c);
    /* numerators at the top of the range: biased exponent ec - 1022 and below */
    {
      const int top = ec - 1022 - (int)(rnd() % 6);
      if (top >= 1) check(from(sg | ((uint64_t)top << 52) | (rnd() & 0x000fffffffffffffull)), c);
      else check(from(sg | ((rnd() & 0x000fffffffffffffull) >> (1 - top))), c);
    }
    /* exact quotients: x = N * c * 2^-1074 for small N and c with a short significand */
    {
      const double cs = from(bits(c) & 0xfffffff000000000ull);
      const double X = (double)(rnd() % (1ull << 20)) * from(bits(fabs(cs)) & 0x7ff0000000000000ull) * 0x1p30;
      if (X > 0 && X < 0x1p52) check(from(sg | bits(ldexp(X, -1074))), from(bits(cs) & 0x7ff0000000000000ull));
    }
    /* q0 next to 2^53: the largest significands over the smallest */
    {
      const int j = (int)(rnd() % 40);
      const double cm = from(((uint64_t)(1023 + j) << 52) | (rnd() % 64));
      const int top = 1023 + j - 1022;
      if (top >= 1) check(from(sg | ((uint64_t)top << 52) | (0x000fffffffffffffull - (rnd() % 64))), cm);
    }
    /* ties at the top: c = 2^j (j >= 1), X = (2I + 1) * 2^(j - 1), X/c = I + 1/2, I in [2^50, 2^52) */
    {
      const int j = 1 + (int)(rnd() % 30);
      const uint64_t I = (1ull << 50) + (rnd() % (3ull << 50));
      const double X = ldexp((double)(2 * I + 1), j - 1);
      check(from(sg | bits(ldexp(X, -1074))), ldexp(1.0, j));
      check(from(sg | bits(ldexp(X, -1074))), -ldexp(1.0, j));
    }
    /* ties: c = 3 * 2^j (j >= 1), X = (2k + 1) * 3 * 2^(j - 1), X/c = k + 1/2 */
    {
      const int j = 1 + (int)(rnd() % 20);
      const double ct = 3.0 * ldexp(1.0, j);
      const uint64_t k = rnd() % (1ull << 28);
      const double X = (double)(2 * k + 1) * 3.0 * ldexp(1.0, j - 1);
      check(from(sg | bits(ldexp(X, -1074))), (rnd() & 1) ? -ct : ct);
      check(from(sg | bits(ldexp(X + 1.0, -1074))), ct);
      check(from(sg | bits(ldexp(X - 1.0, -1074))), ct);
    }
  }
  printf("%ld %ld %ld\n", bad, cases, upper_cases);
  return 0;
}
