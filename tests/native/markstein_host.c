/* Host check of the operand windows in which the bit-faithful FP64 policy
 * divides through a reciprocal: y = RN(1/b), q = RN(a*y), e = a - q*b (one
 * fma), result RN(q + e*y), or q itself for a zero numerator.  Inside the
 * windows the result must equal RN(a/b) bit for bit; just below them (tiny
 * numerators) it need not, which is why the device falls back there.
 * The windows: for a grid-independent c in [2^-100, 2^100], numerators of
 * exponent in [-960, 960] whose quotient's exponent is in [-1000, 1000];
 * for a shared reciprocal, both operands in [2^-400, 2^400]; and normal
 * numerators below the first window, scaled by 2^256 into it, whose quotient
 * (exponent at least -1000) is scaled back.
 * Uses the host's correctly rounded fma.  Prints "mismatches_inside outside". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s = 88172645463325252ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double from(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

static double mant_operand(int lo, int hi, int mode) {
  uint64_t m = rnd() & 0x000fffffffffffffull;
  if (mode == 1) m = 0x000fffffffffffffull - (rnd() & 0xffff);   /* top of the binade */
  if (mode == 2) m = rnd() & 0xffff;                              /* bottom */
  int e = lo + (int)(rnd() % (uint64_t)(hi - lo + 1));
  return from(((rnd() & 1) << 63) | ((uint64_t)e << 52) | m);
}

static double corrected(double a, double b, double y) {
  double q = a * y, e = fma(-q, b, a);
  return (bits(a) << 1) == 0 ? q : fma(e, y, q);
}

int main(int argc, char** argv) {
  long n = argc > 1 ? atol(argv[1]) : 10000000;
  long inside = 0, outside = 0;
  for (long i = 0; i < n; ++i) {
    /* divisions by constants: c in [2^-100, 2^100], numerator exponent in
       [-960, 960] with the quotient's exponent in [-1000, 1000] */
    double c = mant_operand(1023 - 100, 1023 + 100, (int)(i % 3));
    int ec = (int)((bits(c) >> 52) & 0x7ff) - 1023;
    int lo = -960 > ec - 1000 ? -960 : ec - 1000, hi = 960 < ec + 1000 ? 960 : ec + 1000;
    double x = (i % 50 == 0) ? from((rnd() & 1) << 63) : mant_operand(1023 + lo, 1023 + hi, (int)(i % 3));
    double r = corrected(x, c, 1.0 / c), w = x / c;
    inside += bits(r) != bits(w);
    /* shared reciprocals: both operands in [2^-400, 2^400] */
    double b = mant_operand(1023 - 400, 1023 + 400, (int)((i / 3) % 3));
    double a = mant_operand(1023 - 400, 1023 + 400, (int)((i / 9) % 3));
    r = corrected(a, b, 1.0 / b);
    w = a / b;
    inside += bits(r) != bits(w);
    /* below the window: subnormal and lowest normal numerators */
    double t = from(((rnd() & 1) << 63) | ((rnd() % 40) << 52) | (rnd() & 0x000fffffffffffffull));
    /* the lowest exponents of the window, against the smallest constants */
    double c2 = mant_operand(1023 - 100, 1023 - 90, (int)(i % 3));
    double x2 = mant_operand(1023 - 960, 1023 - 950, (int)((i / 3) % 3));
    r = corrected(x2, c2, 1.0 / c2);
    w = x2 / c2;
    inside += bits(r) != bits(w);
    /* tiny normal numerators below the window whose quotient is normal:
       scaled by 2^256 into the window and the quotient scaled back */
    double c4 = mant_operand(1023 - 100, 1023 + 100, (int)(i % 3));
    int e4 = (int)((bits(c4) >> 52) & 0x7ff) - 1023;
    int lo4 = -1022 > e4 - 1000 ? -1022 : e4 - 1000;
    if (lo4 <= -961) {
      double x4 = mant_operand(1023 + lo4, 1023 - 961, (int)((i / 3) % 3));
      r = ldexp(corrected(ldexp(x4, 256), c4, 1.0 / c4), -256);
      w = x4 / c4;
      inside += bits(r) != bits(w);
    }
    /* the quotient's lowest exponents: large constants, small numerators */
    double c3 = mant_operand(1023 + 90, 1023 + 100, (int)(i % 3));
    int e3 = (int)((bits(c3) >> 52) & 0x7ff) - 1023;
    double x3 = mant_operand(1023 + e3 - 1000, 1023 + e3 - 990, (int)((i / 3) % 3));
    r = corrected(x3, c3, 1.0 / c3);
    w = x3 / c3;
    inside += bits(r) != bits(w);
    r = corrected(t, c, 1.0 / c);
    w = t / c;
    outside += bits(r) != bits(w);
  }
  printf("%ld %ld\n", inside, outside);
  return 0;
}
