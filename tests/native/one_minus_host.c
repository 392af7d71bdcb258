/* Host check of the bit-faithful FP64 policy's 1 - x on the integer pipe
 * (fgb::F64Exact::one_minus_exact): for x in [0.5, 2) (sign 0, exponent
 * field 1022 or 1023) 1 - x is exact by Sterbenz's lemma; with
 * x = X * 2^-53 the integer 2^53 - X is normalised by its leading bit.  The
 * same integer steps as the device code, compared with the host's IEEE
 * subtraction.  Cases: random significands in both binades, the ends of the
 * range and their neighbours, x = 1, and significands with a single bit or
 * a run of low bits set (results far below 1).
 * Prints "mismatches window_cases out_of_window_checked". */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s = 0x13198a2e03707344ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double from(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }

static int window(double x) { return (unsigned)(bits(x) >> 53) == 511u; }

/* the device's one_minus_exact, step for step */
static double one_minus_exact(double x) {
  const uint64_t xb = bits(x);
  const unsigned hi = (unsigned)(xb >> 32), lo = (unsigned)xb;
  const uint64_t X = ((((uint64_t)((hi & 0xfffffu) | 0x100000u)) << 32) | lo) << ((hi >> 20) & 1u);
  const int64_t d = (int64_t)(1ull << 53) - (int64_t)X;
  const uint64_t a = d < 0 ? (uint64_t)(-d) : (uint64_t)d;
  const int n = a ? __builtin_clzll(a) : 64;
  const uint64_t b = ((uint64_t)(1032 - n) << 52) + (a << ((n - 11) & 63));
  return from(a == 0 ? 0ull : (b | (d < 0 ? 0x8000000000000000ull : 0ull)));
}

static long bad = 0, cases = 0, outside = 0;

static void check(double x) {
  if (!window(x)) {
    ++outside;
    /* the window test must refuse exactly the values outside [0.5, 2) */
    bad += (x >= 0.5 && x < 2.0);
    return;
  }
  ++cases;
  bad += !(x >= 0.5 && x < 2.0);
  bad += bits(one_minus_exact(x)) != bits(1.0 - x);
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 10000000;
  const double edges[] = {0.5, 1.0, 2.0, 0.25, -0.5, -1.0, 0.0, -0.0};
  for (unsigned i = 0; i < sizeof(edges) / sizeof(edges[0]); ++i) {
    const uint64_t b = bits(edges[i]);
    for (int k = -3; k <= 3; ++k) check(from(b + (uint64_t)(int64_t)k));
  }
  for (long i = 0; i < n; ++i) {
    const uint64_t e = 1022 + (rnd() & 1);
    const uint64_t m = rnd() & 0x000fffffffffffffull;
    check(from((e << 52) | m));
    check(from((e << 52) | (1ull << (rnd() % 52))));
    check(from((e << 52) | (m >> (rnd() % 53))));
    check(from((e << 52) | (0x000fffffffffffffull ^ (m >> (rnd() % 53)))));
    check(from(rnd()));   /* any bit pattern: mostly outside */
  }
  printf("%ld %ld %ld\n", bad, cases, outside);
  return 0;
}
