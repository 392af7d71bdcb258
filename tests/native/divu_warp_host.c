/* Host check of the bit-faithful FP64 policy's division by a
 * grid-independent constant as a warp takes it (fgb::F64Exact::divu and
 * divu_outside, divu_mixed): 32 lanes share the divisor, and the warp picks
 * its form from all lanes' tests (window; window or tiny; window, tiny or
 * below 2^-1021; else the IEEE division).  The device's integer steps and
 * FP64 operations are restated on the host's correctly rounded fma and
 * compared lane by lane with the host's IEEE division.  Warps mix numerator
 * classes (moderate, tiny normal, subnormal, the top of the integer-grid
 * range, zeros, and numerators between the scaled form and the window for
 * divisors above 2^40) so that every form, and the lanes of each kind
 * inside the mixed one, are taken.
 * Prints "mismatches lanes warps_window warps_tiny warps_mixed warps_ieee". */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s = 0xa4093822299f31d0ull;
static uint64_t rnd(void) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
static double from(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
static uint64_t bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
static int clz64(uint64_t v) { return v ? __builtin_clzll(v) : 64; }
static unsigned expo(double x) { return (unsigned)(bits(x) >> 52) & 0x7ffu; }
static int is_zero(double x) { return (bits(x) << 1) == 0; }
static int within(double x, unsigned w) { return expo(x) - (1023u - w) <= 2u * w; }
static int eff_of(double x) {
  const unsigned ex = expo(x);
  const uint64_t m = bits(x) & 0x000fffffffffffffull;
  return ex != 0u ? (int)ex : 12 - clz64(m);
}

static int divu_window(double x, double c) {
  const unsigned ex = expo(x);
  return within(c, 100) && (is_zero(x) || (ex - 63u <= 1920u && ex - expo(c) + 1000u <= 2000u));
}
static int divu_tiny(double x, double c) {
  const unsigned ex = expo(x);
  const uint64_t m = bits(x) & 0x000fffffffffffffull;
  return within(c, 100) && ex < 63u && m + ex != 0ull && eff_of(x) + 1021 >= (int)expo(c);
}
static int divu_sub(double x, double c) {
  const uint64_t m = bits(x) & 0x000fffffffffffffull;
  return within(c, 100) && m + expo(x) != 0ull && eff_of(x) - (int)expo(c) <= -1022;
}

static double scale_up(double x, int k) {
  uint64_t b = bits(x);
  if (expo(x) != 0u) {
    b += (uint64_t)k << 52;
  } else {
    const uint64_t m = b & 0x000fffffffffffffull;
    const int sh = clz64(m) - 11;
    b = (b & 0x8000000000000000ull) | ((uint64_t)(k + 1 - sh) << 52) | ((m << sh) & 0x000fffffffffffffull);
  }
  return from(b);
}
static double scale_down(double q) { return from(bits(q) - (256ull << 52)); }

static double round_quotient(double x, double c, double q0, double r, int* fits) {
  const uint64_t qb = bits(q0), rb = bits(r), cb = bits(c);
  const unsigned qhi = (unsigned)(qb >> 32), qlo = (unsigned)qb, rhi = (unsigned)(rb >> 32), chi = (unsigned)(cb >> 32);
  const unsigned eq = (qhi >> 20) & 0x7ffu, ec = (chi >> 20) & 0x7ffu;
  const uint64_t m = ((uint64_t)(qhi & 0xfffffu) << 32) | qlo;
  const int et = (int)ec + (int)eq - 1076;
  const int zero = is_zero(x);
  *fits = zero || (m - 2ull <= (1ull << 52) - 5ull && (unsigned)(et - 2) <= 2044u);
  const uint64_t t = ((uint64_t)((chi & 0xfffffu) | ((unsigned)et << 20)) << 32) | (unsigned)cb;
  const uint64_t a = ((uint64_t)(rhi & 0x7fffffffu) << 32) | (unsigned)rb;
  const int step = a > t || (a == t && (qlo & 1u));
  const int up = ((rhi ^ chi ^ qhi) >> 31) == 0;
  const uint64_t res = qb + (step ? (up ? 1ull : ~0ull) : 0ull);
  return zero ? q0 : from(res);
}
static double markstein_last(double x, double q0, double r, double y) { return is_zero(x) ? q0 : fma(r, y, q0); }

/* one warp: the divisor c and its host reciprocal rc, 32 numerators */
static long forms[4];
static void warp_divide(const double* x, double c, double rc, double* out) {
  int win[32], tiny[32], sub[32], all_w = 1, all_wt = 1, all_wts = 1;
  for (int l = 0; l < 32; ++l) {
    win[l] = divu_window(x[l], c);
    tiny[l] = divu_tiny(x[l], c);
    sub[l] = divu_sub(x[l], c);
    all_w &= win[l];
    all_wt &= win[l] || tiny[l];
    all_wts &= win[l] || tiny[l] || sub[l];
  }
  if (all_w || all_wt) {   /* quotient(), on the scaled numerators where tiny */
    ++forms[all_w ? 0 : 1];
    double q0[32], r[32], q[32], a[32];
    int fits[32], all_fit = 1;
    for (int l = 0; l < 32; ++l) {
      a[l] = tiny[l] ? scale_up(x[l], 256) : x[l];
      q0[l] = a[l] * rc;
      r[l] = fma(-q0[l], c, a[l]);
      q[l] = round_quotient(a[l], c, q0[l], r[l], &fits[l]);
      all_fit &= fits[l];
    }
    for (int l = 0; l < 32; ++l) {
      const double ql = all_fit ? q[l] : markstein_last(a[l], q0[l], r[l], rc);
      out[l] = tiny[l] ? scale_down(ql) : ql;
    }
    return;
  }
  if (all_wts) {   /* divu_mixed */
    ++forms[2];
    double a[32], q0[32], r[32], q[32];
    uint64_t base[32];
    int fits[32], halfq[32], all_ok = 1;
    for (int l = 0; l < 32; ++l) {
      const uint64_t xb = bits(x[l]), cb = bits(c);
      a[l] = sub[l] ? scale_up(from(xb & 0x7fffffffffffffffull), 1074) : (tiny[l] ? scale_up(x[l], 256) : x[l]);
      const double cc = sub[l] ? from(cb & 0x7fffffffffffffffull) : c;
      q0[l] = a[l] * (sub[l] ? from(bits(rc) & 0x7fffffffffffffffull) : rc);
      const uint64_t qb = bits(q0[l]);
      const int e = (int)((qb >> 52) & 0x7ff) - 1023;
      const uint64_t qm = (qb & 0x000fffffffffffffull) | (1ull << 52);
      int sh = 52 - e;
      sh = sh < 1 ? 1 : (sh > 53 ? 53 : sh);
      const uint64_t n0 = e < -1 ? 0ull : (qm + (1ull << (sh - 1))) >> sh;
      const int lead = 63 - clz64(n0 | 1ull);
      const uint64_t nb = n0 == 0ull ? 0ull : (((uint64_t)(lead + 1023) << 52) | ((n0 << (52 - lead)) & 0x000fffffffffffffull));
      const int upper = e >= 51;
      base[l] = upper ? (e >= 52 ? qm << (e - 52 < 11 ? e - 52 : 11) : qm >> 1) : n0;
      halfq[l] = e == 51 && (qm & 1ull);
      r[l] = fma(-((sub[l] && !upper) ? from(nb) : q0[l]), cc, a[l]);
      q[l] = round_quotient(a[l], c, q0[l], r[l], &fits[l]);
      all_ok &= fits[l] || sub[l];
    }
    for (int l = 0; l < 32; ++l) {
      double ql = q[l];
      if (!all_ok && !sub[l]) ql = markstein_last(a[l], q0[l], r[l], rc);
      const uint64_t rb = bits(r[l]), cb = bits(c);
      const uint64_t ar = rb & 0x7fffffffffffffffull, half = (cb & 0x7fffffffffffffffull) - (1ull << 52);
      const int rneg = (int)(rb >> 63);
      const int step = halfq[l] ? ((!rneg && ar != 0ull) || (ar == 0ull && (base[l] & 1ull)))
                                : (ar > half || (ar == half && (base[l] & 1ull)));
      const uint64_t n = base[l] + (step ? ((rneg && !halfq[l]) ? ~0ull : 1ull) : 0ull);
      const uint64_t sb = n | ((bits(x[l]) ^ cb) & 0x8000000000000000ull);
      out[l] = sub[l] ? from(sb) : (tiny[l] ? scale_down(ql) : ql);
    }
    return;
  }
  ++forms[3];
  for (int l = 0; l < 32; ++l) out[l] = x[l] / c;
}

static double numerator(int cls, int ec) {
  const uint64_t sg = (rnd() & 1) << 63, m = rnd() & 0x000fffffffffffffull;
  switch (cls) {
    case 0: return from(sg | ((uint64_t)(1023 - 60 + (int)(rnd() % 121)) << 52) | m);   /* moderate */
    case 1: {   /* tiny normal with a normal quotient */
      const int lo = ec - 1021 > 1 ? ec - 1021 : 1;
      return lo <= 62 ? from(sg | ((uint64_t)(lo + (int)(rnd() % (uint64_t)(63 - lo))) << 52) | m) : 0.0;
    }
    case 2: return from(sg | (m >> (rnd() % 53)));   /* subnormal (or zero) */
    case 3: {   /* the top of the integer-grid range */
      const int top = ec - 1022 - (int)(rnd() % 3);
      return top >= 1 ? from(sg | ((uint64_t)top << 52) | m) : from(sg | (m >> (1 - top)));
    }
    case 4: return from(sg);   /* signed zero */
    default: {   /* above the scaled form, below the window: the IEEE division (divisors above 2^40) */
      const int ex = ec - 1010;
      return ex >= 63 ? from(sg | ((uint64_t)ex << 52) | m) : from(sg);
    }
  }
}

int main(int argc, char** argv) {
  const long warps = argc > 1 ? atol(argv[1]) : 100000;
  long bad = 0, lanes = 0;
  double x[32], out[32];
  for (long w = 0; w < warps; ++w) {
    const int ec = 1023 - 100 + (int)(rnd() % 201);
    const double c = from(((rnd() & 1) << 63) | ((uint64_t)ec << 52) | (rnd() & 0x000fffffffffffffull));
    const double rc = 1.0 / c;
    const int mode = (int)(rnd() % 7);
    for (int l = 0; l < 32; ++l) {
      const int cls = mode < 6 ? (l % (mode + 1) == 0 ? mode : (int)(rnd() % 5)) : (int)(rnd() % 6);
      x[l] = numerator(mode == 0 ? 0 : cls, ec);
    }
    warp_divide(x, c, rc, out);
    for (int l = 0; l < 32; ++l) {
      ++lanes;
      const double want = x[l] / c;
      if (bits(out[l]) != bits(want) && !(out[l] != out[l] && want != want)) {
        if (bad < 5) printf("# x=%a c=%a got %a want %a\n", x[l], c, out[l], want);
        ++bad;
      }
    }
  }
  printf("%ld %ld %ld %ld %ld %ld\n", bad, lanes, forms[0], forms[1], forms[2], forms[3]);
  return 0;
}
