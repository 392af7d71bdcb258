// Host build of the integer-pipe binary64 operations for the CPU tests:
// each entry applies one operation elementwise and reports, per element,
// whether the fast path applied (the result is only defined then).
#include "../../formura_gb300/csrc/fgb_softf64.h"

using namespace fgb::soft;

extern "C" {

void soft_add(const double* a, const double* b, double* r, unsigned char* fast, long n) {
  for (long i = 0; i < n; ++i) {
    uint64_t R = 0;
    fast[i] = add_bits(to_bits(a[i]), to_bits(b[i]), R);
    r[i] = from_bits(R);
  }
}

void soft_sub(const double* a, const double* b, double* r, unsigned char* fast, long n) {
  for (long i = 0; i < n; ++i) {
    uint64_t R = 0;
    fast[i] = add_bits(to_bits(a[i]), to_bits(b[i]) ^ kSign, R);
    r[i] = from_bits(R);
  }
}

void soft_mul(const double* a, const double* b, double* r, unsigned char* fast, long n) {
  for (long i = 0; i < n; ++i) {
    uint64_t R = 0;
    fast[i] = mul_bits(to_bits(a[i]), to_bits(b[i]), R);
    r[i] = from_bits(R);
  }
}

// c*h + t with c = (negate ? -1 : 1) * 2^k
void soft_scaled_add(const double* h, const double* t, double* r, unsigned char* fast, long n, int k, int negate) {
  for (long i = 0; i < n; ++i) {
    uint64_t R = 0;
    double c = negate ? -1.0 : 1.0;
    for (int j = 0; j < k; ++j) c *= 2.0;
    for (int j = 0; j > k; --j) c *= 0.5;
    fast[i] = scaled_add_bits(to_bits(c), to_bits(h[i]), to_bits(t[i]), R);
    r[i] = from_bits(R);
  }
}

}  // extern "C"
