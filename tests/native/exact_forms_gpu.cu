// GPU check of the shortened operations of the bit-faithful FP64 policy
// (fgb::F64Exact::divu, ::divr with ::rcp, ::fma with a power-of-two factor,
// ::one_minus)
// against the reference's separately rounded IEEE operations, bit for bit,
// wherever the form's range flag stays set.  Operand classes: moderate, wide,
// subnormal and tiny, huge and non-finite, signed zeros, any bit pattern.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../formura_gb300/csrc/fgb_templates.cuh"

using fgb::F64Exact;
using fgb::F64Ieee;

__device__ __forceinline__ uint64_t mix(uint64_t x) {
  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ double make(uint64_t sign, int e, uint64_t mant) {
  e = e < 0 ? 0 : (e > 2047 ? 2047 : e);
  return __longlong_as_double((long long)((sign << 63) | ((uint64_t)e << 52) | (mant & 0x000fffffffffffffull)));
}

// one operand of class `cls` (the same for the whole warp)
__device__ double operand(uint64_t key, int cls) {
  const uint64_t r = mix(key), m = mix(key ^ 0xabcdef);
  const uint64_t sign = r >> 63;
  switch (cls) {
    case 0:  return make(sign, 1023 - 60 + (int)(r % 121), m);          // moderate
    case 1:  return make(sign, 1023 - 380 + (int)(r % 761), m);         // wide, inside the windows
    case 2:  return make(sign, (int)(r % 90), m >> (r % 53));           // subnormal and lowest binades
    case 3:  return make(sign, 1960 + (int)(r % 88), m);                // huge, infinity and NaN
    case 4:  return (r & 2) ? make(sign, 0, 0) : make(sign, 1023 - 60 + (int)(r % 121), m);  // signed zeros
    default: return __longlong_as_double((long long)r);                 // any bit pattern
  }
}

__device__ __forceinline__ bool same(double a, double b) {
  // bitwise, except that any NaN matches any NaN
  return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}

// A division must give the IEEE result's bits for every lane (it falls back
// to the IEEE division by itself); the multiply-add wherever its range flag
// stays set (where it drops, the kernels evaluate with F64Ieee instead).
// Counts per operation: mismatches, and lanes inside the shortened window;
// then the mismatches of the integer-pipe comparisons, and of the divisions'
// integer rounding step taken lane by lane, with the lanes it applied to;
// then the mismatches of 1 - x (warp by warp, and its integer form lane by
// lane) with the lanes in that form's window; then the mismatches of the
// quotients below 2^-1021 on the integer grid, lane by lane, with their lanes.
__global__ void check(uint64_t seed, uint64_t n, unsigned long long* out) {
  unsigned long long bad[4] = {0, 0, 0, 0}, fast[3] = {0, 0, 0}, step_used = 0, step_bad = 0;
  unsigned long long om_bad = 0, om_used = 0, sub_bad = 0, sub_used = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t key = seed * 0x100000000ull + i;
    const uint64_t warp = i / 32;
    const int ca = (int)(mix(warp * 3 + seed) % 6), cb = (int)(mix(warp * 5 + seed) % 6);
    // divu: uniform divisor per warp (grid-independent), numerator per lane
    double c = operand(warp * 11 + seed, ca == 3 ? 1 : ca % 2);
    if ((warp & 3) == 3)   // powers of two, whose quotient is one product
      c = __longlong_as_double((long long)(__double_as_longlong(c) & 0xfff0000000000000ull));
    double x = operand(key * 7 + 1, cb == 5 ? (int)(mix(key) % 6) : cb);
    if ((warp & 7) == 6) {
      // one warp with quotients below 2^-1021, numerators in the window and
      // tiny numerators with a normal quotient (c in [2^10, 2^60])
      const uint64_t rw = mix(warp * 17 + seed), r2 = mix(key * 5 + 9);
      const int ecb = 1023 + 10 + (int)(rw % 51);
      c = make(rw >> 63, ecb, mix(rw));
      if (i % 3 == 0)   // quotients below 2^-1021: subnormal numerators, and the top of the range
        x = (r2 & 2) ? make(r2 >> 63, 0, mix(r2) >> (r2 % 52)) : make(r2 >> 63, ecb - 1022 - (int)(r2 % 3), mix(r2));
      else if (i % 3 == 1) x = make(r2 >> 63, 1023 - 60 + (int)(r2 % 121), mix(r2));
      else x = make(r2 >> 63, ecb - 1021 + (int)(r2 % (uint64_t)(63 - (ecb - 1021))), mix(r2));
    }
    const double rc = 1.0 / c;
    bool ok = true;
    if ((warp & 3) == 3) {   // the power-of-two policy's single product, for every numerator
      if (!same(fgb::F64ExactP2::divu(x, c, rc, ok), __ddiv_rn(x, c))) ++bad[0];
    }
    double r = F64Exact::divu(x, c, rc, ok);
    fast[0] += F64Exact::divu_window(x, c);
    bad[0] += ok && !same(r, __ddiv_rn(x, c));
    // the integer rounding step on its own, lane by lane (the kernels take it
    // only where every lane of a warp fits)
    if (F64Exact::divu_window(x, c)) {
      const double q0 = __dmul_rn(x, rc), rem = __fma_rn(-q0, c, x);
      bool fits;
      const double q = F64Exact::round_quotient(x, c, q0, rem, fits);
      step_used += fits;
      step_bad += fits && !same(q, __ddiv_rn(x, c));
    }
    // quotients below 2^-1021 on the integer grid, lane by lane
    if (F64Exact::divu_sub(x, c)) {
      ++sub_used;
      sub_bad += !same(F64Exact::divu_mixed(x, c, rc, false, true), __ddiv_rn(x, c));
    }
    // divr: grid numerator and denominator
    const double a = operand(key * 7 + 2, ca == 5 ? (int)(mix(key ^ 1) % 6) : ca);
    const double b = operand(key * 7 + 3, cb);
    ok = true;
    r = F64Exact::divr(a, b, F64Exact::rcp(b), ok);
    fast[1] += F64Exact::divr_window(a, b);
    bad[1] += ok && !same(r, __ddiv_rn(a, b));
    if (F64Exact::divr_window(a, b)) {
      const double y = F64Exact::rcp(b), q0 = __dmul_rn(a, y), rem = __fma_rn(-q0, b, a);
      bool fits;
      const double q = F64Exact::round_quotient(a, b, q0, rem, fits);
      step_used += fits;
      step_bad += fits && !same(q, __ddiv_rn(a, b));
    }
    // fma with a = +-2^k, k in [-3, 3]: RN(RN(a*h) + t)
    const int k = (int)(mix(warp * 7 + seed) % 7) - 3;
    const double f = ((warp & 1) ? -1.0 : 1.0) * ldexp(1.0, k);
    const double h = operand(key * 7 + 4, cb), t = operand(key * 7 + 5, (cb + 1) % 6);
    ok = true;
    r = F64Exact::fma(f, h, t, ok);
    fast[2] += ok;
    bad[2] += ok && !same(r, __dadd_rn(__dmul_rn(f, h), t));
    // comparisons on the integer pipe against the hardware's, every operand
    // class against every other (signed zeros, infinities and NaNs included),
    // and each value against itself and its negation
    const double p = operand(key * 7 + 6, (int)(mix(key ^ 2) % 6)), q = (i & 8) ? -p : (i & 16) ? p : b;
    const bool hw[6] = {p < q, p > q, p <= q, p >= q, p == q, p != q};
    const bool in[6] = {F64Exact::lt(p, q), F64Exact::gt(p, q), F64Exact::le(p, q),
                        F64Exact::ge(p, q), F64Exact::eq(p, q), F64Exact::ne(p, q)};
    for (int j = 0; j < 6; ++j) bad[3] += hw[j] != in[j];
    bad[3] += !same(F64Exact::fabs(p), fabs(p)) || (__double_as_longlong(F64Exact::fabs(p)) >> 63) != 0;
    // 1 - x: whole warps in [0.5, 2), warps with one lane outside, and any
    // operand class
    const int cm = (int)(mix(warp * 13 + seed) % 3);
    const uint64_t sm = mix(key ^ 3);
    double u = __longlong_as_double((long long)(((1022ull + (sm & 1)) << 52) | ((sm >> 1) & 0x000fffffffffffffull)));
    if (cm == 1 && (i & 31) == (warp & 31)) u = operand(key * 7 + 7, (int)(sm % 6));
    if (cm == 2) u = operand(key * 7 + 7, (int)(sm % 6));
    om_bad += !same(F64Exact::one_minus(u), __dsub_rn(1.0, u));
    if (F64Exact::one_minus_window(u)) {
      ++om_used;
      om_bad += !same(F64Exact::one_minus_exact(u), __dsub_rn(1.0, u));
    }
  }
  for (int j = 0; j < 3; ++j) {
    atomicAdd(&out[j], bad[j]);
    atomicAdd(&out[3 + j], fast[j]);
  }
  atomicAdd(&out[6], bad[3]);
  atomicAdd(&out[7], step_bad);
  atomicAdd(&out[8], step_used);
  atomicAdd(&out[9], om_bad);
  atomicAdd(&out[10], om_used);
  atomicAdd(&out[11], sub_bad);
  atomicAdd(&out[12], sub_used);
}

extern "C" int exact_forms_gpu_check(unsigned long long seed, unsigned long long n, unsigned long long* host_out) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 13 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  cudaMemset(d, 0, 13 * sizeof(unsigned long long));
  check<<<152 * 8, 256>>>(seed, n, d);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(host_out, d, 13 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : 2;
}
