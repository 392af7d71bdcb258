// GPU check of the integer-pipe binary64 operations against the hardware
// instructions, on counter-generated operands: random bit patterns, nearby
// exponents of both signs, sparse mantissas (exact results and ties) and
// O(1) stencil-like values.  Reports mismatches and fast-path hits per op.
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../formura_gb300/csrc/fgb_softf64.h"

using namespace fgb::soft;

__device__ __forceinline__ uint64_t mix(uint64_t x) {
  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

__device__ uint64_t operand(uint64_t key, int kind, int e_ref, int& e_out) {
  const uint64_t r = mix(key), s = mix(key ^ 0x5555);
  uint64_t sign = (r >> 63) << 63;
  uint64_t mant = s & kMant;
  int e;
  switch (kind) {
    case 0:  // any bit pattern
      e_out = (int)((r >> 52) & 0x7ff);
      return r;
    case 1:  // exponent near the reference, full mantissa
      e = e_ref + (int)(r % 141) - 70;
      break;
    case 2: {  // sparse mantissa
      mant = 0;
      for (int j = 0; j < 4; ++j) mant |= 1ull << ((s >> (6 * j)) % 52);
      e = e_ref + (int)(r % 113) - 56;
      break;
    }
    default:  // O(1) values and their neighbours
      e = 1023 - (int)(r % 8);
      break;
  }
  e = e < 0 ? 0 : (e > 2046 ? 2046 : e);
  e_out = e;
  if (e == 0) mant &= 0xffffffffull;
  return sign | ((uint64_t)e << 52) | mant;
}

__global__ void check(uint64_t seed, uint64_t n, unsigned long long* out) {
  unsigned long long bad[4] = {0, 0, 0, 0}, fast[4] = {0, 0, 0, 0};
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t key = seed * 0x100000000ull + i;
    const int kind = (int)(i & 3);
    const int e_ref = 100 + (int)(mix(key * 3) % 1800);
    int ea, eb;
    const uint64_t A = operand(key * 7 + 1, kind, e_ref, ea);
    const uint64_t B = operand(key * 7 + 2, kind, kind == 0 ? e_ref : ea, eb);
    const double a = from_bits(A), b = from_bits(B);
    uint64_t R;
    if (add_bits(A, B, R)) {
      ++fast[0];
      bad[0] += R != to_bits(__dadd_rn(a, b));
    }
    if (add_bits(A, B ^ kSign, R)) {
      ++fast[1];
      bad[1] += R != to_bits(__dsub_rn(a, b));
    }
    // products: bring b near 1 so that most exponents stay in range
    const uint64_t B1 = (B & ~(0x7ffull << 52)) | ((uint64_t)(1023 - 200 + (int)(mix(key * 5) % 401)) << 52);
    if (mul_bits(A, B1, R)) {
      ++fast[2];
      bad[2] += R != to_bits(__dmul_rn(a, from_bits(B1)));
    }
    const double c = (i & 4) ? -2.0 : 0.5;
    if (scaled_add_bits(to_bits(c), B, A, R)) {
      ++fast[3];
      bad[3] += R != to_bits(__fma_rn(c, b, a));
    }
  }
  for (int k = 0; k < 4; ++k) {
    atomicAdd(&out[k], bad[k]);
    atomicAdd(&out[4 + k], fast[k]);
  }
}

extern "C" int softf64_gpu_check(unsigned long long seed, unsigned long long n, unsigned long long* host_out) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 8 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  cudaMemset(d, 0, 8 * sizeof(unsigned long long));
  check<<<152 * 8, 256>>>(seed, n, d);
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(host_out, d, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : 2;
}
