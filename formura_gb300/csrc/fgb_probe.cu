// Throughput probe of the FP64 fused multiply-add pipe.
//
// The bit-faithful FP64 stencil kernels are bound by this part's FP64 rate,
// not by HBM, so their roofline is the DFMA rate: this probe measures it on
// the device at hand.  Every thread runs kChains independent dependency
// chains of a = fma(a, b, c) (latency hidden by the chains and by 8 resident
// 256-thread blocks per SM); the result is stored so that nothing is
// eliminated.  fgb_probe_dfma_rate returns the best of `reps` timed launches
// in FMA instructions per second (divide by 1e9 for G/s; one FMA is two
// flops).
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) dfma_chains(double b, double c, int iters, double* out) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = (double)(threadIdx.x + k) * 1e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = __fma_rn(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int fgb_probe_dfma_rate(int reps, double* fma_per_second) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.0f;
  int rc = 0;
  for (int r = 0; r < reps + 1 && rc == 0; ++r) {
    cudaEventRecord(e0);
    // b slightly below 1 and c small: the chains stay finite and normal
    dfma_chains<<<blocks, threads>>>(0.999999, 1e-7, iters, out);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = -1;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && (best == 0.0f || ms < best)) best = ms;  // the first launch is a warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (rc != 0 || best <= 0.0f) return -1;
  *fma_per_second = (double)blocks * threads * kChains * iters / (best * 1e-3);
  return 0;
}
