// Test kernel for the library's bounded mbarrier wait (fgb_wait.cuh): each
// block initialises an mbarrier that expects one arrival.  With `arrive`
// set, thread 0 arrives and the phase completes; without it nothing ever
// completes the phase, so the bounded wait runs out.  A block whose wait
// ran out raises the error word the way the library's tile kernels do (value
// 1) and skips its store; nothing is in flight (no copies are issued).
#include <cuda_runtime.h>
#include <stdint.h>

#include "fgb_wait.cuh"

__global__ void wait_kernel(int arrive, int* err, int* stored) {
  __shared__ __align__(8) uint64_t bar;
  const uint32_t b = (uint32_t)__cvta_generic_to_shared(&bar);
  if (threadIdx.x == 0) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
  __syncthreads();
  if (arrive && threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(b) : "memory");
  const bool ok = __syncthreads_and(fgb::mbar_wait_bounded(b, 0u));
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
    return;
  }
  if (threadIdx.x == 0) atomicAdd(stored, 1);
}

// Runs the kernel on `blocks` blocks of 128 threads and waits for it;
// returns the CUDA status, the number of blocks that stored, and the time.
extern "C" int bounded_wait_run(int arrive, int blocks, int* err_dev, int* stored_host, float* ms) {
  int* stored = nullptr;
  cudaError_t e = cudaMalloc(&stored, sizeof(int));
  if (e != cudaSuccess) return (int)e;
  cudaMemset(stored, 0, sizeof(int));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  wait_kernel<<<blocks, 128>>>(arrive, err_dev, stored);
  cudaEventRecord(e1);
  e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventElapsedTime(ms, e0, e1);
  cudaMemcpy(stored_host, stored, sizeof(int), cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(stored);
  return (int)e;
}
