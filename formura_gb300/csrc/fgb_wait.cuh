// Bounded waits on an mbarrier phase.  No kernel of this library waits
// without a limit: a wait that runs out returns false, the kernel raises its
// launch's error word (FgbLaunch::err) and returns, so the context stays
// usable and the host reports the failure (fgb_synchronize, fgb_download).
#pragma once
#include <stdint.h>

namespace fgb {

// Limit of an ordinary wait for a TMA copy (normally a few microseconds),
// and of the drain of copies still in flight after such a wait ran out.
constexpr uint64_t kWaitLimitNs = 1000000000ull;
constexpr uint64_t kDrainLimitNs = 2000000000ull;

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// One poll of the phase of parity `parity` of the mbarrier at shared address
// `bar`; the thread may be suspended for up to about 10 microseconds while
// the phase is incomplete.
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(parity), "r"(10000u)
      : "memory");
  return done != 0;
}

// Waits for that phase for at most `limit_ns` nanoseconds of the global
// timer; true once the phase has completed, false if the wait ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity,
                                                  uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

}  // namespace fgb
