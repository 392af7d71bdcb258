// Lazy synchronisation of the host copy of the state (formura_data).
//
// The reference keeps the state in host memory; a driver may read or write
// formura_data between any two Formura_Forward calls.  The eager drop-in
// uploads and downloads it on every call.  In lazy mode the device keeps the
// state across calls and the host pages are protected instead:
//   after a forward step  -> pages PROT_NONE (the device copy is newer);
//   first access           -> SIGSEGV: download, pages read-only (clean);
//   first write afterwards -> SIGSEGV: pages read-write (dirty);
//   next forward step      -> upload only if dirty.
// A driver that touches formura_data every N steps pays one copy per N steps.
// Faults outside the registered regions are passed on to the previous
// handler.  The region must be page aligned and span whole pages (the
// generated drop-in places formura_data in a page-aligned, page-padded block).
#include <cuda_runtime.h>
#include <signal.h>
#include <stdint.h>
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>
#include <atomic>

#include "../../include/formura_gb300.h"

int fgb_internal_set_error(int code, const char* message);

namespace {

enum { kDirty = 0, kClean = 1, kDeviceNewer = 2 };
const int kMaxRegions = 16;

struct Region {
  std::atomic<fgb_grid*> grid{nullptr};
  char* lo = nullptr;
  size_t len = 0;
  std::atomic<int> state{kDirty};
  std::atomic<int> lock{0};
  std::atomic<int64_t> downloads{0}, uploads{0};
};

Region g_regions[kMaxRegions];
struct sigaction g_previous;
std::atomic<int> g_installed{0};

void region_lock(Region& r) {
  int expected = 0;
  while (!r.lock.compare_exchange_weak(expected, 1)) expected = 0;
}
void region_unlock(Region& r) { r.lock.store(0); }

void chain(int sig, siginfo_t* si, void* ctx) {
  if (g_previous.sa_flags & SA_SIGINFO) {
    if (g_previous.sa_sigaction) {
      g_previous.sa_sigaction(sig, si, ctx);
      return;
    }
  } else if (g_previous.sa_handler != SIG_DFL && g_previous.sa_handler != SIG_IGN) {
    g_previous.sa_handler(sig);
    return;
  }
  // default action: restore it and let the fault happen again
  signal(sig, SIG_DFL);
}

void on_fault(int sig, siginfo_t* si, void* ctx) {
  char* a = static_cast<char*>(si->si_addr);
  for (int i = 0; i < kMaxRegions; ++i) {
    Region& r = g_regions[i];
    fgb_grid* g = r.grid.load();
    if (!g || a < r.lo || a >= r.lo + r.len) continue;
    // The fault is synchronous: this thread is in the driver's code reading
    // or writing formura_data, never inside the CUDA runtime.
    region_lock(r);
    const int st = r.state.load();
    if (st == kDeviceNewer) {
      mprotect(r.lo, r.len, PROT_READ | PROT_WRITE);
      fgb_download(g, reinterpret_cast<double*>(r.lo));
      ++r.downloads;
      mprotect(r.lo, r.len, PROT_READ);
      r.state.store(kClean);
    } else if (st == kClean) {
      mprotect(r.lo, r.len, PROT_READ | PROT_WRITE);
      r.state.store(kDirty);
    }
    region_unlock(r);
    return;
  }
  chain(sig, si, ctx);
}

int install() {
  int expected = 0;
  if (!g_installed.compare_exchange_strong(expected, 1)) return FGB_OK;
  struct sigaction sa;
  memset(&sa, 0, sizeof sa);
  sa.sa_sigaction = on_fault;
  sa.sa_flags = SA_SIGINFO | SA_NODEFER;
  sigemptyset(&sa.sa_mask);
  if (sigaction(SIGSEGV, &sa, &g_previous) != 0) {
    g_installed.store(0);
    return fgb_internal_set_error(FGB_E_ARG, "sigaction(SIGSEGV) failed");
  }
  return FGB_OK;
}

Region* find(fgb_grid* g) {
  for (int i = 0; i < kMaxRegions; ++i)
    if (g_regions[i].grid.load() == g) return &g_regions[i];
  return nullptr;
}

}  // namespace

extern "C" {

int fgb_lazy_attach(fgb_grid* g, void* host_state, size_t bytes) {
  const size_t page = (size_t)sysconf(_SC_PAGESIZE);
  if (!g || !host_state || bytes == 0) return fgb_internal_set_error(FGB_E_ARG, "bad lazy region");
  if (((uintptr_t)host_state % page) != 0 || bytes % page != 0)
    return fgb_internal_set_error(FGB_E_ARG, "lazy region must be page aligned and whole pages");
  if (find(g)) return fgb_internal_set_error(FGB_E_ARG, "grid already has a lazy region");
  int rc = install();
  if (rc != FGB_OK) return rc;
  for (int i = 0; i < kMaxRegions; ++i) {
    Region& r = g_regions[i];
    fgb_grid* expected = nullptr;
    if (r.grid.load() == nullptr) {
      r.lo = static_cast<char*>(host_state);
      r.len = bytes;
      r.state.store(kDirty);
      r.downloads.store(0);
      r.uploads.store(0);
      if (r.grid.compare_exchange_strong(expected, g)) return FGB_OK;
    }
  }
  return fgb_internal_set_error(FGB_E_ARG, "too many lazy regions");
}

// Upload if the host copy was written, advance, and leave the host pages
// protected (the device copy is the newer one).
int fgb_lazy_forward(fgb_grid* g, int nsteps) {
  Region* r = find(g);
  if (!r) return fgb_internal_set_error(FGB_E_ARG, "grid has no lazy region");
  region_lock(*r);
  int rc = FGB_OK;
  if (r->state.load() == kDirty) {
    rc = fgb_upload(g, reinterpret_cast<const double*>(r->lo));
    ++r->uploads;
  }
  if (rc == FGB_OK) rc = fgb_forward(g, nsteps);
  if (rc == FGB_OK) {
    mprotect(r->lo, r->len, PROT_NONE);
    r->state.store(kDeviceNewer);
  }
  region_unlock(*r);
  return rc;
}

// Bring the host copy up to date and unprotect it.
int fgb_lazy_detach(fgb_grid* g) {
  Region* r = find(g);
  if (!r) return FGB_OK;
  region_lock(*r);
  mprotect(r->lo, r->len, PROT_READ | PROT_WRITE);
  int rc = FGB_OK;
  if (r->state.load() == kDeviceNewer) rc = fgb_download(g, reinterpret_cast<double*>(r->lo));
  r->state.store(kDirty);
  r->grid.store(nullptr);
  region_unlock(*r);
  return rc;
}

int fgb_lazy_stats(fgb_grid* g, int64_t* uploads, int64_t* downloads) {
  Region* r = find(g);
  if (!r) return fgb_internal_set_error(FGB_E_ARG, "grid has no lazy region");
  if (uploads) *uploads = r->uploads.load();
  if (downloads) *downloads = r->downloads.load();
  return FGB_OK;
}

}  // extern "C"
