// fgb_forward_noalloc: time steps on caller-owned device buffers without any
// device allocation.
//
// Some callers cannot call cudaMalloc while they run: a host framework that
// owns all device memory through its own pool, a plug-in host that forbids
// new device allocations once a run has started, or a solver stepping while
// the device is nearly full.  This entry point takes the input and output
// state from the caller; every other byte it needs (the uniform table, the
// second buffer of the ping-pong between steps, the intermediate stage arrays
// of multi-stage programs) comes from one fixed array that is part of the
// library's device image.  That array is FGB_NOALLOC_SCRATCH_BYTES (64 MiB)
// on every GPU that loads the library, held until the process exits.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <mutex>

#include "fgb_internal.h"
#include "../../include/formura_gb300.h"

extern "C" const FgbProgramGetter fgb_builtin_programs[];
extern "C" const int fgb_builtin_program_count;
int fgb_internal_set_error(int code, const char* message);

#define FGB_NOALLOC_MAX_DEVICES 64
#define FGB_NOALLOC_MAX_UNIFORMS 1024

static __device__ __align__(256) unsigned char fgb_noalloc_scratch[FGB_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_setup_mutex;
unsigned char* g_scratch[FGB_NOALLOC_MAX_DEVICES];  // device address per device, set once

int error(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return fgb_internal_set_error(code, buf);
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// a normal power of two: division by it is one exact product, so FP64 steps
// may use the program's launch_p2 kernels (the choice fgb_open makes)
bool is_pow2(double c) {
  uint64_t u;
  memcpy(&u, &c, sizeof u);
  const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
  return (u & 0x000fffffffffffffull) == 0 && e >= 1u && e <= 2046u;
}

// The uniform table travels as a kernel parameter (copied at launch), so no
// host buffer has to outlive the call and no pageable copy is queued.
struct UniformTable {
  double v[FGB_NOALLOC_MAX_UNIFORMS];
};
static_assert(sizeof(UniformTable) <= 16384, "uniform table exceeds the kernel parameter space used here");

__global__ void write_uniforms(UniformTable t, int n, int as_float, void* dst) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (as_float)
      static_cast<float*>(dst)[i] = (float)t.v[i];
    else
      static_cast<double*>(dst)[i] = t.v[i];
  }
}

// The device address of the scratch array on the current device.  In host
// code `fgb_noalloc_scratch` is only a host-side stand-in for the symbol, so
// the address is looked up once per device with that device current.
int scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return error(FGB_E_NODEV, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= FGB_NOALLOC_MAX_DEVICES) return error(FGB_E_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, fgb_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return error(FGB_E_CUDA, "cudaGetSymbolAddress(fgb_noalloc_scratch): %s", cudaGetErrorString(e));
    g_scratch[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch[dev];
  return FGB_OK;
}

}  // namespace

extern "C" int fgb_forward_noalloc(const char* program, const int* shape, int ndim, int precision,
                                   const double* uniforms, int nuniforms, const void* in_state,
                                   void* out_state, int nsteps, void* stream) {
  const FgbProgramDesc* d = nullptr;
  for (int i = 0; program && i < fgb_builtin_program_count; ++i) {
    const FgbProgramDesc* c = fgb_builtin_programs[i]();
    if (strcmp(c->name, program) == 0) d = c;
  }
  if (!d) return error(FGB_E_PROGRAM, "unknown program '%s'", program ? program : "(null)");
  if (ndim != d->dim || !shape) return error(FGB_E_ARG, "program %s is %d-dimensional", d->name, d->dim);
  if (precision < 0 || precision >= FGB_NUM_PRECISIONS) return error(FGB_E_ARG, "unknown precision %d", precision);
  if (nuniforms != d->nuniforms || (nuniforms > 0 && !uniforms))
    return error(FGB_E_ARG, "program %s needs %d uniform values, got %d", d->name, d->nuniforms, nuniforms);
  if (nuniforms > FGB_NOALLOC_MAX_UNIFORMS) return error(FGB_E_ARG, "too many uniform values");
  if (nsteps < 0 || !in_state || !out_state) return error(FGB_E_ARG, "bad state pointers or step count");
  int n[3] = {1, 1, 1};
  size_t cells = 1;
  const int need_pts = d->reach > d->shift ? d->reach : d->shift;
  for (int a = 0; a < ndim; ++a) {
    if (shape[a] < 1 || shape[a] < need_pts)
      return error(FGB_E_ARG, "axis %d has %d points; program %s reads %d points away", a, shape[a], d->name, need_pts);
    n[3 - ndim + a] = shape[a];
    cells *= (size_t)shape[a];
  }
  // the stage kernels index fields and cells with 32-bit integers
  if (cells * (size_t)d->nfields >= ((size_t)1 << 32) || cells >= ((size_t)1 << 31))
    return error(FGB_E_ARG, "grid of %zu points is larger than this build supports", cells);
  const size_t es = precision <= FGB_F64_FAST ? 8 : (precision == FGB_F32 ? 4 : 2);
  const size_t cs = precision <= FGB_F64_FAST ? 8 : 4;
  const size_t state_bytes = cells * d->nfields * es;
  const char* in_c = static_cast<const char*>(in_state);
  const char* out_c = static_cast<const char*>(out_state);
  if (in_c < out_c + state_bytes && out_c < in_c + state_bytes)
    return error(FGB_E_ARG, "input and output states overlap");

  // scratch layout: uniform table | second state buffer | intermediate arrays
  const size_t off_state = align256((size_t)nuniforms * cs);
  const size_t off_mids = off_state + (nsteps > 1 ? align256(state_bytes) : 0);
  const size_t mid_bytes = align256(cells * cs);
  const size_t need = off_mids + (size_t)d->nmids * mid_bytes;
  if (need > FGB_NOALLOC_SCRATCH_BYTES)
    return error(FGB_E_ARG, "%s on this grid needs %zu bytes of scratch; fgb_forward_noalloc has %llu",
                 d->name, need, (unsigned long long)FGB_NOALLOC_SCRATCH_BYTES);

  unsigned char* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc != FGB_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
  if (nsteps == 0) {
    e = cudaMemcpyAsync(out_state, in_state, state_bytes, cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? FGB_OK : error(FGB_E_CUDA, "copy: %s", cudaGetErrorString(e));
  }
  if (nuniforms > 0) {
    UniformTable t;
    memcpy(t.v, uniforms, (size_t)nuniforms * sizeof(double));
    write_uniforms<<<1, 128, 0, st>>>(t, nuniforms, cs == 4, scratch);
    e = cudaGetLastError();
    if (e != cudaSuccess) return error(FGB_E_CUDA, "uniform table: %s", cudaGetErrorString(e));
  }
  bool p2 = false;
  if (precision == FGB_F64 && d->ndivisors > 0) {
    p2 = true;
    for (int i = 0; i < d->ndivisors; ++i) p2 = p2 && is_pow2(uniforms[d->divisors[i]]);
  }
  void* bufs[2] = {out_state, scratch + off_state};
  FgbLaunch L;
  memset(&L, 0, sizeof L);
  for (int k = 0; k < d->nmids; ++k) L.mid[k] = scratch + off_mids + k * mid_bytes;
  L.uniforms = scratch;
  for (int a = 0; a < 3; ++a) L.n[a] = n[a];
  L.fused_steps = 1;
  for (int f = 0; f < d->nfields; ++f) {
    L.scale[f] = 1.0f;
    L.inv_scale[f] = 1.0f;
  }
  const void* src = in_state;
  for (int s = 0; s < nsteps; ++s) {
    // the last step writes into out_state
    void* dst = bufs[(nsteps - 1 - s) % 2];
    for (int f = 0; f < d->nfields; ++f) {
      L.in[f] = static_cast<const char*>(src) + f * cells * es;
      L.out[f] = static_cast<char*>(dst) + f * cells * es;
    }
    for (int stg = 0; stg < d->nstages; ++stg) {
      e = (p2 ? d->launch_p2[stg] : d->launch[precision][stg])(&L, st);
      if (e != cudaSuccess) return error(FGB_E_CUDA, "stage launch: %s", cudaGetErrorString(e));
    }
    src = dst;
  }
  return FGB_OK;
}
