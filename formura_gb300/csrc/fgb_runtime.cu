// Runtime of the GB300 backend: device-resident grids, host<->device
// transfer of formura_data, and the time loop that replaces
// Formura_Forward's halo assembly + OpenMP loop nests
// (src/Formura/Generator/Templates.hs:295-346).
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <string>
#include <vector>

#include "fgb_internal.h"
#include "../../include/formura_gb300.h"

extern "C" const FgbProgramGetter fgb_builtin_programs[];
extern "C" const int fgb_builtin_program_count;

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? FGB_E_NOMEM : FGB_E_CUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

#define FGB_CUDA(call, what)                   \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

const FgbProgramDesc* find_program(const char* name) {
  if (!name) return nullptr;
  for (int i = 0; i < fgb_builtin_program_count; ++i) {
    const FgbProgramDesc* d = fgb_builtin_programs[i]();
    if (strcmp(d->name, name) == 0) return d;
  }
  return nullptr;
}

size_t storage_size(int precision) {
  switch (precision) {
    case FGB_F64: case FGB_F64_FAST: return 8;
    case FGB_F32: return 4;
    default: return 2;
  }
}
size_t compute_size(int precision) { return precision <= FGB_F64_FAST ? 8 : 4; }

// conversion between the host's FP64 state and the device storage format
template <class S>
__global__ void to_storage(const double* __restrict__ src, S* __restrict__ dst, size_t n, float inv_scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if constexpr (sizeof(S) == 2) dst[i] = __float2half_rn((float)src[i] * inv_scale);
    else dst[i] = (S)src[i];
  }
}
template <class S>
__global__ void from_storage(const S* __restrict__ src, double* __restrict__ dst, size_t n, float scale) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if constexpr (sizeof(S) == 2) dst[i] = (double)(__half2float(src[i]) * scale);
    else dst[i] = (double)src[i];
  }
}

}  // namespace

struct fgb_grid {
  const FgbProgramDesc* prog = nullptr;
  int precision = 0;
  int n[3] = {1, 1, 1};
  size_t cells = 0;
  cudaStream_t stream = nullptr;
  void* state[2] = {nullptr, nullptr};  // two buffers of nfields * cells storage elements
  void* mids = nullptr;                 // nmids * cells compute elements
  void* uniforms = nullptr;
  double* staging = nullptr;            // FP64 staging for F32/F16 transfers
  int cur = 0;
  float scale[FGB_MAX_FIELDS];
  int64_t launches = 0;
  cudaGraphExec_t graph = nullptr;      // a chunk of kGraphSteps steps
  int graph_cur = -1;
};

static const int kGraphSteps = 16;

static void fill_launch(const fgb_grid* g, int cur, FgbLaunch* L) {
  memset(L, 0, sizeof *L);
  const size_t es = storage_size(g->precision), cs = compute_size(g->precision);
  for (int f = 0; f < g->prog->nfields; ++f) {
    L->in[f] = (const char*)g->state[cur] + f * g->cells * es;
    L->out[f] = (char*)g->state[cur ^ 1] + f * g->cells * es;
    L->scale[f] = g->scale[f];
    L->inv_scale[f] = 1.0f / g->scale[f];
  }
  for (int k = 0; k < g->prog->nmids; ++k) L->mid[k] = (char*)g->mids + k * g->cells * cs;
  L->uniforms = g->uniforms;
  for (int a = 0; a < 3; ++a) L->n[a] = g->n[a];
  L->fused_steps = 1;
}

static int run_steps(fgb_grid* g, int nsteps) {
  FgbLaunch L[2];
  fill_launch(g, 0, &L[0]);
  fill_launch(g, 1, &L[1]);
  for (int s = 0; s < nsteps; ++s) {
    for (int st = 0; st < g->prog->nstages; ++st) {
      cudaError_t e = g->prog->launch[g->precision][st](&L[g->cur], g->stream);
      if (e != cudaSuccess) return cuda_fail(e, "stage launch");
      ++g->launches;
    }
    g->cur ^= 1;
  }
  return FGB_OK;
}

extern "C" {

const char* fgb_last_error(void) { return g_last_error.c_str(); }

int fgb_program_count(void) { return fgb_builtin_program_count; }

const char* fgb_program_name(int index) {
  if (index < 0 || index >= fgb_builtin_program_count) return nullptr;
  return fgb_builtin_programs[index]()->name;
}

int fgb_program_query(const char* program, int* dim, int* nfields, int* nuniforms, int* sleeve,
                      int* shift) {
  const FgbProgramDesc* d = find_program(program);
  if (!d) return fail(FGB_E_PROGRAM, "unknown program '%s'", program ? program : "(null)");
  if (dim) *dim = d->dim;
  if (nfields) *nfields = d->nfields;
  if (nuniforms) *nuniforms = d->nuniforms;
  if (sleeve) *sleeve = d->sleeve;
  if (shift) *shift = d->shift;
  return FGB_OK;
}

const char* fgb_program_field(const char* program, int index) {
  const FgbProgramDesc* d = find_program(program);
  if (!d || index < 0 || index >= d->nfields) return nullptr;
  return d->field_names[index];
}

int fgb_open(const char* program, const int* shape, int ndim, int precision, const double* uniforms,
             int nuniforms, fgb_grid** out) {
  if (!out) return fail(FGB_E_ARG, "out is null");
  *out = nullptr;
  const FgbProgramDesc* d = find_program(program);
  if (!d) return fail(FGB_E_PROGRAM, "unknown program '%s'", program ? program : "(null)");
  if (ndim != d->dim || !shape) return fail(FGB_E_ARG, "program %s is %d-dimensional", d->name, d->dim);
  if (precision < 0 || precision >= FGB_NUM_PRECISIONS)
    return fail(FGB_E_ARG, "unknown precision %d", precision);
  if (nuniforms != d->nuniforms || (nuniforms > 0 && !uniforms))
    return fail(FGB_E_ARG, "program %s needs %d uniform values, got %d", d->name, d->nuniforms, nuniforms);
  int n[3] = {1, 1, 1};
  size_t cells = 1;
  for (int a = 0; a < ndim; ++a) {
    const int v = shape[a];
    const int need = d->reach > d->shift ? d->reach : d->shift;
    if (v < 1 || v < need)
      return fail(FGB_E_ARG, "axis %d has %d points; program %s reads %d points away", a, v, d->name, need);
    n[3 - ndim + a] = v;
    cells *= (size_t)v;
  }
  if (cells * (size_t)d->nfields >= ((size_t)1 << 32) || cells >= ((size_t)1 << 31))
    return fail(FGB_E_ARG, "grid of %zu points is larger than this build supports", cells);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(FGB_E_NODEV, "no CUDA device");

  fgb_grid* g = new fgb_grid();
  g->prog = d;
  g->precision = precision;
  memcpy(g->n, n, sizeof n);
  g->cells = cells;
  for (int f = 0; f < FGB_MAX_FIELDS; ++f) g->scale[f] = 1.0f;
  const size_t es = storage_size(precision), cs = compute_size(precision);
  cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) e = cudaMalloc(&g->state[b], cells * d->nfields * es);
  if (e == cudaSuccess && d->nmids > 0) e = cudaMalloc(&g->mids, cells * d->nmids * cs);
  if (e == cudaSuccess && d->nuniforms > 0) e = cudaMalloc(&g->uniforms, d->nuniforms * cs);
  if (e == cudaSuccess && precision >= FGB_F32) e = cudaMalloc((void**)&g->staging, cells * d->nfields * 8);
  if (e == cudaSuccess && d->nuniforms > 0) {
    if (cs == 8) {
      e = cudaMemcpy(g->uniforms, uniforms, d->nuniforms * 8, cudaMemcpyHostToDevice);
    } else {
      std::vector<float> u(uniforms, uniforms + d->nuniforms);
      e = cudaMemcpy(g->uniforms, u.data(), d->nuniforms * 4, cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(g->state[0], 0, cells * d->nfields * es, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) {
    int rc = cuda_fail(e, "fgb_open");
    fgb_close(g);
    return rc;
  }
  *out = g;
  return FGB_OK;
}

int fgb_close(fgb_grid* g) {
  if (!g) return FGB_OK;
  if (g->stream) cudaStreamSynchronize(g->stream);
  if (g->graph) cudaGraphExecDestroy(g->graph);
  cudaFree(g->state[0]);
  cudaFree(g->state[1]);
  cudaFree(g->mids);
  cudaFree(g->uniforms);
  cudaFree(g->staging);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
  return FGB_OK;
}

int fgb_set_scales(fgb_grid* g, const float* scales, int nfields) {
  if (!g || !scales || nfields != g->prog->nfields) return fail(FGB_E_ARG, "bad scale arguments");
  for (int f = 0; f < nfields; ++f) {
    if (!(scales[f] > 0.0f)) return fail(FGB_E_ARG, "scale of field %d must be positive", f);
  }
  for (int f = 0; f < nfields; ++f) g->scale[f] = scales[f];
  if (g->graph) {
    cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
  }
  return FGB_OK;
}

int fgb_upload(fgb_grid* g, const double* host) {
  if (!g || !host) return fail(FGB_E_ARG, "null argument");
  const size_t n = g->cells * g->prog->nfields;
  if (g->precision <= FGB_F64_FAST) {
    FGB_CUDA(cudaMemcpyAsync(g->state[g->cur], host, n * 8, cudaMemcpyHostToDevice, g->stream), "upload");
  } else {
    FGB_CUDA(cudaMemcpyAsync(g->staging, host, n * 8, cudaMemcpyHostToDevice, g->stream), "upload");
    for (int f = 0; f < g->prog->nfields; ++f) {
      const double* src = g->staging + f * g->cells;
      if (g->precision == FGB_F32)
        to_storage<float><<<1024, 256, 0, g->stream>>>(src, (float*)g->state[g->cur] + f * g->cells, g->cells, 1.0f);
      else
        to_storage<__half><<<1024, 256, 0, g->stream>>>(src, (__half*)g->state[g->cur] + f * g->cells, g->cells,
                                                        1.0f / g->scale[f]);
      ++g->launches;
    }
    FGB_CUDA(cudaGetLastError(), "upload conversion");
  }
  FGB_CUDA(cudaStreamSynchronize(g->stream), "upload");
  return FGB_OK;
}

int fgb_download(fgb_grid* g, double* host) {
  if (!g || !host) return fail(FGB_E_ARG, "null argument");
  const size_t n = g->cells * g->prog->nfields;
  if (g->precision <= FGB_F64_FAST) {
    FGB_CUDA(cudaMemcpyAsync(host, g->state[g->cur], n * 8, cudaMemcpyDeviceToHost, g->stream), "download");
  } else {
    for (int f = 0; f < g->prog->nfields; ++f) {
      double* dst = g->staging + f * g->cells;
      if (g->precision == FGB_F32)
        from_storage<float><<<1024, 256, 0, g->stream>>>((const float*)g->state[g->cur] + f * g->cells, dst, g->cells, 1.0f);
      else
        from_storage<__half><<<1024, 256, 0, g->stream>>>((const __half*)g->state[g->cur] + f * g->cells, dst,
                                                          g->cells, g->scale[f]);
      ++g->launches;
    }
    FGB_CUDA(cudaGetLastError(), "download conversion");
    FGB_CUDA(cudaMemcpyAsync(host, g->staging, n * 8, cudaMemcpyDeviceToHost, g->stream), "download");
  }
  FGB_CUDA(cudaStreamSynchronize(g->stream), "download");
  return FGB_OK;
}

int fgb_forward(fgb_grid* g, int nsteps) {
  if (!g || nsteps < 0) return fail(FGB_E_ARG, "bad forward arguments");
  // Long runs replay a captured chunk of kGraphSteps steps (an even count,
  // so the buffer parity is unchanged after each replay).
  int done = 0;
  if (nsteps >= kGraphSteps) {
    if (!g->graph || g->graph_cur != g->cur) {
      if (g->graph) {
        cudaGraphExecDestroy(g->graph);
        g->graph = nullptr;
      }
      cudaGraph_t graph;
      const int cur0 = g->cur;
      const int64_t l0 = g->launches;
      FGB_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal), "graph capture");
      int rc = run_steps(g, kGraphSteps);
      cudaError_t e = cudaStreamEndCapture(g->stream, &graph);
      g->cur = cur0;
      g->launches = l0;
      if (rc != FGB_OK) return rc;
      if (e != cudaSuccess) return cuda_fail(e, "graph capture");
      e = cudaGraphInstantiate(&g->graph, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
      g->graph_cur = g->cur;
    }
    const int64_t per = (int64_t)kGraphSteps * g->prog->nstages;
    while (nsteps - done >= kGraphSteps) {
      FGB_CUDA(cudaGraphLaunch(g->graph, g->stream), "graph launch");
      g->launches += per;
      done += kGraphSteps;
    }
  }
  return run_steps(g, nsteps - done);
}

int fgb_synchronize(fgb_grid* g) {
  if (!g) return fail(FGB_E_ARG, "null grid");
  FGB_CUDA(cudaStreamSynchronize(g->stream), "synchronize");
  return FGB_OK;
}

void* fgb_stream(fgb_grid* g) { return g ? (void*)g->stream : nullptr; }

int fgb_state_device(fgb_grid* g, void** ptrs, int nfields) {
  if (!g || !ptrs || nfields != g->prog->nfields) return fail(FGB_E_ARG, "bad arguments");
  const size_t es = storage_size(g->precision);
  for (int f = 0; f < nfields; ++f) ptrs[f] = (char*)g->state[g->cur] + f * g->cells * es;
  return FGB_OK;
}

int64_t fgb_launch_count(fgb_grid* g) { return g ? g->launches : -1; }

int fgb_host_register(void* ptr, size_t bytes) {
  FGB_CUDA(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault), "host register");
  return FGB_OK;
}

int fgb_host_unregister(void* ptr) {
  FGB_CUDA(cudaHostUnregister(ptr), "host unregister");
  return FGB_OK;
}

}  // extern "C"

// Lets other translation units of the library report through fgb_last_error().
int fgb_internal_set_error(int code, const char* message) { return fail(code, "%s", message); }
