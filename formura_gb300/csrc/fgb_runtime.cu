// Runtime of the GB300 backend: device-resident grids, host<->device
// transfer of formura_data, and the time loop that replaces
// Formura_Forward's halo assembly + OpenMP loop nests
// (src/Formura/Generator/Templates.hs:295-346).
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <algorithm>
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

// FP64 sums of every field (conserved totals), whatever the storage type.
// One partial sum per block in FP64, then the host adds the partials in a
// fixed order, so the result does not depend on scheduling.
template <class S>
__global__ void field_partial_sums(const S* __restrict__ a, size_t n, double* __restrict__ partial) {
  __shared__ double red[256];
  double acc = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if constexpr (sizeof(S) == 2) acc += (double)__half2float(a[i]);
    else acc += (double)a[i];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

}  // namespace

// a normal power of two (+-2^k): division by it is exact as one product
// with its reciprocal, which is then a power of two as well
static bool is_pow2(double c) {
  uint64_t u;
  memcpy(&u, &c, sizeof u);
  const unsigned e = (unsigned)(u >> 52) & 0x7ffu;
  return (u & 0x000fffffffffffffull) == 0 && e >= 1u && e <= 2046u;
}

struct fgb_grid {
  const FgbProgramDesc* prog = nullptr;
  int precision = 0;
  bool p2 = false;   // FP64 steps through launch_p2 (every divisor a power of two)
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
  int variant = -1;                     // temporal-blocking kernel in use, -1: one step per launch
  // reverse mode
  void* lam[2] = {nullptr, nullptr};    // adjoint state, storage precision
  int lcur = 0;
  void* lam_mids = nullptr;             // multi-stage adjoint: adjoints of the forward arrays
  void* pairs = nullptr;                // and the partial sums of one stage (compute type)
  void* tmaps = nullptr;                // TMA tensor maps [2 state buffers][nfields], or null
  int* err = nullptr;                   // device flag of bounded waits that ran out
  std::vector<void*> snaps;             // checkpoints of the forward state
  int grad_steps = -1;                  // steps recorded by fgb_gradient_forward
  int64_t grad_fwd = 0, grad_adj = 0;   // forward steps (incl. recomputation) and adjoint steps
  // first_step / filter functions of the program (Templates.hs:252-270)
  struct Sub {
    const FgbProgramDesc* prog = nullptr;
    void* uniforms = nullptr;
    void* mids = nullptr;
  } sub[2];
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
  L->tmap = g->tmaps ? (const char*)g->tmaps + (size_t)cur * g->prog->nfields * FGB_TMA_MAP_BYTES : nullptr;
  L->err = g->err;
}

// TMA tensor maps of the two state buffers (2D or 3D, FP64/FP32 storage,
// rows of a multiple of 16 bytes): boxes of FGB_TMA_BOX^2 elements for the 2D
// tile kernels, planes of FGB_TMA_BOX x FGB_TMA_BOX3_Y for the 3D streaming
// kernels.  Without them (other grids, or no driver entry point) the
// kernels load their tiles with ordinary loads.
static void make_tensor_maps(fgb_grid* g) {
  const FgbProgramDesc* d = g->prog;
  const size_t es = storage_size(g->precision);
  const int boxy = d->dim == 3 ? FGB_TMA_BOX3_Y : FGB_TMA_BOX;
  if (d->dim < 2 || g->precision > FGB_F32 || (g->n[2] * es) % 16 != 0 || g->n[2] < FGB_TMA_BOX ||
      g->n[1] < boxy)
    return;
  static_assert(sizeof(CUtensorMap) == FGB_TMA_MAP_BYTES, "tensor map size");
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return;
  auto encode = reinterpret_cast<CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                              CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                              CUtensorMapFloatOOBfill)>(fn);
  std::vector<CUtensorMap> maps(2 * d->nfields);
  const cuuint32_t rank = (cuuint32_t)d->dim;
  const cuuint64_t dims[3] = {(cuuint64_t)g->n[2], (cuuint64_t)g->n[1], (cuuint64_t)g->n[0]};
  const cuuint64_t strides[2] = {(cuuint64_t)g->n[2] * es, (cuuint64_t)g->n[2] * g->n[1] * es};
  const cuuint32_t box[3] = {FGB_TMA_BOX, (cuuint32_t)boxy, 1};
  const cuuint32_t unit[3] = {1, 1, 1};
  const CUtensorMapDataType type = es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
  for (int b = 0; b < 2; ++b)
    for (int f = 0; f < d->nfields; ++f) {
      void* base = (char*)g->state[b] + f * g->cells * es;
      if (encode(&maps[b * d->nfields + f], type, rank, base, dims, strides, box, unit, CU_TENSOR_MAP_INTERLEAVE_NONE,
                 CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                 CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return;
    }
  void* dev = nullptr;
  if (cudaMalloc(&dev, maps.size() * sizeof(CUtensorMap)) != cudaSuccess) return;
  if (cudaMemcpy(dev, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaFree(dev);
    return;
  }
  g->tmaps = dev;
}

// Device address of a grid's error word (not part of the public header):
// lets a test raise the word from its own kernel, whose bounded wait runs out
// on a barrier nothing completes, and check how the runtime reports it.
extern "C" int* fgb_internal_error_word(fgb_grid* g) { return g ? g->err : nullptr; }

// a kernel's bounded wait ran out: report it once and clear the flag
static int check_device_flag(fgb_grid* g) {
  if (!g->err) return FGB_OK;
  int v = 0;
  FGB_CUDA(cudaMemcpy(&v, g->err, sizeof v, cudaMemcpyDeviceToHost), "device flag");
  if (v == 0) return FGB_OK;
  cudaMemset(g->err, 0, sizeof(int));
  return fail(FGB_E_CUDA, "a %s tile kernel's wait for its TMA load ran out", v == 2 ? "3D" : "2D");
}

static int run_steps(fgb_grid* g, int nsteps) {
  FgbLaunch L[2];
  fill_launch(g, 0, &L[0]);
  fill_launch(g, 1, &L[1]);
  if (g->variant >= 0) {
    const FgbFusedVariant& v = g->prog->fused[g->precision][g->variant];
    while (nsteps >= v.steps) {
      cudaError_t e = v.launch(&L[g->cur], g->stream);
      if (e != cudaSuccess) return cuda_fail(e, "fused launch");
      ++g->launches;
      g->cur ^= 1;
      nsteps -= v.steps;
    }
  }
  for (int s = 0; s < nsteps; ++s) {
    for (int st = 0; st < g->prog->nstages; ++st) {
      cudaError_t e = (g->p2 ? g->prog->launch_p2[st] : g->prog->launch[g->precision][st])(&L[g->cur], g->stream);
      if (e != cudaSuccess) return cuda_fail(e, "stage launch");
      ++g->launches;
    }
    g->cur ^= 1;
  }
  return FGB_OK;
}

extern "C" {

static void free_snaps(fgb_grid* g);

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
  const int nmids = std::max(d->nmids, d->nmids_adj);   // the forward's arrays, or the adjoint's
  if (e == cudaSuccess && nmids > 0) e = cudaMalloc(&g->mids, cells * nmids * cs);
  if (e == cudaSuccess && d->nuniforms > 0) e = cudaMalloc(&g->uniforms, d->nuniforms * cs);
  if (e == cudaSuccess && precision >= FGB_F32) e = cudaMalloc((void**)&g->staging, cells * d->nfields * 8);
  if (precision == FGB_F64 && d->ndivisors > 0) {
    g->p2 = true;
    for (int i = 0; i < d->ndivisors; ++i) g->p2 = g->p2 && is_pow2(uniforms[d->divisors[i]]);
  }
  if (e == cudaSuccess && d->nuniforms > 0) {
    if (cs == 8) {
      e = cudaMemcpy(g->uniforms, uniforms, d->nuniforms * 8, cudaMemcpyHostToDevice);
    } else {
      std::vector<float> u(uniforms, uniforms + d->nuniforms);
      e = cudaMemcpy(g->uniforms, u.data(), d->nuniforms * 4, cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(g->state[0], 0, cells * d->nfields * es, g->stream);
  if (e == cudaSuccess) e = cudaMalloc((void**)&g->err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(g->err, 0, sizeof(int), g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  if (e != cudaSuccess) {
    int rc = cuda_fail(e, "fgb_open");
    fgb_close(g);
    return rc;
  }
  make_tensor_maps(g);
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
  cudaFree(g->lam[0]);
  cudaFree(g->lam[1]);
  cudaFree(g->lam_mids);
  cudaFree(g->pairs);
  cudaFree(g->tmaps);
  cudaFree(g->err);
  for (auto& sb : g->sub) {
    cudaFree(sb.uniforms);
    cudaFree(sb.mids);
  }
  free_snaps(g);
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
  return check_device_flag(g);
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

int fgb_variant_count(fgb_grid* g) { return g ? g->prog->nfused[g->precision] : 0; }

int fgb_variant_info(fgb_grid* g, int index, int* tile_x, int* tile_y, int* steps) {
  if (!g || index < 0 || index >= g->prog->nfused[g->precision]) return fail(FGB_E_ARG, "no such variant");
  const FgbFusedVariant& v = g->prog->fused[g->precision][index];
  if (tile_x) *tile_x = v.tile_x;
  if (tile_y) *tile_y = v.tile_y;
  if (steps) *steps = v.steps;
  return FGB_OK;
}

static bool variant_fits(const fgb_grid* g, int index) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const FgbFusedVariant& v = g->prog->fused[g->precision][index];
  return v.smem_bytes <= (size_t)optin && (v.x_multiple <= 1 || g->n[2] % v.x_multiple == 0);
}

int fgb_set_variant(fgb_grid* g, int index) {
  if (!g || index < -1 || index >= g->prog->nfused[g->precision]) return fail(FGB_E_ARG, "no such variant");
  if (index >= 0 && !variant_fits(g, index))
    return fail(FGB_E_ARG, "variant %d does not fit this grid (it needs %zu bytes of shared memory and "
                "a contiguous axis that is a multiple of %d)", index,
                g->prog->fused[g->precision][index].smem_bytes, g->prog->fused[g->precision][index].x_multiple);
  if (index != g->variant && g->graph) {
    cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
  }
  g->variant = index;
  return FGB_OK;
}

int fgb_variant(fgb_grid* g) { return g ? g->variant : -1; }

int fgb_autotune(fgb_grid* g, int trial_steps, int* chosen) {
  if (!g || trial_steps < 8) return fail(FGB_E_ARG, "autotune needs a grid and at least 8 trial steps");
  const int nv = g->prog->nfused[g->precision];
  if (nv == 0) {
    if (chosen) *chosen = -1;
    return fgb_set_variant(g, -1);
  }
  const size_t bytes = g->cells * g->prog->nfields * storage_size(g->precision);
  void* backup = nullptr;
  FGB_CUDA(cudaMalloc(&backup, bytes), "autotune backup");
  FGB_CUDA(cudaMemcpyAsync(backup, g->state[g->cur], bytes, cudaMemcpyDeviceToDevice, g->stream), "autotune");
  const int64_t launches0 = g->launches;
  const int old_variant = g->variant;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.0f;
  int best_i = -1;
  int rc = FGB_OK;
  for (int i = -1; i < nv && rc == FGB_OK; ++i) {
    if (i >= 0 && !variant_fits(g, i)) continue;
    g->variant = i;
    const int k = i >= 0 ? g->prog->fused[g->precision][i].steps : 1;
    const int steps = ((trial_steps + k - 1) / k) * k;
    rc = run_steps(g, k);                       // warm-up (and kernel attribute set-up)
    if (rc != FGB_OK) break;
    cudaEventRecord(e0, g->stream);
    rc = run_steps(g, steps);
    cudaEventRecord(e1, g->stream);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "autotune");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    const float per_step = ms / steps;
    if (rc == FGB_OK && (i == -1 || per_step < best)) {
      best = per_step;
      best_i = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemcpyAsync(g->state[g->cur], backup, bytes, cudaMemcpyDeviceToDevice, g->stream);
  cudaStreamSynchronize(g->stream);
  cudaFree(backup);
  g->launches = launches0;
  g->variant = old_variant;
  if (rc != FGB_OK) return rc;
  if (chosen) *chosen = best_i;
  return fgb_set_variant(g, best_i);
}

// ---------------------------------------------------------------------------
// reverse mode: adjoint steps and checkpointed gradients
// ---------------------------------------------------------------------------
static size_t state_bytes(const fgb_grid* g) { return g->cells * g->prog->nfields * storage_size(g->precision); }

static bool stage_adjoint(const fgb_grid* g) {
  return g->prog->nstages > 1 && g->prog->adj_partial[g->precision][0] != nullptr;
}

static int ensure_adjoint(fgb_grid* g) {
  if (!g->prog->adjoint[g->precision] && !stage_adjoint(g))
    return fail(FGB_E_ARG, "program %s has no adjoint in this precision", g->prog->name);
  for (int b = 0; b < 2; ++b)
    if (!g->lam[b]) FGB_CUDA(cudaMalloc(&g->lam[b], state_bytes(g)), "adjoint state");
  if (stage_adjoint(g)) {
    const size_t cs = compute_size(g->precision);
    int most = 0;
    for (int s = 0; s < g->prog->nstages; ++s) most = std::max(most, g->prog->adj_pairs[s]);
    if (!g->lam_mids && g->prog->nmids_adj > 0)
      FGB_CUDA(cudaMalloc(&g->lam_mids, g->cells * g->prog->nmids_adj * cs), "adjoint of the forward arrays");
    if (!g->pairs && most > 0) FGB_CUDA(cudaMalloc(&g->pairs, g->cells * most * cs), "adjoint partial sums");
  }
  return FGB_OK;
}

// host FP64 (formura_data layout) <-> device state in storage precision
static int host_to_state(fgb_grid* g, const double* host, void* dst) {
  const size_t n = g->cells * g->prog->nfields;
  if (g->precision <= FGB_F64_FAST) {
    FGB_CUDA(cudaMemcpyAsync(dst, host, n * 8, cudaMemcpyHostToDevice, g->stream), "copy in");
  } else {
    FGB_CUDA(cudaMemcpyAsync(g->staging, host, n * 8, cudaMemcpyHostToDevice, g->stream), "copy in");
    if (g->precision == FGB_F32) to_storage<float><<<1024, 256, 0, g->stream>>>(g->staging, (float*)dst, n, 1.0f);
    else to_storage<__half><<<1024, 256, 0, g->stream>>>(g->staging, (__half*)dst, n, 1.0f);
    ++g->launches;
    FGB_CUDA(cudaGetLastError(), "copy in");
  }
  return FGB_OK;
}

static int state_to_host(fgb_grid* g, const void* src, double* host) {
  const size_t n = g->cells * g->prog->nfields;
  if (g->precision <= FGB_F64_FAST) {
    FGB_CUDA(cudaMemcpyAsync(host, src, n * 8, cudaMemcpyDeviceToHost, g->stream), "copy out");
  } else {
    if (g->precision == FGB_F32) from_storage<float><<<1024, 256, 0, g->stream>>>((const float*)src, g->staging, n, 1.0f);
    else from_storage<__half><<<1024, 256, 0, g->stream>>>((const __half*)src, g->staging, n, 1.0f);
    ++g->launches;
    FGB_CUDA(cudaGetLastError(), "copy out");
    FGB_CUDA(cudaMemcpyAsync(host, g->staging, n * 8, cudaMemcpyDeviceToHost, g->stream), "copy out");
  }
  FGB_CUDA(cudaStreamSynchronize(g->stream), "copy out");
  return FGB_OK;
}

// Multi-stage step: recompute from u the forward arrays that the partial
// sums read (the generator works out which; a linear last stage needs none
// of the arrays it reads), then run the adjoint passes of each stage from
// the last stage to the first.
static int stage_adjoint_step(fgb_grid* g, const void* u) {
  const FgbProgramDesc* d = g->prog;
  const size_t es = storage_size(g->precision), cs = compute_size(g->precision);
  FgbLaunch L;
  fill_launch(g, g->cur, &L);
  for (int f = 0; f < d->nfields; ++f) L.in[f] = (const char*)u + f * g->cells * es;
  // the program's own arrays, which the adjoint reads (the buffer holds
  // the larger of the two counts)
  for (int k = 0; k < d->nmids_adj; ++k) L.mid[k] = (char*)g->mids + k * g->cells * cs;
  // The arrays recomputed here only feed the partial sums, which evaluate
  // their own forward values in contracted arithmetic: in the FP64 form
  // they are recomputed with the contracted FP64 kernels too (same storage,
  // same uniform table).  The forward steps of a gradient stay exact.
  const int rp = g->precision == FGB_F64 ? FGB_F64_FAST : g->precision;
  for (int st = 0; st + 1 < d->nstages; ++st) {
    if (!d->adj_recompute[st]) continue;
    cudaError_t e = d->adj_launch[rp][st](&L, g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "stage launch");
    ++g->launches;
  }
  FgbAdjLaunch A;
  memset(&A, 0, sizeof A);
  for (int f = 0; f < d->nfields; ++f) {
    A.u[f] = (const char*)u + f * g->cells * es;
    A.lnext[f] = (const char*)g->lam[g->lcur] + f * g->cells * es;
    A.lprev[f] = (char*)g->lam[g->lcur ^ 1] + f * g->cells * es;
    A.scale[f] = g->scale[f];
  }
  for (int k = 0; k < d->nmids_adj; ++k) {
    A.mid[k] = (const char*)g->mids + k * g->cells * cs;
    A.lmid[k] = (char*)g->lam_mids + k * g->cells * cs;
  }
  for (int s = 0; s < d->nstages; ++s)
    if (d->adj_pairs[s] > FGB_MAX_PAIRS) return fail(FGB_E_ARG, "stage %d reads too many arrays", s);
  A.uniforms = g->uniforms;
  for (int a = 0; a < 3; ++a) A.n[a] = g->n[a];
  for (int s = d->nstages - 1; s >= 0; --s) {
    for (int j = 0; j < d->adj_pairs[s]; ++j) A.pair[j] = (char*)g->pairs + (size_t)j * g->cells * cs;
    cudaError_t e = d->adj_partial[g->precision][s](&A, g->stream);
    if (e == cudaSuccess) e = d->adj_gather[g->precision][s](&A, g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
    g->launches += d->adj_parts[s] + 1;
  }
  ++g->grad_adj;
  g->lcur ^= 1;
  return FGB_OK;
}

// lambda <- (dF/du at `u`)^T lambda
static int adjoint_step(fgb_grid* g, const void* u) {
  if (!g->prog->adjoint[g->precision]) return stage_adjoint_step(g, u);
  FgbLaunch L;
  fill_launch(g, g->cur, &L);
  const size_t es = storage_size(g->precision);
  for (int f = 0; f < g->prog->nfields; ++f) {
    L.in[f] = (const char*)u + f * g->cells * es;
    L.mid[f] = (char*)g->lam[g->lcur] + f * g->cells * es;
    L.out[f] = (char*)g->lam[g->lcur ^ 1] + f * g->cells * es;
  }
  cudaError_t e = g->prog->adjoint[g->precision](&L, g->stream);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
  ++g->launches;
  ++g->grad_adj;
  g->lcur ^= 1;
  return FGB_OK;
}

static int64_t binom(int s, int t) {   // C(s + t, s), saturating
  double r = 1.0;
  for (int i = 1; i <= s; ++i) r = r * (t + i) / i;
  return r > 4e18 ? (int64_t)4e18 : (int64_t)(r + 0.5);
}

struct Reversal {
  fgb_grid* g;
  std::vector<int> free_slots;
  size_t bytes;

  int restore(int slot) {
    FGB_CUDA(cudaMemcpyAsync(g->state[g->cur], g->snaps[slot], bytes, cudaMemcpyDeviceToDevice, g->stream),
             "restore checkpoint");
    return FGB_OK;
  }
  int advance(int n) {
    g->grad_fwd += n;
    return run_steps(g, n);
  }
  // u_l is in checkpoint `slot`; lambda holds lambda_r; leaves lambda_l.
  int reverse(int l, int r, int slot) {
    int rc;
    if (r - l == 1) {
      if ((rc = restore(slot)) != FGB_OK) return rc;
      return adjoint_step(g, g->state[g->cur]);
    }
    const int s = (int)free_slots.size();
    if (s == 0) {
      // no free checkpoint: recompute each state from u_l
      for (int k = r - 1; k >= l; --k) {
        if ((rc = restore(slot)) != FGB_OK) return rc;
        if ((rc = advance(k - l)) != FGB_OK) return rc;
        if ((rc = adjoint_step(g, g->state[g->cur])) != FGB_OK) return rc;
      }
      return FGB_OK;
    }
    // binomial split: [m, r) is reversed with s-1 free checkpoints and
    // [l, m) with s, each within t sweeps (Griewank's revolve bound)
    int t = 1;
    while (binom(s, t) < r - l) ++t;
    int m = r - (int)std::min<int64_t>(binom(s - 1, t), r - l - 1);
    if (m <= l) m = l + 1;
    if ((rc = restore(slot)) != FGB_OK) return rc;
    if ((rc = advance(m - l)) != FGB_OK) return rc;
    const int sm = free_slots.back();
    free_slots.pop_back();
    FGB_CUDA(cudaMemcpyAsync(g->snaps[sm], g->state[g->cur], bytes, cudaMemcpyDeviceToDevice, g->stream),
             "store checkpoint");
    rc = reverse(m, r, sm);
    free_slots.push_back(sm);
    if (rc != FGB_OK) return rc;
    return reverse(l, m, slot);
  }
};

static void free_snaps(fgb_grid* g) {
  for (void* p : g->snaps) cudaFree(p);
  g->snaps.clear();
}

int fgb_backward(fgb_grid* g, const double* lambda_next, double* lambda) {
  if (!g || !lambda_next || !lambda) return fail(FGB_E_ARG, "null argument");
  int rc = ensure_adjoint(g);
  if (rc != FGB_OK) return rc;
  if ((rc = host_to_state(g, lambda_next, g->lam[g->lcur])) != FGB_OK) return rc;
  if ((rc = adjoint_step(g, g->state[g->cur])) != FGB_OK) return rc;
  return state_to_host(g, g->lam[g->lcur], lambda);
}

int fgb_adjoint_steps(fgb_grid* g, int nsteps) {
  if (!g || nsteps < 0) return fail(FGB_E_ARG, "bad arguments");
  int rc = ensure_adjoint(g);
  for (int i = 0; i < nsteps && rc == FGB_OK; ++i) rc = adjoint_step(g, g->state[g->cur]);
  return rc;
}

int fgb_gradient_forward(fgb_grid* g, int nsteps, int snapshots) {
  if (!g || nsteps < 1 || snapshots < 1) return fail(FGB_E_ARG, "need nsteps >= 1 and snapshots >= 1");
  int rc = ensure_adjoint(g);
  if (rc != FGB_OK) return rc;
  free_snaps(g);
  for (int i = 0; i < snapshots; ++i) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, state_bytes(g));
    if (e != cudaSuccess) {
      free_snaps(g);
      return cuda_fail(e, "checkpoint buffers");
    }
    g->snaps.push_back(p);
  }
  FGB_CUDA(cudaMemcpyAsync(g->snaps[0], g->state[g->cur], state_bytes(g), cudaMemcpyDeviceToDevice, g->stream),
           "checkpoint u0");
  g->grad_fwd = nsteps;
  g->grad_adj = 0;
  g->grad_steps = nsteps;
  return run_steps(g, nsteps);
}

static int gradient_backward(fgb_grid* g) {
  if (g->grad_steps < 1) return fail(FGB_E_ARG, "fgb_gradient_forward was not called");
  Reversal R{g, {}, state_bytes(g)};
  for (int i = (int)g->snaps.size() - 1; i >= 1; --i) R.free_slots.push_back(i);
  int rc = R.reverse(0, g->grad_steps, 0);
  if (rc == FGB_OK) rc = R.restore(0);          // the state is u_0 again
  g->grad_steps = -1;
  if (rc == FGB_OK) {
    cudaError_t e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "gradient");
  }
  free_snaps(g);
  return rc;
}

int fgb_gradient_backward(fgb_grid* g, const double* seed, double* grad) {
  if (!g || !seed || !grad) return fail(FGB_E_ARG, "null argument");
  int rc = ensure_adjoint(g);
  if (rc != FGB_OK) return rc;
  if ((rc = host_to_state(g, seed, g->lam[g->lcur])) != FGB_OK) return rc;
  if ((rc = gradient_backward(g)) != FGB_OK) return rc;
  return state_to_host(g, g->lam[g->lcur], grad);
}

int fgb_gradient_backward_device(fgb_grid* g, const void* seed, void* grad) {
  if (!g || !seed || !grad) return fail(FGB_E_ARG, "null argument");
  int rc = ensure_adjoint(g);
  if (rc != FGB_OK) return rc;
  FGB_CUDA(cudaMemcpyAsync(g->lam[g->lcur], seed, state_bytes(g), cudaMemcpyDeviceToDevice, g->stream), "seed");
  if ((rc = gradient_backward(g)) != FGB_OK) return rc;
  FGB_CUDA(cudaMemcpyAsync(grad, g->lam[g->lcur], state_bytes(g), cudaMemcpyDeviceToDevice, g->stream), "gradient");
  FGB_CUDA(cudaStreamSynchronize(g->stream), "gradient");
  return FGB_OK;
}

int fgb_gradient_stats(fgb_grid* g, int64_t* forward_steps, int64_t* adjoint_steps) {
  if (!g) return fail(FGB_E_ARG, "null grid");
  if (forward_steps) *forward_steps = g->grad_fwd;
  if (adjoint_steps) *adjoint_steps = g->grad_adj;
  return FGB_OK;
}

static int sub_index(const char* which) {
  if (!which) return -1;
  if (strcmp(which, "first_step") == 0) return 0;
  if (strcmp(which, "filter") == 0) return 1;
  return -1;
}

int fgb_attach(fgb_grid* g, const char* which, const double* uniforms, int nuniforms) {
  const int k = sub_index(which);
  if (!g || k < 0) return fail(FGB_E_ARG, "attach: expected \"first_step\" or \"filter\"");
  char name[256];
  snprintf(name, sizeof name, "%s__%s", g->prog->name, which);
  const FgbProgramDesc* d = find_program(name);
  if (!d) return fail(FGB_E_PROGRAM, "program %s has no %s function in this library", g->prog->name, which);
  if (d->nfields != g->prog->nfields || d->dim != g->prog->dim)
    return fail(FGB_E_ARG, "%s does not match the step's state", name);
  if (nuniforms != d->nuniforms || (nuniforms > 0 && !uniforms))
    return fail(FGB_E_ARG, "%s needs %d uniform values, got %d", name, d->nuniforms, nuniforms);
  // every axis of the program (not only those longer than one point) must
  // hold the attached function's reach and roll
  for (int a = 3 - d->dim; a < 3; ++a) {
    const int need = d->reach > d->shift ? d->reach : d->shift;
    if (g->n[a] < need) return fail(FGB_E_ARG, "grid too small for %s", name);
  }
  fgb_grid::Sub& s = g->sub[k];
  cudaFree(s.uniforms);
  cudaFree(s.mids);
  s = fgb_grid::Sub();
  const size_t cs = compute_size(g->precision);
  if (d->nuniforms > 0) {
    FGB_CUDA(cudaMalloc(&s.uniforms, d->nuniforms * cs), "attach");
    if (cs == 8) {
      FGB_CUDA(cudaMemcpy(s.uniforms, uniforms, d->nuniforms * 8, cudaMemcpyHostToDevice), "attach");
    } else {
      std::vector<float> u(uniforms, uniforms + d->nuniforms);
      FGB_CUDA(cudaMemcpy(s.uniforms, u.data(), u.size() * 4, cudaMemcpyHostToDevice), "attach");
    }
  }
  if (d->nmids > 0) FGB_CUDA(cudaMalloc(&s.mids, g->cells * d->nmids * cs), "attach");
  s.prog = d;
  return FGB_OK;
}

int fgb_apply(fgb_grid* g, const char* which) {
  const int k = sub_index(which);
  if (!g || k < 0 || !g->sub[k].prog) return fail(FGB_E_ARG, "%s is not attached", which ? which : "(null)");
  const fgb_grid::Sub& s = g->sub[k];
  FgbLaunch L;
  fill_launch(g, g->cur, &L);
  const size_t cs = compute_size(g->precision);
  for (int m = 0; m < s.prog->nmids; ++m) L.mid[m] = (char*)s.mids + m * g->cells * cs;
  L.uniforms = s.uniforms;
  for (int st = 0; st < s.prog->nstages; ++st) {
    cudaError_t e = s.prog->launch[g->precision][st](&L, g->stream);
    if (e != cudaSuccess) return cuda_fail(e, "apply");
    ++g->launches;
  }
  g->cur ^= 1;
  return FGB_OK;
}

int fgb_totals(fgb_grid* g, double* sums, int nfields) {
  if (!g || !sums || nfields != g->prog->nfields) return fail(FGB_E_ARG, "bad totals arguments");
  const int blocks = 608;   // 4 per SM on 152 SMs
  double* partial = nullptr;
  FGB_CUDA(cudaMalloc(&partial, (size_t)blocks * nfields * sizeof(double)), "totals");
  const size_t es = storage_size(g->precision);
  for (int f = 0; f < nfields; ++f) {
    const void* a = (const char*)g->state[g->cur] + f * g->cells * es;
    double* p = partial + (size_t)f * blocks;
    if (es == 8) field_partial_sums<double><<<blocks, 256, 0, g->stream>>>((const double*)a, g->cells, p);
    else if (es == 4) field_partial_sums<float><<<blocks, 256, 0, g->stream>>>((const float*)a, g->cells, p);
    else field_partial_sums<__half><<<blocks, 256, 0, g->stream>>>((const __half*)a, g->cells, p);
    ++g->launches;
  }
  std::vector<double> h((size_t)blocks * nfields);
  cudaError_t e = cudaMemcpyAsync(h.data(), partial, h.size() * sizeof(double), cudaMemcpyDeviceToHost, g->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
  cudaFree(partial);
  if (e != cudaSuccess) return cuda_fail(e, "totals");
  for (int f = 0; f < nfields; ++f) {
    double s = 0.0;
    for (int b = 0; b < blocks; ++b) s += h[(size_t)f * blocks + b];
    sums[f] = f < (int)FGB_MAX_FIELDS && g->precision == FGB_F16 ? s * g->scale[f] : s;
  }
  return FGB_OK;
}

int fgb_synchronize(fgb_grid* g) {
  if (!g) return fail(FGB_E_ARG, "null grid");
  FGB_CUDA(cudaStreamSynchronize(g->stream), "synchronize");
  return check_device_flag(g);
}

void* fgb_stream(fgb_grid* g) { return g ? (void*)g->stream : nullptr; }

int fgb_state_device(fgb_grid* g, void** ptrs, int nfields) {
  if (!g || !ptrs || nfields != g->prog->nfields) return fail(FGB_E_ARG, "bad arguments");
  const size_t es = storage_size(g->precision);
  for (int f = 0; f < nfields; ++f) ptrs[f] = (char*)g->state[g->cur] + f * g->cells * es;
  return FGB_OK;
}

int64_t fgb_launch_count(fgb_grid* g) { return g ? g->launches : -1; }

// A refused registration leaves the memory pageable (copies still work,
// more slowly).  Its error is not sticky, so it is cleared here: otherwise
// the runtime would report it again at the next launch check.
int fgb_host_register(void* ptr, size_t bytes) {
  const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return cuda_fail(e, "host register");
  }
  return FGB_OK;
}

int fgb_host_unregister(void* ptr) {
  const cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return cuda_fail(e, "host unregister");
  }
  return FGB_OK;
}

}  // extern "C"

// Lets other translation units of the library report through fgb_last_error().
int fgb_internal_set_error(int code, const char* message) { return fail(code, "%s", message); }
