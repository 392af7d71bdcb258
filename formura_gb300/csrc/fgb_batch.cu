// Batched ensembles of one single-stage 2D program: many independent periodic
// grids of different extents and per-grid parameters, advanced together by
// persistent launches over a tile queue that spans every grid.  A chunk of
// steps is captured once in a CUDA graph and replayed for the time loop.
// The reference runs one grid per process; this is an extension for
// ensembles (parameter sweeps) on one GPU.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#include "fgb_internal.h"
#include "../../include/formura_gb300.h"

extern "C" const FgbProgramGetter fgb_builtin_programs[];
extern "C" const int fgb_builtin_program_count;
int fgb_internal_set_error(int code, const char* message);

namespace {

int error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return fgb_internal_set_error(code, buf);
}

int cuda_error(cudaError_t e, const char* what) {
  return error(e == cudaErrorMemoryAllocation ? FGB_E_NOMEM : FGB_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define BATCH_CUDA(call, what)                               \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_error(e_, what);      \
  } while (0)

const int kChunkSteps = 64;   // steps per captured graph (a multiple of every fused depth)

}  // namespace

struct fgb_batch {
  const FgbProgramDesc* prog = nullptr;
  int precision = 0;
  int count = 0;
  std::vector<int> ny, nx;
  std::vector<size_t> offset;        // element offset of each grid's buffer pair
  size_t total = 0;                  // elements of one buffer set
  void* states = nullptr;            // [2][total] storage elements
  void* uniforms = nullptr;          // [count][nuniforms] compute elements
  FgbBatchInstance* d_inst = nullptr;
  FgbBatchTile* d_tiles[2] = {nullptr, nullptr};   // queue of the selected variant, of variant 0
  int ntiles[2] = {0, 0};
  int blocks[2] = {0, 0};
  double* staging = nullptr;         // FP64 staging for one grid (F32 transfers)
  size_t staging_cells = 0;
  cudaStream_t stream = nullptr;
  int parity = 0;
  int variant = 0;
  int64_t launches = 0;
  cudaGraphExec_t graph = nullptr;
  int graph_parity = -1;
  int64_t graph_per = 0;             // kernel launches in one captured chunk
};

static size_t batch_es(int p) { return p <= FGB_F64_FAST ? 8 : 4; }

// Tile queue (and persistent grid size) for variant `v` into slot `q`.
static int build_queue(fgb_batch* b, int q, int v) {
  const FgbBatchVariant& var = b->prog->batch[b->precision][v];
  std::vector<FgbBatchTile> tiles;
  for (int i = 0; i < b->count; ++i)
    for (int y0 = 0; y0 < b->ny[i]; y0 += var.tile_y)
      for (int x0 = 0; x0 < b->nx[i]; x0 += var.tile_x) tiles.push_back({i, y0, x0, 0});
  BATCH_CUDA(cudaStreamSynchronize(b->stream), "tile queue");
  cudaFree(b->d_tiles[q]);
  b->d_tiles[q] = nullptr;
  BATCH_CUDA(cudaMalloc(&b->d_tiles[q], tiles.size() * sizeof(FgbBatchTile)), "tile queue");
  BATCH_CUDA(cudaMemcpy(b->d_tiles[q], tiles.data(), tiles.size() * sizeof(FgbBatchTile), cudaMemcpyHostToDevice),
             "tile queue");
  b->ntiles[q] = (int)tiles.size();
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = var.blocks_per_sm();
  if (per_sm < 1) return error(FGB_E_ARG, "batch variant %d does not fit on this device", v);
  b->blocks[q] = sms * per_sm < b->ntiles[q] ? sms * per_sm : b->ntiles[q];   // persistent grid
  return FGB_OK;
}

static int build_tiles(fgb_batch* b) {
  int rc = build_queue(b, 0, b->variant);
  if (rc == FGB_OK) rc = build_queue(b, 1, 0);
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return rc;
}

static int batch_launch(fgb_batch* b, int variant, int q) {
  const FgbBatchVariant& v = b->prog->batch[b->precision][variant];
  FgbBatchLaunch L{b->d_inst, b->d_tiles[q], b->ntiles[q], b->parity};
  cudaError_t e = v.launch(&L, b->stream, b->blocks[q]);
  if (e != cudaSuccess) return cuda_error(e, "batch launch");
  ++b->launches;
  b->parity ^= 1;
  return FGB_OK;
}

// Steps with the selected variant; leftovers with the one-step kernel
// (variant 0) on its own tile queue.
static int batch_steps(fgb_batch* b, int nsteps) {
  const int k = b->prog->batch[b->precision][b->variant].steps;
  int rc = FGB_OK;
  while (nsteps >= k && rc == FGB_OK) {
    rc = batch_launch(b, b->variant, 0);
    nsteps -= k;
  }
  while (nsteps-- > 0 && rc == FGB_OK) rc = batch_launch(b, 0, 1);
  return rc;
}

extern "C" {

int fgb_batch_open(const char* program, int count, const int* shapes, int precision, const double* uniforms,
                   int nuniforms, fgb_batch** out) {
  if (!out) return error(FGB_E_ARG, "out is null");
  *out = nullptr;
  const FgbProgramDesc* d = nullptr;
  for (int i = 0; program && i < fgb_builtin_program_count; ++i)
    if (strcmp(fgb_builtin_programs[i]()->name, program) == 0) d = fgb_builtin_programs[i]();
  if (!d) return error(FGB_E_PROGRAM, "unknown program '%s'", program ? program : "(null)");
  if (precision < 0 || precision >= FGB_NUM_PRECISIONS || d->nbatch[precision] == 0)
    return error(FGB_E_ARG, "program %s has no batched kernels in precision %d", d->name, precision);
  if (count < 1 || !shapes) return error(FGB_E_ARG, "empty batch");
  if (nuniforms != d->nuniforms || (nuniforms > 0 && !uniforms))
    return error(FGB_E_ARG, "program %s needs %d uniform values per grid", d->name, d->nuniforms);
  fgb_batch* b = new fgb_batch();
  b->prog = d;
  b->precision = precision;
  b->count = count;
  const int need = d->reach > d->shift ? d->reach : d->shift;
  size_t maxcells = 0;
  for (int i = 0; i < count; ++i) {
    const int y = shapes[2 * i], x = shapes[2 * i + 1];
    if (y < need || x < need) {
      delete b;
      return error(FGB_E_ARG, "grid %d is %dx%d; the program reads %d points away", i, y, x, need);
    }
    b->ny.push_back(y);
    b->nx.push_back(x);
    b->offset.push_back(b->total);
    const size_t cells = (size_t)y * x;
    b->total += cells * d->nfields;
    if (cells > maxcells) maxcells = cells;
  }
  const size_t es = batch_es(precision);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&b->states, 2 * b->total * es);
  if (e == cudaSuccess && nuniforms > 0) e = cudaMalloc(&b->uniforms, (size_t)count * nuniforms * es);
  if (e == cudaSuccess) e = cudaMalloc(&b->d_inst, count * sizeof(FgbBatchInstance));
  if (e == cudaSuccess && precision == FGB_F32) {
    b->staging_cells = maxcells * d->nfields;
    e = cudaMalloc((void**)&b->staging, b->staging_cells * 8);
  }
  if (e == cudaSuccess && nuniforms > 0) {
    if (es == 8) {
      e = cudaMemcpy(b->uniforms, uniforms, (size_t)count * nuniforms * 8, cudaMemcpyHostToDevice);
    } else {
      std::vector<float> u(uniforms, uniforms + (size_t)count * nuniforms);
      e = cudaMemcpy(b->uniforms, u.data(), u.size() * 4, cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess) {
    std::vector<FgbBatchInstance> inst(count);
    for (int i = 0; i < count; ++i) {
      inst[i].state[0] = (char*)b->states + b->offset[i] * es;
      inst[i].state[1] = (char*)b->states + (b->total + b->offset[i]) * es;
      inst[i].uniforms = (char*)b->uniforms + (size_t)i * nuniforms * es;
      inst[i].ny = b->ny[i];
      inst[i].nx = b->nx[i];
    }
    e = cudaMemcpy(b->d_inst, inst.data(), count * sizeof(FgbBatchInstance), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(b->states, 0, 2 * b->total * es);
  int rc = e == cudaSuccess ? build_tiles(b) : cuda_error(e, "fgb_batch_open");
  if (rc != FGB_OK) {
    fgb_batch_close(b);
    return rc;
  }
  *out = b;
  return FGB_OK;
}

int fgb_batch_close(fgb_batch* b) {
  if (!b) return FGB_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  cudaFree(b->states);
  cudaFree(b->uniforms);
  cudaFree(b->d_inst);
  cudaFree(b->d_tiles[0]);
  cudaFree(b->d_tiles[1]);
  cudaFree(b->staging);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return FGB_OK;
}

static __global__ void batch_to_f32(const double* src, float* dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}
static __global__ void batch_from_f32(const float* src, double* dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}

int fgb_batch_upload(fgb_batch* b, int index, const double* host) {
  if (!b || !host || index < 0 || index >= b->count) return error(FGB_E_ARG, "bad batch upload");
  const size_t n = (size_t)b->ny[index] * b->nx[index] * b->prog->nfields;
  char* dst = (char*)b->states + (b->parity * b->total + b->offset[index]) * batch_es(b->precision);
  if (b->precision <= FGB_F64_FAST) {
    BATCH_CUDA(cudaMemcpyAsync(dst, host, n * 8, cudaMemcpyHostToDevice, b->stream), "batch upload");
  } else {
    BATCH_CUDA(cudaMemcpyAsync(b->staging, host, n * 8, cudaMemcpyHostToDevice, b->stream), "batch upload");
    batch_to_f32<<<256, 256, 0, b->stream>>>(b->staging, (float*)dst, n);
    ++b->launches;
  }
  BATCH_CUDA(cudaStreamSynchronize(b->stream), "batch upload");
  return FGB_OK;
}

int fgb_batch_download(fgb_batch* b, int index, double* host) {
  if (!b || !host || index < 0 || index >= b->count) return error(FGB_E_ARG, "bad batch download");
  const size_t n = (size_t)b->ny[index] * b->nx[index] * b->prog->nfields;
  const char* src = (const char*)b->states + (b->parity * b->total + b->offset[index]) * batch_es(b->precision);
  if (b->precision <= FGB_F64_FAST) {
    BATCH_CUDA(cudaMemcpyAsync(host, src, n * 8, cudaMemcpyDeviceToHost, b->stream), "batch download");
  } else {
    batch_from_f32<<<256, 256, 0, b->stream>>>((const float*)src, b->staging, n);
    ++b->launches;
    BATCH_CUDA(cudaMemcpyAsync(host, b->staging, n * 8, cudaMemcpyDeviceToHost, b->stream), "batch download");
  }
  BATCH_CUDA(cudaStreamSynchronize(b->stream), "batch download");
  return FGB_OK;
}

int fgb_batch_variant_count(fgb_batch* b) { return b ? b->prog->nbatch[b->precision] : 0; }

int fgb_batch_variant_info(fgb_batch* b, int index, int* tile_x, int* tile_y, int* steps) {
  if (!b || index < 0 || index >= b->prog->nbatch[b->precision]) return error(FGB_E_ARG, "no such variant");
  const FgbBatchVariant& v = b->prog->batch[b->precision][index];
  if (tile_x) *tile_x = v.tile_x;
  if (tile_y) *tile_y = v.tile_y;
  if (steps) *steps = v.steps;
  return FGB_OK;
}

int fgb_batch_set_variant(fgb_batch* b, int index) {
  if (!b || index < 0 || index >= b->prog->nbatch[b->precision]) return error(FGB_E_ARG, "no such variant");
  const int old = b->variant;
  b->variant = index;
  int rc = build_tiles(b);
  if (rc != FGB_OK) {
    b->variant = old;
    build_tiles(b);
  }
  return rc;
}

int fgb_batch_variant(fgb_batch* b) { return b ? b->variant : -1; }

int fgb_batch_forward(fgb_batch* b, int nsteps) {
  if (!b || nsteps < 0) return error(FGB_E_ARG, "bad batch forward");
  int done = 0;
  if (nsteps >= kChunkSteps) {
    if (!b->graph || b->graph_parity != b->parity) {
      if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
      }
      const int p0 = b->parity;
      const int64_t l0 = b->launches;
      cudaGraph_t graph;
      BATCH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "batch capture");
      int rc = batch_steps(b, kChunkSteps);
      cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
      b->graph_per = b->launches - l0;
      b->parity = p0;
      b->launches = l0;
      if (rc != FGB_OK) return rc;
      if (e != cudaSuccess) return cuda_error(e, "batch capture");
      e = cudaGraphInstantiate(&b->graph, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return cuda_error(e, "batch graph");
      b->graph_parity = p0;
    }
    while (nsteps - done >= kChunkSteps) {
      BATCH_CUDA(cudaGraphLaunch(b->graph, b->stream), "batch graph launch");
      b->launches += b->graph_per;
      b->parity ^= (int)(b->graph_per & 1);
      done += kChunkSteps;
      if (b->graph_per & 1) break;     // parity changed: the captured chunk no longer applies
    }
  }
  if (nsteps - done >= kChunkSteps) return fgb_batch_forward(b, nsteps - done);
  return batch_steps(b, nsteps - done);
}

int fgb_batch_autotune(fgb_batch* b, int trial_steps, int* chosen) {
  if (!b || trial_steps < 8) return error(FGB_E_ARG, "autotune needs at least 8 trial steps");
  // time every variant on a copy of the state, then restore it
  const size_t bytes = 2 * b->total * batch_es(b->precision);
  void* backup = nullptr;
  BATCH_CUDA(cudaMalloc(&backup, bytes), "batch autotune");
  BATCH_CUDA(cudaMemcpyAsync(backup, b->states, bytes, cudaMemcpyDeviceToDevice, b->stream), "batch autotune");
  const int p0 = b->parity, v0 = b->variant;
  const int64_t l0 = b->launches;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.0f;
  int best_i = -1, rc = FGB_OK;
  for (int i = 0; i < b->prog->nbatch[b->precision] && rc == FGB_OK; ++i) {
    if (b->prog->batch[b->precision][i].blocks_per_sm() < 1) continue;
    b->variant = i;
    if ((rc = build_tiles(b)) != FGB_OK) break;
    const int k = b->prog->batch[b->precision][i].steps;
    const int steps = ((trial_steps + k - 1) / k) * k;
    if ((rc = batch_steps(b, k)) != FGB_OK) break;
    cudaEventRecord(e0, b->stream);
    rc = batch_steps(b, steps);
    cudaEventRecord(e1, b->stream);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rc == FGB_OK && (best_i < 0 || ms / steps < best)) {
      best = ms / steps;
      best_i = i;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaMemcpyAsync(b->states, backup, bytes, cudaMemcpyDeviceToDevice, b->stream);
  cudaStreamSynchronize(b->stream);
  cudaFree(backup);
  b->parity = p0;
  b->launches = l0;
  b->variant = best_i >= 0 ? best_i : v0;
  int rc2 = build_tiles(b);
  if (rc != FGB_OK) return rc;
  if (chosen) *chosen = b->variant;
  return rc2;
}

int fgb_batch_synchronize(fgb_batch* b) {
  if (!b) return error(FGB_E_ARG, "null batch");
  BATCH_CUDA(cudaStreamSynchronize(b->stream), "batch synchronize");
  return FGB_OK;
}

void* fgb_batch_stream(fgb_batch* b) { return b ? (void*)b->stream : nullptr; }

int64_t fgb_batch_launch_count(fgb_batch* b) { return b ? b->launches : -1; }

}  // extern "C"
