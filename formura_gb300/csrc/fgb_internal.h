// Internal interface between the runtime (fgb_runtime.cu) and the
// per-program kernel instantiations (generated from each program's step
// function, compiled against fgb_templates.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define FGB_MAX_FIELDS 16
#define FGB_MAX_MIDS 160
#define FGB_MAX_STAGES 8
#define FGB_NUM_PRECISIONS 4
#define FGB_MAX_DIVISORS 64

// Arguments of one stage launch.  Field and intermediate pointers are
// device pointers; their element type is fixed by the precision (storage
// type for state fields, compute type for intermediates and uniforms).
struct FgbLaunch {
  const void* in[FGB_MAX_FIELDS];
  void* out[FGB_MAX_FIELDS];
  void* mid[FGB_MAX_MIDS];
  const void* uniforms;
  float scale[FGB_MAX_FIELDS];      // half storage: value = stored * scale
  float inv_scale[FGB_MAX_FIELDS];
  int n[3];                         // grid extent, leading axes padded with 1
  int fused_steps;                  // >1: temporal blocking inside one launch
  // 2D and 3D grids in FP64/FP32 storage: one TMA tensor map per field of
  // `in` (device memory; boxes of FGB_TMA_BOX x FGB_TMA_BOX elements in 2D,
  // one plane of FGB_TMA_BOX x FGB_TMA_BOX3_Y in 3D), or null
  const void* tmap;
  int* err;                         // set by a kernel whose bounded wait ran out
};

#define FGB_TMA_BOX 64        // 2D box: 64 x 64; 3D box: 64 x FGB_TMA_BOX3_Y x 1
#define FGB_TMA_BOX3_Y 32
#define FGB_TMA_MAP_BYTES 128

#define FGB_MAX_FUSED 12

typedef cudaError_t (*FgbStageLaunch)(const FgbLaunch* args, cudaStream_t stream);

// One temporal-blocking kernel: `steps` time steps per launch on tiles of
// tile_x x tile_y output cells (single-stage programs only).
struct FgbFusedVariant {
  FgbStageLaunch launch;
  int tile_x, tile_y, steps;
  size_t smem_bytes;
  int x_multiple;          // the contiguous axis must be a multiple of this
};

// Batched ensembles: many independent 2D grids of one single-stage program,
// each with its own extent and uniform table, advanced together.
struct FgbBatchInstance {
  void* state[2];          // the two state buffers (fields back to back)
  const void* uniforms;    // this grid's uniform table (compute type)
  int ny, nx;              // extent; x is the contiguous axis
};
struct FgbBatchTile {
  int inst, y0, x0, pad;
};
struct FgbBatchLaunch {
  const FgbBatchInstance* inst;
  const FgbBatchTile* tiles;
  int ntiles;
  int parity;              // state buffer read by this launch
};
typedef cudaError_t (*FgbBatchFn)(const FgbBatchLaunch* args, cudaStream_t stream, int blocks);
typedef int (*FgbOccupancyFn)(void);
struct FgbBatchVariant {
  FgbBatchFn launch;
  FgbOccupancyFn blocks_per_sm;
  int tile_x, tile_y, steps;
  size_t smem_bytes;
};

// Adjoint of a multi-stage step (two passes per stage, see the generator's
// adjoint.py): u and mid are the forward state u_n and the step's forward
// arrays; lnext / lprev the adjoint of the new and of the old state (storage
// type); lmid the adjoints of the forward arrays and pair the per-point
// partial sums of one stage (compute type).
#define FGB_MAX_PAIRS 256
struct FgbAdjLaunch {
  const void* u[FGB_MAX_FIELDS];
  const void* mid[FGB_MAX_MIDS];
  const void* lnext[FGB_MAX_FIELDS];
  void* lprev[FGB_MAX_FIELDS];
  void* lmid[FGB_MAX_MIDS];
  void* pair[FGB_MAX_PAIRS];
  const void* uniforms;
  float scale[FGB_MAX_FIELDS];
  int n[3];
};
typedef cudaError_t (*FgbAdjLaunchFn)(const FgbAdjLaunch* args, cudaStream_t stream);

struct FgbProgramDesc {
  const char* name;
  int dim, nfields, nmids, nstages, sleeve, shift, reach, nuniforms;
  const char* const* field_names;
  FgbStageLaunch launch[FGB_NUM_PRECISIONS][FGB_MAX_STAGES];
  FgbFusedVariant fused[FGB_NUM_PRECISIONS][FGB_MAX_FUSED];
  int nfused[FGB_NUM_PRECISIONS];
  // Adjoint step (transpose of the step's Jacobian), single-stage programs:
  // in = forward state u_n, mid[f] = lambda_{n+1}, out = lambda_n.
  FgbStageLaunch adjoint[FGB_NUM_PRECISIONS];
  FgbBatchVariant batch[FGB_NUM_PRECISIONS][FGB_MAX_FUSED];
  int nbatch[FGB_NUM_PRECISIONS];
  // Adjoint of a multi-stage step: per stage, the partial-sum pass and the
  // gather pass, and the number of (input array, cursor) pairs it reads.
  FgbAdjLaunchFn adj_partial[FGB_NUM_PRECISIONS][FGB_MAX_STAGES];
  FgbAdjLaunchFn adj_gather[FGB_NUM_PRECISIONS][FGB_MAX_STAGES];
  int adj_pairs[FGB_MAX_STAGES];
  int adj_parts[FGB_MAX_STAGES];   // partial-sum kernels per stage
  int adj_recompute[FGB_MAX_STAGES];   // forward arrays of the stage read by the partial sums
  // The forward stages whose arrays the adjoint reads, and how many arrays
  // they store: the program's own stored arrays, which may differ from the
  // ones the forward step stores (the generator chooses those for HBM
  // traffic); the same as launch / nmids when they do not differ.
  FgbStageLaunch adj_launch[FGB_NUM_PRECISIONS][FGB_MAX_STAGES];
  int nmids_adj;
  // Uniform-table slots of the grid-independent divisors; when all of them
  // are powers of two for a grid, its FP64 steps use launch_p2, whose
  // division by them is one product.
  int ndivisors;
  int divisors[FGB_MAX_DIVISORS];
  FgbStageLaunch launch_p2[FGB_MAX_STAGES];
};

typedef const FgbProgramDesc* (*FgbProgramGetter)(void);
