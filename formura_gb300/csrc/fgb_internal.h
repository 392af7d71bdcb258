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
};

typedef cudaError_t (*FgbStageLaunch)(const FgbLaunch* args, cudaStream_t stream);
// Fused multi-step launch for single-stage programs (nullptr when absent).
typedef cudaError_t (*FgbFusedLaunch)(const FgbLaunch* args, cudaStream_t stream);

struct FgbProgramDesc {
  const char* name;
  int dim, nfields, nmids, nstages, sleeve, shift, reach, nuniforms;
  const char* const* field_names;
  FgbStageLaunch launch[FGB_NUM_PRECISIONS][FGB_MAX_STAGES];
  FgbFusedLaunch fused[FGB_NUM_PRECISIONS];
  int fused_max_steps;
};

typedef const FgbProgramDesc* (*FgbProgramGetter)(void);
