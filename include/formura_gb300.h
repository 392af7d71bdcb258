/* formura_gb300: C ABI of the GB300 backend for Formura-generated stencil code.
 *
 * The reference's boundary is the C pair that Formura writes for each program
 * (src/Formura/Generator/Encode.hs:11-27): the header declares
 * `Formura_Grid_Struct formura_data`, `Formura_Navi`, `to_pos_*`,
 * `Formura_Init`, `Formura_Forward` and `Formura_Finalize`
 * (src/Formura/Generator/Templates.hs:53-115, 221-250, 295-334, 383-386).
 * That API stays unchanged: the generator of this backend writes the same
 * header and a C body whose Formura_Forward calls the entry points below
 * instead of running the OpenMP loop nests.  Every entry point returns 0 on
 * success or a negative FGB_E* code; fgb_last_error() describes the last
 * failure of the calling thread.  No entry point exits the process (the
 * reference's only error path is exit(1) on an MPI size mismatch,
 * Templates.hs:243).
 */
#ifndef FORMURA_GB300_H
#define FORMURA_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FGB_OK 0
#define FGB_E_ARG (-1)       /* invalid argument */
#define FGB_E_PROGRAM (-2)   /* unknown program name */
#define FGB_E_CUDA (-3)      /* CUDA runtime error */
#define FGB_E_NOMEM (-4)     /* device allocation failed */
#define FGB_E_NODEV (-5)     /* no CUDA device */

/* Arithmetic forms of the state update. */
#define FGB_F64 0       /* FP64, rounded like the reference's C (bit-faithful) */
#define FGB_F64_FAST 1  /* FP64 with fused multiply-add and reciprocal products */
#define FGB_F32 2       /* FP32 storage and arithmetic */
#define FGB_F16 3       /* FP16 storage with a per-field scale, FP32 arithmetic */

typedef struct fgb_grid fgb_grid;

/* Programs compiled into the library.  A program is the step function of a
 * .fmr file; its kernels are the hand-written templates instantiated with
 * the program's stencil expression. */
int fgb_program_count(void);
const char* fgb_program_name(int index);
/* dim, number of state fields, size of the uniform table, sleeve
 * (calcSleeve, src/Formura/OrthotopeMachine/Translate.hs:613-623) and the
 * per-step roll of the array content (Templates.hs:346). */
int fgb_program_query(const char* program, int* dim, int* nfields, int* nuniforms,
                      int* sleeve, int* shift);
/* Name of state field `index` (fields are in name order, like the members of
 * Formura_Grid_Struct, Templates.hs:53-73). */
const char* fgb_program_field(const char* program, int index);

/* Create a device-resident grid of `program` with extent shape[0..ndim-1]
 * (the grid_per_node of the numerical config) in the given precision.
 * `uniforms` holds the grid-independent values of the step function for
 * this configuration, in the order the generator reports. Replaces the
 * static buffers of Templates.hs:125-186. */
int fgb_open(const char* program, const int* shape, int ndim, int precision,
             const double* uniforms, int nuniforms, fgb_grid** out);
int fgb_close(fgb_grid* grid);

/* FP16 storage: value = stored * scales[f]. */
int fgb_set_scales(fgb_grid* grid, const float* scales, int nfields);

/* Copy the whole state between the host and the device.  `host_state`
 * points at a Formura_Grid_Struct: one C-order array per field, fields back
 * to back in name order, FP64 (the layout of formura_data). */
int fgb_upload(fgb_grid* grid, const double* host_state);
int fgb_download(fgb_grid* grid, double* host_state);

/* Advance `nsteps` time steps (enqueued on the grid's stream).  Each step
 * rolls the array content by the program's shift along every axis, exactly
 * as Formura_Forward does (Templates.hs:300-310, 336-346). */
int fgb_forward(fgb_grid* grid, int nsteps);
int fgb_synchronize(fgb_grid* grid);

/* The grid's CUDA stream (a cudaStream_t), for events and interop. */
void* fgb_stream(fgb_grid* grid);
/* Device pointers of the current state fields (storage precision). */
int fgb_state_device(fgb_grid* grid, void** field_ptrs, int nfields);
/* Number of kernels this grid has launched so far. */
int64_t fgb_launch_count(fgb_grid* grid);

/* Temporal-blocking kernels.  Programs whose step is a single stage also
 * have kernels that advance several steps per launch in shared-memory tiles
 * (they replace the reference's CPU temporal blocking, Templates.hs:311-381);
 * 3D programs also have one-step kernels on row vectors, and multi-stage 3D
 * programs in FP32/FP16 a one-launch kernel with every stage's arrays in
 * shared memory.
 * fgb_autotune times every variant that fits on this device and the
 * one-step kernel over `trial_steps` steps, restores the state, and selects
 * the fastest; fgb_set_variant selects one by index (-1: one step per
 * launch).  FP64 results do not depend on the choice, nor do FP32 results
 * of single-stage programs; the FP32 results of the one-launch multi-stage
 * kernels agree with the stage kernels' to rounding (nvcc fuses products and
 * sums into FMAs differently in different kernels).  With FP16 storage the
 * tiles keep FP32 values between the steps of one launch. */
int fgb_variant_count(fgb_grid* grid);
int fgb_variant_info(fgb_grid* grid, int index, int* tile_x, int* tile_y, int* steps);
int fgb_set_variant(fgb_grid* grid, int index);
int fgb_variant(fgb_grid* grid);
int fgb_autotune(fgb_grid* grid, int trial_steps, int* chosen);

/* Reverse mode (no counterpart in the reference: the Formura_Backward
 * extension of the generated API).  The adjoint step is generated from the
 * program's own step function by reverse-mode differentiation: one pass for
 * single-stage steps, two passes per stage for multi-stage steps (programs
 * built with gpu_adjoint: 1), in FP64 and FP32.
 *
 * fgb_backward: one adjoint step at the current state u_n:
 *   lambda = (dF/du at u_n)^T lambda_next   (host FP64, formura_data layout).
 * fgb_gradient_forward / fgb_gradient_backward: gradient of a scalar loss of
 * the state `nsteps` steps ahead with respect to the current state.  The
 * forward call checkpoints the current state u_0 and advances to u_T; the
 * caller computes seed = dJ/du_T; the backward call returns dJ/du_0 and
 * leaves the state at u_0.  `snapshots` device checkpoints (u_0 included)
 * bound the memory; the reversal places them by the binomial rule of
 * Griewank's revolve and recomputes forward segments in between.
 * fgb_gradient_stats: forward steps (including recomputation) and adjoint
 * steps of the last gradient. */
int fgb_backward(fgb_grid* grid, const double* lambda_next, double* lambda);
int fgb_gradient_forward(fgb_grid* grid, int nsteps, int snapshots);
int fgb_gradient_backward(fgb_grid* grid, const double* seed, double* grad);
int fgb_gradient_backward_device(fgb_grid* grid, const void* seed, void* grad);
int fgb_gradient_stats(fgb_grid* grid, int64_t* forward_steps, int64_t* adjoint_steps);
/* Apply the adjoint step `nsteps` times to the device adjoint state at the
 * current forward state (enqueued; for linear steps and for timing). */
int fgb_adjoint_steps(fgb_grid* grid, int nsteps);

/* Batched ensembles (no counterpart in the reference, which runs one grid
 * per process): `count` independent periodic 2D grids of one single-stage
 * program, grid i of extent shapes[2i] x shapes[2i+1] with its own uniform
 * table uniforms[i*nuniforms ...] (e.g. per-grid feed and kill rates).  All
 * grids advance together: persistent CTAs walk one tile queue spanning every
 * grid, several steps per launch in shared memory; fgb_batch_forward replays
 * a CUDA graph of 64 steps for long runs; fgb_batch_autotune picks the tile
 * shape and steps per launch.  FP64 and FP32 only.  Each grid's result is
 * bit-identical to running it alone with fgb_open / fgb_forward. */
typedef struct fgb_batch fgb_batch;
int fgb_batch_open(const char* program, int count, const int* shapes, int precision,
                   const double* uniforms, int nuniforms, fgb_batch** out);
int fgb_batch_close(fgb_batch* batch);
int fgb_batch_upload(fgb_batch* batch, int index, const double* host_state);
int fgb_batch_download(fgb_batch* batch, int index, double* host_state);
int fgb_batch_forward(fgb_batch* batch, int nsteps);
int fgb_batch_synchronize(fgb_batch* batch);
int fgb_batch_variant_count(fgb_batch* batch);
int fgb_batch_variant_info(fgb_batch* batch, int index, int* tile_x, int* tile_y, int* steps);
int fgb_batch_set_variant(fgb_batch* batch, int index);
int fgb_batch_variant(fgb_batch* batch);
int fgb_batch_autotune(fgb_batch* batch, int trial_steps, int* chosen);
void* fgb_batch_stream(fgb_batch* batch);
int64_t fgb_batch_launch_count(fgb_batch* batch);

/* The program's first_step and filter functions (Templates.hs:252-270).
 * fgb_attach(grid, "first_step" | "filter", uniforms, n) loads the function
 * with its own uniform table; fgb_apply runs it once on the current state,
 * with its own roll (its sleeve), as Formura_First_Step / Formura_Filter do. */
int fgb_attach(fgb_grid* grid, const char* which, const double* uniforms, int nuniforms);
int fgb_apply(fgb_grid* grid, const char* which);

/* FP64 sum of every state field of the current state (conserved totals of
 * mass, momentum and energy for conservative programs), whatever the
 * storage precision; deterministic for a given grid size. */
int fgb_totals(fgb_grid* grid, double* sums, int nfields);

/* Lazy host synchronisation (opt-in; the drop-in's gpu_host_sync: lazy).
 * The host state region (page aligned, whole pages) stays protected while
 * the device copy is newer; the first access downloads it (SIGSEGV handler,
 * faults elsewhere go to the previous handler), the first write marks it
 * dirty, and fgb_lazy_forward uploads only a dirty copy.  fgb_lazy_detach
 * downloads if needed and unprotects. */
int fgb_lazy_attach(fgb_grid* grid, void* host_state, size_t bytes);
int fgb_lazy_forward(fgb_grid* grid, int nsteps);
int fgb_lazy_detach(fgb_grid* grid);
int fgb_lazy_stats(fgb_grid* grid, int64_t* uploads, int64_t* downloads);

/* Pin a host range (e.g. formura_data) for faster copies; optional. */
int fgb_host_register(void* ptr, size_t bytes);
int fgb_host_unregister(void* ptr);

const char* fgb_last_error(void);

/* Size of the fixed device array that fgb_forward_noalloc draws on. */
#define FGB_NOALLOC_SCRATCH_BYTES (64ull << 20)

/* Advance a caller-owned device state by `nsteps` steps without allocating
 * any device memory.  This entry point has no counterpart in the reference
 * (whose generated code keeps every buffer in static host arrays); it serves
 * callers that cannot call cudaMalloc while they run, such as a framework
 * that owns all device memory through its own pool, or a plug-in host that
 * forbids device allocation once a run has started.
 *
 * in_state / out_state: device pointers to the whole state in the
 * formura_data layout (fields back to back, name order), in the storage
 * type of `precision` (FGB_F16 uses unit scales).  They must not overlap;
 * in_state is left unchanged.  The uniform table, the second buffer of the
 * step-to-step ping-pong and the intermediate arrays of multi-stage programs
 * come from one static device array of FGB_NOALLOC_SCRATCH_BYTES (64 MiB),
 * which every GPU that loads the library holds until the process exits.  A
 * grid that needs more returns FGB_E_ARG with the required size.  Nothing in
 * that array has to start at zero: every byte a call reads was written
 * earlier by the same call.  All calls share the array, so calls that
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  The first call on each device looks up the
 * array's device address; make that first call before any stream capture.
 * Work is queued on `stream` (a cudaStream_t; NULL is the legacy default
 * stream) and is complete when that stream is. */
int fgb_forward_noalloc(const char* program, const int* shape, int ndim, int precision,
                        const double* uniforms, int nuniforms, const void* in_state,
                        void* out_state, int nsteps, void* stream);

#ifdef __cplusplus
}
#endif
#endif
