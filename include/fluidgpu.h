/*
 * fluidgpu.h -- C ABI of the GB300 simulation step for pkg/fluid.
 *
 * One `fg_fluid` handle stands in for one Go `*fluid.Fluid`.  Every entry
 * point below replaces one method (or one exported field access) of the Go
 * package pkg/fluid of TheFellow/fluid; the replaced symbol is cited as
 * file:line inside that package.  The signatures use plain C types only, so a
 * cgo, ctypes or JNI binding can call them directly.
 *
 * Memory model.  The fields live in device memory (HBM), pitched, x-major
 * like the reference (cell (i, j) at i*pitch + j, j contiguous).  Each field
 * also has a pinned host mirror of NumX*NumY floats laid out exactly like the
 * Go slices (index i*NumY + j), returned by fg_field().  The device copy is
 * authoritative: fg_download() refreshes a mirror, fg_mark_dirty() schedules
 * a mirror for upload before the next device operation.  The tool calls
 * (fg_set_solid, fg_set_velocity, ...) update a mirror that is current and
 * queue the same edit for the device, so they need no transfer of whole
 * fields.
 *
 * Threading.  A handle is not safe for concurrent use (neither is the Go
 * type).  Calls may come from different OS threads (cgo moves goroutines):
 * each call binds the handle's device first.
 *
 * Errors.  Every call returns FG_OK (0) or a negative FG_ERR_* code;
 * fg_last_error() gives the text of the last failure on the handle.  Index
 * errors (FG_ERR_INDEX) are the cases where the Go methods panic.
 */
#ifndef FLUIDGPU_H
#define FLUIDGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define FG_OK 0
#define FG_ERR_INVALID (-1)     /* bad argument: dimensions, pointer, parameter range   */
#define FG_ERR_INDEX (-2)       /* cell index out of range (the Go API panics)          */
#define FG_ERR_CUDA (-3)        /* a CUDA runtime call failed                            */
#define FG_ERR_UNSUPPORTED (-4) /* option not available on this path (see the call)      */
#define FG_ERR_MASK (-5)        /* S holds a value other than 0 or 1                     */
#define FG_ERR_TIMEOUT (-6)     /* a bounded device-side wait gave up                    */
#define FG_ERR_NOMEM (-7)       /* device or pinned allocation failed                    */
#define FG_ERR_TOO_LARGE (-8)   /* fg_project_noalloc: grid beyond its scratch or indices */
#define FG_ERR_NONFINITE (-9)   /* a statistic of the last step is NaN or infinite        */

/* Field identifiers (Fluid.U, .V, .newU, .newV, .p, .S, .M, .newM). */
enum {
  FG_U = 0,
  FG_V = 1,
  FG_NEWU = 2,
  FG_NEWV = 3,
  FG_P = 4,
  FG_S = 5,
  FG_M = 6,
  FG_NEWM = 7,
  FG_NUM_FIELDS = 8
};
#define FG_FIELD_BIT(f) (1u << (f))
#define FG_ALL_FIELDS 0xFFu

/* Pressure schemes.  LEXSOR is the reference's serial lexicographic SOR
 * (fluid.go:157-234) reproduced exactly by a wavefront kernel; JACOBI is the
 * parallel weighted-Jacobi relaxation of the same masked Poisson system with
 * temporal blocking.  MULTIGRID solves that system by num_iters parallel
 * V(2,2) cycles (the role the reference's UseMultigrid V-cycle,
 * fluid.go:559-758, plays for its serial scheme): levels of half the
 * interior size down to a side of 8, damped Jacobi smoothing with weight
 * 0.8 * PressureDamping (jacobi_omega, tb_depth and early_exit are not
 * used), residuals summed into the coarse right-hand side, bilinear
 * interpolation of the correction; refine_sweeps must be 0. */
enum { FG_SCHEME_LEXSOR = 0, FG_SCHEME_JACOBI = 1, FG_SCHEME_MULTIGRID = 3 };

typedef struct fg_params {
  /* Exported tuning fields of fluid.Fluid (fluid.go:25-39). */
  float confinement;          /* Confinement                                  */
  float viscosity_diffusion;  /* ViscosityDiffusion                           */
  float pressure_damping;     /* PressureDamping                              */
  float turbulence_strength;  /* TurbulenceStrength                           */
  float smoke_advection;      /* SmokeAdvection                               */
  int use_multigrid;          /* UseMultigrid: the reference's V-cycle, bit for bit */
  int multigrid_levels;       /* MultigridLevels                              */
  int use_bfecc;              /* UseBFECC                                     */
  float relaxation;           /* package var fluid.Relaxation (fluid.go:7-9)  */
  /* Constants the reference hard-codes in Simulate / solveSingleGrid. */
  int num_iters;              /* numIters = 8 (fluid.go:81)                   */
  float tolerance;            /* early-exit tolerance 1e-5 (fluid.go:159)     */
  int early_exit;             /* 1 = stop when max|div| < tolerance           */
  /* GPU scheme selection. */
  int scheme;                 /* FG_SCHEME_*                                  */
  float jacobi_omega;         /* Jacobi relaxation weight (times damping)     */
  int tb_depth;               /* Jacobi sweeps per launch; also the early-exit check interval */
  int refine_sweeps;          /* FP64-residual outer correction sweeps (0 = off) */
  int use_graphs;             /* capture each step in a CUDA graph            */
  int precise_coords;         /* 1: advection departure points relative to their face
                                 (no counterpart in the reference; 0 = the reference's
                                 absolute float coordinates, fluid.go:357-398) */
  int reserved[6];
} fg_params;

/* Per-step diagnostics, accumulated in FP64 on the device. */
typedef struct fg_stats {
  double div_l2_post;    /* sqrt(sum div^2) over fluid interior cells after the projection */
  double div_max_post;   /* max |div| after the projection                               */
  double div_count_post; /* number of fluid interior cells                               */
  double resid_l2;       /* FP64 L2 norm of the pressure residual (parallel schemes)      */
  double resid_max;      /* FP64 max |residual|                                           */
  double smoke_mass;     /* sum of M over interior cells after the step                   */
  double last_maxdiv;    /* max |div| seen by the last pressure sweep                     */
  int sweeps;            /* pressure sweeps executed (early exit included)                */
  int jacobi_kernel;     /* FG_JACOBI_KERNEL_*: the kernel of the last JACOBI-scheme solve */
  int reserved[6];
} fg_stats;

/* fg_stats.jacobi_kernel: which kernel ran the sweeps of the last step's main
 * JACOBI-scheme solve (host-side record of what was enqueued or captured).
 * NONE for the other schemes and for batches; SWEEP is the per-launch kernel
 * that loads its tiles itself (early exit, depths below 8, grids without a
 * tensor map); TMA the per-launch kernel fed by the tensor memory
 * accelerator; DATAFLOW the one cooperative launch that runs every full
 * 8-sweep phase (fixed sweep counts of at least 16 on grids of at least one
 * tile per SM). */
#define FG_JACOBI_KERNEL_NONE 0
#define FG_JACOBI_KERNEL_SWEEP 1
#define FG_JACOBI_KERNEL_TMA 2
#define FG_JACOBI_KERNEL_DATAFLOW 3

typedef struct fg_fluid fg_fluid;

/* Defaults of fluid.New (fluid.go:42-68) plus numIters = 8, LEXSOR. */
int fg_params_default(fg_params* out);

/* fluid.New(density, width, height, h) -- fluid.go:42-68.  Allocates the
 * NumX = width+2 by NumY = height+2 grid on the current device.  Cells are
 * indexed with 32-bit integers: NumX * (NumY rounded up to 32) above 2^30
 * returns FG_ERR_INVALID (before any device call). */
int fg_create(int width, int height, float density, float h, const fg_params* params,
              fg_fluid** out);
/* Releases the handle (no counterpart: Go frees by GC). */
int fg_destroy(fg_fluid* f);
int fg_dims(const fg_fluid* f, int* num_x, int* num_y);
/* Fluid.H() -- fluid.go:71. */
float fg_h(const fg_fluid* f);
/* Reads / writes the exported tuning fields (fluid.go:25-39). */
int fg_get_params(const fg_fluid* f, fg_params* out);
int fg_set_params(fg_fluid* f, const fg_params* params);

/* Host mirror of a field (the Go slices Fluid.U/.V/.S/.M and the private
 * p/newU/newV/newM the white-box tests read). */
int fg_field(fg_fluid* f, int field, float** host_ptr);
/* Schedules the mirrors in `mask` for upload before the next device call. */
int fg_mark_dirty(fg_fluid* f, unsigned mask);
/* Copies the device fields in `mask` into their mirrors (waits). */
int fg_download(fg_fluid* f, unsigned mask);
/* Copies the smoke field (mask = FG_FIELD_BIT(FG_M); other fields:
 * FG_ERR_UNSUPPORTED) of the work queued so far into its mirror on a second
 * stream, and returns at once.  The copy runs beside the next fg_simulate
 * (which writes the other smoke buffer), started once that step's pressure
 * projection is done; any other call on the handle, and fg_download_wait,
 * start it at once.  The mirror is current after fg_download_wait
 * (fg_download and the next fg_download_async wait too); do not read or
 * write it before.  For a frame loop that reads the smoke every frame:
 * simulate, wait, read, start the next copy. */
int fg_download_async(fg_fluid* f, unsigned mask);
int fg_download_wait(fg_fluid* f);
/* Waits for all queued work on the handle's stream. */
int fg_synchronize(fg_fluid* f);
/* The handle's CUDA stream (cudaStream_t), for callers that time it. */
void* fg_stream(fg_fluid* f);

/* (*Fluid).Simulate(dt) -- fluid.go:79-109.  Enqueues one step; returns when
 * it is queued.  Results are read with fg_download / fg_get_stats. */
int fg_simulate(fg_fluid* f, float dt);
/* Statistics of the last step or stage (waits).  With the statistics filled
 * in, FG_ERR_TIMEOUT when a bounded device-side wait of that step gave up
 * (its fields are then not to be used), else FG_ERR_NONFINITE when one of
 * the statistics is NaN or infinite (the step produced non-finite values). */
int fg_get_stats(fg_fluid* f, fg_stats* out);

/* Stage entry points (the unexported methods the reference tests call). */
int fg_make_incompressible(fg_fluid* f, int num_iters, float dt); /* fluid.go:144-155 */
int fg_advect_velocity(fg_fluid* f, float dt);                    /* fluid.go:291-333 */
int fg_advect_smoke(fg_fluid* f, float dt);                       /* fluid.go:400-434 */
int fg_advect_velocity_bfecc(fg_fluid* f, float dt);              /* fluid.go:911-994 */
int fg_advect_smoke_bfecc(fg_fluid* f, float dt);                 /* fluid.go:997-1051 */
int fg_handle_borders(fg_fluid* f);                               /* fluid.go:236-289 */
int fg_apply_vorticity_confinement(fg_fluid* f, float dt);        /* fluid.go:449-493 */
int fg_apply_viscosity(fg_fluid* f, float dt);                    /* fluid.go:112-142 */
int fg_add_turbulence(fg_fluid* f, float dt);                     /* fluid.go:496-526 */
int fg_clear_pressure(fg_fluid* f);                               /* fill(f.p, 0) fluid.go:83 */
/* copyBorder(dst, src) -- fluid.go:436-446, on two host arrays of
 * NumX*NumY floats (run through the device kernel). */
int fg_copy_border(fg_fluid* f, float* dst, const float* src);

/* Tools (walls.go:5-93, fluid.go:760-796, 893-907). */
int fg_set_solid(fg_fluid* f, int i, int j, int value);          /* walls.go:5-49   */
int fg_is_solid(const fg_fluid* f, int i, int j, int* out);      /* walls.go:51-60  */
int fg_set_velocity(fg_fluid* f, int i, int j, float u, float v);/* walls.go:62-72  */
int fg_add_smoke(fg_fluid* f, int i, int j, float smoke);        /* walls.go:74-83  */
int fg_reset(fg_fluid* f);                                       /* walls.go:85-93  */
int fg_apply_force(fg_fluid* f, int i, int j, float fx, float fy);                 /* fluid.go:761-771 */
int fg_apply_force_radius(fg_fluid* f, int cx, int cy, float fx, float fy, int r); /* fluid.go:774-796 */
int fg_set_circular_obstacle(fg_fluid* f, int cx, int cy, int radius);             /* fluid.go:894-907 */

/* Batched forms of SetVelocity / AddSmoke: the same as n calls in order. */
int fg_set_velocity_many(fg_fluid* f, int n, const int* i, const int* j, const float* u,
                         const float* v);
int fg_add_smoke_many(fg_fluid* f, int n, const int* i, const int* j, const float* smoke);

/* Persistent sources, applied on the device at the start of every
 * fg_simulate, in list order: the per-frame SetVelocity / AddSmoke calls the
 * reference app makes before Simulate for its jet and its sources
 * (main/main.go:236-241, 474-486).  mode bit 0: skip the source while its
 * cell is solid (applySources' IsSolid check); bit 1: set U and V to u, v;
 * bit 2: add `smoke` to M; bit 3: set M to `smoke` (the reference tests' jet
 * assignment M[i*n+j] = 1, fluid_test.go:396-401; it takes precedence over
 * bit 2).  Other bits: FG_ERR_INVALID.  n = 0 clears the list. */
#define FG_SRC_SKIP_SOLID 1
#define FG_SRC_SET_VELOCITY 2
#define FG_SRC_ADD_SMOKE 4
#define FG_SRC_SET_SMOKE 8
int fg_set_sources(fg_fluid* f, int n, const int* i, const int* j, const float* u,
                   const float* v, const float* smoke, const int* mode);

/* Views and diagnostics (fluid.go:798-891, 529-557; pressure.go, smoke.go). */
int fg_max_divergence(fg_fluid* f, float* out);                                  /* fluid.go:876-891 */
int fg_vorticity(fg_fluid* f, float* out_host, float* min_val, float* max_val);  /* fluid.go:806-838 */
int fg_velocity_magnitude(fg_fluid* f, float* out_host, float* min_val, float* max_val); /* fluid.go:841-873 */
int fg_field_min_max(fg_fluid* f, int field, float* min_val, float* max_val);    /* pressure.go:5-24, smoke.go:5-24 */
int fg_sample_velocity(fg_fluid* f, float x, float y, float* u, float* v);       /* fluid.go:799-803 */
int fg_adaptive_time_step(fg_fluid* f, float basedt, float* out);                /* fluid.go:529-557 */

/* Measurement hooks (no counterpart in the reference).  With profiling on,
 * CUDA events bracket the main Jacobi launches of each pressure solve;
 * fg_profile_jacobi waits and returns that span and its number of sweep
 * blocks (per-launch kernels, or phases of the one dataflow launch).
 * fg_launch_count is the number of kernels the handle has enqueued;
 * fg_edit_bytes the bytes of queued tool edits sent to the device so far
 * (the edit kernel reads them from pinned host memory). */
int fg_profile_enable(fg_fluid* f, int on);
int fg_profile_jacobi(fg_fluid* f, float* ms, int* launches);
/* Per-stage times (ms) of the last profiled step; returns the number of
 * stages written (<= max), names[k] naming the stage that ended at mark k. */
int fg_profile_stages(fg_fluid* f, int max, float* ms, const char** names);
unsigned long long fg_launch_count(const fg_fluid* f);
unsigned long long fg_edit_bytes(const fg_fluid* f);

/* Pressure projection that allocates nothing (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc when they project: an
 * engine whose own allocator owns the device memory, a frame loop that must
 * not risk the device-wide synchronisation an allocation can cause, or code
 * where allocation is forbidden.  It runs the JACOBI projection of
 * fg_make_incompressible (same kernels, same results) on caller-owned device
 * fields: u, v (in/out, staggered faces), p (out) and s (in, 0 = solid,
 * 1 = fluid; any nonzero value counts as fluid), each num_x rows of `pitch`
 * floats (pitch >= num_y), cell (i, j) at i*pitch + j.  Its scratch is a
 * fixed array inside the library of FG_NOALLOC_MAX_CELLS cells (about
 * 21 MiB, held on every GPU that loads the library until the process exits):
 * num_x * (num_y rounded up to 32) above FG_NOALLOC_MAX_CELLS, num_x * pitch
 * above 2^31 - 1 (cells are indexed with 32-bit integers), or more than
 * 4096 Jacobi launches (num_iters / tb_depth), returns FG_ERR_TOO_LARGE.  The work is
 * enqueued on `stream` (a cudaStream_t; NULL = the legacy default stream)
 * and the call returns without waiting.  The first call on a device looks up
 * the scratch array's device address; make that first call before any stream
 * capture.  The address is kept per CUDA context, so a caller that makes its
 * own context current (cuCtxCreate / cuCtxSetCurrent) or resets the device
 * gets the array of the context it runs in; the first call in each context
 * does the look-up.  All calls on a device share the one scratch array, so calls
 * whose work can overlap on the GPU (other streams, other host threads) race
 * and must be ordered by the caller.
 * The call returns before the GPU work ends, so a bounded device-side wait
 * that gives up (the TMA-fed Jacobi kernel's copy wait, about a second)
 * cannot be reported by it: the wait sets a status word in the scratch
 * array, the call's remaining kernels still run, and the fields it wrote are
 * then not a projection.  fg_project_noalloc_status(stream) waits for
 * `stream` and returns FG_ERR_TIMEOUT when the last call's status word is
 * set, FG_OK otherwise (FG_ERR_CUDA when the read fails); it allocates
 * nothing either.  Call it outside stream capture, after the call whose
 * status it reads and before the next one. */
#define FG_NOALLOC_MAX_CELLS (1 << 20)
int fg_project_noalloc(float* u, float* v, float* p, const float* s, int num_x, int num_y,
                       int pitch, float density, float h, float dt, int num_iters,
                       float jacobi_omega, float pressure_damping, int tb_depth, int early_exit,
                       float tolerance, void* stream);
int fg_project_noalloc_status(void* stream);

/* Differentiable rollouts: a Step / StepAdjoint pair standing in for an
 * autograd Function (no counterpart in the reference, which has no
 * derivatives; the forward step is fg_simulate's, fluid.go:79-109).
 *
 * fg_tape_begin(f, max_steps, every) starts a recorded rollout from the
 * current state and saves it as the first checkpoint.  It needs the JACOBI
 * scheme with early_exit 0 and viscosity_diffusion 0 (else
 * FG_ERR_UNSUPPORTED); the outer correction (refine_sweeps > 0) and
 * precise_coords are differentiated.  The parameters, the sources and
 * the state must not change until fg_tape_end (else FG_ERR_INVALID).
 *
 * fg_step_forward(f, dt, force_u, force_v) runs one step with the force
 * field (force_u, force_v) added to U, V before the sources (both NULL: no
 * force).  Every `every` steps the state is checkpointed on the device.
 *
 * fg_tape_seed sets the adjoint of the final state (dL/dU, dL/dV, dL/dM;
 * NULL = zero); fg_tape_seed_smoke_l2 sets it for L = ||M - target||_2 over
 * the interior cells and returns L (summed in double-float, returned in
 * FP64).
 *
 * fg_step_adjoint reverses the latest step not yet reversed: the adjoint
 * becomes that of the state before the step, and dL/d(force_u, force_v) of
 * that step is written to grad_force_u / grad_force_v (NULL: skipped).  The
 * steps of a checkpoint interval are recomputed from its checkpoint when the
 * interval is first reversed (each step's pressure potential is kept from the
 * forward pass, so the recomputation skips the pressure solve).  After the
 * last step is reversed the handle's state is back at the end of the forward
 * pass, and fg_tape_grad returns dL/d(initial U, V, M, newU, newV, newM).
 *
 * fg_tape_end closes the rollout (restoring the end-of-rollout state if it
 * was left mid-reverse).  The rollout's device buffers (per step: two force
 * fields and a potential; one interval of 13 recorded fields; 6 fields per
 * checkpoint) stay allocated for the next rollout until fg_destroy.
 *
 * All fields (forces, seeds, target, gradients) use the mirrors' layout
 * (NumX * NumY floats, index i*NumY + j) in host or device memory.  Adjoint
 * advection scatters with FP32 atomics: gradients reproduce to about 1e-6
 * relative, not bit for bit. */
int fg_tape_begin(fg_fluid* f, int max_steps, int every);
int fg_step_forward(fg_fluid* f, float dt, const float* force_u, const float* force_v);
int fg_tape_seed(fg_fluid* f, const float* dU, const float* dV, const float* dM);
int fg_tape_seed_smoke_l2(fg_fluid* f, const float* target, double* loss);
int fg_step_adjoint(fg_fluid* f, float* grad_force_u, float* grad_force_v);
int fg_tape_grad(fg_fluid* f, float* dU, float* dV, float* dM, float* dNU, float* dNV, float* dNM);
int fg_tape_steps(const fg_fluid* f, int* forward, int* reversed);
int fg_tape_end(fg_fluid* f);

/* Batches: many independent scenes of different sizes stepped together (no
 * counterpart in the reference, which steps one Fluid at a time).
 *
 * fg_batch_create(scenes, n, &batch) packs the state of n scene handles into
 * one batch handle: every stage then runs as one launch over all scenes
 * (each scene keeping its own size, obstacles, sources and pressure sweep
 * count), and fg_simulate / fg_batch_step capture a whole batch step in one
 * CUDA graph.  The members must use the JACOBI scheme without early exit,
 * refinement, viscosity or multigrid, and share every parameter except
 * num_iters (>= 1); else FG_ERR_UNSUPPORTED / FG_ERR_INVALID.  A batch step
 * gives each scene the same bits as fg_simulate on its handle; it computes
 * no statistics.  The members are left as they were: fg_batch_scatter copies
 * the batch's state into them, fg_batch_gather copies theirs into the batch
 * (the sources and parameters are fixed at creation).  Destroy the batch
 * before its members.
 *
 * A batch takes the recorded-rollout calls (fg_tape_begin, fg_step_forward
 * without force fields, fg_step_adjoint without force gradients,
 * fg_tape_end); fg_batch_seed_smoke_l2 seeds L_s = ||M_s - target_s||_2 per
 * scene (targets[s]: NumX_s * NumY_s values) and returns the n losses;
 * fg_batch_grad returns scene s's dL_s/d(initial U, V, M).
 *
 * fg_batch_autotune times each candidate thread-block shape of the per-cell
 * kernels and Jacobi sweeps per launch (tb_depth) on `reps` steps of this
 * batch from its current state (restored afterwards), keeps the fastest and
 * reports it.  The choice changes no result bit.
 *
 * Entry points that address one scene's cells, mirrors or views return
 * FG_ERR_UNSUPPORTED on a batch handle. */
int fg_batch_create(fg_fluid* const* scenes, int n, fg_fluid** batch);
int fg_batch_size(const fg_fluid* batch, int* n);
int fg_batch_step(fg_fluid* batch, float dt);
int fg_batch_step_adjoint(fg_fluid* batch);
int fg_batch_gather(fg_fluid* batch);
int fg_batch_scatter(fg_fluid* batch);
int fg_batch_seed_smoke_l2(fg_fluid* batch, const float* const* targets, double* losses);
int fg_batch_grad(fg_fluid* batch, int scene, float* dU, float* dV, float* dM);
int fg_batch_autotune(fg_fluid* batch, float dt, int reps, int* tb_depth, int* block_x,
                      int* block_y, float* ms_per_step);

/* Tracer particles: the app's advectParticles (main/main.go:512-546) on the
 * device.  fg_particles_add appends n particles at world positions (x, y)
 * with age 0, the given maximum age and colour (rgb: 3 bytes each), keeping
 * the total at most max_total (the app's maxParticles; <= 0: no limit);
 * host or device arrays.  fg_particles_advect(dt) ages every particle, drops
 * those older than their maximum age, moves the others by RK2 midpoint steps
 * through SampleVelocity (fluid.go:799-803) and drops those that leave the
 * grid or enter a solid cell, keeping the survivors in order.
 * fg_particles_get copies the live particles out (NULL: skipped; fg_particles
 * _count gives their number). */
int fg_particles_add(fg_fluid* f, int n, const float* x, const float* y, const float* max_age,
                     const unsigned char* rgb, int max_total);
int fg_particles_advect(fg_fluid* f, float dt);
int fg_particles_count(fg_fluid* f, int* n);
int fg_particles_get(fg_fluid* f, float* x, float* y, float* age, float* max_age,
                     unsigned char* rgb);
int fg_particles_clear(fg_fluid* f);

/* Renders a field as the app draws it (main/main.go:619-650): an RGBA8
 * image of NumX x NumY pixels, row stride 4 * NumX, pixel (i, j) showing cell
 * (i, NumY - 1 - j); smoke, pressure and speed with the scientific colormap
 * (getSciValue, main/colors.go:47-84) between the view's min and max,
 * vorticity with the blue-white-red one (getDivergingColor,
 * main/colors.go:10-44).  rgba: NumX * NumY * 4 bytes, host or device. */
enum { FG_RENDER_SMOKE = 0, FG_RENDER_PRESSURE = 1, FG_RENDER_SPEED = 2, FG_RENDER_VORTICITY = 3 };
int fg_render(fg_fluid* f, int kind, void* rgba);

/* Text of the last error on the handle ("" if none); static text for a
 * NULL handle. */
const char* fg_last_error(const fg_fluid* f);

/* Fault injection (no counterpart in the reference), for tests of the
 * error paths without a GPU fault.
 * fg_debug_fail_alloc(n): the n-th next device or pinned allocation made by
 * the library (counting from 0, process-wide) fails as if memory were
 * exhausted; n < 0 disarms.  The call that made it returns FG_ERR_NOMEM (or
 * FG_ERR_CUDA where a CUDA failure is reported) and frees what it took.
 * fg_debug_stall_tile(f, t): the dataflow Jacobi kernel never publishes tile
 * t of the handle's solves, so the tiles that read it wait until their
 * bounded waits (about a second) give up; the step's fg_get_stats returns
 * FG_ERR_TIMEOUT.  t < 0 disarms.  Changes the handle's captured graphs.
 * fg_debug_stall_tile(NULL, t): in later fg_project_noalloc calls, the
 * TMA-fed Jacobi kernel's copy barrier of tile t expects 16 bytes more than
 * its copies bring, so the block that sweeps tile t gives up after its
 * bounded waits (about nine seconds) and fg_project_noalloc_status returns
 * FG_ERR_TIMEOUT; every copy issued still lands.  t < 0 disarms. */
int fg_debug_fail_alloc(int n);
int fg_debug_stall_tile(fg_fluid* f, int tile);

#ifdef __cplusplus
}
#endif

#endif /* FLUIDGPU_H */
