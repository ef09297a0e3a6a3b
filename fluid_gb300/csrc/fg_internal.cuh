// Internal declarations shared by the CUDA translation units of libfluidgpu.
//
// Device layout: every field is an array of NX rows of `pitch` floats
// (pitch = NY rounded up to 32, so rows start on 128-byte boundaries);
// cell (i, j) sits at i*pitch + j.  Padding cells (j >= NY) are never read
// by a kernel.  Arithmetic on the simulated fields is FP32 with every
// operation separately rounded (the library is compiled with -fmad=false;
// fused multiply-adds appear only as explicit __fmaf_rn calls in the
// parallel pressure schemes), so a step reproduces the CPU restatement of
// pkg/fluid bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/fluidgpu.h"

namespace fg {

// Per-cell flag byte (built from S when S changes).
enum : uint8_t {
  F_W = 1,          // S[i-1, j] != 0
  F_E = 2,          // S[i+1, j] != 0
  F_S = 4,          // S[i, j-1] != 0
  F_N = 8,          // S[i, j+1] != 0
  F_FLUID = 16,     // S[i, j] != 0
  F_INTERIOR = 32,  // 1 <= i <= NX-2 and 1 <= j <= NY-2
};
__host__ __device__ inline int flag_count(uint8_t f) {
  return (f & 1) + ((f >> 1) & 1) + ((f >> 2) & 1) + ((f >> 3) & 1);
}
// A cell the pressure relaxation updates: interior, fluid, >= 1 fluid neighbour.
__host__ __device__ inline bool flag_active(uint8_t f) {
  return (f & (F_FLUID | F_INTERIOR)) == (F_FLUID | F_INTERIOR) && (f & 15) != 0;
}

struct Grid {
  int NX, NY, P;   // NumX, NumY, device pitch (floats)
  float h;         // grid spacing
  float h1;        // float32(1.0 / h)           fluid.go:360
  float hh;        // 0.5 * h  (== h / 2)        fluid.go:298, 361, 406
  float NXh, NYh;  // float32(NumX) * h, float32(NumY) * h   fluid.go:363-364
  int precise;     // departure points relative to their face (fg_params.precise_coords)
};

inline Grid make_grid(int NX, int NY, int P, float h) {
  Grid g;
  g.NX = NX;
  g.NY = NY;
  g.P = P;
  g.h = h;
  g.h1 = 1.0f / h;
  g.hh = 0.5f * h;
  g.NXh = (float)NX * h;
  g.NYh = (float)NY * h;
  g.precise = 0;
  return g;
}

// ---------------------------------------------------------------- device helpers
#ifdef __CUDACC__
__device__ __forceinline__ float canon_nan() { return __int_as_float(0x7fc00000); }
// Go's builtin min / max on float32: a NaN argument gives NaN, -0 < +0.
__device__ __forceinline__ float go_min(float a, float b) {
  if (isnan(a) || isnan(b)) return canon_nan();
  if (a == b) return signbit(a) ? a : b;
  return a < b ? a : b;
}
__device__ __forceinline__ float go_max(float a, float b) {
  if (isnan(a) || isnan(b)) return canon_nan();
  if (a == b) return signbit(a) ? b : a;
  return a > b ? a : b;
}
__device__ __forceinline__ float fbit(uint8_t f, uint8_t bit) { return (f & bit) ? 1.0f : 0.0f; }

// Programmatic dependent launch.  A kernel launched by launch_pdl may be
// scheduled while the kernel before it on the stream still runs; it calls
// pdl_enter before touching global memory, which waits for that kernel to
// complete (its writes visible) and lets the kernel after it be scheduled in
// turn.  Both instructions are no-ops in a plain launch.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The bilinear stencil of one sample: corner indices, weights and whether
// each coordinate lies inside the clamp range.
struct Bilin {
  int x0, x1, y0, y1;
  float tx, ty;
  bool inx, iny;
};

// sampleField / sampleFieldFrom (fluid.go:357-398, 1055-1091) at the
// absolute point (x, y).  dx, dy are the staggering offsets of the sampled
// field (U: 0,h/2; V: h/2,0; M: h/2,h/2).  The clamp of the coordinates uses
// fminf/fmaxf: for any non-NaN coordinate they equal Go's min/max here (the
// bounds are positive, so no signed-zero ties); a NaN coordinate, where the
// reference's int conversion of the floor gives an out-of-range index and
// panics, clamps to the upper bound.
__device__ __forceinline__ Bilin bilin_abs(float x, float y, float dx, float dy, const Grid& g) {
  Bilin s;
  float xc = fmaxf(fminf(x, g.NXh), g.h);
  float yc = fmaxf(fminf(y, g.NYh), g.h);
  s.inx = xc == x;
  s.iny = yc == y;
  float xs = xc - dx;
  float ys = yc - dy;
  s.x0 = min((int)floorf(xs * g.h1), g.NX - 1);
  s.tx = (xs - (float)s.x0 * g.h) * g.h1;
  s.x1 = min(s.x0 + 1, g.NX - 1);
  s.y0 = min((int)floorf(ys * g.h1), g.NY - 1);
  s.ty = (ys - (float)s.y0 * g.h) * g.h1;
  s.y1 = min(s.y0 + 1, g.NY - 1);
  return s;
}

// The same stencil for a point given relative to index (i, j): its sample
// coordinates in cells are (i + a, j + b), on a field staggered by (dxr,
// dyr) cells (0 or 0.5).  Absolute float coordinates near index 2048 are
// resolved to 2^-12 cells only, which shifts the weights by up to ~1e-4;
// here the integer part is exact and the weights keep float precision of
// the displacement.  The clamp to [h, NumX h] (fluid.go:363-364) becomes
// a in [1 - dxr - i, NumX - dxr - i].
__device__ __forceinline__ Bilin bilin_local(int i, int j, float a, float b, float dxr, float dyr,
                                             const Grid& g) {
  Bilin s;
  float ac = fmaxf(fminf(a, (float)(g.NX - i) - dxr), (float)(1 - i) - dxr);
  float bc = fmaxf(fminf(b, (float)(g.NY - j) - dyr), (float)(1 - j) - dyr);
  s.inx = ac == a;
  s.iny = bc == b;
  float fa = floorf(ac), fb = floorf(bc);
  s.x0 = i + (int)fa;
  s.tx = ac - fa;
  if (s.x0 > g.NX - 1) {
    s.x0 = g.NX - 1;
    s.tx = ac - (float)(s.x0 - i);
  }
  s.y0 = j + (int)fb;
  s.ty = bc - fb;
  if (s.y0 > g.NY - 1) {
    s.y0 = g.NY - 1;
    s.ty = bc - (float)(s.y0 - j);
  }
  s.x1 = min(s.x0 + 1, g.NX - 1);
  s.y1 = min(s.y0 + 1, g.NY - 1);
  return s;
}

// Stencil at the departure point of face / cell (i, j): the point
// (i h + ox, j h + oy), ox and oy 0 or h/2 (hx, hy), moved by (-su, -sv)
// (su, sv: the products sdt * u, sdt * v), on a field staggered by the same
// half cells.  Without g.precise the coordinates are formed as the reference
// forms them (fluid.go:304-330, 411-414, 940-960).
__device__ __forceinline__ Bilin bilin_dep(int i, int j, float su, float sv, bool hx, bool hy,
                                           const Grid& g) {
  if (g.precise)
    return bilin_local(i, j, -su * g.h1, -sv * g.h1, hx ? 0.5f : 0.0f, hy ? 0.5f : 0.0f, g);
  float x = hx ? ((float)i * g.h + g.hh) - su : (float)i * g.h - su;
  float y = hy ? ((float)j * g.h + g.hh) - sv : (float)j * g.h - sv;
  return bilin_abs(x, y, hx ? g.hh : 0.0f, hy ? g.hh : 0.0f, g);
}

// The bilinear value over a stencil; d(i, j) reads the field.
template <typename A>
__device__ __forceinline__ float bilin_sample(const A& d, const Bilin& s) {
  float sx = 1.0f - s.tx;
  float sy = 1.0f - s.ty;
  return sx * sy * d(s.x0, s.y0) + s.tx * sy * d(s.x1, s.y0) + s.tx * s.ty * d(s.x1, s.y1) +
         sx * s.ty * d(s.x0, s.y1);
}

// A field in global memory with pitch P.
struct PtrAcc {
  const float* __restrict__ p;
  int P;
  __device__ __forceinline__ float operator()(int i, int j) const { return p[i * P + j]; }
};

__device__ __forceinline__ float sample_field(const float* __restrict__ d, float x, float y,
                                              float dx, float dy, const Grid& g) {
  return bilin_sample(PtrAcc{d, g.P}, bilin_abs(x, y, dx, dy, g));
}
// Sample of d at the departure point of face / cell (i, j) (bilin_dep).
__device__ __forceinline__ float sample_dep(const float* __restrict__ d, int i, int j, float su,
                                            float sv, bool hx, bool hy, const Grid& g) {
  return bilin_sample(PtrAcc{d, g.P}, bilin_dep(i, j, su, sv, hx, hy, g));
}
#endif

// ---------------------------------------------------------------- handle
struct EditRec {  // one queued tool edit
  uint32_t field;
  uint32_t cell;  // host index i*NY + j
  uint32_t op;    // 0 = set, 1 = add
  float value;
};

struct SourceRec {  // one persistent per-step source (applied at the start of a step)
  uint32_t cell;      // host index i*NY + j
  uint32_t mode;      // bit 0: skip if the cell is solid, bit 1: set U,V, bit 2: add smoke
  float u, v, smoke;
};

struct DevStats {  // device-side accumulation target (finalised per step)
  double div_l2_sq, div_max, div_count;
  double resid_l2_sq, resid_max;
  double smoke_mass;
  double last_maxdiv;
  int sweeps;
  int timeout;  // 1: a bounded device-side wait of the step gave up
};

// ---------------------------------------------------------------- batches
// A batch packs many scenes of different sizes into the same per-field
// arrays: scene s occupies NX_s rows of pitch P_s starting at element
// offset off_s of every field (the flag bytes and noise pairs at the same
// element offset of theirs).  Kernels run over a block table: one entry per
// thread block naming the scene and the tile within it.
struct BScene {
  Grid g;
  long long off;  // element offset of the scene in the packed arrays
  int iters;      // Jacobi sweeps of the scene's pressure solve
  int pad;
};
struct BTile {
  int s, x, y, pad;  // scene, tile column, tile row (per-cell and border tables)
};
// A per-cell block of a batch with its scene's grid and offset in the same
// entry, so the block's first read is its last table read.
struct BCell {
  Grid g;
  long long off;
  int x, y;  // tile column, tile row
  int pad[2];
};
static_assert(sizeof(BCell) == 64, "one 64-byte entry per block");
// A per-launch Jacobi block (k_pressure.cu) sweeps a region of 64 rows (8
// warps; 32 with 4 warps on small grids) x 128 columns in registers and
// writes the cells of it that are exact after its sweeps.  Inside the grid a region edge costs a halo of 8 cells; at the
// grid's edge it costs none: the cells past the grid are zero and stay zero,
// and the grid's outermost ring has w = bw = 0, so whatever a region-edge
// thread reads beside it (a warp shuffle at lane 0 or 31 returns the
// thread's own value) is multiplied by 0.  Along an axis of n cells, region
// t of length R starts at t S (S = R - 2 halo); the first owns from the
// grid's edge, the one that reaches n owns up to n, the others own [t S +
// halo, t S + R - halo).  A batch's Jacobi BTile holds the region's first
// column and row in x and y and the owned window in pad.
constexpr int kJacRegionRows = 64, kJacRegionCols = 128, kJacHalo = 8;
__host__ __device__ inline int span_count(int n, int R) {
  const int S = R - 2 * kJacHalo;
  return n <= R ? 1 : (n - R + S - 1) / S + 1;
}
// Owned window of region t in region coordinates: first | end << 8.
__host__ __device__ inline uint32_t span_own(int t, int n, int R) {
  const int a = t * (R - 2 * kJacHalo);
  const uint32_t lo = t ? kJacHalo : 0, hi = a + R >= n ? n - a : R - kJacHalo;
  return lo | hi << 8;
}

struct BatchGeom {
  int n = 0;
  std::vector<BScene> scenes;
  std::vector<fg_fluid*> members;  // the scene handles (not owned)
  BScene* scenes_dev = nullptr;
  int bx = 32, by = 8;  // thread-block shape of the per-cell kernels (autotuned)
  BTile* cell_tiles = nullptr;
  BCell* cell_blocks = nullptr;  // the same tiles with their scenes (per-cell kernels)
  int n_cell_tiles = 0;
  int* cell_range = nullptr;  // device: [first, end) cell tiles of each scene (2 n entries)
  BTile* border_tiles = nullptr;
  int n_border_tiles = 0;
  BTile* jac_tiles = nullptr;  // scenes with more sweeps first (see jac_iters)
  int n_jac_tiles = 0;
  // Per scene in the Jacobi table's order: its sweeps and its regions, so a
  // launch runs only the table's prefix of scenes that have started.
  std::vector<int> jac_iters, jac_regions;
  int max_iters = 0;
  int* src_scene = nullptr;  // device: scene of each source group
  double* losses = nullptr;  // device: per-scene loss of the last seed, then n floats 1 / L
};

// One level of the MULTIGRID scheme's hierarchy (k_pressure.cu).  Level 0
// names the handle's own solver arrays; the coarser levels own theirs.
struct MgLevelDev {
  Grid g;
  float* S = nullptr;        // fluid mask (1 = fluid)
  uint8_t* flags = nullptr;  // flag bytes built from S
  float* w = nullptr;        // smoothing weight / s on active cells
  float* b = nullptr;        // right-hand side
  float* bw = nullptr;       // w * b
  float* x[2] = {nullptr, nullptr};  // iterate (ping-pong)
};
// The MULTIGRID scheme's smoothing weight (times PressureDamping) and the
// interior side below which it stops coarsening.
constexpr float kMgOmega = 0.8f;
constexpr int kMgMinSide = 8;
struct MgHier {
  std::vector<MgLevelDev> lv;
  void* block = nullptr;  // one allocation holding the coarse levels' arrays
  void* ctl = nullptr;    // control block of the smoothing launches
  float omega = -1.0f;    // smoothing weight the coarse weights hold
};

}  // namespace fg

struct fg_fluid {
  int device = 0;
  int NX = 0, NY = 0, P = 0;
  float density = 0, h = 0;
  fg_params prm;
  fg::Grid g;
  cudaStream_t stream = nullptr;

  // State fields on the device (indexed by FG_*), plus one rotation partner
  // for U, V and M (out-of-place stages swap state and partner).
  float* d[FG_NUM_FIELDS] = {};
  float* partner[FG_NUM_FIELDS] = {};
  // Scratch.
  float *fwdU = nullptr, *fwdV = nullptr, *fwdM = nullptr;
  float *corrU = nullptr, *corrV = nullptr, *corrM = nullptr;
  // Coarse levels of the MULTIGRID scheme (allocated on its first step).
  fg::MgHier* mg = nullptr;
  float *phi = nullptr, *phi2 = nullptr, *rhs = nullptr;
  float *err = nullptr, *err2 = nullptr, *rhs_e = nullptr;
  float *wgt = nullptr, *bw = nullptr, *bwe = nullptr;  // Jacobi w = om/s, w*b, w*b_e
  float* curl = nullptr;
  float* view = nullptr;       // output of the vorticity / magnitude views
  float2* noise = nullptr;     // per-cell float32(sin(seed)) pairs for addTurbulence
  uint8_t* flags = nullptr;    // per-cell flag byte
  float* partials = nullptr;   // block partial rows of the reductions (float pairs)
  int n_partials = 0;          // floats
  fg::DevStats* dstats = nullptr;
  void* pctl = nullptr;   // control block of the main Jacobi solve (k_pressure.cu PCtl)
  int* tile_done = nullptr;  // dataflow Jacobi kernel: per-tile phase flags + item counter
  int stall_tile = -1;       // fault injection: a tile the dataflow kernel never publishes
  int jacobi_kernel = 0;     // FG_JACOBI_KERNEL_* of the last main solve (fg_stats)
  float* skew[3] = {};       // diagonal-major U, V, p of the wavefront SOR (or none)
  uint8_t* skew_flags = nullptr;
  int skew_sp = 0;           // their row stride (cells per diagonal)
  unsigned* lex_scratch = nullptr;  // grid-wide wavefront: sweep maxima, barrier words
  void* ectl = nullptr;   // control block of the FP64-residual correction solve
  int n_slots = 0;        // launch slots per control block
  float* copy_tmp = nullptr;        // fg_copy_border staging (2 fields)

  // Host mirrors (pinned) and bookkeeping.
  float* hm[FG_NUM_FIELDS] = {};  // pinned host mirrors (NX*NY, Go slice layout)
  bool host_valid[FG_NUM_FIELDS] = {};
  unsigned dirty = 0;
  bool masks_stale = true;
  std::vector<fg::EditRec> edits;
  // Two staging slots for queued edits, used alternately; a slot is reused
  // once the event recorded after its upload has completed.
  fg::EditRec* edit_pinned[2] = {};   // the edit log, double-buffered (pinned)
  fg::EditRec* edit_dev[2] = {};      // the same memory as the device addresses it
  uint32_t* edit_off_pinned[2] = {};
  uint32_t* edit_off_dev[2] = {};
  cudaEvent_t edit_ev[2] = {};
  size_t edit_cap[2] = {};
  int edit_slot = 0;
  unsigned long long edit_bytes = 0;  // bytes of queued edits uploaded so far
  // Persistent sources, grouped by cell on the host (offsets into src_dev).
  fg::SourceRec* src_dev = nullptr;
  uint32_t* src_off_dev = nullptr;
  int n_src_groups = 0;
  // Differentiable rollouts: the adjoint of the state (U, V, M and the
  // staging fields) and the adjoint work fields, allocated by the first
  // recorded rollout; the rollout's tape (fg_api.cu).
  enum { A_U, A_V, A_M, A_NU, A_NV, A_NM, A_CU, A_CV, A_FU, A_FV, A_CM, A_FM,
         A_COUNT };
  float* adj[A_COUNT] = {};
  struct Tape* tape = nullptr;
  // The force field of the recorded step being enqueued (added to U, V by
  // the pressure setup and the gradient kernel), null otherwise.
  const float* step_fu = nullptr;
  const float* step_fv = nullptr;
  // Where the gradient kernel also writes the projected field before the
  // turbulence it applies (a recorded step's U2, V2), null otherwise.
  float* step_u2 = nullptr;
  float* step_v2 = nullptr;
  // Tracer particles (structure of arrays, two buffers) and the render
  // target, allocated on first use.
  struct Particles {
    int cap = 0, n_upper = 0, cur = 0;
    float* a[2][4] = {};  // x, y, age, max age
    uint32_t* rgb[2] = {};
    int* count = nullptr;      // device: live particles
    uint8_t* keep = nullptr;   // device: survivor flags (cap rounded up to whole blocks)
    int* block_keep = nullptr;
  } parts;
  uint32_t* image = nullptr;
  void* image_pinned = nullptr;  // pinned staging of fg_render's frames for pageable targets
  // Non-null when this handle is a batch of scenes (fg_batch_create).
  fg::BatchGeom* batch = nullptr;
  // Asynchronous smoke download (fg_download_async): a copy stream, the event
  // it starts after and the copy's completion event; device operations after
  // the first one that follows the copy wait for it.
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t async_ev[2] = {};
  bool async_pending = false;
  int async_ops = 0;
  // A smoke read-back requested but not issued yet (fg_download_async): the
  // buffer to copy, and whether the operation being enqueued is a step that
  // issues it after its projection (mid_ev, recorded inside every step).
  bool async_deferred = false;
  const float* async_src = nullptr;
  bool async_defer_ok = false;
  bool step_mid = false;  // the step being enqueued records mid_ev
  cudaEvent_t mid_ev = nullptr;
  bool src_smoke = false;  // a persistent source writes M in place
  // Kernel launches enqueued so far (graph replays add the captured count).
  unsigned long long launches = 0;
  // Optional CUDA-event bracket around the main Jacobi launches of a solve.
  bool profile = false;
  cudaEvent_t prof_ev[2] = {};
  int prof_launches = 0;
  // With profiling on, events at the stage boundaries of each step.
  static constexpr int kMaxMarks = 16;
  cudaEvent_t mark_ev[kMaxMarks] = {};
  const char* mark_name[kMaxMarks] = {};
  int n_marks = 0;
  float* scalar_pinned = nullptr;  // small D2H results
  fg::DevStats* stats_pinned = nullptr;
  std::string last_error;

  // CUDA graphs of the step, keyed by the state pointers and dt.
  struct GraphEntry {
    float* key[8];   // state pointers before the step
    float* post[6];  // state pointers after it
    unsigned long long launches;  // kernels in the graph
    uint32_t dt_bits;
    uint64_t version;
    bool mid;  // records mid_ev after the projection (a read-back is deferred to the step)
    cudaGraphExec_t exec;
  };
  std::vector<GraphEntry> graphs;
  uint64_t params_version = 1;
};

namespace fg {

// Launchers implemented in the kernel translation units.  All enqueue on
// f->stream and return cudaGetLastError().
// k_forces.cu
cudaError_t launch_build_flags(fg_fluid* f);
cudaError_t launch_build_flags_on(cudaStream_t st, const float* S, uint8_t* flags, const Grid& g);
cudaError_t launch_apply_edits(fg_fluid* f, int n_groups, int slot);
cudaError_t launch_apply_sources(fg_fluid* f);
cudaError_t launch_viscosity(fg_fluid* f, float dt);  // U,V -> partner, newU/newV = result; swaps
cudaError_t launch_confinement_turbulence(fg_fluid* f, float dt, bool conf, bool turb);
cudaError_t launch_borders(fg_fluid* f);
cudaError_t launch_copy_border(fg_fluid* f, float* dst, const float* src);
cudaError_t launch_noise_table(fg_fluid* f);
// k_advect.cu
cudaError_t launch_advect_velocity(fg_fluid* f, float dt);
cudaError_t launch_advect_smoke(fg_fluid* f, float dt);
cudaError_t launch_advect_velocity_bfecc(fg_fluid* f, float dt);
cudaError_t launch_advect_smoke_bfecc(fg_fluid* f, float dt);
// k_pressure.cu
// Pressure solve + gradient subtract + post-projection divergence statistics;
// with fuse_turb (parallel scheme only) also addTurbulence.
cudaError_t launch_pressure(fg_fluid* f, int num_iters, float dt, bool fuse_turb);
// The MULTIGRID scheme's levels: masks, flags and weights rebuilt from the
// fine flags (the allocation is fg_api.cu's, outside stream capture).
cudaError_t launch_mg_rebuild(fg_fluid* f);
cudaError_t mg_kernel_setup();  // the bottom kernel's shared-memory limit (outside capture)
void mg_free(fg_fluid* f);
// solveMultigridVCycle (fluid.go:559-594) with the reference's serial
// smoothers, bit for bit.
cudaError_t launch_multigrid(fg_fluid* f, int num_iters, float dt);
// K Jacobi sweeps of A x = b from x = 0 (no early exit); ctl->sel names the
// buffer holding x.
void init_jacobi_tma();
void init_lexsor_cluster();
int lexsor_scratch_words();
int jacobi_tile_count(int NX, int NY);
cudaError_t launch_jacobi_solve(fg_fluid* f, void* ctl, const float* b, const float* bw, float* x0,
                                float* x1, int iters);
// Copies the last solve's potential to dst.
cudaError_t launch_store_phi(fg_fluid* f, float* dst);
// Gradient subtract with a stored potential (a recorded step's replay).
cudaError_t launch_grad_replay(fg_fluid* f, float dt, const float* phi, bool fuse_turb);
// k_adjoint.cu
constexpr int kTapeFields = 13;  // U2 V2 U4 V4 fwdU fwdV corrU corrV U5 V5 M1 fwdM corrM
cudaError_t launch_add_forces(fg_fluid* f, const float* fu, const float* fv);
// Zeroes a force field on the cells whose velocity the sources set (they
// overwrite the forced value), so the forces can be added after them.
cudaError_t launch_mask_forces(fg_fluid* f, float* fu, float* fv);
// Adjoint of one recorded step: adj[A_U..A_NM] go from the adjoint of the
// state after the step to that of the state before it; adj[A_U], adj[A_V]
// then also hold the adjoint of the step's force field.
cudaError_t launch_step_adjoint(fg_fluid* f, float dt, float* const* tape);
cudaError_t launch_loss_seed(fg_fluid* f, const float* target, double* dev_loss);
// k_diag.cu
cudaError_t launch_div_stats(fg_fluid* f);
cudaError_t launch_smoke_mass(fg_fluid* f);
// Combines the smoke-mass block partials the final smoke pass wrote.
cudaError_t launch_store_mass(fg_fluid* f, int nb);
cudaError_t launch_clear_stats(fg_fluid* f);
cudaError_t launch_max_divergence(fg_fluid* f, float* dev_out);
cudaError_t launch_view(fg_fluid* f, int kind, float* dev_minmax);  // 0 vorticity, 1 magnitude
cudaError_t launch_field_minmax(fg_fluid* f, int field, float* dev_minmax);
cudaError_t launch_sample_velocity(fg_fluid* f, float x, float y, float* dev_uv);
cudaError_t launch_max_speed(fg_fluid* f, float* dev_out);
// k_particles.cu: one advectParticles step from buffers `in` (x, y, age,
// max age; rgb_in) into `out`, survivors in order; *count is the live
// count, read and rewritten on the device; n_upper bounds it.
cudaError_t launch_particles_advect(fg_fluid* f, float dt, int n_upper, const float* const* in,
                                    const uint32_t* rgb_in, float* const* out, uint32_t* rgb_out,
                                    int* count, uint8_t* keep, int* block_keep);
// Renders `field` with the scientific (or, with diverging, the blue-white-
// red) colormap between dev_minmax[0..1] into an NX x NY RGBA8 image.
cudaError_t launch_render(fg_fluid* f, const float* field, const float* dev_minmax, int diverging,
                          uint32_t* img);
// Device-to-device copy of an NX x NY field between two row pitches.
cudaError_t launch_repitch(fg_fluid* f, float* dst, const float* src, int dpitch, int spitch);

// Grid of the reduction kernels: 32 x 8 threads per block over (j, i), at
// most about 1200 blocks; each block strides down the rows, so the single-
// block combine of the block partials stays short.
inline dim3 reduce_grid(const fg_fluid* f) {
  int gx = (f->NY + 31) / 32;
  int gy = (f->NX + 7) / 8;
  int cap = 1216 / gx;
  if (cap < 1) cap = 1;
  if (gy > cap) gy = cap;
  return dim3(gx, gy);
}

// True when a reduction with `ns` partials per block over `nb` blocks, plus
// its two-level combine, fits the partials buffer without reaching the
// scalar result slots at its end.
// Launches kernel k(args...) with programmatic stream serialization: it may
// be scheduled before the previous kernel on `st` finishes and must call
// pdl_enter first (see above).
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

inline bool partials_fit(const fg_fluid* f, int ns, int nb) {
  size_t rows = (size_t)nb + (size_t)((nb + 2047) / 2048) + 1;
  return 2 * (size_t)ns * rows + 8 <= (size_t)f->n_partials;
}

// Records a stage-boundary event named `name` (profiling only).
inline void mark(fg_fluid* f, const char* name) {
  if (!f->profile || f->n_marks >= fg_fluid::kMaxMarks) return;
  cudaEventRecord(f->mark_ev[f->n_marks], f->stream);
  f->mark_name[f->n_marks] = name;
  f->n_marks++;
}

// Counts one kernel launch on the handle (for the benchmark's launch tally).
inline void count(fg_fluid* f, int n = 1) { f->launches += (unsigned long long)n; }

inline void swap_state(fg_fluid* f, int field) {
  float* t = f->d[field];
  f->d[field] = f->partner[field];
  f->partner[field] = t;
}

}  // namespace fg
