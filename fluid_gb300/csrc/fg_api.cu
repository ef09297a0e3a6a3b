// C ABI of libfluidgpu: handle lifetime, host mirrors, tool edits, the step
// sequence and the views.  The kernels live in k_*.cu.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "fg_internal.cuh"

namespace fg {
size_t pctl_bytes(int n_slots);
int jacobi_launches(const fg_fluid* f, int iters);
void set_noalloc_stall(int tile);
}  // namespace fg

using namespace fg;

namespace {

constexpr int kSlots = 4096;

void tape_free(fg_fluid* f);  // differentiable rollouts, at the end of the file
void batch_free(fg::BatchGeom* b);  // batches, at the end of the file

// Entry points that address one scene's cells, mirrors or views are not
// available on a batch handle.
bool is_batch(const fg_fluid* f) { return f && f->batch; }
int batch_unsupported(const fg_fluid* f) {
  const_cast<fg_fluid*>(f)->last_error = "not available on a batch handle";
  return FG_ERR_UNSUPPORTED;
}

// Allocation-failure injection (fg_debug_fail_alloc): -1 off, else the
// number of allocations still to succeed before one fails.
std::atomic<int> g_alloc_fail_in{-1};
bool inject_alloc_failure() {
  int v = g_alloc_fail_in.load();
  while (v >= 0) {
    if (g_alloc_fail_in.compare_exchange_weak(v, v - 1)) return v == 0;
  }
  return false;
}
cudaError_t dev_malloc(void** p, size_t n) {
  if (inject_alloc_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, n);
}
cudaError_t host_malloc(void** p, size_t n) {
  if (inject_alloc_failure()) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMallocHost(p, n);
}

int fail(fg_fluid* f, int code, const char* what, cudaError_t e = cudaSuccess) {
  if (f) {
    char buf[512];
    if (e != cudaSuccess)
      snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    else
      snprintf(buf, sizeof buf, "%s", what);
    f->last_error = buf;
  }
  return code;
}

#define CK(f, call, what)                                  \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return fail(f, FG_ERR_CUDA, what, e_); \
  } while (0)

float host_go_min(float a, float b) {
  if (std::isnan(a) || std::isnan(b)) return std::nanf("");
  if (a == b) return std::signbit(a) ? a : b;
  return a < b ? a : b;
}
float host_go_max(float a, float b) {
  if (std::isnan(a) || std::isnan(b)) return std::nanf("");
  if (a == b) return std::signbit(a) ? b : a;
  return a > b ? a : b;
}

bool in_grid(const fg_fluid* f, int i, int j) { return i >= 0 && i < f->NX && j >= 0 && j < f->NY; }

int bind(fg_fluid* f) {
  cudaError_t e = cudaSetDevice(f->device);
  if (e != cudaSuccess) return fail(f, FG_ERR_CUDA, "cudaSetDevice", e);
  return FG_OK;
}

size_t field_bytes(const fg_fluid* f) { return sizeof(float) * (size_t)f->NX * f->P; }

int alloc_dev(fg_fluid* f, float** p) {
  cudaError_t e = dev_malloc((void**)p, field_bytes(f));
  if (e != cudaSuccess) return fail(f, FG_ERR_NOMEM, "cudaMalloc", e);
  e = cudaMemsetAsync(*p, 0, field_bytes(f), f->stream);
  if (e != cudaSuccess) return fail(f, FG_ERR_CUDA, "cudaMemsetAsync", e);
  return FG_OK;
}

int upload_field(fg_fluid* f, int k) {
  CK(f, cudaMemcpy2DAsync(f->d[k], sizeof(float) * f->P, f->hm[k], sizeof(float) * f->NY,
                          sizeof(float) * f->NY, f->NX, cudaMemcpyHostToDevice, f->stream),
     "upload");
  return FG_OK;
}

int download_field(fg_fluid* f, int k) {
  CK(f, cudaMemcpy2DAsync(f->hm[k], sizeof(float) * f->NY, f->d[k], sizeof(float) * f->P,
                          sizeof(float) * f->NY, f->NX, cudaMemcpyDeviceToHost, f->stream),
     "download");
  return FG_OK;
}

int check_mask(fg_fluid* f) {
  const float* S = f->hm[FG_S];
  size_t n = (size_t)f->NX * f->NY;
  for (size_t k = 0; k < n; ++k)
    if (!(S[k] == 0.0f || S[k] == 1.0f)) {
      char buf[160];
      snprintf(buf, sizeof buf, "S[%zu] = %g: the GPU step supports S values 0 and 1 only", k,
               (double)S[k]);
      return fail(f, FG_ERR_MASK, buf);
    }
  return FG_OK;
}

// Applies pending mirror uploads and queued tool edits, rebuilds the flag
// bytes if S changed.  Called at the start of every device operation.
// Orders device work after a pending asynchronous smoke download: the copy
// reads the smoke buffer of the step before it; the next operation writes
// the other buffer and may run beside it unless something writes M in place
// (an upload, an edit, a smoke source); every later operation waits for it.
// Issues the deferred smoke read-back on the copy stream once `after` (an
// event of the handle's stream) has happened.
int issue_async_copy(fg_fluid* f, cudaEvent_t after) {
  if (!f->async_deferred) return FG_OK;
  f->async_deferred = false;
  CK(f, cudaStreamWaitEvent(f->copy_stream, after, 0), "copy event");
  CK(f, cudaMemcpy2DAsync(f->hm[FG_M], sizeof(float) * f->NY, f->async_src, sizeof(float) * f->P,
                          sizeof(float) * f->NY, f->NX, cudaMemcpyDeviceToHost, f->copy_stream),
     "async download");
  CK(f, cudaEventRecord(f->async_ev[1], f->copy_stream), "copy event");
  return FG_OK;
}

int async_guard(fg_fluid* f) {
  if (!f->async_pending) return FG_OK;
  bool in_place = (f->dirty & FG_FIELD_BIT(FG_M)) || f->src_smoke;
  for (const EditRec& e : f->edits) in_place = in_place || e.field == (uint32_t)FG_M;
  // A step that writes M only out of place starts the copy itself, after its
  // projection; anything else starts it now.
  if (in_place || !f->async_defer_ok || f->async_ops > 0) {
    int rc = issue_async_copy(f, f->async_ev[0]);
    if (rc) return rc;
  }
  if (in_place || f->async_ops > 0)
    CK(f, cudaStreamWaitEvent(f->stream, f->async_ev[1], 0), "async wait");
  f->async_ops++;
  return FG_OK;
}

int flush(fg_fluid* f) {
  int rc = bind(f);
  if (rc) return rc;
  if ((rc = async_guard(f))) return rc;
  unsigned up = f->dirty;
  if (up & FG_FIELD_BIT(FG_S)) {
    if ((rc = check_mask(f))) {
      f->dirty &= ~FG_FIELD_BIT(FG_S);
      return rc;
    }
    f->masks_stale = true;
  }
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if (up & FG_FIELD_BIT(k))
      if ((rc = upload_field(f, k))) return rc;
  if (up) {
    // The caller may write the mirrors again as soon as we return.
    CK(f, cudaStreamSynchronize(f->stream), "upload sync");
  }
  f->dirty = 0;
  if (!f->edits.empty()) {
    std::vector<EditRec> ed;
    ed.reserve(f->edits.size());
    for (const EditRec& r : f->edits)
      if (!(up & FG_FIELD_BIT(r.field))) ed.push_back(r);
    f->edits.clear();
    if (!ed.empty()) {
      std::stable_sort(ed.begin(), ed.end(), [](const EditRec& a, const EditRec& b) {
        return a.field != b.field ? a.field < b.field : a.cell < b.cell;
      });
      std::vector<uint32_t> off;
      off.push_back(0);
      for (size_t k = 1; k < ed.size(); ++k)
        if (ed[k].field != ed[k - 1].field || ed[k].cell != ed[k - 1].cell) off.push_back((uint32_t)k);
      off.push_back((uint32_t)ed.size());
      size_t ng = off.size() - 1;
      int sl = f->edit_slot;
      f->edit_slot ^= 1;
      // The edit kernel reads the log straight from the slot's pinned
      // buffers (mapped into the device's address space: no upload); the
      // slot's previous kernel must have finished reading them.
      CK(f, cudaEventSynchronize(f->edit_ev[sl]), "edit slot wait");
      if (ed.size() > f->edit_cap[sl] || off.size() > f->edit_cap[sl] + 1) {
        cudaFreeHost(f->edit_pinned[sl]);
        cudaFreeHost(f->edit_off_pinned[sl]);
        f->edit_pinned[sl] = nullptr;
        f->edit_off_pinned[sl] = nullptr;
        f->edit_dev[sl] = nullptr;
        f->edit_off_dev[sl] = nullptr;
        f->edit_cap[sl] = 0;
        size_t cap = std::max<size_t>(ed.size(), off.size()) * 2;
        CK(f, host_malloc((void**)&f->edit_pinned[sl], cap * sizeof(EditRec)), "edit alloc");
        CK(f, host_malloc((void**)&f->edit_off_pinned[sl], (cap + 1) * sizeof(uint32_t)),
           "edit alloc");
        CK(f, cudaHostGetDevicePointer((void**)&f->edit_dev[sl], f->edit_pinned[sl], 0),
           "edit map");
        CK(f, cudaHostGetDevicePointer((void**)&f->edit_off_dev[sl], f->edit_off_pinned[sl], 0),
           "edit map");
        f->edit_cap[sl] = cap;
      }
      memcpy(f->edit_pinned[sl], ed.data(), ed.size() * sizeof(EditRec));
      memcpy(f->edit_off_pinned[sl], off.data(), off.size() * sizeof(uint32_t));
      f->edit_bytes += ed.size() * sizeof(EditRec) + off.size() * sizeof(uint32_t);
      CK(f, launch_apply_edits(f, (int)ng, sl), "apply edits");
      CK(f, cudaEventRecord(f->edit_ev[sl], f->stream), "edit event");
    }
  }
  if (f->masks_stale) {
    CK(f, launch_build_flags(f), "build flags");
    if (f->mg) CK(f, launch_mg_rebuild(f), "multigrid levels");
    f->masks_stale = false;
  }
  return FG_OK;
}

void invalidate(fg_fluid* f, unsigned mask) {
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if ((mask & FG_FIELD_BIT(k)) && k != FG_S) f->host_valid[k] = false;
}

constexpr unsigned kStepFields = FG_ALL_FIELDS & ~FG_FIELD_BIT(FG_S);

// Records a tool edit of `field` at host index `cell`: applied to a current
// mirror at once, and queued for the device unless the mirror is scheduled
// for upload anyway.
void edit(fg_fluid* f, int field, int cell, int op, float value) {
  if (f->host_valid[field]) {
    float& m = f->hm[field][cell];
    m = op == 0 ? value : m + value;
  }
  if (!(f->dirty & FG_FIELD_BIT(field))) f->edits.push_back(EditRec{(uint32_t)field, (uint32_t)cell, (uint32_t)op, value});
}

int check_params(fg_fluid* f, const fg_params* p) {
  if (p->num_iters < 0) return fail(f, FG_ERR_INVALID, "num_iters < 0");
  if (p->scheme != FG_SCHEME_LEXSOR && p->scheme != FG_SCHEME_JACOBI &&
      p->scheme != FG_SCHEME_MULTIGRID)
    return fail(f, FG_ERR_INVALID, "unknown pressure scheme");
  if (p->scheme == FG_SCHEME_MULTIGRID && p->refine_sweeps > 0)
    return fail(f, FG_ERR_UNSUPPORTED, "MULTIGRID takes no outer correction (refine_sweeps 0)");
  if (p->refine_sweeps < 0) return fail(f, FG_ERR_INVALID, "refine_sweeps < 0");
  return FG_OK;
}

void clear_graphs(fg_fluid* f) {
  for (auto& g : f->graphs) cudaGraphExecDestroy(g.exec);
  f->graphs.clear();
}

int check_iters(fg_fluid* f, int iters) {
  if (iters < 0) return fail(f, FG_ERR_INVALID, "num_iters < 0");
  if (f->prm.scheme == FG_SCHEME_JACOBI) {
    // In 64 bits; a count whose control block would pass 2^24 launch slots
    // (64 MiB) is refused rather than allowed to wrap.
    const long long need =
        (long long)std::max(jacobi_launches(f, iters), jacobi_launches(f, f->prm.refine_sweeps)) +
        1;
    if (need > (1ll << 24)) return fail(f, FG_ERR_INVALID, "num_iters: too many Jacobi launches");
    if (need > f->n_slots) {
      CK(f, cudaStreamSynchronize(f->stream), "sync");
      cudaFree(f->pctl);
      cudaFree(f->ectl);
      f->n_slots = (int)need * 2;
      CK(f, dev_malloc(&f->pctl, pctl_bytes(f->n_slots)), "pctl alloc");
      CK(f, dev_malloc(&f->ectl, pctl_bytes(f->n_slots)), "pctl alloc");
      CK(f, cudaMemsetAsync(f->pctl, 0, pctl_bytes(f->n_slots), f->stream), "pctl");
      CK(f, cudaMemsetAsync(f->ectl, 0, pctl_bytes(f->n_slots), f->stream), "pctl");
      clear_graphs(f);
    }
  }
  return FG_OK;
}

// Enqueues makeIncompressible's solve with the statistics of the projected
// field.
// fuse_turb: run addTurbulence inside the parallel scheme's gradient kernel.
bool multigrid(const fg_fluid* f) { return f->prm.use_multigrid && f->prm.multigrid_levels > 1; }

int enqueue_pressure(fg_fluid* f, int iters, float dt, bool fuse_turb) {
  if (multigrid(f)) {
    // UseMultigrid (fluid.go:148-149) runs the reference's V-cycle whatever
    // the single-grid scheme.
    CK(f, launch_multigrid(f, iters, dt), "multigrid");
    CK(f, launch_div_stats(f), "div stats");
    return FG_OK;
  }
  CK(f, launch_pressure(f, iters, dt, fuse_turb), "pressure");
  if (f->prm.scheme == FG_SCHEME_LEXSOR) CK(f, launch_div_stats(f), "div stats");
  return FG_OK;
}

// One Simulate(dt) (fluid.go:79-109) as a kernel sequence; swaps the state
// pointers as the out-of-place stages run.
int enqueue_step(fg_fluid* f, float dt) {
  const fg_params& p = f->prm;
  f->n_marks = 0;
  mark(f, "start");
  CK(f, launch_apply_sources(f), "sources");
  CK(f, launch_clear_stats(f), "clear stats");
  if (p.scheme == FG_SCHEME_LEXSOR || multigrid(f))
    CK(f, cudaMemsetAsync(f->d[FG_P], 0, field_bytes(f), f->stream), "fill p");
  if (p.viscosity_diffusion > 0.0f) CK(f, launch_viscosity(f, dt), "viscosity");
  mark(f, "sources+viscosity");
  const bool conf = p.confinement != 0.0f, turb = p.turbulence_strength > 0.0f;
  const bool fuse_turb = (p.scheme == FG_SCHEME_JACOBI || p.scheme == FG_SCHEME_MULTIGRID) &&
                         !multigrid(f) && !conf && turb;
  int rc = enqueue_pressure(f, p.num_iters, dt, fuse_turb);
  if (rc) return rc;
  mark(f, "gradient+div stats");
  // The projection is done: a smoke read-back deferred to this step may
  // start (an event-record node when the step is captured).  Only steps
  // with a deferred read-back record it, and they are captured into graphs
  // of their own: the node costs a replay about 4 us.  (Recorded on a side
  // branch of the graph instead, it cost 2.5 us, but the copy then started
  // later and the step with the read-back ran 7-9 us longer.)
  if (f->step_mid) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(f, cudaStreamIsCapturing(f->stream, &cs), "capture status");
    CK(f, cs == cudaStreamCaptureStatusActive
              ? cudaEventRecordWithFlags(f->mid_ev, f->stream, cudaEventRecordExternal)
              : cudaEventRecord(f->mid_ev, f->stream),
       "mid-step event");
  }
  if (!fuse_turb) CK(f, launch_confinement_turbulence(f, dt, conf, turb), "confinement/turbulence");
  CK(f, launch_borders(f), "borders");
  mark(f, "confinement/turbulence+borders");
  if (p.use_bfecc) {
    CK(f, launch_advect_velocity_bfecc(f, dt), "advect velocity");
    mark(f, "advect velocity");
    CK(f, launch_advect_smoke_bfecc(f, dt), "advect smoke");
  } else {
    CK(f, launch_advect_velocity(f, dt), "advect velocity");
    mark(f, "advect velocity");
    CK(f, launch_advect_smoke(f, dt), "advect smoke");
  }
  mark(f, "advect smoke+mass");
  return FG_OK;
}

void state_key(const fg_fluid* f, float* key[8]) {
  key[0] = f->d[FG_U];
  key[1] = f->d[FG_V];
  key[2] = f->d[FG_M];
  key[3] = f->partner[FG_U];
  key[4] = f->partner[FG_V];
  key[5] = f->partner[FG_M];
  key[6] = nullptr;
  key[7] = nullptr;
}

}  // namespace

extern "C" {

int fg_params_default(fg_params* out) {
  if (!out) return FG_ERR_INVALID;
  memset(out, 0, sizeof *out);
  out->confinement = 0.0f;
  out->viscosity_diffusion = 0.0f;
  out->pressure_damping = 1.0f;
  out->turbulence_strength = 0.02f;
  out->smoke_advection = 1.0f;
  out->use_multigrid = 0;
  out->multigrid_levels = 2;
  out->use_bfecc = 0;
  out->relaxation = 1.9f;
  out->num_iters = 8;
  out->tolerance = 1e-5f;
  out->early_exit = 1;
  out->scheme = FG_SCHEME_LEXSOR;
  out->jacobi_omega = 1.0f;
  out->tb_depth = 8;
  out->refine_sweeps = 0;
  out->use_graphs = 1;
  return FG_OK;
}

int fg_create(int width, int height, float density, float h, const fg_params* params,
              fg_fluid** out) {
  if (!out || width < 1 || height < 1 || !(h > 0.0f)) return FG_ERR_INVALID;
  // Cell indices are 32-bit: the padded grid (rows of NY rounded up to 32)
  // stays within 2^30 cells.
  const long long nx = (long long)width + 2, pitch = ((long long)height + 2 + 31) / 32 * 32;
  if (nx * pitch > (1ll << 30)) return FG_ERR_INVALID;
  *out = nullptr;
  fg_fluid* f = new fg_fluid();
  fg_params_default(&f->prm);
  if (params) {
    if (check_params(f, params)) {
      delete f;
      return FG_ERR_INVALID;
    }
    f->prm = *params;
  }
  f->NX = width + 2;
  f->NY = height + 2;
  f->P = (f->NY + 31) / 32 * 32;
  f->density = density;
  f->h = h;
  f->g = make_grid(f->NX, f->NY, f->P, h);
  f->g.precise = f->prm.precise_coords ? 1 : 0;
  int rc = FG_OK;
  auto bail = [&](int code) {
    fg_destroy(f);
    return code;
  };
  if (cudaGetDevice(&f->device) != cudaSuccess) return bail(FG_ERR_CUDA);
  // The per-context set-up below needs a current context, which
  // cudaGetDevice does not create; cudaFree(nullptr) makes the runtime use
  // the caller's current context or create the device's primary one.
  if (cudaFree(nullptr) != cudaSuccess) return bail(FG_ERR_CUDA);
  init_jacobi_tma();
  init_lexsor_cluster();
  if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(FG_ERR_CUDA);
  for (int k = 0; k < 2; ++k) {
    if (cudaEventCreateWithFlags(&f->edit_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return bail(FG_ERR_CUDA);
    if (cudaEventCreate(&f->prof_ev[k]) != cudaSuccess) return bail(FG_ERR_CUDA);
  }
  if (cudaEventCreateWithFlags(&f->mid_ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(FG_ERR_CUDA);
  for (int k = 0; k < fg_fluid::kMaxMarks; ++k)
    if (cudaEventCreate(&f->mark_ev[k]) != cudaSuccess) return bail(FG_ERR_CUDA);
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if ((rc = alloc_dev(f, &f->d[k]))) return bail(rc);
  for (int k : {FG_U, FG_V, FG_M})
    if ((rc = alloc_dev(f, &f->partner[k]))) return bail(rc);
  float** scratch[] = {&f->fwdU, &f->fwdV, &f->fwdM, &f->corrU, &f->corrV, &f->corrM,
                       &f->phi,  &f->phi2, &f->rhs,  &f->err,   &f->err2,  &f->rhs_e,
                       &f->curl, &f->view, &f->wgt,  &f->bw,    &f->bwe};
  for (float** s : scratch)
    if ((rc = alloc_dev(f, s))) return bail(rc);
  size_t cells = (size_t)f->NX * f->P;
  if (dev_malloc((void**)&f->noise, cells * sizeof(float2)) != cudaSuccess) return bail(FG_ERR_NOMEM);
  if (dev_malloc((void**)&f->flags, cells) != cudaSuccess) return bail(FG_ERR_NOMEM);
  int nb = ((f->NY + 31) / 32) * ((f->NX + 7) / 8);
  // Rows of up to 5 float-pair slots per block, the combine levels and the
  // scalar result slots at the end.
  f->n_partials = 16 * nb + 512;
  if (dev_malloc((void**)&f->partials, sizeof(float) * f->n_partials) != cudaSuccess)
    return bail(FG_ERR_NOMEM);
  if (dev_malloc((void**)&f->dstats, sizeof(DevStats)) != cudaSuccess) return bail(FG_ERR_NOMEM);
  f->n_slots = kSlots;
  if (dev_malloc(&f->pctl, pctl_bytes(f->n_slots)) != cudaSuccess) return bail(FG_ERR_NOMEM);
  if (dev_malloc(&f->ectl, pctl_bytes(f->n_slots)) != cudaSuccess) return bail(FG_ERR_NOMEM);
  if (dev_malloc((void**)&f->tile_done, sizeof(int) * ((size_t)jacobi_tile_count(f->NX, f->NY) + 1)) !=
      cudaSuccess)
    return bail(FG_ERR_NOMEM);
  cudaMemsetAsync(f->pctl, 0, pctl_bytes(f->n_slots), f->stream);
  cudaMemsetAsync(f->ectl, 0, pctl_bytes(f->n_slots), f->stream);
  cudaMemsetAsync(f->dstats, 0, sizeof(DevStats), f->stream);
  cudaMemsetAsync(f->flags, 0, cells, f->stream);
  size_t hbytes = sizeof(float) * (size_t)f->NX * f->NY;
  for (int k = 0; k < FG_NUM_FIELDS; ++k) {
    if (host_malloc((void**)&f->hm[k], hbytes) != cudaSuccess) return bail(FG_ERR_NOMEM);
    memset(f->hm[k], 0, hbytes);
    f->host_valid[k] = true;
  }
  if (host_malloc((void**)&f->scalar_pinned, 64 * sizeof(float)) != cudaSuccess)
    return bail(FG_ERR_NOMEM);
  if (host_malloc((void**)&f->stats_pinned, sizeof(DevStats)) != cudaSuccess)
    return bail(FG_ERR_NOMEM);
  if (launch_noise_table(f) != cudaSuccess) return bail(FG_ERR_CUDA);
  f->masks_stale = true;
  if (flush(f) || cudaStreamSynchronize(f->stream) != cudaSuccess) return bail(FG_ERR_CUDA);
  *out = f;
  return FG_OK;
}

int fg_destroy(fg_fluid* f) {
  if (!f) return FG_ERR_INVALID;
  cudaSetDevice(f->device);
  if (f->stream) cudaStreamSynchronize(f->stream);
  if (f->copy_stream) cudaStreamSynchronize(f->copy_stream);
  clear_graphs(f);
  tape_free(f);
  batch_free(f->batch);
  mg_free(f);
  for (int k = 0; k < fg_fluid::A_COUNT; ++k) cudaFree(f->adj[k]);
  for (int b = 0; b < 2; ++b) {
    for (int q = 0; q < 4; ++q) cudaFree(f->parts.a[b][q]);
    cudaFree(f->parts.rgb[b]);
  }
  cudaFree(f->parts.count);
  cudaFree(f->parts.keep);
  cudaFree(f->parts.block_keep);
  cudaFree(f->image);
  if (f->copy_stream) cudaStreamDestroy(f->copy_stream);
  for (int k = 0; k < 2; ++k)
    if (f->async_ev[k]) cudaEventDestroy(f->async_ev[k]);
  if (f->mid_ev) cudaEventDestroy(f->mid_ev);
  for (int k = 0; k < FG_NUM_FIELDS; ++k) {
    cudaFree(f->d[k]);
    cudaFree(f->partner[k]);
    cudaFreeHost(f->hm[k]);
  }
  float* scratch[] = {f->fwdU, f->fwdV, f->fwdM, f->corrU, f->corrV, f->corrM, f->phi,
                      f->phi2, f->rhs,  f->err,  f->err2,  f->rhs_e, f->curl,  f->view,
                      f->wgt,  f->bw,   f->bwe,  f->copy_tmp};
  for (float* s : scratch) cudaFree(s);
  cudaFree(f->noise);
  cudaFree(f->flags);
  cudaFree(f->src_dev);
  cudaFree(f->src_off_dev);
  cudaFree(f->partials);
  cudaFree(f->dstats);
  cudaFree(f->pctl);
  cudaFree(f->ectl);
  cudaFree(f->tile_done);
  if (f->image_pinned) cudaFreeHost(f->image_pinned);
  for (float* q : f->skew) cudaFree(q);
  cudaFree(f->skew_flags);
  cudaFree(f->lex_scratch);
  for (int k = 0; k < 2; ++k) {
    cudaFreeHost(f->edit_pinned[k]);  // edit_dev / edit_off_dev map these
    cudaFreeHost(f->edit_off_pinned[k]);
    if (f->edit_ev[k]) cudaEventDestroy(f->edit_ev[k]);
    if (f->prof_ev[k]) cudaEventDestroy(f->prof_ev[k]);
  }
  for (int k = 0; k < fg_fluid::kMaxMarks; ++k)
    if (f->mark_ev[k]) cudaEventDestroy(f->mark_ev[k]);
  cudaFreeHost(f->scalar_pinned);
  cudaFreeHost(f->stats_pinned);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
  return FG_OK;
}

int fg_dims(const fg_fluid* f, int* nx, int* ny) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !nx || !ny) return FG_ERR_INVALID;
  *nx = f->NX;
  *ny = f->NY;
  return FG_OK;
}

float fg_h(const fg_fluid* f) { return f ? f->h : 0.0f; }

int fg_get_params(const fg_fluid* f, fg_params* out) {
  if (!f || !out) return FG_ERR_INVALID;
  *out = f->prm;
  return FG_OK;
}

int fg_set_params(fg_fluid* f, const fg_params* p) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !p) return FG_ERR_INVALID;
  int rc = check_params(f, p);
  if (rc) return rc;
  if (memcmp(&f->prm, p, sizeof *p) != 0) {
    f->prm = *p;
    f->g.precise = p->precise_coords ? 1 : 0;
    f->params_version++;
  }
  return FG_OK;
}

int fg_field(fg_fluid* f, int field, float** host_ptr) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !host_ptr || field < 0 || field >= FG_NUM_FIELDS) return FG_ERR_INVALID;
  *host_ptr = f->hm[field];
  return FG_OK;
}

int fg_mark_dirty(fg_fluid* f, unsigned mask) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if ((mask & FG_FIELD_BIT(k)) && !f->host_valid[k])
      return fail(f, FG_ERR_INVALID, "mirror is not current: fg_download it before writing");
  f->dirty |= mask & FG_ALL_FIELDS;
  return FG_OK;
}

int fg_download_wait(fg_fluid* f);

int fg_download(fg_fluid* f, unsigned mask) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = fg_download_wait(f);
  if (rc) return rc;
  if ((rc = flush(f))) return rc;
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if ((mask & FG_FIELD_BIT(k)) && !f->host_valid[k])
      if ((rc = download_field(f, k))) return rc;
  CK(f, cudaStreamSynchronize(f->stream), "download sync");
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if (mask & FG_FIELD_BIT(k)) f->host_valid[k] = true;
  return FG_OK;
}

// Copies the smoke field M of the work enqueued so far into its host mirror
// on a second stream, beside the next step (after that step's projection);
// fg_download_wait completes it (the mirror is not current until then).
int fg_download_async(fg_fluid* f, unsigned mask) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  if (mask & ~FG_FIELD_BIT(FG_M))
    return fail(f, FG_ERR_UNSUPPORTED, "asynchronous downloads take the smoke field only");
  int rc = fg_download_wait(f);
  if (rc || !mask) return rc;
  if ((rc = flush(f))) return rc;
  if (f->host_valid[FG_M]) return FG_OK;
  if (!f->copy_stream) {
    CK(f, cudaStreamCreateWithFlags(&f->copy_stream, cudaStreamNonBlocking), "copy stream");
    for (int k = 0; k < 2; ++k)
      CK(f, cudaEventCreateWithFlags(&f->async_ev[k], cudaEventDisableTiming), "copy event");
  }
  // The copy is issued later: by the next step, once that step's
  // projection is done (a copy beside the pressure solve slows it, whose
  // arrays live in L2), or at once by anything else (issue_async_copy).
  CK(f, cudaEventRecord(f->async_ev[0], f->stream), "copy event");
  f->async_src = f->d[FG_M];
  f->async_deferred = true;
  f->async_pending = true;
  f->async_ops = 0;
  return FG_OK;
}

int fg_download_wait(fg_fluid* f) {
  if (!f) return FG_ERR_INVALID;
  if (!f->async_pending) return FG_OK;
  int rc = bind(f);
  if (rc) return rc;
  if ((rc = issue_async_copy(f, f->async_ev[0]))) return rc;
  CK(f, cudaEventSynchronize(f->async_ev[1]), "async download");
  f->async_pending = false;
  // The mirror holds the copied frame; it is the device's M only if nothing
  // has run since the copy was issued.
  f->host_valid[FG_M] = f->async_ops == 0;
  return FG_OK;
}

int fg_synchronize(fg_fluid* f) {
  if (!f) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  CK(f, cudaStreamSynchronize(f->stream), "synchronize");
  return FG_OK;
}

void* fg_stream(fg_fluid* f) { return f ? (void*)f->stream : nullptr; }

// The diagonal-major copies of the wavefront SOR (LEXSOR and the multigrid
// smoothers), allocated before the first step that uses them (outside any
// capture); without them the row-major kernel runs.
void ensure_skew(fg_fluid* f) {
  if (f->skew[0] || f->batch || !(f->prm.scheme == FG_SCHEME_LEXSOR || multigrid(f))) return;
  const int sp = (f->NX + 31) / 32 * 32;
  const size_t n = (size_t)(f->NX + f->NY - 1) * sp;
  // The wavefront kernels index the copies with 32-bit integers: a grid much
  // wider than tall whose copies exceed that keeps the row-major kernel.
  if (n > (size_t)INT_MAX) return;
  float* a[3] = {};
  uint8_t* fl = nullptr;
  bool ok = true;
  for (auto& q : a) ok = ok && dev_malloc((void**)&q, n * sizeof(float)) == cudaSuccess;
  ok = ok && dev_malloc((void**)&fl, n) == cudaSuccess;
  unsigned* lex = nullptr;
  ok = ok && dev_malloc((void**)&lex, sizeof(unsigned) * lexsor_scratch_words()) == cudaSuccess;
  if (!ok) {
    for (auto& q : a) cudaFree(q);
    cudaFree(fl);
    cudaFree(lex);
    cudaGetLastError();
    return;
  }
  f->lex_scratch = lex;
  for (int k = 0; k < 3; ++k) f->skew[k] = a[k];
  f->skew_flags = fl;
  f->skew_sp = sp;
  f->params_version++;  // captured steps run the other kernel sequence
}

// Allocates the MULTIGRID scheme's levels below the handle's grid (interior
// sides halved until the shorter is at most kMgMinSide) and builds their
// masks, flags and weights; called outside stream capture before a solve.
// Rebuilds the coarse weights when PressureDamping changed since.
static int mg_prepare(fg_fluid* f) {
  if (f->prm.scheme != FG_SCHEME_MULTIGRID || f->batch) return FG_OK;
  if (f->mg) {
    if (f->mg->omega != kMgOmega * f->prm.pressure_damping) {
      CK(f, launch_mg_rebuild(f), "multigrid levels");
      f->params_version++;
    }
    return FG_OK;
  }
  if (std::min(f->NX, f->NY) - 2 <= kMgMinSide)
    return fail(f, FG_ERR_UNSUPPORTED, "MULTIGRID needs an interior side above 8 cells");
  MgHier* h = new MgHier();
  MgLevelDev l0;
  l0.g = f->g;
  l0.S = f->d[FG_S];
  l0.flags = f->flags;
  l0.w = f->wgt;
  l0.b = f->rhs;
  l0.bw = f->bw;
  l0.x[0] = f->phi;
  l0.x[1] = f->phi2;
  h->lv.push_back(l0);
  std::vector<size_t> off;
  size_t total = 0;
  int nx = f->NX, ny = f->NY;
  while (std::min(nx, ny) - 2 > kMgMinSide) {
    nx = (nx - 2 + 1) / 2 + 2;
    ny = (ny - 2 + 1) / 2 + 2;
    MgLevelDev c;
    c.g = make_grid(nx, ny, (ny + 31) / 32 * 32, f->h);
    h->lv.push_back(c);
    off.push_back(total);
    total += (6 * sizeof(float) + 1) * (size_t)nx * c.g.P;
    total = (total + 255) / 256 * 256;
  }
  if (dev_malloc(&h->block, total) != cudaSuccess || dev_malloc(&h->ctl, 64) != cudaSuccess) {
    cudaFree(h->block);
    delete h;
    return fail(f, FG_ERR_NOMEM, "multigrid levels");
  }
  for (size_t l = 1; l < h->lv.size(); ++l) {
    MgLevelDev& c = h->lv[l];
    const size_t cells = (size_t)c.g.NX * c.g.P;
    float* base = reinterpret_cast<float*>(static_cast<unsigned char*>(h->block) + off[l - 1]);
    c.S = base;
    c.w = base + cells;
    c.b = base + 2 * cells;
    c.bw = base + 3 * cells;
    c.x[0] = base + 4 * cells;
    c.x[1] = base + 5 * cells;
    c.flags = reinterpret_cast<uint8_t*>(base + 6 * cells);
  }
  f->mg = h;
  // Zeroed once: the padding columns and the ghost rings are never written
  // and must read as 0.
  CK(f, mg_kernel_setup(), "multigrid levels");
  CK(f, cudaMemsetAsync(h->block, 0, total, f->stream), "multigrid levels");
  CK(f, cudaMemsetAsync(h->ctl, 0, 64, f->stream), "multigrid levels");
  CK(f, launch_mg_rebuild(f), "multigrid levels");
  f->params_version++;
  return FG_OK;
}

static int simulate_enqueue(fg_fluid* f, float dt);

int fg_simulate(fg_fluid* f, float dt) {
  if (!f) return FG_ERR_INVALID;
  f->async_defer_ok = true;
  int rc = simulate_enqueue(f, dt);
  f->async_defer_ok = false;
  f->step_mid = false;
  // A read-back deferred to this step starts after its projection, or after
  // the copied work when the step was not enqueued.
  if (f->async_deferred) {
    int rc2 = issue_async_copy(f, rc == FG_OK ? f->mid_ev : f->async_ev[0]);
    if (!rc) rc = rc2;
  }
  return rc;
}

static int simulate_enqueue(fg_fluid* f, float dt) {
  int rc = flush(f);
  if (rc) return rc;
  f->step_mid = f->async_deferred;
  ensure_skew(f);
  if ((rc = check_iters(f, f->prm.num_iters))) return rc;
  if ((rc = mg_prepare(f))) return rc;
  invalidate(f, kStepFields);
  // Profiling brackets the Jacobi launches with timed events, which plain
  // capture would turn into graph-internal dependencies: run it uncaptured.
  if (!f->prm.use_graphs || f->profile) return enqueue_step(f, dt);
  float* key[8];
  state_key(f, key);
  uint32_t dtb;
  memcpy(&dtb, &dt, 4);
  for (auto& g : f->graphs) {
    if (g.dt_bits == dtb && g.version == f->params_version && g.mid == f->step_mid &&
        memcmp(g.key, key, sizeof key) == 0) {
      CK(f, cudaGraphLaunch(g.exec, f->stream), "graph launch");
      f->launches += g.launches;
      // Apply the pointer rotation the captured step performed.
      f->d[FG_U] = g.post[0];
      f->d[FG_V] = g.post[1];
      f->d[FG_M] = g.post[2];
      f->partner[FG_U] = g.post[3];
      f->partner[FG_V] = g.post[4];
      f->partner[FG_M] = g.post[5];
      return FG_OK;
    }
  }
  // Capture this configuration (at most two entries per configuration: the
  // rotation alternates between two pointer states).
  if (f->graphs.size() >= 8) clear_graphs(f);
  fg_fluid::GraphEntry ent;
  memcpy(ent.key, key, sizeof key);
  ent.dt_bits = dtb;
  ent.version = f->params_version;
  ent.mid = f->step_mid;
  // The Jacobi kernels' per-context set-up cannot run inside a capture: do
  // it first (a no-op once done), so the captured step gets the TMA-fed and
  // dataflow kernels even if this thread's context changed since fg_create.
  init_jacobi_tma();
  CK(f, cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  unsigned long long before = f->launches;
  rc = enqueue_step(f, dt);
  ent.launches = f->launches - before;
  f->launches = before;
  cudaGraph_t graph = nullptr;
  cudaError_t ec = cudaStreamEndCapture(f->stream, &graph);
  if (rc || ec != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    // Restore the pre-step pointers; nothing was executed.
    f->d[FG_U] = key[0];
    f->d[FG_V] = key[1];
    f->d[FG_M] = key[2];
    f->partner[FG_U] = key[3];
    f->partner[FG_V] = key[4];
    f->partner[FG_M] = key[5];
    return rc ? rc : fail(f, FG_ERR_CUDA, "end capture", ec);
  }
  ent.post[0] = f->d[FG_U];
  ent.post[1] = f->d[FG_V];
  ent.post[2] = f->d[FG_M];
  ent.post[3] = f->partner[FG_U];
  ent.post[4] = f->partner[FG_V];
  ent.post[5] = f->partner[FG_M];
  ec = cudaGraphInstantiate(&ent.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ec != cudaSuccess) return fail(f, FG_ERR_CUDA, "graph instantiate", ec);
  f->graphs.push_back(ent);
  CK(f, cudaGraphLaunch(ent.exec, f->stream), "graph launch");
  f->launches += ent.launches;
  return FG_OK;
}

int fg_get_stats(fg_fluid* f, fg_stats* out) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !out) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  CK(f, cudaMemcpyAsync(f->stats_pinned, f->dstats, sizeof(DevStats), cudaMemcpyDeviceToHost,
                        f->stream), "stats");
  CK(f, cudaStreamSynchronize(f->stream), "stats sync");
  const DevStats& s = *f->stats_pinned;
  memset(out, 0, sizeof *out);
  out->div_l2_post = std::sqrt(s.div_l2_sq);
  out->div_max_post = s.div_max;
  out->div_count_post = s.div_count;
  out->resid_l2 = std::sqrt(s.resid_l2_sq);
  out->resid_max = s.resid_max;
  out->smoke_mass = s.smoke_mass;
  out->last_maxdiv = s.last_maxdiv;
  out->sweeps = s.sweeps;
  out->jacobi_kernel = f->jacobi_kernel;
  if (s.timeout) return fail(f, FG_ERR_TIMEOUT, "a device-side wait of the last step gave up");
  for (double v : {s.div_l2_sq, s.div_max, s.resid_l2_sq, s.resid_max, s.smoke_mass, s.last_maxdiv})
    if (!std::isfinite(v)) return fail(f, FG_ERR_NONFINITE, "the last step produced non-finite values");
  return FG_OK;
}

// ------------------------------------------------------------------ stages
#define STAGE_PROLOGUE(f)       \
  if (!(f)) return FG_ERR_INVALID; \
  int rc = flush(f);            \
  if (rc) return rc;

int fg_make_incompressible(fg_fluid* f, int num_iters, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  ensure_skew(f);
  if ((rc = check_iters(f, num_iters))) return rc;
  if ((rc = mg_prepare(f))) return rc;
  invalidate(f, kStepFields);
  CK(f, launch_clear_stats(f), "clear stats");
  // copyBorder(newU, U), copyBorder(newV, V) (fluid.go:145-146).
  CK(f, launch_copy_border(f, f->d[FG_NEWU], f->d[FG_U]), "copy border");
  CK(f, launch_copy_border(f, f->d[FG_NEWV], f->d[FG_V]), "copy border");
  return enqueue_pressure(f, num_iters, dt, false);
}

int fg_advect_velocity(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, kStepFields);
  CK(f, launch_advect_velocity(f, dt), "advect velocity");
  return FG_OK;
}

int fg_advect_smoke(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, kStepFields);
  CK(f, launch_advect_smoke(f, dt), "advect smoke");
  return FG_OK;
}

int fg_advect_velocity_bfecc(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, kStepFields);
  CK(f, launch_advect_velocity_bfecc(f, dt), "advect velocity bfecc");
  return FG_OK;
}

int fg_advect_smoke_bfecc(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, kStepFields);
  CK(f, launch_advect_smoke_bfecc(f, dt), "advect smoke bfecc");
  return FG_OK;
}

int fg_handle_borders(fg_fluid* f) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, kStepFields);
  CK(f, launch_borders(f), "borders");
  return FG_OK;
}

int fg_apply_vorticity_confinement(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, kStepFields);
  CK(f, launch_confinement_turbulence(f, dt, true, false), "confinement");
  return FG_OK;
}

int fg_apply_viscosity(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  if (!(f->prm.viscosity_diffusion > 0.0f)) return FG_OK;  // fluid.go:113-115
  invalidate(f, kStepFields);
  CK(f, launch_viscosity(f, dt), "viscosity");
  return FG_OK;
}

int fg_add_turbulence(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  if (!(f->prm.turbulence_strength > 0.0f)) return FG_OK;  // fluid.go:497-499
  invalidate(f, kStepFields);
  CK(f, launch_confinement_turbulence(f, dt, false, true), "turbulence");
  return FG_OK;
}

int fg_clear_pressure(fg_fluid* f) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  invalidate(f, FG_FIELD_BIT(FG_P));
  CK(f, cudaMemsetAsync(f->d[FG_P], 0, field_bytes(f), f->stream), "fill p");
  return FG_OK;
}

int fg_copy_border(fg_fluid* f, float* dst, const float* src) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  if (!dst || !src) return fail(f, FG_ERR_INVALID, "null buffer");
  if (!f->copy_tmp)
    CK(f, dev_malloc((void**)&f->copy_tmp, 2 * field_bytes(f)), "copy_border alloc");
  float* dd = f->copy_tmp;
  float* ds = f->copy_tmp + (size_t)f->NX * f->P;
  size_t hp = sizeof(float) * f->NY, dp = sizeof(float) * f->P;
  CK(f, cudaMemcpy2DAsync(dd, dp, dst, hp, hp, f->NX, cudaMemcpyHostToDevice, f->stream), "copy");
  CK(f, cudaMemcpy2DAsync(ds, dp, src, hp, hp, f->NX, cudaMemcpyHostToDevice, f->stream), "copy");
  CK(f, launch_copy_border(f, dd, ds), "copy border");
  CK(f, cudaMemcpy2DAsync(dst, hp, dd, dp, hp, f->NX, cudaMemcpyDeviceToHost, f->stream), "copy");
  CK(f, cudaStreamSynchronize(f->stream), "copy sync");
  return FG_OK;
}

// ------------------------------------------------------------------ tools
int fg_set_solid(fg_fluid* f, int i, int j, int value) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  if (!in_grid(f, i, j)) return fail(f, FG_ERR_INDEX, i < 0 || i >= f->NX ? "invalid x-index" : "invalid y-index");
  int n = f->NY;
  int cell = i * n + j;
  f->hm[FG_S][cell] = value ? 0.0f : 1.0f;
  f->dirty |= FG_FIELD_BIT(FG_S);
  if (value) {
    for (int fld : {FG_U, FG_NEWU}) {
      edit(f, fld, cell, 0, 0.0f);
      if (i + 1 < f->NX) edit(f, fld, (i + 1) * n + j, 0, 0.0f);
    }
    for (int fld : {FG_V, FG_NEWV}) {
      edit(f, fld, cell, 0, 0.0f);
      if (j + 1 < f->NY) edit(f, fld, cell + 1, 0, 0.0f);
    }
  }
  return FG_OK;
}

int fg_is_solid(const fg_fluid* f, int i, int j, int* out) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !out) return FG_ERR_INVALID;
  if (!in_grid(f, i, j)) return FG_ERR_INDEX;
  *out = f->hm[FG_S][i * f->NY + j] == 0.0f ? 1 : 0;
  return FG_OK;
}

int fg_set_velocity(fg_fluid* f, int i, int j, float u, float v) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  if (!in_grid(f, i, j)) return fail(f, FG_ERR_INDEX, i < 0 || i >= f->NX ? "invalid x-index" : "invalid y-index");
  int cell = i * f->NY + j;
  edit(f, FG_U, cell, 0, u);
  edit(f, FG_V, cell, 0, v);
  return FG_OK;
}

int fg_add_smoke(fg_fluid* f, int i, int j, float smoke) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  if (!in_grid(f, i, j)) return fail(f, FG_ERR_INDEX, i < 0 || i >= f->NX ? "invalid x-index" : "invalid y-index");
  edit(f, FG_M, i * f->NY + j, 1, smoke);
  return FG_OK;
}

int fg_set_velocity_many(fg_fluid* f, int n, const int* is, const int* js, const float* us,
                         const float* vs) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || n < 0 || (n && (!is || !js || !us || !vs))) return FG_ERR_INVALID;
  for (int k = 0; k < n; ++k)
    if (!in_grid(f, is[k], js[k])) return fail(f, FG_ERR_INDEX, "invalid index");
  for (int k = 0; k < n; ++k) {
    int cell = is[k] * f->NY + js[k];
    edit(f, FG_U, cell, 0, us[k]);
    edit(f, FG_V, cell, 0, vs[k]);
  }
  return FG_OK;
}

int fg_add_smoke_many(fg_fluid* f, int n, const int* is, const int* js, const float* ss) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || n < 0 || (n && (!is || !js || !ss))) return FG_ERR_INVALID;
  for (int k = 0; k < n; ++k)
    if (!in_grid(f, is[k], js[k])) return fail(f, FG_ERR_INDEX, "invalid index");
  for (int k = 0; k < n; ++k) edit(f, FG_M, is[k] * f->NY + js[k], 1, ss[k]);
  return FG_OK;
}

int fg_set_sources(fg_fluid* f, int n, const int* is, const int* js, const float* us,
                   const float* vs, const float* smoke, const int* mode) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || n < 0 || (n && (!is || !js || !mode))) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  std::vector<SourceRec> recs;
  for (int k = 0; k < n; ++k) {
    if (!in_grid(f, is[k], js[k])) return fail(f, FG_ERR_INDEX, "invalid source index");
    if (mode[k] & ~15) return fail(f, FG_ERR_INVALID, "unknown source mode bits");
    SourceRec r;
    r.cell = (uint32_t)(is[k] * f->NY + js[k]);
    r.mode = (uint32_t)mode[k];
    r.u = us ? us[k] : 0.0f;
    r.v = vs ? vs[k] : 0.0f;
    r.smoke = smoke ? smoke[k] : 0.0f;
    recs.push_back(r);
  }
  std::stable_sort(recs.begin(), recs.end(),
                   [](const SourceRec& a, const SourceRec& b) { return a.cell < b.cell; });
  std::vector<uint32_t> off;
  if (!recs.empty()) {
    off.push_back(0);
    for (size_t k = 1; k < recs.size(); ++k)
      if (recs[k].cell != recs[k - 1].cell) off.push_back((uint32_t)k);
    off.push_back((uint32_t)recs.size());
  }
  CK(f, cudaStreamSynchronize(f->stream), "sources sync");
  cudaFree(f->src_dev);
  cudaFree(f->src_off_dev);
  f->src_dev = nullptr;
  f->src_off_dev = nullptr;
  f->n_src_groups = 0;
  if (!recs.empty()) {
    CK(f, dev_malloc((void**)&f->src_dev, recs.size() * sizeof(SourceRec)), "sources alloc");
    CK(f, dev_malloc((void**)&f->src_off_dev, off.size() * sizeof(uint32_t)), "sources alloc");
    CK(f, cudaMemcpy(f->src_dev, recs.data(), recs.size() * sizeof(SourceRec),
                     cudaMemcpyHostToDevice), "sources upload");
    CK(f, cudaMemcpy(f->src_off_dev, off.data(), off.size() * sizeof(uint32_t),
                     cudaMemcpyHostToDevice), "sources upload");
    f->n_src_groups = (int)off.size() - 1;
  }
  f->src_smoke = false;
  for (const SourceRec& r : recs) f->src_smoke = f->src_smoke || (r.mode & 12u) != 0;
  f->params_version++;  // the step graph embeds the source list
  return FG_OK;
}

int fg_reset(fg_fluid* f) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  const int fields[] = {FG_U, FG_V, FG_NEWU, FG_NEWV, FG_P, FG_M, FG_NEWM};
  unsigned mask = 0;
  for (int k : fields) mask |= FG_FIELD_BIT(k);
  std::vector<EditRec> keep;
  for (const EditRec& r : f->edits)
    if (!(mask & FG_FIELD_BIT(r.field))) keep.push_back(r);
  f->edits.swap(keep);
  f->dirty &= ~mask;
  size_t hbytes = sizeof(float) * (size_t)f->NX * f->NY;
  for (int k : fields) {
    CK(f, cudaMemsetAsync(f->d[k], 0, field_bytes(f), f->stream), "reset");
    memset(f->hm[k], 0, hbytes);
    f->host_valid[k] = true;
  }
  return FG_OK;
}

int fg_apply_force(fg_fluid* f, int i, int j, float fx, float fy) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  if (i < 1 || i >= f->NX - 1 || j < 1 || j >= f->NY - 1) return FG_OK;  // fluid.go:762-764
  int cell = i * f->NY + j;
  if (f->hm[FG_S][cell] == 0.0f) return FG_OK;
  edit(f, FG_U, cell, 1, fx);
  edit(f, FG_V, cell, 1, fy);
  return FG_OK;
}

int fg_apply_force_radius(fg_fluid* f, int cx, int cy, float fx, float fy, int radius) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  if (radius <= 0) return fg_apply_force(f, cx, cy, fx, fy);
  float r2 = (float)(radius * radius);
  for (int i = cx - radius; i <= cx + radius; ++i)
    for (int j = cy - radius; j <= cy + radius; ++j) {
      if (i < 1 || i >= f->NX - 1 || j < 1 || j >= f->NY - 1) continue;
      float dx = (float)(i - cx), dy = (float)(j - cy);
      float dist2 = dx * dx + dy * dy;
      if (dist2 > r2) continue;
      float weight = (float)std::exp((double)(-3.0f * dist2 / r2));  // fluid.go:792
      fg_apply_force(f, i, j, fx * weight, fy * weight);
    }
  return FG_OK;
}

int fg_set_circular_obstacle(fg_fluid* f, int cx, int cy, int radius) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  for (int i = cx - radius; i <= cx + radius; ++i)
    for (int j = cy - radius; j <= cy + radius; ++j) {
      if (i < 0 || i >= f->NX || j < 0 || j >= f->NY) continue;
      float dx = (float)(i - cx), dy = (float)(j - cy);
      if (dx * dx + dy * dy <= (float)(radius * radius)) fg_set_solid(f, i, j, 1);
    }
  return FG_OK;
}

// ------------------------------------------------------------------ views
static int read_scalars(fg_fluid* f, int n) {
  CK(f, cudaStreamSynchronize(f->stream), "view sync");
  (void)n;
  return FG_OK;
}

static float* dev_scalar_slot(fg_fluid* f) {
  // The last 8 floats of the partials buffer hold small device results; the
  // reductions never reach them (partials_fit).
  return f->partials + (size_t)f->n_partials - 8;
}

int fg_max_divergence(fg_fluid* f, float* out) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  if (!out) return FG_ERR_INVALID;
  float* slot = dev_scalar_slot(f);
  CK(f, launch_max_divergence(f, slot), "maxdiv");
  CK(f, cudaMemcpyAsync(f->scalar_pinned, slot, sizeof(float), cudaMemcpyDeviceToHost, f->stream),
     "maxdiv");
  if ((rc = read_scalars(f, 1))) return rc;
  *out = f->scalar_pinned[0];
  return FG_OK;
}

static int view_common(fg_fluid* f, int kind, float* out_host, float* mn, float* mx) {
  float* slot = dev_scalar_slot(f);
  CK(f, launch_view(f, kind, slot), "view");
  CK(f, cudaMemcpyAsync(f->scalar_pinned, slot, 2 * sizeof(float), cudaMemcpyDeviceToHost,
                        f->stream), "view");
  if (out_host) {
    size_t hp = sizeof(float) * f->NY, dp = sizeof(float) * f->P;
    CK(f, cudaMemcpy2DAsync(out_host, hp, f->view, dp, hp, f->NX, cudaMemcpyDeviceToHost,
                            f->stream), "view");
  }
  int rc = read_scalars(f, 2);
  if (rc) return rc;
  if (mn) *mn = f->scalar_pinned[0];
  if (mx) *mx = f->scalar_pinned[1];
  return FG_OK;
}

int fg_vorticity(fg_fluid* f, float* out_host, float* mn, float* mx) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  return view_common(f, 0, out_host, mn, mx);
}

int fg_velocity_magnitude(fg_fluid* f, float* out_host, float* mn, float* mx) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  return view_common(f, 1, out_host, mn, mx);
}

int fg_field_min_max(fg_fluid* f, int field, float* mn, float* mx) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  if (field < 0 || field >= FG_NUM_FIELDS) return fail(f, FG_ERR_INVALID, "bad field");
  float* slot = dev_scalar_slot(f);
  CK(f, launch_field_minmax(f, field, slot), "minmax");
  CK(f, cudaMemcpyAsync(f->scalar_pinned, slot, 2 * sizeof(float), cudaMemcpyDeviceToHost,
                        f->stream), "minmax");
  if ((rc = read_scalars(f, 2))) return rc;
  if (mn) *mn = f->scalar_pinned[0];
  if (mx) *mx = f->scalar_pinned[1];
  return FG_OK;
}

int fg_sample_velocity(fg_fluid* f, float x, float y, float* u, float* v) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  float* slot = dev_scalar_slot(f);
  CK(f, launch_sample_velocity(f, x, y, slot), "sample");
  CK(f, cudaMemcpyAsync(f->scalar_pinned, slot, 2 * sizeof(float), cudaMemcpyDeviceToHost,
                        f->stream), "sample");
  if ((rc = read_scalars(f, 2))) return rc;
  if (u) *u = f->scalar_pinned[0];
  if (v) *v = f->scalar_pinned[1];
  return FG_OK;
}

int fg_adaptive_time_step(fg_fluid* f, float basedt, float* out) {
  if (is_batch(f)) return batch_unsupported(f);
  STAGE_PROLOGUE(f);
  if (!out) return FG_ERR_INVALID;
  float* slot = dev_scalar_slot(f);
  CK(f, launch_max_speed(f, slot), "max speed");
  CK(f, cudaMemcpyAsync(f->scalar_pinned, slot, sizeof(float), cudaMemcpyDeviceToHost, f->stream),
     "max speed");
  if ((rc = read_scalars(f, 1))) return rc;
  float maxVel = f->scalar_pinned[0];
  if (maxVel == 0.0f) {
    *out = basedt;
    return FG_OK;
  }
  // fluid.go:550-556 in float32 arithmetic with Go's min / max.
  float cflFactor = 0.8f;
  float adaptivedt = cflFactor * f->h / maxVel;
  *out = host_go_max(host_go_min(adaptivedt, basedt * 2.0f), basedt * 0.1f);
  return FG_OK;
}

int fg_profile_enable(fg_fluid* f, int on) {
  if (!f) return FG_ERR_INVALID;
  if (f->profile != (on != 0)) {
    f->profile = on != 0;
    f->params_version++;  // recapture with or without the event nodes
  }
  return FG_OK;
}

int fg_profile_jacobi(fg_fluid* f, float* ms, int* launches) {
  if (!f || !ms || !launches) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  CK(f, cudaStreamSynchronize(f->stream), "profile sync");
  if (!f->profile || f->prof_launches == 0) return fail(f, FG_ERR_INVALID, "no profiled solve");
  CK(f, cudaEventElapsedTime(ms, f->prof_ev[0], f->prof_ev[1]), "profile elapsed");
  *launches = f->prof_launches;
  return FG_OK;
}

int fg_profile_stages(fg_fluid* f, int max, float* ms, const char** names) {
  if (!f || max < 0 || (max && (!ms || !names))) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  CK(f, cudaStreamSynchronize(f->stream), "profile sync");
  int n = 0;
  for (int k = 1; k < f->n_marks && n < max; ++k, ++n) {
    CK(f, cudaEventElapsedTime(&ms[n], f->mark_ev[k - 1], f->mark_ev[k]), "profile elapsed");
    names[n] = f->mark_name[k];
  }
  return n;
}

unsigned long long fg_launch_count(const fg_fluid* f) { return f ? f->launches : 0ull; }

unsigned long long fg_edit_bytes(const fg_fluid* f) { return f ? f->edit_bytes : 0ull; }

const char* fg_last_error(const fg_fluid* f) {
  if (!f) return "invalid handle";
  return f->last_error.c_str();
}

}  // extern "C"

// ===========================================================================
// Differentiable rollouts: the Step / StepAdjoint pair.
//
// fg_tape_begin saves the current state as checkpoint 0; each
// fg_step_forward runs one step with an optional force field and saves a
// checkpoint every `every` steps; fg_tape_seed / fg_tape_seed_smoke_l2 set the
// adjoint of the final state; each fg_step_adjoint reverses the latest step
// not yet reversed.  Reversing a step needs the intermediates of its forward
// pass: the steps of one checkpoint interval are recomputed from their
// checkpoint, recording them (the last interval is recorded during the
// forward pass itself).  The forward pass also keeps each step's pressure
// potential (one field per step), so a recomputed step replays the gradient
// subtract instead of repeating the Jacobi solve.  Memory: one interval of
// records, the checkpoints, the potentials and the forces; the buffers are
// kept for the next rollout until the handle is destroyed.  When the last
// step has been reversed, the handle's state is restored to the end of the
// forward pass.
// ===========================================================================
struct Tape {
  bool active = false;
  int max_steps = 0, every = 0;
  int n_fwd = 0, n_rev = 0;
  int n_ckpt = 0;
  int seg_loaded = -1;  // interval whose steps' records fill the record slots
  bool seeded = false;
  bool final_saved = false;
  uint64_t version = 0;
  std::vector<float> dts;
  std::vector<char> has_force;
  // Capacity of the buffers (steps, record slots, checkpoint slots).
  int cap_steps = 0, cap_every = 0, cap_ckpt = 0;
  float* forces = nullptr;  // cap_steps x {Fu, Fv}
  float* phis = nullptr;    // cap_steps potentials
  float* ckpt = nullptr;    // cap_ckpt x {U, V, M, newU, newV, newM}; slot n_ckpt: the final state
  float* rec = nullptr;     // cap_every x kTapeFields
  float* aux = nullptr;     // loss target
  // CUDA graphs of recorded, replayed and adjoint steps (see run_graphed).
  struct Graph {
    int kind;
    uint32_t dt_bits;
    uint64_t version;
    const void* ptrs[4];
    float* pre[6 + fg_fluid::A_COUNT];
    float* post[6 + fg_fluid::A_COUNT];
    unsigned long long launches;
    cudaGraphExec_t exec;
  };
  std::vector<Graph> graphs;
};

namespace {

constexpr int kStateFields[6] = {FG_U, FG_V, FG_M, FG_NEWU, FG_NEWV, FG_NEWM};

size_t field_elems(const fg_fluid* f) { return (size_t)f->NX * f->P; }

void tape_clear_graphs(Tape* t) {
  for (auto& g : t->graphs) cudaGraphExecDestroy(g.exec);
  t->graphs.clear();
}

void tape_free(fg_fluid* f) {
  if (!f->tape) return;
  cudaStreamSynchronize(f->stream);
  tape_clear_graphs(f->tape);
  cudaFree(f->tape->forces);
  cudaFree(f->tape->phis);
  cudaFree(f->tape->ckpt);
  cudaFree(f->tape->rec);
  cudaFree(f->tape->aux);
  delete f->tape;
  f->tape = nullptr;
}

int tape_supported(fg_fluid* f) {
  const fg_params& p = f->prm;
  if (p.scheme != FG_SCHEME_JACOBI)
    return fail(f, FG_ERR_UNSUPPORTED, "recorded rollouts need the parallel (Jacobi) scheme");
  if (p.early_exit)
    return fail(f, FG_ERR_UNSUPPORTED, "recorded rollouts need a fixed sweep count (early_exit 0)");
  if (p.viscosity_diffusion > 0.0f)
    return fail(f, FG_ERR_UNSUPPORTED, "recorded rollouts do not support viscosity");
  if (p.use_multigrid && p.multigrid_levels > 1)
    return fail(f, FG_ERR_UNSUPPORTED, "recorded rollouts do not support UseMultigrid");
  return FG_OK;
}

int copy_field(fg_fluid* f, float* dst, const float* src) {
  CK(f, cudaMemcpyAsync(dst, src, field_bytes(f), cudaMemcpyDeviceToDevice, f->stream), "copy");
  return FG_OK;
}

int save_state(fg_fluid* f, float* dst) {
  for (int k = 0; k < 6; ++k) {
    int rc = copy_field(f, dst + k * field_elems(f), f->d[kStateFields[k]]);
    if (rc) return rc;
  }
  return FG_OK;
}

int load_state(fg_fluid* f, const float* src) {
  for (int k = 0; k < 6; ++k) {
    int rc = copy_field(f, f->d[kStateFields[k]], src + k * field_elems(f));
    if (rc) return rc;
  }
  return FG_OK;
}

// Copies a field in the Go slice layout (host or device memory) to a
// pitched device field, or back.
bool on_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
int put_field(fg_fluid* f, float* dev, const float* src) {
  if (on_device(src)) {
    CK(f, launch_repitch(f, dev, src, f->P, f->NY), "upload");
    return FG_OK;
  }
  size_t hp = sizeof(float) * f->NY, dp = sizeof(float) * f->P;
  CK(f, cudaMemcpy2DAsync(dev, dp, src, hp, hp, f->NX, cudaMemcpyDefault, f->stream), "upload");
  return FG_OK;
}
int get_field(fg_fluid* f, float* dst, const float* dev) {
  if (on_device(dst)) {
    CK(f, launch_repitch(f, dst, dev, f->NY, f->P), "download");
    return FG_OK;
  }
  size_t hp = sizeof(float) * f->NY, dp = sizeof(float) * f->P;
  CK(f, cudaMemcpy2DAsync(dst, hp, dev, dp, hp, f->NX, cudaMemcpyDefault, f->stream), "download");
  return FG_OK;
}

// One recorded step: Simulate (fluid.go:79-109) with the force field added
// to U, V before the sources (`fu`, `fv` already zero where the sources set
// U, V), confinement / turbulence run as their own pass, and the
// intermediates the adjoint reads written to `rec`
// (kTapeFields fields: U2 V2 U4 V4 fwdU fwdV corrU corrV U5 V5 M1 fwdM
// corrM).  The BFECC
// intermediates are produced in place: the scratch pointers are redirected
// to the record for the step.  The pressure potential is stored to `phi`
// (replay = false) or, on a replay of a step already run, read from it in
// place of the solve; both give the same bits.
int enqueue_step_record(fg_fluid* f, float dt, const float* fu, const float* fv, float* rec,
                        float* phi, bool replay) {
  const fg_params& p = f->prm;
  const size_t n = field_elems(f);
  auto R = [&](int k) { return rec + (size_t)k * n; };
  int rc;
  CK(f, launch_apply_sources(f), "sources");
  // The forces (zero where the sources set U, V) are added by the pressure
  // setup and the gradient kernel as they read U, V: U1 = sources(U0 + F).
  // Without confinement the gradient kernel also applies the turbulence and
  // writes U2 to the record; with it, U2 is copied and confinement and
  // turbulence run as their own pass.
  const bool conf = p.confinement != 0.0f, turb = p.turbulence_strength > 0.0f;
  const bool fuse = turb && !conf;
  f->step_fu = fu;
  f->step_fv = fv;
  if (fuse) {
    f->step_u2 = R(0);
    f->step_v2 = R(1);
  }
  cudaError_t ep = cudaSuccess;
  rc = FG_OK;
  if (replay) {
    ep = launch_grad_replay(f, dt, phi, fuse);
  } else {
    ep = launch_clear_stats(f);
    if (ep == cudaSuccess) rc = enqueue_pressure(f, p.num_iters, dt, fuse);
    if (ep == cudaSuccess && !rc) ep = launch_store_phi(f, phi);
  }
  f->step_fu = f->step_fv = nullptr;
  f->step_u2 = f->step_v2 = nullptr;
  if (rc) return rc;
  if (ep != cudaSuccess) return fail(f, FG_ERR_CUDA, "pressure", ep);
  if (conf) {
    if ((rc = copy_field(f, R(0), f->d[FG_U])) || (rc = copy_field(f, R(1), f->d[FG_V]))) return rc;
    CK(f, launch_confinement_turbulence(f, dt, conf, turb), "confinement/turbulence");
  }
  CK(f, launch_borders(f), "borders");
  if ((rc = copy_field(f, R(2), f->d[FG_U])) || (rc = copy_field(f, R(3), f->d[FG_V]))) return rc;
  float* keep[6] = {f->fwdU, f->fwdV, f->corrU, f->corrV, f->fwdM, f->corrM};
  f->fwdU = R(4);
  f->fwdV = R(5);
  f->corrU = R(6);
  f->corrV = R(7);
  f->fwdM = R(11);
  f->corrM = R(12);
  cudaError_t e = p.use_bfecc ? launch_advect_velocity_bfecc(f, dt) : launch_advect_velocity(f, dt);
  if (e == cudaSuccess) {
    if ((rc = copy_field(f, R(8), f->d[FG_U])) || (rc = copy_field(f, R(9), f->d[FG_V])) ||
        (rc = copy_field(f, R(10), f->d[FG_M]))) {
      e = cudaErrorUnknown;
    } else {
      e = p.use_bfecc ? launch_advect_smoke_bfecc(f, dt) : launch_advect_smoke(f, dt);
    }
  }
  f->fwdU = keep[0];
  f->fwdV = keep[1];
  f->corrU = keep[2];
  f->corrV = keep[3];
  f->fwdM = keep[4];
  f->corrM = keep[5];
  if (e != cudaSuccess) return fail(f, FG_ERR_CUDA, "advection", e);
  return FG_OK;
}

int tape_usable(fg_fluid* f) {
  Tape* t = f->tape;
  if (!t || !t->active) return fail(f, FG_ERR_INVALID, "no recorded rollout (fg_tape_begin)");
  if (t->version != f->params_version)
    return fail(f, FG_ERR_INVALID, "parameters or sources changed during a recorded rollout");
  if (!f->edits.empty() || f->dirty || f->masks_stale)
    return fail(f, FG_ERR_INVALID, "the state was edited during a recorded rollout");
  int rc = bind(f);
  if (rc) return rc;
  return async_guard(f);
}

float* ckpt_at(fg_fluid* f, int k) { return f->tape->ckpt + (size_t)k * 6 * field_elems(f); }
float* rec_at(fg_fluid* f, int k) { return f->tape->rec + (size_t)k * kTapeFields * field_elems(f); }
float* force_at(fg_fluid* f, int t, int c) {
  return f->tape->forces + ((size_t)t * 2 + c) * field_elems(f);
}
float* phi_at(fg_fluid* f, int t) { return f->tape->phis + (size_t)t * field_elems(f); }

// The pointers a captured step bakes in and may rotate: the state and its
// rotation partners, and the adjoint fields.
constexpr int kSnap = 6 + fg_fluid::A_COUNT;
void snap_ptrs(const fg_fluid* f, float** out) {
  out[0] = f->d[FG_U];
  out[1] = f->d[FG_V];
  out[2] = f->d[FG_M];
  out[3] = f->partner[FG_U];
  out[4] = f->partner[FG_V];
  out[5] = f->partner[FG_M];
  for (int k = 0; k < fg_fluid::A_COUNT; ++k) out[6 + k] = f->adj[k];
}
void set_ptrs(fg_fluid* f, float* const* in) {
  f->d[FG_U] = in[0];
  f->d[FG_V] = in[1];
  f->d[FG_M] = in[2];
  f->partner[FG_U] = in[3];
  f->partner[FG_V] = in[4];
  f->partner[FG_M] = in[5];
  for (int k = 0; k < fg_fluid::A_COUNT; ++k) f->adj[k] = in[6 + k];
}

// Runs enqueue() as a CUDA graph: replays the graph captured for the same
// kind, dt, parameters, tape pointers (ptrs) and rotation state, or captures
// a new one.  The tape buffers persist across rollouts, so a training loop
// captures each step once.  Profiling or use_graphs = 0 run it uncaptured.
template <class Fn>
int run_graphed(fg_fluid* f, int kind, float dt, const void* const* ptrs, Fn&& enqueue) {
  Tape* t = f->tape;
  if (!f->prm.use_graphs || f->profile) return enqueue();
  float* pre[kSnap];
  snap_ptrs(f, pre);
  uint32_t dtb;
  memcpy(&dtb, &dt, 4);
  for (auto& g : t->graphs) {
    if (g.kind == kind && g.dt_bits == dtb && g.version == f->params_version &&
        memcmp(g.ptrs, ptrs, sizeof g.ptrs) == 0 && memcmp(g.pre, pre, sizeof pre) == 0) {
      CK(f, cudaGraphLaunch(g.exec, f->stream), "graph launch");
      f->launches += g.launches;
      set_ptrs(f, g.post);
      return FG_OK;
    }
  }
  if (t->graphs.size() >= (size_t)(4 * t->cap_steps + 64)) tape_clear_graphs(t);
  Tape::Graph ent;
  ent.kind = kind;
  ent.dt_bits = dtb;
  ent.version = f->params_version;
  memcpy(ent.ptrs, ptrs, sizeof ent.ptrs);
  memcpy(ent.pre, pre, sizeof pre);
  init_jacobi_tma();  // outside the capture, as for the step graphs
  CK(f, cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  unsigned long long before = f->launches;
  int rc = enqueue();
  ent.launches = f->launches - before;
  f->launches = before;
  cudaGraph_t graph = nullptr;
  cudaError_t ec = cudaStreamEndCapture(f->stream, &graph);
  if (rc || ec != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    set_ptrs(f, pre);  // nothing ran
    return rc ? rc : fail(f, FG_ERR_CUDA, "end capture", ec);
  }
  snap_ptrs(f, ent.post);
  ec = cudaGraphInstantiate(&ent.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (ec != cudaSuccess) {
    set_ptrs(f, pre);
    return fail(f, FG_ERR_CUDA, "graph instantiate", ec);
  }
  t->graphs.push_back(ent);
  CK(f, cudaGraphLaunch(ent.exec, f->stream), "graph launch");
  f->launches += ent.launches;
  return FG_OK;
}

enum { kGraphForward = 1, kGraphReplay = 2, kGraphAdjoint = 3 };

// Recomputes the steps of interval s from its checkpoint, recording them.
int tape_load_interval(fg_fluid* f, int s) {
  Tape* t = f->tape;
  int rc = load_state(f, ckpt_at(f, s));
  if (rc) return rc;
  int t1 = std::min((s + 1) * t->every, t->n_fwd);
  for (int k = s * t->every; k < t1; ++k) {
    bool hf = t->has_force[k] != 0;
    const float* fu = hf ? force_at(f, k, 0) : nullptr;
    const float* fv = hf ? force_at(f, k, 1) : nullptr;
    float* rec = rec_at(f, k - s * t->every);
    float* phi = phi_at(f, k);
    const void* ptrs[4] = {rec, phi, fu, fv};
    rc = run_graphed(f, kGraphReplay, t->dts[k], ptrs, [&] {
      return enqueue_step_record(f, t->dts[k], fu, fv, rec, phi, true);
    });
    if (rc) return rc;
  }
  t->seg_loaded = s;
  return FG_OK;
}

}  // namespace

extern "C" {

int fg_tape_begin(fg_fluid* f, int max_steps, int every) {
  if (!f || max_steps < 1 || every < 1) return FG_ERR_INVALID;
  int rc = flush(f);
  if (rc) return rc;
  if ((rc = tape_supported(f))) return rc;
  if ((rc = check_iters(f, f->prm.num_iters))) return rc;
  for (int k = 0; k < fg_fluid::A_COUNT; ++k)
    if (!f->adj[k] && (rc = alloc_dev(f, &f->adj[k]))) return rc;
  every = std::min(every, max_steps);
  int n_ckpt = (max_steps + every - 1) / every;
  Tape* t = f->tape;
  if (t && (t->cap_steps < max_steps || t->cap_every < every || t->cap_ckpt < n_ckpt + 1)) {
    tape_free(f);
    t = nullptr;
  }
  if (!t) {
    t = new Tape();
    f->tape = t;
    t->cap_steps = max_steps;
    t->cap_every = every;
    t->cap_ckpt = n_ckpt + 1;
    size_t fb = field_bytes(f);
    cudaError_t e;
    if ((e = dev_malloc((void**)&t->forces, fb * 2 * max_steps)) != cudaSuccess ||
        (e = dev_malloc((void**)&t->phis, fb * max_steps)) != cudaSuccess ||
        (e = dev_malloc((void**)&t->ckpt, fb * 6 * t->cap_ckpt)) != cudaSuccess ||
        (e = dev_malloc((void**)&t->rec, fb * kTapeFields * every)) != cudaSuccess ||
        (e = dev_malloc((void**)&t->aux, fb)) != cudaSuccess) {
      tape_free(f);
      return fail(f, FG_ERR_NOMEM, "tape allocation", e);
    }
    // Record fields a step leaves unwritten (U2, V2 without turbulence) and
    // the padding columns stay zero.
    CK(f, cudaMemsetAsync(t->rec, 0, fb * kTapeFields * every, f->stream), "tape");
    CK(f, cudaMemsetAsync(t->aux, 0, fb, f->stream), "tape");
  }
  if (t->version != f->params_version) tape_clear_graphs(t);
  t->active = true;
  t->max_steps = max_steps;
  t->every = every;
  t->n_ckpt = n_ckpt;
  t->n_fwd = t->n_rev = 0;
  t->seg_loaded = -1;
  t->seeded = t->final_saved = false;
  t->version = f->params_version;
  t->dts.assign(max_steps, 0.0f);
  t->has_force.assign(max_steps, 0);
  return save_state(f, ckpt_at(f, 0));
}

int fg_tape_end(fg_fluid* f) {
  if (!f) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  Tape* t = f->tape;
  if (!t || !t->active) return FG_OK;
  if (t->final_saved && t->n_rev < t->n_fwd) {
    // Abandoned mid-reverse: put the end-of-rollout state back.
    if ((rc = load_state(f, ckpt_at(f, t->n_ckpt)))) return rc;
    invalidate(f, kStepFields);
  }
  t->active = false;
  return FG_OK;
}

int fg_step_forward(fg_fluid* f, float dt, const float* force_u, const float* force_v) {
  if (!f) return FG_ERR_INVALID;
  int rc = tape_usable(f);
  if (rc) return rc;
  Tape* t = f->tape;
  if (t->n_rev > 0 || t->seeded)
    return fail(f, FG_ERR_INVALID, "the rollout is being reversed: no further forward steps");
  if (t->n_fwd >= t->max_steps) return fail(f, FG_ERR_INVALID, "rollout longer than max_steps");
  if ((force_u == nullptr) != (force_v == nullptr))
    return fail(f, FG_ERR_INVALID, "give both force components or neither");
  if (f->batch && force_u) return fail(f, FG_ERR_UNSUPPORTED, "batches take no force fields");
  int k = t->n_fwd;
  if (k > 0 && k % t->every == 0 && (rc = save_state(f, ckpt_at(f, k / t->every)))) return rc;
  if (force_u) {
    if ((rc = put_field(f, force_at(f, k, 0), force_u)) ||
        (rc = put_field(f, force_at(f, k, 1), force_v)))
      return rc;
    CK(f, launch_mask_forces(f, force_at(f, k, 0), force_at(f, k, 1)), "forces");
  }
  invalidate(f, kStepFields);
  {
    const float* fu = force_u ? force_at(f, k, 0) : nullptr;
    const float* fv = force_u ? force_at(f, k, 1) : nullptr;
    float* rec = rec_at(f, k % t->every);
    float* phi = phi_at(f, k);
    const void* ptrs[4] = {rec, phi, fu, fv};
    rc = run_graphed(f, kGraphForward, dt, ptrs,
                     [&] { return enqueue_step_record(f, dt, fu, fv, rec, phi, false); });
    if (rc) return rc;
  }
  t->dts[k] = dt;
  t->has_force[k] = force_u ? 1 : 0;
  t->seg_loaded = k / t->every;
  t->n_fwd = k + 1;
  return FG_OK;
}

int fg_tape_seed(fg_fluid* f, const float* dU, const float* dV, const float* dM) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = tape_usable(f);
  if (rc) return rc;
  Tape* t = f->tape;
  if (t->n_fwd == 0 || t->n_rev > 0)
    return fail(f, FG_ERR_INVALID, "seed the adjoint after the forward steps, before reversing");
  const float* src[3] = {dU, dV, dM};
  const int dst[3] = {fg_fluid::A_U, fg_fluid::A_V, fg_fluid::A_M};
  for (int k = 0; k < 3; ++k) {
    CK(f, cudaMemsetAsync(f->adj[dst[k]], 0, field_bytes(f), f->stream), "seed");
    if (src[k] && (rc = put_field(f, f->adj[dst[k]], src[k]))) return rc;
  }
  for (int k : {fg_fluid::A_NU, fg_fluid::A_NV, fg_fluid::A_NM})
    CK(f, cudaMemsetAsync(f->adj[k], 0, field_bytes(f), f->stream), "seed");
  t->seeded = true;
  return FG_OK;
}

int fg_tape_seed_smoke_l2(fg_fluid* f, const float* target, double* loss) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !target) return FG_ERR_INVALID;
  int rc = tape_usable(f);
  if (rc) return rc;
  Tape* t = f->tape;
  if (t->n_fwd == 0 || t->n_rev > 0)
    return fail(f, FG_ERR_INVALID, "seed the adjoint after the forward steps, before reversing");
  if ((rc = put_field(f, t->aux, target))) return rc;
  // An 8-byte aligned double in the scalar slots.
  double* slot = (double*)dev_scalar_slot(f);
  CK(f, launch_loss_seed(f, t->aux, slot), "loss");
  t->seeded = true;
  if (loss) {
    CK(f, cudaMemcpyAsync(f->scalar_pinned, slot, sizeof(double), cudaMemcpyDeviceToHost,
                          f->stream), "loss");
    CK(f, cudaStreamSynchronize(f->stream), "loss sync");
    memcpy(loss, f->scalar_pinned, sizeof(double));
  }
  return FG_OK;
}

int fg_step_adjoint(fg_fluid* f, float* grad_force_u, float* grad_force_v) {
  if (!f) return FG_ERR_INVALID;
  int rc = tape_usable(f);
  if (rc) return rc;
  Tape* t = f->tape;
  if (!t->seeded) return fail(f, FG_ERR_INVALID, "seed the adjoint first (fg_tape_seed)");
  if (f->batch && (grad_force_u || grad_force_v))
    return fail(f, FG_ERR_UNSUPPORTED, "batches take no force fields");
  if (t->n_rev >= t->n_fwd) return fail(f, FG_ERR_INVALID, "every recorded step is reversed");
  if (!t->final_saved) {
    if ((rc = save_state(f, ckpt_at(f, t->n_ckpt)))) return rc;
    t->final_saved = true;
  }
  int k = t->n_fwd - 1 - t->n_rev;
  int s = k / t->every;
  if (t->seg_loaded != s && (rc = tape_load_interval(f, s))) return rc;
  float* rec[kTapeFields];
  for (int q = 0; q < kTapeFields; ++q)
    rec[q] = rec_at(f, k - s * t->every) + (size_t)q * field_elems(f);
  const void* ptrs[4] = {rec[0], nullptr, nullptr, nullptr};
  rc = run_graphed(f, kGraphAdjoint, t->dts[k], ptrs, [&] {
    cudaError_t e = launch_step_adjoint(f, t->dts[k], rec);
    return e == cudaSuccess ? FG_OK : fail(f, FG_ERR_CUDA, "step adjoint", e);
  });
  if (rc) return rc;
  if (grad_force_u && (rc = get_field(f, grad_force_u, f->adj[fg_fluid::A_U]))) return rc;
  if (grad_force_v && (rc = get_field(f, grad_force_v, f->adj[fg_fluid::A_V]))) return rc;
  t->n_rev++;
  if (t->n_rev == t->n_fwd) {
    if ((rc = load_state(f, ckpt_at(f, t->n_ckpt)))) return rc;
    t->seg_loaded = -1;
  }
  invalidate(f, kStepFields);
  return FG_OK;
}

int fg_tape_grad(fg_fluid* f, float* dU, float* dV, float* dM, float* dNU, float* dNV, float* dNM) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  if (!f->tape || !f->tape->active || !f->tape->seeded)
    return fail(f, FG_ERR_INVALID, "no seeded rollout");
  float* out[6] = {dU, dV, dM, dNU, dNV, dNM};
  const int src[6] = {fg_fluid::A_U, fg_fluid::A_V, fg_fluid::A_M,
                      fg_fluid::A_NU, fg_fluid::A_NV, fg_fluid::A_NM};
  for (int k = 0; k < 6; ++k)
    if (out[k] && (rc = get_field(f, out[k], f->adj[src[k]]))) return rc;
  CK(f, cudaStreamSynchronize(f->stream), "grad sync");
  return FG_OK;
}

int fg_tape_steps(const fg_fluid* f, int* forward, int* reversed) {
  if (!f || !forward || !reversed) return FG_ERR_INVALID;
  bool on = f->tape && f->tape->active;
  *forward = on ? f->tape->n_fwd : 0;
  *reversed = on ? f->tape->n_rev : 0;
  return FG_OK;
}

}  // extern "C"

// ===========================================================================
// Batches: many independent scenes of different sizes stepped together.
//
// fg_batch_create packs the state of n scene handles into one handle whose
// fields are the concatenation of the scenes' pitched fields.  Every stage
// then runs as one launch over a block table that names each block's scene
// and tile (a pressure solve runs each scene's own sweep count), so a step
// of the whole batch is a few dozen launches, captured in one CUDA graph by
// fg_simulate like a single scene's.  The batch handle accepts fg_simulate,
// the recorded-rollout calls (without force fields) and the batch calls
// below; entry points that address one scene's cells or mirrors return
// FG_ERR_UNSUPPORTED.  The member handles are not touched until
// fg_batch_scatter copies the batch's state back into them.
// ===========================================================================
namespace {

// Thread-block shapes (x = j, y = i) the autotuner tries for the per-cell
// kernels of a batch.
constexpr int kBatchShapes[5][2] = {{32, 4}, {32, 8}, {32, 16}, {64, 4}, {128, 2}};

void batch_free(fg::BatchGeom* b) {
  if (!b) return;
  cudaFree(b->scenes_dev);
  cudaFree(b->cell_tiles);
  cudaFree(b->cell_blocks);
  cudaFree(b->cell_range);
  cudaFree(b->border_tiles);
  cudaFree(b->jac_tiles);
  cudaFree(b->src_scene);
  cudaFree(b->losses);
  delete b;
}

// Order in which scenes' blocks are laid out: largest first, so the long
// scenes start early and the small ones fill the tail.
std::vector<int> batch_order(const fg::BatchGeom* b) {
  std::vector<int> ord(b->n);
  for (int s = 0; s < b->n; ++s) ord[s] = s;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c) {
    return (long long)b->scenes[a].g.NX * b->scenes[a].g.NY >
           (long long)b->scenes[c].g.NX * b->scenes[c].g.NY;
  });
  return ord;
}

template <class T>
int upload_table(fg_fluid* f, T** dev, const std::vector<T>& host) {
  cudaFree(*dev);
  *dev = nullptr;
  if (host.empty()) return FG_OK;
  CK(f, dev_malloc((void**)dev, host.size() * sizeof(T)), "batch table");
  CK(f, cudaMemcpy(*dev, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice),
     "batch table");
  return FG_OK;
}

// Block table of the per-cell kernels for a bx x by thread-block shape.
int batch_cell_tiles(fg_fluid* f, int bx, int by) {
  fg::BatchGeom* b = f->batch;
  std::vector<BTile> tiles;
  std::vector<BCell> blocks;
  std::vector<int> range(2 * b->n);
  for (int s : batch_order(b)) {
    const Grid& g = b->scenes[s].g;
    range[2 * s] = (int)tiles.size();
    for (int ty = 0; ty < (g.NX + by - 1) / by; ++ty)
      for (int tx = 0; tx < (g.NY + bx - 1) / bx; ++tx) {
        tiles.push_back(BTile{s, tx, ty, 0});
        blocks.push_back(BCell{g, b->scenes[s].off, tx, ty, {0, 0}});
      }
    range[2 * s + 1] = (int)tiles.size();
  }
  CK(f, cudaStreamSynchronize(f->stream), "batch sync");
  int rc = upload_table(f, &b->cell_tiles, tiles);
  if (rc || (rc = upload_table(f, &b->cell_blocks, blocks)) ||
      (rc = upload_table(f, &b->cell_range, range)))
    return rc;
  b->bx = bx;
  b->by = by;
  b->n_cell_tiles = (int)tiles.size();
  return FG_OK;
}

// Copies the members' state, flags and noise into the packed fields.
int batch_pack(fg_fluid* f) {
  fg::BatchGeom* b = f->batch;
  for (int s = 0; s < b->n; ++s) {
    fg_fluid* m = b->members[s];
    int rc = flush(m);
    if (rc) return fail(f, rc, "member flush failed");
    CK(f, cudaStreamSynchronize(m->stream), "member sync");
    long long off = b->scenes[s].off;
    size_t n = (size_t)m->NX * m->P;
    for (int k = 0; k < FG_NUM_FIELDS; ++k)
      CK(f, cudaMemcpyAsync(f->d[k] + off, m->d[k], n * sizeof(float), cudaMemcpyDeviceToDevice,
                            f->stream), "batch pack");
    CK(f, cudaMemcpyAsync(f->flags + off, m->flags, n, cudaMemcpyDeviceToDevice, f->stream),
       "batch pack");
    CK(f, cudaMemcpyAsync(f->noise + off, m->noise, n * sizeof(float2), cudaMemcpyDeviceToDevice,
                          f->stream), "batch pack");
  }
  CK(f, cudaStreamSynchronize(f->stream), "batch pack");
  return FG_OK;
}

int batch_check_member(fg_fluid* f, const fg_fluid* m, const fg_fluid* m0) {
  const fg_params& p = m->prm;
  if (m->batch) return fail(f, FG_ERR_INVALID, "a batch cannot hold a batch");
  if (m->device != m0->device) return fail(f, FG_ERR_INVALID, "batch members on different devices");
  if (p.scheme != FG_SCHEME_JACOBI || p.early_exit || p.refine_sweeps > 0 ||
      p.viscosity_diffusion > 0.0f || (p.use_multigrid && p.multigrid_levels > 1))
    return fail(f, FG_ERR_UNSUPPORTED,
                "batch members need the Jacobi scheme without early exit, refinement, "
                "viscosity or multigrid");
  if (p.num_iters < 1) return fail(f, FG_ERR_INVALID, "batch members need num_iters >= 1");
  fg_params a = p, c = m0->prm;
  a.num_iters = c.num_iters = 0;
  a.tb_depth = c.tb_depth = 0;
  a.use_graphs = c.use_graphs = 0;
  if (memcmp(&a, &c, sizeof a) != 0 || m->density != m0->density || m->h != m0->h)
    return fail(f, FG_ERR_INVALID, "batch members must share parameters except num_iters");
  return FG_OK;
}

}  // namespace

extern "C" {

int fg_batch_create(fg_fluid* const* scenes, int n, fg_fluid** out) {
  if (!scenes || n < 1 || !out) return FG_ERR_INVALID;
  *out = nullptr;
  for (int s = 0; s < n; ++s)
    if (!scenes[s]) return FG_ERR_INVALID;
  fg_fluid* f = new fg_fluid();
  auto bail = [&](int code) {
    std::string msg = f->last_error;
    fg_destroy(f);
    // The reason stays readable on the first member.
    if (!msg.empty()) scenes[0]->last_error = msg;
    return code;
  };
  f->batch = new fg::BatchGeom();
  fg::BatchGeom* b = f->batch;
  b->n = n;
  int rc;
  for (int s = 0; s < n; ++s)
    if ((rc = batch_check_member(f, scenes[s], scenes[0]))) return bail(rc);
  f->device = scenes[0]->device;
  if (cudaSetDevice(f->device) != cudaSuccess) return bail(FG_ERR_CUDA);
  f->prm = scenes[0]->prm;
  f->density = scenes[0]->density;
  f->h = scenes[0]->h;
  // Packed layout: scene s at element offset off_s, each slice a multiple of
  // 32 floats (128 bytes) long.
  long long total = 0;
  for (int s = 0; s < n; ++s) {
    const fg_fluid* m = scenes[s];
    BScene sc;
    sc.g = m->g;
    sc.off = total;
    sc.iters = m->prm.num_iters;
    sc.pad = 0;
    b->scenes.push_back(sc);
    b->members.push_back(scenes[s]);
    b->max_iters = std::max(b->max_iters, m->prm.num_iters);
    total += (long long)m->NX * m->P;
  }
  f->prm.num_iters = b->max_iters;
  f->NX = 1;
  f->NY = (int)std::min<long long>(total, 1 << 30);
  f->P = (int)total;
  if (total >= (1ll << 31)) return bail(fail(f, FG_ERR_INVALID, "batch larger than 2^31 cells"));
  f->g = make_grid(1, f->NY, f->P, f->h);
  if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(FG_ERR_CUDA);
  for (int k = 0; k < 2; ++k) {
    if (cudaEventCreateWithFlags(&f->edit_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return bail(FG_ERR_CUDA);
    if (cudaEventCreate(&f->prof_ev[k]) != cudaSuccess) return bail(FG_ERR_CUDA);
  }
  if (cudaEventCreateWithFlags(&f->mid_ev, cudaEventDisableTiming) != cudaSuccess)
    return bail(FG_ERR_CUDA);
  for (int k = 0; k < fg_fluid::kMaxMarks; ++k)
    if (cudaEventCreate(&f->mark_ev[k]) != cudaSuccess) return bail(FG_ERR_CUDA);
  for (int k = 0; k < FG_NUM_FIELDS; ++k)
    if ((rc = alloc_dev(f, &f->d[k]))) return bail(rc);
  for (int k : {FG_U, FG_V, FG_M})
    if ((rc = alloc_dev(f, &f->partner[k]))) return bail(rc);
  float** scratch[] = {&f->fwdU, &f->fwdV, &f->fwdM, &f->corrU, &f->corrV, &f->corrM,
                       &f->phi,  &f->phi2, &f->rhs,  &f->err,   &f->err2,  &f->rhs_e,
                       &f->curl, &f->view, &f->wgt,  &f->bw,    &f->bwe};
  for (float** sp : scratch)
    if ((rc = alloc_dev(f, sp))) return bail(rc);
  if (dev_malloc((void**)&f->noise, total * sizeof(float2)) != cudaSuccess ||
      dev_malloc((void**)&f->flags, total) != cudaSuccess)
    return bail(fail(f, FG_ERR_NOMEM, "batch allocation"));
  cudaMemsetAsync(f->flags, 0, total, f->stream);
  f->n_slots = kSlots;
  if (dev_malloc(&f->pctl, pctl_bytes(f->n_slots)) != cudaSuccess ||
      dev_malloc(&f->ectl, pctl_bytes(f->n_slots)) != cudaSuccess ||
      dev_malloc((void**)&f->dstats, sizeof(DevStats)) != cudaSuccess ||
      dev_malloc((void**)&b->losses, sizeof(double) * 2 * n) != cudaSuccess)
    return bail(fail(f, FG_ERR_NOMEM, "batch allocation"));
  cudaMemsetAsync(f->pctl, 0, pctl_bytes(f->n_slots), f->stream);
  cudaMemsetAsync(f->ectl, 0, pctl_bytes(f->n_slots), f->stream);
  cudaMemsetAsync(f->dstats, 0, sizeof(DevStats), f->stream);
  if (host_malloc((void**)&f->scalar_pinned, 64 * sizeof(float)) != cudaSuccess ||
      host_malloc((void**)&f->stats_pinned, sizeof(DevStats)) != cudaSuccess)
    return bail(fail(f, FG_ERR_NOMEM, "batch allocation"));
  // Block tables.
  if ((rc = upload_table(f, &b->scenes_dev, b->scenes))) return bail(rc);
  if ((rc = batch_cell_tiles(f, 32, 8))) return bail(rc);
  std::vector<BTile> bt, jt;
  for (int s : batch_order(b)) {
    const Grid& g = b->scenes[s].g;
    for (int t = 0; t < (std::max(g.NX, g.NY) + 127) / 128; ++t) bt.push_back(BTile{s, t, 0, 0});
  }
  // Jacobi regions: scenes with more sweeps first (then larger first), so
  // the scenes that have started by any launch are a prefix of the table.
  std::vector<int> jord = batch_order(b);
  b->jac_iters.clear();
  b->jac_regions.clear();
  std::stable_sort(jord.begin(), jord.end(),
                   [&](int a, int c) { return b->scenes[a].iters > b->scenes[c].iters; });
  for (int s : jord) {
    const Grid& g = b->scenes[s].g;
    b->jac_iters.push_back(b->scenes[s].iters);
    b->jac_regions.push_back(span_count(g.NX, kJacRegionRows) * span_count(g.NY, kJacRegionCols));
    for (int ti = 0; ti < span_count(g.NX, kJacRegionRows); ++ti)
      for (int tj = 0; tj < span_count(g.NY, kJacRegionCols); ++tj)
        jt.push_back(BTile{s, tj * (kJacRegionCols - 2 * kJacHalo),
                           ti * (kJacRegionRows - 2 * kJacHalo),
                           (int)(span_own(ti, g.NX, kJacRegionRows) |
                                 span_own(tj, g.NY, kJacRegionCols) << 16)});
  }
  if ((rc = upload_table(f, &b->border_tiles, bt)) || (rc = upload_table(f, &b->jac_tiles, jt)))
    return bail(rc);
  b->n_border_tiles = (int)bt.size();
  b->n_jac_tiles = (int)jt.size();
  // Partial rows of the per-scene loss: one float pair per cell tile for the
  // block shape with the most tiles, plus the reserve partials_fit keeps.
  long long max_tiles = 0;
  for (const auto& sh : kBatchShapes) {
    long long nt = 0;
    for (const BScene& sc : b->scenes)
      nt += (long long)((sc.g.NX + sh[1] - 1) / sh[1]) * ((sc.g.NY + sh[0] - 1) / sh[0]);
    max_tiles = std::max(max_tiles, nt);
  }
  f->n_partials = (int)(2 * (max_tiles + max_tiles / 2048 + 2) + 512);
  if (dev_malloc((void**)&f->partials, sizeof(float) * f->n_partials) != cudaSuccess)
    return bail(fail(f, FG_ERR_NOMEM, "batch allocation"));
  // Sources: the members' groups, each tagged with its scene.
  std::vector<SourceRec> recs;
  std::vector<uint32_t> off;
  std::vector<int> gscene;
  for (int s = 0; s < n; ++s) {
    const fg_fluid* m = scenes[s];
    if (m->n_src_groups <= 0) continue;
    std::vector<uint32_t> moff(m->n_src_groups + 1);
    if (cudaMemcpy(moff.data(), m->src_off_dev, moff.size() * sizeof(uint32_t),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
      return bail(FG_ERR_CUDA);
    std::vector<SourceRec> mr(moff.back());
    if (cudaMemcpy(mr.data(), m->src_dev, mr.size() * sizeof(SourceRec),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
      return bail(FG_ERR_CUDA);
    for (int k = 0; k < m->n_src_groups; ++k) {
      off.push_back((uint32_t)recs.size());
      for (uint32_t q = moff[k]; q < moff[k + 1]; ++q) recs.push_back(mr[q]);
      gscene.push_back(s);
    }
  }
  if (!recs.empty()) {
    off.push_back((uint32_t)recs.size());
    if ((rc = upload_table(f, &f->src_dev, recs)) || (rc = upload_table(f, &f->src_off_dev, off)) ||
        (rc = upload_table(f, &b->src_scene, gscene)))
      return bail(rc);
    f->n_src_groups = (int)gscene.size();
  }
  if ((rc = batch_pack(f))) return bail(rc);
  f->masks_stale = false;
  *out = f;
  return FG_OK;
}

int fg_batch_step(fg_fluid* f, float dt) {
  if (!f || !f->batch) return FG_ERR_INVALID;
  return fg_simulate(f, dt);
}

int fg_batch_step_adjoint(fg_fluid* f) {
  if (!f || !f->batch) return FG_ERR_INVALID;
  return fg_step_adjoint(f, nullptr, nullptr);
}

int fg_batch_size(const fg_fluid* f, int* n) {
  if (!f || !f->batch || !n) return FG_ERR_INVALID;
  *n = f->batch->n;
  return FG_OK;
}

int fg_batch_gather(fg_fluid* f) {
  if (!f || !f->batch) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  if (f->tape && f->tape->active) return fail(f, FG_ERR_INVALID, "a recorded rollout is open");
  return batch_pack(f);
}

int fg_batch_scatter(fg_fluid* f) {
  if (!f || !f->batch) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  const fg::BatchGeom* b = f->batch;
  CK(f, cudaStreamSynchronize(f->stream), "batch sync");
  for (int s = 0; s < b->n; ++s) {
    fg_fluid* m = b->members[s];
    size_t n = (size_t)m->NX * m->P;
    for (int k = 0; k < FG_NUM_FIELDS; ++k) {
      if (k == FG_S) continue;
      CK(f, cudaMemcpyAsync(m->d[k], f->d[k] + b->scenes[s].off, n * sizeof(float),
                            cudaMemcpyDeviceToDevice, f->stream), "batch scatter");
    }
    invalidate(m, kStepFields);
  }
  CK(f, cudaStreamSynchronize(f->stream), "batch scatter");
  return FG_OK;
}

// Seeds a batch's rollout with L_s = ||M_s - target_s||_2 for every scene
// (targets[s]: the scene's NumX * NumY values, host or device memory).
int fg_batch_seed_smoke_l2(fg_fluid* f, const float* const* targets, double* losses) {
  if (!f || !f->batch || !targets) return FG_ERR_INVALID;
  int rc = tape_usable(f);
  if (rc) return rc;
  Tape* t = f->tape;
  if (t->n_fwd == 0 || t->n_rev > 0)
    return fail(f, FG_ERR_INVALID, "seed the adjoint after the forward steps, before reversing");
  const fg::BatchGeom* b = f->batch;
  CK(f, cudaMemsetAsync(t->aux, 0, field_bytes(f), f->stream), "seed");
  for (int s = 0; s < b->n; ++s) {
    if (!targets[s]) return fail(f, FG_ERR_INVALID, "missing target");
    const Grid& g = b->scenes[s].g;
    size_t hp = sizeof(float) * g.NY, dp = sizeof(float) * g.P;
    CK(f, cudaMemcpy2DAsync(t->aux + b->scenes[s].off, dp, targets[s], hp, hp, g.NX,
                            cudaMemcpyDefault, f->stream), "target upload");
  }
  CK(f, launch_loss_seed(f, t->aux, nullptr), "loss");
  t->seeded = true;
  if (losses) {
    CK(f, cudaMemcpyAsync(losses, b->losses, sizeof(double) * b->n, cudaMemcpyDefault, f->stream),
       "losses");
    CK(f, cudaStreamSynchronize(f->stream), "losses");
  }
  return FG_OK;
}

// dL/d(initial U, V, M) of scene s after a batch's reverse pass (the
// scene's NumX * NumY layout; NULL: skipped).
int fg_batch_grad(fg_fluid* f, int s, float* dU, float* dV, float* dM) {
  if (!f || !f->batch || s < 0 || s >= f->batch->n) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  if (!f->tape || !f->tape->active || !f->tape->seeded)
    return fail(f, FG_ERR_INVALID, "no seeded rollout");
  const BScene& sc = f->batch->scenes[s];
  float* out[3] = {dU, dV, dM};
  const int src[3] = {fg_fluid::A_U, fg_fluid::A_V, fg_fluid::A_M};
  size_t hp = sizeof(float) * sc.g.NY, dp = sizeof(float) * sc.g.P;
  for (int k = 0; k < 3; ++k)
    if (out[k])
      CK(f, cudaMemcpy2DAsync(out[k], hp, f->adj[src[k]] + sc.off, dp, hp, sc.g.NX,
                              cudaMemcpyDefault, f->stream), "grad");
  CK(f, cudaStreamSynchronize(f->stream), "grad sync");
  return FG_OK;
}

// Picks the per-cell thread-block shape and the Jacobi sweeps per launch
// that step this batch fastest: each candidate runs `reps` timed steps
// (after one untimed step that also captures its graph) from the same
// saved state, which is restored afterwards.  Neither choice changes any
// result bit.
int fg_batch_autotune(fg_fluid* f, float dt, int reps, int* tb_depth, int* block_x, int* block_y,
                      float* ms_per_step) {
  if (!f || !f->batch || reps < 1) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  if (f->tape && f->tape->active) return fail(f, FG_ERR_INVALID, "a recorded rollout is open");
  const auto& shapes = kBatchShapes;
  static const int depths[] = {4, 6, 8};
  size_t fb = field_bytes(f);
  float* saved = nullptr;
  CK(f, dev_malloc((void**)&saved, fb * 7), "autotune");
  auto save = [&]() {
    int r = save_state(f, saved);
    if (!r) r = copy_field(f, saved + 6 * field_elems(f), f->d[FG_P]);
    return r;
  };
  auto restore = [&]() {
    int r = load_state(f, saved);
    if (!r) r = copy_field(f, f->d[FG_P], saved + 6 * field_elems(f));
    return r;
  };
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bb = 0, bd = 0;
  rc = save();
  for (int si = 0; !rc && si < (int)(sizeof shapes / sizeof shapes[0]); ++si) {
    if ((rc = batch_cell_tiles(f, shapes[si][0], shapes[si][1]))) break;
    for (int di = 0; !rc && di < (int)(sizeof depths / sizeof depths[0]); ++di) {
      f->prm.tb_depth = depths[di];
      f->params_version++;
      clear_graphs(f);
      if ((rc = fg_simulate(f, dt))) break;
      cudaEventRecord(e0, f->stream);
      for (int r = 0; r < reps && !rc; ++r) rc = fg_simulate(f, dt);
      cudaEventRecord(e1, f->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(f, FG_ERR_CUDA, "autotune");
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      ms /= (float)reps;
      if (!rc && ms < best) {
        best = ms;
        bb = si;
        bd = di;
      }
      if (!rc) rc = restore();
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!rc) rc = batch_cell_tiles(f, shapes[bb][0], shapes[bb][1]);
  f->prm.tb_depth = depths[bd];
  f->params_version++;
  clear_graphs(f);
  cudaStreamSynchronize(f->stream);
  cudaFree(saved);
  if (rc) return rc;
  if (tb_depth) *tb_depth = depths[bd];
  if (block_x) *block_x = shapes[bb][0];
  if (block_y) *block_y = shapes[bb][1];
  if (ms_per_step) *ms_per_step = best;
  return FG_OK;
}

}  // extern "C"

// ===========================================================================
// Tracer particles (main/main.go:489-546) and rendering (main/main.go:619-650,
// main/colors.go:10-84).
// ===========================================================================
namespace {

constexpr int kParticleBlock = 1024;

int particles_read_count(fg_fluid* f, int* out) {
  auto& P = f->parts;
  if (!P.count) {
    *out = 0;
    return FG_OK;
  }
  CK(f, cudaMemcpyAsync(f->scalar_pinned, P.count, sizeof(int), cudaMemcpyDeviceToHost,
                        f->stream), "particle count");
  CK(f, cudaStreamSynchronize(f->stream), "particle count");
  memcpy(out, f->scalar_pinned, sizeof(int));
  P.n_upper = *out;
  return FG_OK;
}

// Grows the particle buffers to hold `need` particles, keeping the first n.
int particles_reserve(fg_fluid* f, int need, int n) {
  auto& P = f->parts;
  if (need <= P.cap && P.count) return FG_OK;
  int cap = std::max(need, std::max(2 * P.cap, kParticleBlock));
  cap = (cap + kParticleBlock - 1) / kParticleBlock * kParticleBlock;
  fg_fluid::Particles Q;
  Q.cap = cap;
  Q.cur = 0;
  Q.n_upper = P.n_upper;
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    for (int q = 0; q < 4 && e == cudaSuccess; ++q)
      e = dev_malloc((void**)&Q.a[b][q], sizeof(float) * cap);
    if (e == cudaSuccess) e = dev_malloc((void**)&Q.rgb[b], sizeof(uint32_t) * cap);
  }
  if (e == cudaSuccess) e = dev_malloc((void**)&Q.keep, cap);
  if (e == cudaSuccess) e = dev_malloc((void**)&Q.block_keep, sizeof(int) * (cap / kParticleBlock));
  if (e == cudaSuccess && !P.count) {
    e = dev_malloc((void**)&Q.count, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(Q.count, 0, sizeof(int), f->stream);
  } else {
    Q.count = P.count;
  }
  if (e == cudaSuccess) e = cudaMemsetAsync(Q.keep, 0, cap, f->stream);
  for (int q = 0; q < 4 && e == cudaSuccess && n > 0; ++q)
    e = cudaMemcpyAsync(Q.a[0][q], P.a[P.cur][q], sizeof(float) * n, cudaMemcpyDeviceToDevice,
                        f->stream);
  if (e == cudaSuccess && n > 0)
    e = cudaMemcpyAsync(Q.rgb[0], P.rgb[P.cur], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice,
                        f->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
  if (e != cudaSuccess) {
    for (int b = 0; b < 2; ++b) {
      for (int q = 0; q < 4; ++q) cudaFree(Q.a[b][q]);
      cudaFree(Q.rgb[b]);
    }
    cudaFree(Q.keep);
    cudaFree(Q.block_keep);
    if (Q.count != P.count) cudaFree(Q.count);
    return fail(f, FG_ERR_NOMEM, "particle buffers", e);
  }
  for (int b = 0; b < 2; ++b) {
    for (int q = 0; q < 4; ++q) cudaFree(P.a[b][q]);
    cudaFree(P.rgb[b]);
  }
  cudaFree(P.keep);
  cudaFree(P.block_keep);
  P = Q;
  return FG_OK;
}

}  // namespace

extern "C" {

int fg_particles_add(fg_fluid* f, int n, const float* x, const float* y, const float* max_age,
                     const unsigned char* rgb, int max_total) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || n < 0 || (n && (!x || !y || !max_age || !rgb))) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  int have = 0;
  if ((rc = particles_read_count(f, &have))) return rc;
  if (max_total > 0) n = std::max(0, std::min(n, max_total - have));
  if (n == 0) return FG_OK;
  if ((rc = particles_reserve(f, have + n, have))) return rc;
  auto& P = f->parts;
  std::vector<float> age(n, 0.0f);
  std::vector<uint32_t> packed(n);
  for (int k = 0; k < n; ++k)
    packed[k] = (uint32_t)rgb[3 * k] | ((uint32_t)rgb[3 * k + 1] << 8) |
                ((uint32_t)rgb[3 * k + 2] << 16);
  const float* src[4] = {x, y, age.data(), max_age};
  for (int q = 0; q < 4; ++q)
    CK(f, cudaMemcpyAsync(P.a[P.cur][q] + have, src[q], sizeof(float) * n, cudaMemcpyDefault,
                          f->stream), "particle upload");
  CK(f, cudaMemcpyAsync(P.rgb[P.cur] + have, packed.data(), sizeof(uint32_t) * n,
                        cudaMemcpyHostToDevice, f->stream), "particle upload");
  int total = have + n;
  CK(f, cudaMemcpyAsync(P.count, &total, sizeof(int), cudaMemcpyHostToDevice, f->stream),
     "particle count");
  CK(f, cudaStreamSynchronize(f->stream), "particle upload");
  P.n_upper = total;
  return FG_OK;
}

int fg_particles_advect(fg_fluid* f, float dt) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = flush(f);
  if (rc) return rc;
  auto& P = f->parts;
  if (!P.count || P.n_upper == 0) return FG_OK;
  const int o = P.cur ^ 1;
  const float* in[4] = {P.a[P.cur][0], P.a[P.cur][1], P.a[P.cur][2], P.a[P.cur][3]};
  float* out[4] = {P.a[o][0], P.a[o][1], P.a[o][2], P.a[o][3]};
  CK(f, launch_particles_advect(f, dt, P.n_upper, in, P.rgb[P.cur], out, P.rgb[o], P.count,
                                P.keep, P.block_keep), "particles");
  P.cur = o;
  return FG_OK;
}

int fg_particles_count(fg_fluid* f, int* n) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !n) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  return particles_read_count(f, n);
}

int fg_particles_get(fg_fluid* f, float* x, float* y, float* age, float* max_age,
                     unsigned char* rgb) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  int n = 0;
  if ((rc = particles_read_count(f, &n))) return rc;
  if (n == 0) return FG_OK;
  auto& P = f->parts;
  float* dst[4] = {x, y, age, max_age};
  for (int q = 0; q < 4; ++q)
    if (dst[q])
      CK(f, cudaMemcpyAsync(dst[q], P.a[P.cur][q], sizeof(float) * n, cudaMemcpyDefault,
                            f->stream), "particle download");
  std::vector<uint32_t> packed(rgb ? n : 0);
  if (rgb)
    CK(f, cudaMemcpyAsync(packed.data(), P.rgb[P.cur], sizeof(uint32_t) * n,
                          cudaMemcpyDeviceToHost, f->stream), "particle download");
  CK(f, cudaStreamSynchronize(f->stream), "particle download");
  for (int k = 0; rgb && k < n; ++k) {
    rgb[3 * k] = (unsigned char)(packed[k] & 0xff);
    rgb[3 * k + 1] = (unsigned char)((packed[k] >> 8) & 0xff);
    rgb[3 * k + 2] = (unsigned char)((packed[k] >> 16) & 0xff);
  }
  return FG_OK;
}

int fg_particles_clear(fg_fluid* f) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f) return FG_ERR_INVALID;
  int rc = bind(f);
  if (rc) return rc;
  if (f->parts.count)
    CK(f, cudaMemsetAsync(f->parts.count, 0, sizeof(int), f->stream), "particles");
  f->parts.n_upper = 0;
  return FG_OK;
}

int fg_render(fg_fluid* f, int kind, void* rgba) {
  if (is_batch(f)) return batch_unsupported(f);
  if (!f || !rgba || kind < FG_RENDER_SMOKE || kind > FG_RENDER_VORTICITY) return FG_ERR_INVALID;
  int rc = flush(f);
  if (rc) return rc;
  size_t bytes = (size_t)f->NX * f->NY * 4;
  if (!f->image) CK(f, dev_malloc((void**)&f->image, bytes), "render target");
  float* mm = dev_scalar_slot(f);
  const float* field = nullptr;
  if (kind == FG_RENDER_SMOKE || kind == FG_RENDER_PRESSURE) {
    int fld = kind == FG_RENDER_SMOKE ? FG_M : FG_P;
    CK(f, launch_field_minmax(f, fld, mm), "render");
    field = f->d[fld];
  } else {
    CK(f, launch_view(f, kind == FG_RENDER_VORTICITY ? 0 : 1, mm), "render");
    field = f->view;
  }
  CK(f, launch_render(f, field, mm, kind == FG_RENDER_VORTICITY ? 1 : 0, f->image), "render");
  // Pageable host memory (an app's image buffer) gets the frame through a
  // pinned staging copy: the device copy into pageable memory runs at a
  // fraction of the link's rate.
  cudaPointerAttributes pa{};
  const bool pageable = cudaPointerGetAttributes(&pa, rgba) == cudaSuccess
                            ? pa.type == cudaMemoryTypeUnregistered
                            : (cudaGetLastError(), true);
  if (pageable && !f->image_pinned &&
      host_malloc((void**)&f->image_pinned, bytes) != cudaSuccess) {
    f->image_pinned = nullptr;
    cudaGetLastError();
  }
  if (pageable && f->image_pinned) {
    CK(f, cudaMemcpyAsync(f->image_pinned, f->image, bytes, cudaMemcpyDeviceToHost, f->stream),
       "render");
    CK(f, cudaStreamSynchronize(f->stream), "render");
    memcpy(rgba, f->image_pinned, bytes);
    return FG_OK;
  }
  CK(f, cudaMemcpyAsync(rgba, f->image, bytes, cudaMemcpyDefault, f->stream), "render");
  CK(f, cudaStreamSynchronize(f->stream), "render");
  return FG_OK;
}

}  // extern "C"


// ------------------------------------------------------------ fault injection
int fg_debug_fail_alloc(int n) {
  g_alloc_fail_in.store(n < 0 ? -1 : n);
  return FG_OK;
}

int fg_debug_stall_tile(fg_fluid* f, int tile) {
  if (!f) {  // the allocation-free projection's TMA-fed Jacobi launches
    set_noalloc_stall(tile);
    return FG_OK;
  }
  if (is_batch(f)) return batch_unsupported(f);
  int rc = flush(f);
  if (rc) return rc;
  f->stall_tile = tile < 0 ? -1 : tile;
  f->params_version++;  // captured steps embed the kernel's arguments
  return FG_OK;
}
