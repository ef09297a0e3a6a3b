// Mask build, tool-edit application, viscosity, vorticity confinement,
// turbulence and border kernels.
//
// Each kernel restates one stage of pkg/fluid/fluid.go with the same float32
// operation order (the file is compiled with -fmad=false), so the results
// match the reference arithmetic bit for bit.
#include <cmath>

#include "fg_batch.cuh"
#include "fg_internal.cuh"

namespace fg {
namespace {

constexpr int BX = 32, BY = 8;  // j (contiguous) along x of the block

inline dim3 cell_grid(const fg_fluid* f) {
  return dim3((f->NY + BX - 1) / BX, (f->NX + BY - 1) / BY);
}

// Flag byte per cell from S (S is validated to hold only 0 and 1).
__global__ void k_build_flags(const float* __restrict__ S, uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  int c = i * g.P + j;
  uint8_t fl = 0;
  if (S[c] != 0.0f) fl |= F_FLUID;
  if (i > 0 && S[c - g.P] != 0.0f) fl |= F_W;
  if (i < g.NX - 1 && S[c + g.P] != 0.0f) fl |= F_E;
  if (j > 0 && S[c - 1] != 0.0f) fl |= F_S;
  if (j < g.NY - 1 && S[c + 1] != 0.0f) fl |= F_N;
  if (i >= 1 && i <= g.NX - 2 && j >= 1 && j <= g.NY - 2) fl |= F_INTERIOR;
  flags[c] = fl;
}

// Queued tool edits, grouped by (field, cell) in call order: one thread per
// group applies its set / add operations sequentially.  recs and off are the
// host's pinned edit log, read across the host link (no upload).
struct FieldPtrs {
  float* p[FG_NUM_FIELDS];
};
__global__ void k_apply_edits(const EditRec* __restrict__ recs, const uint32_t* __restrict__ off,
                              int n_groups, FieldPtrs fp, Grid g) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_groups) return;
  uint32_t b = off[k], e = off[k + 1];
  EditRec r0 = recs[b];
  int i = (int)(r0.cell / (uint32_t)g.NY);
  int j = (int)(r0.cell % (uint32_t)g.NY);
  float* ptr = fp.p[r0.field] + (size_t)i * g.P + j;
  float v = *ptr;
  for (uint32_t q = b; q < e; ++q) {
    EditRec r = recs[q];
    if (r.op == 0)
      v = r.value;
    else
      v = v + r.value;
  }
  *ptr = v;
}

// Persistent sources: per cell group, in list order, the app's
// SetVelocity(i, j, u, v) and AddSmoke(i, j, s) calls made before each step
// (main/main.go:236-241 jet, 474-486 sources) or a smoke assignment
// (fluid_test.go:396-401), optionally skipped on solid cells (the IsSolid
// check of applySources).
__device__ __forceinline__ void apply_sources_group(const SourceRec* __restrict__ recs,
                                                    uint32_t b, uint32_t e, float* U, float* V,
                                                    float* M, const uint8_t* __restrict__ flags,
                                                    const Grid& g) {
  uint32_t cell = recs[b].cell;
  int i = (int)(cell / (uint32_t)g.NY), j = (int)(cell % (uint32_t)g.NY);
  int c = i * g.P + j;
  bool fluid = (flags[c] & F_FLUID) != 0;
  float u = U[c], v = V[c], m = M[c];
  for (uint32_t q = b; q < e; ++q) {
    SourceRec r = recs[q];
    if ((r.mode & 1u) && !fluid) continue;
    if (r.mode & 2u) {
      u = r.u;
      v = r.v;
    }
    if (r.mode & 8u)
      m = r.smoke;
    else if (r.mode & 4u)
      m = m + r.smoke;
  }
  U[c] = u;
  V[c] = v;
  M[c] = m;
}

__global__ void k_apply_sources(const SourceRec* __restrict__ recs,
                                const uint32_t* __restrict__ off, int n_groups, float* U,
                                float* V, float* M, const uint8_t* __restrict__ flags, Grid g) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_groups) return;
  apply_sources_group(recs, off[k], off[k + 1], U, V, M, flags, g);
}

// A batch's sources: group k belongs to scene gs[k].
__global__ void kb_apply_sources(const SourceRec* __restrict__ recs,
                                 const uint32_t* __restrict__ off, const int* __restrict__ gs,
                                 int n_groups, float* U, float* V, float* M,
                                 const uint8_t* __restrict__ flags,
                                 const BScene* __restrict__ sc) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_groups) return;
  const BScene& s = sc[gs[k]];
  apply_sources_group(recs, off[k], off[k + 1], U + s.off, V + s.off, M + s.off, flags + s.off,
                      s.g);
}

// applyViscosity (fluid.go:112-142): out = U + visc*lap(U) on fluid interior
// cells, U elsewhere; newU takes the same values (copy(f.newU, f.U) then the
// update then copy(f.U, f.newU)).
__global__ void k_viscosity(const float* __restrict__ U, const float* __restrict__ V,
                            float* __restrict__ Uo, float* __restrict__ Vo,
                            float* __restrict__ nU, float* __restrict__ nV,
                            const uint8_t* __restrict__ flags, float visc, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  int c = i * g.P + j;
  float u = U[c], v = V[c];
  uint8_t fl = flags[c];
  if ((fl & (F_INTERIOR | F_FLUID)) == (F_INTERIOR | F_FLUID)) {
    float uLap = U[c - g.P] + U[c + g.P] + U[c - 1] + U[c + 1] - 4.0f * u;
    float vLap = V[c - g.P] + V[c + g.P] + V[c - 1] + V[c + 1] - 4.0f * v;
    u = u + visc * uLap;
    v = v + visc * vLap;
  }
  Uo[c] = u;
  Vo[c] = v;
  nU[c] = u;
  nV[c] = v;
}

// Curl pass of applyVorticityConfinement (fluid.go:455-466); zero on cells
// the reference leaves at the fresh array's zero.
__device__ __forceinline__ void curl_cell(int i, int j, const float* __restrict__ U,
                                          const float* __restrict__ V, float* __restrict__ curl,
                                          const uint8_t* __restrict__ flags, const Grid& g) {
  int c = i * g.P + j;
  float w = 0.0f;
  uint8_t fl = flags[c];
  if ((fl & (F_INTERIOR | F_FLUID)) == (F_INTERIOR | F_FLUID)) {
    float dvdx = (V[c + g.P] - V[c - g.P]) * 0.5f / g.h;
    float dudy = (U[c + 1] - U[c - 1]) * 0.5f / g.h;
    w = dvdx - dudy;
  }
  curl[c] = w;
}
__global__ void k_curl(const float* __restrict__ U, const float* __restrict__ V,
                       float* __restrict__ curl, const uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  curl_cell(i, j, U, V, curl, flags, g);
}

// Force pass of applyVorticityConfinement (fluid.go:468-492) followed by
// addTurbulence (fluid.go:496-526).  Both touch only the cell's own U, V, so
// running them per cell in that order equals the reference's two loops.
__device__ __forceinline__ void conf_turb_cell(int i, int j, float* __restrict__ U,
                                               float* __restrict__ V,
                                               const float* __restrict__ curl,
                                               const float2* __restrict__ noise,
                                               const uint8_t* __restrict__ flags, float conf,
                                               float dt, float turbStrength, int do_conf,
                                               int do_turb, const Grid& g) {
  int c = i * g.P + j;
  uint8_t fl = flags[c];
  if ((fl & (F_INTERIOR | F_FLUID)) != (F_INTERIOR | F_FLUID)) return;
  float u = U[c], v = V[c];
  if (do_conf) {
    const float eps = 1e-5f;
    float gx = (fabsf(curl[c + g.P]) - fabsf(curl[c - g.P])) * 0.5f / g.h;
    float gy = (fabsf(curl[c + 1]) - fabsf(curl[c - 1])) * 0.5f / g.h;
    float mag = sqrtf(gx * gx + gy * gy) + eps;
    gx /= mag;
    gy /= mag;
    float vort = curl[c];
    float localVel = sqrtf(u * u + v * v);
    float adaptiveStrength = conf * (1.0f + localVel * 0.1f);
    u += adaptiveStrength * gy * vort * dt;
    v -= adaptiveStrength * gx * vort * dt;
  }
  if (do_turb) {
    float2 nz = noise[c];
    float noiseU = nz.x * turbStrength;
    float noiseV = nz.y * turbStrength;
    float localVel = sqrtf(u * u + v * v);
    if (localVel > 0.1f) {
      float turbulenceFactor = go_min(localVel * 0.5f, 1.0f);
      u += noiseU * turbulenceFactor;
      v += noiseV * turbulenceFactor;
    }
  }
  U[c] = u;
  V[c] = v;
}
__global__ void k_conf_turb(float* __restrict__ U, float* __restrict__ V,
                            const float* __restrict__ curl, const float2* __restrict__ noise,
                            const uint8_t* __restrict__ flags, float conf, float dt,
                            float turbStrength, int do_conf, int do_turb, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  conf_turb_cell(i, j, U, V, curl, noise, flags, conf, dt, turbStrength, do_conf, do_turb, g);
}

// handleBorders (fluid.go:236-289): thread t does the ghost rows j = 0 and
// j = NY-1 of U for i = t, and the ghost columns i = 0 and i = NX-1 of V for
// j = t.  The two loops touch disjoint data.
__device__ __forceinline__ void borders_border(int t, float* __restrict__ U, float* __restrict__ V,
                                               const uint8_t* __restrict__ flags, const Grid& g) {
  const int P = g.P, NX = g.NX, NY = g.NY;
  auto fluid = [&](int i, int j) { return (flags[i * P + j] & F_FLUID) != 0; };
  if (t < NX) {
    int i = t;
    float* u = U + (size_t)i * P;
    if (!fluid(i, 0) || !fluid(i, 1)) {
      u[0] = 0.0f;
    } else if (i > 0 && i < NX - 1 && fluid(i, 2)) {
      u[0] = 2.0f * u[1] - u[2];
    } else {
      u[0] = u[1];
    }
    if (!fluid(i, NY - 1) || !fluid(i, NY - 2)) {
      u[NY - 1] = 0.0f;
    } else if (i > 0 && i < NX - 1 && fluid(i, NY - 3)) {
      u[NY - 1] = 2.0f * u[NY - 2] - u[NY - 3];
    } else {
      u[NY - 1] = u[NY - 2];
    }
  }
  if (t < NY) {
    int j = t;
    if (!fluid(0, j) || !fluid(1, j)) {
      V[j] = 0.0f;
    } else if (j > 0 && j < NY - 1 && fluid(2, j)) {
      V[j] = 2.0f * V[P + j] - V[2 * P + j];
    } else {
      V[j] = V[P + j];
    }
    int a = (NX - 1) * P + j, b = (NX - 2) * P + j, cc = (NX - 3) * P + j;
    if (!fluid(NX - 1, j) || !fluid(NX - 2, j)) {
      V[a] = 0.0f;
    } else if (j > 0 && j < NY - 1 && fluid(NX - 3, j)) {
      V[a] = 2.0f * V[b] - V[cc];
    } else {
      V[a] = V[b];
    }
  }
}
__global__ void k_borders(float* __restrict__ U, float* __restrict__ V,
                          const uint8_t* __restrict__ flags, Grid g) {
  pdl_enter();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  borders_border(t, U, V, flags, g);
}

// copyBorder (fluid.go:436-446).
__global__ void k_copy_border(float* __restrict__ dst, const float* __restrict__ src, Grid g) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < g.NX) {
    dst[t * g.P] = src[t * g.P];
    dst[t * g.P + g.NY - 1] = src[t * g.P + g.NY - 1];
  }
  if (t < g.NY) {
    dst[t] = src[t];
    dst[(g.NX - 1) * g.P + t] = src[(g.NX - 1) * g.P + t];
  }
}

}  // namespace

cudaError_t launch_build_flags_on(cudaStream_t st, const float* S, uint8_t* flags, const Grid& g) {
  k_build_flags<<<dim3((g.NY + BX - 1) / BX, (g.NX + BY - 1) / BY), dim3(BX, BY), 0, st>>>(S, flags,
                                                                                       g);
  return cudaGetLastError();
}

cudaError_t launch_build_flags(fg_fluid* f) {
  count(f);
  k_build_flags<<<cell_grid(f), dim3(BX, BY), 0, f->stream>>>(f->d[FG_S], f->flags, f->g);
  return cudaGetLastError();
}

cudaError_t launch_apply_edits(fg_fluid* f, int n_groups, int slot) {
  if (n_groups <= 0) return cudaSuccess;
  FieldPtrs fp;
  for (int k = 0; k < FG_NUM_FIELDS; ++k) fp.p[k] = f->d[k];
  count(f);
  k_apply_edits<<<(n_groups + 255) / 256, 256, 0, f->stream>>>(
      f->edit_dev[slot], f->edit_off_dev[slot], n_groups, fp, f->g);
  return cudaGetLastError();
}

cudaError_t launch_apply_sources(fg_fluid* f) {
  if (f->n_src_groups <= 0) return cudaSuccess;
  count(f);
  if (f->batch)
    kb_apply_sources<<<(f->n_src_groups + 255) / 256, 256, 0, f->stream>>>(
        f->src_dev, f->src_off_dev, f->batch->src_scene, f->n_src_groups, f->d[FG_U],
        f->d[FG_V], f->d[FG_M], f->flags, f->batch->scenes_dev);
  else
    k_apply_sources<<<(f->n_src_groups + 255) / 256, 256, 0, f->stream>>>(
        f->src_dev, f->src_off_dev, f->n_src_groups, f->d[FG_U], f->d[FG_V], f->d[FG_M],
        f->flags, f->g);
  return cudaGetLastError();
}

cudaError_t launch_viscosity(fg_fluid* f, float dt) {
  float visc = f->prm.viscosity_diffusion * dt;
  count(f);
  k_viscosity<<<cell_grid(f), dim3(BX, BY), 0, f->stream>>>(
      f->d[FG_U], f->d[FG_V], f->partner[FG_U], f->partner[FG_V], f->d[FG_NEWU], f->d[FG_NEWV],
      f->flags, visc, f->g);
  swap_state(f, FG_U);
  swap_state(f, FG_V);
  return cudaGetLastError();
}

cudaError_t launch_confinement_turbulence(fg_fluid* f, float dt, bool conf, bool turb) {
  if (!conf && !turb) return cudaSuccess;
  if (conf) {
    count(f);
    FG_CELLS(f, k_curl, curl_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V], f->curl,
             (const uint8_t*)f->flags);
  }
  float turbStrength = f->prm.turbulence_strength * dt;
  count(f);
  FG_CELLS(f, k_conf_turb, conf_turb_cell, f->d[FG_U], f->d[FG_V], (const float*)f->curl,
           (const float2*)f->noise, (const uint8_t*)f->flags, f->prm.confinement, dt,
           turbStrength, conf ? 1 : 0, turb ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_borders(fg_fluid* f) {
  count(f);
  if (f->batch) {
    FG_BORDER(f, k_borders, borders_border, f->d[FG_U], f->d[FG_V], (const uint8_t*)f->flags);
  } else {
    const int n = f->NX > f->NY ? f->NX : f->NY;
    launch_pdl(k_borders, dim3((n + 127) / 128), dim3(128), 0, f->stream, f->d[FG_U], f->d[FG_V],
               f->flags, f->g);
  }
  return cudaGetLastError();
}

cudaError_t launch_copy_border(fg_fluid* f, float* dst, const float* src) {
  int n = f->NX > f->NY ? f->NX : f->NY;
  count(f);
  k_copy_border<<<(n + 127) / 128, 128, 0, f->stream>>>(dst, src, f->g);
  return cudaGetLastError();
}

// The turbulence noise depends on the cell only: float32(math.Sin(float64(
// float32(i*137 + j*241) * 0.01))) and the same with 157, 263 (fluid.go:509-514).
// It is evaluated once on the host in double precision and stored as a
// float2 table (8 bytes per cell), rather than evaluating a double-precision
// sine per cell on a part with low FP64 throughput.
cudaError_t launch_noise_table(fg_fluid* f) {
  std::vector<float2> tab((size_t)f->NX * f->P, make_float2(0.f, 0.f));
  for (int i = 0; i < f->NX; ++i)
    for (int j = 0; j < f->NY; ++j) {
      float seedU = (float)(i * 137 + j * 241) * 0.01f;
      float seedV = (float)(i * 157 + j * 263) * 0.01f;
      tab[(size_t)i * f->P + j] =
          make_float2((float)std::sin((double)seedU), (float)std::sin((double)seedV));
    }
  cudaError_t e = cudaMemcpyAsync(f->noise, tab.data(), tab.size() * sizeof(float2),
                                  cudaMemcpyHostToDevice, f->stream);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(f->stream);
}

}  // namespace fg
