// Diagnostics and field views (pkg/fluid/fluid.go:529-557, 798-891;
// pressure.go, smoke.go): reductions accumulate in FP64 through fixed-slot
// block partials, so repeated runs give identical numbers.
#include <cfloat>

#include "fg_internal.cuh"
#include "fg_reduce.cuh"

namespace fg {
namespace {

constexpr int BX = 32, BY = 8;
inline dim3 cell_grid(const fg_fluid* f) {
  return dim3((f->NY + BX - 1) / BX, (f->NX + BY - 1) / BY);
}
__device__ __forceinline__ int block_id() { return blockIdx.y * gridDim.x + blockIdx.x; }
__device__ __forceinline__ bool fluid_interior(uint8_t fl) {
  return (fl & (F_FLUID | F_INTERIOR)) == (F_FLUID | F_INTERIOR);
}

// Post-projection divergence statistics: rows {sum div^2, max |div|, count}
// over fluid interior cells.
__global__ void k_div_partials(const float* __restrict__ U, const float* __restrict__ V,
                               const uint8_t* __restrict__ flags, float* __restrict__ part,
                               Grid g) {
  __shared__ float sh[64 * 3];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
  if (j < g.NY && i < g.NX) {
    int c = i * g.P + j;
    if (fluid_interior(flags[c])) {
      float div = U[c + g.P] - U[c] + V[c + 1] - V[c];
      v[0] = ff_sq(div);
      v[1].hi = fabsf(div);
      v[2].hi = 1.0f;
    }
  }
  block_row<3>(v, 2u, sh, part + 6 * (size_t)block_id());
}

__global__ void k_store_div(const float* __restrict__ r, DevStats* st) {
  st->div_l2_sq = row_sum(r, 0);
  st->div_max = (double)r[2];
  st->div_count = row_sum(r, 2);
}

// sum of M over interior cells.
__global__ void k_mass_partials(const float* __restrict__ M, float* __restrict__ part, Grid g) {
  __shared__ float sh[64];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[1] = {{0.0f, 0.0f}};
  if (i >= 1 && i <= g.NX - 2 && j >= 1 && j <= g.NY - 2) v[0].hi = M[i * g.P + j];
  block_row<1>(v, 0u, sh, part + 2 * (size_t)block_id());
}

struct StoreMass {
  DevStats* st;
  __device__ void operator()(const float* r) const { st->smoke_mass = row_sum(r, 0); }
};

// MaxDivergence (fluid.go:876-891): float32 |div|, NaN ignored (fmaxf).
__global__ void k_maxdiv_partials(const float* __restrict__ U, const float* __restrict__ V,
                                  const uint8_t* __restrict__ flags, float* __restrict__ part,
                                  Grid g) {
  __shared__ float sh[64];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[1] = {{0.0f, 0.0f}};
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    if (fluid_interior(flags[c])) {
      float div = U[c + g.P] - U[c] + V[c + 1] - V[c];
      v[0].hi = fabsf(div);
    }
  }
  block_row<1>(v, 1u, sh, part + 2 * (size_t)block_id());
}

// |U| + |V| on fluid interior cells (GetAdaptiveTimeStep fluid.go:534-543).
__global__ void k_speed_partials(const float* __restrict__ U, const float* __restrict__ V,
                                 const uint8_t* __restrict__ flags, float* __restrict__ part,
                                 Grid g) {
  __shared__ float sh[64];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[1] = {{0.0f, 0.0f}};
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    if (fluid_interior(flags[c])) v[0].hi = fabsf(U[c]) + fabsf(V[c]);
  }
  block_row<1>(v, 1u, sh, part + 2 * (size_t)block_id());
}

// Vorticity (fluid.go:806-838, kind 0) and VelocityMagnitude (fluid.go:841-873,
// kind 1) on fluid interior cells, 0 elsewhere; rows {max v, max -v} over
// the computed cells (-inf when a block saw none).
__global__ void k_view(const float* __restrict__ U, const float* __restrict__ V,
                       const uint8_t* __restrict__ flags, float* __restrict__ out, int kind,
                       float* __restrict__ part, Grid g) {
  __shared__ float sh[128];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[2] = {{-INFINITY, 0.0f}, {-INFINITY, 0.0f}};
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    float x = 0.0f;
    if (fluid_interior(flags[c])) {
      if (kind == 0) {
        float dvdx = (V[c + g.P] - V[c - g.P]) * 0.5f / g.h;
        float dudy = (U[c + 1] - U[c - 1]) * 0.5f / g.h;
        x = dvdx - dudy;
      } else {
        float u = (U[c] + U[c + g.P]) * 0.5f;
        float w = (V[c] + V[c + 1]) * 0.5f;
        x = sqrtf(u * u + w * w);
      }
      if (!isnan(x)) {
        v[0].hi = x;
        v[1].hi = -x;
      }
    }
    out[c] = x;
  }
  block_row<2>(v, 3u, sh, part + 4 * (size_t)block_id());
}

// min / max over all cells of a field (Pressure(), Smoke()).
__global__ void k_minmax_partials(const float* __restrict__ F, float* __restrict__ part, Grid g) {
  __shared__ float sh[128];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[2] = {{-INFINITY, 0.0f}, {-INFINITY, 0.0f}};
  if (i < g.NX && j < g.NY) {
    float x = F[i * g.P + j];
    if (!isnan(x)) {
      v[0].hi = x;
      v[1].hi = -x;
    }
  }
  block_row<2>(v, 3u, sh, part + 4 * (size_t)block_id());
}

// (max v, max -v) -> float (min, max), with the reference's initial values
// (MaxFloat32, -MaxFloat32) when no cell was seen.
__global__ void k_store_minmax(const float* __restrict__ r, float* __restrict__ out) {
  float hi = r[0], nlo = r[2];
  out[0] = nlo == -INFINITY ? FLT_MAX : -nlo;
  out[1] = hi == -INFINITY ? -FLT_MAX : hi;
}

// A max slot of a final row -> float, 0 when no cell was seen.
__global__ void k_store_max0(const float* __restrict__ r, float* __restrict__ out) {
  out[0] = r[0] < 0.0f ? 0.0f : r[0];
}

__global__ void k_sample_velocity(const float* __restrict__ U, const float* __restrict__ V,
                                  float x, float y, float* __restrict__ out, Grid g) {
  out[0] = sample_field(U, x, y, 0.0f, g.hh, g);
  out[1] = sample_field(V, x, y, g.hh, 0.0f, g);
}

}  // namespace

cudaError_t launch_clear_stats(fg_fluid* f) {
  return cudaMemsetAsync(f->dstats, 0, sizeof(DevStats), f->stream);
}

cudaError_t launch_div_stats(fg_fluid* f) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 3, nb)) return cudaErrorInvalidValue;
  count(f);
  k_div_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags,
                                                     f->partials, f->g);
  float* out = nullptr;
  count(f, combine_rows<3>(f->stream, f->partials, nb, 2u, &out));
  count(f);
  k_store_div<<<1, 1, 0, f->stream>>>(out, f->dstats);
  return cudaGetLastError();
}

cudaError_t launch_store_mass(fg_fluid* f, int nb) {
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  launch_pdl(k_combine_store<1, StoreMass>, dim3(1), dim3(1024), 0, f->stream, f->partials, nb,
             0u, StoreMass{f->dstats});
  return cudaGetLastError();
}

cudaError_t launch_smoke_mass(fg_fluid* f) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_mass_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_M], f->partials, f->g);
  return launch_store_mass(f, nb);
}

static cudaError_t finish_max0(fg_fluid* f, int nb, float* dev_out) {
  float* out = nullptr;
  count(f, combine_rows<1>(f->stream, f->partials, nb, 1u, &out));
  count(f);
  k_store_max0<<<1, 1, 0, f->stream>>>(out, dev_out);
  return cudaGetLastError();
}

cudaError_t launch_max_divergence(fg_fluid* f, float* dev_out) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_maxdiv_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags,
                                                        f->partials, f->g);
  return finish_max0(f, nb, dev_out);
}

cudaError_t launch_max_speed(fg_fluid* f, float* dev_out) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_speed_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags,
                                                       f->partials, f->g);
  return finish_max0(f, nb, dev_out);
}

static cudaError_t finish_minmax(fg_fluid* f, int nb, float* dev_minmax) {
  float* out = nullptr;
  count(f, combine_rows<2>(f->stream, f->partials, nb, 3u, &out));
  count(f);
  k_store_minmax<<<1, 1, 0, f->stream>>>(out, dev_minmax);
  return cudaGetLastError();
}

cudaError_t launch_view(fg_fluid* f, int kind, float* dev_minmax) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 2, nb)) return cudaErrorInvalidValue;
  count(f);
  k_view<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags, f->view, kind,
                                             f->partials, f->g);
  return finish_minmax(f, nb, dev_minmax);
}

cudaError_t launch_field_minmax(fg_fluid* f, int field, float* dev_minmax) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 2, nb)) return cudaErrorInvalidValue;
  count(f);
  k_minmax_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[field], f->partials, f->g);
  return finish_minmax(f, nb, dev_minmax);
}

cudaError_t launch_sample_velocity(fg_fluid* f, float x, float y, float* dev_uv) {
  count(f);
  k_sample_velocity<<<1, 1, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], x, y, dev_uv, f->g);
  return cudaGetLastError();
}

// Copies between the mirrors' layout (rows of NY floats) and the device
// pitch, on the device (faster than a strided DMA copy for device sources).
__global__ void k_repitch(float* __restrict__ dst, const float* __restrict__ src, int rows,
                          int cols, int dpitch, int spitch) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= rows || j >= cols) return;
  dst[(size_t)i * dpitch + j] = src[(size_t)i * spitch + j];
}

cudaError_t launch_repitch(fg_fluid* f, float* dst, const float* src, int dpitch, int spitch) {
  count(f);
  dim3 gr((f->NY + 31) / 32, (f->NX + 7) / 8);
  k_repitch<<<gr, dim3(32, 8), 0, f->stream>>>(dst, src, f->NX, f->NY, dpitch, spitch);
  return cudaGetLastError();
}

}  // namespace fg
