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

// sum div^2 (float pairs in the block, FP64 across blocks), max |div| and
// the count of fluid interior cells.
__global__ void k_div_partials(const float* __restrict__ U, const float* __restrict__ V,
                               const uint8_t* __restrict__ flags, double* __restrict__ part,
                               Grid g) {
  __shared__ double red[32];
  __shared__ float redf[32];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF s2{0.0f, 0.0f};
  float mx = 0.0f;
  int n = 0;
  if (j < g.NY && i < g.NX) {
    int c = i * g.P + j;
    if (fluid_interior(flags[c])) {
      float div = U[c + g.P] - U[c] + V[c + 1] - V[c];
      s2 = ff_sq(div);
      mx = fabsf(div);
      n = 1;
    }
  }
  double a = block_sum_ff(s2, red);
  float b = block_max_f(mx, redf);
  double cn = block_sum_ff(FF{(float)n, 0.0f}, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    double* o = part + 3 * (size_t)block_id();
    o[0] = a;
    o[1] = (double)b;
    o[2] = cn;
  }
}

__global__ void k_store_div(const double* __restrict__ r, DevStats* st) {
  st->div_l2_sq = r[0];
  st->div_max = r[1];
  st->div_count = r[2];
}

// sum of M over interior cells (float pairs in the block, FP64 across blocks).
__global__ void k_mass_partials(const float* __restrict__ M, double* __restrict__ part, Grid g) {
  __shared__ double red[32];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  FF m{0.0f, 0.0f};
  if (j >= 1 && j <= g.NY - 2) {
    for (int i = blockIdx.y * blockDim.y + threadIdx.y; i < g.NX; i += gridDim.y * blockDim.y)
      if (i >= 1 && i <= g.NX - 2) m = ff_add(m, FF{M[i * g.P + j], 0.0f});
  }
  double a = block_sum_ff(m, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) part[block_id()] = a;
}

__global__ void k_store_mass(const double* __restrict__ r, DevStats* st) { st->smoke_mass = r[0]; }

// MaxDivergence (fluid.go:876-891): float32 |div|, NaN ignored.
__global__ void k_maxdiv_partials(const float* __restrict__ U, const float* __restrict__ V,
                                  const uint8_t* __restrict__ flags, double* __restrict__ part,
                                  Grid g) {
  __shared__ double red[32];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  double mx = 0.0;
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    if (fluid_interior(flags[c])) {
      float div = U[c + g.P] - U[c] + V[c + 1] - V[c];
      float a = fabsf(div);
      if (a > 0.0f) mx = (double)a;
    }
  }
  double b = block_reduce<true>(mx, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) part[block_id()] = b;
}

// |U| + |V| on fluid interior cells (GetAdaptiveTimeStep fluid.go:534-543).
__global__ void k_speed_partials(const float* __restrict__ U, const float* __restrict__ V,
                                 const uint8_t* __restrict__ flags, double* __restrict__ part,
                                 Grid g) {
  __shared__ double red[32];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  double mx = 0.0;
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    if (fluid_interior(flags[c])) {
      float vel = fabsf(U[c]) + fabsf(V[c]);
      if (vel > 0.0f) mx = (double)vel;
    }
  }
  double b = block_reduce<true>(mx, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) part[block_id()] = b;
}

// Vorticity (fluid.go:806-838, kind 0) and VelocityMagnitude (fluid.go:841-873,
// kind 1) on fluid interior cells, 0 elsewhere; partials hold max(v), max(-v)
// over the computed cells.
__global__ void k_view(const float* __restrict__ U, const float* __restrict__ V,
                       const uint8_t* __restrict__ flags, float* __restrict__ out, int kind,
                       double* __restrict__ part, Grid g) {
  __shared__ double red[32];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  double hi = -DBL_MAX, nlo = -DBL_MAX;
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    float v = 0.0f;
    if (fluid_interior(flags[c])) {
      if (kind == 0) {
        float dvdx = (V[c + g.P] - V[c - g.P]) * 0.5f / g.h;
        float dudy = (U[c + 1] - U[c - 1]) * 0.5f / g.h;
        v = dvdx - dudy;
      } else {
        float u = (U[c] + U[c + g.P]) * 0.5f;
        float w = (V[c] + V[c + 1]) * 0.5f;
        v = sqrtf(u * u + w * w);
      }
      if (!isnan(v)) {
        hi = (double)v;
        nlo = -(double)v;
      }
    }
    out[c] = v;
  }
  double a = block_reduce<true>(hi, red);
  double b = block_reduce<true>(nlo, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    part[2 * (size_t)block_id()] = a;
    part[2 * (size_t)block_id() + 1] = b;
  }
}

// min / max over all cells of a field (Pressure(), Smoke()).
__global__ void k_minmax_partials(const float* __restrict__ F, double* __restrict__ part, Grid g) {
  __shared__ double red[32];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  double hi = -DBL_MAX, nlo = -DBL_MAX;
  if (i < g.NX && j < g.NY) {
    float v = F[i * g.P + j];
    if (!isnan(v)) {
      hi = (double)v;
      nlo = -(double)v;
    }
  }
  double a = block_reduce<true>(hi, red);
  double b = block_reduce<true>(nlo, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    part[2 * (size_t)block_id()] = a;
    part[2 * (size_t)block_id() + 1] = b;
  }
}

// Converts combined (max, max of negation) into float (min, max) with the
// reference's initial values when nothing was seen.
__global__ void k_store_minmax(const double* __restrict__ r, float* __restrict__ out) {
  double hi = r[0], nlo = r[1];
  out[0] = nlo == -DBL_MAX ? FLT_MAX : (float)(-nlo);
  out[1] = hi == -DBL_MAX ? -FLT_MAX : (float)hi;
}

// k_combine with max starts from 0.0; the view partials are -DBL_MAX when a
// block saw nothing, which never exceeds a real value, and a combined 0.0
// from an empty field is mapped back below by the caller's initial values.
__global__ void k_combine_max2(const double* __restrict__ part, int n, double* __restrict__ out) {
  __shared__ double red[32];
  for (int s = 0; s < 2; ++s) {
    double v = -DBL_MAX;
    for (int k = threadIdx.x; k < n; k += blockDim.x) v = fmax(v, part[2 * (size_t)k + s]);
    v = block_reduce<true>(v, red);
    if (threadIdx.x == 0) out[s] = v;
  }
}

__global__ void k_store_float(const double* __restrict__ r, float* __restrict__ out) {
  out[0] = (float)r[0];
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
  double* out = nullptr;
  count(f, combine_partials<3>(f->stream, f->partials, nb, 2u, &out));
  count(f);
  k_store_div<<<1, 1, 0, f->stream>>>(out, f->dstats);
  return cudaGetLastError();
}

cudaError_t launch_smoke_mass(fg_fluid* f) {
  dim3 gr = reduce_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_mass_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_M], f->partials, f->g);
  double* out = nullptr;
  count(f, combine_partials<1>(f->stream, f->partials, nb, 0u, &out));
  count(f);
  k_store_mass<<<1, 1, 0, f->stream>>>(out, f->dstats);
  return cudaGetLastError();
}

cudaError_t launch_store_mass(fg_fluid* f, int nb) {
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  double* out = nullptr;
  count(f, combine_partials<1>(f->stream, f->partials, nb, 0u, &out));
  count(f);
  k_store_mass<<<1, 1, 0, f->stream>>>(out, f->dstats);
  return cudaGetLastError();
}

cudaError_t launch_max_divergence(fg_fluid* f, float* dev_out) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_maxdiv_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags,
                                                        f->partials, f->g);
  double* out = nullptr;
  count(f, combine_partials<1>(f->stream, f->partials, nb, 1u, &out));
  count(f);
  k_store_float<<<1, 1, 0, f->stream>>>(out, dev_out);
  return cudaGetLastError();
}

cudaError_t launch_max_speed(fg_fluid* f, float* dev_out) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_speed_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags,
                                                       f->partials, f->g);
  double* out = nullptr;
  count(f, combine_partials<1>(f->stream, f->partials, nb, 1u, &out));
  count(f);
  k_store_float<<<1, 1, 0, f->stream>>>(out, dev_out);
  return cudaGetLastError();
}

cudaError_t launch_view(fg_fluid* f, int kind, float* dev_minmax) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 2, nb)) return cudaErrorInvalidValue;
  count(f);
  k_view<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->flags, f->view, kind,
                                             f->partials, f->g);
  double* out = f->partials + 2 * (size_t)nb;
  count(f);
  k_combine_max2<<<1, 1024, 0, f->stream>>>(f->partials, nb, out);
  count(f);
  k_store_minmax<<<1, 1, 0, f->stream>>>(out, dev_minmax);
  return cudaGetLastError();
}

cudaError_t launch_field_minmax(fg_fluid* f, int field, float* dev_minmax) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 2, nb)) return cudaErrorInvalidValue;
  count(f);
  k_minmax_partials<<<gr, dim3(BX, BY), 0, f->stream>>>(f->d[field], f->partials, f->g);
  double* out = f->partials + 2 * (size_t)nb;
  count(f);
  k_combine_max2<<<1, 1024, 0, f->stream>>>(f->partials, nb, out);
  count(f);
  k_store_minmax<<<1, 1, 0, f->stream>>>(out, dev_minmax);
  return cudaGetLastError();
}

cudaError_t launch_sample_velocity(fg_fluid* f, float x, float y, float* dev_uv) {
  count(f);
  k_sample_velocity<<<1, 1, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], x, y, dev_uv, f->g);
  return cudaGetLastError();
}

}  // namespace fg
