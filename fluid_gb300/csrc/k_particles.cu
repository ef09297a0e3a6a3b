// Tracer particles and field rendering: the app-side loops that read the
// simulation every frame (main/main.go:489-546 advectParticles,
// main/main.go:619-650 drawScalarField / drawVorticityField with the
// colormaps of main/colors.go:10-84), as kernels on the resident fields.
//
// Particles are stored as structure-of-arrays on the device (x, y, age,
// max age, packed RGB) in two buffers; a step advects every live particle
// and writes the survivors, in their original order, to the other buffer.
// The live count stays on the device: the kernels read it there, so a step
// needs no host round trip.
#include "fg_internal.cuh"

namespace fg {
namespace {

constexpr int PB = 1024;  // particles per block

// One advectParticles iteration for particle k: age, RK2 midpoint through
// SampleVelocity (fluid.go:799-803), bounds and solid checks.
__global__ void k_particles_advect(float* __restrict__ px, float* __restrict__ py,
                                   float* __restrict__ age, const float* __restrict__ maxage,
                                   const int* __restrict__ count, uint8_t* __restrict__ keep,
                                   int* __restrict__ block_keep, const float* __restrict__ U,
                                   const float* __restrict__ V, const uint8_t* __restrict__ flags,
                                   float dt, Grid g) {
  const int k = blockIdx.x * PB + threadIdx.x;
  const int n = *count;
  bool alive = false;
  if (k < n) {
    float a = age[k] + dt;
    age[k] = a;
    if (!(a > maxage[k])) {
      float x = px[k], y = py[k];
      float u1 = sample_field(U, x, y, 0.0f, g.hh, g);
      float v1 = sample_field(V, x, y, g.hh, 0.0f, g);
      float mx = x + 0.5f * dt * u1;
      float my = y + 0.5f * dt * v1;
      float u2 = sample_field(U, mx, my, 0.0f, g.hh, g);
      float v2 = sample_field(V, mx, my, g.hh, 0.0f, g);
      x += dt * u2;
      y += dt * v2;
      px[k] = x;
      py[k] = y;
      // int(p.X / h): truncation toward zero, as Go converts.
      float qi = x / g.h, qj = y / g.h;
      if (qi > -2147483648.0f && qi < 2147483648.0f && qj > -2147483648.0f &&
          qj < 2147483648.0f) {
        int fi = (int)qi, fj = (int)qj;
        if (fi >= 0 && fi < g.NX && fj >= 0 && fj < g.NY)
          alive = (flags[fi * g.P + fj] & F_FLUID) != 0;
      }
    }
  }
  keep[k] = alive ? 1 : 0;  // every slot of the grid: the compaction reads whole blocks
  const unsigned bal = __ballot_sync(0xffffffffu, alive);
  __shared__ int wsum[PB / 32];
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < PB / 32; ++w) s += wsum[w];
    block_keep[blockIdx.x] = s;
  }
}

// Writes the survivors of block b at (survivors of blocks < b) + (their
// rank within the block), preserving order; block 0 also stores the new
// count.
__global__ void k_particles_compact(const float* __restrict__ px, const float* __restrict__ py,
                                    const float* __restrict__ age,
                                    const float* __restrict__ maxage,
                                    const uint32_t* __restrict__ rgb,
                                    const uint8_t* __restrict__ keep,
                                    const int* __restrict__ block_keep, int nblocks,
                                    int* __restrict__ count, float* __restrict__ ox,
                                    float* __restrict__ oy, float* __restrict__ oage,
                                    float* __restrict__ omax, uint32_t* __restrict__ orgb) {
  __shared__ int part[PB / 32];
  __shared__ int base;
  // Survivors of the earlier blocks (and, for block 0, of all blocks).
  const int upto = blockIdx.x == 0 ? nblocks : (int)blockIdx.x;
  int s = 0;
  for (int b = threadIdx.x; b < upto; b += PB) s += block_keep[b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < PB / 32; ++w) t += part[w];
    base = blockIdx.x == 0 ? 0 : t;
    if (blockIdx.x == 0) *count = t;
  }
  __syncthreads();
  const int k = blockIdx.x * PB + threadIdx.x;
  const bool alive = keep[k] != 0;  // keep is sized to whole blocks, zero past the count
  const unsigned bal = __ballot_sync(0xffffffffu, alive);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) part[w] = __popc(bal);
  __syncthreads();
  if (!alive) return;
  int r = __popc(bal & ((1u << lane) - 1u));
  for (int q = 0; q < w; ++q) r += part[q];
  const int d = base + r;
  ox[d] = px[k];
  oy[d] = py[k];
  oage[d] = age[k];
  omax[d] = maxage[k];
  orgb[d] = rgb[k];
}

// ---------------------------------------------------------------- colormaps
__device__ __forceinline__ uint32_t pack(float r, float g, float b) {
  // uint8(255 * c): truncation of a value in [0, 255], as Go converts.
  uint32_t R = (uint32_t)(255.0f * r), G = (uint32_t)(255.0f * g), B = (uint32_t)(255.0f * b);
  return R | (G << 8) | (B << 16) | (0xffu << 24);
}

// getSciValue (main/colors.go:47-84).
__device__ __forceinline__ uint32_t sci_color(float val, float mn, float mx) {
  val = go_min(go_max(val, mn), mx - 0.0001f);
  float d = mx - mn;
  if (d <= 0.0f)
    val = 0.5f;
  else
    val = (val - mn) / d;
  const float m = 0.25f;
  float num = floorf(val / m);
  float s = (val - num * m) / m;
  float r = 0.0f, g = 0.0f, b = 0.0f;
  if (num == 0.0f) {
    r = 0.0f;
    g = s;
    b = 1.0f;
  } else if (num == 1.0f) {
    r = 0.0f;
    g = 1.0f;
    b = 1.0f - s;
  } else if (num == 2.0f) {
    r = s;
    g = 1.0f;
    b = 0.0f;
  } else if (num == 3.0f) {
    r = 1.0f;
    g = 1.0f - s;
    b = 0.0f;
  }
  return pack(r, g, b);
}

// getDivergingColor (main/colors.go:10-44).
__device__ __forceinline__ uint32_t diverging_color(float val, float mn, float mx) {
  float absMax = (float)fmax(fabs((double)mn), fabs((double)mx));
  if (absMax < 1e-8f) return 0xffffffffu;
  float t = val / absMax;
  if (t > 1.0f) t = 1.0f;
  if (t < -1.0f) t = -1.0f;
  float r, g, b;
  if (t >= 0.0f) {
    r = 1.0f;
    g = 1.0f - t;
    b = 1.0f - t;
  } else {
    float a = -t;
    r = 1.0f - a;
    g = 1.0f - a;
    b = 1.0f;
  }
  return pack(r, g, b);
}

// drawScalarField / drawVorticityField: pixel (i, j) of the NX x NY image
// (row stride NX) shows the field at (i, NY - 1 - j).
__global__ void k_render(const float* __restrict__ F, const float* __restrict__ minmax,
                         int diverging, uint32_t* __restrict__ img, Grid g) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  float v = F[i * g.P + (g.NY - 1 - j)];
  float mn = minmax[0], mx = minmax[1];
  img[(size_t)j * g.NX + i] = diverging ? diverging_color(v, mn, mx) : sci_color(v, mn, mx);
}

}  // namespace

cudaError_t launch_particles_advect(fg_fluid* f, float dt, int n_upper, const float* const* in,
                                    const uint32_t* rgb_in, float* const* out, uint32_t* rgb_out,
                                    int* live, uint8_t* keep, int* block_keep) {
  int nb = (n_upper + PB - 1) / PB;
  if (nb == 0) return cudaSuccess;
  count(f, 2);
  k_particles_advect<<<nb, PB, 0, f->stream>>>(
      (float*)in[0], (float*)in[1], (float*)in[2], in[3], live, keep, block_keep, f->d[FG_U],
      f->d[FG_V], f->flags, dt, f->g);
  k_particles_compact<<<nb, PB, 0, f->stream>>>(in[0], in[1], in[2], in[3], rgb_in, keep,
                                                block_keep, nb, live, out[0], out[1], out[2],
                                                out[3], rgb_out);
  return cudaGetLastError();
}

cudaError_t launch_render(fg_fluid* f, const float* field, const float* dev_minmax,
                          int diverging, uint32_t* img) {
  count(f);
  dim3 gr((f->NX + 31) / 32, (f->NY + 7) / 8);
  k_render<<<gr, dim3(32, 8), 0, f->stream>>>(field, dev_minmax, diverging, img, f->g);
  return cudaGetLastError();
}

}  // namespace fg
