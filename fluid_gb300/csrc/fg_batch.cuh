// Batched launches: the per-cell kernels of a batch run over a block table
// (BTile) and read each block's scene (BScene) from a device table; every
// field pointer argument is shifted to the scene's slice of the packed
// arrays, so one launch covers every scene of the batch.
#pragma once

#include "fg_internal.cuh"

namespace fg {

// Field pointers move to the scene's slice; everything else (scalars,
// control blocks, tables) passes unchanged.
template <class T>
__device__ __forceinline__ T bshift(T v, long long) {
  return v;
}
__device__ __forceinline__ float* bshift(float* p, long long o) { return p ? p + o : p; }
__device__ __forceinline__ const float* bshift(const float* p, long long o) {
  return p ? p + o : p;
}
__device__ __forceinline__ uint8_t* bshift(uint8_t* p, long long o) { return p ? p + o : p; }
__device__ __forceinline__ const uint8_t* bshift(const uint8_t* p, long long o) {
  return p ? p + o : p;
}
__device__ __forceinline__ float2* bshift(float2* p, long long o) { return p ? p + o : p; }
__device__ __forceinline__ const float2* bshift(const float2* p, long long o) {
  return p ? p + o : p;
}

// Body(i, j, args..., grid) over the cells of every scene.  The block's
// table entry (constant) is read before waiting on the previous kernel.
template <auto Body, class... A>
__global__ void kb_cells(const BCell* __restrict__ blocks, A... a) {
  const BCell c = blocks[blockIdx.x];
  pdl_enter();
  const int j = c.x * blockDim.x + threadIdx.x;
  const int i = c.y * blockDim.y + threadIdx.y;
  if (i >= c.g.NX || j >= c.g.NY) return;
  Body(i, j, bshift(a, c.off)..., c.g);
}

// kb_cells<Body> over the batch's cell blocks, with programmatic stream
// serialization.
template <auto Body, class... A>
inline cudaError_t launch_cells(const fg_fluid* f, A... a) {
  const BatchGeom* b = f->batch;
  return launch_pdl(kb_cells<Body, A...>, dim3(b->n_cell_tiles), dim3(b->bx, b->by), 0,
                    f->stream, b->cell_blocks, a...);
}

// Body(t, args..., grid) over the border threads (t < max(NX, NY)) of
// every scene; blocks are one-dimensional.
template <auto Body, class... A>
__global__ void kb_border(const BTile* __restrict__ tiles, const BScene* __restrict__ sc, A... a) {
  const BTile t = tiles[blockIdx.x];
  const Grid g = sc[t.s].g;
  Body(t.x * blockDim.x + threadIdx.x, bshift(a, sc[t.s].off)..., g);
}

// Launches a per-cell stage: the single-scene kernel K over the handle's
// grid, or the batched wrapper of BODY over the batch's block table.
#define FG_CELLS(f, K, BODY, ...)                                                            \
  do {                                                                                       \
    if ((f)->batch) {                                                                        \
      launch_cells<BODY>((f), __VA_ARGS__);                                                  \
    } else {                                                                                 \
      K<<<dim3(((f)->NY + 31) / 32, ((f)->NX + 7) / 8), dim3(32, 8), 0, (f)->stream>>>(      \
          __VA_ARGS__, (f)->g);                                                              \
    }                                                                                        \
  } while (0)

// The batched wrapper of BODY only (for stages whose single-scene kernel
// takes other arguments).
#define FG_CELLS_BATCH(f, BODY, ...) launch_cells<BODY>((f), __VA_ARGS__)

#define FG_BORDER(f, K, BODY, ...)                                                           \
  do {                                                                                       \
    if ((f)->batch) {                                                                        \
      const BatchGeom* b_ = (f)->batch;                                                      \
      kb_border<BODY><<<b_->n_border_tiles, 128, 0, (f)->stream>>>(b_->border_tiles,         \
                                                                   b_->scenes_dev,           \
                                                                   __VA_ARGS__);             \
    } else {                                                                                 \
      int n_ = (f)->NX > (f)->NY ? (f)->NX : (f)->NY;                                        \
      K<<<(n_ + 127) / 128, 128, 0, (f)->stream>>>(__VA_ARGS__, (f)->g);                     \
    }                                                                                        \
  } while (0)

}  // namespace fg
