// Deterministic block reductions: every block writes its partials to fixed
// slots; a single-block pass combines the slots in a fixed tree order, so the
// result does not depend on scheduling or on atomics.
#pragma once

#include <cfloat>

#include "fg_internal.cuh"

namespace fg {
namespace {

// Sum (MAX = false) or max (MAX = true) of one double per thread over the
// block; the result is valid in thread 0.  The block size must be a
// multiple of 32 and at most 1024; sh holds 32 doubles.
template <bool MAX>
__device__ __forceinline__ double block_reduce(double v, double* sh) {
  int tid = threadIdx.x + threadIdx.y * blockDim.x;
  int nt = blockDim.x * blockDim.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_down_sync(0xffffffffu, v, o);
    v = MAX ? fmax(v, w) : v + w;
  }
  __syncthreads();  // sh may still be read by a previous reduction
  if ((tid & 31) == 0) sh[tid >> 5] = v;
  __syncthreads();
  if (tid < 32) {
    v = tid < (nt >> 5) ? sh[tid] : (MAX ? -DBL_MAX : 0.0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double w = __shfl_down_sync(0xffffffffu, v, o);
      v = MAX ? fmax(v, w) : v + w;
    }
  }
  return v;
}

// Combines n rows of NS partials (partials[k*NS + s]); bit s of max_mask
// selects max instead of sum for slot s.  One block of 1024 threads.
template <int NS>
__global__ void k_combine(const double* __restrict__ partials, int n, unsigned max_mask,
                          double* __restrict__ out) {
  __shared__ double sh[32];
  for (int s = 0; s < NS; ++s) {
    bool mx = (max_mask >> s) & 1u;
    double v = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      double w = partials[(size_t)k * NS + s];
      v = mx ? fmax(v, w) : v + w;
    }
    v = mx ? block_reduce<true>(v, sh) : block_reduce<false>(v, sh);
    if (threadIdx.x == 0) out[s] = v;
  }
}

}  // namespace
}  // namespace fg
