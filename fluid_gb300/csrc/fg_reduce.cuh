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

// Combines rows [b*per, min(n, (b+1)*per)) of NS partials (partials[k*NS +
// s]) into out[b*NS + s], one block b of 1024 threads per output row; bit s
// of max_mask selects max instead of sum for slot s.
template <int NS>
__global__ void k_combine(const double* __restrict__ partials, int n, int per, unsigned max_mask,
                          double* __restrict__ out) {
  __shared__ double sh[32];
  int k0 = blockIdx.x * per;
  int k1 = min(n, k0 + per);
  for (int s = 0; s < NS; ++s) {
    bool mx = (max_mask >> s) & 1u;
    double v = 0.0;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
      double w = partials[(size_t)k * NS + s];
      v = mx ? fmax(v, w) : v + w;
    }
    v = mx ? block_reduce<true>(v, sh) : block_reduce<false>(v, sh);
    if (threadIdx.x == 0) out[(size_t)blockIdx.x * NS + s] = v;
  }
}

// Deterministic two-level combine of n rows of NS partials starting at
// `part`; the result (NS doubles) is written at *out_ptr, which points past
// the level-one rows inside the same buffer.  Returns the number of kernels.
template <int NS>
inline int combine_partials(cudaStream_t st, double* part, int n, unsigned max_mask,
                            double** out_ptr) {
  double* lvl = part + (size_t)NS * n;
  const int per = 2048;
  if (n <= per) {
    k_combine<NS><<<1, 1024, 0, st>>>(part, n, n, max_mask, lvl);
    *out_ptr = lvl;
    return 1;
  }
  int g = (n + per - 1) / per;
  k_combine<NS><<<g, 1024, 0, st>>>(part, n, per, max_mask, lvl);
  double* out = lvl + (size_t)NS * g;
  k_combine<NS><<<1, 1024, 0, st>>>(lvl, g, g, max_mask, out);
  *out_ptr = out;
  return 2;
}

}  // namespace
}  // namespace fg

// ---------------------------------------------------------------------------
// Double-float ("float-float") accumulation.  This part's FP64 rate is about
// 1/64 of its FP32 rate, so the per-cell and intra-block work of the FP64
// reductions uses error-free FP32 transformations (Knuth's TwoSum, the exact
// product error by fma), which carry about 48 significant bits; block totals
// are converted exactly to double and combined across blocks in IEEE FP64.
// ---------------------------------------------------------------------------
namespace fg {
namespace {

struct FF {
  float hi, lo;
};

// Knuth's TwoSum: s + e == a + b exactly.
__host__ __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

__host__ __device__ __forceinline__ FF ff_add(FF a, FF b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = e + (a.lo + b.lo);
  float h, l;
  two_sum(s, e, h, l);
  return FF{h, l};
}

// x*x as an unevaluated float pair (exact).
__device__ __forceinline__ FF ff_sq(float x) {
  float p = x * x;
  return FF{p, __fmaf_rn(x, x, -p)};
}

// Residual b + (pw + pe + ps + pn) - s*x of FP32 inputs as a normalised float
// pair (hi = the residual rounded to float): the product s*x is split
// exactly by fma and the seven terms are summed with a TwoSum cascade.
__host__ __device__ __forceinline__ FF resid_ff(float b, float pw, float pe, float ps, float pn,
                                                float s, float x) {
  float p = s * x;
#ifdef __CUDA_ARCH__
  float pl = __fmaf_rn(s, x, -p);
#else
  float pl = fmaf(s, x, -p);
#endif
  float hi = b, lo = 0.0f, t, e;
  two_sum(hi, pw, t, e); hi = t; lo = lo + e;
  two_sum(hi, pe, t, e); hi = t; lo = lo + e;
  two_sum(hi, ps, t, e); hi = t; lo = lo + e;
  two_sum(hi, pn, t, e); hi = t; lo = lo + e;
  two_sum(hi, -p, t, e); hi = t; lo = lo + e;
  lo = lo - pl;
  two_sum(hi, lo, t, e);
  return FF{t, e};
}

// Warp-level reduction of NS float-pair sums, NM float maxima and a count
// of predicates, then one block-level combine in double: the block's totals
// land in out[0..NS+NM] (sums, maxima, count) written by thread 0.  The tree
// adds pairs with one TwoSum per level and renormalises at the end.  sh
// holds 8 * (NS + NM + 1) doubles (blocks of up to 256 threads).
template <int NS, int NM>
__device__ __forceinline__ void block_stats(FF (&s)[NS], float (&m)[NM], bool pred, double* sh,
                                            double* out) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = (blockDim.x * blockDim.y) >> 5;
  const int cnt = __popc(__ballot_sync(0xffffffffu, pred));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      float bh = __shfl_down_sync(0xffffffffu, s[k].hi, o);
      float bl = __shfl_down_sync(0xffffffffu, s[k].lo, o);
      float t, e;
      two_sum(s[k].hi, bh, t, e);
      s[k].hi = t;
      s[k].lo = (s[k].lo + bl) + e;
    }
#pragma unroll
    for (int k = 0; k < NM; ++k) m[k] = fmaxf(m[k], __shfl_down_sync(0xffffffffu, m[k], o));
  }
  constexpr int R = NS + NM + 1;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < NS; ++k) sh[wid * R + k] = (double)s[k].hi + (double)s[k].lo;
#pragma unroll
    for (int k = 0; k < NM; ++k) sh[wid * R + NS + k] = (double)m[k];
    sh[wid * R + NS + NM] = (double)cnt;
  }
  __syncthreads();
  if (tid < R) {
    double v = 0.0;
    bool mx = tid >= NS && tid < NS + NM;
    for (int w = 0; w < nw; ++w) v = mx ? fmax(v, sh[w * R + tid]) : v + sh[w * R + tid];
    out[tid] = v;
  }
}

// Sum of a float pair per thread over the block, as a double in thread 0.
// Warp level in float-float, block level in double.  sh: 32 doubles.
__device__ __forceinline__ double block_sum_ff(FF v, double* sh) {
  int tid = threadIdx.x + threadIdx.y * blockDim.x;
  int nt = blockDim.x * blockDim.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    FF w{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
    v = ff_add(v, w);
  }
  __syncthreads();
  if ((tid & 31) == 0) sh[tid >> 5] = (double)v.hi + (double)v.lo;
  __syncthreads();
  double r = 0.0;
  if (tid == 0)
    for (int k = 0; k < (nt >> 5); ++k) r += sh[k];
  return r;
}

// Max of a non-negative float per thread over the block (thread 0).
__device__ __forceinline__ float block_max_f(float v, float* sh) {
  int tid = threadIdx.x + threadIdx.y * blockDim.x;
  int nt = blockDim.x * blockDim.y;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((tid & 31) == 0) sh[tid >> 5] = v;
  __syncthreads();
  float r = 0.0f;
  if (tid == 0)
    for (int k = 0; k < (nt >> 5); ++k) r = fmaxf(r, sh[k]);
  return r;
}

}  // namespace
}  // namespace fg
