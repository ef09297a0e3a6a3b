// Deterministic reductions in double-float arithmetic.
//
// This part retires only two FP64 operations per cycle per SM (1/64 of its
// FP32 rate), so a single double operation per warp per block already
// dominates a bandwidth-bound reduction pass.  The statistics are therefore
// accumulated as unevaluated pairs of floats ("double-float", about 48
// significant bits) with error-free transformations -- Knuth's TwoSum and
// the exact product error by fma -- at every level: per thread, warp, block
// and across blocks.  Only the final totals are converted to IEEE FP64.
// Every block writes its partial row to a fixed slot and the rows are
// combined in a fixed tree order, so results do not depend on scheduling.
//
// A partial row holds NS slots of two floats.  A slot is either a sum (hi,
// lo) or a maximum (hi; lo unused), chosen by bit s of `max_mask`; a sum
// whose bit is set in `exact_mask` holds small integers (cell counts) that
// float addition sums exactly, so it skips the error term.
#pragma once

#include <math.h>

#include "fg_internal.cuh"

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

#ifdef __CUDACC__
// x*x as an unevaluated float pair (exact).
__device__ __forceinline__ FF ff_sq(float x) {
  float p = x * x;
  return FF{p, __fmaf_rn(x, x, -p)};
}
#endif

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

#ifdef __CUDACC__
// Combines slot values of two threads / rows.
template <int NS, unsigned EXACT = 0u>
__device__ __forceinline__ void slots_merge(FF (&a)[NS], const FF (&b)[NS], unsigned max_mask) {
#pragma unroll
  for (int s = 0; s < NS; ++s) {
    if ((max_mask >> s) & 1u) {
      a[s].hi = fmaxf(a[s].hi, b[s].hi);
    } else if ((EXACT >> s) & 1u) {
      a[s].hi = a[s].hi + b[s].hi;
    } else {
      float t, e;
      two_sum(a[s].hi, b[s].hi, t, e);
      a[s].hi = t;
      a[s].lo = (a[s].lo + b[s].lo) + e;
    }
  }
}

template <int NS>
__device__ __forceinline__ void slots_identity(FF (&a)[NS], unsigned max_mask) {
#pragma unroll
  for (int s = 0; s < NS; ++s) a[s] = FF{((max_mask >> s) & 1u) ? -INFINITY : 0.0f, 0.0f};
}

template <int NS, unsigned EXACT = 0u>
__device__ __forceinline__ void warp_merge(FF (&v)[NS], unsigned max_mask) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    FF w[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      w[s].hi = __shfl_down_sync(0xffffffffu, v[s].hi, o);
      // Maxima and exact sums carry no error term.
      w[s].lo = ((max_mask | EXACT) >> s) & 1u ? 0.0f : __shfl_down_sync(0xffffffffu, v[s].lo, o);
    }
    slots_merge<NS, EXACT>(v, w, max_mask);
  }
}

// Reduces the per-thread slot values over the block (at most 32 warps) and
// writes the block's row (NS x {hi, lo}) from thread 0.  sh holds 64 * NS
// floats.  Every thread of the block must call it.
template <int NS, unsigned EXACT = 0u>
__device__ __forceinline__ void block_row(FF (&v)[NS], unsigned max_mask, float* sh, float* row) {
  const int tid = threadIdx.x + threadIdx.y * blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = (blockDim.x * blockDim.y + 31) >> 5;
  warp_merge<NS, EXACT>(v, max_mask);
  if (lane == 0) {
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      sh[(wid * NS + s) * 2] = v[s].hi;
      sh[(wid * NS + s) * 2 + 1] = v[s].lo;
    }
  }
  __syncthreads();
  if (wid == 0) {
    FF u[NS];
    if (lane < nw) {
#pragma unroll
      for (int s = 0; s < NS; ++s) u[s] = FF{sh[(lane * NS + s) * 2], sh[(lane * NS + s) * 2 + 1]};
    } else {
      slots_identity<NS>(u, max_mask);
    }
    warp_merge<NS, EXACT>(u, max_mask);
    if (lane == 0) {
#pragma unroll
      for (int s = 0; s < NS; ++s) {
        float h = u[s].hi, l = u[s].lo;
        if (!((max_mask >> s) & 1u)) two_sum(u[s].hi, u[s].lo, h, l);
        row[2 * s] = h;
        row[2 * s + 1] = l;
      }
    }
  }
}

// Combines rows [b*per, min(n, (b+1)*per)) of `in` into row b of `out`.
template <int NS>
__global__ void __launch_bounds__(1024)
    k_combine_rows(const float* __restrict__ in, int n, int per, unsigned max_mask,
                   float* __restrict__ out) {
  __shared__ float sh[64 * NS];
  FF v[NS];
  slots_identity<NS>(v, max_mask);
  int k1 = min(n, (int)blockIdx.x * per + per);
  for (int k = blockIdx.x * per + threadIdx.x; k < k1; k += blockDim.x) {
    FF w[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s)
      w[s] = FF{in[(size_t)k * 2 * NS + 2 * s], in[(size_t)k * 2 * NS + 2 * s + 1]};
    slots_merge<NS>(v, w, max_mask);
  }
  block_row<NS>(v, max_mask, sh, out + (size_t)blockIdx.x * 2 * NS);
}

// Two-level combine of n rows at `part`; the final row is written past the
// level-one rows in the same buffer and returned in *out_row.  Returns the
// number of kernels launched.
template <int NS>
inline int combine_rows(cudaStream_t st, float* part, int n, unsigned max_mask, float** out_row) {
  float* lvl = part + (size_t)2 * NS * n;
  const int per = 2048;
  if (n <= per) {
    k_combine_rows<NS><<<1, 1024, 0, st>>>(part, n, n, max_mask, lvl);
    *out_row = lvl;
    return 1;
  }
  int g = (n + per - 1) / per;
  k_combine_rows<NS><<<g, 1024, 0, st>>>(part, n, per, max_mask, lvl);
  float* out = lvl + (size_t)2 * NS * g;
  k_combine_rows<NS><<<1, 1024, 0, st>>>(lvl, g, g, max_mask, out);
  *out_row = out;
  return 2;
}

// Combines all n rows of `in` in one block -- thread k merges rows k,
// k + blockDim.x, ... in turn, then the block's fixed tree -- and hands the
// total row to store(row) on thread 0: the per-step statistics in one
// launch instead of a two-level combine and a store kernel.
template <int NS, typename Store>
__global__ void __launch_bounds__(1024)
    k_combine_store(const float* __restrict__ in, int n, unsigned max_mask, Store store) {
  __shared__ float sh[64 * NS];
  __shared__ float row[2 * NS];
  pdl_enter();
  FF v[NS];
  slots_identity<NS>(v, max_mask);
  // U rows' loads are issued before their merges (in the same order), so
  // a thread waits for one round trip per U rows instead of one per row.
  constexpr int U = NS > 2 ? 4 : 8;
  int k = threadIdx.x;
  for (; k + (U - 1) * (int)blockDim.x < n; k += U * blockDim.x) {
    FF w[U][NS];
#pragma unroll
    for (int q = 0; q < U; ++q) {
      const size_t r = (size_t)(k + q * blockDim.x) * 2 * NS;
#pragma unroll
      for (int s = 0; s < NS; ++s) w[q][s] = FF{in[r + 2 * s], in[r + 2 * s + 1]};
    }
#pragma unroll
    for (int q = 0; q < U; ++q) slots_merge<NS>(v, w[q], max_mask);
  }
  for (; k < n; k += blockDim.x) {
    FF w[NS];
#pragma unroll
    for (int s = 0; s < NS; ++s)
      w[s] = FF{in[(size_t)k * 2 * NS + 2 * s], in[(size_t)k * 2 * NS + 2 * s + 1]};
    slots_merge<NS>(v, w, max_mask);
  }
  block_row<NS>(v, max_mask, sh, row);  // thread 0 writes the row
  if (threadIdx.x == 0) store(row);
}

// Total of a sum slot of a final row, in FP64.
__device__ __forceinline__ double row_sum(const float* row, int s) {
  return (double)row[2 * s] + (double)row[2 * s + 1];
}
#endif

}  // namespace
}  // namespace fg
