// Pressure projection (pkg/fluid/fluid.go:144-234).
//
// Two schemes:
//  * LEXSOR reproduces solveSingleGrid / pressureJacobiIteration exactly: the
//    serial lexicographic SOR sweep in velocity form with the relaxation
//    schedule 1.9 -> 1.2 and the early exit on max|div| < tolerance.  Cell
//    (i, j) of a sweep depends on (i-1, j) and (i, j-1) of the same sweep and
//    on (i+1, j), (i, j+1) of the previous one, so the sweep runs as a
//    wavefront over anti-diagonals, with consecutive sweeps pipelined two
//    diagonals apart.  Every face sees the same sequence of floating-point
//    updates as in the serial loop, so the result is bit-identical.  The
//    wavefront runs on one block (k_lexsor) or an 8-block cluster
//    (k_lexsor_cl), on diagonal-major copies of the fields; the early exit
//    either waits, step by step, for the previous sweep to be known not to
//    exit, or runs speculatively (all sweeps, then an exact re-run of the
//    sweeps the serial loop makes when one falls below the tolerance).
//  * JACOBI relaxes the same masked Poisson system for the cell potential
//    phi (the accumulated per-cell correction of the SOR loop):
//        s_c phi_c - sum_n phi_n = -div_c,   phi = 0 off the active cells,
//    then applies U_face += S_R phi_L - S_L phi_R (and likewise V) and
//    p = cp * phi.  Sweeps run temporally blocked: a block relaxes a tile
//    with a halo as wide as its sweep count (8) in registers, so memory sees
//    one read and one write of phi per block of sweeps (k_jacobi_rb; fed by
//    TMA copies in k_jacobi_tma; a whole fixed-count solve as one cooperative
//    dataflow launch in k_jacobi_flow).  Optional outer correction: an
//    FP64-class residual of the FP32 iterate, a correction solve on it,
//    phi += e.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <mutex>

#include "fg_batch.cuh"
#include "fg_internal.cuh"
#include "fg_reduce.cuh"

namespace fg {

// Device control block of the parallel schemes.
struct PCtl {
  int stop;         // early-exit latch
  int sel;          // buffer holding the latest phi (0: phi, 1: phi2)
  int sweeps;       // sweeps executed
  int last_launch;  // index of the last executed launch
  int esel;         // buffer holding the latest correction (0: err, 1: err2)
  int pad[3];
  unsigned slots[1];  // per-launch max |r| of its last sweep (float bits)
};

namespace {

constexpr unsigned long long MBAR_WAIT_NS = 1000000000ull;  // 1 s
constexpr int MBAR_MAX_TRIES = 1 << 24;
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

constexpr int BX = 32, BY = 8;
inline dim3 cell_grid(const fg_fluid* f) {
  return dim3((f->NY + BX - 1) / BX, (f->NX + BY - 1) / BY);
}

// q / n and q % n for 0 <= q < 2^24, n > 0, from a float reciprocal and one
// correction step (exact: q and the candidate products are exact in float
// range, and the float quotient is off by at most one).
__device__ __forceinline__ int div_small(int q, int n, float inv_n, int& rem) {
  int t = __float2int_rz((float)q * inv_n);
  int r = q - t * n;
  if (r < 0) {
    --t;
    r += n;
  } else if (r >= n) {
    ++t;
    r -= n;
  }
  rem = r;
  return t;
}

// ------------------------------------------------------------------ LEXSOR
constexpr int LEX_THREADS = 1024;
constexpr int LEX_RING = 4096;  // sweeps in flight (a new sweep waits while the ring is full)
constexpr int LEX_CHUNK = 4;    // cells whose loads a thread issues together

__global__ void __launch_bounds__(LEX_THREADS)
    k_lexsor(float* U, float* V, float* p, const uint8_t* __restrict__ flags, Grid g,
             int numIters, float relax0, float damping, float cp, float tol, int early_exit,
             DevStats* st, float minRelax = 1.2f, const int* __restrict__ stop = nullptr,
             int SP = 0, int* __restrict__ exit_out = nullptr,
             const int* __restrict__ run_from = nullptr) {
  __shared__ int s_start[LEX_RING];
  __shared__ unsigned s_max[LEX_RING];
  __shared__ uint8_t s_cont[LEX_RING];
  __shared__ int s_lo, s_hi, s_done, s_exit, s_last;
  const int P = g.P;
  const int ni = g.NX - 2, nj = g.NY - 2;  // interior extent
  const int D = ni + nj - 1;               // anti-diagonals d = i + j in [2, NX+NY-4]
  // Row-major fields (SP = 0): cell (i, j) at i * P + j, its east face +P,
  // its north face +1.  Diagonal-major copies (SP > 0): cell (i, j) at
  // (i + j) * SP + i, east +SP+1, north +SP, so a step's accesses are
  // contiguous along the diagonal.
  const int offE = SP ? SP + 1 : P, offN = SP ? SP : 1;
  const int L = ni < nj ? ni : nj;         // longest diagonal
  if (threadIdx.x == 0) {
    s_lo = 0;
    s_hi = 0;
    s_done = 0;
    s_exit = 0;
    s_last = -1;
  }
  __syncthreads();
  if (numIters <= 0 || ni <= 0 || nj <= 0) return;
  if (stop && *stop) return;  // a multigrid solve that already converged
  // The cells of the W sweeps lo .. lo+W-1 that step tau reaches; sweep t is
  // on diagonal 2 + delta_of(t) (out of range: not running) and its max
  // |div| goes to s_max[r] (r = t mod LEX_RING).
  auto step = [&](long long tau, int lo, int W, auto delta_of, int runIters, bool all) {
      // Each warp takes 32 cells of one sweep's diagonal (the diagonal length
      // padded to a multiple of 32), so the sweep's max |div| and its
      // "cannot exit" mark are reduced in the warp and stored once per warp.
      // The cells a step updates share no face or pressure value (cells of one
      // diagonal are not neighbours; sweeps in flight are two diagonals
      // apart), so a thread loads the inputs of LEX_CHUNK cells at once and
      // then updates them: one memory round trip per chunk instead of one per
      // cell.
      const int Lp = (L + 31) & ~31;
      const float invLp = 1.0f / (float)Lp;
      const int items = W * Lp;
      for (int base = 0; base < items; base += LEX_CHUNK * LEX_THREADS) {
        int cc[LEX_CHUNK], rr[LEX_CHUNK], tt[LEX_CHUNK];
        bool act[LEX_CHUNK] = {};
        uint8_t fl[LEX_CHUNK];
        float u0[LEX_CHUNK], u1[LEX_CHUNK], v0[LEX_CHUNK], v1[LEX_CHUNK], p0[LEX_CHUNK];
#pragma unroll
        for (int m = 0; m < LEX_CHUNK; ++m) {
          if (base + m * LEX_THREADS >= items) break;  // (block-uniform)
          const int q = base + m * LEX_THREADS + (int)threadIdx.x;
          int k;
          const int t = lo + (items < (1 << 24) ? div_small(q, Lp, invLp, k) : (k = q % Lp, q / Lp));
          const int r = t & (LEX_RING - 1);
          const int delta = q < items ? delta_of(t) : -1;
          const int d = 2 + delta;
          const int i_lo = max(1, d - nj), i_hi = min(ni, d - 1);
          const int i = i_lo + k;
          const bool in = delta >= 0 && delta < D && k < L && i <= i_hi;
          const int c = in ? (SP ? d * SP + i : i * P + (d - i)) : 0;
          cc[m] = c;
          rr[m] = r;
          tt[m] = t;
          act[m] = in;
          fl[m] = in ? flags[c] : 0;
          u0[m] = in ? U[c] : 0.0f;
          u1[m] = in ? U[c + offE] : 0.0f;
          v0[m] = in ? V[c] : 0.0f;
          v1[m] = in ? V[c + offN] : 0.0f;
          p0[m] = in ? p[c] : 0.0f;
        }
#pragma unroll
        for (int m = 0; m < LEX_CHUNK; ++m) {
          if (base + m * LEX_THREADS >= items) break;  // (whole warps: items is a multiple of 32)
          const uint8_t f = fl[m];
          bool a = act[m] && (f & F_FLUID);
          const float sx0 = fbit(f, F_W), sx1 = fbit(f, F_E), sy0 = fbit(f, F_S),
                      sy1 = fbit(f, F_N);
          const float s = sx0 + sx1 + sy0 + sy1;
          a = a && s != 0.0f;
          const float div = a ? u1[m] - u0[m] + v1[m] - v0[m] : 0.0f;
          const float absDiv = fabsf(div);
          const bool counted = a && !isnan(absDiv);
          const unsigned mx = __reduce_max_sync(0xffffffffu, counted ? __float_as_uint(absDiv) : 0u);
          const bool cont = __any_sync(0xffffffffu, counted && absDiv >= tol);
          // (Without the early exit only the last sweep's max is reported,
          // and more sweeps than ring slots may be in flight.)
          if ((threadIdx.x & 31) == 0 && (early_exit || all || tt[m] == runIters - 1)) {
            if (mx) atomicMax(&s_max[rr[m]], mx);
            if (cont) s_cont[rr[m]] = 1;
          }
          if (!a) continue;
          const int c = cc[m];
          // Relaxation of sweep t (fluid.go:169-170).
          float iterProgress = (float)tt[m] / (float)numIters;
          float rel = relax0 - (relax0 - minRelax) * iterProgress;
          float pp = -div / s;
          pp *= rel;
          pp *= damping;
          p[c] = p0[m] + cp * pp;
          U[c] = u0[m] - sx0 * pp;
          U[c + offE] = u1[m] + sx1 * pp;
          V[c] = v0[m] - sy0 * pp;
          V[c + offN] = v1[m] + sy1 * pp;
        }
      }
  };
  if (!early_exit) {
    // Without the early exit sweep t always starts at step 2t (two steps
    // after the previous one, as the bookkeeping below would start it):
    // sweep t covers steps 2t .. 2t + D - 1 and the steps need no
    // bookkeeping between them, one barrier each.  With exit_out (the
    // speculative pass of an early-exit solve) every sweep's max |div| is
    // kept until the sweep retires and the first sweep below the tolerance
    // is recorded; with run_from (the re-run) only sweeps 0 .. *run_from run,
    // and nothing at all when no sweep was below it.
    int runIters = numIters;
    if (run_from) {
      const int e = *run_from;
      if (e < 0 || e >= numIters) return;
      runIters = e + 1;
    }
    for (int r = threadIdx.x; r < LEX_RING; r += LEX_THREADS) s_max[r] = 0u;
    __shared__ unsigned s_lastmax;
    if (threadIdx.x == 0) s_lastmax = 0u;
    __syncthreads();
    const long long steps = (long long)D + 2LL * (runIters - 1);
    for (long long tau = 0; tau < steps; ++tau) {
      int t_lo = (int)((tau - D + 2) / 2);
      if (t_lo < 0) t_lo = 0;
      while (tau - 2LL * t_lo >= D) ++t_lo;
      int t_hi = (int)(tau / 2);
      if (t_hi > runIters - 1) t_hi = runIters - 1;
      step(tau, t_lo, t_hi - t_lo + 1, [&](int t) { return (int)(tau - 2LL * t); }, runIters,
           exit_out != nullptr);
      __syncthreads();
      // The sweep whose last diagonal ran in this step retires.
      const long long rt = tau - (D - 1);
      if (threadIdx.x == 0 && rt >= 0 && (rt & 1) == 0 && rt / 2 < runIters) {
        const int t = (int)(rt / 2), r = t & (LEX_RING - 1);
        const unsigned m = s_max[r];
        if (exit_out && __uint_as_float(m) < tol) atomicMin(exit_out, t);
        if (t == runIters - 1) s_lastmax = m;
        s_max[r] = 0u;  // (slot reused by sweep t + LEX_RING, not yet started)
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      st->sweeps = runIters;
      st->last_maxdiv = (double)__uint_as_float(s_lastmax);
    }
    return;
  }
  // Start sweep 0 at step 0.
  if (threadIdx.x == 0) {
    s_start[0] = 0;
    s_max[0] = 0u;
    s_cont[0] = 0;
    s_hi = 1;
  }
  __syncthreads();
  // Bounded: each sweep takes D steps and starts at most D + 2 steps after
  // the previous one.
  const long long max_steps = (long long)numIters * (D + 2) + D + 4;
  for (long long tau = 0; tau < max_steps; ++tau) {
    const int lo = s_lo, hi = s_hi;
    step(tau, lo, hi - lo, [&](int t) { return (int)(tau - s_start[t & (LEX_RING - 1)]); },
         numIters, false);
    __syncthreads();
    if (threadIdx.x == 0) {
      // Retire sweeps whose last diagonal ran in this step.
      while (s_lo < s_hi && tau - s_start[s_lo & (LEX_RING - 1)] >= D - 1) {
        int r = s_lo & (LEX_RING - 1);
        s_last = s_lo;
        if (early_exit && __uint_as_float(s_max[r]) < tol) s_exit = 1;
        ++s_lo;
      }
      // Start the next sweep if allowed.
      int nxt = s_hi;
      if (!s_exit && nxt < numIters) {
        int pr = (nxt - 1) & (LEX_RING - 1);
        bool prev_done = s_lo > nxt - 1;
        bool gap_ok = prev_done || (tau + 1 - s_start[pr] >= 2);
        bool safe = !early_exit || prev_done || s_cont[pr];
        if (gap_ok && safe && nxt - s_lo < LEX_RING) {
          int r = nxt & (LEX_RING - 1);
          s_start[r] = (int)(tau + 1);
          s_max[r] = 0u;
          s_cont[r] = 0;
          s_hi = nxt + 1;
        }
      }
      if (s_lo == s_hi && (s_exit || s_hi >= numIters)) s_done = 1;
    }
    __syncthreads();
    if (s_done) break;
  }
  if (threadIdx.x == 0) {
    st->sweeps = s_hi;
    st->last_maxdiv = s_last >= 0 ? (double)__uint_as_float(s_max[s_last & (LEX_RING - 1)]) : 0.0;
  }
}

// ------------------------------------------------------------------ LEXSOR on a cluster
// k_lexsor's schedule on a thread-block cluster of LEX_CLUSTER blocks (one
// SM each): the cells of a step are spread over all of the cluster's
// threads and every step ends with a cluster barrier (release / acquire, so
// the steps' global stores are ordered for the whole cluster; the fields are
// read past L1).  The sweep bookkeeping (start steps, maxima, "cannot exit"
// marks, retire / start decisions) lives in the shared memory of block rank
// 0; the other blocks read and update it through distributed shared memory.
// With the early exit a step takes two cluster barriers (the step, then rank
// 0's decisions); without it the closed-form schedule needs one.
constexpr int LEX_CLUSTER = 8;

__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;"
               ::: "memory");
}
// Shared-window address of `p` (a shared variable) in block `rank` of the cluster.
__device__ __forceinline__ uint32_t cl_map(const void* p, unsigned rank) {
  uint32_t a;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(p)), "r"(rank));
  return a;
}
__device__ __forceinline__ int cl_ld(uint32_t a) {
  int v;
  asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ void cl_st8(uint32_t a, unsigned v) {
  asm volatile("st.shared::cluster.u8 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void cl_max(uint32_t a, unsigned v) {
  asm volatile("red.shared::cluster.max.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

__global__ void __launch_bounds__(LEX_THREADS)
    k_lexsor_cl(float* U, float* V, float* p, const uint8_t* __restrict__ flags, Grid g,
                int numIters, float relax0, float damping, float cp, float tol, int early_exit,
                DevStats* st, float minRelax, const int* __restrict__ stop, int SP,
                int* __restrict__ exit_out, const int* __restrict__ run_from) {
  __shared__ int s_start[LEX_RING];
  __shared__ unsigned s_max[LEX_RING];
  __shared__ uint8_t s_cont[LEX_RING];
  __shared__ int s_lo, s_hi, s_done, s_exit, s_last;
  const unsigned rank = cl_rank();
  const int P = g.P;
  const int ni = g.NX - 2, nj = g.NY - 2;
  const int D = ni + nj - 1;
  const int offE = SP ? SP + 1 : P, offN = SP ? SP : 1;
  const int L = ni < nj ? ni : nj;
  // Rank 0's bookkeeping, as seen from this block.
  const uint32_t a_start = cl_map(s_start, 0), a_max = cl_map(s_max, 0),
                 a_cont = cl_map(s_cont, 0), a_lo = cl_map(&s_lo, 0), a_hi = cl_map(&s_hi, 0),
                 a_done = cl_map(&s_done, 0);
  if (rank == 0) {
    for (int r = threadIdx.x; r < LEX_RING; r += LEX_THREADS) {
      s_max[r] = 0u;
      s_cont[r] = 0;
    }
    if (threadIdx.x == 0) {
      s_start[0] = 0;
      s_lo = 0;
      s_hi = 1;
      s_done = 0;
      s_exit = 0;
      s_last = -1;
    }
  }
  cl_sync();
  if (numIters <= 0 || ni <= 0 || nj <= 0) return;  // (the same in every block)
  if (stop && *stop) return;
  const int gt = (int)rank * LEX_THREADS + (int)threadIdx.x;
  const int stride = LEX_CLUSTER * LEX_THREADS;
  const int Lp = (L + 31) & ~31;
  const float invLp = 1.0f / (float)Lp;
  auto step = [&](long long tau, int lo, int W, auto delta_of, int runIters, bool all) {
    const int items = W * Lp;
    for (int base = 0; base < items; base += LEX_CHUNK * stride) {
      int cc[LEX_CHUNK], rr[LEX_CHUNK], tt[LEX_CHUNK];
      bool act[LEX_CHUNK] = {};
      uint8_t fl[LEX_CHUNK];
      float u0[LEX_CHUNK], u1[LEX_CHUNK], v0[LEX_CHUNK], v1[LEX_CHUNK], p0[LEX_CHUNK];
#pragma unroll
      for (int m = 0; m < LEX_CHUNK; ++m) {
        if (base + m * stride >= items) break;  // (uniform over the cluster)
        const int q = base + m * stride + gt;
        int k;
        const int t = lo + (items < (1 << 24) ? div_small(q, Lp, invLp, k) : (k = q % Lp, q / Lp));
        const int r = t & (LEX_RING - 1);
        const int delta = q < items ? delta_of(t) : -1;
        const int d = 2 + delta;
        const int i_lo = max(1, d - nj), i_hi = min(ni, d - 1);
        const int i = i_lo + k;
        const bool in = delta >= 0 && delta < D && k < L && i <= i_hi;
        const int c = in ? (SP ? d * SP + i : i * P + (d - i)) : 0;
        cc[m] = c;
        rr[m] = r;
        tt[m] = t;
        act[m] = in;
        fl[m] = in ? __ldcg(flags + c) : 0;
        u0[m] = in ? __ldcg(U + c) : 0.0f;
        u1[m] = in ? __ldcg(U + c + offE) : 0.0f;
        v0[m] = in ? __ldcg(V + c) : 0.0f;
        v1[m] = in ? __ldcg(V + c + offN) : 0.0f;
        p0[m] = in ? __ldcg(p + c) : 0.0f;
      }
#pragma unroll
      for (int m = 0; m < LEX_CHUNK; ++m) {
        if (base + m * stride >= items) break;  // (whole warps: items is a multiple of 32)
        const uint8_t f = fl[m];
        bool a = act[m] && (f & F_FLUID);
        const float sx0 = fbit(f, F_W), sx1 = fbit(f, F_E), sy0 = fbit(f, F_S),
                    sy1 = fbit(f, F_N);
        const float s = sx0 + sx1 + sy0 + sy1;
        a = a && s != 0.0f;
        const float div = a ? u1[m] - u0[m] + v1[m] - v0[m] : 0.0f;
        const float absDiv = fabsf(div);
        const bool counted = a && !isnan(absDiv);
        const unsigned mx = __reduce_max_sync(0xffffffffu, counted ? __float_as_uint(absDiv) : 0u);
        const bool cont = __any_sync(0xffffffffu, counted && absDiv >= tol);
        if ((threadIdx.x & 31) == 0 && (early_exit || all || tt[m] == runIters - 1)) {
          if (mx) cl_max(a_max + 4u * rr[m], mx);
          if (cont) cl_st8(a_cont + (unsigned)rr[m], 1u);
        }
        if (!a) continue;
        const int c = cc[m];
        // Relaxation of sweep t (fluid.go:169-170).
        float iterProgress = (float)tt[m] / (float)numIters;
        float rel = relax0 - (relax0 - minRelax) * iterProgress;
        float pp = -div / s;
        pp *= rel;
        pp *= damping;
        p[c] = p0[m] + cp * pp;
        U[c] = u0[m] - sx0 * pp;
        U[c + offE] = u1[m] + sx1 * pp;
        V[c] = v0[m] - sy0 * pp;
        V[c + offN] = v1[m] + sy1 * pp;
      }
    }
  };
  if (!early_exit) {
    // The closed-form schedule, as in k_lexsor (exit_out / run_from alike);
    // rank 0's thread 0 retires the sweeps.
    int runIters = numIters;
    if (run_from) {
      const int e = *run_from;
      if (e < 0 || e >= numIters) {
        cl_sync();
        return;
      }
      runIters = e + 1;
    }
    const long long steps = (long long)D + 2LL * (runIters - 1);
    for (long long tau = 0; tau < steps; ++tau) {
      int t_lo = (int)((tau - D + 2) / 2);
      if (t_lo < 0) t_lo = 0;
      while (tau - 2LL * t_lo >= D) ++t_lo;
      int t_hi = (int)(tau / 2);
      if (t_hi > runIters - 1) t_hi = runIters - 1;
      step(tau, t_lo, t_hi - t_lo + 1, [&](int t) { return (int)(tau - 2LL * t); }, runIters,
           exit_out != nullptr);
      cl_sync();
      const long long rt = tau - (D - 1);
      if (rank == 0 && threadIdx.x == 0 && rt >= 0 && (rt & 1) == 0 && rt / 2 < runIters) {
        const int t = (int)(rt / 2), r = t & (LEX_RING - 1);
        const unsigned m = s_max[r];
        if (exit_out && __uint_as_float(m) < tol) atomicMin(exit_out, t);
        if (t == runIters - 1) s_last = (int)m;
        s_max[r] = 0u;  // (slot reused by sweep t + LEX_RING, not yet started)
      }
    }
    cl_sync();
    if (rank == 0 && threadIdx.x == 0) {
      st->sweeps = runIters;
      st->last_maxdiv = (double)__uint_as_float((unsigned)s_last);
    }
    cl_sync();  // (no block leaves while others may still address rank 0)
    return;
  }
  const long long max_steps = (long long)numIters * (D + 2) + D + 4;
  for (long long tau = 0; tau < max_steps; ++tau) {
    const int lo = cl_ld(a_lo), hi = cl_ld(a_hi);
    step(tau, lo, hi - lo,
         [&](int t) { return (int)(tau - cl_ld(a_start + 4u * (t & (LEX_RING - 1)))); },
         numIters, false);
    cl_sync();
    if (rank == 0 && threadIdx.x == 0) {
      // Retire sweeps whose last diagonal ran in this step.
      while (s_lo < s_hi && tau - s_start[s_lo & (LEX_RING - 1)] >= D - 1) {
        int r = s_lo & (LEX_RING - 1);
        s_last = s_lo;
        if (__uint_as_float(s_max[r]) < tol) s_exit = 1;
        ++s_lo;
      }
      // Start the next sweep if allowed.
      int nxt = s_hi;
      if (!s_exit && nxt < numIters) {
        int pr = (nxt - 1) & (LEX_RING - 1);
        bool prev_done = s_lo > nxt - 1;
        bool gap_ok = prev_done || (tau + 1 - s_start[pr] >= 2);
        bool safe = prev_done || s_cont[pr];
        if (gap_ok && safe && nxt - s_lo < LEX_RING) {
          int r = nxt & (LEX_RING - 1);
          s_start[r] = (int)(tau + 1);
          s_max[r] = 0u;
          s_cont[r] = 0;
          s_hi = nxt + 1;
        }
      }
      if (s_lo == s_hi && (s_exit || s_hi >= numIters)) s_done = 1;
    }
    cl_sync();
    if (cl_ld(a_done)) break;
  }
  if (rank == 0 && threadIdx.x == 0) {
    st->sweeps = s_hi;
    st->last_maxdiv = s_last >= 0 ? (double)__uint_as_float(s_max[s_last & (LEX_RING - 1)]) : 0.0;
  }
  cl_sync();
}

// ------------------------------------------------------------------ LEXSOR on the whole GPU
// The closed-form schedule (no early exit, or the speculative early exit's
// two passes) over every SM: a cooperative launch of one block per SM, a
// grid barrier per step.  For solves with many sweeps in flight (a step
// then holds hundreds of thousands of cells: the reference's 200-sweep
// workload at 2048^2) the step is compute-bound and the cluster's 8 SMs are
// too few.  Scratch (lex): [0, LEX_RING) the sweeps' maxima, then the
// barrier's arrival count and generation, then its give-up flag.
constexpr int LEX_GRID_SCRATCH = LEX_RING + 4;

// A grid barrier: the block's last arrival advances the generation; the
// others wait for it, for at most about a second (then *fail is set and
// they go on; the solve's result is then not to be used).  Release / acquire
// at GPU scope around it order the steps' stores.
__device__ __forceinline__ void grid_barrier(unsigned* count, unsigned* gen, unsigned nblocks,
                                             int* fail) {
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned g0;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(g0) : "l"(gen) : "memory");
    __threadfence();
    if (atomicAdd(count, 1u) == nblocks - 1) {
      *count = 0u;
      __threadfence();
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(gen) : "memory");
    } else {
      const unsigned long long t0 = global_ns();
      for (int it = 0; it < MBAR_MAX_TRIES; ++it) {
        unsigned gv;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(gv) : "l"(gen) : "memory");
        if (gv != g0) break;
        if (global_ns() - t0 > MBAR_WAIT_NS) {
          atomicExch(fail, 1);
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
}

__global__ void __launch_bounds__(LEX_THREADS)
    k_lexsor_grid(float* U, float* V, float* p, const uint8_t* __restrict__ flags, Grid g,
                  int numIters, float relax0, float damping, float cp, float tol, DevStats* st,
                  float minRelax, int SP, int* __restrict__ exit_out,
                  const int* __restrict__ run_from, unsigned* __restrict__ lex, int* err) {
  const int P = g.P;
  const int ni = g.NX - 2, nj = g.NY - 2;
  const int D = ni + nj - 1;
  const int offE = SP ? SP + 1 : P, offN = SP ? SP : 1;
  const int L = ni < nj ? ni : nj;
  unsigned* gmax = lex;
  unsigned* bcount = lex + LEX_RING;
  unsigned* bgen = lex + LEX_RING + 1;
  int* bfail = reinterpret_cast<int*>(lex + LEX_RING + 2);
  const unsigned nb = gridDim.x;
  if (numIters <= 0 || ni <= 0 || nj <= 0) return;  // (the same in every block)
  int runIters = numIters;
  if (run_from) {
    const int e = *run_from;
    if (e < 0 || e >= numIters) return;
    runIters = e + 1;
  }
  // (gmax and the barrier words were zeroed before the launch.)
  const int gt = (int)blockIdx.x * LEX_THREADS + (int)threadIdx.x;
  const int stride = (int)nb * LEX_THREADS;
  const int Lp = (L + 31) & ~31;
  const float invLp = 1.0f / (float)Lp;
  const long long steps = (long long)D + 2LL * (runIters - 1);
  for (long long tau = 0; tau < steps; ++tau) {
    int t_lo = (int)((tau - D + 2) / 2);
    if (t_lo < 0) t_lo = 0;
    while (tau - 2LL * t_lo >= D) ++t_lo;
    int t_hi = (int)(tau / 2);
    if (t_hi > runIters - 1) t_hi = runIters - 1;
    const int lo = t_lo, W = t_hi - t_lo + 1;
    const int items = W * Lp;
    for (int base = 0; base < items; base += LEX_CHUNK * stride) {
      int cc[LEX_CHUNK], rr[LEX_CHUNK], tt[LEX_CHUNK];
      bool act[LEX_CHUNK] = {};
      uint8_t fl[LEX_CHUNK];
      float u0[LEX_CHUNK], u1[LEX_CHUNK], v0[LEX_CHUNK], v1[LEX_CHUNK], p0[LEX_CHUNK];
#pragma unroll
      for (int m = 0; m < LEX_CHUNK; ++m) {
        if (base + m * stride >= items) break;  // (uniform over the grid)
        const int q = base + m * stride + gt;
        int k;
        const int t = lo + (items < (1 << 24) ? div_small(q, Lp, invLp, k) : (k = q % Lp, q / Lp));
        const int r = t & (LEX_RING - 1);
        const int delta = q < items ? (int)(tau - 2LL * t) : -1;
        const int d = 2 + delta;
        const int i_lo = max(1, d - nj), i_hi = min(ni, d - 1);
        const int i = i_lo + k;
        const bool in = delta >= 0 && delta < D && k < L && i <= i_hi;
        const int c = in ? (SP ? d * SP + i : i * P + (d - i)) : 0;
        cc[m] = c;
        rr[m] = r;
        tt[m] = t;
        act[m] = in;
        fl[m] = in ? __ldcg(flags + c) : 0;
        u0[m] = in ? __ldcg(U + c) : 0.0f;
        u1[m] = in ? __ldcg(U + c + offE) : 0.0f;
        v0[m] = in ? __ldcg(V + c) : 0.0f;
        v1[m] = in ? __ldcg(V + c + offN) : 0.0f;
        p0[m] = in ? __ldcg(p + c) : 0.0f;
      }
#pragma unroll
      for (int m = 0; m < LEX_CHUNK; ++m) {
        if (base + m * stride >= items) break;  // (the slots the loads filled)
        const uint8_t f = fl[m];
        bool a = act[m] && (f & F_FLUID);
        const float sx0 = fbit(f, F_W), sx1 = fbit(f, F_E), sy0 = fbit(f, F_S),
                    sy1 = fbit(f, F_N);
        const float s = sx0 + sx1 + sy0 + sy1;
        a = a && s != 0.0f;
        const float div = a ? u1[m] - u0[m] + v1[m] - v0[m] : 0.0f;
        const float absDiv = fabsf(div);
        const bool counted = a && !isnan(absDiv);
        const unsigned mx = __reduce_max_sync(0xffffffffu, counted ? __float_as_uint(absDiv) : 0u);
        if ((threadIdx.x & 31) == 0 && mx && (exit_out || tt[m] == runIters - 1))
          atomicMax(&gmax[rr[m]], mx);
        if (!a) continue;
        const int c = cc[m];
        // Relaxation of sweep t (fluid.go:169-170).
        float iterProgress = (float)tt[m] / (float)numIters;
        float rel = relax0 - (relax0 - minRelax) * iterProgress;
        float pp = -div / s;
        pp *= rel;
        pp *= damping;
        p[c] = p0[m] + cp * pp;
        U[c] = u0[m] - sx0 * pp;
        U[c + offE] = u1[m] + sx1 * pp;
        V[c] = v0[m] - sy0 * pp;
        V[c + offN] = v1[m] + sy1 * pp;
      }
    }
    grid_barrier(bcount, bgen, nb, bfail);
    // Block 0 retires the sweep whose last diagonal ran in this step (its
    // slot is next used LEX_RING sweeps later).
    const long long rt = tau - (D - 1);
    if (blockIdx.x == 0 && threadIdx.x == 0 && rt >= 0 && (rt & 1) == 0 && rt / 2 < runIters) {
      const int t = (int)(rt / 2), r = t & (LEX_RING - 1);
      const unsigned m = atomicExch(&gmax[r], 0u);
      if (exit_out && __uint_as_float(m) < tol) atomicMin(exit_out, t);
      if (t == runIters - 1) {
        st->sweeps = runIters;
        st->last_maxdiv = (double)__uint_as_float(m);
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && *bfail) atomicExch(err, 1);
}

// Copies of U, V, p and the flags into the diagonal-major layout of the
// wavefront kernel (cell (i, j) at (i + j) * SP + i) and of U, V, p back.
__global__ void k_skew_in(const float* __restrict__ U, const float* __restrict__ V,
                          const float* __restrict__ p, const uint8_t* __restrict__ flags,
                          float* __restrict__ sU, float* __restrict__ sV, float* __restrict__ sp,
                          uint8_t* __restrict__ sf, Grid g, int SP,
                          const int* __restrict__ only_if = nullptr, int limit = 0) {
  if (only_if && *only_if >= limit) return;  // (the re-run copy: only when it runs)
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const size_t c = (size_t)i * g.P + j, s = (size_t)(i + j) * SP + i;
  sU[s] = U[c];
  sV[s] = V[c];
  sp[s] = p[c];
  sf[s] = flags[c];
}
__global__ void k_skew_out(const float* __restrict__ sU, const float* __restrict__ sV,
                           const float* __restrict__ sp, float* __restrict__ U,
                           float* __restrict__ V, float* __restrict__ p, Grid g, int SP) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const size_t c = (size_t)i * g.P + j, s = (size_t)(i + j) * SP + i;
  U[c] = sU[s];
  V[c] = sV[s];
  p[c] = sp[s];
}

// ------------------------------------------------------------------ multigrid
// solveMultigridVCycle (fluid.go:559-594) with its helpers (fluid.go:596-758,
// 1122-1149): per iteration three SOR sweeps at relaxation 1.5 (k_lexsor),
// the early exit on the last sweep's max |div|, the residual restricted by
// full weighting to the (NX+1)/2 x (NY+1)/2 grid, 40 lexicographic
// Gauss-Seidel sweeps there at relaxation 1.6, the bilinear prolongation
// applied to p and the faces, three SOR sweeps at 1.2.  Every stage keeps
// the reference's per-cell operation order; the serial loops become a
// wavefront (the SOR sweeps, the coarse sweeps) or a per-face kernel that
// applies a face's two updates in the loop's order (the correction).  Once
// a solve exits early, *stop makes every later kernel of it return.

// After the three pre-smoothing sweeps: count them and latch the exit when
// the last one's max |div| is below the tolerance.
__global__ void k_mg_check(const DevStats* __restrict__ sm, DevStats* st, int* stop, float tol,
                           int post) {
  if (*stop) return;
  st->sweeps += 3;
  if (post) return;
  float maxDiv = (float)sm->last_maxdiv;
  st->last_maxdiv = sm->last_maxdiv;
  if (maxDiv < tol) *stop = 1;
}

// computePressureResidual (fluid.go:596-628): r = -div - laplacian(p) on
// fluid interior cells, 0 elsewhere.
__global__ void k_mg_residual(const float* __restrict__ U, const float* __restrict__ V,
                              const float* __restrict__ p, const uint8_t* __restrict__ flags,
                              float* __restrict__ r, const int* __restrict__ stop, Grid g) {
  if (*stop) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const int P = g.P;
  int c = i * P + j;
  uint8_t fl = flags[c];
  float out = 0.0f;
  if ((fl & (F_FLUID | F_INTERIOR)) == (F_FLUID | F_INTERIOR)) {
    float div = U[c + P] - U[c] + V[c + 1] - V[c];
    float sx0 = fbit(fl, F_W), sx1 = fbit(fl, F_E), sy0 = fbit(fl, F_S), sy1 = fbit(fl, F_N);
    float lap = sx0 * (p[c - P] - p[c]) + sx1 * (p[c + P] - p[c]) + sy0 * (p[c - 1] - p[c]) +
                sy1 * (p[c + 1] - p[c]);
    out = -div - lap;
  }
  r[c] = out;
}

// restrictResidual (fluid.go:630-660) into the coarse grid (pitch cP = cNY).
// Coarse-grid index of cell (i, j): row-major i * cNY + j (CSP = 0) or
// diagonal-major (i + j) * CSP + i.
__device__ __forceinline__ int cidx(int i, int j, int cNY, int CSP) {
  return CSP ? (i + j) * CSP + i : i * cNY + j;
}

// The coarse solid mask: the fine cell (2i, 2j) (fluid.go:672-685).
__device__ __forceinline__ float coarse_s(const uint8_t* __restrict__ flags, int i, int j,
                                          const Grid& g) {
  int fi = 2 * i, fj = 2 * j;
  if (fi >= g.NX || fj >= g.NY) return 0.0f;
  return (flags[fi * g.P + fj] & F_FLUID) ? 1.0f : 0.0f;
}

// restrictResidual (fluid.go:630-660) into cr at cidx; with CSP > 0 also the
// coarse mask of every coarse cell into cmask (same layout).
__global__ void k_mg_restrict(const float* __restrict__ r, float* __restrict__ cr,
                              const int* __restrict__ stop, Grid g, int cNX, int cNY, int CSP,
                              const uint8_t* __restrict__ flags, uint8_t* __restrict__ cmask) {
  if (*stop) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= cNX || j >= cNY) return;
  float out = 0.0f;
  int fi = 2 * i, fj = 2 * j;
  if (i >= 1 && i < cNX - 1 && j >= 1 && j < cNY - 1 && fi < g.NX - 1 && fj < g.NY - 1) {
    const int P = g.P;
    int c = fi * P + fj;
    float center = r[c] * 0.25f;
    float nb = (r[c - P] + r[c + P] + r[c - 1] + r[c + 1]) * 0.125f;
    float cr4 = (r[c - P - 1] + r[c + P - 1] + r[c - P + 1] + r[c + P + 1]) * 0.0625f;
    out = center + nb + cr4;
  }
  const int ci = cidx(i, j, cNY, CSP);
  cr[ci] = out;
  if (CSP) cmask[ci] = coarse_s(flags, i, j, g) != 0.0f ? 1 : 0;
}

// solveCoarseGrid (fluid.go:662-715): 40 lexicographic Gauss-Seidel sweeps
// from zero, in one block.  Cell (i, j) of a sweep needs (i-1, j), (i, j-1)
// of that sweep and (i+1, j), (i, j+1) of the previous one, so the sweeps
// run as anti-diagonal wavefronts, each two diagonals behind the previous.
constexpr int MG_THREADS = 1024;
constexpr int MG_CHUNK = 4;  // cells whose loads a thread issues together
// CLUSTER: the same schedule on a thread-block cluster of LEX_CLUSTER blocks
// (a step's cells over all of its threads, a cluster barrier per step, the
// solution read past L1), for coarse grids whose steps hold many cells.
template <bool CLUSTER>
__global__ void __launch_bounds__(MG_THREADS)
    k_mg_coarse(const float* __restrict__ cr, float* __restrict__ cp_,
                const uint8_t* __restrict__ flags, const int* __restrict__ stop, Grid g, int cNX,
                int cNY, int sweeps, float relaxation, int CSP,
                const uint8_t* __restrict__ cmask) {
  if (*stop) return;  // (the same in every block)
  const int ni = cNX - 2, nj = cNY - 2;
  // Row-major (CSP = 0): neighbours at -cNY, +cNY, -1, +1.  Diagonal-major:
  // west -(CSP+1), east +(CSP+1), south -CSP, north +CSP, and the cells of a
  // step contiguous along their diagonal.
  const int oW = CSP ? CSP + 1 : cNY, oS = CSP ? CSP : 1;
  const int n0 = CSP ? (cNX + cNY - 1) * CSP : cNX * cNY;
  const int gt = CLUSTER ? (int)cl_rank() * MG_THREADS + (int)threadIdx.x : (int)threadIdx.x;
  const int stride = CLUSTER ? LEX_CLUSTER * MG_THREADS : MG_THREADS;
  auto barrier = [] {
    if (CLUSTER)
      cl_sync();
    else
      __syncthreads();
  };
  for (int k = gt; k < n0; k += stride) cp_[k] = 0.0f;
  barrier();
  if (ni <= 0 || nj <= 0) return;
  const int D = ni + nj - 1;
  const int L = ni < nj ? ni : nj;
  const float invL = 1.0f / (float)L;
  const long long steps = (long long)D + 2LL * (sweeps - 1);
  for (long long tau = 0; tau < steps; ++tau) {
    // Sweeps t with 0 <= tau - 2t < D, each on diagonal d = tau - 2t + 2.
    int t_lo = (int)((tau - D + 2) / 2);
    if (t_lo < 0) t_lo = 0;
    while (tau - 2LL * t_lo >= D) ++t_lo;
    int t_hi = (int)(tau / 2);
    if (t_hi > sweeps - 1) t_hi = sweeps - 1;
    int nact = t_hi - t_lo + 1;
    // The cells of a step are independent (one diagonal per sweep in flight,
    // sweeps two diagonals apart, no cell reads another's value): a thread
    // loads the inputs of MG_CHUNK cells at once, then updates them.
    const int items = nact * L;
    for (int base = 0; base < items; base += MG_CHUNK * stride) {
      int cc[MG_CHUNK];
      bool in[MG_CHUNK] = {};  // (slots past the step's cells stay out)
      float s0[MG_CHUNK], s1[MG_CHUNK], s2[MG_CHUNK], s3[MG_CHUNK], sc[MG_CHUNK];
      float pc[MG_CHUNK], pw[MG_CHUNK], pe[MG_CHUNK], ps[MG_CHUNK], pn[MG_CHUNK], rc[MG_CHUNK];
#pragma unroll
      for (int m = 0; m < MG_CHUNK; ++m) {
        if (base + m * stride >= items) break;  // (uniform over the block or cluster)
        const int q = base + m * stride + gt;
        int k;
        const int t = t_lo + (items < (1 << 24) ? div_small(q, L, invL, k) : (k = q % L, q / L));
        const int d = (int)(tau - 2LL * t) + 2;
        const int i_lo = max(1, d - nj), i_hi = min(ni, d - 1);
        const int i = i_lo + k;
        const bool ok = q < items && i <= i_hi;
        const int j = d - i;
        const int c = ok ? cidx(i, j, cNY, CSP) : 0;
        cc[m] = c;
        in[m] = ok;
        if (CSP) {
          sc[m] = ok ? (float)cmask[c] : 0.0f;
          s0[m] = ok ? (float)cmask[c - oW] : 0.0f;
          s1[m] = ok ? (float)cmask[c + oW] : 0.0f;
          s2[m] = ok ? (float)cmask[c - oS] : 0.0f;
          s3[m] = ok ? (float)cmask[c + oS] : 0.0f;
        } else {
          sc[m] = ok ? coarse_s(flags, i, j, g) : 0.0f;
          s0[m] = ok ? coarse_s(flags, i - 1, j, g) : 0.0f;
          s1[m] = ok ? coarse_s(flags, i + 1, j, g) : 0.0f;
          s2[m] = ok ? coarse_s(flags, i, j - 1, g) : 0.0f;
          s3[m] = ok ? coarse_s(flags, i, j + 1, g) : 0.0f;
        }
        auto ld = [&](int a) { return CLUSTER ? __ldcg(cp_ + a) : cp_[a]; };
        pc[m] = ok ? ld(c) : 0.0f;
        pw[m] = ok ? ld(c - oW) : 0.0f;
        pe[m] = ok ? ld(c + oW) : 0.0f;
        ps[m] = ok ? ld(c - oS) : 0.0f;
        pn[m] = ok ? ld(c + oS) : 0.0f;
        rc[m] = ok ? cr[c] : 0.0f;
      }
#pragma unroll
      for (int m = 0; m < MG_CHUNK; ++m) {
        if (base + m * stride >= items) break;  // (the slots the loads filled)
        if (!in[m] || sc[m] == 0.0f) continue;
        const float sx0 = s0[m], sx1 = s1[m], sy0 = s2[m], sy1 = s3[m];
        const float s = sx0 + sx1 + sy0 + sy1;
        if (s == 0.0f) continue;
        const float p0 = pc[m];
        float lap = sx0 * (pw[m] - p0) + sx1 * (pe[m] - p0) + sy0 * (ps[m] - p0) +
                    sy1 * (pn[m] - p0);
        float residual = rc[m] - lap;
        float correction = -residual / s * relaxation;
        cp_[cc[m]] = p0 + correction;
      }
    }
    barrier();
  }
}

// prolongateCorrection (fluid.go:717-758) at fine cell (i, j).
__device__ __forceinline__ float mg_corr(const float* __restrict__ cc, int i, int j, int cNX,
                                         int cNY, int CSP) {
  int ci = i / 2, cj = j / 2;
  if (ci >= cNX - 1 || cj >= cNY - 1) return 0.0f;
  float fI = (float)(i % 2) * 0.5f, fJ = (float)(j % 2) * 0.5f;
  return (1.0f - fI) * (1.0f - fJ) * cc[cidx(ci, cj, cNY, CSP)] +
         fI * (1.0f - fJ) * cc[cidx(ci + 1, cj, cNY, CSP)] +
         (1.0f - fI) * fJ * cc[cidx(ci, cj + 1, cNY, CSP)] +
         fI * fJ * cc[cidx(ci + 1, cj + 1, cNY, CSP)];
}

// applePressureCorrection (fluid.go:1122-1149): p += corr * cp on fluid
// interior cells; face (i, j) of U first gets + S_i corr(i-1, j) from cell
// (i-1, j), then - S_{i-1} corr(i, j) from cell (i, j), as the loop visits
// them; V likewise along j.
__global__ void k_mg_apply(float* __restrict__ U, float* __restrict__ V, float* __restrict__ p,
                           const float* __restrict__ cc, const uint8_t* __restrict__ flags,
                           const int* __restrict__ stop, float cp, Grid g, int cNX, int cNY,
                           int CSP) {
  if (*stop) return;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const int P = g.P;
  int c = i * P + j;
  auto fluid_int = [&](int a, int b) {
    return a >= 1 && a <= g.NX - 2 && b >= 1 && b <= g.NY - 2 &&
           (flags[a * P + b] & F_FLUID) != 0;
  };
  bool self = fluid_int(i, j);
  float corr = self ? mg_corr(cc, i, j, cNX, cNY, CSP) : 0.0f;
  if (self) p[c] += corr * cp;
  uint8_t fl = flags[c];
  if (i >= 1) {
    float u = U[c];
    if (fluid_int(i - 1, j)) u += fbit(fl, F_FLUID) * mg_corr(cc, i - 1, j, cNX, cNY, CSP);
    if (self) u -= fbit(fl, F_W) * corr;
    U[c] = u;
  }
  if (j >= 1) {
    float v = V[c];
    if (fluid_int(i, j - 1)) v += fbit(fl, F_FLUID) * mg_corr(cc, i, j - 1, cNX, cNY, CSP);
    if (self) v -= fbit(fl, F_S) * corr;
    V[c] = v;
  }
}

// ------------------------------------------------------------------ parallel scheme
struct WTab {
  float w[5];  // w[s] = (omega * damping) / s
};

// Per cell: b = -div, w = om / s and bw = w * b on active cells, all 0
// elsewhere (ring included); phi = 0 when `zero_phi` (a solve with no sweeps
// reads it directly).
// U, V use the grid pitch g.P, the solver arrays the pitch Ps.
// U + Fu at face u (the force field of a recorded step, null otherwise).
__device__ __forceinline__ float with_force(const float* __restrict__ U,
                                            const float* __restrict__ F, int u) {
  return F ? U[u] + F[u] : U[u];
}

__device__ __forceinline__ void setup_cell_p(int i, int j, const float* __restrict__ U,
                                             const float* __restrict__ V, float* __restrict__ phi,
                                             float* __restrict__ rhs, float* __restrict__ W,
                                             float* __restrict__ BW,
                                             const uint8_t* __restrict__ flags, float om,
                                             int zero_phi, const Grid& g, int Ps,
                                             const float* __restrict__ Fu = nullptr,
                                             const float* __restrict__ Fv = nullptr) {
  int u = i * g.P + j;
  int c = i * Ps + j;
  float b = 0.0f, w = 0.0f, bw = 0.0f;
  uint8_t fl = flags[c];
  // Active cells are interior.  Below the last row and column the four face
  // loads are in range whatever the flags say, so they issue beside the flag
  // load and the flags only select the result.
  if (i <= g.NX - 2 && j <= g.NY - 2) {
    float div = with_force(U, Fu, u + g.P) - with_force(U, Fu, u) + with_force(V, Fv, u + 1) -
                with_force(V, Fv, u);
    bool act = flag_active(fl);
    b = act ? -div : 0.0f;
    w = act ? om / (float)flag_count(fl) : 0.0f;
    bw = w * b;
  }
  rhs[c] = b;
  W[c] = w;
  BW[c] = bw;
  if (zero_phi) phi[c] = 0.0f;
}
__device__ __forceinline__ void setup_cell(int i, int j, const float* __restrict__ U,
                                           const float* __restrict__ V, float* __restrict__ phi,
                                           float* __restrict__ rhs, float* __restrict__ W,
                                           float* __restrict__ BW,
                                           const uint8_t* __restrict__ flags, float om,
                                           int zero_phi, const Grid& g) {
  setup_cell_p(i, j, U, V, phi, rhs, W, BW, flags, om, zero_phi, g, g.P);
}
__global__ void k_setup_system(const float* __restrict__ U, const float* __restrict__ V,
                               float* __restrict__ phi, float* __restrict__ rhs,
                               float* __restrict__ W, float* __restrict__ BW,
                               const uint8_t* __restrict__ flags, float om, int zero_phi, Grid g,
                               int Ps, const float* __restrict__ Fu, const float* __restrict__ Fv) {
  pdl_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  setup_cell_p(i, j, U, V, phi, rhs, W, BW, flags, om, zero_phi, g, Ps, Fu, Fv);
}

// Register-blocked, temporally blocked Jacobi.  A CTA of 8 warps holds a
// 64 x 128 region (rows i x columns j) in registers: each thread a block of
// RT = 8 rows by JT = 4 consecutive columns.  Vertical neighbours come from
// the thread's own rows, or through shared memory from the warp above/below
// at its first/last row; horizontal neighbours from the thread's own columns
// or a warp shuffle.  `ns` <= H sweeps run per launch; inside the grid the
// region carries a halo of H = 8 cells, so the CTA owns the inner 48 x 112
// cells, and at the grid's edges it owns up to the edge (span_count and
// span_own, fg_internal.cuh); it writes only what it owns.  Cells outside
// the grid or inactive have w = bw = 0 and stay 0.  The TMA-fed kernels
// below keep regions at t S - H with the inner 48 x 112 owned.  Launch k
// first decides whether the solve already stopped
// (thread 0 of every CTA reads the same control words, so all CTAs agree);
// a running launch records the max |r| of its last sweep over the active
// cells it owns, r = fma(-s, phi, b + nb), in slots[k].
constexpr int JT = 4, RT = 8, NWARP = 8, TMAX = 8;
constexpr int RJ = 32 * JT;        // 128 region columns
constexpr int RI = NWARP * RT;     // 64 region rows
constexpr int OJ = RJ - 2 * TMAX;  // 112 owned columns
constexpr int OI = RI - 2 * TMAX;  // 48 owned rows
constexpr int TB_THREADS = 32 * NWARP;
static_assert(RI == kJacRegionRows && RJ == kJacRegionCols && TMAX == kJacHalo,
              "Jacobi region geometry");

// RINIT (first launch of the outer correction): instead of loading bw, the
// kernel loads the main potential phi (from the buffer the main solve's
// control block names), b and the flags, forms the correction right-hand
// side b_e = r(phi) = resid_ff(...) rounded to float on every region cell
// (garbage only on the region's outermost ring, which the halo absorbs),
// sets bw = w * b_e, starts the correction from 0 and, when more launches
// follow, writes b_e and bw_e of the owned cells to rhs_e / bwe.
template <bool OMEGA1, bool FULL, bool CHECK, bool RINIT, int NW = NWARP>
__device__ __forceinline__ void jacobi_tile(
    int ri0, int rj0, uint32_t own, bool lead, const float* __restrict__ src, float* __restrict__ dst,
    const float* __restrict__ W, const float* __restrict__ BW, const float* __restrict__ rhs,
    const uint8_t* __restrict__ flags, float om1, PCtl* ctl, int k, int t0, int ns, float tol,
    int out_sel, int zero_init, Grid g, const float* __restrict__ mphi0,
    const float* __restrict__ mphi1, const PCtl* __restrict__ mctl, float* __restrict__ rhs_e,
    float* __restrict__ bwe) {
  __shared__ float4 xch[2][2][NW][32];
  __shared__ float red[NW];
  __shared__ int skip;
  pdl_enter();
  if (threadIdx.x == 0) {
    int sk = ctl->stop;
    if (!sk && CHECK && k > 0 && __uint_as_float(ctl->slots[k - 1]) < tol) {
      sk = 1;
      ctl->stop = 1;
    }
    skip = sk;
  }
  __syncthreads();
  if (skip) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gi0 = ri0 + warp * RT;
  const int gj = rj0 + lane * JT;
  const int oi0 = own & 255, oi1 = own >> 8 & 255, oj0 = own >> 16 & 255, oj1 = own >> 24;
  // gj is a multiple of 4 (rj0 is) and the pitch a multiple of 4: a 4-column
  // group is either wholly left of the grid or a 16-byte aligned read inside
  // the row.
  const bool colok = gj >= 0 && gj < g.P;
  float x[RT][JT], w[RT][JT], bw[RT][JT];
  uint32_t fr[RINIT ? RT : 1];
  const float* ph = RINIT ? (mctl->sel ? mphi1 : mphi0) : src;
#pragma unroll
  for (int r = 0; r < RT; ++r) {
    int gi = gi0 + r;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), ww = a, bb = a;
    uint32_t f4 = 0;
    if (colok && gi >= 0 && gi < g.NX) {
      size_t c = (size_t)gi * g.P + gj;
      if (RINIT || !zero_init) a = *reinterpret_cast<const float4*>(ph + c);
      ww = *reinterpret_cast<const float4*>(W + c);
      bb = *reinterpret_cast<const float4*>((RINIT ? rhs : BW) + c);
      if (RINIT) f4 = *reinterpret_cast<const uint32_t*>(flags + c);
    }
    x[r][0] = a.x; x[r][1] = a.y; x[r][2] = a.z; x[r][3] = a.w;
    w[r][0] = ww.x; w[r][1] = ww.y; w[r][2] = ww.z; w[r][3] = ww.w;
    bw[r][0] = bb.x; bw[r][1] = bb.y; bw[r][2] = bb.z; bw[r][3] = bb.w;
    if (RINIT) fr[r] = f4;
#pragma unroll
    for (int q = 0; q < JT; ++q)
      if (gj + q >= g.NY) {
        x[r][q] = 0.0f;
        w[r][q] = 0.0f;
        bw[r][q] = 0.0f;
        if (RINIT) fr[r] &= ~(0xffu << (8 * q));
      }
  }
  const bool own_col = lane * JT >= oj0 && lane * JT < oj1;
  if (RINIT) {
    // Residual of the main potential held in x, with b in bw.
    xch[1][0][warp][lane] = make_float4(x[0][0], x[0][1], x[0][2], x[0][3]);
    xch[1][1][warp][lane] = make_float4(x[RT - 1][0], x[RT - 1][1], x[RT - 1][2], x[RT - 1][3]);
    __syncthreads();
    float4 u4 = warp > 0 ? xch[1][1][warp - 1][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 d4 = warp < NW - 1 ? xch[1][0][warp + 1][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    float prev[JT] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      float lf = __shfl_up_sync(0xffffffffu, x[r][JT - 1], 1);
      float rt = __shfl_down_sync(0xffffffffu, x[r][0], 1);
      float nxt[JT];
      if (r < RT - 1) {
#pragma unroll
        for (int q = 0; q < JT; ++q) nxt[q] = x[r + 1][q];
      } else {
        nxt[0] = d4.x; nxt[1] = d4.y; nxt[2] = d4.z; nxt[3] = d4.w;
      }
      float be[JT];
#pragma unroll
      for (int q = 0; q < JT; ++q) {
        uint8_t fl = (uint8_t)(fr[r] >> (8 * q));
        float left = q == 0 ? lf : x[r][q - 1];
        float right = q == JT - 1 ? rt : x[r][q + 1];
        be[q] = 0.0f;
        if (flag_active(fl))
          be[q] = resid_ff(bw[r][q], prev[q], nxt[q], left, right, (float)flag_count(fl), x[r][q]).hi;
      }
#pragma unroll
      for (int q = 0; q < JT; ++q) {
        prev[q] = x[r][q];
        bw[r][q] = w[r][q] * be[q];
      }
      if (rhs_e && own_col && warp * RT + r >= oi0 && warp * RT + r < oi1) {
        int gi = gi0 + r;
        if (gi < g.NX && gj < g.NY) {
          size_t c = (size_t)gi * g.P + gj;
          if (gj + JT <= g.NY) {
            *reinterpret_cast<float4*>(rhs_e + c) = make_float4(be[0], be[1], be[2], be[3]);
            *reinterpret_cast<float4*>(bwe + c) =
                make_float4(bw[r][0], bw[r][1], bw[r][2], bw[r][3]);
          } else {
#pragma unroll
            for (int q = 0; q < JT; ++q)
              if (gj + q < g.NY) {
                rhs_e[c + q] = be[q];
                bwe[c + q] = bw[r][q];
              }
          }
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RT; ++r)
#pragma unroll
      for (int q = 0; q < JT; ++q) x[r][q] = 0.0f;
    __syncthreads();  // xch[1] is read above and written again by the second sweep
  }
  float mx = 0.0f;
  auto sweep = [&](int sw, bool last) {
    const int buf = sw & 1;
    xch[buf][0][warp][lane] = make_float4(x[0][0], x[0][1], x[0][2], x[0][3]);
    xch[buf][1][warp][lane] = make_float4(x[RT - 1][0], x[RT - 1][1], x[RT - 1][2], x[RT - 1][3]);
    __syncthreads();
    float4 u4 = warp > 0 ? xch[buf][1][warp - 1][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 d4 = warp < NW - 1 ? xch[buf][0][warp + 1][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
    float prev[JT] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      float lf = __shfl_up_sync(0xffffffffu, x[r][JT - 1], 1);
      float rt = __shfl_down_sync(0xffffffffu, x[r][0], 1);
      float nxt[JT];
      if (r < RT - 1) {
#pragma unroll
        for (int q = 0; q < JT; ++q) nxt[q] = x[r + 1][q];
      } else {
        nxt[0] = d4.x; nxt[1] = d4.y; nxt[2] = d4.z; nxt[3] = d4.w;
      }
      float nw[JT];
      float nbv[JT];
#pragma unroll
      for (int q = 0; q < JT; ++q) {
        float left = q == 0 ? lf : x[r][q - 1];
        float right = q == JT - 1 ? rt : x[r][q + 1];
        float nb = prev[q] + nxt[q] + left + right;  // (i-1) + (i+1) + (j-1) + (j+1)
        nbv[q] = nb;
        float y = __fmaf_rn(w[r][q], nb, bw[r][q]);
        if (!OMEGA1) y = __fmaf_rn(om1, x[r][q], y);
        nw[q] = y;
      }
      if (CHECK && last) {
        const int ri = warp * RT + r;
        const int gi = gi0 + r;
        if (own_col && ri >= oi0 && ri < oi1 && gi < g.NX && gj < g.NY) {
          size_t c = (size_t)gi * g.P + gj;
          float4 b4 = *reinterpret_cast<const float4*>(rhs + c);
          uint32_t f4 = *reinterpret_cast<const uint32_t*>(flags + c);
          float bq[JT] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
          for (int q = 0; q < JT; ++q) {
            uint8_t fl = (uint8_t)(f4 >> (8 * q));
            if (gj + q < g.NY && flag_active(fl)) {
              float rr = __fmaf_rn(-(float)flag_count(fl), x[r][q], bq[q] + nbv[q]);
              float ar = fabsf(rr);
              if (ar > mx) mx = ar;
            }
          }
        }
      }
#pragma unroll
      for (int q = 0; q < JT; ++q) {
        prev[q] = x[r][q];
        x[r][q] = nw[q];
      }
    }
  };
  if (FULL) {
#pragma unroll
    for (int sw = 0; sw < TMAX; ++sw) sweep(sw, sw == TMAX - 1);
  } else {
    for (int sw = 0; sw < ns; ++sw) sweep(sw, sw == ns - 1);
  }
  // Owned cells: rows [oi0, oi1), columns [oj0, oj1) of the region.
  if (own_col) {
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      int gi = gi0 + r;
      if (warp * RT + r < oi0 || warp * RT + r >= oi1 || gi >= g.NX || gj >= g.NY) continue;
      size_t c = (size_t)gi * g.P + gj;
      if (gj + JT <= g.NY) {
        *reinterpret_cast<float4*>(dst + c) = make_float4(x[r][0], x[r][1], x[r][2], x[r][3]);
      } else {
#pragma unroll
        for (int q = 0; q < JT; ++q)
          if (gj + q < g.NY) dst[c + q] = x[r][q];
      }
    }
  }
  if (CHECK) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if (lane == 0) red[warp] = mx;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (CHECK) {
      float m = 0.0f;
#pragma unroll
      for (int q = 0; q < NW; ++q) m = fmaxf(m, red[q]);
      if (m > 0.0f) atomicMax(&ctl->slots[k], __float_as_uint(m));
    }
    if (lead) {
      ctl->sweeps = t0 + ns;
      ctl->last_launch = k;
      ctl->sel = out_sel;
    }
  }
}

// NW warps (8, or 4 on grids with fewer 8-warp regions than SMs): a region
// of 8 NW rows x 128 columns, so a small grid spreads over more SMs.
template <bool OMEGA1, bool FULL, bool CHECK, bool RINIT, int NW = NWARP>
__global__ void __launch_bounds__(32 * NW, 2 * NWARP / NW)
    k_jacobi_rb(const float* __restrict__ src, float* __restrict__ dst,
                const float* __restrict__ W, const float* __restrict__ BW,
                const float* __restrict__ rhs, const uint8_t* __restrict__ flags, float om1,
                PCtl* ctl, int k, int t0, int ns, float tol, int out_sel, int zero_init, Grid g,
                const float* __restrict__ mphi0, const float* __restrict__ mphi1,
                const PCtl* __restrict__ mctl, float* __restrict__ rhs_e,
                float* __restrict__ bwe) {
  constexpr int R = NW * RT;  // region rows
  jacobi_tile<OMEGA1, FULL, CHECK, RINIT, NW>((int)blockIdx.y * (R - 2 * TMAX), (int)blockIdx.x * OJ,
                                              span_own(blockIdx.y, g.NX, R) |
                                                  span_own(blockIdx.x, g.NY, RJ) << 16,
                                              blockIdx.x == 0 && blockIdx.y == 0, src, dst, W,
                                              BW, rhs, flags, om1, ctl, k, t0, ns, tol, out_sel,
                                              zero_init, g, mphi0, mphi1, mctl, rhs_e, bwe);
}

// A batch's Jacobi launch k of L: scene s runs its nl_s = ceil(iters_s / T)
// launches as the last nl_s of the L, the first of them with the remainder
// sweeps, so every scene ends in the same buffer.  The table lists the
// scenes with more sweeps first and launch k runs only the prefix of
// scenes that have started (a block of another would return at once).
// Each block's table entry gives its region's origin and owned window
// (fg_internal.cuh): regions at a scene's edges start or end there and own
// up to it, so a scene is cut into fewer regions than whole 48 x 112 tiles
// with halos on every side.  The tables are constant and read before
// jacobi_tile waits on the previous launch (programmatic dependent launch).
template <bool OMEGA1>
__global__ void __launch_bounds__(TB_THREADS, 2)
    kb_jacobi(const BTile* __restrict__ tiles, const BScene* __restrict__ sc,
              const float* __restrict__ src, float* __restrict__ dst, const float* __restrict__ W,
              const float* __restrict__ BW, const uint8_t* __restrict__ flags, float om1,
              PCtl* ctl, int k, int L, int T, int out_sel) {
  const BTile t = tiles[blockIdx.x];
  const BScene& s = sc[t.s];
  const int nl = (s.iters + T - 1) / T;
  const int first = L - nl;
  if (k < first) return;
  const int ns = k == first ? s.iters - (nl - 1) * T : T;
  const long long o = s.off;
  if (ns == TMAX)
    jacobi_tile<OMEGA1, true, false, false>(t.y, t.x, (uint32_t)t.pad, blockIdx.x == 0, src + o, dst + o, W + o,
                                            BW + o, nullptr, flags + o, om1, ctl, k, 0, ns, 0.0f,
                                            out_sel, k == first, s.g, nullptr, nullptr, nullptr,
                                            nullptr, nullptr);
  else
    jacobi_tile<OMEGA1, false, false, false>(t.y, t.x, (uint32_t)t.pad, blockIdx.x == 0, src + o, dst + o, W + o,
                                             BW + o, nullptr, flags + o, om1, ctl, k, 0, ns, 0.0f,
                                             out_sel, k == first, s.g, nullptr, nullptr, nullptr,
                                             nullptr, nullptr);
}


// ------------------------------------------------------------------ TMA-fed Jacobi
// The full 8-sweep launches without residual check, as a persistent kernel:
// each block (two per SM) walks tiles t = blockIdx.x, + gridDim.x, ...; the
// tensor memory accelerator copies the next tile's phi, w and w*b boxes (64 x
// 128, zero outside the arrays) into shared memory while the block sweeps the
// current tile in registers, so the loads no longer sit in front of the
// sweeps.  Same per-cell arithmetic as k_jacobi_rb, same results.
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load_2d(float* dst, const CUtensorMap* tm, int x, int y,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

constexpr int TILE_FLOATS = RI * RJ;  // one 64 x 128 box


// Waits for phase `parity` of the barrier for at most about a second (and a
// bounded number of polls); false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (int it = 0; it < MBAR_MAX_TRIES; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > MBAR_WAIT_NS) return false;
  }
  return false;
}

// After a wait gave up, before the block leaves: waits for its copy in
// flight for up to about eight more seconds, so a copy that is only slow
// lands before the block's shared memory passes to another block.  A copy
// still outstanding after nine seconds means the device is not progressing;
// the wait stays bounded all the same.
constexpr int MBAR_DRAIN_SLICES = 8;
__device__ __forceinline__ void mbar_drain(uint64_t* bar, unsigned parity) {
  for (int s = 0; s < MBAR_DRAIN_SLICES; ++s)
    if (mbar_wait_bounded(bar, parity)) return;
}

// One sweep of a tile in registers, with the arithmetic of jacobi_tile;
// buf alternates between consecutive sweeps (the row exchange is double
// buffered, one barrier per sweep).
template <bool OMEGA1>
__device__ __forceinline__ void tile_sweep(float (&x)[RT][JT], const float (&w)[RT][JT],
                                           const float (&bw)[RT][JT], float om1,
                                           float4 (&xch)[2][2][NWARP][32], int warp, int lane,
                                           int buf) {
  xch[buf][0][warp][lane] = make_float4(x[0][0], x[0][1], x[0][2], x[0][3]);
  xch[buf][1][warp][lane] = make_float4(x[RT - 1][0], x[RT - 1][1], x[RT - 1][2], x[RT - 1][3]);
  __syncthreads();
  float4 u4 = warp > 0 ? xch[buf][1][warp - 1][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
  float4 d4 = warp < NWARP - 1 ? xch[buf][0][warp + 1][lane] : make_float4(0.f, 0.f, 0.f, 0.f);
  float prev[JT] = {u4.x, u4.y, u4.z, u4.w};
#pragma unroll
  for (int r = 0; r < RT; ++r) {
    float lf = __shfl_up_sync(0xffffffffu, x[r][JT - 1], 1);
    float rt = __shfl_down_sync(0xffffffffu, x[r][0], 1);
    float nxt[JT];
    if (r < RT - 1) {
#pragma unroll
      for (int q = 0; q < JT; ++q) nxt[q] = x[r + 1][q];
    } else {
      nxt[0] = d4.x; nxt[1] = d4.y; nxt[2] = d4.z; nxt[3] = d4.w;
    }
    float nw[JT];
#pragma unroll
    for (int q = 0; q < JT; ++q) {
      float left = q == 0 ? lf : x[r][q - 1];
      float right = q == JT - 1 ? rt : x[r][q + 1];
      float nb = prev[q] + nxt[q] + left + right;  // (i-1) + (i+1) + (j-1) + (j+1)
      float y = __fmaf_rn(w[r][q], nb, bw[r][q]);
      if (!OMEGA1) y = __fmaf_rn(om1, x[r][q], y);
      nw[q] = y;
    }
#pragma unroll
    for (int q = 0; q < JT; ++q) {
      prev[q] = x[r][q];
      x[r][q] = nw[q];
    }
  }
}

// The TMAX sweeps of one tile.  hook(sw) runs before sweep sw (sw a
// constant after unrolling), so callers can spread latency-bound side work
// over the sweeps.
struct NoHook {
  __device__ __forceinline__ void operator()(int) const {}
};
template <bool OMEGA1, typename Hook = NoHook>
__device__ __forceinline__ void tile_sweeps(float (&x)[RT][JT], const float (&w)[RT][JT],
                                            const float (&bw)[RT][JT], float om1,
                                            float4 (&xch)[2][2][NWARP][32], int warp, int lane,
                                            Hook hook = Hook()) {
#pragma unroll
  for (int sw = 0; sw < TMAX; ++sw) {
    hook(sw);
    tile_sweep<OMEGA1>(x, w, bw, om1, xch, warp, lane, sw & 1);
  }
}

// 16 bytes from global to shared memory without passing through registers;
// the bytes past src_bytes (0 or 16) are zero-filled.
__device__ __forceinline__ void cp_async16(float* smem, const float* gmem, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem),
               "r"(src_bytes)
               : "memory");
}

// A batch's Jacobi launch k (as kb_jacobi, same regions, same per-cell
// arithmetic, same results) as a persistent kernel: block b runs the
// started scenes' regions b, b + G, ... in turn, and while it sweeps one,
// its threads' asynchronous copies bring the next region's boxes (phi, w,
// w*b; zero outside the scene's rows and pitch) into shared memory, so the
// loads no longer sit in front of the sweeps.  The tables are constant;
// the copies read the previous launch's result, after the programmatic
// wait.
template <bool OMEGA1>
__global__ void __launch_bounds__(TB_THREADS, 2)
    kb_jacobi_pf(const BTile* __restrict__ tiles, const BScene* __restrict__ sc, int n,
                 const float* __restrict__ src, float* __restrict__ dst,
                 const float* __restrict__ W, const float* __restrict__ BW, float om1, PCtl* ctl,
                 int k, int L, int T, int out_sel) {
  extern __shared__ __align__(128) float4 pbuf4[];  // [3][RI][RJ] floats: phi, w, w*b
  float* pbuf = reinterpret_cast<float*>(pbuf4);
  __shared__ float4 xch[2][2][NWARP][32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // Thread tid copies float4 q = tid + 256 m (m < 8) of each box: region
  // row q / 32, columns 4 (q % 32) .. + 3, for a region starting at (ri0,
  // rj0) of a scene of NX rows of pitch P at element offset off.
  auto issue_at = [&](int ri0, int rj0, int NX, int P, long long off, bool zi) {
    const float* xs = src + off;
    const float* ws = W + off;
    const float* bs = BW + off;
#pragma unroll
    for (int m = 0; m < TILE_FLOATS / 4 / TB_THREADS; ++m) {
      const int q = tid + TB_THREADS * m;
      const int row = q / (RJ / JT), col = JT * (q % (RJ / JT));
      const int gi = ri0 + row, gj = rj0 + col;
      const bool ok = gi >= 0 && gi < NX && gj >= 0 && gj < P;
      const size_t c = ok ? (size_t)gi * P + gj : 0;
      float* d = pbuf + row * RJ + col;
      cp_async16(d, xs + c, ok && !zi ? 16 : 0);
      cp_async16(d + TILE_FLOATS, ws + c, ok ? 16 : 0);
      cp_async16(d + 2 * TILE_FLOATS, bs + c, ok ? 16 : 0);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  // (A scene's first launch starts from 0: its phi box is not copied.)
  auto issue = [&](int i) {
    const BTile t = tiles[i];
    const BScene& s = sc[t.s];
    issue_at(t.y, t.x, s.g.NX, s.g.P, s.off, k == L - (s.iters + T - 1) / T);
  };
  int i = blockIdx.x;
  pdl_enter();
  if (i < n) issue(i);
  while (i < n) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();  // every thread's copies of region i landed
    const BTile t = tiles[i];
    const BScene& s = sc[t.s];
    const Grid g = s.g;
    const int nl = (s.iters + T - 1) / T;
    const int ns = k == L - nl ? s.iters - (nl - 1) * T : T;
    const int gi0 = t.y + warp * RT, gj = t.x + lane * JT;
    float x[RT][JT], w[RT][JT], bw[RT][JT];
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      const int o = (warp * RT + r) * RJ + lane * JT;
      const float4 a = *reinterpret_cast<const float4*>(pbuf + o);
      const float4 ww = *reinterpret_cast<const float4*>(pbuf + TILE_FLOATS + o);
      const float4 bb = *reinterpret_cast<const float4*>(pbuf + 2 * TILE_FLOATS + o);
      x[r][0] = a.x; x[r][1] = a.y; x[r][2] = a.z; x[r][3] = a.w;
      w[r][0] = ww.x; w[r][1] = ww.y; w[r][2] = ww.z; w[r][3] = ww.w;
      bw[r][0] = bb.x; bw[r][1] = bb.y; bw[r][2] = bb.z; bw[r][3] = bb.w;
#pragma unroll
      for (int q = 0; q < JT; ++q)
        if (gj + q >= g.NY) {  // the pitch padding: outside the grid
          x[r][q] = 0.0f;
          w[r][q] = 0.0f;
          bw[r][q] = 0.0f;
        }
    }
    const int nx = i + gridDim.x;
    if (i == 0 && tid == 0) ctl->sweeps = ns;
    // (The host launches the started scenes' regions only; a region of a
    // scene that has not started would be left alone.)
    const bool run = k >= L - nl;
    if (run && ns == TMAX) {
      // The next region's table entry is read before sweep 0, its scene's
      // before sweep 1, and its copies start before sweep 2 (sweep 0's
      // barrier has ordered every thread's register fill before them), so
      // neither the dependent table reads nor the copies sit in front of a
      // sweep.
      BTile tn{};
      int nNX = 0, nP = 0, nit = 0;
      long long noff = 0;
      auto hook = [&](int sw) {
        if (nx >= n) return;
        if (sw == 0) {
          tn = tiles[nx];
        } else if (sw == 1) {
          const BScene& sn = sc[tn.s];
          nNX = sn.g.NX;
          nP = sn.g.P;
          noff = sn.off;
          nit = sn.iters;
        } else if (sw == 2) {
          issue_at(tn.y, tn.x, nNX, nP, noff, k == L - (nit + T - 1) / T);
        }
      };
      tile_sweeps<OMEGA1>(x, w, bw, om1, xch, warp, lane, hook);
    } else {
      __syncthreads();  // the boxes are in registers: the buffer takes the next region
      if (nx < n) issue(nx);
      if (run)
        for (int sw = 0; sw < ns; ++sw) tile_sweep<OMEGA1>(x, w, bw, om1, xch, warp, lane, sw & 1);
    }
    const uint32_t own = (uint32_t)t.pad;
    const int oi0 = own & 255, oi1 = own >> 8 & 255, oj0 = own >> 16 & 255, oj1 = own >> 24;
    if (run && lane * JT >= oj0 && lane * JT < oj1) {
      float* xd = dst + s.off;
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        const int gi = gi0 + r;
        if (warp * RT + r < oi0 || warp * RT + r >= oi1 || gi >= g.NX || gj >= g.NY) continue;
        const size_t c = (size_t)gi * g.P + gj;
        if (gj + JT <= g.NY) {
          *reinterpret_cast<float4*>(xd + c) = make_float4(x[r][0], x[r][1], x[r][2], x[r][3]);
        } else {
#pragma unroll
          for (int q = 0; q < JT; ++q)
            if (gj + q < g.NY) xd[c + q] = x[r][q];
        }
      }
    }
    i = nx;
  }
  if (blockIdx.x == 0 && tid == 0) {
    ctl->last_launch = k;
    ctl->sel = out_sel;
  }
}

template <bool OMEGA1>
__global__ void __launch_bounds__(TB_THREADS, 2)
    k_jacobi_tma(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmw,
                 const __grid_constant__ CUtensorMap tmb, float* __restrict__ dst, float om1,
                 PCtl* ctl, int k, int t0, int out_sel, int zero_init, Grid g, int ntx,
                 int ntiles, int* err, int stall_tile) {
  extern __shared__ __align__(128) float4 tbuf4[];  // [3][RI][RJ] floats: phi, w, w*b
  float* tbuf = reinterpret_cast<float*>(tbuf4);
  __shared__ float4 xch[2][2][NWARP][32];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_skip;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_skip = ctl->stop;
    if (!s_skip) mbar_init(&bar, 1);
  }
  __syncthreads();
  if (s_skip) return;
  const unsigned bytes = (zero_init ? 2u : 3u) * TILE_FLOATS * 4u;
  auto issue = [&](int t) {
    const int ty = t / ntx, tx = t - ty * ntx;
    const int x = tx * OJ - TMAX, y = ty * OI - TMAX;  // x: a multiple of 4 floats (16 bytes)
    // Order this block's earlier shared-memory reads before the copy's writes.
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    // Fault injection: tile `stall_tile` expects 16 bytes more than its
    // copies bring, so its barrier phase never completes and the bounded
    // wait below gives up (every copy issued still lands).
    mbar_expect_tx(&bar, bytes + (t == stall_tile ? 16u : 0u));
    if (!zero_init) tma_load_2d(tbuf, &tmx, x, y, &bar);
    tma_load_2d(tbuf + TILE_FLOATS, &tmw, x, y, &bar);
    tma_load_2d(tbuf + 2 * TILE_FLOATS, &tmb, x, y, &bar);
  };
  if (tid == 0 && (int)blockIdx.x < ntiles) issue(blockIdx.x);
  unsigned parity = 0;
  const bool own_col = lane * JT >= TMAX && lane * JT < RJ - TMAX;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const bool landed = mbar_wait_bounded(&bar, parity);
    if (__syncthreads_or(!landed)) {
      // A copy did not land in time (the whole block agrees): flag it, let
      // it land (bounded), stop.  The next tile's copy is issued only after
      // this one landed, so nothing else is in flight.
      if (tid == 0) {
        atomicExch(&ctl->pad[0], 1);
        if (err) atomicExch(err, 1);
      }
      if (!landed) mbar_drain(&bar, parity);
      return;
    }
    parity ^= 1u;
    const int ty = t / ntx, tx = t - ty * ntx;
    const int gi0 = ty * OI - TMAX + warp * RT;
    const int gj = tx * OJ - TMAX + lane * JT;
    float x[RT][JT], w[RT][JT], bw[RT][JT];
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      const int o = (warp * RT + r) * RJ + lane * JT;
      float4 a = zero_init ? make_float4(0.f, 0.f, 0.f, 0.f)
                           : *reinterpret_cast<const float4*>(tbuf + o);
      float4 ww = *reinterpret_cast<const float4*>(tbuf + TILE_FLOATS + o);
      float4 bb = *reinterpret_cast<const float4*>(tbuf + 2 * TILE_FLOATS + o);
      x[r][0] = a.x; x[r][1] = a.y; x[r][2] = a.z; x[r][3] = a.w;
      w[r][0] = ww.x; w[r][1] = ww.y; w[r][2] = ww.z; w[r][3] = ww.w;
      bw[r][0] = bb.x; bw[r][1] = bb.y; bw[r][2] = bb.z; bw[r][3] = bb.w;
#pragma unroll
      for (int q = 0; q < JT; ++q)
        if (gj + q >= g.NY) {  // the pitch padding (outside the grid: zero-filled)
          x[r][q] = 0.0f;
          w[r][q] = 0.0f;
          bw[r][q] = 0.0f;
        }
    }
    __syncthreads();  // the boxes are in registers: the buffer takes the next tile
    if (tid == 0 && t + (int)gridDim.x < ntiles) issue(t + gridDim.x);
    tile_sweeps<OMEGA1>(x, w, bw, om1, xch, warp, lane);
    if (own_col && warp >= TMAX / RT && warp < NWARP - TMAX / RT) {
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        int gi = gi0 + r;
        if (gi >= g.NX || gj >= g.NY) continue;
        size_t c = (size_t)gi * g.P + gj;
        if (gj + JT <= g.NY) {
          *reinterpret_cast<float4*>(dst + c) = make_float4(x[r][0], x[r][1], x[r][2], x[r][3]);
        } else {
#pragma unroll
          for (int q = 0; q < JT; ++q)
            if (gj + q < g.NY) dst[c + q] = x[r][q];
        }
      }
    }
  }
  if (tid == 0 && blockIdx.x == 0) {
    ctl->sweeps = t0 + TMAX;
    ctl->last_launch = k;
    ctl->sel = out_sel;
  }
}

// ------------------------------------------------------------------ dataflow Jacobi
// A whole fixed-count solve (nphase launches of TMAX sweeps) as one
// cooperative persistent kernel.  Items (phase, tile) are numbered phase
// by phase and handed out by an atomic counter (done[ntiles]): a block
// claims its next item while it sweeps the current one, so the tensor
// memory accelerator copies the next boxes meanwhile.  Item (ph, t) starts
// once the up to nine tiles whose owned cells its region reads have
// finished phase ph - 1 (done[n] >= ph; done[t] = ph + 1 is published with
// release semantics after the tile's stores).  That one wait covers both
// hazards of the ping-pong buffers: the neighbours' phase ph - 1 results
// are in src(ph), and they no longer read src(ph - 1), which this item
// overwrites.  Items are claimed in increasing order and depend only on
// smaller ones, so the smallest unfinished item can always proceed (all
// blocks are resident: cooperative launch).  No block idles at a launch
// boundary or in a partial last wave.  Same per-cell arithmetic, same
// results.
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Whether the tiles around t (3 x 3, clipped to the tile grid) finished
// phase ph - 1.  All 32 lanes of a warp call it: lane l < 9 reads the flag
// of neighbour (l / 3 - 1, l % 3 - 1) with a relaxed load followed by an
// acquire fence.
__device__ __forceinline__ bool flow_ready_warp(const int* done, int ph, int t, int ntx, int nty,
                                                int lane) {
  bool ok = true;
  if (ph > 0 && lane < 9) {
    const int ty = t / ntx, tx = t - ty * ntx;
    const int y = ty + lane / 3 - 1, x = tx + lane % 3 - 1;
    if (y >= 0 && y < nty && x >= 0 && x < ntx) {
      int v;
      asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(done + y * ntx + x)
                   : "memory");
      ok = v >= ph;
      asm volatile("fence.acq_rel.gpu;" ::: "memory");
    }
  }
  return __all_sync(0xffffffffu, ok);
}

template <bool OMEGA1>
__global__ void __launch_bounds__(TB_THREADS, 2)
    k_jacobi_flow(const __grid_constant__ CUtensorMap tm0, const __grid_constant__ CUtensorMap tm1,
                  const __grid_constant__ CUtensorMap tmw, const __grid_constant__ CUtensorMap tmb,
                  float* __restrict__ x0, float* __restrict__ x1, float om1, PCtl* ctl,
                  int* __restrict__ done, int nphase, int zero_first, Grid g, int ntx, int nty,
                  int* err, int stall_tile) {
  extern __shared__ __align__(128) float4 tbuf4[];  // [3][RI][RJ] floats: phi, w, w*b
  float* tbuf = reinterpret_cast<float*>(tbuf4);
  __shared__ float4 xch[2][2][NWARP][32];
  __shared__ __align__(8) uint64_t bar;
  __shared__ int s_item;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int ntiles = ntx * nty, total = ntiles * nphase;
  int* counter = done + ntiles;
  // Thread 0: copy item i's boxes (phi of its phase's source, w, w*b).
  auto issue = [&](int i) {
    const int ph = i / ntiles, t = i - ph * ntiles;
    const int ty = t / ntx, tx = t - ty * ntx;
    const int x = tx * OJ - TMAX, y = ty * OI - TMAX;  // x: a multiple of 4 floats (16 bytes)
    const bool zi = zero_first && ph == 0;
    // The neighbours' (generic) stores, acquired above, before the copy's
    // reads; this block's earlier shared-memory reads before its writes.
    asm volatile("fence.proxy.async.global;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar, (zi ? 2u : 3u) * TILE_FLOATS * 4u);
    if (!zi) tma_load_2d(tbuf, (ph & 1) ? &tm1 : &tm0, x, y, &bar);
    tma_load_2d(tbuf + TILE_FLOATS, &tmw, x, y, &bar);
    tma_load_2d(tbuf + 2 * TILE_FLOATS, &tmb, x, y, &bar);
  };
  // Warp 0 (all lanes): whether item i's inputs are final.
  auto ready = [&](int i) {
    const int ph = i / ntiles;
    return flow_ready_warp(done, ph, i - ph * ntiles, ntx, nty, lane);
  };
  // Warp 0: bounded wait (about a second) for item i's inputs.
  auto wait_ready = [&](int i) -> bool {
    if (ready(i)) return true;
    const unsigned long long t0 = global_ns();
    for (int it = 0; it < MBAR_MAX_TRIES; ++it) {
      if (ready(i)) return true;
      if (global_ns() - t0 > MBAR_WAIT_NS) return false;
    }
    return false;
  };
  int fail = 0;            // thread 0: a wait gave up
  bool in_flight = false;  // thread 0: a copy issued and not consumed
  if (warp == 0) {
    int i = 0;
    if (lane == 0) {
      mbar_init(&bar, 1);
      i = atomicAdd(counter, 1);
    }
    i = __shfl_sync(0xffffffffu, i, 0);
    const bool ok = i < total ? wait_ready(i) : true;
    if (lane == 0) {
      if (i < total) {
        if (ok) {
          issue(i);
          in_flight = true;
        } else {
          fail = 1;
        }
      }
      s_item = i;
    }
  }
  unsigned parity = 0;
  const bool own_col = lane * JT >= TMAX && lane * JT < RJ - TMAX;
  while (true) {
    if (__syncthreads_or(fail)) break;
    const int item = s_item;
    if (item >= total) break;
    const bool landed = mbar_wait_bounded(&bar, parity);
    if (__syncthreads_or(!landed)) {
      if (tid == 0) fail = 1;
      break;
    }
    if (tid == 0) in_flight = false;
    parity ^= 1u;
    const int ph = item / ntiles, t = item - ph * ntiles;
    const int ty = t / ntx, tx = t - ty * ntx;
    const int gi0 = ty * OI - TMAX + warp * RT;
    const int gj = tx * OJ - TMAX + lane * JT;
    const bool zi = zero_first && ph == 0;
    float x[RT][JT], w[RT][JT], bw[RT][JT];
#pragma unroll
    for (int r = 0; r < RT; ++r) {
      const int o = (warp * RT + r) * RJ + lane * JT;
      float4 a = zi ? make_float4(0.f, 0.f, 0.f, 0.f) : *reinterpret_cast<const float4*>(tbuf + o);
      float4 ww = *reinterpret_cast<const float4*>(tbuf + TILE_FLOATS + o);
      float4 bb = *reinterpret_cast<const float4*>(tbuf + 2 * TILE_FLOATS + o);
      x[r][0] = a.x; x[r][1] = a.y; x[r][2] = a.z; x[r][3] = a.w;
      w[r][0] = ww.x; w[r][1] = ww.y; w[r][2] = ww.z; w[r][3] = ww.w;
      bw[r][0] = bb.x; bw[r][1] = bb.y; bw[r][2] = bb.z; bw[r][3] = bb.w;
#pragma unroll
      for (int q = 0; q < JT; ++q)
        if (gj + q >= g.NY) {  // the pitch padding (outside the grid: zero-filled)
          x[r][q] = 0.0f;
          w[r][q] = 0.0f;
          bw[r][q] = 0.0f;
        }
    }
    __syncthreads();  // the boxes are in registers: the buffer takes the next item
    // Warp 0 claims and prepares the next item while it sweeps this one:
    // the claim is sent before sweep 0, the neighbours' flags are read
    // before sweep 2 and looked at before sweep 4, where the copy of the
    // next boxes starts if they are final (else after this tile).  No wait
    // on an atomic or a flag sits in front of a sweep barrier.
    int next = total, flag = 0;
    bool pending = false;
    auto hook = [&](int sw) {
      if (warp != 0) return;
      if (sw == 0) {
        if (lane == 0) next = atomicAdd(counter, 1);
      } else if (sw == 2) {
        next = __shfl_sync(0xffffffffu, next, 0);
        flag = INT_MAX;
        const int nph = next / ntiles, nt = next - nph * ntiles;
        if (next < total && nph > 0 && lane < 9) {
          const int nty0 = nt / ntx, ntx0 = nt - nty0 * ntx;
          const int y = nty0 + lane / 3 - 1, xx = ntx0 + lane % 3 - 1;
          if (y >= 0 && y < nty && xx >= 0 && xx < ntx)
            asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];"
                         : "=r"(flag)
                         : "l"(done + y * ntx + xx)
                         : "memory");
        }
      } else if (sw == 4) {
        const bool ok = __all_sync(0xffffffffu, flag >= next / ntiles);
        if (next < total) {
          if (ok) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");  // the flags acquired
            __syncwarp();
            if (lane == 0) {
              issue(next);
              in_flight = true;
            }
          } else {
            pending = true;  // issued after this tile, once its inputs are final
          }
        }
      }
    };
    tile_sweeps<OMEGA1>(x, w, bw, om1, xch, warp, lane, hook);
    float* dst = (ph & 1) ? x0 : x1;
    if (own_col && warp >= TMAX / RT && warp < NWARP - TMAX / RT) {
#pragma unroll
      for (int r = 0; r < RT; ++r) {
        int gi = gi0 + r;
        if (gi >= g.NX || gj >= g.NY) continue;
        size_t c = (size_t)gi * g.P + gj;
        if (gj + JT <= g.NY) {
          *reinterpret_cast<float4*>(dst + c) = make_float4(x[r][0], x[r][1], x[r][2], x[r][3]);
        } else {
#pragma unroll
          for (int q = 0; q < JT; ++q)
            if (gj + q < g.NY) dst[c + q] = x[r][q];
        }
      }
    }
    __syncthreads();  // the tile's stores precede its publication
    if (warp == 0) {
      if (lane == 0 && t != stall_tile) {  // (a stalled tile: fault injection)
        __threadfence();
        st_release(done + t, ph + 1);
      }
      if (pending) {
        const bool ok = wait_ready(next);
        if (lane == 0) {
          if (ok) {
            issue(next);
            in_flight = true;
          } else {
            fail = 1;
          }
        }
      }
      if (lane == 0) s_item = next;
    }
  }
  if (tid == 0) {
    if (fail) {
      atomicExch(&ctl->pad[0], 1);
      if (err) atomicExch(err, 1);
    }
    if (in_flight) mbar_drain(&bar, parity);  // a copy still landing
    if (blockIdx.x == 0 && nphase > 0) {
      ctl->sweeps = nphase * TMAX;
      ctl->last_launch = nphase - 1;
      ctl->sel = ((nphase - 1) & 1) ? 0 : 1;
    }
  }
}

// Final potential at cell c: the main iterate, plus the outer correction on
// active cells when one ran (phi = phi + e, fluid.go's p accumulation aside).
__device__ __forceinline__ float phi_final(const float* __restrict__ phi,
                                           const float* __restrict__ e, int c, bool act) {
  float x = phi[c];
  if (e && act) x = x + e[c];
  return x;
}

// Gradient subtract and pressure: U_face += S_R phi_L - S_L phi_R on faces
// with an active neighbour, V likewise, p = cp * phi on active cells, 0
// elsewhere (fill(f.p, 0) fluid.go:83 plus p += cp * delta fluid.go:224).
// U, V, p use the grid pitch g.P; phi, e and the flags the pitch Ps.
__global__ void k_grad(float* __restrict__ U, float* __restrict__ V, float* __restrict__ p,
                       const float* __restrict__ phi0, const float* __restrict__ phi1,
                       const PCtl* __restrict__ ctl, const float* __restrict__ e0,
                       const float* __restrict__ e1, const PCtl* __restrict__ ectl,
                       const uint8_t* __restrict__ flags, float cp, Grid g, int Ps) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const float* phi = ctl->sel ? phi1 : phi0;
  const float* e = ectl ? (ectl->sel ? e1 : e0) : nullptr;
  int c = i * Ps + j;
  int u = i * g.P + j;
  uint8_t fl = flags[c];
  bool act = flag_active(fl);
  float pc = phi_final(phi, e, c, act);
  if (i >= 1 && j >= 1 && j <= g.NY - 2) {
    uint8_t fL = flags[c - Ps];
    bool actL = flag_active(fL);
    if (act || actL) {
      float d = fbit(fl, F_FLUID) * phi_final(phi, e, c - Ps, actL) - fbit(fl, F_W) * pc;
      U[u] = U[u] + d;
    }
  }
  if (j >= 1 && i >= 1 && i <= g.NX - 2) {
    uint8_t fB = flags[c - 1];
    bool actB = flag_active(fB);
    if (act || actB) {
      float d = fbit(fl, F_FLUID) * phi_final(phi, e, c - 1, actB) - fbit(fl, F_S) * pc;
      V[u] = V[u] + d;
    }
  }
  p[u] = act ? cp * pc : 0.0f;
}

// Gradient subtract for the parallel scheme, fused with what follows it in
// the step: the post-projection divergence statistics (sum div^2 in float
// pairs, max |div|, fluid cell count), the residual statistics of the final
// potential (resid_ff per cell, sum r^2 and max |r|) and, when confinement
// is off, addTurbulence (fluid.go:496-526), which only touches a cell's own
// U, V.  Reads U, V and writes the rotated buffers Uo, Vo, so the divergence
// can recompute a neighbour's projected face from its original value.  A
// thread handles GR consecutive cells of one column (k_grad_fused below).
constexpr int GR = 8;
struct GradAcc {
  FF d2, r2;
  float dmax, rmax, n;
};

// A cell's inputs: its flags and its four neighbours', the final potential
// (phi + e) there (0 past the domain edge), U and V at its faces (plus the
// recorded step's forces) and at the faces (i+1, j), (i, j+1), b and the
// turbulence noise.
struct GradIn {
  uint8_t fl, fL, fR, fB, fT;
  float pc, pL, pR, pB, pT;
  float u, v, uR0, vT0, bc;
  float2 nz;
};

// The cell's update from its inputs: the projected faces, p, the residual
// and divergence statistics, turbulence; writes Uo, Vo, p (and the
// pre-turbulence faces U2o, V2o of a recorded step).
__device__ __forceinline__ void grad_apply(int c, bool hasL, bool hasR, bool hasB, bool hasT,
                                           const GradIn& in, float* __restrict__ Uo,
                                           float* __restrict__ Vo, float* __restrict__ p,
                                           float cp, float turbStrength, int do_turb,
                                           GradAcc& acc, float* __restrict__ U2o,
                                           float* __restrict__ V2o) {
  const uint8_t fl = in.fl, fR = in.fR, fT = in.fT;
  const bool act = flag_active(fl), aL = flag_active(in.fL), aR = flag_active(fR);
  const bool aB = flag_active(in.fB), aT = flag_active(fT);
  const float pc = in.pc, pL = in.pL, pR = in.pR, pB = in.pB, pT = in.pT;
  float u = in.u, v = in.v;
  if (hasL && hasB && hasT && (act || aL)) u = u + (fbit(fl, F_FLUID) * pL - fbit(fl, F_W) * pc);
  if (hasB && hasL && hasR && (act || aB)) v = v + (fbit(fl, F_FLUID) * pB - fbit(fl, F_S) * pc);
  p[c] = act ? cp * pc : 0.0f;
  if (act) {
    FF r = resid_ff(in.bc, pL, pR, pB, pT, (float)flag_count(fl), pc);
    FF q = ff_sq(r.hi);
    q.lo = q.lo + 2.0f * r.hi * r.lo;
    acc.r2 = ff_add(acc.r2, q);
    acc.rmax = fmaxf(acc.rmax, fabsf(r.hi));
  }
  if ((fl & (F_FLUID | F_INTERIOR)) == (F_FLUID | F_INTERIOR)) {
    // Projected faces (i+1, j) and (i, j+1), as their own threads compute them.
    float uR = in.uR0;
    if (act || aR) uR = uR + (fbit(fR, F_FLUID) * pc - fbit(fR, F_W) * pR);
    float vT = in.vT0;
    if (act || aT) vT = vT + (fbit(fT, F_FLUID) * pc - fbit(fT, F_S) * pT);
    float div = uR - u + vT - v;
    acc.d2 = ff_add(acc.d2, ff_sq(div));
    acc.dmax = fmaxf(acc.dmax, fabsf(div));
    acc.n = acc.n + 1.0f;
    if (U2o) {
      // The projected field before turbulence (a recorded step keeps it).
      U2o[c] = u;
      V2o[c] = v;
    }
    if (do_turb) {
      float noiseU = in.nz.x * turbStrength;
      float noiseV = in.nz.y * turbStrength;
      float localVel = sqrtf(u * u + v * v);
      if (localVel > 0.1f) {
        float turbulenceFactor = go_min(localVel * 0.5f, 1.0f);
        u += noiseU * turbulenceFactor;
        v += noiseV * turbulenceFactor;
      }
    }
  }
  if (U2o && (fl & (F_FLUID | F_INTERIOR)) != (F_FLUID | F_INTERIOR)) {
    U2o[c] = u;
    V2o[c] = v;
  }
  Uo[c] = u;
  Vo[c] = v;
}

__device__ __forceinline__ void grad_cell(int i, int j, const float* __restrict__ U,
                                          const float* __restrict__ V, float* __restrict__ Uo,
                                          float* __restrict__ Vo, float* __restrict__ p,
                                          const float* __restrict__ phi,
                                          const float* __restrict__ e,
                                          const float* __restrict__ rhs,
                                          const uint8_t* __restrict__ flags, float cp,
                                          const float2* __restrict__ noise, float turbStrength,
                                          int do_turb, const Grid& g, GradAcc& acc,
                                          const float* __restrict__ Fu = nullptr,
                                          const float* __restrict__ Fv = nullptr,
                                          float* __restrict__ U2o = nullptr,
                                          float* __restrict__ V2o = nullptr) {
  const int P = g.P;
  const int c = i * P + j;
  const bool hasL = i >= 1, hasR = i <= g.NX - 2, hasB = j >= 1, hasT = j <= g.NY - 2;
  // Neighbour indices clamped to the cell at the domain edge, so every load
  // below is issued at once and valid; the edge values are masked after.
  const int cL = hasL ? c - P : c, cR = hasR ? c + P : c;
  const int cB = hasB ? c - 1 : c, cT = hasT ? c + 1 : c;
  GradIn in;
  in.fl = flags[c];
  in.fL = hasL ? flags[cL] : 0;
  in.fR = hasR ? flags[cR] : 0;
  in.fB = hasB ? flags[cB] : 0;
  in.fT = hasT ? flags[cT] : 0;
  // phi and the correction are both exactly 0 off the active cells, so the
  // final potential phi + e needs no activity test.
  float pc = phi[c], pL = phi[cL], pR = phi[cR], pB = phi[cB], pT = phi[cT];
  if (e) {
    pc = pc + e[c];
    pL = pL + e[cL];
    pR = pR + e[cR];
    pB = pB + e[cB];
    pT = pT + e[cT];
  }
  if (!hasL) pL = 0.0f;
  if (!hasR) pR = 0.0f;
  if (!hasB) pB = 0.0f;
  if (!hasT) pT = 0.0f;
  in.pc = pc;
  in.pL = pL;
  in.pR = pR;
  in.pB = pB;
  in.pT = pT;
  // U1 = U + the recorded step's forces (when given).
  in.u = with_force(U, Fu, c);
  in.v = with_force(V, Fv, c);
  in.uR0 = with_force(U, Fu, cR);
  in.vT0 = with_force(V, Fv, cT);
  in.bc = rhs[c];
  in.nz = do_turb ? noise[c] : make_float2(0.0f, 0.0f);
  grad_apply(c, hasL, hasR, hasB, hasT, in, Uo, Vo, p, cp, turbStrength, do_turb, acc, U2o, V2o);
}

// The gradient subtract and its fused statistics over GR consecutive rows
// per thread (a block of 32 x 8 threads covers 32 columns x 8 GR rows): on
// interior strips the flags, the final potential and U of rows i-1, i, i+1
// roll from row to row instead of being loaded again (about 14 loads per
// cell instead of 19); each cell's inputs and update are grad_cell's.
// Strips at the domain edge run grad_cell row by row.
__device__ __forceinline__ float phi_fin(const float* __restrict__ phi,
                                         const float* __restrict__ e, int c) {
  float x = phi[c];
  if (e) x = x + e[c];
  return x;
}
__global__ void __launch_bounds__(256)
    k_grad_fused(const float* __restrict__ U, const float* __restrict__ V,
                 float* __restrict__ Uo, float* __restrict__ Vo, float* __restrict__ p,
                 const float* __restrict__ phi0, const float* __restrict__ phi1,
                 const PCtl* __restrict__ ctl, const float* __restrict__ e0,
                 const float* __restrict__ e1, const PCtl* __restrict__ ectl,
                 const float* __restrict__ rhs, const uint8_t* __restrict__ flags, float cp,
                 const float2* __restrict__ noise, float turbStrength, int do_turb,
                 float* __restrict__ part, Grid g, const float* __restrict__ Fu,
                 const float* __restrict__ Fv, float* __restrict__ U2o,
                 float* __restrict__ V2o) {
  __shared__ float shr[64 * 5];
  pdl_enter();
  const float* phi = ctl->sel ? phi1 : phi0;
  const float* e = ectl ? (ectl->sel ? e1 : e0) : nullptr;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * GR;
  GradAcc acc{{0.0f, 0.0f}, {0.0f, 0.0f}, 0.0f, 0.0f, 0.0f};
  if (j < g.NY && i0 < g.NX) {
    if (j >= 1 && j <= g.NY - 2 && i0 >= 1 && i0 + GR - 1 <= g.NX - 2) {
      const int P = g.P;
      int c = i0 * P + j;
      uint8_t fprev = flags[c - P], fcur = flags[c];
      float pprev = phi_fin(phi, e, c - P), pcur = phi_fin(phi, e, c);
      float ucur = with_force(U, Fu, c);
#pragma unroll
      for (int r = 0; r < GR; ++r) {
        const uint8_t fnext = flags[c + P];
        const float pnext = phi_fin(phi, e, c + P);
        const float unext = with_force(U, Fu, c + P);
        GradIn in;
        in.fl = fcur;
        in.fL = fprev;
        in.fR = fnext;
        in.fB = flags[c - 1];
        in.fT = flags[c + 1];
        in.pc = pcur;
        in.pL = pprev;
        in.pR = pnext;
        in.pB = phi_fin(phi, e, c - 1);
        in.pT = phi_fin(phi, e, c + 1);
        in.u = ucur;
        in.v = with_force(V, Fv, c);
        in.uR0 = unext;
        in.vT0 = with_force(V, Fv, c + 1);
        in.bc = rhs[c];
        in.nz = do_turb ? noise[c] : make_float2(0.0f, 0.0f);
        grad_apply(c, true, true, true, true, in, Uo, Vo, p, cp, turbStrength, do_turb, acc, U2o,
                   V2o);
        fprev = fcur;
        fcur = fnext;
        pprev = pcur;
        pcur = pnext;
        ucur = unext;
        c += P;
      }
    } else {
      for (int r = 0; r < GR && i0 + r < g.NX; ++r)
        grad_cell(i0 + r, j, U, V, Uo, Vo, p, phi, e, rhs, flags, cp, noise, turbStrength,
                  do_turb, g, acc, Fu, Fv, U2o, V2o);
    }
  }
  // Row slots: sum div^2, max |div|, fluid cells (exact), sum r^2, max |r|.
  FF row[5] = {acc.d2, {acc.dmax, 0.0f}, {acc.n, 0.0f}, acc.r2, {acc.rmax, 0.0f}};
  block_row<5, 0x4u>(row, 0x12u, shr, part + 10 * (size_t)(blockIdx.y * gridDim.x + blockIdx.x));
}

// Copies the solve's final potential (the buffer the control block names),
// plus the outer correction when one ran (both exactly 0 off the active
// cells, as k_grad_fused adds them).
__global__ void k_store_phi(const float* __restrict__ phi0, const float* __restrict__ phi1,
                            const PCtl* __restrict__ ctl, const float* __restrict__ e0,
                            const float* __restrict__ e1, const PCtl* __restrict__ ectl,
                            float* __restrict__ dst, int n) {
  const float* src = ctl->sel ? phi1 : phi0;
  const float* e = ectl ? (ectl->sel ? e1 : e0) : nullptr;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) dst[k] = e ? src[k] + e[k] : src[k];
}

// A batch's gradient subtract: grad_cell without the statistics.
__device__ __forceinline__ void grad_batch_cell(int i, int j, const float* __restrict__ U,
                                                const float* __restrict__ V,
                                                float* __restrict__ Uo, float* __restrict__ Vo,
                                                float* __restrict__ p,
                                                const float* __restrict__ phi0,
                                                const float* __restrict__ phi1,
                                                const PCtl* __restrict__ ctl,
                                                const float* __restrict__ rhs,
                                                const uint8_t* __restrict__ flags, float cp,
                                                const float2* __restrict__ noise,
                                                float turbStrength, int do_turb,
                                                float* __restrict__ U2o, float* __restrict__ V2o,
                                                const Grid& g) {
  GradAcc acc{{0.0f, 0.0f}, {0.0f, 0.0f}, 0.0f, 0.0f, 0.0f};
  grad_cell(i, j, U, V, Uo, Vo, p, ctl->sel ? phi1 : phi0, nullptr, rhs, flags, cp, noise,
            turbStrength, do_turb, g, acc, nullptr, nullptr, U2o, V2o);
}

// The step's statistics from the combined row of k_grad_fused's partials
// (sum div^2, max |div|, fluid cells, sum r^2, max |r|) and, after a solve,
// its sweep count and last checked max |r| from the control block.
struct StoreDivP {
  DevStats* st;
  const PCtl* ctl;
  __device__ void operator()(const float* r) const {
    st->div_l2_sq = row_sum(r, 0);
    st->div_max = (double)r[2];
    st->div_count = row_sum(r, 2);
    st->resid_l2_sq = row_sum(r, 3);
    st->resid_max = (double)r[8];
    if (ctl) {
      st->sweeps = ctl->sweeps;
      st->last_maxdiv = (double)__uint_as_float(ctl->slots[ctl->last_launch]);
    }
  }
};


}  // namespace

size_t pctl_bytes(int n_slots) { return sizeof(PCtl) + sizeof(unsigned) * (size_t)n_slots; }

// Tensor maps of the TMA-fed Jacobi kernel: a 2D float array of rows x
// pitch, boxes of 64 rows x 128 columns, zero outside.  false when the
// driver entry point or the encoding is unavailable (the plain kernel runs).
// Per CUDA context: the SM count, the dataflow kernel's blocks per SM,
// whether the set-up ran (the kernels' shared-memory limit is state of the
// context the module is loaded in).
constexpr int kMaxContexts = 64;
struct TmaDevice {
  std::once_flag once;
  std::atomic<bool> ready{false};
  int sms = 0;
  int flow_per_sm = 0;
  int batch_pf_per_sm = 0;  // blocks of kb_jacobi_pf per SM (0: the plain batch kernel runs)
};
static TmaDevice g_tma_dev[kMaxContexts];
static unsigned long long g_tma_key[kMaxContexts];
static int g_tma_used = 0;
static std::mutex g_tma_mu;
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

// Identity of the CUDA context current on the calling thread: its
// cuCtxGetId value (unique for the life of the process) with the top bit
// clear, or, when the driver entry points are missing, the device ordinal
// with the top bit set; 0 when neither is known (no context yet).  Module
// state -- a __device__ array's address, a kernel's shared-memory limit --
// belongs to a context, and a caller may make its own context current
// (cuCtxCreate, cuCtxSetCurrent) or replace the primary one
// (cudaDeviceReset), so caches of that state are keyed by this value.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);
static PfnCtxGetCurrent g_ctx_current = nullptr;
static PfnCtxGetId g_ctx_id = nullptr;
static std::once_flag g_ctx_once;

unsigned long long context_key() {
  std::call_once(g_ctx_once, [] {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_current = reinterpret_cast<PfnCtxGetCurrent>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_id = reinterpret_cast<PfnCtxGetId>(fn);
    cudaGetLastError();
  });
  if (g_ctx_current && g_ctx_id) {
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (g_ctx_id(c, &id) != CUDA_SUCCESS) return 0;
    return (id & ~(1ull << 63)) + 1;  // nonzero, top bit clear
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return (1ull << 63) | (unsigned long long)dev;
}

static bool encode_box_map(CUtensorMap* tm, const float* base, int rows, int pitch) {
  if (!g_encode || (reinterpret_cast<uintptr_t>(base) & 15) || (pitch % 4) != 0) return false;
  cuuint64_t dims[2] = {(cuuint64_t)pitch, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)pitch * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)RJ, (cuuint32_t)RI};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// The current context's entry, or nullptr (no context identity, or more
// contexts than entries: the plain kernels run).
static TmaDevice* tma_device() {
  const unsigned long long key = context_key();
  if (!key) return nullptr;
  std::lock_guard<std::mutex> lk(g_tma_mu);
  for (int k = 0; k < g_tma_used; ++k)
    if (g_tma_key[k] == key) return &g_tma_dev[k];
  if (g_tma_used == kMaxContexts) return nullptr;
  g_tma_key[g_tma_used] = key;
  return &g_tma_dev[g_tma_used++];
}

// Resolves the tensor-map encoder (once per process) and, once per device,
// the SM count and the TMA kernels' shared-memory limit (outside any stream
// capture).
void init_jacobi_tma() {
  std::call_once(g_encode_once, [] {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    cudaGetLastError();
  });
  TmaDevice* d = tma_device();
  if (!d) return;
  std::call_once(d->once, [d] {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess)
      d->sms = n;
    const int smem = 3 * TILE_FLOATS * (int)sizeof(float);
    if (cudaFuncSetAttribute(k_jacobi_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess ||
        cudaFuncSetAttribute(k_jacobi_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
      d->sms = 0;
    // Blocks of the dataflow kernel that fit on one SM (co-residency bound).
    int b1 = 0, b2 = 0;
    if (cudaFuncSetAttribute(k_jacobi_flow<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) == cudaSuccess &&
        cudaFuncSetAttribute(k_jacobi_flow<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_jacobi_flow<true>, TB_THREADS,
                                                      smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_jacobi_flow<false>, TB_THREADS,
                                                      smem) == cudaSuccess)
      d->flow_per_sm = b1 < b2 ? b1 : b2;
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop)
      d->flow_per_sm = 0;
    int p1 = 0, p2 = 0;
    if (cudaFuncSetAttribute(kb_jacobi_pf<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) == cudaSuccess &&
        cudaFuncSetAttribute(kb_jacobi_pf<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p1, kb_jacobi_pf<true>, TB_THREADS,
                                                      smem) == cudaSuccess &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p2, kb_jacobi_pf<false>, TB_THREADS,
                                                      smem) == cudaSuccess)
      d->batch_pf_per_sm = p1 < p2 ? p1 : p2;
    cudaGetLastError();
    d->ready.store(true);
  });
}

// The current device's set-up, done here unless the stream is capturing
// (then nullptr: the plain kernels run).
static const TmaDevice* tma_ready(cudaStream_t st) {
  TmaDevice* d = tma_device();
  if (!d) return nullptr;
  if (!d->ready.load()) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusActive;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
      cudaGetLastError();
      return nullptr;
    }
    init_jacobi_tma();
  }
  return d->ready.load() ? d : nullptr;
}

// Launches one full, unchecked Jacobi launch through the TMA-fed kernel;
// false (nothing launched) when the tensor maps cannot be made.
static bool launch_jacobi_tma(cudaStream_t st, const Grid& g, PCtl* ctl, const float* src,
                              float* dst, const float* W, const float* BW, float om1, bool o1,
                              int k, int t0, int sel, int zero_init, int* err, int stall_tile) {
  const TmaDevice* dv = tma_ready(st);
  if (!dv) return false;
  CUtensorMap tmx, tmw, tmb;
  if (!encode_box_map(&tmx, src, g.NX, g.P) || !encode_box_map(&tmw, W, g.NX, g.P) ||
      !encode_box_map(&tmb, BW, g.NX, g.P))
    return false;
  const int nsm = dv->sms;
  if (nsm <= 0) return false;
  const int ntx = (g.NY + OJ - 1) / OJ, nty = (g.NX + OI - 1) / OI;
  const int ntiles = ntx * nty;
  const int grid = ntiles < 2 * nsm ? ntiles : 2 * nsm;
  const size_t smem = 3 * (size_t)TILE_FLOATS * sizeof(float);
  if (o1)
    k_jacobi_tma<true><<<grid, TB_THREADS, smem, st>>>(tmx, tmw, tmb, dst, om1, ctl, k, t0, sel,
                                                       zero_init, g, ntx, ntiles, err, stall_tile);
  else
    k_jacobi_tma<false><<<grid, TB_THREADS, smem, st>>>(tmx, tmw, tmb, dst, om1, ctl, k, t0, sel,
                                                        zero_init, g, ntx, ntiles, err, stall_tile);
  return true;
}

inline int clamp_tb(int t) { return t < 1 ? 1 : (t > TMAX ? TMAX : t); }

int jacobi_launches(const fg_fluid* f, int iters) {
  // In 64 bits: iters near INT_MAX must not wrap (at most INT_MAX launches).
  const long long T = clamp_tb(f->prm.tb_depth);
  return (int)(((long long)iters + T - 1) / T);
}

int jacobi_tile_count(int NX, int NY) {
  return ((NY + OJ - 1) / OJ) * ((NX + OI - 1) / OI);
}

// Launches the first `nphase` full phases of a fixed-count solve as one
// cooperative dataflow kernel (x0 -> x1 -> x0 ...); `done` holds one flag
// per tile and the item counter.  false (nothing launched) when the grid is
// below one tile per SM, the flags are missing, or the tensor maps or the
// cooperative launch are unavailable.
static bool launch_jacobi_flow(cudaStream_t st, const Grid& g, PCtl* ctl, float* x0, float* x1,
                               const float* W, const float* BW, float om1, bool o1, int nphase,
                               int* done, int* err, int stall_tile) {
  if (!done || nphase < 2) return false;
  const TmaDevice* dv = tma_ready(st);
  if (!dv || dv->flow_per_sm <= 0 || dv->sms <= 0) return false;
  const int ntx = (g.NY + OJ - 1) / OJ, nty = (g.NX + OI - 1) / OI;
  const int ntiles = ntx * nty;
  // Below one tile per SM the per-launch kernels were measured faster
  // (128^2 jet 68.3 against 64.6 us per step, 512x256 Karman street 138.5
  // against 121.7 us).
  if (ntiles < dv->sms) return false;
  CUtensorMap tm0, tm1, tmw, tmb;
  if (!encode_box_map(&tm0, x0, g.NX, g.P) || !encode_box_map(&tm1, x1, g.NX, g.P) ||
      !encode_box_map(&tmw, W, g.NX, g.P) || !encode_box_map(&tmb, BW, g.NX, g.P))
    return false;
  // The tile flags and the item counter.
  if (cudaMemsetAsync(done, 0, sizeof(int) * ((size_t)ntiles + 1), st) != cudaSuccess) return false;
  const int cap = dv->flow_per_sm * dv->sms;
  const int grid = ntiles < cap ? ntiles : cap;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(TB_THREADS);
  cfg.dynamicSmemBytes = 3 * (size_t)TILE_FLOATS * sizeof(float);
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  const int zero_first = 1;
  cudaError_t e = o1 ? cudaLaunchKernelEx(&cfg, k_jacobi_flow<true>, tm0, tm1, tmw, tmb, x0, x1,
                                          om1, ctl, done, nphase, zero_first, g, ntx, nty, err,
                                          stall_tile)
                     : cudaLaunchKernelEx(&cfg, k_jacobi_flow<false>, tm0, tm1, tmw, tmb, x0, x1,
                                          om1, ctl, done, nphase, zero_first, g, ntx, nty, err,
                                          stall_tile);
  return e == cudaSuccess;
}

// Enqueues `iters` Jacobi sweeps of A x = b from x = 0 in launches of T
// sweeps; x ping-pongs between x0 and x1 and ctl->sel names the buffer that
// holds the result.  The grid g's pitch is the solver arrays' pitch.
// With `mphi0` set, the first launch forms the right-hand side from the main
// potential (RINIT): b is then the main right-hand side, and b_e / bw_e are
// written to rhs_e / bwe when more launches follow (which then read them).
static cudaError_t enqueue_jacobi(cudaStream_t st, const Grid& g, PCtl* ctl, const float* b,
                                  const float* bw, const float* W, const uint8_t* flags, float* x0,
                                  float* x1, int iters, int T, float om, int check, float tol,
                                  int* n_launched, const float* mphi0 = nullptr,
                                  const float* mphi1 = nullptr, const PCtl* mctl = nullptr,
                                  float* rhs_e = nullptr, float* bwe = nullptr,
                                  int* err = nullptr, int* done = nullptr,
                                  int stall_tile = -1, int tma_stall_tile = -1,
                                  int* kind = nullptr) {
  float om1 = 1.0f - om;
  int used = FG_JACOBI_KERNEL_SWEEP;
  bool o1 = om1 == 0.0f;
  dim3 gr(span_count(g.NY, RJ), span_count(g.NX, RI));
  // Grids with fewer 8-warp regions than SMs run every launch on 4-warp
  // regions (half the rows), spread over twice the SMs.
  const TmaDevice* dv = tma_ready(st);
  const bool narrow = dv && dv->sms > 0 && (long long)gr.x * gr.y < dv->sms;
  const dim3 gr4(span_count(g.NY, RJ), span_count(g.NX, RI / 2));
  int nlaunch = (int)(((long long)iters + T - 1) / T);
  int k0 = 0, kernels = 0;
  // Fixed sweep counts in full launches: the leading full phases as one
  // dataflow kernel where the grid is large enough.
  if (!check && !mphi0 && T == TMAX && iters / TMAX >= 2 &&
      launch_jacobi_flow(st, g, ctl, x0, x1, W, bw, om1, o1, iters / TMAX, done, err,
                         stall_tile)) {
    k0 = iters / TMAX;
    kernels = 1;
    used = FG_JACOBI_KERNEL_DATAFLOW;
  }
  for (int k = k0; k < nlaunch; ++k) {
    ++kernels;
    int t0 = k * T;
    int ns = iters - t0 < T ? iters - t0 : T;
    const float* src = (k & 1) ? x1 : x0;
    float* dst = (k & 1) ? x0 : x1;
    int sel = (k & 1) ? 0 : 1;
    int zi = k == 0 ? 1 : 0;
    bool full = ns == TMAX;
    bool rinit = k == 0 && mphi0 != nullptr;
    const float* bk = rinit ? b : (mphi0 ? rhs_e : b);
    const float* bwk = mphi0 && k > 0 ? bwe : bw;
    float* re = rinit && nlaunch > 1 ? rhs_e : nullptr;
    if (full && !check && !rinit && !mphi0 && !narrow &&
        launch_jacobi_tma(st, g, ctl, src, dst, W, bwk, om1, o1, k, t0, sel, zi, err,
                          tma_stall_tile)) {
      if (used == FG_JACOBI_KERNEL_SWEEP) used = FG_JACOBI_KERNEL_TMA;
      continue;
    }
#define FG_JAC(O, F, C, R)                                                                      \
  (narrow ? launch_pdl(k_jacobi_rb<O, F, C, R, NWARP / 2>, gr4, dim3(TB_THREADS / 2), 0, st, src, \
                       dst, W, bwk, bk, flags, om1, ctl, k, t0, ns, tol, sel, zi, g, mphi0,     \
                       mphi1, mctl, re, bwe)                                                    \
          : launch_pdl(k_jacobi_rb<O, F, C, R>, gr, dim3(TB_THREADS), 0, st, src, dst, W, bwk, \
                       bk, flags, om1, ctl, k, t0, ns, tol, sel, zi, g, mphi0, mphi1, mctl, re, \
                       bwe))
    if (rinit) {
      if (o1) { if (full) FG_JAC(true, true, false, true); else FG_JAC(true, false, false, true); }
      else { if (full) FG_JAC(false, true, false, true); else FG_JAC(false, false, false, true); }
    } else if (o1) {
      if (full) { if (check) FG_JAC(true, true, true, false); else FG_JAC(true, true, false, false); }
      else { if (check) FG_JAC(true, false, true, false); else FG_JAC(true, false, false, false); }
    } else {
      if (full) { if (check) FG_JAC(false, true, true, false); else FG_JAC(false, true, false, false); }
      else { if (check) FG_JAC(false, false, true, false); else FG_JAC(false, false, false, false); }
    }
#undef FG_JAC
  }
  *n_launched = kernels;
  if (kind) *kind = used;
  return cudaGetLastError();
}

// A batch's solves: every scene runs its own sweep count, no early exit.
static cudaError_t jacobi_solve_batch(fg_fluid* f, PCtl* ctl, const float* bw, float* x0,
                                      float* x1) {
  const BatchGeom* bt = f->batch;
  int T = clamp_tb(f->prm.tb_depth);
  int L = (bt->max_iters + T - 1) / T;
  cudaError_t e = cudaMemsetAsync(ctl, 0, sizeof(PCtl), f->stream);
  if (e != cudaSuccess) return e;
  float om = f->prm.jacobi_omega * f->prm.pressure_damping;
  float om1 = 1.0f - om;
  const TmaDevice* dv = tma_ready(f->stream);
  const int pf_blocks = dv && dv->sms > 0 ? dv->batch_pf_per_sm * dv->sms : 0;
  size_t sc = 0;  // scenes (in the table's order) started by launch k
  int n_act = 0;  // their regions: the prefix of the table launch k runs
  for (int k = 0; k < L; ++k) {
    while (sc < bt->jac_iters.size() && L - (bt->jac_iters[sc] + T - 1) / T <= k)
      n_act += bt->jac_regions[sc++];
    const float* src = (k & 1) ? x1 : x0;
    float* dst = (k & 1) ? x0 : x1;
    int sel = (k & 1) ? 0 : 1;
    if (n_act == 0) continue;
    if (pf_blocks > 0)
      launch_pdl(om1 == 0.0f ? kb_jacobi_pf<true> : kb_jacobi_pf<false>,
                 dim3(n_act < pf_blocks ? n_act : pf_blocks), dim3(TB_THREADS),
                 3 * (size_t)TILE_FLOATS * sizeof(float), f->stream, bt->jac_tiles,
                 bt->scenes_dev, n_act, src, dst, f->wgt, bw, om1, ctl, k, L, T, sel);
    else
      launch_pdl(om1 == 0.0f ? kb_jacobi<true> : kb_jacobi<false>, dim3(n_act),
                 dim3(TB_THREADS), 0, f->stream, bt->jac_tiles, bt->scenes_dev, src, dst, f->wgt,
                 bw, f->flags, om1, ctl, k, L, T, sel);
  }
  count(f, L);
  return cudaGetLastError();
}

// kind: where to record the kernel that ran the sweeps (the main solve's).
static cudaError_t jacobi_solve(fg_fluid* f, PCtl* ctl, const float* b, const float* bw, float* x0,
                                float* x1, int iters, bool allow_exit, bool rinit = false,
                                int* kind = nullptr) {
  if (f->batch) return jacobi_solve_batch(f, ctl, bw, x0, x1);
  int T = clamp_tb(f->prm.tb_depth);
  const long long nlaunch = ((long long)iters + T - 1) / T;
  if (nlaunch > f->n_slots) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(ctl, 0, pctl_bytes((int)nlaunch), f->stream);
  if (e != cudaSuccess) return e;
  int check = allow_exit && f->prm.early_exit ? 1 : 0;
  const bool prof = f->profile && allow_exit;
  if (prof && (e = cudaEventRecord(f->prof_ev[0], f->stream)) != cudaSuccess) return e;
  int n = 0;
  if (rinit)
    e = enqueue_jacobi(f->stream, f->g, ctl, b, bw, f->wgt, f->flags, x0, x1, iters, T,
                       f->prm.jacobi_omega * f->prm.pressure_damping, 0, f->prm.tolerance, &n,
                       f->phi, f->phi2, (const PCtl*)f->pctl, f->rhs_e, f->bwe);
  else
    e = enqueue_jacobi(f->stream, f->g, ctl, b, bw, f->wgt, f->flags, x0, x1, iters, T,
                       f->prm.jacobi_omega * f->prm.pressure_damping, check, f->prm.tolerance, &n,
                       nullptr, nullptr, nullptr, nullptr, nullptr, &f->dstats->timeout,
                       f->tile_done, f->stall_tile, -1, kind);
  count(f, n);
  if (e != cudaSuccess) return e;
  if (prof) {
    if ((e = cudaEventRecord(f->prof_ev[1], f->stream)) != cudaSuccess) return e;
    f->prof_launches = (int)nlaunch;
  }
  return cudaGetLastError();
}

cudaError_t launch_jacobi_solve(fg_fluid* f, void* ctl, const float* b, const float* bw, float* x0,
                                float* x1, int iters) {
  return jacobi_solve(f, (PCtl*)ctl, b, bw, x0, x1, iters, false);
}

// One k_lexsor solve on the handle's fields: on the diagonal-major copies
// when the handle has them (copied in and back around the solve), else on
// the row-major fields.
// Blocks of the grid-wide wavefront the GPU holds at once (0: unavailable);
// checked once per process by init_lexsor_cluster.
static std::atomic<int> g_lex_grid_blocks{0};

// Whether the cluster form of the wavefront can run on this device (checked
// once per process, outside any capture: fg_create calls it).
static std::atomic<int> g_lex_cluster{-1};
void init_lexsor_cluster() {
  if (g_lex_cluster.load() >= 0) return;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(LEX_CLUSTER);
  cfg.blockDim = dim3(LEX_THREADS);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = LEX_CLUSTER;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  const bool ok = cudaOccupancyMaxActiveClusters(&n, k_lexsor_cl, &cfg) == cudaSuccess && n >= 1;
  cudaGetLastError();
  g_lex_cluster.store(ok ? 1 : 0);
  int dev = 0, coop = 0, per = 0, sms = 0;
  if (cudaGetDevice(&dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) == cudaSuccess && coop &&
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lexsor_grid, LEX_THREADS, 0) ==
          cudaSuccess &&
      per >= 1)
    g_lex_grid_blocks.store(per * sms);
  cudaGetLastError();
}

int lexsor_scratch_words() { return LEX_GRID_SCRATCH; }

// One wavefront solve: the cluster kernel when a step gives its threads work
// (diagonals of at least 256 cells, at least 8 sweeps in the pipeline), else
// one block (whose barrier is cheaper than the cluster's).
static void lexsor_kernel(fg_fluid* f, float* U, float* V, float* p, const uint8_t* flags,
                          int iters, float relax0, float cp, int early_exit, DevStats* st,
                          float minRelax, const int* stop, int SP, int* exit_out = nullptr,
                          const int* run_from = nullptr) {
  const int L = std::min(f->NX - 2, f->NY - 2);
  // Many sweeps in flight on long diagonals (the closed-form schedule only;
  // no multigrid stop latch): every SM, a grid barrier per step.
  const int nblk = g_lex_grid_blocks.load();
  const int D = f->NX + f->NY - 5;  // (sweeps in flight must fit the maxima's ring)
  if (!early_exit && !stop && f->lex_scratch && nblk > 0 && L >= 256 && iters >= 32 &&
      D / 2 + 4 < LEX_RING) {
    cudaMemsetAsync(f->lex_scratch, 0, sizeof(unsigned) * LEX_GRID_SCRATCH, f->stream);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nblk);
    cfg.blockDim = dim3(LEX_THREADS);
    cfg.stream = f->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_lexsor_grid, U, V, p, flags, f->g, iters, relax0,
                           f->prm.pressure_damping, cp, f->prm.tolerance, st, minRelax, SP,
                           exit_out, run_from, f->lex_scratch, &f->dstats->timeout) ==
        cudaSuccess) {
      count(f);
      return;
    }
    cudaGetLastError();
  }
  if (L >= 256 && iters >= 8 && g_lex_cluster.load() == 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(LEX_CLUSTER);
    cfg.blockDim = dim3(LEX_THREADS);
    cfg.stream = f->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = LEX_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_lexsor_cl, U, V, p, flags, f->g, iters, relax0,
                           f->prm.pressure_damping, cp, f->prm.tolerance, early_exit, st,
                           minRelax, stop, SP, exit_out, run_from) == cudaSuccess)
      return;
    cudaGetLastError();
  }
  k_lexsor<<<1, LEX_THREADS, 0, f->stream>>>(U, V, p, flags, f->g, iters, relax0,
                                              f->prm.pressure_damping, cp, f->prm.tolerance,
                                              early_exit, st, minRelax, stop, SP, exit_out,
                                              run_from);
}

static void run_lexsor(fg_fluid* f, int iters, float relax0, float cp, int early_exit,
                       DevStats* st, float minRelax, const int* stop, int* exit_slot) {
  if (f->skew[0]) {
    dim3 gr = cell_grid(f), bl(BX, BY);
    const Grid& g = f->g;
    k_skew_in<<<gr, bl, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->d[FG_P], f->flags, f->skew[0],
                                        f->skew[1], f->skew[2], f->skew_flags, g, f->skew_sp);
    const int D = f->NX + f->NY - 5;  // anti-diagonals of the interior
    if (early_exit && exit_slot && D / 2 + 4 < LEX_RING) {
      // The early exit, speculatively: all sweeps on the closed-form
      // schedule, recording the first sweep whose max |div| is below the
      // tolerance; if there is one, the fields (untouched so far) are copied
      // in again and exactly that many sweeps run.  Sweeps up to that one
      // are the same in both runs, so this is the serial loop's result and
      // the steps never wait for a "cannot exit" mark.
      cudaMemsetAsync(exit_slot, 0x7f, sizeof(int), f->stream);
      lexsor_kernel(f, f->skew[0], f->skew[1], f->skew[2], f->skew_flags, iters, relax0, cp, 0,
                    st, minRelax, stop, f->skew_sp, exit_slot, nullptr);
      k_skew_in<<<gr, bl, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->d[FG_P], f->flags,
                                          f->skew[0], f->skew[1], f->skew[2], f->skew_flags, g,
                                          f->skew_sp, exit_slot, iters);
      lexsor_kernel(f, f->skew[0], f->skew[1], f->skew[2], f->skew_flags, iters, relax0, cp, 0,
                    st, minRelax, stop, f->skew_sp, nullptr, exit_slot);
      count(f, 3);
    } else {
      lexsor_kernel(f, f->skew[0], f->skew[1], f->skew[2], f->skew_flags, iters, relax0, cp,
                    early_exit, st, minRelax, stop, f->skew_sp);
    }
    k_skew_out<<<gr, bl, 0, f->stream>>>(f->skew[0], f->skew[1], f->skew[2], f->d[FG_U],
                                         f->d[FG_V], f->d[FG_P], g, f->skew_sp);
    count(f, 2);
  } else {
    lexsor_kernel(f, f->d[FG_U], f->d[FG_V], f->d[FG_P], f->flags, iters, relax0, cp, early_exit,
                  st, minRelax, stop, 0);
  }
}

// solveCoarseGrid's 40 sweeps: on the cluster when the coarse diagonals hold
// at least 128 cells (a step then spans thousands), else on one block.
static void launch_mg_coarse(fg_fluid* f, const int* stop, int cNX, int cNY, int CSP,
                             const uint8_t* cmask) {
  const int L = std::min(cNX - 2, cNY - 2);
  if (CSP && L >= 128 && g_lex_cluster.load() == 1) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(LEX_CLUSTER);
    cfg.blockDim = dim3(MG_THREADS);
    cfg.stream = f->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = LEX_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_mg_coarse<true>, (const float*)f->err, f->err2,
                           (const uint8_t*)f->flags, stop, f->g, cNX, cNY, 40, 1.6f, CSP,
                           cmask) == cudaSuccess)
      return;
    cudaGetLastError();
  }
  k_mg_coarse<false><<<1, MG_THREADS, 0, f->stream>>>(f->err, f->err2, f->flags, stop, f->g,
                                                       cNX, cNY, 40, 1.6f, CSP, cmask);
}

cudaError_t launch_multigrid(fg_fluid* f, int num_iters, float dt) {
  float cp = f->density * f->h / dt;  // fluid.go:560
  const int cNX = (f->NX + 1) / 2, cNY = (f->NY + 1) / 2;
  if ((size_t)cNX * cNY > (size_t)f->NX * f->P) return cudaErrorInvalidValue;
  // Scratch: the fine residual in rhs, the coarse right-hand side and
  // solution in err / err2, the stop latch and the smoothers' statistics in
  // the correction solve's control block (unused by this scheme).
  int* stop = reinterpret_cast<int*>(f->ectl);
  DevStats* sm = reinterpret_cast<DevStats*>(reinterpret_cast<char*>(f->ectl) + 64);
  cudaError_t e = cudaMemsetAsync(f->ectl, 0, 64 + sizeof(DevStats), f->stream);
  if (e != cudaSuccess) return e;
  dim3 gr = cell_grid(f), bl(BX, BY);
  dim3 cg((cNY + BX - 1) / BX, (cNX + BY - 1) / BY);
  // The coarse grid diagonal-major when it fits the scratch fields (err,
  // err2; its mask in rhs_e) and the fine one is (the handle has the copies).
  const int csp = (cNX + 31) / 32 * 32;
  const int CSP = f->skew[0] && (size_t)(cNX + cNY - 1) * csp <= (size_t)f->NX * f->P ? csp : 0;
  uint8_t* cmask = reinterpret_cast<uint8_t*>(f->rhs_e);
  for (int it = 0; it < num_iters; ++it) {
    count(f, 8);
    run_lexsor(f, 3, 1.5f, cp, 0, sm, 1.5f, stop, nullptr);
    k_mg_check<<<1, 1, 0, f->stream>>>(sm, f->dstats, stop, f->prm.tolerance, 0);
    k_mg_residual<<<gr, bl, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->d[FG_P], f->flags, f->rhs,
                                            stop, f->g);
    k_mg_restrict<<<cg, bl, 0, f->stream>>>(f->rhs, f->err, stop, f->g, cNX, cNY, CSP, f->flags,
                                            cmask);
    launch_mg_coarse(f, stop, cNX, cNY, CSP, cmask);
    k_mg_apply<<<gr, bl, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->d[FG_P], f->err2, f->flags,
                                         stop, cp, f->g, cNX, cNY, CSP);
    run_lexsor(f, 3, 1.2f, cp, 0, sm, 1.2f, stop, nullptr);
    k_mg_check<<<1, 1, 0, f->stream>>>(sm, f->dstats, stop, f->prm.tolerance, 1);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------------------ multigrid Jacobi
// The MULTIGRID scheme: V(2,2) cycles on the masked Poisson system of the
// Jacobi scheme.  A coarse cell covers up to 2 x 2 fine cells (the ghost
// ring coarsens along its own row or column) and is fluid if any of them is;
// its flag bytes come from that mask as the fine ones come from S.  The
// smoother is the Jacobi scheme's sweep kernel with weight kMgOmega *
// PressureDamping (undamped Jacobi leaves the high frequencies a coarse grid
// cannot see); the coarse right-hand side is the sum of the children's
// residuals (the coarse operator has the fine one's form at twice the
// spacing, so the sum is the scaled average); the correction returns by
// bilinear interpolation (weights 9, 3, 3, 1) over the active coarse cells
// around each fine cell.  Every operation has a fixed order, restated by
// the oracle, so the result is bitwise reproducible.
constexpr int kMgPre = 2, kMgPost = 2, kMgCoarse = 32;

namespace {

// Rows of the fine grid (NXf rows) under coarse row I of NXc: the ring row
// under the ring, else rows 2I-1 and 2I of the interior.
__host__ __device__ __forceinline__ void mg_children(int I, int NXc, int NXf, int& a, int& b) {
  if (I == 0) {
    a = b = 0;
  } else if (I == NXc - 1) {
    a = b = NXf - 1;
  } else {
    a = 2 * I - 1;
    b = min(2 * I, NXf - 2);
  }
}

__global__ void k_mg_mask(const float* __restrict__ Sf, Grid gf, float* __restrict__ Sc, Grid gc) {
  int J = blockIdx.x * blockDim.x + threadIdx.x;
  int I = blockIdx.y * blockDim.y + threadIdx.y;
  if (I >= gc.NX || J >= gc.NY) return;
  int a0, a1, b0, b1;
  mg_children(I, gc.NX, gf.NX, a0, a1);
  mg_children(J, gc.NY, gf.NY, b0, b1);
  float v = 0.0f;
  for (int a = a0; a <= a1; ++a)
    for (int b = b0; b <= b1; ++b) v = fmaxf(v, Sf[a * gf.P + b]);
  Sc[I * gc.P + J] = v;
}

__global__ void k_mg_weights(const uint8_t* __restrict__ flags, float* __restrict__ w, float om,
                             Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const uint8_t fl = flags[i * g.P + j];
  w[i * g.P + j] = flag_active(fl) ? om / (float)flag_count(fl) : 0.0f;
}

// Coarse right-hand side at coarse cell (I, J): the sum of the active
// children's residuals b - (s x - (x_w + x_e + x_s + x_n)), and w * b.
__device__ __forceinline__ void mg_restrict_cell(int I, int J, const float* __restrict__ xf,
                                                 const float* __restrict__ bf,
                                                 const uint8_t* __restrict__ flf, const Grid& gf,
                                                 const uint8_t* __restrict__ flc,
                                                 const float* __restrict__ wc,
                                                 float* __restrict__ bc, float* __restrict__ bwc,
                                                 const Grid& gc) {
  const int cc = I * gc.P + J;
  float rs = 0.0f;
  if (flag_active(flc[cc])) {
    int a0, a1, b0, b1;
    mg_children(I, gc.NX, gf.NX, a0, a1);
    mg_children(J, gc.NY, gf.NY, b0, b1);
    for (int a = a0; a <= a1; ++a)
      for (int b = b0; b <= b1; ++b) {
        const int cf = a * gf.P + b;
        const uint8_t fl = flf[cf];
        if (!flag_active(fl)) continue;
        float nb = xf[cf - gf.P] + xf[cf + gf.P] + xf[cf - 1] + xf[cf + 1];
        float ax = (float)flag_count(fl) * xf[cf] - nb;
        rs = rs + (bf[cf] - ax);
      }
  }
  bc[cc] = rs;
  bwc[cc] = wc[cc] * rs;
}
__global__ void k_mg_restrict(const float* __restrict__ xf, const float* __restrict__ bf,
                              const uint8_t* __restrict__ flf, Grid gf,
                              const uint8_t* __restrict__ flc, const float* __restrict__ wc,
                              float* __restrict__ bc, float* __restrict__ bwc, Grid gc) {
  int J = blockIdx.x * blockDim.x + threadIdx.x;
  int I = blockIdx.y * blockDim.y + threadIdx.y;
  if (I < 1 || J < 1 || I > gc.NX - 2 || J > gc.NY - 2) return;
  mg_restrict_cell(I, J, xf, bf, flf, gf, flc, wc, bc, bwc, gc);
}

// x_f += the bilinear interpolation of x_c over the active coarse cells
// around the active fine cell (i, j).
__device__ __forceinline__ void mg_prolong_cell(int i, int j, const float* __restrict__ xc,
                                                const uint8_t* __restrict__ flc, const Grid& gc,
                                                float* __restrict__ xf,
                                                const uint8_t* __restrict__ flf, const Grid& gf) {
  const int cf = i * gf.P + j;
  if (!flag_active(flf[cf])) return;
  const int I = (i - 1) / 2 + 1, J = (j - 1) / 2 + 1;
  const int di = ((i - 1) & 1) ? 1 : -1, dj = ((j - 1) & 1) ? 1 : -1;
  const int ci[4] = {I, I + di, I, I + di}, cj[4] = {J, J, J + dj, J + dj};
  const float wt[4] = {9.0f, 3.0f, 3.0f, 1.0f};
  float num = 0.0f, den = 0.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int cc = ci[k] * gc.P + cj[k];
    if (!flag_active(flc[cc])) continue;
    num = num + wt[k] * xc[cc];
    den = den + wt[k];
  }
  const float e = den > 0.0f ? num / den : 0.0f;
  xf[cf] = xf[cf] + e;
}
__global__ void k_mg_prolong(const float* __restrict__ xc, const uint8_t* __restrict__ flc, Grid gc,
                             float* __restrict__ xf, const uint8_t* __restrict__ flf, Grid gf) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i < 1 || j < 1 || i > gf.NX - 2 || j > gf.NY - 2) return;
  mg_prolong_cell(i, j, xc, flc, gc, xf, flf, gf);
}

// The bottom of the V-cycle in one block, in shared memory: levels l0 ..
// n-1 (a launch per operation would cost more than their work, and their
// arrays fit on one SM).  The block copies the levels' weights and flags
// and level l0's right-hand side into shared memory (rows of NY, no pitch
// padding), zeroes the iterates, runs the same per-cell operations as the
// launches above and the Jacobi sweep kernel -- zero-started pre-smoothing
// and restriction down to the coarsest level, its sweeps, then
// prolongation and post-smoothing back up -- and writes level l0's iterate
// back to its buffer 0.  Every level starts in buffer 0 and makes an even
// number of sweeps, so its iterate ends in buffer 0; only interior cells
// are written and the ghost rings stay 0 as the sweep kernel leaves them.
constexpr int kMgFuseLevels = 12, kMgFuseThreads = 1024;
constexpr int kMgSmemBytes = 200 * 1024;  // dynamic shared memory of k_mg_bottom
struct MgFused {
  Grid gg[kMgFuseLevels];               // the levels in global memory (pitched)
  Grid gs[kMgFuseLevels];               // the same in shared memory (pitch NY)
  const uint8_t* flags[kMgFuseLevels];  // global
  const float* w[kMgFuseLevels];        // global
  const float* b0;                      // level l0's right-hand side and w * b (global)
  const float* bw0;
  float* x0;                            // level l0's buffer 0 (global): the result
  int foff[kMgFuseLevels];              // first float of each level's arrays in shared memory
  int boff[kMgFuseLevels];              // first byte of each level's flags in shared memory
  int n;                                // levels held (the first is l0)
};
// A level's arrays in shared memory: five float arrays of NX * NY, then flags.
struct MgSm {
  float *x0, *x1, *b, *bw, *w;
  uint8_t* fl;
};
__device__ __forceinline__ MgSm mg_sm(const MgFused& m, int l, float* fs, uint8_t* bs) {
  const int n = m.gs[l].NX * m.gs[l].NY;
  float* p = fs + m.foff[l];
  return MgSm{p, p + n, p + 2 * n, p + 3 * n, p + 4 * n, bs + m.boff[l]};
}

__device__ __forceinline__ void mg_fused_sweeps(const MgSm& a, const Grid& g, int ns, bool zero,
                                                float om1) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kMgFuseThreads / 32;
  for (int s = 0; s < ns; ++s) {
    const float* xs = (s & 1) ? a.x1 : a.x0;
    float* xd = (s & 1) ? a.x0 : a.x1;
    const bool z = zero && s == 0;
    for (int i = 1 + warp; i < g.NX - 1; i += nw)
      for (int j = 1 + lane; j < g.NY - 1; j += 32) {
        const int c = i * g.P + j;
        float xc = 0.0f, nb;
        if (!z) {
          xc = xs[c];
          nb = xs[c - g.P] + xs[c + g.P] + xs[c - 1] + xs[c + 1];
        } else {
          nb = 0.0f + 0.0f + 0.0f + 0.0f;
        }
        float y = __fmaf_rn(a.w[c], nb, a.bw[c]);
        y = __fmaf_rn(om1, xc, y);
        xd[c] = y;
      }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kMgFuseThreads)
    k_mg_bottom(const __grid_constant__ MgFused m, float om1) {
  extern __shared__ __align__(16) float mg_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kMgFuseThreads / 32;
  uint8_t* bsm = reinterpret_cast<uint8_t*>(mg_smem);
  const int last = m.n - 1;
  for (int l = 0; l <= last; ++l) {
    const MgSm a = mg_sm(m, l, mg_smem, bsm);
    const Grid& gg = m.gg[l];
    const Grid& gs = m.gs[l];
    for (int i = warp; i < gs.NX; i += nw)
      for (int j = lane; j < gs.NY; j += 32) {
        const int cs = i * gs.P + j, cg = i * gg.P + j;
        a.w[cs] = m.w[l][cg];
        a.fl[cs] = m.flags[l][cg];
        a.b[cs] = l == 0 ? m.b0[cg] : 0.0f;
        a.bw[cs] = l == 0 ? m.bw0[cg] : 0.0f;
        a.x0[cs] = 0.0f;
        a.x1[cs] = 0.0f;
      }
  }
  __syncthreads();
  for (int l = 0; l < last; ++l) {
    const MgSm f = mg_sm(m, l, mg_smem, bsm), c = mg_sm(m, l + 1, mg_smem, bsm);
    mg_fused_sweeps(f, m.gs[l], kMgPre, true, om1);
    const Grid& gf = m.gs[l];
    const Grid& gc = m.gs[l + 1];
    for (int I = 1 + warp; I < gc.NX - 1; I += nw)
      for (int J = 1 + lane; J < gc.NY - 1; J += 32)
        mg_restrict_cell(I, J, f.x0, f.b, f.fl, gf, c.fl, c.w, c.b, c.bw, gc);
    __syncthreads();
  }
  mg_fused_sweeps(mg_sm(m, last, mg_smem, bsm), m.gs[last], kMgCoarse, true, om1);
  for (int l = last - 1; l >= 0; --l) {
    const MgSm f = mg_sm(m, l, mg_smem, bsm), c = mg_sm(m, l + 1, mg_smem, bsm);
    const Grid& gf = m.gs[l];
    const Grid& gc = m.gs[l + 1];
    for (int i = 1 + warp; i < gf.NX - 1; i += nw)
      for (int j = 1 + lane; j < gf.NY - 1; j += 32)
        mg_prolong_cell(i, j, c.x0, c.fl, gc, f.x0, f.fl, gf);
    __syncthreads();
    mg_fused_sweeps(f, gf, kMgPost, false, om1);
  }
  const MgSm a = mg_sm(m, 0, mg_smem, bsm);
  for (int i = warp; i < m.gs[0].NX; i += nw)
    for (int j = lane; j < m.gs[0].NY; j += 32) m.x0[i * m.gg[0].P + j] = a.x0[i * m.gs[0].P + j];
}

inline dim3 level_grid(const Grid& g) { return dim3((g.NY + BX - 1) / BX, (g.NX + BY - 1) / BY); }

// ns (<= TMAX) damped Jacobi sweeps src -> dst on one level (4-warp
// regions on levels with fewer 8-warp regions than SMs, as enqueue_jacobi).
void mg_sweeps(cudaStream_t st, const MgLevelDev& v, const float* src, float* dst, float om1,
               PCtl* ctl, int t0, int ns, int sel, int zero) {
  dim3 gr(span_count(v.g.NY, RJ), span_count(v.g.NX, RI));
  const TmaDevice* dv = tma_ready(st);
  const bool narrow = dv && dv->sms > 0 && (long long)gr.x * gr.y < dv->sms;
#define FG_MGJ(F, NW)                                                                           \
  k_jacobi_rb<false, F, false, false, NW>                                                       \
      <<<dim3(gr.x, span_count(v.g.NX, RT * NW)), 32 * NW, 0, st>>>(                            \
          src, dst, v.w, v.bw, nullptr, v.flags, om1, ctl, 0, t0, ns, 0.0f, sel, zero, v.g,     \
          nullptr, nullptr, nullptr, nullptr, nullptr)
  if (narrow) {
    if (ns == TMAX) FG_MGJ(true, NWARP / 2); else FG_MGJ(false, NWARP / 2);
  } else {
    if (ns == TMAX) FG_MGJ(true, NWARP); else FG_MGJ(false, NWARP);
  }
#undef FG_MGJ
}

// The V-cycles of one solve.  cur[l] names the buffer of level l holding
// its iterate; the last smoothing of level 0 reports to the main control
// block (sweeps = cycles, sel = the buffer of the result).
// The first coarse level from which all levels down fit k_mg_bottom's
// shared memory (at most kMgFuseLevels of them); the level count when none
// does.
int mg_bottom_level(const MgHier* h) {
  const int L = (int)h->lv.size();
  long long bytes = 0;
  int bottom = L;
  for (int l = L - 1; l >= 1 && L - l <= kMgFuseLevels; --l) {
    bytes += (5 * (long long)sizeof(float) + 1) * h->lv[l].g.NX * h->lv[l].g.NY;
    if (bytes > kMgSmemBytes - 64) break;
    bottom = l;
  }
  return bottom;
}

struct MgRun {
  fg_fluid* f;
  MgHier* h;
  float om1;
  int cycles;
  std::vector<int> cur;
  int bottom;  // the first level run by k_mg_bottom (levels below it included)
  int launches = 0;
  void smooth(int l, int ns, bool zero, bool last) {
    MgLevelDev& v = h->lv[l];
    const int to = 1 - cur[l];
    PCtl* ctl = last ? (PCtl*)f->pctl : (PCtl*)h->ctl;
    mg_sweeps(f->stream, v, v.x[cur[l]], v.x[to], om1, ctl, last ? cycles - ns : 0, ns, to,
              zero ? 1 : 0);
    cur[l] = to;
    ++launches;
  }
  void cycle(int l, bool zero, bool last) {
    const int L = (int)h->lv.size();
    if (l == bottom) {
      MgFused m{};
      m.n = L - l;
      int fo = 0;
      for (int k = 0; k < m.n; ++k) {
        const MgLevelDev& v = h->lv[l + k];
        m.gg[k] = v.g;
        m.gs[k] = make_grid(v.g.NX, v.g.NY, v.g.NY, v.g.h);
        m.flags[k] = v.flags;
        m.w[k] = v.w;
        m.foff[k] = fo;
        fo += 5 * v.g.NX * v.g.NY;
      }
      int bo = fo * (int)sizeof(float);
      for (int k = 0; k < m.n; ++k) {
        m.boff[k] = bo;
        bo += h->lv[l + k].g.NX * h->lv[l + k].g.NY;
      }
      m.b0 = h->lv[l].b;
      m.bw0 = h->lv[l].bw;
      m.x0 = h->lv[l].x[0];
      k_mg_bottom<<<1, kMgFuseThreads, bo, f->stream>>>(m, om1);
      cur[l] = 0;
      ++launches;
      return;
    }
    if (l == L - 1) {
      for (int k = 0; k < kMgCoarse / TMAX; ++k) smooth(l, TMAX, zero && k == 0, false);
      return;
    }
    MgLevelDev& v = h->lv[l];
    MgLevelDev& c = h->lv[l + 1];
    smooth(l, kMgPre, zero, false);
    k_mg_restrict<<<level_grid(c.g), dim3(BX, BY), 0, f->stream>>>(v.x[cur[l]], v.b, v.flags, v.g,
                                                                   c.flags, c.w, c.b, c.bw, c.g);
    ++launches;
    cycle(l + 1, true, false);
    k_mg_prolong<<<level_grid(v.g), dim3(BX, BY), 0, f->stream>>>(c.x[cur[l + 1]], c.flags, c.g,
                                                                  v.x[cur[l]], v.flags, v.g);
    ++launches;
    smooth(l, kMgPost, false, last && l == 0);
  }
};

cudaError_t mg_solve(fg_fluid* f, int cycles, float om) {
  MgHier* h = f->mg;
  if (!h || h->lv.size() < 2) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(h->ctl, 0, sizeof(PCtl), f->stream);
  if (e != cudaSuccess) return e;
  const int L = (int)h->lv.size();
  const int bottom = mg_bottom_level(h);
  MgRun run{f, h, 1.0f - om, cycles, std::vector<int>(h->lv.size(), 0), bottom};
  for (int k = 0; k < cycles; ++k) run.cycle(0, k == 0, k == cycles - 1);
  count(f, run.launches);
  return cudaGetLastError();
}

}  // namespace

cudaError_t mg_kernel_setup() {
  return cudaFuncSetAttribute(k_mg_bottom, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              kMgSmemBytes);
}

void mg_free(fg_fluid* f) {
  if (!f->mg) return;
  cudaFree(f->mg->block);
  cudaFree(f->mg->ctl);
  delete f->mg;
  f->mg = nullptr;
}

cudaError_t launch_mg_rebuild(fg_fluid* f) {
  MgHier* h = f->mg;
  if (!h) return cudaSuccess;
  const float om = kMgOmega * f->prm.pressure_damping;
  for (size_t l = 1; l < h->lv.size(); ++l) {
    const MgLevelDev& p = h->lv[l - 1];
    const MgLevelDev& c = h->lv[l];
    k_mg_mask<<<level_grid(c.g), dim3(BX, BY), 0, f->stream>>>(p.S, p.g, c.S, c.g);
    cudaError_t e = launch_build_flags_on(f->stream, c.S, c.flags, c.g);
    if (e != cudaSuccess) return e;
    k_mg_weights<<<level_grid(c.g), dim3(BX, BY), 0, f->stream>>>(c.flags, c.w, om, c.g);
  }
  h->omega = om;
  return cudaGetLastError();
}

cudaError_t launch_pressure(fg_fluid* f, int num_iters, float dt, bool fuse_turb) {
  float cp = f->density * f->h / dt;  // fluid.go:158
  cudaError_t e;
  f->jacobi_kernel = FG_JACOBI_KERNEL_NONE;
  if (f->prm.scheme == FG_SCHEME_LEXSOR) {
    count(f);
    // (The correction solve's control block is free in this scheme: its
    // first words hold the speculative early exit's sweep index.)
    run_lexsor(f, num_iters, f->prm.relaxation, cp, f->prm.early_exit, f->dstats, 1.2f, nullptr,
               reinterpret_cast<int*>(f->ectl));
    return cudaGetLastError();
  }
  PCtl* ctl = (PCtl*)f->pctl;
  PCtl* ectl = (PCtl*)f->ectl;
  dim3 gr = cell_grid(f), bl(BX, BY);
  const bool mgs = f->prm.scheme == FG_SCHEME_MULTIGRID && !f->batch;
  float om = mgs ? kMgOmega * f->prm.pressure_damping
                 : f->prm.jacobi_omega * f->prm.pressure_damping;
  if (f->batch) {
    // Every scene solves (the batch forbids early exit and refinement);
    // no statistics.
    count(f);
    FG_CELLS_BATCH(f, setup_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V], f->phi,
                   f->rhs, f->wgt, f->bw, (const uint8_t*)f->flags, om, 1);
    if ((e = jacobi_solve_batch(f, ctl, f->bw, f->phi, f->phi2)) != cudaSuccess) return e;
    count(f);
    FG_CELLS_BATCH(f, grad_batch_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V],
                   f->partner[FG_U], f->partner[FG_V], f->d[FG_P], (const float*)f->phi,
                   (const float*)f->phi2, (const PCtl*)ctl, (const float*)f->rhs,
                   (const uint8_t*)f->flags, cp, (const float2*)f->noise,
                   f->prm.turbulence_strength * dt, fuse_turb ? 1 : 0, f->step_u2, f->step_v2);
    swap_state(f, FG_U);
    swap_state(f, FG_V);
    return cudaGetLastError();
  }
  // sel = 0 (phi) until a launch runs.
  if ((e = cudaMemsetAsync(ctl, 0, sizeof(PCtl), f->stream)) != cudaSuccess) return e;
  count(f);
  launch_pdl(k_setup_system, gr, bl, 0, f->stream, f->d[FG_U], f->d[FG_V], f->phi, f->rhs,
             f->wgt, f->bw, f->flags, om, num_iters == 0 ? 1 : 0, f->g, f->P, f->step_fu,
             f->step_fv);
  mark(f, "pressure setup");
  if (num_iters > 0) {
    e = mgs ? mg_solve(f, num_iters, om)
            : jacobi_solve(f, ctl, f->rhs, f->bw, f->phi, f->phi2, num_iters, true, false,
                           &f->jacobi_kernel);
    if (e != cudaSuccess) return e;
  }
  mark(f, "jacobi sweeps");
  bool refine = f->prm.refine_sweeps > 0;
  if (refine) {
    if ((e = jacobi_solve(f, ectl, f->rhs, f->bw, f->err, f->err2, f->prm.refine_sweeps, false,
                          true)) != cudaSuccess)
      return e;
    mark(f, "outer correction");
  }
  dim3 rg((f->NY + BX - 1) / BX, (f->NX + BY * GR - 1) / (BY * GR));
  int nb = rg.x * rg.y;
  if (!partials_fit(f, 5, nb)) return cudaErrorInvalidValue;
  count(f);
  launch_pdl(k_grad_fused, rg, bl, 0, f->stream, f->d[FG_U], f->d[FG_V], f->partner[FG_U],
             f->partner[FG_V], f->d[FG_P], f->phi, f->phi2, ctl, f->err, f->err2,
             refine ? ectl : nullptr, f->rhs, f->flags, cp, f->noise,
             f->prm.turbulence_strength * dt, fuse_turb ? 1 : 0, f->partials, f->g, f->step_fu,
             f->step_fv, f->step_u2, f->step_v2);
  swap_state(f, FG_U);
  swap_state(f, FG_V);
  count(f);
  launch_pdl(k_combine_store<5, StoreDivP>, dim3(1), dim3(1024), 0, f->stream, f->partials, nb,
             0x12u, StoreDivP{f->dstats, num_iters > 0 ? ctl : nullptr});
  return cudaGetLastError();
}

cudaError_t launch_store_phi(fg_fluid* f, float* dst) {
  int n = f->NX * f->P;
  count(f);
  const bool refine = f->prm.refine_sweeps > 0;
  k_store_phi<<<(n + 255) / 256, 256, 0, f->stream>>>(f->phi, f->phi2, (const PCtl*)f->pctl,
                                                      f->err, f->err2,
                                                      refine ? (const PCtl*)f->ectl : nullptr,
                                                      dst, n);
  return cudaGetLastError();
}

cudaError_t launch_grad_replay(fg_fluid* f, float dt, const float* phi, bool fuse_turb) {
  float cp = f->density * f->h / dt;  // fluid.go:158
  if (f->batch) {
    count(f);
    FG_CELLS_BATCH(f, grad_batch_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V],
                   f->partner[FG_U], f->partner[FG_V], f->d[FG_P], phi, phi,
                   (const PCtl*)f->pctl, (const float*)f->rhs, (const uint8_t*)f->flags, cp,
                   (const float2*)f->noise, f->prm.turbulence_strength * dt, fuse_turb ? 1 : 0,
                   f->step_u2, f->step_v2);
    swap_state(f, FG_U);
    swap_state(f, FG_V);
    return cudaGetLastError();
  }
  dim3 rg((f->NY + BX - 1) / BX, (f->NX + BY * GR - 1) / (BY * GR)), bl(BX, BY);
  if (!partials_fit(f, 5, rg.x * rg.y)) return cudaErrorInvalidValue;
  count(f);
  // The potential is the same buffer whichever one the control block names;
  // the statistics partials it writes are not combined.
  k_grad_fused<<<rg, bl, 0, f->stream>>>(
      f->d[FG_U], f->d[FG_V], f->partner[FG_U], f->partner[FG_V], f->d[FG_P], phi, phi,
      (const PCtl*)f->pctl, nullptr, nullptr, nullptr, f->rhs, f->flags, cp, f->noise,
      f->prm.turbulence_strength * dt, fuse_turb ? 1 : 0, f->partials, f->g, f->step_fu,
      f->step_fv, f->step_u2, f->step_v2);
  swap_state(f, FG_U);
  swap_state(f, FG_V);
  return cudaGetLastError();
}

}  // namespace fg

// ===========================================================================
// Projection without allocation.
//
// Some callers cannot allocate device memory at the moment they need a
// projection: an embedding engine whose allocator owns all of the device
// memory, a real-time loop that forbids cudaMalloc (it may synchronise the
// device), or code running where allocation is not allowed at all.  For them
// fg_project_noalloc runs the Jacobi projection on caller-owned fields using
// the scratch array below instead of the handle's buffers.  The array is a
// fixed part of the library image, so every GPU that loads the library holds
// it (about 21 MiB) until the process exits.
// ===========================================================================
namespace fg {
namespace {

constexpr size_t kNoAllocMaxCells = (size_t)FG_NOALLOC_MAX_CELLS;  // num_x * padded num_y
constexpr int kNoAllocSlots = 4096;                                  // Jacobi launches per call
constexpr size_t kNoAllocCtlBytes = 256 + sizeof(unsigned) * kNoAllocSlots;
// The status word: nonzero when a bounded wait of the last call gave up.
constexpr size_t kNoAllocStatusOff = 21 * kNoAllocMaxCells + kNoAllocCtlBytes;
constexpr size_t kNoAllocBytes = kNoAllocStatusOff + 256;

// Scratch shared by every call on a device: phi, phi2, rhs, w, bw (floats),
// the flag bytes, the control block and the status word, carved at fixed
// offsets with the solver's own pitch (num_y rounded up to 32).  It keeps
// the previous call's contents; each call rewrites or clears what it reads.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Flag bytes from a caller-owned S (nonzero = fluid).
__global__ void k_noalloc_flags(const float* __restrict__ S, uint8_t* __restrict__ flags, Grid g,
                                int Ps) {
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
  flags[i * Ps + j] = fl;
}

// The scratch array's address per CUDA context (context_key), looked up by
// the first call made in each context.  A full table is not an error: the
// address is then looked up on every call.
constexpr int kNoAllocCtx = 64;
std::mutex g_noalloc_mu;
unsigned long long g_noalloc_key[kNoAllocCtx] = {};
void* g_noalloc_ptr[kNoAllocCtx] = {};
int g_noalloc_used = 0;
std::atomic<int> g_noalloc_stall{-1};

cudaError_t noalloc_scratch(void** out) {
  unsigned long long key = context_key();
  if (key) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    for (int k = 0; k < g_noalloc_used; ++k)
      if (g_noalloc_key[k] == key) {
        *out = g_noalloc_ptr[k];
        return cudaSuccess;
      }
  }
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return e;
  if (!key) key = context_key();  // the lookup made the primary context current
  if (key) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_used < kNoAllocCtx) {
      g_noalloc_key[g_noalloc_used] = key;
      g_noalloc_ptr[g_noalloc_used++] = ptr;
    }
  }
  *out = ptr;
  return cudaSuccess;
}

}  // namespace

void set_noalloc_stall(int tile) { g_noalloc_stall.store(tile < 0 ? -1 : tile); }

}  // namespace fg

extern "C" int fg_project_noalloc(float* u, float* v, float* p, const float* s, int num_x,
                                  int num_y, int pitch, float density, float h, float dt,
                                  int num_iters, float jacobi_omega, float pressure_damping,
                                  int tb_depth, int early_exit, float tolerance, void* stream) {
  using namespace fg;
  if (!u || !v || !p || !s || num_x < 3 || num_y < 3 || pitch < num_y || num_iters < 0 ||
      !(h > 0.0f) || dt == 0.0f)
    return FG_ERR_INVALID;
  const int Ps = (num_y + 31) / 32 * 32;  // solver pitch inside the scratch
  if ((size_t)num_x * (size_t)Ps > kNoAllocMaxCells) return FG_ERR_TOO_LARGE;
  // The caller's fields are indexed with 32-bit integers too.
  if ((size_t)num_x * (size_t)pitch > (size_t)INT_MAX) return FG_ERR_TOO_LARGE;
  const int T = clamp_tb(tb_depth);
  // In 64 bits: a num_iters near INT_MAX must not wrap below the limit.
  const long long nlaunch = ((long long)num_iters + T - 1) / T;
  if (nlaunch > kNoAllocSlots) return FG_ERR_TOO_LARGE;
  void* base = nullptr;
  if (noalloc_scratch(&base) != cudaSuccess) return FG_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* b = (unsigned char*)base;
  float* phi = (float*)b;
  float* phi2 = (float*)(b + 4 * kNoAllocMaxCells);
  float* rhs = (float*)(b + 8 * kNoAllocMaxCells);
  float* W = (float*)(b + 12 * kNoAllocMaxCells);
  float* BW = (float*)(b + 16 * kNoAllocMaxCells);
  uint8_t* flags = b + 20 * kNoAllocMaxCells;
  PCtl* ctl = (PCtl*)(b + 21 * kNoAllocMaxCells);
  int* status = (int*)(b + kNoAllocStatusOff);
  Grid g = make_grid(num_x, num_y, pitch, h);   // caller fields
  Grid gs = make_grid(num_x, num_y, Ps, h);     // solver arrays
  float om = jacobi_omega * pressure_damping;
  float cp = density * h / dt;
  dim3 gr((num_y + BX - 1) / BX, (num_x + BY - 1) / BY), bl(BX, BY);
  // The control words and the status word start at zero (sel = 0 until a
  // launch runs).
  if (cudaMemsetAsync(ctl, 0, pctl_bytes((int)nlaunch), st) != cudaSuccess ||
      cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess)
    return FG_ERR_CUDA;
  k_noalloc_flags<<<gr, bl, 0, st>>>(s, flags, g, Ps);
  k_setup_system<<<gr, bl, 0, st>>>(u, v, phi, rhs, W, BW, flags, om, num_iters == 0 ? 1 : 0, g,
                                    Ps, nullptr, nullptr);
  int n = 0;
  if (num_iters > 0 &&
      enqueue_jacobi(st, gs, ctl, rhs, BW, W, flags, phi, phi2, num_iters, T, om,
                     early_exit ? 1 : 0, tolerance, &n, nullptr, nullptr, nullptr, nullptr,
                     nullptr, status, nullptr, -1, g_noalloc_stall.load()) != cudaSuccess)
    return FG_ERR_CUDA;
  k_grad<<<gr, bl, 0, st>>>(u, v, p, phi, phi2, ctl, nullptr, nullptr, nullptr, flags, cp, g, Ps);
  return cudaGetLastError() == cudaSuccess ? FG_OK : FG_ERR_CUDA;
}

extern "C" int fg_project_noalloc_status(void* stream) {
  using namespace fg;
  int v = 0;
  cudaStream_t st = (cudaStream_t)stream;
  // The symbol is resolved in the current context, like the scratch itself.
  if (cudaMemcpyFromSymbolAsync(&v, g_noalloc_scratch, sizeof(int), kNoAllocStatusOff,
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return FG_ERR_CUDA;
  return v ? FG_ERR_TIMEOUT : FG_OK;
}
