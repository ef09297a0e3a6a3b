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
//    updates as in the serial loop, so the result is bit-identical.  One CTA
//    owns one grid; a new sweep starts only once the previous sweep is known
//    not to trigger the early exit (some cell with |div| >= tolerance).
//  * JACOBI relaxes the same masked Poisson system for the cell potential
//    phi (the accumulated per-cell correction of the SOR loop):
//        s_c phi_c - sum_n phi_n = -div_c,   phi = 0 off the active cells,
//    then applies U_face += S_R phi_L - S_L phi_R (and likewise V) and
//    p = cp * phi.  Sweeps run temporally blocked: each launch loads a tile
//    with a halo as wide as its sweep count into shared memory and relaxes it
//    there, so HBM sees one read and one write of phi per launch.  Optional
//    outer correction: an FP64 residual of the FP32 iterate, a correction
//    solve on it, phi += e.
#include <mutex>

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

constexpr int BX = 32, BY = 8;
inline dim3 cell_grid(const fg_fluid* f) {
  return dim3((f->NY + BX - 1) / BX, (f->NX + BY - 1) / BY);
}

// ------------------------------------------------------------------ LEXSOR
constexpr int LEX_THREADS = 1024;
constexpr int LEX_RING = 2048;  // sweeps in flight (a new sweep waits while the ring is full)

__global__ void __launch_bounds__(LEX_THREADS)
    k_lexsor(float* U, float* V, float* p, const uint8_t* __restrict__ flags, Grid g,
             int numIters, float relax0, float damping, float cp, float tol, int early_exit,
             DevStats* st) {
  __shared__ int s_start[LEX_RING];
  __shared__ unsigned s_max[LEX_RING];
  __shared__ int s_cont[LEX_RING];
  __shared__ int s_lo, s_hi, s_done, s_exit, s_last;
  const int P = g.P;
  const int ni = g.NX - 2, nj = g.NY - 2;  // interior extent
  const int D = ni + nj - 1;               // anti-diagonals d = i + j in [2, NX+NY-4]
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
  // Start sweep 0 at step 0.
  if (threadIdx.x == 0) {
    s_start[0] = 0;
    s_max[0] = 0u;
    s_cont[0] = 0;
    s_hi = 1;
  }
  __syncthreads();
  const float minRelax = 1.2f;
  // Bounded: each sweep takes D steps and starts at most D + 2 steps after
  // the previous one.
  const long long max_steps = (long long)numIters * (D + 2) + D + 4;
  for (long long tau = 0; tau < max_steps; ++tau) {
    int lo = s_lo, hi = s_hi;
    int W = hi - lo;
    int items = W * L;
    for (int q = threadIdx.x; q < items; q += LEX_THREADS) {
      int t = lo + q / L;
      int k = q - (q / L) * L;
      int r = t & (LEX_RING - 1);
      int delta = (int)(tau - s_start[r]);
      if (delta < 0 || delta >= D) continue;
      int d = 2 + delta;
      int i_lo = max(1, d - nj), i_hi = min(ni, d - 1);
      int i = i_lo + k;
      if (i > i_hi) continue;
      int j = d - i;
      int c = i * P + j;
      uint8_t fl = flags[c];
      if (!(fl & F_FLUID)) continue;
      float sx0 = fbit(fl, F_W), sx1 = fbit(fl, F_E), sy0 = fbit(fl, F_S), sy1 = fbit(fl, F_N);
      float s = sx0 + sx1 + sy0 + sy1;
      if (s == 0.0f) continue;
      float div = U[c + P] - U[c] + V[c + 1] - V[c];
      float absDiv = fabsf(div);
      if (!isnan(absDiv)) {
        atomicMax(&s_max[r], __float_as_uint(absDiv));
        if (absDiv >= tol) s_cont[r] = 1;
      }
      // Relaxation of sweep t (fluid.go:169-170).
      float iterProgress = (float)t / (float)numIters;
      float rel = relax0 - (relax0 - minRelax) * iterProgress;
      float pp = -div / s;
      pp *= rel;
      pp *= damping;
      p[c] += cp * pp;
      U[c] -= sx0 * pp;
      U[c + P] += sx1 * pp;
      V[c] -= sy0 * pp;
      V[c + 1] += sy1 * pp;
    }
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

// ------------------------------------------------------------------ parallel scheme
struct WTab {
  float w[5];  // w[s] = (omega * damping) / s
};

// b = -div on active cells, phi = 0 everywhere (ring included).
__global__ void k_setup_system(const float* __restrict__ U, const float* __restrict__ V,
                               float* __restrict__ phi, float* __restrict__ phi2,
                               float* __restrict__ rhs, const uint8_t* __restrict__ flags,
                               Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  int c = i * g.P + j;
  float b = 0.0f;
  if (flag_active(flags[c])) {
    float div = U[c + g.P] - U[c] + V[c + 1] - V[c];
    b = -div;
  }
  rhs[c] = b;
  phi[c] = 0.0f;
  phi2[c] = 0.0f;
}

__device__ __forceinline__ float jacobi_cell(float x, float nb, float b, int s, const WTab& w,
                                             float* r_out) {
  float t1 = b + nb;
  float r = __fmaf_rn(-(float)s, x, t1);
  *r_out = r;
  return __fmaf_rn(w.w[s], r, x);
}

// Temporally blocked Jacobi: `ns` sweeps of a TI x TJ tile with a halo of
// TMAX cells (ns <= TMAX) in shared memory.  Launch k of a solve first
// decides whether the solve already stopped (thread 0 of every CTA reads the
// same control words, so all CTAs agree); a running launch records the max
// |r| of its last sweep over the cells it owns in slots[k].
constexpr int TI = 32, TJ = 48, TMAX = 8;
constexpr int RI = TI + 2 * TMAX, RJ = TJ + 2 * TMAX;
constexpr int TB_THREADS = 256;

__global__ void __launch_bounds__(TB_THREADS)
    k_jacobi_tb(const float* __restrict__ src, float* __restrict__ dst,
                const float* __restrict__ rhs, const uint8_t* __restrict__ flags, WTab w,
                PCtl* ctl, int k, int t0, int ns, int check, float tol, int out_sel, Grid g) {
  __shared__ float ph[2][RI * RJ];
  __shared__ float rh[RI * RJ];
  __shared__ uint8_t sc[RI * RJ];
  __shared__ double red[32];
  __shared__ int skip;
  if (threadIdx.x == 0) {
    int sk = ctl->stop;
    if (!sk && check && k > 0 && __uint_as_float(ctl->slots[k - 1]) < tol) {
      sk = 1;
      ctl->stop = 1;
    }
    skip = sk;
  }
  __syncthreads();
  if (skip) return;
  const int i0 = blockIdx.y * TI - TMAX, j0 = blockIdx.x * TJ - TMAX;
  for (int q = threadIdx.x; q < RI * RJ; q += TB_THREADS) {
    int ri = q / RJ, rj = q - (q / RJ) * RJ;
    int gi = i0 + ri, gj = j0 + rj;
    float x = 0.0f, b = 0.0f;
    uint8_t s = 0;
    if (gi >= 0 && gi < g.NX && gj >= 0 && gj < g.NY) {
      int c = gi * g.P + gj;
      uint8_t fl = flags[c];
      x = src[c];
      if (flag_active(fl)) {
        s = (uint8_t)flag_count(fl);
        b = rhs[c];
      }
    }
    ph[0][q] = x;
    rh[q] = b;
    sc[q] = s;
  }
  __syncthreads();
  float mx = 0.0f;
  int cur = 0;
  for (int sw = 1; sw <= ns; ++sw) {
    const float* a = ph[cur];
    float* o = ph[cur ^ 1];
    const bool last = sw == ns;
    for (int q = threadIdx.x; q < RI * RJ; q += TB_THREADS) {
      int ri = q / RJ, rj = q - (q / RJ) * RJ;
      if (ri < sw || ri >= RI - sw || rj < sw || rj >= RJ - sw) continue;
      int s = sc[q];
      float y = 0.0f;
      if (s) {
        float nb = a[q - RJ] + a[q + RJ] + a[q - 1] + a[q + 1];
        float r;
        y = jacobi_cell(a[q], nb, rh[q], s, w, &r);
        if (last && ri >= TMAX && ri < TMAX + TI && rj >= TMAX && rj < TMAX + TJ) {
          float ar = fabsf(r);
          if (ar > mx) mx = ar;
        }
      }
      o[q] = y;
    }
    __syncthreads();
    cur ^= 1;
  }
  // Write the owned cells.
  for (int q = threadIdx.x; q < TI * TJ; q += TB_THREADS) {
    int oi = q / TJ, oj = q - (q / TJ) * TJ;
    int gi = i0 + TMAX + oi, gj = j0 + TMAX + oj;
    if (gi < g.NX && gj < g.NY) dst[gi * g.P + gj] = ph[cur][(oi + TMAX) * RJ + oj + TMAX];
  }
  double m = block_reduce<true>((double)mx, red);
  if (threadIdx.x == 0) {
    if (m > 0.0) atomicMax(&ctl->slots[k], __float_as_uint((float)m));
    if (blockIdx.x == 0 && blockIdx.y == 0) {
      ctl->sweeps = t0 + ns;
      ctl->last_launch = k;
      ctl->sel = out_sel;
    }
  }
}

// FP64 residual r = b - A phi of the current iterate: writes r (rounded to
// float) as the correction right-hand side and the block partials
// (sum r^2, max |r|).
__global__ void k_resid64(const float* __restrict__ phi0, const float* __restrict__ phi1,
                          const PCtl* __restrict__ ctl, const float* __restrict__ rhs,
                          const uint8_t* __restrict__ flags, float* __restrict__ rhs_e,
                          float* __restrict__ err, float* __restrict__ err2,
                          double* __restrict__ partials, Grid g) {
  __shared__ double red[32];
  const float* phi = ctl->sel ? phi1 : phi0;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  double r2 = 0.0, ra = 0.0;
  if (i < g.NX && j < g.NY) {
    int c = i * g.P + j;
    uint8_t fl = flags[c];
    float re = 0.0f;
    if (flag_active(fl)) {
      double nb = (double)phi[c - g.P] + (double)phi[c + g.P] + (double)phi[c - 1] +
                  (double)phi[c + 1];
      double r = ((double)rhs[c] + nb) - (double)flag_count(fl) * (double)phi[c];
      re = (float)r;
      r2 = r * r;
      ra = fabs(r);
    }
    if (rhs_e) {
      rhs_e[c] = re;
      err[c] = 0.0f;
      err2[c] = 0.0f;
    }
  }
  double s = block_reduce<false>(r2, red);
  double m = block_reduce<true>(ra, red);
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    int b = blockIdx.y * gridDim.x + blockIdx.x;
    partials[2 * b] = s;
    partials[2 * b + 1] = m;
  }
}

__global__ void k_add_correction(float* __restrict__ phi0, float* __restrict__ phi1,
                                 const float* __restrict__ e0, const float* __restrict__ e1,
                                 const PCtl* __restrict__ ctl, const PCtl* __restrict__ ectl,
                                 const uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  int c = i * g.P + j;
  if (!flag_active(flags[c])) return;
  float* phi = ctl->sel ? phi1 : phi0;
  const float* e = ectl->sel ? e1 : e0;
  phi[c] = phi[c] + e[c];
}

// Gradient subtract and pressure: U_face += S_R phi_L - S_L phi_R on faces
// with an active neighbour, V likewise, p = cp * phi on active cells, 0
// elsewhere (fill(f.p, 0) fluid.go:83 plus p += cp * delta fluid.go:224).
__global__ void k_grad(float* __restrict__ U, float* __restrict__ V, float* __restrict__ p,
                       const float* __restrict__ phi0, const float* __restrict__ phi1,
                       const PCtl* __restrict__ ctl, const uint8_t* __restrict__ flags, float cp,
                       Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  const float* phi = ctl->sel ? phi1 : phi0;
  int c = i * g.P + j;
  uint8_t fl = flags[c];
  bool act = flag_active(fl);
  if (i >= 1 && j >= 1 && j <= g.NY - 2) {
    bool actL = flag_active(flags[c - g.P]);
    if (act || actL) {
      float d = fbit(fl, F_FLUID) * phi[c - g.P] - fbit(fl, F_W) * phi[c];
      U[c] = U[c] + d;
    }
  }
  if (j >= 1 && i >= 1 && i <= g.NX - 2) {
    bool actB = flag_active(flags[c - 1]);
    if (act || actB) {
      float d = fbit(fl, F_FLUID) * phi[c - 1] - fbit(fl, F_S) * phi[c];
      V[c] = V[c] + d;
    }
  }
  p[c] = act ? cp * phi[c] : 0.0f;
}

__global__ void k_finish_parallel(const PCtl* __restrict__ ctl, DevStats* st) {
  st->sweeps = ctl->sweeps;
  st->last_maxdiv = (double)__uint_as_float(ctl->slots[ctl->last_launch]);
}

__global__ void k_store_resid(const double* __restrict__ r, DevStats* st) {
  st->resid_l2_sq = r[0];
  st->resid_max = r[1];
}

}  // namespace

static cudaError_t resid_stats(fg_fluid* f, bool write_rhs_e) {
  dim3 gr = cell_grid(f);
  int nb = gr.x * gr.y;
  count(f);
  k_resid64<<<gr, dim3(BX, BY), 0, f->stream>>>(
      f->phi, f->phi2, (PCtl*)f->pctl, f->rhs, f->flags, write_rhs_e ? f->rhs_e : nullptr,
      f->err, f->err2, f->partials, f->g);
  double* out = f->partials + 2 * (size_t)nb;
  count(f);
  k_combine<2><<<1, 1024, 0, f->stream>>>(f->partials, nb, 2u, out);
  count(f);
  k_store_resid<<<1, 1, 0, f->stream>>>(out, f->dstats);
  return cudaGetLastError();
}

size_t pctl_bytes(int n_slots) { return sizeof(PCtl) + sizeof(unsigned) * (size_t)n_slots; }

// Runs `iters` Jacobi sweeps of A x = b in launches of tb_depth sweeps; x
// ping-pongs between x0 and x1 and ctl->sel names the buffer holding the
// result.
static cudaError_t jacobi_solve(fg_fluid* f, PCtl* ctl, const float* b, float* x0, float* x1,
                                int iters, bool allow_exit) {
  WTab w;
  float om = f->prm.jacobi_omega * f->prm.pressure_damping;
  w.w[0] = 0.0f;
  for (int s = 1; s <= 4; ++s) w.w[s] = om / (float)s;
  int T = f->prm.tb_depth;
  if (T < 1) T = 1;
  if (T > TMAX) T = TMAX;
  dim3 gr((f->NY + TJ - 1) / TJ, (f->NX + TI - 1) / TI);
  int nlaunch = (iters + T - 1) / T;
  if (nlaunch > f->n_slots) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(ctl, 0, pctl_bytes(nlaunch), f->stream);
  if (e != cudaSuccess) return e;
  int check = allow_exit && f->prm.early_exit ? 1 : 0;
  const bool prof = f->profile && allow_exit;
  if (prof && (e = cudaEventRecord(f->prof_ev[0], f->stream)) != cudaSuccess) return e;
  for (int k = 0; k < nlaunch; ++k) {
    int t0 = k * T;
    int ns = iters - t0 < T ? iters - t0 : T;
    const float* src = (k & 1) ? x1 : x0;
    float* dst = (k & 1) ? x0 : x1;
    count(f);
    k_jacobi_tb<<<gr, TB_THREADS, 0, f->stream>>>(src, dst, b, f->flags, w, ctl, k, t0, ns, check,
                                                  f->prm.tolerance, (k & 1) ? 0 : 1, f->g);
  }
  if (prof) {
    if ((e = cudaEventRecord(f->prof_ev[1], f->stream)) != cudaSuccess) return e;
    f->prof_launches = nlaunch;
  }
  return cudaGetLastError();
}

int jacobi_launches(const fg_fluid* f, int iters) {
  int T = f->prm.tb_depth;
  if (T < 1) T = 1;
  if (T > TMAX) T = TMAX;
  return (iters + T - 1) / T;
}

cudaError_t launch_pressure(fg_fluid* f, int num_iters, float dt) {
  float cp = f->density * f->h / dt;  // fluid.go:158
  cudaError_t e;
  if (f->prm.scheme == FG_SCHEME_LEXSOR) {
    count(f);
    k_lexsor<<<1, LEX_THREADS, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->d[FG_P], f->flags,
                                                f->g, num_iters, f->prm.relaxation,
                                                f->prm.pressure_damping, cp, f->prm.tolerance,
                                                f->prm.early_exit, f->dstats);
    return cudaGetLastError();
  }
  PCtl* ctl = (PCtl*)f->pctl;
  PCtl* ectl = (PCtl*)f->ectl;
  dim3 gr = cell_grid(f), bl(BX, BY);
  // sel = 0 (phi) until a launch runs.
  if ((e = cudaMemsetAsync(ctl, 0, sizeof(PCtl), f->stream)) != cudaSuccess) return e;
  count(f);
  k_setup_system<<<gr, bl, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->phi, f->phi2, f->rhs,
                                           f->flags, f->g);
  if (num_iters > 0) {
    if ((e = jacobi_solve(f, ctl, f->rhs, f->phi, f->phi2, num_iters, true)) != cudaSuccess)
      return e;
    count(f);
    k_finish_parallel<<<1, 1, 0, f->stream>>>(ctl, f->dstats);
  }
  bool refine = f->prm.refine_sweeps > 0;
  if ((e = resid_stats(f, refine)) != cudaSuccess) return e;
  if (refine) {
    if ((e = jacobi_solve(f, ectl, f->rhs_e, f->err, f->err2, f->prm.refine_sweeps, false)) !=
        cudaSuccess)
      return e;
    count(f);
    k_add_correction<<<gr, bl, 0, f->stream>>>(f->phi, f->phi2, f->err, f->err2, ctl, ectl,
                                               f->flags, f->g);
    if ((e = resid_stats(f, false)) != cudaSuccess) return e;
  }
  count(f);
  k_grad<<<gr, bl, 0, f->stream>>>(f->d[FG_U], f->d[FG_V], f->d[FG_P], f->phi, f->phi2, ctl,
                                   f->flags, cp, f->g);
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
// it (about 13 MiB) until the process exits.
// ===========================================================================
namespace fg {
namespace {

constexpr size_t kNoAllocMaxCells = (size_t)FG_NOALLOC_MAX_CELLS;  // num_x * pitch
constexpr int kNoAllocSlots = 4096;                                  // Jacobi launches per call
constexpr size_t kNoAllocCtlBytes = 256 + sizeof(unsigned) * kNoAllocSlots;
constexpr size_t kNoAllocBytes = 13 * kNoAllocMaxCells + kNoAllocCtlBytes;

// Scratch shared by every call on a device: phi, phi2, rhs (floats), the
// flag bytes and the control block, carved at fixed offsets.  It keeps the
// previous call's contents; each call rewrites or clears what it reads.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Flag bytes from a caller-owned S (nonzero = fluid).
__global__ void k_noalloc_flags(const float* __restrict__ S, uint8_t* __restrict__ flags, Grid g) {
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

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[256] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the first call on each device does it).
cudaError_t noalloc_scratch(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace fg

extern "C" int fg_project_noalloc(float* u, float* v, float* p, const float* s, int num_x,
                                  int num_y, int pitch, float density, float h, float dt,
                                  int num_iters, float jacobi_omega, float pressure_damping,
                                  int tb_depth, int early_exit, float tolerance, void* stream) {
  using namespace fg;
  if (!u || !v || !p || !s || num_x < 3 || num_y < 3 || pitch < num_y || num_iters < 0 ||
      !(h > 0.0f) || dt == 0.0f)
    return FG_ERR_INVALID;
  if ((size_t)num_x * (size_t)pitch > kNoAllocMaxCells) return FG_ERR_TOO_LARGE;
  int T = tb_depth < 1 ? 1 : (tb_depth > TMAX ? TMAX : tb_depth);
  int nlaunch = (num_iters + T - 1) / T;
  if (nlaunch > kNoAllocSlots) return FG_ERR_TOO_LARGE;
  void* base = nullptr;
  if (noalloc_scratch(&base) != cudaSuccess) return FG_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* b = (unsigned char*)base;
  float* phi = (float*)b;
  float* phi2 = (float*)(b + 4 * kNoAllocMaxCells);
  float* rhs = (float*)(b + 8 * kNoAllocMaxCells);
  uint8_t* flags = b + 12 * kNoAllocMaxCells;
  PCtl* ctl = (PCtl*)(b + 13 * kNoAllocMaxCells);
  Grid g = make_grid(num_x, num_y, pitch, h);
  WTab w;
  float om = jacobi_omega * pressure_damping;
  w.w[0] = 0.0f;
  for (int k = 1; k <= 4; ++k) w.w[k] = om / (float)k;
  float cp = density * h / dt;
  dim3 gr((num_y + BX - 1) / BX, (num_x + BY - 1) / BY), bl(BX, BY);
  // The control words start at zero (sel = 0 until a launch runs).
  if (cudaMemsetAsync(ctl, 0, pctl_bytes(nlaunch), st) != cudaSuccess) return FG_ERR_CUDA;
  k_noalloc_flags<<<gr, bl, 0, st>>>(s, flags, g);
  k_setup_system<<<gr, bl, 0, st>>>(u, v, phi, phi2, rhs, flags, g);
  dim3 tg((num_y + TJ - 1) / TJ, (num_x + TI - 1) / TI);
  int check = early_exit ? 1 : 0;
  for (int k = 0; k < nlaunch; ++k) {
    int t0 = k * T;
    int ns = num_iters - t0 < T ? num_iters - t0 : T;
    const float* src = (k & 1) ? phi2 : phi;
    float* dst = (k & 1) ? phi : phi2;
    k_jacobi_tb<<<tg, TB_THREADS, 0, st>>>(src, dst, rhs, flags, w, ctl, k, t0, ns, check,
                                           tolerance, (k & 1) ? 0 : 1, g);
  }
  k_grad<<<gr, bl, 0, st>>>(u, v, p, phi, phi2, ctl, flags, cp, g);
  return cudaGetLastError() == cudaSuccess ? FG_OK : FG_ERR_CUDA;
}
