// Semi-Lagrangian and BFECC advection of the staggered velocity and the
// cell-centred smoke (pkg/fluid/fluid.go:291-434 and 909-1120).
//
// The reference stages results in the persistent newU/newV/newM buffers and
// copies them back (fluid.go:331-332, 433); faces or cells it does not
// advect keep whatever that buffer held ("stale" values, e.g. faces next to
// a solid).  The kernels reproduce that: a face takes the advected value if
// it is advected, else the border value of the field being advected if it
// lies on the ghost ring (copyBorder, fluid.go:293-294), else the stale
// staging value.  The result is written to the rotation partner of the state
// field and to the staging buffer, after which state and partner swap.
#include "fg_batch.cuh"
#include "fg_internal.cuh"
#include "fg_reduce.cuh"

namespace fg {
namespace {

constexpr int BX = 32, BY = 8;

inline dim3 cell_grid(const fg_fluid* f) {
  return dim3((f->NY + BX - 1) / BX, (f->NX + BY - 1) / BY);
}

__device__ __forceinline__ bool on_ring(int i, int j, const Grid& g) {
  return i == 0 || j == 0 || i == g.NX - 1 || j == g.NY - 1;
}

// U face (i, j) is advected iff 1 <= i <= NX-1, 1 <= j <= NY-2, and both
// adjacent cells are fluid (fluid.go:304).
__device__ __forceinline__ bool u_advected(uint8_t fl, int i, int j, const Grid& g) {
  return i >= 1 && j >= 1 && j <= g.NY - 2 && (fl & F_FLUID) && (fl & F_W);
}
// V face (i, j): 1 <= i <= NX-2, 1 <= j <= NY-1, both cells fluid (fluid.go:317).
__device__ __forceinline__ bool v_advected(uint8_t fl, int i, int j, const Grid& g) {
  return i >= 1 && i <= g.NX - 2 && j >= 1 && (fl & F_FLUID) && (fl & F_S);
}

// Backtrace of the U face (i, j) through the velocity (Ut, Vt); sdt = dt
// traces backward in time (x - dt*u), sdt = -dt forward (x + dt*u, BFECC's
// reverse pass fluid.go:951-952).
__device__ __forceinline__ float trace_sample_u(const float* __restrict__ Ut,
                                                const float* __restrict__ Vt,
                                                const float* __restrict__ Fs, int i, int j,
                                                float sdt, const Grid& g) {
  int c = i * g.P + j;
  float u = Ut[c];
  float v = (Vt[c - g.P] + Vt[c] + Vt[c - g.P + 1] + Vt[c + 1]) * 0.25f;  // avgV fluid.go:342-347
  return sample_dep(Fs, i, j, sdt * u, sdt * v, false, true, g);
}
__device__ __forceinline__ float trace_sample_v(const float* __restrict__ Ut,
                                                const float* __restrict__ Vt,
                                                const float* __restrict__ Fs, int i, int j,
                                                float sdt, const Grid& g) {
  int c = i * g.P + j;
  float u = (Ut[c - 1] + Ut[c] + Ut[c + g.P - 1] + Ut[c + g.P]) * 0.25f;  // avgU fluid.go:335-340
  float v = Vt[c];
  return sample_dep(Fs, i, j, sdt * u, sdt * v, true, false, g);
}

// Interior cells (1 <= i <= NX-2, 1 <= j <= NY-2): every load of the two
// traces is in range whatever the flags say, so the interior paths below
// issue them beside the flag load instead of after it, and sample before
// selecting.  The departure points are formed as in trace_sample_u/v, so
// the results are bitwise the same.
__device__ __forceinline__ bool interior_ij(int i, int j, const Grid& g) {
  return i >= 1 && j >= 1 && i <= g.NX - 2 && j <= g.NY - 2;
}
struct Departure {
  float su_u, sv_u;  // sdt * (u, v) at the U face
  float su_v, sv_v;  // sdt * (u, v) at the V face
};
__device__ __forceinline__ Departure departures(const float* __restrict__ Ut,
                                                const float* __restrict__ Vt, int i, int j,
                                                int c, float sdt, const Grid& g) {
  float uu = Ut[c];
  float vu = (Vt[c - g.P] + Vt[c] + Vt[c - g.P + 1] + Vt[c + 1]) * 0.25f;
  float uv = (Ut[c - 1] + Ut[c] + Ut[c + g.P - 1] + Ut[c + g.P]) * 0.25f;
  float vv = Vt[c];
  Departure d;
  d.su_u = sdt * uu;
  d.sv_u = sdt * vu;
  d.su_v = sdt * uv;
  d.sv_v = sdt * vv;
  return d;
}

// advectVelocity (fluid.go:291-333) with trace field = sampled field =
// border field = (Ui, Vi); stale values from the staging buffers nU, nV;
// result to (Uo, Vo) and back into (nU, nV).
__device__ __forceinline__ void sl_velocity_cell(int i, int j, const float* __restrict__ Ui,
                                                 const float* __restrict__ Vi,
                                                 float* __restrict__ Uo, float* __restrict__ Vo,
                                                 float* nU, float* nV,
                                                 const uint8_t* __restrict__ flags, float dt,
                                                 const Grid& g) {
  int c = i * g.P + j;
  float u, v;
  if (interior_ij(i, j, g)) {
    uint8_t fl = flags[c];
    Departure d = departures(Ui, Vi, i, j, c, dt, g);
    float su = sample_dep(Ui, i, j, d.su_u, d.sv_u, false, true, g);
    float sv = sample_dep(Vi, i, j, d.su_v, d.sv_v, true, false, g);
    u = u_advected(fl, i, j, g) ? su : nU[c];
    v = v_advected(fl, i, j, g) ? sv : nV[c];
    Uo[c] = u;
    Vo[c] = v;
    nU[c] = u;
    nV[c] = v;
    return;
  }
  uint8_t fl = flags[c];
  bool ring = on_ring(i, j, g);
  if (u_advected(fl, i, j, g))
    u = trace_sample_u(Ui, Vi, Ui, i, j, dt, g);
  else
    u = ring ? Ui[c] : nU[c];
  if (v_advected(fl, i, j, g))
    v = trace_sample_v(Ui, Vi, Vi, i, j, dt, g);
  else
    v = ring ? Vi[c] : nV[c];
  Uo[c] = u;
  Vo[c] = v;
  nU[c] = u;
  nV[c] = v;
}

// BFECC pass 1 (fluid.go:923): forward advection of the original field into
// (Fu, Fv).  The staging buffers are not written: the final pass reads the
// same stale values from them (newU = fwdU on the faces that are stale).
__device__ __forceinline__ void bfecc_vel_fwd_cell(int i, int j, const float* __restrict__ Ui,
                                                   const float* __restrict__ Vi,
                                                   const float* __restrict__ nU,
                                                   const float* __restrict__ nV,
                                                   float* __restrict__ Fu, float* __restrict__ Fv,
                                                   const uint8_t* __restrict__ flags, float dt,
                                                   const Grid& g) {
  int c = i * g.P + j;
  if (interior_ij(i, j, g)) {
    uint8_t fl = flags[c];
    Departure d = departures(Ui, Vi, i, j, c, dt, g);
    float su = sample_dep(Ui, i, j, d.su_u, d.sv_u, false, true, g);
    float sv = sample_dep(Vi, i, j, d.su_v, d.sv_v, true, false, g);
    Fu[c] = u_advected(fl, i, j, g) ? su : nU[c];
    Fv[c] = v_advected(fl, i, j, g) ? sv : nV[c];
    return;
  }
  uint8_t fl = flags[c];
  bool ring = on_ring(i, j, g);
  Fu[c] = u_advected(fl, i, j, g) ? trace_sample_u(Ui, Vi, Ui, i, j, dt, g) : (ring ? Ui[c] : nU[c]);
  Fv[c] = v_advected(fl, i, j, g) ? trace_sample_v(Ui, Vi, Vi, i, j, dt, g) : (ring ? Vi[c] : nV[c]);
}

// One row of a 3-wide window: columns j-1, j, j+1, with their min and max.
struct Row3 {
  float l, c, r, mn, mx;
};
__device__ __forceinline__ Row3 row3(const float* __restrict__ src, int c) {
  Row3 w;
  w.l = src[c - 1];
  w.c = src[c];
  w.r = src[c + 1];
  w.mn = fminf(fminf(w.l, w.c), w.r);
  w.mx = fmaxf(fmaxf(w.l, w.c), w.r);
  return w;
}

// The range of clampToNeighbors (fluid.go:1094-1120: lo = hi = the centre,
// then a scan of the 3x3 block row by row that replaces lo on v < lo and hi
// on v > hi) over the rows a, b, c around the centre b.c, bit for bit, with
// min / max trees instead of 18 compare-and-selects.  For a centre that is
// not NaN the scan ignores NaN neighbours, as fminf / fmaxf do, and ends on
// the first element (in scan order) of the minimum's value; a nonzero
// minimum has a single bit pattern, so the tree's value is it; a zero
// minimum with a zero centre is the centre (scanned first, nothing compares
// below it); a NaN centre is never replaced.  Only a zero extreme with a
// nonzero centre (a -0/+0 tie that scan order decides) runs the scan.
__device__ __forceinline__ void range_rows(const Row3& a, const Row3& b, const Row3& c, float& lo,
                                           float& hi) {
  const float ctr = b.c;
  const float m = fminf(fminf(a.mn, b.mn), c.mn);
  const float M = fmaxf(fmaxf(a.mx, b.mx), c.mx);
  if (ctr != ctr) {
    lo = hi = ctr;
    return;
  }
  const float v[9] = {a.l, a.c, a.r, b.l, b.c, b.r, c.l, c.c, c.r};
  if (m != 0.0f) {
    lo = m;
  } else if (ctr == 0.0f) {
    lo = ctr;
  } else {
    lo = ctr;
#pragma unroll
    for (int k = 0; k < 9; ++k)
      if (v[k] < lo) lo = v[k];
  }
  if (M != 0.0f) {
    hi = M;
  } else if (ctr == 0.0f) {
    hi = ctr;
  } else {
    hi = ctr;
#pragma unroll
    for (int k = 0; k < 9; ++k)
      if (v[k] > hi) hi = v[k];
  }
}

// clampToNeighbors' range (fluid.go:1094-1120) for an interior cell (all 3x3
// neighbours in range): range3x3 through the min / max trees, for the
// velocity; range3x3_scan as the reference scans, for the smoke (measured
// faster there: a field of zeros always ends in the centre's case, and the
// smoke pass has fewer instructions to save).
__device__ __forceinline__ void range3x3(const float* __restrict__ src, int c, int P, float& lo,
                                         float& hi) {
  range_rows(row3(src, c - P), row3(src, c), row3(src, c + P), lo, hi);
}
__device__ __forceinline__ void range3x3_scan(const float* __restrict__ src, int c, int P,
                                              float& lo, float& hi) {
  lo = src[c];
  hi = src[c];
#pragma unroll
  for (int di = -1; di <= 1; ++di)
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
      float v = src[c + di * P + dj];
      if (v < lo) lo = v;
      if (v > hi) hi = v;
    }
}
__device__ __forceinline__ float clamp_to(float val, float lo, float hi) {
  if (val < lo) return lo;
  if (val > hi) return hi;
  return val;
}

// BFECC passes 2-3 (fluid.go:931-987): reverse advection of the forward
// result traced with the original velocity, error compensation on every
// interior face (non-advected faces see bwd = 0), clamp to the original
// field's 3x3 range.  Ring faces keep the original value.
__device__ __forceinline__ void bfecc_vel_correct_cell(int i, int j, const float* __restrict__ Ui,
                                                       const float* __restrict__ Vi,
                                                       const float* __restrict__ Fu,
                                                       const float* __restrict__ Fv,
                                                       float* __restrict__ Cu,
                                                       float* __restrict__ Cv,
                                                       const uint8_t* __restrict__ flags, float dt,
                                                       const Grid& g) {
  int c = i * g.P + j;
  if (on_ring(i, j, g)) {
    Cu[c] = Ui[c];
    Cv[c] = Vi[c];
    return;
  }
  // Off the ring every cell is interior: all loads below are in range, so
  // they are issued together and the samples are taken before selecting.
  uint8_t fl = flags[c];
  Departure d = departures(Ui, Vi, i, j, c, -dt, g);
  float ou = Ui[c], ov = Vi[c];
  float lou, hiu, lov, hiv;
  range3x3(Ui, c, g.P, lou, hiu);
  range3x3(Vi, c, g.P, lov, hiv);
  float su = sample_dep(Fu, i, j, d.su_u, d.sv_u, false, true, g);
  float sv = sample_dep(Fv, i, j, d.su_v, d.sv_v, true, false, g);
  float bu = u_advected(fl, i, j, g) ? su : 0.0f;
  float bv = v_advected(fl, i, j, g) ? sv : 0.0f;
  float cu = ou - (bu - ou) * 0.5f;
  float cv = ov - (bv - ov) * 0.5f;
  Cu[c] = clamp_to(cu, lou, hiu);
  Cv[c] = clamp_to(cv, lov, hiv);
}
__global__ void k_bfecc_vel_correct(const float* __restrict__ Ui, const float* __restrict__ Vi,
                                    const float* __restrict__ Fu, const float* __restrict__ Fv,
                                    float* __restrict__ Cu, float* __restrict__ Cv,
                                    const uint8_t* __restrict__ flags, float dt, Grid g) {
  pdl_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  bfecc_vel_correct_cell(i, j, Ui, Vi, Fu, Fv, Cu, Cv, flags, dt, g);
}

// advectSmoke (fluid.go:400-434).  Trace velocity (Ut, Vt); sampled field Ms
// (which also feeds the optional diffusion term); ring cells from Ms; stale
// cells from nM.  Result to Mo and back into nM.
__device__ __forceinline__ float smoke_value(const float* __restrict__ Ut,
                                             const float* __restrict__ Vt,
                                             const float* __restrict__ Ms, int i, int j,
                                             float sdt, float smokeAdv, const Grid& g) {
  int c = i * g.P + j;
  float u = (Ut[c] + Ut[c + g.P]) * 0.5f * smokeAdv;
  float v = (Vt[c] + Vt[c + 1]) * 0.5f * smokeAdv;
  return sample_dep(Ms, i, j, sdt * u, sdt * v, true, true, g);
}


// One cell of advectSmoke: writes Mo and nM, returns the new value.
__device__ __forceinline__ float sl_smoke_value(int i, int j, const float* __restrict__ Ut,
                                                const float* __restrict__ Vt,
                                                const float* __restrict__ Ms,
                                                float* __restrict__ Mo, float* nM,
                                                const uint8_t* __restrict__ flags, float dt,
                                                float smokeAdv, int diffuse,
                                                float smokeDiffusion, const Grid& g) {
  int c = i * g.P + j;
  uint8_t fl = flags[c];
  float m;
  if (interior_ij(i, j, g)) {
    // The trace's loads are in range on interior cells: the sample is taken
    // whatever the flags say (its loads issue beside the flag load) and
    // kept on fluid cells.
    float s = smoke_value(Ut, Vt, Ms, i, j, dt, smokeAdv, g);
    if (fl & F_FLUID) {
      if (diffuse) {
        float neighbors = Ms[c - g.P] + Ms[c + g.P] + Ms[c - 1] + Ms[c + 1] - 4.0f * Ms[c];
        s += smokeDiffusion * neighbors;
      }
      m = go_max(s, 0.0f);
    } else {
      m = nM[c];
    }
  } else {
    m = Ms[c];  // off the interior every cell is on the ring
  }
  Mo[c] = m;
  nM[c] = m;
  return m;
}
__device__ __forceinline__ void sl_smoke_cell(int i, int j, const float* __restrict__ Ut,
                                              const float* __restrict__ Vt,
                                              const float* __restrict__ Ms,
                                              float* __restrict__ Mo, float* nM,
                                              const uint8_t* __restrict__ flags, float dt,
                                              float smokeAdv, int diffuse, float smokeDiffusion,
                                              const Grid& g) {
  sl_smoke_value(i, j, Ut, Vt, Ms, Mo, nM, flags, dt, smokeAdv, diffuse, smokeDiffusion, g);
}

__global__ void k_sl_smoke(const float* __restrict__ Ut, const float* __restrict__ Vt,
                           const float* __restrict__ Ms, float* __restrict__ Mo, float* nM,
                           const uint8_t* __restrict__ flags, float dt, float smokeAdv,
                           int diffuse, float smokeDiffusion, float* __restrict__ mass_part,
                           Grid g) {
  __shared__ float sh[64];
  pdl_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF mass{0.0f, 0.0f};
  if (i < g.NX && j < g.NY) {
    float m = sl_smoke_value(i, j, Ut, Vt, Ms, Mo, nM, flags, dt, smokeAdv, diffuse,
                             smokeDiffusion, g);
    if (!on_ring(i, j, g)) mass.hi = m;
  }
  // Smoke mass of the result over interior cells (float pairs within the
  // block, FP64 across blocks).
  if (mass_part) {
    FF v[1] = {mass};
    block_row<1>(v, 0u, sh, mass_part + 2 * (size_t)(blockIdx.y * gridDim.x + blockIdx.x));
  }
}

// BFECC smoke pass 1 (fluid.go:1007): forward advection into Fm without
// touching the staging buffer.
__device__ __forceinline__ void bfecc_smoke_fwd_cell(int i, int j, const float* __restrict__ Ut,
                                                     const float* __restrict__ Vt,
                                                     const float* __restrict__ Ms,
                                                     const float* __restrict__ nM,
                                                     float* __restrict__ Fm,
                                                     const uint8_t* __restrict__ flags, float dt,
                                                     float smokeAdv, int diffuse,
                                                     float smokeDiffusion, const Grid& g) {
  int c = i * g.P + j;
  uint8_t fl = flags[c];
  float m;
  if (interior_ij(i, j, g)) {
    // The trace's loads are in range on interior cells: the sample is taken
    // whatever the flags say (its loads issue beside the flag load) and
    // kept on fluid cells.
    float s = smoke_value(Ut, Vt, Ms, i, j, dt, smokeAdv, g);
    if (fl & F_FLUID) {
      if (diffuse) {
        float neighbors = Ms[c - g.P] + Ms[c + g.P] + Ms[c - 1] + Ms[c + 1] - 4.0f * Ms[c];
        s += smokeDiffusion * neighbors;
      }
      m = go_max(s, 0.0f);
    } else {
      m = nM[c];
    }
  } else {
    m = Ms[c];  // off the interior every cell is on the ring
  }
  Fm[c] = m;
}
__global__ void k_bfecc_smoke_fwd(const float* __restrict__ Ut, const float* __restrict__ Vt,
                                  const float* __restrict__ Ms, const float* __restrict__ nM,
                                  float* __restrict__ Fm, const uint8_t* __restrict__ flags,
                                  float dt, float smokeAdv, int diffuse, float smokeDiffusion,
                                  Grid g) {
  pdl_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  bfecc_smoke_fwd_cell(i, j, Ut, Vt, Ms, nM, Fm, flags, dt, smokeAdv, diffuse, smokeDiffusion, g);
}

// BFECC smoke passes 2-3 (fluid.go:1013-1046): reverse advection of the
// forward result, compensation on every interior cell (non-fluid cells see
// bwd = 0), clamp to the original 3x3 range, then to >= 0.
__device__ __forceinline__ void bfecc_smoke_correct_cell(int i, int j, const float* __restrict__ Ut,
                                                         const float* __restrict__ Vt,
                                                         const float* __restrict__ Mi,
                                                         const float* __restrict__ Fm,
                                                         float* __restrict__ Cm,
                                                         const uint8_t* __restrict__ flags,
                                                         float dt, float smokeAdv, const Grid& g) {
  int c = i * g.P + j;
  if (on_ring(i, j, g)) {
    Cm[c] = Mi[c];
    return;
  }
  // Off the ring every cell is interior: the sample's loads are in range and
  // issue with the flag load.
  uint8_t fl = flags[c];
  float o = Mi[c];
  float lo, hi;
  range3x3_scan(Mi, c, g.P, lo, hi);
  float s = smoke_value(Ut, Vt, Fm, i, j, -dt, smokeAdv, g);
  float b = (fl & F_FLUID) ? s : 0.0f;
  float cm = o - (b - o) * 0.5f;
  cm = clamp_to(cm, lo, hi);
  if (cm < 0.0f) cm = 0.0f;
  Cm[c] = cm;
}
__global__ void k_bfecc_smoke_correct(const float* __restrict__ Ut, const float* __restrict__ Vt,
                                      const float* __restrict__ Mi, const float* __restrict__ Fm,
                                      float* __restrict__ Cm, const uint8_t* __restrict__ flags,
                                      float dt, float smokeAdv, Grid g) {
  pdl_enter();
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  bfecc_smoke_correct_cell(i, j, Ut, Vt, Mi, Fm, Cm, flags, dt, smokeAdv, g);
}

// ------------------------------------------------------------ strip kernels
// The single-scene velocity passes without a clamp (BFECC pass 1 and the
// final advection) run R consecutive rows of one column per thread (a block
// of 32 x 8 threads covers 32 columns x 8R rows).  Interior strips keep the
// departure velocities' neighbouring rows in registers, so each U and V load
// is made once per row instead of twice; the arithmetic of every cell is
// the same, operation for operation.  Strips that touch the ghost ring (or
// pass the last row) run the per-cell bodies.  The clamping passes and the
// smoke passes stay one cell per thread: their strips took 48-64 registers,
// which halved the resident warps of these load-latency-bound passes and
// cost more than the shared loads saved (velocity correction 56.8 against
// 50.4 us, smoke passes +5 to +12 us each, at 2048^2).
constexpr int kStripRows = 4;

template <int R>
__device__ __forceinline__ bool strip_interior(int i0, int j, const Grid& g) {
  return j >= 1 && j <= g.NY - 2 && i0 >= 1 && i0 + R - 1 <= g.NX - 2;
}

// advectVelocity's interior cells (sl_velocity_cell, MODE 1: result to
// Uo, Vo and the staging buffers) or BFECC pass 1 (bfecc_vel_fwd_cell,
// MODE 0: result to Uo = Fu, Vo = Fv; the staging buffers only read).  The
// departure velocities of row i need U on rows i, i+1 (columns j-1, j) and
// V on rows i-1, i (columns j, j+1).
template <int R, int MODE>
__global__ void __launch_bounds__(256, 4)
    k_vel_strip(const float* __restrict__ Ui, const float* __restrict__ Vi, float* __restrict__ Uo,
                float* __restrict__ Vo, float* nU, float* nV, const uint8_t* __restrict__ flags,
                float dt, Grid g) {
  pdl_enter();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = (blockIdx.y * blockDim.y + threadIdx.y) * R;
  if (j >= g.NY || i0 >= g.NX) return;
  if (!strip_interior<R>(i0, j, g)) {
    for (int r = 0; r < R && i0 + r < g.NX; ++r) {
      if (MODE == 1)
        sl_velocity_cell(i0 + r, j, Ui, Vi, Uo, Vo, nU, nV, flags, dt, g);
      else
        bfecc_vel_fwd_cell(i0 + r, j, Ui, Vi, nU, nV, Uo, Vo, flags, dt, g);
    }
    return;
  }
  const int P = g.P;
  int c = i0 * P + j;
  float ul = Ui[c - 1], uc = Ui[c];          // U row i
  float vp = Vi[c - P], vpr = Vi[c - P + 1];  // V row i-1
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int i = i0 + r;
    const float uln = Ui[c + P - 1], ucn = Ui[c + P];  // U row i+1
    const float vc = Vi[c], vcr = Vi[c + 1];           // V row i
    const uint8_t fl = flags[c];
    // departures(): avgV at the U face, avgU at the V face.
    const float vu = (vp + vc + vpr + vcr) * 0.25f;
    const float uv = (ul + uc + uln + ucn) * 0.25f;
    const float su = sample_dep(Ui, i, j, dt * uc, dt * vu, false, true, g);
    const float sv = sample_dep(Vi, i, j, dt * uv, dt * vc, true, false, g);
    const float u = u_advected(fl, i, j, g) ? su : nU[c];
    const float v = v_advected(fl, i, j, g) ? sv : nV[c];
    Uo[c] = u;
    Vo[c] = v;
    if (MODE == 1) {
      nU[c] = u;
      nV[c] = v;
    }
    ul = uln;
    uc = ucn;
    vp = vc;
    vpr = vcr;
    c += P;
  }
}

inline dim3 strip_grid(const fg_fluid* f) {
  return dim3((f->NY + BX - 1) / BX, (f->NX + BY * kStripRows - 1) / (BY * kStripRows));
}

}  // namespace

// advectVelocity over (Ui, Vi) into the rotation partners and the staging
// buffers.
static void sl_velocity_pass(fg_fluid* f, const float* Ui, const float* Vi, float dt) {
  count(f);
  if (f->batch) {
    FG_CELLS_BATCH(f, sl_velocity_cell, Ui, Vi, f->partner[FG_U], f->partner[FG_V],
                   f->d[FG_NEWU], f->d[FG_NEWV], (const uint8_t*)f->flags, dt);
    return;
  }
  launch_pdl(k_vel_strip<kStripRows, 1>, strip_grid(f), dim3(BX, BY), 0, f->stream, Ui, Vi,
             f->partner[FG_U], f->partner[FG_V], f->d[FG_NEWU], f->d[FG_NEWV], f->flags, dt, f->g);
}

cudaError_t launch_advect_velocity(fg_fluid* f, float dt) {
  sl_velocity_pass(f, f->d[FG_U], f->d[FG_V], dt);
  swap_state(f, FG_U);
  swap_state(f, FG_V);
  return cudaGetLastError();
}

static float smoke_diffusion(const fg_fluid* f, float dt, int* diffuse) {
  *diffuse = f->prm.viscosity_diffusion > 0.0f ? 1 : 0;
  return f->prm.viscosity_diffusion * 0.3f * dt;  // fluid.go:422
}

// Final smoke pass from Ms; a single handle also sums the smoke mass.
static cudaError_t smoke_pass(fg_fluid* f, const float* Ms, float dt) {
  int diffuse;
  float sd = smoke_diffusion(f, dt, &diffuse);
  float sa = f->prm.smoke_advection;
  count(f);
  if (f->batch) {
    FG_CELLS_BATCH(f, sl_smoke_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V], Ms,
                   f->partner[FG_M], f->d[FG_NEWM], (const uint8_t*)f->flags, dt, sa, diffuse,
                   sd);
    swap_state(f, FG_M);
    return cudaGetLastError();
  }
  dim3 gr = cell_grid(f);
  if (!partials_fit(f, 1, gr.x * gr.y)) return cudaErrorInvalidValue;
  launch_pdl(k_sl_smoke, gr, dim3(BX, BY), 0, f->stream, f->d[FG_U], f->d[FG_V], Ms,
             f->partner[FG_M], f->d[FG_NEWM], f->flags, dt, sa, diffuse, sd, f->partials, f->g);
  swap_state(f, FG_M);
  return launch_store_mass(f, gr.x * gr.y);
}

cudaError_t launch_advect_smoke(fg_fluid* f, float dt) { return smoke_pass(f, f->d[FG_M], dt); }

cudaError_t launch_advect_velocity_bfecc(fg_fluid* f, float dt) {
  count(f);
  if (f->batch)
    FG_CELLS_BATCH(f, bfecc_vel_fwd_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V],
                   (const float*)f->d[FG_NEWU], (const float*)f->d[FG_NEWV], f->fwdU, f->fwdV,
                   (const uint8_t*)f->flags, dt);
  else
    launch_pdl(k_vel_strip<kStripRows, 0>, strip_grid(f), dim3(BX, BY), 0, f->stream,
               f->d[FG_U], f->d[FG_V], f->fwdU, f->fwdV, f->d[FG_NEWU], f->d[FG_NEWV], f->flags,
               dt, f->g);
  count(f);
  if (f->batch)
    FG_CELLS_BATCH(f, bfecc_vel_correct_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V],
                   (const float*)f->fwdU, (const float*)f->fwdV, f->corrU, f->corrV,
                   (const uint8_t*)f->flags, dt);
  else
    launch_pdl(k_bfecc_vel_correct, cell_grid(f), dim3(BX, BY), 0, f->stream, f->d[FG_U],
               f->d[FG_V], f->fwdU, f->fwdV, f->corrU, f->corrV, f->flags, dt, f->g);
  // Pass 4 (fluid.go:991-993): advect the corrected field with itself.
  sl_velocity_pass(f, f->corrU, f->corrV, dt);
  swap_state(f, FG_U);
  swap_state(f, FG_V);
  return cudaGetLastError();
}

cudaError_t launch_advect_smoke_bfecc(fg_fluid* f, float dt) {
  int diffuse;
  float sd = smoke_diffusion(f, dt, &diffuse);
  float sa = f->prm.smoke_advection;
  count(f);
  if (f->batch)
    FG_CELLS_BATCH(f, bfecc_smoke_fwd_cell, (const float*)f->d[FG_U], (const float*)f->d[FG_V],
                   (const float*)f->d[FG_M], (const float*)f->d[FG_NEWM], f->fwdM,
                   (const uint8_t*)f->flags, dt, sa, diffuse, sd);
  else
    launch_pdl(k_bfecc_smoke_fwd, cell_grid(f), dim3(BX, BY), 0, f->stream, f->d[FG_U],
               f->d[FG_V], f->d[FG_M], f->d[FG_NEWM], f->fwdM, f->flags, dt, sa, diffuse, sd,
               f->g);
  count(f);
  if (f->batch)
    FG_CELLS_BATCH(f, bfecc_smoke_correct_cell, (const float*)f->d[FG_U],
                   (const float*)f->d[FG_V], (const float*)f->d[FG_M], (const float*)f->fwdM,
                   f->corrM, (const uint8_t*)f->flags, dt, sa);
  else
    launch_pdl(k_bfecc_smoke_correct, cell_grid(f), dim3(BX, BY), 0, f->stream, f->d[FG_U],
               f->d[FG_V], f->d[FG_M], f->fwdM, f->corrM, f->flags, dt, sa, f->g);
  return smoke_pass(f, f->corrM, dt);
}

}  // namespace fg
