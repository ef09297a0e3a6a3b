// Adjoint (reverse-mode derivative) of the simulation step for the parallel
// pressure scheme.
//
// The forward step of a differentiable rollout is Simulate (fluid.go:79-109)
// with two additions: an optional force field added to U and V before the
// sources, and the pressure scheme fixed to Jacobi without early exit.  The
// stages and their adjoints:
//   forces       U += Fu, V += Fv            -> dFu = dU, dFv = dV
//   sources      U, V set / M added          -> dU, dV zeroed on set cells
//   projection   U2 = U1 + G P_K (-div U1)    -> dU1 = dU2 - div^T P_K G^T dU2
//                (K Jacobi sweeps from 0 apply P_K = sum_k M^k W with M W =
//                W M^T, so P_K is symmetric: its adjoint is the same solve)
//   turbulence   pointwise, gated on |u| > 0.1 (fluid.go:496-526)
//   borders      linear rules on the ghost rows (fluid.go:236-289)
//   advection    bilinear gathers: transposed as scatters with atomics, plus
//                the derivative of the backtrace position through the
//                velocity that traced it; BFECC composes three of them with
//                the compensation and the 3x3 clamp (fluid.go:909-1120)
// Subgradient conventions at non-smooth points: a coordinate clamped to the
// domain contributes no position derivative; the bilinear cell choice
// (floor) is locally constant; a clamped BFECC value takes the derivative of
// the neighbour that bounded it (the first in the reference's scan order);
// max(x, 0) passes the derivative for x >= 0; min(0.5|u|, 1) has derivative
// 0.5 below the kink and 0 at or above it; the turbulence gate passes the
// noise term only for |u| > 0.1.
//
// The scatters use FP32 atomic adds, so an adjoint run is reproducible to
// about 1e-7 relative, not bit for bit.
#include <utility>

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
__device__ __forceinline__ bool u_advected(uint8_t fl, int i, int j, const Grid& g) {
  return i >= 1 && j >= 1 && j <= g.NY - 2 && (fl & F_FLUID) && (fl & F_W);
}
__device__ __forceinline__ bool v_advected(uint8_t fl, int i, int j, const Grid& g) {
  return i >= 1 && i <= g.NX - 2 && j >= 1 && (fl & F_FLUID) && (fl & F_S);
}
__device__ __forceinline__ bool fluid_interior(uint8_t fl) {
  return (fl & (F_FLUID | F_INTERIOR)) == (F_FLUID | F_INTERIOR);
}

// Forward: U += Fu, V += Fv on every cell.
__device__ __forceinline__ void add_forces_cell(int i, int j, float* __restrict__ U,
                                                float* __restrict__ V, const float* __restrict__ Fu,
                                                const float* __restrict__ Fv, const Grid& g) {
  int c = i * g.P + j;
  U[c] = U[c] + Fu[c];
  V[c] = V[c] + Fv[c];
}
__global__ void k_add_forces(float* __restrict__ U, float* __restrict__ V,
                             const float* __restrict__ Fu, const float* __restrict__ Fv, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  add_forces_cell(i, j, U, V, Fu, Fv, g);
}

// Adjoint of a bilinear sample of field F at (x, y) (sampleField): scatters
// lam * weights into dF and returns d value / d x, d value / d y (0 along a
// clamped coordinate).
__device__ __forceinline__ void sample_adjoint(const float* __restrict__ F, float* dF,
                                               const Bilin& s, float lam, const Grid& g,
                                               float* dvdx, float* dvdy) {
  const int x0 = s.x0, x1 = s.x1, y0 = s.y0, y1 = s.y1;
  const float tx = s.tx, ty = s.ty;
  float sx = 1.0f - tx, sy = 1.0f - ty;
  const int P = g.P;
  float f00 = F[x0 * P + y0], f10 = F[x1 * P + y0], f11 = F[x1 * P + y1], f01 = F[x0 * P + y1];
  if (lam != 0.0f) {
    atomicAdd(&dF[x0 * P + y0], sx * sy * lam);
    atomicAdd(&dF[x1 * P + y0], tx * sy * lam);
    atomicAdd(&dF[x1 * P + y1], tx * ty * lam);
    atomicAdd(&dF[x0 * P + y1], sx * ty * lam);
  }
  *dvdx = s.inx ? g.h1 * (sy * (f10 - f00) + ty * (f11 - f01)) : 0.0f;
  *dvdy = s.iny ? g.h1 * (sx * (f01 - f00) + tx * (f11 - f10)) : 0.0f;
}

// Adjoint of a semi-Lagrangian velocity pass (advectVelocity fluid.go:291-333
// and BFECC's passes): out = advected ? sample(Fs; trace with (Ut, Vt), sdt)
// : ring ? R : stale.  lamU/lamV hold the output adjoint.  Accumulates into
// dFu/dFv (sampled field), dUt/dVt (tracing velocity), dRu/dRv (ring source,
// may be null: no ring term) and dNu/dNv (stale source, may be null).
__device__ __forceinline__ void adj_sl_velocity_cell(int i, int j, const float* __restrict__ lamU,
                                                     const float* __restrict__ lamV,
                                                     const float* __restrict__ Ut,
                                                     const float* __restrict__ Vt,
                                                     const float* __restrict__ Fu,
                                                     const float* __restrict__ Fv, float* dUt,
                                                     float* dVt, float* dFu, float* dFv, float* dRu,
                                                     float* dRv, float* dNu, float* dNv,
                                                     const uint8_t* __restrict__ flags, float sdt,
                                                     const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  uint8_t fl = flags[c];
  bool ring = on_ring(i, j, g);
  float lu = lamU[c], lv = lamV[c];
  if (u_advected(fl, i, j, g)) {
    float u = Ut[c];
    float v = (Vt[c - P] + Vt[c] + Vt[c - P + 1] + Vt[c + 1]) * 0.25f;
    float gx, gy;
    sample_adjoint(Fu, dFu, bilin_dep(i, j, sdt * u, sdt * v, false, true, g), lu, g, &gx, &gy);
    float du = -sdt * gx * lu, dv = -sdt * gy * lu;
    if (du != 0.0f) atomicAdd(&dUt[c], du);
    if (dv != 0.0f) {
      float q = 0.25f * dv;
      atomicAdd(&dVt[c - P], q);
      atomicAdd(&dVt[c], q);
      atomicAdd(&dVt[c - P + 1], q);
      atomicAdd(&dVt[c + 1], q);
    }
  } else if (ring) {
    if (dRu && lu != 0.0f) atomicAdd(&dRu[c], lu);
  } else if (dNu) {
    dNu[c] += lu;
  }
  if (v_advected(fl, i, j, g)) {
    float u = (Ut[c - 1] + Ut[c] + Ut[c + P - 1] + Ut[c + P]) * 0.25f;
    float v = Vt[c];
    float gx, gy;
    sample_adjoint(Fv, dFv, bilin_dep(i, j, sdt * u, sdt * v, true, false, g), lv, g, &gx, &gy);
    float du = -sdt * gx * lv, dv = -sdt * gy * lv;
    if (dv != 0.0f) atomicAdd(&dVt[c], dv);
    if (du != 0.0f) {
      float q = 0.25f * du;
      atomicAdd(&dUt[c - 1], q);
      atomicAdd(&dUt[c], q);
      atomicAdd(&dUt[c + P - 1], q);
      atomicAdd(&dUt[c + P], q);
    }
  } else if (ring) {
    if (dRv && lv != 0.0f) atomicAdd(&dRv[c], lv);
  } else if (dNv) {
    dNv[c] += lv;
  }
}
__global__ void k_adj_sl_velocity(const float* __restrict__ lamU, const float* __restrict__ lamV,
                                  const float* __restrict__ Ut, const float* __restrict__ Vt,
                                  const float* __restrict__ Fu, const float* __restrict__ Fv,
                                  float* dUt, float* dVt, float* dFu, float* dFv, float* dRu,
                                  float* dRv, float* dNu, float* dNv,
                                  const uint8_t* __restrict__ flags, float sdt, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_sl_velocity_cell(i, j, lamU, lamV, Ut, Vt, Fu, Fv, dUt, dVt, dFu, dFv, dRu, dRv, dNu, dNv, flags, sdt, g);
}

// clampToNeighbors (fluid.go:1094-1120) on an interior cell: returns the
// offset (in elements) of the neighbour whose value bounded `val`, or -1 if
// val was inside the range.  Ties keep the first value in scan order, as the
// strict comparisons of the reference do.
__device__ __forceinline__ int clamp_source(float val, const float* __restrict__ src, int c, int P) {
  float lo = src[c], hi = src[c];
  int klo = 0, khi = 0;
#pragma unroll
  for (int di = -1; di <= 1; ++di)
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
      int k = di * P + dj;
      float v = src[c + k];
      if (v < lo) {
        lo = v;
        klo = k;
      }
      if (v > hi) {
        hi = v;
        khi = k;
      }
    }
  if (val < lo) return klo + 0x40000000;  // tagged: a neighbour offset
  if (val > hi) return khi + 0x40000000;
  return -1;
}

// Adjoint of BFECC's passes 2-3 for velocity (fluid.go:931-987), fused:
// bwd = sample(fwd; trace with (Ou, Ov) at -dt) on advected interior faces
// (0 on the others), corr = clamp(o - (bwd - o) * 0.5) on interior faces,
// corr = o on the ring.  Reads lamC (adjoint of corr); accumulates into dO
// (the original field, which is also the tracing velocity) and dF (fwd).
__device__ __forceinline__ void adj_bfecc_vel_cell(int i, int j, const float* __restrict__ lamCu,
                                                   const float* __restrict__ lamCv,
                                                   const float* __restrict__ Ou,
                                                   const float* __restrict__ Ov,
                                                   const float* __restrict__ Fu,
                                                   const float* __restrict__ Fv, float* dOu,
                                                   float* dOv, float* dFu, float* dFv,
                                                   const uint8_t* __restrict__ flags, float dt,
                                                   const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  float lu = lamCu[c], lv = lamCv[c];
  if (on_ring(i, j, g)) {
    if (lu != 0.0f) atomicAdd(&dOu[c], lu);
    if (lv != 0.0f) atomicAdd(&dOv[c], lv);
    return;
  }
  uint8_t fl = flags[c];
#pragma unroll
  for (int comp = 0; comp < 2; ++comp) {
    const float* O = comp == 0 ? Ou : Ov;
    const float* F = comp == 0 ? Fu : Fv;
    float* dO = comp == 0 ? dOu : dOv;
    float lam = comp == 0 ? lu : lv;
    bool adv = comp == 0 ? u_advected(fl, i, j, g) : v_advected(fl, i, j, g);
    float b = 0.0f;
    Bilin st{};
    if (adv) {
      // The reverse trace of trace_sample_u / _v with sdt = -dt.
      if (comp == 0) {
        float u = Ou[c];
        float v = (Ov[c - P] + Ov[c] + Ov[c - P + 1] + Ov[c + 1]) * 0.25f;
        st = bilin_dep(i, j, -dt * u, -dt * v, false, true, g);
      } else {
        float u = (Ou[c - 1] + Ou[c] + Ou[c + P - 1] + Ou[c + P]) * 0.25f;
        float v = Ov[c];
        st = bilin_dep(i, j, -dt * u, -dt * v, true, false, g);
      }
      b = bilin_sample(PtrAcc{F, P}, st);
    }
    float o = O[c];
    float raw = o - (b - o) * 0.5f;
    int src = clamp_source(raw, O, c, P);
    if (src >= 0) {
      if (lam != 0.0f) atomicAdd(&dO[c + (src - 0x40000000)], lam);
      continue;
    }
    if (lam == 0.0f) continue;
    atomicAdd(&dO[c], 1.5f * lam);
    if (!adv) continue;
    float lb = -0.5f * lam;  // adjoint of bwd
    float gx, gy;
    sample_adjoint(F, comp == 0 ? dFu : dFv, st, lb, g, &gx, &gy);
    float du = dt * gx * lb, dv = dt * gy * lb;
    if (comp == 0) {
      if (du != 0.0f) atomicAdd(&dOu[c], du);
      if (dv != 0.0f) {
        float q = 0.25f * dv;
        atomicAdd(&dOv[c - P], q);
        atomicAdd(&dOv[c], q);
        atomicAdd(&dOv[c - P + 1], q);
        atomicAdd(&dOv[c + 1], q);
      }
    } else {
      if (dv != 0.0f) atomicAdd(&dOv[c], dv);
      if (du != 0.0f) {
        float q = 0.25f * du;
        atomicAdd(&dOu[c - 1], q);
        atomicAdd(&dOu[c], q);
        atomicAdd(&dOu[c + P - 1], q);
        atomicAdd(&dOu[c + P], q);
      }
    }
  }
}
__global__ void k_adj_bfecc_vel(const float* __restrict__ lamCu, const float* __restrict__ lamCv,
                                const float* __restrict__ Ou, const float* __restrict__ Ov,
                                const float* __restrict__ Fu, const float* __restrict__ Fv,
                                float* dOu, float* dOv, float* dFu, float* dFv,
                                const uint8_t* __restrict__ flags, float dt, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_bfecc_vel_cell(i, j, lamCu, lamCv, Ou, Ov, Fu, Fv, dOu, dOv, dFu, dFv, flags, dt, g);
}

// Adjoint of a semi-Lagrangian smoke pass (advectSmoke fluid.go:400-434,
// without the diffusion term): out = fluid interior ? max(sample(Ms), 0) :
// ring ? Ms : stale.  With bwd = 1 the pass is BFECC's reverse sample (no
// max, non-fluid cells constant 0, no ring / stale terms).  The trace
// velocity is ((U[c] + U[c+P]) / 2 * SA, (V[c] + V[c+1]) / 2 * SA).
__device__ __forceinline__ void adj_sl_smoke_cell(int i, int j, const float* __restrict__ lamM,
                                                  const float* __restrict__ U,
                                                  const float* __restrict__ V,
                                                  const float* __restrict__ Ms, float* dU,
                                                  float* dV, float* dMs, float* dN,
                                                  const uint8_t* __restrict__ flags, float sdt,
                                                  float smokeAdv, int bwd, const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  uint8_t fl = flags[c];
  float lam = lamM[c];
  bool interior = !on_ring(i, j, g);
  bool advected = bwd ? (interior && (fl & F_FLUID)) : fluid_interior(fl);
  if (advected) {
    float u = (U[c] + U[c + P]) * 0.5f * smokeAdv;
    float v = (V[c] + V[c + 1]) * 0.5f * smokeAdv;
    const Bilin st = bilin_dep(i, j, sdt * u, sdt * v, true, true, g);
    if (!bwd) {
      float s = bilin_sample(PtrAcc{Ms, P}, st);
      if (!(s >= 0.0f)) lam = 0.0f;  // max(s, 0) clamped
    }
    float gx, gy;
    sample_adjoint(Ms, dMs, st, lam, g, &gx, &gy);
    float du = -sdt * gx * lam * 0.5f * smokeAdv, dv = -sdt * gy * lam * 0.5f * smokeAdv;
    if (du != 0.0f) {
      atomicAdd(&dU[c], du);
      atomicAdd(&dU[c + P], du);
    }
    if (dv != 0.0f) {
      atomicAdd(&dV[c], dv);
      atomicAdd(&dV[c + 1], dv);
    }
  } else if (!bwd) {
    if (!interior) {
      if (lam != 0.0f) atomicAdd(&dMs[c], lam);
    } else if (dN) {
      dN[c] += lam;
    }
  }
}
__global__ void k_adj_sl_smoke(const float* __restrict__ lamM, const float* __restrict__ U,
                               const float* __restrict__ V, const float* __restrict__ Ms,
                               float* dU, float* dV, float* dMs, float* dN,
                               const uint8_t* __restrict__ flags, float sdt, float smokeAdv,
                               int bwd, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_sl_smoke_cell(i, j, lamM, U, V, Ms, dU, dV, dMs, dN, flags, sdt, smokeAdv, bwd, g);
}

// Adjoint of BFECC's smoke passes 2-3 (fluid.go:1013-1046), fused: bwd =
// sample(fwd; trace with (U, V) at -dt) on fluid interior cells (0 on the
// others), corr = max(clamp(o - (bwd - o) * 0.5), 0) on interior cells, o on
// the ring.  Reads lamC; accumulates into dO (original smoke), dF (fwd) and
// dU, dV (the tracing velocity).
__device__ __forceinline__ void adj_bfecc_smoke_cell(int i, int j, const float* __restrict__ lamC,
                                                     const float* __restrict__ U,
                                                     const float* __restrict__ V,
                                                     const float* __restrict__ Mo,
                                                     const float* __restrict__ Fm, float* dO,
                                                     float* dF, float* dU, float* dV,
                                                     const uint8_t* __restrict__ flags, float dt,
                                                     float smokeAdv, const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  float lam = lamC[c];
  if (on_ring(i, j, g)) {
    if (lam != 0.0f) atomicAdd(&dO[c], lam);
    return;
  }
  uint8_t fl = flags[c];
  bool adv = (fl & F_FLUID) != 0;
  float b = 0.0f;
  Bilin st{};
  if (adv) {
    float u = (U[c] + U[c + P]) * 0.5f * smokeAdv;
    float v = (V[c] + V[c + 1]) * 0.5f * smokeAdv;
    st = bilin_dep(i, j, -dt * u, -dt * v, true, true, g);
    b = bilin_sample(PtrAcc{Fm, P}, st);
  }
  float o = Mo[c];
  float raw = o - (b - o) * 0.5f;
  int src = clamp_source(raw, Mo, c, P);
  float cm = src >= 0 ? Mo[c + (src - 0x40000000)] : raw;
  if (cm < 0.0f || lam == 0.0f) return;  // the final max(., 0) passes nothing
  if (src >= 0) {
    atomicAdd(&dO[c + (src - 0x40000000)], lam);
    return;
  }
  atomicAdd(&dO[c], 1.5f * lam);
  if (!adv) return;
  float lb = -0.5f * lam;
  float gx, gy;
  sample_adjoint(Fm, dF, st, lb, g, &gx, &gy);
  float du = dt * gx * lb * 0.5f * smokeAdv, dv = dt * gy * lb * 0.5f * smokeAdv;
  if (du != 0.0f) {
    atomicAdd(&dU[c], du);
    atomicAdd(&dU[c + P], du);
  }
  if (dv != 0.0f) {
    atomicAdd(&dV[c], dv);
    atomicAdd(&dV[c + 1], dv);
  }
}
__global__ void k_adj_bfecc_smoke(const float* __restrict__ lamC, const float* __restrict__ U,
                                  const float* __restrict__ V, const float* __restrict__ Mo,
                                  const float* __restrict__ Fm, float* dO, float* dF, float* dU,
                                  float* dV, const uint8_t* __restrict__ flags, float dt,
                                  float smokeAdv, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_bfecc_smoke_cell(i, j, lamC, U, V, Mo, Fm, dO, dF, dU, dV, flags, dt, smokeAdv, g);
}

// Adjoint of handleBorders (fluid.go:236-289), in place on (dU, dV): each
// ghost value was written from interior values or 0.  Thread t reverses the
// U rows of column i = t (bottom row first: it was written last) and the V
// columns of row j = t.
__device__ __forceinline__ void adj_borders_border(int t, float* __restrict__ dU,
                                                   float* __restrict__ dV,
                                                   const uint8_t* __restrict__ flags,
                                                   const Grid& g) {
  const int P = g.P, NX = g.NX, NY = g.NY;
  auto fluid = [&](int i, int j) { return (flags[i * P + j] & F_FLUID) != 0; };
  if (t < NX) {
    int i = t;
    float* d = dU + (size_t)i * P;
    float l = d[NY - 1];
    d[NY - 1] = 0.0f;
    if (fluid(i, NY - 1) && fluid(i, NY - 2)) {
      if (i > 0 && i < NX - 1 && fluid(i, NY - 3)) {
        d[NY - 2] += 2.0f * l;
        d[NY - 3] -= l;
      } else {
        d[NY - 2] += l;
      }
    }
    l = d[0];
    d[0] = 0.0f;
    if (fluid(i, 0) && fluid(i, 1)) {
      if (i > 0 && i < NX - 1 && fluid(i, 2)) {
        d[1] += 2.0f * l;
        d[2] -= l;
      } else {
        d[1] += l;
      }
    }
  }
  if (t < NY) {
    int j = t;
    int a = (NX - 1) * P + j, b = (NX - 2) * P + j, cc = (NX - 3) * P + j;
    float l = dV[a];
    dV[a] = 0.0f;
    if (fluid(NX - 1, j) && fluid(NX - 2, j)) {
      if (j > 0 && j < NY - 1 && fluid(NX - 3, j)) {
        dV[b] += 2.0f * l;
        dV[cc] -= l;
      } else {
        dV[b] += l;
      }
    }
    l = dV[j];
    dV[j] = 0.0f;
    if (fluid(0, j) && fluid(1, j)) {
      if (j > 0 && j < NY - 1 && fluid(2, j)) {
        dV[P + j] += 2.0f * l;
        dV[2 * P + j] -= l;
      } else {
        dV[P + j] += l;
      }
    }
  }
}
__global__ void k_adj_borders(float* __restrict__ dU, float* __restrict__ dV,
                              const uint8_t* __restrict__ flags, Grid g) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  adj_borders_border(t, dU, dV, flags, g);
}

// Adjoint of addTurbulence (fluid.go:496-526) at the pre-turbulence field
// (U2, V2), in place on (dU, dV).
__device__ __forceinline__ void adj_turbulence_cell(int i, int j, float* __restrict__ dU,
                                                    float* __restrict__ dV,
                                                    const float* __restrict__ U2,
                                                    const float* __restrict__ V2,
                                                    const float2* __restrict__ noise,
                                                    const uint8_t* __restrict__ flags,
                                                    float turbStrength, const Grid& g) {
  int c = i * g.P + j;
  if (!fluid_interior(flags[c])) return;
  float u = U2[c], v = V2[c];
  float r = sqrtf(u * u + v * v);
  if (!(r > 0.1f)) return;
  float fp = 0.5f * r < 1.0f ? 0.5f : 0.0f;  // d min(0.5 r, 1) / d r
  if (fp == 0.0f) return;
  float2 nz = noise[c];
  float nu = nz.x * turbStrength, nv = nz.y * turbStrength;
  float au = u / r, av = v / r;  // d r / d u, d r / d v
  float lu = dU[c], lv = dV[c];
  float s = (lu * nu + lv * nv) * fp;
  dU[c] = lu + s * au;
  dV[c] = lv + s * av;
}
__global__ void k_adj_turbulence(float* __restrict__ dU, float* __restrict__ dV,
                                 const float* __restrict__ U2, const float* __restrict__ V2,
                                 const float2* __restrict__ noise,
                                 const uint8_t* __restrict__ flags, float turbStrength, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_turbulence_cell(i, j, dU, dV, U2, V2, noise, flags, turbStrength, g);
}

// ---------------------------------------------------------------- confinement
// applyVorticityConfinement (fluid.go:449-493) followed by addTurbulence on
// the pre-confinement field (U2, V2).  curl_at restates k_curl for one cell.
__device__ __forceinline__ float curl_at(const float* __restrict__ U, const float* __restrict__ V,
                                         const uint8_t* __restrict__ flags, int c, const Grid& g) {
  if (!fluid_interior(flags[c])) return 0.0f;
  float dvdx = (V[c + g.P] - V[c - g.P]) * 0.5f / g.h;
  float dudy = (U[c + 1] - U[c - 1]) * 0.5f / g.h;
  return dvdx - dudy;
}

// Per fluid interior cell: the turbulence adjoint at the post-confinement
// velocity (recomputed), then the confinement adjoint of the cell's own
// terms.  In place on (dU, dV) for the identity and speed terms; writes the
// adjoint of the cell's curl through its direct use (lw) and of the
// normalised gradient's inputs (lgx, lgy: d/d gx, d/d gy), 0 on every other
// cell.  Subgradients: |curl| passes sign(curl) (0 at 0); at |grad| = 0 the
// normalisation's derivative is I / eps.
__device__ __forceinline__ void adj_conf_local_cell(int i, int j, float* __restrict__ dU,
                                                    float* __restrict__ dV,
                                                    const float* __restrict__ U2,
                                                    const float* __restrict__ V2,
                                                    const float2* __restrict__ noise,
                                                    const uint8_t* __restrict__ flags, float conf,
                                                    float dt, float turbStrength, int do_turb,
                                                    float* __restrict__ lw, float* __restrict__ lgx,
                                                    float* __restrict__ lgy, const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  if (!fluid_interior(flags[c])) {
    lw[c] = 0.0f;
    lgx[c] = 0.0f;
    lgy[c] = 0.0f;
    return;
  }
  const float eps = 1e-5f;
  float w = curl_at(U2, V2, flags, c, g);
  float aE = fabsf(curl_at(U2, V2, flags, c + P, g)), aW = fabsf(curl_at(U2, V2, flags, c - P, g));
  float aN = fabsf(curl_at(U2, V2, flags, c + 1, g)), aS = fabsf(curl_at(U2, V2, flags, c - 1, g));
  float gx = (aE - aW) * 0.5f / g.h;
  float gy = (aN - aS) * 0.5f / g.h;
  float rg = sqrtf(gx * gx + gy * gy);
  float m = rg + eps;
  float nx = gx / m, ny = gy / m;
  float u = U2[c], v = V2[c];
  float r = sqrtf(u * u + v * v);
  float K = conf * (1.0f + r * 0.1f);
  // Forward confinement (as k_conf_turb), then the turbulence adjoint at it.
  float u1 = u + K * ny * w * dt;
  float v1 = v - K * nx * w * dt;
  float lu = dU[c], lv = dV[c];
  if (do_turb) {
    float r1 = sqrtf(u1 * u1 + v1 * v1);
    if (r1 > 0.1f && 0.5f * r1 < 1.0f) {
      float2 nz = noise[c];
      float s = (lu * nz.x * turbStrength + lv * nz.y * turbStrength) * 0.5f;
      lu = lu + s * (u1 / r1);
      lv = lv + s * (v1 / r1);
    }
  }
  // Confinement: u1 = u + K ny w dt, v1 = v - K nx w dt.
  float a = lu * dt, b = -lv * dt;
  float S = a * ny + b * nx;
  float lK = w * S;
  float ou = lu, ov = lv;
  if (r > 0.0f) {
    ou = ou + lK * conf * 0.1f * (u / r);
    ov = ov + lK * conf * 0.1f * (v / r);
  }
  dU[c] = ou;
  dV[c] = ov;
  lw[c] = K * S;
  float Lnx = K * w * b, Lny = K * w * a;
  float im = 1.0f / m;
  float qx = Lnx * im, qy = Lny * im;
  if (rg > 0.0f) {
    float t = (Lnx * gx + Lny * gy) / (rg * m * m);
    qx = qx - t * gx;
    qy = qy - t * gy;
  }
  lgx[c] = qx;
  lgy[c] = qy;
}
__global__ void k_adj_conf_local(float* __restrict__ dU, float* __restrict__ dV,
                                 const float* __restrict__ U2, const float* __restrict__ V2,
                                 const float2* __restrict__ noise,
                                 const uint8_t* __restrict__ flags, float conf, float dt,
                                 float turbStrength, int do_turb, float* __restrict__ lw,
                                 float* __restrict__ lgx, float* __restrict__ lgy, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_conf_local_cell(i, j, dU, dV, U2, V2, noise, flags, conf, dt, turbStrength, do_turb, lw, lgx, lgy, g);
}

// Adjoint of every cell's curl: its direct use plus the |curl| terms of the
// four neighbours' gradients.  Gathers lgx, lgy from the neighbours.
__device__ __forceinline__ void adj_conf_curl_cell(int i, int j, const float* __restrict__ U2,
                                                   const float* __restrict__ V2,
                                                   const float* __restrict__ lwd,
                                                   const float* __restrict__ lgx,
                                                   const float* __restrict__ lgy,
                                                   float* __restrict__ lw,
                                                   const uint8_t* __restrict__ flags,
                                                   const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  float out = 0.0f;
  if (fluid_interior(flags[c])) {
    float w = curl_at(U2, V2, flags, c, g);
    float sg = w > 0.0f ? 1.0f : (w < 0.0f ? -1.0f : 0.0f);
    float k = 0.5f / g.h;
    out = lwd[c] + sg * k * ((lgx[c - P] - lgx[c + P]) + (lgy[c - 1] - lgy[c + 1]));
  }
  lw[c] = out;
}
__global__ void k_adj_conf_curl(const float* __restrict__ U2, const float* __restrict__ V2,
                                const float* __restrict__ lwd, const float* __restrict__ lgx,
                                const float* __restrict__ lgy, float* __restrict__ lw,
                                const uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_conf_curl_cell(i, j, U2, V2, lwd, lgx, lgy, lw, flags, g);
}

// curl^T: dU[m] += (lw[m+1] - lw[m-1]) / 2h, dV[m] += (lw[m-P] - lw[m+P]) / 2h
// (lw is 0 off the fluid interior cells).
__device__ __forceinline__ void adj_conf_apply_cell(int i, int j, float* __restrict__ dU,
                                                    float* __restrict__ dV,
                                                    const float* __restrict__ lw, const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  float k = 0.5f / g.h;
  float wN = j + 1 < g.NY ? lw[c + 1] : 0.0f, wS = j >= 1 ? lw[c - 1] : 0.0f;
  float wE = i + 1 < g.NX ? lw[c + P] : 0.0f, wW = i >= 1 ? lw[c - P] : 0.0f;
  dU[c] = dU[c] + k * (wN - wS);
  dV[c] = dV[c] + k * (wW - wE);
}
__global__ void k_adj_conf_apply(float* __restrict__ dU, float* __restrict__ dV,
                                 const float* __restrict__ lw, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_conf_apply_cell(i, j, dU, dV, lw, g);
}

// G^T: the adjoint of the gradient subtract with respect to phi, as the
// Jacobi right-hand side of the adjoint solve: rhs = G^T (dU, dV) on active
// cells, and bw = w * rhs.
__device__ __forceinline__ void adj_grad_t_cell(int i, int j, const float* __restrict__ dU,
                                                const float* __restrict__ dV,
                                                const float* __restrict__ W,
                                                float* __restrict__ rhs, float* __restrict__ BW,
                                                const uint8_t* __restrict__ flags, const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  uint8_t fl = flags[c];
  float r = 0.0f;
  if (flag_active(fl)) {
    r = fbit(fl, F_E) * dU[c + P] - fbit(fl, F_W) * dU[c] + fbit(fl, F_N) * dV[c + 1] -
        fbit(fl, F_S) * dV[c];
  }
  rhs[c] = r;
  BW[c] = W[c] * r;
}
__global__ void k_adj_grad_t(const float* __restrict__ dU, const float* __restrict__ dV,
                             const float* __restrict__ W, float* __restrict__ rhs,
                             float* __restrict__ BW, const uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_grad_t_cell(i, j, dU, dV, W, rhs, BW, flags, g);
}

// The adjoint of the outer correction's right-hand side: r = lam - A e on
// active cells (e: the correction solve run on lam), the exact residual
// rounded once as resid_ff forms it, and w * r for the main solve that
// follows.  e is exactly 0 off the active cells.
__device__ __forceinline__ void adj_resid_cell(int i, int j, const float* __restrict__ lam,
                                               const float* __restrict__ e0,
                                               const float* __restrict__ e1,
                                               const void* __restrict__ esel,
                                               const float* __restrict__ W,
                                               float* __restrict__ rhs, float* __restrict__ BW,
                                               const uint8_t* __restrict__ flags, const Grid& g) {
  const int P = g.P;
  int c = i * P + j;
  uint8_t fl = flags[c];
  float r = 0.0f;
  if (flag_active(fl)) {
    const float* e = (*(const int*)esel) ? e1 : e0;
    r = resid_ff(lam[c], e[c - P], e[c + P], e[c - 1], e[c + 1], (float)flag_count(fl), e[c]).hi;
  }
  rhs[c] = r;
  BW[c] = W[c] * r;
}
__global__ void k_adj_resid(const float* __restrict__ lam, const float* __restrict__ e0,
                            const float* __restrict__ e1, const void* __restrict__ esel,
                            const float* __restrict__ W, float* __restrict__ rhs,
                            float* __restrict__ BW, const uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_resid_cell(i, j, lam, e0, e1, esel, W, rhs, BW, flags, g);
}

// div^T: with b = -div on active cells, d(face) += db(cell on its high side)
// - db(cell on its low side), db = the adjoint solve's result (0 off active)
// plus, with the outer correction, the correction solve's (e0/e1, else null).
__device__ __forceinline__ void adj_div_t_cell(int i, int j, float* __restrict__ dU,
                                               float* __restrict__ dV, const float* __restrict__ x0,
                                               const float* __restrict__ x1,
                                               const void* __restrict__ ctl_sel,
                                               const float* __restrict__ e0,
                                               const float* __restrict__ e1,
                                               const void* __restrict__ esel,
                                               const uint8_t* __restrict__ flags, const Grid& g) {
  const int P = g.P;
  const float* db = (*(const int*)ctl_sel) ? x1 : x0;
  const float* de = e0 ? ((*(const int*)esel) ? e1 : e0) : nullptr;
  int c = i * P + j;
  auto val = [&](int k) { return de ? db[k] + de[k] : db[k]; };
  bool act = flag_active(flags[c]);
  float bc = act ? val(c) : 0.0f;
  if (i >= 1) {
    float bl = flag_active(flags[c - P]) ? val(c - P) : 0.0f;
    dU[c] = dU[c] + (bc - bl);
  }
  if (j >= 1) {
    float bb = flag_active(flags[c - 1]) ? val(c - 1) : 0.0f;
    dV[c] = dV[c] + (bc - bb);
  }
}
__global__ void k_adj_div_t(float* __restrict__ dU, float* __restrict__ dV,
                            const float* __restrict__ x0, const float* __restrict__ x1,
                            const void* __restrict__ ctl_sel, const float* __restrict__ e0,
                            const float* __restrict__ e1, const void* __restrict__ esel,
                            const uint8_t* __restrict__ flags, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  adj_div_t_cell(i, j, dU, dV, x0, x1, ctl_sel, e0, e1, esel, flags, g);
}

// Sources that set U, V (SetVelocity) or M (a smoke assignment) cut the
// derivative there.
__device__ __forceinline__ void adj_sources_group(float* dU, float* dV, float* dM,
                                                  const SourceRec* __restrict__ recs, uint32_t b,
                                                  uint32_t e, const uint8_t* __restrict__ flags,
                                                  const Grid& g) {
  uint32_t cell = recs[b].cell;
  int i = (int)(cell / (uint32_t)g.NY), j = (int)(cell % (uint32_t)g.NY);
  int c = i * g.P + j;
  bool fluid = (flags[c] & F_FLUID) != 0;
  bool set = false, set_m = false;
  for (uint32_t q = b; q < e; ++q) {
    SourceRec r = recs[q];
    if ((r.mode & 1u) && !fluid) continue;
    if (r.mode & 2u) set = true;
    if (r.mode & 8u) set_m = true;
  }
  if (set) {
    dU[c] = 0.0f;
    dV[c] = 0.0f;
  }
  if (set_m) dM[c] = 0.0f;
}
__global__ void k_adj_sources(float* __restrict__ dU, float* __restrict__ dV,
                              float* __restrict__ dM, const SourceRec* __restrict__ recs,
                              const uint32_t* __restrict__ off, int n_groups,
                              const uint8_t* __restrict__ flags, Grid g) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_groups) return;
  adj_sources_group(dU, dV, dM, recs, off[k], off[k + 1], flags, g);
}
__global__ void kb_adj_sources(float* __restrict__ dU, float* __restrict__ dV,
                               float* __restrict__ dM, const SourceRec* __restrict__ recs,
                               const uint32_t* __restrict__ off, const int* __restrict__ gs,
                               int n_groups, const uint8_t* __restrict__ flags,
                               const BScene* __restrict__ sc) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_groups) return;
  const BScene& s = sc[gs[k]];
  adj_sources_group(dU + s.off, dV + s.off, dM + s.off, recs, off[k], off[k + 1], flags + s.off,
                    s.g);
}

// Zeroes the force field where a source sets U, V (the forward adds the
// forces before the sources, which overwrite those cells).
__global__ void k_mask_forces(float* __restrict__ Fu, float* __restrict__ Fv,
                              const SourceRec* __restrict__ recs,
                              const uint32_t* __restrict__ off, int n_groups,
                              const uint8_t* __restrict__ flags, Grid g) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_groups) return;
  uint32_t cell = recs[off[k]].cell;
  int i = (int)(cell / (uint32_t)g.NY), j = (int)(cell % (uint32_t)g.NY);
  int c = i * g.P + j;
  bool fluid = (flags[c] & F_FLUID) != 0;
  for (uint32_t q = off[k]; q < off[k + 1]; ++q) {
    SourceRec r = recs[q];
    if ((r.mode & 1u) && !fluid) continue;
    if (r.mode & 2u) {
      Fu[c] = 0.0f;
      Fv[c] = 0.0f;
    }
  }
}

// A batch's loss: L_s = ||M_s - target_s||_2 per scene.  Block rows of the
// sums of squares per cell tile, one block per scene to combine its tiles'
// rows, then the seed dL/dM_s = (M_s - target_s) / L_s.
__global__ void kb_loss_partials(const BTile* __restrict__ tiles, const BScene* __restrict__ sc,
                                 const float* __restrict__ M, const float* __restrict__ T,
                                 float* __restrict__ part) {
  __shared__ float sh[64];
  const BTile t = tiles[blockIdx.x];
  const BScene& s = sc[t.s];
  int j = t.x * blockDim.x + threadIdx.x;
  int i = t.y * blockDim.y + threadIdx.y;
  FF v[1] = {{0.0f, 0.0f}};
  if (i >= 1 && i <= s.g.NX - 2 && j >= 1 && j <= s.g.NY - 2) {
    long long c = s.off + (long long)i * s.g.P + j;
    v[0] = ff_sq(M[c] - T[c]);
  }
  block_row<1>(v, 0u, sh, part + 2 * (size_t)blockIdx.x);
}
__global__ void kb_loss_combine(const float* __restrict__ part, const int* __restrict__ range,
                                double* __restrict__ losses) {
  __shared__ float sh[64];
  __shared__ float row[2];
  const int s = blockIdx.x;
  FF v[1] = {{0.0f, 0.0f}};
  for (int k = range[2 * s] + threadIdx.x; k < range[2 * s + 1]; k += blockDim.x) {
    FF w[1] = {{part[2 * (size_t)k], part[2 * (size_t)k + 1]}};
    slots_merge<1>(v, w, 0u);
  }
  block_row<1>(v, 0u, sh, row);
  __syncthreads();
  if (threadIdx.x == 0) {
    double L = sqrt((double)row[0] + (double)row[1]);
    losses[s] = L;
    // 1 / L_s as floats after the n losses.
    reinterpret_cast<float*>(losses + gridDim.x)[s] = L > 0.0 ? (float)(1.0 / L) : 0.0f;
  }
}
__global__ void kb_loss_seed(const BTile* __restrict__ tiles, const BScene* __restrict__ sc,
                             const float* __restrict__ M, const float* __restrict__ T,
                             const double* __restrict__ losses, int n_scenes,
                             float* __restrict__ lamM) {
  const BTile t = tiles[blockIdx.x];
  const BScene& s = sc[t.s];
  int j = t.x * blockDim.x + threadIdx.x;
  int i = t.y * blockDim.y + threadIdx.y;
  if (i >= s.g.NX || j >= s.g.NY) return;
  long long c = s.off + (long long)i * s.g.P + j;
  float inv = reinterpret_cast<const float*>(losses + n_scenes)[t.s];
  float v = 0.0f;
  if (i >= 1 && i <= s.g.NX - 2 && j >= 1 && j <= s.g.NY - 2) v = (M[c] - T[c]) * inv;
  lamM[c] = v;
}

// Loss L = ||M - target||_2 over interior cells: float-pair block rows of
// sum (M - target)^2, combined later.
__global__ void k_loss_partials(const float* __restrict__ M, const float* __restrict__ T,
                                float* __restrict__ part, Grid g) {
  __shared__ float sh[64];
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  FF v[1] = {{0.0f, 0.0f}};
  if (i >= 1 && i <= g.NX - 2 && j >= 1 && j <= g.NY - 2) {
    int c = i * g.P + j;
    v[0] = ff_sq(M[c] - T[c]);
  }
  block_row<1>(v, 0u, sh, part + 2 * (size_t)(blockIdx.y * gridDim.x + blockIdx.x));
}

// L = sqrt(sum) in FP64 (the float-pair sum carries ~48 bits, so
// differences of nearby losses stay resolved) and 1 / L rounded to float.
__global__ void k_loss_finish(const float* __restrict__ row, double* __restrict__ loss,
                              float* __restrict__ inv) {
  double L = sqrt((double)row[0] + (double)row[1]);
  loss[0] = L;
  inv[0] = L > 0.0 ? (float)(1.0 / L) : 0.0f;
}

// Seeds the adjoint state with dL/dM = (M - target) / L on interior cells,
// zero elsewhere.
__global__ void k_loss_seed(const float* __restrict__ M, const float* __restrict__ T,
                            const float* __restrict__ inv, float* __restrict__ lamM, Grid g) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.NX || j >= g.NY) return;
  int c = i * g.P + j;
  float v = 0.0f;
  if (i >= 1 && i <= g.NX - 2 && j >= 1 && j <= g.NY - 2) v = (M[c] - T[c]) * inv[0];
  lamM[c] = v;
}

// Start of a step's adjoint: the state after the step holds U5, V5 and M2
// twice (state and staging copy), so their adjoints add; the staging
// adjoints restart at zero (they collect the stale reads of the step), as
// do the work fields that accumulate.
__global__ void k_adj_begin(float* __restrict__ aU, float* __restrict__ aV, float* __restrict__ aM,
                            float* __restrict__ aNU, float* __restrict__ aNV,
                            float* __restrict__ aNM, float* __restrict__ w0,
                            float* __restrict__ w1, float* __restrict__ w2,
                            float* __restrict__ w3, float* __restrict__ w4,
                            float* __restrict__ w5, int n) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  aU[k] = aU[k] + aNU[k];
  aV[k] = aV[k] + aNV[k];
  aM[k] = aM[k] + aNM[k];
  aNU[k] = 0.0f;
  aNV[k] = 0.0f;
  aNM[k] = 0.0f;
  w0[k] = 0.0f;
  w1[k] = 0.0f;
  w2[k] = 0.0f;
  w3[k] = 0.0f;
  w4[k] = 0.0f;
  w5[k] = 0.0f;
}

}  // namespace

cudaError_t launch_loss_seed(fg_fluid* f, const float* target, double* dev_loss) {
  if (f->batch) {
    const BatchGeom* b = f->batch;
    if (!partials_fit(f, 1, b->n_cell_tiles)) return cudaErrorInvalidValue;
    count(f, 3);
    kb_loss_partials<<<b->n_cell_tiles, dim3(b->bx, b->by), 0, f->stream>>>(
        b->cell_tiles, b->scenes_dev, f->d[FG_M], target, f->partials);
    kb_loss_combine<<<b->n, 256, 0, f->stream>>>(f->partials, b->cell_range, b->losses);
    kb_loss_seed<<<b->n_cell_tiles, dim3(b->bx, b->by), 0, f->stream>>>(
        b->cell_tiles, b->scenes_dev, f->d[FG_M], target, b->losses, b->n,
        f->adj[fg_fluid::A_M]);
    size_t bytes = sizeof(float) * (size_t)f->NX * f->P;
    for (int k : {fg_fluid::A_U, fg_fluid::A_V, fg_fluid::A_NU, fg_fluid::A_NV, fg_fluid::A_NM}) {
      cudaError_t e = cudaMemsetAsync(f->adj[k], 0, bytes, f->stream);
      if (e != cudaSuccess) return e;
    }
    (void)dev_loss;
    return cudaGetLastError();
  }
  dim3 gr = cell_grid(f), bl(BX, BY);
  int nb = gr.x * gr.y;
  if (!partials_fit(f, 1, nb)) return cudaErrorInvalidValue;
  count(f);
  k_loss_partials<<<gr, bl, 0, f->stream>>>(f->d[FG_M], target, f->partials, f->g);
  float* row = nullptr;
  count(f, combine_rows<1>(f->stream, f->partials, nb, 0u, &row));
  // 1 / L in the float after the FP64 loss (the scalar slots hold 8 floats).
  float* inv = reinterpret_cast<float*>(dev_loss) + 2;
  count(f, 2);
  k_loss_finish<<<1, 1, 0, f->stream>>>(row, dev_loss, inv);
  k_loss_seed<<<gr, bl, 0, f->stream>>>(f->d[FG_M], target, inv, f->adj[fg_fluid::A_M], f->g);
  size_t bytes = sizeof(float) * (size_t)f->NX * f->P;
  for (int k : {fg_fluid::A_U, fg_fluid::A_V, fg_fluid::A_NU, fg_fluid::A_NV, fg_fluid::A_NM}) {
    cudaError_t e = cudaMemsetAsync(f->adj[k], 0, bytes, f->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

// Adjoint of one recorded step (see the file comment).  On entry adj[A_U..
// A_NM] hold the adjoint of the state after the step; on exit the adjoint of
// the state before it, and adj[A_FORCE_U/V] the adjoint of the step's force
// fields.  tape: the kTapeFields fields recorded by the forward step.
cudaError_t launch_step_adjoint(fg_fluid* f, float dt, float* const* tape) {
  const fg_params& p = f->prm;
  const Grid& g = f->g;
  size_t bytes = sizeof(float) * (size_t)f->NX * f->P;
  float** A = f->adj;
  using F = fg_fluid;
  float *U2 = tape[0], *V2 = tape[1], *U4 = tape[2], *V4 = tape[3], *fwdU = tape[4],
        *fwdV = tape[5], *corrU = tape[6], *corrV = tape[7], *U5 = tape[8], *V5 = tape[9],
        *M1 = tape[10], *fwdM = tape[11], *corrM = tape[12];
  cudaStream_t st = f->stream;
  cudaError_t e;
  const int n = f->NX * f->P;
  count(f);
  k_adj_begin<<<(n + 255) / 256, 256, 0, st>>>(A[F::A_U], A[F::A_V], A[F::A_M], A[F::A_NU],
                                               A[F::A_NV], A[F::A_NM], A[F::A_CU], A[F::A_CV],
                                               A[F::A_FU], A[F::A_FV], A[F::A_CM], A[F::A_FM], n);
  float sa = p.smoke_advection;
  // ---- smoke (the trace velocity is the final U5, V5)
  // dU5, dV5 accumulate into A_U, A_V (already holding dU5 from the state).
  if (p.use_bfecc) {
    // pass 4: final SL of corrM
    count(f);
    FG_CELLS(f, k_adj_sl_smoke, adj_sl_smoke_cell, A[F::A_M], U5, V5, corrM, A[F::A_U], A[F::A_V], A[F::A_CM],
                                      A[F::A_NM], f->flags, dt, sa, 0);
    // compensation + clamp and the reverse sample of fwdM traced with U5,
    // V5 at +dt: dM1 (orig), dfwdM, dU5
    if ((e = cudaMemsetAsync(A[F::A_M], 0, bytes, st)) != cudaSuccess) return e;
    count(f);
    FG_CELLS(f, k_adj_bfecc_smoke, adj_bfecc_smoke_cell, A[F::A_CM], U5, V5, M1, fwdM, A[F::A_M], A[F::A_FM],
                                         A[F::A_U], A[F::A_V], f->flags, dt, sa);
    // pass 1: forward SL of M1
    count(f);
    FG_CELLS(f, k_adj_sl_smoke, adj_sl_smoke_cell, A[F::A_FM], U5, V5, M1, A[F::A_U], A[F::A_V], A[F::A_M],
                                      A[F::A_NM], f->flags, dt, sa, 0);
  } else {
    // single SL pass of M1: dM2 moves to the zeroed work field, dM1
    // accumulates in the other
    std::swap(A[F::A_M], A[F::A_CM]);
    count(f);
    FG_CELLS(f, k_adj_sl_smoke, adj_sl_smoke_cell, A[F::A_CM], U5, V5, M1, A[F::A_U], A[F::A_V], A[F::A_M],
                                      A[F::A_NM], f->flags, dt, sa, 0);
  }
  // ---- velocity advection: A_U/A_V hold dU5/dV5; produce dU4 in A_CU..
  if (p.use_bfecc) {
    // pass 4: final SL of corr traced with corr: d -> dcorr (A_CU/A_CV)
    count(f);
    FG_CELLS(f, k_adj_sl_velocity, adj_sl_velocity_cell, A[F::A_U], A[F::A_V], corrU, corrV, corrU, corrV,
                                         A[F::A_CU], A[F::A_CV], A[F::A_CU], A[F::A_CV],
                                         A[F::A_CU], A[F::A_CV], A[F::A_NU], A[F::A_NV], f->flags,
                                         dt);
    // dU4 accumulates into A_U/A_V (reset first); compensation + clamp and
    // the reverse sample of fwd traced with U4 at +dt: dfwd (A_FU/A_FV), dU4
    if ((e = cudaMemsetAsync(A[F::A_U], 0, bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(A[F::A_V], 0, bytes, st)) != cudaSuccess) return e;
    count(f);
    FG_CELLS(f, k_adj_bfecc_vel, adj_bfecc_vel_cell, A[F::A_CU], A[F::A_CV], U4, V4, fwdU, fwdV, A[F::A_U],
                                       A[F::A_V], A[F::A_FU], A[F::A_FV], f->flags, dt);
    // pass 1: forward SL of U4 traced with U4
    count(f);
    FG_CELLS(f, k_adj_sl_velocity, adj_sl_velocity_cell, A[F::A_FU], A[F::A_FV], U4, V4, U4, V4, A[F::A_U],
                                         A[F::A_V], A[F::A_U], A[F::A_V], A[F::A_U], A[F::A_V],
                                         A[F::A_NU], A[F::A_NV], f->flags, dt);
  } else {
    std::swap(A[F::A_U], A[F::A_CU]);
    std::swap(A[F::A_V], A[F::A_CV]);
    count(f);
    FG_CELLS(f, k_adj_sl_velocity, adj_sl_velocity_cell, A[F::A_CU], A[F::A_CV], U4, V4, U4, V4, A[F::A_U],
                                         A[F::A_V], A[F::A_U], A[F::A_V], A[F::A_U], A[F::A_V],
                                         A[F::A_NU], A[F::A_NV], f->flags, dt);
  }
  // ---- borders, confinement + turbulence (A_U/A_V: dU4 -> dU3 -> dU2)
  count(f);
  FG_BORDER(f, k_adj_borders, adj_borders_border, A[F::A_U], A[F::A_V],
            (const uint8_t*)f->flags);
  if (p.confinement != 0.0f) {
    // Work fields A_CU, A_CV, A_FU, A_FV are free again here.
    count(f, 3);
    FG_CELLS(f, k_adj_conf_local, adj_conf_local_cell, A[F::A_U], A[F::A_V], U2, V2, f->noise, f->flags,
                                        p.confinement, dt, p.turbulence_strength * dt,
                                        p.turbulence_strength > 0.0f ? 1 : 0, A[F::A_CU],
                                        A[F::A_CV], A[F::A_FU]);
    FG_CELLS(f, k_adj_conf_curl, adj_conf_curl_cell, U2, V2, A[F::A_CU], A[F::A_CV], A[F::A_FU], A[F::A_FV],
                                       f->flags);
    FG_CELLS(f, k_adj_conf_apply, adj_conf_apply_cell, A[F::A_U], A[F::A_V], A[F::A_FV]);
  } else if (p.turbulence_strength > 0.0f) {
    count(f);
    FG_CELLS(f, k_adj_turbulence, adj_turbulence_cell, A[F::A_U], A[F::A_V], U2, V2, f->noise, f->flags,
                                        p.turbulence_strength * dt);
  }
  // ---- projection: dU1 = dU2 + div^T M^T G^T dU2, where the potential is
  // M b with M = P_K (K sweeps from 0) and, with the outer correction,
  // M = P_K + P_c (I - A P_K) (P_c: its K_c sweeps).  P_K, P_c and A are
  // symmetric, so M^T lam = P_K (lam - A P_c lam) + P_c lam: the correction
  // solve runs first, on lam, then the main solve on the residual.
  count(f);
  FG_CELLS(f, k_adj_grad_t, adj_grad_t_cell, A[F::A_U], A[F::A_V], f->wgt, f->rhs, f->bw, f->flags);
  const bool refine = p.refine_sweeps > 0;
  const float* rhs_main = f->rhs;
  const float* bw_main = f->bw;
  if (refine) {
    if ((e = launch_jacobi_solve(f, f->pctl, f->rhs, f->bw, f->err, f->err2,
                                 p.refine_sweeps)) != cudaSuccess)
      return e;
    count(f);
    FG_CELLS(f, k_adj_resid, adj_resid_cell, (const float*)f->rhs, (const float*)f->err,
             (const float*)f->err2, (const void*)((const int*)f->pctl + 1),
             (const float*)f->wgt, f->rhs_e, f->bwe, (const uint8_t*)f->flags);
    rhs_main = f->rhs_e;
    bw_main = f->bwe;
  }
  if (p.num_iters > 0) {
    if ((e = launch_jacobi_solve(f, f->ectl, rhs_main, bw_main, f->phi, f->phi2, p.num_iters)) !=
        cudaSuccess)
      return e;
  } else {
    if ((e = cudaMemsetAsync(f->phi, 0, bytes, st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(f->ectl, 0, sizeof(int) * 8, st)) != cudaSuccess) return e;
  }
  count(f);
  FG_CELLS(f, k_adj_div_t, adj_div_t_cell, A[F::A_U], A[F::A_V], f->phi, f->phi2,
           (const void*)((const int*)f->ectl + 1), refine ? (const float*)f->err : nullptr,
           (const float*)f->err2, (const void*)((const int*)f->pctl + 1),
           (const uint8_t*)f->flags);
  // ---- sources (the forces' adjoint is then the state's)
  if (f->n_src_groups > 0) {
    count(f);
    if (f->batch)
      kb_adj_sources<<<(f->n_src_groups + 255) / 256, 256, 0, st>>>(
          A[F::A_U], A[F::A_V], A[F::A_M], f->src_dev, f->src_off_dev, f->batch->src_scene,
          f->n_src_groups, f->flags, f->batch->scenes_dev);
    else
      k_adj_sources<<<(f->n_src_groups + 255) / 256, 256, 0, st>>>(
          A[F::A_U], A[F::A_V], A[F::A_M], f->src_dev, f->src_off_dev, f->n_src_groups, f->flags,
          g);
  }
  return cudaGetLastError();
}

cudaError_t launch_mask_forces(fg_fluid* f, float* fu, float* fv) {
  if (f->n_src_groups <= 0 || f->batch) return cudaSuccess;
  count(f);
  k_mask_forces<<<(f->n_src_groups + 255) / 256, 256, 0, f->stream>>>(
      fu, fv, f->src_dev, f->src_off_dev, f->n_src_groups, f->flags, f->g);
  return cudaGetLastError();
}

cudaError_t launch_add_forces(fg_fluid* f, const float* fu, const float* fv) {
  count(f);
  FG_CELLS(f, k_add_forces, add_forces_cell, f->d[FG_U], f->d[FG_V], fu, fv);
  return cudaGetLastError();
}

}  // namespace fg
