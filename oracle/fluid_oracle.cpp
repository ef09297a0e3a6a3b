// CPU oracle for the fluid simulation step (test infrastructure only).
//
// This file restates, in C++17, the simulation step of the Go package
// pkg/fluid (TheFellow/fluid).  It is the checker for the CUDA path: only the
// test-suite, the smoke entry and the CPU-baseline leg of the benchmark load
// it, and nothing in the product links against it.
//
// Two kinds of restatement live here, selected per instance:
//   * the reference scheme (Scheme::LexSOR): the exact operation order of
//     pkg/fluid/fluid.go, including the serial lexicographic SOR pressure loop
//     with its relaxation schedule and early exit (fluid.go:157-234), the
//     stage order of Simulate (fluid.go:79-109) and the hidden newU/newV/newM
//     staging state (fluid.go:291-434, walls.go:26-47);
//   * the GPU scheme (Scheme::Jacobi / Scheme::RedBlack): the same step with
//     the pressure loop replaced by the parallel relaxation the CUDA kernels
//     run, with the identical per-cell operation order, so the FP32 GPU
//     result can be compared bit for bit.
// The template parameter T is float (FP32-faithful: Go's float32 arithmetic,
// math.* evaluated in double and rounded back) or double (the FP64 oracle).
//
// Build with -O2 -ffp-contract=off and without -ffast-math: every float op is
// a separately rounded IEEE op, which is what Go's compiler emits on amd64.
//
// Parity pin: the reference's own known-answer and threshold tests
// (pkg/fluid/fluid_test.go, confinement_test.go) are ported under tests/ and
// run against this oracle.  There is no Go toolchain to produce golden field
// dumps, so bit-level agreement with the Go binary itself is unpinned.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

namespace orc {

enum Scheme { LexSOR = 0, Jacobi = 1, RedBlack = 2, MgJacobi = 3 };

// ---------------------------------------------------------------------------
// Thread pool standing in for parallelRange (pkg/fluid/parallel.go:10-39):
// static contiguous chunks of [start,end) over the worker count.
// ---------------------------------------------------------------------------
class Pool {
 public:
  explicit Pool(int n) : n_(std::max(1, n)) {
    for (int w = 1; w < n_; ++w) threads_.emplace_back([this, w] { loop(w); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }
  int size() const { return n_; }
  void range(int start, int end, const std::function<void(int)>& fn) {
    int total = end - start;
    if (total <= 0) return;
    int workers = std::min(n_, total);
    if (workers == 1) {
      for (int i = start; i < end; ++i) fn(i);
      return;
    }
    int chunk = (total + workers - 1) / workers;
    {
      std::lock_guard<std::mutex> g(m_);
      fn_ = &fn;
      start_ = start;
      end_ = end;
      chunk_ = chunk;
      workers_ = workers;
      pending_ = workers - 1;
      ++gen_;
    }
    cv_.notify_all();
    run_chunk(0);
    std::unique_lock<std::mutex> lk(m_);
    done_cv_.wait(lk, [this] { return pending_ == 0; });
    fn_ = nullptr;
  }

 private:
  void run_chunk(int w) {
    int s = start_ + w * chunk_;
    int e = std::min(s + chunk_, end_);
    for (int i = s; i < e; ++i) (*fn_)(i);
  }
  void loop(int w) {
    uint64_t seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return gen_ != seen; });
      seen = gen_;
      if (stop_) return;
      bool mine = w < workers_;
      lk.unlock();
      if (mine) {
        run_chunk(w);
        std::lock_guard<std::mutex> g(m_);
        if (--pending_ == 0) done_cv_.notify_all();
      }
    }
  }
  int n_;
  std::vector<std::thread> threads_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* fn_ = nullptr;
  int start_ = 0, end_ = 0, chunk_ = 0, workers_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// ---------------------------------------------------------------------------
// Go semantics helpers.
// ---------------------------------------------------------------------------
// Go's builtin min/max on floats: NaN wins, and -0 < +0.
template <typename T>
inline T go_min(T a, T b) {
  if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<T>::quiet_NaN();
  if (a == b) return std::signbit(a) ? a : b;
  return a < b ? a : b;
}
template <typename T>
inline T go_max(T a, T b) {
  if (std::isnan(a) || std::isnan(b)) return std::numeric_limits<T>::quiet_NaN();
  if (a == b) return std::signbit(a) ? b : a;
  return a > b ? a : b;
}
// float32(math.Sqrt(float64(x))) / math.Sqrt for T=double.
template <typename T>
inline T go_sqrt(T x) { return (T)std::sqrt((double)x); }
template <typename T>
inline T go_abs(T x) { return (T)std::fabs((double)x); }

struct Stats {
  double div_l2_post = 0, div_max_post = 0, div_count_post = 0;
  double resid_l2 = 0, resid_max = 0;
  double smoke_mass = 0;
  int sweeps = 0;
  double last_maxdiv = 0;
};

template <typename T>
struct Fluid {
  T density, h;
  int NX, NY, N;
  std::vector<T> U, V, newU, newV, p, S, M, newM;
  T Confinement = 0, ViscosityDiffusion = 0, PressureDamping = 1,
    TurbulenceStrength = (T)0.02, SmokeAdvection = 1;
  bool UseMultigrid = false;
  int MultigridLevels = 2;
  bool UseBFECC = false;
  T Relaxation = (T)1.9;  // package var Relaxation (fluid.go:7-9)

  // Extensions shared with the CUDA path.
  int num_iters = 8;        // numIters, hard-coded to 8 in Simulate (fluid.go:81)
  T tolerance = (T)1e-5;    // fluid.go:159
  bool early_exit = true;
  int scheme = LexSOR;
  T jacobi_omega = 1;       // relaxation of the parallel schemes
  int check_every = 1;      // early-exit check interval (sweeps) of the parallel schemes
  int refine_sweeps = 0;    // FP64-residual outer correction sweeps (0 = off)
  // Departure points of the advection relative to their face (the GPU's
  // fg_params.precise_coords); off: the reference's absolute coordinates.
  bool precise_coords = false;

  // Parallel-scheme work arrays.
  std::vector<T> phi, phi2, rhs, err, err2;
  std::vector<uint8_t> cnt;  // neighbour fluid count of active cells, 0 = inactive
  Stats st;
  Pool* pool;

  Fluid(T density_, int width, int height, T h_, Pool* pool_)
      : density(density_), h(h_), NX(width + 2), NY(height + 2),
        N((width + 2) * (height + 2)), pool(pool_) {
    U.assign(N, 0); V.assign(N, 0); newU.assign(N, 0); newV.assign(N, 0);
    p.assign(N, 0); S.assign(N, 0); M.assign(N, 0); newM.assign(N, 0);
  }
  inline int ix(int i, int j) const { return i * NY + j; }
  void par(int s, int e, const std::function<void(int)>& fn) { pool->range(s, e, fn); }

  // ---------------------------------------------------------------- Simulate
  // fluid.go:79-109
  void simulate(T dt) {
    int numIters = num_iters;
    std::fill(p.begin(), p.end(), (T)0);
    if (ViscosityDiffusion > 0) applyViscosity(dt);
    makeIncompressible(numIters, dt);
    if (Confinement != 0) applyVorticityConfinement(dt);
    if (TurbulenceStrength > 0) addTurbulence(dt);
    handleBorders();
    if (UseBFECC) {
      advectVelocityBFECC(dt);
      advectSmokeBFECC(dt);
    } else {
      advectVelocity(dt);
      advectSmoke(dt);
    }
    st.smoke_mass = smokeMass();
  }

  // fluid.go:112-142
  void applyViscosity(T dt) {
    if (ViscosityDiffusion <= 0) return;
    int n = NY;
    T visc = ViscosityDiffusion * dt;
    newU = U;
    newV = V;
    par(1, NX - 1, [&](int i) {
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] > 0) {
          T uLap = U[(i - 1) * n + j] + U[(i + 1) * n + j] + U[i * n + j - 1] +
                   U[i * n + j + 1] - (T)4 * U[i * n + j];
          newU[i * n + j] = U[i * n + j] + visc * uLap;
          T vLap = V[(i - 1) * n + j] + V[(i + 1) * n + j] + V[i * n + j - 1] +
                   V[i * n + j + 1] - (T)4 * V[i * n + j];
          newV[i * n + j] = V[i * n + j] + visc * vLap;
        }
      }
    });
    U = newU;
    V = newV;
  }

  // fluid.go:144-155
  void makeIncompressible(int numIters, T dt) {
    copyBorder(newU, U);
    copyBorder(newV, V);
    if (UseMultigrid && MultigridLevels > 1) {
      solveMultigridVCycle(numIters, dt);
    } else if (scheme == LexSOR) {
      solveSingleGrid(numIters, dt);
    } else {
      solveParallel(numIters, dt);
    }
    postProjectionStats();
  }

  // fluid.go:157-186
  void solveSingleGrid(int numIters, T dt) {
    T cp = density * h / dt;
    T tol = tolerance;
    T initialRelaxation = Relaxation;
    T minRelaxation = (T)1.2;
    st.sweeps = 0;
    for (int iter = 0; iter < numIters; ++iter) {
      T iterProgress = (T)(unsigned)iter / (T)(unsigned)numIters;
      T currentRelaxation =
          initialRelaxation - (initialRelaxation - minRelaxation) * iterProgress;
      T maxDiv = pressureJacobiIteration(currentRelaxation, cp);
      st.sweeps = iter + 1;
      st.last_maxdiv = maxDiv;
      if (early_exit && maxDiv < tol) break;
    }
  }

  // fluid.go:188-234 (serial, in place, lexicographic i-major then j)
  T pressureJacobiIteration(T relaxation, T cp) {
    int n = NY;
    T maxDiv = 0;
    for (int i = 1; i < NX - 1; ++i) {
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T sx0 = S[(i - 1) * n + j];
        T sx1 = S[(i + 1) * n + j];
        T sy0 = S[i * n + j - 1];
        T sy1 = S[i * n + j + 1];
        T s = sx0 + sx1 + sy0 + sy1;
        if (s == 0) continue;
        T div = U[(i + 1) * n + j] - U[i * n + j] + V[i * n + j + 1] - V[i * n + j];
        T absDiv = go_abs(div);
        if (absDiv > maxDiv) maxDiv = absDiv;
        T pp = -div / s;
        pp *= relaxation;
        pp *= PressureDamping;
        p[i * n + j] += cp * pp;
        U[i * n + j] -= sx0 * pp;
        U[(i + 1) * n + j] += sx1 * pp;
        V[i * n + j] -= sy0 * pp;
        V[i * n + j + 1] += sy1 * pp;
      }
    }
    return maxDiv;
  }

  // ---------------------------------------------------- parallel GPU schemes
  // The masked Poisson system the SOR loop above relaxes, written for the
  // cell potential phi (the accumulated per-cell velocity correction):
  //   s_c phi_c - sum_{n} phi_n = b_c = -div_c,
  // with phi = 0 on inactive cells (solid, border ring, no fluid neighbour),
  // followed by U_face += S_R phi_L - S_L phi_R (and the same for V) and
  // p = cp phi.  Jacobi and red-black relaxations of it run on the GPU.
  // Per active cell c with s_c fluid neighbours, the Jacobi update is
  //   phi' = (1 - om) phi + w_c (nb + b_c),   w_c = om / s_c,  om = omega * damping,
  // evaluated as fma(w_c, nb, bw_c) with bw_c = w_c * b_c precomputed (and an
  // outer fma with 1 - om when om != 1); W = BW = 0 off the active cells.
  void setupSystem() { setupSystemOm(jacobi_omega * PressureDamping); }
  void setupSystemOm(T om) {
    int n = NY;
    phi.assign(N, 0); phi2.assign(N, 0); rhs.assign(N, 0); cnt.assign(N, 0);
    Wc.assign(N, 0); BWc.assign(N, 0);
    par(1, NX - 1, [&](int i) {
      for (int j = 1; j < NY - 1; ++j) {
        int c = i * n + j;
        if (S[c] == 0) continue;
        T s = S[(i - 1) * n + j] + S[(i + 1) * n + j] + S[i * n + j - 1] + S[i * n + j + 1];
        if (s == 0) continue;
        T div = U[(i + 1) * n + j] - U[c] + V[c + 1] - V[c];
        rhs[c] = -div;
        cnt[c] = (uint8_t)s;
        Wc[c] = om / s;
        BWc[c] = Wc[c] * rhs[c];
      }
    });
  }
  std::vector<T> Wc, BWc, BWe;
  // One Jacobi sweep src -> dst; returns max |r| over the active cells, with
  // r = fma(-s, phi, b + nb) the residual of the input iterate.
  T sweepJacobi(const std::vector<T>& b, const std::vector<T>& bw, const std::vector<T>& src,
                std::vector<T>& dst) {
    int n = NY;
    T om1 = (T)1 - jacobi_omega * PressureDamping;
    std::vector<T> rowmax(NX, 0);
    par(1, NX - 1, [&](int i) {
      T mx = 0;
      for (int j = 1; j < NY - 1; ++j) {
        int c = i * n + j;
        T nb = src[c - n] + src[c + n] + src[c - 1] + src[c + 1];
        T y = std::fma(Wc[c], nb, bw[c]);
        if (om1 != 0) y = std::fma(om1, src[c], y);
        int s = cnt[c];
        if (s) {
          T r = std::fma(-(T)s, src[c], b[c] + nb);
          T a = go_abs(r);
          if (a > mx) mx = a;
        }
        dst[c] = y;
      }
      rowmax[i] = mx;
    });
    T mx = 0;
    for (int i = 1; i < NX - 1; ++i)
      if (rowmax[i] > mx) mx = rowmax[i];
    return mx;
  }
  // Red-black SOR half sweep (CPU-only variant), in place.
  T sweepRB(const std::vector<T>& b, std::vector<T>& x, int colour, T omega_scale) {
    int n = NY;
    T w[5];
    for (int s = 1; s <= 4; ++s) w[s] = (omega_scale * PressureDamping) / (T)s;
    std::vector<T> rowmax(NX, 0);
    par(1, NX - 1, [&](int i) {
      T mx = 0;
      for (int j = 1; j < NY - 1; ++j) {
        int c = i * n + j;
        if (((i + j) & 1) != colour) continue;
        int s = cnt[c];
        if (s == 0) continue;
        T nb = x[c - n] + x[c + n] + x[c - 1] + x[c + 1];
        T r = std::fma(-(T)s, x[c], b[c] + nb);
        T a = go_abs(r);
        if (a > mx) mx = a;
        x[c] = std::fma(w[s], r, x[c]);
      }
      rowmax[i] = mx;
    });
    T mx = 0;
    for (int i = 1; i < NX - 1; ++i)
      if (rowmax[i] > mx) mx = rowmax[i];
    return mx;
  }
  // Runs `iters` sweeps on x (ping-pong with tmp); early exit checked after
  // sweeps whose count is a multiple of check_every.  Returns sweeps done.
  int relax(const std::vector<T>& b, const std::vector<T>& bw, std::vector<T>& x,
            std::vector<T>& tmp, int iters, bool allow_exit) {
    int done = 0;
    for (int t = 0; t < iters; ++t) {
      T mx;
      if (scheme == RedBlack) {
        // Red-black SOR with the reference's relaxation schedule.
        T prog = (T)(unsigned)t / (T)(unsigned)iters;
        T om = Relaxation - (Relaxation - (T)1.2) * prog;
        T m0 = sweepRB(b, x, 0, om);
        T m1 = sweepRB(b, x, 1, om);
        mx = m0 > m1 ? m0 : m1;
      } else {
        mx = sweepJacobi(b, bw, x, tmp);
        std::swap(x, tmp);
      }
      done = t + 1;
      // The GPU scheme measures |r| only when it checks the early exit.
      st.last_maxdiv = (allow_exit && early_exit) || scheme == RedBlack ? mx : (T)0;
      if (allow_exit && early_exit && ((t + 1) % check_every) == 0 && mx < tolerance) break;
    }
    return done;
  }
  // ---------------------------------------------------------------- multigrid Jacobi
  // The GPU's parallel V-cycle (scheme MgJacobi) for the same system
  // s_c phi_c - sum_n phi_n = b_c: levels of half the interior size (a
  // coarse cell is fluid if any of its up to 2 x 2 children is; the ghost
  // ring coarsens along its own row or column), damped Jacobi smoothing
  // (weight kMgOmega * PressureDamping, the Jacobi scheme's per-cell
  // arithmetic), the residuals of the children summed into the coarse
  // right-hand side, and the coarse correction interpolated back bilinearly
  // (weights 9, 3, 3, 1 over the active coarse cells around the child).
  // V(2, 2) cycles, 32 sweeps on the coarsest level (interior side <= 8).
  static constexpr float kMgOmega = 0.8f;
  static constexpr int kMgPre = 2, kMgPost = 2, kMgCoarse = 32, kMgMinSide = 8;
  struct MgLevel {
    int NX, NY;
    std::vector<T> S, w, b, bw, x, tmp;
    std::vector<uint8_t> cnt;
  };
  std::vector<MgLevel> mg;
  // Children rows of coarse row I (fine rows of NXf): the ring row for the
  // ring, else the interior rows 2I-1 and 2I that exist.
  static void mgChildren(int I, int NXc, int NXf, int& a, int& b) {
    if (I == 0) { a = b = 0; return; }
    if (I == NXc - 1) { a = b = NXf - 1; return; }
    a = 2 * I - 1;
    b = std::min(2 * I, NXf - 2);
  }
  void mgCounts(MgLevel& L, T om) {
    int n = L.NY;
    L.cnt.assign((size_t)L.NX * n, 0);
    L.w.assign((size_t)L.NX * n, 0);
    for (int i = 1; i < L.NX - 1; ++i)
      for (int j = 1; j < L.NY - 1; ++j) {
        int c = i * n + j;
        if (L.S[c] == 0) continue;
        T s = L.S[c - n] + L.S[c + n] + L.S[c - 1] + L.S[c + 1];
        if (s == 0) continue;
        L.cnt[c] = (uint8_t)s;
        L.w[c] = om / s;
      }
  }
  void mgBuild(T om) {
    mg.assign(1, MgLevel());
    MgLevel& L0 = mg[0];
    L0.NX = NX; L0.NY = NY;
    L0.S = S; L0.cnt = cnt; L0.w = Wc; L0.b = rhs; L0.bw = BWc;
    L0.x.assign(N, 0); L0.tmp.assign(N, 0);
    while (std::min(mg.back().NX, mg.back().NY) - 2 > kMgMinSide) {
      const MgLevel& F = mg.back();
      MgLevel C;
      C.NX = (F.NX - 2 + 1) / 2 + 2;
      C.NY = (F.NY - 2 + 1) / 2 + 2;
      C.S.assign((size_t)C.NX * C.NY, 0);
      for (int I = 0; I < C.NX; ++I)
        for (int J = 0; J < C.NY; ++J) {
          int a0, a1, b0, b1;
          mgChildren(I, C.NX, F.NX, a0, a1);
          mgChildren(J, C.NY, F.NY, b0, b1);
          T v = 0;
          for (int a = a0; a <= a1; ++a)
            for (int b = b0; b <= b1; ++b) v = std::max(v, F.S[a * F.NY + b]);
          C.S[I * C.NY + J] = v;
        }
      mgCounts(C, om);
      size_t nc = (size_t)C.NX * C.NY;
      C.b.assign(nc, 0); C.bw.assign(nc, 0); C.x.assign(nc, 0); C.tmp.assign(nc, 0);
      mg.push_back(std::move(C));
    }
  }
  void mgSmooth(MgLevel& L, int ns, bool zero, T om1) {
    int n = L.NY;
    if (zero) std::fill(L.x.begin(), L.x.end(), (T)0);
    for (int t = 0; t < ns; ++t) {
      par(1, L.NX - 1, [&](int i) {
        for (int j = 1; j < L.NY - 1; ++j) {
          int c = i * n + j;
          T nb = L.x[c - n] + L.x[c + n] + L.x[c - 1] + L.x[c + 1];
          T y = std::fma(L.w[c], nb, L.bw[c]);
          if (om1 != 0) y = std::fma(om1, L.x[c], y);
          L.tmp[c] = y;
        }
      });
      std::swap(L.x, L.tmp);
    }
  }
  void mgRestrict(const MgLevel& F, MgLevel& C) {
    int nf = F.NY, nc = C.NY;
    par(1, C.NX - 1, [&](int I) {
      for (int J = 1; J < C.NY - 1; ++J) {
        int cc = I * nc + J;
        T rs = 0;
        if (C.cnt[cc]) {
          int a0, a1, b0, b1;
          mgChildren(I, C.NX, F.NX, a0, a1);
          mgChildren(J, C.NY, F.NY, b0, b1);
          for (int a = a0; a <= a1; ++a)
            for (int b = b0; b <= b1; ++b) {
              int cf = a * nf + b;
              if (!F.cnt[cf]) continue;
              T nb = F.x[cf - nf] + F.x[cf + nf] + F.x[cf - 1] + F.x[cf + 1];
              T ax = (T)F.cnt[cf] * F.x[cf] - nb;
              rs = rs + (F.b[cf] - ax);
            }
        }
        C.b[cc] = rs;
        C.bw[cc] = C.w[cc] * rs;
      }
    });
  }
  void mgProlong(const MgLevel& C, MgLevel& F) {
    int nf = F.NY, nc = C.NY;
    par(1, F.NX - 1, [&](int i) {
      for (int j = 1; j < F.NY - 1; ++j) {
        int cf = i * nf + j;
        if (!F.cnt[cf]) continue;
        int I = (i - 1) / 2 + 1, J = (j - 1) / 2 + 1;
        int di = ((i - 1) & 1) ? 1 : -1, dj = ((j - 1) & 1) ? 1 : -1;
        const int ci[4] = {I, I + di, I, I + di}, cj[4] = {J, J, J + dj, J + dj};
        const T wt[4] = {(T)9, (T)3, (T)3, (T)1};
        T num = 0, den = 0;
        for (int k = 0; k < 4; ++k) {
          int cc = ci[k] * nc + cj[k];
          if (!C.cnt[cc]) continue;
          num = num + wt[k] * C.x[cc];
          den = den + wt[k];
        }
        T e = den > 0 ? num / den : (T)0;
        F.x[cf] = F.x[cf] + e;
      }
    });
  }
  void mgCycle(int l, bool zero, T om1) {
    MgLevel& L = mg[l];
    if (l == (int)mg.size() - 1) {
      mgSmooth(L, kMgCoarse, true, om1);
      return;
    }
    mgSmooth(L, kMgPre, zero, om1);
    mgRestrict(L, mg[l + 1]);
    mgCycle(l + 1, true, om1);
    mgProlong(mg[l + 1], L);
    mgSmooth(L, kMgPost, false, om1);
  }
  void solveMg(int numCycles, T dt) {
    T om = (T)kMgOmega * PressureDamping;
    setupSystemOm(om);
    mgBuild(om);
    for (int k = 0; k < numCycles; ++k) mgCycle(0, k == 0, (T)1 - om);
    phi = mg[0].x;
    st.sweeps = numCycles;
    st.last_maxdiv = 0;
    residualFP64();
    gradientAndPressure(dt);
  }

  void solveParallel(int numIters, T dt) {
    if (scheme == MgJacobi) {
      solveMg(numIters, dt);
      return;
    }
    T cp = density * h / dt;
    (void)cp;
    setupSystem();
    st.sweeps = relax(rhs, BWc, phi, phi2, numIters, true);
    residualFP64();
    if (refine_sweeps > 0) {
      // Outer correction: FP64 residual of the FP32 iterate, a correction
      // solve A e = r by the same relaxation, then phi += e.
      std::vector<T> r(N, 0);
      BWe.assign(N, 0);
      for (int c = 0; c < N; ++c)
        if (cnt[c]) {
          r[c] = (T)resid64_[c];
          BWe[c] = Wc[c] * r[c];
        }
      err.assign(N, 0); err2.assign(N, 0);
      T keep = st.last_maxdiv;
      relax(r, BWe, err, err2, refine_sweeps, false);
      st.last_maxdiv = keep;
      for (int c = 0; c < N; ++c)
        if (cnt[c]) phi[c] = phi[c] + err[c];
      // Statistics: the residual of the final potential.
      residualFP64();
    }
    gradientAndPressure(dt);
  }
  // Gradient subtract + pressure from the potential phi.
  void gradientAndPressure(T dt) {
    int n = NY;
    T cp = density * h / dt;
    par(1, NX, [&](int i) {
      for (int j = 1; j < NY - 1; ++j) {
        int c = i * n + j;
        int cl = c - n;
        if (cnt[cl] || (i < NX - 1 && cnt[c])) {
          T d = S[c] * phi[cl] - S[cl] * phi[c];
          U[c] = U[c] + d;
        }
      }
    });
    par(1, NX - 1, [&](int i) {
      for (int j = 1; j < NY; ++j) {
        int c = i * n + j;
        int cb = c - 1;
        if (cnt[cb] || (j < NY - 1 && cnt[c])) {
          T d = S[c] * phi[cb] - S[cb] * phi[c];
          V[c] = V[c] + d;
        }
      }
    });
    for (int c = 0; c < N; ++c) p[c] = cnt[c] ? cp * phi[c] : (T)0;
  }
  std::vector<double> resid64_;
  // Knuth's TwoSum: s + e == a + b exactly.
  static void twoSum(float a, float b, float& s, float& e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
  }
  // Residual b + (pw + pe + ps + pn) - s*x of float inputs as a normalised
  // float pair: the product split exactly by fma, the terms summed by a
  // TwoSum cascade (the GPU scheme's residual, bit for bit).
  static void residFF(float b, float pw, float pe, float ps, float pn, float s, float x,
                      float& rhi, float& rlo) {
    float p = s * x;
    float pl = std::fma(s, x, -p);
    float hi = b, lo = 0.0f, t, e;
    twoSum(hi, pw, t, e); hi = t; lo = lo + e;
    twoSum(hi, pe, t, e); hi = t; lo = lo + e;
    twoSum(hi, ps, t, e); hi = t; lo = lo + e;
    twoSum(hi, pn, t, e); hi = t; lo = lo + e;
    twoSum(hi, -p, t, e); hi = t; lo = lo + e;
    lo = lo - pl;
    twoSum(hi, lo, rhi, rlo);
  }
  // Residual r = b - A phi of the current iterate in ~FP64 accuracy: float
  // pairs per cell for the FP32 oracle, doubles for the FP64 one; its
  // L2 norm and max accumulate in double.
  void residualFP64() {
    int n = NY;
    resid64_.assign(N, 0.0);
    double l2 = 0, mx = 0;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        int c = i * n + j;
        if (!cnt[c]) continue;
        double r, a;
        if constexpr (std::is_same<T, float>::value) {
          float hi, lo;
          residFF(rhs[c], phi[c - n], phi[c + n], phi[c - 1], phi[c + 1], (float)cnt[c], phi[c],
                  hi, lo);
          r = (double)hi + (double)lo;
          a = std::fabs((double)hi);
        } else {
          double nb = (double)phi[c - n] + (double)phi[c + n] + (double)phi[c - 1] +
                      (double)phi[c + 1];
          r = ((double)rhs[c] + nb) - (double)cnt[c] * (double)phi[c];
          a = std::fabs(r);
        }
        resid64_[c] = r;
        l2 += r * r;
        if (a > mx) mx = a;
      }
    st.resid_l2 = std::sqrt(l2);
    st.resid_max = mx;
  }
  void postProjectionStats() {
    int n = NY;
    double l2 = 0, mx = 0, cntc = 0;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        int c = i * n + j;
        if (S[c] == 0) continue;
        T div = U[c + n] - U[c] + V[c + 1] - V[c];
        double d = (double)div;
        l2 += d * d;
        if (std::fabs(d) > mx) mx = std::fabs(d);
        cntc += 1;
      }
    st.div_l2_post = std::sqrt(l2);
    st.div_max_post = mx;
    st.div_count_post = cntc;
  }
  double smokeMass() const {
    double m = 0;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) m += (double)M[i * NY + j];
    return m;
  }

  // fluid.go:236-289
  void handleBorders() {
    int n = NY;
    par(0, NX, [&](int i) {
      if (S[i * n + 0] == 0 || S[i * n + 1] == 0) {
        U[i * n + 0] = 0;
      } else {
        if (i > 0 && i < NX - 1 && S[i * n + 2] > 0)
          U[i * n + 0] = (T)2 * U[i * n + 1] - U[i * n + 2];
        else
          U[i * n + 0] = U[i * n + 1];
      }
      if (S[i * n + NY - 1] == 0 || S[i * n + NY - 2] == 0) {
        U[i * n + NY - 1] = 0;
      } else {
        if (i > 0 && i < NX - 1 && S[i * n + NY - 3] > 0)
          U[i * n + NY - 1] = (T)2 * U[i * n + NY - 2] - U[i * n + NY - 3];
        else
          U[i * n + NY - 1] = U[i * n + NY - 2];
      }
    });
    par(0, NY, [&](int j) {
      if (S[0 * n + j] == 0 || S[1 * n + j] == 0) {
        V[0 * n + j] = 0;
      } else {
        if (j > 0 && j < NY - 1 && S[2 * n + j] > 0)
          V[0 * n + j] = (T)2 * V[1 * n + j] - V[2 * n + j];
        else
          V[0 * n + j] = V[1 * n + j];
      }
      if (S[(NX - 1) * n + j] == 0 || S[(NX - 2) * n + j] == 0) {
        V[(NX - 1) * n + j] = 0;
      } else {
        if (j > 0 && j < NY - 1 && S[(NX - 3) * n + j] > 0)
          V[(NX - 1) * n + j] = (T)2 * V[(NX - 2) * n + j] - V[(NX - 3) * n + j];
        else
          V[(NX - 1) * n + j] = V[(NX - 2) * n + j];
      }
    });
  }

  // fluid.go:436-446
  void copyBorder(std::vector<T>& dst, const std::vector<T>& src) {
    int n = NY;
    for (int i = 0; i < NX; ++i) {
      dst[i * n + 0] = src[i * n + 0];
      dst[i * n + NY - 1] = src[i * n + NY - 1];
    }
    for (int j = 0; j < NY; ++j) {
      dst[0 * n + j] = src[0 * n + j];
      dst[(NX - 1) * n + j] = src[(NX - 1) * n + j];
    }
  }

  // fluid.go:335-347
  inline T avgU(const std::vector<T>& Uf, int i, int j) const {
    int n = NY;
    return (Uf[i * n + j - 1] + Uf[i * n + j] + Uf[(i + 1) * n + j - 1] + Uf[(i + 1) * n + j]) *
           (T)0.25;
  }
  inline T avgV(const std::vector<T>& Vf, int i, int j) const {
    int n = NY;
    return (Vf[(i - 1) * n + j] + Vf[i * n + j] + Vf[(i - 1) * n + j + 1] + Vf[i * n + j + 1]) *
           (T)0.25;
  }

  // fluid.go:357-398 and fluid.go:1055-1091; fld: 0 = U, 1 = V, 2 = M
  T sampleFrom(T x, T y, const std::vector<T>& data, int fld) const {
    int n = NY;
    T h1 = (T)1.0 / h;
    T h2 = (T)0.5 * h;
    // fmin/fmax equal Go's min/max for every non-NaN coordinate here (the
    // bounds are positive); a NaN coordinate, which makes the reference
    // panic on its index, clamps to the upper bound as on the GPU.
    x = std::fmax(std::fmin(x, (T)NX * h), h);
    y = std::fmax(std::fmin(y, (T)NY * h), h);
    T dx = 0, dy = 0;
    if (fld == 0) dy = h2;
    else if (fld == 1) dx = h2;
    else { dx = h2; dy = h2; }
    int x0 = std::min((int)std::floor((double)((x - dx) * h1)), NX - 1);
    T tx = ((x - dx) - (T)x0 * h) * h1;
    int x1 = std::min(x0 + 1, NX - 1);
    int y0 = std::min((int)std::floor((double)((y - dy) * h1)), NY - 1);
    T ty = ((y - dy) - (T)y0 * h) * h1;
    int y1 = std::min(y0 + 1, NY - 1);
    T sx = (T)1.0 - tx;
    T sy = (T)1.0 - ty;
    return sx * sy * data[x0 * n + y0] + tx * sy * data[x1 * n + y0] +
           tx * ty * data[x1 * n + y1] + sx * ty * data[x0 * n + y1];
  }

  // Sample at the departure point of face / cell (i, j) moved by (-su, -sv)
  // (su, sv: the products dt * u, dt * v; fld as sampleFrom, whose
  // staggering is also the face's offset in the cell).  Without
  // precise_coords the point is formed in absolute coordinates exactly as
  // the reference forms it (fluid.go:304-330, 411-414, 940-960); with it,
  // as index plus offset in cells, (i + a, j + b), a = -su / h: the floor
  // and the weights are taken from the small offset, exact to the float
  // precision of the displacement.
  T sampleDep(int i, int j, T su, T sv, const std::vector<T>& data, int fld) const {
    const bool hx = fld != 0, hy = fld != 1;
    const T h2 = h / (T)2;
    if (!precise_coords) {
      T x = hx ? ((T)i * h + h2) - su : (T)i * h - su;
      T y = hy ? ((T)j * h + h2) - sv : (T)j * h - sv;
      return sampleFrom(x, y, data, fld);
    }
    const int n = NY;
    const T h1 = (T)1.0 / h;
    const T dxr = hx ? (T)0.5 : (T)0, dyr = hy ? (T)0.5 : (T)0;
    T a = -su * h1, b = -sv * h1;
    a = std::fmax(std::fmin(a, (T)(NX - i) - dxr), (T)(1 - i) - dxr);
    b = std::fmax(std::fmin(b, (T)(NY - j) - dyr), (T)(1 - j) - dyr);
    T fa = std::floor(a), fb = std::floor(b);
    int x0 = i + (int)fa, y0 = j + (int)fb;
    T tx = a - fa, ty = b - fb;
    if (x0 > NX - 1) {
      x0 = NX - 1;
      tx = a - (T)(x0 - i);
    }
    if (y0 > NY - 1) {
      y0 = NY - 1;
      ty = b - (T)(y0 - j);
    }
    int x1 = std::min(x0 + 1, NX - 1), y1 = std::min(y0 + 1, NY - 1);
    T sx = (T)1.0 - tx;
    T sy = (T)1.0 - ty;
    return sx * sy * data[x0 * n + y0] + tx * sy * data[x1 * n + y0] +
           tx * ty * data[x1 * n + y1] + sx * ty * data[x0 * n + y1];
  }

  // fluid.go:291-333
  void advectVelocity(T dt) {
    copyBorder(newU, U);
    copyBorder(newV, V);
    int n = NY;
    T hh = h;
    T h2 = hh / (T)2;
    par(1, NX, [&](int i) {
      for (int j = 1; j < NY; ++j) {
        if (S[i * n + j] != 0 && S[(i - 1) * n + j] != 0 && j < NY - 1) {
          T u = U[i * n + j];
          T v = avgV(V, i, j);
          newU[i * n + j] = sampleDep(i, j, dt * u, dt * v, U, 0);
        }
        if (S[i * n + j] != 0 && S[i * n + j - 1] != 0 && i < NX - 1) {
          T u = avgU(U, i, j);
          T v = V[i * n + j];
          newV[i * n + j] = sampleDep(i, j, dt * u, dt * v, V, 1);
        }
      }
    });
    U = newU;
    V = newV;
  }

  // fluid.go:400-434
  void advectSmoke(T dt) {
    copyBorder(newM, M);
    int n = NY;
    T hh = h;
    T h2 = (T)0.5 * hh;
    par(1, NX - 1, [&](int i) {
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] != 0) {
          T u = (U[i * n + j] + U[(i + 1) * n + j]) * (T)0.5 * SmokeAdvection;
          T v = (V[i * n + j] + V[i * n + j + 1]) * (T)0.5 * SmokeAdvection;
          T smokeValue = sampleDep(i, j, dt * u, dt * v, M, 2);
          if (ViscosityDiffusion > 0) {
            T smokeDiffusion = ViscosityDiffusion * (T)0.3 * dt;
            T neighbors = M[(i - 1) * n + j] + M[(i + 1) * n + j] + M[i * n + j - 1] +
                          M[i * n + j + 1] - (T)4 * M[i * n + j];
            smokeValue += smokeDiffusion * neighbors;
          }
          newM[i * n + j] = go_max(smokeValue, (T)0.0);
        }
      }
    });
    M = newM;
  }

  // fluid.go:449-493 (two serial passes; curl is a fresh zeroed array)
  void applyVorticityConfinement(T dt) {
    int n = NY;
    T hh = h;
    std::vector<T> curl(N, 0);
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T dvdx = (V[(i + 1) * n + j] - V[(i - 1) * n + j]) * (T)0.5 / hh;
        T dudy = (U[i * n + j + 1] - U[i * n + j - 1]) * (T)0.5 / hh;
        curl[i * n + j] = dvdx - dudy;
      }
    T eps = (T)1e-5;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T gx = (go_abs(curl[(i + 1) * n + j]) - go_abs(curl[(i - 1) * n + j])) * (T)0.5 / hh;
        T gy = (go_abs(curl[i * n + j + 1]) - go_abs(curl[i * n + j - 1])) * (T)0.5 / hh;
        T mag = go_sqrt(gx * gx + gy * gy) + eps;
        gx /= mag;
        gy /= mag;
        T vort = curl[i * n + j];
        T localVel = go_sqrt(U[i * n + j] * U[i * n + j] + V[i * n + j] * V[i * n + j]);
        T adaptiveStrength = Confinement * ((T)1.0 + localVel * (T)0.1);
        U[i * n + j] += adaptiveStrength * gy * vort * dt;
        V[i * n + j] -= adaptiveStrength * gx * vort * dt;
      }
  }

  // fluid.go:496-526
  void addTurbulence(T dt) {
    if (TurbulenceStrength <= 0) return;
    int n = NY;
    T turbStrength = TurbulenceStrength * dt;
    par(1, NX - 1, [&](int i) {
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] > 0) {
          T seedU = (T)(i * 137 + j * 241) * (T)0.01;
          T seedV = (T)(i * 157 + j * 263) * (T)0.01;
          T noiseU = (T)std::sin((double)seedU) * turbStrength;
          T noiseV = (T)std::sin((double)seedV) * turbStrength;
          T localVel = go_sqrt(U[i * n + j] * U[i * n + j] + V[i * n + j] * V[i * n + j]);
          if (localVel > (T)0.1) {
            T turbulenceFactor = go_min(localVel * (T)0.5, (T)1.0);
            U[i * n + j] += noiseU * turbulenceFactor;
            V[i * n + j] += noiseV * turbulenceFactor;
          }
        }
      }
    });
  }

  // fluid.go:529-557
  T getAdaptiveTimeStep(T basedt) const {
    T maxVel = 0;
    int n = NY;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j)
        if (S[i * n + j] > 0) {
          T vel = go_abs(U[i * n + j]) + go_abs(V[i * n + j]);
          if (vel > maxVel) maxVel = vel;
        }
    if (maxVel == 0) return basedt;
    T cflFactor = (T)0.8;
    T adaptivedt = cflFactor * h / maxVel;
    adaptivedt = go_max(go_min(adaptivedt, basedt * (T)2.0), basedt * (T)0.1);
    return adaptivedt;
  }

  // ------------------------------------------------ multigrid (fluid.go:559-758, 1122-1149)
  void solveMultigridVCycle(int numIters, T dt) {
    T cp = density * h / dt;
    T tol = tolerance;
    st.sweeps = 0;
    for (int iter = 0; iter < numIters; ++iter) {
      T maxDiv = 0;
      for (int sm = 0; sm < 3; ++sm) maxDiv = pressureJacobiIteration((T)1.5, cp);
      st.sweeps += 3;
      if (maxDiv < tol) break;
      std::vector<T> residual = computePressureResidual();
      std::vector<T> coarseRHS = restrictResidual(residual);
      std::vector<T> coarse = solveCoarseGrid(coarseRHS);
      std::vector<T> corr = prolongateCorrection(coarse);
      applyPressureCorrection(corr, cp);
      for (int sm = 0; sm < 3; ++sm) pressureJacobiIteration((T)1.2, cp);
      st.sweeps += 3;
    }
  }
  std::vector<T> computePressureResidual() {
    int n = NY;
    std::vector<T> r(N, 0);
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T div = U[(i + 1) * n + j] - U[i * n + j] + V[i * n + j + 1] - V[i * n + j];
        T sx0 = S[(i - 1) * n + j], sx1 = S[(i + 1) * n + j];
        T sy0 = S[i * n + j - 1], sy1 = S[i * n + j + 1];
        T lap = sx0 * (p[(i - 1) * n + j] - p[i * n + j]) +
                sx1 * (p[(i + 1) * n + j] - p[i * n + j]) +
                sy0 * (p[i * n + j - 1] - p[i * n + j]) +
                sy1 * (p[i * n + j + 1] - p[i * n + j]);
        r[i * n + j] = -div - lap;
      }
    return r;
  }
  std::vector<T> restrictResidual(const std::vector<T>& fr) {
    int cNX = (NX + 1) / 2, cNY = (NY + 1) / 2;
    std::vector<T> c(cNX * cNY, 0);
    for (int i = 1; i < cNX - 1; ++i)
      for (int j = 1; j < cNY - 1; ++j) {
        int fi = i * 2, fj = j * 2;
        if (fi < NX - 1 && fj < NY - 1) {
          T center = fr[fi * NY + fj] * (T)0.25;
          T nbr = (fr[(fi - 1) * NY + fj] + fr[(fi + 1) * NY + fj] + fr[fi * NY + fj - 1] +
                   fr[fi * NY + fj + 1]) * (T)0.125;
          T crn = (fr[(fi - 1) * NY + fj - 1] + fr[(fi + 1) * NY + fj - 1] +
                   fr[(fi - 1) * NY + fj + 1] + fr[(fi + 1) * NY + fj + 1]) * (T)0.0625;
          c[i * cNY + j] = center + nbr + crn;
        }
      }
    return c;
  }
  std::vector<T> solveCoarseGrid(const std::vector<T>& rhsc) {
    int cNX = (NX + 1) / 2, cNY = (NY + 1) / 2;
    std::vector<T> cP(cNX * cNY, 0), cS(cNX * cNY, 0);
    for (int i = 0; i < cNX; ++i)
      for (int j = 0; j < cNY; ++j) {
        int fi = i * 2, fj = j * 2;
        cS[i * cNY + j] = (fi < NX && fj < NY) ? S[fi * NY + fj] : (T)0;
      }
    T relaxation = (T)1.6;
    for (int it = 0; it < 40; ++it)
      for (int i = 1; i < cNX - 1; ++i)
        for (int j = 1; j < cNY - 1; ++j) {
          if (cS[i * cNY + j] == 0) continue;
          T sx0 = cS[(i - 1) * cNY + j], sx1 = cS[(i + 1) * cNY + j];
          T sy0 = cS[i * cNY + j - 1], sy1 = cS[i * cNY + j + 1];
          T s = sx0 + sx1 + sy0 + sy1;
          if (s == 0) continue;
          T lap = sx0 * (cP[(i - 1) * cNY + j] - cP[i * cNY + j]) +
                  sx1 * (cP[(i + 1) * cNY + j] - cP[i * cNY + j]) +
                  sy0 * (cP[i * cNY + j - 1] - cP[i * cNY + j]) +
                  sy1 * (cP[i * cNY + j + 1] - cP[i * cNY + j]);
          T residual = rhsc[i * cNY + j] - lap;
          T correction = -residual / s * relaxation;
          cP[i * cNY + j] += correction;
        }
    return cP;
  }
  std::vector<T> prolongateCorrection(const std::vector<T>& cc) {
    std::vector<T> corr(N, 0);
    int cNY = (NY + 1) / 2, cNX = (NX + 1) / 2;
    for (int i = 0; i < NX; ++i)
      for (int j = 0; j < NY; ++j) {
        int ci = i / 2, cj = j / 2;
        if (ci >= cNX - 1 || cj >= cNY - 1) continue;
        T fI = (T)(i % 2) * (T)0.5, fJ = (T)(j % 2) * (T)0.5;
        corr[i * NY + j] = ((T)1 - fI) * ((T)1 - fJ) * cc[ci * cNY + cj] +
                           fI * ((T)1 - fJ) * cc[(ci + 1) * cNY + cj] +
                           ((T)1 - fI) * fJ * cc[ci * cNY + cj + 1] +
                           fI * fJ * cc[(ci + 1) * cNY + cj + 1];
      }
    return corr;
  }
  void applyPressureCorrection(const std::vector<T>& corr, T cp) {
    int n = NY;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        p[i * n + j] += corr[i * n + j] * cp;
        T sx0 = S[(i - 1) * n + j], sx1 = S[(i + 1) * n + j];
        T sy0 = S[i * n + j - 1], sy1 = S[i * n + j + 1];
        T pc = corr[i * n + j];
        U[i * n + j] -= sx0 * pc;
        U[(i + 1) * n + j] += sx1 * pc;
        V[i * n + j] -= sy0 * pc;
        V[i * n + j + 1] += sy1 * pc;
      }
  }

  // ------------------------------------------------ tools (walls.go, fluid.go:760-907)
  // Return 0 on success, -1 on an index the reference would panic on.
  int setSolid(int i, int j, bool value) {
    if (i < 0 || i >= NX || j < 0 || j >= NY) return -1;
    int cell = i * NY + j;
    S[cell] = value ? (T)0 : (T)1;
    if (value) {
      int n = NY;
      U[i * n + j] = 0;
      if (i + 1 < NX) U[(i + 1) * n + j] = 0;
      V[i * n + j] = 0;
      if (j + 1 < NY) V[i * n + j + 1] = 0;
      newU[i * n + j] = 0;
      if (i + 1 < NX) newU[(i + 1) * n + j] = 0;
      newV[i * n + j] = 0;
      if (j + 1 < NY) newV[i * n + j + 1] = 0;
    }
    return 0;
  }
  int isSolid(int i, int j) const {
    if (i < 0 || i >= NX || j < 0 || j >= NY) return -1;
    return S[i * NY + j] == 0 ? 1 : 0;
  }
  int setVelocity(int i, int j, T u, T v) {
    if (i < 0 || i >= NX || j < 0 || j >= NY) return -1;
    U[i * NY + j] = u;
    V[i * NY + j] = v;
    return 0;
  }
  int addSmoke(int i, int j, T s) {
    if (i < 0 || i >= NX || j < 0 || j >= NY) return -1;
    M[i * NY + j] += s;
    return 0;
  }
  void reset() {
    std::fill(U.begin(), U.end(), (T)0); std::fill(V.begin(), V.end(), (T)0);
    std::fill(newU.begin(), newU.end(), (T)0); std::fill(newV.begin(), newV.end(), (T)0);
    std::fill(p.begin(), p.end(), (T)0); std::fill(M.begin(), M.end(), (T)0);
    std::fill(newM.begin(), newM.end(), (T)0);
  }
  void applyForce(int i, int j, T fx, T fy) {
    if (i < 1 || i >= NX - 1 || j < 1 || j >= NY - 1) return;
    if (S[i * NY + j] == 0) return;
    U[i * NY + j] += fx;
    V[i * NY + j] += fy;
  }
  void applyForceRadius(int cx, int cy, T fx, T fy, int radius) {
    if (radius <= 0) { applyForce(cx, cy, fx, fy); return; }
    T r2 = (T)(radius * radius);
    for (int i = cx - radius; i <= cx + radius; ++i)
      for (int j = cy - radius; j <= cy + radius; ++j) {
        if (i < 1 || i >= NX - 1 || j < 1 || j >= NY - 1) continue;
        T dx = (T)(i - cx), dy = (T)(j - cy);
        T dist2 = dx * dx + dy * dy;
        if (dist2 > r2) continue;
        T weight = (T)std::exp((double)((T)-3.0 * dist2 / r2));
        applyForce(i, j, fx * weight, fy * weight);
      }
  }
  void setCircularObstacle(int cx, int cy, int radius) {
    for (int i = cx - radius; i <= cx + radius; ++i)
      for (int j = cy - radius; j <= cy + radius; ++j) {
        if (i < 0 || i >= NX || j < 0 || j >= NY) continue;
        T dx = (T)(i - cx), dy = (T)(j - cy);
        if (dx * dx + dy * dy <= (T)(radius * radius)) setSolid(i, j, true);
      }
  }

  // ------------------------------------------------ views (fluid.go:798-891)
  T maxDivergence() const {
    int n = NY;
    T maxDiv = 0;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T div = U[(i + 1) * n + j] - U[i * n + j] + V[i * n + j + 1] - V[i * n + j];
        T a = go_abs(div);
        if (a > maxDiv) maxDiv = a;
      }
    return maxDiv;
  }
  void vorticity(T* out, T* mn, T* mx) const {
    int n = NY;
    T minVal = std::numeric_limits<T>::max(), maxVal = -(std::numeric_limits<T>::max() - 1);
    std::fill(out, out + N, (T)0);
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T dvdx = (V[(i + 1) * n + j] - V[(i - 1) * n + j]) * (T)0.5 / h;
        T dudy = (U[i * n + j + 1] - U[i * n + j - 1]) * (T)0.5 / h;
        T c = dvdx - dudy;
        out[i * n + j] = c;
        if (c < minVal) minVal = c;
        if (c > maxVal) maxVal = c;
      }
    *mn = minVal;
    *mx = maxVal;
  }
  void velocityMagnitude(T* out, T* mn, T* mx) const {
    int n = NY;
    T minVal = std::numeric_limits<T>::max(), maxVal = -(std::numeric_limits<T>::max() - 1);
    std::fill(out, out + N, (T)0);
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] == 0) continue;
        T u = (U[i * n + j] + U[(i + 1) * n + j]) * (T)0.5;
        T v = (V[i * n + j] + V[i * n + j + 1]) * (T)0.5;
        T mag = go_sqrt(u * u + v * v);
        out[i * n + j] = mag;
        if (mag < minVal) minVal = mag;
        if (mag > maxVal) maxVal = mag;
      }
    *mn = minVal;
    *mx = maxVal;
  }

  // ------------------------------------------------ BFECC (fluid.go:909-1120)
  T clampToNeighbors(T val, const std::vector<T>& src, int i, int j) const {
    int n = NY;
    T lo = src[i * n + j], hi = src[i * n + j];
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj) {
        int ni = i + di, nj = j + dj;
        if (ni >= 0 && ni < NX && nj >= 0 && nj < NY) {
          T v = src[ni * n + nj];
          if (v < lo) lo = v;
          if (v > hi) hi = v;
        }
      }
    if (val < lo) return lo;
    if (val > hi) return hi;
    return val;
  }
  // keep (optional): receives fwdU, fwdV, corrU, corrV for the adjoint.
  void advectVelocityBFECC(T dt, std::vector<T>* keep = nullptr) {
    int n = NY;
    T hh = h, h2 = hh / (T)2;
    std::vector<T> origU = U, origV = V;
    advectVelocity(dt);
    std::vector<T> fwdU = U, fwdV = V;
    U = origU;
    V = origV;
    std::vector<T> bwdU(N, 0), bwdV(N, 0);
    copyBorder(bwdU, fwdU);
    copyBorder(bwdV, fwdV);
    par(1, NX, [&](int i) {
      for (int j = 1; j < NY; ++j) {
        if (S[i * n + j] != 0 && S[(i - 1) * n + j] != 0 && j < NY - 1) {
          T u = U[i * n + j], v = avgV(V, i, j);
          bwdU[i * n + j] = sampleDep(i, j, -dt * u, -dt * v, fwdU, 0);
        }
        if (S[i * n + j] != 0 && S[i * n + j - 1] != 0 && i < NX - 1) {
          T u = avgU(U, i, j), v = V[i * n + j];
          bwdV[i * n + j] = sampleDep(i, j, -dt * u, -dt * v, fwdV, 1);
        }
      }
    });
    std::vector<T> corrU = origU, corrV = origV;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        corrU[i * n + j] = origU[i * n + j] - (bwdU[i * n + j] - origU[i * n + j]) * (T)0.5;
        corrV[i * n + j] = origV[i * n + j] - (bwdV[i * n + j] - origV[i * n + j]) * (T)0.5;
      }
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        corrU[i * n + j] = clampToNeighbors(corrU[i * n + j], origU, i, j);
        corrV[i * n + j] = clampToNeighbors(corrV[i * n + j], origV, i, j);
      }
    if (keep) {
      keep[0] = fwdU;
      keep[1] = fwdV;
      keep[2] = corrU;
      keep[3] = corrV;
    }
    U = corrU;
    V = corrV;
    advectVelocity(dt);
  }
  // keep (optional): receives fwdM, corrM for the adjoint.
  void advectSmokeBFECC(T dt, std::vector<T>* keep = nullptr) {
    int n = NY;
    T hh = h, h2 = (T)0.5 * hh;
    std::vector<T> origM = M;
    advectSmoke(dt);
    std::vector<T> fwdM = M;
    std::vector<T> bwdM(N, 0);
    copyBorder(bwdM, fwdM);
    par(1, NX - 1, [&](int i) {
      for (int j = 1; j < NY - 1; ++j) {
        if (S[i * n + j] != 0) {
          T u = (U[i * n + j] + U[(i + 1) * n + j]) * (T)0.5 * SmokeAdvection;
          T v = (V[i * n + j] + V[i * n + j + 1]) * (T)0.5 * SmokeAdvection;
          bwdM[i * n + j] = sampleDep(i, j, -dt * u, -dt * v, fwdM, 2);
        }
      }
    });
    std::vector<T> corrM = origM;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j)
        corrM[i * n + j] = origM[i * n + j] - (bwdM[i * n + j] - origM[i * n + j]) * (T)0.5;
    for (int i = 1; i < NX - 1; ++i)
      for (int j = 1; j < NY - 1; ++j) {
        corrM[i * n + j] = clampToNeighbors(corrM[i * n + j], origM, i, j);
        if (corrM[i * n + j] < 0) corrM[i * n + j] = 0;
      }
    if (keep) {
      keep[0] = fwdM;
      keep[1] = corrM;
    }
    M = corrM;
    advectSmoke(dt);
  }
};

}  // namespace orc

// ===========================================================================
// App-side loops that read the simulation every frame: tracer particles
// (main/main.go:512-546 advectParticles) and the field rendering
// (main/main.go:619-650 drawScalarField / drawVorticityField with
// main/colors.go:10-84).
// ===========================================================================
namespace orc {

// advectParticles: ages, culls, RK2-advects and bounds-checks the particles
// in place, keeping the survivors in order; returns their number.
template <typename T>
int advect_particles(const Fluid<T>& f, int n, T* X, T* Y, T* Age, T* MaxAge, uint32_t* RGB,
                     T dt) {
  const T h = f.h;
  int w = 0;
  for (int k = 0; k < n; ++k) {
    T age = Age[k] + dt;
    if (age > MaxAge[k]) continue;
    T x = X[k], y = Y[k];
    T u1 = f.sampleFrom(x, y, f.U, 0), v1 = f.sampleFrom(x, y, f.V, 1);
    T midX = x + (T)0.5 * dt * u1;
    T midY = y + (T)0.5 * dt * v1;
    T u2 = f.sampleFrom(midX, midY, f.U, 0), v2 = f.sampleFrom(midX, midY, f.V, 1);
    x += dt * u2;
    y += dt * v2;
    T qi = x / h, qj = y / h;
    if (!(qi > (T)-2147483648.0 && qi < (T)2147483648.0 && qj > (T)-2147483648.0 &&
          qj < (T)2147483648.0))
      continue;
    int fi = (int)qi, fj = (int)qj;
    if (fi < 0 || fi >= f.NX || fj < 0 || fj >= f.NY) continue;
    if (f.S[fi * f.NY + fj] == 0) continue;
    X[w] = x;
    Y[w] = y;
    Age[w] = age;
    MaxAge[w] = MaxAge[k];
    RGB[w] = RGB[k];
    ++w;
  }
  return w;
}

template <typename T>
void rgba_store(uint8_t* px, T r, T g, T b) {
  px[0] = (uint8_t)(T)(255 * r);
  px[1] = (uint8_t)(T)(255 * g);
  px[2] = (uint8_t)(T)(255 * b);
  px[3] = 0xff;
}

// getSciValue (main/colors.go:47-84)
template <typename T>
void sci_value(T val, T mn, T mx, uint8_t* px) {
  val = go_min(go_max(val, mn), mx - (T)0.0001);
  T d = mx - mn;
  if (d <= 0)
    val = (T)0.5;
  else
    val = (val - mn) / d;
  T m = (T)0.25;
  T num = (T)std::floor((double)(val / m));
  T s = (val - num * m) / m;
  T r = 0, g = 0, b = 0;
  if (num == 0) {
    g = s;
    b = 1;
  } else if (num == 1) {
    g = 1;
    b = 1 - s;
  } else if (num == 2) {
    r = s;
    g = 1;
  } else if (num == 3) {
    r = 1;
    g = 1 - s;
  }
  rgba_store(px, r, g, b);
}

// getDivergingColor (main/colors.go:10-44)
template <typename T>
void diverging_color(T val, T mn, T mx, uint8_t* px) {
  T absMax = (T)std::max(std::fabs((double)mn), std::fabs((double)mx));
  if (absMax < (T)1e-8) {
    px[0] = px[1] = px[2] = px[3] = 255;
    return;
  }
  T t = val / absMax;
  if (t > 1) t = 1;
  if (t < -1) t = -1;
  T r, g, b;
  if (t >= 0) {
    r = 1;
    g = 1 - t;
    b = 1 - t;
  } else {
    T a = -t;
    r = 1 - a;
    g = 1 - a;
    b = 1;
  }
  rgba_store(px, r, g, b);
}

// kind: 0 smoke, 1 pressure, 2 speed, 3 vorticity.  out: NX x NY RGBA8,
// pixel (i, j) showing cell (i, NY - 1 - j).
template <typename T>
void render(const Fluid<T>& f, int kind, uint8_t* out) {
  std::vector<T> vals(f.N);
  T mn = std::numeric_limits<T>::max(), mx = -(std::numeric_limits<T>::max() - 1);
  if (kind == 0 || kind == 1) {
    const std::vector<T>& F = kind == 0 ? f.M : f.p;
    for (int c = 0; c < f.N; ++c) {
      vals[c] = F[c];
      if (F[c] < mn) mn = F[c];
      if (F[c] > mx) mx = F[c];
    }
  } else if (kind == 2) {
    f.velocityMagnitude(vals.data(), &mn, &mx);
  } else {
    f.vorticity(vals.data(), &mn, &mx);
  }
  for (int i = 0; i < f.NX; ++i)
    for (int j = 0; j < f.NY; ++j) {
      T v = vals[i * f.NY + (f.NY - j - 1)];
      uint8_t* px = out + 4 * ((size_t)j * f.NX + i);
      if (kind == 3)
        diverging_color(v, mn, mx, px);
      else
        sci_value(v, mn, mx, px);
    }
}

}  // namespace orc

// ===========================================================================
// Reverse mode of a recorded rollout: the FP64 reference for the CUDA
// adjoint (test infrastructure; the reference has no derivatives).  A step
// is Simulate (fluid.go:79-109) with the parallel Jacobi scheme and a fixed
// sweep count, a force field added to U, V before the sources, and the
// sources of the rollout (the app's per-step SetVelocity / smoke calls).
// Every step's intermediates are kept (small grids only); the reverse pass
// runs the transposed stages sequentially, so it is deterministic.  The
// subgradient conventions are those of the CUDA adjoint: a clamped sample
// coordinate passes no position derivative, floor is locally constant, a
// clamped BFECC value takes the derivative of the first bounding neighbour
// in scan order, max(x, 0) passes for x >= 0, |x| passes sign(x) (0 at 0),
// the turbulence gate passes its term only for |u| > 0.1 and below the
// min(0.5|u|, 1) kink.
// ===========================================================================
namespace orc {

struct Source {
  int i, j;
  double u, v, smoke;
  int mode;  // bit 0 skip if solid, 1 set U V, 2 add smoke, 3 set smoke
};

template <typename T>
struct Rollout {
  Fluid<T>& f;
  std::vector<Source> src;
  struct Rec {
    std::vector<T> U2, V2, U4, V4, k[4], U5, V5, M1, km[2];
  };
  std::vector<Rec> recs;
  std::vector<T> dts;
  std::vector<T> aU, aV, aM, aNU, aNV, aNM;
  explicit Rollout(Fluid<T>& f_) : f(f_) {}

  int n() const { return f.NY; }
  bool ring(int i, int j) const { return i == 0 || j == 0 || i == f.NX - 1 || j == f.NY - 1; }
  bool uadv(int i, int j) const {
    return i >= 1 && j >= 1 && j <= f.NY - 2 && f.S[i * n() + j] != 0 && f.S[(i - 1) * n() + j] != 0;
  }
  bool vadv(int i, int j) const {
    return i >= 1 && i <= f.NX - 2 && j >= 1 && f.S[i * n() + j] != 0 && f.S[i * n() + j - 1] != 0;
  }
  bool fluid_interior(int i, int j) const {
    return i >= 1 && i <= f.NX - 2 && j >= 1 && j <= f.NY - 2 && f.S[i * n() + j] != 0;
  }

  void apply_sources() {
    for (const Source& s : src) {
      int c = s.i * n() + s.j;
      if ((s.mode & 1) && f.S[c] == 0) continue;
      if (s.mode & 2) {
        f.U[c] = (T)s.u;
        f.V[c] = (T)s.v;
      }
      if (s.mode & 8)
        f.M[c] = (T)s.smoke;
      else if (s.mode & 4)
        f.M[c] = f.M[c] + (T)s.smoke;
    }
  }

  void step(T dt, const T* fu, const T* fv) {
    Rec r;
    if (fu)
      for (int c = 0; c < f.N; ++c) {
        f.U[c] += fu[c];
        f.V[c] += fv[c];
      }
    apply_sources();
    std::fill(f.p.begin(), f.p.end(), (T)0);
    f.makeIncompressible(f.num_iters, dt);
    r.U2 = f.U;
    r.V2 = f.V;
    if (f.Confinement != 0) f.applyVorticityConfinement(dt);
    if (f.TurbulenceStrength > 0) f.addTurbulence(dt);
    f.handleBorders();
    r.U4 = f.U;
    r.V4 = f.V;
    if (f.UseBFECC)
      f.advectVelocityBFECC(dt, r.k);
    else
      f.advectVelocity(dt);
    r.U5 = f.U;
    r.V5 = f.V;
    r.M1 = f.M;
    if (f.UseBFECC)
      f.advectSmokeBFECC(dt, r.km);
    else
      f.advectSmoke(dt);
    recs.push_back(std::move(r));
    dts.push_back(dt);
  }

  // d sample / d (x, y) and the scatter of lam into dD (sampleFrom's
  // bilinear weights); fld as sampleFrom.
  void sample_adj(T x, T y, const std::vector<T>& D, std::vector<T>& dD, int fld, T lam, T* gx,
                  T* gy) const {
    const int NX = f.NX, NY = f.NY;
    const T h = f.h, h1 = (T)1.0 / h, h2 = (T)0.5 * h;
    T xc = std::fmax(std::fmin(x, (T)NX * h), h), yc = std::fmax(std::fmin(y, (T)NY * h), h);
    T dx = fld == 0 ? 0 : h2, dy = fld == 1 ? 0 : h2;
    int x0 = std::min((int)std::floor((double)((xc - dx) * h1)), NX - 1);
    T tx = ((xc - dx) - (T)x0 * h) * h1;
    int x1 = std::min(x0 + 1, NX - 1);
    int y0 = std::min((int)std::floor((double)((yc - dy) * h1)), NY - 1);
    T ty = ((yc - dy) - (T)y0 * h) * h1;
    int y1 = std::min(y0 + 1, NY - 1);
    T sx = 1 - tx, sy = 1 - ty;
    T f00 = D[x0 * NY + y0], f10 = D[x1 * NY + y0], f11 = D[x1 * NY + y1], f01 = D[x0 * NY + y1];
    dD[x0 * NY + y0] += sx * sy * lam;
    dD[x1 * NY + y0] += tx * sy * lam;
    dD[x1 * NY + y1] += tx * ty * lam;
    dD[x0 * NY + y1] += sx * ty * lam;
    *gx = xc == x ? h1 * (sy * (f10 - f00) + ty * (f11 - f01)) : (T)0;
    *gy = yc == y ? h1 * (sx * (f01 - f00) + tx * (f11 - f10)) : (T)0;
  }

  // Adjoint of advectVelocity with trace field = sampled field = border
  // field (Ut, Vt) traced at sdt (-dt: BFECC's reverse sample, whose faces
  // that are not advected are constant 0: dR = dN = null).
  void sl_vel_adj(const std::vector<T>& lu, const std::vector<T>& lv, const std::vector<T>& Ut,
                  const std::vector<T>& Vt, const std::vector<T>& Fu, const std::vector<T>& Fv,
                  std::vector<T>& dUt, std::vector<T>& dVt, std::vector<T>& dFu,
                  std::vector<T>& dFv, std::vector<T>* dRu, std::vector<T>* dRv,
                  std::vector<T>* dNu, std::vector<T>* dNv, T sdt) const {
    const int nn = n();
    const T h = f.h, h2 = h / (T)2;
    for (int i = 0; i < f.NX; ++i)
      for (int j = 0; j < f.NY; ++j) {
        int c = i * nn + j;
        if (uadv(i, j)) {
          T x = (T)i * h - sdt * Ut[c];
          T y = (T)j * h + h2 - sdt * f.avgV(Vt, i, j);
          T gx, gy;
          sample_adj(x, y, Fu, dFu, 0, lu[c], &gx, &gy);
          dUt[c] += -sdt * gx * lu[c];
          T q = (T)0.25 * (-sdt * gy * lu[c]);
          dVt[c - nn] += q;
          dVt[c] += q;
          dVt[c - nn + 1] += q;
          dVt[c + 1] += q;
        } else if (ring(i, j)) {
          if (dRu) (*dRu)[c] += lu[c];
        } else if (dNu) {
          (*dNu)[c] += lu[c];
        }
        if (vadv(i, j)) {
          T x = (T)i * h + h2 - sdt * f.avgU(Ut, i, j);
          T y = (T)j * h - sdt * Vt[c];
          T gx, gy;
          sample_adj(x, y, Fv, dFv, 1, lv[c], &gx, &gy);
          dVt[c] += -sdt * gy * lv[c];
          T q = (T)0.25 * (-sdt * gx * lv[c]);
          dUt[c - 1] += q;
          dUt[c] += q;
          dUt[c + nn - 1] += q;
          dUt[c + nn] += q;
        } else if (ring(i, j)) {
          if (dRv) (*dRv)[c] += lv[c];
        } else if (dNv) {
          (*dNv)[c] += lv[c];
        }
      }
  }

  // Offset of the neighbour that bounded val in clampToNeighbors' scan, or
  // INT_MIN when val was inside the range.
  int clamp_src(T val, const std::vector<T>& O, int i, int j) const {
    const int nn = n();
    T lo = O[i * nn + j], hi = lo;
    int klo = 0, khi = 0;
    for (int di = -1; di <= 1; ++di)
      for (int dj = -1; dj <= 1; ++dj) {
        T v = O[(i + di) * nn + j + dj];
        if (v < lo) {
          lo = v;
          klo = di * nn + dj;
        }
        if (v > hi) {
          hi = v;
          khi = di * nn + dj;
        }
      }
    if (val < lo) return klo;
    if (val > hi) return khi;
    return INT32_MIN;
  }

  // Adjoint of a semi-Lagrangian smoke pass traced with (U, V) at sdt; bwd:
  // BFECC's reverse sample (no max, non-fluid cells constant 0).
  void sl_smoke_adj(const std::vector<T>& lam, const std::vector<T>& U, const std::vector<T>& V,
                    const std::vector<T>& Ms, std::vector<T>& dU, std::vector<T>& dV,
                    std::vector<T>& dMs, std::vector<T>* dN, T sdt, bool bwd) const {
    const int nn = n();
    const T h = f.h, h2 = (T)0.5 * h, sa = f.SmokeAdvection;
    for (int i = 0; i < f.NX; ++i)
      for (int j = 0; j < f.NY; ++j) {
        int c = i * nn + j;
        T l = lam[c];
        if (fluid_interior(i, j)) {
          T u = (U[c] + U[c + nn]) * (T)0.5 * sa;
          T v = (V[c] + V[c + 1]) * (T)0.5 * sa;
          T x = (T)i * h + h2 - sdt * u;
          T y = (T)j * h + h2 - sdt * v;
          if (!bwd && !(f.sampleFrom(x, y, Ms, 2) >= 0)) l = 0;
          T gx, gy;
          sample_adj(x, y, Ms, dMs, 2, l, &gx, &gy);
          T du = -sdt * gx * l * (T)0.5 * sa, dv = -sdt * gy * l * (T)0.5 * sa;
          dU[c] += du;
          dU[c + nn] += du;
          dV[c] += dv;
          dV[c + 1] += dv;
        } else if (!bwd) {
          if (ring(i, j))
            dMs[c] += l;
          else if (dN)
            (*dN)[c] += l;
        }
      }
  }

  void adjoint_step(int k, std::vector<T>* dfu, std::vector<T>* dfv) {
    const Rec& r = recs[k];
    const T dt = dts[k];
    const int N = f.N, nn = n(), NX = f.NX, NY = f.NY;
    std::vector<T> dU5(N), dV5(N), dM2(N);
    for (int c = 0; c < N; ++c) {
      dU5[c] = aU[c] + aNU[c];
      dV5[c] = aV[c] + aNV[c];
      dM2[c] = aM[c] + aNM[c];
    }
    std::fill(aNU.begin(), aNU.end(), (T)0);
    std::fill(aNV.begin(), aNV.end(), (T)0);
    std::fill(aNM.begin(), aNM.end(), (T)0);
    // ---- smoke
    std::vector<T> dM1(N, 0);
    if (f.UseBFECC) {
      const std::vector<T>&fwdM = r.km[0], &corrM = r.km[1];
      std::vector<T> dcorr(N, 0), dfwd(N, 0);
      sl_smoke_adj(dM2, r.U5, r.V5, corrM, dU5, dV5, dcorr, &aNM, dt, false);
      for (int i = 1; i < NX - 1; ++i)
        for (int j = 1; j < NY - 1; ++j) {
          int c = i * nn + j;
          T lam = dcorr[c];
          bool adv = f.S[c] != 0;
          T b = 0, x = 0, y = 0;
          if (adv) {
            T u = (r.U5[c] + r.U5[c + nn]) * (T)0.5 * f.SmokeAdvection;
            T v = (r.V5[c] + r.V5[c + 1]) * (T)0.5 * f.SmokeAdvection;
            x = (T)i * f.h + (T)0.5 * f.h + dt * u;
            y = (T)j * f.h + (T)0.5 * f.h + dt * v;
            b = f.sampleFrom(x, y, fwdM, 2);
          }
          T o = r.M1[c];
          T raw = o - (b - o) * (T)0.5;
          int sk = clamp_src(raw, r.M1, i, j);
          T cm = sk != INT32_MIN ? r.M1[c + sk] : raw;
          if (cm < 0) continue;
          if (sk != INT32_MIN) {
            dM1[c + sk] += lam;
            continue;
          }
          dM1[c] += (T)1.5 * lam;
          if (!adv) continue;
          T lb = (T)-0.5 * lam, gx, gy;
          sample_adj(x, y, fwdM, dfwd, 2, lb, &gx, &gy);
          T du = dt * gx * lb * (T)0.5 * f.SmokeAdvection;
          T dv = dt * gy * lb * (T)0.5 * f.SmokeAdvection;
          dU5[c] += du;
          dU5[c + nn] += du;
          dV5[c] += dv;
          dV5[c + 1] += dv;
        }
      for (int i = 0; i < NX; ++i)
        for (int j = 0; j < NY; ++j)
          if (ring(i, j)) dM1[i * nn + j] += dcorr[i * nn + j];
      sl_smoke_adj(dfwd, r.U5, r.V5, r.M1, dU5, dV5, dM1, &aNM, dt, false);
    } else {
      sl_smoke_adj(dM2, r.U5, r.V5, r.M1, dU5, dV5, dM1, &aNM, dt, false);
    }
    // ---- velocity
    std::vector<T> dU(N, 0), dV(N, 0);  // dU4, dV4
    if (f.UseBFECC) {
      const std::vector<T>&fwdU = r.k[0], &fwdV = r.k[1], &corrU = r.k[2], &corrV = r.k[3];
      std::vector<T> dcU(N, 0), dcV(N, 0), dfU(N, 0), dfV(N, 0);
      sl_vel_adj(dU5, dV5, corrU, corrV, corrU, corrV, dcU, dcV, dcU, dcV, &dcU, &dcV, &aNU, &aNV,
                 dt);
      for (int i = 0; i < NX; ++i)
        for (int j = 0; j < NY; ++j) {
          int c = i * nn + j;
          if (ring(i, j)) {
            dU[c] += dcU[c];
            dV[c] += dcV[c];
            continue;
          }
          for (int comp = 0; comp < 2; ++comp) {
            const std::vector<T>& O = comp == 0 ? r.U4 : r.V4;
            const std::vector<T>& F = comp == 0 ? fwdU : fwdV;
            std::vector<T>& dO = comp == 0 ? dU : dV;
            T lam = comp == 0 ? dcU[c] : dcV[c];
            bool adv = comp == 0 ? uadv(i, j) : vadv(i, j);
            T b = 0, x = 0, y = 0;
            if (adv) {
              if (comp == 0) {
                x = (T)i * f.h + dt * r.U4[c];
                y = (T)j * f.h + f.h / (T)2 + dt * f.avgV(r.V4, i, j);
              } else {
                x = (T)i * f.h + f.h / (T)2 + dt * f.avgU(r.U4, i, j);
                y = (T)j * f.h + dt * r.V4[c];
              }
              b = f.sampleFrom(x, y, F, comp);
            }
            T o = O[c];
            T raw = o - (b - o) * (T)0.5;
            int sk = clamp_src(raw, O, i, j);
            if (sk != INT32_MIN) {
              dO[c + sk] += lam;
              continue;
            }
            dO[c] += (T)1.5 * lam;
            if (!adv) continue;
            T lb = (T)-0.5 * lam, gx, gy;
            sample_adj(x, y, F, comp == 0 ? dfU : dfV, comp, lb, &gx, &gy);
            T du = dt * gx * lb, dv = dt * gy * lb;
            if (comp == 0) {
              dU[c] += du;
              T q = (T)0.25 * dv;
              dV[c - nn] += q;
              dV[c] += q;
              dV[c - nn + 1] += q;
              dV[c + 1] += q;
            } else {
              dV[c] += dv;
              T q = (T)0.25 * du;
              dU[c - 1] += q;
              dU[c] += q;
              dU[c + nn - 1] += q;
              dU[c + nn] += q;
            }
          }
        }
      sl_vel_adj(dfU, dfV, r.U4, r.V4, r.U4, r.V4, dU, dV, dU, dV, &dU, &dV, &aNU, &aNV, dt);
    } else {
      sl_vel_adj(dU5, dV5, r.U4, r.V4, r.U4, r.V4, dU, dV, dU, dV, &dU, &dV, &aNU, &aNV, dt);
    }
    // ---- borders (fluid.go:236-289), reversed: the last write first
    auto fl = [&](int i, int j) { return f.S[i * nn + j] != 0; };
    for (int i = 0; i < NX; ++i) {
      T* d = &dU[i * nn];
      T l = d[NY - 1];
      d[NY - 1] = 0;
      if (fl(i, NY - 1) && fl(i, NY - 2)) {
        if (i > 0 && i < NX - 1 && fl(i, NY - 3)) {
          d[NY - 2] += 2 * l;
          d[NY - 3] -= l;
        } else {
          d[NY - 2] += l;
        }
      }
      l = d[0];
      d[0] = 0;
      if (fl(i, 0) && fl(i, 1)) {
        if (i > 0 && i < NX - 1 && fl(i, 2)) {
          d[1] += 2 * l;
          d[2] -= l;
        } else {
          d[1] += l;
        }
      }
    }
    for (int j = 0; j < NY; ++j) {
      int a = (NX - 1) * nn + j, b = (NX - 2) * nn + j, c3 = (NX - 3) * nn + j;
      T l = dV[a];
      dV[a] = 0;
      if (fl(NX - 1, j) && fl(NX - 2, j)) {
        if (j > 0 && j < NY - 1 && fl(NX - 3, j)) {
          dV[b] += 2 * l;
          dV[c3] -= l;
        } else {
          dV[b] += l;
        }
      }
      l = dV[j];
      dV[j] = 0;
      if (fl(0, j) && fl(1, j)) {
        if (j > 0 && j < NY - 1 && fl(2, j)) {
          dV[nn + j] += 2 * l;
          dV[2 * nn + j] -= l;
        } else {
          dV[nn + j] += l;
        }
      }
    }
    // ---- confinement (fluid.go:449-493) and turbulence (fluid.go:496-526)
    std::vector<T> Uc = r.U2, Vc = r.V2;  // after confinement
    std::vector<T> curl(N, 0);
    const T h = f.h;
    if (f.Confinement != 0) {
      std::swap(f.U, Uc);
      std::swap(f.V, Vc);
      f.applyVorticityConfinement(dt);
      std::swap(f.U, Uc);
      std::swap(f.V, Vc);
      for (int i = 1; i < NX - 1; ++i)
        for (int j = 1; j < NY - 1; ++j)
          if (f.S[i * nn + j] != 0)
            curl[i * nn + j] = (r.V2[(i + 1) * nn + j] - r.V2[(i - 1) * nn + j]) * (T)0.5 / h -
                               (r.U2[i * nn + j + 1] - r.U2[i * nn + j - 1]) * (T)0.5 / h;
    }
    if (f.TurbulenceStrength > 0) {
      T ts = f.TurbulenceStrength * dt;
      for (int i = 1; i < NX - 1; ++i)
        for (int j = 1; j < NY - 1; ++j) {
          int c = i * nn + j;
          if (f.S[c] == 0) continue;
          T u = Uc[c], v = Vc[c];
          T rr = go_sqrt(u * u + v * v);
          if (!(rr > (T)0.1) || !((T)0.5 * rr < 1)) continue;
          T seedU = (T)(i * 137 + j * 241) * (T)0.01;
          T seedV = (T)(i * 157 + j * 263) * (T)0.01;
          T nU = (T)std::sin((double)seedU) * ts, nV = (T)std::sin((double)seedV) * ts;
          T sc = (dU[c] * nU + dV[c] * nV) * (T)0.5;
          dU[c] += sc * u / rr;
          dV[c] += sc * v / rr;
        }
    }
    if (f.Confinement != 0) {
      const T conf = f.Confinement, eps = (T)1e-5, k2 = (T)0.5 / h;
      std::vector<T> lwd(N, 0), lgx(N, 0), lgy(N, 0);
      for (int i = 1; i < NX - 1; ++i)
        for (int j = 1; j < NY - 1; ++j) {
          int c = i * nn + j;
          if (f.S[c] == 0) continue;
          T gx = (go_abs(curl[c + nn]) - go_abs(curl[c - nn])) * (T)0.5 / h;
          T gy = (go_abs(curl[c + 1]) - go_abs(curl[c - 1])) * (T)0.5 / h;
          T rg = go_sqrt(gx * gx + gy * gy), m = rg + eps;
          T nx = gx / m, ny = gy / m, w = curl[c];
          T u = r.U2[c], v = r.V2[c], rr = go_sqrt(u * u + v * v);
          T K = conf * ((T)1.0 + rr * (T)0.1);
          T a = dU[c] * dt, b = -dV[c] * dt;
          T Sm = a * ny + b * nx;
          if (rr > 0) {
            dU[c] += w * Sm * conf * (T)0.1 * u / rr;
            dV[c] += w * Sm * conf * (T)0.1 * v / rr;
          }
          lwd[c] = K * Sm;
          T Lnx = K * w * b, Lny = K * w * a;
          T qx = Lnx / m, qy = Lny / m;
          if (rg > 0) {
            T t = (Lnx * gx + Lny * gy) / (rg * m * m);
            qx -= t * gx;
            qy -= t * gy;
          }
          lgx[c] = qx;
          lgy[c] = qy;
        }
      std::vector<T> lw(N, 0);
      for (int i = 1; i < NX - 1; ++i)
        for (int j = 1; j < NY - 1; ++j) {
          int c = i * nn + j;
          if (f.S[c] == 0) continue;
          T w = curl[c];
          T sg = w > 0 ? (T)1 : (w < 0 ? (T)-1 : (T)0);
          lw[c] = lwd[c] + sg * k2 * ((lgx[c - nn] - lgx[c + nn]) + (lgy[c - 1] - lgy[c + 1]));
        }
      for (int i = 1; i < NX - 1; ++i)
        for (int j = 1; j < NY - 1; ++j) {
          int c = i * nn + j;
          T l = lw[c] * k2;
          if (l == 0) continue;
          dV[c + nn] += l;
          dV[c - nn] -= l;
          dU[c + 1] -= l;
          dU[c - 1] += l;
        }
    }
    // ---- projection: dU1 = dU2 + div^T P_K G^T dU2 (P_K symmetric)
    {
      std::vector<T> g(N, 0), bw(N, 0), x(N, 0), tmp(N, 0);
      for (int c = 0; c < N; ++c)
        if (f.cnt[c]) {
          g[c] = f.S[c + nn] * dU[c + nn] - f.S[c - nn] * dU[c] + f.S[c + 1] * dV[c + 1] -
                 f.S[c - 1] * dV[c];
          bw[c] = f.Wc[c] * g[c];
        }
      T keep = f.st.last_maxdiv;
      f.relax(g, bw, x, tmp, f.num_iters, false);
      f.st.last_maxdiv = keep;
      for (int i = 1; i < NX; ++i)
        for (int j = 0; j < NY; ++j) {
          int c = i * nn + j;
          dU[c] += x[c] - x[c - nn];
        }
      for (int i = 0; i < NX; ++i)
        for (int j = 1; j < NY; ++j) {
          int c = i * nn + j;
          dV[c] += x[c] - x[c - 1];
        }
    }
    // ---- sources, forces
    for (const Source& s : src) {
      int c = s.i * nn + s.j;
      if ((s.mode & 1) && f.S[c] == 0) continue;
      if (s.mode & 2) dU[c] = dV[c] = 0;
      if (s.mode & 8) dM1[c] = 0;
    }
    if (dfu) *dfu = dU;
    if (dfv) *dfv = dV;
    aU = dU;
    aV = dV;
    aM = dM1;
  }
};

}  // namespace orc

// ===========================================================================
// C ABI (loaded with ctypes by the tests and the benchmark's CPU leg).
// Fields: 0 U, 1 V, 2 newU, 3 newV, 4 p, 5 S, 6 M, 7 newM.
// ===========================================================================
namespace {
struct Handle {
  int prec;
  orc::Pool* pool;
  orc::Fluid<float>* f32;
  orc::Fluid<double>* f64;
};
template <typename F>
auto with(Handle* h, F&& fn) {
  if (h->prec == 32) return fn(*h->f32);
  return fn(*h->f64);
}
template <typename T>
std::vector<T>* field_of(orc::Fluid<T>& f, int k) {
  switch (k) {
    case 0: return &f.U;
    case 1: return &f.V;
    case 2: return &f.newU;
    case 3: return &f.newV;
    case 4: return &f.p;
    case 5: return &f.S;
    case 6: return &f.M;
    case 7: return &f.newM;
    case 8: return &f.phi;
    case 9: return &f.rhs;
  }
  return nullptr;
}
}  // namespace

extern "C" {

void* orc_create(int prec, int width, int height, double density, double h, int threads) {
  if ((prec != 32 && prec != 64) || width < 1 || height < 1) return nullptr;
  Handle* hd = new Handle{prec, new orc::Pool(threads), nullptr, nullptr};
  if (prec == 32)
    hd->f32 = new orc::Fluid<float>((float)density, width, height, (float)h, hd->pool);
  else
    hd->f64 = new orc::Fluid<double>(density, width, height, h, hd->pool);
  return hd;
}

void orc_destroy(void* p) {
  Handle* h = (Handle*)p;
  if (!h) return;
  delete h->f32;
  delete h->f64;
  delete h->pool;
  delete h;
}

int orc_dims(void* p, int* nx, int* ny) {
  return with((Handle*)p, [&](auto& f) { *nx = f.NX; *ny = f.NY; return 0; });
}

void* orc_field(void* p, int k) {
  return with((Handle*)p, [&](auto& f) -> void* {
    auto* v = field_of(f, k);
    if (!v || v->empty()) return nullptr;
    return (void*)v->data();
  });
}

int orc_set_param(void* p, const char* name, double value) {
  std::string k(name);
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    if (k == "Confinement") f.Confinement = (T)value;
    else if (k == "ViscosityDiffusion") f.ViscosityDiffusion = (T)value;
    else if (k == "PressureDamping") f.PressureDamping = (T)value;
    else if (k == "TurbulenceStrength") f.TurbulenceStrength = (T)value;
    else if (k == "SmokeAdvection") f.SmokeAdvection = (T)value;
    else if (k == "UseMultigrid") f.UseMultigrid = value != 0;
    else if (k == "MultigridLevels") f.MultigridLevels = (int)value;
    else if (k == "UseBFECC") f.UseBFECC = value != 0;
    else if (k == "Relaxation") f.Relaxation = (T)value;
    else if (k == "num_iters") f.num_iters = (int)value;
    else if (k == "tolerance") f.tolerance = (T)value;
    else if (k == "early_exit") f.early_exit = value != 0;
    else if (k == "scheme") f.scheme = (int)value;
    else if (k == "jacobi_omega") f.jacobi_omega = (T)value;
    else if (k == "check_every") f.check_every = std::max(1, (int)value);
    else if (k == "refine_sweeps") f.refine_sweeps = (int)value;
    else if (k == "precise_coords") f.precise_coords = value != 0;
    else return -1;
    return 0;
  });
}

double orc_get_param(void* p, const char* name) {
  std::string k(name);
  return with((Handle*)p, [&](auto& f) -> double {
    if (k == "Confinement") return f.Confinement;
    if (k == "ViscosityDiffusion") return f.ViscosityDiffusion;
    if (k == "PressureDamping") return f.PressureDamping;
    if (k == "TurbulenceStrength") return f.TurbulenceStrength;
    if (k == "SmokeAdvection") return f.SmokeAdvection;
    if (k == "UseMultigrid") return f.UseMultigrid;
    if (k == "MultigridLevels") return f.MultigridLevels;
    if (k == "UseBFECC") return f.UseBFECC;
    if (k == "Relaxation") return f.Relaxation;
    if (k == "num_iters") return f.num_iters;
    if (k == "tolerance") return f.tolerance;
    if (k == "early_exit") return f.early_exit;
    if (k == "scheme") return f.scheme;
    if (k == "jacobi_omega") return f.jacobi_omega;
    if (k == "check_every") return f.check_every;
    if (k == "refine_sweeps") return f.refine_sweeps;
    if (k == "precise_coords") return f.precise_coords ? 1 : 0;
    if (k == "h") return f.h;
    if (k == "density") return f.density;
    return std::nan("");
  });
}

void orc_simulate(void* p, double dt) {
  with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    f.simulate((T)dt);
    return 0;
  });
}

// Stage entry points (the white-box tests of the reference call these).
// stage: 0 makeIncompressible(iters, dt) 1 advectVelocity 2 advectSmoke
// 3 handleBorders 4 applyVorticityConfinement 5 applyViscosity
// 6 addTurbulence 7 advectVelocityBFECC 8 advectSmokeBFECC
// 9 fill(p, 0)
int orc_stage(void* p, int stage, int iters, double dt) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    T d = (T)dt;
    switch (stage) {
      case 0: f.makeIncompressible(iters, d); break;
      case 1: f.advectVelocity(d); break;
      case 2: f.advectSmoke(d); break;
      case 3: f.handleBorders(); break;
      case 4: f.applyVorticityConfinement(d); break;
      case 5: f.applyViscosity(d); break;
      case 6: f.addTurbulence(d); break;
      case 7: f.advectVelocityBFECC(d); break;
      case 8: f.advectSmokeBFECC(d); break;
      case 9: std::fill(f.p.begin(), f.p.end(), (T)0); break;
      default: return -1;
    }
    return 0;
  });
}

// copyBorder(dst, src) on two caller buffers of NX*NY elements of the
// instance's precision.
int orc_copy_border(void* p, void* dst, const void* src) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    std::vector<T> d((T*)dst, (T*)dst + f.N), s((const T*)src, (const T*)src + f.N);
    f.copyBorder(d, s);
    std::memcpy(dst, d.data(), sizeof(T) * f.N);
    return 0;
  });
}

int orc_set_solid(void* p, int i, int j, int v) {
  return with((Handle*)p, [&](auto& f) { return f.setSolid(i, j, v != 0); });
}
int orc_is_solid(void* p, int i, int j) {
  return with((Handle*)p, [&](auto& f) { return f.isSolid(i, j); });
}
int orc_set_velocity(void* p, int i, int j, double u, double v) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    return f.setVelocity(i, j, (T)u, (T)v);
  });
}
int orc_add_smoke(void* p, int i, int j, double s) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    return f.addSmoke(i, j, (T)s);
  });
}
void orc_reset(void* p) { with((Handle*)p, [&](auto& f) { f.reset(); return 0; }); }
void orc_apply_force(void* p, int i, int j, double fx, double fy) {
  with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    f.applyForce(i, j, (T)fx, (T)fy);
    return 0;
  });
}
void orc_apply_force_radius(void* p, int cx, int cy, double fx, double fy, int r) {
  with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    f.applyForceRadius(cx, cy, (T)fx, (T)fy, r);
    return 0;
  });
}
void orc_set_circular_obstacle(void* p, int cx, int cy, int r) {
  with((Handle*)p, [&](auto& f) { f.setCircularObstacle(cx, cy, r); return 0; });
}
double orc_max_divergence(void* p) {
  return with((Handle*)p, [&](auto& f) -> double { return f.maxDivergence(); });
}
double orc_adaptive_dt(void* p, double basedt) {
  return with((Handle*)p, [&](auto& f) -> double {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    return f.getAdaptiveTimeStep((T)basedt);
  });
}
// out: NX*NY elements of the instance precision; mnmx[2] (double)
int orc_vorticity(void* p, void* out, double* mnmx) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    T mn, mx;
    f.vorticity((T*)out, &mn, &mx);
    mnmx[0] = mn;
    mnmx[1] = mx;
    return 0;
  });
}
int orc_velocity_magnitude(void* p, void* out, double* mnmx) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    T mn, mx;
    f.velocityMagnitude((T*)out, &mn, &mx);
    mnmx[0] = mn;
    mnmx[1] = mx;
    return 0;
  });
}
int orc_sample_velocity(void* p, double x, double y, double* uv) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    uv[0] = f.sampleFrom((T)x, (T)y, f.U, 0);
    uv[1] = f.sampleFrom((T)x, (T)y, f.V, 1);
    return 0;
  });
}
// stats: div_l2_post, div_max_post, div_count_post, resid_l2, resid_max,
// smoke_mass, sweeps, last_maxdiv
int orc_stats(void* p, double* out) {
  return with((Handle*)p, [&](auto& f) {
    out[0] = f.st.div_l2_post;
    out[1] = f.st.div_max_post;
    out[2] = f.st.div_count_post;
    out[3] = f.st.resid_l2;
    out[4] = f.st.resid_max;
    out[5] = f.st.smoke_mass;
    out[6] = f.st.sweeps;
    out[7] = f.st.last_maxdiv;
    return 0;
  });
}
int orc_threads(void* p) { return ((Handle*)p)->pool->size(); }

// Tracer particles: advances n particles in place (the survivors first, in
// order); returns their number.  Arrays hold the handle's precision.
int orc_particles_advect(void* p, int n, void* x, void* y, void* age, void* max_age,
                         uint32_t* rgb, double dt) {
  return with((Handle*)p, [&](auto& f) {
    using T = typename std::remove_reference<decltype(f.U[0])>::type;
    return orc::advect_particles(f, n, (T*)x, (T*)y, (T*)age, (T*)max_age, rgb, (T)dt);
  });
}

// Renders field `kind` (0 smoke, 1 pressure, 2 speed, 3 vorticity) into out
// (NX x NY RGBA8).
int orc_render(void* p, int kind, uint8_t* out) {
  return with((Handle*)p, [&](auto& f) {
    orc::render(f, kind, out);
    return 0;
  });
}

// Recorded rollout of `steps` steps from the handle's state (FP64 handles
// only) with per-step forces (steps x 2 x N, NULL = none) and n_src sources
// applied before every step; loss L = ||M - target||_2 over interior cells
// and its reverse pass.  Outputs dL/d(initial U, V, M) and dL/d(forces)
// (steps x 2 x N, may be NULL).  The handle ends at the end of the rollout.
int orc_rollout_grad(void* p, int steps, double dt, const double* forces, int n_src,
                     const int* si, const int* sj, const double* su, const double* sv,
                     const double* ssmoke, const int* smode, const double* target, double* loss,
                     double* dU, double* dV, double* dM, double* dF) {
  Handle* hd = (Handle*)p;
  if (hd->prec != 64 || steps < 1) return -1;
  orc::Fluid<double>& f = *hd->f64;
  if (f.scheme != orc::Jacobi || f.early_exit || f.refine_sweeps > 0 ||
      f.ViscosityDiffusion > 0)
    return -4;
  orc::Rollout<double> r(f);
  for (int k = 0; k < n_src; ++k)
    r.src.push_back(orc::Source{si[k], sj[k], su[k], sv[k], ssmoke[k], smode[k]});
  const int N = f.N;
  for (int t = 0; t < steps; ++t)
    r.step(dt, forces ? forces + (size_t)t * 2 * N : nullptr,
           forces ? forces + (size_t)t * 2 * N + N : nullptr);
  double L2 = 0;
  for (int i = 1; i < f.NX - 1; ++i)
    for (int j = 1; j < f.NY - 1; ++j) {
      double d = f.M[i * f.NY + j] - target[i * f.NY + j];
      L2 += d * d;
    }
  double L = std::sqrt(L2);
  *loss = L;
  r.aU.assign(N, 0);
  r.aV.assign(N, 0);
  r.aM.assign(N, 0);
  r.aNU.assign(N, 0);
  r.aNV.assign(N, 0);
  r.aNM.assign(N, 0);
  for (int i = 1; i < f.NX - 1; ++i)
    for (int j = 1; j < f.NY - 1; ++j) {
      int c = i * f.NY + j;
      r.aM[c] = L > 0 ? (f.M[c] - target[c]) / L : 0;
    }
  std::vector<double> gu, gv;
  for (int t = steps - 1; t >= 0; --t) {
    r.adjoint_step(t, &gu, &gv);
    if (dF) {
      std::copy(gu.begin(), gu.end(), dF + (size_t)t * 2 * N);
      std::copy(gv.begin(), gv.end(), dF + (size_t)t * 2 * N + N);
    }
  }
  if (dU) std::copy(r.aU.begin(), r.aU.end(), dU);
  if (dV) std::copy(r.aV.begin(), r.aV.end(), dV);
  if (dM) std::copy(r.aM.begin(), r.aM.end(), dM);
  return 0;
}

}  // extern "C"
