"""Gradients of recorded rollouts (fg_step_forward / fg_step_adjoint).

The reference has no derivatives; the adjoint is checked the way a
hand-written reverse mode is checked:

* directional derivatives <grad, d> against central differences of the
  FP64 oracle's forward pass on the same scene, forces and sources (the
  oracle is the FP64 restatement of Simulate, fluid.go:79-109, with the
  force field added to U, V before the sources),
* against central differences of the GPU's own FP32 forward pass
  (eps = 1e-3, the rollout benchmark's check),
* reproducibility, independence of the checkpoint interval, and the state
  after the reverse pass equal to the end of the forward pass bit for bit,
* recorded forward steps without forces equal fg_simulate bit for bit,
* the error cases of the C ABI.
"""
import numpy as np
import pytest

import scenes
from oracle.pyoracle import OracleFluid

pytestmark = pytest.mark.gpu

W, H, DT, ITERS = 26, 22, 0.1, 20
STEPS = 6


@pytest.fixture(scope="module")
def gpu():
    import fluid_gb300

    fluid_gb300.build()
    return fluid_gb300


def jet_sources(f):
    """Jet inlet as persistent sources: U = 2 and +1 smoke on 8 rows at i = 1."""
    rows = np.array(list(scenes.jet_rows(f)), np.int32)
    f.set_sources(np.ones_like(rows), rows, u=2.0, v=0.0, smoke=1.0, mode=1 | 2 | 4)


def oracle_jet_sources(o):
    for j in scenes.jet_rows(o):
        if not o.IsSolid(1, j):
            o.SetVelocity(1, j, 2.0, 0.0)
            o.AddSmoke(1, j, 1.0)


def initial_state(f, seed=11):
    """Smooth seeded velocity and smoke on the fluid cells."""
    rng = np.random.default_rng(seed)
    nx, ny = f.NumX, f.NumY
    x = np.arange(nx)[:, None] / nx
    y = np.arange(ny)[None, :] / ny
    U = np.zeros((nx, ny))
    V = np.zeros((nx, ny))
    M = np.zeros((nx, ny))
    for _ in range(3):
        a, b, c, d = rng.uniform(0.5, 3.0, 4)
        U += rng.uniform(-0.6, 0.6) * np.sin(a * np.pi * x + c) * np.cos(b * np.pi * y + d)
        V += rng.uniform(-0.6, 0.6) * np.cos(a * np.pi * x + d) * np.sin(b * np.pi * y + c)
        M += rng.uniform(0.2, 0.6) * np.exp(-((x - rng.uniform(0.2, 0.8)) ** 2
                                              + (y - rng.uniform(0.2, 0.8)) ** 2) / 0.02)
    S = f.S.reshape(nx, ny) != 0
    U[1:, :] *= S[1:, :] * S[:-1, :]
    V[:, 1:] *= S[:, 1:] * S[:, :-1]
    U[0, :] = 0
    V[:, 0] = 0
    M *= S
    return U.ravel(), V.ravel(), M.ravel()


def target_field(nx, ny, seed=4):
    """Sum of 4 seeded isotropic Gaussian blobs (sigma 2-6 cells, amplitude 0.5-1)."""
    rng = np.random.default_rng(seed)
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    T = np.zeros((nx, ny))
    for _ in range(4):
        s = rng.uniform(2.0, 6.0)
        a = rng.uniform(0.5, 1.0)
        ci, cj = rng.uniform(1, nx - 1), rng.uniform(1, ny - 1)
        T += a * np.exp(-((i - ci) ** 2 + (j - cj) ** 2) / (2 * s * s))
    return T.ravel()


def make_gpu(gpu, **extra):
    params = dict(scheme=1, num_iters=ITERS, tb_depth=8, early_exit=False, UseBFECC=True)
    params.update(extra)
    f = gpu.Fluid(1.0, W, H, 1.0, auto_sync=False, **params)
    scenes.fast_walls(f)
    f.mark_dirty()
    f.download()
    return f


def seeded_forces(n, steps, seed=7, amp=0.05):
    rng = np.random.default_rng(seed)
    return [(rng.uniform(-amp, amp, n).astype(np.float32), rng.uniform(-amp, amp, n).astype(np.float32))
            for _ in range(steps)]


def gpu_rollout(gpu, U0, V0, M0, forces, target, every=4, steps=STEPS, **extra):
    f = make_gpu(gpu, **extra)
    jet_sources(f)
    f.U[:] = U0
    f.V[:] = V0
    f.M[:] = M0
    f.mark_dirty()
    out = f.rollout_grad(DT, steps, target.astype(np.float32), forces, every=every)
    return f, out


def gpu_loss(gpu, U0, V0, M0, forces, target, steps=STEPS, **extra):
    f = make_gpu(gpu, **extra)
    jet_sources(f)
    f.U[:] = U0
    f.V[:] = V0
    f.M[:] = M0
    f.mark_dirty()
    f.tape_begin(steps, 4)
    for t in range(steps):
        f.step_forward(DT, *forces[t])
    loss = f.tape_seed_smoke_l2(target.astype(np.float32))
    f.tape_end()
    return loss


def oracle_loss(U0, V0, M0, forces, target, steps=STEPS, S=None, bfecc=True, conf=0.0, **extra):
    o = OracleFluid(1.0, W, H, 1.0, prec=64, scheme=1, num_iters=ITERS, check_every=8,
                    early_exit=False, UseBFECC=bfecc, Confinement=conf, **extra)
    o.S[:] = S
    o.U[:] = U0
    o.V[:] = V0
    o.M[:] = M0
    for t in range(steps):
        fu, fv = forces[t]
        o.U[:] += fu
        o.V[:] += fv
        oracle_jet_sources(o)
        o.Simulate(DT)
    d = (o.M - target).reshape(o.NumX, o.NumY)[1:-1, 1:-1]
    return float(np.sqrt(np.sum(d * d)))


def directions(nx, ny, S, k, seed=21):
    """Seeded random directions on U0, V0 (interior faces) and the forces."""
    rng = np.random.default_rng(seed + k)
    n = nx * ny
    dU = rng.standard_normal(n) * 0.5
    dV = rng.standard_normal(n) * 0.5
    dF = [(rng.standard_normal(n) * 0.05, rng.standard_normal(n) * 0.05) for _ in range(STEPS)]
    return dU, dV, dF


def directional(out, dU, dV, dF):
    g = float(np.dot(out["U"].astype(np.float64), dU) + np.dot(out["V"].astype(np.float64), dV))
    for t, (du, dv) in enumerate(dF):
        g += float(np.dot(out["force_u"][t].astype(np.float64), du)
                   + np.dot(out["force_v"][t].astype(np.float64), dv))
    return g


@pytest.fixture(scope="module")
def problem(gpu):
    f = make_gpu(gpu)
    S = f.S.astype(np.float64).copy()
    U0, V0, M0 = initial_state(f)
    forces = seeded_forces(f.numCells, STEPS)
    target = target_field(f.NumX, f.NumY)
    _, out = gpu_rollout(gpu, U0, V0, M0, forces, target)
    return dict(S=S, U0=U0, V0=V0, M0=M0, forces=forces, target=target, out=out)


def test_loss_matches_fp64_oracle(gpu, problem):
    p = problem
    f64 = [(fu.astype(np.float64), fv.astype(np.float64)) for fu, fv in p["forces"]]
    lo = oracle_loss(p["U0"], p["V0"], p["M0"], f64, p["target"], S=p["S"])
    assert p["out"]["loss"] == pytest.approx(lo, rel=1e-4)


@pytest.mark.parametrize("k", range(8))
def test_directional_derivative_vs_fp64_central_differences(gpu, problem, k):
    p = problem
    dU, dV, dF = directions(W + 2, H + 2, p["S"], k)
    g = directional(p["out"], dU, dV, dF)
    eps = 1e-6
    f64 = [(fu.astype(np.float64), fv.astype(np.float64)) for fu, fv in p["forces"]]

    def at(s):
        fs = [(fu + s * du, fv + s * dv) for (fu, fv), (du, dv) in zip(f64, dF)]
        return oracle_loss(p["U0"] + s * dU, p["V0"] + s * dV, p["M0"], fs, p["target"], S=p["S"])

    fd = (at(eps) - at(-eps)) / (2 * eps)
    print("direction %d: adjoint %.8g  fp64 central difference %.8g" % (k, g, fd))
    # The BFECC clamps make the loss piecewise smooth: at eps 1e-5 the FP64
    # differences still cross clamp switches (they scatter by ~3e-5); at
    # 1e-6 and 1e-7 they agree with each other to ~1e-8.
    assert g == pytest.approx(fd, rel=1e-3, abs=5e-6)


@pytest.mark.parametrize("k", range(4))
def test_directional_derivative_without_bfecc(gpu, problem, k):
    """Semi-Lagrangian advection only (no clamps): a tighter bound."""
    p = problem
    _, out = gpu_rollout(gpu, p["U0"], p["V0"], p["M0"], p["forces"], p["target"], UseBFECC=False)
    dU, dV, dF = directions(W + 2, H + 2, p["S"], 50 + k)
    g = directional(out, dU, dV, dF)
    eps = 1e-6
    f64 = [(fu.astype(np.float64), fv.astype(np.float64)) for fu, fv in p["forces"]]

    def at(s):
        fs = [(fu + s * du, fv + s * dv) for (fu, fv), (du, dv) in zip(f64, dF)]
        return oracle_loss(p["U0"] + s * dU, p["V0"] + s * dV, p["M0"], fs, p["target"],
                           S=p["S"], bfecc=False)

    fd = (at(eps) - at(-eps)) / (2 * eps)
    print("no-BFECC direction %d: adjoint %.8g  fp64 central difference %.8g" % (k, g, fd))
    assert g == pytest.approx(fd, rel=1e-3, abs=5e-6)


@pytest.mark.parametrize("k", range(4))
def test_directional_derivative_with_confinement(gpu, problem, k):
    """Vorticity confinement (curl, |curl| gradient, normalisation, speed
    scaling) followed by turbulence, without BFECC."""
    p = problem
    _, out = gpu_rollout(gpu, p["U0"], p["V0"], p["M0"], p["forces"], p["target"], UseBFECC=False,
                         Confinement=0.3)
    dU, dV, dF = directions(W + 2, H + 2, p["S"], 70 + k)
    g = directional(out, dU, dV, dF)
    eps = 1e-6
    f64 = [(fu.astype(np.float64), fv.astype(np.float64)) for fu, fv in p["forces"]]

    def at(s):
        fs = [(fu + s * du, fv + s * dv) for (fu, fv), (du, dv) in zip(f64, dF)]
        return oracle_loss(p["U0"] + s * dU, p["V0"] + s * dV, p["M0"], fs, p["target"],
                           S=p["S"], bfecc=False, conf=0.3)

    fd = (at(eps) - at(-eps)) / (2 * eps)
    print("confinement direction %d: adjoint %.8g  fp64 central difference %.8g" % (k, g, fd))
    assert g == pytest.approx(fd, rel=1e-3, abs=5e-6)


REFINED = dict(refine_sweeps=8, precise_coords=True)


@pytest.fixture(scope="module")
def problem_refined(gpu):
    f = make_gpu(gpu, **REFINED)
    S = f.S.astype(np.float64).copy()
    U0, V0, M0 = initial_state(f, seed=12)
    forces = seeded_forces(f.numCells, STEPS, seed=8)
    target = target_field(f.NumX, f.NumY, seed=5)
    _, out = gpu_rollout(gpu, U0, V0, M0, forces, target, **REFINED)
    return dict(S=S, U0=U0, V0=V0, M0=M0, forces=forces, target=target, out=out)


@pytest.mark.parametrize("k", range(4))
def test_directional_derivative_with_outer_correction(gpu, problem_refined, k):
    """The headline forward's chosen forms in a recorded rollout: the 8-sweep
    outer correction of the potential (its adjoint: the correction solve on
    the adjoint right-hand side, then the main solve on that solve's
    residual) and face-relative departure points.  Directional derivatives
    against FP64 central differences of the oracle's forward pass with the
    same settings."""
    p = problem_refined
    dU, dV, dF = directions(W + 2, H + 2, p["S"], k, seed=31)
    g = directional(p["out"], dU, dV, dF)
    eps = 1e-6
    f64 = [(fu.astype(np.float64), fv.astype(np.float64)) for fu, fv in p["forces"]]

    def at(s):
        fs = [(fu + s * du, fv + s * dv) for (fu, fv), (du, dv) in zip(f64, dF)]
        return oracle_loss(p["U0"] + s * dU, p["V0"] + s * dV, p["M0"], fs, p["target"],
                           S=p["S"], **REFINED)

    fd = (at(eps) - at(-eps)) / (2 * eps)
    print("direction %d (outer correction): adjoint %.8g  fp64 central difference %.8g"
          % (k, g, fd))
    assert g == pytest.approx(fd, rel=1e-3, abs=5e-6)


def test_smoke_gradient_vs_fp64_central_differences(gpu, problem):
    """Relative perturbations of the initial smoke: cells whose smoke is 0
    (where max(s, 0) has a kink, so central differences see half a slope)
    stay unperturbed."""
    p = problem
    rng = np.random.default_rng(5)
    dM = rng.standard_normal(p["M0"].size) * 0.5 * p["M0"]
    g = float(np.dot(p["out"]["M"].astype(np.float64), dM))
    eps = 1e-6
    f64 = [(fu.astype(np.float64), fv.astype(np.float64)) for fu, fv in p["forces"]]
    fd = (oracle_loss(p["U0"], p["V0"], p["M0"] + eps * dM, f64, p["target"], S=p["S"])
          - oracle_loss(p["U0"], p["V0"], p["M0"] - eps * dM, f64, p["target"], S=p["S"])) / (2 * eps)
    print("smoke direction: adjoint %.8g  fp64 central difference %.8g" % (g, fd))
    assert g == pytest.approx(fd, rel=1e-3, abs=5e-6)


@pytest.mark.parametrize("k", range(4))
def test_directional_derivative_vs_fp32_gpu_differences(gpu, problem, k):
    """Central differences of the GPU's FP32 forward with eps = 1e-3.  The
    loss (about 22) is resolved to 2e-6 in float, so the differences carry
    about 1e-3 of quantisation."""
    p = problem
    dU, dV, dF = directions(W + 2, H + 2, p["S"], 100 + k)
    g = directional(p["out"], dU, dV, dF)
    eps = 1e-3

    def at(s):
        fs = [((fu + s * du).astype(np.float32), (fv + s * dv).astype(np.float32))
              for (fu, fv), (du, dv) in zip(p["forces"], dF)]
        return gpu_loss(gpu, (p["U0"] + s * dU).astype(np.float32),
                        (p["V0"] + s * dV).astype(np.float32), p["M0"].astype(np.float32), fs,
                        p["target"])

    fd = (at(eps) - at(-eps)) / (2 * eps)
    print("direction %d: adjoint %.6g  fp32 central difference %.6g" % (k, g, fd))
    assert g == pytest.approx(fd, rel=2e-2, abs=2e-3)


def test_checkpoint_interval_does_not_change_gradients(gpu, problem):
    p = problem
    ref = p["out"]
    for every in (1, 3, STEPS):
        _, out = gpu_rollout(gpu, p["U0"], p["V0"], p["M0"], p["forces"], p["target"], every=every)
        assert out["loss"] == ref["loss"]
        for k in ("U", "V", "M"):
            scale = float(np.abs(ref[k]).max())
            assert np.abs(out[k] - ref[k]).max() <= 1e-5 * scale, (every, k)
        for t in range(STEPS):
            scale = float(np.abs(ref["force_u"][t]).max())
            assert np.abs(out["force_u"][t] - ref["force_u"][t]).max() <= 1e-5 * scale


def test_reverse_pass_restores_final_state(gpu, problem):
    p = problem
    f = make_gpu(gpu)
    jet_sources(f)
    f.U[:], f.V[:], f.M[:] = p["U0"], p["V0"], p["M0"]
    f.mark_dirty()
    f.tape_begin(STEPS, 4)
    for t in range(STEPS):
        f.step_forward(DT, *p["forces"][t])
    f.download()
    end = {k: getattr(f, k).copy() for k in ("U", "V", "M", "newU", "newV", "newM")}
    f.tape_seed_smoke_l2(p["target"].astype(np.float32))
    for t in range(STEPS):
        assert f.tape_steps() == (STEPS, t)
        f.step_adjoint()
    f.download()
    for k, v in end.items():
        assert np.array_equal(getattr(f, k).view(np.uint32), v.view(np.uint32)), k
    f.tape_end()


@pytest.mark.parametrize("extra", [{}, {"refine_sweeps": 8, "precise_coords": True}],
                         ids=["plain", "refined"])
def test_recorded_steps_equal_simulate(gpu, problem, extra):
    """Recorded steps (the BFECC passes written to the tape, the potential
    stored with its outer correction) equal fg_simulate's bit for bit."""
    p = problem
    a = make_gpu(gpu, TurbulenceStrength=0.05, **extra)
    b = make_gpu(gpu, TurbulenceStrength=0.05, **extra)
    for f in (a, b):
        jet_sources(f)
        f.U[:], f.V[:], f.M[:] = p["U0"], p["V0"], p["M0"]
        f.mark_dirty()
    a.tape_begin(STEPS, 4)
    for _ in range(STEPS):
        a.step_forward(DT)
        b.Simulate(DT)
    a.tape_end()
    a.download()
    b.download()
    for k in ("U", "V", "M", "newU", "newV", "newM"):
        assert np.array_equal(getattr(a, k).view(np.uint32), getattr(b, k).view(np.uint32)), k


def test_unsupported_and_invalid(gpu):
    from fluid_gb300 import FluidError

    f = gpu.Fluid(1.0, 8, 8, 1.0, auto_sync=False)  # reference scheme
    with pytest.raises(FluidError) as e:
        f.tape_begin(4)
    assert e.value.code == -4
    f = make_gpu(gpu, ViscosityDiffusion=0.1)
    with pytest.raises(FluidError) as e:
        f.tape_begin(4)
    assert e.value.code == -4
    f = make_gpu(gpu)
    f.tape_begin(2, 1)
    f.step_forward(DT)
    f.SetVelocity(3, 3, 1.0, 0.0)  # an edit inside a recorded rollout
    with pytest.raises(FluidError):
        f.step_forward(DT)
    f.tape_end()
    f = make_gpu(gpu)
    f.tape_begin(1, 1)
    with pytest.raises(FluidError):
        f.step_adjoint()  # not seeded
    f.step_forward(DT)
    with pytest.raises(FluidError):
        f.step_forward(DT)  # beyond max_steps
    f.tape_seed()
    f.step_adjoint()
    with pytest.raises(FluidError):
        f.step_adjoint()  # nothing left to reverse
    f.tape_end()


# ------------------------------------------------------------------ 256^2 jet rollout
R_SIDE, R_STEPS, R_ITERS, R_EVERY = 256, 64, 60, 8


def rollout_fluid(gpu):
    f = gpu.Fluid(1.0, R_SIDE, R_SIDE, 1.0, auto_sync=False, scheme=1, num_iters=R_ITERS,
                  tb_depth=8, early_exit=False, UseBFECC=True)
    scenes.jet_rollout_scene(f)
    return f


def rollout_loss(f, U0, V0, forces, target):
    """L after R_STEPS steps from (U0, V0) with the given forces (GPU, FP32)."""
    f.Reset()
    f.download()
    f.U[:], f.V[:] = U0, V0
    f.mark_dirty((1 << 0) | (1 << 1))
    f.tape_begin(R_STEPS, R_EVERY)
    for t in range(R_STEPS):
        f.step_forward(DT, forces[t][0], forces[t][1])
    loss = f.tape_seed_smoke_l2(target)
    f.tape_end()
    return loss


@pytest.fixture(scope="module")
def rollout256(gpu):
    f = rollout_fluid(gpu)
    n = f.numCells
    target = scenes.gaussian_target(f.NumX, f.NumY, seed=4)
    U0 = np.zeros(n, np.float32)
    V0 = np.zeros(n, np.float32)
    forces = [(np.zeros(n, np.float32), np.zeros(n, np.float32)) for _ in range(R_STEPS)]
    out = f.rollout_grad(DT, R_STEPS, target, forces, every=R_EVERY)
    return dict(f=f, target=target, U0=U0, V0=V0, forces=forces, out=out)


def rollout_directions(n, k):
    rng = np.random.default_rng(4000 + k)
    dU = rng.standard_normal(n).astype(np.float32)
    dV = rng.standard_normal(n).astype(np.float32)
    dF = [(rng.standard_normal(n).astype(np.float32) * 0.1, rng.standard_normal(n).astype(np.float32) * 0.1)
          for _ in range(R_STEPS)]
    return dU, dV, dF


def oracle_rollout_loss(S, U0, V0, forces, target):
    """The same rollout on the FP64 oracle (host sources before each step)."""
    import os

    o = OracleFluid(1.0, R_SIDE, R_SIDE, 1.0, prec=64, threads=os.cpu_count() or 1, scheme=1,
                    num_iters=R_ITERS, check_every=8, early_exit=False, UseBFECC=True)
    o.S[:] = S
    o.U[:], o.V[:] = U0, V0
    rows = list(scenes.jet_rows(o))
    for t in range(R_STEPS):
        o.U[:] += forces[t][0]
        o.V[:] += forces[t][1]
        for j in rows:
            if not o.IsSolid(1, j):
                o.SetVelocity(1, j, 2.0, 0.0)
                o.M[1 * o.NumY + j] = 1.0
        o.Simulate(DT)
    d = (o.M - target).reshape(o.NumX, o.NumY)[1:-1, 1:-1]
    return float(np.sqrt(np.sum(d * d)))


def rollout_directional(out, dU, dV, dF):
    g = float(np.dot(out["U"].astype(np.float64), dU) + np.dot(out["V"].astype(np.float64), dV))
    for t in range(R_STEPS):
        g += float(np.dot(out["force_u"][t].astype(np.float64), dF[t][0])
                   + np.dot(out["force_v"][t].astype(np.float64), dF[t][1]))
    return g


def test_rollout256_vs_fp64_oracle_differences(gpu, rollout256):
    """256^2 jet rollout: directional derivatives on 8 seeded directions
    against central differences of the FP64 oracle's forward.  Over 64 steps
    of 66k cells, eps 1e-5 and even 1e-6 still cross BFECC clamp switches
    on some directions; the differences settle for eps <= 3e-7."""
    r = rollout256
    f, out = r["f"], r["out"]
    f.download()
    S = f.S.astype(np.float64).copy()
    n = f.numCells
    for k in range(8):
        dU, dV, dF = rollout_directions(n, k)
        g = rollout_directional(out, dU, dV, dF)
        eps = 1e-7
        vals = []
        for s in (eps, -eps):
            fs = [(r["forces"][t][0] + s * dF[t][0].astype(np.float64),
                   r["forces"][t][1] + s * dF[t][1].astype(np.float64)) for t in range(R_STEPS)]
            vals.append(oracle_rollout_loss(S, r["U0"] + s * dU.astype(np.float64),
                                            r["V0"] + s * dV.astype(np.float64), fs, r["target"]))
        fd = (vals[0] - vals[1]) / (2 * eps)
        print("rollout256 direction %d: adjoint %.8g  fp64 central difference %.8g" % (k, g, fd))
        assert g == pytest.approx(fd, rel=1e-3, abs=1e-5)


def test_rollout256_fp32_central_differences_32_directions(gpu, rollout256):
    """256^2 jet, 64 steps, BFECC, 60 sweeps, checkpoint every 8: the
    adjoint's directional derivatives against central differences of the
    FP32 forward pass (loss returned in FP64) with eps = 1e-3 on 32 seeded
    directions.  These differences carry the FP32 trajectory's rounding and
    the clamp switches a 1e-3 perturbation of every cell causes (a few
    percent); the FP64 check above is the tight one."""
    r = rollout256
    f, out = r["f"], r["out"]
    n = f.numCells
    eps = 1e-3
    rows = []
    for k in range(32):
        dU, dV, dF = rollout_directions(n, k)
        g = rollout_directional(out, dU, dV, dF)
        vals = []
        for s in (eps, -eps):
            fs = [(r["forces"][t][0] + s * dF[t][0], r["forces"][t][1] + s * dF[t][1])
                  for t in range(R_STEPS)]
            vals.append(rollout_loss(f, r["U0"] + s * dU, r["V0"] + s * dV, fs, r["target"]))
        rows.append((g, (vals[0] - vals[1]) / (2 * eps)))
    g = np.array([x[0] for x in rows])
    fd = np.array([x[1] for x in rows])
    rel = np.abs(g - fd) / np.abs(fd)
    print("rollout256: loss %.6g  |dL/dU0| %.4g  median rel err %.3g  max %.3g"
          % (out["loss"], float(np.linalg.norm(out["U"])), np.median(rel), rel.max()))
    assert np.median(rel) < 5e-2


# ------------------------------------------------------------------ 64^2 vs the FP64 reverse mode
@pytest.mark.parametrize("precise", [False, True])
def test_rollout64_gradient_fields_vs_fp64_reference_adjoint(gpu, precise):
    """64^2 jet, 64 steps, BFECC, 60 sweeps, checkpoint every 8: every
    gradient field (initial U, V, M and all 64 x 2 force fields) against the
    oracle's FP64 reverse mode of the same rollout.  The GPU trajectory is
    FP32, so the fields agree to FP32 accuracy, not bit for bit.  With
    precise_coords the forward and adjoint samples take their weights from
    face-relative offsets (the FP64 reverse mode's absolute coordinates are
    exact enough for either)."""
    side, steps = 64, 64
    f = gpu.Fluid(1.0, side, side, 1.0, auto_sync=False, scheme=1, num_iters=R_ITERS,
                  tb_depth=8, early_exit=False, UseBFECC=True, precise_coords=precise)
    scenes.jet_rollout_scene(f)
    n = f.numCells
    target = scenes.gaussian_target(f.NumX, f.NumY, seed=4, sigma=(2.5, 7.5))
    rng = np.random.default_rng(64)
    forces = [(rng.uniform(-0.02, 0.02, n).astype(np.float32),
               rng.uniform(-0.02, 0.02, n).astype(np.float32)) for _ in range(steps)]
    out = f.rollout_grad(DT, steps, target, forces, every=R_EVERY)
    f.download()
    o = OracleFluid(1.0, side, side, 1.0, prec=64, scheme=1, num_iters=R_ITERS, check_every=8,
                    early_exit=False, UseBFECC=True)
    o.S[:] = f.S
    srcs = [(1, j, 2.0, 0.0, 1.0, 1 | 2 | 8) for j in scenes.jet_rows(o)]
    F = np.stack([np.stack([a, b]) for a, b in forces]).astype(np.float64)
    ref = o.rollout_grad(DT, steps, target.astype(np.float64), F, srcs)
    assert out["loss"] == pytest.approx(ref["loss"], rel=1e-5)
    errs = {}
    for k in ("U", "V", "M"):
        errs[k] = float(np.linalg.norm(out[k] - ref[k]) / np.linalg.norm(ref[k]))
    gf = np.stack([np.stack([a, b]) for a, b in zip(out["force_u"], out["force_v"])])
    rf = np.stack([ref["force_u"], ref["force_v"]], axis=1)
    errs["forces"] = float(np.linalg.norm(gf - rf) / np.linalg.norm(rf))
    print("rollout64 relative L2 error of the gradient fields vs FP64 reverse mode:", errs)
    for k, e in errs.items():
        assert e < 1e-3, (k, e)


# ------------------------------------------------------------------ large-grid rollouts
def test_rollout_gradients_independent_of_sweep_blocking_on_large_grid(gpu):
    """700x1200 (165 Jacobi tiles: the solves of 8-sweep blocks run as one
    dataflow kernel, inside the captured forward, replay and adjoint graphs)
    against 4-sweep blocks (plain per-launch kernels).  Jacobi with a fixed
    sweep count does not depend on the blocking: the loss and the final
    state agree bit for bit; the gradients agree to the rounding of the
    adjoint's atomic scatter sums (whose order varies from run to run)."""
    outs = []
    for tb in (8, 4):
        f = gpu.Fluid(1.0, 700, 1200, 1.0, auto_sync=False, scheme=1, num_iters=24,
                      tb_depth=tb, early_exit=False, UseBFECC=True)
        scenes.jet_rollout_scene(f)
        n = f.numCells
        target = scenes.gaussian_target(f.NumX, f.NumY, seed=4)
        rng = np.random.default_rng(7)
        forces = [(rng.uniform(-0.02, 0.02, n).astype(np.float32),
                   rng.uniform(-0.02, 0.02, n).astype(np.float32)) for _ in range(4)]
        out = f.rollout_grad(DT, 4, target, forces, every=2)
        f.download()
        out["final"] = (f.U.copy(), f.V.copy(), f.M.copy())
        outs.append(out)
        del f
    a, b = outs
    assert a["loss"] == b["loss"]
    for x, y in zip(a["final"], b["final"]):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    pairs = [(a[k], b[k]) for k in ("U", "V", "M")]
    pairs += list(zip(a["force_u"], b["force_u"])) + list(zip(a["force_v"], b["force_v"]))
    for x, y in pairs:
        x, y = np.asarray(x, np.float64), np.asarray(y, np.float64)
        assert np.abs(x - y).max() <= 1e-5 * np.abs(y).max()
