"""Parity of the CUDA step (through the C ABI) with the CPU oracle.

* Reference scheme (LEXSOR, the default): the GPU step must equal the
  FP32-faithful restatement of pkg/fluid bit for bit, field by field,
  including the hidden staging buffers newU/newV/newM.
* Parallel scheme (JACOBI): bit-identical to the oracle's FP32 Jacobi
  variant for every temporal-blocking depth, and within the stated
  tolerances of the FP64 oracle: velocity max-abs error <= 1e-4 relative to
  the field's max, post-projection divergence L2 within 1e-5.
"""
import os

import numpy as np
import pytest

import reference_cases as rc
import scenes
from oracle.pyoracle import OracleFluid

pytestmark = pytest.mark.gpu

FIELDS = ("U", "V", "M", "p", "S", "newU", "newV", "newM")


@pytest.fixture(scope="module")
def gpu():
    import fluid_gb300

    fluid_gb300.build()
    return fluid_gb300


def both(gpu, width, height, density=1.0, h=1.0, **params):
    g = gpu.Fluid(density, width, height, h, **params)
    oparams = dict(params)
    oparams.pop("use_graphs", None)
    if "tb_depth" in oparams:
        oparams["check_every"] = oparams.pop("tb_depth")
    elif oparams.get("scheme", 0) == 1:
        oparams["check_every"] = 8
    o = OracleFluid(density, width, height, h, prec=32, **oparams)
    return g, o


def assert_bitwise(g, o, fields=FIELDS, where=""):
    for k in fields:
        a, b = getattr(g, k), getattr(o, k)
        if not np.array_equal(a.view(np.uint32), b.view(np.uint32)):
            bad = np.flatnonzero(a.view(np.uint32) != b.view(np.uint32))
            c = bad[0]
            raise AssertionError("%s %s differs at %d cells; first (i=%d, j=%d): gpu %r oracle %r"
                                 % (where, k, bad.size, c // g.NumY, c % g.NumY, a[c], b[c]))


# ------------------------------------------------------------------ reference tests on the GPU
@pytest.mark.parametrize("case", rc.ALL_CASES + [rc.case_multigrid_stability],
                         ids=lambda c: c.__name__)
def test_reference_case_on_gpu(gpu, case):
    case(lambda d, w, h, hh: gpu.Fluid(d, w, h, hh))


# ------------------------------------------------------------------ bitwise parity, reference scheme
@pytest.mark.parametrize("bfecc", [False, True])
def test_jet_128_bitwise_lexsor(gpu, bfecc):
    """Config 1 shape: 128x128 jet, 40 iterations, 60 steps, every field."""
    g, o = both(gpu, 128, 128, num_iters=40, UseBFECC=bfecc)
    for f in (g, o):
        scenes.jet_scene(f)
    for step in range(60):
        for f in (g, o):
            scenes.jet_inject(f)
            f.Simulate(0.1)
        if step % 20 == 19:
            assert_bitwise(g, o, where="step %d" % step)
    assert g.stats()["sweeps"] == o.stats()["sweeps"]


def test_all_stages_bitwise_lexsor(gpu):
    """Viscosity, confinement, turbulence, BFECC, an obstacle, odd sizes."""
    g, o = both(gpu, 37, 29, density=1000.0, h=0.01, ViscosityDiffusion=0.1, Confinement=0.3,
                PressureDamping=0.95, SmokeAdvection=1.2, UseBFECC=True, num_iters=20)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(15, 14, 4)
    for step in range(25):
        for f in (g, o):
            scenes.jet_inject(f, speed=4.0)
            if step % 7 == 0:
                f.ApplyForceRadius(20, 10, 3.0, -2.0, 3)
                f.AddSmoke(10, 20, 0.5)
            f.Simulate(1.0 / 120.0)
    assert_bitwise(g, o)


@pytest.mark.parametrize("amp,dt", [(0.5, 0.1), (20.0, 0.5)])
def test_bfecc_displacements_bitwise(gpu, amp, dt):
    """BFECC advection with departure points within a cell and many cells
    away (clamped at the walls), smoke diffusion, confinement, an obstacle
    and a grid that is no multiple of the thread blocks: every field stays
    bit for bit the oracle's."""
    g, o = both(gpu, 95, 70, num_iters=10, UseBFECC=True, ViscosityDiffusion=0.05,
                Confinement=0.1)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(40, 35, 7)
        scenes.random_state(f, seed=8, amp=amp)
    for _ in range(3):
        for f in (g, o):
            f.Simulate(dt)
    assert_bitwise(g, o)


@pytest.mark.parametrize("scheme", [0, 1])
def test_precise_coords_bitwise(gpu, scheme):
    """precise_coords: advection departure points as face index plus a
    displacement in cells.  The oracle restates the same arithmetic, so
    every field stays bit for bit its own: BFECC and plain steps, smoke
    diffusion, an obstacle, displacements below a cell and of several."""
    params = dict(scheme=scheme, num_iters=20, precise_coords=True, ViscosityDiffusion=0.05)
    if scheme == 1:
        params.update(tb_depth=4, early_exit=False, refine_sweeps=4)
    for bfecc, amp, dt in ((True, 0.5, 0.1), (True, 6.0, 0.5), (False, 3.0, 0.5)):
        g, o = both(gpu, 95, 70, UseBFECC=bfecc, **params)
        for f in (g, o):
            scenes.jet_scene(f)
            f.SetCircularObstacle(40, 35, 7)
            scenes.random_state(f, seed=9, amp=amp)
        for _ in range(3):
            for f in (g, o):
                scenes.jet_inject(f, speed=2.0)
                f.Simulate(dt)
        assert_bitwise(g, o, where="BFECC %s amp %g" % (bfecc, amp))


@pytest.mark.parametrize("w,h,cycles", [(70, 45, 2), (95, 70, 3), (333, 222, 2), (9, 30, 1),
                                         (1100, 1500, 1)])
def test_multigrid_jacobi_bitwise(gpu, w, h, cycles):
    """The MULTIGRID scheme (parallel V(2,2) cycles: damped Jacobi smoothing,
    summed residuals, bilinear correction, levels down to a side of 8)
    against the oracle's restatement, bit for bit: odd and even sizes, a
    grid with one coarse level, an obstacle, BFECC, confinement."""
    g, o = both(gpu, w, h, scheme=3, num_iters=cycles, early_exit=False, UseBFECC=True,
                Confinement=0.1)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(w // 3, h // 2, max(2, min(w, h) // 8))
    for _ in range(3):
        for f in (g, o):
            scenes.jet_inject(f, speed=2.0)
            f.Simulate(0.1)
    assert_bitwise(g, o, where="%dx%d" % (w, h))
    sg, so = g.stats(), o.stats()
    assert sg["sweeps"] == so["sweeps"] == cycles
    assert sg["resid_l2"] == pytest.approx(so["resid_l2"], rel=1e-9, abs=1e-12)


def test_multigrid_jacobi_residual_below_200_sweeps(gpu):
    """On a 512^2 lid-driven cavity one V-cycle leaves a smaller pressure
    residual than 200 Jacobi sweeps, and each further cycle shrinks it by
    about ten."""
    res = {}
    for name, kw in (("jacobi200", dict(scheme=1, num_iters=200, tb_depth=8)),
                     ("mg1", dict(scheme=3, num_iters=1)), ("mg2", dict(scheme=3, num_iters=2))):
        f = gpu.Fluid(1.0, 512, 512, 1.0, auto_sync=False, early_exit=False, UseBFECC=True, **kw)
        scenes.fast_walls(f, top=True, bottom=True, left=True, right=True)
        f.mark_dirty()
        i = np.arange(2, f.NumX - 2, dtype=np.int32)
        f.set_sources(i, np.full_like(i, f.NumY - 2), u=1.0, v=0.0,
                      mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY)
        for _ in range(3):
            f.Simulate(0.1)
        res[name] = f.stats()["resid_l2"]
    print("resid_l2 after 3 steps:", res)
    assert res["mg1"] < res["jacobi200"]
    assert res["mg2"] < res["mg1"] / 5


def test_multigrid_rejects_refinement_and_tiny_grids(gpu):
    from fluid_gb300 import FluidError

    with pytest.raises(FluidError):
        gpu.Fluid(1.0, 64, 64, 1.0, scheme=3, refine_sweeps=4)
    f = gpu.Fluid(1.0, 6, 40, 1.0, scheme=3, num_iters=1)
    with pytest.raises(FluidError):
        f.Simulate(0.1)


def test_early_exit_matches(gpu):
    g, o = both(gpu, 30, 20, num_iters=40)
    for f in (g, o):
        f.S[:] = 1.0
        f.ApplyForceRadius(10, 10, 0.01, 0.0, 3)
        f.Simulate(0.1)
    assert g.stats()["sweeps"] == o.stats()["sweeps"] < 40
    assert_bitwise(g, o)


def test_zero_field_exits_after_one_sweep(gpu):
    g, o = both(gpu, 40, 30)
    for f in (g, o):
        scenes.jet_scene(f)
        f.Simulate(1 / 120)
    assert g.stats()["sweeps"] == o.stats()["sweeps"] == 1
    assert_bitwise(g, o)


# ------------------------------------------------------------------ bitwise parity, Jacobi scheme
@pytest.mark.parametrize("tb", [1, 3, 8])
def test_jacobi_bitwise(gpu, tb):
    g, o = both(gpu, 70, 45, scheme=1, num_iters=30, tb_depth=tb, UseBFECC=True, Confinement=0.2)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(30, 22, 6)
    for _ in range(15):
        for f in (g, o):
            scenes.jet_inject(f, speed=3.0)
            f.Simulate(0.1)
    assert_bitwise(g, o)
    sg, so = g.stats(), o.stats()
    assert sg["sweeps"] == so["sweeps"]
    assert sg["resid_l2"] == pytest.approx(so["resid_l2"], rel=1e-9, abs=1e-12)


def test_jacobi_early_exit_bitwise(gpu):
    g, o = both(gpu, 33, 33, scheme=1, num_iters=200, tb_depth=4, tolerance=1e-3)
    for f in (g, o):
        f.S[:] = 1.0
        f.S[: f.NumY] = 0.0
        scenes.random_state(f, seed=3, amp=0.01)
        f.makeIncompressible(200, 0.1)
    assert g.stats()["sweeps"] == o.stats()["sweeps"] < 200
    assert_bitwise(g, o, fields=("U", "V", "p"))


def test_jacobi_refinement_bitwise(gpu):
    g, o = both(gpu, 50, 40, scheme=1, num_iters=40, tb_depth=8, refine_sweeps=16, early_exit=False)
    for f in (g, o):
        scenes.cavity_scene(f)
        scenes.random_state(f, seed=5)
        f.makeIncompressible(40, 0.1)
    assert_bitwise(g, o, fields=("U", "V", "p"))
    sg, so = g.stats(), o.stats()
    assert sg["resid_l2"] == pytest.approx(so["resid_l2"], rel=1e-9)


@pytest.mark.parametrize("w,h", [(70, 45), (333, 222), (1100, 1500), (9000, 100), (300, 2700)])
def test_jacobi_fixed_sweeps_bitwise(gpu, w, h):
    """Fixed sweep counts in full 8-sweep launches against the oracle, bit for
    bit: the per-launch kernel on 4-warp regions (70x45, 333x222: fewer 8-warp
    regions than SMs) and the dataflow kernel (1100x1500: 322 tiles; 9000x100:
    one tile column of 188 tiles; 300x2700: 7 tile rows of 25)."""
    g, o = both(gpu, w, h, scheme=1, num_iters=40, tb_depth=8, early_exit=False, UseBFECC=True)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(w // 3, h // 2, max(3, min(w, h) // 8))
    for _ in range(3):
        for f in (g, o):
            scenes.jet_inject(f, speed=3.0)
            f.Simulate(0.1)
    assert_bitwise(g, o, where="%dx%d" % (w, h))


@pytest.mark.parametrize("w,h", [(1100, 1500), (400, 2700)])
def test_jacobi_4_sweep_launches_bitwise(gpu, w, h):
    """tb_depth 4 on grids large enough for the dataflow kernel: ten 4-sweep
    launches of the per-launch kernel (the dataflow kernel runs 8-sweep
    phases only), bit for bit against the oracle."""
    g, o = both(gpu, w, h, scheme=1, num_iters=40, tb_depth=4, early_exit=False, UseBFECC=True)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(w // 3, h // 2, max(3, min(w, h) // 8))
    for _ in range(3):
        for f in (g, o):
            scenes.jet_inject(f, speed=3.0)
            f.Simulate(0.1)
    assert_bitwise(g, o, where="%dx%d" % (w, h))
    assert g.stats()["jacobi_kernel"] == gpu.JACOBI_KERNEL_SWEEP


def test_jacobi_dataflow_then_partial_launch_bitwise(gpu):
    """44 sweeps at 1100x1500: five dataflow phases, then one 4-sweep launch
    of the per-launch kernel continuing from the dataflow result."""
    g, o = both(gpu, 1100, 1500, scheme=1, num_iters=44, tb_depth=8, early_exit=False)
    for f in (g, o):
        scenes.cavity_scene(f)
        scenes.random_state(f, seed=21)
        f.makeIncompressible(44, 0.1)
    assert_bitwise(g, o, fields=("U", "V", "p"))
    assert g.stats()["sweeps"] == 44
    assert g.stats()["jacobi_kernel"] == gpu.JACOBI_KERNEL_DATAFLOW


def test_jacobi_fixed_sweeps_2048_matches_checked_launches(gpu):
    """At 2046x2046 (817 tiles) the unchecked launches give the same fields
    as the residual-checking kernel with a tolerance that never stops."""
    fs = [gpu.Fluid(1.0, 2046, 2046, 1.0, scheme=1, num_iters=200, tb_depth=8, UseBFECC=True,
                    early_exit=ee, tolerance=0.0) for ee in (False, True)]
    for f in fs:
        scenes.cavity_scene(f)
        scenes.random_state(f, seed=11)
    for _ in range(2):
        for f in fs:
            f.Simulate(0.05)
    for k in ("U", "V", "p", "M"):
        a, b = getattr(fs[0], k), getattr(fs[1], k)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), k
    assert fs[0].stats()["sweeps"] == fs[1].stats()["sweeps"] == 200
    assert fs[0].stats()["jacobi_kernel"] == gpu.JACOBI_KERNEL_DATAFLOW
    assert fs[1].stats()["jacobi_kernel"] == gpu.JACOBI_KERNEL_SWEEP


FRESH_PROCESS = r"""
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
import fluid_gb300 as fg
# No CUDA call before the handle: the library creates the context itself.
f = fg.Fluid(1.0, 1200, 800, 1.0, auto_sync=False, scheme=1, num_iters=40, tb_depth=8,
             early_exit=False)
S = f.S.reshape(f.NumX, f.NumY)
S[:] = 1.0
S[:, 0] = S[:, -1] = S[0, :] = 0.0
f.mark_dirty()
kinds = []
for _ in range(3):
    f.Simulate(0.1)  # the first call captures the step graph, the others replay it
    kinds.append(f.stats()["jacobi_kernel"])
print("KINDS", kinds)
assert kinds == [fg.JACOBI_KERNEL_DATAFLOW] * 3, kinds
"""


def test_dataflow_kernel_in_graph_of_handle_made_before_any_cuda_call(gpu):
    """A handle created in a process that has made no CUDA call yet (no
    context exists) still captures the dataflow kernel in its step graph:
    the per-context set-up needs a current context, which the library
    creates before it."""
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FRESH_PROCESS, root], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "KINDS [3, 3, 3]" in r.stdout


def test_jacobi_against_fp64_oracle(gpu):
    """Per-step error of the FP32 GPU step against the FP64 oracle."""
    g = gpu.Fluid(1.0, 96, 64, 1.0, scheme=1, num_iters=100, tb_depth=8, UseBFECC=True,
                  Confinement=0.3)
    o = OracleFluid(1.0, 96, 64, 1.0, prec=64, scheme=1, num_iters=100, check_every=8,
                    UseBFECC=True, Confinement=0.3)
    for f in (g, o):
        scenes.karman_scene(f, radius=8)
    for _ in range(5):
        for f in (g, o):
            scenes.karman_inflow(f)
            f.Simulate(0.1)
    scale = float(np.abs(o.U).max())
    err = max(float(np.abs(g.U.astype(np.float64) - o.U).max()),
              float(np.abs(g.V.astype(np.float64) - o.V).max())) / scale
    assert err <= 1e-4, err
    assert abs(g.stats()["div_l2_post"] - o.stats()["div_l2_post"]) <= 1e-5


@pytest.mark.parametrize("scheme", [0, 1])
def test_app_size_bitwise(gpu, scheme):
    """The reference app's grid (300 x 251, main/main.go:22-23) with BFECC,
    the outer correction (parallel scheme) and the app's jet; large enough
    for the multi-block reductions and several Jacobi tiles."""
    params = dict(scheme=scheme, num_iters=24, UseBFECC=True, early_exit=scheme == 0)
    if scheme == 1:
        params.update(tb_depth=8, refine_sweeps=8)
    g, o = both(gpu, 300, 251, density=1000.0, h=0.01, **params)
    for f in (g, o):
        scenes.apply_walls(f, top=True, bottom=True, left=True, right=False)
    for _ in range(4):
        for f in (g, o):
            n = f.NumY
            for j in range(f.NumY // 2 - 50, f.NumY // 2 + 50):
                f.SetVelocity(1, j, 4.0, 0.0)
                f.AddSmoke(1, j, 1.0)
            f.Simulate(1.0 / 120.0)
    assert_bitwise(g, o)
    sg, so = g.stats(), o.stats()
    for k in ("div_l2_post", "div_max_post", "smoke_mass"):
        assert sg[k] == pytest.approx(so[k], rel=1e-9, abs=1e-12), k
    assert sg["div_count_post"] == so["div_count_post"]
    if scheme == 1:
        assert sg["resid_l2"] == pytest.approx(so["resid_l2"], rel=1e-9, abs=1e-12)
        assert sg["resid_max"] == pytest.approx(so["resid_max"], rel=1e-9, abs=1e-12)


# ------------------------------------------------------------------ API behaviour
def test_graphs_do_not_change_results(gpu):
    a = gpu.Fluid(1.0, 40, 30, 1.0, use_graphs=True, UseBFECC=True, num_iters=20)
    b = gpu.Fluid(1.0, 40, 30, 1.0, use_graphs=False, UseBFECC=True, num_iters=20)
    for f in (a, b):
        scenes.jet_scene(f)
    for _ in range(12):
        for f in (a, b):
            scenes.jet_inject(f)
            f.Simulate(0.1)
    for k in FIELDS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


def test_explicit_sync_mode_matches_auto(gpu):
    """auto_sync=False: tool calls only, device authoritative, one download."""
    a = gpu.Fluid(1.0, 48, 40, 1.0, num_iters=20)
    b = gpu.Fluid(1.0, 48, 40, 1.0, num_iters=20, auto_sync=False)
    for f in (a, b):
        scenes.apply_walls(f)
    for step in range(10):
        for f in (a, b):
            for j in scenes.jet_rows(f):
                f.SetVelocity(1, j, 2.0, 0.0)
                f.AddSmoke(1, j, 1.0)
            f.Simulate(0.1)
    b.download()
    for k in FIELDS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


def test_views_match_oracle(gpu):
    g, o = both(gpu, 30, 25, num_iters=10)
    for f in (g, o):
        scenes.jet_scene(f)
    for _ in range(10):
        for f in (g, o):
            scenes.jet_inject(f, speed=5.0)
            f.Simulate(0.05)
    assert g.MaxDivergence() == np.float32(o.MaxDivergence())
    for name in ("Vorticity", "VelocityMagnitude"):
        vg, vo = getattr(g, name)(), getattr(o, name)()
        assert np.array_equal(vg.values, vo.values), name
        assert vg.MinValue == np.float32(vo.MinValue) and vg.MaxValue == np.float32(vo.MaxValue)
    for x, y in ((3.3, 7.1), (0.0, 0.0), (100.0, 100.0), (12.5, 12.5)):
        ug, vg_ = g.SampleVelocity(x, y)
        uo, vo_ = o.SampleVelocity(x, y)
        assert (ug, vg_) == (np.float32(uo), np.float32(vo_))
    assert g.GetAdaptiveTimeStep(0.08) == np.float32(o.GetAdaptiveTimeStep(0.08))
    sm = g.Smoke()
    assert sm.MinValue == float(o.M.min()) and sm.MaxValue == float(o.M.max())


def test_stage_entry_points_bitwise(gpu):
    g, o = both(gpu, 21, 17, ViscosityDiffusion=0.2, Confinement=1.0)
    for f in (g, o):
        f.S[:] = 1.0
        f.S[5 * f.NumY + 5] = 0.0
        scenes.random_state(f, seed=7)
    for name, args in (("applyViscosity", (0.1,)), ("makeIncompressible", (12, 0.1)),
                       ("applyVorticityConfinement", (0.1,)), ("addTurbulence", (0.1,)),
                       ("handleBorders", ()), ("advectVelocity", (0.1,)), ("advectSmoke", (0.1,)),
                       ("advectVelocityBFECC", (0.1,)), ("advectSmokeBFECC", (0.1,))):
        for f in (g, o):
            getattr(f, name)(*args)
        assert_bitwise(g, o, where=name)


@pytest.mark.parametrize("w,h", [(1, 1), (2, 3), (3, 30), (31, 7), (33, 34), (62, 29), (95, 70),
                                 (130, 66)])
def test_bfecc_stages_bitwise_across_strip_alignments(gpu, w, h):
    """The velocity passes run four rows per thread, blocks of 32 x 32
    cells; strips that reach the ghost ring or pass the last row run cell by
    cell.  Grids whose rows end inside a strip, with fewer rows than a
    strip, or one cell wide, with an obstacle and random state: BFECC and
    plain advection stay bit for bit the oracle's."""
    g, o = both(gpu, w, h, Confinement=0.3)
    for f in (g, o):
        f.S[:] = 1.0
        if w > 4 and h > 4:
            f.S[(w // 2) * f.NumY + h // 2] = 0.0
        scenes.random_state(f, seed=w * 1000 + h, amp=2.0)
    for name in ("advectVelocityBFECC", "advectSmokeBFECC", "advectVelocity", "advectSmoke"):
        for f in (g, o):
            getattr(f, name)(0.4)
        assert_bitwise(g, o, where="%s %dx%d" % (name, w, h))


def test_bfecc_clamp_ties_and_nan_centres(gpu):
    """The velocity correction forms clampToNeighbors' 3x3 range with min /
    max trees; it must end on the same element as the reference's scan,
    including -0/+0 ties (a zero extreme with a nonzero centre, decided by
    scan order), zero centres, and NaN centres (never replaced) or NaN
    neighbours (skipped).  Fields drawn from {-1, -0, +0, 1/2, 1} with a
    few NaNs; every bit equal to the oracle's except NaN payloads, which
    the two machines form differently (all NaNs compare equal here)."""
    g, o = both(gpu, 61, 43)
    rng = np.random.default_rng(12)
    vals = np.array([-1.0, -0.0, 0.0, 0.5, 1.0], np.float32)
    U = vals[rng.integers(0, 5, g.numCells)]
    V = vals[rng.integers(0, 5, g.numCells)]
    for a in (U, V):
        a[rng.integers(0, g.numCells, 6)] = np.nan
    for f in (g, o):
        f.S[:] = 1.0
        f.U[:] = U
        f.V[:] = V
        f.advectVelocityBFECC(0.3)
    for k in ("U", "V", "newU", "newV"):
        a, b = getattr(g, k), getattr(o, k)
        same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
        assert same.all(), (k, int((~same).sum()))
    # The ties occur: zero extremes with a nonzero centre are in the data.
    assert (np.signbit(U) & (U == 0)).sum() > 100


def test_invalid_mask_fails_loudly(gpu):
    f = gpu.Fluid(1.0, 8, 8, 1.0)
    f.S[:] = 0.5
    with pytest.raises(gpu.FluidError) as e:
        f.Simulate(0.1)
    assert e.value.code == -5


@pytest.mark.parametrize("w,h,early,iters", [(300, 280, True, 30), (300, 280, False, 30),
                                              (640, 300, True, 30), (300, 280, False, 40),
                                              (300, 280, True, 40)])
def test_lexsor_cluster_bitwise(gpu, w, h, early, iters):
    """Grids whose diagonals hold at least 256 cells: the reference SOR runs
    as the cluster form of the wavefront (30 sweeps) or, with 32 sweeps or
    more, on every SM with a grid barrier per step; with the early exit as
    the speculative passes; bit for bit, sweep count included."""
    g, o = both(gpu, w, h, num_iters=iters, UseBFECC=True, early_exit=early, tolerance=1e-3)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(w // 3, h // 2, 12)
    for _ in range(4):
        for f in (g, o):
            scenes.jet_inject(f, speed=3.0)
            f.Simulate(0.1)
    assert_bitwise(g, o, where="%dx%d early %s" % (w, h, early))
    assert g.stats()["sweeps"] == o.stats()["sweeps"]


@pytest.mark.parametrize("w,h", [(8200, 10), (8000, 300)])
def test_lexsor_bookkeeping_early_exit_bitwise(gpu, w, h):
    """Grids whose diagonals outnumber the sweep ring (NX + NY > 8190): the
    early exit runs with the step-by-step bookkeeping (one block; the
    cluster with the bookkeeping in rank 0's shared memory), bit for bit."""
    g, o = both(gpu, w, h, num_iters=30, UseBFECC=True, tolerance=1e-3)
    for f in (g, o):
        scenes.jet_scene(f)
        scenes.jet_inject(f, speed=3.0)
        f.Simulate(0.1)
    assert_bitwise(g, o, where="%dx%d" % (w, h))
    assert g.stats()["sweeps"] == o.stats()["sweeps"]


@pytest.mark.parametrize("w,h", [(40, 30), (320, 300), (4000, 100)])
def test_lexsor_early_exit_mid_solve_bitwise(gpu, w, h):
    """A nearly divergence-free state whose solve stops part way: the
    speculative early exit (all sweeps, then a re-run of exactly the sweeps
    the serial loop makes) on one block, on the cluster, and with more than
    2048 sweeps' worth of diagonals in the ring (4000x100), bit for bit."""
    g, o = both(gpu, w, h, num_iters=60, tolerance=1e-3)
    for f in (g, o):
        f.S[:] = 1.0
        f.S[: f.NumY] = 0.0
        scenes.random_state(f, seed=17, amp=1e-3)
        f.makeIncompressible(60, 0.1)
    sg, so = g.stats(), o.stats()
    assert sg["sweeps"] == so["sweeps"] < 60
    assert_bitwise(g, o, fields=("U", "V", "p"))


@pytest.mark.parametrize("w,h,bfecc", [(70, 45, True), (33, 20, False), (64, 64, True),
                                         (12, 9, False), (600, 520, True)])
def test_multigrid_bitwise(gpu, w, h, bfecc):
    """UseMultigrid (fluid.go:559-758, 1122-1149): the V-cycle with the
    reference's serial smoothers and coarse Gauss-Seidel, bit for bit, on
    odd and even grid sizes, with obstacles and the app's jet."""
    g, o = both(gpu, w, h, UseMultigrid=True, UseBFECC=bfecc, Confinement=0.1)
    for f in (g, o):
        scenes.jet_scene(f)
        if w > 20:
            f.SetCircularObstacle(w // 2, h // 2, 4)
    for _ in range(10):
        for f in (g, o):
            scenes.jet_inject(f, speed=2.5)
            f.Simulate(0.1)
    assert_bitwise(g, o)
    assert g.stats()["sweeps"] == o.stats()["sweeps"]


def test_multigrid_early_break(gpu):
    """A field already divergence-free leaves the V-cycle after the first
    three smoothing sweeps."""
    g, o = both(gpu, 24, 18, UseMultigrid=True)
    for f in (g, o):
        scenes.jet_scene(f)
        f.Simulate(0.1)
    assert g.stats()["sweeps"] == o.stats()["sweeps"] == 3
    assert_bitwise(g, o)


@pytest.mark.parametrize("w,h", [(1, 1), (1, 7), (9, 1), (2, 3), (65, 33)])
def test_small_and_ragged_grids_bitwise(gpu, w, h):
    for scheme in (0, 1):
        g, o = both(gpu, w, h, scheme=scheme, num_iters=6, tb_depth=2, UseBFECC=True)
        for f in (g, o):
            f.S[:] = 1.0
            f.S[: f.NumY] = 0.0
            scenes.random_state(f, seed=w * 100 + h)
        for _ in range(3):
            for f in (g, o):
                f.Simulate(0.05)
        assert_bitwise(g, o, where="%dx%d scheme %d" % (w, h, scheme))


def test_karman_512x256_fp32_against_fp64_every_100_steps(gpu):
    """The Karman vortex street at 512x256 (disc r = 24 at (128, 128), inflow
    U = 1 on the left, open right, walls top and bottom, U0 = 1 + U(-1e-3,
    1e-3) seed 2, BFECC, confinement 0.3, 100 Jacobi sweeps) for 1000 steps.
    Every 100 steps an FP64 oracle is set to the GPU's state and both run
    the next step: that step's velocity max-abs error (relative to max |U|)
    must stay within 1e-4 and its post-projection divergence L2 within 1e-5
    of FP64.  A free-running FP64 oracle beside it shows how the two
    trajectories of this vortex-shedding (chaotic) flow drift apart over
    hundreds of steps; that drift is reported, not bounded."""
    import os

    W, H, R = 512, 256, 24
    th = os.cpu_count() or 1
    params = dict(scheme=1, num_iters=100, early_exit=False, UseBFECC=True, Confinement=0.3)
    g = gpu.Fluid(1.0, W, H, 1.0, auto_sync=False, tb_depth=4, **params)
    free = OracleFluid(1.0, W, H, 1.0, prec=64, threads=th, check_every=4, **params)
    sync = OracleFluid(1.0, W, H, 1.0, prec=64, threads=th, check_every=4, **params)
    scenes.fast_walls(g, top=True, bottom=True, left=False, right=False)
    g.mark_dirty()
    g.SetCircularObstacle(128, 128, R)
    g.download()
    rng = np.random.default_rng(2)
    U0 = ((1.0 + rng.uniform(-1e-3, 1e-3, g.numCells)) * (g.S != 0)).reshape(g.NumX, g.NumY)
    U0[0, :] = 0.0
    U0[:, 0] = U0[:, -1] = 0.0
    g.U[:] = U0.ravel()
    g.mark_dirty()
    for o in (free, sync):
        o.S[:] = g.S
        o.U[:] = g.U
    rows = np.arange(1, g.NumY - 1, dtype=np.int32)
    g.set_sources(np.ones_like(rows), rows, u=1.0, v=0.0, mode=g.SRC_SKIP_SOLID | g.SRC_SET_VELOCITY)
    state = ("U", "V", "M", "newU", "newV", "newM")
    per_step, drift = [], []
    for step in range(1, 1001):
        check = step % 100 == 1
        if check:
            g.download()
            for k in state:
                getattr(sync, k)[:] = getattr(g, k)
        g.Simulate(0.1)
        scenes.karman_inflow(free)
        free.Simulate(0.1)
        if check:
            scenes.karman_inflow(sync)
            sync.Simulate(0.1)
            g.download()
            scale = float(np.abs(sync.U).max())
            err = max(float(np.abs(g.U.astype(np.float64) - sync.U).max()),
                      float(np.abs(g.V.astype(np.float64) - sync.V).max())) / scale
            per_step.append((step, err, g.stats()["div_l2_post"], sync.stats()["div_l2_post"]))
        if step % 100 == 0:
            g.download()
            scale = float(np.abs(free.U).max())
            err = max(float(np.abs(g.U.astype(np.float64) - free.U).max()),
                      float(np.abs(g.V.astype(np.float64) - free.V).max())) / scale
            drift.append((step, err, g.stats()["div_l2_post"], free.stats()["div_l2_post"]))
    print("one step from the GPU state: step, vel max-abs err / max|U|, div L2 GPU, div L2 FP64")
    for r in per_step:
        print("%4d  %.3e  %.6e  %.6e" % r)
    print("free-running: step, vel max-abs err / max|U|, div L2 GPU, div L2 FP64")
    for r in drift:
        print("%4d  %.3e  %.4e  %.4e" % r)
    for step, err, dg, do in per_step:
        assert err <= 1e-4, (step, err)
        assert abs(dg - do) <= 1e-5, (step, dg, do)


def test_async_smoke_download_frames(gpu):
    """The frame loop with fg_download_async / fg_download_wait: every
    frame's smoke equals a synchronous download's, with smoke sources and
    smoke edits writing M in place between frames."""
    a = gpu.Fluid(1.0, 40, 30, 1.0, auto_sync=False, UseBFECC=True)
    b = gpu.Fluid(1.0, 40, 30, 1.0, auto_sync=False, UseBFECC=True)
    for f in (a, b):
        scenes.fast_walls(f)
        f.mark_dirty()
        rows = np.array(list(scenes.jet_rows(f)), np.int32)
        f.set_sources(np.ones_like(rows), rows, u=2.0, v=0.0, smoke=0.5,
                      mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY | f.SRC_ADD_SMOKE)
    prev = None
    for k in range(12):
        for f in (a, b):
            if k % 4 == 3:
                f.AddSmoke(10, 10, 1.0)
            f.Simulate(0.1)
        a.download_wait()
        if prev is not None:
            assert np.array_equal(a.M.view(np.uint32), prev.view(np.uint32)), k
        a.download_async()
        b.download(1 << gpu.FIELDS["M"])
        prev = b.M.copy()
    a.download_wait()
    assert np.array_equal(a.M.view(np.uint32), prev.view(np.uint32))


@pytest.mark.parametrize("scheme,graphs", [(1, True), (0, True), (1, False)])
def test_async_smoke_download_deferred_paths(gpu, scheme, graphs):
    """fg_download_async leaves the copy to the next step, which starts it
    once its projection is done; every other path starts it at once.  The
    mirror must hold the smoke of the frame the call was made after: with
    two steps before the wait (the second waits for the copy before it
    overwrites that buffer), a stage call or a view in between, a wait right
    away, and a synchronous download while a copy is deferred."""
    kw = dict(scheme=scheme, UseBFECC=True, use_graphs=graphs, auto_sync=False)
    if scheme == 1:
        kw.update(num_iters=24, tb_depth=8, early_exit=False)
    a = gpu.Fluid(1.0, 150, 170, 1.0, **kw)
    b = gpu.Fluid(1.0, 150, 170, 1.0, **kw)
    for f in (a, b):
        scenes.fast_walls(f)
        f.mark_dirty()
        rows = np.array(list(scenes.jet_rows(f)), np.int32)
        f.set_sources(np.ones_like(rows), rows, u=2.0, v=0.0, smoke=0.5,
                      mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY | f.SRC_SET_SMOKE)
    mbit = 1 << gpu.FIELDS["M"]

    def ref():
        b.download(mbit)
        return b.M.copy()

    def same(x, y, what):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), what

    for f in (a, b):
        for _ in range(3):
            f.Simulate(0.1)
    for rnd in range(3):
        want = ref()
        # Two steps before the wait.
        a.download_async()
        for f in (a, b):
            f.Simulate(0.1)
            f.Simulate(0.1)
        a.download_wait()
        same(a.M, want, "two steps, round %d" % rnd)
        # A stage call and a view before the wait.
        want = ref()
        a.download_async()
        for f in (a, b):
            f.advectSmoke(0.05)
            f.Vorticity()
        a.download_wait()
        same(a.M, want, "stage and view, round %d" % rnd)
        # The wait at once, then a synchronous download while one is deferred.
        want = ref()
        a.download_async()
        a.download_wait()
        same(a.M, want, "wait at once, round %d" % rnd)
        a.download_async()
        for f in (a, b):
            f.Simulate(0.1)
        a.download(mbit)
        same(a.M, ref(), "synchronous download, round %d" % rnd)


def test_jet128_against_golden_fixtures(gpu):
    """The 128x128 jet of the golden fixtures (200 steps, 40 iterations, the
    reference's early exit): the GPU's reference scheme equals the FP32
    fixture bit for bit, and stays within 1e-4 of max |U| (velocity) of the
    FP64 fixture."""
    import os
    import sys

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_golden

    gold = np.load(os.path.join(here, "jet128_fp32.npz"))
    f, trace = make_golden.run(lambda *a: gpu.Fluid(*a))
    for k in ("U", "V", "M", "p", "newU", "newV", "newM", "S"):
        a = np.asarray(getattr(f, k))
        assert np.array_equal(a.view(np.uint32), gold[k].view(np.uint32)), k
    gold64 = np.load(os.path.join(here, "jet128_fp64.npz"))
    scale = float(np.abs(gold64["U"]).max())
    err = max(float(np.abs(f.U.astype(np.float64) - gold64["U"]).max()),
              float(np.abs(f.V.astype(np.float64) - gold64["V"]).max())) / scale
    print("jet128 after 200 steps: velocity max-abs error vs FP64 / max|U| = %.3e" % err)
    assert err <= 1e-4, err
