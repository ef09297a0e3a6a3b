"""Batched ensembles (fg_batch_create): many scenes of different sizes
stepped by one launch per stage must give every scene the same bits as
stepping its own handle, before and after autotuning, and the same
gradients (to the FP32 atomics' reproducibility) in recorded rollouts."""
import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

# Grids (w + 2) x (h + 2): Jacobi regions of 64 rows x 128 columns cut them
# into one to three regions per axis, starting and ending at scene edges.
SIDES = [(30, 20), (64, 48), (17, 33), (100, 90), (40, 40), (128, 64), (9, 9), (150, 140),
         (60, 250), (62, 126)]
DT = 0.1


@pytest.fixture(scope="module")
def gpu():
    import fluid_gb300

    fluid_gb300.build()
    return fluid_gb300


def make_scenes(gpu, seed=3, **params):
    rng = np.random.default_rng(seed)
    out = []
    for k, (w, h) in enumerate(SIDES):
        p = dict(scheme=1, tb_depth=8, early_exit=False, UseBFECC=True, auto_sync=False)
        p.update(params)
        p["num_iters"] = int(rng.integers(10, 41))
        f = gpu.Fluid(1.0, w, h, 1.0, **p)
        scenes.ensemble_scene(f, np.random.default_rng(100 + k), radius=(2.0, 8.0))
        out.append(f)
    return out


FIELDS = ("U", "V", "M", "newU", "newV", "newM", "p")


def assert_same(a, b, where):
    a.download()
    b.download()
    for k in FIELDS:
        x, y = getattr(a, k), getattr(b, k)
        if not np.array_equal(x.view(np.uint32), y.view(np.uint32)):
            bad = np.flatnonzero(x.view(np.uint32) != y.view(np.uint32))
            raise AssertionError("%s: %s differs at %d cells (first %d: %r vs %r)"
                                 % (where, k, bad.size, bad[0], x[bad[0]], y[bad[0]]))


@pytest.mark.parametrize("conf", [0.0, 0.3])
def test_batch_step_bitwise_equals_single_scenes(gpu, conf):
    ref = make_scenes(gpu, Confinement=conf)
    mem = make_scenes(gpu, Confinement=conf)
    batch = gpu.Batch(mem)
    for _ in range(12):
        for f in ref:
            f.Simulate(DT)
        batch.step(DT)
    batch.scatter()
    for k, (a, b) in enumerate(zip(ref, mem)):
        assert_same(a, b, "scene %d" % k)


@pytest.mark.parametrize("omega,tb", [(0.8, 8), (1.0, 4), (0.8, 6)])
def test_batch_damped_and_short_blocks_bitwise(gpu, omega, tb):
    """Damped Jacobi (omega < 1: the relaxation term in every sweep) and
    blocking depths below 8 (every launch's sweeps counted at run time),
    each scene against its own handle, bit for bit."""
    ref = make_scenes(gpu, seed=8, jacobi_omega=omega, tb_depth=tb)
    mem = make_scenes(gpu, seed=8, jacobi_omega=omega, tb_depth=tb)
    batch = gpu.Batch(mem)
    for _ in range(6):
        for f in ref:
            f.Simulate(DT)
        batch.step(DT)
    batch.scatter()
    for k, (a, b) in enumerate(zip(ref, mem)):
        assert_same(a, b, "scene %d (omega %g, tb %d)" % (k, omega, tb))


def test_autotune_keeps_results(gpu):
    ref = make_scenes(gpu, seed=4)
    mem = make_scenes(gpu, seed=4)
    batch = gpu.Batch(mem)
    for _ in range(3):
        for f in ref:
            f.Simulate(DT)
        batch.step(DT)
    tb, bx, by, ms = batch.autotune(DT, reps=2)
    assert tb in (4, 6, 8) and bx * by in (128, 256, 512) and ms > 0
    for _ in range(5):
        for f in ref:
            f.Simulate(DT)
        batch.step(DT)
    batch.scatter()
    for k, (a, b) in enumerate(zip(ref, mem)):
        assert_same(a, b, "scene %d after autotune" % k)


def test_batch_rollout_gradients_match_single_scenes(gpu):
    ref = make_scenes(gpu, seed=6)
    mem = make_scenes(gpu, seed=6)
    targets = [scenes.gaussian_target(f.NumX, f.NumY, seed=10 + k, sigma=(2.0, 6.0))
               for k, f in enumerate(ref)]
    batch = gpu.Batch(mem)
    losses, grads = batch.rollout_grad(DT, 10, targets, every=4)
    for k, f in enumerate(ref):
        out = f.rollout_grad(DT, 10, targets[k], every=4)
        assert losses[k] == pytest.approx(out["loss"], rel=1e-12)
        for key in ("U", "V", "M"):
            scale = max(float(np.abs(out[key]).max()), 1e-30)
            err = float(np.abs(grads[k][key] - out[key]).max()) / scale
            assert err <= 1e-5, (k, key, err)
    # Both reverse passes leave the state at the end of the forward pass.
    batch.scatter()
    for k, (a, b) in enumerate(zip(ref, mem)):
        assert_same(a, b, "scene %d after the rollout" % k)


def test_batch_rejects_single_scene_calls_and_mixed_params(gpu):
    from fluid_gb300 import FluidError

    mem = make_scenes(gpu, seed=7)
    batch = gpu.Batch(mem)
    import ctypes

    L = batch._L
    mn, mx = ctypes.c_float(), ctypes.c_float()
    assert L.fg_field_min_max(batch.handle, 0, ctypes.byref(mn), ctypes.byref(mx)) == -4
    assert L.fg_max_divergence(batch.handle, ctypes.byref(mn)) == -4
    assert L.fg_set_velocity(batch.handle, 1, 1, 1.0, 0.0) == -4
    a = gpu.Fluid(1.0, 8, 8, 1.0, scheme=1, early_exit=False, UseBFECC=True)
    b = gpu.Fluid(1.0, 8, 8, 1.0, scheme=1, early_exit=False, UseBFECC=False)
    with pytest.raises(FluidError):
        gpu.Batch([a, b])
    c = gpu.Fluid(1.0, 8, 8, 1.0)  # reference scheme
    with pytest.raises(FluidError):
        gpu.Batch([c])
