"""Error paths exercised without a GPU fault: allocation failures injected
on the host, a Jacobi tile whose completion flag is never published (the
dependent tiles' bounded waits give up and the step reports FG_ERR_TIMEOUT,
after which the handle keeps working), and non-finite values reported by
the step statistics."""
import time

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import fluid_gb300

    fluid_gb300.build()
    return fluid_gb300


def test_allocation_failures_are_reported_and_leak_nothing(gpu):
    import torch
    from fluid_gb300 import _lib

    gpu.Fluid(1.0, 64, 48, 1.0)  # library and context set up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    failures = 0
    for n in range(0, 64):
        gpu.debug_fail_alloc(n)
        try:
            f = gpu.Fluid(1.0, 64, 48, 1.0)
        except gpu.FluidError as e:
            assert e.code in (_lib.FG_ERR_NOMEM, _lib.FG_ERR_CUDA), e
            failures += 1
            continue
        finally:
            gpu.debug_fail_alloc(-1)
        del f  # every allocation of a create succeeded: n is past them
        break
    assert failures > 20  # each of the create's allocations failed once
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0 - (2 << 20)
    f = gpu.Fluid(1.0, 64, 48, 1.0, scheme=1)
    scenes.jet_scene(f)
    scenes.jet_inject(f)
    f.Simulate(0.1)
    assert np.isfinite(f.U).all()


def test_stalled_jacobi_tile_times_out_and_handle_recovers(gpu):
    from fluid_gb300 import _lib

    w, h = 1100, 1500  # 322 Jacobi tiles: the dataflow kernel
    params = dict(scheme=1, num_iters=24, tb_depth=8, early_exit=False, UseBFECC=True)
    a = gpu.Fluid(1.0, w, h, 1.0, **params)
    b = gpu.Fluid(1.0, w, h, 1.0, **params)
    for f in (a, b):
        scenes.jet_scene(f)
        scenes.random_state(f, seed=3, amp=0.5)
    saved = {k: getattr(a, k).copy() for k in gpu.FIELDS}
    a.debug_stall_tile(40)
    t0 = time.time()
    a.Simulate(0.05)
    with pytest.raises(gpu.FluidError) as ei:
        a.stats()
    elapsed = time.time() - t0
    assert ei.value.code == _lib.FG_ERR_TIMEOUT
    assert elapsed < 30.0, elapsed
    # Disarmed, with the state restored, the handle steps like a fresh one.
    a.debug_stall_tile(-1)
    for k, v in saved.items():
        getattr(a, k)[:] = v
    a.mark_dirty()
    for f in (a, b):
        f.Simulate(0.05)
        f.stats()
    for k in ("U", "V", "M", "p"):
        x, y = getattr(a, k), getattr(b, k)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), k


def test_non_finite_values_are_reported(gpu):
    from fluid_gb300 import _lib

    f = gpu.Fluid(1.0, 40, 30, 1.0, scheme=1, early_exit=False, num_iters=16)
    scenes.jet_scene(f)
    scenes.jet_inject(f)
    f.Simulate(0.1)
    f.stats()
    f.U[10 * f.NumY + 12] = np.nan
    f.mark_dirty()
    f.Simulate(0.1)
    with pytest.raises(gpu.FluidError) as ei:
        f.stats()
    assert ei.value.code == _lib.FG_ERR_NONFINITE


def test_concurrent_dataflow_solves_on_two_streams(gpu):
    """Two handles (each with its own stream) whose steps run the cooperative
    dataflow Jacobi kernel at the same time: both finish without a timeout
    and equal the same steps run one handle after the other."""
    w, h = 1100, 1500
    params = dict(scheme=1, num_iters=40, tb_depth=8, early_exit=False, UseBFECC=True)

    def make(seed):
        f = gpu.Fluid(1.0, w, h, 1.0, auto_sync=False, **params)
        scenes.jet_scene(f)
        scenes.random_state(f, seed=seed, amp=0.5)
        f.mark_dirty()
        return f

    a, b = make(1), make(2)
    for _ in range(4):  # enqueued back to back: the two streams overlap
        a.Simulate(0.05)
        b.Simulate(0.05)
    a.synchronize()
    b.synchronize()
    a.stats()
    b.stats()
    for seed, f in ((1, a), (2, b)):
        r = make(seed)
        for _ in range(4):
            r.Simulate(0.05)
        r.synchronize()
        f.download()
        r.download()
        for k in ("U", "V", "M", "p"):
            x, y = getattr(f, k), getattr(r, k)
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), (seed, k)


def test_reference_sor_without_its_copies_falls_back_bitwise(gpu):
    """When the diagonal-major copies cannot be allocated (an injected
    allocation failure at the first step), the reference SOR runs on the
    row-major fields and still equals the oracle bit for bit."""
    from oracle.pyoracle import OracleFluid

    for w, h in ((60, 40), (300, 280)):  # one block, the cluster
        g = gpu.Fluid(1.0, w, h, 1.0, num_iters=30, UseBFECC=True, tolerance=1e-3)
        o = OracleFluid(1.0, w, h, 1.0, prec=32, num_iters=30, UseBFECC=True, tolerance=1e-3)
        for f in (g, o):
            scenes.jet_scene(f)
            scenes.random_state(f, seed=5, amp=0.5)
        g.mark_dirty()
        g.download()  # (queued edits and mirrors reach the device first)
        gpu.debug_fail_alloc(0)
        try:
            g.Simulate(0.1)
        finally:
            gpu.debug_fail_alloc(-1)
        o.Simulate(0.1)
        for k in ("U", "V", "M", "p"):
            a, b = getattr(g, k), getattr(o, k)
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (w, k)
        assert g.stats()["sweeps"] == o.stats()["sweeps"]
