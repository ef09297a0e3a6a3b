"""fg_project_noalloc: the projection for callers that cannot allocate.

Callers that cannot call cudaMalloc when they project (an engine whose
allocator owns the device memory, a frame loop that must not risk the
synchronisation an allocation can cause) pass their own device fields and
the library uses a fixed scratch array instead of allocating.  The test
calls it through the C ABI on caller-owned buffers (torch tensors with a
pitch unlike the library's own) twice in a row, with different grids, and
checks U, V and p bit for bit against the handle-based projection
fg_make_incompressible with the same settings.  This file sorts last so a
run that stops at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    import fluid_gb300
    from fluid_gb300 import _lib

    fluid_gb300.build()
    torch.cuda.init()
    return torch, fluid_gb300, _lib.lib(), _lib


def reference_projection(fluid_gb300, width, height, seed, iters, tb, early_exit, tol, dt):
    f = fluid_gb300.Fluid(1.0, width, height, 1.0, scheme=fluid_gb300.SCHEME_JACOBI,
                          num_iters=iters, tb_depth=tb, early_exit=early_exit, tolerance=tol)
    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = S[:, -1] = S[0, :] = 0.0
    f.SetCircularObstacle(f.NumX // 3, f.NumY // 2, max(2, min(width, height) // 8))
    scenes.random_state(f, seed=seed, amp=0.5, smoke=False)
    inputs = {k: getattr(f, k).copy() for k in ("U", "V", "S")}
    f.makeIncompressible(iters, dt)
    return inputs, {k: getattr(f, k).copy() for k in ("U", "V", "p")}, f.stats()["sweeps"]


def noalloc_projection(torch, L, inputs, nx, ny, iters, tb, early_exit, tol, dt):
    pitch = ny + 5  # any pitch >= num_y
    dev = {}
    for k in ("U", "V", "S"):
        t = torch.zeros((nx, pitch), dtype=torch.float32, device="cuda")
        t[:, :ny] = torch.from_numpy(inputs[k].reshape(nx, ny)).cuda()
        dev[k] = t
    p = torch.full((nx, pitch), 123.0, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.fg_project_noalloc(dev["U"].data_ptr(), dev["V"].data_ptr(), p.data_ptr(),
                              dev["S"].data_ptr(), nx, ny, pitch, ctypes.c_float(1.0),
                              ctypes.c_float(1.0), ctypes.c_float(dt), iters, ctypes.c_float(1.0),
                              ctypes.c_float(1.0), tb, int(early_exit), ctypes.c_float(tol),
                              ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 0, rc
    return {"U": dev["U"][:, :ny].cpu().numpy().ravel(), "V": dev["V"][:, :ny].cpu().numpy().ravel(),
            "p": p[:, :ny].cpu().numpy().ravel()}


def test_noalloc_projection_matches_handle_path_twice(env):
    torch, fluid_gb300, L, _lib = env
    cases = [
        # width, height, seed, iters, tb, early_exit, tolerance, dt
        (120, 90, 11, 40, 8, False, 1e-5, 0.1),
        (77, 133, 12, 200, 4, True, 0.1, 0.05),
    ]
    for width, height, seed, iters, tb, ee, tol, dt in cases:
        inputs, want, sweeps = reference_projection(fluid_gb300, width, height, seed, iters, tb, ee,
                                                    tol, dt)
        got = noalloc_projection(torch, L, inputs, width + 2, height + 2, iters, tb, ee, tol, dt)
        for k in ("U", "V", "p"):
            assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), (width, k)
        if ee:
            assert sweeps < iters  # the early exit was exercised


def test_noalloc_allocates_nothing_and_rejects_oversize(env):
    torch, fluid_gb300, L, _lib = env
    inputs, _, _ = reference_projection(fluid_gb300, 64, 64, 3, 16, 8, False, 1e-5, 0.1)
    noalloc_projection(torch, L, inputs, 66, 66, 16, 8, False, 1e-5, 0.1)  # device set-up done
    free0, _ = torch.cuda.mem_get_info()
    noalloc_projection(torch, L, inputs, 66, 66, 16, 8, False, 1e-5, 0.1)
    free1, _ = torch.cuda.mem_get_info()
    # Only the test's own tensors come and go (torch caches them); the call
    # itself takes no device memory.
    assert free1 >= free0
    big = _lib.NOALLOC_MAX_CELLS // 1000 + 1
    rc = L.fg_project_noalloc(1, 1, 1, 1, big, 998, 1000, ctypes.c_float(1.0), ctypes.c_float(1.0),
                              ctypes.c_float(0.1), 10, ctypes.c_float(1.0), ctypes.c_float(1.0), 8, 0,
                              ctypes.c_float(1e-5), None)
    assert rc == _lib.FG_ERR_TOO_LARGE
