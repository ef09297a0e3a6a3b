"""fg_project_noalloc: the projection for callers that cannot allocate.

Callers that cannot call cudaMalloc when they project (an engine whose
allocator owns the device memory, a frame loop that must not risk the
synchronisation an allocation can cause) pass their own device fields and
the library uses a fixed scratch array instead of allocating.  The tests
call it through the C ABI on caller-owned buffers (torch tensors with a
pitch unlike the library's own) several times in a row -- with no sweeps,
with a smaller grid before a larger one and the reverse, with the early
exit -- and check U, V and p bit for bit against the handle-based
projection fg_make_incompressible with the same settings.  They also check
that a device-side wait that gives up is reported by
fg_project_noalloc_status, and that a context the caller creates itself
gets the scratch array of that context.  This file sorts last so a run that
stops at the first failure has run every other test before it.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

import scenes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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


def noalloc_projection(torch, L, inputs, nx, ny, iters, tb, early_exit, tol, dt, status=True):
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
    assert rc == 0, rc
    st = L.fg_project_noalloc_status(ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    if status:
        assert st == 0, st
    out = {"U": dev["U"][:, :ny].cpu().numpy().ravel(), "V": dev["V"][:, :ny].cpu().numpy().ravel(),
           "p": p[:, :ny].cpu().numpy().ravel()}
    return (out, st) if not status else out


def assert_bitwise(got, want, where):
    for k in ("U", "V", "p"):
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), (where, k)


def test_noalloc_projection_matches_handle_path_twice(env):
    torch, fluid_gb300, L, _lib = env
    cases = [
        # width, height, seed, iters, tb, early_exit, tolerance, dt
        (120, 90, 11, 40, 8, False, 1e-5, 0.1),
        (77, 133, 12, 200, 4, True, 0.1, 0.05),
        (1000, 1000, 13, 16, 8, False, 1e-5, 0.1),  # 189 regions: the TMA-fed kernel
    ]
    for width, height, seed, iters, tb, ee, tol, dt in cases:
        inputs, want, sweeps = reference_projection(fluid_gb300, width, height, seed, iters, tb, ee,
                                                    tol, dt)
        got = noalloc_projection(torch, L, inputs, width + 2, height + 2, iters, tb, ee, tol, dt)
        assert_bitwise(got, want, width)
        if ee:
            assert sweeps < iters  # the early exit was exercised


def test_noalloc_zero_sweeps_and_growing_grids(env):
    """No sweeps at all (the potential is cleared in the set-up and no Jacobi
    launch runs), then a small grid followed by a larger one in rows and
    columns (the second call reads nothing the first one left behind), then
    the small one again."""
    torch, fluid_gb300, L, _lib = env
    cases = [
        (50, 40, 21, 0, 8, False, 1e-5, 0.1),
        (30, 20, 22, 24, 8, False, 1e-5, 0.1),
        (300, 260, 23, 24, 8, False, 1e-5, 0.1),
        (30, 20, 22, 24, 8, False, 1e-5, 0.1),
        (64, 64, 24, 0, 4, True, 1e-5, 0.1),
    ]
    for width, height, seed, iters, tb, ee, tol, dt in cases:
        inputs, want, _ = reference_projection(fluid_gb300, width, height, seed, iters, tb, ee,
                                               tol, dt)
        got = noalloc_projection(torch, L, inputs, width + 2, height + 2, iters, tb, ee, tol, dt)
        assert_bitwise(got, want, (width, height, iters))


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


def test_noalloc_reports_a_wait_that_gave_up(env):
    """A copy barrier that never completes (fault injection: tile 0 expects
    16 bytes more than its copies bring; no fault, every copy lands) makes
    the TMA-fed Jacobi kernel's bounded wait give up (a 1000x1000 grid: at
    least one 8-warp region per SM, where that kernel runs).  The call itself
    returns FG_OK (its work is still queued); fg_project_noalloc_status
    reports FG_ERR_TIMEOUT.  Disarmed, the next call is bit for bit the
    handle path's again, whatever the stalled call left in the scratch."""
    torch, fluid_gb300, L, _lib = env
    width, height, seed, iters, tb = 1000, 1000, 31, 8, 8
    inputs, want, _ = reference_projection(fluid_gb300, width, height, seed, iters, tb, False,
                                           1e-5, 0.1)
    assert L.fg_debug_stall_tile(None, 0) == 0
    try:
        _, st = noalloc_projection(torch, L, inputs, width + 2, height + 2, iters, tb, False, 1e-5,
                                   0.1, status=False)
    finally:
        L.fg_debug_stall_tile(None, -1)
    assert st == _lib.FG_ERR_TIMEOUT, st
    got = noalloc_projection(torch, L, inputs, width + 2, height + 2, iters, tb, False, 1e-5, 0.1)
    assert_bitwise(got, want, "after the stalled call")


CONTEXT_SCRIPT = textwrap.dedent(r'''
    import ctypes, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    from fluid_gb300 import _lib
    L = _lib.lib()
    cu = ctypes.CDLL("libcuda.so.1")
    if not hasattr(cu, "cuCtxCreate_v2"):
        print("SKIP cuCtxCreate_v2 not exported"); sys.exit(0)
    def ck(r, what):
        if r != 0:
            raise SystemExit("%s failed: %d" % (what, r))
    ck(cu.cuInit(0), "cuInit")
    dev = ctypes.c_int()
    ck(cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
    NX, NY, P, ITERS = 98, 74, 80, 24
    rng = np.random.default_rng(7)
    S = np.ones((NX, P), np.float32)
    S[:, 0] = S[:, NY - 1] = S[0, :] = 0.0
    S[:, NY:] = 0.0
    U = (rng.uniform(-0.5, 0.5, (NX, P)) * S).astype(np.float32)
    V = (rng.uniform(-0.5, 0.5, (NX, P)) * S).astype(np.float32)
    def project():
        # fields allocated by the caller in the context current now
        ptrs = {}
        for k, a in (("U", U), ("V", V), ("S", S), ("p", np.zeros_like(U))):
            d = ctypes.c_uint64()
            ck(cu.cuMemAlloc_v2(ctypes.byref(d), ctypes.c_size_t(a.nbytes)), "cuMemAlloc")
            ck(cu.cuMemcpyHtoD_v2(d, a.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(a.nbytes)),
               "cuMemcpyHtoD")
            ptrs[k] = d
        f = ctypes.c_float
        rc = L.fg_project_noalloc(ctypes.c_void_p(ptrs["U"].value), ctypes.c_void_p(ptrs["V"].value),
                                  ctypes.c_void_p(ptrs["p"].value), ctypes.c_void_p(ptrs["S"].value),
                                  NX, NY, P, f(1.0), f(1.0), f(0.1), ITERS, f(1.0), f(1.0), 8, 0,
                                  f(1e-5), None)
        ck(rc, "fg_project_noalloc")
        ck(L.fg_project_noalloc_status(None), "fg_project_noalloc_status")
        ck(cu.cuCtxSynchronize(), "cuCtxSynchronize")
        out = {}
        for k in ("U", "V", "p"):
            a = np.empty_like(U)
            ck(cu.cuMemcpyDtoH_v2(a.ctypes.data_as(ctypes.c_void_p), ptrs[k],
                                  ctypes.c_size_t(a.nbytes)), "cuMemcpyDtoH")
            out[k] = a[:, :NY].copy()
        for d in ptrs.values():
            ck(cu.cuMemFree_v2(d), "cuMemFree")
        return out
    prim = ctypes.c_void_p()
    ck(cu.cuDevicePrimaryCtxRetain(ctypes.byref(prim), dev), "cuDevicePrimaryCtxRetain")
    ck(cu.cuCtxSetCurrent(prim), "cuCtxSetCurrent")
    a = project()                       # the primary context
    own = ctypes.c_void_p()
    ck(cu.cuCtxCreate_v2(ctypes.byref(own), 0, dev), "cuCtxCreate")  # now current
    b = project()                       # a context the caller made
    ck(cu.cuCtxDestroy_v2(own), "cuCtxDestroy")
    ck(cu.cuCtxSetCurrent(prim), "cuCtxSetCurrent")
    c = project()                       # the primary context again
    for k in ("U", "V", "p"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), ("own context", k)
        assert np.array_equal(a[k].view(np.uint32), c[k].view(np.uint32)), ("primary again", k)
    assert np.abs(a["p"]).max() > 0
    print("OK")
''')


def test_noalloc_in_a_context_the_caller_created(env):
    """The scratch array's address belongs to a CUDA context.  A caller that
    creates its own context (cuCtxCreate) and calls the projection there
    gets that context's array: the results equal the primary context's bit
    for bit, before and after the caller's context is destroyed.  Runs in a
    child process that uses the driver API directly (no torch), so the
    contexts it makes and destroys touch nothing else."""
    r = subprocess.run([sys.executable, "-c", CONTEXT_SCRIPT, ROOT], capture_output=True,
                       text=True, timeout=300)
    out = r.stdout + r.stderr
    if r.returncode == 0 and out.startswith("SKIP"):
        pytest.skip(out.strip())
    assert r.returncode == 0 and "OK" in r.stdout, out
