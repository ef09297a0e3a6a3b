"""The C ABI library loads on a machine without a GPU and exports every
symbol include/fluidgpu.h declares (no device calls here)."""
import ctypes
import os
import re

import pytest

from fluid_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "fluidgpu.h")).read()
    return sorted(set(re.findall(r"\b(fg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_api():
    names = declared_symbols()
    assert "fg_simulate" in names and "fg_create" in names
    assert len(names) >= 35


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_params_default_matches_fluid_new():
    L = _lib.load()
    p = _lib.Params()
    assert L.fg_params_default(ctypes.byref(p)) == 0
    # fluid.New defaults (fluid.go:59-66) and the hard-coded Simulate constants.
    assert p.confinement == 0 and p.viscosity_diffusion == 0
    assert p.pressure_damping == 1.0
    assert p.turbulence_strength == pytest.approx(0.02)
    assert p.smoke_advection == 1.0 and p.use_multigrid == 0 and p.multigrid_levels == 2
    assert p.use_bfecc == 0 and p.relaxation == pytest.approx(1.9)
    assert p.num_iters == 8 and p.tolerance == pytest.approx(1e-5) and p.early_exit == 1
    assert p.scheme == 0


def test_null_handle_is_rejected_without_device():
    L = _lib.load()
    assert L.fg_params_default(None) == _lib.FG_ERR_INVALID
    assert L.fg_last_error(None) == b"invalid handle"
    assert L.fg_simulate(None, 0.1) == _lib.FG_ERR_INVALID
    assert L.fg_destroy(None) == _lib.FG_ERR_INVALID


def test_oversized_grids_are_rejected_before_any_device_call():
    """Cell indices are 32-bit: fg_create refuses a padded grid above 2^30
    cells and fg_project_noalloc a caller pitch whose fields exceed 2^31
    cells, both before touching a device (so this runs without a GPU)."""
    L = _lib.load()
    h = _lib._vp()
    for w, hh in ((2 ** 15, 2 ** 15), (40_000_000, 1), (2 ** 31 - 2, 1), (1, 2 ** 31 - 2)):
        assert L.fg_create(w, hh, 1.0, 1.0, None, ctypes.byref(h)) == _lib.FG_ERR_INVALID, (w, hh)
        assert not h.value
    # A normal grid passes the check: without a GPU it stops at the device.
    rc = L.fg_create(64, 48, 1.0, 1.0, None, ctypes.byref(h))
    if rc == 0:
        L.fg_destroy(h)
    assert rc in (0, _lib.FG_ERR_CUDA)
    dummy = ctypes.c_void_p(256)
    rc = L.fg_project_noalloc(dummy, dummy, dummy, dummy, 3, 3, 2 ** 30, 1.0, 1.0, 0.1, 8,
                              1.0, 1.0, 8, 0, 1e-5, None)
    assert rc == _lib.FG_ERR_TOO_LARGE


def test_noalloc_sweep_counts_near_int_max_are_rejected():
    """The allocation-free projection's launch count is formed in 64 bits: a
    num_iters near 2^31 must not wrap below the 4096-launch limit (it is
    refused before any device call, so this runs without a GPU)."""
    L = _lib.load()
    dummy = ctypes.c_void_p(256)
    for iters, tb in ((2 ** 31 - 1, 8), (2 ** 31 - 1, 1), (2 ** 31 - 8, 4), (4096 * 8 + 1, 8)):
        rc = L.fg_project_noalloc(dummy, dummy, dummy, dummy, 16, 16, 16, 1.0, 1.0, 0.1, iters,
                                  1.0, 1.0, tb, 0, 1e-5, None)
        assert rc == _lib.FG_ERR_TOO_LARGE, (iters, tb, rc)


def test_struct_layouts_and_constants_match_the_header(tmp_path):
    """The ctypes mirrors of fg_params and fg_stats have the C layout (every
    field's offset and the size), and the FG_JACOBI_KERNEL_* values are the
    Python constants: a C probe compiled against include/fluidgpu.h prints
    them."""
    import shutil
    import subprocess

    import fluid_gb300

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "fluidgpu.h"', "int main(void) {"]
    for cname, pyt in (("fg_params", _lib.Params), ("fg_stats", _lib.Stats)):
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for name, _ in pyt._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, name, cname, name))
    for k in ("NONE", "SWEEP", "TMA", "DATAFLOW"):
        lines.append('printf("FG_JACOBI_KERNEL_%s %%d\\n", FG_JACOBI_KERNEL_%s);' % (k, k))
    lines.append("return 0; }")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], check=True, capture_output=True,
                                                         text=True).stdout.splitlines())
    for cname, pyt in (("fg_params", _lib.Params), ("fg_stats", _lib.Stats)):
        assert int(out["%s size" % cname]) == ctypes.sizeof(pyt), cname
        for name, _ in pyt._fields_:
            assert int(out["%s %s" % (cname, name)]) == getattr(pyt, name).offset, (cname, name)
    for k in ("NONE", "SWEEP", "TMA", "DATAFLOW"):
        assert int(out["FG_JACOBI_KERNEL_%s" % k]) == getattr(fluid_gb300, "JACOBI_KERNEL_%s" % k)
