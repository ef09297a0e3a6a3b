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
