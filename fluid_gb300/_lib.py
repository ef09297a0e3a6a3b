"""ctypes binding of include/fluidgpu.h (libfluidgpu.so built in-tree).

Loading fails loudly: there is no CPU fallback for the step.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

FG_OK = 0
FG_ERR_INVALID = -1
FG_ERR_INDEX = -2
FG_ERR_CUDA = -3
FG_ERR_UNSUPPORTED = -4
FG_ERR_MASK = -5
FG_ERR_TIMEOUT = -6
FG_ERR_NOMEM = -7
FG_ERR_TOO_LARGE = -8
FG_ERR_NONFINITE = -9
NOALLOC_MAX_CELLS = 1 << 20

_c_i, _c_f, _c_d = ctypes.c_int, ctypes.c_float, ctypes.c_double


class Params(ctypes.Structure):
    _fields_ = [
        ("confinement", _c_f), ("viscosity_diffusion", _c_f), ("pressure_damping", _c_f),
        ("turbulence_strength", _c_f), ("smoke_advection", _c_f), ("use_multigrid", _c_i),
        ("multigrid_levels", _c_i), ("use_bfecc", _c_i), ("relaxation", _c_f),
        ("num_iters", _c_i), ("tolerance", _c_f), ("early_exit", _c_i), ("scheme", _c_i),
        ("jacobi_omega", _c_f), ("tb_depth", _c_i), ("refine_sweeps", _c_i),
        ("use_graphs", _c_i), ("precise_coords", _c_i), ("reserved", _c_i * 6),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("div_l2_post", _c_d), ("div_max_post", _c_d), ("div_count_post", _c_d),
        ("resid_l2", _c_d), ("resid_max", _c_d), ("smoke_mass", _c_d), ("last_maxdiv", _c_d),
        ("sweeps", _c_i), ("jacobi_kernel", _c_i), ("reserved", _c_i * 6),
    ]


# name -> (restype, argtypes); every symbol of include/fluidgpu.h.
_vp, _fp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float)
SIGNATURES = {
    "fg_params_default": (_c_i, [ctypes.POINTER(Params)]),
    "fg_create": (_c_i, [_c_i, _c_i, _c_f, _c_f, ctypes.POINTER(Params), ctypes.POINTER(_vp)]),
    "fg_destroy": (_c_i, [_vp]),
    "fg_dims": (_c_i, [_vp, ctypes.POINTER(_c_i), ctypes.POINTER(_c_i)]),
    "fg_h": (_c_f, [_vp]),
    "fg_get_params": (_c_i, [_vp, ctypes.POINTER(Params)]),
    "fg_set_params": (_c_i, [_vp, ctypes.POINTER(Params)]),
    "fg_field": (_c_i, [_vp, _c_i, ctypes.POINTER(_fp)]),
    "fg_mark_dirty": (_c_i, [_vp, ctypes.c_uint]),
    "fg_download": (_c_i, [_vp, ctypes.c_uint]),
    "fg_synchronize": (_c_i, [_vp]),
    "fg_download_async": (_c_i, [_vp, ctypes.c_uint]),
    "fg_download_wait": (_c_i, [_vp]),
    "fg_stream": (_vp, [_vp]),
    "fg_simulate": (_c_i, [_vp, _c_f]),
    "fg_get_stats": (_c_i, [_vp, ctypes.POINTER(Stats)]),
    "fg_make_incompressible": (_c_i, [_vp, _c_i, _c_f]),
    "fg_advect_velocity": (_c_i, [_vp, _c_f]),
    "fg_advect_smoke": (_c_i, [_vp, _c_f]),
    "fg_advect_velocity_bfecc": (_c_i, [_vp, _c_f]),
    "fg_advect_smoke_bfecc": (_c_i, [_vp, _c_f]),
    "fg_handle_borders": (_c_i, [_vp]),
    "fg_apply_vorticity_confinement": (_c_i, [_vp, _c_f]),
    "fg_apply_viscosity": (_c_i, [_vp, _c_f]),
    "fg_add_turbulence": (_c_i, [_vp, _c_f]),
    "fg_clear_pressure": (_c_i, [_vp]),
    "fg_copy_border": (_c_i, [_vp, _vp, _vp]),
    "fg_set_solid": (_c_i, [_vp, _c_i, _c_i, _c_i]),
    "fg_is_solid": (_c_i, [_vp, _c_i, _c_i, ctypes.POINTER(_c_i)]),
    "fg_set_velocity": (_c_i, [_vp, _c_i, _c_i, _c_f, _c_f]),
    "fg_add_smoke": (_c_i, [_vp, _c_i, _c_i, _c_f]),
    "fg_reset": (_c_i, [_vp]),
    "fg_set_velocity_many": (_c_i, [_vp, _c_i, _vp, _vp, _vp, _vp]),
    "fg_add_smoke_many": (_c_i, [_vp, _c_i, _vp, _vp, _vp]),
    "fg_set_sources": (_c_i, [_vp, _c_i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fg_apply_force": (_c_i, [_vp, _c_i, _c_i, _c_f, _c_f]),
    "fg_apply_force_radius": (_c_i, [_vp, _c_i, _c_i, _c_f, _c_f, _c_i]),
    "fg_set_circular_obstacle": (_c_i, [_vp, _c_i, _c_i, _c_i]),
    "fg_max_divergence": (_c_i, [_vp, _fp]),
    "fg_vorticity": (_c_i, [_vp, _vp, _fp, _fp]),
    "fg_velocity_magnitude": (_c_i, [_vp, _vp, _fp, _fp]),
    "fg_field_min_max": (_c_i, [_vp, _c_i, _fp, _fp]),
    "fg_sample_velocity": (_c_i, [_vp, _c_f, _c_f, _fp, _fp]),
    "fg_adaptive_time_step": (_c_i, [_vp, _c_f, _fp]),
    "fg_profile_enable": (_c_i, [_vp, _c_i]),
    "fg_profile_jacobi": (_c_i, [_vp, _fp, ctypes.POINTER(_c_i)]),
    "fg_profile_stages": (_c_i, [_vp, _c_i, _fp, ctypes.POINTER(ctypes.c_char_p)]),
    "fg_launch_count": (ctypes.c_ulonglong, [_vp]),
    "fg_edit_bytes": (ctypes.c_ulonglong, [_vp]),
    "fg_project_noalloc": (_c_i, [_vp, _vp, _vp, _vp, _c_i, _c_i, _c_i, _c_f, _c_f, _c_f, _c_i,
                                  _c_f, _c_f, _c_i, _c_i, _c_f, _vp]),
    "fg_project_noalloc_status": (_c_i, [_vp]),
    "fg_debug_fail_alloc": (_c_i, [_c_i]),
    "fg_debug_stall_tile": (_c_i, [_vp, _c_i]),
    "fg_tape_begin": (_c_i, [_vp, _c_i, _c_i]),
    "fg_step_forward": (_c_i, [_vp, _c_f, _vp, _vp]),
    "fg_tape_seed": (_c_i, [_vp, _vp, _vp, _vp]),
    "fg_tape_seed_smoke_l2": (_c_i, [_vp, _vp, ctypes.POINTER(_c_d)]),
    "fg_step_adjoint": (_c_i, [_vp, _vp, _vp]),
    "fg_tape_grad": (_c_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fg_tape_steps": (_c_i, [_vp, ctypes.POINTER(_c_i), ctypes.POINTER(_c_i)]),
    "fg_tape_end": (_c_i, [_vp]),
    "fg_batch_create": (_c_i, [_vp, _c_i, ctypes.POINTER(_vp)]),
    "fg_batch_size": (_c_i, [_vp, ctypes.POINTER(_c_i)]),
    "fg_batch_step": (_c_i, [_vp, _c_f]),
    "fg_batch_step_adjoint": (_c_i, [_vp]),
    "fg_batch_gather": (_c_i, [_vp]),
    "fg_batch_scatter": (_c_i, [_vp]),
    "fg_batch_seed_smoke_l2": (_c_i, [_vp, _vp, ctypes.POINTER(_c_d)]),
    "fg_batch_grad": (_c_i, [_vp, _c_i, _vp, _vp, _vp]),
    "fg_batch_autotune": (_c_i, [_vp, _c_f, _c_i, ctypes.POINTER(_c_i), ctypes.POINTER(_c_i),
                                 ctypes.POINTER(_c_i), _fp]),
    "fg_particles_add": (_c_i, [_vp, _c_i, _vp, _vp, _vp, _vp, _c_i]),
    "fg_particles_advect": (_c_i, [_vp, _c_f]),
    "fg_particles_count": (_c_i, [_vp, ctypes.POINTER(_c_i)]),
    "fg_particles_get": (_c_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "fg_particles_clear": (_c_i, [_vp]),
    "fg_render": (_c_i, [_vp, _c_i, _vp]),
    "fg_last_error": (ctypes.c_char_p, [_vp]),
}

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libfluidgpu.so (building it first if absent) without touching the GPU."""
    global _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                if not build_if_missing:
                    raise ImportError("libfluidgpu.so is not built: run fluid_gb300._build.build()")
                _build.build()
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def lib():
    return load()
