"""GB300-native simulation step of pkg/fluid (TheFellow/fluid).

The CUDA kernels sit behind the C ABI declared in include/fluidgpu.h
(libfluidgpu.so, built in-tree by fluid_gb300._build).  ``Fluid`` is the
Python mirror of the Go type ``fluid.Fluid`` over that ABI.
"""
from . import fluid as _fluid_mod
from ._build import build
from .fluid import (ALL_FIELDS, FIELDS, JACOBI_KERNEL_DATAFLOW, JACOBI_KERNEL_NONE,
                    JACOBI_KERNEL_SWEEP, JACOBI_KERNEL_TMA, SCHEME_JACOBI, SCHEME_LEXSOR,
                    SCHEME_MULTIGRID, Batch, Fluid, FluidError, ScalarField, VectorField,
                    debug_fail_alloc)


def __getattr__(name):
    if name == "Relaxation":
        return _fluid_mod.Relaxation
    raise AttributeError(name)


def set_relaxation(value: float) -> None:
    """Sets the package variable fluid.Relaxation (fluid.go:7-9)."""
    _fluid_mod.Relaxation = float(value)


__all__ = ["Fluid", "Batch", "FluidError", "ScalarField", "VectorField", "build", "set_relaxation",
           "FIELDS", "ALL_FIELDS", "SCHEME_LEXSOR", "SCHEME_JACOBI", "SCHEME_MULTIGRID",
           "JACOBI_KERNEL_NONE", "JACOBI_KERNEL_SWEEP", "JACOBI_KERNEL_TMA",
           "JACOBI_KERNEL_DATAFLOW", "debug_fail_alloc"]
