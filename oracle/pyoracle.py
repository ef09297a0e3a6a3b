"""ctypes front end of the CPU oracle (test infrastructure only).

``OracleFluid`` exposes the same surface as the Go type ``fluid.Fluid``
(pkg/fluid/fluid.go:11-68, walls.go, the field views) and as
``fluid_gb300.Fluid``, so the ported reference tests run unchanged against
both.  Only tests/, the smoke entry and the benchmark's CPU leg import this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

# Pressure schemes (shared numbering with the CUDA library).
LEXSOR, JACOBI, REDBLACK = 0, 1, 2

_FIELDS = {"U": 0, "V": 1, "newU": 2, "newV": 3, "p": 4, "S": 5, "M": 6, "newM": 7}


def build(force: bool = False) -> str:
    """Compile the oracle shared library (g++, no CUDA)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "fluid_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            vp, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
            sig = {
                "orc_create": (vp, [i, i, i, d, d, i]),
                "orc_destroy": (None, [vp]),
                "orc_dims": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
                "orc_field": (vp, [vp, i]),
                "orc_set_param": (i, [vp, ctypes.c_char_p, d]),
                "orc_get_param": (d, [vp, ctypes.c_char_p]),
                "orc_simulate": (None, [vp, d]),
                "orc_stage": (i, [vp, i, i, d]),
                "orc_copy_border": (i, [vp, vp, vp]),
                "orc_set_solid": (i, [vp, i, i, i]),
                "orc_is_solid": (i, [vp, i, i]),
                "orc_set_velocity": (i, [vp, i, i, d, d]),
                "orc_add_smoke": (i, [vp, i, i, d]),
                "orc_reset": (None, [vp]),
                "orc_apply_force": (None, [vp, i, i, d, d]),
                "orc_apply_force_radius": (None, [vp, i, i, d, d, i]),
                "orc_set_circular_obstacle": (None, [vp, i, i, i]),
                "orc_max_divergence": (d, [vp]),
                "orc_adaptive_dt": (d, [vp, d]),
                "orc_vorticity": (i, [vp, vp, ctypes.POINTER(d)]),
                "orc_velocity_magnitude": (i, [vp, vp, ctypes.POINTER(d)]),
                "orc_sample_velocity": (i, [vp, d, d, ctypes.POINTER(d)]),
                "orc_stats": (i, [vp, ctypes.POINTER(d)]),
                "orc_threads": (i, [vp]),
                "orc_particles_advect": (i, [vp, i, vp, vp, vp, vp, vp, d]),
                "orc_render": (i, [vp, i, vp]),
                "orc_rollout_grad": (i, [vp, i, d, vp, i, vp, vp, vp, vp, vp, vp, vp,
                                         ctypes.POINTER(d), vp, vp, vp, vp]),
            }
            for name, (res, args) in sig.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class ScalarField:
    """pkg/fluid/scalar_field.go:7-22."""

    def __init__(self, nx, ny, values, mn, mx):
        self.NumX, self.NumY = nx, ny
        self.values = values
        self.MinValue, self.MaxValue = mn, mx

    def Value(self, i, j):
        if i < 0 or i >= self.NumX:
            return 0.0, "x index (%d) out of range, must be between 0 and %d" % (i, self.NumX - 1)
        if j < 0 or j >= self.NumY:
            return 0.0, "y index (%d) out of range, must be between 0 and %d" % (j, self.NumY - 1)
        return float(self.values[i * self.NumY + j]), None


class VectorField:
    """pkg/fluid/vector_field.go:5-19."""

    def __init__(self, nx, ny, u, v):
        self.NumX, self.NumY = nx, ny
        self.valuesU, self.valuesV = u, v

    def Value(self, i, j):
        if i < 0 or i >= self.NumX:
            return 0.0, 0.0, "x index out of range, must be between 0 and %d" % (self.NumX - 1)
        if j < 0 or j >= self.NumY:
            return 0.0, 0.0, "y index out of range, must be between 0 and %d" % (self.NumY - 1)
        k = i * self.NumY + j
        return float(self.valuesU[k]), float(self.valuesV[k]), None


_PARAMS = (
    "Confinement", "ViscosityDiffusion", "PressureDamping", "TurbulenceStrength",
    "SmokeAdvection", "UseMultigrid", "MultigridLevels", "UseBFECC", "Relaxation",
    "num_iters", "tolerance", "early_exit", "scheme", "jacobi_omega", "check_every",
    "refine_sweeps", "precise_coords",
)
_BOOL_PARAMS = ("UseMultigrid", "UseBFECC", "early_exit", "precise_coords")
_INT_PARAMS = ("MultigridLevels", "num_iters", "scheme", "check_every", "refine_sweeps")


class OracleFluid:
    """CPU restatement of ``fluid.Fluid``; ``prec`` is 32 (FP32-faithful) or 64."""

    def __init__(self, density, width, height, h, prec=32, threads=1, **params):
        self._lib = lib()
        self._h = self._lib.orc_create(prec, width, height, density, h, threads)
        if not self._h:
            raise ValueError("invalid oracle arguments")
        self.prec = prec
        self.dtype = np.float32 if prec == 32 else np.float64
        nx, ny = ctypes.c_int(), ctypes.c_int()
        self._lib.orc_dims(self._h, ctypes.byref(nx), ctypes.byref(ny))
        self.NumX, self.NumY = nx.value, ny.value
        self.numCells = self.NumX * self.NumY
        for k, v in params.items():
            setattr(self, k, v)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._lib.orc_destroy(h)
            self._h = None

    # ------------------------------------------------------------ fields
    def _field(self, name):
        ptr = self._lib.orc_field(self._h, _FIELDS[name])
        ct = ctypes.c_float if self.prec == 32 else ctypes.c_double
        return np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ct)), shape=(self.numCells,))

    U = property(lambda self: self._field("U"))
    V = property(lambda self: self._field("V"))
    S = property(lambda self: self._field("S"))
    M = property(lambda self: self._field("M"))
    p = property(lambda self: self._field("p"))
    newU = property(lambda self: self._field("newU"))
    newV = property(lambda self: self._field("newV"))
    newM = property(lambda self: self._field("newM"))

    @property
    def density(self):
        return self._lib.orc_get_param(self._h, b"density")

    def H(self):
        return self._lib.orc_get_param(self._h, b"h")

    def __getattr__(self, name):
        if name in _PARAMS:
            v = self._lib.orc_get_param(self.__dict__["_h"], name.encode())
            if name in _BOOL_PARAMS:
                return bool(v)
            if name in _INT_PARAMS:
                return int(v)
            return v
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in _PARAMS:
            if self._lib.orc_set_param(self._h, name.encode(), float(value)) != 0:
                raise AttributeError(name)
        else:
            object.__setattr__(self, name, value)

    # ------------------------------------------------------------ step + stages
    def Simulate(self, dt):
        self._lib.orc_simulate(self._h, dt)

    def _stage(self, k, iters=0, dt=0.0):
        if self._lib.orc_stage(self._h, k, iters, dt) != 0:
            raise RuntimeError("stage %d failed" % k)

    def makeIncompressible(self, numIters, dt):
        self._stage(0, numIters, dt)

    def advectVelocity(self, dt):
        self._stage(1, 0, dt)

    def advectSmoke(self, dt):
        self._stage(2, 0, dt)

    def handleBorders(self):
        self._stage(3)

    def applyVorticityConfinement(self, dt):
        self._stage(4, 0, dt)

    def applyViscosity(self, dt):
        self._stage(5, 0, dt)

    def addTurbulence(self, dt):
        self._stage(6, 0, dt)

    def advectVelocityBFECC(self, dt):
        self._stage(7, 0, dt)

    def advectSmokeBFECC(self, dt):
        self._stage(8, 0, dt)

    def copyBorder(self, dst, src):
        assert dst.dtype == self.dtype and src.dtype == self.dtype
        assert dst.flags.c_contiguous and src.flags.c_contiguous
        self._lib.orc_copy_border(self._h, dst.ctypes.data, src.ctypes.data)

    # ------------------------------------------------------------ tools
    def _check(self, rc, i, j):
        if rc < 0:
            if i < 0 or i >= self.NumX:
                raise IndexError("invalid x-index: %d" % i)
            raise IndexError("invalid y-index: %d" % j)
        return rc

    def SetSolid(self, i, j, value):
        self._check(self._lib.orc_set_solid(self._h, i, j, int(bool(value))), i, j)

    def IsSolid(self, i, j):
        return bool(self._check(self._lib.orc_is_solid(self._h, i, j), i, j))

    def SetVelocity(self, i, j, u, v):
        self._check(self._lib.orc_set_velocity(self._h, i, j, u, v), i, j)

    def AddSmoke(self, i, j, s):
        self._check(self._lib.orc_add_smoke(self._h, i, j, s), i, j)

    def Reset(self):
        self._lib.orc_reset(self._h)

    def ApplyForce(self, i, j, fx, fy):
        self._lib.orc_apply_force(self._h, i, j, fx, fy)

    def ApplyForceRadius(self, cx, cy, fx, fy, radius):
        self._lib.orc_apply_force_radius(self._h, cx, cy, fx, fy, radius)

    def SetCircularObstacle(self, cx, cy, radius):
        self._lib.orc_set_circular_obstacle(self._h, cx, cy, radius)

    # ------------------------------------------------------------ views
    def MaxDivergence(self):
        return self._lib.orc_max_divergence(self._h)

    def GetAdaptiveTimeStep(self, basedt):
        return self._lib.orc_adaptive_dt(self._h, basedt)

    def SampleVelocity(self, x, y):
        uv = (ctypes.c_double * 2)()
        self._lib.orc_sample_velocity(self._h, x, y, uv)
        return uv[0], uv[1]

    def _view(self, fn):
        out = np.zeros(self.numCells, dtype=self.dtype)
        mm = (ctypes.c_double * 2)()
        fn(self._h, out.ctypes.data, mm)
        return ScalarField(self.NumX, self.NumY, out, mm[0], mm[1])

    def Vorticity(self):
        return self._view(self._lib.orc_vorticity)

    def VelocityMagnitude(self):
        return self._view(self._lib.orc_velocity_magnitude)

    def Pressure(self):
        p = self.p
        return ScalarField(self.NumX, self.NumY, p, float(p.min()), float(p.max()))

    def Smoke(self):
        m = self.M
        return ScalarField(self.NumX, self.NumY, m, float(m.min()), float(m.max()))

    def Velocity(self):
        return VectorField(self.NumX, self.NumY, self.U, self.V)

    def stats(self):
        out = (ctypes.c_double * 8)()
        self._lib.orc_stats(self._h, out)
        keys = ("div_l2_post", "div_max_post", "div_count_post", "resid_l2", "resid_max",
                "smoke_mass", "sweeps", "last_maxdiv")
        return dict(zip(keys, list(out)))

    def rollout_grad(self, dt, steps, target, forces=None, sources=()):
        """FP64 reverse-mode reference of a recorded rollout (prec=64 only):
        `steps` steps with per-step forces (steps x 2 x N array or None) and
        sources [(i, j, u, v, smoke, mode)] applied before every step, loss
        ||M - target||_2 over the interior.  Returns {"loss", "U", "V", "M",
        "force_u", "force_v"}; the oracle ends at the end of the rollout."""
        n = self.NumX * self.NumY
        tgt = np.ascontiguousarray(target, np.float64)
        fr = None if forces is None else np.ascontiguousarray(forces, np.float64)
        src = list(sources)
        si = np.array([s[0] for s in src] or [0], np.int32)
        sj = np.array([s[1] for s in src] or [0], np.int32)
        su = np.array([s[2] for s in src] or [0], np.float64)
        sv = np.array([s[3] for s in src] or [0], np.float64)
        ss = np.array([s[4] for s in src] or [0], np.float64)
        sm = np.array([s[5] for s in src] or [0], np.int32)
        out = [np.zeros(n) for _ in range(3)]
        dF = np.zeros((steps, 2, n))
        loss = ctypes.c_double()
        rc = self._lib.orc_rollout_grad(self._h, int(steps), float(dt),
                                      None if fr is None else fr.ctypes.data, len(src),
                                      si.ctypes.data, sj.ctypes.data, su.ctypes.data,
                                      sv.ctypes.data, ss.ctypes.data, sm.ctypes.data,
                                      tgt.ctypes.data, ctypes.byref(loss), out[0].ctypes.data,
                                      out[1].ctypes.data, out[2].ctypes.data, dF.ctypes.data)
        if rc != 0:
            raise RuntimeError("orc_rollout_grad failed (%d)" % rc)
        return {"loss": loss.value, "U": out[0], "V": out[1], "M": out[2],
                "force_u": dF[:, 0], "force_v": dF[:, 1]}

    def particles_advect(self, dt, x, y, age, max_age, rgb):
        """advectParticles (main/main.go:512-546) on arrays of this oracle's
        precision, in place; returns the number of survivors (first)."""
        return self._lib.orc_particles_advect(self._h, len(x), x.ctypes.data, y.ctypes.data,
                                              age.ctypes.data, max_age.ctypes.data,
                                              rgb.ctypes.data, float(dt))

    def render(self, kind):
        """drawScalarField / drawVorticityField: NumX * NumY * 4 bytes."""
        out = np.zeros(self.NumX * self.NumY * 4, np.uint8)
        self._lib.orc_render(self._h, int(kind), out.ctypes.data)
        return out

