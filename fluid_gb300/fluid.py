"""Python front end of libfluidgpu with the surface of the Go type fluid.Fluid.

``Fluid`` mirrors pkg/fluid (fluid.go:11-68 for the state and tuning fields,
walls.go for the tools, the view files for ScalarField/VectorField) over the
C ABI of include/fluidgpu.h.  Its exported slices U, V, S, M are numpy views
of the library's pinned host mirrors, laid out like the Go slices (index
i*NumY + j).

With ``auto_sync=True`` (the default) every call behaves like the Go
methods: before a device call all mirrors are uploaded, after it they are
downloaded, so code may read and write the arrays freely between calls.
With ``auto_sync=False`` the device copy is authoritative: use the tool
methods for edits and ``download()`` before reading arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

Relaxation = 1.9  # package var fluid.Relaxation (fluid.go:7-9)

FIELDS = {"U": 0, "V": 1, "newU": 2, "newV": 3, "p": 4, "S": 5, "M": 6, "newM": 7}
ALL_FIELDS = 0xFF
SCHEME_LEXSOR, SCHEME_JACOBI, SCHEME_MULTIGRID = 0, 1, 3
# stats()["jacobi_kernel"]: the kernel of the last JACOBI-scheme solve (FG_JACOBI_KERNEL_*).
JACOBI_KERNEL_NONE, JACOBI_KERNEL_SWEEP, JACOBI_KERNEL_TMA, JACOBI_KERNEL_DATAFLOW = 0, 1, 2, 3

# Python attribute -> fg_params member.
_PARAMS = {
    "Confinement": "confinement",
    "ViscosityDiffusion": "viscosity_diffusion",
    "PressureDamping": "pressure_damping",
    "TurbulenceStrength": "turbulence_strength",
    "SmokeAdvection": "smoke_advection",
    "UseMultigrid": "use_multigrid",
    "MultigridLevels": "multigrid_levels",
    "UseBFECC": "use_bfecc",
    "num_iters": "num_iters",
    "tolerance": "tolerance",
    "early_exit": "early_exit",
    "scheme": "scheme",
    "jacobi_omega": "jacobi_omega",
    "tb_depth": "tb_depth",
    "check_every": "tb_depth",
    "refine_sweeps": "refine_sweeps",
    "use_graphs": "use_graphs",
    "precise_coords": "precise_coords",
}
_BOOL = {"UseMultigrid", "UseBFECC", "early_exit", "use_graphs", "precise_coords"}


def debug_fail_alloc(n):
    """Fault injection: the n-th next device or pinned allocation of the
    library (process-wide, from 0) fails as if memory were exhausted; n < 0
    disarms."""
    _lib.lib().fg_debug_fail_alloc(int(n))


class FluidError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


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


class Fluid:
    """fluid.New(density, width, height, h) on the GPU."""

    dtype = np.float32

    def __init__(self, density, width, height, h, auto_sync=True, **params):
        L = _lib.lib()
        object.__setattr__(self, "_L", L)
        object.__setattr__(self, "_h", ctypes.c_void_p())
        object.__setattr__(self, "auto_sync", auto_sync)
        prm = _lib.Params()
        L.fg_params_default(ctypes.byref(prm))
        object.__setattr__(self, "_prm", prm)
        rc = L.fg_create(int(width), int(height), float(density), float(h), ctypes.byref(prm),
                         ctypes.byref(self._h))
        if rc != 0:
            raise FluidError(rc, "fg_create failed")
        nx, ny = ctypes.c_int(), ctypes.c_int()
        L.fg_dims(self._h, ctypes.byref(nx), ctypes.byref(ny))
        object.__setattr__(self, "NumX", nx.value)
        object.__setattr__(self, "NumY", ny.value)
        object.__setattr__(self, "numCells", nx.value * ny.value)
        object.__setattr__(self, "_density", float(np.float32(density)))
        views = {}
        for name, k in FIELDS.items():
            ptr = ctypes.POINTER(ctypes.c_float)()
            L.fg_field(self._h, k, ctypes.byref(ptr))
            views[name] = np.ctypeslib.as_array(ptr, shape=(self.numCells,))
        object.__setattr__(self, "_views", views)
        for k, v in params.items():
            setattr(self, k, v)

    def __del__(self):
        h = self.__dict__.get("_h")
        if h:
            self._L.fg_destroy(h)
            object.__setattr__(self, "_h", None)

    # ------------------------------------------------------------ plumbing
    def _check(self, rc, what="call"):
        if rc != 0:
            msg = self._L.fg_last_error(self._h)
            raise FluidError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def _push_params(self):
        self._prm.relaxation = float(Relaxation)
        self._check(self._L.fg_set_params(self._h, ctypes.byref(self._prm)), "fg_set_params")

    def _before(self):
        self._push_params()
        if self.auto_sync:
            self._check(self._L.fg_mark_dirty(self._h, ALL_FIELDS), "fg_mark_dirty")

    def _after(self):
        if self.auto_sync:
            self._check(self._L.fg_download(self._h, ALL_FIELDS), "fg_download")

    def _device(self, fn, *args, what=None):
        self._before()
        self._check(fn(self._h, *args), what or fn.__name__)
        self._after()

    def download(self, mask=ALL_FIELDS):
        self._check(self._L.fg_download(self._h, mask), "fg_download")

    def download_async(self, mask=1 << FIELDS["M"]):
        """Copies the smoke field beside the next step, after its projection
        (download_wait completes it)."""
        self._check(self._L.fg_download_async(self._h, mask), "fg_download_async")

    def download_wait(self):
        self._check(self._L.fg_download_wait(self._h), "fg_download_wait")

    def mark_dirty(self, mask=ALL_FIELDS):
        self._check(self._L.fg_mark_dirty(self._h, mask), "fg_mark_dirty")

    def synchronize(self):
        self._check(self._L.fg_synchronize(self._h), "fg_synchronize")

    @property
    def stream(self):
        return self._L.fg_stream(self._h)

    @property
    def handle(self):
        return self._h

    # ------------------------------------------------------------ fields / params
    U = property(lambda self: self._views["U"])
    V = property(lambda self: self._views["V"])
    S = property(lambda self: self._views["S"])
    M = property(lambda self: self._views["M"])
    p = property(lambda self: self._views["p"])
    newU = property(lambda self: self._views["newU"])
    newV = property(lambda self: self._views["newV"])
    newM = property(lambda self: self._views["newM"])

    @property
    def density(self):
        return self._density

    def H(self):
        return self._L.fg_h(self._h)

    def __getattr__(self, name):
        if name in _PARAMS:
            v = getattr(self.__dict__["_prm"], _PARAMS[name])
            return bool(v) if name in _BOOL else v
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in _PARAMS:
            field = _PARAMS[name]
            ctype = dict(_lib.Params._fields_)[field]
            setattr(self._prm, field, int(value) if ctype is ctypes.c_int else float(value))
            self._push_params()
        else:
            object.__setattr__(self, name, value)

    # ------------------------------------------------------------ step + stages
    def Simulate(self, dt):
        """(*Fluid).Simulate fluid.go:79-109."""
        self._device(self._L.fg_simulate, ctypes.c_float(dt), what="Simulate")

    def stats(self):
        st = _lib.Stats()
        self._check(self._L.fg_get_stats(self._h, ctypes.byref(st)), "fg_get_stats")
        return {k: getattr(st, k) for k, _ in _lib.Stats._fields_ if k != "reserved"}

    def makeIncompressible(self, numIters, dt):
        self._device(self._L.fg_make_incompressible, int(numIters), ctypes.c_float(dt))

    def advectVelocity(self, dt):
        self._device(self._L.fg_advect_velocity, ctypes.c_float(dt))

    def advectSmoke(self, dt):
        self._device(self._L.fg_advect_smoke, ctypes.c_float(dt))

    def advectVelocityBFECC(self, dt):
        self._device(self._L.fg_advect_velocity_bfecc, ctypes.c_float(dt))

    def advectSmokeBFECC(self, dt):
        self._device(self._L.fg_advect_smoke_bfecc, ctypes.c_float(dt))

    def handleBorders(self):
        self._device(self._L.fg_handle_borders)

    def applyVorticityConfinement(self, dt):
        self._device(self._L.fg_apply_vorticity_confinement, ctypes.c_float(dt))

    def applyViscosity(self, dt):
        self._device(self._L.fg_apply_viscosity, ctypes.c_float(dt))

    def addTurbulence(self, dt):
        self._device(self._L.fg_add_turbulence, ctypes.c_float(dt))

    def clearPressure(self):
        self._device(self._L.fg_clear_pressure)

    def copyBorder(self, dst, src):
        assert dst.dtype == np.float32 and src.dtype == np.float32
        assert dst.size == self.numCells and src.size == self.numCells
        self._before()
        self._check(self._L.fg_copy_border(self._h, dst.ctypes.data, src.ctypes.data), "copyBorder")
        self._after()

    # ------------------------------------------------------------ tools
    def _index(self, rc, i, j):
        if rc == _lib.FG_ERR_INDEX:
            if i < 0 or i >= self.NumX:
                raise IndexError("invalid x-index: %d" % i)
            raise IndexError("invalid y-index: %d" % j)
        self._check(rc)

    def SetSolid(self, i, j, value):
        self._index(self._L.fg_set_solid(self._h, i, j, int(bool(value))), i, j)

    def IsSolid(self, i, j):
        out = ctypes.c_int()
        self._index(self._L.fg_is_solid(self._h, i, j, ctypes.byref(out)), i, j)
        return bool(out.value)

    def SetVelocity(self, i, j, u, v):
        self._index(self._L.fg_set_velocity(self._h, i, j, ctypes.c_float(u), ctypes.c_float(v)), i, j)

    def AddSmoke(self, i, j, s):
        self._index(self._L.fg_add_smoke(self._h, i, j, ctypes.c_float(s)), i, j)

    def SetVelocityMany(self, i, j, u, v):
        """n SetVelocity calls in order (one C call)."""
        i, j = np.ascontiguousarray(i, np.int32), np.ascontiguousarray(j, np.int32)
        u = np.ascontiguousarray(np.broadcast_to(u, i.shape), np.float32)
        v = np.ascontiguousarray(np.broadcast_to(v, i.shape), np.float32)
        rc = self._L.fg_set_velocity_many(self._h, i.size, i.ctypes.data, j.ctypes.data,
                                          u.ctypes.data, v.ctypes.data)
        if rc == _lib.FG_ERR_INDEX:
            raise IndexError("invalid index")
        self._check(rc, "SetVelocityMany")

    def AddSmokeMany(self, i, j, s):
        i, j = np.ascontiguousarray(i, np.int32), np.ascontiguousarray(j, np.int32)
        s = np.ascontiguousarray(np.broadcast_to(s, i.shape), np.float32)
        rc = self._L.fg_add_smoke_many(self._h, i.size, i.ctypes.data, j.ctypes.data, s.ctypes.data)
        if rc == _lib.FG_ERR_INDEX:
            raise IndexError("invalid index")
        self._check(rc, "AddSmokeMany")

    SRC_SKIP_SOLID, SRC_SET_VELOCITY, SRC_ADD_SMOKE, SRC_SET_SMOKE = 1, 2, 4, 8

    def set_sources(self, i, j, u=None, v=None, smoke=None, mode=None):
        """Persistent per-step sources applied on the device before every step."""
        i = np.ascontiguousarray(i, np.int32)
        j = np.ascontiguousarray(j, np.int32)
        n = i.size

        def arr(x, dt, default):
            return np.ascontiguousarray(np.broadcast_to(default if x is None else x, (n,)), dt)

        u, v, sm = arr(u, np.float32, 0.0), arr(v, np.float32, 0.0), arr(smoke, np.float32, 0.0)
        md = arr(mode, np.int32, self.SRC_SET_VELOCITY)
        rc = self._L.fg_set_sources(self._h, n, i.ctypes.data, j.ctypes.data, u.ctypes.data,
                                    v.ctypes.data, sm.ctypes.data, md.ctypes.data)
        if rc == _lib.FG_ERR_INDEX:
            raise IndexError("invalid source index")
        self._check(rc, "set_sources")

    def launch_count(self):
        return int(self._L.fg_launch_count(self._h))

    def edit_bytes(self):
        return int(self._L.fg_edit_bytes(self._h))

    def profile(self, on=True):
        self._check(self._L.fg_profile_enable(self._h, int(bool(on))), "fg_profile_enable")

    def jacobi_span(self):
        """(milliseconds, sweep blocks) of the main Jacobi solve of the last step
        (blocks of tb_depth sweeps: launches, or phases of the dataflow kernel)."""
        ms, n = ctypes.c_float(), ctypes.c_int()
        self._check(self._L.fg_profile_jacobi(self._h, ctypes.byref(ms), ctypes.byref(n)),
                    "fg_profile_jacobi")
        return ms.value, n.value

    def stage_times(self):
        """[(stage, ms)] of the last step run with profiling on."""
        ms = (ctypes.c_float * 16)()
        names = (ctypes.c_char_p * 16)()
        n = self._L.fg_profile_stages(self._h, 16, ms, names)
        if n < 0:
            self._check(n, "fg_profile_stages")
        return [(names[k].decode(), ms[k]) for k in range(n)]

    # ------------------------------------------------------------ differentiable rollouts
    # The Step / StepAdjoint pair of include/fluidgpu.h.  Fields (forces,
    # seeds, targets, gradients) are numpy float32 arrays of numCells values
    # in the mirrors' layout, or float32 torch tensors of that size (host or
    # device memory).  During a recorded rollout the mirrors are not kept in
    # sync: call download() to read the state.
    def _field_ptr(self, x, writable=False):
        if x is None:
            return None
        if isinstance(x, np.ndarray):
            if x.dtype != np.float32 or x.size != self.numCells or not x.flags.c_contiguous:
                raise ValueError("expected a contiguous float32 array of %d values" % self.numCells)
            if writable and not x.flags.writeable:
                raise ValueError("output array is read-only")
            return x.ctypes.data
        if hasattr(x, "data_ptr"):
            import torch

            if x.dtype != torch.float32 or x.numel() != self.numCells or not x.is_contiguous():
                raise ValueError("expected a contiguous float32 tensor of %d values" % self.numCells)
            return x.data_ptr()
        raise TypeError("expected a numpy array or a torch tensor")

    def tape_begin(self, max_steps, every=8):
        """Starts a recorded rollout from the current state (fg_tape_begin)."""
        self._before()
        self._check(self._L.fg_tape_begin(self._h, int(max_steps), int(every)), "fg_tape_begin")

    def step_forward(self, dt, force_u=None, force_v=None):
        """One recorded step with an optional force field (fg_step_forward)."""
        self._check(self._L.fg_step_forward(self._h, ctypes.c_float(dt), self._field_ptr(force_u),
                                            self._field_ptr(force_v)), "fg_step_forward")

    def tape_seed(self, dU=None, dV=None, dM=None):
        self._check(self._L.fg_tape_seed(self._h, self._field_ptr(dU), self._field_ptr(dV),
                                         self._field_ptr(dM)), "fg_tape_seed")

    def tape_seed_smoke_l2(self, target):
        """Seeds dL/dM for L = ||M - target||_2 over the interior; returns L (FP64)."""
        loss = ctypes.c_double()
        self._check(self._L.fg_tape_seed_smoke_l2(self._h, self._field_ptr(target),
                                                  ctypes.byref(loss)), "fg_tape_seed_smoke_l2")
        return loss.value

    def step_adjoint(self, grad_force_u=None, grad_force_v=None):
        """Reverses the latest step; writes that step's force gradient if given."""
        self._check(self._L.fg_step_adjoint(self._h, self._field_ptr(grad_force_u, True),
                                            self._field_ptr(grad_force_v, True)), "fg_step_adjoint")

    def tape_grad(self):
        """dL/d(initial U, V, M, newU, newV, newM) as numpy arrays."""
        out = [np.zeros(self.numCells, np.float32) for _ in range(6)]
        self._check(self._L.fg_tape_grad(self._h, *[o.ctypes.data for o in out]), "fg_tape_grad")
        return dict(zip(("U", "V", "M", "newU", "newV", "newM"), out))

    def tape_steps(self):
        a, b = ctypes.c_int(), ctypes.c_int()
        self._check(self._L.fg_tape_steps(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def tape_end(self):
        self._check(self._L.fg_tape_end(self._h), "fg_tape_end")

    def rollout_grad(self, dt, steps, target, forces=None, every=8):
        """Loss L = ||M_T - target||_2 after `steps` steps from the current
        state with per-step forces (a list of (force_u, force_v) or None), and
        its gradients: {"loss", "U", "V", "M", "newU", "newV", "newM",
        "force_u": [steps arrays], "force_v": [...]}.  The state ends where
        the forward pass ended."""
        self.tape_begin(steps, every)
        try:
            for t in range(steps):
                fu, fv = forces[t] if forces is not None else (None, None)
                self.step_forward(dt, fu, fv)
            loss = self.tape_seed_smoke_l2(target)
            gfu = [np.zeros(self.numCells, np.float32) for _ in range(steps)]
            gfv = [np.zeros(self.numCells, np.float32) for _ in range(steps)]
            for t in reversed(range(steps)):
                self.step_adjoint(gfu[t], gfv[t])
            out = self.tape_grad()
        finally:
            self.tape_end()
        out.update(loss=loss, force_u=gfu, force_v=gfv)
        return out

    # ------------------------------------------------------------ particles, rendering
    def particles_add(self, x, y, max_age, rgb, max_total=0):
        """Appends particles at world positions (x, y) with age 0 (the app's
        spawnParticles, main/main.go:489-510); rgb: (n, 3) uint8."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        ma = np.ascontiguousarray(np.broadcast_to(max_age, x.shape), np.float32)
        c = np.ascontiguousarray(np.broadcast_to(rgb, (x.size, 3)), np.uint8)
        self._check(self._L.fg_particles_add(self._h, x.size, x.ctypes.data, y.ctypes.data,
                                             ma.ctypes.data, c.ctypes.data, int(max_total)),
                    "fg_particles_add")

    def particles_advect(self, dt):
        """advectParticles (main/main.go:512-546) on the device."""
        self._check(self._L.fg_particles_advect(self._h, ctypes.c_float(dt)),
                    "fg_particles_advect")

    def particles(self):
        n = ctypes.c_int()
        self._check(self._L.fg_particles_count(self._h, ctypes.byref(n)), "fg_particles_count")
        out = {k: np.zeros(n.value, np.float32) for k in ("X", "Y", "Age", "MaxAge")}
        rgb = np.zeros((n.value, 3), np.uint8)
        self._check(self._L.fg_particles_get(self._h, out["X"].ctypes.data, out["Y"].ctypes.data,
                                             out["Age"].ctypes.data, out["MaxAge"].ctypes.data,
                                             rgb.ctypes.data), "fg_particles_get")
        out["RGB"] = rgb
        return out

    def debug_stall_tile(self, tile):
        """Fault injection: the dataflow Jacobi kernel never publishes `tile`,
        so the step's bounded waits give up and stats() raises FG_ERR_TIMEOUT
        (tile < 0 disarms)."""
        self._check(self._L.fg_debug_stall_tile(self._h, int(tile)), "fg_debug_stall_tile")

    def particles_clear(self):
        self._check(self._L.fg_particles_clear(self._h), "fg_particles_clear")

    RENDER_SMOKE, RENDER_PRESSURE, RENDER_SPEED, RENDER_VORTICITY = 0, 1, 2, 3

    def render(self, kind):
        """The app's drawScalarField / drawVorticityField image (NumX * NumY *
        4 bytes RGBA, pixel (i, j) showing cell (i, NumY - 1 - j))."""
        self._before()
        out = np.zeros(self.numCells * 4, np.uint8)
        self._check(self._L.fg_render(self._h, int(kind), out.ctypes.data), "fg_render")
        self._after()
        return out

    def Reset(self):
        self._check(self._L.fg_reset(self._h), "Reset")

    def ApplyForce(self, i, j, fx, fy):
        self._check(self._L.fg_apply_force(self._h, i, j, ctypes.c_float(fx), ctypes.c_float(fy)))

    def ApplyForceRadius(self, cx, cy, fx, fy, radius):
        self._check(self._L.fg_apply_force_radius(self._h, cx, cy, ctypes.c_float(fx),
                                                  ctypes.c_float(fy), radius))

    def SetCircularObstacle(self, cx, cy, radius):
        self._check(self._L.fg_set_circular_obstacle(self._h, cx, cy, radius))

    # ------------------------------------------------------------ views
    def _scalar(self, fn, *args):
        self._before()
        outs = [ctypes.c_float() for _ in range(2)]
        self._check(fn(self._h, *args, *[ctypes.byref(o) for o in outs]))
        self._after()
        return [o.value for o in outs]

    def MaxDivergence(self):
        self._before()
        out = ctypes.c_float()
        self._check(self._L.fg_max_divergence(self._h, ctypes.byref(out)), "MaxDivergence")
        self._after()
        return out.value

    def GetAdaptiveTimeStep(self, basedt):
        self._before()
        out = ctypes.c_float()
        self._check(self._L.fg_adaptive_time_step(self._h, ctypes.c_float(basedt), ctypes.byref(out)))
        self._after()
        return out.value

    def SampleVelocity(self, x, y):
        return tuple(self._scalar(self._L.fg_sample_velocity, ctypes.c_float(x), ctypes.c_float(y)))

    def _view(self, fn):
        self._before()
        out = np.zeros(self.numCells, dtype=np.float32)
        mn, mx = ctypes.c_float(), ctypes.c_float()
        self._check(fn(self._h, out.ctypes.data, ctypes.byref(mn), ctypes.byref(mx)))
        self._after()
        return ScalarField(self.NumX, self.NumY, out, mn.value, mx.value)

    def Vorticity(self):
        return self._view(self._L.fg_vorticity)

    def VelocityMagnitude(self):
        return self._view(self._L.fg_velocity_magnitude)

    def _minmax_view(self, field):
        mn, mx = self._scalar(self._L.fg_field_min_max, FIELDS[field])
        if not self.auto_sync:
            self.download(1 << FIELDS[field])
        return ScalarField(self.NumX, self.NumY, self._views[field], mn, mx)

    def Pressure(self):
        return self._minmax_view("p")

    def Smoke(self):
        return self._minmax_view("M")

    def Velocity(self):
        if not self.auto_sync:
            self.download((1 << FIELDS["U"]) | (1 << FIELDS["V"]))
        return VectorField(self.NumX, self.NumY, self.U, self.V)


class Batch:
    """Many Fluid scenes stepped together (fg_batch_create).

    The scenes keep their own sizes, obstacles, sources and num_iters; they
    must share every other parameter (Jacobi scheme, no early exit,
    refinement or viscosity).  ``step`` advances every scene; ``scatter``
    copies the batch's state back into the scene objects (whose mirrors are
    then refreshed on ``download``).  The scene objects must outlive the
    batch; the batch holds references to them.
    """

    def __init__(self, scenes):
        scenes = list(scenes)
        if not scenes:
            raise ValueError("empty batch")
        L = _lib.lib()
        self._L = L
        self.scenes = scenes
        for s in scenes:
            s._before()  # push parameters and, with auto_sync, the mirrors
        arr = (ctypes.c_void_p * len(scenes))(*[s.handle.value for s in scenes])
        h = ctypes.c_void_p()
        rc = L.fg_batch_create(arr, len(scenes), ctypes.byref(h))
        if rc != 0:
            msg = L.fg_last_error(scenes[0].handle)
            raise FluidError(rc, "fg_batch_create: %s" % (msg.decode() if msg else ""))
        self._h = h

    def __del__(self):
        h = self.__dict__.get("_h")
        if h:
            self._L.fg_destroy(h)
            self._h = None

    def close(self):
        self.__del__()

    def __len__(self):
        return len(self.scenes)

    def _check(self, rc, what):
        if rc != 0:
            msg = self._L.fg_last_error(self._h)
            raise FluidError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    @property
    def handle(self):
        return self._h

    @property
    def stream(self):
        return self._L.fg_stream(self._h)

    def step(self, dt):
        self._check(self._L.fg_batch_step(self._h, ctypes.c_float(dt)), "fg_batch_step")

    def synchronize(self):
        self._check(self._L.fg_synchronize(self._h), "fg_synchronize")

    def scatter(self):
        """Copies every scene's state from the batch into its Fluid object."""
        self._check(self._L.fg_batch_scatter(self._h), "fg_batch_scatter")
        for s in self.scenes:
            if s.auto_sync:
                s.download()

    def gather(self):
        """Copies every Fluid object's state into the batch."""
        for s in self.scenes:
            s._before()
        self._check(self._L.fg_batch_gather(self._h), "fg_batch_gather")

    def autotune(self, dt, reps=3):
        """(tb_depth, block_x, block_y, ms_per_step) of the fastest candidate."""
        tb, bx, by = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = ctypes.c_float()
        self._check(self._L.fg_batch_autotune(self._h, ctypes.c_float(dt), int(reps),
                                              ctypes.byref(tb), ctypes.byref(bx),
                                              ctypes.byref(by), ctypes.byref(ms)),
                    "fg_batch_autotune")
        return tb.value, bx.value, by.value, ms.value

    def launch_count(self):
        return int(self._L.fg_launch_count(self._h))

    def profile(self, on=True):
        self._check(self._L.fg_profile_enable(self._h, int(bool(on))), "fg_profile_enable")

    # ------------------------------------------------------------ recorded rollouts
    def tape_begin(self, max_steps, every=8):
        self._check(self._L.fg_tape_begin(self._h, int(max_steps), int(every)), "fg_tape_begin")

    def step_forward(self, dt):
        self._check(self._L.fg_step_forward(self._h, ctypes.c_float(dt), None, None),
                    "fg_step_forward")

    def seed_smoke_l2(self, targets):
        """Seeds L_s = ||M_s - targets[s]||_2 per scene; returns the n losses."""
        keep = [np.ascontiguousarray(t, np.float32) if isinstance(t, np.ndarray) else t
                for t in targets]
        ptrs = (ctypes.c_void_p * len(keep))(
            *[t.ctypes.data if isinstance(t, np.ndarray) else t.data_ptr() for t in keep])
        losses = (ctypes.c_double * len(keep))()
        self._check(self._L.fg_batch_seed_smoke_l2(self._h, ptrs, losses),
                    "fg_batch_seed_smoke_l2")
        return np.array(losses[:], np.float64)

    def step_adjoint(self):
        self._check(self._L.fg_batch_step_adjoint(self._h), "fg_batch_step_adjoint")

    def grad(self, s):
        """dL_s/d(initial U, V, M) of scene s."""
        n = self.scenes[s].numCells
        out = [np.zeros(n, np.float32) for _ in range(3)]
        self._check(self._L.fg_batch_grad(self._h, int(s), *[o.ctypes.data for o in out]),
                    "fg_batch_grad")
        return dict(zip(("U", "V", "M"), out))

    def tape_end(self):
        self._check(self._L.fg_tape_end(self._h), "fg_tape_end")

    def rollout_grad(self, dt, steps, targets, every=8):
        """Per-scene losses ||M_s - targets[s]||_2 after `steps` steps and each
        scene's gradients w.r.t. its initial U, V, M."""
        self.tape_begin(steps, every)
        try:
            for _ in range(steps):
                self.step_forward(dt)
            losses = self.seed_smoke_l2(targets)
            for _ in range(steps):
                self.step_adjoint()
            grads = [self.grad(s) for s in range(len(self.scenes))]
        finally:
            self.tape_end()
        return losses, grads
