"""Seeded synthetic scenes shared by the parity tests and the benchmark.

Walls and sources follow the reference app's presets (main/main.go:761-793,
840-849); every scene only calls the Go API surface, so it runs unchanged on
the CPU oracle and on the CUDA path.
"""
from __future__ import annotations

import numpy as np


def apply_walls(f, top=True, bottom=True, left=True, right=False):
    """applyWallSettings (main/main.go:840-849) after clearing every cell."""
    for i in range(f.NumX):
        for j in range(f.NumY):
            f.SetSolid(i, j, False)
    for i in range(f.NumX):
        f.SetSolid(i, 0, bottom)
        f.SetSolid(i, f.NumY - 1, top)
    for j in range(f.NumY):
        f.SetSolid(0, j, left)
        f.SetSolid(f.NumX - 1, j, right)


def fast_walls(f, top=True, bottom=True, left=True, right=False):
    """Same mask as apply_walls, written directly into S (for large grids)."""
    S = f.S.reshape(f.NumX, f.NumY)
    S[:] = 1.0
    S[:, 0] = 0.0 if bottom else 1.0
    S[:, -1] = 0.0 if top else 1.0
    S[0, :] = 0.0 if left else 1.0
    S[-1, :] = 0.0 if right else 1.0


def jet_rows(f, half=4):
    return range(f.NumY // 2 - half, f.NumY // 2 + half)


def jet_inject(f, speed=2.0, smoke=1.0, half=4):
    """Jet inlet on the left wall: U = speed, M = smoke on 2*half rows at i = 1."""
    n = f.NumY
    for j in jet_rows(f, half):
        f.SetVelocity(1, j, speed, 0.0)
        f.M[1 * n + j] = smoke


def jet_scene(f):
    apply_walls(f, top=True, bottom=True, left=True, right=False)


def karman_scene(f, radius=24, seed=2, noise=1e-3):
    """Inflow left, outflow right, slip walls top/bottom, disc at (W/4, H/2)."""
    apply_walls(f, top=True, bottom=True, left=False, right=False)
    cx, cy = (f.NumX - 2) // 4, (f.NumY - 2) // 2
    f.SetCircularObstacle(cx, cy, radius)
    rng = np.random.default_rng(seed)
    U = f.U.reshape(f.NumX, f.NumY)
    S = f.S.reshape(f.NumX, f.NumY)
    U[1:-1, 1:-1] = (1.0 + rng.uniform(-noise, noise, (f.NumX - 2, f.NumY - 2))) * (S[1:-1, 1:-1] != 0)


def karman_inflow(f, speed=1.0):
    n = f.NumY
    for j in range(1, f.NumY - 1):
        if f.S[1 * n + j] != 0:
            f.SetVelocity(1, j, speed, 0.0)


def cavity_scene(f):
    apply_walls(f, top=True, bottom=True, left=True, right=True)


def cavity_lid(f, speed=1.0):
    """Source row under the top wall (main/main.go:774-779), without smoke."""
    j = f.NumY - 2
    for i in range(2, f.NumX - 2):
        f.SetVelocity(i, j, speed, 0.0)


def random_state(f, seed=0, amp=1.0, smoke=True):
    rng = np.random.default_rng(seed)
    f.U[:] = rng.uniform(-amp, amp, f.numCells).astype(f.dtype)
    f.V[:] = rng.uniform(-amp, amp, f.numCells).astype(f.dtype)
    if smoke:
        f.M[:] = rng.uniform(0, 1, f.numCells).astype(f.dtype)


# ---------------------------------------------------------------- differentiable rollout
def jet_rollout_scene(f, speed=2.0, smoke=1.0, half=4):
    """Jet scene of the differentiable rollout: walls left, top and bottom,
    open right; a jet of 2*half rows at i = 1 held by device sources (U =
    speed, V = 0, M = smoke assigned before every step, as fluid_test.go
    :396-401 does on the host).  Zero initial state."""
    fast_walls(f)
    f.mark_dirty()
    rows = np.array(list(jet_rows(f, half)), np.int32)
    f.set_sources(np.ones_like(rows), rows, u=speed, v=0.0, smoke=smoke,
                  mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY | f.SRC_SET_SMOKE)


def gaussian_target(nx, ny, seed=4, n=4, sigma=(10.0, 30.0), amp=(0.5, 1.0)):
    """Sum of n seeded isotropic Gaussian blobs (sigma and amplitude drawn
    uniformly, centres uniform over the interior), as NX*NY float32."""
    rng = np.random.default_rng(seed)
    i = np.arange(nx)[:, None]
    j = np.arange(ny)[None, :]
    T = np.zeros((nx, ny))
    for _ in range(n):
        s = rng.uniform(*sigma)
        a = rng.uniform(*amp)
        ci, cj = rng.uniform(1, nx - 1), rng.uniform(1, ny - 1)
        T += a * np.exp(-((i - ci) ** 2 + (j - cj) ** 2) / (2 * s * s))
    return T.ravel().astype(np.float32)


# ---------------------------------------------------------------- ensembles
def ensemble_scene(f, rng, radius=(4.0, 32.0), speed=(0.5, 2.0)):
    """One scene of a batched ensemble on f: walls left, top and bottom, open
    right; 0-5 solid discs (radius drawn from `radius`, capped at a sixth of
    the smaller side) and 1-3 jet inlets of 8 rows on the left wall (U drawn
    from `speed`, smoke assigned 1) held by device sources."""
    fast_walls(f)
    f.mark_dirty()
    nx, ny = f.NumX - 2, f.NumY - 2
    for _ in range(int(rng.integers(0, 6))):
        r = int(min(rng.uniform(*radius), max(1, min(nx, ny) // 6)))
        cx = int(rng.uniform(nx * 0.3, max(nx * 0.3 + 1, nx - r - 1)))
        cy = int(rng.uniform(r + 2, max(r + 3, ny - r - 2)))
        f.SetCircularObstacle(cx, cy, r)
    rows, us = [], []
    for _ in range(int(rng.integers(1, 4))):
        c = int(rng.uniform(5, max(6, ny - 4)))
        sp = float(rng.uniform(*speed))
        for j in range(max(1, c - 4), min(ny + 1, c + 4)):
            rows.append(j)
            us.append(sp)
    rows = np.array(rows, np.int32)
    f.set_sources(np.ones_like(rows), rows, u=np.array(us, np.float32), v=0.0, smoke=1.0,
                  mode=f.SRC_SKIP_SOLID | f.SRC_SET_VELOCITY | f.SRC_SET_SMOKE)


def ensemble_sides(n, seed=5, lo=64, hi=512):
    """Square grid sides drawn log-uniformly from [lo, hi] (seeded)."""
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))))) for _ in range(n)]
