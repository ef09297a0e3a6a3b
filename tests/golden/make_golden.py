"""Writes the golden fixtures of the 128x128 jet (the CPU-runnable parity
configuration): 128x128 MAC grid, h = 1, dt = 0.1, density 1, walls left,
top and bottom, open right, an 8-cell jet at mid-height on the left wall
(U = 2 set and smoke M = 1 assigned before every step, as fluid_test.go:396-
401 does), semi-Lagrangian advection, no confinement, the New() turbulence
0.02, 40 pressure iterations per step with the reference's early exit, zero
initial state, 200 steps.

jet128_fp32.npz: the FP32-faithful oracle (the reference's float32 step with
the serial SOR) after 200 steps, every state field, plus the max |U| after
every 20 steps.  jet128_fp64.npz: the FP64 oracle after 200 steps (U, V, M,
p), stored as float64.

Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import scenes  # noqa: E402
from oracle.pyoracle import OracleFluid  # noqa: E402

W = H = 128
STEPS = 200
ITERS = 40


def run(make, steps=STEPS, every=20):
    f = make(1.0, W, H, 1.0)
    f.num_iters = ITERS
    scenes.jet_scene(f)
    trace = []
    for k in range(1, steps + 1):
        scenes.jet_inject(f, speed=2.0, smoke=1.0)
        f.Simulate(0.1)
        if k % every == 0:
            trace.append(float(np.abs(np.asarray(f.U, np.float64)).max()))
    return f, np.array(trace)


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    f, trace = run(lambda *a: OracleFluid(*a, prec=32))
    np.savez_compressed(os.path.join(here, "jet128_fp32.npz"),
                        **{k: np.asarray(getattr(f, k)).copy() for k in
                           ("U", "V", "M", "p", "newU", "newV", "newM", "S")},
                        max_u_every_20=trace)
    g, _ = run(lambda *a: OracleFluid(*a, prec=64))
    np.savez_compressed(os.path.join(here, "jet128_fp64.npz"),
                        **{k: np.asarray(getattr(g, k)).copy() for k in ("U", "V", "M", "p")})


if __name__ == "__main__":
    main()
