"""The CPU oracle against the reference's own tests (no GPU needed).

The reference has no golden field dumps; its known-answer and threshold tests
(pkg/fluid/fluid_test.go, confinement_test.go) are the pin.  They run here
against the FP32-faithful and the FP64 restatement of the reference scheme.
"""
import numpy as np
import pytest

import reference_cases as rc
from oracle.pyoracle import JACOBI, LEXSOR, REDBLACK, OracleFluid


def _maker(**kw):
    return lambda d, w, h, hh: OracleFluid(d, w, h, hh, **kw)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("case", rc.ALL_CASES + [rc.case_multigrid_stability], ids=lambda c: c.__name__)
def test_reference_case_on_oracle(case, prec):
    case(_maker(prec=prec))


def _jet(f, steps, dt=0.1):
    """128x128 jet scene: left/top/bottom walls solid, right open; 8-cell jet."""
    n = f.NumY
    for i in range(f.NumX):
        for j in range(f.NumY):
            f.SetSolid(i, j, False)
    for i in range(f.NumX):
        f.SetSolid(i, 0, True)
        f.SetSolid(i, f.NumY - 1, True)
    for j in range(f.NumY):
        f.SetSolid(0, j, True)
        f.SetSolid(f.NumX - 1, j, False)
    for _ in range(steps):
        for j in range(f.NumY // 2 - 4, f.NumY // 2 + 4):
            f.SetVelocity(1, j, 2.0, 0.0)
            f.M[1 * n + j] = 1.0
        f.Simulate(dt)


def test_fp32_tracks_fp64_on_jet():
    a = OracleFluid(1.0, 48, 48, 1.0, prec=32, num_iters=40)
    b = OracleFluid(1.0, 48, 48, 1.0, prec=64, num_iters=40)
    _jet(a, 20)
    _jet(b, 20)
    for k in ("U", "V", "M"):
        x, y = getattr(a, k).astype(np.float64), getattr(b, k)
        scale = max(1.0, float(np.abs(y).max()))
        assert float(np.abs(x - y).max()) / scale < 1e-3, k


@pytest.mark.parametrize("scheme", [JACOBI, REDBLACK])
def test_parallel_scheme_threads_do_not_change_bits(scheme):
    a = OracleFluid(1.0, 40, 30, 1.0, threads=1, scheme=scheme, num_iters=30, UseBFECC=True)
    b = OracleFluid(1.0, 40, 30, 1.0, threads=4, scheme=scheme, num_iters=30, UseBFECC=True)
    _jet(a, 10)
    _jet(b, 10)
    for k in ("U", "V", "M", "p", "newU", "newV", "newM"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


def test_jacobi_converges_to_small_divergence():
    f = OracleFluid(1.0, 16, 16, 1.0, scheme=JACOBI, early_exit=False)
    f.S[:] = 1.0
    rng = np.random.default_rng(0)
    f.U[:] = rng.uniform(-1, 1, f.numCells).astype(np.float32)
    f.V[:] = rng.uniform(-1, 1, f.numCells).astype(np.float32)
    f.makeIncompressible(2000, 0.1)
    st = f.stats()
    assert st["div_max_post"] < 1e-4
    assert st["resid_max"] < 1e-4


def test_early_exit_check_interval():
    f = OracleFluid(1.0, 16, 16, 1.0, scheme=JACOBI, check_every=4, tolerance=1e30)
    f.S[:] = 1.0
    f.makeIncompressible(40, 0.1)
    assert f.stats()["sweeps"] == 4
    g = OracleFluid(1.0, 16, 16, 1.0, scheme=LEXSOR, tolerance=1e30)
    g.S[:] = 1.0
    g.makeIncompressible(40, 0.1)
    assert g.stats()["sweeps"] == 1


def test_refinement_reduces_fp64_residual():
    kw = dict(scheme=JACOBI, early_exit=False)
    a = OracleFluid(1.0, 24, 24, 1.0, **kw)
    b = OracleFluid(1.0, 24, 24, 1.0, refine_sweeps=200, **kw)
    for f in (a, b):
        f.S[:] = 1.0
        f.S[: f.NumY] = 0.0
        rng = np.random.default_rng(1)
        f.U[:] = rng.uniform(-1, 1, f.numCells).astype(np.float32)
        f.makeIncompressible(50, 0.1)
    # The statistics are those of the final potential: the correction lowers
    # its residual and the divergence of the projected field.
    assert b.stats()["resid_l2"] < a.stats()["resid_l2"]
    assert b.stats()["div_l2_post"] < a.stats()["div_l2_post"]


def test_oracle_reproduces_golden_jet128():
    """The committed fixtures of the 128x128 jet (tests/golden/make_golden.py)
    pin the oracle: the FP32 restatement reproduces them bit for bit and the
    FP64 one exactly."""
    import os
    import sys

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    sys.path.insert(0, here)
    import make_golden

    gold = np.load(os.path.join(here, "jet128_fp32.npz"))
    f, trace = make_golden.run(lambda *a: OracleFluid(*a, prec=32))
    for k in ("U", "V", "M", "p", "newU", "newV", "newM", "S"):
        assert np.array_equal(np.asarray(getattr(f, k)).view(np.uint32), gold[k].view(np.uint32)), k
    assert np.array_equal(trace, gold["max_u_every_20"])
    gold64 = np.load(os.path.join(here, "jet128_fp64.npz"))
    g, _ = make_golden.run(lambda *a: OracleFluid(*a, prec=64))
    for k in ("U", "V", "M", "p"):
        assert np.array_equal(np.asarray(getattr(g, k)), gold64[k]), k
