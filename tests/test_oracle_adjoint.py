"""The FP64 reverse-mode reference of recorded rollouts (oracle
orc_rollout_grad) against central differences of the FP64 oracle's own
forward pass: it is the full-field reference the CUDA adjoint is compared
with, so it is pinned here on its own (no GPU)."""
import numpy as np
import pytest

import scenes
from oracle.pyoracle import OracleFluid

W, H, DT, ITERS, STEPS = 22, 18, 0.1, 16, 5


def make(conf, bfecc):
    o = OracleFluid(1.0, W, H, 1.0, prec=64, scheme=1, num_iters=ITERS, check_every=8,
                    early_exit=False, UseBFECC=bfecc, Confinement=conf)
    scenes.fast_walls(o)
    return o


def state(o, seed=1):
    rng = np.random.default_rng(seed)
    nx, ny = o.NumX, o.NumY
    x = np.arange(nx)[:, None] / nx
    y = np.arange(ny)[None, :] / ny
    U = 0.8 * np.sin(2.1 * np.pi * x + 0.3) * np.cos(1.3 * np.pi * y)
    V = 0.6 * np.cos(1.7 * np.pi * x) * np.sin(2.4 * np.pi * y + 0.5)
    # Off-centre: a blob centred on a cell row makes mirror cells tie exactly,
    # where the BFECC clamp has a kink.
    M = np.exp(-((x - 0.4137) ** 2 + (y - 0.5291) ** 2) / 0.03)
    S = o.S.reshape(nx, ny) != 0
    U[1:, :] *= S[1:, :] * S[:-1, :]
    V[:, 1:] *= S[:, 1:] * S[:, :-1]
    F = rng.uniform(-0.05, 0.05, (STEPS, 2, nx * ny))
    T = np.exp(-((x - 0.7) ** 2 + (y - 0.4) ** 2) / 0.05).ravel()
    return U.ravel(), V.ravel(), (M * S).ravel(), F, T


def loss(conf, bfecc, U0, V0, M0, F, T, srcs):
    o = make(conf, bfecc)
    o.U[:], o.V[:], o.M[:] = U0, V0, M0
    for t in range(STEPS):
        o.U[:] += F[t, 0]
        o.V[:] += F[t, 1]
        for (i, j, u, v, s, mode) in srcs:
            o.SetVelocity(i, j, u, v)
            o.AddSmoke(i, j, s)
        o.Simulate(DT)
    d = (o.M - T).reshape(o.NumX, o.NumY)[1:-1, 1:-1]
    return float(np.sqrt(np.sum(d * d)))


@pytest.mark.parametrize("conf,bfecc", [(0.0, True), (0.3, False), (0.3, True)])
def test_fp64_adjoint_matches_fp64_central_differences(conf, bfecc):
    o = make(conf, bfecc)
    U0, V0, M0, F, T = state(o)
    srcs = [(1, j, 2.0, 0.0, 1.0, 1 | 2 | 4) for j in scenes.jet_rows(o)]
    o.U[:], o.V[:], o.M[:] = U0, V0, M0
    out = o.rollout_grad(DT, STEPS, T, F, srcs)
    assert out["loss"] == pytest.approx(loss(conf, bfecc, U0, V0, M0, F, T, srcs), rel=1e-13)
    n = o.NumX * o.NumY
    for k in range(3):
        rng = np.random.default_rng(30 + k)
        dU, dV = rng.standard_normal(n) * 0.5, rng.standard_normal(n) * 0.5
        dF = rng.standard_normal((STEPS, 2, n)) * 0.05
        dM = rng.standard_normal(n) * 0.5 * M0
        g = (np.dot(out["U"], dU) + np.dot(out["V"], dV) + np.dot(out["M"], dM)
             + np.sum(out["force_u"] * dF[:, 0]) + np.sum(out["force_v"] * dF[:, 1]))
        eps = 1e-7
        fd = (loss(conf, bfecc, U0 + eps * dU, V0 + eps * dV, M0 + eps * dM, F + eps * dF, T, srcs)
              - loss(conf, bfecc, U0 - eps * dU, V0 - eps * dV, M0 - eps * dM, F - eps * dF, T,
                     srcs)) / (2 * eps)
        assert g == pytest.approx(fd, rel=2e-5, abs=1e-8), (k, g, fd)
