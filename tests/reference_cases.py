"""The reference's own tests for pkg/fluid, restated as backend-neutral cases.

Each ``case_*`` follows one Go test of pkg/fluid/fluid_test.go or
pkg/fluid/confinement_test.go (cited per case) with the same set-up, the
same stage calls and the same thresholds.  ``make(density, width, height, h)``
builds a fluid that exposes the Go ``Fluid`` surface (the CPU oracle or the
CUDA path); stage calls (``makeIncompressible``, ``advectVelocity``...) are
the white-box entry points those Go tests call.
"""
from __future__ import annotations

import math

import numpy as np

f32 = np.float32


def _all_fluid(f):
    f.S[:] = 1.0


def calculate_divergence(f):
    """fluid_test.go:266-285 (mean |div| over fluid cells, float32 sums)."""
    n = f.NumY
    U, V, S = f.U, f.V, f.S
    total = f32(0.0)
    count = 0
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            if S[i * n + j] > 0:
                div = f32(U[(i + 1) * n + j]) - f32(U[i * n + j]) + f32(V[i * n + j + 1]) - f32(V[i * n + j])
                total = f32(total + f32(abs(div)))
                count += 1
    return float(total / f32(count)) if count else 0.0


def case_copy_border(make):
    """TestCopyBorder fluid_test.go:8-35."""
    f = make(1.0, 3, 3, 1.0)
    src = np.arange(1, f.numCells + 1, dtype=f.dtype)
    dst = np.zeros(f.numCells, dtype=f.dtype)
    f.copyBorder(dst, src)
    n = f.NumY
    for i in range(f.NumX):
        assert dst[i * n + 0] == src[i * n + 0]
        assert dst[i * n + f.NumY - 1] == src[i * n + f.NumY - 1]
    for j in range(f.NumY):
        assert dst[0 * n + j] == src[0 * n + j]
        assert dst[(f.NumX - 1) * n + j] == src[(f.NumX - 1) * n + j]


def case_diffusion_behavior(make):
    """TestDiffusionBehavior fluid_test.go:37-82."""
    f = make(1.0, 10, 10, 1.0)
    _all_fluid(f)
    n = f.NumY
    cx, cy = f.NumX // 2, f.NumY // 2
    f.U[cx * n + cy] = 10.0
    f.V[cx * n + cy] = 10.0
    initialU = f.U.copy()
    f.makeIncompressible(10, 0.01)
    tol = 0.05
    assert f.U[cx * n + cy] < initialU[cx * n + cy]
    for i, j in ((cx - 1, cy), (cx + 1, cy), (cx, cy - 1), (cx, cy + 1)):
        if 0 < i < f.NumX - 1 and 0 < j < f.NumY - 1:
            assert not (abs(f.U[i * n + j]) < tol and abs(f.V[i * n + j]) < tol), (i, j)


def case_velocity_advection(make):
    """TestVelocityAdvection fluid_test.go:84-147."""
    f = make(1.0, 10, 10, 1.0)
    _all_fluid(f)
    n = f.NumY
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            f.U[i * n + j] = 2.0
            f.V[i * n + j] = 0.0
    tx, ty = 3, 5
    f.V[tx * n + ty] = 5.0
    initialV = f.V.copy()
    f.advectVelocity(0.1)
    ax = tx + 1
    if ax < f.NumX - 1:
        assert f.V[ax * n + ty] > initialV[ax * n + ty]
    assert f.V[tx * n + ty] < f32(5.0) * f32(0.9)
    tot = f32(0.0)
    cnt = 0
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            tot = f32(tot + f.U[i * n + j])
            cnt += 1
    assert tot / cnt >= 2.0 * 0.8


def case_smoke_advection(make):
    """TestSmokeAdvection fluid_test.go:149-208."""
    f = make(1.0, 10, 10, 1.0)
    _all_fluid(f)
    n = f.NumY
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            f.U[i * n + j] = 3.0
            f.V[i * n + j] = 0.0
    sx, sy = 2, 5
    f.M[sx * n + sy] = 1.0
    initialM = f.M.copy()
    f.advectSmoke(0.1)
    moved = any(f.M[i * n + sy] > initialM[i * n + sy] + 0.01 for i in range(sx, min(sx + 3, f.NumX - 1)))
    assert moved
    it = f32(0.0)
    ft = f32(0.0)
    M = f.M
    for k in range(f.numCells):
        it = f32(it + initialM[k])
        ft = f32(ft + M[k])
    assert abs(float(ft - it)) <= 0.1


def case_pressure_projection(make):
    """TestPressureProjection fluid_test.go:210-264."""
    f = make(1.0, 8, 8, 1.0)
    _all_fluid(f)
    n = f.NumY
    cx, cy = f.NumX // 2, f.NumY // 2
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            dx = f32(i - cx)
            dy = f32(j - cy)
            dist = f32(math.sqrt(float(dx * dx + dy * dy))) + f32(0.1)
            f.U[i * n + j] = dx / dist
            f.V[i * n + j] = dy / dist
    initial = calculate_divergence(f)
    f.makeIncompressible(20, 0.01)
    final = calculate_divergence(f)
    assert final < initial * 0.5, (initial, final)
    U, V = f.U, f.V
    mx = 0.0
    for i in range(2, f.NumX - 2):
        for j in range(2, f.NumY - 2):
            div = U[(i + 1) * n + j] - U[i * n + j] + V[i * n + j + 1] - V[i * n + j]
            mx = max(mx, abs(float(div)))
    assert mx <= 0.4, mx


def case_boundary_conditions(make):
    """TestBoundaryConditions fluid_test.go:287-355."""
    f = make(1.0, 6, 6, 1.0)
    _all_fluid(f)
    n = f.NumY
    ox, oy = 3, 3
    f.S[ox * n + oy] = 0.0
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            f.U[i * n + j] = 1.0
            f.V[i * n + j] = 0.5
    f.handleBorders()
    S, U = f.S, f.U
    for i in range(f.NumX):
        if S[i * n + 0] == 0 or (i > 0 and S[i * n + 1] == 0):
            assert U[i * n + 0] == 0
        bj = f.NumY - 1
        if S[i * n + bj] == 0 or (i > 0 and S[i * n + bj - 1] == 0):
            assert U[i * n + bj] == 0
    f.makeIncompressible(10, 0.01)
    U, V = f.U, f.V
    effect = False
    for i, j in ((ox - 1, oy), (ox + 1, oy), (ox, oy - 1), (ox, oy + 1)):
        if 0 < i < f.NumX - 1 and 0 < j < f.NumY - 1:
            if abs(float(U[i * n + j]) - 1.0) > 0.05 or abs(float(V[i * n + j]) - 0.5) > 0.05:
                effect = True
                break
    assert effect


def case_realistic_jet(make):
    """TestRealisticJetSimulation fluid_test.go:357-477."""
    f = make(1.0, 30, 20, 1.0)
    _all_fluid(f)
    n = f.NumY
    jetX, jetH = 1, 8
    jc = f.NumY // 2
    js, je = jc - jetH // 2, jc + jetH // 2
    jv = 15.0
    for j in range(js, je):
        if 0 < j < f.NumY - 1:
            f.U[jetX * n + j] = jv
            f.V[jetX * n + j] = 0.0
    for j in range(js, je):
        if 0 < j < f.NumY - 1:
            f.M[jetX * n + j] = 1.0
    for _ in range(20):
        f.Simulate(0.05)
        for j in range(js, je):
            if 0 < j < f.NumY - 1:
                f.U[jetX * n + j] = jv
                f.M[jetX * n + j] = 1.0
    U, M = f.U, f.M
    avg = f32(0.0)
    cells = 0
    for j in range(js, je):
        if 0 < j < f.NumY - 1:
            avg = f32(avg + U[(jetX + 1) * n + j])
            cells += 1
    avg = avg / cells
    assert avg >= jv * 0.6, avg
    prev = 0.0
    for dist in (3, 6, 10):
        tx = jetX + dist
        if tx >= f.NumX - 1:
            continue
        spread = sum(1.0 for j in range(1, f.NumY - 1) if U[tx * n + j] > jv * 0.1)
        assert not (prev > 0 and spread < prev * 0.9), (dist, spread, prev)
        prev = spread
    transported = any(
        M[i * n + j] > 0.1
        for i in range(jetX + 2, min(jetX + 10, f.NumX - 1))
        for j in range(js, je)
        if 0 < j < f.NumY - 1
    )
    assert transported
    mom = f32(0.0)
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            mom = f32(mom + U[i * n + j] * f32(f.density))
    assert mom >= jv * jetH * f.density * 0.3, mom


def case_obstacle_vortex_shedding(make):
    """TestObstacleVortexShedding fluid_test.go:479-648."""
    f = make(1.0, 40, 25, 1.0)
    _all_fluid(f)
    n = f.NumY
    ox, oy, orad = 15, f.NumY // 2, 3
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            dx, dy = f32(i - ox), f32(j - oy)
            if dx * dx + dy * dy <= f32(orad * orad):
                f.S[i * n + j] = 0.0
    jetX, jetH = 3, 6
    jc = f.NumY // 2
    js, je = jc - jetH // 2, jc + jetH // 2
    jv = 12.0
    f.Confinement = 0.1
    for j in range(js, je):
        if 0 < j < f.NumY - 1:
            f.M[jetX * n + j] = 1.0
    for _ in range(120):
        f.Simulate(0.025)
        for j in range(js, je):
            if 0 < j < f.NumY - 1:
                f.U[jetX * n + j] = jv
                f.M[jetX * n + j] = 1.0
    U, V, S, M, P = f.U, f.V, f.S, f.M, f.p
    infl = False
    cr = orad + 2
    for i in range(ox - cr, ox + cr + 1):
        for j in range(oy - cr, oy + cr + 1):
            if 0 < i < f.NumX - 1 and 0 < j < f.NumY - 1 and S[i * n + j] > 0:
                if abs(float(V[i * n + j])) > 1.0:
                    infl = True
    assert infl
    maxc = 0.0
    h = f32(f.H())
    for i in range(ox + orad + 1, min(ox + 15, f.NumX - 2)):
        for j in range(2, f.NumY - 2):
            if S[i * n + j] > 0:
                dvdx = (V[(i + 1) * n + j] - V[(i - 1) * n + j]) / (f32(2.0) * h)
                dudy = (U[i * n + j + 1] - U[i * n + j - 1]) / (f32(2.0) * h)
                maxc = max(maxc, abs(float(dvdx - dudy)))
    assert maxc >= 0.2, maxc
    tot = 0.0
    front = -1
    for i in range(jetX + 1, f.NumX - 1):
        has = False
        for j in range(1, f.NumY - 1):
            if S[i * n + j] > 0:
                tot += float(M[i * n + j])
                if M[i * n + j] > 0.01:
                    has = True
                    front = i
        if not has and front > 0:
            break
    assert not (front < ox - 2 or tot < 0.1), (front, tot)
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            dx, dy = f32(i - ox), f32(j - oy)
            if dx * dx + dy * dy <= f32(orad * orad):
                assert S[i * n + j] == 0.0
    pv = False
    for i in range(ox - 2, ox + 5):
        for j in range(oy - 2, oy + 3):
            if 0 < i < f.NumX - 1 and 0 < j < f.NumY - 1 and S[i * n + j] > 0:
                if abs(float(P[i * n + j])) > 0.1:
                    pv = True
    assert pv


def _max_uv(f):
    n = f.NumY
    U = f.U.reshape(f.NumX, n)[1:-1, 1:-1]
    V = f.V.reshape(f.NumX, n)[1:-1, 1:-1]
    return float(np.abs(U).max()), float(np.abs(V).max())


def case_bfecc_stability(make):
    """TestBFECCStability fluid_test.go:650-702."""
    f = make(1.0, 20, 20, 1.0)
    _all_fluid(f)
    n = f.NumY
    for i in range(1, f.NumX - 1):
        for j in range(1, f.NumY - 1):
            f.U[i * n + j] = 2.0
            f.V[i * n + j] = 1.0
    for step in range(100):
        mu, mv = _max_uv(f)
        assert not (mu > 1000 or mv > 1000 or math.isnan(mu) or math.isnan(mv)), step
        f.Simulate(0.2)
        if step % 10 == 0:
            f.U[5 * n + 5] = 3.0
            f.V[5 * n + 5] = 2.0


def case_bfecc_jet_stability(make):
    """TestBFECCJetStability fluid_test.go:704-758."""
    f = make(1.0, 30, 20, 1.0)
    _all_fluid(f)
    n = f.NumY
    jc = f.NumY // 2
    js, je = jc - 3, jc + 3
    for step in range(30):
        for j in range(js, je):
            if 0 < j < f.NumY - 1:
                f.U[1 * n + j] = 20.0
                f.V[1 * n + j] = 0.0
        mu, mv = _max_uv(f)
        assert not (mu > 500 or mv > 500 or math.isnan(mu) or math.isnan(mv)), step
        f.Simulate(0.1)


def case_visual_enhancements_low_iterations(make):
    """TestVisualEnhancementsLowIterations fluid_test.go:760-839."""
    f = make(1.0, 20, 15, 1.0)
    _all_fluid(f)
    f.ViscosityDiffusion = 0.1
    f.PressureDamping = 0.95
    f.Confinement = 0.05
    n = f.NumY
    jetX, jc = 2, f.NumY // 2
    js, je = jc - 2, jc + 2
    f.S[10 * n + jc] = 0.0
    for step in range(15):
        for j in range(js, je):
            if 0 < j < f.NumY - 1:
                f.U[jetX * n + j] = 10.0
                f.M[jetX * n + j] = 1.0
        f.Simulate(0.1)
        mu, mv = _max_uv(f)
        assert not (mu > 50 or mv > 50), (step, mu, mv)
        assert not (math.isnan(mu) or math.isnan(mv))
    M = f.M
    tot = sum(float(M[i * n + j]) for i in range(jetX + 2, f.NumX - 1) for j in range(1, f.NumY - 1))
    assert tot >= 1.0, tot


def case_performance_comparison(make):
    """TestPerformanceComparison fluid_test.go:841-899."""
    for visc, damp, conf in ((0.1, 0.95, 0.05), (0.0, 1.0, 0.0)):
        f = make(1.0, 15, 10, 1.0)
        _all_fluid(f)
        f.ViscosityDiffusion = visc
        f.PressureDamping = damp
        f.Confinement = conf
        n = f.NumY
        for _ in range(10):
            f.U[2 * n + f.NumY // 2] = 8.0
            f.Simulate(0.1)
        mv = float(np.max(np.abs(f.U).astype(np.float32) + np.abs(f.V).astype(np.float32)))
        assert not (math.isnan(mv) or mv > 100.0), mv


def case_advanced_visual_enhancements(make):
    """TestAdvancedVisualEnhancements fluid_test.go:901-1022."""
    f = make(1.0, 25, 15, 1.0)
    _all_fluid(f)
    f.ViscosityDiffusion = 0.15
    f.PressureDamping = 0.92
    f.Confinement = 0.08
    f.TurbulenceStrength = 0.03
    f.SmokeAdvection = 1.2
    n = f.NumY
    jetX, jc = 3, f.NumY // 2
    js, je = jc - 3, jc + 3
    for ox, oy in ((12, jc), (18, jc - 3), (18, jc + 3)):
        if ox < f.NumX and 0 <= oy < f.NumY:
            f.S[ox * n + oy] = 0.0
    for step in range(20):
        adt = f.GetAdaptiveTimeStep(0.08)
        for j in range(js, je):
            if 0 < j < f.NumY - 1:
                f.U[jetX * n + j] = 12.0
                f.M[jetX * n + j] = 1.0
        f.Simulate(adt)
        mu, mv = _max_uv(f)
        assert not (mu > 100 or mv > 100), (step, mu, mv)
        assert not (math.isnan(mu) or math.isnan(mv))
        assert not np.isnan(f.M).any()
    M = f.M
    tot = sum(float(M[i * n + j]) for i in range(jetX + 5, f.NumX - 1) for j in range(1, f.NumY - 1))
    assert tot >= 2.0, tot


def case_apply_force(make):
    """TestApplyForce fluid_test.go:1134-1160 (exact values)."""
    f = make(1.0, 10, 10, 1.0)
    _all_fluid(f)
    n = f.NumY
    f.ApplyForce(5, 5, 3.0, -2.0)
    assert f.U[5 * n + 5] == 3.0
    assert f.V[5 * n + 5] == -2.0
    f.S[6 * n + 6] = 0.0
    f.ApplyForce(6, 6, 10.0, 10.0)
    assert f.U[6 * n + 6] == 0 and f.V[6 * n + 6] == 0
    f.ApplyForce(0, 0, 1.0, 1.0)


def case_apply_force_radius(make):
    """TestApplyForceRadius fluid_test.go:1162-1190."""
    f = make(1.0, 20, 20, 1.0)
    _all_fluid(f)
    n = f.NumY
    cx, cy = 10, 10
    f.ApplyForceRadius(cx, cy, 5.0, 0.0, 3)
    U = f.U
    assert U[cx * n + cy] >= 4.5
    edge = U[(cx + 3) * n + cy]
    assert edge < U[cx * n + cy] and edge > 0
    assert U[(cx + 4) * n + cy] == 0


def case_force_does_not_break_incompressibility(make):
    """TestForceDoesNotBreakIncompressibility fluid_test.go:1192-1208."""
    f = make(1.0, 20, 15, 1.0)
    _all_fluid(f)
    f.ApplyForceRadius(10, 7, 20.0, 10.0, 4)
    f.Simulate(0.05)
    md = f.MaxDivergence()
    assert md <= 1.0, md


def case_bfecc_accuracy(make):
    """TestBFECCAccuracy fluid_test.go:1210-1268 (logs only; runs both paths)."""
    out = {}
    for use in (False, True):
        f = make(1.0, 30, 30, 1.0)
        _all_fluid(f)
        n = f.NumY
        inner = np.zeros((f.NumX, n), dtype=bool)
        inner[1:-1, 1:-1] = True
        inner = inner.ravel()
        f.U[inner] = 3.0
        for i in range(8, 13):
            for j in range(13, 18):
                f.M[i * n + j] = 1.0
        f.UseBFECC = use
        for _ in range(50):
            f.Simulate(0.05)
            f.U[inner] = 3.0
        out[use] = float(f.M.max())
    assert all(math.isfinite(v) for v in out.values())
    return out


def case_bfecc_stability_long_run(make):
    """TestBFECCStabilityLongRun fluid_test.go:1270-1314."""
    f = make(1.0, 30, 20, 1.0)
    _all_fluid(f)
    f.UseBFECC = True
    n = f.NumY
    f.SetCircularObstacle(15, f.NumY // 2, 3)
    for step in range(200):
        for j in range(f.NumY // 2 - 4, f.NumY // 2 + 4):
            if 0 < j < f.NumY - 1:
                f.U[1 * n + j] = 15.0
                f.M[1 * n + j] = 1.0
        f.Simulate(0.05)
        inner = np.concatenate([
            f.U.reshape(f.NumX, n)[1:-1, 1:-1].ravel(),
            f.V.reshape(f.NumX, n)[1:-1, 1:-1].ravel(),
            f.M.reshape(f.NumX, n)[1:-1, 1:-1].ravel(),
        ])
        assert np.isfinite(inner).all(), step
    assert (f.M >= -0.001).all()


def case_interaction_stability(make):
    """TestInteractionStability fluid_test.go:1316-1358."""
    f = make(1.0, 30, 20, 1.0)
    _all_fluid(f)
    for step in range(100):
        if step % 5 == 0:
            f.ApplyForceRadius(10 + step % 10, 10, 10.0, 5.0, 3)
        if step % 3 == 0:
            f.AddSmoke(5, 10, 1.0)
        if step % 20 == 0:
            f.SetSolid(15, 10, True)
        if step % 20 == 10:
            f.SetSolid(15, 10, False)
        f.Simulate(0.05)
        mu, mv = _max_uv(f)
        m = max(mu, mv)
        assert not (math.isnan(m) or m > 500), (step, m)


def case_smoke_non_negative(make):
    """TestSmokeNonNegative fluid_test.go:1360-1379."""
    f = make(1.0, 20, 15, 1.0)
    _all_fluid(f)
    f.ViscosityDiffusion = 0.1
    n = f.NumY
    for _ in range(50):
        f.U[3 * n + 7] = 10.0
        f.M[3 * n + 7] = 1.0
        f.Simulate(0.08)
    assert (f.M >= -0.01).all()


def case_vorticity_field(make):
    """TestVorticityField fluid_test.go:1381-1402."""
    f = make(1.0, 10, 10, 1.0)
    _all_fluid(f)
    n = f.NumY
    f.U[5 * n + 4] = 1
    f.U[5 * n + 6] = -1
    f.V[4 * n + 5] = -1
    f.V[6 * n + 5] = 1
    v, err = f.Vorticity().Value(5, 5)
    assert err is None
    assert abs(v) >= 0.1


def case_velocity_magnitude_field(make):
    """TestVelocityMagnitudeField fluid_test.go:1404-1425."""
    f = make(1.0, 10, 10, 1.0)
    _all_fluid(f)
    n = f.NumY
    f.U[5 * n + 5] = 3.0
    f.U[6 * n + 5] = 3.0
    f.V[5 * n + 5] = 4.0
    f.V[5 * n + 6] = 4.0
    v, err = f.VelocityMagnitude().Value(5, 5)
    assert err is None
    assert abs(v - 5.0) <= 0.1


def case_set_circular_obstacle(make):
    """TestSetCircularObstacle fluid_test.go:1427-1445."""
    f = make(1.0, 20, 20, 1.0)
    _all_fluid(f)
    f.SetCircularObstacle(10, 10, 3)
    assert f.IsSolid(10, 10)
    assert f.IsSolid(12, 10)
    assert not f.IsSolid(14, 10)


def case_apply_vorticity_confinement(make):
    """TestApplyVorticityConfinement confinement_test.go:6-27."""
    f = make(1, 4, 4, 1)
    for i in range(f.NumX):
        for j in range(f.NumY):
            f.SetSolid(i, j, False)
    f.SetVelocity(3, 2, 1, 0)
    f.SetVelocity(2, 3, -1, 0)
    f.SetVelocity(2, 2, 0, 1)
    f.SetVelocity(3, 3, 0, -1)
    f.Confinement = 5
    idx = 2 * f.NumY + 2
    u0, v0 = float(f.U[idx]), float(f.V[idx])
    f.applyVorticityConfinement(1)
    assert not (f.U[idx] == u0 and f.V[idx] == v0)


def case_set_solid_panics(make):
    """walls.go:6-11, 52-57, 63-68, 75-80: out-of-range indices panic."""
    import pytest

    f = make(1.0, 4, 4, 1.0)
    for call in (lambda: f.SetSolid(-1, 0, True), lambda: f.IsSolid(0, f.NumY),
                 lambda: f.SetVelocity(f.NumX, 0, 1, 1), lambda: f.AddSmoke(0, -1, 1)):
        with pytest.raises(IndexError):
            call()
    v, err = f.Smoke().Value(f.NumX, 0)
    assert err is not None and v == 0.0


# Cases driving Simulate with the reference's iteration count; the multigrid
# cases (TestMultigridPerformance, TestMultigridStability) cover the
# reference's optional two-level solver, which the CUDA path does not build.
ALL_CASES = [
    case_copy_border, case_diffusion_behavior, case_velocity_advection,
    case_smoke_advection, case_pressure_projection, case_boundary_conditions,
    case_realistic_jet, case_obstacle_vortex_shedding, case_bfecc_stability,
    case_bfecc_jet_stability, case_visual_enhancements_low_iterations,
    case_performance_comparison, case_advanced_visual_enhancements, case_apply_force,
    case_apply_force_radius, case_force_does_not_break_incompressibility,
    case_bfecc_accuracy, case_bfecc_stability_long_run, case_interaction_stability,
    case_smoke_non_negative, case_vorticity_field, case_velocity_magnitude_field,
    case_set_circular_obstacle, case_apply_vorticity_confinement, case_set_solid_panics,
]


def case_multigrid_stability(make):
    """TestMultigridStability fluid_test.go:1470-1547."""
    f = make(1.0, 30, 20, 1.0)
    _all_fluid(f)
    f.UseMultigrid = True
    f.MultigridLevels = 2
    f.ViscosityDiffusion = 0.1
    f.PressureDamping = 0.95
    f.Confinement = 0.05
    n = f.NumY
    jc = f.NumY // 2
    for ox, oy in ((15, jc), (22, jc - 2), (22, jc + 2)):
        f.S[ox * n + oy] = 0.0
    for step in range(25):
        for j in range(jc - 3, jc + 3):
            f.U[3 * n + j] = 18.0
            f.M[3 * n + j] = 1.0
        f.Simulate(0.08)
        mu, mv = _max_uv(f)
        assert not (mu > 100 or mv > 100), step
    assert calculate_divergence(f) <= 5.0
