"""Tracer particles and rendering on the device against the oracle's
restatement of the app loops (main/main.go:489-546 advectParticles,
main/main.go:619-650 and main/colors.go:10-84): on the reference scheme the
fields are bit-identical, so particle positions, ages, survivors and every
rendered byte must be identical too."""
import numpy as np
import pytest

import scenes
from oracle.pyoracle import OracleFluid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import fluid_gb300

    fluid_gb300.build()
    return fluid_gb300


def hue_rgb(h):
    """hueToRGB (main/main.go:871-894) for the spawn colours."""
    h = h % 360.0
    x = 1.0 - abs((h / 60.0) % 2 - 1)
    r, g, b = [(1, x, 0), (x, 1, 0), (0, 1, x), (0, x, 1), (x, 0, 1), (1, 0, x)][int(h // 60) % 6]
    return np.array([int(255 * r), int(255 * g), int(255 * b)], np.uint8)


def test_particles_and_render_bitwise(gpu):
    W, H = 64, 48
    g = gpu.Fluid(1.0, W, H, 1.0, UseBFECC=True, Confinement=0.2)
    o = OracleFluid(1.0, W, H, 1.0, prec=32, UseBFECC=True, Confinement=0.2)
    for f in (g, o):
        scenes.jet_scene(f)
        f.SetCircularObstacle(30, 24, 5)
    h = g.H()
    ox = np.zeros(0, np.float32)
    oy, oage, omax = ox.copy(), ox.copy(), ox.copy()
    orgb = np.zeros(0, np.uint32)
    hue = 0.0
    for frame in range(60):
        for f in (g, o):
            scenes.jet_inject(f, speed=2.0)
            f.Simulate(0.1)
        if frame % 3 == 0:
            # spawnParticles at the jet cells: cell centres, age 0, max age 15
            cells = [(1, j) for j in scenes.jet_rows(g)] + [(20, 10), (50, 40), (31, 24)]
            xs = np.array([(ci + 0.5) * h for ci, cj in cells], np.float32)
            ys = np.array([(cj + 0.5) * h for ci, cj in cells], np.float32)
            col = hue_rgb(hue)
            hue = (hue + 2.0) % 360.0
            g.particles_add(xs, ys, 1.5, col, max_total=60)
            room = max(0, 60 - ox.size)
            xs, ys = xs[:room], ys[:room]
            ox = np.concatenate([ox, xs])
            oy = np.concatenate([oy, ys])
            oage = np.concatenate([oage, np.zeros(xs.size, np.float32)])
            omax = np.concatenate([omax, np.full(xs.size, 1.5, np.float32)])
            packed = np.uint32(col[0]) | (np.uint32(col[1]) << 8) | (np.uint32(col[2]) << 16)
            orgb = np.concatenate([orgb, np.full(xs.size, packed, np.uint32)])
        g.particles_advect(0.1)
        n = o.particles_advect(0.1, ox, oy, oage, omax, orgb)
        ox, oy, oage, omax, orgb = ox[:n], oy[:n], oage[:n], omax[:n], orgb[:n]
        p = g.particles()
        assert p["X"].size == n, (frame, p["X"].size, n)
        for a, b in ((p["X"], ox), (p["Y"], oy), (p["Age"], oage), (p["MaxAge"], omax)):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), frame
        rgb = (orgb[:, None] >> np.array([0, 8, 16], np.uint32)) & 0xff
        assert np.array_equal(p["RGB"], rgb.astype(np.uint8))
    assert 0 < n <= 60
    for kind in range(4):
        a, b = g.render(kind), o.render(kind)
        bad = np.flatnonzero(a != b)
        assert bad.size == 0, (kind, bad.size, bad[:4])
