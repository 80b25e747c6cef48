"""Headless colour buffers and point view (the Demo programs' VBOs without GL):
the colours equal the reference's rules restated here in float32 (colorRamp,
fluidSystem.cpp:97-114, 165-181; poiseuilleFlowSystem.cpp:152-166; Coloring,
PeristalsisSystem.cpp:409-442), and the PPM view is a well-formed image."""
import numpy as np
import pytest

import cmag_gb300 as cm
from cmag_gb300 import presets

pytestmark = pytest.mark.gpu

F = np.float32
RAMP = np.array([[1.0, 0.0, 0.0], [1.0, 0.5, 0.0], [1.0, 1.0, 0.0], [0.0, 1.0, 0.0],
                 [0.0, 1.0, 1.0], [0.0, 0.0, 1.0], [1.0, 0.0, 1.0]], np.float32)


def color_ramp(t):
    t = F(F(t) * F(6.0))
    i = int(t)
    u = F(t - F(np.floor(t)))
    return np.array([F(RAMP[i, k] + F(u * F(RAMP[i + 1, k] - RAMP[i, k]))) for k in range(3)], np.float32)


def test_dambreak_colors(gpu):
    s = cm.DamBreakSystem((16, 32, 1), 1, (64, 64, 4), 1.0 / 256)
    s.reset()
    got = s.colors()
    n = s.getNumParticles()
    p = s.params
    fluid = 16 * 32
    type_one = fluid + (p.grid_size[0] - p.boundary_offset + 1) + 2 * (p.grid_size[1] - p.boundary_offset)
    want = np.empty((n, 4), np.float32)
    for i in range(n):
        t = 0.7
        if i < type_one:
            t = 0.2
        if i < fluid:
            t = 0.5
        want[i, :3] = color_ramp(t)
        want[i, 3] = 1.0
    assert np.array_equal(got, want)
    s.close()


def test_poiseuille_colors(gpu):
    kw = presets.poiseuille_dump()
    s = cm.PoiseuilleFlowSystem(kw["fluid_size"], kw["boundary_offset"], kw["grid_size"], kw["radius"])
    s.reset()
    got = s.colors()
    fluid = kw["fluid_size"][0] * kw["fluid_size"][1]
    gx = kw["grid_size"][0]
    for i in (0, 1, gx, gx + 3, fluid - 1, fluid, s.getNumParticles() - 1):
        t = 0.5 if i < fluid else 0.7
        if i % gx == 0 and i < fluid:
            t = 0.2
        assert np.array_equal(got[i, :3], color_ramp(t)), i
    s.close()


def test_peristalsis_colors_and_view(gpu, tmp_path):
    kw = presets.peristalsis_report()
    s = cm.PeristalsisSystem(kw["dt"], kw["fluid_size"], kw["amplitude"], kw["wave_speed"],
                             kw["soundspeed"], kw["gravity"], kw["boundary_offset"], kw["grid_size"],
                             kw["radius"])
    s.reset()
    s.update_n(20)
    pos = s.getArray(cm.POSITION)
    got = s.colors()
    p = s.params
    edge = F(F(p.world_origin[0]) + F(4.0) * F(p.particle_radius))
    want = np.where(pos[:, 3:4] != 0, [0, 0, 0, 1], np.where(pos[:, 0:1] < edge, [255, 0, 0, 1], [255, 255, 255, 1]))
    assert np.array_equal(got, want.astype(np.float32))
    path = tmp_path / "view.ppm"
    s.render_ppm(path, 512)
    data = path.read_bytes()
    magic, size, mx, body = data.split(b"\n", 3)
    w, h = (int(v) for v in size.split())
    assert magic == b"P6" and w == 512 and int(mx) == 255 and len(body) == 3 * w * h
    pix = np.frombuffer(body, np.uint8).reshape(h, w, 3)
    assert (pix == 255).all(axis=2).sum() > 1000  # white fluid
    assert ((pix[..., 0] == 255) & (pix[..., 1] == 0)).sum() > 0  # red marker column
    s.close()
