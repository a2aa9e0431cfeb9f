"""Headless renderer: the GPU canvas after each Renderer pass equals, bit for
bit, the CPU restatement of Renderer.cpp / Canvas.cpp (itself pinned to the
reference's own sources in test_oracle_vs_reference.py), including the line
and fill colours the canvas keeps, the PPM bytes, and pixels that many
metaballs overlap."""
import numpy as np
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import build as fsbuild
from fluid_simulation_gb300 import scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

def bits(a: np.ndarray) -> np.ndarray:
    """Float bits with every NaN made the same NaN: a canvas narrower than 40
    pixels makes the reference divide 0 by 0 for zero-length velocity lines
    (Renderer.cpp:121), and CPUs and GPUs write different NaN payloads."""
    a = np.array(a, np.float32)
    a[np.isnan(a)] = np.float32("nan")
    return a.view(np.uint32)


PASSES = [fsg.RENDER_CLEAR, fsg.RENDER_CELLS, fsg.RENDER_VELOCITIES, fsg.RENDER_PARTICLES, fsg.RENDER_METABALLS]


@pytest.fixture(scope="module")
def states():
    fsbuild.build()
    sc = scenes.dam_break_small()
    g = fsg.FluidSim(sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio,
                     cg_tolerance=sc.cg_tolerance, cg_max_iterations=400)
    o = po.OracleSim("restatement", sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    o.set_cg(sc.cg_tolerance, 400)
    solid = scenes.disc_mask(64, 64, 45.0, 20.0, 8.0)
    g.set_solid_mask(solid)
    o.set_solid_mask(solid)
    parts = sc.particles.copy()
    parts[:7, 0] = [-3.0, 70.0, 10.0, 63.9, 0.0, 20.0, 30.0]
    g.set_particles(parts)
    o.set_particles(parts)
    for _ in range(12):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
    return g, o


@pytest.mark.parametrize("what", PASSES)
@pytest.mark.parametrize("size,area", [((96, 80), (0.0, 64.0, 0.0, 64.0)), ((160, 200), (-0.05, 66.0, 0.02, 60.0)),
                                       ((30, 25), (0.0, 64.0, 0.0, 64.0)), ((20, 20), (0.0, 64.0, 0.0, 64.0))])
def test_render_pass_matches_restatement(states, what, size, area):
    g, o = states
    w, h = size
    rng = np.random.default_rng(what * 7 + w)
    start = rng.random((h, w, 3), dtype=np.float32)
    cols = rng.random(6, dtype=np.float32)
    c = fsg.Canvas(w, h)
    c.set_pixels(start)
    c.set_colors(cols[:3], cols[3:])
    g.render(c, what, area)
    ref, kref = start.copy(), cols.copy()
    o.render(what, area, ref, kref)
    got = c.pixels()
    bad = np.argwhere(np.any(bits(got) != bits(ref), axis=2))
    assert len(bad) == 0, (len(bad), bad[:3].tolist(), got[tuple(bad[0])], ref[tuple(bad[0])])
    assert np.array_equal(bits(c.colors()), bits(kref))


def test_canvas_bytes_and_ppm(states, tmp_path):
    g, o = states
    c = fsg.Canvas(128, 128)
    area = (0.0, 64.0, 0.0, 64.0)
    for what in (fsg.RENDER_CLEAR, fsg.RENDER_CELLS, fsg.RENDER_PARTICLES):
        g.render(c, what, area)
    rgb = c.pixels()
    assert np.array_equal(c.bytes(), po.canvas_bytes(rgb))
    path = str(tmp_path / "frame.ppm")
    c.write_ppm(path)
    data = open(path, "rb").read()
    head = b"P6\n128 128\n255\n"
    assert data.startswith(head) and data[len(head):] == po.canvas_bytes(rgb).tobytes()
