"""The C restatement against the reference's own code, run side by side
(only where the reference checkout exists, i.e. where oracle/_ref builds)."""
import numpy as np
import pytest

from fluid_simulation_gb300 import scenes
from oracle import pyoracle as po

pytestmark = pytest.mark.skipif(not po.reference_available(), reason="reference build unavailable")


def _pair(sc, cg_maxit=400):
    sims = []
    for kind in ("restatement", "reference"):
        s = po.OracleSim(kind, sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
        s.set_cg(sc.cg_tolerance, cg_maxit)
        s.set_particles(sc.particles)
        sims.append(s)
    return sims


def _same(a, b):
    sa, sb = a.state(), b.state()
    for k in sa:
        assert np.array_equal(sa[k].view(np.uint8), sb[k].view(np.uint8)), k


@pytest.mark.parametrize("method", [po.STEP_PICFLIP, po.STEP_PIC, po.STEP_FLIP, po.STEP_SEMI_LAGRANGIAN])
def test_step_methods(method):
    sc = scenes.dam_break_small()
    a, b = _pair(sc)
    for _ in range(15):
        assert a.step(method, sc.dt) == 0 and b.step(method, sc.dt) == 0
    _same(a, b)


def test_phase_sequence_equals_stock_step():
    """The harness's explicit phase sequence equals FluidSolver::stepPICFLIP."""
    sc = scenes.dam_break_small()
    a, b = _pair(sc)
    _, c = _pair(sc)
    c.set_use_stock(False)
    for _ in range(10):
        b.step(po.STEP_PICFLIP, sc.dt)
        c.step(po.STEP_PICFLIP, sc.dt)
    _same(b, c)


@pytest.mark.parametrize("ph", [po.PH_CLASSIFY, po.PH_P2G, po.PH_SAVE_PREV, po.PH_GRAVITY, po.PH_DIRICHLET,
                                po.PH_EXTEND, po.PH_PRESSURE, po.PH_SAVE_DIFF, po.PH_G2P_PICFLIP,
                                po.PH_G2P_PIC, po.PH_G2P_FLIP, po.PH_ADVECT_SAFE, po.PH_ADVECT,
                                po.PH_SL_VELOCITY, po.PH_SL_PARTICLES])
def test_single_phase_on_random_state(ph):
    """Each phase on a randomised mid-simulation state (random velocities,
    jittered particles incl. negative and out-of-cell positions)."""
    sc = scenes.dam_break_small()
    a, b = _pair(sc)
    for s in (a, b):
        for _ in range(3):
            s.step(po.STEP_PICFLIP, sc.dt)
    rng = np.random.default_rng(ph)
    grids = {w: rng.standard_normal((sc.size_y, sc.size_x)).astype(np.float32) for w in range(8)}
    parts = a.particles()
    parts[:, 2:] = rng.standard_normal((parts.shape[0], 2)).astype(np.float32)
    if ph == po.PH_PRESSURE:
        # pressureSolve counts particles without clamping (FluidSolver.cpp:353-360):
        # a particle outside the grid is undefined behaviour there.
        parts[:3, 0] = np.array([-0.3, 0.0, 63.99], np.float32)
    else:
        parts[:5, 0] = np.array([-0.3, -2.5, 0.0, 63.99, 70.0], np.float32)
    for s in (a, b):
        for w, g in grids.items():
            s.set_grid(w, g)
        s.set_particles(parts)
        s.set_pic_ratio(0.3)
        assert s.phase(ph, sc.dt) == 0
    _same(a, b)


def test_fluid_source_and_obstacle():
    sc = scenes.dam_break_small()
    disc = scenes.disc_mask(64, 64, 45.0, 20.0, 8.0)
    sims = []
    for kind in ("restatement", "reference"):
        s = po.OracleSim(kind, 64, 64, 64.0, 64.0, sc.density, sc.pic_ratio)
        s.set_cg(1e-6, 500)
        s.set_solid_mask(disc)
        s.set_gravity(0.0, -9.81)
        s.add_source(2.0, 10.0, 40.0, 50.0, 1.0, 1.0, 3.0, 0.0, 0.05, 3)
        sims.append(s)
    for _ in range(40):
        for s in sims:
            s.update(sc.dt)
            assert s.step(po.STEP_PICFLIP, sc.dt) == 0
    _same(*sims)


def test_non_square_cells_rejected_like_reference():
    """dx != dy: the solver's pool copy keeps dx for dy, so validate() fails
    and every step throws in the reference (FluidSolver.cpp:56-62, 215-221)."""
    for kind in ("restatement", "reference"):
        s = po.OracleSim(kind, 32, 16, 32.0, 32.0, 0.005, 0.05)
        assert s.step(po.STEP_PICFLIP, 0.005) == -1


def test_clear_sources_matches_reference():
    """FluidDomain::clearFluidSources between spawns: restatement == reference."""
    sims = []
    for kind in ("restatement", "reference"):
        sc = scenes.dam_break_small()
        s = po.OracleSim(kind, sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
        s.set_cg(sc.cg_tolerance, 400)
        s.add_source(3.3, 11.1, 44.0, 52.5, 0.7, 1.3, 2.5, -1.0, 0.02, -1)
        sims.append(s)
    for k in range(12):
        for s in sims:
            if k == 6:
                s.clear_sources()
                s.add_source(40.0, 47.0, 20.0, 30.0, 1.1, 0.9, 0.0, 0.0, 0.05, 3)
            s.update(0.005)
            assert s.step(po.STEP_PICFLIP, 0.005) == 0
        a, b = sims[0].state(), sims[1].state()
        for key in a:
            assert np.array_equal(a[key].view(np.uint8), b[key].view(np.uint8)), (k, key)


def _render_pair(steps=12):
    sims = []
    for kind in ("restatement", "reference"):
        sc = scenes.dam_break_small()
        s = po.OracleSim(kind, sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
        s.set_cg(sc.cg_tolerance, 400)
        s.set_solid_mask(scenes.disc_mask(64, 64, 45.0, 20.0, 8.0))
        parts = sc.particles.copy()
        parts[:7, 0] = [-3.0, 70.0, 10.0, 63.9, 0.0, 20.0, 30.0]  # off the canvas and on its edges
        s.set_particles(parts)
        for _ in range(steps):
            s.step(po.STEP_PICFLIP, sc.dt)
        sims.append(s)
    return sims


@pytest.mark.parametrize("what", [po.RENDER_CLEAR, po.RENDER_CELLS, po.RENDER_VELOCITIES, po.RENDER_PARTICLES,
                                  po.RENDER_METABALLS])
# (the reference offsets the canvas by half of x_min * width pixels, so only
# small offsets of the area keep the drawing on the canvas)
@pytest.mark.parametrize("size,area", [((96, 80), (0.0, 64.0, 0.0, 64.0)), ((160, 200), (-0.05, 66.0, 0.02, 60.0)),
                                       ((30, 25), (0.0, 64.0, 0.0, 64.0))])
def test_renderer_restatement_matches_reference(what, size, area):
    """Renderer.cpp / Canvas.cpp: the restatement paints the same canvas bit
    for bit, from a random starting canvas (the renderers draw over it)."""
    w, h = size
    rng = np.random.default_rng(what * 7 + w)
    start = rng.random((h, w, 3), dtype=np.float32)
    cols = rng.random(6, dtype=np.float32)
    out = []
    for s in _render_pair():
        c, k = start.copy(), cols.copy()
        s.render(what, area, c, k)
        out.append((c, k))
    (a, ka), (b, kb) = out
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(ka.view(np.uint32), kb.view(np.uint32))
    if what != po.RENDER_CLEAR:
        assert not np.array_equal(a, start)  # something was drawn


def test_canvas_bytes_and_metaball_weights_match_reference():
    rng = np.random.default_rng(3)
    c = (rng.random((40, 50, 3), dtype=np.float32) * 1.4 - 0.2).astype(np.float32)
    assert np.array_equal(po.canvas_bytes(c, "restatement"), po.canvas_bytes(c, "reference"))
    for j in range(-5, 5):
        for i in range(-5, 5):
            a, b = po.metaball_weight(i, j, "restatement"), po.metaball_weight(i, j, "reference")
            assert np.float32(a).view(np.uint32) == np.float32(b).view(np.uint32)


def _level_set_pair(nx, ny, steps=6):
    sims = []
    for kind in ("restatement", "reference"):
        s = po.OracleSim(kind, nx, ny, float(nx), float(ny), 0.005, 0.02)
        s.set_cg(1e-6, 400)
        s.set_particles(scenes.block_particles(nx, ny, float(nx), float(ny), 1, nx // 2, 1, ny // 2, 4, 9))
        for _ in range(steps):
            s.step(po.STEP_PICFLIP, 0.005)
        jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
        s.set_level_set((np.hypot(ii + 0.5 - nx / 3, jj + 0.5 - ny / 3) - nx / 5).astype(np.float32))
        sims.append(s)
    return sims


def test_level_set_square_grid_matches_reference():
    """FluidDomain::advectLevelSet on a square grid: every row but the last,
    whose velocities the reference reads past the end of its arrays; then
    classifyCells(LevelSet&) and the level-set render pass."""
    a, b = _level_set_pair(64, 64)
    for s in (a, b):
        s.advect_level_set(0.05)
    la, lb = a.level_set(), b.level_set()
    assert np.array_equal(la[:-1].view(np.uint32), lb[:-1].view(np.uint32))
    assert not np.array_equal(la[:-1], _level_set_pair(64, 64, steps=0)[0].level_set()[:-1])
    for s in (a, b):
        s.set_level_set(la)  # the same (defined) field on both, then classify and draw it
        s.classify_level_set()
    assert np.array_equal(a.labels(), b.labels())
    start = np.random.default_rng(1).random((70, 90, 3), dtype=np.float32)
    out = []
    for s in (a, b):
        c, k = start.copy(), np.zeros(6, np.float32)
        s.render(po.RENDER_LEVEL_SET, (0.0, 64.0, 0.0, 64.0), c, k)
        out.append((c, k))
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.array_equal(out[0][1].view(np.uint32), out[1][1].view(np.uint32))


def test_level_set_narrow_grid_matches_reference_everywhere():
    """size_x < size_y: the swapped loop bounds (FluidDomain.cpp:111-113) alias
    writes but stay inside the arrays, so every cell is defined and equal."""
    a, b = _level_set_pair(40, 64)
    for k in range(3):
        for s in (a, b):
            s.advect_level_set(0.05)
        assert np.array_equal(a.level_set().view(np.uint32), b.level_set().view(np.uint32)), k
