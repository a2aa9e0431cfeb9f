"""GPU parity: the CUDA path (through the C ABI) against the CPU restatement of
the reference (oracle/fs_oracle.c, itself pinned bit-exact against the
reference's own code) and against the fixtures recorded from the reference.

Everything here is compared bit for bit: labels, fluid indices and particle
counts (integers), and every float array (velocity grids front/back/previous/
difference, pressure, particle positions and velocities).  The GPU follows
the reference's float evaluation order, and its CG sums its dot products along
the same fixed tree as the oracle's CG (in float, the reference's precision,
or in double as an option), so no tolerance is needed."""
import os

import numpy as np
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import build as fsbuild
from fluid_simulation_gb300 import scenes
from oracle import pyoracle as po
from tests.golden import make_golden as mg

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    fsbuild.build()
    fsg.load_library()


def pair(sc, cg_tol=None, cg_maxit=None, precision=fsg.CG_FLOAT):
    tol = sc.cg_tolerance if cg_tol is None else cg_tol
    maxit = sc.cg_max_iterations if cg_maxit is None else cg_maxit
    g = fsg.FluidSim(sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio,
                     cg_tolerance=tol, cg_max_iterations=maxit, gravity=sc.gravity)
    o = po.OracleSim("restatement", sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    o.set_cg(tol, maxit)
    g.set_cg_precision(precision)
    o.set_cg_precision(precision)
    o.set_gravity(*sc.gravity)
    if sc.solid is not None:
        g.set_solid_mask(sc.solid)
        o.set_solid_mask(sc.solid)
    g.set_particles(sc.particles)
    o.set_particles(sc.particles)
    return g, o


def assert_same(g_state, o_state, keys=None, where=""):
    for k in keys or o_state.keys():
        a, b = g_state[k], o_state[k]
        assert a.shape == b.shape, (where, k, a.shape, b.shape)
        if not np.array_equal(a.view(np.uint8), b.view(np.uint8)):
            bad = np.argwhere(a != b) if a.dtype != np.uint8 or True else None
            first = tuple(bad[0]) if bad is not None and len(bad) else None
            raise AssertionError("%s %s differs at %d entries, first %s: gpu %r oracle %r" % (
                where, k, 0 if bad is None else len(bad), first,
                None if first is None else a[first], None if first is None else b[first]))


@pytest.mark.parametrize("method", [fsg.STEP_PICFLIP, fsg.STEP_PIC, fsg.STEP_FLIP, fsg.STEP_SEMI_LAGRANGIAN])
def test_step_methods_bit_exact(method):
    sc = scenes.dam_break_small()
    g, o = pair(sc, cg_maxit=400)
    for k in range(12):
        g.step(method, sc.dt)
        assert o.step(method, sc.dt) == 0
        assert_same(g.state(), o.state(), where="method %d step %d" % (method, k))


@pytest.mark.parametrize("graphs", [True, False], ids=["graph", "launches"])
@pytest.mark.parametrize("method", [fsg.STEP_PICFLIP, fsg.STEP_SEMI_LAGRANGIAN])
def test_steps_on_a_caller_stream_bit_exact(method, graphs):
    """A handle whose work is queued on a stream the caller owns
    (fs_set_stream), replayed through its graph or launched kernel by kernel:
    each step forks its v splat onto the handle's second stream and joins it
    back, and every result equals the oracle's."""
    import torch

    sc = scenes.dam_break_small()
    g, o = pair(sc, cg_maxit=400)
    s = torch.cuda.Stream()
    g.set_stream(s.cuda_stream)
    g.set_graphs(graphs)
    for k in range(6):
        g.step(method, sc.dt)
        assert o.step(method, sc.dt) == 0
        assert_same(g.state(), o.state(), where="method %d step %d" % (method, k))
    g.close()  # before the caller's stream goes away


@pytest.mark.parametrize("precision", [fsg.CG_FLOAT, fsg.CG_DOUBLE])
def test_picflip_200_steps_bit_exact_with_graphs(precision):
    """The 64x64 dam break of the small configuration, 200 steps, replayed
    through the cached CUDA graph of the step; both CG precisions."""
    sc = scenes.dam_break_small()
    g, o = pair(sc, precision=precision)
    for k in range(200):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
        if k % 20 == 19 or k < 3:
            assert_same(g.state(), o.state(), where="step %d" % k)
            st = g.stats()
            it, err, nf = o.cg_stats()
            assert st["cg_iterations"] == it and st["n_fluid"] == nf
            assert st["cg_residual"] == pytest.approx(err, rel=1e-12, abs=0)


@pytest.mark.parametrize("case", sorted(mg.CASES))
def test_against_reference_fixtures(case, golden_dir):
    """The GPU against the states recorded from the reference's own code
    (the fluid-source case spawns its particles on the device)."""
    ref = np.load(os.path.join(golden_dir, case + ".npz"))
    method, steps, scene, opt = mg.CASES[case]
    sc = scenes.dam_break_small()
    g = fsg.FluidSim(sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio,
                     cg_tolerance=sc.cg_tolerance, cg_max_iterations=sc.cg_max_iterations)
    if "disc" in opt:
        g.set_solid_mask(scenes.disc_mask(sc.size_x, sc.size_y, *opt["disc"]))
    if scene == "source":
        g.add_fluid_source(2.0, 10.0, 40.0, 50.0, 1.0, 1.0, 3.0, 0.0, 0.05, 5)
    else:
        g.set_particles(sc.particles)
    for k in range(1, max(steps) + 1):
        if scene == "source":
            g.update(sc.dt)
        g.step(method, sc.dt)
        if k in steps:
            st = g.state()
            for key in mg.FULL_KEYS:
                a, b = st[key], ref["s%d_%s" % (k, key)]
                assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (case, k, key)


PHASES = [fsg.PH_CLASSIFY, fsg.PH_P2G, fsg.PH_SAVE_PREV, fsg.PH_GRAVITY, fsg.PH_DIRICHLET, fsg.PH_EXTEND,
          fsg.PH_PRESSURE, fsg.PH_SAVE_DIFF, fsg.PH_G2P_PICFLIP, fsg.PH_G2P_PIC, fsg.PH_G2P_FLIP,
          fsg.PH_ADVECT_SAFE, fsg.PH_ADVECT, fsg.PH_SL_VELOCITY, fsg.PH_SL_PARTICLES, fsg.PH_SWAP]


@pytest.mark.parametrize("ph", PHASES)
@pytest.mark.parametrize("n", [64, 97])
def test_single_phase_on_random_state(ph, n):
    """Each phase from an identical randomised state: random velocities on all
    eight grids, particles jittered (incl. negative and out-of-grid positions
    where the reference clamps), a solid obstacle, pic ratio 0.3."""
    rng = np.random.default_rng(1000 * ph + n)
    sc = scenes.dam_break_small() if n == 64 else scenes.Scene(
        n, n, float(n), float(n), 0.005, 0.05, 0.005,
        scenes.block_particles(n, n, float(n), float(n), 1, n // 2, 1, 2 * n // 3, 5, 7),
        solid=scenes.disc_mask(n, n, 0.7 * n, 0.3 * n, 0.1 * n), cg_tolerance=1e-6, cg_max_iterations=500)
    g, o = pair(sc)
    for s in (g, o):
        s.step(fsg.STEP_PICFLIP, sc.dt)
    parts = o.particles()
    parts[:, 2:] = rng.standard_normal((parts.shape[0], 2)).astype(np.float32)
    if ph != fsg.PH_PRESSURE:
        parts[:6, 0] = np.array([-0.3, -2.5, 0.0, n - 0.01, n + 6.0, -1e-8], np.float32)
        parts[6:9, 1] = np.array([-0.7, n + 0.2, 0.5], np.float32)
    grids = [rng.standard_normal((n, n)).astype(np.float32) for _ in range(8)]
    for s in (g, o):
        for w, arr in enumerate(grids):
            s.set_grid(w, arr)
        s.set_particles(parts)
        s.set_pic_ratio(0.3)
    g.phase(ph, sc.dt)
    assert o.phase(ph, sc.dt) == 0
    assert_same(g.state(), o.state(), where="phase %d" % ph)


def test_obstacle_and_gravity_override():
    n = 80
    solid = scenes.disc_mask(n, n, 55.0, 20.0, 9.0)
    sc = scenes.Scene(n, n, float(n), float(n), 0.005, 0.05, 0.005,
                      scenes.block_particles(n, n, float(n), float(n), 1, 30, 1, 50, 4, 3, solid),
                      solid=solid, gravity=(0.0, -9.81), cg_tolerance=1e-5, cg_max_iterations=3000)
    g, o = pair(sc)
    for k in range(60):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
    assert_same(g.state(), o.state(), where="obstacle")


@pytest.mark.parametrize("precision", [fsg.CG_FLOAT, fsg.CG_DOUBLE, fsg.CG_DS])
def test_large_grid_one_step_bit_exact(precision):
    """512x512 dam break with an obstacle (~430k particles), one full step:
    multi-CTA CG with grid barriers, register-resident CG state (at most 4
    chunks per CTA)."""
    sc = scenes.dam_break_large(512)
    g, o = pair(sc, precision=precision)
    g.step(fsg.STEP_PICFLIP, sc.dt)
    o.step(po.STEP_PICFLIP, sc.dt)
    assert_same(g.state(), o.state(), where="512")
    st = g.stats()
    it, err, nf = o.cg_stats()
    assert (st["cg_iterations"], st["n_fluid"]) == (it, nf)
    assert st["cg_residual"] < sc.cg_tolerance


def test_benchmark_workload_three_steps_bit_exact():
    """The benchmark's own workload (1024x1024 dam break, disc obstacle,
    1,716,100 particles, CG to 1e-5, stepPICFLIP): three steps, every array
    bit-identical to the oracle after each, with the same CG iteration counts."""
    sc = scenes.dam_break_large(1024)
    g, o = pair(sc)
    for k in range(3):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        assert o.step(po.STEP_PICFLIP, sc.dt) == 0
        st = g.stats()
        it, err, nf = o.cg_stats()
        assert (st["cg_iterations"], st["n_fluid"]) == (it, nf), k
        assert st["cg_iterations"] > 1000 and st["cg_residual"] < sc.cg_tolerance
        assert_same(g.state(), o.state(), where="1024 step %d" % k)


@pytest.mark.parametrize("precision", [fsg.CG_FLOAT, fsg.CG_DOUBLE])
def test_streaming_cg_matches_oracle(precision):
    """A fluid region too large for k_cg's register-resident CG (11 chunks of
    1024 fluid cells per CTA): with float dot products k_cg_large's 12-chunk
    form, with double dot products k_cg's streaming form."""
    n = 1280
    sc = scenes.Scene(n, n, float(n), float(n), 0.01, 0.05, 0.01,
                      scenes.block_particles(n, n, float(n), float(n), 1, n - 1, 1, n - 1, 1, 11),
                      cg_tolerance=1e-3, cg_max_iterations=60)
    g, o = pair(sc, precision=precision)
    g.step(fsg.STEP_PICFLIP, sc.dt)
    o.step(po.STEP_PICFLIP, sc.dt)
    st = g.stats()
    it, err, nf = o.cg_stats()
    assert nf > 8 * 1024 * 152
    assert (st["cg_iterations"], st["n_fluid"]) == (it, nf)
    assert_same(g.state(), o.state(), keys=["pressure", "u_front", "v_front", "labels", "particles"], where="1280")


@pytest.mark.parametrize("precision", [fsg.CG_FLOAT, fsg.CG_DOUBLE])
def test_eight_chunk_register_form_matches_oracle(precision):
    """5 to 8 chunks of 1024 fluid cells per CTA: the register-resident CG
    with r and p in shared memory and the larger halo."""
    n = 1024
    sc = scenes.Scene(n, n, float(n), float(n), 0.01, 0.05, 0.01,
                      scenes.block_particles(n, n, float(n), float(n), 1, 1000, 1, 800, 1, 12),
                      cg_tolerance=1e-3, cg_max_iterations=60)
    g, o = pair(sc, precision=precision)
    g.step(fsg.STEP_PICFLIP, sc.dt)
    o.step(po.STEP_PICFLIP, sc.dt)
    st = g.stats()
    it, err, nf = o.cg_stats()
    assert 4 * 1024 * 152 < nf <= 8 * 1024 * 152
    assert (st["cg_iterations"], st["n_fluid"]) == (it, nf)
    assert_same(g.state(), o.state(), keys=["pressure", "u_front", "v_front", "labels", "particles"], where="1024")


@pytest.mark.parametrize("precision", [fsg.CG_FLOAT, fsg.CG_DOUBLE])
def test_resident_and_streaming_ctas_in_one_solve(precision):
    """8192 cells wide: the CTAs owning the full-width rows have halos of two
    8190-cell rows, more than the 8-chunk form holds, and stream their state,
    while the CTAs owning the narrow column above stay register-resident; all
    share the solve's barriers and reduction tree."""
    nx, ny = 8192, 400
    wide = scenes.block_particles(nx, ny, float(nx), float(ny), 1, nx - 1, 1, 60, 1, 13)
    narrow = scenes.block_particles(nx, ny, float(nx), float(ny), 1, 1500, 60, ny - 1, 1, 14)
    sc = scenes.Scene(nx, ny, float(nx), float(ny), 0.01, 0.05, 0.01, np.concatenate([wide, narrow]),
                      cg_tolerance=1e-3, cg_max_iterations=60)
    g, o = pair(sc, precision=precision)
    g.step(fsg.STEP_PICFLIP, sc.dt)
    o.step(po.STEP_PICFLIP, sc.dt)
    st = g.stats()
    it, err, nf = o.cg_stats()
    assert 4 * 1024 * 152 < nf <= 8 * 1024 * 152
    assert (st["cg_iterations"], st["n_fluid"]) == (it, nf)
    assert_same(g.state(), o.state(), keys=["pressure", "u_front", "v_front", "labels", "particles"], where="mixed")
    # the case mixes the two forms: per-CTA halo extents (152 CTAs, chunks of 1024) around the
    # 8-chunk form's capacity of 10,237 halo cells (204,800 B of shared memory, 16 B per owned cell)
    liquid = g.labels() == 0
    fidx = np.full(liquid.shape, -1, np.int64)
    fidx[liquid] = np.arange(int(liquid.sum()))  # j-major, as the fluid indexing
    down = np.full(liquid.shape, -1, np.int64)
    up = np.full(liquid.shape, -1, np.int64)
    down[1:] = np.where(liquid[:-1], fidx[:-1], -1)
    up[:-1] = np.where(liquid[1:], fidx[1:], -1)
    dn_of, up_of = down[liquid], up[liquid]
    nchunks = (nf + 1023) // 1024
    halos = []
    for cta in range(152):
        c0, c1 = cta * nchunks // 152, (cta + 1) * nchunks // 152
        e0, e1 = c0 * 1024, min(c1 * 1024, nf)
        lo = min(e0, dn_of[e0:e1][dn_of[e0:e1] >= 0].min(initial=e0), e0 - 1)
        hi = max(e1, up_of[e0:e1].max(initial=e1) + 1, e1 + 1)
        halos.append((e0 - lo) + (hi - e1))
    assert max(halos) > 10237 and min(halos) <= 10237, (min(halos), max(halos))


def test_non_square_cells_rejected_like_reference():
    g = fsg.FluidSim(32, 16, 32.0, 32.0, 0.005, 0.05)
    with pytest.raises(fsg.FsError) as ei:
        g.step(fsg.STEP_PICFLIP, 0.005)
    assert ei.value.code == 2


def test_empty_domain_and_no_fluid():
    """No particles: no fluid cell, the pressure solve returns before solving
    and swapping (src/FluidSolver.cpp:347-350)."""
    sc = scenes.dam_break_small()
    sc.particles = sc.particles[:0]
    g, o = pair(sc)
    rng = np.random.default_rng(5)
    grids = [rng.standard_normal((64, 64)).astype(np.float32) for _ in range(8)]
    for s in (g, o):
        for w, arr in enumerate(grids):
            s.set_grid(w, arr)
    for _ in range(3):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
    assert_same(g.state(), o.state(), where="empty")
    assert g.stats()["n_fluid"] == 0


def test_p2g_on_4096_grid_reaches_the_last_cells():
    """4096 x 4096 cells make 4096^2 + 1 splat bins, more tiles than one block
    of the tile-sum scan covers in one round; particles next to the last
    cell must still land in the right bins."""
    n = 4096
    rng = np.random.default_rng(3)
    k = 4000
    corner = np.stack([n - 2 + rng.random(k) * 1.9, n - 2 + rng.random(k) * 1.9,
                       rng.standard_normal(k), rng.standard_normal(k)], axis=1).astype(np.float32)
    spread = np.stack([1 + rng.random(k) * (n - 2), 1 + rng.random(k) * (n - 2),
                       rng.standard_normal(k), rng.standard_normal(k)], axis=1).astype(np.float32)
    parts = np.concatenate([corner, spread])
    g = fsg.FluidSim(n, n, float(n), float(n), 1.0, 0.02)
    o = po.OracleSim("restatement", n, n, float(n), float(n), 1.0, 0.02)
    g.set_particles(parts)
    o.set_particles(parts)
    for ph in (fsg.PH_CLASSIFY, fsg.PH_P2G):
        g.phase(ph, 0.005)
        o.phase(ph, 0.005)
    for w in (fsg.U_FRONT, fsg.V_FRONT):
        a, b = g.grid(w), o.grid(w)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), w
        assert np.count_nonzero(a[n - 3:, n - 3:]) > 0


def test_fluid_sources_on_device_match_oracle():
    """Two sources (one unlimited, one limited, odd spacings whose float
    accumulation matters) on top of existing particles, with a clear and a
    particle reset midway."""
    sc = scenes.dam_break_small()
    g, o = pair(sc, cg_maxit=400)
    args = [(3.3, 11.1, 44.0, 52.5, 0.7, 1.3, 2.5, -1.0, 0.02, -1), (40.0, 47.0, 20.0, 30.0, 1.1, 0.9, 0.0, 0.0, 0.05, 3)]
    for a in args:
        g.add_fluid_source(*a)
        o.add_source(*a)
    for k in range(40):
        if k == 25:
            g.clear_fluid_sources()
            o.clear_sources()
            g.add_fluid_source(*args[0])
            o.add_source(*args[0])
        if k == 30:
            g.reset_particles()
            o.set_particles(np.zeros((0, 4), np.float32))
        g.update(sc.dt)
        o.update(sc.dt)
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
        assert g.num_particles() == len(o.particles()), k
        assert_same(g.state(), o.state(), where="source step %d" % k)


def test_fluid_source_lattice_that_cannot_advance_is_rejected():
    g = fsg.FluidSim(16, 16, 16.0, 16.0, 1.0, 0.0)
    with pytest.raises(fsg.FsError) as e:
        g.add_fluid_source(1.0e8, 1.0e8 + 64.0, 1.0, 2.0, 1.0, 1.0, 0.0, 0.0, 0.0, 1)
    assert e.value.code == 1


def test_snapshot_and_restore_replay_bit_exact():
    sc = scenes.dam_break_small()
    g, o = pair(sc, cg_maxit=400)
    g.add_fluid_source(2.0, 10.0, 40.0, 50.0, 1.0, 1.0, 3.0, 0.0, 0.02, 4)
    for _ in range(5):
        g.update(sc.dt)
        g.step(fsg.STEP_PICFLIP, sc.dt)
    snap = g.snapshot()
    for _ in range(7):
        g.update(sc.dt)
        g.step(fsg.STEP_PICFLIP, sc.dt)
    first = g.state()
    g.restore(snap)
    for _ in range(7):
        g.update(sc.dt)
        g.step(fsg.STEP_PICFLIP, sc.dt)
    assert_same(g.state(), first, where="replay from snapshot")
    other = fsg.FluidSim(sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    with pytest.raises(fsg.FsError):
        other.restore(snap)
    g.clear_fluid_sources()
    with pytest.raises(fsg.FsError):
        g.restore(snap)


def test_cg_barrier_timeout_is_reported_and_the_handle_recovers():
    """Failure detection without a GPU fault: the CG's grid barrier is made to
    wait for CTAs that do not exist (a bounded 50 ms wait); every CTA gives
    up, the host reads FS_ERR_TIMEOUT, and the handle keeps working: restored
    from a snapshot it continues bit-exact with the oracle."""
    sc = scenes.dam_break_large(256)
    g, o = pair(sc, cg_maxit=5000)
    for _ in range(2):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
    assert g.stats()["n_fluid"] > 16 * 1024  # the solve runs grid-wide
    snap = g.snapshot()
    assert g.lib.fs_debug_set_cg_barrier_fault(g.h, 1, 0.05) == 0
    g.step(fsg.STEP_PICFLIP, sc.dt)
    with pytest.raises(fsg.FsError) as e:
        g.synchronize()
    assert e.value.code == 4
    assert g.lib.fs_debug_set_cg_barrier_fault(g.h, 0, 2.0) == 0
    g.restore(snap)
    for k in range(2):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
        assert_same(g.state(), o.state(), where="after recovery, step %d" % k)


@pytest.mark.parametrize("n,chunks", [(1280, (9, 12)), (2048, (20, 32))], ids=["resident12", "pipelined"])
def test_large_system_cg_barrier_timeout_recovers(n, chunks):
    """The same failure path in the large-system kernel: a box of fluid of
    1280^2 (about 1.6M fluid cells, 11 chunks of 1024 per CTA on 152 SMs:
    k_cg_large's 12-chunk form) or 2048^2 (about 4.1M, 27 chunks per CTA: its
    cp.async pipeline).  With the barrier waiting for a CTA that does not
    exist every CTA gives up after 50 ms (and waits for its own copies in
    flight), the host reads FS_ERR_TIMEOUT, and the handle, restored from a
    snapshot, steps bit-exact with a handle that never failed."""
    import torch

    parts = scenes.block_particles(n, n, float(n), float(n), 1, n - 1, 1, n - 20, 4, 11)
    sims = []
    for _ in range(2):
        s = fsg.FluidSim(n, n, float(n), float(n), 0.005, 0.05, cg_tolerance=1e-5, cg_max_iterations=60)
        s.set_particles(parts)
        s.step(fsg.STEP_PICFLIP, 0.005)
        sims.append(s)
    g, ref = sims
    nf = g.stats()["n_fluid"]
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    per_cta = (-(-nf // 1024) + sms - 1) // sms
    assert chunks[0] <= per_cta <= chunks[1]
    snap = g.snapshot()
    assert g.lib.fs_debug_set_cg_barrier_fault(g.h, 1, 0.05) == 0
    g.step(fsg.STEP_PICFLIP, 0.005)
    with pytest.raises(fsg.FsError) as e:
        g.synchronize()
    assert e.value.code == 4
    assert g.lib.fs_debug_set_cg_barrier_fault(g.h, 0, 2.0) == 0
    g.restore(snap)
    for k in range(2):
        g.step(fsg.STEP_PICFLIP, 0.005)
        ref.step(fsg.STEP_PICFLIP, 0.005)
        assert_same(g.state(), ref.state(), where="after recovery, step %d" % k)


@pytest.mark.parametrize("shape", [(64, 64), (40, 64)])
def test_level_set_path_matches_oracle(shape):
    """FluidDomain::advectLevelSet and classifyCells(LevelSet&) on the device,
    square and narrow grids (the reference's swapped loop bounds), several
    advections interleaved with steps, then the level-set render pass."""
    nx, ny = shape
    sc = scenes.dam_break_small()
    g = fsg.FluidSim(nx, ny, float(nx), float(ny), 0.005, 0.02, cg_tolerance=1e-6, cg_max_iterations=400)
    o = po.OracleSim("restatement", nx, ny, float(nx), float(ny), 0.005, 0.02)
    o.set_cg(1e-6, 400)
    parts = scenes.block_particles(nx, ny, float(nx), float(ny), 1, nx // 2, 1, ny // 2, 4, 9)
    g.set_particles(parts)
    o.set_particles(parts)
    jj, ii = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    ls = (np.hypot(ii + 0.5 - nx / 3, jj + 0.5 - ny / 3) - nx / 5).astype(np.float32)
    g.set_level_set(ls)
    o.set_level_set(ls)
    for k in range(4):
        g.step(fsg.STEP_PICFLIP, sc.dt)
        o.step(po.STEP_PICFLIP, sc.dt)
        g.advect_level_set(0.05)
        o.advect_level_set(0.05)
        assert np.array_equal(g.level_set().view(np.uint32), o.level_set().view(np.uint32)), k
    g.classify_level_set()
    o.classify_level_set()
    assert np.array_equal(g.labels(), o.labels())
    c = fsg.Canvas(90, 70)
    g.render(c, fsg.RENDER_LEVEL_SET, (0.0, float(nx), 0.0, float(ny)))
    ref, k6 = np.ones((70, 90, 3), np.float32), np.array([0, 0, 0, 1, 1, 1], np.float32)
    o.render(po.RENDER_LEVEL_SET, (0.0, float(nx), 0.0, float(ny)), ref, k6)
    assert np.array_equal(c.pixels().view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(c.colors().view(np.uint32), k6.view(np.uint32))


def test_p2g_weight_threshold_edge():
    """transferVelocityToGridSpread keeps a face's previous back value unless
    its weight exceeds 1e-6 (src/FluidSolver.cpp:898-917): isolated particles
    a hair from a grid line put weights just below, at and above it."""
    n = 32
    rng = np.random.default_rng(5)
    offs = np.array([1e-7, 4e-7, 9.9e-7, 1e-6, 1.05e-6, 3e-6, 1 - 1e-7, 1 - 9.9e-7, 1 - 1.05e-6], np.float64)
    parts = []
    for k, f in enumerate(offs):
        i, j = 3 + 3 * k, 4 + (k % 3) * 7
        parts.append([i + f, j + 0.5 + f, 1.0 + k, -2.0 + k])  # u footprint at (x, y - 0.5)
        parts.append([i + 0.5 + f, j + 1 - f, -1.0 - k, 3.0 - k])
    parts = np.array(parts, np.float32)
    g = fsg.FluidSim(n, n, float(n), float(n), 1.0, 0.0)
    o = po.OracleSim("restatement", n, n, float(n), float(n), 1.0, 0.0)
    grids = [rng.standard_normal((n, n)).astype(np.float32) for _ in range(8)]
    for s in (g, o):
        for w, arr in enumerate(grids):
            s.set_grid(w, arr)
        s.set_particles(parts)
    g.phase(fsg.PH_P2G, 0.005)
    o.phase(po.PH_P2G, 0.005)
    assert_same(g.state(), o.state(), where="P2G threshold")
    # the edge is exercised: some touched faces kept their old value, others were replaced
    ub0 = grids[fsg.U_BACK]
    uf = g.grid(fsg.U_FRONT)  # the back buffer became the front
    assert (uf == ub0).sum() > 0 and (uf != ub0).sum() > 0


@pytest.mark.parametrize("method", [fsg.STEP_PICFLIP, fsg.STEP_SEMI_LAGRANGIAN])
@pytest.mark.parametrize("length", [48.0, 12.0])
def test_particles_on_cell_corners_and_faces(method, length):
    """Particles exactly on grid lines: cell classification truncates x / dx at
    an integer (src/FluidDomain.cpp:150-180) and the bilinear weights of the
    splat and the gather are exactly 0 and 1 (include/Grid.h:117-184)."""
    n = 48
    dx = length / n
    ii, jj = np.meshgrid(np.arange(4, 28) * 0.5, np.arange(4, 36) * 0.5)  # corners and face centres
    rng = np.random.default_rng(9)
    parts = np.stack([ii.ravel() * dx, jj.ravel() * dx,
                      rng.standard_normal(ii.size), rng.standard_normal(ii.size)], 1).astype(np.float32)
    g = fsg.FluidSim(n, n, length, length, 1.0, 0.05, cg_tolerance=1e-6, cg_max_iterations=2000)
    o = po.OracleSim("restatement", n, n, length, length, 1.0, 0.05)
    o.set_cg(1e-6, 2000)
    g.set_particles(parts)
    o.set_particles(parts)
    for k in range(5):
        g.step(method, 0.005)
        assert o.step(method, 0.005) == 0
        assert_same(g.state(), o.state(), where="grid-line particles step %d" % k)


@pytest.mark.parametrize("method", [fsg.STEP_PICFLIP, fsg.STEP_SEMI_LAGRANGIAN])
def test_particles_outside_the_domain(method):
    """Particles beyond every wall and on the domain's edge: classification,
    the splat and the gather clamp their cells to the grid like the reference
    (src/FluidDomain.cpp:150-180, include/Grid.h:117-184); the per-cell
    particle count, which the reference does not clamp (src/FluidSolver.cpp:
    353-360, undefined there), skips them here and in the oracle alike."""
    n, length = 40, 40.0
    rng = np.random.default_rng(21)
    block = scenes.block_particles(n, n, length, length, 2, 14, 2, 20, 2, 21)
    xs = np.array([-2.5, -0.3, -1e-3, 0.0, length, length + 1e-3, 1.7 * length, 3.25 * length], np.float32)
    ys = np.array([-1.5, -0.01, 0.0, 7.25, length, 1.2 * length, 2.0 * length, 19.5], np.float32)
    xx, yy = np.meshgrid(xs, ys)
    outside = np.stack([xx.ravel(), yy.ravel(), rng.standard_normal(xx.size), rng.standard_normal(xx.size)],
                       1).astype(np.float32)
    parts = np.concatenate([block, outside])
    g = fsg.FluidSim(n, n, length, length, 1.0, 0.05, cg_tolerance=1e-6, cg_max_iterations=2000)
    o = po.OracleSim("restatement", n, n, length, length, 1.0, 0.05)
    o.set_cg(1e-6, 2000)
    g.set_particles(parts)
    o.set_particles(parts)
    for k in range(5):
        g.step(method, 0.005)
        assert o.step(method, 0.005) == 0
        assert_same(g.state(), o.state(), where="outside particles step %d" % k)
