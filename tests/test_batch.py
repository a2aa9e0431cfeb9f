"""Batch of independent simulations (fs_batch_*): after every step, each
simulation's state is bit-identical to the CPU restatement of the reference
stepping that simulation alone (velocity grids front/back/previous/
difference, labels, pressure, particles, CG iteration counts)."""
import numpy as np
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import build as fsbuild
from fluid_simulation_gb300 import scenes
from oracle import pyoracle as po

KEYS = ("u_front", "v_front", "u_back", "v_back", "u_prev", "v_prev", "u_diff", "v_diff", "labels", "pressure",
        "particles")


def oracle_for(sc):
    o = po.OracleSim("restatement", sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    o.set_cg(sc.cg_tolerance, sc.cg_max_iterations)
    o.set_gravity(*sc.gravity)
    if sc.solid is not None:
        o.set_solid_mask(sc.solid)
    o.set_particles(sc.particles)
    return o


def assert_same(a_state, o_state, where):
    for k in KEYS:
        a, b = a_state[k], o_state[k]
        assert a.shape == b.shape, (where, k)
        if not np.array_equal(a.view(np.uint8), b.view(np.uint8)):
            bad = np.argwhere(a != b)
            raise AssertionError("%s: %s differs at %d entries, first %s" % (where, k, len(bad),
                                                                              tuple(bad[0]) if len(bad) else None))


def mixed_scenes():
    """Small random members plus one of each CG cluster class (1, 2, 4 and 8
    CTAs per simulation at 8 chunks per CTA)."""
    sc = scenes.batch_scenes(n=5, seed=11, min_side=24, max_side=72)
    big = scenes.batch_scenes(n=40, seed=12, min_side=96, max_side=256)
    want = [(96, 130), (130, 182), (182, 257)]
    for lo, hi in want:
        sc.append(next(s for s in big if lo <= s.size_x < hi))
    return sc


def test_batch_scenes_are_deterministic_and_in_range():
    a = scenes.batch_scenes(n=24)
    b = scenes.batch_scenes(n=24)
    for x, y in zip(a, b):
        assert x.size_x == y.size_x and np.array_equal(x.particles, y.particles)
        assert 32 <= x.size_x <= 256 and x.size_x == x.size_y
        assert 0.0 <= x.pic_ratio <= 0.1 + 1e-7
        i0, i1, j0, j1 = x.meta["block"]
        assert 1 <= i0 < i1 <= x.size_x - 1 and 1 <= j0 < j1 <= x.size_y - 1
        p = x.particles
        assert np.all((p[:, 0] >= i0) & (p[:, 0] < i1) & (p[:, 1] >= j0) & (p[:, 1] < j1))
        if x.solid is not None:
            assert not x.solid[p[:, 1].astype(int), p[:, 0].astype(int)].any()


def test_batch_rejects_simulations_beyond_its_limits():
    lib = fsg.load_library()
    cfg = fsg.fs_config()
    lib.fs_config_init(fsg.C.byref(cfg), 300, 300)
    with pytest.raises(fsg.FsError) as e:
        fsg.FluidBatch([cfg])
    assert e.value.code == 5
    with pytest.raises(fsg.FsError) as e:
        fsg.FluidBatch([])
    assert e.value.code == 1
    # double-single dot products are a handle and Poisson option only
    lib.fs_config_init(fsg.C.byref(cfg), 64, 64)
    cfg.cg_precision = fsg.CG_DS
    with pytest.raises(fsg.FsError) as e:
        fsg.FluidBatch([cfg])
    assert e.value.code == 1 and "double-single" in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("method", [fsg.STEP_PICFLIP, fsg.STEP_SEMI_LAGRANGIAN, fsg.STEP_PIC, fsg.STEP_FLIP])
def test_batch_matches_oracle_per_simulation(method):
    fsbuild.build()
    sc = mixed_scenes() if method == fsg.STEP_PICFLIP else scenes.batch_scenes(n=4, seed=21, max_side=64)
    b = fsg.FluidBatch.from_scenes(sc)
    os_ = [oracle_for(s) for s in sc]
    nsteps = 4 if method == fsg.STEP_PICFLIP else 3
    for k in range(nsteps):
        b.step(method, 0.005)
        for s, o in enumerate(os_):
            assert o.step(method, 0.005) == 0
            assert_same(b.state(s), o.state(), "method %d step %d sim %d (%dx%d)" % (
                method, k, s, sc[s].size_x, sc[s].size_y))
            it, res, nf = o.cg_stats()
            st = b.stats(s)
            assert (st["cg_iterations"], st["n_fluid"]) == (it, nf), (k, s)
    # the comparison is not vacuous: the fields and the particles moved
    last = len(sc) - 1
    assert np.abs(os_[-1].state()["v_front"]).max() > 0
    assert not np.array_equal(b.state(last)["particles"][:, :2], sc[last].particles[:, :2])


@pytest.mark.gpu
def test_batch_tune_leaves_state_and_continues_bit_exact():
    fsbuild.build()
    sc = scenes.batch_scenes(n=6, seed=31, max_side=96)
    b = fsg.FluidBatch.from_scenes(sc)
    os_ = [oracle_for(s) for s in sc]
    b.step(fsg.STEP_PICFLIP, 0.005)
    for o in os_:
        o.step(po.STEP_PICFLIP, 0.005)
    before = [b.state(s) for s in range(len(sc))]
    t = b.tune(fsg.STEP_PICFLIP, 0.005, steps=1)
    assert t["chunks_per_cta"] in (1, 2, 4, 8) and all(v > 0 for v in t["ms_per_step"].values())
    for s in range(len(sc)):
        assert_same(b.state(s), before[s], "after tune sim %d" % s)
    for k in range(2):
        b.step(fsg.STEP_PICFLIP, 0.005)
        for s, o in enumerate(os_):
            o.step(po.STEP_PICFLIP, 0.005)
            assert_same(b.state(s), o.state(), "tuned step %d sim %d" % (k, s))


@pytest.mark.gpu
@pytest.mark.parametrize("plan", [1, 2, 4, 8])
def test_batch_every_cluster_plan_and_direct_launches_agree(plan):
    fsbuild.build()
    sc = mixed_scenes()
    ref = fsg.FluidBatch.from_scenes(sc)
    alt = fsg.FluidBatch.from_scenes(sc)
    alt.set_tuning(plan)
    alt.set_graphs(False)
    for k in range(2):
        ref.step(fsg.STEP_PICFLIP, 0.005)
        alt.step(fsg.STEP_PICFLIP, 0.005)
    for s in range(len(sc)):
        assert_same(alt.state(s), ref.state(s), "plan %d sim %d" % (plan, s))


@pytest.mark.gpu
def test_batch_validate_quirk_and_empty_members():
    """A member with dx != dy fails every step (FluidSolver::validate against
    the pool's dx-for-dy copy, src/FluidSolver.cpp:56-62,89-97); members
    without particles step like an empty domain."""
    fsbuild.build()
    lib = fsg.load_library()
    cfgs = []
    for nx, ny, lx, ly in ((40, 40, 40.0, 40.0), (40, 30, 40.0, 60.0)):
        c = fsg.fs_config()
        lib.fs_config_init(fsg.C.byref(c), nx, ny)
        c.length_x, c.length_y = lx, ly
        cfgs.append(c)
    b = fsg.FluidBatch(cfgs)
    with pytest.raises(fsg.FsError) as e:
        b.step(fsg.STEP_PICFLIP, 0.005)
    assert e.value.code == 2 and "simulation 1" in str(e.value)
    sc = scenes.batch_scenes(n=2, seed=41, max_side=48)
    b = fsg.FluidBatch.from_scenes(sc)
    b.set_particles(1, np.zeros((0, 4), np.float32))
    o = oracle_for(sc[0])
    e_ = po.OracleSim("restatement", sc[1].size_x, sc[1].size_y, sc[1].length_x, sc[1].length_y, sc[1].density,
                      sc[1].pic_ratio)
    e_.set_cg(sc[1].cg_tolerance, sc[1].cg_max_iterations)
    if sc[1].solid is not None:
        e_.set_solid_mask(sc[1].solid)
    for k in range(2):
        b.step(fsg.STEP_PICFLIP, 0.005)
        o.step(po.STEP_PICFLIP, 0.005)
        e_.step(po.STEP_PICFLIP, 0.005)
        assert_same(b.state(0), o.state(), "step %d sim 0" % k)
        assert_same(b.state(1), e_.state(), "step %d empty sim" % k)


@pytest.mark.gpu
def test_batch_member_outgrowing_its_cluster_plan_stays_exact():
    """A plan made after a step (here by fs_batch_set_tuning, as the tuner
    does) sizes each member's cluster for its current fluid cells; a member
    whose fluid then grows past that size solves from global memory, with the
    same results."""
    fsbuild.build()
    sc = scenes.batch_scenes(n=3, seed=51, min_side=120, max_side=200)
    s0 = sc[0]
    small = scenes.block_particles(s0.size_x, s0.size_y, s0.length_x, s0.length_y, 1, 9, 1, 9, 4, 77, s0.solid)
    b = fsg.FluidBatch.from_scenes(sc)
    b.set_particles(0, small)
    os_ = [oracle_for(s) for s in sc]
    os_[0].set_particles(small)
    b.step(fsg.STEP_PICFLIP, 0.005)
    for o in os_:
        o.step(po.STEP_PICFLIP, 0.005)
    b.set_tuning(8)  # after a step: sized for the fluid cells that step counted
    b.set_particles(0, s0.particles)
    os_[0].set_particles(s0.particles)
    for k in range(3):
        b.step(fsg.STEP_PICFLIP, 0.005)
        for s, o in enumerate(os_):
            o.step(po.STEP_PICFLIP, 0.005)
            assert_same(b.state(s), o.state(), "grown step %d sim %d" % (k, s))
    assert b.stats(0)["n_fluid"] > 4 * 1024 * 5 // 4


def _launch_class(n_fluid, interior, target):
    """(chunks per CTA footprint, CTAs per cluster) of a member planned from
    n_fluid fluid cells for the tuner's target chunks per CTA (the planning
    rule of fs_batch: current fluid cells plus 25%, at most the interior,
    in 1024-cell chunks; the smallest power-of-two cluster up to 8 that keeps
    the chunks per CTA at or under the target)."""
    ch = max(1, min((n_fluid * 5 // 4 + 1023) // 1024, max(1, (interior + 1023) // 1024)))
    c = 1
    while c < 8 and -(-ch // c) > target:
        c *= 2
    return (4 if -(-ch // c) <= 4 else 8, c)


@pytest.mark.gpu
def test_full_batch_workload_members_bit_exact_after_tuning():
    """The benchmark's batched workload itself -- 512 members of sides
    U{32..256} (seed 0xC3), 12.9M cells -- tuned as the benchmark tunes it,
    then stepped: after each of three steps, at least 32 members are
    bit-identical to the restatement stepping each alone, among them every
    member of side 248 or more, members with three discs, and the first
    member of every CG launch class of the tuned plan."""
    fsbuild.build()
    sc = scenes.batch_scenes(512)
    b = fsg.FluidBatch.from_scenes(sc)
    b.step(fsg.STEP_PICFLIP, 0.005)
    nf = [b.stats(s)["n_fluid"] for s in range(len(sc))]
    t = b.tune(fsg.STEP_PICFLIP, 0.005, steps=2)
    target = t["chunks_per_cta"]
    classes = {}
    for s, x in enumerate(sc):
        classes.setdefault(_launch_class(nf[s], (x.size_x - 2) * (x.size_y - 2), target), []).append(s)
    pick = {v[0] for v in classes.values()}
    pick |= {s for s, x in enumerate(sc) if x.size_x >= 248}
    pick |= set([s for s, x in enumerate(sc) if x.meta["discs"] == 3][:8])
    pick |= set(range(0, 512, 32))
    pick = sorted(pick)
    assert len(pick) >= 32 and len(classes) >= 3, (len(pick), sorted(classes))
    os_ = {s: oracle_for(sc[s]) for s in pick}
    for o in os_.values():
        assert o.step(po.STEP_PICFLIP, 0.005) == 0
    for k in range(3):
        b.step(fsg.STEP_PICFLIP, 0.005)
        for s in pick:
            o = os_[s]
            assert o.step(po.STEP_PICFLIP, 0.005) == 0
            assert_same(b.state(s), o.state(), "tuned 512-member batch, step %d, sim %d (%dx%d)"
                        % (k + 2, s, sc[s].size_x, sc[s].size_y))
            it, res, n = o.cg_stats()
            st = b.stats(s)
            assert (st["cg_iterations"], st["n_fluid"]) == (it, n), (k, s)
    assert max(sc[s].size_x for s in pick) >= 250
