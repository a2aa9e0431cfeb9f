"""The allocation-free pressure solve (fs_pressure_solve_noalloc) through the C
ABI, against the pressure the regular handle path computes from the same
state (fs_phase(FS_PH_PRESSURE) + fs_get_pressure).

fs_pressure_solve_noalloc serves callers that must not allocate device
memory once they run (a frame loop that cannot afford the stall of a
cudaMalloc, a plugin confined to its host's memory budget); it keeps its
scratch in a static device array shared by every call.  Two calls in a row
must both match, so the second call sees whatever the first left in that
array.  The test itself allocates its input and output buffers freely; only
the entry point may not.  This file is collected last so that a run stopping
at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import build as fsbuild
from fluid_simulation_gb300 import scenes

pytestmark = pytest.mark.gpu

NX, NY = 128, 112  # 14336 cells, under the 16384-cell limit


def _state_before_pressure(sim, dt):
    for ph in (fsg.PH_CLASSIFY, fsg.PH_P2G, fsg.PH_SAVE_PREV, fsg.PH_GRAVITY, fsg.PH_DIRICHLET, fsg.PH_EXTEND):
        sim.phase(ph, dt)
    return sim.labels(), sim.grid(fsg.U_FRONT), sim.grid(fsg.V_FRONT)


@pytest.mark.parametrize("precision", [fsg.CG_FLOAT, fsg.CG_DOUBLE])
def test_noalloc_pressure_matches_handle_path_two_calls(precision):
    torch = pytest.importorskip("torch")
    fsbuild.build()
    lib = fsg.load_library()
    solid = scenes.disc_mask(NX, NY, 95.0, 30.0, 12.0)
    parts = scenes.block_particles(NX, NY, float(NX), float(NY), 1, 50, 1, 70, 4, 21, solid)
    tol, maxit, dt = 1e-5, 5000, 0.005
    sim = fsg.FluidSim(NX, NY, float(NX), float(NY), dt, 0.05, cg_tolerance=tol, cg_max_iterations=maxit)
    sim.set_cg_precision(precision)
    sim.set_solid_mask(solid)
    sim.set_particles(parts)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        for _ in range(3 + 5 * call):
            sim.step(fsg.STEP_PICFLIP, dt)
        labels, u, v = _state_before_pressure(sim, dt)
        d_lab = torch.from_numpy(labels).cuda()
        d_u = torch.from_numpy(u).cuda()
        d_v = torch.from_numpy(v).cuda()
        d_p = torch.full((NY, NX), float("nan"), dtype=torch.float32, device="cuda")
        it, res = C.c_int(-1), C.c_double(-1.0)
        rc = lib.fs_pressure_solve_noalloc(NX, NY, float(NX), float(NY), d_lab.data_ptr(), d_u.data_ptr(),
                                           d_v.data_ptr(), tol, maxit, precision, d_p.data_ptr(), C.byref(it),
                                           C.byref(res), stream)
        assert rc == 0, lib.fs_last_error(None)
        torch.cuda.synchronize()
        p_noalloc = d_p.cpu().numpy()

        sim.phase(fsg.PH_PRESSURE, dt)
        p_ref = sim.pressure()
        st = sim.stats()
        assert st["n_fluid"] > 1000
        # Same kernels in the same order: identical to the last bit.
        assert np.array_equal(p_noalloc.view(np.uint32), p_ref.view(np.uint32)), "call %d" % call
        assert it.value == st["cg_iterations"]
        assert res.value == st["cg_residual"]


def _noalloc_vs_handle(lib, torch, nx, ny, steps, with_outputs=True):
    """One allocation-free solve of a disc-obstacle dam break of nx x ny after
    `steps` steps, and the handle path's pressure of the same state."""
    solid = scenes.disc_mask(nx, ny, 0.75 * nx, 0.25 * ny, 0.1 * min(nx, ny))
    parts = scenes.block_particles(nx, ny, float(nx), float(ny), 1, int(0.4 * nx), 1, int(0.6 * ny), 4, nx + ny,
                                   solid)
    tol, maxit, dt = 1e-5, 5000, 0.005
    sim = fsg.FluidSim(nx, ny, float(nx), float(ny), dt, 0.05, cg_tolerance=tol, cg_max_iterations=maxit)
    sim.set_solid_mask(solid)
    sim.set_particles(parts)
    for _ in range(steps):
        sim.step(fsg.STEP_PICFLIP, dt)
    labels, u, v = _state_before_pressure(sim, dt)
    d_lab = torch.from_numpy(labels).cuda()
    d_u = torch.from_numpy(u).cuda()
    d_v = torch.from_numpy(v).cuda()
    d_p = torch.full((ny, nx), float("nan"), dtype=torch.float32, device="cuda")
    it, res = C.c_int(-1), C.c_double(-1.0)
    rc = lib.fs_pressure_solve_noalloc(nx, ny, float(nx), float(ny), d_lab.data_ptr(), d_u.data_ptr(),
                                       d_v.data_ptr(), tol, maxit, fsg.CG_FLOAT, d_p.data_ptr(),
                                       C.byref(it) if with_outputs else None,
                                       C.byref(res) if with_outputs else None,
                                       torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.fs_last_error(None)
    torch.cuda.synchronize()
    sim.phase(fsg.PH_PRESSURE, dt)
    assert sim.stats()["n_fluid"] > 100
    return d_p.cpu().numpy(), sim.pressure(), (it.value if with_outputs else None), sim.stats()


def test_noalloc_smaller_grid_after_larger_one():
    """The shared array still holds a 128 x 128 call's values past a smaller
    grid's cells; the 64 x 48 call after it must not see them.  Calls without
    the optional outputs return the same pressure."""
    torch = pytest.importorskip("torch")
    fsbuild.build()
    lib = fsg.load_library()
    for nx, ny, steps, with_outputs in ((128, 128, 6, True), (64, 48, 4, False), (128, 128, 2, False),
                                        (40, 72, 5, True)):
        p_noalloc, p_ref, it, st = _noalloc_vs_handle(lib, torch, nx, ny, steps, with_outputs=with_outputs)
        assert np.array_equal(p_noalloc.view(np.uint32), p_ref.view(np.uint32)), (nx, ny)
        if with_outputs:
            assert it == st["cg_iterations"]


def test_noalloc_rejects_grids_beyond_its_limit():
    torch = pytest.importorskip("torch")
    fsbuild.build()
    lib = fsg.load_library()
    n = 129  # 129 x 129 = 16641 cells > 16384
    d_lab = torch.zeros((n, n), dtype=torch.uint8, device="cuda")
    d_u = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    d_p = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    rc = lib.fs_pressure_solve_noalloc(n, n, float(n), float(n), d_lab.data_ptr(), d_u.data_ptr(), d_u.data_ptr(),
                                       1e-5, 100, 0, d_p.data_ptr(), None, None, None)
    assert rc == 5  # FS_ERR_TOO_LARGE
    assert b"16384-cell limit" in lib.fs_last_error(None)
