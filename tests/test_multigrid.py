"""Multigrid-preconditioned CG (not the reference's method, so checked against
the mathematics rather than bit for bit): the standalone Poisson solve against
an FP64 direct solve, its iteration count against the Jacobi-preconditioned
CG's, and the step with the multigrid pressure solver against the step with
the reference's solver."""
import numpy as np
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import build as fsbuild
from fluid_simulation_gb300 import scenes

pytestmark = pytest.mark.gpu


def direct_solve(labels, rhs):
    """FP64 sparse solve of the reference's system (one unknown pinned per
    connected fluid component without AIR), demeaned where singular."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    from scipy import ndimage

    ny, nx = labels.shape
    fl = labels == 0
    idx = -np.ones(labels.shape, np.int64)
    cells = np.flatnonzero(fl)
    idx.reshape(-1)[cells] = np.arange(cells.size)
    rows, cols, vals = [], [], []
    for di, dj in ((-1, 0), (1, 0), (0, -1), (0, 1)):
        for j, i in zip(*np.nonzero(fl)):
            ii, jj = min(max(i + di, 0), nx - 1), min(max(j + dj, 0), ny - 1)
            t = labels[jj, ii]
            if t != 2:
                rows.append(idx[j, i]); cols.append(idx[j, i]); vals.append(-1.0)
                if t == 0 and (ii, jj) != (i, j):
                    rows.append(idx[j, i]); cols.append(idx[jj, ii]); vals.append(1.0)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(cells.size, cells.size))
    b = rhs.reshape(-1)[cells]
    comp, nc = ndimage.label(fl, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    air_near = ndimage.binary_dilation(labels == 1, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    keep = np.ones(cells.size, bool)
    singular = []
    for c in range(1, nc + 1):
        if not (air_near & (comp == c)).any():
            keep[idx[comp == c][0]] = False
            singular.append(c)
    x = np.zeros(cells.size)
    x[keep] = spla.spsolve(A[keep][:, keep].tocsc(), b[keep])
    cc = comp.reshape(-1)[cells]
    for c in singular:
        m = cc == c
        x[m] -= x[m].mean()
    out = np.zeros(labels.size)
    out[cells] = x
    return out.reshape(labels.shape), singular, comp


def free_surface_problem(n=96, seed=3):
    labels, rhs = scenes.projection_problem(n, seed=seed)
    labels = labels.copy()
    labels[n // 2:, 1:-1] = np.where(labels[n // 2:, 1:-1] == 0, 1, labels[n // 2:, 1:-1])  # AIR above
    rng = np.random.default_rng(seed)
    rhs = np.where(labels == 0, rng.standard_normal(labels.shape), 0.0)
    return labels, rhs


@pytest.mark.parametrize("problem,n", [("neumann", 96), ("free_surface", 96), ("free_surface", 40)])
def test_mgpcg_poisson_against_fp64_direct_solve(problem, n):
    """n = 40: every level of the V-cycle runs in the single-CTA kernel."""
    fsbuild.build()
    labels, rhs = scenes.projection_problem(n, seed=7) if problem == "neumann" else free_surface_problem(n)
    ps = fsg.PoissonSolver(n, n, float(n), float(n))
    ps.set_problem(labels, rhs)
    mg = ps.solve(fsg.POISSON_MGPCG, 1e-6, 2000)
    x = ps.solution()
    jac = ps.solve(fsg.POISSON_FP32, 1e-6, 20000)
    xd, singular, comp = direct_solve(labels, rhs)
    for c in singular:  # the solution is defined up to a constant there
        m = comp == c
        x[m] -= x[m].mean()
    err = np.linalg.norm(x - xd) / np.linalg.norm(xd)
    print(problem, "MGPCG iterations", mg["inner_iterations"], "Jacobi-PCG", jac["inner_iterations"],
          "residual", mg["residual"], "error", err)
    assert mg["residual"] < 1e-4
    assert err < 1e-4
    assert mg["inner_iterations"] * 4 < jac["inner_iterations"]


def divergence(sim):
    """Divergence of the front velocities on fluid cells (unit cells)."""
    u, v, lab = sim.grid(fsg.U_FRONT), sim.grid(fsg.V_FRONT), sim.labels()
    div = (u[:-1, 1:] - u[:-1, :-1]) + (v[1:, :-1] - v[:-1, :-1])
    return div[lab[:-1, :-1] == 0]


def test_step_with_multigrid_pressure_solver():
    fsbuild.build()
    sc = scenes.dam_break_large(256)
    ref = fsg.FluidSim.from_scene(sc)
    for _ in range(3):
        ref.step(fsg.STEP_PICFLIP, sc.dt)
    snap = ref.snapshot()
    ref.set_cg(1e-6, 20000)
    ref.step(fsg.STEP_PICFLIP, sc.dt)
    p_ref, s_ref = ref.pressure(), ref.stats()
    div_ref = divergence(ref)
    ref.restore(snap)
    ref.set_pressure_solver(fsg.SOLVER_MGPCG)
    ref.step(fsg.STEP_PICFLIP, sc.dt)
    p_mg, s_mg = ref.pressure(), ref.stats()
    print("Jacobi-PCG iterations", s_ref["cg_iterations"], "MGPCG", s_mg["cg_iterations"])
    assert s_mg["n_fluid"] == s_ref["n_fluid"]
    assert s_mg["cg_residual"] < 1e-6 and s_mg["cg_iterations"] * 5 < s_ref["cg_iterations"]
    assert np.abs(p_mg - p_ref).max() <= 1e-3 * np.abs(p_ref).max()
    # the step leaves as little divergence as the reference's solver does
    assert np.abs(divergence(ref)).max() <= 1.5 * np.abs(div_ref).max() + 1e-4
    for _ in range(100):
        ref.step(fsg.STEP_PICFLIP, sc.dt)
    assert np.isfinite(ref.particles()).all()


def test_mixed_precision_with_multigrid_corrections_reaches_1e10():
    fsbuild.build()
    n = 128
    labels, rhs = scenes.projection_problem(n, seed=11)
    ps = fsg.PoissonSolver(n, n, float(n), float(n))
    ps.set_problem(labels, rhs)
    mm = ps.solve(fsg.POISSON_MIXED_MG, 1e-10, 2000, inner_tol=1e-3)
    x = ps.solution()
    mj = ps.solve(fsg.POISSON_MIXED, 1e-10, 20000, inner_tol=1e-3)
    xd, singular, comp = direct_solve(labels, rhs)
    for c in singular:
        m = comp == c
        x[m] -= x[m].mean()
    err = np.linalg.norm(x - xd) / np.linalg.norm(xd)
    print("mixed+MG", mm, "mixed+Jacobi", mj, "error", err)
    assert mm["residual"] < 1e-10 and err < 1e-8
    assert mm["inner_iterations"] * 10 < mj["inner_iterations"]


def test_mgpcg_on_a_narrow_grid():
    """A 6 x 200 domain: its coarse levels are one cell wide."""
    fsbuild.build()
    nx, ny = 6, 200
    rng = np.random.default_rng(5)
    labels = np.zeros((ny, nx), np.uint8)
    labels[:, 0] = labels[:, -1] = 2
    labels[0, :] = 2
    labels[-20:, 1:-1] = 1  # AIR on top
    labels[rng.random((ny, nx)) < 0.05] = 2
    rhs = np.where(labels == 0, rng.standard_normal(labels.shape), 0.0)
    ps = fsg.PoissonSolver(nx, ny, float(nx), float(ny))
    ps.set_problem(labels, rhs)
    mg = ps.solve(fsg.POISSON_MGPCG, 1e-6, 2000)
    x = ps.solution()
    jac = ps.solve(fsg.POISSON_FP32, 1e-6, 20000)
    xj = ps.solution()
    xd, singular, comp = direct_solve(labels, rhs)
    for c in singular:
        for v in (x, xj):
            m = comp == c
            v[m] -= v[m].mean()
    err = np.linalg.norm(x - xd) / np.linalg.norm(xd)
    err_j = np.linalg.norm(xj - xd) / np.linalg.norm(xd)
    print("narrow MGPCG iterations", mg["inner_iterations"], "residual", mg["residual"], "error", err,
          "| Jacobi-PCG", jac["inner_iterations"], jac["residual"], err_j)
    # both solve in float vectors; this thin domain is ill-conditioned (cond ~ 200^2)
    assert err < 1e-4 and mg["residual"] < max(1e-4, 10 * jac["residual"])
