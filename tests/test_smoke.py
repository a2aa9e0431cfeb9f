"""Differentiable smoke form: the CPU FP64 restatement's adjoint against
central finite differences (CPU), the GPU forward and adjoint against the
restatement, and the GPU gradient against FP64 central differences along
random directions at the full 256 x 256, 64-step size (GPU).  A
torch.autograd.Function wraps the C ABI here, in the tests only."""
import numpy as np
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import scenes
from oracle.smoke import SmokeOracle

INTEGRATORS = [fsg.INTEGRATOR_EULER, fsg.INTEGRATOR_RK2, fsg.INTEGRATOR_RK3]


def small_problem(n=24):
    return scenes.smoke_problem(n, sigma=4.0, shift=(3.0, 2.0), kmax=3)


def directional(g, d):
    return sum(float(np.sum(a * b)) for a, b in zip(g, d))


@pytest.mark.parametrize("integrator", INTEGRATORS)
def test_restatement_adjoint_matches_central_differences(integrator):
    n, steps, dt = 24, 6, 0.05
    u, v, d, t = small_problem(n)
    solid = np.zeros((n, n), np.uint8)
    solid[10:13, 14:16] = 1
    o = SmokeOracle(n, n, dt=dt, integrator=integrator, solid=solid)
    loss, st = o.forward(u, v, d, t, steps)
    g = o.backward(st, t, loss)
    rng = np.random.default_rng(integrator)
    eps = 1e-6
    for _ in range(4):
        dirs = rng.standard_normal((3, n, n))
        lp = o.forward(u + eps * dirs[0], v + eps * dirs[1], d + eps * dirs[2], t, steps)[0]
        lm = o.forward(u - eps * dirs[0], v - eps * dirs[1], d - eps * dirs[2], t, steps)[0]
        fd = (lp - lm) / (2 * eps)
        ad = directional(g, dirs)
        assert abs(fd - ad) <= 1e-6 * abs(fd), (fd, ad)


def test_restatement_projection_is_a_projection():
    n = 20
    o = SmokeOracle(n, n)
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal((2, n, n))
    u[~o.u_open] = 0
    v[~o.v_open] = 0
    pu, pv = o.project(u, v)
    assert np.abs(o.divergence(pu, pv)).max() < 1e-10
    qu, qv = o.project(pu, pv)
    assert np.allclose(qu, pu, atol=1e-12) and np.allclose(qv, pv, atol=1e-12)


def gpu_smoke(n, dt, integrator, precision, steps_tol=1e-12, checkpoint_every=8, solid=None,
              projection=fsg.POISSON_MIXED):
    from fluid_simulation_gb300 import build as fsbuild

    fsbuild.build()
    s = fsg.Smoke(n, n, dt=dt, integrator=integrator, precision=precision, projection_method=projection,
                  cg_tolerance=steps_tol, checkpoint_every=checkpoint_every)
    if solid is not None:
        s.set_solid_mask(solid)
    return s


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.gpu
@pytest.mark.parametrize("integrator", INTEGRATORS)
@pytest.mark.parametrize("precision", [fsg.SMOKE_FP64, fsg.SMOKE_FP32])
def test_gpu_forward_and_gradient_match_restatement(integrator, precision):
    n, steps, dt = 48, 10, 0.05
    u, v, d, t = scenes.smoke_problem(n, sigma=8.0, shift=(5.0, 3.0), kmax=4)
    solid = np.zeros((n, n), np.uint8)
    solid[20:24, 28:31] = 1
    o = SmokeOracle(n, n, dt=dt, integrator=integrator, solid=solid)
    loss_o, st = o.forward(u, v, d, t, steps)
    go = o.backward(st, t, loss_o)
    s = gpu_smoke(n, dt, integrator, precision, checkpoint_every=3, solid=solid)
    s.set_state(u, v, d)
    s.set_target(t)
    loss = s.forward(steps)
    gu, gv, gd = s.backward()
    # FP64: the projections are CG solves to a relative residual of 1e-12
    # (the restatement solves exactly), a few 1e-10 on the solution at this size
    tol_state, tol_grad = (1e-8, 1e-6) if precision == fsg.SMOKE_FP64 else (2e-5, 2e-3)
    for a, b in zip(s.state(), st[-1]):
        assert rel(a, b) < tol_state
    assert abs(loss - loss_o) <= tol_state * loss_o
    for a, b in zip((gu, gv, gd), go):
        assert rel(a, b) < tol_grad, (rel(a, b), tol_grad)


@pytest.mark.gpu
def test_gpu_gradient_matches_fp64_central_differences_full_size():
    """256 x 256, 64 RK2 steps at dt = 0.01, checkpoints every 8 steps: the
    adjoint against FP64 central differences of the FP64 forward along 16
    random directions (relative error < 1e-4), and against the FP64 CPU
    restatement's gradient."""
    n, steps, dt = 256, 64, 0.01
    u, v, d, t = scenes.smoke_problem(n)
    s64 = gpu_smoke(n, dt, fsg.INTEGRATOR_RK2, fsg.SMOKE_FP64)
    s64.set_state(u, v, d)
    s64.set_target(t)
    loss = s64.forward(steps)
    g64 = s64.backward()
    s32 = gpu_smoke(n, dt, fsg.INTEGRATOR_RK2, fsg.SMOKE_FP32, steps_tol=1e-10)
    s32.set_state(u, v, d)
    s32.set_target(t)
    loss32 = s32.forward(steps)
    g32 = s32.backward()
    s32.close()
    s32t = gpu_smoke(n, dt, fsg.INTEGRATOR_RK2, fsg.SMOKE_FP32_TRACE64, steps_tol=1e-10)
    s32t.set_state(u, v, d)
    s32t.set_target(t)
    loss32t = s32t.forward(steps)
    g32t = s32t.backward()
    s32t.close()
    rng = np.random.default_rng(0xC4)
    eps = 1e-6
    worst64 = worst32 = worst32t = 0.0
    for _ in range(16):
        dirs = rng.standard_normal((3, n, n))
        s64.set_state(u + eps * dirs[0], v + eps * dirs[1], d + eps * dirs[2])
        lp = s64.forward(steps)
        s64.set_state(u - eps * dirs[0], v - eps * dirs[1], d - eps * dirs[2])
        lm = s64.forward(steps)
        fd = (lp - lm) / (2 * eps)
        worst64 = max(worst64, abs(directional(g64, dirs) - fd) / abs(fd))
        worst32 = max(worst32, abs(directional(g32, dirs) - fd) / abs(fd))
        worst32t = max(worst32t, abs(directional(g32t, dirs) - fd) / abs(fd))
    print("adjoint vs FP64 central differences, worst relative error: fp64 %.3g fp32 %.3g fp32 with double "
          "traces %.3g; loss %.9g / %.9g / %.9g" % (worst64, worst32, worst32t, loss, loss32, loss32t))
    assert worst64 < 1e-4
    # float fields traced in double meet the target; traced in float, positions within float resolution of
    # a node take the other one-sided derivative of the bilinear sampler than the FP64 forward does
    assert worst32t < 1e-4
    assert worst32 < 1e-2
    o = SmokeOracle(n, n, dt=dt, integrator=fsg.INTEGRATOR_RK2)
    loss_o, st = o.forward(u, v, d, t, steps)
    go = o.backward(st, t, loss_o)
    assert abs(loss - loss_o) <= 1e-8 * loss_o
    for a, b in zip(g64, go):
        assert rel(a, b) < 1e-5


@pytest.mark.gpu
def test_gpu_gradient_with_multigrid_projection_full_size():
    """The full-size problem with the projections solved by FP64 refinement
    around multigrid-preconditioned float corrections (FS_POISSON_MIXED_MG)
    instead of Jacobi-preconditioned ones, to the same 1e-10: the FP64
    gradient equals the Jacobi-projected one to 1e-6 relative, and with float
    fields traced in double the directional derivatives along the 16 random
    directions stay within 1e-4 of the FP64 ones."""
    n, steps, dt = 256, 64, 0.01
    u, v, d, t = scenes.smoke_problem(n)
    grads = {}
    for name, prec, proj in (("jacobi64", fsg.SMOKE_FP64, fsg.POISSON_MIXED),
                             ("mg64", fsg.SMOKE_FP64, fsg.POISSON_MIXED_MG),
                             ("mg32t", fsg.SMOKE_FP32_TRACE64, fsg.POISSON_MIXED_MG)):
        s = gpu_smoke(n, dt, fsg.INTEGRATOR_RK2, prec, steps_tol=1e-10, projection=proj)
        s.set_state(u, v, d)
        s.set_target(t)
        s.forward(steps)
        grads[name] = s.backward()
        s.close()
    for a, b in zip(grads["mg64"], grads["jacobi64"]):
        assert rel(a, b) < 1e-6, rel(a, b)
    rng = np.random.default_rng(0xC4)
    worst = 0.0
    for _ in range(16):
        dirs = rng.standard_normal((3, n, n))
        ref = directional(grads["jacobi64"], dirs)
        worst = max(worst, abs(directional(grads["mg32t"], dirs) - ref) / abs(ref))
    print("multigrid-projected gradient, float fields traced in double vs FP64: worst directional %.3g" % worst)
    assert worst < 1e-4


@pytest.mark.gpu
def test_torch_autograd_function_over_the_c_abi():
    torch = pytest.importorskip("torch")
    n, steps = 32, 6
    u, v, d, t = small_problem(n)
    s = gpu_smoke(n, 0.05, fsg.INTEGRATOR_RK2, fsg.SMOKE_FP64)
    s.set_target(t)

    class SmokeLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, tu, tv, td):
            s.set_state(tu.detach().numpy(), tv.detach().numpy(), td.detach().numpy())
            return torch.tensor(s.forward(steps), dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad):
            return tuple(grad * torch.from_numpy(a) for a in s.backward())

    tu, tv, td = (torch.tensor(a, requires_grad=True) for a in (u, v, d))
    loss = 3.0 * SmokeLoss.apply(tu, tv, td)
    loss.backward()
    s.set_state(u, v, d)
    s.forward(steps)
    ref = s.backward()
    # the adjoint adds every node's contributions in a fixed order: bit-identical
    for tg, r in zip((tu.grad, tv.grad, td.grad), ref):
        assert np.array_equal(tg.numpy().view(np.uint64), (3.0 * r).view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [fsg.SMOKE_FP32, fsg.SMOKE_FP64, fsg.SMOKE_FP32_TRACE64])
@pytest.mark.parametrize("integrator", [fsg.INTEGRATOR_EULER, fsg.INTEGRATOR_RK2, fsg.INTEGRATOR_RK3])
def test_gpu_gradient_repeats_bit_for_bit(precision, integrator):
    """Two backward passes of the same forward, and a third after a fresh
    forward, give the same gradient to the last bit: the transpose of the
    advection is a gather in a fixed order, with no float atomics."""
    n, steps = 64, 10
    u, v, d, t = small_problem(n)
    s = gpu_smoke(n, 0.02, integrator, precision)
    s.set_state(u, v, d)
    s.set_target(t)
    s.forward(steps)
    g1 = s.backward()
    g2 = s.backward()
    s.forward(steps)
    g3 = s.backward()
    for a, b, c in zip(g1, g2, g3):
        assert np.abs(a).max() > 0
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
        assert np.array_equal(a.view(np.uint64), c.view(np.uint64))
