"""CPU FP64 restatement of the differentiable smoke form (test infrastructure:
only tests, the smoke check and the bench's CPU leg use it).

The form is not in the reference; its pieces restate the reference's
functions in double precision:
  * bilinear sampling: Grid::valueInterpolated (include/Grid.h:117-144) --
    the fraction is taken before the corner indices are clamped, the +1
    corner after; u faces at (i h, (j + 1/2) h), v faces at ((i + 1/2) h,
    j h) (MacGrid::vel{X,Y}Interpolated, include/MacGrid.h:66-79); density at
    cell centres;
  * back-trace with step -dt: explicit Euler, the midpoint rule (RK2) or the
    RK3 of include/OdeSolver.h:102-113 (k2 at h/2, k3 at 3h/4, (2k1 + 3k2 +
    4k3) h / 9), written in the same operation order;
  * projection: the pressure matrix of FluidSolver::pressureSolve
    (src/FluidSolver.cpp:363-416: diagonal -(non-solid neighbours) / h^2,
    +1 / h^2 to fluid neighbours), divergence as MacGrid::divVel{X,Y}
    (include/MacGrid.h:98-111), u -= grad p on faces between fluid cells;
    faces touching a solid cell are closed (zero).  The singular Neumann
    system is solved exactly: one cell per connected fluid component pinned
    to 0, sparse LU of the rest.
The adjoint (reverse mode, written by hand) is the reference gradient the GPU
adjoint is checked against; central finite differences of `forward` check the
adjoint itself.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
from scipy import ndimage

LIQUID, SOLID = 0, 2
EULER, RK2, RK3 = 0, 1, 2


class Foot:
    __slots__ = ("i", "j", "i1", "j1", "fi", "fj")


class SmokeOracle:
    def __init__(self, nx: int, ny: int, h: float = 1.0, dt: float = 0.01, integrator: int = RK2,
                 solid: np.ndarray | None = None):
        self.nx, self.ny, self.h, self.dt, self.integrator = nx, ny, float(h), float(dt), integrator
        lab = np.full((ny, nx), LIQUID, np.uint8)
        lab[0, :] = lab[-1, :] = SOLID
        lab[:, 0] = lab[:, -1] = SOLID
        if solid is not None:
            lab[np.asarray(solid).reshape(ny, nx) != 0] = SOLID
        self.labels = lab
        sol = lab == SOLID
        # open faces: both neighbouring cells non-solid (u: (i-1, j) and (i, j))
        self.u_open = np.zeros((ny, nx), bool)
        self.u_open[:, 1:] = ~sol[:, 1:] & ~sol[:, :-1]
        self.v_open = np.zeros((ny, nx), bool)
        self.v_open[1:, :] = ~sol[1:, :] & ~sol[:-1, :]
        self.fluid = lab == LIQUID
        self._build_poisson()
        jj, ii = np.meshgrid(np.arange(ny, dtype=np.float64), np.arange(nx, dtype=np.float64), indexing="ij")
        hh = self.h
        self.pos = {"u": (ii * hh, (jj + 0.5) * hh), "v": ((ii + 0.5) * hh, jj * hh),
                    "d": ((ii + 0.5) * hh, (jj + 0.5) * hh)}

    # ---- projection -----------------------------------------------------
    def _build_poisson(self):
        nx, ny, h2 = self.nx, self.ny, self.h * self.h
        fl = self.fluid
        idx = -np.ones((ny, nx), np.int64)
        cells = np.flatnonzero(fl.reshape(-1))
        idx.reshape(-1)[cells] = np.arange(cells.size)
        nf = cells.size
        rows, cols, vals = [], [], []
        non_solid = self.labels != SOLID
        for (di, dj) in ((-1, 0), (1, 0), (0, -1), (0, 1)):
            sh = np.zeros((ny, nx), bool)
            nb_idx = -np.ones((ny, nx), np.int64)
            ys = slice(max(0, -dj), ny - max(0, dj))
            xs = slice(max(0, -di), nx - max(0, di))
            yt = slice(max(0, dj), ny - max(0, -dj))
            xt = slice(max(0, di), nx - max(0, -di))
            sh[ys, xs] = non_solid[yt, xt]
            nb_idx[ys, xs] = idx[yt, xt]
            m = fl & sh
            r = idx[m]
            rows.append(r)
            cols.append(r)
            vals.append(np.full(r.size, -1.0 / h2))
            m2 = m & (nb_idx >= 0)
            rows.append(idx[m2])
            cols.append(nb_idx[m2])
            vals.append(np.full(int(m2.sum()), 1.0 / h2))
        A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nf, nf))
        comp, ncomp = ndimage.label(fl, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
        pins = np.array([idx.reshape(-1)[np.flatnonzero(comp.reshape(-1) == c)[0]] for c in range(1, ncomp + 1)],
                        np.int64)
        keep = np.ones(nf, bool)
        keep[pins] = False
        self._keep = keep
        self._lu = spla.splu(A[keep][:, keep].tocsc()) if keep.any() else None
        self._cells = cells
        self._nf = nf

    def solve(self, rhs: np.ndarray) -> np.ndarray:
        """p on every cell (0 outside fluid, 0 at the pinned cells) with A p = rhs."""
        b = rhs.reshape(-1)[self._cells]
        x = np.zeros(self._nf)
        if self._lu is not None:
            x[self._keep] = self._lu.solve(b[self._keep])
        p = np.zeros(self.nx * self.ny)
        p[self._cells] = x
        return p.reshape(self.ny, self.nx)

    def divergence(self, u, v):
        h = self.h
        r = np.zeros((self.ny, self.nx))
        r[:-1, :-1] = (u[:-1, 1:] - u[:-1, :-1]) / h + (v[1:, :-1] - v[:-1, :-1]) / h
        r[~self.fluid] = 0.0
        return r

    def subtract_gradient(self, u, v, p):
        h, fl = self.h, self.fluid
        u, v = u.copy(), v.copy()
        mu = np.zeros_like(fl)
        mu[:, 1:] = fl[:, 1:] & fl[:, :-1]
        mv = np.zeros_like(fl)
        mv[1:, :] = fl[1:, :] & fl[:-1, :]
        gu = np.zeros_like(u)
        gu[:, 1:] = (p[:, 1:] - p[:, :-1]) / h
        gv = np.zeros_like(v)
        gv[1:, :] = (p[1:, :] - p[:-1, :]) / h
        u[mu] = u[mu] - gu[mu]
        v[mv] = v[mv] - gv[mv]
        return u, v

    def project(self, u, v):
        return self.subtract_gradient(u, v, self.solve(self.divergence(u, v)))

    # ---- sampling ---------------------------------------------------------
    def foot(self, x, y) -> Foot:
        h = self.h
        xs, ys = x / h, y / h
        i = np.trunc(xs).astype(np.int64)
        j = np.trunc(ys).astype(np.int64)
        F = Foot()
        F.fi = xs - i
        F.fj = ys - j
        F.i = np.clip(i, 0, self.nx - 1)
        F.j = np.clip(j, 0, self.ny - 1)
        F.i1 = np.minimum(F.i + 1, self.nx - 1)
        F.j1 = np.minimum(F.j + 1, self.ny - 1)
        return F

    def foot_of(self, kind, x, y) -> Foot:
        h2 = self.h / 2.0
        if kind == "u":
            return self.foot(x, y - h2)
        if kind == "v":
            return self.foot(x - h2, y)
        return self.foot(x - h2, y - h2)

    @staticmethod
    def interp(f, F):
        v00, v10, v01, v11 = f[F.j, F.i], f[F.j, F.i1], f[F.j1, F.i], f[F.j1, F.i1]
        a = (1.0 - F.fi) * v00 + F.fi * v10
        b = (1.0 - F.fi) * v01 + F.fi * v11
        return (1.0 - F.fj) * a + F.fj * b

    def grad(self, f, F):
        v00, v10, v01, v11 = f[F.j, F.i], f[F.j, F.i1], f[F.j1, F.i], f[F.j1, F.i1]
        gx = ((1.0 - F.fj) * (v10 - v00) + F.fj * (v11 - v01)) / self.h
        gy = ((1.0 - F.fi) * (v01 - v00) + F.fi * (v11 - v10)) / self.h
        return gx, gy

    def scatter(self, acc, F, w):
        n = self.nx
        flat = acc.reshape(-1)
        for ii, jj, wt in ((F.i, F.j, (1.0 - F.fi) * (1.0 - F.fj)), (F.i1, F.j, F.fi * (1.0 - F.fj)),
                           (F.i, F.j1, (1.0 - F.fi) * F.fj), (F.i1, F.j1, F.fi * F.fj)):
            flat += np.bincount((ii + jj * n).reshape(-1), weights=(wt * w).reshape(-1), minlength=flat.size)

    def vel(self, u, v, x, y):
        return self.interp(u, self.foot_of("u", x, y)), self.interp(v, self.foot_of("v", x, y))

    def trace(self, u, v, x, y):
        """(stage positions, traced position) of the back-trace from (x, y)."""
        ht = -self.dt
        k1x, k1y = self.vel(u, v, x, y)
        if self.integrator == EULER:
            return [(x, y)], (x + ht * k1x, y + ht * k1y)
        if self.integrator == RK2:
            xm, ym = x + ht / 2.0 * k1x, y + ht / 2.0 * k1y
            k2x, k2y = self.vel(u, v, xm, ym)
            return [(x, y), (xm, ym)], (x + ht * k2x, y + ht * k2y)
        x2, y2 = x + k1x * ht * 1.0 / 2.0, y + k1y * ht * 1.0 / 2.0
        k2x, k2y = self.vel(u, v, x2, y2)
        x3, y3 = x + k2x * ht * 3.0 / 4.0, y + k2y * ht * 3.0 / 4.0
        k3x, k3y = self.vel(u, v, x3, y3)
        ox = x + (k1x * 2.0 + k2x * 3.0 + k3x * 4.0) * ht * 1.0 / 9.0
        oy = y + (k1y * 2.0 + k2y * 3.0 + k3y * 4.0) * ht * 1.0 / 9.0
        return [(x, y), (x2, y2), (x3, y3)], (ox, oy)

    # ---- forward ------------------------------------------------------------
    def advect(self, u, v, d):
        out = {}
        for kind, f in (("u", u), ("v", v), ("d", d)):
            x, y = self.pos[kind]
            _, (ox, oy) = self.trace(u, v, x, y)
            out[kind] = self.interp(f, self.foot_of(kind, ox, oy))
        out["u"][~self.u_open] = 0.0
        out["v"][~self.v_open] = 0.0
        return out["u"], out["v"], out["d"]

    def step(self, u, v, d):
        un, vn, dn = self.advect(u, v, d)
        un, vn = self.project(un, vn)
        return un, vn, dn

    def forward(self, u0, v0, d0, target, steps):
        """(loss, [states 0..steps])"""
        states = [(np.array(u0, np.float64), np.array(v0, np.float64), np.array(d0, np.float64))]
        for _ in range(steps):
            states.append(self.step(*states[-1]))
        loss = float(np.sqrt(np.sum((states[-1][2] - target) ** 2)))
        return loss, states

    # ---- adjoint ------------------------------------------------------------
    def advect_adjoint(self, u, v, d, lu, lv, ld):
        au, av, ad = np.zeros_like(u), np.zeros_like(v), np.zeros_like(d)
        ht = -self.dt
        fields = {"u": (u, au), "v": (v, av), "d": (d, ad)}
        lams = {"u": np.where(self.u_open, lu, 0.0), "v": np.where(self.v_open, lv, 0.0), "d": ld}
        for kind in ("u", "v", "d"):
            x, y = self.pos[kind]
            lam = lams[kind]
            stages, (ox, oy) = self.trace(u, v, x, y)
            f, acc = fields[kind]
            F = self.foot_of(kind, ox, oy)
            self.scatter(acc, F, lam)
            gx, gy = self.grad(f, F)
            lx, ly = lam * gx, lam * gy

            def stage(q, kxa, kya):
                sx, sy = stages[q]
                fu, fv = self.foot_of("u", sx, sy), self.foot_of("v", sx, sy)
                self.scatter(au, fu, kxa)
                self.scatter(av, fv, kya)
                ux, uy = self.grad(u, fu)
                vx, vy = self.grad(v, fv)
                return ux * kxa + vx * kya, uy * kxa + vy * kya

            if self.integrator == EULER:
                stage(0, ht * lx, ht * ly)
            elif self.integrator == RK2:
                px, py = stage(1, ht * lx, ht * ly)
                stage(0, ht / 2.0 * px, ht / 2.0 * py)
            else:
                k1x, k1y = 2.0 * ht / 9.0 * lx, 2.0 * ht / 9.0 * ly
                k2x, k2y = 3.0 * ht / 9.0 * lx, 3.0 * ht / 9.0 * ly
                px, py = stage(2, 4.0 * ht / 9.0 * lx, 4.0 * ht / 9.0 * ly)
                k2x, k2y = k2x + 3.0 * ht / 4.0 * px, k2y + 3.0 * ht / 4.0 * py
                px, py = stage(1, k2x, k2y)
                stage(0, k1x + ht / 2.0 * px, k1y + ht / 2.0 * py)
        return au, av, ad

    def backward(self, states, target, loss):
        """dL/d(u0, v0, d0) for L = ||d_T - target||."""
        lu = np.zeros_like(states[0][0])
        lv = np.zeros_like(states[0][1])
        ld = (states[-1][2] - target) / loss if loss > 0 else np.zeros_like(target)
        for n in range(len(states) - 2, -1, -1):
            lu = np.where(self.u_open, lu, 0.0)
            lv = np.where(self.v_open, lv, 0.0)
            lu, lv = self.project(lu, lv)
            lu, lv, ld = self.advect_adjoint(*states[n], lu, lv, ld)
        return lu, lv, ld
