"""ctypes front end of the oracle C API (oracle/fs_oracle.h); test infrastructure.

``OracleSim("restatement")`` drives the plain-C restatement,
``OracleSim("reference")`` the reference's own code (only where
``oracle/_ref/libfsref.so`` was built, i.e. where the reference checkout
exists).  Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline
leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

U_FRONT, V_FRONT, U_BACK, V_BACK, U_PREV, V_PREV, U_DIFF, V_DIFF = range(8)
STEP_SEMI_LAGRANGIAN, STEP_PIC, STEP_FLIP, STEP_PICFLIP = range(4)
(PH_CLASSIFY, PH_P2G, PH_SAVE_PREV, PH_GRAVITY, PH_DIRICHLET, PH_EXTEND, PH_PRESSURE, PH_SAVE_DIFF,
 PH_G2P_PICFLIP, PH_G2P_PIC, PH_G2P_FLIP, PH_ADVECT_SAFE, PH_ADVECT, PH_SL_VELOCITY, PH_SL_PARTICLES,
 PH_SWAP) = range(16)
LIQUID, AIR, SOLID = 0, 1, 2

_LIBS: dict[str, C.CDLL] = {}


def reference_available() -> bool:
    return os.path.exists(build_oracle.REFERENCE_SO) or build_oracle.build_reference() is not None


def _lib(kind: str) -> C.CDLL:
    if kind in _LIBS:
        return _LIBS[kind]
    if kind == "restatement":
        path = build_oracle.build_restatement()
    elif kind == "reference":
        path = build_oracle.build_reference()
        if path is None:
            raise RuntimeError("the reference build is not available on this machine")
    else:
        raise ValueError(kind)
    lib = C.CDLL(path)
    vp, i, f, d, i64 = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_int64
    sig = {
        "fso_create": (vp, [i, i, f, f, f, f]),
        "fso_destroy": (None, [vp]),
        "fso_set_cg": (None, [vp, d, i]),
        "fso_set_gravity": (None, [vp, f, f]),
        "fso_set_cg_precision": (None, [vp, i]),
        "fso_set_extension_iterations": (None, [vp, i]),
        "fso_set_solid_mask": (None, [vp, vp]),
        "fso_set_use_stock": (None, [vp, i]),
        "fso_set_pic_ratio": (None, [vp, f]),
        "fso_set_particles": (None, [vp, vp, i64]),
        "fso_num_particles": (i64, [vp]),
        "fso_get_particles": (None, [vp, vp]),
        "fso_get_grid": (None, [vp, i, vp]),
        "fso_set_grid": (None, [vp, i, vp]),
        "fso_get_labels": (None, [vp, vp]),
        "fso_set_labels": (None, [vp, vp]),
        "fso_get_fluid_indices": (None, [vp, vp]),
        "fso_get_particle_counts": (None, [vp, vp]),
        "fso_get_pressure": (None, [vp, vp]),
        "fso_get_cg_stats": (None, [vp, C.POINTER(i), C.POINTER(d), C.POINTER(i)]),
        "fso_step": (i, [vp, i, f]),
        "fso_phase": (i, [vp, i, f]),
        "fso_add_source": (None, [vp, f, f, f, f, f, f, f, f, f, i]),
        "fso_update": (None, [vp, f]),
        "fso_clear_sources": (None, [vp]),
        "fso_render": (None, [vp, i, vp, i, i, vp, vp]),
        "fso_get_level_set": (None, [vp, vp]),
        "fso_set_level_set": (None, [vp, vp]),
        "fso_advect_level_set": (None, [vp, f]),
        "fso_classify_level_set": (None, [vp]),
        "fso_canvas_bytes": (None, [vp, i64, vp]),
        "fso_metaball_weight": (f, [i, i]),
        "fso_kind": (C.c_char_p, []),
        "fso_poisson_solve": (i, [i, i, f, f, vp, vp, i, d, i, d, i, vp, C.POINTER(i), C.POINTER(i),
                                  C.POINTER(d)]),
    }
    optional = {"fso_poisson_solve"}   # restatement only: the reference has no standalone solve
    for name, (res, args) in sig.items():
        if name in optional and not hasattr(lib, name):
            continue
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[kind] = lib
    return lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


RENDER_CLEAR, RENDER_CELLS, RENDER_VELOCITIES, RENDER_PARTICLES, RENDER_METABALLS, RENDER_LEVEL_SET = range(6)


def canvas_bytes(canvas: np.ndarray, kind: str = "restatement") -> np.ndarray:
    """Renderer::writeCanvasToPpm's byte conversion of a (h, w, 3) float32 canvas."""
    lib = _lib(kind)
    c = np.ascontiguousarray(canvas, dtype=np.float32)
    out = np.empty(c.shape, np.uint8)
    lib.fso_canvas_bytes(_ptr(c), c.shape[0] * c.shape[1], _ptr(out))
    return out


def metaball_weight(i: int, j: int, kind: str = "restatement") -> float:
    return float(_lib(kind).fso_metaball_weight(i, j))


def poisson_solve(labels: np.ndarray, rhs: np.ndarray, length_x: float, length_y: float, method: int, tol: float,
                  maxit: int, inner_tol: float = 1e-3, inner_precision: int = 0) -> tuple[np.ndarray, dict]:
    """The restatement of the GPU's pressure-projection solver (fs_poisson_*)."""
    lib = _lib("restatement")
    ny, nx = labels.shape
    lab = np.ascontiguousarray(labels, dtype=np.uint8)
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    x = np.empty((ny, nx), np.float64)
    outer, inner, res = C.c_int(), C.c_int(), C.c_double()
    nf = lib.fso_poisson_solve(nx, ny, length_x, length_y, _ptr(lab), _ptr(b), method, tol, maxit, inner_tol,
                               inner_precision, _ptr(x), C.byref(outer), C.byref(inner), C.byref(res))
    return x, {"n_fluid": nf, "outer_iterations": outer.value, "inner_iterations": inner.value,
               "residual": res.value}


class OracleSim:
    """One simulation (FluidDomain + FluidSolver) in an oracle implementation."""

    def __init__(self, kind: str, size_x: int, size_y: int, length_x: float, length_y: float,
                 density: float, pic_ratio: float):
        self.kind = kind
        self.lib = _lib(kind)
        self.nx, self.ny = size_x, size_y
        self.h = self.lib.fso_create(size_x, size_y, length_x, length_y, density, pic_ratio)

    def close(self) -> None:
        if self.h:
            self.lib.fso_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # settings
    def set_cg(self, tol: float, maxit: int) -> None:
        self.lib.fso_set_cg(self.h, float(tol), int(maxit))

    def set_cg_precision(self, precision: int) -> None:
        """0: float dot products (the reference's precision); 1: double; 2: double-single."""
        self.lib.fso_set_cg_precision(self.h, int(precision))

    def set_gravity(self, gx: float, gy: float) -> None:
        self.lib.fso_set_gravity(self.h, gx, gy)

    def set_extension_iterations(self, n: int) -> None:
        self.lib.fso_set_extension_iterations(self.h, n)

    def set_solid_mask(self, mask: np.ndarray | None) -> None:
        if mask is None:
            self.lib.fso_set_solid_mask(self.h, None)
        else:
            m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
            assert m.size == self.nx * self.ny
            self.lib.fso_set_solid_mask(self.h, _ptr(m))

    def set_use_stock(self, on: bool) -> None:
        self.lib.fso_set_use_stock(self.h, int(on))

    def set_pic_ratio(self, r: float) -> None:
        self.lib.fso_set_pic_ratio(self.h, r)

    # particles
    def set_particles(self, xyuv: np.ndarray) -> None:
        a = np.ascontiguousarray(xyuv, dtype=np.float32).reshape(-1, 4)
        self.lib.fso_set_particles(self.h, _ptr(a), a.shape[0])

    def particles(self) -> np.ndarray:
        n = self.lib.fso_num_particles(self.h)
        out = np.empty((n, 4), np.float32)
        if n:
            self.lib.fso_get_particles(self.h, _ptr(out))
        return out

    # grids
    def grid(self, which: int) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float32)
        self.lib.fso_get_grid(self.h, which, _ptr(out))
        return out

    def set_grid(self, which: int, g: np.ndarray) -> None:
        a = np.ascontiguousarray(g, dtype=np.float32).reshape(self.ny, self.nx)
        self.lib.fso_set_grid(self.h, which, _ptr(a))

    def labels(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.uint8)
        self.lib.fso_get_labels(self.h, _ptr(out))
        return out

    def set_labels(self, lab: np.ndarray) -> None:
        a = np.ascontiguousarray(lab, dtype=np.uint8).reshape(self.ny, self.nx)
        self.lib.fso_set_labels(self.h, _ptr(a))

    def fluid_indices(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.int32)
        self.lib.fso_get_fluid_indices(self.h, _ptr(out))
        return out

    def particle_counts(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.uint8)
        self.lib.fso_get_particle_counts(self.h, _ptr(out))
        return out

    def pressure(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float32)
        self.lib.fso_get_pressure(self.h, _ptr(out))
        return out

    def cg_stats(self) -> tuple[int, float, int]:
        it, err, nf = C.c_int(), C.c_double(), C.c_int()
        self.lib.fso_get_cg_stats(self.h, C.byref(it), C.byref(err), C.byref(nf))
        return it.value, err.value, nf.value

    # stepping
    def step(self, method: int, dt: float) -> int:
        return self.lib.fso_step(self.h, method, dt)

    def phase(self, ph: int, dt: float = 0.0) -> int:
        return self.lib.fso_phase(self.h, ph, dt)

    def add_source(self, x_min, x_max, y_min, y_max, dx, dy, vx, vy, time_step, max_spawns) -> None:
        self.lib.fso_add_source(self.h, x_min, x_max, y_min, y_max, dx, dy, vx, vy, time_step, max_spawns)

    def update(self, dt: float) -> None:
        self.lib.fso_update(self.h, dt)

    def clear_sources(self) -> None:
        self.lib.fso_clear_sources(self.h)

    def level_set(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float32)
        self.lib.fso_get_level_set(self.h, _ptr(out))
        return out

    def set_level_set(self, ls: np.ndarray) -> None:
        a = np.ascontiguousarray(ls, dtype=np.float32).reshape(self.ny, self.nx)
        self.lib.fso_set_level_set(self.h, _ptr(a))

    def advect_level_set(self, dt: float) -> None:
        self.lib.fso_advect_level_set(self.h, dt)

    def classify_level_set(self) -> None:
        self.lib.fso_classify_level_set(self.h)

    def render(self, what: int, area, canvas: np.ndarray, colors: np.ndarray) -> None:
        """Renderer (Renderer.cpp) onto canvas (h, w, 3) float32 and colors (6,) float32, in place."""
        a = np.ascontiguousarray(area, dtype=np.float32)
        assert canvas.dtype == np.float32 and canvas.flags.c_contiguous and colors.dtype == np.float32
        h, w = canvas.shape[:2]
        self.lib.fso_render(self.h, what, _ptr(a), w, h, _ptr(canvas), _ptr(colors))

    def state(self) -> dict[str, np.ndarray]:
        """Every observable array, for comparisons."""
        s = {name: self.grid(w) for name, w in (("u_front", U_FRONT), ("v_front", V_FRONT),
                                                 ("u_back", U_BACK), ("v_back", V_BACK),
                                                 ("u_prev", U_PREV), ("v_prev", V_PREV),
                                                 ("u_diff", U_DIFF), ("v_diff", V_DIFF))}
        s["labels"] = self.labels()
        s["fluid_indices"] = self.fluid_indices()
        s["particle_counts"] = self.particle_counts()
        s["pressure"] = self.pressure()
        s["particles"] = self.particles()
        return s
