"""fluid_simulation_gb300: GB300 (sm_103a) implementation of Fluid_Simulation's
per-step PIC/FLIP + MAC-grid + pressure-projection path.

The product is the CUDA library ``_build/libfsgpu.so`` behind the C ABI of
``include/fsgpu.h`` and the C++ drop-in classes in ``dropin/``.  This module is
the Python front end of that C ABI (ctypes), used by the tests and bench.py.
There is no CPU fallback: without the built library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libfsgpu.so")

# Constants of include/fsgpu.h
FS_OK = 0
STATUS_NAMES = {0: "FS_OK", 1: "FS_ERR_INVALID_ARGUMENT", 2: "FS_ERR_VALIDATE", 3: "FS_ERR_CUDA",
                4: "FS_ERR_TIMEOUT", 5: "FS_ERR_TOO_LARGE", 6: "FS_ERR_INTERNAL", 7: "FS_ERR_OUT_OF_MEMORY"}
FS_WARN_PARTICLE_OUTSIDE = 1
FS_WARN_CG_NOT_CONVERGED = 2
U_FRONT, V_FRONT, U_BACK, V_BACK, U_PREV, V_PREV, U_DIFF, V_DIFF = range(8)
STEP_SEMI_LAGRANGIAN, STEP_PIC, STEP_FLIP, STEP_PICFLIP = range(4)
(PH_CLASSIFY, PH_P2G, PH_SAVE_PREV, PH_GRAVITY, PH_DIRICHLET, PH_EXTEND, PH_PRESSURE, PH_SAVE_DIFF,
 PH_G2P_PICFLIP, PH_G2P_PIC, PH_G2P_FLIP, PH_ADVECT_SAFE, PH_ADVECT, PH_SL_VELOCITY, PH_SL_PARTICLES,
 PH_SWAP) = range(16)
CG_FLOAT, CG_DOUBLE, CG_DS = 0, 1, 2
POISSON_FP32, POISSON_FP64, POISSON_MIXED, POISSON_MGPCG, POISSON_MIXED_MG = 0, 1, 2, 3, 4
SOLVER_JACOBI_PCG, SOLVER_MGPCG = 0, 1
INTEGRATOR_EULER, INTEGRATOR_RK2, INTEGRATOR_RK3 = 0, 1, 2
SMOKE_FP32, SMOKE_FP64, SMOKE_FP32_TRACE64 = 0, 1, 2
RENDER_CLEAR, RENDER_CELLS, RENDER_VELOCITIES, RENDER_PARTICLES, RENDER_METABALLS, RENDER_LEVEL_SET = range(6)
TIMED_PHASES = ("classify", "p2g", "forces", "assembly", "cg", "project", "g2p")


class FsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, code), msg))
        self.code = code


class fs_config(C.Structure):
    _fields_ = [("size_x", C.c_int), ("size_y", C.c_int), ("length_x", C.c_float), ("length_y", C.c_float),
                ("density", C.c_float), ("pic_ratio", C.c_float), ("gravity_x", C.c_float),
                ("gravity_y", C.c_float), ("cg_max_iterations", C.c_int), ("cg_tolerance", C.c_double),
                ("extension_iterations", C.c_int), ("device", C.c_int), ("cg_precision", C.c_int),
                ("reserved", C.c_int * 7)]


class fs_poisson_stats(C.Structure):
    _fields_ = [("outer_iterations", C.c_int), ("inner_iterations", C.c_int), ("residual", C.c_double),
                ("ms", C.c_float)]


class fs_smoke_config(C.Structure):
    _fields_ = [("size_x", C.c_int), ("size_y", C.c_int), ("length_x", C.c_float), ("length_y", C.c_float),
                ("dt", C.c_float), ("integrator", C.c_int), ("precision", C.c_int), ("projection_method", C.c_int),
                ("cg_tolerance", C.c_double), ("cg_max_iterations", C.c_int), ("inner_tolerance", C.c_double),
                ("checkpoint_every", C.c_int), ("device", C.c_int), ("reserved", C.c_int * 8)]


class fs_step_stats(C.Structure):
    _fields_ = [("cg_iterations", C.c_int), ("n_fluid", C.c_int), ("cg_residual", C.c_double),
                ("warnings", C.c_uint), ("ms_total", C.c_float), ("ms_phase", C.c_float * 7)]


# Every function include/fsgpu.h declares, with its ctypes signature.
_vp, _i, _f, _d, _i64 = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_int64
SIGNATURES = {
    "fs_config_init": (None, [C.POINTER(fs_config), _i, _i]),
    "fs_create": (_i, [C.POINTER(fs_config), C.POINTER(_vp)]),
    "fs_destroy": (_i, [_vp]),
    "fs_last_error": (C.c_char_p, [_vp]),
    "fs_set_pic_ratio": (_i, [_vp, _f]),
    "fs_set_gravity": (_i, [_vp, _f, _f]),
    "fs_set_cg": (_i, [_vp, _d, _i]),
    "fs_set_cg_precision": (_i, [_vp, _i]),
    "fs_set_extension_iterations": (_i, [_vp, _i]),
    "fs_set_pressure_solver": (_i, [_vp, _i]),
    "fs_set_solid_mask": (_i, [_vp, _vp]),
    "fs_set_particles": (_i, [_vp, _vp, _i64]),
    "fs_set_particles_device": (_i, [_vp, _vp, _i64]),
    "fs_add_particles": (_i, [_vp, _vp, _i64]),
    "fs_num_particles": (_i, [_vp, C.POINTER(_i64)]),
    "fs_get_particles": (_i, [_vp, _vp, _i64]),
    "fs_get_particles_device": (_i, [_vp, _vp, _i64]),
    "fs_get_grid": (_i, [_vp, _i, _vp]),
    "fs_set_grid": (_i, [_vp, _i, _vp]),
    "fs_get_labels": (_i, [_vp, _vp]),
    "fs_set_labels": (_i, [_vp, _vp]),
    "fs_get_fluid_indices": (_i, [_vp, _vp]),
    "fs_get_particle_counts": (_i, [_vp, _vp]),
    "fs_get_pressure": (_i, [_vp, _vp]),
    "fs_step": (_i, [_vp, _i, _f]),
    "fs_phase": (_i, [_vp, _i, _f]),
    "fs_add_fluid_source": (_i, [_vp, _f, _f, _f, _f, _f, _f, _f, _f, _f, _i]),
    "fs_update": (_i, [_vp, _f]),
    "fs_clear_fluid_sources": (_i, [_vp]),
    "fs_num_fluid_sources": (_i, [_vp, C.POINTER(_i)]),
    "fs_set_fluid_source_state": (_i, [_vp, _i, _f, _i]),
    "fs_reset_particles": (_i, [_vp]),
    "fs_snapshot": (_i, [_vp, C.POINTER(_vp)]),
    "fs_restore": (_i, [_vp, _vp]),
    "fs_snapshot_destroy": (_i, [_vp]),
    "fs_debug_set_cg_barrier_fault": (_i, [_vp, _i, _d]),
    "fs_canvas_create": (_i, [_i, _i, _i, C.POINTER(_vp)]),
    "fs_canvas_destroy": (_i, [_vp]),
    "fs_canvas_last_error": (C.c_char_p, [_vp]),
    "fs_canvas_set_pixels": (_i, [_vp, _vp]),
    "fs_canvas_get_pixels": (_i, [_vp, _vp]),
    "fs_canvas_set_colors": (_i, [_vp, _vp, _vp]),
    "fs_canvas_get_colors": (_i, [_vp, _vp, _vp]),
    "fs_canvas_get_bytes": (_i, [_vp, _vp]),
    "fs_canvas_write_ppm": (_i, [_vp, C.c_char_p]),
    "fs_canvas_kernel_launches": (_i64, [_vp]),
    "fs_render": (_i, [_vp, _vp, _i, _vp]),
    "fs_get_level_set": (_i, [_vp, _vp]),
    "fs_set_level_set": (_i, [_vp, _vp]),
    "fs_advect_level_set": (_i, [_vp, _f]),
    "fs_classify_level_set": (_i, [_vp]),
    "fs_synchronize": (_i, [_vp]),
    "fs_get_stats": (_i, [_vp, C.POINTER(fs_step_stats)]),
    "fs_set_timing": (_i, [_vp, _i]),
    "fs_set_graphs": (_i, [_vp, _i]),
    "fs_get_stream": (_vp, [_vp]),
    "fs_set_stream": (_i, [_vp, _vp]),
    "fs_kernel_launches": (_i64, [_vp]),
    "fs_poisson_create": (_i, [_i, _i, _f, _f, _i, C.POINTER(_vp)]),
    "fs_poisson_destroy": (_i, [_vp]),
    "fs_poisson_set_problem": (_i, [_vp, _vp, _vp]),
    "fs_poisson_solve": (_i, [_vp, _i, _d, _i, _d, _i, C.POINTER(fs_poisson_stats)]),
    "fs_poisson_get_solution": (_i, [_vp, _vp]),
    "fs_poisson_kernel_launches": (_i64, [_vp]),
    "fs_batch_create": (_i, [_i, C.POINTER(fs_config), C.POINTER(_vp)]),
    "fs_batch_destroy": (_i, [_vp]),
    "fs_batch_last_error": (C.c_char_p, [_vp]),
    "fs_batch_size": (_i, [_vp]),
    "fs_batch_set_particles": (_i, [_vp, _i, _vp, _i64]),
    "fs_batch_num_particles": (_i, [_vp, _i, C.POINTER(_i64)]),
    "fs_batch_get_particles": (_i, [_vp, _i, _vp, _i64]),
    "fs_batch_set_solid_mask": (_i, [_vp, _i, _vp]),
    "fs_batch_get_grid": (_i, [_vp, _i, _i, _vp]),
    "fs_batch_get_labels": (_i, [_vp, _i, _vp]),
    "fs_batch_get_pressure": (_i, [_vp, _i, _vp]),
    "fs_batch_step": (_i, [_vp, _i, _f]),
    "fs_batch_synchronize": (_i, [_vp]),
    "fs_batch_get_stats": (_i, [_vp, _i, C.POINTER(fs_step_stats)]),
    "fs_batch_tune": (_i, [_vp, _i, _f, _i, _vp]),
    "fs_batch_set_tuning": (_i, [_vp, _i]),
    "fs_batch_get_tuning": (_i, [_vp]),
    "fs_batch_set_graphs": (_i, [_vp, _i]),
    "fs_batch_get_stream": (_vp, [_vp]),
    "fs_batch_kernel_launches": (_i64, [_vp]),
    "fs_smoke_config_init": (None, [C.POINTER(fs_smoke_config), _i, _i]),
    "fs_smoke_create": (_i, [C.POINTER(fs_smoke_config), C.POINTER(_vp)]),
    "fs_smoke_destroy": (_i, [_vp]),
    "fs_smoke_last_error": (C.c_char_p, [_vp]),
    "fs_smoke_set_solid_mask": (_i, [_vp, _vp]),
    "fs_smoke_set_state": (_i, [_vp, _vp, _vp, _vp]),
    "fs_smoke_set_target": (_i, [_vp, _vp]),
    "fs_smoke_forward": (_i, [_vp, _i, C.POINTER(_d)]),
    "fs_smoke_get_state": (_i, [_vp, _vp, _vp, _vp]),
    "fs_smoke_backward": (_i, [_vp, _vp, _vp, _vp]),
    "fs_smoke_kernel_launches": (_i64, [_vp]),
    "fs_pressure_solve_noalloc": (_i, [_i, _i, _f, _f, _vp, _vp, _vp, _d, _i, _i, _vp, C.POINTER(_i),
                                       C.POINTER(_d), _vp]),
}

_LIB: C.CDLL | None = None


def library_path() -> str:
    return LIB_PATH


def load_library(path: str | None = None) -> C.CDLL:
    """Loads libfsgpu.so (built by fluid_simulation_gb300/build.py); raises if absent."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libfsgpu.so is not built (%s); run fluid_simulation_gb300/build.py" % p)
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class FluidSim:
    """One FluidDomain + FluidSolver pair on the GPU (a C-ABI handle)."""

    def __init__(self, size_x: int, size_y: int, length_x: float, length_y: float, density: float,
                 pic_ratio: float, device: int = 0, cg_tolerance: float | None = None,
                 cg_max_iterations: int | None = None, gravity: tuple[float, float] | None = None,
                 extension_iterations: int | None = None):
        self.lib = load_library()
        cfg = fs_config()
        self.lib.fs_config_init(C.byref(cfg), size_x, size_y)
        cfg.length_x, cfg.length_y = length_x, length_y
        cfg.density, cfg.pic_ratio, cfg.device = density, pic_ratio, device
        if cg_tolerance is not None:
            cfg.cg_tolerance = cg_tolerance
        if cg_max_iterations is not None:
            cfg.cg_max_iterations = cg_max_iterations
        if gravity is not None:
            cfg.gravity_x, cfg.gravity_y = gravity
        if extension_iterations is not None:
            cfg.extension_iterations = extension_iterations
        h = C.c_void_p()
        rc = self.lib.fs_create(C.byref(cfg), C.byref(h))
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_last_error(None).decode())
        self.h = h
        self.nx, self.ny = size_x, size_y

    @classmethod
    def from_scene(cls, sc, device: int = 0) -> "FluidSim":
        sim = cls(sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio, device,
                  cg_tolerance=sc.cg_tolerance, cg_max_iterations=sc.cg_max_iterations, gravity=sc.gravity)
        if sc.solid is not None:
            sim.set_solid_mask(sc.solid)
        sim.set_particles(sc.particles)
        return sim

    def _check(self, rc: int) -> None:
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_last_error(self.h).decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # settings
    def set_cg(self, tol: float, maxit: int) -> None:
        self._check(self.lib.fs_set_cg(self.h, float(tol), int(maxit)))

    def set_cg_precision(self, precision: int) -> None:
        """CG_FLOAT (0, the reference's precision), CG_DOUBLE (1) or CG_DS (2, double-single)."""
        self._check(self.lib.fs_set_cg_precision(self.h, int(precision)))

    def set_pressure_solver(self, solver: int) -> None:
        """SOLVER_JACOBI_PCG (the reference's, bit-exact) or SOLVER_MGPCG (multigrid-preconditioned)."""
        self._check(self.lib.fs_set_pressure_solver(self.h, int(solver)))

    def set_gravity(self, gx: float, gy: float) -> None:
        self._check(self.lib.fs_set_gravity(self.h, gx, gy))

    def set_extension_iterations(self, n: int) -> None:
        self._check(self.lib.fs_set_extension_iterations(self.h, n))

    def set_pic_ratio(self, r: float) -> None:
        self._check(self.lib.fs_set_pic_ratio(self.h, r))

    def set_solid_mask(self, mask: np.ndarray | None) -> None:
        if mask is None:
            self._check(self.lib.fs_set_solid_mask(self.h, None))
        else:
            m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(-1)
            assert m.size == self.nx * self.ny
            self._check(self.lib.fs_set_solid_mask(self.h, _ptr(m)))

    def set_timing(self, on: bool) -> None:
        self._check(self.lib.fs_set_timing(self.h, int(on)))

    def set_graphs(self, on: bool) -> None:
        self._check(self.lib.fs_set_graphs(self.h, int(on)))

    def set_stream(self, stream: int) -> None:
        """Queue the handle's work on a caller's CUDA stream (a cudaStream_t as an int)."""
        self._check(self.lib.fs_set_stream(self.h, C.c_void_p(stream)))

    # particles
    def set_particles(self, xyuv: np.ndarray) -> None:
        a = np.ascontiguousarray(xyuv, dtype=np.float32).reshape(-1, 4)
        self._check(self.lib.fs_set_particles(self.h, _ptr(a), a.shape[0]))

    def add_particles(self, xyuv: np.ndarray) -> None:
        a = np.ascontiguousarray(xyuv, dtype=np.float32).reshape(-1, 4)
        self._check(self.lib.fs_add_particles(self.h, _ptr(a), a.shape[0]))

    def num_particles(self) -> int:
        n = C.c_int64()
        self._check(self.lib.fs_num_particles(self.h, C.byref(n)))
        return n.value

    def particles(self) -> np.ndarray:
        n = self.num_particles()
        out = np.empty((n, 4), np.float32)
        self._check(self.lib.fs_get_particles(self.h, _ptr(out), n))
        return out

    # grids
    def grid(self, which: int) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float32)
        self._check(self.lib.fs_get_grid(self.h, which, _ptr(out)))
        return out

    def set_grid(self, which: int, g: np.ndarray) -> None:
        a = np.ascontiguousarray(g, dtype=np.float32).reshape(self.ny, self.nx)
        self._check(self.lib.fs_set_grid(self.h, which, _ptr(a)))

    def labels(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.uint8)
        self._check(self.lib.fs_get_labels(self.h, _ptr(out)))
        return out

    def set_labels(self, lab: np.ndarray) -> None:
        a = np.ascontiguousarray(lab, dtype=np.uint8).reshape(self.ny, self.nx)
        self._check(self.lib.fs_set_labels(self.h, _ptr(a)))

    def fluid_indices(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.int32)
        self._check(self.lib.fs_get_fluid_indices(self.h, _ptr(out)))
        return out

    def particle_counts(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.uint8)
        self._check(self.lib.fs_get_particle_counts(self.h, _ptr(out)))
        return out

    def pressure(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float32)
        self._check(self.lib.fs_get_pressure(self.h, _ptr(out)))
        return out

    # fluid sources (FluidDomain::addFluidSource / update / clearFluidSources)
    def add_fluid_source(self, x_min, x_max, y_min, y_max, delta_x, delta_y, x_velocity, y_velocity, time_step,
                         max_spawns) -> None:
        self._check(self.lib.fs_add_fluid_source(self.h, x_min, x_max, y_min, y_max, delta_x, delta_y, x_velocity,
                                                 y_velocity, time_step, int(max_spawns)))

    def update(self, dt: float) -> None:
        self._check(self.lib.fs_update(self.h, dt))

    def clear_fluid_sources(self) -> None:
        self._check(self.lib.fs_clear_fluid_sources(self.h))

    def reset_particles(self) -> None:
        self._check(self.lib.fs_reset_particles(self.h))

    # level set (FluidDomain::levelSet / advectLevelSet / classifyCells(LevelSet&))
    def level_set(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float32)
        self._check(self.lib.fs_get_level_set(self.h, _ptr(out)))
        return out

    def set_level_set(self, ls: np.ndarray) -> None:
        a = np.ascontiguousarray(ls, dtype=np.float32).reshape(self.ny, self.nx)
        self._check(self.lib.fs_set_level_set(self.h, _ptr(a)))

    def advect_level_set(self, dt: float) -> None:
        self._check(self.lib.fs_advect_level_set(self.h, dt))

    def classify_level_set(self) -> None:
        self._check(self.lib.fs_classify_level_set(self.h))

    # rendering (Renderer.cpp onto a device canvas)
    def render(self, canvas: "Canvas", what: int, area) -> None:
        a = np.ascontiguousarray(area, dtype=np.float32)
        self._check(self.lib.fs_render(self.h, canvas.p, what, _ptr(a)))

    # snapshots
    def snapshot(self) -> "Snapshot":
        p = C.c_void_p()
        self._check(self.lib.fs_snapshot(self.h, C.byref(p)))
        return Snapshot(self.lib, p)

    def restore(self, snap: "Snapshot") -> None:
        self._check(self.lib.fs_restore(self.h, snap.p))

    # stepping
    def step(self, method: int, dt: float) -> None:
        self._check(self.lib.fs_step(self.h, method, dt))

    def phase(self, ph: int, dt: float = 0.0) -> None:
        self._check(self.lib.fs_phase(self.h, ph, dt))

    def synchronize(self) -> None:
        self._check(self.lib.fs_synchronize(self.h))

    def stats(self) -> dict:
        s = fs_step_stats()
        self._check(self.lib.fs_get_stats(self.h, C.byref(s)))
        return {"cg_iterations": s.cg_iterations, "n_fluid": s.n_fluid, "cg_residual": s.cg_residual,
                "warnings": s.warnings, "ms_total": s.ms_total,
                "ms_phase": dict(zip(TIMED_PHASES, list(s.ms_phase)))}

    def stream(self) -> int:
        return self.lib.fs_get_stream(self.h) or 0

    def kernel_launches(self) -> int:
        return self.lib.fs_kernel_launches(self.h)

    def state(self) -> dict[str, np.ndarray]:
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


class Canvas:
    """A device canvas of width x height RGB floats (fs_canvas_*)."""

    def __init__(self, width: int, height: int, device: int = 0):
        self.lib = load_library()
        p = C.c_void_p()
        rc = self.lib.fs_canvas_create(width, height, device, C.byref(p))
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_canvas_last_error(None).decode())
        self.p, self.width, self.height = p, width, height

    def _check(self, rc: int) -> None:
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_canvas_last_error(self.p).decode())

    def close(self) -> None:
        if getattr(self, "p", None):
            self.lib.fs_canvas_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_pixels(self, rgb: np.ndarray) -> None:
        a = np.ascontiguousarray(rgb, dtype=np.float32).reshape(self.height, self.width, 3)
        self._check(self.lib.fs_canvas_set_pixels(self.p, _ptr(a)))

    def pixels(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), np.float32)
        self._check(self.lib.fs_canvas_get_pixels(self.p, _ptr(out)))
        return out

    def set_colors(self, line, fill) -> None:
        l_, f_ = np.asarray(line, np.float32), np.asarray(fill, np.float32)
        self._check(self.lib.fs_canvas_set_colors(self.p, _ptr(l_), _ptr(f_)))

    def colors(self) -> np.ndarray:
        l_, f_ = np.empty(3, np.float32), np.empty(3, np.float32)
        self._check(self.lib.fs_canvas_get_colors(self.p, _ptr(l_), _ptr(f_)))
        return np.concatenate([l_, f_])

    def bytes(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 3), np.uint8)
        self._check(self.lib.fs_canvas_get_bytes(self.p, _ptr(out)))
        return out

    def write_ppm(self, path: str) -> None:
        self._check(self.lib.fs_canvas_write_ppm(self.p, path.encode()))


class Snapshot:
    """A device copy of a FluidSim's state (fs_snapshot); freed with the object."""

    def __init__(self, lib: C.CDLL, p: C.c_void_p):
        self.lib, self.p = lib, p

    def close(self) -> None:
        if getattr(self, "p", None):
            self.lib.fs_snapshot_destroy(self.p)
            self.p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def scene_config(lib: C.CDLL, sc, device: int = 0) -> fs_config:
    """The fs_config of a Scene (fluid_simulation_gb300.scenes)."""
    cfg = fs_config()
    lib.fs_config_init(C.byref(cfg), sc.size_x, sc.size_y)
    cfg.length_x, cfg.length_y = sc.length_x, sc.length_y
    cfg.density, cfg.pic_ratio, cfg.device = sc.density, sc.pic_ratio, device
    cfg.cg_tolerance, cfg.cg_max_iterations = sc.cg_tolerance, sc.cg_max_iterations
    cfg.gravity_x, cfg.gravity_y = sc.gravity
    return cfg


class FluidBatch:
    """Many independent FluidDomain + FluidSolver pairs stepped together (fs_batch_*)."""

    def __init__(self, configs: list, device: int = 0):
        self.lib = load_library()
        n = len(configs)
        arr = (fs_config * n)(*configs)
        h = C.c_void_p()
        rc = self.lib.fs_batch_create(n, arr, C.byref(h))
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_batch_last_error(None).decode())
        self.h = h
        self.shapes = [(c.size_y, c.size_x) for c in configs]

    @classmethod
    def from_scenes(cls, scenes: list, device: int = 0) -> "FluidBatch":
        lib = load_library()
        b = cls([scene_config(lib, sc, device) for sc in scenes], device)
        for s, sc in enumerate(scenes):
            if sc.solid is not None:
                b.set_solid_mask(s, sc.solid)
            b.set_particles(s, sc.particles)
        return b

    def __len__(self) -> int:
        return len(self.shapes)

    def _check(self, rc: int) -> None:
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_batch_last_error(self.h).decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, sim: int, xyuv: np.ndarray) -> None:
        a = np.ascontiguousarray(xyuv, dtype=np.float32).reshape(-1, 4)
        self._check(self.lib.fs_batch_set_particles(self.h, sim, _ptr(a), a.shape[0]))

    def num_particles(self, sim: int) -> int:
        n = C.c_int64()
        self._check(self.lib.fs_batch_num_particles(self.h, sim, C.byref(n)))
        return n.value

    def particles(self, sim: int) -> np.ndarray:
        n = self.num_particles(sim)
        out = np.empty((n, 4), np.float32)
        self._check(self.lib.fs_batch_get_particles(self.h, sim, _ptr(out), n))
        return out

    def set_solid_mask(self, sim: int, mask: np.ndarray | None) -> None:
        if mask is None:
            self._check(self.lib.fs_batch_set_solid_mask(self.h, sim, None))
        else:
            m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(self.shapes[sim])
            self._check(self.lib.fs_batch_set_solid_mask(self.h, sim, _ptr(m)))

    def grid(self, sim: int, which: int) -> np.ndarray:
        out = np.empty(self.shapes[sim], np.float32)
        self._check(self.lib.fs_batch_get_grid(self.h, sim, which, _ptr(out)))
        return out

    def labels(self, sim: int) -> np.ndarray:
        out = np.empty(self.shapes[sim], np.uint8)
        self._check(self.lib.fs_batch_get_labels(self.h, sim, _ptr(out)))
        return out

    def pressure(self, sim: int) -> np.ndarray:
        out = np.empty(self.shapes[sim], np.float32)
        self._check(self.lib.fs_batch_get_pressure(self.h, sim, _ptr(out)))
        return out

    def step(self, method: int, dt: float) -> None:
        self._check(self.lib.fs_batch_step(self.h, method, dt))

    def synchronize(self) -> None:
        self._check(self.lib.fs_batch_synchronize(self.h))

    def stats(self, sim: int) -> dict:
        s = fs_step_stats()
        self._check(self.lib.fs_batch_get_stats(self.h, sim, C.byref(s)))
        return {"cg_iterations": s.cg_iterations, "n_fluid": s.n_fluid, "cg_residual": s.cg_residual,
                "warnings": s.warnings}

    def tune(self, method: int, dt: float, steps: int = 2) -> dict:
        ms = (C.c_float * 4)()
        self._check(self.lib.fs_batch_tune(self.h, method, dt, steps, ms))
        return {"chunks_per_cta": self.lib.fs_batch_get_tuning(self.h),
                "ms_per_step": dict(zip((1, 2, 4, 8), list(ms)))}

    def set_tuning(self, chunks_per_cta: int) -> None:
        self._check(self.lib.fs_batch_set_tuning(self.h, chunks_per_cta))

    def set_graphs(self, on: bool) -> None:
        self._check(self.lib.fs_batch_set_graphs(self.h, int(on)))

    def stream(self) -> int:
        return self.lib.fs_batch_get_stream(self.h) or 0

    def kernel_launches(self) -> int:
        return self.lib.fs_batch_kernel_launches(self.h)

    def state(self, sim: int) -> dict[str, np.ndarray]:
        s = {name: self.grid(sim, w) for name, w in (("u_front", U_FRONT), ("v_front", V_FRONT),
                                                      ("u_back", U_BACK), ("v_back", V_BACK),
                                                      ("u_prev", U_PREV), ("v_prev", V_PREV),
                                                      ("u_diff", U_DIFF), ("v_diff", V_DIFF))}
        s["labels"] = self.labels(sim)
        s["pressure"] = self.pressure(sim)
        s["particles"] = self.particles(sim)
        return s


class Smoke:
    """Differentiable smoke on the GPU (fs_smoke_*): forward steps, the loss
    ||density - target|| and its gradient with respect to the initial state."""

    def __init__(self, size_x: int, size_y: int, dt: float = 0.01, integrator: int = INTEGRATOR_RK2,
                 precision: int = SMOKE_FP32, projection_method: int = POISSON_MIXED, cg_tolerance: float = 1e-10,
                 checkpoint_every: int = 8, device: int = 0, cg_max_iterations: int = 100000,
                 inner_tolerance: float = 1e-3):
        self.lib = load_library()
        cfg = fs_smoke_config()
        self.lib.fs_smoke_config_init(C.byref(cfg), size_x, size_y)
        cfg.dt, cfg.integrator, cfg.precision = dt, integrator, precision
        cfg.projection_method, cfg.cg_tolerance, cfg.checkpoint_every = projection_method, cg_tolerance, checkpoint_every
        cfg.device, cfg.cg_max_iterations, cfg.inner_tolerance = device, cg_max_iterations, inner_tolerance
        h = C.c_void_p()
        rc = self.lib.fs_smoke_create(C.byref(cfg), C.byref(h))
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_smoke_last_error(None).decode())
        self.h = h
        self.shape = (size_y, size_x)

    def _check(self, rc: int) -> None:
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_smoke_last_error(self.h).decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fs_smoke_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arr(self, a) -> np.ndarray:
        return np.ascontiguousarray(a, dtype=np.float64).reshape(self.shape)

    def set_solid_mask(self, mask: np.ndarray | None) -> None:
        if mask is None:
            self._check(self.lib.fs_smoke_set_solid_mask(self.h, None))
        else:
            m = np.ascontiguousarray(mask, dtype=np.uint8).reshape(self.shape)
            self._check(self.lib.fs_smoke_set_solid_mask(self.h, _ptr(m)))

    def set_state(self, u, v, density) -> None:
        u, v, d = self._arr(u), self._arr(v), self._arr(density)
        self._check(self.lib.fs_smoke_set_state(self.h, _ptr(u), _ptr(v), _ptr(d)))

    def set_target(self, target) -> None:
        t = self._arr(target)
        self._check(self.lib.fs_smoke_set_target(self.h, _ptr(t)))

    def forward(self, steps: int) -> float:
        loss = C.c_double()
        self._check(self.lib.fs_smoke_forward(self.h, steps, C.byref(loss)))
        return loss.value

    def state(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        out = [np.empty(self.shape, np.float64) for _ in range(3)]
        self._check(self.lib.fs_smoke_get_state(self.h, *[_ptr(a) for a in out]))
        return tuple(out)

    def backward(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        out = [np.empty(self.shape, np.float64) for _ in range(3)]
        self._check(self.lib.fs_smoke_backward(self.h, *[_ptr(a) for a in out]))
        return tuple(out)

    def kernel_launches(self) -> int:
        return self.lib.fs_smoke_kernel_launches(self.h)


class PoissonSolver:
    """Pressure projection alone on the GPU (fs_poisson_*): labels + double rhs in,
    double pressure out, by the FP32, FP64 or mixed-precision method."""

    def __init__(self, size_x: int, size_y: int, length_x: float, length_y: float, device: int = 0):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.fs_poisson_create(size_x, size_y, length_x, length_y, device, C.byref(h))
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_last_error(None).decode())
        self.h = h
        self.nx, self.ny = size_x, size_y

    def _check(self, rc: int) -> None:
        if rc != FS_OK:
            raise FsError(rc, self.lib.fs_last_error(None).decode())

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fs_poisson_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_problem(self, labels: np.ndarray, rhs: np.ndarray) -> None:
        lab = np.ascontiguousarray(labels, dtype=np.uint8).reshape(self.ny, self.nx)
        b = np.ascontiguousarray(rhs, dtype=np.float64).reshape(self.ny, self.nx)
        self._check(self.lib.fs_poisson_set_problem(self.h, _ptr(lab), _ptr(b)))

    def solve(self, method: int, tol: float, maxit: int, inner_tol: float = 1e-3,
              inner_precision: int = CG_FLOAT) -> dict:
        st = fs_poisson_stats()
        self._check(self.lib.fs_poisson_solve(self.h, method, tol, maxit, inner_tol, inner_precision, C.byref(st)))
        return {"outer_iterations": st.outer_iterations, "inner_iterations": st.inner_iterations,
                "residual": st.residual, "ms": st.ms}

    def solution(self) -> np.ndarray:
        out = np.empty((self.ny, self.nx), np.float64)
        self._check(self.lib.fs_poisson_get_solution(self.h, _ptr(out)))
        return out
