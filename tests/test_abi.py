"""The C-ABI library loads and exports every function include/fsgpu.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import build as fsbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fs_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    fsbuild.build()
    return ctypes.CDLL(fsg.library_path())


def test_every_declared_symbol_is_exported(lib):
    names = _declared("fsgpu.h")
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_front_end_covers_the_header():
    assert sorted(fsg.SIGNATURES) == _declared("fsgpu.h")


def test_library_has_no_cpu_fallback_symbols(lib):
    # The product library never links the oracle.
    assert not hasattr(lib, "fso_create")


def test_load_library_fails_loudly_without_the_build(tmp_path):
    with pytest.raises(RuntimeError):
        fsg.load_library(str(tmp_path / "missing.so"))


def test_config_defaults_are_the_reference_s(lib):
    """fs_config_init: density 1, pic_ratio 0, gravity (0, -9.82)
    (src/FluidSolver.cpp:232), CG maxit 100 and Eigen's default tolerance
    FLT_EPSILON (src/FluidSolver.cpp:81), 2 extension sweeps (:234)."""
    c = fsg.fs_config()
    lib.fs_config_init(ctypes.byref(c), 64, 48)
    assert (c.size_x, c.size_y, c.length_x, c.length_y) == (64, 48, 64.0, 48.0)
    assert (c.density, c.pic_ratio, c.gravity_x) == (1.0, 0.0, 0.0)
    assert c.gravity_y == ctypes.c_float(-9.82).value
    assert (c.cg_max_iterations, c.extension_iterations, c.device) == (100, 2, 0)
    assert c.cg_tolerance == 1.1920928955078125e-07


def test_invalid_arguments_are_reported_before_any_device_work():
    """Argument checks come before any CUDA call, so they hold on a machine
    without a GPU; a null handle is an error, never a crash."""
    lib = fsg.load_library()
    invalid, too_large = 1, 5
    h = ctypes.c_void_p()
    assert lib.fs_create(None, ctypes.byref(h)) == invalid
    assert b"null" in lib.fs_last_error(None)
    for size_x, size_y, length in ((0, 10, 10.0), (10, -1, 10.0), (10, 10, 0.0), (10, 10, float("nan")),
                                   (10, 10, float("inf"))):
        c = fsg.fs_config()
        lib.fs_config_init(ctypes.byref(c), size_x, size_y)
        c.length_x = length
        assert lib.fs_create(ctypes.byref(c), ctypes.byref(h)) == invalid, (size_x, size_y, length)
    c = fsg.fs_config()
    lib.fs_config_init(ctypes.byref(c), 4097, 4096)
    assert lib.fs_create(ctypes.byref(c), ctypes.byref(h)) == too_large
    assert b"16777216" in lib.fs_last_error(None)
    assert lib.fs_step(None, fsg.STEP_PICFLIP, 0.005) == invalid
    assert lib.fs_set_particles(None, None, 0) == invalid
    assert lib.fs_get_particles(None, None, 0) == invalid
    assert lib.fs_destroy(None) == 0
