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
