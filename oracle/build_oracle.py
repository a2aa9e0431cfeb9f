"""Build recipe for the oracle libraries (test infrastructure).

* ``oracle/_build/libfsoracle.so`` -- the C restatement ``oracle/fs_oracle.c``.
  Built on every machine (this container and the GPU machine).
* ``oracle/_ref/libfsref.so`` -- the reference's own sources
  ``src/{FluidSolver,FluidDomain,MacGrid,MarkerParticleSet,LevelSet,Canvas,Renderer}.cpp``,
  compiled where they lie under the reference checkout (``$FS_REFERENCE_DIR``,
  else a checkout named ``reference`` beside this repository's root) against
  the project's Eigen-subset stand-in
  ``oracle/eigen_shim`` plus ``oracle/ref_harness.cpp``.  Built only when the
  reference checkout exists; nothing is copied out of it.

Both use ``-O3 -DNDEBUG -ffp-contract=off``: no FMA contraction (aarch64 GCC
contracts by default), no fast-math, asserts off.

Usage: ``python oracle/build_oracle.py [--force]``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
RESTATEMENT_SO = os.path.join(BUILD_DIR, "libfsoracle.so")
REFERENCE_SO = os.path.join(REF_DIR, "libfsref.so")
REFERENCE_SOURCES = ("FluidSolver", "FluidDomain", "MacGrid", "MarkerParticleSet", "LevelSet", "Canvas", "Renderer")
FLAGS = ["-O3", "-DNDEBUG", "-ffp-contract=off", "-fPIC", "-fno-fast-math"]


def reference_dir() -> str:
    env = os.environ.get("FS_REFERENCE_DIR")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))


def build_restatement(force: bool = False) -> str:
    src = os.path.join(HERE, "fs_oracle.c")
    hdr = os.path.join(HERE, "fs_oracle.h")
    if not force and _newer(RESTATEMENT_SO, [src, hdr, __file__]):
        return RESTATEMENT_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = RESTATEMENT_SO + ".tmp%d" % os.getpid()
    _run(["gcc", "-std=c11", *FLAGS, "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, RESTATEMENT_SO)
    return RESTATEMENT_SO


def build_reference(force: bool = False) -> str | None:
    ref = reference_dir()
    if not os.path.isdir(os.path.join(ref, "src")):
        return None
    srcs = [os.path.join(ref, "src", n + ".cpp") for n in REFERENCE_SOURCES]
    harness = os.path.join(HERE, "ref_harness.cpp")
    shim = os.path.join(HERE, "eigen_shim", "Eigen", "fs_shim_core.h")
    deps = srcs + [harness, shim, os.path.join(HERE, "fs_oracle.h"), __file__]
    if not force and _newer(REFERENCE_SO, deps):
        return REFERENCE_SO
    os.makedirs(REF_DIR, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "eigen_shim"), "-I", os.path.join(ref, "include"), "-I", HERE]
    objs = []

    def compile_one(src: str) -> str:
        obj = os.path.join(REF_DIR, os.path.splitext(os.path.basename(src))[0] + ".o")
        _run(["g++", "-std=c++14", *FLAGS, "-w", *inc, "-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        objs = list(ex.map(compile_one, srcs + [harness]))
    tmp = REFERENCE_SO + ".tmp%d" % os.getpid()
    _run(["g++", "-shared", "-o", tmp, *objs])
    os.replace(tmp, REFERENCE_SO)
    return REFERENCE_SO


def build_reference_program(src: str, name: str) -> str | None:
    """Compiles a program written against the reference's class API with the
    reference's own sources (same stand-in and flags as libfsref.so) into
    oracle/_ref/<name>; None without the reference checkout."""
    if build_reference() is None:
        return None
    ref = reference_dir()
    exe = os.path.join(REF_DIR, name)
    objs = [os.path.join(REF_DIR, n + ".o") for n in REFERENCE_SOURCES]
    if _newer(exe, [src] + objs + [__file__]):
        return exe
    inc = ["-I", os.path.join(HERE, "eigen_shim"), "-I", os.path.join(ref, "include")]
    _run(["g++", "-std=c++14", *FLAGS, "-w", *inc, src, *objs, "-o", exe])
    return exe


def main(argv: list[str]) -> int:
    force = "--force" in argv
    print("restatement:", build_restatement(force))
    print("reference:", build_reference(force) or "not built (no reference checkout)")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
