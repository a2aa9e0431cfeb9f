"""Builds libfsgpu.so (the CUDA kernels + C ABI) in-tree with nvcc for sm_103a.

Output: fluid_simulation_gb300/_build/libfsgpu.so (+ libfsgpu_dropin.so, the
C++ drop-in classes over the C ABI).  Each .cu file is compiled to its own
object in parallel; the library links the CUDA runtime statically.

``-fmad=false`` keeps every float product and sum separately rounded (the
kernels also spell this out with __f*_rn intrinsics), and ``-ffp-contract=off``
does the same for host code (the renderer's weight table), which the bit-exact
parity with the reference's CPU code relies on.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
DROPIN = os.path.join(PKG, "dropin")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libfsgpu.so")
DROPIN_LIB = os.path.join(BUILD, "libfsgpu_dropin.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(ROOT, "include", "fsgpu.h"))
    return hs


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> str:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), res.stdout, res.stderr))
    return res.stdout + res.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    hdrs = _headers()
    objs = []
    jobs = []
    for s in srcs:
        o = os.path.join(BUILD, os.path.splitext(os.path.basename(s))[0] + ".o")
        objs.append(o)
        if force or ptxas_info or _stale(o, [s, __file__] + hdrs):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", s, "-o", o]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                if verbose or ptxas_info:
                    print(out)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
        os.replace(tmp, LIB)
    build_dropin(force)
    return LIB


def build_dropin(force: bool = False) -> str | None:
    """The C++ drop-in classes (reference API) as a shared library over libfsgpu.so."""
    src_dir = os.path.join(DROPIN, "src")
    inc_dir = os.path.join(DROPIN, "include")
    if not os.path.isdir(src_dir):
        return None
    srcs = sorted(os.path.join(src_dir, f) for f in os.listdir(src_dir) if f.endswith(".cpp"))
    hdrs = [os.path.join(inc_dir, f) for f in os.listdir(inc_dir)] + [os.path.join(ROOT, "include", "fsgpu.h")]
    if not force and not _stale(DROPIN_LIB, srcs + hdrs + [LIB, __file__]):
        return DROPIN_LIB
    tmp = DROPIN_LIB + ".tmp%d" % os.getpid()
    _run(["g++", "-std=c++14", "-O2", "-fPIC", "-shared", "-I", inc_dir, "-I", os.path.join(ROOT, "include"),
          *srcs, "-o", tmp, "-L", BUILD, "-lfsgpu", "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, DROPIN_LIB)
    return DROPIN_LIB


def build_example(name: str = "dam_break") -> str:
    """Compiles dropin/examples/<name>.cpp, a program written against the
    reference's class API, against the drop-in headers and libraries."""
    build()
    src = os.path.join(DROPIN, "examples", name + ".cpp")
    exe = os.path.join(BUILD, name + "_gpu")
    if _stale(exe, [src, DROPIN_LIB, LIB]):
        _run(["g++", "-std=c++14", "-O2", "-I", os.path.join(DROPIN, "include"), "-I", os.path.join(ROOT, "include"),
              src, "-o", exe, "-L", BUILD, "-lfsgpu_dropin", "-lfsgpu", "-Wl,-rpath," + BUILD])
    return exe


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
