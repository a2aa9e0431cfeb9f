"""The ncu summaries under profiles/ give the command that produced each;
those commands must stay runnable as the code changes.  For every command:
its bench.py arguments parse with bench.py's own parser, `--clock-control
none` is given, and a `-k regex:` kernel filter matches a kernel that the
CUDA sources define."""
import glob
import os
import re
import shlex
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fluid_simulation_gb300", "csrc")


def _commands():
    """(file, command) for every ncu command, continuation lines joined."""
    out = []
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        lines = open(path).read().splitlines()
        k = 0
        while k < len(lines):
            line = lines[k].strip()
            if line.startswith("ncu "):
                cmd = line
                while cmd.endswith("\\") and k + 1 < len(lines):
                    k += 1
                    cmd = cmd[:-1] + " " + lines[k].strip()
                out.append((os.path.basename(path), cmd))
            k += 1
    return out


COMMANDS = _commands()


def _kernel_names(demangled=False):
    """__global__ function names; with demangled names (ncu
    --kernel-name-base demangled) also the functors the generic kernels take
    as template arguments."""
    names = set()
    for path in glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cuh")):
        src = open(path).read()
        names.update(re.findall(r"__global__\s+void\s+(?:__launch_bounds__\([^)]*\)\s+)?(\w+)", src))
        if demangled:
            names.update(re.findall(r"^struct\s+(\w+)", src, re.M))
    return names


def test_every_profile_has_a_command():
    files = {os.path.basename(p) for p in glob.glob(os.path.join(ROOT, "profiles", "*.md"))}
    assert files and files == {f for f, _ in COMMANDS}


@pytest.mark.parametrize("fname,cmd", COMMANDS, ids=[f for f, _ in COMMANDS])
def test_profile_command_is_runnable(fname, cmd, monkeypatch):
    argv = shlex.split(cmd)
    assert argv[argv.index("--clock-control") + 1] == "none"
    if "-k" in argv:
        pattern = argv[argv.index("-k") + 1]
        assert pattern.startswith("regex:")
        rx = re.compile(pattern[len("regex:"):])
        demangled = "--kernel-name-base" in argv and argv[argv.index("--kernel-name-base") + 1] == "demangled"
        assert any(rx.search(n) for n in _kernel_names(demangled)), (fname, pattern)
    i = argv.index("bench.py")
    assert argv[i - 1] == "python"
    sys.path.insert(0, ROOT)
    try:
        import bench
    finally:
        sys.path.remove(ROOT)
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv[i + 1:])
    args = bench.parse()
    assert args.impl == "gpu"
