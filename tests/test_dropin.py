"""The C++ drop-in: one program written only against the reference's class API
(fluid_simulation_gb300/dropin/examples/dam_break.cpp) is compiled unchanged
against the reference's own sources (where the checkout exists) and against
the drop-in headers over the GPU library; both must produce the oracle's
particles bit for bit."""
import os
import subprocess

import numpy as np
import pytest

from oracle import build_oracle
from oracle import pyoracle as po

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXAMPLE = os.path.join(ROOT, "fluid_simulation_gb300", "dropin", "examples", "dam_break.cpp")
STEPS = 120


def oracle_particles(steps):
    """The example's scene, replayed call by call on the C restatement."""
    s = po.OracleSim("restatement", 64, 64, 64.0, 64.0, 0.005, 0.02)  # FluidSolver defaults: maxit 100, tol eps
    s.add_source(2.0, 24.0, 2.0, 36.0, 1.0, 1.0, 0.0, 0.0, 0.0, 1)
    s.add_source(2.0, 5.0, 48.0, 52.0, 1.0, 1.0, 6.0, 0.0, 0.05, 6)
    for _ in range(steps):
        s.update(0.005)
        assert s.step(po.STEP_PICFLIP, 0.005) == 0
    return s.particles()


def run(exe, tmp_path):
    out = str(tmp_path / "parts.bin")
    res = subprocess.run([exe, str(STEPS), out], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    return np.fromfile(out, dtype=np.float32).reshape(-1, 4)


@pytest.mark.skipif(not po.reference_available(), reason="reference build unavailable")
def test_example_against_reference_equals_oracle(tmp_path):
    exe = build_oracle.build_reference_program(EXAMPLE, "dam_break_ref")
    got = run(exe, tmp_path)
    ref = oracle_particles(STEPS)
    assert got.shape == ref.shape and got.shape[0] > 4000
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.gpu
def test_example_against_dropin_equals_oracle(tmp_path):
    from fluid_simulation_gb300 import build as fsbuild

    exe = fsbuild.build_example("dam_break")
    got = run(exe, tmp_path)
    ref = oracle_particles(STEPS)
    assert got.shape == ref.shape and got.shape[0] > 4000
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
