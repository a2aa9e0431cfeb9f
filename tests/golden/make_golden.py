"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs the reference sources (compiled by oracle/build_oracle.py into
oracle/_ref/libfsref.so against the Eigen-subset stand-in) on seeded scenes
and stores the observable state after selected steps.  The fixtures pin the C
restatement (oracle/fs_oracle.c) and the GPU library on machines without the
reference checkout.

Usage (needs the reference checkout): python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fluid_simulation_gb300 import scenes  # noqa: E402
from oracle import pyoracle as po  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# name -> (method, steps to record, scene builder, options)
CASES = {
    "picflip_dam64": (po.STEP_PICFLIP, (1, 10, 50, 200), "small", {}),
    "pic_dam64": (po.STEP_PIC, (1, 10), "small", {}),
    "flip_dam64": (po.STEP_FLIP, (1, 10), "small", {}),
    "semilagrangian_dam64": (po.STEP_SEMI_LAGRANGIAN, (1, 10), "small", {}),
    "picflip_disc64": (po.STEP_PICFLIP, (1, 30), "small", {"disc": (45.0, 20.0, 8.0)}),
    "picflip_source64": (po.STEP_PICFLIP, (1, 30), "source", {}),
}

FULL_KEYS = ("u_front", "v_front", "u_back", "v_back", "u_prev", "v_prev", "u_diff", "v_diff",
             "labels", "fluid_indices", "particle_counts", "pressure", "particles")


def make_sim(kind: str, case: str):
    method, steps, scene, opt = CASES[case]
    sc = scenes.dam_break_small()
    sim = po.OracleSim(kind, sc.size_x, sc.size_y, sc.length_x, sc.length_y, sc.density, sc.pic_ratio)
    sim.set_cg(sc.cg_tolerance, sc.cg_max_iterations)
    solid = None
    if "disc" in opt:
        solid = scenes.disc_mask(sc.size_x, sc.size_y, *opt["disc"])
        sim.set_solid_mask(solid)
    sources = scene == "source"
    if sources:
        # A FluidSource as in examples/simple.cpp:36, spawning 5 times.
        sim.add_source(2.0, 10.0, 40.0, 50.0, 1.0, 1.0, 3.0, 0.0, 0.05, 5)
    else:
        sim.set_particles(sc.particles)
    return sim, sc, method, steps, solid, sources


def run_case(kind: str, case: str) -> dict[str, np.ndarray]:
    sim, sc, method, steps, solid, sources = make_sim(kind, case)
    out: dict[str, np.ndarray] = {}
    last = max(steps)
    for k in range(1, last + 1):
        if sources:
            sim.update(sc.dt)
        rc = sim.step(method, sc.dt)
        assert rc == 0
        if k in steps:
            st = sim.state()
            for key in FULL_KEYS:
                out["s%d_%s" % (k, key)] = st[key]
            it, err, nf = sim.cg_stats()
            out["s%d_cg" % k] = np.array([it, err, nf], np.float64)
    return out


def main() -> int:
    if not po.reference_available():
        print("reference build unavailable; fixtures not regenerated")
        return 1
    for case in CASES:
        data = run_case("reference", case)
        path = os.path.join(HERE, case + ".npz")
        np.savez_compressed(path, **data)
        print(case, os.path.getsize(path), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
