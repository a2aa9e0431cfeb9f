"""Device memory of a simulation handle against the budget stated for
integrators: about 135 bytes per cell and 72 bytes per particle of capacity
(the capacity doubles from 4096 as particles are added)."""
import pytest

import fluid_simulation_gb300 as fsg
from fluid_simulation_gb300 import scenes

CELL_BYTES = 135
PARTICLE_BYTES = 72


def capacity(n: int) -> int:
    cap = 4096
    while cap < n:
        cap *= 2
    return cap


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1024, 4096])
def test_handle_device_memory_within_budget(n):
    """fs_create + fs_set_particles of the benchmark's dam break at n^2 (1.7M
    and 27.5M particles), measured as the drop in free device memory
    (cudaMalloc rounds each buffer up, so the band is wide)."""
    import torch

    from fluid_simulation_gb300 import build as fsbuild

    fsbuild.build()
    sc = scenes.dam_break_large(n)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    sim = fsg.FluidSim.from_scene(sc)
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    sim.close()
    npart = len(sc.particles)
    budget = CELL_BYTES * sc.size_x * sc.size_y + PARTICLE_BYTES * capacity(npart)
    print(f"handle device memory: {used / 2**20:.1f} MiB measured, {budget / 2**20:.1f} MiB budgeted "
          f"({sc.size_x}x{sc.size_y} cells, {npart} particles, capacity {capacity(npart)})")
    assert 0.8 * budget <= used <= 1.1 * budget + (64 << 20), (used, budget)
