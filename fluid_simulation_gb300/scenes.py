"""Seeded synthetic initial states for the fluid step (host-side workload setup).

The reference ships no datasets; its examples build a dam break with a
``FluidSource`` (examples/simple.cpp:36) or mouse-driven sources
(examples/opengl_example/FluidInteractionHandler.cpp).  The workloads here are
dam breaks whose particles are jittered inside their cells by a SplitMix64
stream, so that every implementation (GPU, oracle, reference) starts from the
same bytes.  SplitMix64 is used instead of ``std::uniform_real_distribution``
because the latter is implementation-defined.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

_M64 = (1 << 64) - 1


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n successive SplitMix64 outputs (Steele, Lea & Flood 2014) as uint64."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = (np.uint64(seed & _M64) + idx * np.uint64(0x9E3779B97F4A7C15))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int) -> np.ndarray:
    """n float32 values in [0, 1): the top 24 bits of each SplitMix64 output."""
    return ((splitmix64(seed, n) >> np.uint64(40)).astype(np.float64) * (2.0 ** -24)).astype(np.float32)


@dataclass
class Scene:
    """Everything needed to construct and fill one simulation."""

    size_x: int
    size_y: int
    length_x: float
    length_y: float
    density: float
    pic_ratio: float
    dt: float
    particles: np.ndarray                     # (n, 4) float32 {x, y, vx, vy}
    solid: np.ndarray | None = None           # (size_y, size_x) uint8 or None
    gravity: tuple[float, float] = (0.0, -9.82)
    cg_tolerance: float = 1.1920928955078125e-07
    cg_max_iterations: int = 100
    description: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.size_x * self.size_y


def block_particles(size_x: int, size_y: int, length_x: float, length_y: float, i0: int, i1: int,
                    j0: int, j1: int, per_cell: int, seed: int,
                    solid: np.ndarray | None = None) -> np.ndarray:
    """per_cell jittered particles in each cell of [i0, i1) x [j0, j1), j-major
    cell order, skipping cells that are solid; positions (i + U, j + U) * delta."""
    dx = np.float32(np.float32(length_x) / np.float32(size_x))
    dy = np.float32(np.float32(length_y) / np.float32(size_y))
    jj, ii = np.meshgrid(np.arange(j0, j1), np.arange(i0, i1), indexing="ij")
    ii = ii.reshape(-1)
    jj = jj.reshape(-1)
    if solid is not None:
        keep = solid[jj, ii] == 0
        ii, jj = ii[keep], jj[keep]
    ncell = ii.size
    u = uniform01(seed, 2 * per_cell * ncell).reshape(ncell, per_cell, 2)
    x = (ii[:, None].astype(np.float32) + u[:, :, 0]) * dx
    y = (jj[:, None].astype(np.float32) + u[:, :, 1]) * dy
    out = np.zeros((ncell * per_cell, 4), np.float32)
    out[:, 0] = x.reshape(-1).astype(np.float32)
    out[:, 1] = y.reshape(-1).astype(np.float32)
    return out


def disc_mask(size_x: int, size_y: int, cx: float, cy: float, radius: float) -> np.ndarray:
    """uint8 mask of cells whose centre lies within radius (in cells) of (cx, cy)."""
    jj, ii = np.meshgrid(np.arange(size_y), np.arange(size_x), indexing="ij")
    d2 = (ii + 0.5 - cx) ** 2 + (jj + 0.5 - cy) ** 2
    return (d2 <= radius * radius).astype(np.uint8)


def dam_break_small(seed: int = 0xC1) -> Scene:
    """64x64 unit cells, solid border, fluid block over the left 40% x 60%,
    4 jittered particles per cell, rho = dt = 0.005, FLIP ratio 0.98
    (pic_ratio 0.02), CG to relative residual 1e-6."""
    n = 64
    i1 = int(np.ceil(0.4 * n))
    j1 = int(np.ceil(0.6 * n))
    parts = block_particles(n, n, float(n), float(n), 1, i1, 1, j1, 4, seed)
    return Scene(n, n, float(n), float(n), 0.005, 0.02, 0.005, parts,
                 cg_tolerance=1e-6, cg_max_iterations=2000,
                 description="dam break 64x64, 4 particles/cell, CG 1e-6",
                 meta={"block": [1, i1, 1, j1], "seed": seed})


def dam_break_large(n: int = 1024, seed: int = 0xC2) -> Scene:
    """n x n unit cells with a circular solid obstacle of radius 100 cells
    (n/1024 scaled) right of a dam-break block sized to ~1.7M particles at
    n = 1024 (655 x 655 cells x 4), rho = dt = 0.005, FLIP ratio 0.95
    (pic_ratio 0.05), CG to relative residual 1e-5."""
    scale = n / 1024.0
    w = max(2, int(round(655 * scale)))
    cx, cy, r = 840.0 * scale, 200.0 * scale, 100.0 * scale
    solid = disc_mask(n, n, cx, cy, r)
    parts = block_particles(n, n, float(n), float(n), 1, 1 + w, 1, 1 + w, 4, seed, solid)
    return Scene(n, n, float(n), float(n), 0.005, 0.05, 0.005, parts, solid=solid,
                 cg_tolerance=1e-5, cg_max_iterations=100000,
                 description="dam break %dx%d + disc r=%g, 4 particles/cell, CG 1e-5" % (n, n, r),
                 meta={"block": [1, 1 + w, 1, 1 + w], "disc": [cx, cy, r], "seed": seed})


def projection_problem(n: int = 4096, seed: int = 0xC5, solid_fraction: float = 0.05):
    """Pressure projection alone: an n x n fluid-filled domain, solid border and
    Bernoulli(solid_fraction) interior solids (seeded), fluid cells with no
    non-solid neighbour turned solid (their matrix row would be zero), and a
    right-hand side of i.i.d. N(0, 1) values (Box-Muller on the SplitMix64
    stream) with the mean of every 4-connected fluid component removed, so
    that each component -- a pure Neumann problem, as nothing is AIR -- is
    consistent.  Returns (labels uint8, rhs float64)."""
    from scipy import ndimage

    LIQUID, SOLID = 0, 2
    u = uniform01(seed, n * n).reshape(n, n)
    labels = np.where(u < solid_fraction, SOLID, LIQUID).astype(np.uint8)
    labels[0, :] = labels[-1, :] = SOLID
    labels[:, 0] = labels[:, -1] = SOLID
    fluid = labels == LIQUID
    nb = np.zeros_like(fluid, dtype=np.int32)
    nb[1:, :] += fluid[:-1, :]
    nb[:-1, :] += fluid[1:, :]
    nb[:, 1:] += fluid[:, :-1]
    nb[:, :-1] += fluid[:, 1:]
    labels[fluid & (nb == 0)] = SOLID
    fluid = labels == LIQUID
    u1 = uniform01(seed ^ 0x5EED, n * n).astype(np.float64).reshape(n, n)
    u2 = uniform01(seed ^ 0xBEEF, n * n).astype(np.float64).reshape(n, n)
    g = np.sqrt(-2.0 * np.log(1.0 - u1)) * np.cos(2.0 * np.pi * u2)
    comp, ncomp = ndimage.label(fluid, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    sums = ndimage.sum(g, comp, index=np.arange(1, ncomp + 1))
    counts = ndimage.sum(np.ones_like(g), comp, index=np.arange(1, ncomp + 1))
    means = np.concatenate([[0.0], sums / counts])
    rhs = np.where(fluid, g - means[comp], 0.0)
    return labels, rhs


def batch_scenes(n: int = 512, seed: int = 0xC3, min_side: int = 32, max_side: int = 256,
                 max_discs: int = 3) -> list[Scene]:
    """n independent square simulations with unit cells: side ~ U{min_side..max_side},
    a random rectangular fluid block (4 jittered particles per non-solid cell),
    0..max_discs random solid discs, FLIP ratio ~ U[0.9, 1.0] (pic_ratio = 1 -
    ratio), rho = dt = 0.005, CG to relative residual 1e-5.  Every draw comes
    from the SplitMix64 stream of (seed, simulation)."""
    out = []
    for s in range(n):
        u = splitmix64((seed << 20) ^ (s * 0x9E37), 16)
        f = (u >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
        side = min_side + int(f[0] * (max_side - min_side + 1))
        side = min(side, max_side)
        # block [i0, i1) x [j0, j1) inside the solid border, at least 2 cells a side
        w = max(2, int((0.2 + 0.5 * f[1]) * (side - 2)))
        h = max(2, int((0.2 + 0.5 * f[2]) * (side - 2)))
        i0 = 1 + int(f[3] * (side - 2 - w))
        j0 = 1 + int(f[4] * (side - 2 - h))
        ndisc = min(max_discs, int(f[5] * (max_discs + 1)))
        solid = np.zeros((side, side), np.uint8)
        for d in range(ndisc):
            r = 2.0 + f[6 + 3 * d] * side / 10.0
            cx = 1.0 + f[7 + 3 * d] * (side - 2)
            cy = 1.0 + f[8 + 3 * d] * (side - 2)
            solid |= disc_mask(side, side, cx, cy, r)
        ratio = 0.9 + 0.1 * f[15]
        pic = float(np.float32(1.0 - ratio))
        parts = block_particles(side, side, float(side), float(side), i0, i0 + w, j0, j0 + h, 4,
                                seed * 1000003 + s, solid if ndisc else None)
        out.append(Scene(side, side, float(side), float(side), 0.005, pic, 0.005, parts,
                         solid=solid if ndisc else None, cg_tolerance=1e-5, cg_max_iterations=20000,
                         description="batch member %d: %dx%d, block %dx%d, %d discs" % (s, side, side, w, h, ndisc),
                         meta={"block": [i0, i0 + w, j0, j0 + h], "discs": ndisc, "seed": seed}))
    return out


def normal01(seed: int, n: int) -> np.ndarray:
    """n N(0, 1) doubles by Box-Muller on two SplitMix64 streams."""
    u1 = uniform01(seed, n).astype(np.float64)
    u2 = uniform01(seed ^ 0xA5A5A5A5, n).astype(np.float64)
    return np.sqrt(-2.0 * np.log(1.0 - u1)) * np.cos(2.0 * np.pi * u2)


def smoke_problem(n: int = 256, seed: int = 0xC4, sigma: float = 20.0, shift: tuple[float, float] = (16.0, 8.0),
                  kmax: int = 8):
    """Differentiable-smoke initial state on an n x n unit-cell grid: a Gaussian
    density blob (sigma cells) at the centre, a target blob shifted by `shift`
    cells, and a velocity of random Fourier modes 1 <= |k| <= kmax (seeded
    N(0, 1) cosine and sine coefficients per component) normalised to RMS 1
    and rounded to float32.  Returns (u, v, density, target) as float64
    arrays of shape (n, n), u(i, j) at (i, j + 1/2), v(i, j) at (i + 1/2, j)."""
    jj, ii = np.meshgrid(np.arange(n, dtype=np.float64), np.arange(n, dtype=np.float64), indexing="ij")
    c = n / 2.0
    d0 = np.exp(-((ii + 0.5 - c) ** 2 + (jj + 0.5 - c) ** 2) / (2 * sigma * sigma))
    tx, ty = c + shift[0], c + shift[1]
    target = np.exp(-((ii + 0.5 - tx) ** 2 + (jj + 0.5 - ty) ** 2) / (2 * sigma * sigma))
    modes = [(kx, ky) for kx in range(-kmax, kmax + 1) for ky in range(0, kmax + 1)
             if 1 <= kx * kx + ky * ky <= kmax * kmax and (ky > 0 or kx > 0)]
    coef = normal01(seed, 4 * len(modes)).reshape(len(modes), 4)
    L = float(n)
    u = np.zeros((n, n))
    v = np.zeros((n, n))
    for (kx, ky), (a, b, cc, d) in zip(modes, coef):
        ph_u = 2 * np.pi * (kx * ii + ky * (jj + 0.5)) / L
        ph_v = 2 * np.pi * (kx * (ii + 0.5) + ky * jj) / L
        u += a * np.cos(ph_u) + b * np.sin(ph_u)
        v += cc * np.cos(ph_v) + d * np.sin(ph_v)
    rms = np.sqrt((np.mean(u * u) + np.mean(v * v)) / 2.0)
    u = (u / rms).astype(np.float32).astype(np.float64)
    v = (v / rms).astype(np.float32).astype(np.float64)
    return u, v, d0.astype(np.float32).astype(np.float64), target.astype(np.float32).astype(np.float64)
