"""Seeded synthetic scenes with the shapes of the benchmark configurations.

No public dataset is involved: every scene is a lattice block of fluid
particles (spacing 2r, positions lo + (i + 1/2) s with x outer / z inner as in
apps/sim_cli/main.cpp:126-135) with a uniform +-0.05 r jitter per axis drawn
from SplitMix64(seed, particle, axis), inside an AABB whose walls are sampled
by sample_aabb_boundary(domain, 2r, 3) (solvers/dfsph/src/boundary_sampler.cpp).

SplitMix64 is the published mixing generator of Steele, Lea and Flood (2014);
it is restated here on numpy uint64 arrays so that the inputs are identical on
every machine.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 output function applied to state x (uint64 array)."""
    with np.errstate(over="ignore"):
        z = x.astype(np.uint64) + _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, index: np.ndarray) -> np.ndarray:
    """Uniform [0, 1) doubles, one per (seed, index) pair."""
    x = (np.uint64(seed) << np.uint64(40)) ^ index.astype(np.uint64)
    return (splitmix64(x) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def lattice_block(lo, counts, spacing: float, jitter: float, seed: int) -> np.ndarray:
    """counts = (nx, ny, nz) particles at lo + (i + 1/2) s, x outer / z inner,
    each axis jittered uniformly in [-jitter, +jitter]."""
    nx, ny, nz = (int(c) for c in counts)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    base = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    pos = np.asarray(lo, dtype=np.float64)[None, :] + (base + 0.5) * spacing
    n = pos.shape[0]
    if jitter > 0:
        idx = np.arange(3 * n, dtype=np.uint64)
        u = uniform01(seed, idx).reshape(n, 3)
        pos += (2.0 * u - 1.0) * jitter
    return pos.astype(np.float32)


def normal(seed: int, n: int, sigma: float) -> np.ndarray:
    """n x 3 normal samples (Box-Muller over SplitMix64 uniforms)."""
    idx = np.arange(6 * n, dtype=np.uint64)
    u = uniform01(seed, idx).reshape(n, 3, 2)
    u1 = np.maximum(u[..., 0], 1e-300)
    r = np.sqrt(-2.0 * np.log(u1))
    return (sigma * r * np.cos(2.0 * np.pi * u[..., 1])).astype(np.float32)


def sample_aabb_boundary(lo, hi, spacing: float, n_layers: int = 3) -> np.ndarray:
    """water::solvers::sample_aabb_boundary through the C ABI (host code)."""
    lib = _lib.load()
    lo3, hi3 = _lib.fvec3(lo), _lib.fvec3(hi)
    n = lib.dfsph_sample_aabb_boundary(lo3, hi3, ctypes.c_float(spacing), n_layers, None, 0)
    if n < 0:
        raise ValueError("sample_aabb_boundary: invalid arguments")
    out = np.empty((n, 3), dtype=np.float32)
    lib.dfsph_sample_aabb_boundary(lo3, hi3, ctypes.c_float(spacing), n_layers,
                                   out.ctypes.data_as(ctypes.c_void_p), n)
    return out


@dataclass
class Scene:
    name: str
    radius: float
    domain_min: tuple
    domain_max: tuple
    fluid: np.ndarray
    velocity: np.ndarray
    boundary: np.ndarray
    dt: float
    steps: int
    viscosity: float = 0.01
    damping: float = 0.5
    max_density_iters: int = 4
    max_divergence_iters: int = 0
    eta_density: float = 0.0
    eta_divergence: float = 0.0
    extra: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.fluid.shape[0])

    @property
    def nb(self) -> int:
        return int(self.boundary.shape[0])

    def config(self, precision: int = _lib.PRECISION_FP32, diagnostics: bool = False,
               capacity: int | None = None) -> _lib.DfsphConfig:
        lib = _lib.load()
        c = _lib.DfsphConfig()
        lib.dfsph_config_init(ctypes.byref(c))
        c.rest_density = 1000.0
        c.particle_radius = self.radius
        c.smoothing_length = np.float32(2.0 * np.float32(self.radius))
        c.viscosity = self.viscosity
        c.damping = self.damping
        c.gravity[0], c.gravity[1], c.gravity[2] = 0.0, -9.81, 0.0
        c.max_density_iters = self.max_density_iters
        c.max_divergence_iters = self.max_divergence_iters
        c.eta_density = self.eta_density
        c.eta_divergence = self.eta_divergence
        for a in range(3):
            c.domain_min[a] = self.domain_min[a]
            c.domain_max[a] = self.domain_max[a]
        c.precision = precision
        c.capacity = capacity if capacity is not None else max(self.n, 1)
        c.boundary_capacity = max(self.nb, 1)
        c.record_diagnostics = 1 if diagnostics else 0
        return c


def puddle(seed: int = 1, sampler=None) -> Scene:
    """Settled puddle: 17^3 particles, r = 0.01, corner (0.3, 0.5, 0.3), box [0,1]^3,
    XSPH 0.01, dt 1e-3, divergence 0.1 % / density 0.01 % tolerances, <= 100 iterations.
    `sampler(lo, hi, spacing, n_layers)` samples the walls (default: the
    library's sample_aabb_boundary)."""
    sampler = sampler or sample_aabb_boundary
    r = 0.01
    s = 2 * r
    fluid = lattice_block((0.3, 0.5, 0.3), (17, 17, 17), s, 0.05 * r, seed)
    lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    return Scene("puddle_4913", r, lo, hi, fluid, np.zeros_like(fluid),
                 sampler(lo, hi, s, 3), dt=1e-3, steps=1500, viscosity=0.01,
                 max_density_iters=100, max_divergence_iters=100, eta_density=1e-4,
                 eta_divergence=1e-3)


def dam_break(scale: int = 1, reference_mode: bool = True, sampler=None) -> Scene:
    """Dam break: a (40 x 80 x 40) * scale column at spacing 0.01 / scale against the
    x = 0 wall of a 1.6 x 1.0 x 0.6 m tank (scale 1: 128,000 particles, scale 2:
    1,024,000). The block starts 3 spacings inside the x = 0 wall and the floor
    (the wall layers occupy [0, 2s]), lattice points at lo + (i + 1/2) s, i.e. at
    cell centres; the column is centred in z. Fixed 4 density iterations and,
    outside reference mode, 2 divergence iterations; dt = 5e-4 / scale.
    `sampler` as for puddle()."""
    sampler = sampler or sample_aabb_boundary
    r = 0.005 / scale
    s = 2 * r
    nx, ny, nz = 40 * scale, 80 * scale, 40 * scale
    lo = (3.0 * s, 3.0 * s, 0.5 * (0.6 - nz * s))
    fluid = lattice_block(lo, (nx, ny, nz), s, 0.05 * r, 2 if scale == 1 else 3)
    dlo, dhi = (0.0, 0.0, 0.0), (1.6, 1.0, 0.6)
    return Scene(f"dam_break_{nx * ny * nz}", r, dlo, dhi, fluid, np.zeros_like(fluid),
                 sampler(dlo, dhi, s, 3), dt=5e-4 / scale,
                 steps=2000 if scale == 1 else 500, viscosity=0.01,
                 max_density_iters=4, max_divergence_iters=0 if reference_mode else 2)


def batched_blocks(n_scenes: int = 64, seed_base: int = 1000, n_min: int = 2000, n_max: int = 60000):
    """Independent falling blocks in the unit box, one per scene: scene k draws
    (from seed seed_base + k) a particle count uniform in [n_min, n_max], block
    aspect ratios x:y and z:y uniform in [0.5, 2] and an XSPH coefficient
    uniform in [0.005, 0.05]; r = 0.01 m, dt = 1e-3 s. All scenes share the
    wall particles of the box. Returns (scenes, viscosities)."""
    r = 0.01
    s = 2 * r
    lo_box, hi_box = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    walls = sample_aabb_boundary(lo_box, hi_box, s, 3)
    max_cells = int(round((1.0 - 6 * s) / s))  # lattice sites between the wall layers
    out, eps = [], []
    for k in range(n_scenes):
        seed = seed_base + k
        u = uniform01(seed, np.arange(4, dtype=np.uint64))
        target = n_min + u[0] * (n_max - n_min)
        ax = 0.5 + 1.5 * u[1]
        az = 0.5 + 1.5 * u[2]
        ny = max(1, int(round((target / (ax * az)) ** (1.0 / 3.0))))
        nx = min(max_cells, max(1, int(round(ax * ny))))
        nz = min(max_cells, max(1, int(round(az * ny))))
        ny = min(max_cells, ny)
        lo = (0.5 - 0.5 * nx * s, min(0.3, 1.0 - 3 * s - ny * s), 0.5 - 0.5 * nz * s)
        fluid = lattice_block(lo, (nx, ny, nz), s, 0.05 * r, seed)
        e = 0.005 + 0.045 * u[3]
        sc = Scene(f"batch_{k}", r, lo_box, hi_box, fluid, np.zeros_like(fluid), walls, dt=1e-3, steps=300,
                   viscosity=float(np.float32(e)), max_density_iters=4, max_divergence_iters=0)
        out.append(sc)
        eps.append(float(np.float32(e)))
    return out, eps


def falling_block(n_side=(12, 12, 12), seed: int = 7, radius: float = 0.01,
                  corner=(0.35, 0.4, 0.35), velocity_sigma: float = 0.0,
                  boundary: bool = True) -> Scene:
    """A small jittered block in the unit box (used by tests)."""
    r = radius
    s = 2 * r
    fluid = lattice_block(corner, n_side, s, 0.05 * r, seed)
    vel = normal(seed + 100, fluid.shape[0], velocity_sigma) if velocity_sigma > 0 else np.zeros_like(fluid)
    lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    b = sample_aabb_boundary(lo, hi, s, 3) if boundary else np.zeros((0, 3), np.float32)
    return Scene(f"block_{fluid.shape[0]}", r, lo, hi, fluid, vel, b, dt=1e-3, steps=50, viscosity=0.01,
                 max_density_iters=4, max_divergence_iters=0)


def adjoint_drop(n_side: int = 32, seed: int = 11, velocity_sigma: float = 0.1) -> Scene:
    """Differentiable drop: an n_side^3 block (32^3 = 32,768 particles, r = 0.01 m)
    centred in x and z with its lower corner at y = 0.3 in the unit box, initial
    velocities N(0, sigma^2) per component (seeded), dt = 1e-3 s, 200 steps,
    fixed 2 divergence and 4 density iterations, XSPH 0.01. The loss target is
    the initial block translated by (0.1, 0, 0) m (extra["target_shift"]);
    checkpoints every 20 steps (extra["checkpoint_every"])."""
    r = 0.01
    s = 2 * r
    lo = (0.5 - 0.5 * n_side * s, 0.3, 0.5 - 0.5 * n_side * s)
    fluid = lattice_block(lo, (n_side, n_side, n_side), s, 0.05 * r, seed)
    vel = normal(seed + 100, fluid.shape[0], velocity_sigma)
    dlo, dhi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    return Scene(f"adjoint_drop_{fluid.shape[0]}", r, dlo, dhi, fluid, vel, sample_aabb_boundary(dlo, dhi, s, 3),
                 dt=1e-3, steps=200, viscosity=0.01, max_density_iters=4, max_divergence_iters=2,
                 extra={"target_shift": (0.1, 0.0, 0.0), "checkpoint_every": 20})


def adjoint_puddle(seed: int = 1, velocity_sigma: float = 0.1, steps: int = 40) -> Scene:
    """The settled-puddle block (17^3 = 4913 particles at corner (0.3, 0.5, 0.3))
    with N(0, sigma^2) initial velocities and the adjoint's fixed 2 divergence
    and 4 density iterations: the finite-difference gradient check case."""
    sc = puddle(seed)
    sc.name = "adjoint_puddle_4913"
    sc.velocity = normal(seed + 100, sc.n, velocity_sigma)
    sc.steps = steps
    sc.max_density_iters, sc.max_divergence_iters = 4, 2
    sc.eta_density, sc.eta_divergence = 0.0, 0.0
    sc.extra = {"target_shift": (0.1, 0.0, 0.0), "checkpoint_every": 20}
    return sc
