"""Seeded synthetic scenes for the SPH step (host numpy arrays, float4 per particle).

The reference has no datasets; these generators build the jittered lattices its
configurations describe. All randomness comes from `SplitMix64` (a published 64-bit
generator, Steele et al. 2014) so that the same seed gives the same scene on x86 and Arm.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import Fluid3DParams, KEY_LINEAR_GRID, params_derive

_M64 = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 stream; uniform() maps the top 24 bits to [0, 1)."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & _M64)

    def next_u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            idx = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + idx * np.uint64(0x9E3779B97F4A7C15)
            self.state = self.state + np.uint64(n) * np.uint64(0x9E3779B97F4A7C15)
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            return z ^ (z >> np.uint64(31))

    def uniform(self, n: int) -> np.ndarray:
        return (self.next_u64(n) >> np.uint64(40)).astype(np.float64) / float(1 << 24)

    def normal(self, n: int) -> np.ndarray:
        """Box-Muller on pairs of uniforms."""
        m = (n + 1) // 2
        u1 = np.maximum(self.uniform(m), 1.0 / (1 << 25))
        u2 = self.uniform(m)
        r = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
        return z[:n]


@dataclasses.dataclass
class Scene3D:
    name: str
    pos: np.ndarray      # float32 [N, 4]
    vel: np.ndarray      # float32 [N, 4]
    params: Fluid3DParams

    @property
    def n(self) -> int:
        return self.pos.shape[0]


def lattice(nx: int, ny: int, nz: int, spacing: float, origin, jitter: float, seed: int) -> np.ndarray:
    """Jittered lattice, x fastest; float32 [nx*ny*nz, 4] with w = 0."""
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    p = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64) * spacing
    p += np.asarray(origin, dtype=np.float64)[None, :]
    rng = SplitMix64(seed)
    p += (rng.uniform(p.size).reshape(p.shape) * 2.0 - 1.0) * jitter
    out = np.zeros((p.shape[0], 4), dtype=np.float32)
    out[:, :3] = p
    return out


def fluid_params(h: float, spacing: float, mass: float, rho0: float, stiffness: float,
                 viscosity: float, dt: float, gravity, box_min, box_max, grid_dim,
                 grid_origin=(0.0, 0.0, 0.0), dims: int = 3, velocity_limit: float = 500.0) -> Fluid3DParams:
    p = Fluid3DParams()
    p.deltaTime = dt
    p.particleRadius = 0.5 * spacing
    p.cellSize = h
    p.mass = mass
    p.viscosity = viscosity
    p.pressure = 0.0
    p.density = rho0
    p.spacing = spacing
    p.stiffness = stiffness
    p.velocitylimit = velocity_limit
    p.dims = dims
    params_derive(p)
    for i in range(3):
        p.gravity[i] = gravity[i]
        p.boxMin[i] = box_min[i]
        p.boxMax[i] = box_max[i]
        p.gridOrigin[i] = grid_origin[i]
        p.gridDim[i] = grid_dim[i]
    p.keyMode = KEY_LINEAR_GRID
    return p


def block_collapse_3d(nx: int = 128, ny: int = 64, nz: int = 128, seed: int = 2) -> Scene3D:
    """3D block collapse: nx*ny*nz particles (default 1,048,576) on a lattice of spacing 0.5h
    (h = 0.02), jittered by uniform +-0.05h, resting in the corner of a [0,4]x[0,2]x[0,4]
    box; gravity -9.81 along y, rest density 1000, gas constant 3.0, viscosity 0.05,
    dt = 5e-5, 200x100x200 linear cell grid. The particle mass, rho0*(0.5h)^3 = 1e-3, is a
    choice of this generator (the configuration does not give it)."""
    h, sp = 0.02, 0.01
    pos = lattice(nx, ny, nz, sp, (0.5 * sp, 0.5 * sp, 0.5 * sp), 0.05 * h, seed)
    vel = np.zeros_like(pos)
    prm = fluid_params(h, sp, 1000.0 * sp ** 3, 1000.0, 3.0, 0.05, 5e-5, (0.0, -9.81, 0.0),
                       (0.0, 0.0, 0.0), (4.0, 2.0, 4.0), (200, 100, 200))
    return Scene3D(f"block_collapse_{nx}x{ny}x{nz}", pos, vel, prm)


def differentiable_block(nx: int = 64, ny: int = 32, nz: int = 32, seed: int = 3) -> Scene3D:
    """The differentiable-rollout scene: nx*ny*nz particles (default 65,536) on a lattice of
    spacing 0.01 (h = 0.02) jittered by uniform +-0.05h at the lower corner of a box twice the
    block's extent per axis (here [0,1.28]x[0,0.64]x[0,0.64], a 64x32x32 cell grid), at rest;
    gravity -9.81 along y, rest density 1000, mass 1e-3, gas constant 3.0, viscosity 0.05,
    dt = 5e-5 (the box, gas constant, primal viscosity and dt are choices of this generator)."""
    h, sp = 0.02, 0.01
    pos = lattice(nx, ny, nz, sp, (0.5 * sp, 0.5 * sp, 0.5 * sp), 0.05 * h, seed)
    vel = np.zeros_like(pos)
    box = 2.0 * np.array([nx, ny, nz], np.float64) * sp
    prm = fluid_params(h, sp, 1000.0 * sp ** 3, 1000.0, 3.0, 0.05, 5e-5, (0.0, -9.81, 0.0),
                       (0.0, 0.0, 0.0), tuple(box), tuple(int(np.ceil(b / h - 1e-9)) for b in box))
    return Scene3D(f"differentiable_block_{nx}x{ny}x{nz}", pos, vel, prm)


def perturbed_velocities(vel: np.ndarray, sigma: float = 0.1, seed: int = 6) -> np.ndarray:
    """vel + N(0, sigma^2) per component (x, y, z), float32 [N, 4]: the target run's initial
    velocities of the differentiable rollout."""
    out = vel.copy()
    n = vel.shape[0]
    out[:, :3] += (SplitMix64(seed).normal(3 * n).reshape(n, 3) * sigma).astype(np.float32)
    return out


def dam_break_2d(nx: int = 128, ny: int = 128, seed: int = 1) -> Scene3D:
    """2D dam break: 128x128 particles (spacing 0.5h, h = 0.01) jittered +-0.05h, anchored at
    the lower-left corner of a [0,1]x[0,1] box; gravity -9.81, rest density 1000, gas constant
    3.0, viscosity 0.1, dt = 1e-4, 100x100 cell grid. Mass rho0*(0.5h)^2 = 0.025 (generator's
    choice). The 128x128 block at spacing 0.005 spans 0.64 x 0.64, more than the left quarter
    of the box that the configuration names, so it is anchored at the wall instead."""
    h, sp = 0.01, 0.005
    pos = lattice(nx, ny, 1, sp, (0.5 * sp, 0.5 * sp, 0.0), 0.05 * h, seed)
    pos[:, 2] = 0.0
    vel = np.zeros_like(pos)
    prm = fluid_params(h, sp, 1000.0 * sp ** 2, 1000.0, 3.0, 0.1, 1e-4, (0.0, -9.81, 0.0),
                       (0.0, 0.0, -1.0), (1.0, 1.0, 1.0), (100, 100, 1), dims=2)
    return Scene3D(f"dam_break_2d_{nx}x{ny}", pos, vel, prm)


def reference_test_scene(n: int = 256, seed: int = 7) -> Scene3D:
    """The reference's smoke scene (libCL/TEST/main.cpp:188-240): n particles uniform in
    [-0.5, 0.5]^3 with the default parameters of clInitFluid and the reference hash keys.
    (The reference draws from rand(); here the seeded SplitMix64 stands in.)"""
    from . import default_params
    rng = SplitMix64(seed)
    pos = np.zeros((n, 4), dtype=np.float32)
    pos[:, :3] = (rng.uniform(3 * n).reshape(n, 3) - 0.5).astype(np.float32)
    vel = np.zeros_like(pos)
    return Scene3D(f"reference_smoke_{n}", pos, vel, default_params())


def clone_params(p: Fluid3DParams) -> Fluid3DParams:
    q = Fluid3DParams()
    import ctypes
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(Fluid3DParams))
    return q


@dataclasses.dataclass
class BatchScenes:
    """A batch of independent 3D scenes: concatenated float4 state plus per-scene descriptions."""
    shared: Fluid3DParams
    descs: list
    pos: np.ndarray
    vel: np.ndarray
    firsts: list

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    def scene(self, s: int) -> Scene3D:
        """Scene s as a stand-alone Scene3D (same parameters, same particles)."""
        d = self.descs[s]
        p = clone_params(self.shared)
        p.stiffness = d.stiffness
        p.viscosity = d.viscosity
        p.dims = 3
        params_derive(p)
        for i in range(3):
            p.boxMin[i], p.boxMax[i] = d.boxMin[i], d.boxMax[i]
            p.gridOrigin[i], p.gridDim[i] = d.gridOrigin[i], d.gridDim[i]
        p.keyMode = KEY_LINEAR_GRID
        a, n = self.firsts[s], d.n_particles
        return Scene3D(f"scene{s}", self.pos[a:a + n].copy(), self.vel[a:a + n].copy(), p)


def batched_ensemble(n_scenes: int = 256, seed: int = 5, n_min: int = 4096, n_max: int = 262144) -> BatchScenes:
    """Independent scenes with particle counts drawn log-uniform in [n_min, n_max]: each a
    near-cubic jittered lattice block (spacing 0.01, h = 0.02, jitter +-0.05h) at the lower
    corner of its own box, twice the block's extent per axis (a choice of this generator);
    gas constant uniform in [1, 5], viscosity uniform in [0.01, 0.2]; dt = 5e-5, gravity -9.81
    along y, rest density 1000, mass 1e-3."""
    from . import SceneDesc
    h, sp = 0.02, 0.01
    rng = SplitMix64(seed)
    u = rng.uniform(4 * n_scenes).reshape(n_scenes, 4)
    counts = np.exp(np.log(n_min) + u[:, 0] * (np.log(n_max) - np.log(n_min)))
    shared = fluid_params(h, sp, 1000.0 * sp ** 3, 1000.0, 3.0, 0.05, 5e-5, (0.0, -9.81, 0.0),
                          (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (1, 1, 1))
    descs, pos_l, firsts, first = [], [], [], 0
    for s in range(n_scenes):
        side = max(2, int(round(counts[s] ** (1.0 / 3.0))))
        nx, ny, nz = side, side, max(1, int(round(counts[s] / (side * side))))
        p = lattice(nx, ny, nz, sp, (0.5 * sp,) * 3, 0.05 * h, seed * 1000 + s)
        ext = np.array([nx, ny, nz], np.float64) * sp
        box = 2.0 * ext
        d = SceneDesc()
        d.n_particles = p.shape[0]
        d.stiffness = float(1.0 + 4.0 * u[s, 1])
        d.viscosity = float(0.01 + 0.19 * u[s, 2])
        for i in range(3):
            d.boxMin[i] = 0.0
            d.boxMax[i] = float(box[i])
            d.gridOrigin[i] = 0.0
            d.gridDim[i] = int(np.ceil(box[i] / h))
        descs.append(d)
        pos_l.append(p)
        firsts.append(first)
        first += p.shape[0]
    pos = np.concatenate(pos_l)
    return BatchScenes(shared, descs, pos, np.zeros_like(pos), firsts)


def triangle_soup(n: int, seed: int = 21, extent: float = 1.0, size: float = 0.01):
    """n independent small triangles: centres uniform in [0, extent]^3 (SplitMix64), vertices
    within +-size of the centre. Returns (vertex float32 [3n, 4] with w = 1, index uint32 [3n])."""
    rng = SplitMix64(seed)
    c = rng.uniform(3 * n).reshape(n, 1, 3) * extent
    d = (rng.uniform(9 * n).reshape(n, 3, 3) * 2.0 - 1.0) * size
    v = np.ones((3 * n, 4), np.float32)
    v[:, :3] = (c + d).reshape(3 * n, 3)
    return v, np.arange(3 * n, dtype=np.uint32)


def sphere_mesh(n_lat: int = 64, n_lon: int = 128, radius: float = 0.5, centre=(1.0, 1.0, 1.0)):
    """A UV sphere: (n_lat - 1) * n_lon + 2 shared vertices, 2 * n_lon * (n_lat - 1) triangles.
    Returns (vertex float32 [V, 4] with w = 0, index uint32 [3T])."""
    verts = [(0.0, 0.0, radius)]
    for i in range(1, n_lat):
        th = np.pi * i / n_lat
        for j in range(n_lon):
            ph = 2.0 * np.pi * j / n_lon
            verts.append((radius * np.sin(th) * np.cos(ph), radius * np.sin(th) * np.sin(ph), radius * np.cos(th)))
    verts.append((0.0, 0.0, -radius))
    v = np.zeros((len(verts), 4), np.float32)
    v[:, :3] = np.asarray(verts) + np.asarray(centre)
    tris = []
    for j in range(n_lon):  # north cap
        tris.append((0, 1 + j, 1 + (j + 1) % n_lon))
    for i in range(n_lat - 2):
        a, b = 1 + i * n_lon, 1 + (i + 1) * n_lon
        for j in range(n_lon):
            jn = (j + 1) % n_lon
            tris.append((a + j, b + j, b + jn))
            tris.append((a + j, b + jn, a + jn))
    last, south = 1 + (n_lat - 2) * n_lon, len(verts) - 1
    for j in range(n_lon):  # south cap
        tris.append((last + j, south, last + (j + 1) % n_lon))
    return v, np.asarray(tris, np.uint32).ravel()


def lattice_soup(k: int = 100, seed: int = 22, size: float = 0.002):
    """k^3 small triangles centred on a jittered k x k x k lattice in [0.05, 1.05]^3 (one per
    lattice cell, so with k <= 1024 their Morton keys are distinct), shuffled. Returns (vertex
    float32 [3 k^3, 4] with w = 1, index uint32 [3 k^3])."""
    rng = SplitMix64(seed)
    n = k ** 3
    iz, iy, ix = np.meshgrid(np.arange(k), np.arange(k), np.arange(k), indexing="ij")
    c = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    c = 0.05 + (c + 0.25 + 0.5 * rng.uniform(3 * n).reshape(n, 3)) / k
    c = c[np.argsort(rng.next_u64(n), kind="stable")]
    d = (rng.uniform(9 * n).reshape(n, 3, 3) * 2.0 - 1.0) * size
    v = np.ones((3 * n, 4), np.float32)
    v[:, :3] = (c[:, None, :] + d).reshape(3 * n, 3)
    return v, np.arange(3 * n, dtype=np.uint32)


def segment_soup(n: int, seed: int = 23, extent: float = 65000.0, size: float = 20.0):
    """n independent 2D line segments: midpoints uniform in [0, extent)^2 (SplitMix64), ends
    within +-size of the midpoint, in the integer pixel space oclBvhLines keys on. Returns
    vertex float32 [2n, 2] (two vertices per segment)."""
    rng = SplitMix64(seed)
    c = rng.uniform(2 * n).reshape(n, 1, 2) * extent + size
    d = (rng.uniform(2 * n).reshape(n, 1, 2) * 2.0 - 1.0) * size
    v = np.concatenate([c - d, c + d], axis=1)
    return v.reshape(2 * n, 2).astype(np.float32)


def segment_lattice(k: int = 1000, seed: int = 24):
    """k^2 short segments whose midpoints sit on distinct integer points of a k x k lattice
    (spacing 64, so their Morton keys are distinct for k <= 1024), shuffled. Returns vertex
    float32 [2 k^2, 2]."""
    rng = SplitMix64(seed)
    n = k * k
    iy, ix = np.meshgrid(np.arange(k), np.arange(k), indexing="ij")
    c = np.stack([ix.ravel(), iy.ravel()], axis=1).astype(np.float64) * 64.0 + 16.5
    c = c[np.argsort(rng.next_u64(n), kind="stable")]
    d = (rng.uniform(2 * n).reshape(n, 2) * 2.0 - 1.0) * 8.0
    v = np.stack([c - d, c + d], axis=1)
    return v.reshape(2 * n, 2).astype(np.float32)

