"""Scenes for the reference's 2D relaxation model (oclFluid2D): a block of particles in the
17.68 x 15.76 container with a wall mask around the container's edge."""
import numpy as np

from libcl_gb300.scenes import SplitMix64


def box_mask(w: int = 256, h: int = 256, thickness: int = 8) -> np.ndarray:
    """[h, w, 4] float32 RGBA mask; .w == 1 on a frame `thickness` pixels wide."""
    m = np.zeros((h, w, 4), np.float32)
    m[:thickness, :, 3] = 1
    m[-thickness:, :, 3] = 1
    m[:, :thickness, 3] = 1
    m[:, -thickness:, 3] = 1
    return m


def block_state(nx: int = 128, ny: int = 128, spacing: float = 0.06, origin=(1.0, 1.0), seed: int = 8) -> np.ndarray:
    """gbsph_particle2d[nx*ny] as float32 [N, 6]: jittered lattice, zero velocity, mass 0.7."""
    iy, ix = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    rng = SplitMix64(seed)
    n = nx * ny
    st = np.zeros((n, 6), np.float32)
    st[:, 0] = origin[0] + ix.ravel() * spacing + (rng.uniform(n) - 0.5) * 0.1 * spacing
    st[:, 1] = origin[1] + iy.ravel() * spacing + (rng.uniform(n) - 0.5) * 0.1 * spacing
    st[:, 4] = 0.7
    return st


def emitter2d_expected(state: np.ndarray, emit: int, particle_size: float) -> np.ndarray:
    """The state clEmitter (libCL/phys/oclFluid2D.cl:342-352) leaves: only particle emit+1
    moves, to (1, 14 + (p%4)*12*particleSize) with velocity (25, 1) and age 1."""
    want = state.copy()
    p = emit + 1
    if p < state.shape[0]:
        want[p, :4] = [1.0, np.float32(14.0) + np.float32(p % 4 * 12) * np.float32(particle_size), 25.0, 1.0]
        want[p, 5] = 1.0
    return want
