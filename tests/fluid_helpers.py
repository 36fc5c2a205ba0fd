"""Shared helpers for the fluid tests: loading a scene into a Fluid3D, reading its state,
running the oracle on the same inputs, and the FP32 tolerance used for non-bit-exact paths."""
from __future__ import annotations

import ctypes

import numpy as np

from libcl_gb300 import (BUF_FORCE, BUF_POSITION, BUF_VELOCITY, OPT_CUDA_GRAPH, OPT_FUSED, Fluid3D,
                         Fluid3DParams)
from libcl_gb300.scenes import Scene3D, SplitMix64, clone_params, lattice

# Tolerance of the fast (FMA, rsqrt, reordered sums) kernels against the FP32 restatement,
# per component: |gpu - ref| <= RTOL * (|ref| + RMS(ref)). Bit-exact paths compare with ==.
RTOL = 2e-4


def hash_block(nside: int = 24, seed: int = 11) -> Scene3D:
    """A lattice at the default spacing of clInitFluid, centred in the reference's [-1,1]^3
    box, with the default parameters and the reference hash keys."""
    from libcl_gb300 import default_params
    p = default_params()
    sp = p.spacing
    pos = lattice(nside, nside, nside, sp, (-0.5 * nside * sp,) * 3, 0.1 * sp, seed)
    return Scene3D(f"hash_block_{nside}", pos, np.zeros_like(pos), p)


def set_params(fluid: Fluid3D, params: Fluid3DParams) -> None:
    ctypes.memmove(ctypes.byref(fluid.getParameters()), ctypes.byref(params), ctypes.sizeof(Fluid3DParams))


def make_fluid(scene: Scene3D, fused: bool = True, graph: bool = True, vel=None, force=None) -> Fluid3D:
    import torch
    f = Fluid3D()
    f.compile()
    f.setParticleCount(scene.n)
    set_params(f, scene.params)
    f.set_option(OPT_FUSED, int(fused))
    f.set_option(OPT_CUDA_GRAPH, int(graph))
    f.getPositionBuffer().copy_(torch.from_numpy(scene.pos))
    f.getVelocityBuffer().copy_(torch.from_numpy(scene.vel if vel is None else vel))
    f.getForceBuffer().copy_(torch.from_numpy(np.zeros_like(scene.pos) if force is None else force))
    torch.cuda.synchronize()
    return f


def state(f: Fluid3D):
    import torch
    torch.cuda.synchronize()
    return {k: f.buffer(w).cpu().numpy().copy() for k, w in
            (("pos", BUF_POSITION), ("vel", BUF_VELOCITY), ("force", BUF_FORCE))}


def sorted_outputs(f: Fluid3D, n_cells: int):
    import torch
    cs, ce = f.cell_bounds(n_cells)
    torch.cuda.synchronize()
    return {
        "cell": f.getCellBuffer().cpu().numpy().view(np.uint32).copy(),
        "index": f.getIndexBuffer().cpu().numpy().view(np.uint32).copy(),
        "spos": f.getSortedPositionBuffer().cpu().numpy().copy(),
        "svel": f.getSortedVelocityBuffer().cpu().numpy().copy(),
        "cell_start": cs.cpu().numpy().view(np.uint32).copy(),
        "cell_end": ce.cpu().numpy().view(np.uint32).copy(),
    }


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a-b| / (|b| + RMS(b)) over all entries."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = np.sqrt(np.mean(b * b)) + 1e-30
    return float(np.max(np.abs(a - b) / (np.abs(b) + scale)))


def pos_err(new: np.ndarray, ref: np.ndarray, prev: np.ndarray, ulps: float = 4.0) -> float:
    """Position check that stays meaningful when a step moves particles by less than one ulp:
    max |new - ref| / (ulps * ulp(|ref|) + RTOL * (|ref - prev| + RMS(ref - prev))). <= 1 passes."""
    new = np.asarray(new, np.float64)
    ref64 = np.asarray(ref, np.float64)
    d = ref64 - np.asarray(prev, np.float64)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    den = ulps * ulp + RTOL * (np.abs(d) + np.sqrt(np.mean(d * d)) + 1e-30)
    return float(np.max(np.abs(new - ref64) / den))


def perturbed(scene: Scene3D, seed: int = 5, sigma: float = 0.05) -> np.ndarray:
    rng = SplitMix64(seed)
    v = np.zeros_like(scene.pos)
    v[:, :3] = (rng.normal(3 * scene.n).reshape(scene.n, 3) * sigma).astype(np.float32)
    return v


__all__ = ["hash_block", "make_fluid", "state", "sorted_outputs", "rel_err", "pos_err", "RTOL", "set_params",
           "clone_params", "perturbed"]


def emitter_expected(pos: np.ndarray, vel: np.ndarray, emit: int, speed: float, radius: float):
    """The state clEmitter (libCL/phys/oclFluid3D.cl:273-282) leaves: particles emit+1 ..
    emit+99 go to a 10-wide sheet at y = 0.6 with velocity (0, speed, 0, 1). index = emit -
    particle is negative; / and % truncate as in C. The z lane adds the float product
    index%10*2*radius to the double literal 0.6 in double, then rounds to float."""
    pos, vel = pos.copy(), vel.copy()
    r = np.float32(radius)
    for p in range(emit + 1, min(emit + 100, pos.shape[0])):
        index = emit - p
        q, m = int(index / 10), int(np.fmod(index, 10))
        pos[p] = [np.float32(q * 2) * r, 0.6, np.float32(0.6 + np.float64(np.float32(m * 2) * r)), 1.0]
        vel[p] = [0.0, speed, 0.0, 1.0]
    return pos.astype(np.float32), vel.astype(np.float32)
