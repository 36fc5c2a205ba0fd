"""Generates the golden fixtures of this directory with the pure-Python restatement
(pyref.py), independent of the C++ oracle and of the CUDA library.

    python tests/golden/make_golden.py

Writes ref3d_hash_small.npz: a 6x6x6 jittered lattice at the default spacing of clInitFluid,
random velocities, the default parameters with the reference hash, and everything one step
of oclFluid3D::compute produces (sorted keys, permutation, non-empty cell bounds, sorted
position/velocity with density/pressure in .w, and the updated position/velocity/force).
"""
import math
from pathlib import Path

import numpy as np

import pyref

HERE = Path(__file__).resolve().parent


def default_params():
    """clInitFluid (libCL/phys/oclFluid3D.cl:130-148) in float32, double literals in double."""
    F = np.float32
    P = {"deltaTime": F(0.005), "mass": F(0.006), "density": F(1000), "viscosity": F(6.0), "pressure": F(0),
         "velocitylimit": F(500), "stiffness": F(1)}
    # pow() of float arguments: implementation-defined in OpenCL (<= 16 ulp); double pow
    # rounded to float here. Tests load these exact values, so the step does not depend on it.
    P["spacing"] = F(0.87 * float(F(math.pow(float(F(P["mass"] / P["density"])), float(F(1 / 3.0))))))
    P["particleRadius"] = F(0.5 * float(P["spacing"]))
    P["cellSize"] = F(2.0 * float(P["spacing"]))
    pi = float(F(np.pi))
    p9 = float(F(math.pow(float(P["cellSize"]), 9.0)))
    p6 = float(F(math.pow(float(P["cellSize"]), 6.0)))
    P["kernelConstant"] = F(315.0 / (64.0 * pi * p9))
    P["viscosityConstant"] = F(-float(P["viscosity"]) * (-45.0 / (pi * p6)))
    P["pressureConstant"] = F(-(-45.0 / (pi * p6)))
    P["gravity"] = [F(-9.8) * F(0), F(-9.8) * F(0), F(-9.8) * F(1), F(-9.8) * F(0)]
    P["boxMin"] = [F(-1)] * 3
    P["boxMax"] = [F(1)] * 3
    return P


def main():
    P = default_params()
    rng = np.random.default_rng(2011)
    side = 6
    sp = float(P["spacing"])
    g = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:, ::-1]
    pos = np.zeros((side ** 3, 4), np.float32)
    pos[:, :3] = (g * sp - 0.5 * side * sp + rng.uniform(-0.1 * sp, 0.1 * sp, (side ** 3, 3))).astype(np.float32)
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(0, 0.05, (side ** 3, 3)).astype(np.float32)
    force = np.zeros_like(pos)
    pos0, vel0 = pos.copy(), vel.copy()
    cell, index, spos, svel, cs, ce = pyref.step(pos, vel, force, P)
    occupied = np.nonzero(cs != pyref.EMPTY)[0].astype(np.uint32)
    np.savez_compressed(HERE / "ref3d_hash_small.npz", pos0=pos0, vel0=vel0, cell=cell, index=index,
                        spos=spos, svel=svel, occupied=occupied, cell_start=cs[occupied], cell_end=ce[occupied],
                        pos1=pos, vel1=vel, force1=force,
                        params=np.array([P[k] for k in ("deltaTime", "particleRadius", "cellSize", "mass", "viscosity",
                                                        "pressure", "density", "spacing", "stiffness",
                                                        "viscosityConstant", "pressureConstant", "kernelConstant",
                                                        "velocitylimit")], np.float32))
    print("wrote", HERE / "ref3d_hash_small.npz", "n =", pos.shape[0], "occupied cells =", occupied.size)


if __name__ == "__main__":
    main()
