"""Pure-Python restatement of the reference's 3D SPH step for small particle counts.

A second, independent restatement of libCL/phys/oclFluid3D.cl (written separately from the
C++ oracle, in scalar numpy float32 arithmetic with the same operation order) used to make
the golden fixtures in this directory. Test infrastructure only; O(N * neighbours) Python
loops, so keep N in the hundreds.
"""
from __future__ import annotations

import numpy as np

F = np.float32
BUCKETS = 262144
EMPTY = 0xFFFFFFFF


def hash_key(x: int, y: int, z: int) -> int:
    """hashKey, oclFluid3D.cl:44-52, with Python integers reduced mod 2^32."""
    m = 0xFFFFFFFF
    n = ((73856093 * (x & m)) & m) ^ ((19349663 * (y & m)) & m) ^ ((83492791 * (z & m)) & m)
    return n % BUCKETS


def grid_position(p, h):
    """gridPosition, oclFluid3D.cl:34-42: (int)floor(p / h) per axis, in float32."""
    return tuple(int(np.floor(F(p[i]) / F(h))) for i in range(3))


def find_bounds(cell, n_cells):
    """fill 0xFFFFFFFF + clFindBounds (oclFluid3D.cl:85-113)."""
    cs = np.full(n_cells, EMPTY, np.uint32)
    ce = np.full(n_cells, EMPTY, np.uint32)
    n = len(cell)
    for p in range(n):
        if p == 0:
            cs[cell[0]] = 0
            continue
        if cell[p] != cell[p - 1]:
            ce[cell[p - 1]] = p
            cs[cell[p]] = p
        if p == n - 1:
            ce[cell[p]] = n
    return cs, ce


def flen(x, y, z):
    return F(np.sqrt(F(F(F(x * x) + F(y * y)) + F(z * z))))


def step(pos, vel, force, P):
    """One oclFluid3D::compute with the reference hash; P is a dict of float32 params.
    Returns (cell, index, spos, svel, cs, ce) and updates pos/vel/force in place."""
    n = pos.shape[0]
    h = F(P["cellSize"])
    cell = np.array([hash_key(*grid_position(pos[i], h)) for i in range(n)], np.uint32)
    index = np.argsort(cell, kind="stable").astype(np.uint32)
    cell = cell[index]
    spos = pos[index].copy()
    svel = vel[index].copy()
    cs, ce = find_bounds(cell, BUCKETS)
    fpos = spos.copy()

    def neighbours(i):
        g = grid_position(fpos[i], h)
        for z in (-1, 0, 1):
            for y in (-1, 0, 1):
                for x in (-1, 0, 1):
                    c = hash_key(g[0] + x, g[1] + y, g[2] + z)
                    if cs[c] != EMPTY:
                        yield from range(int(cs[c]), int(ce[c]))

    for i in range(n):  # clCalculateDensity, :150-200
        d, count = F(0), 0
        for j in neighbours(i):
            if j == i:
                continue
            vlen = flen(F(spos[i, 0] - spos[j, 0]), F(spos[i, 1] - spos[j, 1]), F(spos[i, 2] - spos[j, 2]))
            if vlen < h:
                t = F(F(h * h) - F(vlen * vlen))
                d = F(d + F(F(t * t) * t))
                count += 1
        if count > 2:
            rho = max(F(1.0), F(F(F(P["mass"]) * F(P["kernelConstant"])) * d))
            spos[i, 3] = rho
            svel[i, 3] = F(F(P["pressure"]) + F(F(P["stiffness"]) * F(rho - F(P["density"]))))
        else:
            spos[i, 3] = F(P["density"])
            svel[i, 3] = F(P["pressure"])
    for i in range(n):  # clCalculateForces, :202-255
        acc = [F(0)] * 6
        for j in neighbours(i):
            if j == i:
                continue
            v = [F(spos[i, k] - spos[j, k]) for k in range(3)]
            vlen = flen(*v)
            if vlen < h:
                d2 = F(spos[i, 3] * spos[j, 3])
                s = F(F(svel[i, 3] + svel[j, 3]) / d2)
                hr = F(h - vlen)
                for k in range(3):
                    acc[k] = F(acc[k] + F(s * F(F(F(v[k] / vlen) * hr) * hr)))
                    acc[3 + k] = F(acc[3 + k] + F(F(F(svel[j, k] - svel[i, k]) / d2) * hr))
        o = index[i]
        for k in range(3):
            force[o, k] = F(force[o, k] + F(F(F(F(P["pressureConstant"]) * acc[k]) +
                                              F(F(P["viscosityConstant"]) * acc[3 + k])) * F(P["mass"])))
        force[o, 3] = F(0)
    r = F(P["particleRadius"])
    for i in range(n):  # clClipBox, :309-361
        o = index[i]
        walls = ((1, F(1), F(r - F(spos[i, 1] - F(P["boxMin"][1])))),
                 (1, F(-1), F(r - F(F(P["boxMax"][1]) - spos[i, 1]))),
                 (2, F(1), F(r - F(spos[i, 2] - F(P["boxMin"][2])))),
                 (2, F(-1), F(r - F(F(P["boxMax"][2]) - spos[i, 2]))),
                 (0, F(1), F(r - F(spos[i, 0] - F(P["boxMin"][0])))),
                 (0, F(-1), F(r - F(F(P["boxMax"][0]) - spos[i, 0]))))
        for axis, sign, diff in walls:
            if diff > F(0.00001):
                mag = F(F(F(2000) * diff) - F(F(256) * F(sign * svel[i, axis])))
                force[o, axis] = F(force[o, axis] + F(sign * mag))
                force[o, 3] = F(force[o, 3] + F(F(0) * mag))
    dt = F(P["deltaTime"])
    for i in range(n):  # clIntegrateForce, :258-271
        f = force[i].copy()
        speed = F(np.sqrt(F(F(F(F(f[0] * f[0]) + F(f[1] * f[1])) + F(f[2] * f[2])) + F(f[3] * f[3]))))
        if speed > F(P["velocitylimit"]):
            f = (f * F(F(P["velocitylimit"]) / speed)).astype(F)
        vel[i] = (vel[i] + (f * dt).astype(F)).astype(F)
    force[:] = np.array(P["gravity"], F)  # clGravity, :294-298
    pos[:] = (pos + (vel * dt).astype(F)).astype(F)  # clIntegrateVelocity, :284-291
    return cell, index, spos, svel, cs, ce
