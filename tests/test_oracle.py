"""CPU tests that pin the oracle (the C++ restatement of the reference kernels).

The reference's own tests hold no golden vectors for this path (libCL/TEST/main.cpp only
checks sortedness). The oracle is pinned instead by: its restated 4-bit block sort against
the definition of a stable sort, hand-computed hash values, the reference's bounds quirks,
analytic few-particle densities, an independent pure-Python restatement (the fixtures in
tests/golden/, made by make_golden.py), and FP64 agreement."""
from pathlib import Path

import numpy as np
import pytest

import libcl_gb300 as gb
import oracle

GOLDEN = Path(__file__).resolve().parent / "golden"


def _stable(keys, vals, s, e):
    field = (keys.astype(np.uint64) >> np.uint64(s)) & np.uint64((1 << (e - s)) - 1)
    o = np.argsort(field, kind="stable")
    return keys[o], vals[o]


@pytest.mark.parametrize("n", [1, 2, 255, 256, 257, 1000, 65536, 100_003])
@pytest.mark.parametrize("bits", [(0, 32), (0, 24), (8, 20), (28, 32)])
def test_restated_reference_sort_is_a_stable_sort(n, bits):
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    if n > 300:
        keys[::3] = keys[0]  # many duplicates: stability matters
    vals = np.arange(n, dtype=np.uint32)
    k, v = keys.copy(), vals.copy()
    assert oracle.radix_sort_reference(k, v, *bits) == 0
    ek, ev = _stable(keys, vals, *bits)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)
    k2, v2 = keys.copy(), vals.copy()
    oracle.stable_sort(k2, v2, *bits)
    assert np.array_equal(k2, ek) and np.array_equal(v2, ev)


def test_restated_reference_sort_error_codes():
    """oclRadixSort::compute's checks (libCL/sort/oclRadixSort.cpp:64-80)."""
    k = np.zeros(8, np.uint32)
    assert oracle.radix_sort_reference(k, np.zeros(7, np.uint32), 0, 32) == -2
    assert oracle.radix_sort_reference(k, k.copy(), 0, 30) == -4
    big = np.zeros(4194304, np.uint32)
    assert oracle.radix_sort_reference(big, big.copy(), 0, 32) == -3  # n >= cMaxArraySize


def test_reference_sort_smoke_like_the_reference_test():
    """libCL/TEST/main.cpp:133-181: 1024 rand() keys, bits 0..32, keys must not decrease."""
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 2 ** 31, 1024).astype(np.uint32)
    vals = np.arange(1024, dtype=np.uint32)
    assert oracle.radix_sort_reference(keys, vals, 0, 32) == 0
    assert np.all(keys[1:] >= keys[:-1])


def test_hash_known_answers():
    """hashKey by hand: (73856093*x ^ 19349663*y ^ 83492791*z) mod 2^32, then mod 262144."""
    p = gb.default_params()
    cases = {(0, 0, 0): 0,
             (1, 0, 0): 73856093 % 262144,
             (0, 1, 0): 19349663 % 262144,
             (1, 1, 1): (73856093 ^ 19349663 ^ 83492791) % 262144,
             (-1, -1, -1): (((2 ** 32 - 73856093) ^ (2 ** 32 - 19349663) ^ (2 ** 32 - 83492791)) % 2 ** 32) % 262144}
    h = p.cellSize
    pos = np.zeros((len(cases), 4), np.float32)
    for i, c in enumerate(cases):
        pos[i, :3] = [(ci + 0.5) * h for ci in c]
    cell, index = oracle.hash(pos, p)
    assert list(cell) == list(cases.values())
    assert list(index) == list(range(len(cases)))
    assert cases[(1, 0, 0)] == 193629


def test_linear_keys_clamp_to_the_grid():
    p = gb.default_params()
    p.keyMode = gb.KEY_LINEAR_GRID
    p.cellSize = 0.5
    p.gridDim[0], p.gridDim[1], p.gridDim[2] = 4, 3, 2
    pos = np.array([[0.1, 0.1, 0.1, 0], [1.9, 1.4, 0.9, 0], [-5, -5, -5, 0], [50, 50, 50, 0], [0.6, 1.1, 0.6, 0]],
                   np.float32)
    cell, _ = oracle.hash(pos, p)
    assert list(cell) == [0, 3 + 4 * (2 + 3 * 1), 0, 3 + 4 * (2 + 3 * 1), 1 + 4 * (2 + 3 * 1)]


def test_find_bounds_semantics_and_quirks():
    keys = np.array([2, 2, 5, 5, 5, 9], np.uint32)
    cs, ce = oracle.find_bounds(keys, 12)
    assert cs[2] == 0 and ce[2] == 2 and cs[5] == 2 and ce[5] == 5 and cs[9] == 5 and ce[9] == 6
    assert cs[0] == 0xFFFFFFFF and ce[0] == 0xFFFFFFFF
    # reference quirk: particle 0 returns before the last-particle check, so n == 1 leaves
    # cellEnd empty (libCL/phys/oclFluid3D.cl:100-104); the library sets it to 1 instead.
    cs, ce = oracle.find_bounds(np.array([3], np.uint32), 8)
    assert cs[3] == 0 and ce[3] == 0xFFFFFFFF


def test_oracle_matches_independent_python_restatement():
    """The C++ oracle reproduces the pure-Python restatement's fixture bit for bit."""
    g = np.load(GOLDEN / "ref3d_hash_small.npz")
    p = gb.default_params()
    for name, v in zip([f for f, _ in gb.Fluid3DParams._fields_[:13]], g["params"]):
        # clInitFluid's pow() is implementation-defined (OpenCL allows 16 ulp): defaults agree
        # to a few ulp; the step below runs on the fixture's own values
        assert abs(np.float32(getattr(p, name)) - v) <= 4 * np.spacing(np.abs(v)), name
        setattr(p, name, float(v))
    pos, vel, force = g["pos0"].copy(), g["vel0"].copy(), np.zeros_like(g["pos0"])
    r = oracle.step(pos, vel, force, p, ref_sort=True)
    for k, a in (("cell", r.cell), ("index", r.index), ("spos", r.spos), ("svel", r.svel)):
        assert np.array_equal(a.view(np.uint32), g[k].view(np.uint32)), k
    occ = g["occupied"]
    assert np.array_equal(np.nonzero(r.cell_start != 0xFFFFFFFF)[0], occ)
    assert np.array_equal(r.cell_start[occ], g["cell_start"]) and np.array_equal(r.cell_end[occ], g["cell_end"])
    for k, a in (("pos1", pos), ("vel1", vel), ("force1", force)):
        assert np.array_equal(a.view(np.uint32), g[k].view(np.uint32)), k


def _tetra_scene(d, centre):
    """Four particles on a regular tetrahedron of edge d around `centre` (plus one far away)."""
    p = gb.default_params()
    a = d / np.sqrt(2.0)
    pts = np.array([[a, a, a], [a, -a, -a], [-a, a, -a], [-a, -a, a]]) / 2.0 + np.asarray(centre)
    pos = np.zeros((5, 4), np.float32)
    pos[:4, :3] = pts
    pos[4, :3] = [0.9, -0.9, 0.9]
    return p, pos


def _hash_multiplicity(gi, gj):
    """How many of the 27 neighbour offsets of cell gi hash to the bucket of cell gj."""
    import sys
    sys.path.insert(0, str(GOLDEN))
    import pyref
    target = pyref.hash_key(*gj)
    return sum(pyref.hash_key(gi[0] + x, gi[1] + y, gi[2] + z) == target
               for z in (-1, 0, 1) for y in (-1, 0, 1) for x in (-1, 0, 1))


@pytest.mark.parametrize("centre", [(0.41, 0.23, -0.37), (0.0, 0.0, 0.0)])
def test_analytic_density_of_a_tetrahedron(centre):
    """Each vertex has 3 neighbours at distance d (count >= 3 > 2), so rho = mass * K *
    sum over neighbours of m_ij * (h^2 - d^2)^3, where m_ij is the number of times the
    27-cell loop visits j's bucket (libCL/phys/oclFluid3D.cl:160-187). Away from the origin
    m_ij = 1; around the origin the Teschner hash modulo 262144 collides and the reference
    counts some neighbours several times. The lone particle has count 0: rho0 and p0."""
    p, pos = _tetra_scene(0.02, centre)
    cell, index, spos, svel, cs, ce = oracle.front_end(pos, np.zeros_like(pos), p)
    oracle.density(spos, svel, cs, ce, p)
    h = float(p.cellSize)
    g = [tuple(int(np.floor(np.float32(pos[i, k]) / np.float32(h))) for k in range(3)) for i in range(5)]
    rho = {int(index[i]): spos[i, 3] for i in range(5)}
    press = {int(index[i]): svel[i, 3] for i in range(5)}
    mult_total = 0
    for i in range(4):
        want = 0.0
        for j in range(4):
            if j != i:
                d = np.linalg.norm(pos[i, :3].astype(np.float64) - pos[j, :3].astype(np.float64))
                m = _hash_multiplicity(g[i], g[j])
                mult_total += m
                want += m * (h * h - d * d) ** 3
        want = max(1.0, p.mass * p.kernelConstant * want)
        assert abs(rho[i] - want) <= 1e-5 * want
        assert abs(press[i] - p.stiffness * (rho[i] - p.density)) <= 1e-3 * abs(rho[i])
    assert rho[4] == p.density and press[4] == p.pressure
    if centre == (0.0, 0.0, 0.0):
        assert mult_total > 12  # some neighbours visited more than once
    else:
        assert mult_total == 12


def test_two_particles_keep_rest_density():
    """count = 1 <= 2: both particles get rho0 and p0."""
    p = gb.default_params()
    pos = np.array([[0, 0, 0, 0], [0.01, 0, 0, 0]], np.float32)
    cell, index, spos, svel, cs, ce = oracle.front_end(pos, np.zeros_like(pos), p)
    oracle.density(spos, svel, cs, ce, p)
    assert np.all(spos[:, 3] == p.density) and np.all(svel[:, 3] == p.pressure)


def test_fp32_step_agrees_with_fp64_oracle():
    from libcl_gb300.scenes import block_collapse_3d
    sc = block_collapse_3d(16, 8, 16)
    rng = np.random.default_rng(3)
    vel = np.zeros_like(sc.pos)
    vel[:, :3] = rng.normal(0, 0.1, (sc.n, 3))
    pos32, vel32, f32 = sc.pos.copy(), vel.copy(), np.zeros_like(sc.pos)
    r32 = oracle.step(pos32, vel32, f32, sc.params)
    pos64, vel64, f64 = sc.pos.astype(np.float64), vel.astype(np.float64), np.zeros((sc.n, 4))
    r64 = oracle.step_f64(pos64, vel64, f64, sc.params)
    assert np.array_equal(r32.index, r64.index)
    rho_err = np.max(np.abs(r32.spos[:, 3] - r64.spos[:, 3]) / r64.spos[:, 3])
    assert rho_err < 1e-5
    dv32, dv64 = vel32 - vel, vel64 - vel.astype(np.float64)
    scale = np.sqrt(np.mean(dv64 ** 2))
    assert np.max(np.abs(dv32 - dv64)) < 1e-3 * scale


def test_stage_functions_compose_to_the_step():
    """front_end + density + forces + clip + integrate == orc_step."""
    from libcl_gb300.scenes import block_collapse_3d
    sc = block_collapse_3d(12, 6, 12)
    p = sc.params
    pos, vel, f = sc.pos.copy(), sc.vel.copy(), np.zeros_like(sc.pos)
    r = oracle.step(pos, vel, f, p)
    pos2, vel2, f2 = sc.pos.copy(), sc.vel.copy(), np.zeros_like(sc.pos)
    cell, index, spos, svel, cs, ce = oracle.front_end(pos2, vel2, p)
    oracle.density(spos, svel, cs, ce, p)
    oracle.forces(spos, svel, f2, index, cs, ce, p)
    oracle.clip_box(spos, svel, f2, index, p)
    oracle.integrate_force(vel2, f2, p)
    oracle.gravity(f2, p)
    oracle.integrate_velocity(pos2, vel2, p)
    assert np.array_equal(r.spos, spos) and np.array_equal(pos, pos2) and np.array_equal(vel, vel2)
