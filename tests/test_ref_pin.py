"""Pins the oracle restatement to the reference's own kernels (CPU).

oracle/ref/build.py compiles the reference's OpenCL C sources (libCL/phys/oclFluid3D.cl,
libCL/phys/oclFluid2D.cl, libCL/sort/oclRadixSort.cl, libCL/geom/oclBvhTrimesh.cl,
libCL/geom/oclBvhLines.cl) for the host cores through the shim oracle/ref/clshim.h, and
oracle/ref/*.cpp enqueue them as the reference's host classes do (oclFluid3D::compute,
oclFluid2D::compute and computeBorder, oclRadixSort::compute, oclBvhTrimesh::compute,
oclBvhLines::compute). Each test here runs those kernels and the oracle (oracle/*.cpp) on the
same inputs and requires the same bits: sort, keys, permutation, cell bounds, densities,
pressures, forces, positions, velocities, wall images, parameter defaults, emitters, the BVH
builds and the BVH collision. The GPU tests compare the CUDA library with the oracle, so
they inherit this pin.

The shim fixes what OpenCL leaves to the implementation as the oracle does (fast_length and
length as sqrtf of the left-to-right sum of squares, IEEE division, pow(x, 3.0f) as x*x*x);
test_pow_convention_moves_density_by_ulps measures what the pow choice changes.
"""
import numpy as np
import pytest

import libcl_gb300 as gb
import oracle
import oracle.ref as ref
from fluid_helpers import emitter_expected, hash_block
from libcl_gb300.scenes import SplitMix64, block_collapse_3d, sphere_mesh
from scenes2d import block_state, box_mask, emitter2d_expected

pytestmark = pytest.mark.skipif(not ref.available(), reason="reference kernels not built (no reference checkout)")


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_same_bits(a, b, what):
    a, b = bits(a), bits(b)
    bad = np.argwhere(a != b)
    assert bad.size == 0, f"{what}: {len(bad)} words differ, first at {bad[:3].tolist()}"


# ---------------------------------------------------------------------------------------
# Sort (libCL/sort/oclRadixSort.cl, oclRadixSort::compute)
# ---------------------------------------------------------------------------------------
def _keys(dist, n, rng):
    if dist == "uniform":
        return rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    if dist == "few":
        return rng.integers(0, 7, n, dtype=np.uint64).astype(np.uint32) * np.uint32(0x01010101)
    # Morton-like: interleaved lattice cells with 0-20 entries per occupied cell
    cells = rng.integers(0, 1 << 18, max(1, n // 8), dtype=np.uint64).astype(np.uint32)
    return np.sort(cells[rng.integers(0, cells.size, n)])[::-1].copy()


@pytest.mark.parametrize("n", [1, 255, 256, 4097, 65536, 100_003])
@pytest.mark.parametrize("bits_", [(0, 24), (0, 32), (4, 12), (8, 32)])
@pytest.mark.parametrize("dist", ["uniform", "few", "cells"])
def test_sort_matches_the_reference_kernels(n, bits_, dist):
    rng = np.random.default_rng(n * 7 + bits_[0])
    keys = _keys(dist, n, rng)
    vals = np.arange(n, dtype=np.uint32)
    k_ref, v_ref = keys.copy(), vals.copy()
    assert ref.radix_sort(k_ref, v_ref, *bits_) == 0
    k_orc, v_orc = keys.copy(), vals.copy()
    assert oracle.radix_sort_reference(k_orc, v_orc, *bits_) == 0
    k_def, v_def = keys.copy(), vals.copy()
    oracle.stable_sort(k_def, v_def, *bits_)
    for k, v, what in ((k_orc, v_orc, "oracle block sort"), (k_def, v_def, "stable sort")):
        assert_same_bits(k, k_ref, what + " keys")
        assert_same_bits(v, v_ref, what + " values")


def test_sort_refusals_match_the_reference():
    big = np.zeros(4_194_304, np.uint32)
    assert ref.radix_sort(big, big.copy(), 0, 24) == oracle.radix_sort_reference(big, big.copy(), 0, 24) == -3
    k = np.arange(10, dtype=np.uint32)
    assert ref.radix_sort(k, k.copy(), 0, 6) == oracle.radix_sort_reference(k, k.copy(), 0, 6) == -4


# ---------------------------------------------------------------------------------------
# 3D step (libCL/phys/oclFluid3D.cl, oclFluid3D::compute)
# ---------------------------------------------------------------------------------------
def test_init_fluid_defaults_match_the_reference():
    """clInitFluid's 13 values: the oracle's restatement, the library's compile() defaults."""
    want = ref.init_fluid3d()
    o = gb.Fluid3DParams()
    oracle.init_fluid_params(o)
    assert_same_bits(ref.system13(o), want, "oracle defaults")
    assert_same_bits(ref.system13(gb.default_params()), want, "library defaults")


@pytest.mark.parametrize("h,mu", [(0.02, 0.05), (0.0316179, 6.0), (0.01, 0.1), (0.05, 0.2), (0.0173, 0.01)])
def test_kernel_constants_match_the_reference_macros(h, mu):
    """gbsph_fluid3d_params_derive and the oracle's restatement against DensityConstant /
    PressureConstant / ViscosityConstant as clInitFluid applies them
    (libCL/phys/oclFluid3D.cl:123-147)."""
    p = gb.Fluid3DParams()
    p.cellSize, p.viscosity, p.dims = h, mu, 3
    gb.params_derive(p)
    got = np.array([p.kernelConstant, p.viscosityConstant, p.pressureConstant], np.float32)
    want = ref.kernel_constants(np.float32(h), np.float32(mu))
    assert_same_bits(got, want, "library kernel constants")
    assert_same_bits(oracle.kernel_constants(np.float32(h), np.float32(mu)), want, "oracle kernel constants")


def _hash_mode(params, gravity_arg):
    """The library's params set up as the reference runs: hash keys, and the gravity stage's
    value -9.8f * gravity_arg (clGravity, libCL/phys/oclFluid3D.cl:294-298)."""
    p = gb.Fluid3DParams.from_buffer_copy(bytes(params))
    p.keyMode = gb.KEY_REFERENCE_HASH
    g = np.float32(-9.8) * np.asarray(gravity_arg, np.float32)
    for i in range(4):
        p.gravity[i] = float(g[i])
    return p


def _run_both(pos, vel, params, gravity_arg, steps):
    p = _hash_mode(params, gravity_arg)
    sysv = ref.system13(p)
    lo = np.array(list(p.boxMin), np.float32)
    hi = np.array(list(p.boxMax), np.float32)
    a = [pos.copy(), vel.copy(), np.zeros_like(pos)]
    b = [pos.copy(), vel.copy(), np.zeros_like(pos)]
    for s in range(steps):
        r = ref.step3d(*a, sysv, gravity_arg, lo, hi)
        o = oracle.step(*b, p, ref_sort=(s % 2 == 1))
        for name in ("cell", "index", "spos", "svel", "cell_start", "cell_end"):
            assert_same_bits(getattr(o, name), getattr(r, name), f"step {s} {name}")
        for name, x, y in zip(("pos", "vel", "force"), b, a):
            assert_same_bits(x, y, f"step {s} {name}")
    return a


def test_reference_default_scene_steps_bit_exact():
    """clInitFluid's parameters, a jittered lattice centred in the reference's [-1,1]^3 box
    (negative cells, hash collisions around the origin), the reference's gravity argument
    (0,0,1,0): five steps."""
    sc = hash_block(24)
    a = _run_both(sc.pos, sc.vel, sc.params, (0, 0, 1, 0), 5)
    assert np.isfinite(a[0]).all()


def test_block_collapse_steps_bit_exact():
    """The block-collapse scene (h = 0.02, spacing 0.5h, [0,4]x[0,2]x[0,4] box) on the
    reference's hash keys, gravity -9.8f * (0, 9.81f/9.8f, 0): six steps."""
    sc = block_collapse_3d(32, 16, 32)
    garg = (0.0, np.float32(9.81) / np.float32(9.8), 0.0, 0.0)
    _run_both(sc.pos, sc.vel, sc.params, garg, 6)


def test_dense_fast_clouds_bit_exact():
    """Two dense clouds with random velocities, one in the corner of the box (wall forces)
    and one around the origin (hash collisions): pressures large enough that clIntegrateForce
    clamps forces to velocitylimit, neighbours far above 64."""
    p = gb.default_params()
    rng = SplitMix64(17)
    n = 8192
    pos = np.zeros((n, 4), np.float32)
    u = rng.uniform(3 * n).reshape(n, 3)
    pos[:4096, :3] = -0.99 + 0.12 * u[:4096]
    pos[4096:, :3] = -0.06 + 0.12 * u[4096:]
    vel = np.zeros_like(pos)
    vel[:, :3] = rng.normal(3 * n).reshape(n, 3)
    p.velocitylimit = 50.0
    a = _run_both(pos, vel, p, (0, 0, 1, 0), 3)
    assert np.isfinite(a[1]).all()


def test_tetrahedron_with_duplicate_bucket_visits_bit_exact():
    """Four particles on a tetrahedron at the origin (some neighbours' buckets are visited
    more than once by the 27-cell loop) plus 252 isolated particles (count <= 2: rest
    density and pressure)."""
    p = gb.default_params()
    d = 0.02
    a = d / np.sqrt(2.0)
    pos = np.zeros((256, 4), np.float32)
    pos[:4, :3] = np.array([[a, a, a], [a, -a, -a], [-a, a, -a], [-a, -a, a]]) / 2.0
    g = np.stack(np.meshgrid(np.arange(7), np.arange(6), np.arange(6), indexing="ij"), -1).reshape(-1, 3)[:252]
    pos[4:, :3] = 0.2 + g * 0.1
    _run_both(pos, np.zeros_like(pos), p, (0, 0, 1, 0), 2)


def test_pow_convention_moves_density_by_ulps():
    """With the C library's powf in place of x*x*x for pow(x, 3.0f), the reference's density
    moves by a few ulp: keys, permutation and bounds stay bit-exact and density/pressure agree
    within 1e-6 relative (the FP32 freedom OpenCL's 16-ulp pow allows)."""
    sc = block_collapse_3d(16, 8, 16)
    garg = (0.0, np.float32(9.81) / np.float32(9.8), 0.0, 0.0)
    p = _hash_mode(sc.params, garg)
    sysv = ref.system13(p)
    lo, hi = np.array(list(p.boxMin), np.float32), np.array(list(p.boxMax), np.float32)
    ref.set_pow_mode(ref.POW_LIBM)
    try:
        r = ref.step3d(sc.pos.copy(), sc.vel.copy(), np.zeros_like(sc.pos), sysv, garg, lo, hi)
    finally:
        ref.set_pow_mode(ref.POW_INTEGER_CUBE)
    o = oracle.step(sc.pos.copy(), sc.vel.copy(), np.zeros_like(sc.pos), p)
    for name in ("cell", "index", "cell_start", "cell_end"):
        assert_same_bits(getattr(o, name), getattr(r, name), name)
    rel = np.abs(r.spos[:, 3] - o.spos[:, 3]) / np.abs(o.spos[:, 3])
    assert rel.max() < 1e-6
    assert (rel > 0).any(), "powf and x*x*x differ somewhere on this scene"


def test_emitter_matches_the_reference():
    sc = block_collapse_3d(8, 8, 8)
    rng = np.random.default_rng(4)
    vel = rng.normal(0, 0.1, sc.pos.shape).astype(np.float32)
    for radius in (sc.params.particleRadius, 0.0123456, 0.0079044737):
        p = gb.Fluid3DParams.from_buffer_copy(bytes(sc.params))
        p.particleRadius = radius
        pos, v = sc.pos.copy(), vel.copy()
        ref.emit3d(pos, v, 200, 1.5, ref.system13(p))
        want_pos, want_vel = emitter_expected(sc.pos, vel, 200, 1.5, p.particleRadius)
        assert_same_bits(want_pos, pos, "emitted positions")
        assert_same_bits(want_vel, v, "emitted velocities")


def test_collide_bvh_matches_the_reference():
    """clCollideBVH (libCL/phys/oclFluid3D.cl:365-550) on a sphere mesh: particles just
    outside moving inward (most hit), some at rest (no hit), against the oracle's restatement."""
    v, idx = sphere_mesh(16, 32)
    box = np.zeros(8, np.float32)
    nodes, root, _, _ = oracle.bvh_build(v, idx, box)
    p = gb.default_params()
    rng = SplitMix64(5)
    n = 2000
    d = rng.normal(3 * n).reshape(n, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3] = 1.0 + d * (0.505 + 0.002 * rng.uniform(n))[:, None]
    vel[:, :3] = -d * 2.0
    vel[::50] = 0.0
    force = rng.normal(4 * n).reshape(n, 4).astype(np.float32)
    a = [force.copy(), pos.copy(), vel.copy()]
    ref.collide_bvh3d(*a, ref.system13(p), nodes, root, idx, v)
    b = [pos.copy(), vel.copy(), force.copy()]
    oracle.bvh_collide(p, b[0], b[1], b[2], nodes, root, idx, v)
    assert_same_bits(b[0], a[1], "positions")
    assert_same_bits(b[1], a[2], "velocities")
    assert_same_bits(b[2], a[0], "forces")
    assert np.all(a[2] == 0, axis=1).sum() > n // 2


# ---------------------------------------------------------------------------------------
# BVH builds (libCL/geom/oclBvhTrimesh.cl, oclBvhTrimesh::compute; libCL/geom/oclBvhLines.cl,
# oclBvhLines::compute)
# ---------------------------------------------------------------------------------------
def _same_build(o, r, what):
    nodes_o, root_o, sk_o, sv_o = o
    rc, nodes_r, root_r, sk_r, sv_r = r
    assert rc == 0, rc
    assert root_o == root_r, (root_o, root_r)
    np.testing.assert_array_equal(sk_o, sk_r, err_msg=f"{what}: sorted Morton keys")
    np.testing.assert_array_equal(sv_o, sv_r, err_msg=f"{what}: sorted ids")
    assert_same_bits(nodes_o.view(np.uint32), nodes_r.view(np.uint32), f"{what}: nodes")


@pytest.mark.parametrize("mesh", ["soup", "sphere", "around_origin"])
def test_bvh_build_matches_the_reference(mesh):
    """Global box (clAABB), Morton keys, the reference's radix sort, node creation, linking,
    leaves and the bottom-up boxes: every node's 48 bytes, the root and the box."""
    from libcl_gb300.scenes import triangle_soup
    if mesh == "soup":
        v, idx = triangle_soup(3000)
    elif mesh == "sphere":
        v, idx = sphere_mesh(24, 48)
    else:  # a soup that straddles the origin (negative coordinates in every axis)
        v, idx = triangle_soup(2000, seed=9)
        v[:, :3] -= np.array([0.8, 0.3, 0.6], np.float32)
    box_o, box_r = np.zeros(8, np.float32), np.zeros(8, np.float32)
    _same_build(oracle.bvh_build(v, idx, box_o), ref.bvh_build(v, idx, box_r), mesh)
    assert_same_bits(box_o, box_r, "global box")


def test_bvh_box_and_root_persist_across_builds_as_the_reference():
    """bfAABB and mRootNode are kept between builds: a second, smaller and shifted mesh is
    keyed inside the first build's box, and the root given in is what an unlinked build
    would leave."""
    from libcl_gb300.scenes import triangle_soup
    v, idx = triangle_soup(500, extent=2.0)
    box_o, box_r = np.zeros(8, np.float32), np.zeros(8, np.float32)
    oracle.bvh_build(v, idx, box_o)
    ref.bvh_build(v, idx, box_r)
    v2 = v.copy()
    v2[:, :3] = v2[:, :3] * 0.25 + 3.0
    _same_build(oracle.bvh_build(v2, idx, box_o, root=7), ref.bvh_build(v2, idx, box_r, root=7), "second build")
    assert_same_bits(box_o, box_r, "global box after two builds")


def test_bvh_reference_refuses_repeated_morton_keys():
    """Two triangles with the same centroid share a Morton key; the reference's clLinkNodes
    then lets two nodes claim one child, so the reference driver refuses the input (-5)."""
    from libcl_gb300.scenes import triangle_soup
    v, idx = triangle_soup(100)
    idx = idx.copy()
    idx[3:6] = idx[0:3]
    rc = ref.bvh_build(v, idx, np.zeros(8, np.float32))[0]
    assert rc == -5


@pytest.mark.parametrize("scene", ["soup", "lattice"])
def test_bvh_lines_build_matches_the_reference(scene):
    """The 2D segment BVH: Morton keys of the truncated midpoints, the sort, linking, leaves
    and boxes (every node's 32 bytes) and the root."""
    from libcl_gb300.scenes import segment_lattice, segment_soup
    v = segment_soup(5000) if scene == "soup" else segment_lattice(300)
    _same_build(oracle.bvh_lines_build(v), ref.bvh_lines_build(v), scene)


# ---------------------------------------------------------------------------------------
# 2D model (libCL/phys/oclFluid2D.cl, oclFluid2D::compute / computeBorder)
# ---------------------------------------------------------------------------------------
def test_2d_defaults_match_the_reference():
    want = gb.Fluid2DParams()
    ref.init_fluid2d(want)
    o = gb.Fluid2DParams()
    oracle.default_params_2d(o)
    assert bytes(o) == bytes(want), "oracle defaults"
    assert bytes(gb.default_params_2d()) == bytes(want), "library defaults"
    assert ref.table_size_2d(want) == oracle.table_size_2d(want)


def _obstacle_mask():
    m = box_mask(200, 180, 6)
    yy, xx = np.mgrid[0:180, 0:200]
    m[((xx - 120) ** 2 + (yy - 60) ** 2) < 20 ** 2, 3] = 1.0
    return m


@pytest.mark.parametrize("mask", ["frame", "obstacle"])
def test_2d_border_images_match_the_reference(mask):
    p = gb.default_params_2d()
    m = box_mask() if mask == "frame" else _obstacle_mask()
    v_o, s_o = oracle.compute_border_2d(m, p)
    v_r, s_r = ref.compute_border_2d(m, p)
    assert_same_bits(v_o, v_r, "wall vectors")
    assert_same_bits(s_o, s_r, "wall state")


def test_2d_steps_bit_exact():
    p = gb.default_params_2d()
    vec, bst = ref.compute_border_2d(_obstacle_mask(), p)
    a = block_state(64, 64)
    b = a.copy()
    for s in range(8):
        r = ref.step_2d(a, p, bst, vec)
        o = oracle.step_2d(b, p, bst, vec)
        for name in ("cell", "index", "sorted", "pstate", "relaxed", "prev", "cell_start", "cell_end"):
            assert_same_bits(getattr(o, name), getattr(r, name), f"step {s} {name}")
        assert_same_bits(b, a, f"step {s} state")


def test_2d_emitter_matches_the_reference():
    p = gb.default_params_2d()
    st = block_state(64, 64)
    got = st.copy()
    ref.emit2d(got, 101, p)
    assert_same_bits(emitter2d_expected(st, 101, p.particleSize), got, "2D emitter")
