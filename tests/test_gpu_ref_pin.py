"""GPU parity against the reference's own kernels (libCL/phys/oclFluid3D.cl,
libCL/phys/oclFluid2D.cl, libCL/sort/oclRadixSort.cl, libCL/geom/oclBvhTrimesh.cl,
libCL/geom/oclBvhLines.cl built for the host cores by oracle/ref/build.py), run on the same
inputs: the CUDA library's results must be the same bits. Skipped where those kernels are not
built (oracle.ref.available())."""
import numpy as np
import pytest

import oracle.ref as ref
from fluid_helpers import hash_block, make_fluid, perturbed, sorted_outputs, state
from libcl_gb300 import (BUF2D_BORDER_STATE, BUF2D_BORDER_VECTOR, BUF2D_CELL, BUF2D_INDEX, BUF2D_PRESSURE,
                         BUF2D_RELAXED, BUF2D_SORTED_STATE, BUF2D_STATE, OK, REF_BUCKETS, Fluid2D, RadixSort)
from libcl_gb300.scenes import block_collapse_3d
from scenes2d import block_state, box_mask

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref.available(), reason="reference kernels not built")]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def same(a, b, what):
    a, b = bits(a), bits(b)
    bad = np.argwhere(a != b)
    assert bad.size == 0, f"{what}: {len(bad)} words differ, first at {bad[:3].tolist()}"


@pytest.mark.parametrize("fused", [False, True])
def test_hash_mode_steps_equal_the_reference_kernels(cuda, fused):
    """Three steps of the reference's default scene on its hash keys: keys, permutation,
    cell table, density, pressure, force, position and velocity identical to
    oclFluid3D::compute's kernels."""
    sc = hash_block(24)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=fused, vel=vel)
    p = sc.params
    g4 = np.array(list(p.gravity), np.float32)
    garg = g4 / np.float32(-9.8)
    assert np.array_equal(np.float32(-9.8) * garg, g4)
    host = [sc.pos.copy(), vel.copy(), np.zeros_like(sc.pos)]
    lo, hi = np.array(list(p.boxMin), np.float32), np.array(list(p.boxMax), np.float32)
    for step in range(3):
        f.compute()
        g, gs = sorted_outputs(f, REF_BUCKETS), state(f)
        r = ref.step3d(*host, ref.system13(p), garg, lo, hi)
        for k in ("cell", "index", "cell_start", "cell_end", "spos", "svel"):
            same(g[k], getattr(r, k), f"step {step} {k}")
        for k, h in zip(("pos", "vel", "force"), host):
            same(gs[k], h, f"step {step} {k}")
    assert f.sync_status() == OK


@pytest.mark.parametrize("bits_", [(0, 24), (0, 32), (4, 16)])
def test_sort_equals_the_reference_kernels(cuda, bits_):
    import torch
    rng = np.random.default_rng(bits_[1])
    keys = rng.integers(0, 2 ** 32, 300_001, dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(keys.size).astype(np.uint32)
    dk = torch.from_numpy(keys.view(np.int32)).cuda()
    dv = torch.from_numpy(vals.view(np.int32)).cuda()
    RadixSort().compute(dk, dv, *bits_)
    k, v = keys.copy(), vals.copy()
    assert ref.radix_sort(k, v, *bits_) == 0
    same(dk.cpu().numpy(), k, "keys")
    same(dv.cpu().numpy(), v, "values")


def test_fluid2d_equals_the_reference_kernels(cuda):
    """Wall images of computeBorder and six steps of oclFluid2D::compute."""
    import torch
    f = Fluid2D()
    f.compile()
    st = block_state(64, 64)
    f.setParticleCount(st.shape[0])
    p = f.getParameters()
    mask = box_mask()
    f.computeBorder(torch.from_numpy(mask).cuda())
    f.getStateBuffer().copy_(torch.from_numpy(st))
    torch.cuda.synchronize()
    vec, bst = ref.compute_border_2d(mask, p)
    same(f.buffer(BUF2D_BORDER_VECTOR).cpu().numpy().reshape(vec.shape), vec, "wall vectors")
    same(f.buffer(BUF2D_BORDER_STATE).cpu().numpy().reshape(bst.shape), bst, "wall state")
    table = ref.table_size_2d(p)
    host = st.copy()
    for step in range(6):
        f.compute()
        torch.cuda.synchronize()
        r = ref.step_2d(host, p, bst, vec)
        same(f.buffer(BUF2D_CELL).cpu().numpy(), r.cell, f"step {step} keys")
        same(f.buffer(BUF2D_INDEX).cpu().numpy(), r.index, f"step {step} index")
        cs, ce = f.cell_bounds(table)
        same(cs.cpu().numpy(), r.cell_start, f"step {step} cellStart")
        same(ce.cpu().numpy(), r.cell_end, f"step {step} cellEnd")
        same(f.buffer(BUF2D_SORTED_STATE).cpu().numpy(), r.sorted, f"step {step} sorted state")
        same(f.buffer(BUF2D_PRESSURE).cpu().numpy(), r.pstate, f"step {step} pressures")
        same(f.buffer(BUF2D_RELAXED).cpu().numpy(), r.relaxed, f"step {step} relaxed positions")
        same(f.buffer(BUF2D_STATE).cpu().numpy(), host, f"step {step} state")
    assert f.sync_status() == 0


def test_emitter_equals_the_reference_kernel(cuda):
    sc = block_collapse_3d(8, 8, 8)
    vel = perturbed(sc)
    f = make_fluid(sc, vel=vel)
    f.emit(200, 1.5)
    g = state(f)
    pos, v = sc.pos.copy(), vel.copy()
    ref.emit3d(pos, v, 200, 1.5, ref.system13(sc.params))
    same(g["pos"], pos, "positions")
    same(g["vel"], v, "velocities")


def test_bvh_builds_equal_the_reference_kernels(cuda):
    """gbsph_bvh (two builds on one handle: the global box carries over) and gbsph_bvh_lines
    against oclBvhTrimesh::compute and oclBvhLines::compute run through the reference's
    kernels: every node's bytes, the root and the box."""
    import torch
    from libcl_gb300 import BvhLines, BvhTrimesh
    from libcl_gb300.scenes import segment_soup, sphere_mesh, triangle_soup
    b = BvhTrimesh()
    box = np.zeros(8, np.float32)
    root = 0
    for v, idx in (triangle_soup(3000), sphere_mesh(24, 48)):
        b.compute(torch.from_numpy(v).cuda(), torch.from_numpy(idx.view(np.int32)).cuda())
        assert b.sync_status() == 0
        rc, nodes, root, _, _ = ref.bvh_build(v, idx, box, root)
        assert rc == 0
        same(b.getNodeBuffer().cpu().numpy().ravel(), nodes.view(np.uint32), "triangle BVH nodes")
        assert b.getRootNode() == root
        same(np.asarray(b.bounds(), np.float32), box, "global box")
    lines = BvhLines()
    v = segment_soup(5000)
    lines.compute(torch.from_numpy(v).cuda())
    assert lines.sync_status() == 0
    rc, nodes, root, _, _ = ref.bvh_lines_build(v)
    assert rc == 0
    same(lines.getNodeBuffer().cpu().numpy().ravel(), nodes.view(np.uint32), "segment BVH nodes")
    assert lines.getRootNode() == root
