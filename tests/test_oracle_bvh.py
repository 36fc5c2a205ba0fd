"""The oracle's restatement of the reference's BVH build (CPU only): the tree it produces is
a binary tree over all triangles whose boxes nest, and its global box behaves as the
reference's (starts at zero, only grows)."""
import numpy as np
import pytest

import oracle
from libcl_gb300.scenes import segment_lattice, segment_soup, sphere_mesh, triangle_soup


def check_tree(nodes, root, vertex, index):
    n = (nodes.size + 1) // 2
    seen = np.zeros(nodes.size, np.int32)
    stack = [root]
    leaves = []
    while stack:
        i = stack.pop()
        seen[i] += 1
        nd = nodes[i]
        if nd["left"] == nd["right"]:
            assert i >= n - 1
            leaves.append(int(nd["bit"]))
            tri = vertex[index[3 * nd["bit"]:3 * nd["bit"] + 3]]
            np.testing.assert_array_equal(nd["bbMin"][:3], tri[:, :3].min(axis=0))
            np.testing.assert_array_equal(nd["bbMax"][:3], tri[:, :3].max(axis=0))
            continue
        assert i < n - 1 and nd["trav"] == 2
        for c in (nd["left"], nd["right"]):
            assert np.all(nodes[c]["bbMin"] >= nd["bbMin"]) and np.all(nodes[c]["bbMax"] <= nd["bbMax"])
            stack.append(int(c))
    assert np.all(seen == 1), "every node reached exactly once"
    assert sorted(leaves) == list(range(n))


@pytest.mark.parametrize("mesh", ["soup", "sphere"])
def test_bvh_oracle_builds_a_tree(mesh):
    v, idx = triangle_soup(3000) if mesh == "soup" else sphere_mesh(24, 48)
    box = np.zeros(8, np.float32)
    nodes, root, sk, sv = oracle.bvh_build(v, idx, box)
    assert np.all(sk[1:] >= sk[:-1])
    assert len(np.unique(sk)) == sk.size, "this mesh has distinct Morton keys"
    check_tree(nodes, root, v, idx)
    # the global box contains the origin (it starts at zero) and every vertex
    assert np.all(box[:3] <= np.minimum(0, v[:, :3].min(axis=0))) and np.all(box[4:7] >= v[:, :3].max(axis=0))


def test_bvh_oracle_box_only_grows():
    v, idx = triangle_soup(500, extent=2.0)
    box = np.zeros(8, np.float32)
    oracle.bvh_build(v, idx, box)
    first = box.copy()
    v2 = v.copy()
    v2[:, :3] *= 0.25
    oracle.bvh_build(v2, idx, box)
    np.testing.assert_array_equal(box, first)  # a smaller mesh does not shrink it


def test_bvh_oracle_collide_stops_particles_crossing_the_mesh():
    """Particles just outside a sphere mesh moving inward: those whose step crosses a
    triangle within the particle radius stop (velocity 0) and are pushed; the others are left
    as they were."""
    from libcl_gb300 import default_params
    from libcl_gb300.scenes import SplitMix64
    v, idx = sphere_mesh(16, 32)
    box = np.zeros(8, np.float32)
    nodes, root, _, _ = oracle.bvh_build(v, idx, box)
    p = default_params()
    rng = SplitMix64(5)
    n = 2000
    d = rng.normal(3 * n).reshape(n, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos = np.zeros((n, 4), np.float32)
    vel = np.zeros((n, 4), np.float32)
    pos[:, :3] = 1.0 + d * (0.505 + 0.002 * rng.uniform(n))[:, None]
    vel[:, :3] = -d * 2.0
    force = np.zeros_like(pos)
    p0, v0 = pos.copy(), vel.copy()
    oracle.bvh_collide(p, pos, vel, force, nodes, root, idx, v)
    hit = np.all(vel == 0, axis=1)
    assert hit.sum() > n // 2
    np.testing.assert_array_equal(pos[~hit], p0[~hit])
    np.testing.assert_array_equal(vel[~hit], v0[~hit])
    assert np.all(np.any(pos[hit] != p0[hit], axis=1))


def check_tree_2d(nodes, root, vertex):
    n = (nodes.size + 1) // 2
    seen = np.zeros(nodes.size, np.int32)
    stack = [root]
    leaves = []
    while stack:
        i = stack.pop()
        seen[i] += 1
        nd = nodes[i]
        if nd["left"] == nd["right"]:
            assert i >= n - 1
            leaves.append(int(nd["bit"]))
            seg = vertex[2 * nd["bit"]:2 * nd["bit"] + 2]
            np.testing.assert_array_equal(nd["bbMin"], seg.min(axis=0))
            np.testing.assert_array_equal(nd["bbMax"], seg.max(axis=0))
            continue
        assert i < n - 1 and nd["trav"] == 3
        for c in (nd["left"], nd["right"]):
            assert np.all(nodes[c]["bbMin"] >= nd["bbMin"]) and np.all(nodes[c]["bbMax"] <= nd["bbMax"])
            stack.append(int(c))
    assert np.all(seen == 1), "every node reached exactly once"
    assert sorted(leaves) == list(range(n))


@pytest.mark.parametrize("scene", ["soup", "lattice"])
def test_bvh_lines_oracle_builds_a_tree(scene):
    v = segment_soup(3000) if scene == "soup" else segment_lattice(40)
    nodes, root, sk, sv = oracle.bvh_lines_build(v)
    assert np.all(sk[1:] >= sk[:-1])
    assert len(np.unique(sk)) == sk.size, "distinct Morton keys"
    check_tree_2d(nodes, root, v)


def test_bvh_lines_oracle_morton_keys_by_hand():
    """clMorton of oclBvhLines: midpoint (truncated) x in the even bits, y in the odd bits."""
    v = np.array([[0, 0], [2, 2],          # midpoint (1, 1): 0b01 | 0b10 = 3
                  [4, 6], [4, 10],         # (4, 8): x 4 -> 0b10000 (16), y 8 -> 0b1000000 << 1 (128)
                  [3.9, 0.2], [3.9, 0.2],  # (3.9, 0.2) -> (3, 0): 0b101 = 5
                  [65535, 0], [65535, 0],  # x 0xFFFF -> 0x55555555
                  [0, 70000], [0, 70000]],  # y 70000 & 0xFFFF = 4464 = 0b1000101110000
                 np.float32)
    # y: 4464 = 0b1_0001_0111_0000 -> bits 4, 5, 6, 8, 12 -> 2^8 + 2^10 + 2^12 + 2^16 + 2^24, shifted by 1
    want = {0: 3, 1: 16 | 128, 2: 5, 3: 0x55555555, 4: 33696256}
    _, _, sk, sv = oracle.bvh_lines_build(v)
    got = {int(i): int(k) for k, i in zip(sk, sv)}
    assert got == want

