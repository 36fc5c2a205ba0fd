"""CPU checks of the 2D restatement (oracle/oracle2d.cpp) of libCL/phys/oclFluid2D.cl."""
import numpy as np

import libcl_gb300 as gb
import oracle
from scenes2d import block_state, box_mask


def test_default_params_match_clInitFluid():
    p = gb.default_params_2d()
    q = gb.Fluid2DParams()
    oracle.default_params_2d(q)
    for name, _ in gb.Fluid2DParams._fields_:
        assert getattr(p, name) == getattr(q, name), name
    assert (p.cellCountX, p.cellCountY) == (40, 36)          # 17.68/0.44+0.5, 15.76/0.44+0.5
    assert oracle.table_size_2d(p) == 1536                   # (1440/256 + 1) * 256
    assert abs(p.h - 0.22) < 1e-6 and abs(p.particleSize - 0.01) < 1e-8


def test_border_inside_and_outside_the_wall():
    p = gb.default_params_2d()
    mask = box_mask(256, 256, 8)  # pixels of 0.069 x 0.062, closer than h = 0.22
    vec, st = oracle.compute_border_2d(mask, p)
    k_norm = np.float32(20) / (np.float32(2) * np.float32(3.1415926535) * np.float32(0.22) * np.float32(0.22))
    inside = st[1, 1]
    assert abs(inside[0] - 112 * 0.7 * k_norm) / (112 * 0.7 * k_norm) < 1e-3  # half precision
    far = st[128, 128]
    assert far[0] == 0 and far[1] == 0 and np.all(vec[128, 128] == 0)  # no wall within h
    near = st[8, 128]                                                  # first fluid row above the bottom wall
    assert near[0] > 0 and vec[8, 128, 1] > 0.99                        # normal points away from the wall (+y)
    assert np.all(st == st.astype(np.float16).astype(np.float32))   # half-float image values


def test_step_keeps_particles_inside_and_is_deterministic():
    p = gb.default_params_2d()
    vec, bst = oracle.compute_border_2d(box_mask(), p)
    s1 = block_state(32, 32)
    s2 = s1.copy()
    for _ in range(5):
        r1 = oracle.step_2d(s1, p, bst, vec)
        r2 = oracle.step_2d(s2, p, bst, vec)
    assert np.array_equal(s1, s2)
    assert np.isfinite(s1).all()
    assert np.all(np.sort(r1.index) == np.arange(s1.shape[0]))
    assert s1[:, 1].mean() < block_state(32, 32)[:, 1].mean()  # gravity pulls the block down
