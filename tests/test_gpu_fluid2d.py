"""GPU parity of the reference's 2D model (gbsph_fluid2d_*) against oracle/oracle2d.cpp:
wall field, sorted permutation, cell bounds, pressures, relaxed positions and state, all
bit-exact, over several steps."""
import numpy as np
import pytest

import oracle
from libcl_gb300 import (BUF2D_BORDER_STATE, BUF2D_BORDER_VECTOR, BUF2D_CELL, BUF2D_INDEX, BUF2D_PRESSURE,
                         BUF2D_RELAXED, BUF2D_SORTED_STATE, BUF2D_STATE, Fluid2D)
from scenes2d import block_state, box_mask, emitter2d_expected

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_fluid2d_bit_exact_over_steps(cuda):
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
    vec, bst = oracle.compute_border_2d(mask, p)
    assert np.array_equal(bits(f.buffer(BUF2D_BORDER_VECTOR).cpu().numpy().reshape(vec.shape)), bits(vec))
    assert np.array_equal(bits(f.buffer(BUF2D_BORDER_STATE).cpu().numpy().reshape(bst.shape)), bits(bst))
    table = oracle.table_size_2d(p)
    host = st.copy()
    for step in range(6):
        f.compute()
        torch.cuda.synchronize()
        r = oracle.step_2d(host, p, bst, vec)
        assert np.array_equal(f.buffer(BUF2D_CELL).cpu().numpy().view(np.uint32), r.cell), step
        assert np.array_equal(f.buffer(BUF2D_INDEX).cpu().numpy().view(np.uint32), r.index), step
        cs, ce = f.cell_bounds(table)
        assert np.array_equal(cs.cpu().numpy().view(np.uint32), r.cell_start)
        assert np.array_equal(ce.cpu().numpy().view(np.uint32), r.cell_end)
        assert np.array_equal(bits(f.buffer(BUF2D_SORTED_STATE).cpu().numpy()), bits(r.sorted)), step
        assert np.array_equal(bits(f.buffer(BUF2D_PRESSURE).cpu().numpy()), bits(r.pstate)), step
        assert np.array_equal(bits(f.buffer(BUF2D_RELAXED).cpu().numpy()), bits(r.relaxed)), step
        g = f.buffer(BUF2D_STATE).cpu().numpy()
        assert np.array_equal(bits(g), bits(host)), step
    assert f.sync_status() == 0


def test_fluid2d_borrowed_state_and_reference_default_count(cuda):
    import torch
    f = Fluid2D()
    f.compile()
    assert f.getParticleCount() == 128 * 128  # the reference's default (libCL/phys/oclFluid2D.cpp:55)
    st = torch.from_numpy(block_state(128, 128)).cuda()
    f.setStateBuffer(st)
    f.computeBorder(torch.from_numpy(box_mask()).cuda())
    for _ in range(10):
        f.compute()
    torch.cuda.synchronize()
    assert torch.isfinite(st).all()
    assert f.getStateBuffer().data_ptr() == st.data_ptr()


def test_fluid2d_emitter(cuda):
    """clEmitter (libCL/phys/oclFluid2D.cl:342-352): only particle emit+1 changes."""
    import torch
    f = Fluid2D()
    f.compile()
    st = block_state(64, 64)
    f.setParticleCount(st.shape[0])
    f.getStateBuffer().copy_(torch.from_numpy(st))
    f.emit(101)
    torch.cuda.synchronize()
    g = f.getStateBuffer().cpu().numpy()
    want = emitter2d_expected(st, 101, f.getParameters().particleSize)
    np.testing.assert_array_equal(g.view(np.uint32), want.view(np.uint32))
