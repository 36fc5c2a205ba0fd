"""GPU tests of the batched step (gbsph_batch3d_*): every scene of a batch advances exactly as
the same scene run alone through Fluid3D (bit for bit: same grid, same brick width, same
neighbour order), scenes do not interact, and the autotuner leaves the state unchanged."""
import numpy as np
import pytest

from fluid_helpers import make_fluid, state
from libcl_gb300 import (BUF_FORCE, BUF_INDEX, BUF_POSITION, BUF_VELOCITY, OPT_BRICK_WIDTH, Batch3D)
from libcl_gb300.scenes import batched_ensemble

pytestmark = pytest.mark.gpu


def load_batch(b, bw=8):
    import torch
    bt = Batch3D()
    bt.set_scenes(b.shared, b.descs)
    bt.set_option(OPT_BRICK_WIDTH, bw)
    bt.buffer(BUF_POSITION).copy_(torch.from_numpy(b.pos))
    bt.buffer(BUF_VELOCITY).copy_(torch.from_numpy(b.vel))
    bt.buffer(BUF_FORCE).zero_()
    torch.cuda.synchronize()
    return bt


def test_batch_matches_scenes_run_alone(cuda):
    import torch
    b = batched_ensemble(n_scenes=7, seed=9, n_min=500, n_max=30000)
    rng = np.random.default_rng(1)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    bt = load_batch(b, bw=8)
    for _ in range(3):
        bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0
    got = {k: bt.buffer(w).cpu().numpy() for k, w in (("pos", BUF_POSITION), ("vel", BUF_VELOCITY), ("force", BUF_FORCE))}
    idx = bt.buffer(BUF_INDEX).cpu().numpy().view(np.uint32)
    assert np.array_equal(np.sort(idx), np.arange(b.n, dtype=np.uint32))
    for s in range(len(b.descs)):
        sc = b.scene(s)
        f = make_fluid(sc, vel=sc.vel)
        f.set_option(OPT_BRICK_WIDTH, 8)
        for _ in range(3):
            f.compute()
        ref = state(f)
        a, n = bt.scene_range(s)
        for k in ("pos", "vel", "force"):
            assert np.array_equal(got[k][a:a + n].view(np.uint32), ref[k].view(np.uint32)), (s, k)


def test_disordered_batch_matches_scenes_run_alone(cuda):
    """As above with every particle moved by up to 0.9 spacing per axis (cells hold 1 to 20
    particles), so the batched brick kernels take the flat list walk and the whole-warp scan
    of overflowed targets."""
    import torch
    b = batched_ensemble(n_scenes=5, seed=13, n_min=3000, n_max=40000)
    rng = np.random.default_rng(4)
    b.pos[:, :3] += (0.006 + rng.uniform(-0.009, 0.009, (b.n, 3))).astype(np.float32)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    bt = load_batch(b, bw=8)
    for _ in range(3):
        bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0
    got = {k: bt.buffer(w).cpu().numpy() for k, w in (("pos", BUF_POSITION), ("vel", BUF_VELOCITY), ("force", BUF_FORCE))}
    for s in range(len(b.descs)):
        sc = b.scene(s)
        f = make_fluid(sc, vel=sc.vel)
        f.set_option(OPT_BRICK_WIDTH, 8)
        for _ in range(3):
            f.compute()
        ref = state(f)
        a, n = bt.scene_range(s)
        for k in ("pos", "vel", "force"):
            assert np.array_equal(got[k][a:a + n].view(np.uint32), ref[k].view(np.uint32)), (s, k)


def test_autotune_restores_state(cuda):
    import torch
    b = batched_ensemble(n_scenes=16, seed=3, n_min=2000, n_max=40000)
    bt = load_batch(b)
    before = bt.buffer(BUF_POSITION).cpu().numpy().copy()
    best = bt.autotune()
    assert best in (4, 8, 16)
    after = bt.buffer(BUF_POSITION).cpu().numpy()
    assert np.array_equal(before, after)
    bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0
