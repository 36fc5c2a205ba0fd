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


def test_full_ensemble_against_oracle_and_scenes_run_alone(cuda):
    """The batched configuration at full size: 256 scenes of 4,096-262,144 particles
    (log-uniform, seed 5), one batched step from a perturbed state. Eight scenes across the
    size range are compared with the oracle's step (oracle.step on the scene alone) within
    RTOL: density, velocity and position; every one of the 256 scenes is bitwise equal to the
    same scene run alone through Fluid3D."""
    import torch
    import oracle
    from fluid_helpers import RTOL, pos_err, rel_err
    from libcl_gb300 import BUF_SORTED_POSITION
    b = batched_ensemble()
    assert len(b.descs) == 256 and b.n > 15_000_000
    rng = np.random.default_rng(6)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    bt = load_batch(b, bw=16)
    bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0
    got = {k: bt.buffer(w).cpu().numpy() for k, w in (("pos", BUF_POSITION), ("vel", BUF_VELOCITY), ("force", BUF_FORCE))}
    idx = bt.buffer(BUF_INDEX).cpu().numpy().view(np.uint32)
    rho = np.empty(b.n, np.float32)
    rho[idx] = bt.buffer(BUF_SORTED_POSITION)[:, 3].cpu().numpy()
    del bt
    torch.cuda.empty_cache()
    sizes = np.array([d.n_particles for d in b.descs])
    picked = [int(np.argsort(sizes)[k]) for k in np.linspace(0, len(sizes) - 1, 8).astype(int)]
    for s in range(len(b.descs)):
        sc = b.scene(s)
        a, n = b.firsts[s], sc.n
        f = make_fluid(sc, vel=sc.vel)
        f.set_option(OPT_BRICK_WIDTH, 16)
        f.compute()
        ref = state(f)
        for k in ("pos", "vel", "force"):
            assert np.array_equal(got[k][a:a + n].view(np.uint32), ref[k].view(np.uint32)), (s, k)
        del f
        if s in picked:
            pos, vel, force = sc.pos.copy(), sc.vel.copy(), np.zeros_like(sc.pos)
            r = oracle.step(pos, vel, force, sc.params)
            rho_o = np.empty(n, np.float32)
            rho_o[r.index] = r.spos[:, 3]
            assert rel_err(rho[a:a + n], rho_o) <= RTOL, (s, "density")
            assert rel_err(got["vel"][a:a + n], vel) <= RTOL, (s, "velocity")
            assert pos_err(got["pos"][a:a + n], pos, sc.pos) <= 1.0, (s, "position")
            assert np.array_equal(got["force"][a:a + n], force), (s, "force (gravity seed)")
