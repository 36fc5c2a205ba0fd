"""GPU tests of the batched step (gbsph_batch3d_*): every scene of a batch advances exactly as
the same scene run alone through Fluid3D (bit for bit: same grid, same brick width, same
neighbour order), scenes do not interact, and the autotuner leaves the state unchanged."""
import numpy as np
import pytest

from fluid_helpers import make_fluid, state
from libcl_gb300 import (BUF_CELL, BUF_FORCE, BUF_INDEX, BUF_POSITION, BUF_SORTED_POSITION, BUF_SORTED_VELOCITY,
                         BUF_VELOCITY, OPT_BRICK_WIDTH, OPT_PERSISTENT, OPT_RADIX_BITS, OPT_SORT_TILE, Batch3D,
                         GbsphError)
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
    before = {w: bt.buffer(w).cpu().numpy().copy() for w in (BUF_POSITION, BUF_VELOCITY, BUF_FORCE)}
    best = bt.autotune()
    assert best in (4, 8, 16)
    cfg = bt.config()
    assert cfg["brick_width"] == best and cfg["radix_bits"] in (6, 7, 8) and cfg["sort_tile_items"] in (8, 16)
    assert cfg["persistent"] in (0, 1)
    for w, v in before.items():
        assert np.array_equal(v, bt.buffer(w).cpu().numpy()), w
    bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0


ALL_BUFFERS = (BUF_POSITION, BUF_VELOCITY, BUF_FORCE, BUF_INDEX, BUF_CELL, BUF_SORTED_POSITION, BUF_SORTED_VELOCITY)


def _run_batch(b, steps, persistent=0, items=0, bits=8, bw=8):
    import torch
    bt = load_batch(b, bw=bw)
    bt.set_option(OPT_PERSISTENT, persistent)
    bt.set_option(OPT_SORT_TILE, items)
    bt.set_option(OPT_RADIX_BITS, bits)
    for _ in range(steps):
        bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0
    return {w: bt.buffer(w).cpu().numpy().view(np.uint32).copy() for w in ALL_BUFFERS}


@pytest.mark.parametrize("bits,items", [(6, 8), (7, 16), (8, 8), (5, 16)])
def test_sort_digit_width_and_tile_do_not_change_results(cuda, bits, items):
    """The radix sort is stable, so every digit width and tile size yields the same sorted
    order and the same step, bit for bit (3 steps of a 12-scene batch whose keys need 17
    bits: four passes with 5-bit digits, three with 6, 7 or 8)."""
    b = batched_ensemble(n_scenes=12, seed=21, n_min=1000, n_max=60000)
    rng = np.random.default_rng(2)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    ref = _run_batch(b, 3)
    got = _run_batch(b, 3, items=items, bits=bits)
    for w in ALL_BUFFERS:
        assert np.array_equal(ref[w], got[w]), w


@pytest.mark.parametrize("items,bits,bw", [(8, 8, 8), (16, 7, 4), (16, 8, 16), (8, 6, 8)])
def test_persistent_step_matches_staged(cuda, items, bits, bw):
    """The persistent form (one cooperative kernel per step) and the staged graph run the same
    phases in the same order, so 4 steps of a 9-scene batch agree bit for bit in every buffer:
    state, sorted state (density and pressure in .w), sort permutation and cell keys."""
    b = batched_ensemble(n_scenes=9, seed=31, n_min=800, n_max=50000)
    rng = np.random.default_rng(8)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    ref = _run_batch(b, 4, 0, items, bits, bw)
    got = _run_batch(b, 4, 1, items, bits, bw)
    for w in ALL_BUFFERS:
        assert np.array_equal(ref[w], got[w]), w


def test_persistent_step_dense_clumps_match_staged(cuda):
    """Dense, disordered scenes (particles jittered by up to 0.9 spacing, cells of 1 to 20
    particles): bricks too full to stage and targets whose lists overflow take the direct
    global-memory paths of the density and force phases."""
    b = batched_ensemble(n_scenes=5, seed=13, n_min=3000, n_max=40000)
    rng = np.random.default_rng(4)
    b.pos[:, :3] += (0.006 + rng.uniform(-0.009, 0.009, (b.n, 3))).astype(np.float32)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    ref = _run_batch(b, 3, 0, bw=16)
    got = _run_batch(b, 3, 1, bw=16)
    for w in ALL_BUFFERS:
        assert np.array_equal(ref[w], got[w]), w


def test_persistent_full_ensemble_matches_staged(cuda):
    """The 256-scene ensemble (17.3M particles), two steps in each form, bitwise."""
    import torch
    b = batched_ensemble()
    rng = np.random.default_rng(6)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    ref = _run_batch(b, 2, 0, bw=8)
    torch.cuda.empty_cache()
    got = _run_batch(b, 2, 1, bw=8)
    for w in ALL_BUFFERS:
        assert np.array_equal(ref[w], got[w]), w


def test_batch_options(cuda):
    b = batched_ensemble(n_scenes=3, seed=1, n_min=1000, n_max=2000)
    bt = load_batch(b)
    assert bt.config() == {"brick_width": 8, "radix_bits": 8, "sort_tile_items": 0, "cuda_graph": 1,
                           "persistent": 0}
    for opt, bad in ((OPT_RADIX_BITS, 4), (OPT_RADIX_BITS, 9), (OPT_SORT_TILE, 12), (OPT_BRICK_WIDTH, 0)):
        with pytest.raises(GbsphError):
            bt.set_option(opt, bad)
    bt.set_option(OPT_RADIX_BITS, 7)
    bt.set_option(OPT_SORT_TILE, 16)
    bt.set_option(OPT_PERSISTENT, 1)
    assert bt.get_option(OPT_RADIX_BITS) == 7 and bt.get_option(OPT_SORT_TILE) == 16
    assert bt.get_option(OPT_PERSISTENT) == 1


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


def _dense_clump_batch():
    """Four scenes: two ordinary lattice blocks, one whose 2,500 particles sit inside a single
    cell (its brick stages more candidates than fit, so both neighbour passes read global
    memory and every target overflows its lists), and one with a quarter of its particles
    beyond its grid on every side (clamped into the border cells)."""
    b = batched_ensemble(n_scenes=4, seed=41, n_min=2000, n_max=6000)
    rng = np.random.default_rng(12)
    a, n = b.firsts[2], b.descs[2].n_particles
    h = float(b.shared.cellSize)
    b.pos[a:a + n, :3] = (h * (3.0 + rng.uniform(0.05, 0.95, (n, 3)))).astype(np.float32)
    a, n = b.firsts[3], b.descs[3].n_particles
    far = rng.random(n) < 0.25
    ext = np.array([b.descs[3].gridDim[i] * h for i in range(3)], np.float32)
    b.pos[a:a + n, :3][far] = (ext * rng.choice([-0.3, 1.3], (int(far.sum()), 3))).astype(np.float32)
    b.vel[:, :3] = rng.normal(0, 0.05, (b.n, 3)).astype(np.float32)
    return b


def test_persistent_step_matches_staged_on_clumps_and_clamped_particles(cuda):
    b = _dense_clump_batch()
    ref = _run_batch(b, 3, 0, bw=8)
    got = _run_batch(b, 3, 1, bw=8)
    for w in ALL_BUFFERS:
        assert np.array_equal(ref[w], got[w]), w


def test_persistent_step_on_tiny_scenes(cuda):
    """Scenes of 8 to 30 particles (one sort tile, a few bricks, most CTAs of the cooperative
    grid without work): persistent equals staged, and both leave no device error."""
    b = batched_ensemble(n_scenes=3, seed=2, n_min=8, n_max=30)
    ref = _run_batch(b, 5, 0)
    got = _run_batch(b, 5, 1)
    for w in ALL_BUFFERS:
        assert np.array_equal(ref[w], got[w]), w


def test_persistent_step_is_captured_in_a_graph(cuda):
    """On this driver the cooperative launch is captured into the step's graph (a refused
    capture would run eagerly and say so in the handle's last error)."""
    import torch
    b = batched_ensemble(n_scenes=3, seed=1, n_min=1000, n_max=2000)
    bt = load_batch(b)
    bt.set_option(OPT_PERSISTENT, 1)
    for _ in range(3):
        bt.compute()
    torch.cuda.synchronize()
    assert bt.sync_status() == 0
    assert bt._lib.gbsph_batch3d_last_error(bt._h).decode() == ""
