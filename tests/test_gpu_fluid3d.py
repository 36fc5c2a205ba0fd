"""GPU parity of the 3D SPH step against the oracle (the FP32 restatement of oclFluid3D.cl),
driven through the C ABI. Keys, sorted permutation and cell bounds are bit-exact everywhere;
the exact (reference-order) kernels are bit-exact for density, force and state as well; the
fast brick kernels agree within RTOL (tests/fluid_helpers.py)."""
import numpy as np
import pytest

import oracle
from fluid_helpers import (RTOL, emitter_expected, hash_block, make_fluid, perturbed, pos_err, rel_err, set_params,
                           sorted_outputs, state)
from libcl_gb300 import (ERR_ARGUMENT, ERR_NOT_COMPILED, ERR_SIZE_MISMATCH, OK, OPT_BRICK_WIDTH, REF_BUCKETS,
                         STAGE_GRAVITY, STAGE_INTEGRATE_FORCE, STAGE_INTEGRATE_VELOCITY, Fluid3D)
from libcl_gb300.scenes import block_collapse_3d, clone_params, lattice, reference_test_scene

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_bit_exact(a, b, what):
    ba, bb = bits(a), bits(b)
    if not np.array_equal(ba, bb):
        bad = np.argwhere(ba != bb)
        raise AssertionError(f"{what}: {len(bad)} entries differ, first at {bad[0]}: {a[tuple(bad[0])]} vs {b[tuple(bad[0])]}")


def oracle_step(scene, vel, force=None, ref_sort=False):
    pos = scene.pos.copy()
    v = vel.copy()
    f = np.zeros_like(scene.pos) if force is None else force.copy()
    r = oracle.step(pos, v, f, scene.params, ref_sort=ref_sort)
    return r, {"pos": pos, "vel": v, "force": f}


@pytest.mark.parametrize("fused", [False, True])
def test_hash_mode_step_bit_exact(cuda, fused):
    """REFERENCE_HASH keys (262144 buckets, duplicate bucket visits included): everything
    bit-exact against the restatement, including density, pressure, force and state."""
    sc = hash_block(24)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=fused, vel=vel)
    f.compute()
    g, gs = sorted_outputs(f, REF_BUCKETS), state(f)
    r, rs = oracle_step(sc, vel, ref_sort=True)
    assert_bit_exact(g["cell"], r.cell, "keys")
    assert_bit_exact(g["index"], r.index, "index")
    assert_bit_exact(g["cell_start"], r.cell_start, "cellStart")
    assert_bit_exact(g["cell_end"], r.cell_end, "cellEnd")
    assert_bit_exact(g["spos"], r.spos, "sorted position (.w = density)")
    assert_bit_exact(g["svel"], r.svel, "sorted velocity (.w = pressure)")
    for k in ("pos", "vel", "force"):
        assert_bit_exact(gs[k], rs[k], k)
    assert f.sync_status() == OK


def test_hash_mode_fused_lists_and_overflow_bit_exact(cuda):
    """REFERENCE_HASH fused step on a block at 0.7 x the default spacing: about three quarters
    of the particles have more in-range neighbours than the force kernel's recorded lists hold
    (they scan the buckets again), the rest walk their lists; all bit-exact."""
    sc = hash_block(22)
    sp = sc.params.spacing
    sc.pos = lattice(22, 22, 22, 0.7 * sp, (-7.7 * sp,) * 3, 0.1 * sp, 14)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=True, vel=vel)
    f.compute()
    g, gs = sorted_outputs(f, REF_BUCKETS), state(f)
    r, rs = oracle_step(sc, vel, ref_sort=True)
    assert_bit_exact(g["spos"], r.spos, "sorted position (.w = density)")
    assert_bit_exact(g["svel"], r.svel, "sorted velocity (.w = pressure)")
    for k in ("pos", "vel", "force"):
        assert_bit_exact(gs[k], rs[k], k)
    assert f.sync_status() == OK


def test_hash_mode_fused_equals_staged_over_steps(cuda):
    """The fused REFERENCE_HASH step (recorded neighbour lists) against the staged stages
    (the force kernel scanning the buckets): bitwise equal state after each of 6 steps."""
    sc = hash_block(24)
    vel = perturbed(sc, sigma=0.2)
    a = make_fluid(sc, fused=True, vel=vel)
    b = make_fluid(sc, fused=False, vel=vel)
    for step in range(6):
        a.compute()
        b.compute()
        sa, sb = state(a), state(b)
        for k in sa:
            assert_bit_exact(sa[k], sb[k], f"{k} after step {step + 1}")
    assert a.sync_status() == OK and b.sync_status() == OK


def test_linear_staged_step_bit_exact(cuda):
    sc = block_collapse_3d(32, 16, 32)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=False, vel=vel)
    f.compute()
    g, gs = sorted_outputs(f, oracle.table_cells(sc.params)), state(f)
    r, rs = oracle_step(sc, vel)
    for k, rv in (("cell", r.cell), ("index", r.index), ("cell_start", r.cell_start), ("cell_end", r.cell_end),
                  ("spos", r.spos), ("svel", r.svel)):
        assert_bit_exact(g[k], rv, k)
    for k in ("pos", "vel", "force"):
        assert_bit_exact(gs[k], rs[k], k)


def compare_fast(g, gs, r, rs, prev_pos, tol=RTOL):
    """Fast path: integer outputs exact, float outputs within tol."""
    assert_bit_exact(g["cell"], r.cell, "keys")
    assert_bit_exact(g["index"], r.index, "index")
    assert_bit_exact(g["cell_start"], r.cell_start, "cellStart")
    assert_bit_exact(g["cell_end"], r.cell_end, "cellEnd")
    assert_bit_exact(g["spos"][:, :3], r.spos[:, :3], "sorted position xyz")
    assert_bit_exact(g["svel"][:, :3], r.svel[:, :3], "sorted velocity xyz")
    errs = {
        "density": rel_err(g["spos"][:, 3], r.spos[:, 3]),
        "pressure": rel_err(g["svel"][:, 3], r.svel[:, 3]),
        "velocity": rel_err(gs["vel"], rs["vel"]),
    }
    assert_bit_exact(gs["force"], rs["force"], "force (gravity seed)")
    for k, e in errs.items():
        assert e <= tol, f"{k}: relative error {e:.3e} > {tol:.1e}"
    errs["position"] = pos_err(gs["pos"], rs["pos"], prev_pos)
    assert errs["position"] <= 1.0, f"position: {errs['position']:.3f} x (4 ulp + RTOL * displacement)"
    return errs


def test_linear_fused_step_within_tolerance(cuda):
    sc = block_collapse_3d(64, 32, 64)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=True, vel=vel)
    f.compute()
    g, gs = sorted_outputs(f, oracle.table_cells(sc.params)), state(f)
    r, rs = oracle_step(sc, vel)
    errs = compare_fast(g, gs, r, rs, sc.pos)
    print("fused-vs-restatement relative errors:", errs)
    assert f.sync_status() == OK


def test_linear_fused_steps_fed_identical_state(cuda):
    """Several steps; before each, the oracle is fed the GPU's own prior state (trajectories
    are chaotic, so single steps are compared, not long runs)."""
    sc = block_collapse_3d(48, 24, 48)
    vel = perturbed(sc, sigma=0.2)
    f = make_fluid(sc, fused=True, vel=vel)
    cells = oracle.table_cells(sc.params)
    for step in range(4):
        before = state(f)
        f.compute()
        g, gs = sorted_outputs(f, cells), state(f)
        pos, v, frc = before["pos"].copy(), before["vel"].copy(), before["force"].copy()
        r = oracle.step(pos, v, frc, sc.params)
        compare_fast(g, gs, r, {"pos": pos, "vel": v, "force": frc}, before["pos"])


def test_graph_replay_equals_eager(cuda):
    sc = block_collapse_3d(32, 16, 32)
    vel = perturbed(sc)
    a = make_fluid(sc, fused=True, graph=True, vel=vel)
    b = make_fluid(sc, fused=True, graph=False, vel=vel)
    for _ in range(5):
        a.compute()
        b.compute()
    sa, sb = state(a), state(b)
    for k in sa:
        assert_bit_exact(sa[k], sb[k], k)


@pytest.mark.parametrize("bw", [1, 3, 8])
def test_brick_width_does_not_change_results(cuda, bw):
    """Each target's candidate order depends only on its own neighbourhood, not on how cells
    are grouped into bricks."""
    sc = block_collapse_3d(32, 16, 32)
    vel = perturbed(sc)
    a = make_fluid(sc, vel=vel)
    b = make_fluid(sc, vel=vel)
    b.set_option(OPT_BRICK_WIDTH, bw)
    a.compute()
    b.compute()
    sa, sb = state(a), state(b)
    for k in sa:
        assert_bit_exact(sa[k], sb[k], k)


def disordered_block(nx=48, ny=24, nz=48, seed=11):
    """The block collapse's lattice jittered by up to one spacing (half a cell) per axis, so
    cells hold anything from a few to a dozen or more particles: the neighbour passes see
    every group size, sub-list layout (Q = 2 ... 8) and some overflowing sub-lists."""
    sc = block_collapse_3d(nx, ny, nz)
    sc.pos = lattice(nx, ny, nz, 0.01, (0.015, 0.015, 0.015), 0.01, seed)
    return sc


def test_disordered_block_within_tolerance_and_brick_width_free(cuda):
    sc = disordered_block()
    vel = perturbed(sc, sigma=0.2)
    a = make_fluid(sc, fused=True, vel=vel)
    a.compute()
    g, gs = sorted_outputs(a, oracle.table_cells(sc.params)), state(a)
    occ = np.unique(np.bincount(g["cell"].astype(np.int64)))
    assert len(occ) >= 8, occ  # the groups really vary (occupancies 0 ... 12 and more)
    r, rs = oracle_step(sc, vel)
    compare_fast(g, gs, r, rs, sc.pos)
    for bw in (1, 5, 8):
        b = make_fluid(sc, fused=True, vel=vel)
        b.set_option(OPT_BRICK_WIDTH, bw)
        b.compute()
        sb = state(b)
        for k in gs:
            assert_bit_exact(gs[k], sb[k], f"{k} (brick width {bw})")


def test_integrate_hook(cuda):
    """EVT_INTEGRATE as in libCL/TEST/main.cpp:246-343: the handler runs integrate-force,
    gravity and integrate-velocity itself and skips the clip box."""
    sc = hash_block(16)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=True, vel=vel)
    calls = []

    def handler(fluid, stream):
        calls.append(1)
        for st in (STAGE_INTEGRATE_FORCE, STAGE_GRAVITY, STAGE_INTEGRATE_VELOCITY):
            fluid.stage(st, stream)
        return 0

    f.addEventHandler(handler)
    f.compute()
    gs = state(f)
    assert calls == [1]
    p = sc.params
    pos, v, frc = sc.pos.copy(), vel.copy(), np.zeros_like(sc.pos)
    cell, index, spos, svel, cs, ce = oracle.front_end(pos, v, p)
    oracle.density(spos, svel, cs, ce, p)
    oracle.forces(spos, svel, frc, index, cs, ce, p)
    oracle.integrate_force(v, frc, p)
    oracle.gravity(frc, p)
    oracle.integrate_velocity(pos, v, p)
    for k, rv in (("pos", pos), ("vel", v), ("force", frc)):
        assert_bit_exact(gs[k], rv, k)


def test_hook_failure_is_reported(cuda):
    sc = hash_block(8)
    f = make_fluid(sc)
    f.addEventHandler(lambda fluid, stream: 3)
    from libcl_gb300 import ERR_STATE
    assert f.compute_raw() == ERR_STATE
    assert "hook" in f.last_error()


def test_reference_smoke_scene_runs(cuda):
    """The reference's own smoke run (256 particles, defaults): a few steps stay finite and
    particle 0 matches the restatement after one step."""
    sc = reference_test_scene(256)
    f = make_fluid(sc)
    f.compute()
    gs = state(f)
    r, rs = oracle_step(sc, sc.vel, ref_sort=True)
    for k in ("pos", "vel", "force"):
        assert_bit_exact(gs[k], rs[k], k)
    for _ in range(20):
        f.compute()
    assert np.isfinite(state(f)["pos"]).all()


def test_errors_and_validation(cuda):
    import torch
    f = Fluid3D()
    assert f.compute_raw() == ERR_NOT_COMPILED
    f.compile()
    assert f.compute_raw() == OK
    p = f.getParameters()
    saved = clone_params(p)
    p.cellSize = float("nan")
    assert f.compute_raw() == ERR_ARGUMENT
    set_params(f, saved)
    p.keyMode = 1
    p.gridDim[0] = 0
    assert f.compute_raw() == ERR_ARGUMENT
    set_params(f, saved)
    n = f.getParticleCount()
    assert n == 256
    bad = torch.zeros((n + 1, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(Exception) as e:
        f.setPositionBuffer(bad)
    assert e.value.status == ERR_SIZE_MISMATCH
    ok = torch.zeros((n + 8, 4), dtype=torch.float32, device="cuda")
    f.setVelocityBuffer(ok)  # velocity/force accept count >= N
    with pytest.raises(Exception):
        f.set_option(OPT_BRICK_WIDTH, 0)
    with pytest.raises(Exception) as e:
        f.setParticleCount(n + 100)  # the borrowed velocity buffer is too small
    assert e.value.status == ERR_SIZE_MISMATCH
    assert f.compute_raw() == OK
    torch.cuda.synchronize()


def test_borrowed_buffers(cuda):
    """setPositionBuffer/setVelocityBuffer with caller-owned memory (never freed by the fluid)."""
    import torch
    sc = block_collapse_3d(16, 8, 16)
    f = make_fluid(sc)
    pos = torch.from_numpy(sc.pos).cuda()
    vel = torch.zeros_like(pos)
    f.setPositionBuffer(pos)
    f.setVelocityBuffer(vel)
    f.compute()
    torch.cuda.synchronize()
    assert f.getPositionBuffer().data_ptr() == pos.data_ptr()
    assert not torch.equal(pos.cpu(), torch.from_numpy(sc.pos))  # moved in place
    del f
    torch.cuda.synchronize()
    assert torch.isfinite(pos).all()  # still valid memory after the fluid is gone


def test_c2_full_size_one_step(cuda):
    """1,048,576 particles, 200x100x200 grid: one fused step against the restatement."""
    sc = block_collapse_3d()
    f = make_fluid(sc, fused=True)
    f.compute()
    g, gs = sorted_outputs(f, oracle.table_cells(sc.params)), state(f)
    idx = g["index"]
    assert np.array_equal(np.sort(idx), np.arange(sc.n, dtype=np.uint32))
    assert np.all(g["cell"][1:] >= g["cell"][:-1])
    r, rs = oracle_step(sc, sc.vel)
    errs = compare_fast(g, gs, r, rs, sc.pos)
    print("C2 1M fused-vs-restatement relative errors:", errs)


def test_golden_fixture_bit_exact(cuda):
    """The exact kernels reproduce the independent pure-Python restatement's fixture
    (tests/golden/ref3d_hash_small.npz) bit for bit."""
    from pathlib import Path
    from libcl_gb300 import Fluid3DParams, default_params
    from libcl_gb300.scenes import Scene3D
    g = np.load(Path(__file__).resolve().parent / "golden" / "ref3d_hash_small.npz")
    p = default_params()
    for (name, _), v in zip(Fluid3DParams._fields_[:13], g["params"]):
        setattr(p, name, float(v))
    sc = Scene3D("golden", g["pos0"].copy(), g["vel0"].copy(), p)
    for fused in (False, True):
        f = make_fluid(sc, fused=fused)
        f.compute()
        o, s = sorted_outputs(f, REF_BUCKETS), state(f)
        for k in ("cell", "index", "spos", "svel"):
            assert_bit_exact(o[k], g[k], k)
        occ = g["occupied"]
        assert np.array_equal(np.nonzero(o["cell_start"] != 0xFFFFFFFF)[0], occ)
        assert_bit_exact(o["cell_start"][occ], g["cell_start"], "cellStart")
        assert_bit_exact(o["cell_end"][occ], g["cell_end"], "cellEnd")
        for k, gk in (("pos", "pos1"), ("vel", "vel1"), ("force", "force1")):
            assert_bit_exact(s[k], g[gk], k)


def test_dense_clump_takes_the_fallback_paths(cuda):
    """A clump of 3000 particles inside 2x2x2 cells: its bricks exceed the staging capacity
    and its particles have more neighbours than the per-particle lists hold, so the force
    kernel scans instead. Results must still agree with the restatement."""
    from libcl_gb300.scenes import SplitMix64
    sc = block_collapse_3d(24, 12, 24)
    rng = SplitMix64(99)
    clump = np.zeros((3000, 4), np.float32)
    clump[:, :3] = (0.5 + rng.uniform(9000).reshape(3000, 3) * 0.04).astype(np.float32)
    sc.pos = np.concatenate([sc.pos, clump])
    sc.vel = np.zeros_like(sc.pos)
    vel = perturbed(sc)
    f = make_fluid(sc, fused=True, vel=vel)
    f.compute()
    g, gs = sorted_outputs(f, oracle.table_cells(sc.params)), state(f)
    r, rs = oracle_step(sc, vel)
    errs = compare_fast(g, gs, r, rs, sc.pos, tol=1e-3)
    print("clump errors:", errs)
    assert f.sync_status() == OK


def test_dense_cloud_force_change_within_tolerance(cuda):
    """A uniform random cloud at about 15 particles per cell: the lanes' neighbour sub-lists
    of the density kernel are often exactly full, the case where a list entry could be
    overwritten by a later out-of-range candidate. The velocity change of one step (force *
    dt, without the initial velocities that would hide a force error) must agree with the
    restatement within 1e-3."""
    from libcl_gb300.scenes import SplitMix64
    sc = block_collapse_3d(8, 8, 8)
    nxc, nyc, nzc = 20, 10, 20
    n = 15 * nxc * nyc * nzc
    rng = SplitMix64(123)
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (rng.uniform(3 * n).reshape(n, 3) * np.array([nxc, nyc, nzc]) * 0.02 + 0.04).astype(np.float32)
    sc.pos = pos
    sc.vel = np.zeros_like(pos)
    vel = perturbed(sc, sigma=0.05)
    f = make_fluid(sc, fused=True, vel=vel)
    f.compute()
    gs = state(f)
    r, rs = oracle_step(sc, vel)
    e = rel_err(gs["vel"] - vel, rs["vel"] - vel)
    print("velocity-change relative error:", e)
    assert e <= 1e-3, e
    assert f.sync_status() == OK


def test_dam_break_2d_staged_bit_exact(cuda):
    """The 2D dam break (dims = 2: poly6/spiky constants for 2D, 9 neighbour cells, no z
    walls), exact kernels: bit-exact against the restatement."""
    from libcl_gb300.scenes import dam_break_2d
    sc = dam_break_2d()
    vel = perturbed(sc)
    vel[:, 2] = 0.0
    f = make_fluid(sc, fused=False, vel=vel)
    f.compute()
    g, gs = sorted_outputs(f, oracle.table_cells(sc.params)), state(f)
    r, rs = oracle_step(sc, vel)
    for k, rv in (("cell", r.cell), ("index", r.index), ("cell_start", r.cell_start), ("cell_end", r.cell_end),
                  ("spos", r.spos), ("svel", r.svel)):
        assert_bit_exact(g[k], rv, k)
    for k in ("pos", "vel", "force"):
        assert_bit_exact(gs[k], rs[k], k)


def test_dam_break_2d_fused_steps_fed_identical_state(cuda):
    """The 2D dam break on the brick kernels (3 neighbour rows): several steps, each compared
    with the restatement fed the GPU's prior state."""
    from libcl_gb300.scenes import dam_break_2d
    sc = dam_break_2d()
    vel = perturbed(sc)
    vel[:, 2] = 0.0
    f = make_fluid(sc, fused=True, vel=vel)
    cells = oracle.table_cells(sc.params)
    for _ in range(3):
        before = state(f)
        f.compute()
        g, gs = sorted_outputs(f, cells), state(f)
        pos, v, frc = before["pos"].copy(), before["vel"].copy(), before["force"].copy()
        r = oracle.step(pos, v, frc, sc.params)
        compare_fast(g, gs, r, {"pos": pos, "vel": v, "force": frc}, before["pos"])
    assert f.sync_status() == OK


def test_disordered_2d_block_within_tolerance_and_brick_width_free(cuda):
    """dims = 2 on the brick kernels with the dam break's lattice jittered by up to one spacing
    per axis: cells hold 0 to 9 particles, so every 2D group size and sub-list layout occurs."""
    from libcl_gb300.scenes import dam_break_2d
    sc = dam_break_2d()
    sc.pos = lattice(128, 128, 1, 0.005, (0.01, 0.01, 0.0), 0.005, 12)
    sc.pos[:, 2] = 0.0
    vel = perturbed(sc, sigma=0.2)
    vel[:, 2] = 0.0
    a = make_fluid(sc, fused=True, vel=vel)
    a.compute()
    g, gs = sorted_outputs(a, oracle.table_cells(sc.params)), state(a)
    assert len(np.unique(np.bincount(g["cell"].astype(np.int64)))) >= 7
    r, rs = oracle_step(sc, vel)
    compare_fast(g, gs, r, rs, sc.pos)
    for bw in (1, 6):
        b = make_fluid(sc, fused=True, vel=vel)
        b.set_option(OPT_BRICK_WIDTH, bw)
        b.compute()
        sb = state(b)
        for k in gs:
            assert_bit_exact(gs[k], sb[k], f"{k} (brick width {bw})")


def test_param_buffer_follows_the_host_parameters(cuda):
    """getParamBuffer (libCL/phys/oclFluid3D.cpp:198-201): a device record equal to
    getParameters(); a host edit reaches it with the next compute(), also when the step is a
    replayed graph, and through a stage() call."""
    import torch
    from libcl_gb300 import STAGE_GRAVITY
    sc = block_collapse_3d(16, 8, 16)
    f = make_fluid(sc)
    pb = f.getParamBuffer()
    torch.cuda.synchronize()

    def host_words():
        return np.frombuffer(bytes(f.getParameters()), np.float32)

    assert np.array_equal(pb.cpu().numpy().view(np.uint32), host_words().view(np.uint32))
    for _ in range(3):  # the third step replays the captured graph
        f.compute()
    f.getParameters().viscosity = 0.07
    f.compute()
    torch.cuda.synchronize()
    assert pb.cpu().numpy()[4] == np.float32(0.07)
    assert np.array_equal(pb.cpu().numpy().view(np.uint32), host_words().view(np.uint32))
    f.getParameters().stiffness = 2.5
    f.stage(STAGE_GRAVITY)
    torch.cuda.synchronize()
    assert pb.cpu().numpy()[8] == np.float32(2.5)
    assert f.sync_status() == OK


def test_emitter(cuda):
    """clEmitter (libCL/phys/oclFluid3D.cl:273-282): particles emit+1 .. emit+99 move to the
    sheet, the rest keep their state (expected values: fluid_helpers.emitter_expected, which
    the CPU tests pin to the reference's own kernel)."""
    sc = block_collapse_3d(8, 8, 8)
    vel = perturbed(sc)
    f = make_fluid(sc, vel=vel)
    f.emit(200, 1.5)
    g = state(f)
    pos, v = emitter_expected(sc.pos, vel, 200, 1.5, sc.params.particleRadius)
    np.testing.assert_array_equal(g["pos"].view(np.uint32), pos.view(np.uint32))
    np.testing.assert_array_equal(g["vel"], v)


@pytest.mark.parametrize("mode", ["pinned", "pageable", "staged"])
def test_compute_host_matches_device_steps(cuda, mode):
    """gbsph_fluid3d_compute_host (state uploaded from and downloaded to host memory around
    each step) gives bit for bit the state of the same steps run on device buffers: page-locked
    tensors (the replayed graph with overlapped uploads), pageable numpy arrays, and the
    per-stage kernels."""
    import torch
    sc = block_collapse_3d(48, 24, 48)
    vel = perturbed(sc)
    fused = mode != "staged"
    a = make_fluid(sc, fused=fused, vel=vel)
    b = make_fluid(sc, fused=fused, vel=vel)
    host = [sc.pos.copy(), vel.copy(), np.zeros_like(sc.pos)]
    if mode == "pinned":
        host = [torch.from_numpy(x).pin_memory() for x in host]
    for _ in range(4):
        a.compute()
        b.compute_host(*host)
        torch.cuda.synchronize()
    sa = state(a)
    for k, h in zip(("pos", "vel", "force"), host):
        hv = h.numpy() if hasattr(h, "numpy") else h
        assert_bit_exact(hv, sa[k], k)
    assert b.sync_status() == OK
