#!/usr/bin/env python
"""SPH particle-steps/s of the 3D block collapse (1,048,576 particles) on one GB300.

One "step" is one oclFluid3D::compute() of the whole scene: hash, one-sweep sort (+reorder),
cell bounds, density, forces + integration. Default: N=1 GPU, 500 timed steps after 5
warm-up steps, L2 flushed (512 MiB write) between timed steps, each step timed with CUDA
events on the stream it runs on. Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own kernels (libCL/phys/oclFluid3D.cl and
libCL/sort/oclRadixSort.cl, built for the host cores by oracle/ref/build.py through an OpenCL
C shim, OpenMP over work-groups) on the same scene, on its own hash keys, without loading
the product library; where they are not built, the oracle (the CPU port of those kernels).
With N>1 (torchrun) the plain step does not shard: every rank advances its own replica.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "SPH particle-steps/s, 1M 3D block collapse (plain step)"
UNIT = "particle-steps/s"
L2_FLUSH_BYTES = 512 << 20

# Algorithmic bytes per particle-step of each stage (the fixed per-stage figures of the step's
# byte budget: each array counted once per stage; neighbour re-reads, neighbour lists and
# cell-table reads not counted), mapped onto the fused step's launches:
STAGE_BYTES_PER_PARTICLE = {
    "front_end": 16 + 4 + 4,          # hash: R pos 16, W key 4, W index 4
    "sort": (4 + 16 * 3) + 68,        # histogram R key + 3 x 8-bit passes (R/W key, index), and the
                                      # reorder fused into the last pass: R index 4, R pos, vel 32,
                                      # W sorted pos, vel 32
    "bounds": 4,                      # R sorted key (+8 B per occupied cell, added below)
    "density": 16 + 4,                # R sorted pos 16, W density/pressure 4
    "forces": 16 + 16 + 4 + 4 + 32,   # R sorted pos, vel, density/pressure, index; W pos, vel
}
# The step adds 8 B per cell of the table (its initialisation) and 8 B per occupied cell.
TABLE_CELLS = 200 * 100 * 200
# The scene (both arms): the 3D block collapse; `l2` says how the timed steps treat caches.
WORKLOAD = {"workload": "3d_block_collapse_1M", "particles": 128 * 64 * 128, "lattice": [128, 64, 128],
            "grid": [200, 100, 200], "h": 0.02, "dt": 5e-5,
            "l2": "GPU arm: L2 flushed between timed steps (512 MiB write); host arm: not flushed"}


def workload_config(world: int) -> dict:
    return dict(WORKLOAD, parallelism=f"replicas x{world}")


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"]
        if self.gpu_id:
            cmd += ["-i", self.gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
            time.sleep(0.15)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self._t:
                self._t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def gpu_ident(torch) -> str | None:
    try:
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        u = getattr(props, "uuid", None)
        if u is not None:
            s = str(u)
            return s if s.startswith("GPU-") else "GPU-" + s
    except Exception:
        pass
    return None


def neighbour_flops(fluid, params, sample: int = 65536, seed: int = 9) -> dict:
    """Algorithmic FP32 work of the neighbour passes on the fluid's current (sorted) state,
    counted exactly on a random sample of particles: candidates of the 27-cell stencil and
    in-range pairs (the particle itself included), then density = candidates x 9 + in-range
    x 30 flops and forces = in-range x 60 flops per particle (the force pass evaluates only the
    listed pairs)."""
    import torch
    nx, ny, nz = (int(g) for g in params.gridDim[:3])
    cs, ce = fluid.cell_bounds(nx * ny * nz)
    keys = fluid.getCellBuffer().long() & 0xFFFFFFFF
    spos = fluid.getSortedPositionBuffer()[:, :3]
    n = keys.numel()
    g = torch.Generator(device="cuda").manual_seed(seed)
    i = torch.randint(0, n, (min(sample, n),), device="cuda", generator=g)
    k = keys[i]
    x, y, z = k % nx, (k // nx) % ny, k // (nx * ny)
    cs64 = cs.long() & 0xFFFFFFFF
    ce64 = ce.long() & 0xFFFFFFFF
    occ = torch.where(cs64 == 0xFFFFFFFF, torch.zeros_like(cs64), ce64 - cs64)
    maxocc = int(occ.max().item())
    thr = float(params.cellSize) ** 2
    pi = spos[i]
    cand = torch.zeros_like(k)
    inr = torch.zeros_like(k)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                cx, cy, cz = x + dx, y + dy, z + dz
                ok = (cx >= 0) & (cx < nx) & (cy >= 0) & (cy < ny) & (cz >= 0) & (cz < nz)
                c = torch.where(ok, cx + nx * (cy + ny * cz), torch.zeros_like(cx))
                st = cs64[c]
                ln = torch.where(ok, occ[c], torch.zeros_like(c))
                cand += ln
                for m in range(maxocc):
                    v = ln > m
                    j = torch.where(v, st + m, torch.zeros_like(st))
                    r2 = ((spos[j] - pi) ** 2).sum(dim=1)
                    inr += (v & (r2 < thr)).long()
    c_mean = float(cand.float().mean().item())
    r_mean = float(inr.float().mean().item())
    return {"sample_particles": int(i.numel()), "candidates_per_particle": c_mean,
            "in_range_per_particle": r_mean, "density_flops_per_particle": 9 * c_mean + 30 * r_mean,
            "forces_flops_per_particle": 60 * r_mean}


def sm_count(torch) -> int:
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def load_scene(fluid, scene):
    import ctypes
    import torch
    from libcl_gb300 import Fluid3DParams
    fluid.compile()
    fluid.setParticleCount(scene.n)
    ctypes.memmove(ctypes.byref(fluid.getParameters()), ctypes.byref(scene.params), ctypes.sizeof(Fluid3DParams))
    fluid.getPositionBuffer().copy_(torch.from_numpy(scene.pos))
    fluid.getVelocityBuffer().copy_(torch.from_numpy(scene.vel))
    fluid.getForceBuffer().zero_()
    torch.cuda.synchronize()


def reference_stepper(prefer_reference: bool = True):
    """One step of the block collapse as the reference computes it, on the host cores, built
    without the product library: positions from the seeded lattice (numpy), the System block
    from clInitFluid's formulas for h = 0.02 and viscosity 0.05, the reference's hash keys
    (262,144 buckets) and 4-bit block sort, clip box [0,4]x[0,2]x[0,4], gravity argument
    (0, 9.81f/9.8f, 0). With the reference's kernels built (oracle/ref) they run it
    (kind "reference"); otherwise, or with prefer_reference False, the oracle does (kind
    "port"). Returns (step function, kind, threads, particles, description)."""
    import oracle.ref as ref
    from libcl_gb300 import Fluid3DParams, KEY_REFERENCE_HASH
    from libcl_gb300.scenes import lattice
    h, sp = 0.02, 0.01
    pos = lattice(128, 64, 128, sp, (0.5 * sp,) * 3, 0.05 * h, 2)
    vel, force = np.zeros_like(pos), np.zeros_like(pos)
    use_ref = prefer_reference and ref.available()
    if use_ref:
        k = ref.kernel_constants(np.float32(h), np.float32(0.05))
    else:
        import oracle
        k = oracle.kernel_constants(np.float32(h), np.float32(0.05))
    system = np.array([5e-5, 0.5 * sp, h, 1000.0 * sp ** 3, 0.05, 0.0, 1000.0, sp, 3.0, k[1], k[2], k[0], 500.0],
                      np.float32)
    garg = np.array([0.0, np.float32(9.81) / np.float32(9.8), 0.0, 0.0], np.float32)
    lo, hi = np.zeros(4, np.float32), np.array([4.0, 2.0, 4.0, 0.0], np.float32)
    if use_ref:
        threads = ref.set_num_threads(0)

        def step():
            ref.step3d(pos, vel, force, system, garg, lo, hi)
        return step, "reference", threads, pos.shape[0], (
            "the reference's kernels (libCL/phys/oclFluid3D.cl, libCL/sort/oclRadixSort.cl) through an "
            "OpenCL C shim, work-groups on OpenMP threads, barrier kernels as coroutines")
    import oracle
    p = Fluid3DParams()
    for name, v in zip([f for f, _ in Fluid3DParams._fields_[:13]], system):
        setattr(p, name, float(v))
    g = np.float32(-9.8) * garg
    for i in range(4):
        p.gravity[i], p.boxMin[i], p.boxMax[i] = float(g[i]), float(lo[i]), float(hi[i])
    p.keyMode, p.dims = KEY_REFERENCE_HASH, 3

    def step():
        oracle.step(pos, vel, force, p, ref_sort=True)
    return step, "port", oracle.num_threads(), pos.shape[0], (
        "the oracle (the C++ restatement of the reference's kernels, its 4-bit block sort loop-fissioned), "
        "OpenMP")


def time_reference(step, n: int, warmup: int, max_steps: int, seconds: float):
    """Warm-up steps, then timed steps until `max_steps` or `seconds`; (particle-steps/s,
    steps, seconds)."""
    for _ in range(max(1, warmup)):
        step()
    steps, t0 = 0, time.perf_counter()
    while steps < max_steps:
        step()
        steps += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return n * steps / dt, steps, dt


def cpu_baseline(seconds: float = 10.0):
    """The reference's step on the host cores (reference_stepper) for about `seconds`."""
    step, kind, threads, n, what = reference_stepper()
    value, steps, dt = time_reference(step, n, 1, 50, seconds)
    return {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"{steps} full steps of the {n}-particle scene on the reference's hash keys ({dt:.1f} s): "
                      + what}


def _time_steps(fn, steps: int, stream) -> float:
    """Device milliseconds of `steps` calls of fn(), CUDA events on `stream`."""
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def extra_batched(stream, steps: int = 200, options: dict | None = None, loop: bool = True) -> dict:
    """256 independent scenes (log-uniform 4,096-262,144 particles, 17.3M in all): `steps`
    batched steps in the configuration the autotuner chose (step form, brick width, sort digit
    width, sort tile) or in `options` ({option: value}, no autotuning), the other step form
    beside it, and (with `loop`) the plain step looped over the same scenes for as many steps."""
    import torch
    from libcl_gb300 import BUF_FORCE, BUF_POSITION, BUF_VELOCITY, OPT_PERSISTENT, Batch3D, Fluid3D
    from libcl_gb300.scenes import batched_ensemble
    b = batched_ensemble()
    bt = Batch3D()
    bt.set_scenes(b.shared, b.descs)
    bt.buffer(BUF_POSITION).copy_(torch.from_numpy(b.pos))
    bt.buffer(BUF_VELOCITY).zero_()
    bt.buffer(BUF_FORCE).zero_()
    if options is None:
        bt.autotune(stream)
    else:
        for k, v in options.items():
            bt.set_option(k, v)
    cfg = bt.config()
    for _ in range(3):
        bt.compute(stream)
    t_b = _time_steps(lambda: bt.compute(stream), steps, stream)
    assert bt.sync_status() == 0
    # the other step form, same configuration otherwise, from the state reached
    bt.set_option(OPT_PERSISTENT, 1 - cfg["persistent"])
    for _ in range(3):
        bt.compute(stream)
    t_o = _time_steps(lambda: bt.compute(stream), steps, stream)
    assert bt.sync_status() == 0
    del bt
    forms = {cfg["persistent"]: t_b / steps, 1 - cfg["persistent"]: t_o / steps}
    out = {"scenes": len(b.descs), "particles": b.n, "steps": steps,
           "config": {"step_form": "persistent" if cfg["persistent"] else "staged graph",
                      "brick_width": cfg["brick_width"], "radix_bits": cfg["radix_bits"],
                      "sort_tile_keys": 256 * cfg["sort_tile_items"], "autotuned": options is None},
           "batched_particle_steps_per_s": b.n * steps / (t_b * 1e-3), "batched_ms_per_step": t_b / steps,
           "staged_graph_ms_per_step": forms[0], "persistent_ms_per_step": forms[1]}
    if not loop:
        return out
    fluids = []
    for s in range(len(b.descs)):
        f = Fluid3D()
        load_scene(f, b.scene(s))
        fluids.append(f)
    for _ in range(3):
        for f in fluids:
            f.compute(stream)
    t_l = _time_steps(lambda: [f.compute(stream) for f in fluids], steps, stream)
    looped = b.n * steps / (t_l * 1e-3)
    out.update({"looped_particle_steps_per_s": looped, "speedup": out["batched_particle_steps_per_s"] / looped,
                "looped_ms_per_step": t_l / steps})
    return out


def extra_sort(stream) -> dict:
    """16,777,216 (key, index) pairs: uniform 32-bit keys and Morton keys of a jittered lattice
    (0-20 particles per occupied cell, 2^22-cell table) + cell start/end extraction."""
    import torch
    from libcl_gb300 import RadixSort
    from libcl_gb300.scenes import SplitMix64
    n = 1 << 24
    rng = SplitMix64(3)
    uni = torch.from_numpy((rng.next_u64(n) >> np.uint64(32)).astype(np.uint32).view(np.int32)).cuda()
    counts = (SplitMix64(4).next_u64(1 << 22) % np.uint64(21)).astype(np.int64)
    cells = np.nonzero(np.cumsum(counts) <= n)[0]
    cid = np.repeat(cells, counts[cells])

    def spread(v):
        v = v.astype(np.uint64) & np.uint64(0x3FF)
        for sh, m in ((16, 0x030000FF), (8, 0x0300F00F), (4, 0x030C30C3), (2, 0x09249249)):
            v = (v | (v << np.uint64(sh))) & np.uint64(m)
        return v
    mort = (spread(cid % 128) | (spread((cid // 128) % 128) << np.uint64(1)) | (spread(cid // 16384) << np.uint64(2)))
    mort = mort.astype(np.uint32)[np.argsort(SplitMix64(5).next_u64(cid.size), kind="stable")]
    mor = torch.from_numpy(mort.view(np.int32)).cuda()
    sorter = RadixSort()
    out = {}
    for name, keys, bits in (("uniform32", uni, 32), ("morton24", mor, 24)):
        vals = torch.arange(keys.numel(), dtype=torch.int32, device="cuda")
        k, v = keys.clone(), vals.clone()
        sorter.compute(k, v, 0, bits, stream)  # warm-up (allocates)
        reps = 5
        ts = []
        for _ in range(reps):
            k.copy_(keys)
            v.copy_(vals)
            ts.append(_time_steps(lambda: sorter.compute(k, v, 0, bits, stream), 1, stream))
        ms = statistics.median(ts)
        out[name] = {"pairs": keys.numel(), "ms": ms, "pairs_per_s": keys.numel() / (ms * 1e-3),
                     "hbm_gbs_algorithmic": (4 + 16 * ((bits + 7) // 8)) * keys.numel() / (ms * 1e-3) / 1e9}
    cs = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    ce = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    ms = _time_steps(lambda: sorter.cell_bounds(k, cs, ce, stream), 5, stream) / 5
    out["cell_bounds_2^22_ms"] = ms
    assert sorter.sync_status() == 0
    # CPU beside it: the restated reference sort (4-bit passes of 256-key blocks, host cores)
    # at its largest accepted size, 4,190,208 pairs (it refuses 2^22), and std::stable_sort on
    # the 16M uniform pairs
    import oracle
    ku = (SplitMix64(3).next_u64(n) >> np.uint64(32)).astype(np.uint32)
    m = (1 << 22) - 4096
    kk, vv = ku[:m].copy(), np.arange(m, dtype=np.uint32)
    t0 = time.perf_counter()
    assert oracle.radix_sort_reference(kk, vv, 0, 32) == 0
    t_ref = time.perf_counter() - t0
    kk, vv = ku.copy(), np.arange(n, dtype=np.uint32)
    t0 = time.perf_counter()
    oracle.stable_sort(kk, vv, 0, 32)
    t_std = time.perf_counter() - t0
    out["cpu"] = {"cores": oracle.num_threads(),
                  "reference_sort_4190208_pairs_per_s": m / t_ref,
                  "std_stable_sort_16m_pairs_per_s": n / t_std}
    return out


def extra_2d(stream, steps: int = 500) -> dict:
    """The 2D dam break (16,384 particles, poly6/spiky on the 3D step with dims = 2) and the
    reference's own 2D relaxation model (oclFluid2D, 16,384 particles)."""
    import torch
    from libcl_gb300 import Fluid2D, Fluid3D
    from libcl_gb300.scenes import dam_break_2d
    sc = dam_break_2d()
    f = Fluid3D()
    load_scene(f, sc)
    for _ in range(5):
        f.compute(stream)
    t = _time_steps(lambda: f.compute(stream), steps, stream)
    assert f.sync_status() == 0
    out = {"dam_break_poly6_2d": {"particles": sc.n, "ms_per_step": t / steps,
                                  "particle_steps_per_s": sc.n * steps / (t * 1e-3)}}
    g = Fluid2D()
    g.compile()
    n = g.getParticleCount()
    st = np.zeros((n, 6), np.float32)
    side = int(np.sqrt(n))
    iy, ix = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    st[:, 0], st[:, 1], st[:, 4] = 1.0 + ix.ravel() * 0.06, 1.0 + iy.ravel() * 0.06, 0.7
    g.getStateBuffer().copy_(torch.from_numpy(st))
    mask = np.zeros((256, 256, 4), np.float32)
    mask[:8, :, 3] = mask[-8:, :, 3] = mask[:, :8, 3] = mask[:, -8:, 3] = 1
    g.computeBorder(torch.from_numpy(mask).cuda(), stream)
    for _ in range(5):
        g.compute(stream)
    t = _time_steps(lambda: g.compute(stream), steps, stream)
    assert g.sync_status() == 0
    out["reference_relaxation_2d"] = {"particles": n, "ms_per_step": t / steps,
                                      "particle_steps_per_s": n * steps / (t * 1e-3)}
    return out


def extra_hash_mode(stream, steps: int = 50) -> dict:
    """The 1M 3D block collapse on the reference's default keys (262,144-bucket hash, the exact
    kernels in the reference's summation order), from the start of the collapse."""
    import statistics
    from libcl_gb300 import KEY_REFERENCE_HASH, OPT_PROFILE, Fluid3D
    from libcl_gb300.scenes import block_collapse_3d
    sc = block_collapse_3d()
    f = Fluid3D()
    load_scene(f, sc)
    f.getParameters().keyMode = KEY_REFERENCE_HASH
    for _ in range(5):
        f.compute(stream)
    t = _time_steps(lambda: f.compute(stream), steps, stream)
    f.set_option(OPT_PROFILE, 1)
    acc = {}
    for _ in range(5):
        f.compute(stream)
        for k, v in f.stage_times().items():
            acc.setdefault(k, []).append(v)
    f.set_option(OPT_PROFILE, 0)
    assert f.sync_status() == 0
    return {"particles": sc.n, "ms_per_step": t / steps, "particle_steps_per_s": sc.n * steps / (t * 1e-3),
            "stages_ms": {k: statistics.median(v) for k, v in acc.items()}}


def extra_adjoint(stream) -> dict:
    """Forward + adjoint against forward alone: the differentiable rollout (65,536 particles,
    200 steps, checkpoint every 20) and the 1M block collapse (20 steps, checkpoint every 10).
    The adjoint's time covers forward() (the steps plus checkpoints) and backward()
    (recomputation with recording, then the reverse kernels)."""
    import torch
    from libcl_gb300 import Adjoint3D, Fluid3D
    from libcl_gb300.scenes import block_collapse_3d, differentiable_block
    out = {}
    for name, sc, steps, every in (("differentiable_block_64k", differentiable_block(), 200, 20),
                                   ("block_collapse_1M", block_collapse_3d(), 20, 10)):
        f = Fluid3D()
        load_scene(f, sc)
        grav = torch.tensor(list(sc.params.gravity), dtype=torch.float32, device="cuda")
        f.getForceBuffer().copy_(grav.expand(sc.n, 4))
        pos0 = f.getPositionBuffer().clone()
        vel0 = f.getVelocityBuffer().clone()

        def reset():
            f.getPositionBuffer().copy_(pos0)
            f.getVelocityBuffer().copy_(vel0)
            f.getForceBuffer().copy_(grav.expand(sc.n, 4))

        for _ in range(3):
            f.compute(stream)
        reset()
        t_fwd = _time_steps(lambda: f.compute(stream), steps, stream)
        adj = Adjoint3D(f, steps, every)
        gpos = torch.full((sc.n, 4), 1e-6, dtype=torch.float32, device="cuda")
        gp0, gv0 = torch.empty_like(gpos), torch.empty_like(gpos)
        gpar = torch.empty(2, dtype=torch.float64, device="cuda")
        reps = []
        for _ in range(3):  # the first run captures graphs and warms up
            reset()
            t_a = _time_steps(lambda: adj.forward(stream), 1, stream)
            t_b = _time_steps(lambda: adj.backward_raw(gpos, None, gp0, gv0, gpar, stream), 1, stream)
            reps.append((t_a, t_b))
        t_a, t_b = min(reps, key=lambda r: r[0] + r[1])
        assert f.sync_status() == 0
        out[name] = {"particles": sc.n, "steps": steps, "checkpoint_every": every,
                     "forward_ms": t_fwd, "adjoint_forward_ms": t_a, "adjoint_backward_ms": t_b,
                     "fwd_plus_adj_over_fwd": (t_a + t_b) / t_fwd,
                     "fwd_plus_adj_particle_steps_per_s": sc.n * steps / ((t_a + t_b) * 1e-3)}
        if name == "differentiable_block_64k":
            # CPU beside it: the FP64 oracle's forward + adjoint on a 10-step sample (K = 5)
            import oracle
            p64 = sc.pos.astype(np.float64)
            v64 = np.zeros_like(p64)
            f64 = np.zeros_like(p64)
            f64[:, :3] = np.array(list(sc.params.gravity)[:3])
            g64 = np.zeros_like(p64)
            g64[:, :3] = 1e-6
            t0 = time.perf_counter()
            oracle.adjoint_f64(p64, v64, f64, sc.params, 10, 5, g64)
            dt = time.perf_counter() - t0
            out[name]["cpu_fp64_fwd_plus_adj"] = {"cores": oracle.num_threads(), "sample_steps": 10,
                                                  "particle_steps_per_s": sc.n * 10 / dt}
        del adj, f
        torch.cuda.empty_cache()
    return out


def extra_bvh(stream) -> dict:
    """The triangle-mesh BVH build (the reference's other radix-sort user): 1,000,000 small
    triangles on a jittered 100^3 lattice, shuffled; one build = box, Morton keys, 32-bit sort,
    nodes, links, leaves, boxes. The CPU restatement of the reference build, single-threaded,
    on the same mesh beside it."""
    import torch
    import oracle
    from libcl_gb300 import BvhTrimesh
    from libcl_gb300.scenes import lattice_soup
    v, idx = lattice_soup(100)
    dv = torch.from_numpy(v).cuda()
    di = torch.from_numpy(idx.view(np.int32)).cuda()
    b = BvhTrimesh()
    for _ in range(3):
        b.compute(dv, di, stream)
    ts = [_time_steps(lambda: b.compute(dv, di, stream), 1, stream) for _ in range(10)]
    assert b.sync_status() == 0
    ms = statistics.median(ts)
    t0 = time.perf_counter()
    oracle.bvh_build(v, idx, np.zeros(8, np.float32))
    cpu_s = time.perf_counter() - t0
    n = idx.size // 3
    return {"triangles": n, "ms": ms, "triangles_per_s": n / (ms * 1e-3),
            "cpu_reference_port_ms": cpu_s * 1e3, "cpu_cores": 1}


def extra_bvh_lines(stream) -> dict:
    """The 2D segment BVH build (oclBvhLines): 1,000,000 short segments on a 1000^2 lattice
    of distinct integer midpoints, shuffled; one build = Morton keys, 32-bit sort, nodes,
    links, leaves, boxes. The CPU restatement of the reference build, single-threaded, on the
    same segments beside it."""
    import torch
    import oracle
    from libcl_gb300 import BvhLines
    from libcl_gb300.scenes import segment_lattice
    v = segment_lattice(1000)
    dv = torch.from_numpy(v).cuda()
    b = BvhLines()
    for _ in range(3):
        b.compute(dv, stream)
    ts = [_time_steps(lambda: b.compute(dv, stream), 1, stream) for _ in range(10)]
    assert b.sync_status() == 0
    ms = statistics.median(ts)
    t0 = time.perf_counter()
    oracle.bvh_lines_build(v)
    cpu_s = time.perf_counter() - t0
    n = v.shape[0] // 2
    return {"segments": n, "ms": ms, "segments_per_s": n / (ms * 1e-3),
            "cpu_reference_port_ms": cpu_s * 1e3, "cpu_cores": 1}


def profile_suite(stream) -> None:
    """One untimed pass over every hot path, sized for a per-kernel ncu capture (about 1 GB on
    the device at a time): 3 fused steps of the 1M block collapse, on the linear grid and on the
    reference's hash keys (exact kernels); the 16M uniform and Morton
    sorts with cell bounds; 2 steps of a 32-scene batch; a 10-step adjoint (checkpoint every
    5) of the 65,536-particle block; the 1M-triangle and 1M-segment BVH builds and a collision
    pass; 3 steps of the 2D dam break (dims = 2) and of the 2D relaxation model."""
    import torch
    from libcl_gb300 import (BUF_FORCE, BUF_POSITION, BUF_VELOCITY, KEY_REFERENCE_HASH, Adjoint3D, Batch3D,
                             BvhLines, BvhTrimesh, Fluid2D, Fluid3D, RadixSort, default_params)
    from libcl_gb300.scenes import (SplitMix64, batched_ensemble, block_collapse_3d, dam_break_2d,
                                    differentiable_block, lattice_soup, segment_lattice, sphere_mesh)

    def done():
        torch.cuda.synchronize()
        torch.cuda.empty_cache()

    for hash_keys in (False, True):
        f = Fluid3D()
        load_scene(f, block_collapse_3d())
        if hash_keys:
            f.getParameters().keyMode = KEY_REFERENCE_HASH
        for _ in range(3):
            f.compute(stream)
        assert f.sync_status() == 0
        del f
        done()
    n = 1 << 24
    rng = SplitMix64(3)
    keys = torch.from_numpy((rng.next_u64(n) >> np.uint64(32)).astype(np.uint32).view(np.int32)).cuda()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    s = RadixSort()
    s.compute(keys, vals, 0, 32, stream)
    keys.random_(0, 1 << 22)
    s.compute(keys, vals, 0, 24, stream)
    cs = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    ce = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    s.cell_bounds(keys, cs, ce, stream)
    assert s.sync_status() == 0
    del keys, vals, cs, ce, s
    done()
    b = batched_ensemble(n_scenes=32)
    bt = Batch3D()
    bt.set_scenes(b.shared, b.descs)
    bt.buffer(BUF_POSITION).copy_(torch.from_numpy(b.pos))
    bt.buffer(BUF_VELOCITY).zero_()
    bt.buffer(BUF_FORCE).zero_()
    for _ in range(2):
        bt.compute(stream)
    assert bt.sync_status() == 0
    del bt
    done()
    sc = differentiable_block()
    f = Fluid3D()
    load_scene(f, sc)
    adj = Adjoint3D(f, 10, 5)
    gpos = torch.full((sc.n, 4), 1e-6, dtype=torch.float32, device="cuda")
    gp0, gv0 = torch.empty_like(gpos), torch.empty_like(gpos)
    gpar = torch.empty(2, dtype=torch.float64, device="cuda")
    adj.forward(stream)
    adj.backward_raw(gpos, None, gp0, gv0, gpar, stream)
    assert f.sync_status() == 0
    del adj, f
    done()
    v, idx = lattice_soup(100)
    bv = BvhTrimesh()
    bv.compute(torch.from_numpy(v).cuda(), torch.from_numpy(idx.view(np.int32)).cuda(), stream)
    sv, si = sphere_mesh(24, 48)
    dsv, dsi = torch.from_numpy(sv).cuda(), torch.from_numpy(si.view(np.int32)).cuda()
    bv.compute(dsv, dsi, stream)
    npart = 20000
    d = rng.normal(3 * npart).reshape(npart, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pos = np.zeros((npart, 4), np.float32)
    vel = np.zeros((npart, 4), np.float32)
    pos[:, :3] = 1.0 + d * 0.505
    vel[:, :3] = -d * 2.0
    dp, dvl = torch.from_numpy(pos).cuda(), torch.from_numpy(vel).cuda()
    bv.collide(default_params(), dp, dvl, torch.zeros_like(dp), dsv, dsi, stream)
    assert bv.sync_status() == 0
    bl = BvhLines()
    bl.compute(torch.from_numpy(segment_lattice(1000)).cuda(), stream)
    assert bl.sync_status() == 0
    del bv, bl
    done()
    f = Fluid3D()
    load_scene(f, dam_break_2d())
    for _ in range(3):
        f.compute(stream)
    assert f.sync_status() == 0
    del f
    g = Fluid2D()
    g.compile()
    m = g.getParticleCount()
    st = np.zeros((m, 6), np.float32)
    side = int(np.sqrt(m))
    iy, ix = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    st[:, 0], st[:, 1], st[:, 4] = 1.0 + ix.ravel() * 0.06, 1.0 + iy.ravel() * 0.06, 0.7
    g.getStateBuffer().copy_(torch.from_numpy(st))
    mask = np.zeros((256, 256, 4), np.float32)
    mask[:8, :, 3] = mask[-8:, :, 3] = mask[:, :8, 3] = mask[:, -8:, 3] = 1
    g.computeBorder(torch.from_numpy(mask).cuda(), stream)
    for _ in range(3):
        g.compute(stream)
    assert g.sync_status() == 0
    done()
    print("profile suite ok", flush=True)


def run_reference(args, rank, world):
    """--impl reference: the reference's own step on the host cores (reference_stepper; the
    product library is not loaded) on the full 1M scene: `--warmup` untimed steps, then the
    timed steps, at most `--steps` or as many as fit in 120 s. Beside it, the oracle port's
    rate on a 20 s sample of the same scene."""
    if rank != 0:
        return 0
    step, kind, threads, n, what = reference_stepper()
    value, steps, dt = time_reference(step, n, args.warmup, args.steps, 120.0)
    sample = f"{steps} full steps of the {n}-particle scene after {max(1, args.warmup)} warm-up steps: {what}"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded jittered lattice, block_collapse_3d seed 2)",
        "config": workload_config(world),
        "keys": "reference hash (262,144 buckets), 4-bit block radix sort",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    if kind == "reference":
        pstep, _, pthreads, _, pwhat = reference_stepper(prefer_reference=False)
        pvalue, psteps, pdt = time_reference(pstep, n, 1, 50, 20.0)
        line["port"] = {"value": pvalue, "unit": UNIT, "cores": pthreads, "kind": "port",
                        "sample": f"{psteps} full steps ({pdt:.1f} s): {pwhat}"}
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--quick", action="store_true", help="skip e2e/profile/baseline legs (for ncu)")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched / sort / 2D side measurements")
    ap.add_argument("--brick-width", type=int, default=0, help="cells per neighbour brick (0: library default)")
    ap.add_argument("--keys", default="linear", choices=["linear", "reference-hash"],
                    help="cell keys of the timed step: the bounded linear grid (default) or the reference's "
                         "262,144-bucket hash with the exact kernels")
    ap.add_argument("--profile-suite", action="store_true",
                    help="run every hot path once, untimed (the workload of the per-kernel ncu summary)")
    ap.add_argument("--batched-only", action="store_true",
                    help="run only the 256-scene batched step, both forms, --steps timed steps each, in the "
                         "configuration given by --brick-width / --radix-bits / --sort-tile (no autotuning, "
                         "no looped baseline): the workload of the batched step's launch list")
    ap.add_argument("--radix-bits", type=int, default=8, help="--batched-only: sort digit width")
    ap.add_argument("--sort-tile", type=int, default=16, help="--batched-only: sort keys per thread (8 or 16)")
    args = ap.parse_args(argv)
    if args.batched_only:
        import torch
        from libcl_gb300 import OPT_BRICK_WIDTH, OPT_RADIX_BITS, OPT_SORT_TILE
        torch.cuda.set_device(0)
        opts = {OPT_BRICK_WIDTH: args.brick_width or 16, OPT_RADIX_BITS: args.radix_bits, OPT_SORT_TILE: args.sort_tile}
        print(json.dumps(extra_batched(torch.cuda.current_stream(), steps=args.steps, options=opts, loop=False)))
        return 0
    if args.profile_suite:
        import torch
        torch.cuda.set_device(0)
        profile_suite(torch.cuda.current_stream())
        return 0
    rank, world, local = env_rank()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.warmup < 3:
        print("warmup must be >= 3", file=sys.stderr)
        return 2

    import torch
    import torch.distributed as dist
    from libcl_gb300 import OPT_PROFILE, Fluid3D
    from libcl_gb300.scenes import block_collapse_3d
    from libcl_gb300.sharding import max_over_ranks

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    scene = block_collapse_3d()
    fluid = Fluid3D()
    load_scene(fluid, scene)
    if args.brick_width:
        from libcl_gb300 import OPT_BRICK_WIDTH
        fluid.set_option(OPT_BRICK_WIDTH, args.brick_width)
    if args.keys == "reference-hash":
        from libcl_gb300 import KEY_REFERENCE_HASH
        fluid.getParameters().keyMode = KEY_REFERENCE_HASH
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        fluid.compute(stream)
    torch.cuda.synchronize()
    assert fluid.sync_status() == 0, fluid.last_error()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(gpu_ident(torch)) as clocks:
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            fluid.compute(stream)
            ends[i].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    t_ms = float(sum(step_ms))
    t_ms = max_over_ranks(t_ms, device="cuda")
    status = fluid.sync_status()
    if status != 0:
        print(f"device status {status}: {fluid.last_error()}", file=sys.stderr)
        return 1
    value = scene.n * args.steps * world / (t_ms * 1e-3)
    # linear grid: hash, 3 sort passes, bounds, density, forces; reference hash: the same with
    # the exact density and forces, plus the fused clip-box / integration kernel
    launches_per_step = 7 if args.keys == "linear" else 8

    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded jittered lattice, block_collapse_3d seed 2)",
        "config": workload_config(world),
        "keys": ("linear grid 200x100x200, 3 x 8-bit one-sweep passes" if args.keys == "linear" else
                 "reference hash (262,144 buckets), exact kernels"),
        "graph": True,
        "gpu_launches": launches_per_step * args.steps,
        "step_ms_p50": statistics.median(step_ms),
    }
    cs = clocks.summary()
    result["clocks"] = cs

    if not args.quick and rank == 0:
        # per-stage events on the launching stream (eager replay of the same fused kernels)
        fluid.set_option(OPT_PROFILE, 1)
        acc: dict[str, list[float]] = {}
        n_cells_occ = None
        for _ in range(20):
            flush.zero_()
            fluid.compute(stream)
            for k, v in fluid.stage_times().items():
                acc.setdefault(k, []).append(v)
        fluid.set_option(OPT_PROFILE, 0)
        cell = fluid.getCellBuffer()
        n_cells_occ = int((cell[1:] != cell[:-1]).sum().item()) + 1
        stage_ms = {k: statistics.median(v) for k, v in acc.items()}
        peak, peak_kind = measured_peaks()
        stage_gbs = {}
        for k, ms in stage_ms.items():
            b = STAGE_BYTES_PER_PARTICLE[k] * scene.n + (8 * n_cells_occ if k == "bounds" else 0)
            stage_gbs[k] = b / (ms * 1e-3) / 1e9
        dom = max(stage_ms, key=stage_ms.get)
        dom_bytes = STAGE_BYTES_PER_PARTICLE[dom] * scene.n
        ach = stage_gbs[dom]
        if args.keys == "linear":  # byte and flop counts of the linear-grid step's kernels
            # DRAM bytes of one launch from the committed ncu capture named in the file (not
            # measured in this run)
            traffic, traffic_src = None, None
            tp = ROOT / "profiles" / "traffic.json"
            if tp.exists():
                rec = json.loads(tp.read_text()).get(dom)
                if rec:
                    traffic = rec["dram_bytes_per_launch"]
                    traffic_src = f"ncu, {rec['profile']} (kernels of commit {rec['commit']})"
            result["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                                  "frac": ach / peak, "peak_source": peak_kind, "traffic": traffic,
                                  "traffic_source": traffic_src,
                                  "algorithmic_bytes_per_launch": dom_bytes, "avg_launch_ms": stage_ms[dom]}
            fl = neighbour_flops(fluid, scene.params)
            fp32_peak = sm_count(torch) * 128 * 2 * (result["clocks"].get("sm_mhz") or 2070.0) * 1e6 / 1e12
            fl["fp32_peak_tflops"] = fp32_peak
            fl["fp32_peak_source"] = "derived: SMs x 128 FP32 lanes x 2 (FMA) x median SM clock of the timed run"
            for stg in ("density", "forces"):
                tf = fl[f"{stg}_flops_per_particle"] * scene.n / (stage_ms[stg] * 1e-3) / 1e12
                fl[f"{stg}_achieved_tflops"] = tf
                fl[f"{stg}_fp32_frac"] = tf / fp32_peak
            result["flops"] = fl
        step_bytes = sum(STAGE_BYTES_PER_PARTICLE.values()) * scene.n + 8 * TABLE_CELLS + 8 * n_cells_occ
        result["stages"] = {"ms": stage_ms, "gbs": stage_gbs, "occupied_cells": n_cells_occ,
                            "step_algorithmic_bytes": step_bytes,
                            "step_hbm_frac": step_bytes / (t_ms / args.steps * 1e-3) / 1e9 / peak}

        # end to end through the C ABI with host buffers: each step uploads its inputs
        # (position, velocity, force) from pinned memory, computes, and downloads the result
        # (gbsph_fluid3d_compute_host: the velocity and force uploads overlap the hash, sort
        # and density passes)
        from libcl_gb300 import BUF_FORCE, BUF_POSITION, BUF_VELOCITY
        hp = [torch.empty((scene.n, 4), dtype=torch.float32, pin_memory=True) for _ in range(3)]
        for h, w in zip(hp, (BUF_POSITION, BUF_VELOCITY, BUF_FORCE)):
            h.copy_(fluid.buffer(w).cpu())
        k_e2e = min(args.steps, 200)
        fluid.compute_host(*hp, stream=stream)  # captures the step-with-copies graph
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k_e2e):
            fluid.compute_host(*hp, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1)
        result["e2e"] = {"value": scene.n * k_e2e / (e2e_ms * 1e-3), "unit": UNIT,
                         "h2d_bytes_per_step": 3 * 16 * scene.n, "d2h_bytes_per_step": 3 * 16 * scene.n,
                         "steps": k_e2e}
        if not args.no_extras:
            del fluid, flush
            torch.cuda.empty_cache()
            result["extras"] = {"batched_256_scenes": extra_batched(stream), "sort_16m": extra_sort(stream),
                                "reference_hash_keys_1m": extra_hash_mode(stream),
                                "two_d": extra_2d(stream), "adjoint": extra_adjoint(stream),
                                "bvh_1m_triangles": extra_bvh(stream),
                                "bvh_lines_1m_segments": extra_bvh_lines(stream)}
        if world == 1 and not args.no_cpu_baseline:
            result["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
