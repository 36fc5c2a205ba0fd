"""Host logic of the multi-GPU layout on CPU: scene shards and the max-over-ranks timing,
with two gloo ranks."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from libcl_gb300.sharding import max_over_ranks, scene_shards


def test_scene_shards_cover_each_scene_once():
    counts = [4096, 262144, 9000, 70000, 5000, 150000, 4096, 30000]
    for world in (1, 2, 3, 4, 8, 11):
        sh = scene_shards(counts, world)
        assert len(sh) == world
        assert sh[0][0] == 0 and sh[-1][1] == len(counts)
        for (a, b), (c, d) in zip(sh, sh[1:]):
            assert b == c and a <= b
    # balance: with many equal scenes the split is even
    sh = scene_shards([1000] * 64, 4)
    assert [b - a for a, b in sh] == [16, 16, 16, 16]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank times its own replica; the job's time is the slowest rank's
        t = max_over_ranks(10.0 + rank)
        counts = [5000 + 1000 * i for i in range(10)]
        first, last = scene_shards(counts, world)[rank]
        mine = sum(counts[first:last])
        import torch
        tot = torch.tensor([mine], dtype=torch.int64)
        dist.all_reduce(tot)
        out[rank] = (t, int(tot.item()), sum(counts))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_max_timing_and_scene_partition():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        t, tot, want = out[r]
        assert t == 11.0
        assert tot == want
