"""Failure detection without a GPU fault: the library's bounded device waits give up, report
GBSPH_ERR_DEVICE_TIMEOUT through the host, and leave the context usable.

gbsph_selftest_bounded_wait(0) runs the one-sweep sort pass with its tile counter started at
1, so the look-back of tile 1 waits on tile 0's status, which nothing writes;
gbsph_selftest_bounded_wait(1) waits on an mbarrier expecting bytes that no copy delivers;
gbsph_selftest_bounded_wait(3) has two CTAs wait at the persistent batch step's grid-wide
barrier for a third that does not exist. Each wait is bounded by about one second of device
time."""
import time

import numpy as np
import pytest

from libcl_gb300 import ERR_ARGUMENT, ERR_DEVICE_TIMEOUT, OK, RadixSort, load_library

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 3])
def test_bounded_wait_times_out_and_context_survives(cuda, which):
    import torch
    lib = load_library()
    t0 = time.perf_counter()
    rc = lib.gbsph_selftest_bounded_wait(which, None)
    dt = time.perf_counter() - t0
    assert rc == ERR_DEVICE_TIMEOUT, rc
    assert 0.5 < dt < 30.0, dt
    # the context still works: a sort right after is correct
    keys = torch.randint(0, 1 << 30, (100_000,), dtype=torch.int32, device="cuda")
    vals = torch.arange(keys.numel(), dtype=torch.int32, device="cuda")
    ref = torch.sort(keys, stable=True)
    s = RadixSort()
    s.compute(keys, vals, 0, 32)
    torch.cuda.synchronize()
    assert s.sync_status() == OK
    assert torch.equal(keys, ref.values) and torch.equal(vals.long(), ref.indices)


def test_bounded_wait_rejects_unknown_probe(cuda):
    assert load_library().gbsph_selftest_bounded_wait(7, None) == ERR_ARGUMENT
