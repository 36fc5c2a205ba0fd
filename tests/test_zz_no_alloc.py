"""The allocation-free sort entry point, gbsph_radix_sort_noalloc, called through the C ABI.

It exists for callers that cannot allocate device memory (a host framework that owns all
device memory, real-time loops that must not stall on cudaMalloc/cudaFree, plugins with a
fixed footprint); its scratch is a static device array shared by every call. Each check
compares it with the definition of a stable LSD sort (numpy's stable argsort of the key bit
field) and with the allocating entry point, gbsph_radix_sort_compute, on the same input.
The sort is integer work, so the comparisons are exact. Two calls run back to back so that
whatever the first call leaves in the shared scratch array cannot change the second result.
gbsph_radix_sort_noalloc_status reports a device-side fault recorded in the array (a
look-back wait driven to its one-second bound by gbsph_selftest_bounded_wait(2)).
This file is named to be collected last."""
import ctypes
import time

import numpy as np
import pytest

from libcl_gb300 import ERR_DEVICE_TIMEOUT, ERR_TOO_LARGE, OK, RadixSort, load_library
from libcl_gb300.scenes import SplitMix64

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 262144


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def _expected(keys, vals, start, end):
    """Stable sort by key bits [start, end): the definition any stable LSD sort meets."""
    width = end - start
    mask = np.uint64((1 << width) - 1)
    field = (keys.astype(np.uint64) >> np.uint64(start)) & mask
    o = np.argsort(field, kind="stable")
    return keys[o], vals[o]


def _noalloc(keys, vals, start, end, stream=None):
    import torch
    lib = load_library()
    handle = (stream or torch.cuda.current_stream()).cuda_stream
    return lib.gbsph_radix_sort_noalloc(ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(vals.data_ptr()),
                                        keys.numel(), vals.numel(), start, end, ctypes.c_void_p(handle))


def _status(stream=None):
    import torch
    handle = (stream or torch.cuda.current_stream()).cuda_stream
    return load_library().gbsph_radix_sort_noalloc_status(ctypes.c_void_p(handle))


# (sizes of the two calls, bit range, run on a stream of its own): 4, 3, 2 and 1 passes of
# 8 bits, and non-zero start bits (8, 32) and (4, 12)
CASES = [((200_000, 4097), (0, 32), False), ((NOALLOC_MAX, 1000), (0, 24), False),
         ((70_000, 70_000), (0, 16), False), ((65_536, 3), (0, 8), False),
         ((150_000, 99_999), (8, 32), True), ((131_072, 77), (4, 12), True)]


@pytest.mark.parametrize("sizes,bits,own_stream", CASES)
def test_noalloc_matches_stable_sort_and_allocating_sort(cuda, sizes, bits, own_stream):
    import torch
    stream = torch.cuda.Stream() if own_stream else None
    ref = RadixSort()
    for call, n in enumerate(sizes):
        rng = SplitMix64(1000 + call + 17 * bits[0])
        keys = (rng.next_u64(n) >> np.uint64(32)).astype(np.uint32)
        keys[::7] = keys[0]  # runs of equal keys: stability matters
        vals = np.arange(n, dtype=np.uint32)[::-1].copy()
        k1, v1 = _dev(keys), _dev(vals)
        k2, v2 = _dev(keys), _dev(vals)
        torch.cuda.synchronize()
        assert _noalloc(k1, v1, *bits, stream=stream) == OK
        ref.compute(k2, v2, *bits, stream=stream)
        torch.cuda.synchronize()
        want_k, want_v = _expected(keys, vals, *bits)
        assert np.array_equal(_host(k1), want_k), f"keys differ from the stable sort on call {call}"
        assert np.array_equal(_host(v1), want_v), f"values differ from the stable sort on call {call}"
        assert np.array_equal(_host(k1), _host(k2)), f"keys differ from the allocating sort on call {call}"
        assert np.array_equal(_host(v1), _host(v2)), f"values differ from the allocating sort on call {call}"
    assert _status(stream) == OK


def test_noalloc_rejects_sizes_beyond_its_limit(cuda):
    k = _dev(np.zeros(NOALLOC_MAX + 1, np.uint32))
    v = _dev(np.zeros(NOALLOC_MAX + 1, np.uint32))
    assert _noalloc(k, v, 0, 32) == ERR_TOO_LARGE


def test_noalloc_status_reports_a_device_timeout_once(cuda):
    """A look-back wait inside the static array runs out (about one second); the status call
    reports it, clears it, and the next sort is correct."""
    import torch
    lib = load_library()
    assert _status() == OK
    assert lib.gbsph_selftest_bounded_wait(2, None) == OK
    t0 = time.perf_counter()
    rc = _status()
    dt = time.perf_counter() - t0
    assert rc == ERR_DEVICE_TIMEOUT, rc
    assert 0.5 < dt < 30.0, dt
    assert _status() == OK
    rng = SplitMix64(99)
    keys = (rng.next_u64(100_000) >> np.uint64(32)).astype(np.uint32)
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v = _dev(keys), _dev(vals)
    assert _noalloc(k, v, 0, 32) == OK
    torch.cuda.synchronize()
    want_k, want_v = _expected(keys, vals, 0, 32)
    assert np.array_equal(_host(k), want_k) and np.array_equal(_host(v), want_v)
    assert _status() == OK


def test_noalloc_argument_checks_run_on_the_host():
    """Checks that happen before any device work."""
    import libcl_gb300 as gb
    lib = gb.load_library()
    assert lib.gbsph_radix_sort_noalloc(None, None, 10, 9, 0, 32, None) == gb.ERR_SIZE_MISMATCH
    assert lib.gbsph_radix_sort_noalloc(None, None, 262145, 262145, 0, 32, None) == gb.ERR_TOO_LARGE
    assert lib.gbsph_radix_sort_noalloc(None, None, 10, 10, 0, 30, None) == gb.ERR_BIT_RANGE
    assert lib.gbsph_radix_sort_noalloc(None, None, 0, 0, 0, 32, None) == gb.OK
    assert lib.gbsph_radix_sort_noalloc(None, None, 10, 10, 0, 32, None) == gb.ERR_ARGUMENT
