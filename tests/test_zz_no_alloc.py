"""The allocation-free sort entry point, gbsph_radix_sort_noalloc, called through the C ABI.

It exists for callers that cannot allocate device memory (a host framework that owns all
device memory, real-time loops that must not stall on cudaMalloc/cudaFree, plugins with a
fixed footprint); its scratch is a static device array shared by every call. Each check
compares it with the allocating entry point, gbsph_radix_sort_compute, on the same input.
The sort is integer work, so the comparison is exact. Two calls run back to back so that
whatever the first call leaves in the shared scratch array cannot change the second result.
This file is named to be collected last."""
import ctypes

import numpy as np
import pytest

from libcl_gb300 import ERR_TOO_LARGE, OK, RadixSort, load_library
from libcl_gb300.scenes import SplitMix64

pytestmark = pytest.mark.gpu

NOALLOC_MAX = 262144


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def _noalloc(keys, vals, start, end):
    import torch
    lib = load_library()
    stream = torch.cuda.current_stream().cuda_stream
    return lib.gbsph_radix_sort_noalloc(ctypes.c_void_p(keys.data_ptr()), ctypes.c_void_p(vals.data_ptr()),
                                        keys.numel(), vals.numel(), start, end, ctypes.c_void_p(stream))


@pytest.mark.parametrize("sizes,bits", [((200_000, 4097), (0, 32)), ((NOALLOC_MAX, 1000), (0, 24)),
                                        ((70_000, 70_000), (0, 8))])
def test_noalloc_matches_allocating_sort(cuda, sizes, bits):
    import torch
    ref = RadixSort()
    for call, n in enumerate(sizes):
        rng = SplitMix64(1000 + call)
        keys = (rng.next_u64(n) >> np.uint64(32)).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)[::-1].copy()
        k1, v1 = _dev(keys), _dev(vals)
        k2, v2 = _dev(keys), _dev(vals)
        assert _noalloc(k1, v1, *bits) == OK
        ref.compute(k2, v2, *bits)
        torch.cuda.synchronize()
        assert np.array_equal(_host(k1), _host(k2)), f"keys differ on call {call}"
        assert np.array_equal(_host(v1), _host(v2)), f"values differ on call {call}"


def test_noalloc_rejects_sizes_beyond_its_limit(cuda):
    k = _dev(np.zeros(NOALLOC_MAX + 1, np.uint32))
    v = _dev(np.zeros(NOALLOC_MAX + 1, np.uint32))
    assert _noalloc(k, v, 0, 32) == ERR_TOO_LARGE


def test_noalloc_argument_checks_run_on_the_host():
    """Checks that happen before any device work."""
    import libcl_gb300 as gb
    lib = gb.load_library()
    assert lib.gbsph_radix_sort_noalloc(None, None, 10, 9, 0, 32, None) == gb.ERR_SIZE_MISMATCH
    assert lib.gbsph_radix_sort_noalloc(None, None, 262145, 262145, 0, 32, None) == gb.ERR_TOO_LARGE
    assert lib.gbsph_radix_sort_noalloc(None, None, 10, 10, 0, 30, None) == gb.ERR_BIT_RANGE
    assert lib.gbsph_radix_sort_noalloc(None, None, 0, 0, 0, 32, None) == gb.OK
    assert lib.gbsph_radix_sort_noalloc(None, None, 10, 10, 0, 32, None) == gb.ERR_ARGUMENT
