"""GPU parity of the one-sweep radix sort and cell-bounds extraction (through the C ABI).

Bit-exact against numpy's stable argsort (the definition of a stable LSD sort on a bit
field) and against the oracle's restatement of clFindBounds."""
import numpy as np
import pytest

import oracle
from libcl_gb300 import (ERR_BIT_RANGE, ERR_SIZE_MISMATCH, OK, RadixSort)
from libcl_gb300.scenes import SplitMix64

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def _host(t):
    return t.cpu().numpy().view(np.uint32)


def _expected(keys, vals, s, e):
    field = (keys.astype(np.uint64) >> np.uint64(s)) & np.uint64((1 << (e - s)) - 1)
    o = np.argsort(field, kind="stable")
    return keys[o], vals[o]


def _keys(n, seed, dist="uniform"):
    rng = SplitMix64(seed)
    if dist == "uniform":
        return (rng.next_u64(n) >> np.uint64(32)).astype(np.uint32)
    if dist == "equal":
        return np.full(n, 0xA5A5A5A5, dtype=np.uint32)
    if dist == "few":
        return (rng.next_u64(n) % np.uint64(5)).astype(np.uint32) * np.uint32(0x01010101)
    if dist == "sorted":
        return np.sort((rng.next_u64(n) >> np.uint64(32)).astype(np.uint32))
    if dist == "reversed":
        return np.sort((rng.next_u64(n) >> np.uint64(32)).astype(np.uint32))[::-1].copy()
    raise ValueError(dist)


def _run(sorter, keys, vals, s, e):
    import torch
    dk, dv = _dev(keys), _dev(vals)
    sorter.compute(dk, dv, s, e)
    torch.cuda.synchronize()
    assert sorter.sync_status() == OK
    return _host(dk), _host(dv)


@pytest.mark.parametrize("n", [1, 2, 255, 256, 4095, 4096, 4097, 65537, 1_000_003])
@pytest.mark.parametrize("bits", [(0, 32), (0, 24), (4, 16), (8, 12), (0, 4), (28, 32)])
def test_sort_uniform(cuda, n, bits):
    sorter = RadixSort()
    keys = _keys(n, 100 + n)
    vals = np.arange(n, dtype=np.uint32)
    k, v = _run(sorter, keys, vals, *bits)
    ek, ev = _expected(keys, vals, *bits)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


@pytest.mark.parametrize("dist", ["equal", "few", "sorted", "reversed"])
@pytest.mark.parametrize("n", [4097, 300_000])
def test_sort_distributions(cuda, dist, n):
    sorter = RadixSort()
    keys = _keys(n, 7, dist)
    vals = (np.arange(n, dtype=np.uint32) * np.uint32(2654435761))  # arbitrary payload
    k, v = _run(sorter, keys, vals, 0, 32)
    ek, ev = _expected(keys, vals, 0, 32)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


def test_reference_smoke_sort(cuda):
    """libCL/TEST/main.cpp:133-181: 1024 random keys, values 0..1023, bits 0..32; the reference
    only checks that keys do not decrease. Here the permutation is checked too."""
    sorter = RadixSort()
    keys = _keys(1024, 1) >> np.uint32(1)  # rand() range
    vals = np.arange(1024, dtype=np.uint32)
    k, v = _run(sorter, keys, vals, 0, 32)
    assert np.all(k[1:] >= k[:-1])
    assert np.array_equal(keys[v], k)
    # the restated reference sort agrees
    rk, rv = keys.copy(), vals.copy()
    assert oracle.radix_sort_reference(rk, rv, 0, 32) == 0
    assert np.array_equal(rk, k) and np.array_equal(rv, v)


def test_sort_repeated_calls_reuse_buffers(cuda):
    sorter = RadixSort()
    for n in (100_000, 5000, 250_000):
        keys = _keys(n, n)
        vals = np.arange(n, dtype=np.uint32)
        k, v = _run(sorter, keys, vals, 0, 32)
        ek, ev = _expected(keys, vals, 0, 32)
        assert np.array_equal(v, ev)


def test_sort_errors(cuda):
    sorter = RadixSort()
    k, v = _dev(np.zeros(10, np.uint32)), _dev(np.zeros(9, np.uint32))
    assert sorter.compute_raw(k, v, 0, 32) == ERR_SIZE_MISMATCH
    v = _dev(np.zeros(10, np.uint32))
    assert sorter.compute_raw(k, v, 0, 30) == ERR_BIT_RANGE      # not a multiple of 4
    assert sorter.compute_raw(k, v, 8, 4) == ERR_BIT_RANGE
    assert sorter.compute_raw(k, v, 0, 36) == ERR_BIT_RANGE
    assert sorter.compute_raw(k, v, 12, 12) == OK                 # empty range: no-op
    assert "divisible by 4" in sorter.last_error()


def morton3(x, y, z):
    def spread(v):
        v = v.astype(np.uint64) & np.uint64(0x3FF)
        v = (v | (v << np.uint64(16))) & np.uint64(0x030000FF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x0300F00F)
        v = (v | (v << np.uint64(4))) & np.uint64(0x030C30C3)
        v = (v | (v << np.uint64(2))) & np.uint64(0x09249249)
        return v
    return (spread(x) | (spread(y) << np.uint64(1)) | (spread(z) << np.uint64(2))).astype(np.uint32)


def morton_lattice_keys(n_target, seed):
    """Morton keys of a jittered lattice with 0-20 particles per occupied cell in a
    128x128x256 (2^22) cell table."""
    rng = SplitMix64(seed)
    counts = (rng.next_u64(1 << 22) % np.uint64(21)).astype(np.int64)
    cells = np.nonzero(np.cumsum(counts) <= n_target)[0]
    cnt = counts[cells]
    cid = np.repeat(cells, cnt)
    x, y, z = cid % 128, (cid // 128) % 128, cid // (128 * 128)
    keys = morton3(x, y, z)
    # shuffle so the input is not already in cell order
    perm = np.argsort(rng.next_u64(keys.size), kind="stable")
    return keys[perm]


def test_cell_bounds_morton(cuda):
    import torch
    keys = morton_lattice_keys(600_000, 4)
    n = keys.size
    sorter = RadixSort()
    vals = np.arange(n, dtype=np.uint32)
    k, v = _run(sorter, keys, vals, 0, 24)
    ek, ev = _expected(keys, vals, 0, 24)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)
    cs = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    ce = torch.empty(1 << 22, dtype=torch.int32, device="cuda")
    sorter.cell_bounds(_dev(k), cs, ce)
    torch.cuda.synchronize()
    ocs, oce = oracle.find_bounds(k, 1 << 22)
    assert np.array_equal(_host(cs), ocs) and np.array_equal(_host(ce), oce)


def test_cell_bounds_key_out_of_range(cuda):
    import torch
    from libcl_gb300 import ERR_DEVICE_RANGE
    sorter = RadixSort()
    k = _dev(np.array([0, 1, 1, 70], np.uint32))
    cs = torch.empty(64, dtype=torch.int32, device="cuda")
    ce = torch.empty(64, dtype=torch.int32, device="cuda")
    sorter.cell_bounds(k, cs, ce)
    assert sorter.sync_status() == ERR_DEVICE_RANGE
    assert sorter.sync_status() == OK  # cleared


@pytest.mark.parametrize("dist", ["uniform32", "morton"])
def test_sort_16m_pairs(cuda, dist):
    """The 16,777,216-pair configuration (above the reference's 4,194,304 cap)."""
    n = 1 << 24
    if dist == "uniform32":
        keys, bits = _keys(n, 3), (0, 32)
    else:
        keys, bits = morton_lattice_keys(n, 4), (0, 24)
    vals = np.arange(keys.size, dtype=np.uint32)
    k, v = _run(RadixSort(), keys, vals, *bits)
    ek, ev = _expected(keys, vals, *bits)
    assert np.array_equal(k, ek) and np.array_equal(v, ev)


MAX_KEYS = (1 << 30) - 1 - 4096  # the largest sortable count (the C ABI refuses one more)


def test_sort_maximum_size(cuda):
    """The largest accepted sort: 1,073,737,727 random 32-bit pairs, checked on the device
    in 64M-key slices: keys ascending, each output value the input position of its key
    (orig[val] == key), equal keys in input order (stability), and the values a
    permutation. One more key is refused with GBSPH_ERR_TOO_LARGE before any device work."""
    import torch
    from libcl_gb300 import ERR_TOO_LARGE
    n = MAX_KEYS
    g = torch.Generator(device="cuda").manual_seed(7)
    keys = torch.randint(-(1 << 31), 1 << 31, (n,), dtype=torch.int32, device="cuda", generator=g)
    orig = keys.clone()
    vals = torch.arange(n, dtype=torch.int32, device="cuda")
    sorter = RadixSort()
    sorter.compute(keys, vals, 0, 32)
    torch.cuda.synchronize()
    assert sorter.sync_status() == OK
    step = 1 << 26
    mask = 0xFFFFFFFF
    for a in range(0, n, step):
        b = min(n, a + step + 1)  # one key of overlap with the next slice
        k = keys[a:b].to(torch.int64) & mask
        v = vals[a:b].to(torch.int64)
        assert bool((k[1:] >= k[:-1]).all()), f"not sorted in [{a}, {b})"
        eq = k[1:] == k[:-1]
        assert bool((v[1:][eq] > v[:-1][eq]).all()), f"not stable in [{a}, {b})"
        assert bool((orig[vals[a:b].long()] == keys[a:b]).all()), f"value does not index its key in [{a}, {b})"
        del k, v, eq
    vs, _ = torch.sort(vals)
    for a in range(0, n, step):
        b = min(n, a + step)
        assert bool((vs[a:b] == torch.arange(a, b, dtype=torch.int32, device="cuda")).all())
    del vs, keys, orig, vals
    torch.cuda.empty_cache()
    lib = sorter._lib
    assert lib.gbsph_radix_sort_compute(sorter._h, None, None, n + 1, n + 1, 0, 32, None) == ERR_TOO_LARGE
