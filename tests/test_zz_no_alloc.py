"""cmag_sort_particles_noalloc: the stable (hash, index) sort for callers that
cannot allocate device memory where they sort (a latency-critical loop where an
allocation would stall the device, or a host whose device memory all comes from
its own pool).  Its workspace is a fixed array inside the library.  The test
calls it through the C ABI twice in a row (the shared scratch keeps the first
call's contents) and checks each result against the allocating entry point, bit
for bit, as the sort is integer work.
This file sorts last on purpose: run alone or after every other test, it must
pass either way."""
import ctypes

import numpy as np
import pytest

from cmag_gb300._lib import c_u32p, lib

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20


def _device_pair(keys, vals):
    import torch
    k = torch.from_numpy(keys.astype(np.int64)).to(torch.int32).cuda()
    v = torch.from_numpy(vals.astype(np.int64)).to(torch.int32).cuda()
    return k, v


def _sort(fn, keys, vals, bits):
    import torch
    k, v = _device_pair(keys, vals)
    torch.cuda.synchronize()
    rc = fn(ctypes.cast(k.data_ptr(), c_u32p), ctypes.cast(v.data_ptr(), c_u32p), keys.size, bits,
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_twice(gpu):
    import torch
    torch.cuda.init()
    L = lib()
    rng = np.random.default_rng(2024)
    # two calls in a row with different sizes and key widths: the second runs on
    # scratch the first one left behind
    for n, bits in ((MAX_PAIRS, 23), (300_001, 15)):
        keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        rc0, k0, v0 = _sort(L.cmag_sort_particles, keys, vals, bits)
        rc1, k1, v1 = _sort(L.cmag_sort_particles_noalloc, keys, vals, bits)
        assert rc0 == 0 and rc1 == 0, L.cmag_sort_particles_noalloc_error()
        assert np.array_equal(k1, k0)
        assert np.array_equal(v1, v0)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(k1, keys[order]) and np.array_equal(v1, vals[order])


def test_noalloc_sort_rejects_more_than_its_maximum(gpu):
    L = lib()
    rc = L.cmag_sort_particles_noalloc(ctypes.cast(1, c_u32p), ctypes.cast(1, c_u32p), MAX_PAIRS + 1,
                                       24, None)
    assert rc != 0
    assert b"at most 1048576" in L.cmag_sort_particles_noalloc_error()
