"""cmag_sort_particles (sortParticles replacement): stable key/value sort equal to
a stable host sort, for edge sizes and key distributions."""
import numpy as np
import pytest

import cmag_gb300 as cm

pytestmark = pytest.mark.gpu

TILE = 4096


def _run(keys, vals, bits):
    import torch
    k = torch.from_numpy(keys.astype(np.int64)).to(torch.int32).cuda()
    v = torch.from_numpy(vals.astype(np.int64)).to(torch.int32).cuda()
    torch.cuda.synchronize()
    cm.sort_particles(k.data_ptr(), v.data_ptr(), keys.size, bits)
    return (k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32))


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, TILE - 1, TILE, TILE + 1, 3 * TILE + 17,
                               100_000, 1 << 20, 3_000_001])
@pytest.mark.parametrize("bits", [8, 15, 24, 31])
def test_sort_matches_stable_host_sort(gpu, n, bits):
    rng = np.random.default_rng(n * 131 + bits)
    keys = rng.integers(0, 1 << bits, size=n, dtype=np.uint64).astype(np.uint32)
    vals = rng.permutation(n).astype(np.uint32)
    gk, gv = _run(keys, vals, bits)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(gk, keys[order])
    assert np.array_equal(gv, vals[order])


@pytest.mark.parametrize("pattern", ["equal", "sorted", "reverse", "few", "nearly"])
def test_sort_patterns(gpu, pattern):
    n = 777_777
    rng = np.random.default_rng(7)
    if pattern == "equal":
        keys = np.full(n, 12345, np.uint32)
    elif pattern == "sorted":
        keys = np.sort(rng.integers(0, 1 << 24, n)).astype(np.uint32)
    elif pattern == "reverse":
        keys = np.sort(rng.integers(0, 1 << 24, n))[::-1].astype(np.uint32).copy()
    elif pattern == "few":
        keys = rng.choice(np.array([3, 70000, 1 << 23], np.uint32), n)
    else:
        keys = (np.arange(n) // 3).astype(np.uint32)
        sw = rng.integers(0, n - 1, n // 50)
        keys[sw], keys[sw + 1] = keys[sw + 1].copy(), keys[sw].copy()
    vals = np.arange(n, dtype=np.uint32)
    gk, gv = _run(keys, vals, 24)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(gk, keys[order])
    assert np.array_equal(gv, vals[order])
