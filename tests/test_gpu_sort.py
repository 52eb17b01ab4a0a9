"""The broad phase's own stable radix sort and exclusive prefix sum (woodem_gb300/csrc/wg_sort.cuh),
through their self-test entry points, against numpy: the sort must equal a stable sort by the
key bits (equal keys keep their input order, so the values carried along come out in that
order), the scan numpy's exclusive cumulative sum. Sizes around the tile boundaries (4096 keys,
4096 scan values) and past one level of scan totals."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort(lib, keys, bits, vals=None, begin=0):
    out = np.empty_like(keys)
    vout = np.empty_like(vals) if vals is not None else None
    r = lib.wg_test_sort(len(keys), keys.dtype.itemsize, begin, bits, keys.ctypes.data,
                         vals.ctypes.data if vals is not None else None, out.ctypes.data,
                         vout.ctypes.data if vout is not None else None)
    assert r == 0, r
    return out, vout


@pytest.mark.parametrize("n", [1, 100, 4096, 4097, 300_001])
@pytest.mark.parametrize("bits", [1, 8, 13, 21, 32])
def test_sort_u32_pairs(gpu_lib, n, bits):
    rng = np.random.default_rng(n * 131 + bits)
    keys = rng.integers(0, 2 ** bits, n, dtype=np.uint64).astype(np.uint32)
    vals = np.arange(n, dtype=np.int32)
    out, vout = _sort(gpu_lib, keys, bits, vals)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(out, keys[order]) and np.array_equal(vout, vals[order])


@pytest.mark.parametrize("n", [5, 4097, 1_000_003])
@pytest.mark.parametrize("bits", [40, 53, 64])
def test_sort_u64_keys(gpu_lib, n, bits):
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 2 ** 63, n, dtype=np.uint64) * np.uint64(2) + rng.integers(0, 2, n, dtype=np.uint64)
    if bits < 64:
        keys &= np.uint64((1 << bits) - 1)
    out, _ = _sort(gpu_lib, keys, bits)
    assert np.array_equal(out, np.sort(keys))


def test_sort_u64_pairs_duplicates_and_partial_bits(gpu_lib):
    """Many equal keys (the values show the order is stable), and a bit range that leaves the high
    bits out (keys equal in the range keep their order whatever their high bits)."""
    rng = np.random.default_rng(7)
    n = 250_000
    keys = rng.integers(0, 50, n, dtype=np.uint64) | (rng.integers(0, 2 ** 20, n, dtype=np.uint64) << np.uint64(40))
    vals = rng.integers(-2 ** 31, 2 ** 31 - 1, n, dtype=np.int64).astype(np.int32)
    out, vout = _sort(gpu_lib, keys.copy(), 40, vals)
    order = np.argsort(keys & np.uint64((1 << 40) - 1), kind="stable")
    assert np.array_equal(out, keys[order]) and np.array_equal(vout, vals[order])


@pytest.mark.parametrize("n", [1, 5, 4096, 4097, 1_000_003, 5_000_000])
def test_exclusive_scan(gpu_lib, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 5, n, dtype=np.int32)
    out = np.empty_like(x)
    assert gpu_lib.wg_test_scan(n, x.ctypes.data, out.ctypes.data) == 0
    ref = np.concatenate([[0], np.cumsum(x)[:-1]]).astype(np.int32)
    assert np.array_equal(out, ref)
