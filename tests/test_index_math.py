"""The division-free cell-key split of the push and the any-order deposits
(split_key in pic-deposition_gb300/csrc/pic_internal.cuh), checked on the CPU.

For key < 2^24 the kernel takes q = (int)(float(key) * (1.0f / n)) with
round-to-nearest FP32 arithmetic (compiled without contraction), then one
correction step: r = key - q*n; r < 0 -> q-1; r >= n -> q+1. numpy's float32
operations round the same way, so this emulation is exact. The claim: the
estimate is within one of floor(key / n), hence the split equals integer
division for every n and every key < 2^24."""
import numpy as np


def split_fp32(keys: np.ndarray, n: int):
    inv = np.float32(1.0) / np.float32(n)
    q = (keys.astype(np.float32) * inv).astype(np.int64)  # truncation, as (int) on the device
    r = keys.astype(np.int64) - q * n
    assert np.all(np.abs(q - keys // n) <= 1), n  # the estimate is within one
    lo, hi = r < 0, r >= n
    q = q - lo + hi
    r = r + lo * n - hi * n
    return q, r


def check(keys, n):
    keys = keys[keys < (1 << 24)].astype(np.int64)
    q, r = split_fp32(keys, n)
    assert np.array_equal(q, keys // n) and np.array_equal(r, keys % n), n


def test_every_key_for_small_rows():
    keys = np.arange(1 << 24, dtype=np.int64)
    for n in (1, 2, 3, 5, 7, 64, 100, 127, 128, 129, 255, 256, 1000, 1023, 1024, 2047, 2048):
        check(keys, n)


def test_row_boundaries_for_many_widths():
    rng = np.random.default_rng(5)
    widths = np.unique(np.concatenate([np.arange(1, 4097), rng.integers(4097, 1 << 24, 3000), [(1 << 24) - 1]]))
    for n in widths:
        n = int(n)
        rows = np.arange(0, (1 << 24) // n + 1, max(1, ((1 << 24) // n) // 512), dtype=np.int64)
        keys = np.concatenate([rows * n - 1, rows * n, rows * n + 1, rows * n + n - 1, rng.integers(0, 1 << 24, 64)])
        check(keys[keys >= 0], n)
