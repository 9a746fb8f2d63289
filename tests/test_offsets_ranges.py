"""The index logic of the offsets kernel (offsets_from_sorted and offsets_range
in pic-deposition_gb300/csrc/sort.cu), restated in Python and checked on the CPU.

A thread takes four consecutive cell-ordered keys k[0..3] at index i0 and the
key before them. Range j < 4 gives the cells (key before k[j], k[j]] the value
i0 + j; range 4, on the thread holding the last particle, gives the cells after
the last key the value n. Short ranges are written by their thread, long ones by
the whole warp; which thread writes a range does not change what is written, so
the claim checked here is that the ranges of all threads cover cells 0 .. G
exactly once and give offsets[c] = the first index whose key is >= c (a
histogram and an exclusive scan)."""
import numpy as np
import pytest


def offsets_range(j, k, before, i0, cnt, n, G):
    """(from, end, val) or None, as offsets_range on the device."""
    if j < 4:
        if j >= cnt:
            return None
        prev = before if j == 0 else k[j - 1]
        lo = 0 if (j == 0 and i0 == 0) else (G if prev >= G else prev + 1)
        hi = k[j] + 1 if k[j] < G else G
        return lo, hi, i0 + j
    if cnt == 0 or i0 + cnt != n or k[cnt - 1] >= G:
        return None
    return k[cnt - 1] + 1, G + 1, n


def offsets_by_ranges(keys, G):
    n = len(keys)
    out = np.full(G + 1, -1, np.int64)
    hits = np.zeros(G + 1, np.int64)
    padded = np.concatenate([keys, np.zeros(3, np.int64)])  # the arrays' padding past n
    for i0 in range(0, n, 4):
        k = [int(v) for v in padded[i0:i0 + 4]]
        before = int(keys[i0 - 1]) if i0 > 0 else 0
        cnt = min(4, n - i0)
        for j in range(5):
            r = offsets_range(j, k, before, i0, cnt, n, G)
            if r is None:
                continue
            lo, hi, val = r
            if hi > lo:
                out[lo:hi] = val
                hits[lo:hi] += 1
    return out, hits


def expected(keys, G):
    return np.searchsorted(keys, np.arange(G + 1), side="left")


def check(keys, G):
    keys = np.sort(np.asarray(keys, np.int64))
    got, hits = offsets_by_ranges(keys, G)
    if len(keys) == 0:
        return  # the library sets the offsets of an empty set to zero without this kernel
    assert np.all(hits == 1), np.nonzero(hits != 1)[0][:10]
    assert np.array_equal(got, expected(keys, G))


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 8, 9, 31, 32, 33, 127, 1000])
def test_dense_and_ragged_counts(n):
    rng = np.random.default_rng(n)
    for G in (1, 2, 7, 64, 1000):
        check(rng.integers(0, G, n), G)


def test_all_particles_in_one_cell_and_at_the_ends():
    for G in (1, 5, 4096):
        for c in {0, G // 2, G - 1}:
            check(np.full(37, c), G)
    check([0, 0, 0, 4095, 4095], 4096)
    check([4095], 4096)
    check([0], 4096)


def test_sparse_and_lopsided():
    rng = np.random.default_rng(11)
    G = 1 << 16
    check(rng.integers(0, G, 50), G)                       # mostly long runs of empty cells
    check(rng.integers(G // 2, G // 2 + 100, 5000), G)     # one cluster, long gaps on both sides
    check(np.concatenate([rng.integers(0, 10, 300), rng.integers(G - 10, G, 300)]), G)


def test_every_gap_length_around_the_warp_threshold():
    for gap in range(0, 40):
        keys = [3, 3, 3, 3 + gap, 3 + gap, 3 + 2 * gap + 1]
        check(keys, 3 + 2 * gap + 40)
