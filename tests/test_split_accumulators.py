"""The tiled deposit's split shared-memory accumulators (deposit_tiled in
pic-deposition_gb300/csrc/deposit.cu), checked on the CPU.

A run total v (at most 8 particles of one lane: |v| <= 8 * (2^24 + 3) < 2^27) is
added to a node as two native 32-bit atomics: v & (2^15 - 1) to an unsigned low
word (wrapping mod 2^32) and v >> 15 (arithmetic shift) to a signed high word;
the node's total is hi * 2^15 + lo. A node receives at most one addition per run
and a run holds at least one particle, so a tile of fewer than 2^17 particles
adds at most 2^17 - 1 values per node. The claim: both words stay exact."""
import numpy as np

SPLIT = 15
MAX_ADDS = (1 << 17) - 1
VMAX = 8 * ((1 << 24) + 3)


def split_sum(v: np.ndarray):
    v = v.astype(np.int64)
    lo = np.sum((v & ((1 << SPLIT) - 1)).astype(np.uint32), dtype=np.uint32)  # wraps like the 32-bit atomic
    hi = np.sum(v >> SPLIT, dtype=np.int64)
    assert -(1 << 31) <= hi < (1 << 31)  # the signed 32-bit high word does not overflow
    return int(hi) * (1 << SPLIT) + int(lo)


def test_worst_cases_at_the_tile_limit():
    rng = np.random.default_rng(6)
    all_low = VMAX - (VMAX % (1 << SPLIT)) - 1  # largest |v| with all 15 low bits set
    cases = [
        np.full(MAX_ADDS, VMAX), np.full(MAX_ADDS, -VMAX), np.full(MAX_ADDS, all_low), np.full(MAX_ADDS, -all_low),
        np.full(MAX_ADDS, (1 << SPLIT) - 1), np.full(MAX_ADDS, -1),
        rng.integers(-VMAX, VMAX + 1, MAX_ADDS), rng.integers(0, VMAX + 1, MAX_ADDS),
    ]
    for v in cases:
        assert split_sum(v) == int(np.sum(v.astype(np.int64)))


def test_the_limit_is_set_by_the_low_word():
    # 2^17 additions of the largest low part still fit the unsigned low word, 2^18 do not;
    # the high word has room to spare (2^17 additions of at most 2^12 each)
    low = (1 << SPLIT) - 1
    assert (1 << 17) * low < (1 << 32) <= (1 << 18) * low
    assert (1 << 17) * ((VMAX >> SPLIT) + 1) < (1 << 31)
