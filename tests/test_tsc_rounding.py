"""The TSC deposit's rounding shortcut (tsc_accumulate in
pic-deposition_gb300/csrc/deposit.cu), checked on the CPU with exact float32
emulation.

The 12 frame entries outside rows and columns 1..2 are rounded to integers by
one FP32 add of M = 1.5 * 2^23: for |v| < 2^22 the bits of fl(M + v), minus the
bits of M, are rint(v) (round half to even). That needs |v| < 2^22, which holds
because those entries carry a weight of column or row 0 or 3, at most 1/8 for
every FP32 offset in [0, 1), and |qn * 2^24| <= 2^24."""
import numpy as np

M = np.float32(12582912.0)  # 1.5 * 2^23
M_BITS = np.uint32(0x4B400000)


def magic_rint(v: np.ndarray) -> np.ndarray:
    s = (M + v.astype(np.float32)).astype(np.float32)
    return (s.view(np.uint32) - M_BITS).view(np.int32).astype(np.int64)


def test_magic_add_is_round_half_even_below_2_22():
    rng = np.random.default_rng(8)
    k = np.concatenate([rng.integers(-(1 << 22) + 1, 1 << 22, 200_000), np.arange(-2048, 2048),
                        [-(1 << 22) + 1, (1 << 22) - 1]]).astype(np.float64)
    # integers, ties (k + 1/2, which round to even), and fractions near the ties
    frac = np.concatenate([np.zeros(1), [0.5, -0.5, 0.25, 0.75, -0.25], rng.random(4)])
    v = (k[:, None] + frac[None, :]).ravel()
    v = v[np.abs(v) < (1 << 22)].astype(np.float32)
    assert np.array_equal(magic_rint(v), np.rint(v.astype(np.float64)).astype(np.int64))


def tsc_axis(r: np.ndarray):
    """The kernel's branch-free weights of one axis (FP32), columns 0..3."""
    r = r.astype(np.float32)
    s = r >= np.float32(0.5)
    t = np.where(s, (r - np.float32(1.0)).astype(np.float32), r)
    half = np.float32(0.5)
    dl, dr = (half - t).astype(np.float32), (half + t).astype(np.float32)
    L = (half * (dl * dl).astype(np.float32)).astype(np.float32)
    C = (np.float32(0.75) - (t * t).astype(np.float32)).astype(np.float32)
    R = (half * (dr * dr).astype(np.float32)).astype(np.float32)
    z = np.zeros_like(r)
    return (np.where(s, z, L), np.where(s, L, C), np.where(s, C, R), np.where(s, R, z))


def test_outer_columns_weigh_at_most_one_eighth():
    rng = np.random.default_rng(9)
    edges = np.array([0.0, 0.5, 1.0 - 2.0 ** -24, 0.25, 0.75], np.float32)
    near = np.concatenate([np.nextafter(edges, np.float32(1.0)), np.nextafter(edges, np.float32(0.0))])
    r = np.concatenate([edges, near, rng.random(2_000_000).astype(np.float32)])
    r = r[(r >= 0) & (r < 1)].astype(np.float32)
    x0, x1, x2, x3 = tsc_axis(r)
    assert np.all(x0 <= 0.125) and np.all(x3 <= 0.125)
    # with |qn * 2^24| <= 2^24 and every weight <= 0.75, the outer entries stay below 2^22
    aq = np.float32(16777216.0)
    for outer in (x0, x3):
        for other in (x0, x1, x2, x3):  # (aq * Y_j) * X_i with the outer weight on either axis
            for a, b in ((other, outer), (outer, other)):
                v = ((aq * a).astype(np.float32) * b).astype(np.float32)
                assert np.all(np.abs(v) < 2.0 ** 22)
