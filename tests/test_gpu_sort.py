"""Cell-sort parity through the C ABI.

Keys are bit-exact with the reference's particleCellIndex
(src/sorting/cell_sort.cpp:8-13); the permutation is bit-exact with a stable
sort on the same keys (the oracle's counting sort); per-cell offsets are
bit-exact with histogram + exclusive scan; and every cell holds the same
particles as after the reference's own std::sort (tests/golden/small_32.npz).
"""
import os

import numpy as np
import pytest

import workloads
from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def gpu_sort(pg, nx, ny, lx, ly, p):
    n = len(p["x"])
    with pg.Context(nx, ny, lx, ly, max(n, 1)) as c:
        c.upload(p["x"], p["y"], p["q"], p.get("vx"), p.get("vy"), p.get("m"))
        before = c.device_layout()
        keys, perm, offs = c.sort(keys=True, perm=True, offsets=True)
        after = c.device_layout()
    return before, keys, perm, offs, after


def check_sort(port, pg, nx, ny, lx, ly, p):
    before, keys, perm, offs, after = gpu_sort(pg, nx, ny, lx, ly, p)
    cell, xr, yr = port.to_device(nx, ny, lx, ly, p["x"], p["y"])
    assert np.array_equal(before["cell"], cell) and np.array_equal(before["xr"], xr)
    assert np.array_equal(before["yr"], yr)
    wk, wp, wo = port.stable_sort_keys(cell, nx * ny)
    assert np.array_equal(keys, wk)
    assert np.array_equal(perm, wp)
    assert np.array_equal(offs, wo)
    for k in ("cell", "xr", "yr", "vx", "vy", "q"):
        assert np.array_equal(after[k], before[k][perm]), k
    return perm


def test_sort_matches_reference_cells(port, pg):
    g = dict(np.load(os.path.join(GOLDEN, "small_32.npz")))
    p = {k: g[k] for k in ("x", "y", "vx", "vy", "q", "m")}
    perm = check_sort(port, pg, 32, 32, 1.0, 1.0, p)
    keys = g["keys"].astype(np.uint32)
    assert np.array_equal(keys[perm], np.sort(keys))
    # same particles per cell as the reference's sortParticlesByCell
    offs = np.concatenate([[0], np.cumsum(np.bincount(keys, minlength=1024))])
    for c in range(1024):
        a = np.sort(g["x"][perm[offs[c]:offs[c + 1]]])
        b = np.sort(g["sorted_x"][offs[c]:offs[c + 1]])
        assert np.array_equal(a, b)


@pytest.mark.parametrize("grid,n", [((1, 1, 1.0, 1.0), 1000), ((3, 5, 3.0, 5.0), 777), ((256, 256, 1.0, 1.0), 300000),
                                    ((2048, 2048, 2048.0, 2048.0), 2_000_000), ((1000, 7, 1.0, 1.0), 123457),
                                    ((16, 16, 1.0, 1.0), 0), ((16, 16, 1.0, 1.0), 1)])
def test_sort_shapes(port, pg, grid, n):
    nx, ny, lx, ly = grid
    p = port.init_particles(0, nx, ny, lx, ly, n, p0=1.0, seed=31)
    check_sort(port, pg, nx, ny, lx, ly, p)


def test_sort_presorted_reversed_and_one_cell(port, pg):
    p = port.init_particles(0, 64, 64, 1.0, 1.0, 50000, p0=1.0, seed=4)
    keys = np.array([port.cell_index(64, 64, 1.0, 1.0, x, y) for x, y in zip(p["x"], p["y"])])
    for order in (np.argsort(keys, kind="stable"), np.argsort(keys, kind="stable")[::-1]):
        q = {k: v[order].copy() for k, v in p.items()}
        check_sort(port, pg, 64, 64, 1.0, 1.0, q)
    q = dict(p)
    q["x"] = 0.3 / 64 + np.zeros(50000)
    q["y"] = 0.7 / 64 + np.zeros(50000)
    check_sort(port, pg, 64, 64, 1.0, 1.0, q)


def test_sort_twice_is_identity(pg):
    p = workloads.uniform_box(100, 100, 9, seed=2)
    with pg.Context(100, 100, 100.0, 100.0, len(p["x"])) as c:
        c.upload(p["x"], p["y"], p["q"])
        c.sort()
        _, perm, _ = c.sort(perm=True)
    assert np.array_equal(perm, np.arange(len(perm), dtype=np.uint32))


@pytest.mark.slow
def test_sort_config2_full_size(port, pg):
    p = workloads.density_cos(1024, 1024, 64, 0.01, 0.1, seed=42)
    check_sort(port, pg, 1024, 1024, 1024.0, 1024.0, p)


def test_in_order_upload_sparse_offsets(port, pg):
    """An upload already in cell order gets its offsets without a sort; long runs
    of empty cells are filled by whole warps. Particles in three clusters of a
    512 x 512 grid (the first cell, mid-grid, the last cell) deposit as the
    oracle does, and a later sort keeps the order (identity permutation) and
    gives the offsets of a stable counting sort."""
    nx = ny = 512
    rng = np.random.default_rng(8)
    xs, ys = [], []
    for cx, cy in ((0.2, 0.3), (200.5, 311.5), (511.6, 511.4)):
        xs.append(np.clip(cx + rng.normal(0.0, 0.8, 3000), 0.0, 511.999))
        ys.append(np.clip(cy + rng.normal(0.0, 0.8, 3000), 0.0, 511.999))
    x, y = np.concatenate(xs), np.concatenate(ys)
    order = np.argsort(np.floor(y).astype(np.int64) * nx + np.floor(x).astype(np.int64), kind="stable")
    p = {"x": x[order], "y": y[order], "q": np.full(len(x), -1.0)}
    with pg.Context(nx, ny, 512.0, 512.0, len(x)) as c:
        c.upload(p["x"], p["y"], p["q"])
        assert c.is_sorted()
        c.deposit(1, 0.0)
        acc, unit = c.rho_fixed()
        lay = c.device_layout()
        _, perm, offs = c.sort(keys=True, perm=True, offsets=True)
    _, maxq = port.normalize_charge(p["q"])
    want, wunit = port.deposit_fixed(nx, ny, 512.0, 512.0, 1, lay["cell"], lay["xr"], lay["yr"], lay["q"], maxq,
                                     lay["vx"], lay["vy"], 0.0)
    assert unit == wunit and np.array_equal(acc, want)
    assert np.array_equal(perm, np.arange(len(x), dtype=np.uint32))
    _, _, wo = port.stable_sort_keys(lay["cell"], nx * ny)
    assert np.array_equal(offs, wo)
