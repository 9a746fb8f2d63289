"""Deposition parity through the C ABI: GPU vs the CPU oracle.

Bar: the int64 fixed-point grid is bit-identical to the oracle's restatement of
the same arithmetic (pic_oracle.c, orc_deposit_fixed) on the same device
layout; rho is within 1e-5 relative L2 (the stated tolerance) of the reference's
FP64 deposit (pic_oracle.c restates src/deposition/ngp.cpp and is itself pinned
bit-exact to the reference in test_oracle.py).
"""
import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu

NGP, CIC, TSC, ESK = 0, 1, 2, 3
REL_L2_TOL = 1e-5  # rho vs the FP64 reference deposit, per scheme


def gpu_deposit(pg, nx, ny, lx, ly, p, scheme, dt=0.0, order="sorted", tile=None, background=0.0):
    n = len(p["x"])
    with pg.Context(nx, ny, lx, ly, max(n, 1)) as c:
        c.upload(p["x"], p["y"], p["q"], p.get("vx"), p.get("vy"), p.get("m"))
        if order == "sorted":
            c.sort()
        elif order == "atomic":
            c.set_order(pg.ORDER_ATOMIC)
        else:
            c.set_order(pg.ORDER_UNSORTED)
        if tile:
            c.set_tile(*tile)
        rho = c.deposit(scheme, dt, background)
        acc, unit = c.rho_fixed()
        lay = c.device_layout()
    return rho, acc, unit, lay


def rel_l2(port, nx, ny, lx, ly, p, scheme, dt, rho):
    """||rho - ref|| / ||ref||; for nearly neutral grids (||ref|| far below the
    magnitude of the deposited charge) the magnitude ||ref(|q|)|| is the scale."""
    ref = port.deposit_ref(nx, ny, lx, ly, scheme, p, dt=dt)
    pa = dict(p)
    pa["q"] = np.abs(p["q"])
    scale = max(np.linalg.norm(ref), 1e-3 * np.linalg.norm(port.deposit_ref(nx, ny, lx, ly, scheme, pa, dt=dt)))
    return np.linalg.norm(rho - ref) / scale if scale > 0 else 0.0


def check(port, pg, nx, ny, lx, ly, p, scheme, dt=0.0, order="sorted", tile=None, rel_tol=REL_L2_TOL):
    rho, acc, unit, lay = gpu_deposit(pg, nx, ny, lx, ly, p, scheme, dt, order, tile)
    cell, xr, yr = port.to_device(nx, ny, lx, ly, p["x"], p["y"])
    qn, maxq = port.normalize_charge(p["q"])
    if order != "sorted":
        assert np.array_equal(lay["cell"], cell) and np.array_equal(lay["xr"], xr) and np.array_equal(lay["yr"], yr)
        assert np.array_equal(lay["q"], qn)
    want, wunit = port.deposit_fixed(nx, ny, lx, ly, scheme, lay["cell"], lay["xr"], lay["yr"], lay["q"], maxq,
                                     lay["vx"], lay["vy"], dt)
    assert unit == wunit
    assert np.array_equal(acc, want), f"max |diff| {np.max(np.abs(acc - want))}"
    assert np.array_equal(rho, acc.astype(np.float64) * unit)
    # every particle deposits exactly its integer charge
    assert acc.sum() == port.fixed_total(scheme, qn)
    rel = rel_l2(port, nx, ny, lx, ly, p, scheme, dt, rho)
    assert rel <= rel_tol, rel
    return rho, acc


def maxwellian(port, nx, ny, lx, ly, n, seed=123, T=1.0):
    return port.init_particles(0, nx, ny, lx, ly, n, p0=T, seed=seed)


# ---- the reference's own test set-ups (src/main_test.cpp) ----------------
@pytest.mark.parametrize("order", ["sorted", "unsorted"])
@pytest.mark.parametrize("scheme,tol", [(CIC, 1e-10), (TSC, 1e-10), (ESK, 1e-10), (NGP, 0.05)])
def test_scheme_charge_conservation(port, pg, order, scheme, tol):
    # testSchemeChargeConservation, main_test.cpp:25-46
    p = maxwellian(port, 32, 32, 1.0, 1.0, 1000)
    rho, _ = check(port, pg, 32, 32, 1.0, 1.0, p, scheme, 0.0, order)
    err = abs(rho.sum() * (1 / 32) ** 2 - p["q"].sum()) / np.abs(p["q"]).sum()
    assert err <= tol


@pytest.mark.parametrize("order", ["sorted", "unsorted"])
def test_esirkepov_moving_charge_conservation(port, pg, order):
    # testEsirkepovMovingChargeConservation, main_test.cpp:52-72 (some moves exceed a cell: general path)
    p = maxwellian(port, 32, 32, 1.0, 1.0, 1000)
    rho, _ = check(port, pg, 32, 32, 1.0, 1.0, p, ESK, 0.01, order)
    err = abs(rho.sum() * (1 / 32) ** 2 - p["q"].sum()) / np.abs(p["q"]).sum()
    assert err <= 1e-10


def test_gpu_deposit_128(port, pg):
    # testGpuDeposit, main_test.cpp:158-180 (CIC, 128^2, 5000 particles, <= 1e-9)
    p = maxwellian(port, 128, 128, 1.0, 1.0, 5000)
    rho, _ = check(port, pg, 128, 128, 1.0, 1.0, p, CIC)
    err = abs(rho.sum() * (1 / 128) ** 2 - p["q"].sum()) / np.abs(p["q"]).sum()
    assert err <= 1e-9


# ---- shapes, tiles and orders -------------------------------------------
@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
@pytest.mark.parametrize("order", ["sorted", "unsorted", "atomic"])
@pytest.mark.parametrize("grid", [(37, 23, 3.7, 2.3), (64, 64, 64.0, 64.0), (1, 1, 1.0, 1.0), (2, 3, 2.0, 3.0),
                                  (200, 5, 20.0, 0.5)])
def test_grids(port, pg, scheme, order, grid):
    nx, ny, lx, ly = grid
    p = maxwellian(port, nx, ny, lx, ly, 20000, seed=7, T=0.3)
    check(port, pg, nx, ny, lx, ly, p, scheme, 0.05, order)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
@pytest.mark.parametrize("tile", [(1, 1), (7, 3), (64, 32), (16, 16), (32, 8)])
def test_tiles(port, pg, scheme, tile):
    p = maxwellian(port, 96, 80, 96.0, 80.0, 60000, seed=3, T=0.01)
    check(port, pg, 96, 80, 96.0, 80.0, p, scheme, 0.1, "sorted", tile)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_sorted_equals_unsorted_bitwise(port, pg, scheme):
    p = maxwellian(port, 50, 70, 5.0, 7.0, 100000, seed=21, T=0.5)
    _, a, ua, _ = gpu_deposit(pg, 50, 70, 5.0, 7.0, p, scheme, 0.02, "sorted")
    _, b, ub, _ = gpu_deposit(pg, 50, 70, 5.0, 7.0, p, scheme, 0.02, "unsorted")
    _, c, _, _ = gpu_deposit(pg, 50, 70, 5.0, 7.0, p, scheme, 0.02, "sorted", (5, 9))
    _, d, _, _ = gpu_deposit(pg, 50, 70, 5.0, 7.0, p, scheme, 0.02, "atomic")
    assert ua == ub and np.array_equal(a, b) and np.array_equal(a, c) and np.array_equal(a, d)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_nearly_sorted_after_push(port, pg, scheme):
    # sort, then push: particles are nearly cell-ordered; AUTO uses the run-aggregating kernel
    p = maxwellian(port, 64, 48, 6.4, 4.8, 200000, seed=12, T=0.05)
    with pg.Context(64, 48, 6.4, 4.8, len(p["x"])) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        c.sort()
        c.push(0.3)
        assert not c.is_sorted()
        c.deposit(scheme, 0.05, download=False)
        acc, unit = c.rho_fixed()
        lay = c.device_layout()
        c.set_order(pg.ORDER_ATOMIC)
        c.deposit(scheme, 0.05, download=False)
        acc2, _ = c.rho_fixed()
    _, maxq = port.normalize_charge(p["q"])
    want, wunit = port.deposit_fixed(64, 48, 6.4, 4.8, scheme, lay["cell"], lay["xr"], lay["yr"], lay["q"], maxq,
                                     lay["vx"], lay["vy"], 0.05)
    assert unit == wunit and np.array_equal(acc, want) and np.array_equal(acc2, want)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_pushed_since_sort_uses_stale_ranges(port, pg, scheme):
    """After a sort and a push of several cells, PIC_ORDER_SORTED still walks the
    sort's cell ranges; particles that left their tile row go straight to the
    global grid. Bit-identical to the oracle and to the other kernels."""
    p = maxwellian(port, 64, 48, 6.4, 4.8, 150000, seed=13, T=3.0)
    with pg.Context(64, 48, 6.4, 4.8, len(p["x"])) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        c.sort()
        c.set_tile(16, 4)
        c.push(0.2)
        assert not c.is_sorted()
        c.deposit(scheme, 0.02, download=False)
        acc, unit = c.rho_fixed()
        c.set_order(pg.ORDER_SORTED)
        c.deposit(scheme, 0.02, download=False)
        acc_s, _ = c.rho_fixed()
        c.set_order(pg.ORDER_UNSORTED)
        c.deposit(scheme, 0.02, download=False)
        acc_u, _ = c.rho_fixed()
        lay = c.device_layout()
    _, maxq = port.normalize_charge(p["q"])
    want, wunit = port.deposit_fixed(64, 48, 6.4, 4.8, scheme, lay["cell"], lay["xr"], lay["yr"], lay["q"], maxq,
                                     lay["vx"], lay["vy"], 0.02)
    assert unit == wunit
    assert np.array_equal(acc, want) and np.array_equal(acc_s, want) and np.array_equal(acc_u, want)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_uniform_charge_skips_the_charge_stream(port, pg, scheme):
    """One charge for every particle is detected at upload (the kernels then do not
    read the charge stream, and the sort leaves the charge array in place); mixed
    charges are read per particle. Both give the oracle's grid bit for bit."""
    base = maxwellian(port, 48, 40, 4.8, 4.0, 30000, seed=31, T=0.4)
    for q, want_uniform in ((np.full(30000, -2.5), -1.0), (np.full(30000, 0.75), 1.0),
                            (np.where(np.arange(30000) % 7 == 0, 1.0, -1.0), 0.0)):
        p = dict(base, q=q)
        with pg.Context(48, 40, 4.8, 4.0, len(q)) as c:
            c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
            assert c.charge_uniform() == want_uniform
            c.sort()
            lay = c.device_layout()
            if want_uniform:
                assert np.all(lay["q"] == np.float32(want_uniform))
        check(port, pg, 48, 40, 4.8, 4.0, p, scheme, 0.03, "sorted")
        check(port, pg, 48, 40, 4.8, 4.0, p, scheme, 0.03, "unsorted")
    with pg.Context(16, 16, 16.0, 16.0, 1000) as c:
        c.generate(1000, vth=0.1, charge=-0.5, seed=3)
        assert c.charge_uniform() == -1.0


# ---- edge cases ------------------------------------------------------------
@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
@pytest.mark.parametrize("order", ["sorted", "unsorted"])
def test_empty(pg, scheme, order):
    p = dict(x=np.zeros(0), y=np.zeros(0), q=np.zeros(0))
    rho, acc, _, _ = gpu_deposit(pg, 8, 8, 1.0, 1.0, p, scheme, 0.0, order)
    assert not acc.any() and not rho.any()


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_single_particle_and_boundaries(port, pg, scheme):
    lx = 10.0
    xs = np.array([0.0, lx - 1e-13, -0.25, lx + 0.25, 4.5, 4.5 - 1e-12, 9.999999, 5.0, 0.5 - 2 ** -30])
    ys = np.array([3.3, 0.0, lx - 1e-15, -3.0, 4.5, 2.0, 0.0, 7.0 + 1e-14, 0.5])
    p = dict(x=xs, y=ys, q=np.linspace(-2.0, 3.0, len(xs)), vx=np.linspace(-0.5, 0.5, len(xs)),
             vy=np.linspace(0.3, -0.3, len(xs)), m=np.ones(len(xs)))
    check(port, pg, 10, 10, lx, lx, p, scheme, 0.3, "sorted", rel_tol=1e-5)
    # A single particle is a set with one charge: TSC then deposits exact integer
    # weights at 2^-15 resolution (every node within 2^-14 of the FP64 weight
    # product), a relative L2 error of up to about 1e-4 for one particle; the
    # 1e-5 bound holds for populated grids (the 64-particles-per-cell benchmark
    # density reaches 2.3e-6).
    for i in range(len(xs)):
        one = {k: v[i:i + 1] for k, v in p.items()}
        rho, _ = check(port, pg, 10, 10, lx, lx, one, scheme, 0.3, "sorted",
                       rel_tol=2e-4 if scheme == TSC else 1e-5)
        if scheme == TSC:
            ref = port.deposit_ref(10, 10, lx, lx, scheme, one, dt=0.3)
            assert np.max(np.abs(rho - ref)) <= 2.0 ** -14 * abs(one["q"][0])


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_all_particles_in_one_cell(port, pg, scheme):
    rng = np.random.default_rng(5)
    n = 40000
    p = dict(x=5.0 + rng.random(n), y=7.0 + rng.random(n), q=rng.choice([-1.0, 1.0], n),
             vx=rng.normal(0, 0.2, n), vy=rng.normal(0, 0.2, n), m=np.ones(n))
    for order in ("sorted", "unsorted"):
        check(port, pg, 16, 16, 16.0, 16.0, p, scheme, 0.5, order)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC])
@pytest.mark.parametrize("n", [131000, 200000])
@pytest.mark.parametrize("order", ["sorted", "unsorted"])
def test_dense_tile_same_sign(port, pg, scheme, n, order):
    """Tiles below 2^17 particles use the split 32-bit shared accumulators,
    denser ones add their runs straight to the global grid; both exact. Equal
    charges at one corner node give the largest per-node sums (n * 2^24), and
    long runs of them the largest int32 partial sums in a warp."""
    rng = np.random.default_rng(n)
    x = np.where(rng.random(n) < 0.5, 5.0, 5.0 + rng.random(n))
    p = dict(x=x, y=np.full(n, 7.0), q=np.ones(n), vx=np.zeros(n), vy=np.zeros(n), m=np.ones(n))
    check(port, pg, 16, 16, 16.0, 16.0, p, scheme, 0.0, order)


@pytest.mark.parametrize("order", ["sorted", "unsorted"])
def test_esirkepov_long_moves(port, pg, order):
    # moves of up to ~20 cells take the general trajectory loop
    p = maxwellian(port, 40, 40, 4.0, 4.0, 5000, seed=9, T=25.0)
    check(port, pg, 40, 40, 4.0, 4.0, p, ESK, 0.08, order)


def test_deterministic_repeats(port, pg):
    p = maxwellian(port, 64, 64, 1.0, 1.0, 200000, seed=1)
    outs = [gpu_deposit(pg, 64, 64, 1.0, 1.0, p, TSC, 0.0, "sorted")[1] for _ in range(3)]
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def test_bad_inputs_are_errors(pg):
    with pg.Context(8, 8, 1.0, 1.0, 4) as c:
        with pytest.raises(pg.PicError) as e:
            c.upload(np.array([0.1, np.nan]), np.array([0.1, 0.2]), np.array([1.0, 1.0]))
        assert e.value.code == -9
        c.upload(np.array([0.5, 0.1]), np.array([0.2, 0.1]), np.array([1.0, 1.0]))  # not in cell order
        assert not c.is_sorted()
        with pytest.raises(pg.PicError):
            c.deposit(7)
        c.set_order(pg.ORDER_SORTED)
        with pytest.raises(pg.PicError) as e:
            c.deposit(CIC)
        assert e.value.code == -4
        with pytest.raises(pg.PicError):
            c.upload(np.zeros(5), np.zeros(5), np.zeros(5))
        with pytest.raises(pg.PicError):
            c.set_tile(0, 4)


# ---- the benchmark shapes ----------------------------------------------------
def test_config1_cic_256(port, pg):
    """256x256, dx=1, 1,048,576 particles of charge -1 from the reference's
    initializeUniformMaxwellian positions (seed 42) plus the neutralising
    background N/V; checked against the reference's golden checksums."""
    import os
    from conftest import GOLDEN

    g = dict(np.load(os.path.join(GOLDEN, "config1_cic.npz")))
    n = 1 << 20
    p = port.init_particles(0, 256, 256, 256.0, 256.0, n, p0=1.0, seed=42)
    p["q"] = -np.ones(n)
    rho, acc = check(port, pg, 256, 256, 256.0, 256.0, p, CIC)
    assert abs(rho.sum() - g["sum"]) <= 1e-9 * abs(g["sum"])
    assert np.max(np.abs(rho[::997] - g["sample"])) <= 1e-5
    rho_bg, _, _, _ = gpu_deposit(pg, 256, 256, 256.0, 256.0, p, CIC, background=16.0)
    assert np.max(np.abs(rho_bg - (rho + 16.0))) == 0.0


@pytest.mark.slow
@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_config2_full_size(port, pg, scheme):
    """1024x1024, 64 particles per cell (67,108,864), density 1+0.01cos(2 pi x/1024),
    vth 0.1, Esirkepov dt 0.1; random order and cell-sorted; bit-exact vs the
    oracle and within tolerance of the FP64 deposit."""
    p = workloads.density_cos(1024, 1024, 64, 0.01, 0.1, seed=42)
    n = len(p["x"])
    ref = port.deposit_ref(1024, 1024, 1024.0, 1024.0, scheme, p, dt=0.1, threads=16)
    with pg.Context(1024, 1024, 1024.0, 1024.0, n) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        c.set_order(pg.ORDER_UNSORTED)
        c.deposit(scheme, 0.1, download=False)
        acc_u, unit = c.rho_fixed()
        c.set_order(pg.ORDER_AUTO)
        c.sort()
        rho = c.deposit(scheme, 0.1)
        acc_s, unit_s = c.rho_fixed()
        lay = c.device_layout()
    assert unit == unit_s and np.array_equal(acc_u, acc_s)
    _, maxq = port.normalize_charge(p["q"])
    want, wunit = port.deposit_fixed(1024, 1024, 1024.0, 1024.0, scheme, lay["cell"], lay["xr"], lay["yr"], lay["q"],
                                     maxq, lay["vx"], lay["vy"], 0.1)
    assert unit == wunit and np.array_equal(acc_s, want)
    rel = np.linalg.norm(rho - ref) / np.linalg.norm(ref)
    assert rel <= REL_L2_TOL, rel


@pytest.mark.parametrize("grid", [(64, 48, 64.0, 48.0), (37, 23, 3.7, 2.3)])
def test_pinned_upload_matches_pageable(port, pg, grid):
    """Page-locked inputs are read by the conversion kernel over the host link;
    the device layout must equal the staged (pageable) upload's bit for bit."""
    nx, ny, lx, ly = grid
    p = maxwellian(port, nx, ny, lx, ly, 300000, seed=17)
    pins = {k: pg.PinnedArray(len(p["x"])) for k in ("x", "y", "vx", "vy", "q")}
    try:
        for k, a in pins.items():
            a.array[:] = p[k]
        with pg.Context(nx, ny, lx, ly, len(p["x"])) as c:
            c.upload(pins["x"].array, pins["y"].array, pins["q"].array, pins["vx"].array, pins["vy"].array)
            a = c.device_layout()
            c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"])
            b = c.device_layout()
        for k in a:
            assert np.array_equal(a[k], b[k]), k
        cell, xr, yr = port.to_device(nx, ny, lx, ly, p["x"], p["y"])
        assert np.array_equal(a["cell"], cell) and np.array_equal(a["xr"], xr) and np.array_equal(a["yr"], yr)
    finally:
        for v in pins.values():
            v.free()
