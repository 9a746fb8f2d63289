"""Fields, FFT Poisson, diagnostics, gather and push through the C ABI vs the oracle.

* FFT Poisson (cuFFT FP64) vs the reference's own solver (golden fixture from
  oracle/_ref, tests/golden/small_32.npz) and the numpy restatement
  (poisson_fft.cpp:45-94): relative max error <= 1e-12.
* E-field from a given phi: bit-exact with the oracle's restatement of
  poisson_fft.cpp:77-93.
* gather / push / fused: bit-exact with the oracle's restatement of the GPU's
  FP32 cell-relative arithmetic, and close to the reference's FP64 gather/push
  (deposition.cpp:335-374).
* diagnostics: FP64 sums within 1e-12 relative of the oracle's sums.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def ctx_with(pg, nx, ny, lx, ly, p):
    c = pg.Context(nx, ny, lx, ly, max(len(p["x"]), 1))
    c.upload(p["x"], p["y"], p["q"], p.get("vx"), p.get("vy"), p.get("m"))
    return c


def test_poisson_fft_matches_reference_golden(pg, oracle_mod):
    g = dict(np.load(os.path.join(GOLDEN, "small_32.npz")))
    with pg.Context(32, 32, 1.0, 1.0, 1) as c:
        c.set_rho(g["poisson_rho"])
        c.poisson_fft()
        phi, ex, ey = c.fields()
    for got, want in ((phi, g["fft_phi"]), (ex, g["fft_ex"]), (ey, g["fft_ey"])):
        assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("grid", [(64, 48, 6.4, 1.2), (256, 256, 256.0, 256.0), (30, 18, 3.0, 1.8), (1, 8, 1.0, 2.0)])
def test_poisson_fft_vs_numpy(pg, oracle_mod, grid):
    nx, ny, lx, ly = grid
    rng = np.random.default_rng(3)
    rho = rng.normal(size=nx * ny)
    with pg.Context(nx, ny, lx, ly, 1) as c:
        c.set_rho(rho)
        c.poisson_fft()
        phi, ex, ey = c.fields()
    wphi, wex, wey = oracle_mod.poisson_fft(nx, ny, lx, ly, rho)
    for got, want in ((phi, wphi), (ex, wex), (ey, wey)):
        assert np.max(np.abs(got - want)) <= 1e-12 * max(np.max(np.abs(want)), 1e-300)


def test_efield_bit_exact(pg, port):
    rng = np.random.default_rng(4)
    rho = rng.normal(size=40 * 24)
    with pg.Context(40, 24, 4.0, 2.4, 1) as c:
        c.set_rho(rho)
        c.poisson_fft()
        phi, ex, ey = c.fields()
    wex, wey = port.efield(40, 24, 4.0, 2.4, phi)
    assert np.array_equal(ex, wex) and np.array_equal(ey, wey)


@pytest.mark.parametrize("mass", [False, True])
@pytest.mark.parametrize("dt", [0.05, 1.7])
def test_gather_push_bit_exact(pg, port, mass, dt):
    nx, ny, lx, ly = 48, 40, 4.8, 4.0
    p = port.init_particles(0, nx, ny, lx, ly, 30000, p0=1.0, seed=6)
    if mass:
        p["m"] = 1.0 + np.random.default_rng(1).random(len(p["x"]))
    rng = np.random.default_rng(7)
    ex, ey = rng.normal(size=nx * ny), rng.normal(size=nx * ny)
    qn, maxq = port.normalize_charge(p["q"])
    m32 = p["m"].astype(np.float32) if mass else None
    for mode in ("gather", "push", "gather_push"):
        with ctx_with(pg, nx, ny, lx, ly, p) as c:
            c.set_fields(ex=ex, ey=ey)
            before = c.device_layout()
            getattr(c, mode)(dt)
            after = c.device_layout()
        want = port.move_f32(nx, ny, lx, ly, before, maxq, ex, ey, dt, gather=mode != "push",
                             push=mode != "gather", m=m32)
        for k in ("cell", "xr", "yr", "vx", "vy"):
            assert np.array_equal(after[k], want[k]), (mode, k)


def test_gather_push_close_to_fp64_reference(pg, port):
    nx, ny, lx, ly = 64, 64, 1.0, 1.0
    p = port.init_particles(0, nx, ny, lx, ly, 20000, p0=1.0, seed=8)
    rng = np.random.default_rng(9)
    ex, ey = rng.normal(size=nx * ny), rng.normal(size=nx * ny)
    dt = 0.01
    with ctx_with(pg, nx, ny, lx, ly, p) as c:
        c.set_fields(ex=ex, ey=ey)
        c.gather(dt)
        c.push(dt)
        got = c.download()
    vx, vy = port.gather_ref(nx, ny, lx, ly, p, ex, ey, dt)
    q = dict(p)
    q["vx"], q["vy"] = vx, vy
    x, y = port.push_ref(nx, ny, lx, ly, q, dt)
    assert np.max(np.abs(got["vx"] - vx)) <= 1e-5 * np.max(np.abs(vx))
    dxw = np.abs(got["x"] - x)
    dxw = np.minimum(dxw, lx - dxw)  # periodic distance
    assert np.max(dxw) <= 1e-6 * lx


def test_diagnostics_vs_oracle(pg, port):
    nx, ny, lx, ly = 64, 32, 2.0, 1.0
    p = port.init_particles(0, nx, ny, lx, ly, 50000, p0=0.5, seed=10)
    with ctx_with(pg, nx, ny, lx, ly, p) as c:
        rho = c.deposit(1)
        c.poisson_fft()
        d = c.diagnostics()
        lay = c.device_layout()
        _, ex, ey = c.fields()
    qn, maxq = port.normalize_charge(p["q"])
    q32 = (qn * np.float32(maxq)).astype(np.float64)
    vx, vy = lay["vx"].astype(np.float64), lay["vy"].astype(np.float64)
    ke = np.sum(0.5 * (vx * vx + vy * vy))
    ir = port.integrated_rho(nx, ny, lx, ly, rho)
    fe = port.field_energy(nx, ny, lx, ly, ex, ey)
    assert abs(d["kinetic_energy"] - ke) <= 1e-12 * ke
    assert abs(d["field_energy"] - fe) <= 1e-12 * fe
    assert abs(d["total_charge"] - q32.sum()) <= 1e-12 * np.abs(q32).sum()
    assert abs(d["integrated_rho"] - ir) <= 1e-12 * np.abs(q32).sum()
    assert d["charge_error"] <= 1e-10


def test_diagnostics_deterministic(pg, port):
    p = port.init_particles(0, 128, 128, 1.0, 1.0, 300000, p0=1.0, seed=11)
    outs = []
    for _ in range(2):
        with ctx_with(pg, 128, 128, 1.0, 1.0, p) as c:
            c.deposit(2)
            c.poisson_fft()
            outs.append(c.diagnostics())
    assert outs[0] == outs[1]
