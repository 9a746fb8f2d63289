"""Esirkepov current (Jx, Jy) through the C ABI.

No reference implementation exists (the reference's "Esirkepov" deposits
charge only, src/deposition/ngp.cpp:13-84); the oracle restates Esirkepov,
Comput. Phys. Commun. 135 (2001) 144 (CIC shape) in FP64 and the GPU's integer
form exactly. Checks:
  * int64 grids bit-exact with the oracle's integer restatement;
  * J within 1e-5 relative L2 of the FP64 Esirkepov current;
  * continuity exactly zero in integers: CIC(after push) - CIC(before) + div J = 0;
  * the FP64 continuity residual of the GPU's J, rho in physical units, at
    round-off of the FP32 state;
  * |v| dt >= cell size is PIC_ERR_COURANT.
"""
import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu

# J must balance the FP32-rounded integer charge difference R1 - R0 exactly, so its
# error against the FP64 current is about one charge unit per node and particle:
# rel-L2 ~1e-5..3e-5 at |v|dt ~ 0.01 cell, smaller for larger moves.
REL_L2_TOL = 5e-5


def run_current(pg, nx, ny, lx, ly, p, dt, sort=False):
    with pg.Context(nx, ny, lx, ly, len(p["x"])) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        if sort:
            c.sort()
        lay = c.device_layout()
        c.deposit(1, download=False)
        r0, unit = c.rho_fixed()
        jx_f, jy_f = c.deposit_current(dt)
        jx, jy, ux, uy = c.current_fixed()
        c.push(dt)
        c.deposit(1, download=False)
        r1, _ = c.rho_fixed()
    return lay, jx, jy, ux, uy, jx_f, jy_f, r0, r1, unit


@pytest.mark.parametrize("grid,n,T,dt", [((32, 32, 32.0, 32.0), 20000, 0.01, 0.5), ((48, 40, 4.8, 2.0), 60000, 0.5, 0.01),
                                         ((8, 6, 8.0, 6.0), 5000, 0.01, 1.0), ((1, 1, 1.0, 1.0), 100, 0.01, 1.0)])
@pytest.mark.parametrize("sort", [False, True])
def test_current_parity_and_exact_continuity(pg, port, grid, n, T, dt, sort):
    nx, ny, lx, ly = grid
    p = port.init_particles(0, nx, ny, lx, ly, n, p0=T, seed=13)
    lay, jx, jy, ux, uy, jx_f, jy_f, r0, r1, unit = run_current(pg, nx, ny, lx, ly, p, dt, sort)
    _, maxq = port.normalize_charge(p["q"])
    wjx, wjy, wux, wuy = port.esirkepov_j_fixed(nx, ny, lx, ly, lay, maxq, dt)
    assert ux == wux and uy == wuy
    assert np.array_equal(jx, wjx) and np.array_equal(jy, wjy)
    assert np.array_equal(jx_f, jx * ux) and np.array_equal(jy_f, jy * uy)
    JX, JY = jx.reshape(ny, nx), jy.reshape(ny, nx)
    div = (JX - np.roll(JX, 1, axis=1)) + (JY - np.roll(JY, 1, axis=0))
    assert not ((r1 - r0).reshape(ny, nx) + div).any()
    rjx, rjy = port.esirkepov_j_ref(nx, ny, lx, ly, p, dt)
    pa = dict(p)
    pa["q"] = np.abs(p["q"])
    ajx, ajy = port.esirkepov_j_ref(nx, ny, lx, ly, pa, dt)
    for got, want, mag in ((jx_f, rjx, ajx), (jy_f, rjy, ajy)):
        # scale: ||J|| (or the magnitude ||J(|q|)|| when mixed charges cancel on a tiny grid)
        nrm = max(np.linalg.norm(want), 1e-3 * np.linalg.norm(mag))
        assert np.linalg.norm(got - want) / nrm <= REL_L2_TOL


def test_current_config2_shape_slice(pg, port):
    """1024x1024 workload shape (density 1+0.01cos, vth 0.1, dt 0.1) on a 1/16 slice of the particles."""
    p = workloads.density_cos(1024, 1024, 4, 0.01, 0.1, seed=42)
    lay, jx, jy, ux, uy, jx_f, jy_f, r0, r1, unit = run_current(pg, 1024, 1024, 1024.0, 1024.0, p, 0.1, sort=True)
    JX, JY = jx.reshape(1024, 1024), jy.reshape(1024, 1024)
    div = (JX - np.roll(JX, 1, axis=1)) + (JY - np.roll(JY, 1, axis=0))
    assert not ((r1 - r0).reshape(1024, 1024) + div).any()
    rjx, rjy = port.esirkepov_j_ref(1024, 1024, 1024.0, 1024.0, p, 0.1)
    assert np.linalg.norm(jx_f - rjx) / np.linalg.norm(rjx) <= REL_L2_TOL
    assert np.linalg.norm(jy_f - rjy) / np.linalg.norm(rjy) <= REL_L2_TOL


@pytest.mark.parametrize("sort", [False, True])
def test_courant_violation_is_an_error(pg, port, sort):
    p = port.init_particles(0, 16, 16, 16.0, 16.0, 1000, p0=1.0, seed=1)
    p["vx"][7] = 50.0
    with pg.Context(16, 16, 16.0, 16.0, 1000) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        if sort:
            c.sort()
        with pytest.raises(pg.PicError) as e:
            c.deposit_current(0.1)
        assert e.value.code == -6
        p["vx"][7] = 0.0
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        if sort:
            c.sort()
        c.deposit_current(0.1)  # context still usable
