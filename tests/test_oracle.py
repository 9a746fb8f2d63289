"""The CPU oracle, pinned before it is trusted.

* against the reference itself (oracle/_ref, compiled from the reference
  sources; skipped where the reference checkout is absent),
* against the golden fixtures in tests/golden (made by the reference),
* against the reference's archived noise study (data/benchmarks/noise_vs_grid.csv:2-13),
* and with the reference's own test conditions (src/main_test.cpp:25-72).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

NGP, CIC, TSC, ESK = 0, 1, 2, 3


def small():
    return dict(np.load(os.path.join(GOLDEN, "small_32.npz")))


# ---- against the compiled reference -------------------------------------
@pytest.mark.parametrize("kind,args", [(0, dict(p0=1.0)), (1, dict(p0=0.01, mode=2)),
                                       (2, dict(p0=0.05, p1=0.1, mode=1)), (3, dict(p0=0.3, p1=0.01)),
                                       (4, dict(p0=0.2, p1=0.02))])
def test_initialisers_bit_exact_vs_reference(port, ref, kind, args):
    a = port.init_particles(kind, 32, 16, 1.0, 2.0, 777, seed=9, **args)
    b = ref.init_particles(kind, 32, 16, 1.0, 2.0, 777, seed=9, **args)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
@pytest.mark.parametrize("dt", [0.0, 0.01, 0.2])
def test_deposit_bit_exact_vs_reference(port, ref, scheme, dt):
    p = port.init_particles(0, 24, 40, 1.5, 2.5, 3000, p0=1.0, seed=5)
    a = port.deposit_ref(24, 40, 1.5, 2.5, scheme, p, dt=dt)
    b = ref.deposit(24, 40, 1.5, 2.5, scheme, p, dt=dt)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("scheme", [NGP, CIC, ESK])
def test_parallel_deposit_vs_reference(port, ref, scheme):
    # the reference merges thread grids in arrival order; equal up to FP64 rounding
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 20000, p0=1.0, seed=3)
    a = port.deposit_ref(32, 32, 1.0, 1.0, scheme, p, dt=0.01, threads=4)
    b = ref.deposit(32, 32, 1.0, 1.0, scheme, p, dt=0.01, threads=4)
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))


def test_parallel_tsc_of_the_port(port, ref):
    # the reference's privatised TSC is not used (it writes past its per-thread grid);
    # the port's parallel TSC equals the serial one and the reference's serial TSC
    # up to the FP64 summation order
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 20000, p0=1.0, seed=5)
    a = port.deposit_ref(32, 32, 1.0, 1.0, TSC, p, threads=4)
    b = port.deposit_ref(32, 32, 1.0, 1.0, TSC, p, threads=1)
    c = ref.deposit(32, 32, 1.0, 1.0, TSC, p, threads=1)
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    assert np.max(np.abs(a - c)) <= 1e-12 * np.max(np.abs(c))


def test_sort_keys_and_cells_vs_reference(port, ref):
    p = port.init_particles(0, 20, 12, 2.0, 1.0, 5000, p0=1.0, seed=11)
    keys, perm, offs = port.stable_cell_sort(20, 12, 2.0, 1.0, p["x"], p["y"])
    for i in range(0, 5000, 97):
        assert port.cell_index(20, 12, 2.0, 1.0, p["x"][i], p["y"][i]) == ref.lib.ref_cell_index(
            20, 12, 2.0, 1.0, p["x"][i], p["y"][i])
    r = ref.sort(20, 12, 2.0, 1.0, p)
    rkeys = np.array([port.cell_index(20, 12, 2.0, 1.0, x, y) for x, y in zip(r["x"], r["y"])])
    assert np.array_equal(rkeys, keys)  # same key sequence
    # each cell holds the same multiset of particles
    for c in range(240):
        a = np.sort(p["x"][perm[offs[c]:offs[c + 1]]])
        b = np.sort(r["x"][offs[c]:offs[c + 1]])
        assert np.array_equal(a, b)


def test_gather_push_vs_reference(port, ref):
    p = port.init_particles(0, 16, 16, 1.0, 1.0, 2000, p0=1.0, seed=2)
    rng = np.random.default_rng(0)
    ex, ey = rng.normal(size=256), rng.normal(size=256)
    a = port.gather_ref(16, 16, 1.0, 1.0, p, ex, ey, 0.05)
    b = ref.gather(16, 16, 1.0, 1.0, p, ex, ey, 0.05)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    p["vx"] *= 30.0
    a = port.push_ref(16, 16, 1.0, 1.0, p, 0.05)
    b = ref.push(16, 16, 1.0, 1.0, p, 0.05)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_gs_and_fft_vs_reference(port, ref, oracle_mod):
    g = small()
    rho = g["poisson_rho"]
    phi, ex, ey, _ = port.gs_ref(32, 32, 1.0, 1.0, rho, 500, 1e-6)
    rphi, rex, rey = ref.poisson_gs(32, 32, 1.0, 1.0, rho, 500, 1e-6)
    assert np.array_equal(phi, rphi) and np.array_equal(ex, rex)
    fphi, fex, fey = oracle_mod.poisson_fft(32, 32, 1.0, 1.0, rho)
    qphi, qex, qey = ref.poisson_fft(32, 32, 1.0, 1.0, rho)
    assert np.max(np.abs(fphi - qphi)) <= 1e-12 * np.max(np.abs(qphi))
    assert np.max(np.abs(fex - qex)) <= 1e-12 * np.max(np.abs(qex))


# ---- against the committed golden fixtures (no reference needed) ---------
def test_port_matches_golden_small(port):
    g = small()
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 1000, p0=1.0, seed=123)
    for k in ("x", "y", "q", "m"):
        assert np.array_equal(p[k], g[k]), k
    # velocities come from libm log/sqrt; allow the last bit across platforms
    assert np.allclose(p["vx"], g["vx"], rtol=1e-15, atol=0)
    for i in range(1000):
        assert port.cell_index(32, 32, 1.0, 1.0, p["x"][i], p["y"][i]) == g["keys"][i]
    for scheme in range(4):
        for dt in (0.0, 0.01):
            pp = dict(g)
            a = port.deposit_ref(32, 32, 1.0, 1.0, scheme, dict(x=g["x"], y=g["y"], vx=g["vx"], vy=g["vy"],
                                                                q=g["q"]), dt=dt)
            assert np.array_equal(a, pp[f"rho_s{scheme}_dt{dt}"]), (scheme, dt)


def test_port_matches_golden_poisson(port, oracle_mod):
    g = small()
    phi, ex, ey, _ = port.gs_ref(32, 32, 1.0, 1.0, g["poisson_rho"], 500, 1e-6)
    assert np.array_equal(phi, g["gs_phi"]) and np.array_equal(ey, g["gs_ey"])
    fphi, fex, fey = oracle_mod.poisson_fft(32, 32, 1.0, 1.0, g["poisson_rho"])
    assert np.max(np.abs(fphi - g["fft_phi"])) <= 1e-12 * np.max(np.abs(g["fft_phi"]))


def test_port_matches_golden_config1(port):
    g = dict(np.load(os.path.join(GOLDEN, "config1_cic.npz")))
    n = 1 << 20
    p = port.init_particles(0, 256, 256, 256.0, 256.0, n, p0=1.0, seed=42)
    assert np.array_equal(p["x"][:64], g["x_head"]) and np.array_equal(p["y"][:64], g["y_head"])
    p["q"] = -np.ones(n)
    rho = port.deposit_ref(256, 256, 256.0, 256.0, CIC, p)
    assert rho.sum() == g["sum"] and (rho * rho).sum() == g["sumsq"]
    assert np.array_equal(rho[::997], g["sample"])


# data/benchmarks/noise_vs_grid.csv:2-13 (runNoiseVsGridStudy, src/pic/validation.cpp:445-472)
NOISE_VS_GRID = {
    (64, NGP): 0.6090021848, (64, CIC): 0.4003197697, (64, TSC): 0.2659117765, (64, ESK): 0.4003197697,
    (128, NGP): 0.5826140746, (128, CIC): 0.3747387341, (128, TSC): 0.2435981661, (128, ESK): 0.3747387341,
    (256, NGP): 0.5659049422, (256, CIC): 0.3631346553, (256, TSC): 0.2342248984, (256, ESK): 0.3631346553,
}


@pytest.mark.parametrize("g", [64, 128, 256])
def test_noise_vs_grid_golden(port, oracle_mod, g):
    p = port.init_particles(0, g, g, 1.0, 1.0, 100000, p0=1.0, seed=42)
    for s in range(4):
        rho = port.deposit_ref(g, g, 1.0, 1.0, s, p)
        assert round(oracle_mod.spectral_noise(g, g, rho), 10) == NOISE_VS_GRID[(g, s)]


# ---- the reference's own tests, on the oracle (src/main_test.cpp) ---------
@pytest.mark.parametrize("scheme,tol", [(CIC, 1e-10), (TSC, 1e-10), (ESK, 1e-10), (NGP, 0.05)])
def test_scheme_charge_conservation(port, scheme, tol):
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 1000, p0=1.0, seed=123)
    rho = port.deposit_ref(32, 32, 1.0, 1.0, scheme, p, dt=0.0)
    err = abs(port.integrated_rho(32, 32, 1.0, 1.0, rho) - p["q"].sum()) / np.abs(p["q"]).sum()
    assert err <= tol


def test_esirkepov_moving_charge_conservation(port):
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 1000, p0=1.0, seed=123)
    rho = port.deposit_ref(32, 32, 1.0, 1.0, ESK, p, dt=0.01)
    err = abs(port.integrated_rho(32, 32, 1.0, 1.0, rho) - p["q"].sum()) / np.abs(p["q"]).sum()
    assert err <= 1e-10


# ---- the oracle's GPU-arithmetic restatement against its FP64 restatement --
@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_fixed_point_restatement_close_to_fp64(port, scheme):
    p = port.init_particles(0, 64, 48, 64.0, 48.0, 50000, p0=0.04, seed=8)
    cell, xr, yr = port.to_device(64, 48, 64.0, 48.0, p["x"], p["y"])
    qn, maxq = port.normalize_charge(p["q"])
    acc, unit = port.deposit_fixed(64, 48, 64.0, 48.0, scheme, cell, xr, yr, qn, maxq, p["vx"].astype(np.float32),
                                   p["vy"].astype(np.float32), dt=0.1)
    got = acc * unit
    want = port.deposit_ref(64, 48, 64.0, 48.0, scheme, p, dt=0.1)
    rel = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert rel < 1e-6
    # every particle deposits exactly its integer charge, so the grid total is exact
    assert acc.sum() == port.fixed_total(scheme, qn)
    assert abs(acc.sum() * unit - p["q"].sum()) <= 1e-12 * np.abs(p["q"]).sum()


def test_tsc_one_charge_exact_integer_form(port):
    """One charge for every particle: TSC deposits exact integer weights (each axis'
    three weights rounded to 2^-15 and summing to 2^15 exactly). On the benchmark's
    density (1 + 0.01 cos, 64 particles per cell, a 128x128 slice) rho stays within
    3e-6 relative L2 of the reference-pinned FP64 deposit, a third of the 1e-5 gate,
    and the grid total is exactly n * 2^30 units (the charge sits in the unit)."""
    import workloads

    nx = ny = 128
    p = workloads.density_cos(nx, ny, 64, 0.01, 0.1, seed=5)
    n = len(p["x"])
    cell, xr, yr = port.to_device(nx, ny, float(nx), float(ny), p["x"], p["y"])
    qn, maxq = port.normalize_charge(p["q"])
    assert port.charge_uniform(qn) and not port.charge_uniform(np.where(np.arange(n) == 7, 1, -1).astype(np.float32))
    acc, unit = port.deposit_fixed(nx, ny, float(nx), float(ny), TSC, cell, xr, yr, qn, maxq)
    assert unit == -2.0 ** -30 and acc.min() >= 0
    assert acc.sum() == port.fixed_total(TSC, qn) == n << 30
    want = port.deposit_ref(nx, ny, float(nx), float(ny), TSC, p, threads=4)
    rel = np.linalg.norm(acc * unit - want) / np.linalg.norm(want)
    assert rel <= 3e-6, rel
    # one particle at a time: its 16 frame values are WX[i] * WY[j] with each axis summing to 2^15
    for r in (0.0, 0.25, 0.5 - 2 ** -24, 0.5, 0.75, 1.0 - 2 ** -24):
        one_c, one_x, one_y = np.array([5 * 16 + 5], np.uint32), np.array([r], np.float32), np.array([0.5], np.float32)
        a1, _ = port.deposit_fixed(16, 16, 16.0, 16.0, TSC, one_c, one_x, one_y, np.array([1.0], np.float32), 1.0)
        g = a1.reshape(16, 16)
        wy = g.sum(axis=1)  # a row's sum is 2^15 * WY[j]
        wx = g.sum(axis=0)
        assert wy.sum() == 2 ** 30 and np.all(wy % 2 ** 15 == 0) and np.all(wx % 2 ** 15 == 0)
        xi = 5.0 + r
        i0 = int(np.floor(xi - 0.5))
        t = xi - i0
        w = np.array([0.5 * (1.5 - t) ** 2, 0.75 - (t - 1) ** 2, 0.5 * (t - 0.5) ** 2])
        got = wx[i0:i0 + 3] / 2.0 ** 30
        assert np.max(np.abs(got - w)) <= 2.0 ** -15, (r, got, w)


def test_to_device_keeps_ngp_choice(port):
    # offsets just below 0.5 must not round up to 0.5f (ngp.cpp:116-117 uses wx >= 0.5)
    x = np.array([0.5 - 2 ** -30, 0.5, 3.5 - 2 ** -40, 1.0 - 2 ** -30, 0.0])
    cell, xr, yr = port.to_device(8, 8, 8.0, 8.0, x, x)
    assert xr[0] < 0.5 and xr[1] == 0.5 and xr[2] < 0.5 and cell[2] == 3 * 8 + 3
    assert xr[3] == 1.0  # rounds to the cell's far edge; the key stays in cell 0
    assert cell[3] == 0


def test_stable_sort_restatement(port):
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 50, size=10000).astype(np.uint32)
    ks, perm, offs = port.stable_sort_keys(keys, 50)
    order = np.argsort(keys, kind="stable")
    assert np.array_equal(perm, order) and np.array_equal(ks, keys[order])
    assert np.array_equal(offs, np.concatenate([[0], np.cumsum(np.bincount(keys, minlength=50))]))


def test_rbgs_matches_converged_lexicographic_gs(port):
    g = small()
    rho = g["poisson_rho"]
    phi_rb, it, res = port.rbgs(32, 32, 1.0, 1.0, rho, tol=1e-10, max_iters=200000)
    assert res <= 1e-10
    phi_gs, _, _, _ = port.gs_ref(32, 32, 1.0, 1.0, rho, 200000, 1e-15)
    phi_gs = phi_gs - phi_gs.mean()
    assert np.max(np.abs(phi_rb - phi_gs)) <= 1e-8 * np.max(np.abs(phi_gs))


# ---- the oracle's time loop and frequency estimator vs the reference -------
@pytest.mark.parametrize("scheme", [CIC, ESK])
def test_simulate_matches_reference_simulation(port, ref, oracle_mod, scheme):
    # Simulation::run (simulation.cpp:69-145) on a uniform Maxwellian, FFT Poisson
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 2000, p0=1.0, seed=42)
    h, _ = oracle_mod.simulate(port, 32, 32, 1.0, 1.0, p, scheme, 0.005, 30)
    r = ref.simulation_run(32, 32, 1.0, 1.0, 0.005, 30, scheme, 2000, seed=42, mode=0, temperature=1.0)
    assert np.allclose(h[:, 5], r["total"], rtol=1e-10, atol=0)
    assert np.allclose(h[:, 3], r["kinetic"], rtol=1e-10, atol=0)


def test_dominant_frequency_matches_reference(port, ref, oracle_mod):
    # runLangmuirValidation (validation.cpp:200-261) on a shortened run
    out = ref.langmuir_validation(64, 64, 1.0, 1.0, 0.002, 2048, CIC, 200, amplitude=0.05, mode_number=1)
    p = port.init_particles(1, 64, 64, 1.0, 1.0, 200, p0=0.05, mode=1, seed=42)
    h, _ = oracle_mod.simulate(port, 64, 64, 1.0, 1.0, p, CIC, 0.002, 2048, background=1.0)
    assert oracle_mod.dominant_frequency(h[2048 // 4:, 4], 0.002) == out["omega_measured"]


def test_port_deposit_speed_matches_the_reference(port, ref):
    """The port is the timed CPU baseline on hosts where the reference does not build,
    so its all-core CIC deposit must run at the reference's speed when both are timed
    the reference's way (depositChargeTimedSoA: untimed warm-ups, then the timed
    clear + deposit). Best of three at 4 M and 8 M cell-sorted particles, all cores;
    the port may not be more than 1.3x slower (timing noise)."""
    import workloads

    threads = os.cpu_count() or 1
    base = workloads.density_cos(1024, 1024, 8, 0.01, 0.1, seed=3)
    key = np.floor(base["y"]).astype(np.int64) * 1024 + np.floor(base["x"]).astype(np.int64)
    o = np.argsort(key, kind="stable")
    base = {k: v[o] for k, v in base.items()}
    for n in (4_000_000, 8_000_000):
        p = {k: np.ascontiguousarray(v[:n]) for k, v in base.items()}
        t_port = min(port.deposit_timed(1024, 1024, 1024.0, 1024.0, CIC, p, threads=threads, repeats=3)
                     for _ in range(3))
        t_ref = min(ref.deposit_timed(1024, 1024, 1024.0, 1024.0, CIC, p, threads=threads, repeats=3)["deposit_ms"]
                    for _ in range(3))
        assert t_port <= 1.3 * t_ref, (n, t_port, t_ref)


@pytest.mark.parametrize("n,T,dt", [(1000, 0.25, 0.01), (20000, 1.0, 0.004)])
def test_esirkepov_j_fp64_continuity(port, ref, n, T, dt):
    """The FP64 Esirkepov current (the oracle's restatement of Esirkepov, CPC 135
    (2001) 144; the reference has none) conserves charge against the reference's own
    CIC deposit: (rho_CIC(x + v dt) - rho_CIC(x)) / dt + div J = 0 to round-off, on
    the set-up of the reference's moving-charge test (src/main_test.cpp:52-72: a
    Maxwellian in the unit box, 32 x 32 cells)."""
    nx = ny = 32
    p = port.init_particles(0, nx, ny, 1.0, 1.0, n, p0=T, seed=123)
    moved = dict(p, x=p["x"] + p["vx"] * dt, y=p["y"] + p["vy"] * dt)
    r0 = ref.deposit(nx, ny, 1.0, 1.0, CIC, p)
    r1 = ref.deposit(nx, ny, 1.0, 1.0, CIC, moved)
    jx, jy = port.esirkepov_j_ref(nx, ny, 1.0, 1.0, p, dt)
    JX, JY = jx.reshape(ny, nx), jy.reshape(ny, nx)
    dx = dy = 1.0 / nx
    div = (JX - np.roll(JX, 1, axis=1)) / dx + (JY - np.roll(JY, 1, axis=0)) / dy
    res = (r1 - r0).reshape(ny, nx) / dt + div
    scale = np.max(np.abs(r0)) / dt
    assert np.max(np.abs(res)) <= 1e-12 * scale, np.max(np.abs(res)) / scale
    assert np.max(np.abs(div)) > 1e-3 * scale  # the current is not trivially zero


def test_two_stream_tsc_simulation_matches_reference_2000_steps(port, ref, oracle_mod):
    """The oracle's FP64 time loop (the checker of the GPU's two-stream TSC run) against
    the reference's own Simulation::run (src/pic/simulation.cpp:69-145) at the reduced
    size of the large time-step configuration: 64 x 64 cells, 16 particles per cell,
    initializeTwoStream (beams +-0.2, perturbation 0.01; charge -1/N, background 1/V),
    TSC, FFT Poisson, dt 0.05, all 2000 steps. Energies agree to FP64 round-off."""
    nx = ny = 64
    n = nx * ny * 16
    steps, dt = 2000, 0.05
    p = port.init_particles(3, nx, ny, float(nx), float(ny), n, p0=0.2, p1=0.01, seed=17)
    h, _ = oracle_mod.simulate(port, nx, ny, float(nx), float(ny), p, TSC, dt, steps, background=1.0 / (nx * ny))
    r = ref.simulation_run(nx, ny, float(nx), float(ny), dt, steps, TSC, n, seed=17, mode=3, beam_velocity=0.2,
                           perturbation=0.01)
    assert np.allclose(h[:, 5], r["total"], rtol=1e-9, atol=0)
    assert np.allclose(h[:, 3], r["kinetic"], rtol=1e-9, atol=0)
    assert np.allclose(h[:, 4], r["field"], rtol=1e-6, atol=1e-12 * np.max(np.abs(r["field"])))
    drift_port = (h[-1, 5] - h[0, 5]) / abs(h[0, 5])
    drift_ref = (r["total"][-1] - r["total"][0]) / abs(r["total"][0])
    assert abs(drift_port - drift_ref) <= 1e-9


@pytest.mark.parametrize("grid,n", [((20, 12, 2.0, 1.0), 5000), ((256, 256, 256.0, 256.0), 400_000)])
def test_cell_sort_restatement_vs_reference(port, ref, grid, n):
    """The port's restatement of sortParticlesByCell (std::sort of indices by cell
    key, then a gather of the six arrays; the CPU baseline of the sort where the
    reference does not build) orders the particles exactly as the reference does."""
    nx, ny, lx, ly = grid
    p = port.init_particles(0, nx, ny, lx, ly, n, p0=1.0, seed=21)
    a = port.sort_by_cell(nx, ny, lx, ly, p)
    b = ref.sort(nx, ny, lx, ly, p)
    for k in ("x", "y", "vx", "vy", "q", "m"):
        assert np.array_equal(a[k], b[k]), k
