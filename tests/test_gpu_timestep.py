"""Time stepping (pic_gpu_run) and red-black Gauss-Seidel through the C ABI.

* The step loop against the oracle's FP64 restatement of Simulation::run
  (src/pic/simulation.cpp:82-131): energies within 1e-4 over the first steps
  (the GPU state is FP32 cell-relative, the oracle FP64).
* The sort interval and CUDA-graph replay change no bit of the result (the
  deposit is order independent).
* Langmuir validation (src/pic/validation.cpp:200-261, the set-up of
  src/main_validation.cpp:7-17): the dominant field-energy frequency bin equals
  the reference's archived 0.1220703125 (data/benchmarks/validation.csv:2-5).
* Conservation study set-up (main_validation.cpp:29-36): charge error stays at
  round-off and the energy drift is small.
* RBGS converges to the oracle's red-black solution; a warm start at the
  solution takes no sweep.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NGP, CIC, TSC, ESK = 0, 1, 2, 3


def start(pg, nx, ny, lx, ly, p):
    c = pg.Context(nx, ny, lx, ly, len(p["x"]))
    c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
    return c


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_run_tracks_fp64_oracle(pg, port, oracle_mod, scheme):
    nx = ny = 32
    p = port.init_particles(0, nx, ny, 1.0, 1.0, 4000, p0=1.0, seed=42)
    with start(pg, nx, ny, 1.0, 1.0, p) as c:
        got = c.run(20, scheme=scheme, dt=0.005, sort_interval=5)
    want, _ = oracle_mod.simulate(port, nx, ny, 1.0, 1.0, p, scheme, 0.005, 20)
    for col in (3, 4, 5):  # kinetic, field, total
        rel = np.max(np.abs(got[:, col] - want[:, col]) / np.abs(want[:, col]))
        assert rel <= 1e-4, (col, rel)
    assert np.max(got[:, 0]) <= 1e-12  # charge error (reference test: <= 1e-10)


def test_sort_interval_and_graph_do_not_change_bits(pg, port):
    nx = ny = 64
    p = port.init_particles(0, nx, ny, 1.0, 1.0, 50000, p0=1.0, seed=3)
    outs = []
    for k, graph in ((0, False), (1, False), (7, True), (3, True)):
        with start(pg, nx, ny, 1.0, 1.0, p) as c:
            h = c.run(25, scheme=TSC, dt=0.004, sort_interval=k, use_graph=graph)
            lay = c.device_layout()
        # compare the particle state as a set (order differs with the sort interval)
        key = np.lexsort((lay["vy"], lay["vx"], lay["yr"], lay["xr"], lay["cell"]))
        outs.append((h, {kk: v[key] for kk, v in lay.items()}))
    for h, lay in outs[1:]:
        # particle state and every grid quantity are bit-identical ...
        for kk in lay:
            assert np.array_equal(lay[kk], outs[0][1][kk])
        for col in (0, 1, 2, 4):  # charge error, total charge, integrated rho, field energy
            assert np.array_equal(h[:, col], outs[0][0][:, col])
        # ... the FP64 kinetic-energy sum runs over the particles in their current order
        assert np.allclose(h[:, 3], outs[0][0][:, 3], rtol=1e-13, atol=0)


@pytest.mark.parametrize("scheme", [NGP, CIC, TSC, ESK])
def test_langmuir_frequency_bin(pg, port, oracle_mod, scheme):
    # main_validation.cpp:7-17: 64x64, L=1, dt=0.002, 16384 steps, 200 particles,
    # amplitude 0.05, mode 1; background 1/V (validation.cpp:56-61)
    nx = ny = 64
    steps = 16384
    p = port.init_particles(1, nx, ny, 1.0, 1.0, 200, p0=0.05, mode=1, seed=42)
    with start(pg, nx, ny, 1.0, 1.0, p) as c:
        h = c.run(steps, scheme=scheme, dt=0.002, background=1.0, use_graph=True)
    fe = h[steps // 4:, 4]
    omega = oracle_mod.dominant_frequency(fe, 0.002)
    assert omega == 0.1220703125  # data/benchmarks/validation.csv:2-5


@pytest.mark.parametrize("scheme", [CIC, TSC])
def test_conservation_study_setup(pg, port, scheme):
    # main_validation.cpp:29-36: 64x64, L=1, dt=0.005, 2000 steps, 10000 particles
    p = port.init_particles(0, 64, 64, 1.0, 1.0, 10000, p0=1.0, seed=42)
    with start(pg, 64, 64, 1.0, 1.0, p) as c:
        h = c.run(2000, scheme=scheme, dt=0.005, sort_interval=1, use_graph=True)
    drift = (h[-1, 5] - h[0, 5]) / abs(h[0, 5])
    assert np.max(h[:, 0]) <= 1e-12
    # reference drifts (conservation_study.csv:3-4): CIC -1.8e-6, TSC -1.9e-5
    assert abs(drift) <= 1e-4, drift


def test_kinetic_sum_and_charge_cache(pg, port):
    """The kinetic diagnostic (double-FP32 per thread, FP64 across threads) agrees
    with an FP64 sum over the device's FP32 velocities to 1e-13; the total charge,
    summed once per particle set, follows a new upload of different charges."""
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 50000, p0=2.0, seed=8)
    with start(pg, 32, 32, 1.0, 1.0, p) as c:
        c.deposit(CIC, 0.0, download=False)
        c.poisson_fft()
        d = c.diagnostics()
        lay = c.device_layout()
        ke = 0.5 * np.sum(lay["vx"].astype(np.float64) ** 2 + lay["vy"].astype(np.float64) ** 2)
        assert abs(d["kinetic_energy"] - ke) <= 1e-13 * ke
        assert d["total_charge"] == pytest.approx(np.sum(p["q"]), rel=1e-6)
        h = c.run(3, scheme=CIC, dt=0.002)
        q2 = np.where(np.arange(len(p["q"])) % 3 == 0, 2.0, -1.0) * abs(p["q"][0])
        c.upload(p["x"], p["y"], q2, p["vx"], p["vy"], p["m"])
        h2 = c.run(3, scheme=CIC, dt=0.002)
    assert h[0, 1] == pytest.approx(np.sum(p["q"]), rel=1e-6)
    assert h2[0, 1] == pytest.approx(np.sum(q2), rel=1e-6) and h2[0, 1] != h[0, 1]


def test_sort_by_moved_fraction(pg, port):
    """Sorts triggered by the measured disorder (pic_run_config.sort_moved_fraction)
    give the fixed interval's particles and grid quantities bit for bit; a lower
    threshold sorts more often; an out-of-range threshold is rejected."""
    nx = ny = 64
    p = port.init_particles(0, nx, ny, 1.0, 1.0, 50000, p0=1.0, seed=3)
    outs, sorts = [], {}
    for k, f, graph in ((3, 0.0, True), (0, 0.05, True), (0, 0.95, False), (8, 0.6, True)):
        with start(pg, nx, ny, 1.0, 1.0, p) as c:
            n0 = c.sort_count()
            h = c.run(30, scheme=TSC, dt=0.004, sort_interval=k, use_graph=graph, sort_moved_fraction=f)
            sorts[(k, f)] = c.sort_count() - n0
            lay = c.device_layout()
            if f == 0.95:
                with pytest.raises(pg.PicError) as e:
                    c.run(2, scheme=TSC, dt=0.004, sort_moved_fraction=1.5)
                assert e.value.code == -1
        key = np.lexsort((lay["vy"], lay["vx"], lay["yr"], lay["xr"], lay["cell"]))
        outs.append((h, {kk: v[key] for kk, v in lay.items()}))
    for h, lay in outs[1:]:
        for kk in lay:
            assert np.array_equal(lay[kk], outs[0][1][kk])
        for col in (0, 1, 2, 4):
            assert np.array_equal(h[:, col], outs[0][0][:, col])
        assert np.allclose(h[:, 3], outs[0][0][:, 3], rtol=1e-13, atol=0)
    assert sorts[(3, 0.0)] == 10
    assert sorts[(0, 0.05)] > sorts[(0, 0.95)] >= 1
    assert sorts[(8, 0.6)] >= 30 // 8


@pytest.mark.parametrize("scheme", [CIC, TSC])
def test_hot_plasma_switches_to_any_order_between_sorts(pg, port, scheme):
    """Particles fast enough (about 0.7 cells per step and axis) that most leave
    their cell every step: after the first deposit between sorts
    finds most of them out of their cell, the following deposits take the
    any-order kernel (a choice made on the device) until the next sort. The run
    gives the particles and the energy history of the run that sorts every step
    bit for bit (kinetic energy to 1e-13), with and without graphs."""
    nx = ny = 64
    p = port.init_particles(0, nx, ny, 1.0, 1.0, 40000, p0=8.0, seed=5)
    outs = []
    for k, graph in ((1, False), (10, True), (10, False)):
        with start(pg, nx, ny, 1.0, 1.0, p) as c:
            h = c.run(25, scheme=scheme, dt=0.004, sort_interval=k, use_graph=graph)
            lay = c.device_layout()
        key = np.lexsort((lay["vy"], lay["vx"], lay["yr"], lay["xr"], lay["cell"]))
        outs.append((h, {kk: v[key] for kk, v in lay.items()}))
    for h, lay in outs[1:]:
        for kk in lay:
            assert np.array_equal(lay[kk], outs[0][1][kk])
        for col in (0, 1, 2, 4):
            assert np.array_equal(h[:, col], outs[0][0][:, col])
        assert np.allclose(h[:, 3], outs[0][0][:, 3], rtol=1e-13, atol=0)


def test_rbgs_matches_oracle(pg, port):
    nx, ny = 64, 48
    rng = np.random.default_rng(0)
    rho = rng.normal(size=nx * ny)
    with pg.Context(nx, ny, 6.4, 4.8, 1) as c:
        c.set_rho(rho)
        it, res = c.poisson_rbgs(tol=1e-10, max_iters=200000, warm_start=False, check_every=50)
        phi, ex, ey = c.fields()
        it2, res2 = c.poisson_rbgs(tol=1e-10, warm_start=True, check_every=50)
    assert res <= 1e-10 and it > 0
    assert it2 == 0 and res2 <= 1e-10
    want, wit, wres = port.rbgs(nx, ny, 6.4, 4.8, rho, tol=1e-10, max_iters=200000, check_every=50)
    assert abs(it - wit) <= 50
    assert np.max(np.abs(phi - want)) <= 1e-8 * np.max(np.abs(want))
    wex, wey = port.efield(nx, ny, 6.4, 4.8, phi)
    assert np.array_equal(ex, wex) and np.array_equal(ey, wey)


def test_rbgs_fixed_sweeps_close_to_oracle(pg, port):
    nx, ny = 32, 32
    rng = np.random.default_rng(1)
    rho = rng.normal(size=nx * ny)
    with pg.Context(nx, ny, 1.0, 1.0, 1) as c:
        c.set_rho(rho)
        it, _ = c.poisson_rbgs(tol=0.0, max_iters=37, warm_start=False, check_every=1000)
        phi, _, _ = c.fields()
    want, wit, _ = port.rbgs(nx, ny, 1.0, 1.0, rho, tol=0.0, max_iters=37, check_every=1000)
    assert it == wit == 37
    # same arithmetic per sweep; the mean of the right-hand side is summed in another order
    assert np.max(np.abs(phi - want)) <= 1e-12 * np.max(np.abs(want))


@pytest.mark.parametrize("nx,ny", [(64, 48), (512, 512), (16, 8)])
def test_rbgs_one_launch_equals_per_colour_launches(pg, nx, ny):
    """The one-launch solve (even check_every and max_iters) and the per-colour
    launches (odd check_every) give the same phi bit for bit after the same sweeps."""
    rng = np.random.default_rng(2)
    rho = rng.normal(size=nx * ny)
    out = []
    for check_every in (40, 5):
        with pg.Context(nx, ny, 1.0, 1.0, 1) as c:
            c.set_rho(rho)
            it, _ = c.poisson_rbgs(tol=0.0, max_iters=40, warm_start=False, check_every=check_every)
            out.append((it, c.fields()[0]))
    assert out[0][0] == out[1][0] == 40
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("nx,ny", [(512, 512), (64, 48)])
def test_rbgs_mixed_precision_meets_the_same_fp64_test(pg, nx, ny):
    """FP32 sweeps on FP64-refined corrections stop on the same FP64 relative
    residual and give the FP64 solve's answer to within that tolerance."""
    rng = np.random.default_rng(4)
    rho = rng.normal(size=nx * ny)
    out = []
    for mixed in (False, True):
        with pg.Context(nx, ny, float(nx), float(ny), 1) as c:
            c.set_rho(rho)
            c.set_rbgs_precision(mixed)
            it, res = c.poisson_rbgs(tol=1e-10, max_iters=2_000_000, warm_start=False, check_every=16)
            out.append((it, res, c.fields()[0]))
    (it0, r0, p0), (it1, r1, p1) = out
    assert r0 <= 1e-10 and r1 <= 1e-10
    assert it1 <= 1.5 * it0 + 64
    assert np.max(np.abs(p1 - p0)) <= 1e-6 * np.max(np.abs(p0))


@pytest.mark.parametrize("absent", [5, 0])
def test_rbgs_barrier_timeout_reported_and_context_usable(pg, port, absent):
    """One CTA of the one-launch solve leaves before its first grid barrier:
    every other CTA's wait runs out after 1 ms and returns, the call reports
    PIC_ERR_TIMEOUT, and the same context then solves and deposits exactly as a
    fresh one does."""
    nx, ny = 512, 512  # 64x32 tiles: 128 CTAs in one cooperative launch
    rng = np.random.default_rng(5)
    rho = rng.normal(size=nx * ny)
    p = port.init_particles(0, nx, ny, 1.0, 1.0, 20000, p0=1.0, seed=9)
    out = []
    for fault in (False, True):
        with pg.Context(nx, ny, 1.0, 1.0, len(p["x"])) as c:
            c.set_rho(rho)
            if fault:
                c.test_rbgs_barrier_timeout(-1, 1.0)  # nobody absent: completes
                with pytest.raises(pg.PicError) as e:
                    c.test_rbgs_barrier_timeout(absent, 1.0)
                assert e.value.code == -7 and "timed out" in str(e.value)
            it, _ = c.poisson_rbgs(tol=0.0, max_iters=40, warm_start=False, check_every=40)
            phi = c.fields()[0]
            c.upload(p["x"], p["y"], p["q"])
            rho_dep = c.deposit(CIC)
            out.append((it, phi, rho_dep))
    assert out[0][0] == out[1][0] == 40
    assert np.array_equal(out[0][1], out[1][1])
    assert np.array_equal(out[0][2], out[1][2])


def test_rbgs_odd_grid_rejected(pg):
    with pg.Context(33, 32, 1.0, 1.0, 1) as c:
        c.set_rho(np.zeros(33 * 32))
        with pytest.raises(pg.PicError) as e:
            c.poisson_rbgs()
        assert e.value.code == -8


def test_run_with_rbgs_poisson(pg, port):
    p = port.init_particles(0, 32, 32, 1.0, 1.0, 3000, p0=1.0, seed=5)
    with start(pg, 32, 32, 1.0, 1.0, p) as c:
        h_fft = c.run(5, scheme=CIC, dt=0.005)
    with start(pg, 32, 32, 1.0, 1.0, p) as c:
        h_gs = c.run(5, scheme=CIC, dt=0.005, poisson=1, rbgs_tol=1e-12, rbgs_max_iters=200000)
    # FFT uses the continuous k^2, GS the 5-point Laplacian: same physics, different discretisation
    assert np.allclose(h_gs[:, 3], h_fft[:, 3], rtol=1e-3)
