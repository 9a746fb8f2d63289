"""Device-side particle generation (pic_gpu_generate) and the two-stream time step
of the large configuration at a reduced size.

* Generated particles are in exactly the layout an upload of the same FP64
  positions produces (the conversion is the upload's).
* Their statistics are the requested ones (beams, thermal spread, density mode).
* The two-stream set-up (ParticlesSoA::initializeTwoStream conventions: charge
  -1/N, m = 1, background 1/V) advanced with TSC, a cell sort every 10 steps and
  the FFT solve tracks the oracle's FP64 restatement of Simulation::run
  (src/pic/simulation.cpp:82-131; pinned to the reference's own Simulation::run
  over 2000 steps in test_oracle.py) within 1e-5 in total energy over all 2000
  steps of the large configuration, at 64 x 64 cells.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TSC = 2


def test_generated_layout_equals_upload(pg):
    nx, ny, n = 128, 64, 200_000
    with pg.Context(nx, ny, 12.8, 6.4, n) as a, pg.Context(nx, ny, 12.8, 6.4, n) as b:
        a.generate(n, amplitude=0.1, mode=2, vth=0.3, v0=0.5, charge=-2.5, mass=3.0, seed=9)
        p = a.download()
        b.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        la, lb = a.device_layout(), b.device_layout()
    for k in ("cell", "xr", "yr", "vx", "vy", "q"):
        assert np.array_equal(la[k], lb[k]), k
    assert np.all(p["q"] == -2.5) and np.allclose(p["m"], 3.0)


def test_generated_statistics(pg):
    nx = ny = 256
    n = 2_000_000
    with pg.Context(nx, ny, float(nx), float(ny), n) as c:
        c.generate(n, amplitude=0.05, mode=1, vth=0.01, v0=0.2, seed=3)
        p = c.download()
    h = n // 2
    assert abs(p["vx"][:h].mean() - 0.2) < 1e-4 and abs(p["vx"][h:].mean() + 0.2) < 1e-4
    assert abs(p["vx"][:h].std() - 0.01) < 2e-4 and abs(p["vy"].std() - 0.01) < 2e-4
    # density mode 1 in x: <cos(2 pi x / L)> = amplitude / 2
    m = np.mean(np.cos(2 * np.pi * p["x"] / nx))
    assert abs(m - 0.025) < 3e-3
    assert p["x"].min() >= 0 and p["x"].max() < nx and p["y"].min() >= 0 and p["y"].max() < ny


def test_two_stream_tsc_tracks_fp64_oracle(pg, port, oracle_mod):
    nx = ny = 64
    n = nx * ny * 16
    steps, dt = 2000, 0.05
    with pg.Context(nx, ny, float(nx), float(ny), n) as c:
        c.generate(n, vth=0.01, v0=0.2, charge=-1.0 / n, mass=1.0, seed=5)
        p = c.download()
        got = c.run(steps, scheme=TSC, dt=dt, background=1.0 / (nx * ny), sort_interval=10, use_graph=True)
    want, _ = oracle_mod.simulate(port, nx, ny, float(nx), float(ny), p, TSC, dt, steps,
                                  background=1.0 / (nx * ny))
    rel = np.max(np.abs(got[:, 5] - want[:, 5]) / np.abs(want[:, 5]))
    assert rel <= 1e-5, rel
    # the energy-drift series at the marks the benchmark reports
    for k in (0, 500, 1000, 1500, steps - 1):
        drift_gpu = (got[k, 5] - got[0, 5]) / abs(got[0, 5])
        drift_ref = (want[k, 5] - want[0, 5]) / abs(want[0, 5])
        assert abs(drift_gpu - drift_ref) <= 1e-5, (k, drift_gpu, drift_ref)
