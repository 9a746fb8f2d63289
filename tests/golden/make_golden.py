"""Generates the golden fixtures in this folder from the reference itself.

Run where the reference checkout exists (it compiles oracle/_ref from the
reference's own sources, see oracle/Makefile):

    python tests/golden/make_golden.py

Fixtures (all produced by the reference's code through oracle/_ref):
  small_32.npz     -- src/main_test.cpp:25-72 setup: 32x32 grid, Lx=Ly=1, 1000
                      particles from initializeUniformMaxwellian(T=1, seed=123).
                      Particle arrays, particleCellIndex keys, the reference's
                      (unstable) sorted arrays, rho for every scheme at
                      esirkepov_dt 0 and 0.01, GS and FFT Poisson of the CIC rho
                      made neutral.
  config1_cic.npz  -- 256x256, dx=1 (Lx=Ly=256), 1,048,576 particles: positions
                      from the reference's initializeUniformMaxwellian(T=1,
                      seed=42), charge -1 each; checksums and a strided sample
                      of the reference's FP64 CIC rho (no background).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402


def main():
    oracle.build(ref=True)
    R = oracle.Ref()
    out = {}
    p = R.init_particles(0, 32, 32, 1.0, 1.0, 1000, p0=1.0, seed=123)
    for k, v in p.items():
        out[k] = v
    import ctypes

    out["keys"] = np.array([R.lib.ref_cell_index(32, 32, 1.0, 1.0, ctypes.c_double(x), ctypes.c_double(y))
                            for x, y in zip(p["x"], p["y"])], np.int32)
    s = R.sort(32, 32, 1.0, 1.0, p)
    for k, v in s.items():
        out["sorted_" + k] = v
    for scheme in range(4):
        for dt in (0.0, 0.01):
            out[f"rho_s{scheme}_dt{dt}"] = R.deposit(32, 32, 1.0, 1.0, scheme, p, dt=dt)
    rho = R.deposit(32, 32, 1.0, 1.0, 1, p)
    rho_n = rho - rho.mean()
    out["poisson_rho"] = rho_n
    phi, ex, ey = R.poisson_gs(32, 32, 1.0, 1.0, rho_n, 500, 1e-6)
    out["gs_phi"], out["gs_ex"], out["gs_ey"] = phi, ex, ey
    phi, ex, ey = R.poisson_fft(32, 32, 1.0, 1.0, rho_n)
    out["fft_phi"], out["fft_ex"], out["fft_ey"] = phi, ex, ey
    np.savez_compressed(os.path.join(HERE, "small_32.npz"), **out)

    n = 1 << 20
    p = R.init_particles(0, 256, 256, 256.0, 256.0, n, p0=1.0, seed=42)
    p["q"] = -np.ones(n)
    rho = R.deposit(256, 256, 256.0, 256.0, 1, p)
    np.savez_compressed(os.path.join(HERE, "config1_cic.npz"), sum=np.array(rho.sum()),
                        sumsq=np.array((rho * rho).sum()), sample=rho[::997].copy(),
                        x_head=p["x"][:64].copy(), y_head=p["y"][:64].copy())
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
