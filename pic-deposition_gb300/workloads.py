"""Seeded synthetic particle sets with the shapes of the benchmark configurations.

The reference's benchmark inputs come from its own initialisers
(src/pic/particles_aos.cpp); the larger configurations below are new and are
drawn with numpy's PCG64 generator so that 67M-particle sets take seconds.

  * ``uniform_box``   -- config "1": positions uniform on [0,L)^2, charge -1.
  * ``density_cos``   -- configs "2" and "5": x from density 1 + a*cos(2*pi*x/Lx)
                         by rejection sampling, y uniform, Maxwellian v with
                         thermal speed vth per component, charge -1.
  * ``two_stream``    -- config "3": uniform positions, two equal beams +-v0,
                         thermal spread vth.
All arrays are FP64 (the reference's ParticlesSoA layout), in generation order,
which is random with respect to cells.
"""
from __future__ import annotations

import numpy as np


def uniform_box(nx: int, ny: int, ppc: int, lx: float | None = None, ly: float | None = None, seed: int = 42):
    lx = float(nx) if lx is None else lx
    ly = float(ny) if ly is None else ly
    n = nx * ny * ppc
    rng = np.random.default_rng(seed)
    x = rng.random(n) * lx
    y = rng.random(n) * ly
    return dict(x=x, y=y, vx=np.zeros(n), vy=np.zeros(n), q=-np.ones(n), m=np.ones(n))


def density_cos(nx: int, ny: int, ppc: int, amp: float, vth: float, lx: float | None = None,
                ly: float | None = None, seed: int = 42):
    lx = float(nx) if lx is None else lx
    ly = float(ny) if ly is None else ly
    n = nx * ny * ppc
    rng = np.random.default_rng(seed)
    parts = []
    need = n
    k = 2.0 * np.pi / lx
    while need > 0:
        m = int(need * (1.0 + amp) * 1.02) + 4096
        cand = rng.random(m) * lx
        u = rng.random(m) * (1.0 + amp)
        keep = cand[u < 1.0 + amp * np.cos(k * cand)]
        parts.append(keep[:need])
        need -= len(parts[-1])
    x = np.concatenate(parts)
    y = rng.random(n) * ly
    vx = rng.normal(0.0, vth, n)
    vy = rng.normal(0.0, vth, n)
    return dict(x=x, y=y, vx=vx, vy=vy, q=-np.ones(n), m=np.ones(n))


def two_stream(nx: int, ny: int, ppc: int, v0: float, vth: float, lx: float | None = None,
               ly: float | None = None, seed: int = 42):
    lx = float(nx) if lx is None else lx
    ly = float(ny) if ly is None else ly
    n = nx * ny * ppc
    rng = np.random.default_rng(seed)
    x = rng.random(n) * lx
    y = rng.random(n) * ly
    sign = np.where(np.arange(n) < n // 2, 1.0, -1.0)
    vx = sign * v0 + rng.normal(0.0, vth, n)
    vy = rng.normal(0.0, vth, n)
    return dict(x=x, y=y, vx=vx, vy=vy, q=-np.ones(n), m=np.ones(n))
