"""bench.py's CPU legs without a GPU: the per-scheme, per-thread-count timing of the
reference's CPU deposit and its cell sort (cpu_baseline.detail of the benchmark line),
with the compiled reference and with the port alone (as on a host where the reference
is not built)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench_mod():
    sys.path.insert(0, ROOT)
    import bench

    return bench


@pytest.fixture(scope="module")
def sorted_sample(bench_mod):
    rng = np.random.default_rng(2)
    n = 200_000
    nx = bench_mod.NX
    p = dict(x=rng.random(n) * nx, y=rng.random(n) * nx, vx=rng.normal(0, 0.1, n), vy=rng.normal(0, 0.1, n),
             q=-np.ones(n), m=np.ones(n))
    o = bench_mod.sorted_order(p)
    return {k: v[o] for k, v in p.items()}


def check_rows(d, threads):
    assert d["unit"] == "particles/s" and d["sample_particles"] == 100_000
    for name in ("NGP", "CIC", "Esirkepov"):
        assert set(d["schemes"][name]) == {"threads_1", f"threads_{threads}"}
    assert set(d["schemes"]["TSC"]) == {"threads_1"}
    assert all(v > 0 for row in d["schemes"].values() for v in row.values())


def test_detail_with_the_port_only(bench_mod, sorted_sample, monkeypatch):
    import oracle

    monkeypatch.setattr(oracle.Ref, "available", staticmethod(lambda: False))
    d = bench_mod.cpu_detail(sorted_sample, 2, sample=100_000)
    check_rows(d, 2)
    assert d["kind"] == "port" and "unavailable" in d["sort"]


def test_detail_with_the_reference(bench_mod, sorted_sample, ref):
    d = bench_mod.cpu_detail(sorted_sample, 2, sample=100_000)
    check_rows(d, 2)
    assert d["kind"] == "reference" and d["sort"]["particles_per_s"] > 0
