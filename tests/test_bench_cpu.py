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
    assert d["kind"] == "port" and d["sort"]["kind"] == "port" and d["sort"]["particles_per_s"] > 0


def test_detail_with_the_reference(bench_mod, sorted_sample, ref):
    d = bench_mod.cpu_detail(sorted_sample, 2, sample=100_000)
    check_rows(d, 2)
    assert d["kind"] == "reference" and d["sort"]["particles_per_s"] > 0


def test_fp64_errors_and_summary(bench_mod):
    """The error report compares GPU grids with the oracle's FP64 deposits (here the
    oracle's own results stand in for the GPU's: every error is zero), and the
    summary that closes the benchmark line is compact and carries every figure."""
    import oracle

    port = oracle.Port()
    rng = np.random.default_rng(4)
    n = 20_000
    nx = bench_mod.NX
    p = dict(x=rng.random(n) * nx, y=rng.random(n) * nx, vx=rng.normal(0, 0.1, n), vy=rng.normal(0, 0.1, n),
             q=-np.ones(n), m=np.ones(n))
    fake = {nm: port.deposit_ref(nx, nx, float(nx), float(nx), code, p, dt=bench_mod.ESK_DT, threads=2)
            for nm, code in bench_mod.SCHEMES.items()}
    fake["Jx"], fake["Jy"] = port.esirkepov_j_ref(nx, nx, float(nx), float(nx), p, bench_mod.ESK_DT)
    err = bench_mod.fp64_errors(p, fake, 2)
    assert set(err) == {"NGP", "CIC", "TSC", "ESK_rho", "Jx", "Jy", "workload"}
    assert all(err[k]["max_abs"] == 0.0 and err[k]["rel_l2"] == 0.0 for k in err if k != "workload")
    res = {"roofline": {"frac": 0.612345}, "errors_vs_fp64": err,
           "extra": {"CIC_sorted": {"kernel_ms": 0.17812345, "frac": 0.4567891}, "poisson_fft_1024x1024": {"ms": 0.38}},
           "timestep_2048": {"ms_per_step": 18.6, "steps": 2000,
                             "energy_drift_at_steps": {"0": 0.0, "500": 1.23456e-15, "1999": -3e-15}},
           "ensemble": {"ms_per_step": 68.0},
           "gs_warm_start": {"speedup_learned_vs_plain": 4.2, "speedup_extrapolated_vs_plain": 3.3,
                             "speedup_net_vs_extrapolated": 1.28},
           "conv_kernels": {k: {"frac_of_bf16_peak": 0.1} for k in ("conv_fwd", "conv_dgrad", "conv_wgrad")}}
    s = bench_mod.summary(res)
    assert s["kernels"]["CIC_sorted"] == [0.1781, 0.4568] and s["kernels"]["poisson_fft_1024x1024"] == 0.38
    assert s["roofline_frac"] == 0.6123 and s["errors_vs_fp64"]["Jx"] == [0.0, 0.0]
    assert s["timestep_2048"]["drift"]["500"] == 1.235e-15 and s["gs"]["speedup_net_vs_extrapolated"] == 1.28
    import json

    assert len(json.dumps(s)) < 1500
