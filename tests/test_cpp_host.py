"""The C++ host interface (pic_gb300_host.hpp: the reference's pic:: hot-path API
over the C ABI) driven by a C++ program written like the reference's
src/main_test.cpp.

CPU: the program builds against the header, and its particle initialisers give
bit-for-bit the particles of the oracle's initialisers (which test_oracle.py pins
to the reference's ParticlesSoA::initialize*, particles_aos.cpp:67-180).
GPU: the program's checks pass, and rho from pic::depositChargeSoA equals the
oracle's fixed-point deposit of the same particles bit for bit.
"""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pic-deposition_gb300")
LIBDIR = os.path.join(PKG, "lib")
SRC = os.path.join(ROOT, "tests", "cpp", "main_test_gb300.cpp")
EXE = os.path.join(LIBDIR, "main_test_gb300")

INIT_KINDS = {"maxwellian": (0, 0.7, 0.0, 1), "langmuir": (1, 0.01, 0.0, 2), "warm": (2, 0.05, 0.1, 1),
              "twostream": (3, 0.3, 0.01, 1), "quasi1d": (4, 0.3, 0.01, 1)}
SCHEMES = {"NGP": 0, "CIC": 1, "TSC": 2, "Esirkepov": 3}


@pytest.fixture(scope="module")
def exe():
    import build_lib

    build_lib.build()
    hdr = os.path.join(PKG, "host", "pic_gb300_host.hpp")
    if build_lib._stale(EXE, [SRC, hdr, build_lib.HOSTLIB]):
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(PKG, "host"), SRC, "-o", EXE, "-L" + LIBDIR, "-lpicgb300_host",
                        "-lpicgb300", "-Wl,-rpath," + LIBDIR], check=True)
    return EXE


def read_dump(path, with_rho):
    raw = np.fromfile(path, dtype=np.uint8)
    n, nx, ny = (int(v) for v in raw[:24].view(np.uint64))
    body = raw[24:].view(np.float64)
    cols = {k: body[i * n:(i + 1) * n] for i, k in enumerate(("x", "y", "vx", "vy", "q", "m"))}
    rho = body[6 * n:6 * n + nx * ny] if with_rho else None
    return n, nx, ny, cols, rho


@pytest.mark.parametrize("kind", sorted(INIT_KINDS))
def test_initialisers_match_oracle(exe, port, tmp_path, kind):
    out = str(tmp_path / f"{kind}.bin")
    subprocess.run([exe, "init", kind, out], check=True)
    n, nx, ny, got, _ = read_dump(out, False)
    code, p0, p1, mode = INIT_KINDS[kind]
    want = port.init_particles(code, nx, ny, 2.0, 1.5, n, p0=p0, p1=p1, mode=mode, seed=42)
    for k in ("x", "y", "vx", "vy", "q", "m"):
        assert np.array_equal(got[k], want[k]), k


def test_wrong_sizes_are_rejected_before_device_work(exe):
    r = subprocess.run([exe, "sizes"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "PASS sizes" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_main_test_program(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    lines = r.stdout.splitlines()
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stderr
    assert sum(ln.startswith("PASS") for ln in lines) >= 28, r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", sorted(SCHEMES))
def test_deposit_matches_oracle(exe, port, tmp_path, scheme):
    out = str(tmp_path / f"dep_{scheme}.bin")
    subprocess.run([exe, "deposit", scheme, out], check=True, timeout=120)
    n, nx, ny, p, rho = read_dump(out, True)
    dt = 0.001 if scheme == "Esirkepov" else 0.0
    lx = ly = 1.0  # pic::Domain defaults
    cell, xr, yr = port.to_device(nx, ny, lx, ly, p["x"], p["y"])
    qn, maxq = port.normalize_charge(p["q"])
    acc, unit = port.deposit_fixed(nx, ny, lx, ly, SCHEMES[scheme], cell, xr, yr, qn, maxq,
                                   p["vx"].astype(np.float32), p["vy"].astype(np.float32), dt)
    assert np.array_equal(rho, acc.astype(np.float64) * unit)
    ref = port.deposit_ref(nx, ny, lx, ly, SCHEMES[scheme], p, dt=dt)
    assert np.linalg.norm(rho - ref) <= 1e-5 * np.linalg.norm(ref)
