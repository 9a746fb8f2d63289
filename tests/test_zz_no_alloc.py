"""pic_gpu_deposit_noalloc: the deposit for callers that cannot allocate device
memory (hosts that own the GPU's whole memory budget, or loops that must not
pay cudaMalloc's synchronisation) -- checked against the context-based
pic_gpu_deposit on the same particles, on two calls in a row, through the C ABI.

This file is collected last on purpose: the entry point keeps its scratch in a
fixed device array shared by every call, and the test must pass both alone in
a fresh process and after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NGP, CIC, TSC = 0, 1, 2
REL_L2_TOL = 1e-5  # the tolerance the deposit tests use against the FP64 deposit


class DeviceBuffers:
    """Plain cudaMalloc'd buffers owned by the test (the test itself may allocate)."""

    def __init__(self):
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        self.rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
        self.rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
        self.rt.cudaFree.argtypes = [C.c_void_p]
        self.ptrs = []

    def put(self, a: np.ndarray) -> C.c_void_p:
        a = np.ascontiguousarray(a)
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), max(a.nbytes, 16)) == 0
        if a.nbytes:
            assert self.rt.cudaMemcpy(p, a.ctypes.data_as(C.c_void_p), a.nbytes, 1) == 0  # H2D
        self.ptrs.append(p)
        return p

    def empty(self, nbytes: int) -> C.c_void_p:
        p = C.c_void_p()
        assert self.rt.cudaMalloc(C.byref(p), max(nbytes, 16)) == 0
        self.ptrs.append(p)
        return p

    def get(self, p: C.c_void_p, n: int, dtype) -> np.ndarray:
        out = np.zeros(n, dtype)
        assert self.rt.cudaDeviceSynchronize() == 0
        assert self.rt.cudaMemcpy(out.ctypes.data_as(C.c_void_p), p, out.nbytes, 2) == 0  # D2H
        return out

    def free(self):
        for p in self.ptrs:
            self.rt.cudaFree(p)
        self.ptrs = []


def reference_deposit(pg, nx, ny, lx, ly, p, scheme, background=0.0):
    """The existing entry point: context upload + pic_gpu_deposit (global-atomic path)."""
    with pg.Context(nx, ny, lx, ly, max(len(p["x"]), 1)) as c:
        c.upload(p["x"], p["y"], p["q"])
        c.set_order(pg.ORDER_UNSORTED)
        rho = c.deposit(scheme, 0.0, background)
        lay = c.device_layout()
    return rho, lay


def noalloc_deposit(pg, dev, nx, ny, lx, ly, lay, maxq, scheme, background=0.0):
    n = len(lay["cell"])
    cell, xr, yr, qn = (dev.put(lay[k]) for k in ("cell", "xr", "yr", "q"))
    rho = dev.empty(nx * ny * 8)
    L = pg.lib()
    L.pic_gpu_deposit_noalloc.restype = C.c_int
    L.pic_gpu_deposit_noalloc.argtypes = [C.POINTER(pg._Domain), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_size_t, C.c_float, C.c_double, C.c_void_p, C.c_void_p]
    rc = L.pic_gpu_deposit_noalloc(C.byref(pg._Domain(lx, ly, nx, ny)), scheme, cell, xr, yr, qn, n, maxq,
                                   background, rho, None)
    assert rc == 0, L.pic_gpu_last_error()
    return dev.get(rho, nx * ny, np.float64)


def particles(nx, ny, lx, ly, n, seed):
    rng = np.random.default_rng(seed)
    return dict(x=rng.random(n) * lx, y=rng.random(n) * ly, q=rng.choice([-1.0, 1.0], n) * 0.5)


def test_noalloc_matches_context_deposit_two_calls(pg):
    dev = DeviceBuffers()
    try:
        # first call: the larger grid; later calls: smaller grids, so stale sums
        # left in the shared scratch by an earlier call would show up
        for scheme, (nx, ny, lx, ly), n, seed, bg in ((CIC, (256, 192, 25.6, 19.2), 300_000, 1, 0.0),
                                                     (TSC, (64, 48, 6.4, 4.8), 40_000, 2, 0.0),
                                                     (NGP, (40, 30, 4.0, 3.0), 20_000, 3, 2.5)):
            p = particles(nx, ny, lx, ly, n, seed)
            want, lay = reference_deposit(pg, nx, ny, lx, ly, p, scheme, bg)
            maxq = float(np.max(np.abs(p["q"].astype(np.float32))))
            got = noalloc_deposit(pg, dev, nx, ny, lx, ly, lay, maxq, scheme, bg)
            rel = np.linalg.norm(got - want) / np.linalg.norm(want)
            assert rel <= REL_L2_TOL, rel
            assert np.array_equal(got, want)  # same fixed-point arithmetic: identical
    finally:
        dev.free()


def test_noalloc_skips_keys_outside_the_grid(pg, port):
    """Particles whose cell key is not below Nx*Ny are left out: the result equals the
    existing entry point's deposit of the remaining particles bit for bit, and the
    FP64 deposit of the remaining particles within the tests' tolerance."""
    nx, ny, lx, ly = 50, 40, 5.0, 4.0
    dev = DeviceBuffers()
    try:
        p = particles(nx, ny, lx, ly, 30_000, 4)
        _, lay = reference_deposit(pg, nx, ny, lx, ly, p, CIC)
        bad = np.array([0, 17, 1000, 29_999])
        lay["cell"][bad[:2]] = nx * ny
        lay["cell"][bad[2:]] = 0xFFFFFFFF
        keep = np.setdiff1d(np.arange(len(p["x"])), bad)
        rest = {k: v[keep] for k, v in p.items()}
        maxq = float(np.max(np.abs(p["q"].astype(np.float32))))
        for scheme in (NGP, CIC, TSC):
            got = noalloc_deposit(pg, dev, nx, ny, lx, ly, lay, maxq, scheme)
            want, _ = reference_deposit(pg, nx, ny, lx, ly, rest, scheme)
            assert np.array_equal(got, want), scheme
            ref = port.deposit_ref(nx, ny, lx, ly, scheme, dict(rest, vx=np.zeros(len(keep)), vy=np.zeros(len(keep))))
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= REL_L2_TOL
    finally:
        dev.free()


def test_noalloc_rejects_grid_above_scratch(pg):
    L = pg.lib()
    L.pic_gpu_deposit_noalloc.restype = C.c_int
    L.pic_gpu_deposit_noalloc.argtypes = [C.POINTER(pg._Domain), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_size_t, C.c_float, C.c_double, C.c_void_p, C.c_void_p]
    rc = L.pic_gpu_deposit_noalloc(C.byref(pg._Domain(2048.0, 1024.0, 2048, 1024)), CIC, None, None, None, None, 0,
                                   1.0, 0.0, C.c_void_p(16), None)
    assert rc == -1
    assert b"exceeds the fixed scratch" in L.pic_gpu_last_error()
