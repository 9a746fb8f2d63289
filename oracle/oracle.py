"""CPU oracle for the GB300 PIC deposition path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
legs may import this module, and only as the checker or the timed CPU
baseline; the product never does.

Two backends:
  * ``Port``  -- ctypes over ``oracle/liboracle.so``, this project's C
    restatement of the reference algorithms (pic_oracle.c, each function
    citing the reference file:line) plus the exact restatement of the GPU
    fixed-point arithmetic. Builds anywhere (``make -C oracle port``).
  * ``Ref``   -- ctypes over ``oracle/_ref/libpicref.so``, the reference's own
    sources compiled by ``make -C oracle ref`` (only where the reference
    checkout exists).

FFT-based pieces are restated in numpy:
  * ``spectral_noise``   -- diagnostics.cpp:53-102 (FFTW R2HC x R2HC power ratio)
  * ``poisson_fft``      -- poisson_fft.cpp:23-35,45-94 (continuous k^2, DC=0)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libpicref.so")


def reference_src() -> str | None:
    """The reference checkout, or None where it is absent: $PIC_REFERENCE_SRC when
    set, else the location the build recipe (oracle/Makefile, `make print-ref`) names."""
    path = os.environ.get("PIC_REFERENCE_SRC")
    if not path:
        r = subprocess.run(["make", "-s", "-C", HERE, "print-ref"], capture_output=True, text=True)
        path = r.stdout.strip() if r.returncode == 0 else ""
    return path if path and os.path.isdir(path) else None

NGP, CIC, TSC, ESIRKEPOV = 0, 1, 2, 3

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


class _Domain(C.Structure):
    _fields_ = [("Lx", C.c_double), ("Ly", C.c_double), ("Nx", C.c_int32), ("Ny", C.c_int32)]


def build(ref: bool | None = None) -> None:
    """Compile the port (always) and the reference library (when the reference checkout is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    src = reference_src()
    if ref is None:
        ref = src is not None
    if ref:
        if src is None:
            raise RuntimeError("the reference checkout is absent: set PIC_REFERENCE_SRC")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={src}"], check=True)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


class Port:
    """The project's C restatement (liboracle.so)."""

    def __init__(self, path: str = PORT_LIB):
        if not os.path.exists(path):
            build(ref=False)
        L = C.CDLL(path)
        self.lib = L
        D = C.POINTER(_Domain)
        L.orc_init_particles.argtypes = [C.c_int, D, C.c_size_t, C.c_double, C.c_double, C.c_int, C.c_uint32,
                                         _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_particle_cell_index.argtypes = [D, C.c_double, C.c_double]
        L.orc_deposit_ref.argtypes = [D, C.c_int, C.c_size_t, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, _dp]
        L.orc_sort_particles_by_cell.argtypes = [D, C.c_size_t, _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_deposit_timed.argtypes = [D, C.c_int, C.c_size_t, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                        C.c_int, _dp, C.POINTER(C.c_double)]
        L.orc_stable_cell_sort.argtypes = [D, C.c_size_t, _dp, _dp, _u32p, _u32p, _u32p]
        L.orc_stable_sort_keys.argtypes = [C.c_size_t, C.c_uint32, _u32p, _u32p, _u32p, _u32p]
        L.orc_gather_ref.argtypes = [D, C.c_size_t, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double]
        L.orc_push_ref.argtypes = [D, C.c_size_t, _dp, _dp, _dp, _dp, C.c_double]
        L.orc_gs_ref.argtypes = [D, _dp, C.c_int, C.c_double, _dp, _dp, _dp]
        L.orc_efield.argtypes = [D, _dp, _dp, _dp]
        L.orc_rbgs.argtypes = [D, _dp, _dp, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int),
                               C.POINTER(C.c_double)]
        L.orc_rbgs_residual.argtypes = [D, _dp, _dp]
        L.orc_rbgs_residual.restype = C.c_double
        for f in ("orc_integrated_rho",):
            getattr(L, f).argtypes = [D, _dp]
            getattr(L, f).restype = C.c_double
        L.orc_field_energy.argtypes = [D, _dp, _dp]
        L.orc_field_energy.restype = C.c_double
        L.orc_to_device.argtypes = [D, C.c_size_t, _dp, _dp, _u32p, _fp, _fp]
        L.orc_normalize_charge.argtypes = [C.c_size_t, _dp, _fp, C.POINTER(C.c_float)]
        L.orc_charge_uniform.argtypes = [C.c_size_t, _fp]
        L.orc_charge_uniform.restype = C.c_int
        L.orc_deposit_fixed.argtypes = [D, C.c_int, C.c_size_t, _u32p, _fp, _fp, _fp, _fp, _fp, C.c_float, C.c_double,
                                        _i64p, C.POINTER(C.c_double)]
        L.orc_fixed_to_rho.argtypes = [C.c_size_t, _i64p, C.c_double, C.c_double, _dp]
        L.orc_esirkepov_j_ref.argtypes = [D, C.c_size_t, _dp, _dp, _dp, _dp, _dp, C.c_double, _dp, _dp]
        L.orc_esirkepov_j_fixed.argtypes = [D, C.c_size_t, _u32p, _fp, _fp, _fp, _fp, _fp, C.c_float, C.c_double,
                                            _i64p, _i64p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_move_f32.argtypes = [D, C.c_size_t, _u32p, _fp, _fp, _fp, _fp, _fp, C.c_float, C.c_void_p, _dp, _dp,
                                   C.c_double, C.c_int, C.c_int]

        _u16p = np.ctypeslib.ndpointer(dtype=np.uint16, flags="C_CONTIGUOUS")
        L.orc_conv3x3_fwd.argtypes = [C.c_int] * 5 + [_u16p, _fp, _fp, C.c_int, C.c_void_p]
        L.orc_conv3x3_dgrad.argtypes = [C.c_int] * 5 + [_u16p, _fp, _u16p, _u16p]
        L.orc_conv3x3_wgrad.argtypes = [C.c_int] * 5 + [_u16p, _u16p, _dp, _dp]
        L.orc_net_param_count.restype = C.c_size_t
        L.orc_net_loss_grad.argtypes = [C.c_int] * 3 + [_fp, _fp, _fp, C.c_int, C.POINTER(C.c_double), _dp]
        L.orc_bf16_from_float.argtypes = [C.c_float]
        L.orc_bf16_from_float.restype = C.c_uint16

    # ---- the warm-start network (nn_oracle.c) ----
    @staticmethod
    def bf16(a):
        """Float array -> BF16 bit patterns (round to nearest even)."""
        u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
        r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
        return r

    @staticmethod
    def from_bf16(h):
        return (np.ascontiguousarray(h, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)

    def conv_fwd(self, x, w, bias, relu=True):
        B, H, W, cin = x.shape
        cout = w.shape[1]
        out = np.zeros((B, H, W, cout), np.uint16) if relu else np.zeros((B, H, W), np.float32)
        self.lib.orc_conv3x3_fwd(B, H, W, cin, cout, _c(x, np.uint16), _c(w, np.float32), _c(bias, np.float32),
                                 0 if relu else 1, out.ctypes.data_as(C.c_void_p))
        return out

    def conv_dgrad(self, dy, w, mask):
        B, H, W, cout = dy.shape
        cin = w.shape[2]
        out = np.zeros((B, H, W, cin), np.uint16)
        self.lib.orc_conv3x3_dgrad(B, H, W, cin, cout, _c(dy, np.uint16), _c(w, np.float32), _c(mask, np.uint16),
                                   out)
        return out

    def conv_wgrad(self, x, dy):
        B, H, W, cin = x.shape
        cout = dy.shape[3]
        dw = np.zeros(9 * cout * cin)
        db = np.zeros(cout)
        self.lib.orc_conv3x3_wgrad(B, H, W, cin, cout, _c(x, np.uint16), _c(dy, np.uint16), dw, db)
        return dw.reshape(9, cout, cin), db

    def net_param_count(self):
        return int(self.lib.orc_net_param_count())

    def net_loss_grad(self, params, inp, target, quantize=True):
        B, H, W = inp.shape
        grad = np.zeros(self.net_param_count())
        loss = C.c_double()
        self.lib.orc_net_loss_grad(B, H, W, _c(params, np.float32), _c(inp, np.float32), _c(target, np.float32),
                                   1 if quantize else 0, C.byref(loss), grad)
        return loss.value, grad

    @staticmethod
    def dom(nx, ny, lx, ly):
        return C.byref(_Domain(float(lx), float(ly), int(nx), int(ny)))

    # ---- reference restatements ----
    def init_particles(self, kind, nx, ny, lx, ly, n, p0=1.0, p1=0.0, mode=1, seed=42):
        out = [np.zeros(n) for _ in range(6)]
        rc = self.lib.orc_init_particles(kind, self.dom(nx, ny, lx, ly), n, p0, p1, mode, seed, *out)
        assert rc == 0
        return dict(zip(("x", "y", "vx", "vy", "q", "m"), out))

    def cell_index(self, nx, ny, lx, ly, x, y):
        return self.lib.orc_particle_cell_index(self.dom(nx, ny, lx, ly), x, y)

    def deposit_ref(self, nx, ny, lx, ly, scheme, p, dt=0.0, threads=1):
        rho = np.zeros(nx * ny)
        n = len(p["x"])
        vx = p.get("vx", np.zeros(n))
        vy = p.get("vy", np.zeros(n))
        rc = self.lib.orc_deposit_ref(self.dom(nx, ny, lx, ly), scheme, n, _c(p["x"], np.float64),
                                      _c(p["y"], np.float64), _c(vx, np.float64), _c(vy, np.float64),
                                      _c(p["q"], np.float64), dt, threads, rho)
        assert rc == 0
        return rho

    def deposit_timed(self, nx, ny, lx, ly, scheme, p, dt=0.0, threads=1, warmups=3, repeats=5):
        """Mean ms of `repeats` deposits after `warmups` untimed ones, timed inside the
        library as the reference's depositChargeTimedSoA times its deposits."""
        n = len(p["x"])
        vx = p.get("vx", np.zeros(n))
        vy = p.get("vy", np.zeros(n))
        rho = np.zeros(nx * ny)
        ms = C.c_double(0)
        rc = self.lib.orc_deposit_timed(self.dom(nx, ny, lx, ly), scheme, n, _c(p["x"], np.float64),
                                        _c(p["y"], np.float64), _c(vx, np.float64), _c(vy, np.float64),
                                        _c(p["q"], np.float64), dt, threads, warmups, repeats, rho, C.byref(ms))
        assert rc == 0
        return ms.value

    def sort_by_cell(self, nx, ny, lx, ly, p):
        """The reference's sortParticlesByCell restated (std::sort of an index array by
        cell key, then a gather of x, y, vx, vy, q, m): a sorted copy of `p`."""
        out = {k: _c(p[k], np.float64).copy() for k in ("x", "y", "vx", "vy", "q", "m")}
        rc = self.lib.orc_sort_particles_by_cell(self.dom(nx, ny, lx, ly), len(out["x"]), out["x"], out["y"],
                                                 out["vx"], out["vy"], out["q"], out["m"])
        assert rc == 0
        return out

    def stable_cell_sort(self, nx, ny, lx, ly, x, y):
        n = len(x)
        keys = np.zeros(n, np.uint32)
        perm = np.zeros(n, np.uint32)
        offs = np.zeros(nx * ny + 1, np.uint32)
        rc = self.lib.orc_stable_cell_sort(self.dom(nx, ny, lx, ly), n, _c(x, np.float64), _c(y, np.float64), keys,
                                           perm, offs)
        assert rc == 0
        return keys, perm, offs

    def stable_sort_keys(self, keys, nkeys):
        keys = _c(keys, np.uint32)
        n = len(keys)
        ks = np.zeros(n, np.uint32)
        perm = np.zeros(n, np.uint32)
        offs = np.zeros(nkeys + 1, np.uint32)
        rc = self.lib.orc_stable_sort_keys(n, nkeys, keys, ks, perm, offs)
        assert rc == 0
        return ks, perm, offs

    def gather_ref(self, nx, ny, lx, ly, p, ex, ey, dt):
        vx = _c(p["vx"], np.float64).copy()
        vy = _c(p["vy"], np.float64).copy()
        n = len(vx)
        m = p.get("m", np.ones(n))
        self.lib.orc_gather_ref(self.dom(nx, ny, lx, ly), n, _c(p["x"], np.float64), _c(p["y"], np.float64), vx, vy,
                                _c(p["q"], np.float64), _c(m, np.float64), _c(ex, np.float64), _c(ey, np.float64), dt)
        return vx, vy

    def push_ref(self, nx, ny, lx, ly, p, dt):
        x = _c(p["x"], np.float64).copy()
        y = _c(p["y"], np.float64).copy()
        self.lib.orc_push_ref(self.dom(nx, ny, lx, ly), len(x), x, y, _c(p["vx"], np.float64),
                              _c(p["vy"], np.float64), dt)
        return x, y

    def gs_ref(self, nx, ny, lx, ly, rho, max_iters=500, tol=1e-6):
        phi, ex, ey = np.zeros(nx * ny), np.zeros(nx * ny), np.zeros(nx * ny)
        it = self.lib.orc_gs_ref(self.dom(nx, ny, lx, ly), _c(rho, np.float64), max_iters, tol, phi, ex, ey)
        return phi, ex, ey, it

    def efield(self, nx, ny, lx, ly, phi):
        ex, ey = np.zeros(nx * ny), np.zeros(nx * ny)
        self.lib.orc_efield(self.dom(nx, ny, lx, ly), _c(phi, np.float64), ex, ey)
        return ex, ey

    def rbgs(self, nx, ny, lx, ly, rho, phi0=None, tol=1e-8, max_iters=100000, check_every=1):
        phi = np.zeros(nx * ny) if phi0 is None else _c(phi0, np.float64).copy()
        it = C.c_int(0)
        res = C.c_double(0)
        rc = self.lib.orc_rbgs(self.dom(nx, ny, lx, ly), _c(rho, np.float64), phi, tol, max_iters, check_every,
                               C.byref(it), C.byref(res))
        assert rc == 0
        return phi, it.value, res.value

    def rbgs_residual(self, nx, ny, lx, ly, b, phi):
        return self.lib.orc_rbgs_residual(self.dom(nx, ny, lx, ly), _c(b, np.float64), _c(phi, np.float64))

    def integrated_rho(self, nx, ny, lx, ly, rho):
        return self.lib.orc_integrated_rho(self.dom(nx, ny, lx, ly), _c(rho, np.float64))

    def field_energy(self, nx, ny, lx, ly, ex, ey):
        return self.lib.orc_field_energy(self.dom(nx, ny, lx, ly), _c(ex, np.float64), _c(ey, np.float64))

    # ---- GPU-arithmetic restatements ----
    def to_device(self, nx, ny, lx, ly, x, y):
        n = len(x)
        cell = np.zeros(n, np.uint32)
        xr = np.zeros(n, np.float32)
        yr = np.zeros(n, np.float32)
        self.lib.orc_to_device(self.dom(nx, ny, lx, ly), n, _c(x, np.float64), _c(y, np.float64), cell, xr, yr)
        return cell, xr, yr

    def normalize_charge(self, q):
        """(qn, maxq): the device's normalised FP32 charge and max |(float)q|."""
        q = _c(q, np.float64)
        qn = np.zeros(len(q), np.float32)
        mq = C.c_float(0)
        self.lib.orc_normalize_charge(len(q), q, qn, C.byref(mq))
        return qn, mq.value

    def charge_uniform(self, qn) -> bool:
        """True when every stored charge equals the first, nonzero and finite (the device's upload test)."""
        qn = _c(qn, np.float32)
        return bool(self.lib.orc_charge_uniform(len(qn), qn))

    def fixed_total(self, scheme, qn) -> int:
        """The exact int64 total of a deposit's grid: every particle deposits rint(qn * 2^24)
        units, or 2^30 units in the exact integer TSC form (one charge for all particles)."""
        if scheme == TSC and self.charge_uniform(qn):
            return len(qn) << 30
        return int(np.sum(np.rint(np.asarray(qn, np.float64) * 2 ** 24)))

    def deposit_fixed(self, nx, ny, lx, ly, scheme, cell, xr, yr, qn, maxq, vx32=None, vy32=None, dt=0.0):
        n = len(cell)
        if vx32 is None:
            vx32 = np.zeros(n, np.float32)
        if vy32 is None:
            vy32 = np.zeros(n, np.float32)
        acc = np.zeros(nx * ny, np.int64)
        unit = C.c_double(0)
        rc = self.lib.orc_deposit_fixed(self.dom(nx, ny, lx, ly), scheme, n, _c(cell, np.uint32), _c(xr, np.float32),
                                        _c(yr, np.float32), _c(vx32, np.float32), _c(vy32, np.float32),
                                        _c(qn, np.float32), float(maxq), dt, acc, C.byref(unit))
        assert rc == 0
        return acc, unit.value

    def esirkepov_j_ref(self, nx, ny, lx, ly, p, dt):
        """FP64 Esirkepov (CIC shape) current: (Jx, Jy) at the x / y cell edges."""
        jx, jy = np.zeros(nx * ny), np.zeros(nx * ny)
        rc = self.lib.orc_esirkepov_j_ref(self.dom(nx, ny, lx, ly), len(p["x"]), _c(p["x"], np.float64),
                                          _c(p["y"], np.float64), _c(p["vx"], np.float64), _c(p["vy"], np.float64),
                                          _c(p["q"], np.float64), dt, jx, jy)
        assert rc == 0, "Courant violated"
        return jx, jy

    def esirkepov_j_fixed(self, nx, ny, lx, ly, lay, maxq, dt):
        """The GPU's integer current on the device layout: (jx, jy, unit_x, unit_y)."""
        jx, jy = np.zeros(nx * ny, np.int64), np.zeros(nx * ny, np.int64)
        ux, uy = C.c_double(), C.c_double()
        rc = self.lib.orc_esirkepov_j_fixed(self.dom(nx, ny, lx, ly), len(lay["cell"]), _c(lay["cell"], np.uint32),
                                            _c(lay["xr"], np.float32), _c(lay["yr"], np.float32),
                                            _c(lay["vx"], np.float32), _c(lay["vy"], np.float32),
                                            _c(lay["q"], np.float32), float(maxq), dt, jx, jy, C.byref(ux), C.byref(uy))
        assert rc == 0, "Courant violated"
        return jx, jy, ux.value, uy.value

    def move_f32(self, nx, ny, lx, ly, lay, maxq, ex, ey, dt, gather=True, push=True, m=None):
        """The GPU's FP32 gather/push on a copy of the device layout `lay`."""
        out = {k: _c(lay[k], np.uint32 if k == "cell" else np.float32).copy() for k in ("cell", "xr", "yr", "vx", "vy")}
        mm = None if m is None else _c(m, np.float32)
        self.lib.orc_move_f32(self.dom(nx, ny, lx, ly), len(out["cell"]), out["cell"], out["xr"], out["yr"], out["vx"],
                              out["vy"], _c(lay["q"], np.float32), float(maxq),
                              None if mm is None else mm.ctypes.data_as(C.c_void_p), _c(ex, np.float64),
                              _c(ey, np.float64), dt, int(gather), int(push))
        return out

    @staticmethod
    def fixed_to_rho(acc, unit, background=0.0):
        return acc.astype(np.float64) * unit + background


class Ref:
    """The reference's own sources (oracle/_ref/libpicref.so)."""

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_LIB)

    def __init__(self, path: str = REF_LIB):
        L = C.CDLL(path)
        self.lib = L
        L.ref_init_particles.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_size_t, C.c_double,
                                         C.c_double, C.c_int, C.c_uint, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_cell_index.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        L.ref_deposit.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double,
                                  C.c_size_t, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_deposit_timed.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int,
                                        C.c_double, C.c_int, C.c_size_t, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_sort.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_size_t, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_gather.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_size_t, _dp, _dp, _dp, _dp, _dp, _dp,
                                 _dp, _dp, C.c_double]
        L.ref_push.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_size_t, _dp, _dp, _dp, _dp, C.c_double]
        L.ref_poisson_gs.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_double, _dp, _dp,
                                     _dp]
        L.ref_poisson_fft.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _dp]
        L.ref_spectral_noise.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp]
        L.ref_spectral_noise.restype = C.c_double
        L.ref_simulation_run.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                         C.c_int, C.c_size_t, C.c_uint, C.c_int, C.c_double, C.c_double, C.c_int,
                                         C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp,
                                         C.POINTER(C.c_double)]
        L.ref_langmuir_validation.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                              C.c_size_t, C.c_double, C.c_int, _dp]

    def init_particles(self, kind, nx, ny, lx, ly, n, p0=1.0, p1=0.0, mode=1, seed=42):
        out = [np.zeros(n) for _ in range(6)]
        rc = self.lib.ref_init_particles(kind, nx, ny, lx, ly, n, p0, p1, mode, seed, *out)
        assert rc == 0
        return dict(zip(("x", "y", "vx", "vy", "q", "m"), out))

    def deposit(self, nx, ny, lx, ly, scheme, p, dt=0.0, sorted_=False, threads=1):
        rho = np.zeros(nx * ny)
        n = len(p["x"])
        vx = p.get("vx", np.zeros(n))
        vy = p.get("vy", np.zeros(n))
        m = p.get("m", np.ones(n))
        rc = self.lib.ref_deposit(nx, ny, lx, ly, scheme, int(sorted_), threads, dt, n, _c(p["x"], np.float64),
                                  _c(p["y"], np.float64), _c(vx, np.float64), _c(vy, np.float64),
                                  _c(p["q"], np.float64), _c(m, np.float64), rho)
        assert rc == 0
        return rho

    def deposit_timed(self, nx, ny, lx, ly, scheme, p, dt=0.0, sorted_=False, threads=1, repeats=5):
        st = np.zeros(6)
        n = len(p["x"])
        rc = self.lib.ref_deposit_timed(nx, ny, lx, ly, scheme, int(sorted_), threads, dt, repeats, n,
                                        _c(p["x"], np.float64), _c(p["y"], np.float64), _c(p["vx"], np.float64),
                                        _c(p["vy"], np.float64), _c(p["q"], np.float64), _c(p["m"], np.float64), st)
        assert rc == 0
        return dict(zip(("sort_ms", "deposit_ms", "deposit_std_ms", "throughput", "bandwidth_gbs", "charge_error"),
                        st.tolist()))

    def sort(self, nx, ny, lx, ly, p):
        arrs = [_c(p[k], np.float64).copy() for k in ("x", "y", "vx", "vy", "q", "m")]
        rc = self.lib.ref_sort(nx, ny, lx, ly, len(arrs[0]), *arrs)
        assert rc == 0
        return dict(zip(("x", "y", "vx", "vy", "q", "m"), arrs))

    def gather(self, nx, ny, lx, ly, p, ex, ey, dt):
        vx = _c(p["vx"], np.float64).copy()
        vy = _c(p["vy"], np.float64).copy()
        self.lib.ref_gather(nx, ny, lx, ly, len(vx), _c(p["x"], np.float64), _c(p["y"], np.float64), vx, vy,
                            _c(p["q"], np.float64), _c(p["m"], np.float64), _c(ex, np.float64),
                            _c(ey, np.float64), dt)
        return vx, vy

    def push(self, nx, ny, lx, ly, p, dt):
        x = _c(p["x"], np.float64).copy()
        y = _c(p["y"], np.float64).copy()
        self.lib.ref_push(nx, ny, lx, ly, len(x), x, y, _c(p["vx"], np.float64), _c(p["vy"], np.float64), dt)
        return x, y

    def poisson_gs(self, nx, ny, lx, ly, rho, max_iters=500, tol=1e-6):
        out = [np.zeros(nx * ny) for _ in range(3)]
        self.lib.ref_poisson_gs(nx, ny, lx, ly, _c(rho, np.float64), max_iters, tol, *out)
        return tuple(out)

    def poisson_fft(self, nx, ny, lx, ly, rho):
        out = [np.zeros(nx * ny) for _ in range(3)]
        self.lib.ref_poisson_fft(nx, ny, lx, ly, _c(rho, np.float64), *out)
        return tuple(out)

    def spectral_noise(self, nx, ny, lx, ly, rho):
        return self.lib.ref_spectral_noise(nx, ny, lx, ly, _c(rho, np.float64))

    def simulation_run(self, nx, ny, lx, ly, dt, steps, scheme, n, seed=42, mode=0, temperature=1.0,
                       amplitude=0.01, mode_number=1, landau_temperature=0.1, beam_velocity=0.3,
                       perturbation=0.01, sorted_=False, poisson_gs=False):
        te, ke, fe, ce = (np.zeros(steps) for _ in range(4))
        drift = C.c_double(0)
        rc = self.lib.ref_simulation_run(nx, ny, lx, ly, dt, steps, scheme, int(poisson_gs), n, seed, mode,
                                         temperature, amplitude, mode_number, landau_temperature, beam_velocity,
                                         perturbation, int(sorted_), te, ke, fe, ce, C.byref(drift))
        assert rc == 0
        return dict(total=te, kinetic=ke, field=fe, charge_error=ce, drift=drift.value)

    def langmuir_validation(self, nx, ny, lx, ly, dt, steps, scheme, n, amplitude=0.01, mode_number=1):
        out = np.zeros(5)
        rc = self.lib.ref_langmuir_validation(nx, ny, lx, ly, dt, steps, scheme, n, amplitude, mode_number, out)
        assert rc == 0
        return dict(zip(("omega_theory", "omega_measured", "relative_error", "omega_ratio", "amplitude_decay"),
                        out.tolist()))


# ---------------------------------------------------------------------------
# numpy restatements of the FFT-based reference pieces
# ---------------------------------------------------------------------------
def _r2hc_1d(a: np.ndarray, axis: int) -> np.ndarray:
    """FFTW R2HC along ``axis``: Re X_k at k <= n/2, Im X_k at n-k for 0 < k < (n+1)/2."""
    n = a.shape[axis]
    X = np.fft.fft(a, axis=axis)
    out = np.empty_like(a, dtype=np.float64)
    idx = [slice(None)] * a.ndim

    def put(k_dst, vals):
        idx[axis] = k_dst
        out[tuple(idx)] = vals

    def take(k):
        idx[axis] = k
        return X[tuple(idx)]

    for k in range(0, n // 2 + 1):
        put(k, take(k).real)
    for k in range(1, (n + 1) // 2):
        put(n - k, take(k).imag)
    return out


def spectral_noise(nx: int, ny: int, rho: np.ndarray) -> float:
    """spectralNoiseLevel, src/pic/diagnostics.cpp:53-102: high-k fraction of the
    R2HC x R2HC power of rho, cut at kx >= nx/3 or ky >= ny/3."""
    a = np.asarray(rho, np.float64).reshape(ny, nx)
    out = _r2hc_1d(_r2hc_1d(a, 1), 0)
    power = out * out
    kcx = max(1, nx // 3)
    kcy = max(1, ny // 3)
    i = np.arange(nx)
    j = np.arange(ny)
    kx = np.where(i <= nx // 2, i, nx - i)
    ky = np.where(j <= ny // 2, j, ny - j)
    high = (kx[None, :] >= kcx) | (ky[:, None] >= kcy)
    total = power.sum()
    if total <= 1e-30:
        return 0.0
    return float(power[high].sum() / total)


def simulate(port: "Port", nx, ny, lx, ly, p, scheme, dt, steps, background=0.0, record_field_from=0):
    """pic::Simulation::run's loop (src/pic/simulation.cpp:82-131) in FP64 over
    the port, with the FFT Poisson solve: NGP/CIC/TSC push -> deposit ->
    background -> solve -> gather; Esirkepov deposit -> background -> solve ->
    push -> gather. Returns (history (steps, 6) in pic_diag order, particles)."""
    p = {k: np.array(v, dtype=np.float64, copy=True) for k, v in p.items()}
    n = len(p["x"])
    p.setdefault("m", np.ones(n))
    hist = np.zeros((steps, 6))
    vol = (lx / nx) * (ly / ny)
    qsum, qabs = p["q"].sum(), np.abs(p["q"]).sum()
    for s in range(steps):
        if scheme != ESIRKEPOV:
            p["x"], p["y"] = port.push_ref(nx, ny, lx, ly, p, dt)
        rho = port.deposit_ref(nx, ny, lx, ly, scheme, p, dt=dt) + background
        phi, ex, ey = poisson_fft(nx, ny, lx, ly, rho)
        if scheme == ESIRKEPOV:
            p["x"], p["y"] = port.push_ref(nx, ny, lx, ly, p, dt)
        p["vx"], p["vy"] = port.gather_ref(nx, ny, lx, ly, p, ex, ey, dt)
        ke = float(np.sum(0.5 * p["m"] * (p["vx"] ** 2 + p["vy"] ** 2)))
        fe = 0.5 * float(np.sum(ex * ex + ey * ey)) * vol
        ir = float(rho.sum()) * vol
        hist[s] = (abs(ir - qsum) / max(qabs, 1e-12), qsum, ir, ke, fe, ke + fe)
    return hist, p


def dominant_frequency(signal, dt):
    """estimateDominantFrequency, src/pic/validation.cpp:19-54: the k = 1..n/2-1
    DFT bin of largest power of the mean-removed signal, returned as k/(n*dt)."""
    x = np.asarray(signal, dtype=np.float64)
    n = len(x)
    if n < 8:
        return 0.0
    c = x - x.mean()
    t = np.arange(n)
    best_p, best_k = 0.0, 1
    for k in range(1, n // 2):
        ph = 2.0 * np.pi * (k * t) / n
        re = np.sum(c * np.cos(ph))
        im = -np.sum(c * np.sin(ph))
        pw = re * re + im * im
        if pw > best_p:
            best_p, best_k = pw, k
    return best_k / (n * dt)


def poisson_fft(nx: int, ny: int, lx: float, ly: float, rho: np.ndarray):
    """PoissonSolverFFT::solve, src/pic/poisson_fft.cpp:45-94: phi_hat =
    (rho*dV)_hat / k^2 with continuous k = 2*pi*m/L, DC set to 0, then the
    forward-difference E. Returns (phi, Ex, Ey) flattened."""
    dx, dy = lx / nx, ly / ny
    a = np.asarray(rho, np.float64).reshape(ny, nx) * (dx * dy)
    F = np.fft.fft2(a)
    i = np.arange(nx)
    j = np.arange(ny)
    kx = 2.0 * np.pi * np.where(i <= nx // 2, i, i - nx) / lx
    ky = 2.0 * np.pi * np.where(j <= ny // 2, j, j - ny) / ly
    k2 = kx[None, :] ** 2 + ky[:, None] ** 2
    k2[0, 0] = 1.0
    F = F / k2
    F[0, 0] = 0.0
    phi = np.fft.ifft2(F).real
    ex = -(np.roll(phi, -1, axis=1) - phi) / dx
    ey = -(np.roll(phi, -1, axis=0) - phi) / dy
    return phi.ravel(), ex.ravel(), ey.ravel()
