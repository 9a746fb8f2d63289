"""Python host binding of the GB300 PIC deposition path (ctypes over libpicgb300.so).

Two layers:
  * ``Context`` -- a thin wrapper of the C ABI in include/pic_gb300.h: device-
    resident particles and grid, explicit upload / sort / deposit / download.
  * Mirrors of the reference's interface (ehocine/pic-deposition,
    src/deposition/deposition.hpp, src/pic/*.hpp): ``Domain``, ``ParticlesSoA``,
    ``FieldGrid``, ``DepositionConfig``, ``DepositionScheme``,
    ``DepositionBackend`` and the free functions ``depositChargeSoA``,
    ``sortParticlesByCell``, ``particleCellIndex`` with the same names, argument
    meaning and error behaviour (RuntimeError where the reference throws
    std::runtime_error). The backend value ``DepositionBackend.GB300`` selects
    this library; the reference's CPU and GPU backends are not part of it.

There is no CPU fallback: importing works anywhere, but every call needs the
compiled library and a CUDA device and raises if either is missing.
"""
from __future__ import annotations

import ctypes as C
import enum
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpicgb300.so")

PIC_OK = 0
ERRORS = {
    -1: "PIC_ERR_ARG", -2: "PIC_ERR_CUDA", -3: "PIC_ERR_NOMEM", -4: "PIC_ERR_STATE", -5: "PIC_ERR_OVERFLOW",
    -6: "PIC_ERR_COURANT", -7: "PIC_ERR_TIMEOUT", -8: "PIC_ERR_UNSUPPORTED", -9: "PIC_ERR_DEVICE",
}
ORDER_AUTO, ORDER_SORTED, ORDER_UNSORTED, ORDER_ATOMIC = 0, 1, 2, 3


class PicError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Domain(C.Structure):
    _fields_ = [("Lx", C.c_double), ("Ly", C.c_double), ("Nx", C.c_int32), ("Ny", C.c_int32)]


class _Diag(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("charge_error", "total_charge", "integrated_rho", "kinetic_energy",
                                           "field_energy", "total_energy")]


_lib = None

# (name, restype, argtypes); restype None means int status.
_vp = C.c_void_p
_dp = C.POINTER(C.c_double)
_SIGS = [
    ("pic_gpu_create", [C.POINTER(_Domain), C.c_size_t, C.c_int, C.POINTER(_vp)]),
    ("pic_gpu_destroy", [_vp]),
    ("pic_gpu_synchronize", [_vp]),
    ("pic_gpu_launch_count", [_vp, C.POINTER(C.c_longlong)]),
    ("pic_gpu_get_stream", [_vp, C.POINTER(_vp)]),
    ("pic_gpu_upload_particles", [_vp, _vp, _vp, _vp, _vp, _vp, _vp, C.c_size_t]),
    ("pic_gpu_download_particles", [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("pic_gpu_download_device_layout", [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    ("pic_gpu_num_particles", [_vp, C.POINTER(C.c_size_t)]),
    ("pic_gpu_sort", [_vp, _vp, _vp, _vp]),
    ("pic_gpu_set_deposit_order", [_vp, C.c_int]),
    ("pic_gpu_set_tile", [_vp, C.c_int, C.c_int]),
    ("pic_gpu_deposit", [_vp, C.c_int, C.c_double, C.c_double, _vp]),
    ("pic_gpu_get_rho_fixed", [_vp, _vp, _dp]),
    ("pic_gpu_get_rho", [_vp, _vp]),
    ("pic_gpu_is_sorted", [_vp, C.POINTER(C.c_int)]),
    ("pic_gpu_charge_uniform", [_vp, C.POINTER(C.c_float)]),
    ("pic_gpu_profile_enable", [_vp, C.c_int]),
    ("pic_gpu_profile_read", [_vp, C.c_char_p, _dp, C.POINTER(C.c_longlong)]),
    ("pic_gpu_host_alloc", [C.c_size_t, C.POINTER(_vp)]),
    ("pic_gpu_host_free", [_vp]),
    ("pic_gpu_set_rho", [_vp, _vp]),
    ("pic_gpu_set_fields", [_vp, _vp, _vp, _vp]),
    ("pic_gpu_get_fields", [_vp, _vp, _vp, _vp]),
    ("pic_gpu_poisson_fft", [_vp]),
    ("pic_gpu_gather", [_vp, C.c_double]),
    ("pic_gpu_push", [_vp, C.c_double]),
    ("pic_gpu_gather_push", [_vp, C.c_double]),
    ("pic_gpu_diagnostics", [_vp, C.POINTER(_Diag)]),
    ("pic_gpu_poisson_rbgs", [_vp, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), _dp]),
]


class RunConfig(C.Structure):
    """pic_run_config (include/pic_gb300.h)."""
    _fields_ = [("scheme", C.c_int), ("poisson", C.c_int), ("dt", C.c_double), ("background", C.c_double),
                ("sort_interval", C.c_int), ("use_graph", C.c_int), ("rbgs_tol", C.c_double),
                ("rbgs_max_iters", C.c_int), ("rbgs_check_every", C.c_int), ("rbgs_warm", C.c_int),
                ("sort_moved_fraction", C.c_double)]


_SIGS.append(("pic_gpu_run", [_vp, C.POINTER(RunConfig), C.c_int, C.POINTER(_Diag)]))
_SIGS.append(("pic_gpu_sort_count", [_vp, C.POINTER(C.c_longlong)]))
_SIGS.append(("pic_gpu_deposit_current", [_vp, C.c_double, _vp, _vp]))
_SIGS.append(("pic_gpu_get_current_fixed", [_vp, _vp, _vp, _dp, _dp]))
_SIGS.append(("pic_nn_conv3x3", [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp, _vp]))

NN_FWD_RELU, NN_FWD_OUT, NN_DGRAD, NN_WGRAD = 0, 1, 2, 3


class WsStats(C.Structure):
    """pic_ws_stats (include/pic_gb300.h): one step of the warm-start study."""
    _fields_ = [("iters", C.c_int * 3), ("ms", C.c_double * 3), ("resid", C.c_double * 3),
                ("guess_resid", C.c_double * 3), ("phi_diff", C.c_double)]


_fp = C.POINTER(C.c_float)
_SIGS += [
    ("pic_gpu_ws_init", [_vp, C.c_uint, C.c_size_t]),
    ("pic_gpu_ws_get_params", [_vp, _vp, C.c_size_t]),
    ("pic_gpu_ws_set_params", [_vp, _vp, C.c_size_t]),
    ("pic_gpu_ws_generate", [_vp, C.c_int, C.c_double, C.c_double, C.c_int]),
    ("pic_gpu_ws_dataset_size", [_vp, C.POINTER(C.c_size_t)]),
    ("pic_gpu_ws_train", [_vp, C.c_int, C.c_int, C.c_float, C.c_uint, _vp]),
    ("pic_gpu_ws_loss_grad", [_vp, C.c_int, _vp, _vp, _dp, _vp]),
    ("pic_gpu_ws_predict", [_vp, _vp, _vp]),
    ("pic_gpu_ws_study", [_vp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                          C.POINTER(WsStats)]),
]


def partition_members(runs, world_size: int):
    """Ensemble members split over `world_size` ranks, balanced by particle count.

    The reference's multi-seed sweep (src/pic/physics_studies.cpp:479-560) runs
    its members one after another; here each rank runs a share of them as one
    batched ensemble on its own GPU. Largest members first, each to the rank with
    the fewest particles so far (lowest rank on ties). Returns one ascending list
    of member indices per rank: every member appears exactly once.
    """
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    load = [0] * world_size
    parts = [[] for _ in range(world_size)]
    sizes = [int(n) * int(n) * int(p) for n, p, _ in runs]
    for i in sorted(range(len(runs)), key=lambda i: (-sizes[i], i)):
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += sizes[i]
    return [sorted(p) for p in parts]


def run_ensemble_ranks(runs, steps: int, rank: int = 0, world_size: int = 1, ensemble=None, **cfg):
    """This rank's share of an ensemble (partition_members), advanced `steps` steps.

    A member's run depends only on its own (N, ppc, seed) and the shared
    configuration, so the share runs as its own batched ensemble. The one
    exchange is a final gather of the per-member energy histories to rank 0
    (torch.distributed.gather_object on the initialised process group). Returns
    (field_energy, kinetic_energy), each (steps, len(runs)) in the order of
    `runs`, on rank 0, and None on the other ranks. `ensemble` builds the
    batch (default: Ensemble) and takes (members, **cfg).
    """
    make = ensemble or Ensemble
    mine = partition_members(runs, world_size)[rank]
    fe = ke = np.zeros((steps, 0))
    if mine:
        with make([runs[i] for i in mine], **cfg) as e:
            fe, ke = e.run_member_order(steps)
    part = (mine, np.asarray(fe), np.asarray(ke))
    if world_size > 1:
        import torch.distributed as dist

        got = [None] * world_size if rank == 0 else None
        dist.gather_object(part, got, dst=0)
        if rank != 0:
            return None
    else:
        got = [part]
    out_fe = np.full((steps, len(runs)), np.nan)
    out_ke = np.full((steps, len(runs)), np.nan)
    seen = np.zeros(len(runs), np.int64)
    for idx, f, k in got:
        for j, i in enumerate(idx):
            out_fe[:, i] = f[:, j]
            out_ke[:, i] = k[:, j]
            seen[i] += 1
    if not np.all(seen == 1):
        raise RuntimeError("ensemble ranks: the gathered members do not cover every run exactly once")
    return out_fe, out_ke


def nn_conv3x3(op: int, x: np.ndarray, weight=None, bias=None, aux=None, cin: int = 32, cout: int = 32):
    """One tensor-core convolution layer on host arrays (pic_nn_conv3x3).

    x and aux are uint16 BF16 bit patterns shaped (B, H, W, C); weight is FP32
    (9, cout, cin), bias FP32 (cout,). Returns BF16 bits (B, H, W, C) for ops 0
    and 2, FP32 (B, H, W) for op 1 and (dw (9, cout, cin), db (cout,)) for op 3.
    """
    if np.ndim(x) < 3:
        raise ValueError("x: expected (B, H, W, C)")
    B, H, W = np.shape(x)[:3]
    px = B * H * W
    # channels of x and aux per op (the C side reads these sizes through plain pointers)
    xc, ac = {NN_FWD_RELU: (cin, 0), NN_FWD_OUT: (cin, 0), NN_DGRAD: (cout, cin), NN_WGRAD: (cin, cout)}.get(op, (cin, 0))
    x = _sized(x, np.uint16, px * xc, "x")
    ptr = lambda a: None if a is None else a.ctypes.data_as(_vp)
    w = None if op == NN_WGRAD else _sized(weight, np.float32, 9 * cout * cin, "weight")
    b = _sized(bias, np.float32, cout, "bias") if op in (NN_FWD_RELU, NN_FWD_OUT) else None
    a = _sized(aux, np.uint16, px * ac, "aux") if ac else None
    if op == NN_FWD_RELU:
        out = np.zeros((B, H, W, cout), np.uint16)
    elif op == NN_FWD_OUT:
        out = np.zeros((B, H, W), np.float32)
    elif op == NN_DGRAD:
        out = np.zeros((B, H, W, cin), np.uint16)
    else:
        out = np.zeros(9 * cout * cin + cout, np.float32)
    _check(lib().pic_nn_conv3x3(op, B, H, W, cin, cout, ptr(x), ptr(w), ptr(b), ptr(a), ptr(out)))
    if op == NN_WGRAD:
        return out[:9 * cout * cin].reshape(9, cout, cin), out[9 * cout * cin:]
    return out


class GenConfig(C.Structure):
    """pic_gen_config (include/pic_gb300.h)."""
    _fields_ = [("n", C.c_size_t), ("amplitude", C.c_double), ("mode", C.c_int), ("vth", C.c_double),
                ("v0", C.c_double), ("charge", C.c_double), ("mass", C.c_double), ("seed", C.c_uint)]


_SIGS.append(("pic_gpu_generate", [_vp, C.POINTER(GenConfig)]))
_SIGS.append(("pic_gpu_set_rbgs_precision", [_vp, C.c_int]))
_SIGS.append(("pic_gpu_test_rbgs_barrier_timeout", [_vp, C.c_int, C.c_double]))


class EnsMember(C.Structure):
    _fields_ = [("N", C.c_int), ("ppc", C.c_int), ("seed", C.c_uint)]


class EnsConfig(C.Structure):
    _fields_ = [("dt", C.c_double), ("amplitude", C.c_double), ("vth", C.c_double), ("sort_interval", C.c_int),
                ("use_graph", C.c_int), ("seed", C.c_uint), ("sort_disorder", C.c_double)]


class EnsRunInfo(C.Structure):
    _fields_ = [("N", C.c_int), ("ppc", C.c_int), ("particles", C.c_size_t), ("tile_w", C.c_int),
                ("tile_h", C.c_int)]


_SIGS += [
    ("pic_ens_create", [C.POINTER(EnsMember), C.c_int, C.POINTER(EnsConfig), C.c_int, C.POINTER(_vp)]),
    ("pic_ens_destroy", [_vp]),
    ("pic_ens_run", [_vp, C.c_int, _vp, _vp]),
    ("pic_ens_num_runs", [_vp, C.POINTER(C.c_int)]),
    ("pic_ens_info", [_vp, C.c_int, C.POINTER(EnsRunInfo)]),
    ("pic_ens_launch_count", [_vp, C.POINTER(C.c_longlong)]),
    ("pic_ens_sort_count", [_vp, C.POINTER(C.c_longlong)]),
    ("pic_ens_get_stream", [_vp, C.POINTER(_vp)]),
    ("pic_ens_download_run", [_vp, C.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
]


class Ensemble:
    """A batch of independent Langmuir runs (pic_ens_*). `runs`: list of (N, ppc, seed).
    Runs are reordered by grid size; info(r) gives run r's setup in that order."""

    def __init__(self, runs, dt=0.1, amplitude=0.01, vth=0.05, sort_interval=20, use_graph=True, seed=1,
                 device=0, sort_disorder=0.0):
        arr = (EnsMember * len(runs))(*[EnsMember(int(n), int(p), int(s)) for n, p, s in runs])
        cfg = EnsConfig(float(dt), float(amplitude), float(vth), int(sort_interval), int(use_graph), int(seed),
                        float(sort_disorder))
        h = _vp()
        _check(lib().pic_ens_create(arr, len(runs), C.byref(cfg), int(device), C.byref(h)))
        self.h = h
        self.nruns = len(runs)
        # the library's order: a stable sort of the runs by grid size
        self.order = sorted(range(len(runs)), key=lambda i: int(runs[i][0]))

    def close(self):
        if self.h:
            lib().pic_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def run(self, steps):
        fe = np.zeros((max(steps, 1), self.nruns))
        ke = np.zeros((max(steps, 1), self.nruns))
        _check(lib().pic_ens_run(self.h, int(steps), _ptr(fe), _ptr(ke)))
        return fe[:steps], ke[:steps]

    def run_member_order(self, steps):
        """run(steps) with the columns put back in the order of the `runs` given."""
        fe, ke = self.run(steps)
        back = np.empty(self.nruns, np.int64)
        back[self.order] = np.arange(self.nruns)
        return fe[:, back], ke[:, back]

    def info(self, r):
        i = EnsRunInfo()
        _check(lib().pic_ens_info(self.h, int(r), C.byref(i)))
        return {"N": i.N, "ppc": i.ppc, "particles": i.particles, "tile": (i.tile_w, i.tile_h)}

    def launch_count(self):
        n = C.c_longlong()
        _check(lib().pic_ens_launch_count(self.h, C.byref(n)))
        return n.value

    def sort_count(self):
        """Cell sorts the ensemble has done (pic_ens_sort_count)."""
        n = C.c_longlong()
        _check(lib().pic_ens_sort_count(self.h, C.byref(n)))
        return n.value

    def stream(self):
        s = _vp()
        _check(lib().pic_ens_get_stream(self.h, C.byref(s)))
        return s.value or 0

    def download_run(self, r):
        inf = self.info(r)
        n, g = inf["particles"], inf["N"] ** 2
        out = {k: np.zeros(n) for k in ("x", "y", "vx", "vy")}
        rho, phi = np.zeros(g), np.zeros(g)
        _check(lib().pic_ens_download_run(self.h, int(r), _ptr(out["x"]), _ptr(out["y"]), _ptr(out["vx"]),
                                          _ptr(out["vy"]), _ptr(rho), _ptr(phi)))
        out["rho"], out["phi"] = rho, phi
        return out


class PinnedArray:
    """A page-locked host buffer (pic_gpu_host_alloc) viewed as a numpy array."""

    def __init__(self, n: int, dtype=np.float64):
        dtype = np.dtype(dtype)
        p = _vp()
        _check(lib().pic_gpu_host_alloc(max(n, 1) * dtype.itemsize, C.byref(p)))
        self._p = p
        buf = (C.c_char * (max(n, 1) * dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=n)

    def free(self):
        if self._p:
            self.array = None
            lib().pic_gpu_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def lib():
    """Loads libpicgb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(LIB_PATH)
        L.pic_gpu_last_error.restype = C.c_char_p
        L.pic_gpu_last_error.argtypes = []
        for name, args in _SIGS:
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = C.c_int
            f.argtypes = args
        _lib = L
    return _lib


def _check(rc: int):
    if rc != PIC_OK:
        raise PicError(rc, lib().pic_gpu_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _arr(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


def _sized(a, dt, n: int, what: str):
    """Contiguous `dt` copy of `a` that holds exactly n values (the C side reads n through a
    plain pointer, so a shorter array would be read past its end); None stays None."""
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=dt)
    if a.size != n:
        raise ValueError(f"{what}: expected {n} values, got {a.size}")
    return a


class Context:
    """Device-resident particles and grid on one GPU (C ABI pic_ctx)."""

    def __init__(self, nx: int, ny: int, lx: float, ly: float, capacity: int, device: int = 0):
        self.nx, self.ny, self.lx, self.ly = int(nx), int(ny), float(lx), float(ly)
        self.G = self.nx * self.ny
        self.capacity = int(capacity)
        h = _vp()
        _check(lib().pic_gpu_create(C.byref(_Domain(self.lx, self.ly, self.nx, self.ny)), self.capacity, device,
                                    C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().pic_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- particles ----
    def upload(self, x, y, q, vx=None, vy=None, m=None):
        n = int(np.size(x))
        arrs = [_sized(a, np.float64, n, name) for a, name in zip((x, y, vx, vy, q, m), ("x", "y", "vx", "vy", "q", "m"))]
        self._keep = arrs
        _check(lib().pic_gpu_upload_particles(self.h, *[_ptr(a) for a in arrs], n))
        self.n = n

    def num_particles(self) -> int:
        n = C.c_size_t()
        _check(lib().pic_gpu_num_particles(self.h, C.byref(n)))
        return n.value

    def download(self):
        n = self.num_particles()
        out = [np.zeros(n) for _ in range(6)]
        _check(lib().pic_gpu_download_particles(self.h, *[_ptr(a) for a in out]))
        return dict(zip(("x", "y", "vx", "vy", "q", "m"), out))

    def device_layout(self):
        n = self.num_particles()
        cell = np.zeros(n, np.uint32)
        f = [np.zeros(n, np.float32) for _ in range(5)]
        _check(lib().pic_gpu_download_device_layout(self.h, _ptr(cell), *[_ptr(a) for a in f]))
        return dict(cell=cell, xr=f[0], yr=f[1], vx=f[2], vy=f[3], q=f[4])

    # ---- sort ----
    def sort(self, keys=False, perm=False, offsets=False):
        n = self.num_particles()
        k = np.zeros(n, np.uint32) if keys else None
        p = np.zeros(n, np.uint32) if perm else None
        o = np.zeros(self.G + 1, np.uint32) if offsets else None
        _check(lib().pic_gpu_sort(self.h, _ptr(k), _ptr(p), _ptr(o)))
        return k, p, o

    # ---- deposit ----
    def set_order(self, mode: int):
        _check(lib().pic_gpu_set_deposit_order(self.h, mode))

    def set_tile(self, w: int, h: int):
        _check(lib().pic_gpu_set_tile(self.h, w, h))

    def deposit(self, scheme: int, dt: float = 0.0, background: float = 0.0, download: bool = True):
        rho = np.zeros(self.G) if download else None
        _check(lib().pic_gpu_deposit(self.h, int(scheme), float(dt), float(background), _ptr(rho)))
        return rho

    def rho_fixed(self):
        acc = np.zeros(self.G, np.int64)
        unit = C.c_double()
        _check(lib().pic_gpu_get_rho_fixed(self.h, _ptr(acc), C.byref(unit)))
        return acc, unit.value

    def rho(self):
        r = np.zeros(self.G)
        _check(lib().pic_gpu_get_rho(self.h, _ptr(r)))
        return r

    def is_sorted(self) -> bool:
        v = C.c_int()
        _check(lib().pic_gpu_is_sorted(self.h, C.byref(v)))
        return bool(v.value)

    def charge_uniform(self) -> float:
        """The stored charge q/max|q| shared by every particle (+-1), 0.0 when they differ."""
        v = C.c_float()
        _check(lib().pic_gpu_charge_uniform(self.h, C.byref(v)))
        return v.value

    def profile(self, enable: bool = True):
        _check(lib().pic_gpu_profile_enable(self.h, int(enable)))

    def profile_read(self, kernel: str):
        """(total milliseconds, launches) of `kernel` since the last read (CUDA events on the context stream)."""
        ms = C.c_double()
        cnt = C.c_longlong()
        _check(lib().pic_gpu_profile_read(self.h, kernel.encode(), C.byref(ms), C.byref(cnt)))
        return ms.value, cnt.value

    # ---- fields / Poisson / motion / diagnostics ----
    def set_rho(self, rho):
        r = _sized(rho, np.float64, self.G, "rho")
        _check(lib().pic_gpu_set_rho(self.h, _ptr(r)))

    def set_fields(self, phi=None, ex=None, ey=None):
        a = [_sized(v, np.float64, self.G, name) for v, name in zip((phi, ex, ey), ("phi", "ex", "ey"))]
        _check(lib().pic_gpu_set_fields(self.h, *[_ptr(v) for v in a]))

    def fields(self):
        out = [np.zeros(self.G) for _ in range(3)]
        _check(lib().pic_gpu_get_fields(self.h, *[_ptr(v) for v in out]))
        return tuple(out)

    def poisson_fft(self):
        _check(lib().pic_gpu_poisson_fft(self.h))

    def gather(self, dt):
        _check(lib().pic_gpu_gather(self.h, float(dt)))

    def push(self, dt):
        _check(lib().pic_gpu_push(self.h, float(dt)))

    def gather_push(self, dt):
        _check(lib().pic_gpu_gather_push(self.h, float(dt)))

    def deposit_current(self, dt, download=True):
        jx = np.zeros(self.G) if download else None
        jy = np.zeros(self.G) if download else None
        _check(lib().pic_gpu_deposit_current(self.h, float(dt), _ptr(jx), _ptr(jy)))
        return jx, jy

    def current_fixed(self):
        jx, jy = np.zeros(self.G, np.int64), np.zeros(self.G, np.int64)
        ux, uy = C.c_double(), C.c_double()
        _check(lib().pic_gpu_get_current_fixed(self.h, _ptr(jx), _ptr(jy), C.byref(ux), C.byref(uy)))
        return jx, jy, ux.value, uy.value

    def set_rbgs_precision(self, mixed: bool):
        """False: FP64 sweeps; True: FP32 sweeps on FP64-refined corrections."""
        _check(lib().pic_gpu_set_rbgs_precision(self.h, 1 if mixed else 0))

    def test_rbgs_barrier_timeout(self, absent_block: int, wait_ms: float = 1.0):
        """Test hook: the one-launch FP64 solve with CTA absent_block (-1: none)
        leaving before its first grid barrier and each barrier wait limited to
        wait_ms; raises PicError(PIC_ERR_TIMEOUT) when a wait ran out."""
        _check(lib().pic_gpu_test_rbgs_barrier_timeout(self.h, int(absent_block), float(wait_ms)))

    def poisson_rbgs(self, tol=1e-8, max_iters=1_000_000, warm_start=True, check_every=64):
        it = C.c_int()
        res = C.c_double()
        _check(lib().pic_gpu_poisson_rbgs(self.h, float(tol), int(max_iters), int(warm_start), int(check_every),
                                          C.byref(it), C.byref(res)))
        return it.value, res.value

    def generate(self, n, amplitude=0.0, mode=1, vth=0.0, v0=0.0, charge=-1.0, mass=1.0, seed=1):
        """Device-side particles (pic_gpu_generate)."""
        cfg = GenConfig(int(n), float(amplitude), int(mode), float(vth), float(v0), float(charge), float(mass),
                        int(seed))
        _check(lib().pic_gpu_generate(self.h, C.byref(cfg)))

    # ---- learned warm start (pic_gpu_ws_*) ----
    def ws_init(self, seed: int = 1, dataset_capacity: int = 0):
        _check(lib().pic_gpu_ws_init(self.h, int(seed), int(dataset_capacity)))

    @staticmethod
    def ws_param_count() -> int:
        L = lib()
        L.pic_gpu_ws_param_count.restype = C.c_size_t
        return int(L.pic_gpu_ws_param_count())

    def ws_params(self) -> np.ndarray:
        p = np.zeros(self.ws_param_count(), np.float32)
        _check(lib().pic_gpu_ws_get_params(self.h, _ptr(p), p.size))
        return p

    def ws_set_params(self, p):
        p = _arr(p, np.float32)
        _check(lib().pic_gpu_ws_set_params(self.h, _ptr(p), p.size))

    def ws_generate(self, steps, dt, background=0.0, sort_interval=20) -> int:
        _check(lib().pic_gpu_ws_generate(self.h, int(steps), float(dt), float(background), int(sort_interval)))
        n = C.c_size_t()
        _check(lib().pic_gpu_ws_dataset_size(self.h, C.byref(n)))
        return n.value

    def ws_train(self, epochs, batch, lr=1e-3, seed=1) -> np.ndarray:
        loss = np.zeros(max(int(epochs), 1))
        _check(lib().pic_gpu_ws_train(self.h, int(epochs), int(batch), float(lr), int(seed), _ptr(loss)))
        return loss[:epochs]

    def ws_loss_grad(self, inputs, targets):
        inputs = np.asarray(inputs)
        batch = int(inputs.shape[0]) if inputs.ndim > 1 else 1
        inputs = _sized(inputs, np.float32, batch * self.G, "inputs")
        targets = _sized(targets, np.float32, batch * self.G, "targets")
        grad = np.zeros(self.ws_param_count(), np.float32)
        loss = C.c_double()
        _check(lib().pic_gpu_ws_loss_grad(self.h, batch, _ptr(inputs), _ptr(targets), C.byref(loss), _ptr(grad)))
        return loss.value, grad

    def ws_predict(self, field):
        shape = np.shape(field)
        field = _sized(field, np.float32, self.G, "field")
        out = np.zeros(field.size, np.float32)
        _check(lib().pic_gpu_ws_predict(self.h, _ptr(field), _ptr(out)))
        return out.reshape(shape)

    def ws_study(self, steps, dt, background=0.0, sort_interval=20, tol=1e-8, check_every=16,
                 max_iters=2_000_000) -> dict:
        st = (WsStats * max(int(steps), 1))()
        _check(lib().pic_gpu_ws_study(self.h, int(steps), float(dt), float(background), int(sort_interval), float(tol),
                                      int(check_every), int(max_iters), st))
        st = st[:steps]
        return {"iters": np.array([list(s.iters) for s in st]), "ms": np.array([list(s.ms) for s in st]),
                "resid": np.array([list(s.resid) for s in st]),
                "guess_resid": np.array([list(s.guess_resid) for s in st]),
                "phi_diff": np.array([s.phi_diff for s in st])}

    def run(self, steps, scheme=1, dt=0.01, background=0.0, sort_interval=0, use_graph=False, poisson=0,
            rbgs_tol=1e-8, rbgs_max_iters=100000, rbgs_check_every=64, rbgs_warm=0, sort_moved_fraction=0.0):
        """Advances `steps` time steps; returns the per-step diagnostics as a (steps, 6) array in
        pic_diag order (charge_error, total_charge, integrated_rho, kinetic, field, total).
        sort_moved_fraction > 0 also sorts when that fraction of the particles has left the
        cells of the last sort (pic_run_config)."""
        cfg = RunConfig(int(scheme), int(poisson), float(dt), float(background), int(sort_interval),
                        int(use_graph), float(rbgs_tol), int(rbgs_max_iters), int(rbgs_check_every), int(rbgs_warm),
                        float(sort_moved_fraction))
        hist = (_Diag * max(steps, 1))()
        _check(lib().pic_gpu_run(self.h, C.byref(cfg), int(steps), hist))
        return np.array([[getattr(h, k) for k, _ in _Diag._fields_] for h in hist[:steps]])

    def sort_count(self) -> int:
        """Cell sorts performed on this context (pic_gpu_sort_count)."""
        n = C.c_longlong()
        _check(lib().pic_gpu_sort_count(self.h, C.byref(n)))
        return n.value

    def diagnostics(self) -> dict:
        d = _Diag()
        _check(lib().pic_gpu_diagnostics(self.h, C.byref(d)))
        return {k: getattr(d, k) for k, _ in _Diag._fields_}

    def synchronize(self):
        _check(lib().pic_gpu_synchronize(self.h))

    def launch_count(self) -> int:
        v = C.c_longlong()
        _check(lib().pic_gpu_launch_count(self.h, C.byref(v)))
        return v.value

    def stream(self) -> int:
        s = _vp()
        _check(lib().pic_gpu_get_stream(self.h, C.byref(s)))
        return s.value or 0


# ---------------------------------------------------------------------------
# Mirrors of the reference interface
# ---------------------------------------------------------------------------
class DepositionScheme(enum.IntEnum):
    """pic::DepositionScheme, src/deposition/deposition.hpp:11."""
    NGP = 0
    CIC = 1
    TSC = 2
    Esirkepov = 3


class DepositionBackend(enum.IntEnum):
    """pic::DepositionBackend, src/deposition/deposition.hpp:13, plus the GB300 value."""
    CPU = 0
    GPUAtomics = 1
    GPUPrivatized = 2
    GB300 = 3


class ParticleLayout(enum.IntEnum):
    AoS = 0
    SoA = 1


@dataclass
class Domain:
    """pic::Domain, src/pic/domain.hpp:7-44."""
    Lx: float = 1.0
    Ly: float = 1.0
    Nx: int = 64
    Ny: int = 64
    dt: float = 0.01
    steps: int = 100

    @property
    def dx(self):
        return self.Lx / self.Nx

    @property
    def dy(self):
        return self.Ly / self.Ny

    def updateDerived(self):
        pass

    def cellVolume(self):
        return self.dx * self.dy

    def domainVolume(self):
        return self.Lx * self.Ly


class ParticlesSoA:
    """pic::ParticlesSoA, src/pic/particles.hpp:45-83 (host FP64 arrays)."""

    def __init__(self, count: int = 0):
        self.resize(count)

    def resize(self, count: int):
        self.x, self.y, self.vx, self.vy, self.q = (np.zeros(count) for _ in range(5))
        self.m = np.ones(count)

    def size(self) -> int:
        return len(self.x)

    def totalCharge(self) -> float:
        return float(np.sum(self.q))

    def kineticEnergy(self) -> float:
        return float(np.sum(0.5 * self.m * (self.vx * self.vx + self.vy * self.vy)))


class FieldGrid:
    """pic::FieldGrid, src/pic/field_grid.hpp:9-39."""

    def __init__(self, domain: Domain):
        self._domain = domain
        n = domain.Nx * domain.Ny
        self.rho, self.phi, self.Ex, self.Ey = (np.zeros(n) for _ in range(4))

    def domain(self):
        return self._domain

    def clearRho(self):
        self.rho[:] = 0.0

    def integratedRho(self) -> float:
        return float(np.sum(self.rho)) * self._domain.cellVolume()

    def fieldEnergy(self) -> float:
        return 0.5 * float(np.sum(self.Ex * self.Ex + self.Ey * self.Ey)) * self._domain.cellVolume()


@dataclass
class DepositionConfig:
    """pic::DepositionConfig, src/deposition/deposition.hpp:15-24."""
    scheme: DepositionScheme = DepositionScheme.CIC
    layout: ParticleLayout = ParticleLayout.SoA
    backend: DepositionBackend = DepositionBackend.GB300
    sorted: bool = False
    num_threads: int = 1
    dx_esirkepov: float = 0.0
    dy_esirkepov: float = 0.0
    esirkepov_dt: float = 0.0


_ctx_cache: dict = {}


def _context_for(domain: Domain, n: int) -> Context:
    key = (domain.Nx, domain.Ny, domain.Lx, domain.Ly)
    c = _ctx_cache.get(key)
    if c is None or c.capacity < n:
        if c is not None:
            c.close()
        c = Context(domain.Nx, domain.Ny, domain.Lx, domain.Ly, max(n, 1))
        _ctx_cache[key] = c
    return c


def depositChargeSoA(particles: ParticlesSoA, grid: FieldGrid, config: DepositionConfig) -> None:
    """pic::depositChargeSoA (src/deposition/deposition.cpp:181-200) on the GB300
    backend: clears rho, uploads the particles, sorts them by cell when
    ``config.sorted`` and deposits ``config.scheme`` into ``grid.rho``."""
    if config.backend != DepositionBackend.GB300:
        raise RuntimeError("this library implements only DepositionBackend.GB300")
    d = grid.domain()
    ctx = _context_for(d, particles.size())
    ctx.upload(particles.x, particles.y, particles.q, particles.vx, particles.vy, particles.m)
    if config.sorted:
        ctx.sort()
    grid.rho[:] = ctx.deposit(int(config.scheme), config.esirkepov_dt)


def sortParticlesByCell(particles: ParticlesSoA, domain: Domain) -> None:
    """pic::sortParticlesByCell(ParticlesSoA&, const Domain&) (src/sorting/cell_sort.cpp:22-46),
    stable. Reorders the six host arrays in place."""
    ctx = _context_for(domain, particles.size())
    ctx.upload(particles.x, particles.y, particles.q, particles.vx, particles.vy, particles.m)
    _, perm, _ = ctx.sort(perm=True)
    for k in ("x", "y", "vx", "vy", "q", "m"):
        setattr(particles, k, getattr(particles, k)[perm])


def particleCellIndex(x: float, y: float, domain: Domain) -> int:
    """pic::particleCellIndex (src/sorting/cell_sort.cpp:8-13), via the device key."""
    ctx = _context_for(domain, 1)
    ctx.upload(np.array([x]), np.array([y]), np.array([1.0]))
    return int(ctx.device_layout()["cell"][0])
