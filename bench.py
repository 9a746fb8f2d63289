"""Benchmark of the GB300 PIC deposition path.

Workload (the deposition benchmark shape): 1024x1024 periodic grid, dx = 1,
64 particles per cell = 67,108,864 particles, x drawn from density
1 + 0.01*cos(2*pi*x/1024) by rejection sampling, y uniform, Maxwellian
velocities vth = 0.1, charge -1, seeded synthetic data. The particles are
cell-sorted once before timing.

One step = one CIC charge deposition of all particles into an FP64 rho grid
(clear + sorted fixed-point deposit + conversion), particles resident in HBM.
The sorted deposit reads each particle's in-cell offsets xr, yr (and its charge
when charges differ); the per-cell offsets name every particle's cell, so the
cell keys are not read: 0.54 GB per step (8 B per particle, every particle has
the same charge), far larger than L2 (129 MB), so no L2 flush is needed.

  value   particles/s over the timed steps (CUDA events on the library stream),
          summed over ranks (replicas; one GPU each), max time over ranks.
  e2e     the same metric through the public C ABI with host buffers: every
          step uploads x, y, q (FP64, pinned) and downloads rho (FP64).
  roofline  the deposit kernel alone: algorithmic bytes (16 B per particle:
          x_rel, y_rel, q, cell key; + 8 B per cell: the int64 grid written once)
          / its mean CUDA-event duration, against the measured HBM copy
          bandwidth in MEASURED_PEAKS.json; frac_bytes_read is the same time
          against the bytes the kernel reads (8 B per particle when every
          particle has the same charge, as here -- neither the charge stream nor,
          after a sort, the cell keys are read -- + 12 B per cell).
  summary   last on the line: per-kernel times and fractions of HBM (at the
          algorithmic bytes, and for the deposits at the bytes read), the
          per-scheme errors against the FP64 deposit, and the time-step,
          ensemble, warm-start and convolution headlines, rounded.
  cpu_baseline  the reference's FP64 CPU deposit on the host cores (rank 0);
          its "detail" times every scheme at 1 and at all host threads, and the
          reference's cell sort where it is built, on a 4 M-particle sample.

--impl reference times the reference's own CPU path (oracle/_ref when it loads
on this machine, else the oracle's C restatement of it) on the same workload,
per step a bounded slice of it, with all host threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "pic-deposition_gb300"))

NX = NY = 1024
PPC = 64  # --ppc overrides (profiling runs use a smaller case)
AMP = 0.01
VTH = 0.1
ESK_DT = 0.1
SCHEMES = {"NGP": 0, "CIC": 1, "TSC": 2, "Esirkepov": 3}
# Algorithmic bytes of the sorted deposit: a cell-sorted particle set is read as
# its in-cell offsets x_rel, y_rel (FP32) and charge q (FP32) -- the per-cell
# offsets array (4 B per cell) names every particle's cell, so the cell keys are
# not read -- plus vx, vy for the Esirkepov schemes; the int64 grid is written
# once (8 B per cell).
BYTES_PER_PARTICLE = 12  # x_rel, y_rel, q (FP32)
BYTES_PER_PARTICLE_ESK = 20  # + vx, vy
# with one charge for every particle (the workloads here: q = -1) the kernels
# do not read the charge stream: 4 B less per particle
BYTES_Q = 4
BYTES_PER_CELL = 12  # int64 rho written once + the u32 cell offsets read once
# Algorithmic bytes per unit of work, the figures the roofline is quoted on
# (independent of how a kernel lays out or skips its reads): a deposit reads
# x_rel, y_rel, q (FP32) and the u32 cell key of each particle and writes the
# int64 grid once, 16 B per particle + 8 B per cell; the Esirkepov schemes read
# vx, vy too (24 B per particle; the current writes two grids). For the config
# 1024x1024, 64 per cell: 1.0821e9 B per deposit, so 60 % of the measured HBM
# copy bandwidth is a deposit of at most 0.270 ms. The bytes the sorted kernels
# actually read (above) are reported beside it.
ALG_BYTES_PER_PARTICLE = 16
ALG_BYTES_PER_PARTICLE_ESK = 24
ALG_BYTES_PER_CELL = 8
# learned warm start for red-black Gauss-Seidel: 512x512, 64 particles per cell,
# density 1 + 0.05*cos(2*pi*x/512), vth = 1 (the reference's charge convention,
# total charge -1 and m = 1, with the neutralising background), dt = 0.1
GS_N = 512
GS_PPC = 64
GS_AMP = 0.05
GS_VTH = 1.0
GS_DT = 0.1
GS_TOL = 1e-8
METRIC = "deposit particles/s (CIC, 64M cell-sorted particles, 1024x1024)"
WORKLOAD = "cic_deposit_1024x1024_64ppc_sorted"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profile():
    """dram bytes per deposit launch from the committed ncu summary (None if absent)."""
    path = os.path.join(ROOT, "profiles", "deposit_cells_cic_1024x1024_64ppc.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith("dram_bytes_per_launch_full_size:"):
                try:
                    return float(line.split(":", 1)[1].split()[0])
                except ValueError:
                    return None
    return None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


class CudaEvents:
    """CUDA events on a raw stream handle (libcudart via ctypes)."""

    def __init__(self):
        for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
            try:
                self.rt = C.CDLL(name)
                break
            except OSError:
                continue
        rt = self.rt
        rt.cudaEventCreate.argtypes = [C.POINTER(C.c_void_p)]
        rt.cudaEventRecord.argtypes = [C.c_void_p, C.c_void_p]
        rt.cudaEventSynchronize.argtypes = [C.c_void_p]
        rt.cudaEventElapsedTime.argtypes = [C.POINTER(C.c_float), C.c_void_p, C.c_void_p]
        rt.cudaEventDestroy.argtypes = [C.c_void_p]

    def event(self):
        e = C.c_void_p()
        assert self.rt.cudaEventCreate(C.byref(e)) == 0
        return e

    def record(self, e, stream):
        assert self.rt.cudaEventRecord(e, C.c_void_p(stream)) == 0

    def elapsed_ms(self, a, b):
        assert self.rt.cudaEventSynchronize(b) == 0
        ms = C.c_float()
        assert self.rt.cudaEventElapsedTime(C.byref(ms), a, b) == 0
        return float(ms.value)


def make_workload(seed: int):
    import workloads

    return workloads.density_cos(NX, NY, PPC, AMP, VTH, seed=seed)


def run_deposit_only(args, d: Dist):
    """Reduced run for profilers: upload, sort, then warmup + steps deposits of
    --scheme; prints the mean deposit-kernel time. No e2e, CPU or extra legs."""
    import pic_gb300 as pg

    p = make_workload(42)
    n = len(p["x"])
    with pg.Context(NX, NY, float(NX), float(NY), n) as ctx:
        ctx.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        if args.order == "sorted":
            ctx.sort()
        else:  # the generation order, random with respect to cells
            ctx.set_order(pg.ORDER_UNSORTED)
        ctx.profile(True)
        for _ in range(args.warmup + args.steps):
            ctx.deposit(SCHEMES[args.scheme], ESK_DT, download=False)
        ms, cnt = ctx.profile_read("deposit")
    print(json.dumps({"deposit_only": args.scheme, "order": args.order, "particles": n, "launches": cnt,
                      "mean_kernel_ms": ms / cnt}))


def run_sort_only(args, d: Dist):
    """Reduced run for profilers: warmup + steps cell sorts of the workload, each of the
    random-order (generation-order) upload; prints the mean sort time."""
    import pic_gb300 as pg

    p = make_workload(42)
    n = len(p["x"])
    with pg.Context(NX, NY, float(NX), float(NY), n) as ctx:
        ctx.profile(True)
        ms = []
        for i in range(args.warmup + args.steps):
            ctx.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
            ctx.profile_read("sort")
            ctx.sort()
            t, cnt = ctx.profile_read("sort")
            if i >= args.warmup:
                ms.append(t / cnt)
    print(json.dumps({"sort_only": "random order", "particles": n, "grid": [NX, NY], "mean_sort_ms": sum(ms) / len(ms)}))


def cpu_deposit_timer(threads: int):
    """Returns (fn(p) -> seconds for one FP64 CIC deposit, kind)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    kind = "port"
    ref = None
    if oracle.Ref.available():
        try:
            ref = oracle.Ref()
            kind = "reference"
        except OSError:
            ref = None
    port = oracle.Port()

    def run(p, scheme=1):
        # the reference's own timer, depositChargeTimedSoA (deposition.cpp:257-310): three
        # untimed deposits, then the timed one (clear + deposit); the port restates it
        if ref is not None:
            st = ref.deposit_timed(NX, NY, float(NX), float(NY), scheme, p, dt=ESK_DT, threads=threads, repeats=1)
            return st["deposit_ms"] / 1e3
        return port.deposit_timed(NX, NY, float(NX), float(NY), scheme, p, dt=ESK_DT, threads=threads, warmups=3,
                                  repeats=1) / 1e3

    return run, kind


def cpu_detail(ps, threads_all: int, sample: int = 4_000_000):
    """The reference's CPU path per scheme and thread count, and its cell sort, each on
    the first `sample` particles of the cell-sorted workload (a bounded sample).

    FP64 deposit at 1 thread and at all host threads per scheme; TSC on one thread
    only (the reference's privatised TSC writes past its per-thread grid, so its
    parallel form is not timed). The sort (sortParticlesByCell: std::sort of indices
    by cell, then a gather of the six arrays) is timed on a shuffled copy of the
    sample: the compiled reference where it loads, else the port's restatement."""
    m = min(sample, len(ps["x"]))
    sl = {k: np.ascontiguousarray(v[:m]) for k, v in ps.items()}
    timers = {th: cpu_deposit_timer(th) for th in sorted({1, threads_all})}
    out = {"unit": "particles/s", "sample_particles": m, "kind": timers[1][1], "threads_all": threads_all,
           "schemes": {}}
    for name, code in SCHEMES.items():
        row = {}
        for th in ((1,) if name == "TSC" else sorted({1, threads_all})):
            run = timers[th][0]
            run(sl, code)  # warm-up
            row[f"threads_{th}"] = m / min(run(sl, code) for _ in range(3))
        out["schemes"][name] = row
    import oracle

    ref = None
    if oracle.Ref.available():
        try:
            ref = oracle.Ref()
        except OSError:
            ref = None
    # sortParticlesByCell: the reference where it is built, else the port's restatement of
    # it (oracle/cell_sort_port.cpp, the same std::sort and gather; bit-identical output)
    sorter = ref.sort if ref is not None else oracle.Port().sort_by_cell
    perm = np.random.default_rng(1).permutation(m)
    sh = {k: np.ascontiguousarray(v[perm]) for k, v in sl.items()}
    sorter(NX, NY, float(NX), float(NY), sh)
    t0 = time.perf_counter()
    sorter(NX, NY, float(NX), float(NY), sh)
    t = time.perf_counter() - t0
    out["sort"] = {"particles_per_s": m / t, "order": "random", "kind": "reference" if ref is not None else "port",
                   "threads": 1, "includes": "copies of the six input arrays"}
    return out


def fp64_errors(p, gpu_out, threads):
    """Max-abs and relative L2 of the GPU's rho per scheme (and of the Esirkepov
    current Jx, Jy) against the reference's FP64 deposit of the same particles
    (the oracle's restatement of src/deposition/ngp.cpp, pinned bit for bit to the
    reference; the FP64 Esirkepov-2001 current), computed by the CPU-baseline leg."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    port = oracle.Port()
    out = {}
    for nm, code in SCHEMES.items():
        ref = port.deposit_ref(NX, NY, float(NX), float(NY), code, p, dt=ESK_DT, threads=threads)
        d = gpu_out[nm] - ref
        out["ESK_rho" if nm == "Esirkepov" else nm] = {"max_abs": float(np.max(np.abs(d))),
                                                       "rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref)),
                                                       "ref_max_abs": float(np.max(np.abs(ref)))}
    jx, jy = port.esirkepov_j_ref(NX, NY, float(NX), float(NY), p, ESK_DT)
    for nm, ref in (("Jx", jx), ("Jy", jy)):
        d = gpu_out[nm] - ref
        out[nm] = {"max_abs": float(np.max(np.abs(d))), "rel_l2": float(np.linalg.norm(d) / np.linalg.norm(ref)),
                   "ref_max_abs": float(np.max(np.abs(ref)))}
    out["workload"] = f"{WORKLOAD} (all particles), dt {ESK_DT} for the Esirkepov schemes"
    return out


def r4(x):
    """x rounded to 4 significant digits (None stays None)."""
    if x is None:
        return None
    return float(f"{x:.4g}")


def summary(res):
    """The figures a reader needs, compact, at the end of the line (the part a log tail keeps)."""
    ex = res.get("extra") or {}
    out = {"kernels": {}}
    for k, v in ex.items():
        ms = v.get("kernel_ms", v.get("ms", v.get("ms_per_step")))
        if "frac_bytes_read" in v:
            out["kernels"][k] = [r4(ms), r4(v.get("frac")), r4(v["frac_bytes_read"])]
        else:
            out["kernels"][k] = [r4(ms), r4(v.get("frac"))] if "frac" in v else r4(ms)
    err = res.get("errors_vs_fp64") or {}
    out["errors_vs_fp64"] = {k: [r4(v["max_abs"]), r4(v["rel_l2"])] for k, v in err.items() if isinstance(v, dict)}
    rl = res.get("roofline") or {}
    out["roofline_frac"] = r4(rl.get("frac"))
    out["roofline_frac_bytes_read"] = r4(rl.get("frac_bytes_read"))
    ts = res.get("timestep_2048")
    if ts:
        out["timestep_2048"] = {"ms_per_step": r4(ts["ms_per_step"]), "steps": ts["steps"],
                                "drift": {k: r4(v) for k, v in ts["energy_drift_at_steps"].items()}}
    en = res.get("ensemble")
    if en:
        out["ensemble_ms_per_step"] = r4(en["ms_per_step"])
    gs = res.get("gs_warm_start")
    if gs:
        out["gs"] = {k: r4(gs[k]) for k in ("speedup_learned_vs_plain", "speedup_extrapolated_vs_plain",
                                              "speedup_net_vs_extrapolated")}
    cv = res.get("conv_kernels")
    if cv:
        out["conv_frac_of_bf16"] = {k: r4(cv[k]["frac_of_bf16_peak"]) for k in ("conv_fwd", "conv_dgrad", "conv_wgrad")}
    return out


def sorted_order(p):
    key = np.floor(p["y"]).astype(np.int64) * NX + np.floor(p["x"]).astype(np.int64)
    return np.argsort(key, kind="stable")


def run_reference(args, d: Dist):
    out = {"impl": "reference", "metric": METRIC, "unit": "particles/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic (seeded)"}
    if d.rank != 0:
        return None
    threads = os.cpu_count() or 1
    p = make_workload(42)
    order = sorted_order(p)
    p = {k: v[order] for k, v in p.items()}
    run, kind = cpu_deposit_timer(threads)
    n = len(p["x"])
    # size each step's slice so that warmup + steps take about 90 s of wall time
    # (each timed deposit follows the timer's untimed warm-up deposits)
    probe = min(n, 4_000_000)
    sl = {k: v[:probe] for k, v in p.items()}
    run(sl)
    t0 = time.perf_counter()
    run(sl)
    rate = probe / max(time.perf_counter() - t0, 1e-6)
    per_step = int(min(n, max(1_000_000, rate * 90.0 / max(1, args.steps + args.warmup))))
    sl = {k: v[:per_step] for k, v in p.items()}
    for _ in range(args.warmup):
        run(sl)
    tot = 0.0
    for _ in range(args.steps):
        tot += run(sl)
    value = per_step * args.steps / tot
    out.update(value=value, ms_per_step=1e3 * tot / args.steps,
               config={"workload": WORKLOAD, "grid": [NX, NY], "particles": n, "sample_particles_per_step": per_step,
                       "l2": "inputs larger than L2 not applicable (CPU)"},
               cpu_baseline={"value": value, "unit": "particles/s", "cores": threads, "kind": kind,
                             "sample": f"first {per_step} cell-sorted particles of the workload per step, "
                                       f"FP64 CIC deposit (reference src/deposition/deposition_parallel.cpp "
                                       f"privatised OpenMP form)"},
               e2e={"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    return out


def run_gpu(args, d: Dist):
    import pic_gb300 as pg

    scheme = SCHEMES[args.scheme]
    dev = d.local if d.ws > 1 else 0
    p = make_workload(42 + d.rank)
    n = len(p["x"])
    G = NX * NY
    ev = CudaEvents()
    ctx = pg.Context(NX, NY, float(NX), float(NY), n, device=dev)
    stream = ctx.stream()

    # random-order upload, then a timed full sort
    ctx.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
    ctx.profile(True)
    _, perm, _ = ctx.sort(perm=True)
    ctx.profile_read("sort")  # the first sort also allocates its scratch arrays: not timed
    for _ in range(2):
        ctx.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
        ctx.sort()
    sort_ms, sort_cnt = ctx.profile_read("sort")
    sort_ms /= max(sort_cnt, 1)
    # unsorted (random order) deposits for reference numbers: use the random-order upload
    extras = {}
    ctx.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
    ctx.set_order(pg.ORDER_UNSORTED)
    for nm in ("CIC", "TSC"):
        for _ in range(2):
            ctx.deposit(SCHEMES[nm], ESK_DT, download=False)
        ctx.profile_read("deposit")
        for _ in range(5):
            ctx.deposit(SCHEMES[nm], ESK_DT, download=False)
        ms, cnt = ctx.profile_read("deposit")
        extras[f"{nm}_random_order"] = {"particles_per_s": n / (ms / cnt / 1e3), "kernel_ms": ms / cnt}
    ctx.set_order(pg.ORDER_AUTO)
    ctx.sort()
    assert ctx.is_sorted()
    q_uniform = ctx.charge_uniform() != 0.0

    peak, peak_kind = peaks()
    # per-scheme sorted kernels; each scheme's rho is kept for the error report
    gpu_out = {}
    for nm, s in SCHEMES.items():
        for _ in range(3):
            ctx.deposit(s, ESK_DT, download=False)
        ctx.profile_read("deposit")
        for _ in range(20):
            ctx.deposit(s, ESK_DT, download=False)
        ms, cnt = ctx.profile_read("deposit")
        bpp = (BYTES_PER_PARTICLE_ESK if s == 3 else BYTES_PER_PARTICLE) - (BYTES_Q if q_uniform else 0)
        abpp = ALG_BYTES_PER_PARTICLE_ESK if s == 3 else ALG_BYTES_PER_PARTICLE
        kms = ms / cnt
        gbs = (abpp * n + ALG_BYTES_PER_CELL * G) / (kms / 1e3) / 1e9
        read_gbs = (bpp * n + BYTES_PER_CELL * G) / (kms / 1e3) / 1e9
        extras[f"{nm}_sorted"] = {"particles_per_s": n / (kms / 1e3), "kernel_ms": kms, "kernel_gbs": gbs,
                                  "frac": gbs / peak, "frac_bytes_read": read_gbs / peak,
                                  "bytes_per_particle_read": bpp}
        gpu_out[nm] = ctx.deposit(s, ESK_DT)
    sort_gbs = (48 * n + 4 * (G + 1)) / (sort_ms / 1e3) / 1e9
    extras["sort_random_to_cells"] = {"ms": sort_ms, "particles_per_s": n / (sort_ms / 1e3),
                                      "algorithmic_gbs": sort_gbs, "frac": sort_gbs / peak}
    # Esirkepov current of the sorted particles (24 B/particle + 2 x 8 B/cell)
    for _ in range(2):
        ctx.deposit_current(ESK_DT, download=False)
    ctx.profile_read("current")
    for _ in range(10):
        ctx.deposit_current(ESK_DT, download=False)
    ms, cnt = ctx.profile_read("current")
    extras["Esirkepov_current_sorted"] = {"particles_per_s": n / (ms / cnt / 1e3), "kernel_ms": ms / cnt,
                                          "kernel_gbs": (24 * n + 16 * G) / (ms / cnt / 1e3) / 1e9,
                                          "frac": (24 * n + 16 * G) / (ms / cnt / 1e3) / 1e9 / peak}
    gpu_out["Jx"], gpu_out["Jy"] = ctx.deposit_current(ESK_DT)
    # FFT Poisson on the 1024^2 grid (cuFFT D2Z + k-divide + Z2D), neutral rho
    ctx.deposit(SCHEMES["CIC"], ESK_DT, background=float(PPC), download=False)
    for _ in range(2):
        ctx.poisson_fft()
    ctx.profile_read("poisson_fft")
    for _ in range(10):
        ctx.poisson_fft()
    ms, cnt = ctx.profile_read("poisson_fft")
    extras["poisson_fft_1024x1024"] = {"ms": ms / cnt}
    # fused gather + push (44 B/particle + 2 x 4 B/cell FP32 fields)
    for _ in range(2):
        ctx.gather_push(0.0)
    ctx.profile_read("gather_push")
    for _ in range(10):
        ctx.gather_push(0.0)
    ms, cnt = ctx.profile_read("gather_push")
    # reads cell, xr, yr, vx, vy (+ q when charges differ), writes cell, xr, yr, vx, vy; FP32 Ex, Ey
    gp_bpp = 40 + (0 if q_uniform else 4)
    gp_gbs = (gp_bpp * n + 8 * G) / (ms / cnt / 1e3) / 1e9
    extras["gather_push"] = {"particles_per_s": n / (ms / cnt / 1e3), "kernel_ms": ms / cnt, "kernel_gbs": gp_gbs,
                             "frac": gp_gbs / peak}
    # full time step: push, [sort every 10], TSC deposit + background, FFT Poisson,
    # gather, FP64 diagnostics; CUDA-graph replay; host wall time per step
    ctx.run(3, scheme=SCHEMES["TSC"], dt=ESK_DT, background=float(PPC), sort_interval=10, use_graph=True)
    t0 = time.perf_counter()
    ctx.run(20, scheme=SCHEMES["TSC"], dt=ESK_DT, background=float(PPC), sort_interval=10, use_graph=True)
    extras["timestep_tsc_sort10"] = {"ms_per_step": (time.perf_counter() - t0) * 1e3 / 20,
                                     "particles_per_s": n * 20 / (time.perf_counter() - t0),
                                     "setup": "the headline particles, charge -1 each with a background of 64 per "
                                              "cell: a hot plasma, most particles change cell every step"}
    # the general path: per-particle charges (alternating +-1) are read as a charge stream
    ctx.upload(p["x"], p["y"], np.where(np.arange(n) % 2 == 0, 1.0, -1.0), p["vx"], p["vy"], p["m"])
    ctx.sort()
    for _ in range(3):
        ctx.deposit(SCHEMES["CIC"], ESK_DT, download=False)
    ctx.profile_read("deposit")
    for _ in range(20):
        ctx.deposit(SCHEMES["CIC"], ESK_DT, download=False)
    ms, cnt = ctx.profile_read("deposit")
    gbs = (ALG_BYTES_PER_PARTICLE * n + ALG_BYTES_PER_CELL * G) / (ms / cnt / 1e3) / 1e9
    read_gbs = (BYTES_PER_PARTICLE * n + BYTES_PER_CELL * G) / (ms / cnt / 1e3) / 1e9
    extras["CIC_sorted_per_particle_charges"] = {"particles_per_s": n / (ms / cnt / 1e3), "kernel_ms": ms / cnt,
                                                 "kernel_gbs": gbs, "frac": gbs / peak,
                                                 "frac_bytes_read": read_gbs / peak,
                                                 "bytes_per_particle_read": BYTES_PER_PARTICLE}
    # restore the benchmark state: the random-order particles, cell-sorted
    ctx.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"], p["m"])
    ctx.sort()
    assert ctx.is_sorted()

    # ---- timed region: K deposits of the sorted particles ----
    for _ in range(args.warmup):
        ctx.deposit(scheme, ESK_DT, download=False)
    ctx.synchronize()
    ctx.profile_read("deposit")
    e0, e1 = ev.event(), ev.event()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.2)
    launches0 = ctx.launch_count()
    d.barrier()
    ctx.synchronize()
    ev.record(e0, stream)
    for _ in range(args.steps):
        ctx.deposit(scheme, ESK_DT, download=False)
    ev.record(e1, stream)
    ms = ev.elapsed_ms(e0, e1)
    ctx.synchronize()
    d.barrier()
    launches = ctx.launch_count() - launches0
    clk = clocks.stop()
    kms_tot, kcnt = ctx.profile_read("deposit")
    ms_max = d.max(ms)
    value = n * args.steps * d.ws / (ms_max / 1e3)
    kernel_ms = kms_tot / max(kcnt, 1)
    bpp_main = BYTES_PER_PARTICLE - (BYTES_Q if q_uniform else 0)
    read_bytes = bpp_main * n + BYTES_PER_CELL * G
    alg_bytes = ALG_BYTES_PER_PARTICLE * n + ALG_BYTES_PER_CELL * G
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    traffic = traffic_from_profile()

    # ---- e2e: host buffers through the C ABI (upload x,y,q + deposit + rho download) ----
    order = perm.astype(np.int64)
    pin = {k: pg.PinnedArray(n) for k in ("x", "y", "q")}
    for k in pin:
        pin[k].array[:] = p[k][order]
    rho_host = pg.PinnedArray(G)
    e2e_steps = max(3, min(args.steps, 20))
    for _ in range(2):
        ctx.upload(pin["x"].array, pin["y"].array, pin["q"].array)
        pg._check(pg.lib().pic_gpu_deposit(ctx.h, scheme, ESK_DT, 0.0, pg._ptr(rho_host.array)))
    assert ctx.is_sorted()
    d.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.upload(pin["x"].array, pin["y"].array, pin["q"].array)
        pg._check(pg.lib().pic_gpu_deposit(ctx.h, scheme, ESK_DT, 0.0, pg._ptr(rho_host.array)))
    t_e2e = time.perf_counter() - t0
    t_e2e = d.max(t_e2e)
    e2e_value = n * e2e_steps * d.ws / t_e2e

    # ---- CPU baseline (rank 0): the reference FP64 path on the host cores ----
    cpu = None
    if d.rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        run, kind = cpu_deposit_timer(threads)
        ps = {k: v[order] for k, v in p.items()}
        t_cpu, reps = 0.0, 0
        w0 = time.perf_counter()
        while time.perf_counter() - w0 < args.cpu_seconds or reps == 0:
            t_cpu += run(ps)
            reps += 1
        cpu = {"value": n * reps / t_cpu, "unit": "particles/s", "cores": threads, "kind": kind,
               "sample": f"full workload ({n} cell-sorted particles), FP64 CIC deposit x{reps}, "
                         f"privatised OpenMP form of src/deposition/deposition_parallel.cpp, timed as "
                         f"depositChargeTimedSoA times it (untimed warm-up deposits first)"}
        try:  # per scheme and thread count, and the sort; a failure here leaves the line intact
            cpu["detail"] = cpu_detail(ps, threads)
        except Exception as e:  # noqa: BLE001
            cpu["detail"] = {"error": f"{type(e).__name__}: {e}"}
        try:  # the same leg's FP64 deposits as the checker of the GPU results
            errors = fp64_errors(p, gpu_out, threads)
        except Exception as e:  # noqa: BLE001
            errors = {"error": f"{type(e).__name__}: {e}"}
    else:
        errors = None
    for a in list(pin.values()) + [rho_host]:
        a.free()
    ctx.close()
    if d.rank != 0:
        return None
    return {
        "metric": METRIC, "value": value, "unit": "particles/s", "n_gpus": d.ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64 fixed point (FP32 weights, FP64 rho)", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "grid": [NX, NY], "particles_per_cell": PPC, "particles": n,
                   "density": "1+0.01cos(2*pi*x/1024)", "vth": VTH, "scheme": args.scheme,
                   "l2": f"inputs ({bpp_main * n / 1e9:.2f} GB particle stream) larger than L2; no flush",
                   "charge": ("one charge (-1) for every particle: the charge stream is not read, "
                              f"{bpp_main} B/particle" if q_uniform else f"per-particle charges, {bpp_main} B/particle"),
                   "parallelism": f"replicas{d.ws}"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "kernel": "deposit_cells<CIC>",
                     "kernel_ms": kernel_ms, "algorithmic_bytes_per_launch": alg_bytes,
                     "bytes_read_per_launch": read_bytes,
                     "frac_bytes_read": read_bytes / (kernel_ms / 1e3) / 1e9 / peak},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "particles/s", "h2d_bytes_per_step": 24 * n,
                "d2h_bytes_per_step": 8 * G, "steps": e2e_steps},
        "gpu_launches": launches,
        "clocks": clk,
        "extra": extras,
        "errors_vs_fp64": errors,
    }


def ensemble_members(seed=4, runs=64):
    """64 Langmuir runs: grid N from {128, 256, 512, 1024} and particles per cell
    from {4, 16, 64, 256}, drawn per run from `seed`."""
    rng = np.random.default_rng(seed)
    ns = rng.choice([128, 256, 512, 1024], runs)
    ppcs = rng.choice([4, 16, 64, 256], runs)
    return [(int(n), int(p), int(1000 + i)) for i, (n, p) in enumerate(zip(ns, ppcs))]


def run_ensemble(args, d=None):
    """Batched ensemble: every run's step (gather+push, deposit, FFT Poisson) in one
    persistent launch + batched FFTs per step, replayed as a CUDA graph. Over N
    ranks each rank runs its share of the members (partition_members, balanced
    by particles) as its own batch; the step time is the max over ranks and the
    throughput counts every member (strong scaling: the members are fixed)."""
    import pic_gb300 as pg

    members = ensemble_members(runs=args.ens_runs)
    ws, rank = (d.ws, d.rank) if d is not None else (1, 0)
    mine = pg.partition_members(members, ws)[rank]
    total = sum(n * n * p for n, p, _ in members)
    out = {"workload": f"ensemble_{len(members)}_langmuir_runs", "runs": len(members), "particles": total,
           "cells": sum(n * n for n, _, _ in members), "dt": 0.1, "amplitude": 0.01, "vth": 0.05,
           "sort_interval": args.ens_sort, "steps": args.ens_steps, "ranks": ws,
           "scaling": "strong" if ws > 1 else None}
    ms, fe = 0.0, np.zeros((1, 0))
    if d is not None:
        d.barrier()
    if mine:
        with pg.Ensemble([members[i] for i in mine], dt=0.1, amplitude=0.01, vth=0.05, sort_interval=args.ens_sort,
                         use_graph=True, device=d.local if d is not None else 0) as e:
            e.run(args.ens_sort + 1)  # warm-up: first sort, autotuning, graph capture
            stream = e.stream()
            ev = CudaEvents()
            e0, e1 = ev.event(), ev.event()
            l0 = e.launch_count()
            if d is not None:
                d.barrier()
            ev.record(e0, stream)
            fe, ke = e.run(args.ens_steps)
            ev.record(e1, stream)
            ms = ev.elapsed_ms(e0, e1)
            out["launches_per_step"] = (e.launch_count() - l0) / args.ens_steps
            out["tiles"] = sorted({f"N{e.info(r)['N']}_ppc{e.info(r)['ppc']}": list(e.info(r)["tile"])
                                   for r in range(len(mine))}.items())
    elif d is not None:
        d.barrier()
    if d is not None:
        ms = d.max(ms)
    out["ms_per_step"] = ms / args.ens_steps
    out["particle_steps_per_s"] = total * args.ens_steps / (ms * 1e-3)
    out["field_energy_finite"] = bool(np.all(np.isfinite(fe)))
    return out


# tensor-core work of the warm-start network per 512x512 sample, as executed
# (first layer 16 input channels, last layer 16 output channels, of which one is used)
NN_LAYERS = [(16, 32), (32, 32), (32, 32), (32, 32), (32, 32), (32, 16)]


def run_nn_profile(args):
    """Throughput of the tcgen05 convolution kernels: forward, input gradient and
    weight gradient of the warm-start network on a batch of 512x512 fields."""
    import pic_gb300 as pg

    B, N = args.nn_batch, GS_N
    P = B * N * N
    rng = np.random.default_rng(3)
    inp = rng.normal(size=(B, N, N)).astype(np.float32)
    tgt = rng.normal(size=(B, N, N)).astype(np.float32)
    with pg.Context(N, N, float(N), float(N), 16) as c:
        c.ws_init(seed=1)
        for _ in range(3):
            c.ws_loss_grad(inp, tgt)
        c.profile(True)
        reps = args.nn_reps
        for _ in range(reps):
            c.ws_loss_grad(inp, tgt)
        prof = {k: c.profile_read(k) for k in ("conv_fwd", "conv_dgrad", "conv_wgrad")}
        c.profile(False)
    flops_fwd = sum(2.0 * P * 9 * ci * co for ci, co in NN_LAYERS)
    flops_dgrad = sum(2.0 * P * 9 * ci * co for ci, co in NN_LAYERS[1:])
    flops_wgrad = flops_fwd
    peak = 1890.5
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except (OSError, KeyError, ValueError):
        pass
    out = {"workload": f"conv3x3_net_{N}x{N}_batch{B}", "batch": B, "peak_bf16_tflops": peak}
    for k, fl in (("conv_fwd", flops_fwd), ("conv_dgrad", flops_dgrad), ("conv_wgrad", flops_wgrad)):
        ms, n = prof[k]
        t = ms / reps
        out[k] = {"ms_per_pass": t, "launches_per_pass": n / reps, "tflops": fl / (t * 1e-3) / 1e12,
                  "frac_of_bf16_peak": fl / (t * 1e-3) / 1e12 / peak}
    return out


def run_config3(args):
    """Full electrostatic time step at 2048x2048 with 100 particles per cell
    (419,430,400 particles): two equal beams vx = +-0.2, vth = 0.01, uniform
    positions (the reference's two-stream conventions: charge -1/N, m = 1,
    background 1/V), TSC, cell sort every 10 steps, FFT Poisson, fused graph steps."""
    import pic_gb300 as pg

    N, ppc = args.c3_n, 100
    n = N * N * ppc
    steps, dt = args.c3_steps, 0.1
    out = {"workload": f"timestep_twostream_tsc_{N}x{N}_{ppc}ppc", "particles": n, "steps": steps, "dt": dt,
           "scheme": "TSC", "sort_interval": 10, "poisson": "FFT"}
    with pg.Context(N, N, float(N), float(N), n) as c:
        c.generate(n, vth=0.01, v0=0.2, charge=-1.0 / n, mass=1.0, seed=2024)
        bg = 1.0 / (N * N)
        c.run(10, scheme=2, dt=dt, background=bg, sort_interval=10, use_graph=True)  # warm-up, graph capture
        c.generate(n, vth=0.01, v0=0.2, charge=-1.0 / n, mass=1.0, seed=2024)
        ev = CudaEvents()
        e0, e1 = ev.event(), ev.event()
        ev.record(e0, c.stream())
        h = c.run(steps, scheme=2, dt=dt, background=bg, sort_interval=10, use_graph=True)
        ev.record(e1, c.stream())
        ms = ev.elapsed_ms(e0, e1)
    e = h[:, 5]
    drift = (e - e[0]) / abs(e[0])
    marks = sorted({0, steps // 4, steps // 2, 3 * steps // 4, steps - 1})
    out.update({"ms_per_step": ms / steps, "particle_steps_per_s": n * steps / (ms * 1e-3),
                "energy_drift_at_steps": {str(k): float(drift[k]) for k in marks},
                "max_abs_energy_drift": float(np.max(np.abs(drift))),
                "max_charge_error": float(np.max(h[:, 0])),
                "charge_error_note": "pic::computeDiagnostics' charge_error, |integral of rho - particle charge| / "
                                     "sum |q|: rho includes the neutralising background (+1 in total) and the "
                                     "particles carry -1, so a neutral plasma reads 1 by construction"})
    return out


def run_gs_study(args):
    """Time to a 1e-8 relative residual of red-black Gauss-Seidel from three
    starting guesses (previous phi; cubic extrapolation; extrapolation plus the
    trained network), each step's system solved three times from the same b."""
    import pic_gb300 as pg
    import workloads

    p = workloads.density_cos(GS_N, GS_N, GS_PPC, GS_AMP, GS_VTH, seed=7)
    n = len(p["x"])
    p["q"] = np.full(n, -1.0 / n)
    bg = 1.0 / (GS_N * GS_N)
    out = {"workload": f"rbgs_{GS_N}x{GS_N}_{GS_PPC}ppc_landau", "particles": n, "tol": GS_TOL, "dt": GS_DT,
           "pairs_requested": args.gs_pairs}
    with pg.Context(GS_N, GS_N, float(GS_N), float(GS_N), n) as c:
        c.upload(p["x"], p["y"], p["q"], p["vx"], p["vy"])
        del p
        c.set_rbgs_precision(args.gs_mixed)
        out["sweep_precision"] = "FP32 sweeps, FP64 refinement" if args.gs_mixed else "FP64"
        c.ws_init(seed=1, dataset_capacity=args.gs_pairs)
        t0 = time.time()
        out["pairs"] = c.ws_generate(args.gs_pairs + 3, GS_DT, bg, sort_interval=20)
        out["generate_s"] = time.time() - t0
        t0 = time.time()
        losses = c.ws_train(args.gs_epochs, args.gs_batch, args.gs_lr)
        out["train_s"] = time.time() - t0
        out["train_loss"] = [float(v) for v in losses]
        out["epochs"], out["batch"], out["lr"] = args.gs_epochs, args.gs_batch, args.gs_lr
        st = c.ws_study(args.gs_steps, GS_DT, bg, sort_interval=20, tol=GS_TOL, check_every=args.gs_check)
    names = ["previous_phi", "extrapolated", "extrapolated_plus_net"]
    out["check_every"] = args.gs_check
    out["steps"] = args.gs_steps
    for k, nm in enumerate(names):
        out[nm] = {"sweeps_mean": float(st["iters"][:, k].mean()), "ms_mean": float(st["ms"][:, k].mean()),
                   "guess_resid_mean": float(st["guess_resid"][:, k].mean()),
                   "resid_max": float(st["resid"][:, k].max())}
    out["speedup_learned_vs_plain"] = out[names[0]]["ms_mean"] / out[names[2]]["ms_mean"]
    out["speedup_extrapolated_vs_plain"] = out[names[0]]["ms_mean"] / out[names[1]]["ms_mean"]
    # what the trained network adds to the same method without it
    out["speedup_net_vs_extrapolated"] = out[names[1]]["ms_mean"] / out[names[2]]["ms_mean"]
    out["sweeps_net_vs_extrapolated"] = out[names[1]]["sweeps_mean"] / out[names[2]]["sweeps_mean"]
    out["phi_diff_max"] = float(st["phi_diff"].max())
    return out


def main():
    global PPC
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scheme", default="CIC", choices=list(SCHEMES))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ppc", type=int, default=PPC, help="particles per cell (64 = the benchmark workload)")
    ap.add_argument("--deposit-only", action="store_true", help="reduced run for profilers")
    ap.add_argument("--sort-only", action="store_true", help="reduced run for profilers: cell sorts only")
    ap.add_argument("--order", default="sorted", choices=["sorted", "random"],
                    help="--deposit-only: cell-sorted particles or the generation order")
    ap.add_argument("--gs-only", action="store_true", help="only the Gauss-Seidel warm-start study")
    ap.add_argument("--no-gs", action="store_true", help="skip the Gauss-Seidel warm-start study")
    ap.add_argument("--c3-only", action="store_true", help="only the 2048^2 two-stream time step")
    ap.add_argument("--no-c3", action="store_true", help="skip the 2048^2 two-stream time step")
    ap.add_argument("--c3-steps", type=int, default=2000)
    ap.add_argument("--c3-n", type=int, default=2048, help="grid N x N of the two-stream time step (2048 = the workload)")
    ap.add_argument("--nn-only", action="store_true", help="only the convolution-kernel throughput")
    ap.add_argument("--nn-batch", type=int, default=8)
    ap.add_argument("--nn-reps", type=int, default=5)
    ap.add_argument("--ens-only", action="store_true", help="only the batched ensemble")
    ap.add_argument("--no-ens", action="store_true", help="skip the batched ensemble")
    ap.add_argument("--ens-runs", type=int, default=64)
    ap.add_argument("--ens-steps", type=int, default=500)
    ap.add_argument("--ens-sort", type=int, default=20)
    ap.add_argument("--gs-pairs", type=int, default=20000)
    ap.add_argument("--gs-epochs", type=int, default=2)
    ap.add_argument("--gs-batch", type=int, default=16)
    ap.add_argument("--gs-lr", type=float, default=1e-3)
    ap.add_argument("--gs-steps", type=int, default=8)
    ap.add_argument("--gs-check", type=int, default=16)
    ap.add_argument("--gs-mixed", type=int, default=1, help="1: FP32 sweeps with FP64 refinement, 0: FP64 sweeps")
    args = ap.parse_args()
    PPC = args.ppc
    if args.warmup < 3:
        args.warmup = 3
    if args.gs_only:
        print(json.dumps(run_gs_study(args)), flush=True)
        return
    if args.ens_only:
        d = Dist()
        try:
            res = run_ensemble(args, d)
        finally:
            d.close()
        if d.rank == 0:
            print(json.dumps(res), flush=True)
        return
    if args.nn_only:
        print(json.dumps(run_nn_profile(args)), flush=True)
        return
    if args.c3_only:
        print(json.dumps(run_config3(args)), flush=True)
        return
    d = Dist()
    if args.deposit_only:
        run_deposit_only(args, d)
        d.close()
        return
    if args.sort_only:
        run_sort_only(args, d)
        d.close()
        return
    try:
        res = run_reference(args, d) if args.impl == "reference" else run_gpu(args, d)
        if res is not None and args.impl != "reference" and d.ws == 1:
            if not args.no_ens:
                res["ensemble"] = run_ensemble(args)
            if not args.no_c3:
                res["timestep_2048"] = run_config3(args)
            if not args.no_gs:
                res["gs_warm_start"] = run_gs_study(args)
                res["conv_kernels"] = run_nn_profile(args)
    finally:
        d.close()
    if res is not None:
        if args.impl != "reference":
            res["summary"] = summary(res)
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
