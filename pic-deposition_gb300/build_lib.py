"""Build recipe for libpicgb300.so (the CUDA kernels + C ABI) and the C++ host adapter.

Every translation unit is compiled for sm_103a only, in parallel, then linked:
    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo --fmad=false ...
``--fmad=false`` keeps every FP32/FP64 multiply and add separately rounded, so the
kernels' arithmetic is reproduced bit for bit by the CPU oracle (compiled with
-ffp-contract=off); kernels that want a fused multiply-add call it explicitly.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(LIBDIR, "obj")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(LIBDIR, "libpicgb300.so")
HOSTLIB = os.path.join(LIBDIR, "libpicgb300_host.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE,
                     "-I" + CSRC]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile libpicgb300.so (and the host adapter) in-tree; returns the library path."""
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + [os.path.join(INCLUDE, "pic_gb300.h")]
    objs = []
    jobs = []
    for s in sources:
        o = os.path.join(OBJDIR, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if _stale(o, [s] + headers) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    logs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out in ex.map(_run, jobs):
                logs.append(out)
    if _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "--cudart", "shared", "-o", LIB] + objs + ["-lcufft"])
    host_srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if host_srcs:
        host_hdrs = sorted(glob.glob(os.path.join(HOST, "**", "*.hpp"), recursive=True))
        if _stale(HOSTLIB, host_srcs + host_hdrs + [LIB]):
            _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I" + INCLUDE, "-I" + HOST, "-o", HOSTLIB]
                 + host_srcs + ["-L" + LIBDIR, "-lpicgb300", "-Wl,-rpath,$ORIGIN"])
    if verbose or ptxas_info:
        sys.stdout.write("".join(logs))
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
