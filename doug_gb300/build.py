"""Build libdouggpu.so (sm_103a) in-tree with nvcc and g++.

The library is the product: C++ host setup + CUDA kernels behind the C ABI of
include/doug_gpu.h.  It is written to doug_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdouggpu.so")
CLI = os.path.join(OUT, "doug_gpu")       # command-line driver (flags of the reference's executables)
CLI_GEOM = os.path.join(OUT, "doug_geom_gpu")  # the same driver with doug_geom's setup
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

HOST_SRC = ["host/setup.cpp", "host/geom.cpp", "host/mf_symbolic.cpp"]
CUDA_SRC = ["dg_solver.cu", "dg_residual.cu", "dg_coarse_setup.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale(obj, srcs):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(s) > t for s in srcs)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in ("dg_kernels.cuh", "host/setup.hpp", "host/mf_symbolic.hpp")]
    headers.append(os.path.join(ROOT, "include", "doug_gpu.h"))
    jobs = []
    objs = []
    for src in HOST_SRC:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off",
                         "-Wall", "-c", s, "-o", o])
    for src in CUDA_SRC:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        logs = list(ex.map(_run, jobs))
    if verbose:
        for l in logs:
            print(l)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lpthread"])
    cli_src = os.path.join(CSRC, "doug_gpu_main.cpp")
    for exe, defs in ((CLI, []), (CLI_GEOM, ["-DDG_DRIVER_GEOM"])):
        if force or _stale(exe, [cli_src, LIB, os.path.join(ROOT, "include", "doug_gpu.h")]):
            _run(["g++", "-std=c++17", "-O2", "-Wall"] + defs + [cli_src, "-o", exe, "-L" + OUT, "-ldouggpu",
                  "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
