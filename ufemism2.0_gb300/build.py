"""Build the GB300 library (libufe_gpu.so) in-tree with nvcc, for sm_103a only.

Each translation unit compiles in parallel; the shared object lands in ``_build/`` next to this
file.  ``--fmad=false`` (device code) and ``-ffp-contract=off`` (host code; gcc contracts a*b+c
into one fused rounding on aarch64 by default) keep every a*b+c as two roundings, so operator
applications reproduce the reference's Fortran arithmetic bit for bit on any host.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libufe_gpu.so")
SOURCES = ["ufe_ctx.cu", "ufe_layout.cu", "ufe_operators.cu", "ufe_spmv.cu", "ufe_velocity.cu", "ufe_noalloc.cu",
           "ufe_thermo.cu", "ufe_gnn.cu", "ufe_mass.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(ptxas_verbose: bool) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
                "-I" + os.path.join(HERE, "..", "include")]
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    return f


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile every CUDA source and link the shared library; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = nvcc_path()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "ufe_gpu.h"))
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or ptxas_verbose or _stale(o, [s] + headers):
            jobs.append([nvcc] + _flags(ptxas_verbose) + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    failures = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0 or ptxas_verbose:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                failures.append(cmd[-3])
    if failures:
        raise RuntimeError("nvcc failed for " + ", ".join(failures))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, ptxas_verbose="--ptxas" in sys.argv))
