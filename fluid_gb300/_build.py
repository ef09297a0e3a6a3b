"""Builds libfluidgpu.so (the CUDA step behind the C ABI in include/fluidgpu.h).

Each translation unit is compiled by nvcc for sm_103a in parallel, then the
objects are linked into fluid_gb300/_build/libfluidgpu.so with the CUDA
runtime linked statically.  Device and host code are compiled without
floating-point contraction (-fmad=false, -ffp-contract=off) so the float32
arithmetic of every stage matches the reference operation for operation;
the parallel pressure schemes use explicit fused multiply-adds.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libfluidgpu.so")
SOURCES = ["fg_api.cu", "k_forces.cu", "k_advect.cu", "k_pressure.cu", "k_diag.cu", "k_adjoint.cu", "k_particles.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfluidgpu")


def _flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-I", os.path.join(ROOT, "include"),
    ]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith(".cuh")]
    headers.append(os.path.join(ROOT, "include", "fluidgpu.h"))
    exe = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(SRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([exe] + _flags() + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    if force or _stale(LIB, objs):
        cmd = [exe] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
