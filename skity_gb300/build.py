"""Build step of the GB300 raster backend: compiles the CUDA library
(skity_gb300/_build/libskity_cuda.so) for sm_103a with nvcc, one job per
translation unit, in parallel.

Numerics flags: -fmad=false (no FMA contraction on the device), IEEE
division and square root (nvcc defaults, kept explicit), and
-ffp-contract=off for host code, so float results follow the reference's
operation order on both sides.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libskity_cuda.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true",
              "-prec-sqrt=true", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden"]
SOURCES = ["kernels.cu", "plan.cu", "pipeline.cu", "per_draw.cu", "static_draw.cu", "server.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build skity_gb300")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "skity_cuda.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if not _newer(o, [s] + headers):
            jobs.append([nvcc(), *NVCC_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        run([nvcc(), ARCH, "-shared", *objs, "-o", LIB, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
