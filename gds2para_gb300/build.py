"""Builds the in-tree shared library libgds2para_gb300.so for sm_103a.

Each translation unit compiles in parallel with nvcc; the assembly units
(index maps, stiffness, V0 bases, extraction) are compiled without FMA
contraction so their floating-point results follow the reference's
operation order bit for bit.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libgds2para_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "--extended-lambda", "-lineinfo", "-Xcompiler", "-fPIC",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]
NO_FMA = {"mesh.cu", "v0.cu", "extract.cu", "mesher.cu"}
# host code whose results must not depend on the host compiler contracting
# a * b + c into one rounding (the oracle builds with -ffp-contract=off)
NO_HOST_CONTRACT = {"ingest.cu", "mesher.cu"}
UNITS = ["primitives.cu", "mesh.cu", "v0.cu", "solver.cu", "block_krylov.cu", "coarse.cu", "solve_api.cu", "extract.cu", "fullwave.cu", "stencil.cu", "noalloc.cu", "serve.cu", "mesher.cu",
         "network.cu", "ingest.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit: str) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit.replace(".cu", ".o"))
    flags = ARCH + COMMON + (["--fmad=false"] if unit in NO_FMA else []) + \
        (["-Xcompiler", "-ffp-contract=off"] if unit in NO_HOST_CONTRACT else [])
    cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {unit}:\n{r.stderr[-4000:]}")
    return obj


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "gds2para_gb300.h"),
                                                              os.path.abspath(__file__)]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, UNITS))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
