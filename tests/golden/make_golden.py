"""Generates tests/golden/*.npz from the reference's own sources.

Runs oracle/_ref/ref_pipeline (the reference's mesh.cpp portSet,
generateStiff.cpp, matrixCon.cpp paraGenerator and fdtdMesh members,
compiled unmodified by oracle/build_ref.sh) on seeded synthetic layouts and
stores what it produced.  Arrays up to SMALL elements are stored whole;
larger ones as a SHA-256 of their bytes plus a few statistics, which is
enough to check bit-exact integer and FP64 results.

Needs the reference checkout (the argument, else $G2P_REFERENCE_ROOT, else
/root/reference); the fixtures it writes are self-contained.  Usage:
    python tests/golden/make_golden.py [reference_root] [--cases a,b,...]
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gds2para_gb300 import layout as lay  # noqa: E402
from oracle.harness import run_reference  # noqa: E402

SMALL = 6000

# name -> (generator, kwargs); kept small enough for the reference's CPU code
CASES = {
    "multistrip_small": ("multistrip", dict(nx=24, ny=20, nz=8, n_strips=3, freq_start=1e8, freq_end=1e10,
                                            nfreq=4)),
    "strip_tiny": ("microstrip", dict(nx=13, ny=9, nz=6)),
    "strip_c1": ("microstrip", dict()),
    "manhattan_small": ("manhattan", dict(nx=40, ny=36, nz=12, n_metal=3, wires_per_layer=10, n_ports=3, seed=10,
                                          lmin=6, lmax=24)),
    "manhattan_sweep": ("manhattan", dict(nx=33, ny=29, nz=12, n_metal=2, wires_per_layer=8, n_ports=2, seed=1,
                                          lmin=6, lmax=20, freq_start=1e8, freq_end=1e10, freq_unit=1.0, nfreq=5,
                                          freq_scale=0)),
}

# The bench configurations, pinned by digests of everything the reference
# path produces (its solves take minutes here, so they are generated only
# when named: make_golden.py --cases manhattan_c2,multistrip_c3).  Their
# hypreSolve stand-in stops at SOLVE_RTOL instead of 1e-13.
BENCH_CASES = {
    "manhattan_c2": ("manhattan", dict(nx=512, ny=512, nz=24, n_ports=8, seed=1001)),
    "multistrip_c3": ("multistrip", dict(nx=256, ny=256, nz=16, n_strips=32)),
}
SOLVE_RTOL = {"manhattan_c2": 1e-10}

# The full-wave (Vh) path, which the reference compiles out: run with
# oracle/_ref/ref_pipeline_vh (find_Vh(1000) and the Vh correction built in),
# which also dumps the reference's Vh
VH_CASES = {
    "strip_tiny_vh": ("microstrip", dict(nx=13, ny=9, nz=6, freq_ghz=1.0, freq_end_ghz=10.0, nfreq=3)),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make_layout(gen: str, kw: dict):
    return lay.build(getattr(lay, gen)(**kw))


def main():
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("reference_root", nargs="?", default=os.environ.get("G2P_REFERENCE_ROOT", "/root/reference"))
    ap.add_argument("--cases", default=",".join(CASES),
                    help="comma-separated case names (default: the small cases; bench cases: "
                         + ",".join(BENCH_CASES) + ")")
    ap.add_argument("--no-build", action="store_true", help="use the oracle/_ref binaries already built")
    args = ap.parse_args()
    if not args.no_build:
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), args.reference_root])
    every = dict(CASES, **BENCH_CASES, **VH_CASES)
    import oracle.harness as harness
    for name in args.cases.split(","):
        gen, kw = every[name]
        if name in SOLVE_RTOL:
            os.environ["G2P_REF_SOLVE_RTOL"] = repr(SOLVE_RTOL[name])
        else:
            os.environ.pop("G2P_REF_SOLVE_RTOL", None)
        d = make_layout(gen, kw)
        harness.REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ref_pipeline_vh" if name in VH_CASES else "ref_pipeline")
        R = run_reference(d)
        out = {}
        meta = {"generator": gen, "kwargs": kw, "hashes": {}, "stats": {},
                "solve_rtol": SOLVE_RTOL.get(name, 1e-13)}
        for k, v in R.items():
            if k == "_log":
                continue
            if isinstance(v, int):
                meta[k] = v
                continue
            if v.size <= SMALL:
                out[k] = v
            else:
                meta["hashes"][k] = digest(v)
                meta["stats"][k] = dict(size=int(v.size), dtype=str(v.dtype),
                                        sum=float(np.sum(v.astype(np.float64))),
                                        absmax=float(np.max(np.abs(v))) if v.size else 0.0)
        # the reference's Z is always stored whole
        out["Z"] = R["Z"]
        out["_meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{name}: {os.path.getsize(path) / 1024:.1f} KiB, solves={R.get('solves')}, Z[0]={R['Z'][0]}")


if __name__ == "__main__":
    main()
