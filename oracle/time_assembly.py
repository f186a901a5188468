"""Host timing of the path's assembly: the reference's own compiled functions
(oracle/_ref/ref_pipeline: generateStiff, merge_v0d1, generateAd, merge_v0c,
generateAc, each timed inside the harness) beside the C restatement
(oracle/pipeline.c: S, then the job's index maps and V0d/Ad, V0c/Ac), on
the same seeded layout, one thread each.  Needs the reference build
(oracle/build_ref.sh), so it runs where the reference checkout is.

    python oracle/time_assembly.py [c2|c3|...]
"""
import json
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from gds2para_gb300 import layout  # noqa: E402
from oracle import harness  # noqa: E402


def main():
    cfg = sys.argv[1] if len(sys.argv) > 1 else "c2"
    d = layout.build(layout.config(cfg))
    os.environ["G2P_REF_NO_DUMP"] = "1"
    with tempfile.TemporaryDirectory(prefix="g2pt_") as td:
        t0 = time.perf_counter()
        r = harness.run_reference(d, workdir=td, skip_para=True)
        ref_wall = time.perf_counter() - t0
    ref = {k: r[k] for k in ("t_stiff_ms", "t_v0d_ms", "t_ad_ms", "t_v0c_ms", "t_ac_ms") if k in r}
    O = harness.COracle()
    t0 = time.perf_counter()
    O.stiffness(d)
    t_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    job = O.job(d)
    t_a = time.perf_counter() - t0
    job.close()
    out = {"config": cfg, "reference_compiled_ms": ref,
           "reference_compiled_total_ms": sum(ref.values()),
           "reference_process_wall_s": ref_wall,
           "restatement_ms": {"stiff": 1e3 * t_s, "maps_v0_ad_ac": 1e3 * t_a},
           "restatement_total_ms": 1e3 * (t_s + t_a)}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
