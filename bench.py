"""Benchmark of the extraction hot path on GB300.

One step = one complete V0 extraction of a synthetic layout through the C ABI
(include/gds2para_gb300.h): upload of the fdtdMesh fields, index maps,
generateStiff, V0 bases and Ad/Ac assembly, AMG setup, the three solves of
every port (all ports as one block of right-hand sides) and the Z matrix.

metric: port-frequency solves per second = ports x frequency points / step.
`value` starts from inputs already resident in HBM; `e2e` starts from pinned
host buffers and includes the host->device copies and the Z read-back.

    python bench.py [--gpus N --steps K --warmup W --impl gb300|reference
                     --config c2 --precision mixed|fp64 --batch 1]
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
sys.path.insert(0, ROOT)

METRIC = "port-freq solves/s at 1e-6 rel Z err, mixed+batched vs FP64 GPU; p50/p99 job ms"
UNIT = "port-freq solves/s"
RTOL = {"c1": 1e-10, "c2": 1e-8, "c3": 1e-8, "c4": 1e-8, "c5": 1e-8}
WORKLOAD = {
    "c1": "microstrip 101x41x11 nodes at 1 um, 1 port, 1 GHz, rtol 1e-10",
    "c2": "random Manhattan 512x512x24 nodes, 4 metal layers x 64 wires, 8 ports, 10 GHz, rtol 1e-8",
    "c3": "microstrip stack 256x256x16 nodes, 32 strips/ports x 64 log-spaced points 1e7..1e11 Hz, rtol 1e-8",
    "c4": "served stream of 200 random Manhattan jobs (sides log-uniform 64..1024 nodes in x and y, nz uniform in "
          "{8, 16, 32}, 1..16 ports, 1..32 log-spaced points 1e8..1e10 Hz), Poisson arrivals at 0.8 x the serial "
          "capacity, 150 GB budget, rtol 1e-8",
    "c5": "large random Manhattan 1536x1536x32 nodes (224M edges), 6 metal layers x 256 wires, 16 ports x 8 "
          "log-spaced points 1e8..1e10 Hz, ports in blocks of 4, rtol 1e-8",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c2", choices=list(WORKLOAD))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-ports", type=int, default=1)
    ap.add_argument("--once", action="store_true",
                    help="run one untimed step and exit (for profiler captures; prints no bench line)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows)}
        if not self.rows:
            return out
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        out["sm_mhz"] = statistics.median(sm) if sm else None
        out["sm_max_mhz"] = max(mx) if mx else None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if r[5 + i].lower().startswith("active"):
                    reasons.add(n)
        out["reasons"] = sorted(reasons)
        return out


def max_over_ranks(ms: float, world: int, device: str = "cuda") -> float:
    """Step time of the whole job: the slowest replica's (a MAX all-reduce
    over the ranks; the replicas share no data)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(units_per_replica: int, world: int, ms: float) -> float:
    """Port-frequency solves per second of N replicas each doing one job per
    step, timed by the slowest one (weak scaling)."""
    return world * units_per_replica / (ms / 1e3)


def make_desc(d, place, torch):
    """MeshDesc arrays as torch tensors on `place` ('pinned' or 'cuda')."""
    arrays = dict(
        xn=(d.xn, np.float64), yn=(d.yn, np.float64), zn=(d.zn, np.float64),
        stack_epsn=(d.stack_epsn, np.float64), stack_sign=(d.stack_sign, np.float64),
        mark_node=(d.mark_node, np.int64), mark_edge=(d.mark_edge, np.int64),
        mark_port=(d.mark_port, np.int32), cdt_return=(d.cdt_return, np.uint8),
        port_side_ptr=(d.port_side_ptr, np.int32), side_edge_ptr=(d.side_edge_ptr, np.int64),
        side_edges=(d.side_edges, np.int64), side_area=(d.side_area, np.float64), side_dir=(d.side_dir, np.int32))
    out = {}
    for k, (a, dt) in arrays.items():
        t = torch.from_numpy(np.ascontiguousarray(a, dtype=dt))
        out[k] = t.pin_memory() if place == "pinned" else t.cuda()
    return out


def desc_struct(d, T, _lib):
    p = lambda k: T[k].data_ptr()
    host_ports = ("port_side_ptr", "side_edge_ptr", "side_edges", "side_area", "side_dir")
    return _lib.MeshDescC(d.nx, d.ny, d.nz, p("xn"), p("yn"), p("zn"), p("stack_epsn"), p("stack_sign"),
                          p("mark_node"), p("mark_edge"), d.num_cdt, p("mark_port"), p("cdt_return"), d.num_ports,
                          p("port_side_ptr"), p("side_edge_ptr"), p("side_edges"), p("side_area"), p("side_dir"),
                          d.freq_start, d.freq_end, d.freq_unit, d.nfreq, d.freq_scale)


def run_gb300(args):
    import torch
    from gds2para_gb300 import _lib, layout
    from gds2para_gb300.api import default_params
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    L = _lib.load()
    lay_cfg = layout.config(args.config)
    t0 = time.perf_counter()
    d = layout.build(lay_cfg)
    host_mesh_s = time.perf_counter() - t0
    # c5: the port blocks that fit 280 GB of HBM (4 ports: about 175 GiB)
    big = args.config == "c5"
    batch = (args.batch if args.batch > 1 else 4) if big else args.batch
    # --once (profiler captures) runs one step without the autotuner's trial
    # solves; c2's tuned choice is the untuned one (all ports, degree 2)
    params = default_params(precision=args.precision, batch=batch, rtol=RTOL[args.config],
                            autotune=0 if (big or args.once) else 1)
    dev = make_desc(d, "cuda", torch)
    pin = make_desc(d, "pinned", torch)
    z =torch.zeros(2 * d.nfreq * d.num_ports * d.num_ports, dtype=torch.float64).pin_memory()
    stats = _lib.ExtractStats()

    def step(T, prm=None):
        desc = desc_struct(d, T, _lib)
        h = C.c_void_p()
        _lib.check(L.g2p_mesh_create(C.byref(desc), C.byref(h)))
        n = C.c_int64()
        _lib.check(L.g2p_generate_stiff(h, C.byref(n)))
        _lib.check(L.g2p_para_generator(h, C.byref(prm or params), C.c_void_p(z.data_ptr()), C.byref(stats)))
        L.g2p_mesh_destroy(h)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(T, k, profile=False, prm=None, per_step=None):
        barrier()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(k + 1)]
        n0 = L.g2p_launch_count()
        if profile:
            L.g2p_profile_begin()
        ev[0].record()
        for i in range(k):
            step(T, prm)
            ev[i + 1].record()
        barrier()
        e0, e1 = ev[0], ev[k]
        if per_step is not None:
            per_step.extend(ev[i].elapsed_time(ev[i + 1]) for i in range(k))
        kern = None
        if profile:
            ms, by, nl = C.c_double(), C.c_double(), C.c_int64()
            _lib.check(L.g2p_profile_end(C.byref(ms), C.byref(by), C.byref(nl)))
            bms, bby, bn = (C.c_double * 8)(), (C.c_double * 8)(), (C.c_int64 * 8)()
            L.g2p_profile_buckets(bms, bby, bn)
            kern = (ms.value, by.value, nl.value, list(bms), list(bby), list(bn))
        el = max_over_ranks(e0.elapsed_time(e1) / k, world)
        return el, L.g2p_launch_count() - n0, kern

    if args.once:
        step(dev)
        torch.cuda.synchronize()
        return {"once": True, "config": args.config, "precision": args.precision,
                "iterations": stats.total_iterations}, rank
    for _ in range(max(args.warmup, 3)):
        step(dev)
    clocks = Clocks(local)
    clocks.start()
    step_ms = []
    ms, launches, _ = timed(dev, args.steps, per_step=step_ms)
    clk = clocks.stop()
    last = {"assembly_ms": stats.assembly_ms, "setup_ms": stats.setup_ms, "solve_ms": stats.solve_ms,
            "total_ms": stats.total_ms, "iterations": stats.total_iterations,
            "max_rel_residual": stats.max_rel_residual, "ad_levels": stats.ad_levels, "ac_levels": stats.ac_levels,
            "rhs_block": stats.rhs_block, "ad_degree": stats.ad_degree, "ac_strength": stats.ac_strength,
            "ac_precision": {0: "fp64", 1: "mixed", 2: "fp64_pc32"}.get(stats.ac_precision, stats.ac_precision),
            "ac_iterations": stats.ac_iterations,
            "autotune": ("off: fixed blocks of 4 ports (the HBM budget)" if big else
                         "block width and Chebyshev degree (first Ad solve timed per candidate) and Ac's "
                         "aggregation strength (first Ac solve timed per candidate) picked in the warm-up"),
            "note": "host wall-clock of the phases of the last timed step (assembly and setup are mostly "
                    "enqueue time; the solve phase ends with the host copy of Z)"}
    # kernel-level figures from separate profiled steps (events around every
    # launch add overhead, so they stay out of the timed region above)
    _, _, kern = timed(dev, max(1, min(args.steps, 2)), profile=True)
    ms_e2e, _, _ = timed(pin, max(1, min(args.steps, 3)))
    # accuracy of this run's Z against the plain FP64 GPU method, and that
    # method's own speed (FP64 throughout, one port at a time), untimed above
    z_run = z.numpy().copy()
    zr = z_run.reshape(-1, 2)
    zc = zr[:, 0] + 1j * zr[:, 1]
    z_err = fp64_ms = None
    if not big:      # the plain method would take minutes at c5's size
        p64 = default_params(precision="fp64", batch=0, rtol=RTOL[args.config])
        step(dev, p64)
        zf = z.numpy().copy().reshape(-1, 2)
        z64c = zf[:, 0] + 1j * zf[:, 1]
        z_err = float(np.max(np.abs(zc - z64c)) / max(np.max(np.abs(z64c)), 1e-300))
        fp64_ms, _, _ = timed(dev, 1, prm=p64) if args.precision == "mixed" or args.batch else (ms, 0, None)
    units = d.num_ports * d.nfreq
    value = whole_job_value(units, world, ms)
    e2e = whole_job_value(units, world, ms_e2e)
    h2d = sum(int(pin[k].numel() * pin[k].element_size()) for k in pin)
    d2h = int(z.numel() * z.element_size())
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak_gbs = peaks.get("hbm_gbs", 6800.0)
    k_ms, k_bytes, k_n, b_ms, b_bytes, b_n = kern
    achieved_all = (k_bytes / (k_ms / 1e3)) / 1e9 if k_ms > 0 else None
    # the fine-level operator's launches in the working precision of the
    # preconditioned solves: the largest row class that launched (>= 1M rows
    # for c2 and c4; c3's Ad has fewer rows)
    base = 0 if args.precision == "mixed" else 4
    fi = next((base + q for q in (3, 2, 1, 0) if b_n[base + q]), base + 3)
    row_class = ("rows<64k", "rows<256k", "rows<1M", "rows>=1M")[fi - base]
    f_ms, f_bytes, f_n = b_ms[fi], b_bytes[fi], b_n[fi]
    achieved = (f_bytes / (f_ms / 1e3)) / 1e9 if f_ms > 0 else None
    traffic = None
    tf = os.path.join(ROOT, "profiles", "spmm_traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get(f"{args.config}_{args.precision}_bytes_per_launch")
        except Exception:
            traffic = None
    # S v by the matrix-free curl-curl stencil against the assembled CSR (the
    # full-wave mode's product), device-resident vectors, 10 products each
    from gds2para_gb300 import api as _api
    stiff = None
    if rank == 0:
        with _api.FdtdMesh(d) as _m:
            _api.generateStiff(_m)
            nS = d.N_edge - _m.sizes().bden
            xs = np.random.default_rng(3).normal(size=nS)
            ys, t_mf = _api.stiffApply(_m, xs, matrix_free=True, reps=10)
            yc, t_csr = _api.stiffApply(_m, xs, matrix_free=False, reps=10)
            nnzS = _m.sizes().leng_S
        stiff = {"matrix_free_ms": t_mf, "csr_ms": t_csr, "speedup": t_csr / t_mf if t_mf > 0 else None,
                 "rows": int(nS), "csr_entries": int(nnzS),
                 "csr_algorithmic_GBps": (12.0 * nnzS + 24.0 * nS) / (t_csr / 1e3) / 1e9 if t_csr > 0 else None,
                 "max_rel_diff": float(np.abs(ys - yc).max() / max(np.abs(yc).max(), 1e-300)),
                 "what": "y = S x over the non-PEC edges: TMA-tiled stencil (face circulations, then edge sums) "
                         "vs the assembled CSR (12 bytes per entry); averages of 10 products"}
    # conductor marking, numbering and ports on the GPU (g2p_mesh_mark), from
    # host boxes to host arrays, against the host generator's time
    gpu_mesh_s = None
    if not big:
        _api.meshAndMark(lay_cfg)
        t0 = time.perf_counter()
        _api.meshAndMark(lay_cfg)
        gpu_mesh_s = time.perf_counter() - t0
    # network stage after the extraction: Z -> S on the GPU (g2p_convert_param,
    # host arrays in and out) and the two writers
    import tempfile
    para = _api.Parasitics(np.full(d.num_ports, 50.0))
    para.saveNetworkParam("Z", d.freqs(), zc)
    para.convertParam("S")
    para.saveNetworkParam("Z", d.freqs(), zc)
    t0 = time.perf_counter()
    para.convertParam("S")
    conv_s = time.perf_counter() - t0
    with tempfile.TemporaryDirectory() as td:
        t0 = time.perf_counter()
        _api.dumpCITI(os.path.join(td, "z.citi"), para, WORKLOAD[args.config][:16])
        citi_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        _api.dumpTouchstone(os.path.join(td, "z.snp"), para, WORKLOAD[args.config][:16])
        ts_s = time.perf_counter() - t0
    srt = sorted(step_ms)
    pct = lambda q: srt[min(len(srt) - 1, int(round(q * (len(srt) - 1))))] if srt else None
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded layout generator; no dataset)",
        "config": {"workload": WORKLOAD[args.config], "config": args.config, "precision": args.precision,
                   "batch": bool(args.batch), "ports": d.num_ports, "nfreq": d.nfreq,
                   "rtol": RTOL[args.config], "l2": "inputs larger than L2 (>129 MB per step)",
                   "parallelism": f"replicas x{world}",
                   "sizes": {"N_edge": d.N_edge, "N_node": d.N_node, "leng_S": stats.sizes.leng_S,
                             "leng_v0d": stats.sizes.leng_v0d, "leng_v0c": stats.sizes.leng_v0c,
                             "nnz_ad": stats.sizes.nnz_ad, "nnz_ac": stats.sizes.nnz_ac},
                   "last_step": last},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": ms_e2e},
        "linear_solves_per_s": world * 3 * d.num_ports / (ms / 1e3),
        "linear_solves": {"per_job": 3 * d.num_ports,
                          "what": "the V0 path's linear solves: Ad, Ac, Ad per port (frequency-independent "
                                  "right-hand sides; frequencies after the first are the f0/f rescale)",
                          "e2e_per_s": world * 3 * d.num_ports / (ms_e2e / 1e3)},
        "gpu_launches": int(launches),
        "mesher": {"gpu_ms": 1e3 * gpu_mesh_s if gpu_mesh_s is not None else None,
                   "host_generator_ms": 1e3 * host_mesh_s,
                   "what": "conductor marking, numbering and port edges (g2p_mesh_mark, host arrays in and out) "
                           "vs the numpy/scipy generator that restates meshAndMark/portSet"},
        "network": {"convert_z_to_s_ms": 1e3 * conv_s, "citi_write_ms": 1e3 * citi_s,
                    "touchstone_write_ms": 1e3 * ts_s,
                    "what": "convertParam('S') on the GPU and dumpCITI / dumpTouchstone of this run's Z"},
        "job_ms": {"p50": pct(0.5), "p99": pct(0.99), "per_step": step_ms},
        "stiffness_apply": stiff,
        "accuracy": {"z_rel_err_vs_fp64_gpu": z_err, "bound": 1e-6,
                     "note": "max |Z - Z_fp64| / max |Z_fp64| over all entries and frequencies"},
        "fp64_plain": ({"value": world * units / (fp64_ms / 1e3), "unit": UNIT, "ms_per_step": fp64_ms,
                        "what": "same job, FP64 AMG-FGMRES, one port at a time (batch 0)",
                        "speedup_of_this_run": fp64_ms / ms} if fp64_ms else
                       {"value": None, "what": "not run at this size"}),
        "clocks": clk,
        "roofline": {"bound": "hbm",
                     "kernel": ("k_spmm_sell<f32>" if args.precision == "mixed" else "k_spmm_sell<f64>") +
                               ": sparse matrix x block of right-hand sides on the fine-level Ad "
                               f"(operators of {row_class})",
                     "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                     "frac": (achieved / peak_gbs) if achieved else None, "traffic": traffic,
                     "launches": int(f_n), "avg_launch_us": 1e3 * f_ms / max(f_n, 1),
                     "algorithmic_bytes_per_launch": f_bytes / max(f_n, 1),
                     "all_levels": {"achieved": achieved_all, "launches": int(k_n),
                                    "avg_launch_us": 1e3 * k_ms / max(k_n, 1),
                                    "frac": (achieved_all / peak_gbs) if achieved_all else None},
                     "buckets": {f"{p}{nm}": [b_n[o + q], b_ms[o + q], b_bytes[o + q]]
                                 for o, p in ((0, "f32 "), (4, "f64 "))
                                 for q, nm in enumerate(("rows<64k", "rows<256k", "rows<1M", "rows>=1M")) if b_n[o + q]},
                     "bucket_fields": "launches, ms, algorithmic bytes",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback 6.8 TB/s"},
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = ({"value": None, "kind": "port", "cores": 1,
                                "sample": "CPU baseline infeasible at this size (memory)"} if big
                               else cpu_baseline(d, args, RTOL[args.config]))
    if world > 1:
        torch.distributed.destroy_process_group()
    return out, rank


def c4_jobs(n=200, seed=1004):
    """The served workload: seeded random Manhattan layouts of mixed sizes,
    sides log-uniform in 64..1024 nodes, nz in {8, 16, 32} (2, 3 or 4 metal
    layers), 1..16 ports and 1..32 frequency points."""
    from gds2para_gb300 import layout
    rng = np.random.default_rng(seed)
    jobs = []
    while len(jobs) < n:
        side = int(round(np.exp(rng.uniform(np.log(64), np.log(1024)))))
        nz = int(rng.choice([8, 16, 32]))
        ports = int(rng.integers(1, 17))
        nfreq = int(rng.integers(1, 33))
        try:
            lay = layout.manhattan(nx=side, ny=side, nz=nz, n_metal={8: 2, 16: 3, 32: 4}[nz],
                                   wires_per_layer=max(8, side // 8), n_ports=ports, seed=int(rng.integers(1 << 30)),
                                   lmin=max(6, side // 16), lmax=max(12, side // 3), freq_start=1e8, freq_end=1e10,
                                   freq_unit=1.0, nfreq=nfreq, freq_scale=0 if nfreq > 1 else 1)
            jobs.append(layout.build(lay))
        except (ValueError, RuntimeError):
            continue
    return jobs


def run_c4(args):
    """Continuous batching: jobs arrive (Poisson) while others run; the
    service admits them by memory footprint and runs up to 8 at once."""
    import torch
    from gds2para_gb300 import api
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    jobs = c4_jobs()
    params = api.default_params(precision=args.precision, batch=args.batch, rtol=RTOL["c4"])
    units = sum(d.num_ports * d.nfreq for d in jobs)
    budget = 150 << 30
    # serial pass (one job at a time; also the warm-up): capacity of the GPU
    with api.Server(budget, max_active=1) as srv:
        t0 = time.perf_counter()
        ids = [srv.submit(d, params) for d in jobs]
        for j in ids:
            srv.wait(j)
        serial_s = time.perf_counter() - t0
    # saturated pass: every job queued at once; throughput of the service
    clocks = Clocks(local)
    clocks.start()
    with api.Server(budget, max_active=8) as srv:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ids = [srv.submit(d, params) for d in jobs]
        sat = [srv.wait(j) for j in ids]
        torch.cuda.synchronize()
        sat_s = time.perf_counter() - t0
    clk = clocks.stop()
    # latency pass: Poisson arrivals at 0.8 x the serial capacity
    rate = 0.8 * len(jobs) / serial_s
    gaps = np.random.default_rng(4).exponential(1.0 / rate, size=len(jobs))
    with api.Server(budget, max_active=8) as srv:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ids = []
        for d, g in zip(jobs, gaps):
            time.sleep(g)
            ids.append(srv.submit(d, params))
        res = [srv.wait(j) for j in ids]
        torch.cuda.synchronize()
        span = time.perf_counter() - t0
    lat = sorted(t.total_ms for _, _, t in res)
    pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]
    overlapped = sum(1 for _, _, t in res if not t.ran_alone)
    out = {
        "metric": METRIC, "value": units / sat_s, "unit": UNIT, "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": 1e3 * sat_s, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic (seeded layout generator)",
        "config": {"workload": WORKLOAD["c4"], "config": "c4", "jobs": len(jobs), "port_freq_columns": units,
                   "arrival_rate_per_s": rate, "max_active": 8, "budget_bytes": budget,
                   "l2": "each job's inputs are resident only while it runs"},
        "job_ms": {"p50": pct(0.5), "p99": pct(0.99), "max": lat[-1],
                   "load": "Poisson arrivals at 0.8 x serial capacity", "arrival_span_s": span,
                   "jobs_overlapped": overlapped},
        "serial": {"value": units / serial_s, "seconds": serial_s, "what": "same jobs, one at a time"},
        "served_over_serial": serial_s / sat_s,
        "clocks": clk,
        "e2e": {"value": units / sat_s, "unit": UNIT, "note": "jobs submitted from host arrays; Z read back per job",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": int(sum(16 * d.nfreq * d.num_ports ** 2 for d in jobs))},
    }
    return out, rank


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


class CpuJobSteps:
    """The reference's path on the host, as the oracle's C restatement
    (oracle/pipeline.c, pinned bit-exact against the reference's own sources
    on the golden layouts; the reference's own build needs MKL, HYPRE and
    MPI, and its sources are not on the GPU machine).  One job is four steps,
    each timed in full:
      0  generateStiff and the V0d/Ad, V0c/Ac assembly (one thread: the
         reference's assembly is sequential);
      1  every port's first Ad solve,
      2  every port's Ac solve,
      3  every port's second Ad solve and Z,
    each solve with its own AMG setup as hypreSolve does, the ports spread
    over `threads` host threads.  A job's time is the sum of its four steps;
    nothing is extrapolated."""

    def __init__(self, d, rtol, threads):
        from oracle.harness import COracle
        self.d, self.threads = d, threads
        self.O = COracle()
        self.opts = self.O.default_opts(rtol=rtol, maxit=400, restart=30, reuse_setup=0)
        self.k, self.job, self.cur = 0, None, []
        self.jobs = []          # per complete job: the four step times (s)

    def step(self) -> float:
        t = time.perf_counter()
        if self.k == 0:
            self.O.stiffness(self.d)
            self.job = self.O.job(self.d)
        else:
            self.job.stage(self.k - 1, self.opts, self.threads)
        dt = time.perf_counter() - t
        self.cur.append(dt)
        self.k += 1
        if self.k == 4:
            self.jobs.append(self.cur)
            self.last = dict(iterations=self.job.iterations, max_rel_residual=self.job.max_rel_residual,
                             z=self.job.z())
            self.job.close()
            self.job, self.cur, self.k = None, [], 0
        return dt

    def summary(self, jobs=None):
        jobs = jobs if jobs is not None else self.jobs
        d = self.d
        js = [sum(j) for j in jobs]
        job_s = statistics.median(js)
        med = [statistics.median(j[i] for j in jobs) for i in range(4)]
        units = d.num_ports * d.nfreq
        return {"value": units / job_s, "unit": UNIT, "cores": self.threads, "kind": "port",
                "sample": (f"{len(jobs)} complete job(s) of the oracle/ C restatement on {self.threads} host "
                           f"thread(s) (ports in parallel, one thread each): generateStiff + assembly "
                           f"{med[0]:.2f} s, first Ad solves {med[1]:.2f} s, Ac solves {med[2]:.2f} s, second Ad "
                           f"solves {med[3]:.2f} s (AMG setup per solve, as hypreSolve); median job "
                           f"{job_s:.1f} s"),
                "job_seconds": job_s, "jobs_timed": len(jobs), "step_seconds_median": med,
                "linear_solves_per_s": 3 * d.num_ports / job_s,
                "iterations_last_job": self.last["iterations"],
                "max_rel_residual_last_job": self.last["max_rel_residual"]}


def cpu_baseline(d, args, rtol):
    """One complete job (four steps) on the host: the GPU line's baseline."""
    cj = CpuJobSteps(d, rtol, max(1, min(d.num_ports, host_threads())))
    for _ in range(4):
        cj.step()
    return cj.summary()


def run_reference(args):
    """The reference's CPU path (CpuJobSteps) on the host cores: warm-up and
    timed steps both run real job steps, four to a job; the value is the
    median over the jobs completed within the timed steps."""
    rank, world, _ = dist_info()
    if rank != 0:
        return None, rank
    from gds2para_gb300 import layout
    if args.config == "c4":
        return {"impl": "reference", "unavailable": "the reference extracts one layout per process and has no "
                                                    "service to time on a job stream"}, rank
    if args.config == "c5":
        return {"impl": "reference", "unavailable": "CPU baseline infeasible at this size (memory): the CPU "
                                                    "assembly of S alone needs about 68 GB of COO"}, rank
    d = layout.build(layout.config(args.config))
    rtol = RTOL[args.config]
    threads = max(1, min(d.num_ports, host_threads()))
    cj = CpuJobSteps(d, rtol, threads)
    for _ in range(args.warmup):
        cj.step()
    while cj.k != 0:            # timed steps start at a job boundary
        cj.step()
    n_before = len(cj.jobs)
    step_s = [cj.step() for _ in range(args.steps)]
    timed_jobs = cj.jobs[n_before:]
    if not timed_jobs:          # fewer than four timed steps: finish the job
        while cj.k != 0:
            cj.step()
        timed_jobs = cj.jobs[n_before:]
    cb = cj.summary(timed_jobs)
    v = cb["value"]
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(step_s), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded layout generator)",
           "config": {"workload": WORKLOAD[args.config], "config": args.config, "rtol": rtol,
                      "parallelism": f"{threads} host threads (ports in parallel)",
                      "step": "one quarter of a job: generateStiff + assembly, or one solve of every port"},
           "linear_solves_per_s": cb["linear_solves_per_s"],
           "cpu_baseline": cb,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return out, rank


def main():
    args = parse()
    if args.impl == "reference":
        out, rank = run_reference(args)
    elif args.config == "c4":
        out, rank = run_c4(args)
    else:
        out, rank = run_gb300(args)
    if rank == 0 and out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
