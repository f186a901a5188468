"""Python access to the two CPU oracles -- test infrastructure only.

* ``COracle``: ctypes binding of the C restatement (oracle/solver.c,
  oracle/pipeline.c), compiled into oracle/_build/liboracle.so.  It builds on
  any host with gcc, including the GPU machine.
* ``run_reference``: drives oracle/_ref/ref_pipeline, the reference's own
  sources compiled by oracle/build_ref.sh.  It exists only where the
  reference checkout does, so only fixture generation and the CPU-side pin
  tests use it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from typing import Dict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_pipeline")


def build_coracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("solver.c", "pipeline.c")]
    shim = os.path.join(HERE, "lapacke_shim.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    if not force and os.path.exists(LIB):
        mt = os.path.getmtime(LIB)
        if all(os.path.getmtime(s) <= mt for s in srcs + [hdr, shim]):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.basename(src) + f".{os.getpid()}.o")
        subprocess.check_call(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fPIC", "-c", src, "-o", obj])
        objs.append(obj)
    # the dense stand-ins of the full-wave path, built with the flags the
    # reference-compiled oracle uses for them (oracle/build_ref.sh)
    obj = os.path.join(BUILD, f"lapacke_shim.{os.getpid()}.o")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-c", shim, "-o", obj])
    objs.append(obj)
    subprocess.check_call(["g++", "-shared", "-o", tmp] + objs + ["-lm"])
    for o in objs:
        os.remove(o)
    os.replace(tmp, LIB)
    return LIB


class _Mesh(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("xn", C.c_void_p), ("yn", C.c_void_p), ("zn", C.c_void_p),
                ("stack_epsn", C.c_void_p), ("stack_sign", C.c_void_p),
                ("mark_node", C.c_void_p), ("mark_edge", C.c_void_p),
                ("num_cdt", C.c_int64), ("mark_port", C.c_void_p), ("cdt_return", C.c_void_p),
                ("num_ports", C.c_int32), ("port_side_ptr", C.c_void_p), ("side_edge_ptr", C.c_void_p),
                ("side_edges", C.c_void_p), ("side_area", C.c_void_p), ("side_dir", C.c_void_p),
                ("freq_start", C.c_double), ("freq_end", C.c_double), ("freq_unit", C.c_double),
                ("nfreq", C.c_int32), ("freq_scale", C.c_int32)]


class _Csr(C.Structure):
    _fields_ = [("n", C.c_int64), ("m", C.c_int64), ("ptr", C.POINTER(C.c_int64)),
                ("col", C.POINTER(C.c_int64)), ("val", C.POINTER(C.c_double))]


class _V0(C.Structure):
    _fields_ = [("nnz", C.c_int64), ("ncol", C.c_int64), ("row", C.POINTER(C.c_int64)),
                ("col", C.POINTER(C.c_int64)), ("val", C.POINTER(C.c_double)),
                ("aval", C.POINTER(C.c_double)), ("map", C.POINTER(C.c_int64))]


class SolverOpts(C.Structure):
    _fields_ = [("restart", C.c_int), ("maxit", C.c_int), ("rtol", C.c_double), ("pc_tol", C.c_double),
                ("pc_mod_sweeps", C.c_int), ("coarse_size", C.c_int), ("strength", C.c_double),
                ("reuse_setup", C.c_int), ("stop_after_solves", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("rel_residual", C.c_double), ("levels", C.c_int),
                ("converged", C.c_int)]


class ParaStats(C.Structure):
    _fields_ = [("leng_v0d", C.c_int64), ("leng_v0c", C.c_int64), ("nnz_ad", C.c_int64),
                ("nnz_ac", C.c_int64), ("bden", C.c_int64), ("solves", C.c_int),
                ("total_iterations", C.c_int), ("max_rel_residual", C.c_double),
                ("t_assembly", C.c_double), ("t_setup", C.c_double), ("t_solve", C.c_double),
                ("t_each", C.c_double * 3)]


def _arr(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class COracle:
    def __init__(self):
        self.lib = C.CDLL(build_coracle())
        L = self.lib
        L.g2po_index_maps.restype = C.c_int64
        L.g2po_solver_default_opts.argtypes = [C.POINTER(SolverOpts)]
        L.g2po_para_generator.argtypes = [C.POINTER(_Mesh), C.POINTER(SolverOpts), C.c_int,
                                          C.c_void_p, C.POINTER(ParaStats)]
        L.g2po_solve_coo.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                     C.c_void_p, C.POINTER(SolverOpts), C.POINTER(SolveStats)]

        L.g2po_job_create.restype = C.c_void_p
        L.g2po_job_create.argtypes = [C.POINTER(_Mesh), C.POINTER(ParaStats)]
        L.g2po_job_port_stage.argtypes = [C.c_void_p, C.c_int, C.POINTER(SolverOpts), C.POINTER(SolveStats),
                                          C.POINTER(C.c_double)]
        L.g2po_job_z.argtypes = [C.c_void_p, C.c_void_p]
        L.g2po_job_destroy.argtypes = [C.c_void_p]
        L.g2po_job_enable_vh.argtypes = [C.c_void_p]
        L.g2po_job_nr.argtypes = [C.c_void_p]
        L.g2po_job_nr.restype = C.c_int64
        L.g2po_find_vh.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int64)]
        L.g2po_job_vh_z.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.free.argtypes = [C.c_void_p]

    def _mesh(self, d):
        keep = {
            "xn": _arr(d.xn, np.float64), "yn": _arr(d.yn, np.float64), "zn": _arr(d.zn, np.float64),
            "se": _arr(d.stack_epsn, np.float64), "ss": _arr(d.stack_sign, np.float64),
            "mn": _arr(d.mark_node, np.int64), "me": _arr(d.mark_edge, np.int64),
            "mp": _arr(d.mark_port, np.int32), "cr": _arr(d.cdt_return, np.uint8),
            "psp": _arr(d.port_side_ptr, np.int32), "sep": _arr(d.side_edge_ptr, np.int64),
            "se2": _arr(d.side_edges, np.int64), "sa": _arr(d.side_area, np.float64),
            "sd": _arr(d.side_dir, np.int32),
        }
        p = lambda k: keep[k].ctypes.data
        m = _Mesh(d.nx, d.ny, d.nz, p("xn"), p("yn"), p("zn"), p("se"), p("ss"), p("mn"), p("me"),
                  d.num_cdt, p("mp"), p("cr"), d.num_ports, p("psp"), p("sep"), p("se2"), p("sa"), p("sd"),
                  d.freq_start, d.freq_end, d.freq_unit, d.nfreq, d.freq_scale)
        m._keep = keep
        return m

    def default_opts(self, **kw) -> SolverOpts:
        o = SolverOpts()
        self.lib.g2po_solver_default_opts(C.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o

    def index_maps(self, d):
        m = self._mesh(d)
        me = np.empty(d.N_edge, np.int64)
        pe = np.empty(d.N_edge, np.uint8)
        pn = np.empty(d.N_node, np.uint8)
        bden = self.lib.g2po_index_maps(C.byref(m), me.ctypes.data_as(C.c_void_p),
                                        pe.ctypes.data_as(C.c_void_p), pn.ctypes.data_as(C.c_void_p))
        return me, pe, pn, int(bden)

    def _take_csr(self, c):
        n = c.n
        nnz = c.ptr[n]
        out = (np.ctypeslib.as_array(c.ptr, (n + 1,)).copy(),
               np.ctypeslib.as_array(c.col, (max(nnz, 1),))[:nnz].copy(),
               np.ctypeslib.as_array(c.val, (max(nnz, 1),))[:nnz].copy())
        self.lib.g2po_csr_free(C.byref(c))
        return out

    def _take_v0(self, v, n_node):
        nnz = v.nnz
        f = lambda p, dt: np.ctypeslib.as_array(p, (max(nnz, 1),))[:nnz].copy()
        out = dict(row=f(v.row, None), col=f(v.col, None), val=f(v.val, None), aval=f(v.aval, None),
                   map=np.ctypeslib.as_array(v.map, (n_node,)).copy(), ncol=int(v.ncol))
        return out

    def stiffness(self, d):
        me, pe, pn, _ = self.index_maps(d)
        m = self._mesh(d)
        S = _Csr()
        self.lib.g2po_stiffness(C.byref(m), me.ctypes.data_as(C.c_void_p), pe.ctypes.data_as(C.c_void_p),
                                C.byref(S))
        return self._take_csr(S)

    def v0_and_laplacians(self, d):
        """V0d (+Ad) and V0c (+Ac) exactly as merge_v0d1/generateAd and
        merge_v0c/generateAc produce them."""
        me, pe, pn, _ = self.index_maps(d)
        m = self._mesh(d)
        out = {}
        for tag, fv, fa in (("d", self.lib.g2po_v0d, self.lib.g2po_ad), ("c", self.lib.g2po_v0c, self.lib.g2po_ac)):
            v = _V0()
            fv(C.byref(m), pn.ctypes.data_as(C.c_void_p), C.byref(v))
            A = _Csr()
            fa(C.byref(m), C.byref(v), C.byref(A))
            out["v0" + tag] = self._take_v0(v, d.N_node)
            self.lib.g2po_v0_free(C.byref(v))
            out["A" + tag] = self._take_csr(A)
        return out

    def para_generator(self, d, opts: SolverOpts = None, max_ports: int = 0):
        if opts is None:
            opts = self.default_opts(rtol=1e-12, maxit=3000, restart=50, reuse_setup=1)
        m = self._mesh(d)
        z = np.zeros(2 * d.nfreq * d.num_ports * d.num_ports, np.float64)
        st = ParaStats()
        self.lib.g2po_para_generator(C.byref(m), C.byref(opts), max_ports, z.ctypes.data_as(C.c_void_p),
                                     C.byref(st))
        zc = z[0::2] + 1j * z[1::2]
        return zc.reshape(d.nfreq, d.num_ports, d.num_ports), st

    def job(self, d):
        """The extraction as a job whose ports can run on several host
        threads (g2po_job_*); see OracleJob."""
        return OracleJob(self, d)

    def solve_csr(self, ptr, col, val, b, opts: SolverOpts = None):
        n = len(ptr) - 1
        rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(ptr))
        col = _arr(col, np.int64); val = _arr(val, np.float64); b = _arr(b, np.float64)
        x = np.zeros(n)
        if opts is None:
            opts = self.default_opts(rtol=1e-12, maxit=3000, restart=50)
        st = SolveStats()
        self.lib.g2po_solve_coo(rows.ctypes.data, col.ctypes.data, val.ctypes.data, len(col), b.ctypes.data,
                                n, x.ctypes.data, C.byref(opts), C.byref(st))
        return x, st


def run_reference(d, workdir: str = None, skip_stiff: bool = False, skip_para: bool = False) -> Dict[str, np.ndarray]:
    """Runs the reference-compiled pipeline on a layout and returns its dumps."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError("oracle/_ref/ref_pipeline missing: run oracle/build_ref.sh")
    own = workdir is None
    td = tempfile.mkdtemp(prefix="g2pref_") if own else workdir
    ind = os.path.join(td, "in")
    outd = os.path.join(td, "out")
    os.makedirs(ind, exist_ok=True)
    os.makedirs(outd, exist_ok=True)
    nboxes = int(d.mark_edge_raw[: d.N_edge_s].max()) - 1
    meta = dict(nx=d.nx, ny=d.ny, nz=d.nz, freqStart=d.freq_start, freqEnd=d.freq_end, freqUnit=d.freq_unit,
                nfreq=d.nfreq, freqScale=d.freq_scale, numBoxes=nboxes, numPorts=d.num_ports,
                skipStiff=int(skip_stiff), skipPara=int(skip_para))
    with open(os.path.join(ind, "meta.txt"), "w") as f:
        for k, v in meta.items():
            f.write(f"{k} {v!r}\n")
    for name, a, dt in (("xn.f64", d.xn, np.float64), ("yn.f64", d.yn, np.float64), ("zn.f64", d.zn, np.float64),
                        ("stack_epsn.f64", d.stack_epsn, np.float64), ("stack_sign.f64", d.stack_sign, np.float64),
                        ("mark_edge_raw.i64", d.mark_edge_raw, np.int64),
                        ("mark_node_raw.i64", d.mark_node_raw, np.int64)):
        _arr(a, dt).tofile(os.path.join(ind, name))
    rows = []
    for p in range(d.num_ports):
        for s in range(d.port_side_ptr[p], d.port_side_ptr[p + 1]):
            rows.append([p] + list(d.side_coords[s]) + [d.side_dir[s]])
    np.array(rows, np.float64).tofile(os.path.join(ind, "ports.f64"))
    r = subprocess.run([REF_BIN, ind, outd], cwd=td, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_pipeline failed ({r.returncode}): {r.stderr[-2000:]}")
    out: Dict[str, np.ndarray] = {}
    ext = {"i64": np.int64, "f64": np.float64, "i32": np.int32, "u8": np.uint8, "c128": np.float64}
    for fn in os.listdir(outd):
        stem, _, e = fn.rpartition(".")
        if e in ext:
            a = np.fromfile(os.path.join(outd, fn), ext[e])
            if e == "c128":
                a = a[0::2] + 1j * a[1::2]
            out[stem] = a
    with open(os.path.join(outd, "meta_out.txt")) as f:
        for line in f:
            k, v = line.split()
            out[k] = int(v)
    out["_log"] = r.stderr
    return out


class OracleJob:
    """One V0 extraction on the host: the assembly happens at construction
    (index maps, V0d/Ad, V0c/Ac); stage(k, threads) then runs solve k of
    every port (0: Ad, 1: Ac, 2: Ad, each with its own AMG setup as
    hypreSolve does), the ports spread over host threads (ctypes releases
    the GIL during each call).  z() gives Z once stage 2 has run."""

    def __init__(self, oracle: "COracle", d):
        self.O, self.d = oracle, d
        self.m = oracle._mesh(d)
        self.st = ParaStats()
        self.h = oracle.lib.g2po_job_create(C.byref(self.m), C.byref(self.st))
        self.iterations = 0
        self.max_rel_residual = 0.0

    def stage(self, k: int, opts: SolverOpts, threads: int = 1):
        import concurrent.futures as cf

        def one(p):
            ss, ts = SolveStats(), C.c_double()
            rc = self.O.lib.g2po_job_port_stage(self.h, p, C.byref(opts), C.byref(ss), C.byref(ts))
            if rc != 0:
                raise RuntimeError(f"g2po_job_port_stage(port {p}, stage {k}) failed")
            return ss.iterations, ss.rel_residual

        ports = range(self.d.num_ports)
        if threads <= 1:
            res = [one(p) for p in ports]
        else:
            with cf.ThreadPoolExecutor(max_workers=threads) as ex:
                res = list(ex.map(one, ports))
        for it, rel in res:
            self.iterations += it
            self.max_rel_residual = max(self.max_rel_residual, rel)

    def enable_vh(self):
        """Keep each port's V0 fields for the full-wave path and build S
        (call before any stage)."""
        if self.O.lib.g2po_job_enable_vh(self.h) != 0:
            raise RuntimeError("g2po_job_enable_vh failed")

    def find_vh(self, k: int):
        """find_Vh(k): returns Vh as an (nr, mm) complex array."""
        p = C.POINTER(C.c_double)()
        mm = C.c_int64()
        self.O.lib.g2po_find_vh(self.h, k, C.byref(p), C.byref(mm))
        nr = int(self.O.lib.g2po_job_nr(self.h))
        a = np.ctypeslib.as_array(p, (max(2 * nr * mm.value, 1),))[: 2 * nr * mm.value].copy()
        self.O.lib.free(p)
        vh = (a[0::2] + 1j * a[1::2]).reshape(mm.value, nr).T
        return vh

    def vh_z(self, vh):
        """The Vh-corrected Z of every port and frequency: (z_vh, z_ref),
        each (nfreq, P, P) complex with z[f, p, q] = response at port q to
        port p (sys->x's order before any transposition); z_ref carries the
        reference's first-frequency start from the V0 Z."""
        d = self.d
        nr, mm = vh.shape
        buf = np.empty(2 * nr * mm)
        buf[0::2] = vh.T.reshape(-1).real
        buf[1::2] = vh.T.reshape(-1).imag
        zv = np.zeros(2 * d.nfreq * d.num_ports ** 2)
        zf = np.zeros_like(zv)
        rc = self.O.lib.g2po_job_vh_z(self.h, buf.ctypes.data, mm, zv.ctypes.data, zf.ctypes.data)
        if rc != 0:
            raise RuntimeError("g2po_job_vh_z failed (run every port's stages with enable_vh first)")
        shape = (d.nfreq, d.num_ports, d.num_ports)
        return (zv[0::2] + 1j * zv[1::2]).reshape(shape), (zf[0::2] + 1j * zf[1::2]).reshape(shape)

    def z(self):
        d = self.d
        z = np.zeros(2 * d.nfreq * d.num_ports * d.num_ports, np.float64)
        self.O.lib.g2po_job_z(self.h, z.ctypes.data_as(C.c_void_p))
        zc = z[0::2] + 1j * z[1::2]
        return zc.reshape(d.nfreq, d.num_ports, d.num_ports)

    def close(self):
        if self.h:
            self.O.lib.g2po_job_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
