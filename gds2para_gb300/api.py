"""The reference's entry points on the extraction path, over the C ABI.

    FdtdMesh        <- fdtdMesh (src/fdtd.hpp:182), filled from a MeshDesc
    generateStiff   <- generateStiff (src/generateStiff.cpp:6)
    hypreSolve      <- hypreSolve (src/hypreSolve.cpp:9)
    paraGenerator   <- paraGenerator (src/matrixCon.cpp:11)

Names and argument meanings follow the reference; unlike it, failures raise
G2PError instead of being ignored.  All compute runs in libgds2para_gb300.so
on the GPU.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np

from . import _lib
from ._lib import ExtractStats, G2PError, SolverParams, SolveStats, Sizes, check
from .layout import MeshDesc


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def default_params(parity: bool = False, **kw) -> SolverParams:
    """parity=True gives hypreSolve's settings (KDim 10, 100 iterations,
    rtol 1e-4; src/hypreSolver.h:7-11); otherwise FP64 at rtol 1e-10."""
    p = SolverParams()
    _lib.load().g2p_default_params(C.byref(p), 1 if parity else 0)
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = {"fp64": _lib.G2P_PREC_FP64, "mixed": _lib.G2P_PREC_MIXED, "fp64_pc32": _lib.G2P_PREC_FP64_PC32}[v]
        setattr(p, k, v)
    return p


class FdtdMesh:
    """Device-resident mesh: the fdtdMesh fields the path reads."""

    def __init__(self, desc: MeshDesc):
        L = _lib.load()
        self.desc = desc
        self._keep = dict(
            xn=_c(desc.xn, np.float64), yn=_c(desc.yn, np.float64), zn=_c(desc.zn, np.float64),
            se=_c(desc.stack_epsn, np.float64), ss=_c(desc.stack_sign, np.float64),
            mn=_c(desc.mark_node, np.int64), me=_c(desc.mark_edge, np.int64),
            mp=_c(desc.mark_port, np.int32), cr=_c(desc.cdt_return, np.uint8),
            psp=_c(desc.port_side_ptr, np.int32), sep=_c(desc.side_edge_ptr, np.int64),
            sed=_c(desc.side_edges, np.int64), sa=_c(desc.side_area, np.float64), sd=_c(desc.side_dir, np.int32))
        k = self._keep
        p = lambda n: k[n].ctypes.data
        self._desc = _lib.MeshDescC(desc.nx, desc.ny, desc.nz, p("xn"), p("yn"), p("zn"), p("se"), p("ss"),
                                    p("mn"), p("me"), desc.num_cdt, p("mp"), p("cr"), desc.num_ports, p("psp"),
                                    p("sep"), p("sed"), p("sa"), p("sd"), desc.freq_start, desc.freq_end,
                                    desc.freq_unit, desc.nfreq, desc.freq_scale)
        h = C.c_void_p()
        check(L.g2p_mesh_create(C.byref(self._desc), C.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().g2p_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- index maps (setMapEdge, fdtd.hpp:1508) ----
    def index_maps(self) -> Tuple[np.ndarray, int]:
        bden = C.c_int64()
        me = np.empty(self.desc.N_edge, np.int64)
        check(_lib.load().g2p_index_maps(self.handle, C.byref(bden), me.ctypes.data))
        return me, int(bden.value)

    def sizes(self) -> Sizes:
        s = Sizes()
        check(_lib.load().g2p_mesh_sizes(self.handle, C.byref(s)))
        return s

    def export_stiff(self):
        n = self.sizes().leng_S
        r, c, v = np.empty(n, np.int64), np.empty(n, np.int64), np.empty(n, np.float64)
        check(_lib.load().g2p_export_stiff(self.handle, r.ctypes.data, c.ctypes.data, v.ctypes.data))
        return r, c, v

    def assemble_v0(self) -> Sizes:
        s = Sizes()
        check(_lib.load().g2p_assemble_v0(self.handle, C.byref(s)))
        return s

    def export_v0(self, which: str):
        w = {"d": 0, "c": 1}[which]
        s = self.sizes()
        n = s.nnz_v0d if w == 0 else s.nnz_v0c
        r, c = np.empty(n, np.int64), np.empty(n, np.int64)
        v, a = np.empty(n, np.float64), np.empty(n, np.float64)
        mp = np.empty(self.desc.N_node, np.int64)
        check(_lib.load().g2p_export_v0(self.handle, w, r.ctypes.data, c.ctypes.data, v.ctypes.data, a.ctypes.data,
                                        mp.ctypes.data))
        return dict(row=r, col=c, val=v, aval=a, map=mp, ncol=s.leng_v0d if w == 0 else s.leng_v0c)

    def export_laplacian(self, which: str):
        w = {"d": 0, "c": 1}[which]
        s = self.sizes()
        n = s.nnz_ad if w == 0 else s.nnz_ac
        r, c, v = np.empty(n, np.int64), np.empty(n, np.int64), np.empty(n, np.float64)
        check(_lib.load().g2p_export_laplacian(self.handle, w, r.ctypes.data, c.ctypes.data, v.ctypes.data))
        return r, c, v


def readGDSII(path, ignore_layers=()):
    """The conductor polygons of a GDSII file's top cell, flattened as the
    reference's AsciiDataBase::saveToMesh flattens them (limboint.hpp:2823):
    returns (layer[npoly], vert_ptr[npoly + 1], x[nvert], y[nvert]) with
    coordinates in metres.  Host code; no GPU needed."""
    L = _lib.load()
    ign = np.ascontiguousarray(np.asarray(ignore_layers, np.int32))
    h = C.c_void_p()
    check(L.g2p_gdsii_read(str(path).encode(), ign.ctypes.data if ign.size else None, int(ign.size), C.byref(h)))
    try:
        npoly, nvert = C.c_int64(), C.c_int64()
        check(L.g2p_polygons_size(h, C.byref(npoly), C.byref(nvert)))
        layer = np.empty(npoly.value, np.int32)
        vptr = np.empty(npoly.value + 1, np.int64)
        x, y = np.empty(nvert.value), np.empty(nvert.value)
        check(L.g2p_polygons_get(h, layer.ctypes.data, vptr.ctypes.data, x.ctypes.data, y.ctypes.data))
    finally:
        L.g2p_polygons_free(h)
    return layer, vptr, x, y


def meshGrid(limits, polygons, port_sides, stack):
    """The grid lines of the reference's meshAndMark (mesh.cpp:5-330).
    limits: (xlim1, xlim2, ylim1, ylim2, zlim1, zlim2); polygons: (layer,
    vert_ptr, x, y) as readGDSII returns them; port_sides: (n, 6) rows
    x1 y1 z1 x2 y2 z2; stack: (m, 4) rows z_begin z_end eps_r sigma; metres.
    Returns xn, yn, zn, stack_epsn, stack_sign."""
    L = _lib.load()
    lim = _c(limits, np.float64)
    _, vptr, x, y = polygons
    vptr, x, y = _c(vptr, np.int64), _c(x, np.float64), _c(y, np.float64)
    sides = _c(np.asarray(port_sides, np.float64).reshape(-1, 6), np.float64)
    st = _c(np.asarray(stack, np.float64).reshape(-1, 4), np.float64)
    counts = np.zeros(3, np.int64)
    cap_xy = max(16, 4 * (len(x) + 2 * len(sides)) + 1024)
    cap_z = 2 * (len(st) + len(sides)) + 1
    for _ in range(2):
        xn, yn, zn = np.empty(cap_xy), np.empty(cap_xy), np.empty(cap_z)
        epsn, sign = np.empty(cap_z), np.empty(cap_z)
        rc = L.g2p_mesh_grid(lim.ctypes.data, len(vptr) - 1, vptr.ctypes.data, x.ctypes.data, y.ctypes.data,
                             len(sides), sides.ctypes.data if len(sides) else None, len(st), st.ctypes.data, cap_xy,
                             cap_z, xn.ctypes.data, yn.ctypes.data, zn.ctypes.data, epsn.ctypes.data,
                             sign.ctypes.data, counts.ctypes.data)
        if rc == _lib.G2P_OK:
            nx, ny, nz = (int(v) for v in counts)
            return xn[:nx].copy(), yn[:ny].copy(), zn[:nz].copy(), epsn[:nz].copy(), sign[:nz].copy()
        if counts[0] > cap_xy or counts[1] > cap_xy:
            cap_xy = int(max(counts[0], counts[1]))
            continue
        check(rc)
    check(rc)


def generateStiff(sys: FdtdMesh) -> int:
    """generateStiff (src/generateStiff.cpp:6): builds S on the device and
    returns leng_S."""
    n = C.c_int64()
    check(_lib.load().g2p_generate_stiff(sys.handle, C.byref(n)))
    return int(n.value)


def hypreSolve(sys, ARowId, AColId, Aval, leng_A, bin, leng_v0, solution) -> int:
    """hypreSolve (src/hypreSolve.cpp:9) with the reference's settings.  `sys`
    is unused, as in the reference.  Writes `solution` in place; returns 0 on
    convergence and raises on failure (the reference returns 0 regardless)."""
    r = _c(ARowId, np.int64); c = _c(AColId, np.int64); v = _c(Aval, np.float64); b = _c(bin, np.float64)
    if not (isinstance(solution, np.ndarray) and solution.dtype == np.float64 and solution.flags.c_contiguous):
        raise TypeError("solution must be a contiguous float64 array")
    st = _lib.load().g2p_hypre_solve(r.ctypes.data, c.ctypes.data, v.ctypes.data, int(leng_A), b.ctypes.data,
                                     int(leng_v0), solution.ctypes.data)
    check(st, allow=(_lib.G2P_OK, _lib.G2P_ERR_NOT_CONVERGED))
    return 0


class Solver:
    """A reusable AMG-FGMRES solver over one matrix (row-sorted COO input)."""

    def __init__(self, rows, cols, vals, n, params: Optional[SolverParams] = None):
        self._r, self._c, self._v = _c(rows, np.int64), _c(cols, np.int64), _c(vals, np.float64)
        self.n = int(n)
        h = C.c_void_p()
        p = params if params is not None else default_params()
        check(_lib.load().g2p_solver_create(self._r.ctypes.data, self._c.ctypes.data, self._v.ctypes.data,
                                            len(self._v), self.n, C.byref(p), C.byref(h)))
        self.handle = h

    def solve(self, b: np.ndarray, allow_unconverged: bool = False):
        b = np.asarray(b, np.float64)
        k = 1 if b.ndim == 1 else b.shape[1]
        bc = np.asfortranarray(b.reshape(self.n, k))
        x = np.zeros((self.n, k), np.float64, order="F")
        st = SolveStats()
        rc = _lib.load().g2p_solver_solve(self.handle, bc.ctypes.data, x.ctypes.data, k, C.byref(st))
        check(rc, allow=(_lib.G2P_OK, _lib.G2P_ERR_NOT_CONVERGED) if allow_unconverged else (_lib.G2P_OK,))
        return (x[:, 0] if b.ndim == 1 else x), st

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().g2p_solver_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def paraGenerator(sys: FdtdMesh, params: Optional[SolverParams] = None):
    """paraGenerator (src/matrixCon.cpp:11): returns (Z, stats) with Z shaped
    (nfreq, P, P) in sys->x's storage order: Z[f].ravel()[q + P*p] is the
    response at port q to a unit source at port p for f = 0; later
    frequencies are stored transposed, as print_z_V0 leaves them."""
    d = sys.desc
    z = np.zeros(2 * d.nfreq * d.num_ports * d.num_ports, np.float64)
    st = ExtractStats()
    p = params if params is not None else default_params()
    rc = _lib.load().g2p_para_generator(sys.handle, C.byref(p), z.ctypes.data, C.byref(st))
    check(rc)
    zc = z[0::2] + 1j * z[1::2]
    return zc.reshape(d.nfreq, d.num_ports, d.num_ports), st


def stiffApply(sys: FdtdMesh, x: np.ndarray, matrix_free: bool = True, reps: int = 1):
    """y = S x over the non-PEC edges, by the matrix-free curl-curl stencil
    or the assembled CSR; returns (y, device ms per product)."""
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    ms = C.c_double()
    check(_lib.load().g2p_stiff_apply(sys.handle, 1 if matrix_free else 0, int(reps), x.ctypes.data, y.ctypes.data,
                                      C.byref(ms)))
    return y, ms.value


def findVh(sys: FdtdMesh, k: int = 1000) -> np.ndarray:
    """find_Vh (src/fdtd.hpp:3577-3859): k Arnoldi steps on the device, the
    Hessenberg eigenproblem on the host; returns Vh, complex (N, leng_Vh)
    over the non-PEC edges.  generateStiff must have run."""
    L = _lib.load()
    mm = C.c_int64()
    check(L.g2p_find_vh(sys.handle, int(k), C.byref(mm)))
    n = int(sys.desc.N_edge - sys.sizes().bden)
    v = np.zeros(2 * n * int(mm.value), np.float64)
    if mm.value:
        check(L.g2p_export_vh(sys.handle, v.ctypes.data))
    return (v[0::2] + 1j * v[1::2]).reshape(int(mm.value), n).T


def setVh(sys: FdtdMesh, vh: np.ndarray) -> None:
    """Installs Vh, complex (N, leng_Vh), in place of findVh's (for reuse, or
    to run the correction stage on a Vh computed elsewhere)."""
    vh = np.asarray(vh, np.complex128)
    buf = np.empty(2 * vh.size, np.float64)
    buf[0::2] = vh.T.reshape(-1).real
    buf[1::2] = vh.T.reshape(-1).imag
    if vh.shape[0] != sys.desc.N_edge - sys.sizes().bden:
        raise ValueError("Vh must have one row per non-PEC edge")
    check(_lib.load().g2p_set_vh(sys.handle, buf.ctypes.data, int(vh.shape[1])))


def paraGeneratorVh(sys: FdtdMesh, params: Optional[SolverParams] = None, k: int = 1000):
    """paraGenerator's full-wave path (src/matrixCon.cpp:609-805 with
    Construct_Z_V0_Vh, src/fdtd.hpp:4133-4170): returns (Z_vh, Z_v0, stats).
    Z_vh is (nfreq, P, P) with Z_vh[f].ravel()[q + P*p] the response at port
    q to port p, not rescaled or transposed; Z_v0 is paraGenerator's Z.
    Runs findVh(sys, k) first if it has not run."""
    d = sys.desc
    nz = d.nfreq * d.num_ports * d.num_ports
    zvh = np.zeros(2 * nz, np.float64)
    zv0 = np.zeros(2 * nz, np.float64)
    st = ExtractStats()
    p = params if params is not None else default_params()
    check(_lib.load().g2p_para_generator_vh(sys.handle, C.byref(p), int(k), zvh.ctypes.data, zv0.ctypes.data,
                                            C.byref(st)))
    shape = (d.nfreq, d.num_ports, d.num_ports)
    return (zvh[0::2] + 1j * zvh[1::2]).reshape(shape), (zv0[0::2] + 1j * zv0[1::2]).reshape(shape), st


def hessenbergEigenvalues(h: np.ndarray) -> np.ndarray:
    """Eigenvalues of a real upper Hessenberg matrix with the library's
    dhseqr stand-in (Francis double-shift QR); complex array of length n."""
    a = np.asfortranarray(np.asarray(h, np.float64))
    n = a.shape[0]
    wr = np.zeros(n, np.float64)
    wi = np.zeros(n, np.float64)
    check(_lib.load().g2p_hessenberg_eig(n, a.ctypes.data, wr.ctypes.data, wi.ctypes.data))
    return wr + 1j * wi


__all__ = ["FdtdMesh", "generateStiff", "hypreSolve", "paraGenerator", "Solver", "Server", "meshAndMark",
           "readSimInput", "polygonZ", "meshAndMarkPolygons", "layoutFromGDS",
           "stiffApply", "findVh", "setVh", "paraGeneratorVh", "hessenbergEigenvalues",
           "Parasitics", "dumpTouchstone", "dumpCITI", "dumpXyce", "dumpSPEF", "default_params", "G2PError"]


class Server:
    """Extraction service over the C ABI (g2p_server_*): jobs are queued,
    admitted onto the GPU while their device-memory estimate fits the budget
    and fewer than max_active run, and run concurrently, each on its own
    stream.  No counterpart in the reference, which extracts one layout per
    process."""

    def __init__(self, mem_budget_bytes: int, max_active: int = 4):
        h = C.c_void_p()
        check(_lib.load().g2p_server_create(int(mem_budget_bytes), int(max_active), C.byref(h)))
        self.handle = h
        self._pending = {}

    def submit(self, desc: MeshDesc, params: Optional[SolverParams] = None) -> int:
        keep, cdesc = _pack_desc(desc)      # copied by the library before submit returns
        job = C.c_int64()
        check(_lib.load().g2p_server_submit(self.handle, C.byref(cdesc), C.byref(params) if params else None,
                                            C.byref(job)))
        self._pending[job.value] = desc
        return job.value

    def wait(self, job: int, allow_unconverged: bool = False):
        desc = self._pending.pop(job)
        z = np.zeros(2 * desc.nfreq * desc.num_ports * desc.num_ports)
        st = ExtractStats()
        t = _lib.JobTimes()
        allow = (_lib.G2P_OK, _lib.G2P_ERR_NOT_CONVERGED) if allow_unconverged else (_lib.G2P_OK,)
        check(_lib.load().g2p_server_wait(self.handle, job, z.ctypes.data, C.byref(st), C.byref(t)), allow)
        zc = z[0::2] + 1j * z[1::2]
        return zc.reshape(desc.nfreq, desc.num_ports, desc.num_ports), st, t

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().g2p_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def _pack_desc(desc: MeshDesc):
    keep = dict(
        xn=_c(desc.xn, np.float64), yn=_c(desc.yn, np.float64), zn=_c(desc.zn, np.float64),
        se=_c(desc.stack_epsn, np.float64), ss=_c(desc.stack_sign, np.float64),
        mn=_c(desc.mark_node, np.int64), me=_c(desc.mark_edge, np.int64),
        mp=_c(desc.mark_port, np.int32), cr=_c(desc.cdt_return, np.uint8),
        psp=_c(desc.port_side_ptr, np.int32), sep=_c(desc.side_edge_ptr, np.int64),
        sed=_c(desc.side_edges, np.int64), sa=_c(desc.side_area, np.float64), sd=_c(desc.side_dir, np.int32))
    p = lambda n: keep[n].ctypes.data
    cdesc = _lib.MeshDescC(desc.nx, desc.ny, desc.nz, p("xn"), p("yn"), p("zn"), p("se"), p("ss"),
                           p("mn"), p("me"), desc.num_cdt, p("mp"), p("cr"), desc.num_ports, p("psp"),
                           p("sep"), p("sed"), p("sa"), p("sd"), desc.freq_start, desc.freq_end,
                           desc.freq_unit, desc.nfreq, desc.freq_scale)
    return keep, cdesc


def meshAndMark(layout) -> dict:
    """Conductor marking, numbering and port edges of a Layout on the GPU
    (g2p_mesh_mark: findInsideCond, the conductor labelling and portSet of
    src/mesh.cpp).  Returns the fdtdMesh fields as numpy arrays."""
    L = _lib.load()
    nx, ny, nz = layout.nx, layout.ny, layout.nz
    px, py, pz = layout.pitch
    xn = np.arange(nx, dtype=np.float64) * px
    yn = np.arange(ny, dtype=np.float64) * py
    zn = np.arange(nz, dtype=np.float64) * pz
    boxes = (_lib.BoxC * max(1, len(layout.boxes)))(*[_lib.BoxC(b.x0, b.x1, b.y0, b.y1, b.z0, b.z1)
                                                      for b in layout.boxes])
    sides, sptr = [], [0]
    for port in layout.ports:
        for s in port:
            sides.append(_lib.PortSideC(*s.supply, *s.ret))
        sptr.append(len(sides))
    nsides = len(sides)
    csides = (_lib.PortSideC * max(1, nsides))(*sides)
    sptr = np.array(sptr, np.int32)
    N_node = nx * ny * nz
    Ns = (ny - 1) * nx + (nx - 1) * ny
    N_edge = Ns * nz + nx * ny * (nz - 1)
    mark_node = np.zeros(N_node, np.int64)
    mark_edge = np.zeros(N_edge, np.int64)
    ncdt = C.c_int64()
    max_cdt = len(layout.boxes) + 2
    mark_port = np.zeros(max_cdt, np.int32)
    cdt_return = np.zeros(max_cdt, np.uint8)
    max_e = sum(abs(s.supply[0] - s.ret[0]) + abs(s.supply[1] - s.ret[1]) + abs(s.supply[2] - s.ret[2])
                for p in layout.ports for s in p) + 1
    side_edge_ptr = np.zeros(nsides + 1, np.int64)
    side_edges = np.zeros(max_e, np.int64)
    side_area = np.zeros(max(1, nsides), np.float64)
    side_dir = np.zeros(max(1, nsides), np.int32)
    check(L.g2p_mesh_mark(nx, ny, nz, xn.ctypes.data, yn.ctypes.data, zn.ctypes.data, C.cast(boxes, C.c_void_p),
                          len(layout.boxes), len(layout.ports), sptr.ctypes.data, C.cast(csides, C.c_void_p),
                          mark_node.ctypes.data, mark_edge.ctypes.data, C.byref(ncdt), mark_port.ctypes.data,
                          cdt_return.ctypes.data, max_cdt, side_edge_ptr.ctypes.data, side_edges.ctypes.data,
                          max_e, side_area.ctypes.data, side_dir.ctypes.data))
    n = ncdt.value
    return dict(mark_node=mark_node, mark_edge=mark_edge, num_cdt=n, mark_port=mark_port[:n],
                cdt_return=cdt_return[:n], side_edge_ptr=side_edge_ptr,
                side_edges=side_edges[:side_edge_ptr[-1]], side_area=side_area[:nsides], side_dir=side_dir[:nsides])


def readSimInput(path) -> dict:
    """The reference's .sim_input reader (SolverDataBase::readSimInput,
    src/solnoutclass.hpp:5412) as convertToFDTDMesh hands it on: limits and
    lengths in metres, the frequency sweep, the valid stack layers (rows z
    begin, z end, eps_r, sigma) with their GDSII numbers, and the ports
    (port_side_ptr, side_coords rows supply xyz + return xyz, side_dir).
    Host code; no GPU needed."""
    L = _lib.load()
    h = C.c_void_p()
    check(L.g2p_sim_input_read(str(path).encode(), C.byref(h)))
    try:
        nl, npt, ns = C.c_int32(), C.c_int32(), C.c_int32()
        check(L.g2p_sim_input_sizes(h, C.byref(nl), C.byref(npt), C.byref(ns)))
        lim, units, fc = np.zeros(6), np.zeros(4), np.zeros(2, np.int32)
        layers, gds = np.zeros((nl.value, 4)), np.zeros(nl.value, np.int32)
        sptr, coords, sdir = np.zeros(npt.value + 1, np.int32), np.zeros((ns.value, 6)), np.zeros(ns.value, np.int32)
        check(L.g2p_sim_input_get(h, lim.ctypes.data, units.ctypes.data, fc.ctypes.data, layers.ctypes.data,
                                  gds.ctypes.data, sptr.ctypes.data, coords.ctypes.data, sdir.ctypes.data))
    finally:
        L.g2p_sim_input_free(h)
    return dict(lim=lim, length_unit=units[0], freq_unit=units[1], freq_start=units[2], freq_end=units[3],
                nfreq=int(fc[0]), freq_scale=int(fc[1]), layers=layers, layer_gdsii=gds, port_side_ptr=sptr,
                side_coords=coords, side_dir=sdir)


def polygonZ(polygons, layers, layer_gdsii) -> np.ndarray:
    """Each polygon's (z bottom, z top) from the stack layer with its GDSII
    number, the last such layer winning (convertToFDTDMesh,
    solnoutclass.hpp:5928-5939); (0, 0) when none has it."""
    lay = np.asarray(polygons[0])
    z = np.zeros((len(lay), 2))
    for k in range(len(layer_gdsii)):
        z[lay == layer_gdsii[k]] = layers[k, :2]
    return z


def meshAndMarkPolygons(grid, polygons, poly_z, port_side_ptr, side_coords, side_dir) -> dict:
    """Conductor marking from polygons on the GPU (g2p_mesh_mark_polygons:
    findInsideCond, the conductor numbering, findPortNode and portSet).
    grid: (xn, yn, zn); polygons as readGDSII returns them; poly_z from
    polygonZ; port sides as readSimInput returns them.  Returns the fdtdMesh
    fields as numpy arrays, with the side coordinates as findPortNode left
    them."""
    L = _lib.load()
    xn, yn, zn = (_c(v, np.float64) for v in grid[:3])
    nx, ny, nz = len(xn), len(yn), len(zn)
    _, vptr, vx, vy = polygons
    vptr, vx, vy = _c(vptr, np.int64), _c(vx, np.float64), _c(vy, np.float64)
    pz = _c(np.asarray(poly_z, np.float64).reshape(-1, 2), np.float64)
    sptr = _c(port_side_ptr, np.int32)
    coords = np.array(side_coords, np.float64).reshape(-1, 6).copy()
    sdir_in = _c(side_dir, np.int32)
    nports, nsides = len(sptr) - 1, len(coords)
    N_node = nx * ny * nz
    Ns = (ny - 1) * nx + (nx - 1) * ny
    N_edge = Ns * nz + nx * ny * (nz - 1)
    mark_node = np.zeros(N_node, np.int64)
    mark_edge = np.zeros(N_edge, np.int64)
    ncdt = C.c_int64()
    max_cdt = len(vptr) + 1
    mark_port = np.zeros(max_cdt, np.int32)
    cdt_return = np.zeros(max_cdt, np.uint8)
    max_e = nsides * max(nx, ny, nz) + 1
    side_edge_ptr = np.zeros(nsides + 1, np.int64)
    side_edges = np.zeros(max_e, np.int64)
    side_area = np.zeros(max(1, nsides), np.float64)
    side_dir = np.zeros(max(1, nsides), np.int32)
    check(L.g2p_mesh_mark_polygons(nx, ny, nz, xn.ctypes.data, yn.ctypes.data, zn.ctypes.data, len(vptr) - 1,
                                   vptr.ctypes.data, vx.ctypes.data, vy.ctypes.data, pz.ctypes.data, nports,
                                   sptr.ctypes.data, coords.ctypes.data, sdir_in.ctypes.data, mark_node.ctypes.data,
                                   mark_edge.ctypes.data, C.byref(ncdt), mark_port.ctypes.data,
                                   cdt_return.ctypes.data, max_cdt, side_edge_ptr.ctypes.data,
                                   side_edges.ctypes.data, max_e, side_area.ctypes.data, side_dir.ctypes.data))
    n = ncdt.value
    return dict(mark_node=mark_node, mark_edge=mark_edge, num_cdt=n, mark_port=mark_port[:n],
                cdt_return=cdt_return[:n], side_edge_ptr=side_edge_ptr,
                side_edges=side_edges[:side_edge_ptr[-1]], side_area=side_area[:nsides],
                side_dir=side_dir[:nsides], side_coords=coords)


def layoutFromGDS(gds_path, sim_input_path, ignore_layers=()) -> MeshDesc:
    """A design file and its .sim_input to the fdtdMesh fields of the V0
    path, as the reference's command-line flow gets there (TestMain.cpp:
    readSimInput, the GDSII read and saveToMesh, convertToFDTDMesh,
    meshAndMark, portSet): readSimInput and readGDSII on the host, the grid
    (g2p_mesh_grid) on the host, marking, numbering and ports on the GPU."""
    sim = readSimInput(sim_input_path)
    polys = readGDSII(gds_path, ignore_layers)
    sides = sim["side_coords"]
    xn, yn, zn, epsn, sign = meshGrid(sim["lim"], polys, sides, sim["layers"])
    pz = polygonZ(polys, sim["layers"], sim["layer_gdsii"])
    mk = meshAndMarkPolygons((xn, yn, zn), polys, pz, sim["port_side_ptr"], sides, sim["side_dir"])
    nports = len(sim["port_side_ptr"]) - 1
    return MeshDesc(nx=len(xn), ny=len(yn), nz=len(zn), xn=xn, yn=yn, zn=zn, stack_epsn=epsn, stack_sign=sign,
                    mark_node=mk["mark_node"], mark_edge=mk["mark_edge"],
                    mark_node_raw=(mk["mark_node"] != 0).astype(np.int64),
                    mark_edge_raw=(mk["mark_edge"] != 0).astype(np.int64), num_cdt=mk["num_cdt"],
                    mark_port=mk["mark_port"], cdt_return=mk["cdt_return"], num_ports=nports,
                    port_side_ptr=np.asarray(sim["port_side_ptr"], np.int32), side_edge_ptr=mk["side_edge_ptr"],
                    side_edges=mk["side_edges"], side_area=mk["side_area"], side_dir=mk["side_dir"],
                    side_coords=mk["side_coords"], freq_start=sim["freq_start"], freq_end=sim["freq_end"],
                    freq_unit=sim["freq_unit"], nfreq=sim["nfreq"], freq_scale=sim["freq_scale"],
                    name=str(gds_path))


class Parasitics:
    """Network parameters of one extraction, as the Parasitics class of
    src/solnoutclass.hpp keeps them: a kind ('Z', 'Y' or 'S'), the sweep
    frequencies (Hz), the ports' source impedances and one P x P complex
    matrix per frequency.  convertParam runs on the GPU (g2p_convert_param);
    the writers below are host code, as the reference's are."""

    def __init__(self, z_source, port_names=None, port_dirs=None):
        self.z_source = np.ascontiguousarray(z_source, np.float64)
        n = len(self.z_source)
        self.port_names = list(port_names) if port_names is not None else [f"port{i + 1}" for i in range(n)]
        self.port_dirs = "".join(port_dirs) if port_dirs is not None else "B" * n
        if len(self.port_names) != n or len(self.port_dirs) != n:
            raise ValueError("one name and one direction per port")
        self.param = "\0"
        self.freqs = np.zeros(0)
        self.matParam = np.zeros((0, n, n), np.complex128)
        self.matG = None
        self.matC = None

    def getNPort(self) -> int:
        return len(self.z_source)

    def getParamType(self) -> str:
        return self.param

    def getFreqs(self):
        return self.freqs

    def getParamMatrix(self):
        return self.matParam

    def saveNetworkParam(self, param: str, freqs, p):
        """saveNetworkParam (src/solnoutclass.hpp:1394-1452): p holds
        nfreq*P*P complex values in sys->x's order, entry (i, j) of
        frequency f at (f*P + i)*P + j -- paraGenerator's Z as returned."""
        if param not in ("Z", "Y", "S"):
            raise ValueError("network parameters must be 'Z', 'Y' or 'S'")
        n = self.getNPort()
        self.freqs = np.ascontiguousarray(freqs, np.float64)
        self.matParam = np.ascontiguousarray(p, np.complex128).reshape(len(self.freqs), n, n).copy()
        self.param = param
        self.computeYBusFromParam(0)

    def computeYBusFromParam(self, indFreq: int):
        """computeYBusFromParam (src/solnoutclass.hpp:1662-1748): the nodal
        matrices matG, matC the Xyce and SPEF writers print; None for
        S-parameters, where the reference has none."""
        n = self.getNPort()
        g = np.zeros((n, n))
        c = np.zeros((n, n))
        p0 = np.ascontiguousarray(self.matParam[indFreq]).view(np.float64).ravel()
        rc = _lib.load().g2p_ybus_from_param(self.param.encode(), n, float(self.freqs[indFreq]), p0.ctypes.data,
                                             g.ctypes.data, c.ctypes.data)
        if rc == 5:                          # G2P_ERR_UNSUPPORTED: S-parameters
            self.matG = self.matC = None
            return
        check(rc)
        self.matG, self.matC = g, c

    def terminatePortZ(self, indPort: int, ZLoad):
        """terminatePortZ (src/solnoutclass.hpp:1767-1842) on the GPU: the
        port loaded by ZLoad (its first value, imaginary part scaled with
        frequency) and removed by Kron reduction."""
        _terminate(self, "Z", indPort, ZLoad)

    def terminatePortY(self, indPort: int, YLoad):
        """terminatePortY (src/solnoutclass.hpp:1844-1921), as terminatePortZ."""
        _terminate(self, "Y", indPort, YLoad)

    def computeYParamFromCircuit(self):
        """computeYParamFromCircuit (src/solnoutclass.hpp:1617-1678) on the
        GPU: Y = G + j 2 pi f C at every frequency."""
        n, nf = self.getNPort(), len(self.freqs)
        g = np.ascontiguousarray(self.matG, np.float64)
        c = np.ascontiguousarray(self.matC, np.float64)
        out = np.zeros(2 * nf * n * n)
        check(_lib.load().g2p_y_from_circuit(n, nf, self.freqs.ctypes.data, g.ctypes.data, c.ctypes.data,
                                             out.ctypes.data))
        self.matParam = out.view(np.complex128).reshape(nf, n, n)
        self.param = "Y"

    def convertParam(self, newParam: str):
        """convertParam (src/solnoutclass.hpp:1456-1610) on the GPU."""
        if newParam not in ("Z", "Y", "S"):
            raise ValueError("new network parameters must be 'S', 'Y' or 'Z'")
        if newParam == self.param:
            return
        nf, n = self.matParam.shape[0], self.getNPort()
        buf = np.ascontiguousarray(self.matParam).view(np.float64).ravel().copy()
        check(_lib.load().g2p_convert_param(self.param.encode(), newParam.encode(), n, nf,
                                            self.z_source.ctypes.data, buf.ctypes.data, buf.ctypes.data))
        self.matParam = buf.view(np.complex128).reshape(nf, n, n)
        self.param = newParam


def _terminate(para: "Parasitics", kind: str, indPort: int, load):
    if para.param != kind:
        raise ValueError(f"terminating a port with {'an impedance' if kind == 'Z' else 'an admittance'} needs "
                         f"{kind}-parameters")
    n, nf = para.getNPort(), len(para.freqs)
    ld = np.ascontiguousarray(np.atleast_1d(np.asarray(load, np.complex128))).view(np.float64).ravel()
    buf = np.ascontiguousarray(para.matParam, np.complex128).view(np.float64).ravel()
    out = np.zeros(2 * nf * (n - 1) * (n - 1))
    check(_lib.load().g2p_terminate_port(kind.encode(), n, nf, para.freqs.ctypes.data, int(indPort), len(ld) // 2,
                                         ld.ctypes.data, buf.ctypes.data, out.ctypes.data))
    para.matParam = out.view(np.complex128).reshape(nf, n - 1, n - 1)
    keep = [i for i in range(n) if i != indPort]
    para.z_source = para.z_source[keep].copy()
    para.port_names = [para.port_names[i] for i in keep]
    para.port_dirs = "".join(para.port_dirs[i] for i in keep)


def _dump(fn, path, para: Parasitics, design: str, with_z: bool) -> bool:
    L = _lib.load()
    data = np.ascontiguousarray(para.matParam, np.complex128).view(np.float64).ravel()
    args = [str(path).encode(), para.param.encode(), para.getNPort(), len(para.freqs), para.freqs.ctypes.data]
    if with_z:
        args.append(para.z_source.ctypes.data)
    args += [data.ctypes.data, design.encode()]
    rc = getattr(L, fn)(*args)
    if rc == 1 and "cannot open" in L.g2p_last_error().decode(errors="replace"):
        return False                         # the reference returns false when the file cannot be opened
    check(rc)
    return True


WRITE_THRESH = 1e-5     # src/solnoutclass.hpp:33


def _nodal_args(para: Parasitics):
    if para.matG is None:
        raise ValueError("no nodal matrices: save Z- or Y-parameters first")
    names = (C.c_char_p * para.getNPort())(*[nm.encode() for nm in para.port_names])
    g = np.ascontiguousarray(para.matG, np.float64)
    c = np.ascontiguousarray(para.matC, np.float64)
    return names, g, c


def dumpXyce(path, para: Parasitics, design: str, save_thresh: float = WRITE_THRESH) -> bool:
    """dumpXyce / toXyce (src/solnoutclass.hpp:2094-2225): SPICE subcircuit."""
    L = _lib.load()
    names, g, c = _nodal_args(para)
    rc = L.g2p_write_xyce(str(path).encode(), design.encode(), para.getNPort(), names, float(para.freqs[0]),
                          g.ctypes.data, c.ctypes.data, save_thresh)
    if rc == 1 and "cannot open" in L.g2p_last_error().decode(errors="replace"):
        return False
    check(rc)
    return True


def dumpSPEF(path, para: Parasitics, design: str, save_thresh: float = WRITE_THRESH) -> bool:
    """dumpSPEF / toSPEF (src/solnoutclass.hpp:1972-2091): SPEF file."""
    L = _lib.load()
    names, g, c = _nodal_args(para)
    rc = L.g2p_write_spef(str(path).encode(), design.encode(), para.getNPort(), names, para.port_dirs.encode(),
                          g.ctypes.data, c.ctypes.data, save_thresh)
    if rc == 1 and "cannot open" in L.g2p_last_error().decode(errors="replace"):
        return False
    check(rc)
    return True


def dumpTouchstone(path, para: Parasitics, design: str = "") -> bool:
    """dumpTouchstone (src/solnoutclass.hpp:6118-6226): Touchstone 2.0 file."""
    return _dump("g2p_write_touchstone", path, para, design, True)


def dumpCITI(path, para: Parasitics, design: str = "") -> bool:
    """dumpCITI (src/solnoutclass.hpp:6040-6115): CITIfile."""
    return _dump("g2p_write_citi", path, para, design, False)
