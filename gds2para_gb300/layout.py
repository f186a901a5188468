"""Synthetic layered-interconnect layouts on uniform structured grids.

The reference builds its solver database from GDSII / ``.sim_input`` files
through Limbo and ``meshAndMark`` (mesh.cpp:5-1133) and ``portSet``
(mesh.cpp:1196-1594).  Those front ends are outside the accelerated path, so
this module fills the same fields directly for seeded synthetic layouts:

* conductor boxes are rasterised the way ``findInsideCond`` marks a polygon
  (fdtd.hpp:534-826): an edge is inside a box when it lies in the closed box,
  its ``markEdge`` takes the box index + 1 and both end nodes are marked;
* ``LOWER_BOUNDARY_PEC`` then marks the whole z = 0 plane (mesh.cpp:466-473);
* conductors are the connected components of marked nodes joined by marked
  edges, numbered in order of their lowest node index, the order the BFS of
  mesh.cpp:683-796 produces; ``markEdge`` is recoloured with the conductor id
  (mesh.cpp:1006-1020);
* port sides, ``portArea``, ``portDirection`` and ``markPort`` follow
  portSet (mesh.cpp:1196-1382), positiveCoordFlow (solnoutclass.hpp:898-912)
  and mesh.cpp:884-953.

Everything here is host-side input preparation; nothing is timed.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Sequence, Tuple

import numpy as np

SIGMA_CU = 5.8e7


@dataclasses.dataclass
class Box:
    """Closed box of node indices [x0,x1] x [y0,y1] x [z0,z1]."""
    x0: int
    x1: int
    y0: int
    y1: int
    z0: int
    z1: int


@dataclasses.dataclass
class PortSpec:
    """One port side: supply node -> return node along a single axis."""
    supply: Tuple[int, int, int]
    ret: Tuple[int, int, int]


@dataclasses.dataclass
class Layout:
    name: str
    nx: int
    ny: int
    nz: int
    pitch: Tuple[float, float, float]
    layer_eps: np.ndarray          # [nz-1] relative permittivity per cell layer
    layer_sig: np.ndarray          # [nz-1] conductivity per cell layer
    boxes: List[Box]
    ports: List[List[PortSpec]]    # per port, its sides
    freq_start: float = 1.0
    freq_end: float = 1.0
    freq_unit: float = 1e9
    nfreq: int = 1
    freq_scale: int = 1            # 1 linear, 0 logarithmic (fdtd.hpp:4325-4330)


@dataclasses.dataclass
class MeshDesc:
    """The fdtdMesh fields the hot path consumes (fdtd.hpp:182-356)."""
    nx: int
    ny: int
    nz: int
    xn: np.ndarray
    yn: np.ndarray
    zn: np.ndarray
    stack_epsn: np.ndarray         # [nz]
    stack_sign: np.ndarray         # [nz]
    mark_node: np.ndarray          # int64 [N_node] conductor id or 0
    mark_edge: np.ndarray          # int64 [N_edge] conductor id or 0
    mark_node_raw: np.ndarray      # int64 [N_node] 1 inside a box, before labelling
    mark_edge_raw: np.ndarray      # int64 [N_edge] box index+1, before labelling
    num_cdt: int
    mark_port: np.ndarray          # int32 [num_cdt]
    cdt_return: np.ndarray         # uint8 [num_cdt]
    num_ports: int
    port_side_ptr: np.ndarray      # int32 [P+1]
    side_edge_ptr: np.ndarray      # int64 [S+1]
    side_edges: np.ndarray         # int64
    side_area: np.ndarray          # f64 [S]
    side_dir: np.ndarray           # int32 [S]
    side_coords: np.ndarray        # f64 [S, 6] supply xyz, return xyz (m)
    freq_start: float
    freq_end: float
    freq_unit: float
    nfreq: int
    freq_scale: int
    name: str = ""

    # derived sizes (mesh.cpp:393-406)
    @property
    def Nx(self):
        return self.nx - 1

    @property
    def Ny(self):
        return self.ny - 1

    @property
    def Nz(self):
        return self.nz - 1

    @property
    def N_edge_s(self):
        return self.Ny * (self.Nx + 1) + self.Nx * (self.Ny + 1)

    @property
    def N_edge_v(self):
        return (self.Nx + 1) * (self.Ny + 1)

    @property
    def N_edge(self):
        return self.N_edge_s * (self.Nz + 1) + self.N_edge_v * self.Nz

    @property
    def N_node_s(self):
        return self.N_edge_v

    @property
    def N_node(self):
        return self.nz * self.N_node_s

    def freqs(self) -> np.ndarray:
        """Frequency of each point as print_z_V0 labels it (fdtd.hpp:4249-4300)."""
        out = []
        for i in range(self.nfreq):
            if self.nfreq == 1 or i == 0:
                out.append(self.freq_start * self.freq_unit)
            elif i == self.nfreq - 1:
                out.append(self.freq_end * self.freq_unit)
            elif self.freq_scale == 1:
                out.append((self.freq_start + i * (self.freq_end - self.freq_start) / (self.nfreq - 1)) * self.freq_unit)
            else:
                out.append(self.freq_start * self.freq_unit * (self.freq_end / self.freq_start) ** (i * 1.0 / (self.nfreq - 1)))
        return np.array(out)


def _rasterise(nx, ny, nz, boxes: Sequence[Box]):
    """Raw marks as findInsideCond leaves them, plus the lower PEC plane."""
    Nx, Ny, Nz = nx - 1, ny - 1, nz - 1
    Y = np.zeros((nz, nx, Ny), np.int64)       # y-edges: plane z, node x, cell y
    X = np.zeros((nz, Nx, ny), np.int64)       # x-edges: plane z, cell x, node y
    Z = np.zeros((Nz, nx, ny), np.int64)       # z-edges: cell z, node x, node y
    node = np.zeros((nz, nx, ny), np.int64)
    for b_i, b in enumerate(boxes):
        v = b_i + 1
        Z[b.z0:b.z1, b.x0:b.x1 + 1, b.y0:b.y1 + 1] = v
        Y[b.z0:b.z1 + 1, b.x0:b.x1 + 1, b.y0:b.y1] = v
        X[b.z0:b.z1 + 1, b.x0:b.x1, b.y0:b.y1 + 1] = v
        node[b.z0:b.z1 + 1, b.x0:b.x1 + 1, b.y0:b.y1 + 1] = 1
    # LOWER_BOUNDARY_PEC: markEdge = numCdtRow + 1 on the z = 0 plane
    Y[0] = len(boxes) + 1
    X[0] = len(boxes) + 1
    node[0] = 1
    return Y, X, Z, node


def _pack_edges(Y, X, Z):
    nz = Y.shape[0]
    parts = []
    for iz in range(nz):
        parts.append(Y[iz].ravel())
        parts.append(X[iz].ravel())
        if iz < nz - 1:
            parts.append(Z[iz].ravel())
    return np.concatenate(parts)


def _label(Y, X, Z, node):
    """Connected components over marked edges, numbered by lowest node id."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components
    nz, nx, ny = node.shape
    nid = np.arange(nz * nx * ny, dtype=np.int64).reshape(nz, nx, ny)
    a = [nid[:, :, :-1][Y != 0], nid[:, :-1, :][X != 0], nid[:-1][Z != 0]]
    b = [nid[:, :, 1:][Y != 0], nid[:, 1:, :][X != 0], nid[1:][Z != 0]]
    a = np.concatenate(a)
    b = np.concatenate(b)
    n = nid.size
    g = sp.coo_matrix((np.ones(a.size, np.int8), (a, b)), shape=(n, n)).tocsr()
    _, lab = connected_components(g, directed=False)
    marked = node.ravel() != 0
    lab_m = lab[marked]
    uniq, first = np.unique(lab_m, return_index=True)
    order = np.argsort(first, kind="stable")
    remap = np.zeros(lab.max() + 1, np.int64)
    remap[uniq[order]] = np.arange(1, uniq.size + 1)
    mark_node = np.zeros(n, np.int64)
    mark_node[marked] = remap[lab_m]
    return mark_node.reshape(nz, nx, ny), int(uniq.size)


def build(layout: Layout) -> MeshDesc:
    nx, ny, nz = layout.nx, layout.ny, layout.nz
    px, py, pz = layout.pitch
    xn = np.arange(nx, dtype=np.float64) * px
    yn = np.arange(ny, dtype=np.float64) * py
    zn = np.arange(nz, dtype=np.float64) * pz
    Nx, Ny, Nz = nx - 1, ny - 1, nz - 1
    # stackEpsn / stackSign per node layer: cell layer above, plus the top
    # surface duplicate (mesh.cpp:312-329)
    stack_epsn = np.concatenate([layout.layer_eps, layout.layer_eps[-1:]]).astype(np.float64)
    stack_sign = np.concatenate([layout.layer_sig, layout.layer_sig[-1:]]).astype(np.float64)
    Y, X, Z, node = _rasterise(nx, ny, nz, layout.boxes)
    mark_edge_raw = _pack_edges(Y, X, Z)
    mark_node_raw = node.ravel().copy()
    lab, ncdt = _label(Y, X, Z, node)
    # recolour: an edge inside a conductor takes the conductor id
    Yc = np.where(Y != 0, lab[:, :, :-1], 0)
    Xc = np.where(X != 0, lab[:, :-1, :], 0)
    Zc = np.where(Z != 0, lab[:-1], 0)
    mark_edge = _pack_edges(Yc, Xc, Zc)
    mark_node = lab.ravel()
    Ns = Ny * (Nx + 1) + Nx * (Ny + 1)
    L = Ns + nx * ny
    nns = nx * ny

    def nidx(p):
        return p[2] * nns + p[0] * ny + p[1]

    mark_port = np.zeros(ncdt, np.int32)
    cdt_return = np.zeros(ncdt, np.uint8)
    seen = set()
    side_ptr = [0]
    edge_ptr = [0]
    edges: List[int] = []
    areas: List[float] = []
    dirs: List[int] = []
    coords = []
    for pi, sides in enumerate(layout.ports):
        for s in sides:
            if mark_node[nidx(s.supply)] == 0 or mark_node[nidx(s.ret)] == 0:
                raise ValueError(f"port {pi} end outside a conductor")
        # mesh.cpp:941-953: the last side's conductors are marked; a return
        # conductor gets its PEC-plane sets only when first met as a return
        c1 = int(mark_node[nidx(sides[-1].supply)])
        c2 = int(mark_node[nidx(sides[-1].ret)])
        mark_port[c1 - 1] = pi + 1
        mark_port[c2 - 1] = -1
        if c1 not in seen:
            seen.add(c1)
        if c2 not in seen:
            seen.add(c2)
            cdt_return[c2 - 1] = 1
        for s in sides:
            (x1, y1, z1), (x2, y2, z2) = s.supply, s.ret
            sx, sy, sz = xn[x1], yn[y1], zn[z1]
            e: List[int] = []
            if x1 != x2:
                for j in range(min(x1, x2), max(x1, x2)):
                    e.append(L * z1 + Ny * (Nx + 1) + j * (Ny + 1) + y1)
                area = _side_len(yn, y1, sy, Ny) * _side_len(zn, z1, sz, Nz)
            elif y1 != y2:
                for j in range(min(y1, y2), max(y1, y2)):
                    e.append(L * z1 + Ny * x1 + j)
                area = _side_len(xn, x1, sx, Nx) * _side_len(zn, z1, sz, Nz)
            else:
                for j in range(min(z1, z2), max(z1, z2)):
                    e.append(L * j + Ns + (Ny + 1) * x1 + y1)
                area = _side_len(xn, x1, sx, Nx) * _side_len(yn, y1, sy, Ny)
            edges.extend(e)
            edge_ptr.append(len(edges))
            areas.append(area)
            # positiveCoordFlow: +1 when any supply coordinate exceeds the return's
            dirs.append(1 if (x1 > x2 or y1 > y2 or z1 > z2) else -1)
            coords.append([sx, sy, sz, xn[x2], yn[y2], zn[z2]])
        side_ptr.append(len(edge_ptr) - 1)
    return MeshDesc(
        nx=nx, ny=ny, nz=nz, xn=xn, yn=yn, zn=zn,
        stack_epsn=stack_epsn, stack_sign=stack_sign,
        mark_node=mark_node.astype(np.int64), mark_edge=mark_edge.astype(np.int64),
        mark_node_raw=mark_node_raw.astype(np.int64), mark_edge_raw=mark_edge_raw.astype(np.int64),
        num_cdt=ncdt, mark_port=mark_port, cdt_return=cdt_return,
        num_ports=len(layout.ports),
        port_side_ptr=np.array(side_ptr, np.int32), side_edge_ptr=np.array(edge_ptr, np.int64),
        side_edges=np.array(edges, np.int64), side_area=np.array(areas, np.float64),
        side_dir=np.array(dirs, np.int32), side_coords=np.array(coords, np.float64).reshape(-1, 6),
        freq_start=layout.freq_start, freq_end=layout.freq_end, freq_unit=layout.freq_unit,
        nfreq=layout.nfreq, freq_scale=layout.freq_scale, name=layout.name)


def _side_len(coord, i, c, N):
    """portSet's dual length of a port point (mesh.cpp:1257-1277)."""
    if i == 0:
        return coord[i + 1] - c
    if i == N:
        return c - coord[i - 1]
    return (coord[i + 1] - c) / 2 + (c - coord[i - 1]) / 2


# --------------------------------------------------------------------------
# Named workloads
# --------------------------------------------------------------------------

def microstrip(nx=101, ny=41, nz=11, pitch=1e-6, freq_ghz=1.0, freq_end_ghz=None, nfreq=1,
               freq_scale=1) -> Layout:
    """Single microstrip over a ground slab, one lumped port at x = 0.

    Cell layers: z 0-1 ground (sigma Cu), 1-8 dielectric (eps_r 3.9), 8-9
    strip (4 cells wide at y 18..22 of 41 nodes, full x), 9-10 air.  The
    default is 101 x 41 x 11 nodes at 1 um and one frequency; nfreq > 1
    sweeps freq_ghz..freq_end_ghz (freq_scale 1 linear, 0 logarithmic)."""
    assert nz >= 5
    zs = nz - 1
    strip_z = zs - 2
    eps = np.ones(zs)
    sig = np.zeros(zs)
    eps[1:strip_z] = 3.9
    sig[0] = SIGMA_CU
    sig[strip_z] = SIGMA_CU
    yc = ny // 2
    w = max(1, round(4 * (ny - 1) / 40)) if ny >= 41 else 2
    y0 = yc - w // 2
    boxes = [Box(0, nx - 1, 0, ny - 1, 0, 1), Box(0, nx - 1, y0, y0 + w, strip_z, strip_z + 1)]
    ports = [[PortSpec((0, yc, strip_z), (0, yc, 1))]]
    return Layout("microstrip", nx, ny, nz, (pitch, pitch, pitch), eps, sig, boxes, ports,
                  freq_start=freq_ghz, freq_end=freq_ghz if freq_end_ghz is None else freq_end_ghz, freq_unit=1e9,
                  nfreq=nfreq, freq_scale=freq_scale)


def multistrip(nx=256, ny=256, nz=16, n_strips=32, pitch=1e-6, width=None, freq_start=1e7, freq_end=1e11,
               freq_unit=1.0, nfreq=64, freq_scale=0, eps_r=3.9) -> Layout:
    """The microstrip stack with n_strips parallel strips, one port each.

    Cell layers as in microstrip(): ground 0-1, dielectric up to the strip
    layer, strips along x in the layer below the top air layer.  Strips are
    evenly spaced in y; each port runs from a strip's bottom at x = 0 down to
    the ground top."""
    assert nz >= 5
    zs = nz - 1
    strip_z = zs - 2
    eps = np.ones(zs)
    sig = np.zeros(zs)
    eps[1:strip_z] = eps_r
    sig[0] = SIGMA_CU
    sig[strip_z] = SIGMA_CU
    slot = (ny - 2) // n_strips
    if slot < 2:
        raise ValueError("grid too narrow for the strip count")
    w = width if width is not None else max(1, slot // 2)
    boxes = [Box(0, nx - 1, 0, ny - 1, 0, 1)]
    ports: List[List[PortSpec]] = []
    for s in range(n_strips):
        y0 = 1 + s * slot + (slot - w) // 2
        boxes.append(Box(0, nx - 1, y0, y0 + w, strip_z, strip_z + 1))
        ports.append([PortSpec((0, y0 + w // 2, strip_z), (0, y0 + w // 2, 1))])
    return Layout("multistrip", nx, ny, nz, (pitch, pitch, pitch), eps, sig, boxes, ports,
                  freq_start=freq_start, freq_end=freq_end, freq_unit=freq_unit, nfreq=nfreq, freq_scale=freq_scale)


def manhattan(nx=512, ny=512, nz=24, n_metal=4, wires_per_layer=64, n_ports=8, seed=1001,
              pitch=1e-6, via_p=0.3, freq_start=10.0, freq_end=10.0, nfreq=1, freq_unit=1e9,
              freq_scale=1, wmin=2, wmax=8, lmin=20, lmax=200) -> Layout:
    """Random Manhattan interconnect over the z = 0 ground plane.

    Metal layers are 2 cells thick, separated by dielectrics whose eps_r is
    drawn from U[2.5, 4.2]; wires alternate x / y by layer with width
    U{wmin..wmax} and length U{lmin..lmax} cells at uniform positions; 2 x 2
    cell vias join overlapping wires on adjacent layers with probability
    via_p.  Ports run from a lowest-layer wire end down to z = 0.  Every
    conductor layer carries copper's sigma (the reference keeps sigma per
    layer and applies it only on conductor edges)."""
    rng = np.random.default_rng(seed)
    ncell = nz - 1
    gap = 4
    thick = 2
    need = lambda g: g + n_metal * thick + (n_metal - 1) * g
    while need(gap) > ncell and gap > 1:
        gap -= 1
    if need(gap) > ncell:
        raise ValueError("grid too short for the metal stack")
    bottom_gap = ncell - (n_metal * thick + (n_metal - 1) * gap)
    air = 0
    if bottom_gap > gap + 1:
        air = 1
        bottom_gap -= 1
    eps = np.ones(ncell)
    sig = np.full(ncell, SIGMA_CU)
    z = 0
    metal_z = []
    d_eps = rng.uniform(2.5, 4.2, size=n_metal)
    eps[0:bottom_gap] = d_eps[0]
    z = bottom_gap
    for k in range(n_metal):
        metal_z.append(z)
        eps[z:z + thick] = d_eps[k]
        z += thick
        if k < n_metal - 1:
            eps[z:z + gap] = d_eps[k + 1]
            z += gap
    if air:
        eps[z:] = 1.0
    boxes: List[Box] = []
    layer_wires: List[List[Box]] = []
    for k in range(n_metal):
        wires = []
        along_x = k % 2 == 0
        for _ in range(wires_per_layer):
            w = int(rng.integers(wmin, wmax + 1))
            ln = int(rng.integers(lmin, lmax + 1))
            if along_x:
                ln = min(ln, nx - 3)
                w = min(w, ny - 3)
                x0 = int(rng.integers(1, nx - 1 - ln))
                y0 = int(rng.integers(1, ny - 1 - w))
                b = Box(x0, x0 + ln, y0, y0 + w, metal_z[k], metal_z[k] + thick)
            else:
                ln = min(ln, ny - 3)
                w = min(w, nx - 3)
                x0 = int(rng.integers(1, nx - 1 - w))
                y0 = int(rng.integers(1, ny - 1 - ln))
                b = Box(x0, x0 + w, y0, y0 + ln, metal_z[k], metal_z[k] + thick)
            wires.append(b)
        layer_wires.append(wires)
        boxes.extend(wires)
    for k in range(n_metal - 1):
        for a in layer_wires[k]:
            for b in layer_wires[k + 1]:
                ox0, ox1 = max(a.x0, b.x0), min(a.x1, b.x1)
                oy0, oy1 = max(a.y0, b.y0), min(a.y1, b.y1)
                if ox1 - ox0 >= 2 and oy1 - oy0 >= 2 and rng.random() < via_p:
                    vx = int(rng.integers(ox0, ox1 - 1))
                    vy = int(rng.integers(oy0, oy1 - 1))
                    boxes.append(Box(vx, vx + 2, vy, vy + 2, a.z1, b.z0))
    lay = Layout("manhattan", nx, ny, nz, (pitch, pitch, pitch), eps, sig, boxes, [],
                 freq_start=freq_start, freq_end=freq_end, freq_unit=freq_unit, nfreq=nfreq,
                 freq_scale=freq_scale)
    # ports at wire ends, lowest layers first, each on a distinct net and with
    # a conductor-free column down to the ground plane
    Y, X, Z, node = _rasterise(nx, ny, nz, boxes)
    lab, _ = _label(Y, X, Z, node)
    used = set()
    ports: List[List[PortSpec]] = []
    for k in range(n_metal):
        for b in layer_wires[k]:
            if len(ports) == n_ports:
                break
            along_x = k % 2 == 0
            ends = [(b.x0, (b.y0 + b.y1) // 2), (b.x1, (b.y0 + b.y1) // 2)] if along_x else \
                   [((b.x0 + b.x1) // 2, b.y0), ((b.x0 + b.x1) // 2, b.y1)]
            for xc, yc in ends:
                net = int(lab[b.z0, xc, yc])
                if net in used or np.any(lab[1:b.z0, xc, yc] != 0):
                    continue
                used.add(net)
                ports.append([PortSpec((xc, yc, b.z0), (xc, yc, 0))])
                break
    if len(ports) < n_ports:
        raise ValueError(f"only {len(ports)} distinct port nets available")
    lay.ports = ports
    return lay


def config(name: str, **kw) -> Layout:
    """The named workloads: c1 microstrip, c2 random Manhattan at 10 GHz,
    c3 the microstrip stack with 32 strips (32 ports x 64 log-spaced points
    1e7..1e11 Hz), c5 the large random Manhattan layout (1536 x 1536 x 32
    nodes, 6 metal layers of 256 wires, 16 ports x 8 log-spaced points)."""
    if name == "c1":
        return microstrip(**kw)
    if name == "c2":
        args = dict(nx=512, ny=512, nz=24, n_ports=8, seed=1001)
        args.update(kw)
        return manhattan(**args)
    if name == "c3":
        args = dict(nx=256, ny=256, nz=16, n_strips=32)
        args.update(kw)
        return multistrip(**args)
    if name == "c5":
        args = dict(nx=1536, ny=1536, nz=32, n_metal=6, wires_per_layer=256, n_ports=16, seed=1005,
                    freq_start=1e8, freq_end=1e10, freq_unit=1.0, nfreq=8, freq_scale=0)
        args.update(kw)
        return manhattan(**args)
    raise KeyError(name)
