"""CPU restatement of the reference's network-parameter stage -- test
infrastructure only (the checker for g2p_convert_param, g2p_ybus_from_param
and the four writers).

* ``convert_param`` follows convertParam (src/solnoutclass.hpp:1456-1610)
  with numpy's LAPACK inverse in place of Eigen's.
* ``touchstone_text`` and ``citi_text`` follow dumpTouchstone
  (src/solnoutclass.hpp:6118-6226) and dumpCITI
  (src/solnoutclass.hpp:6040-6115); C++ iostream output of a double at
  precision p in the default float field is printf's %.{p}g, std::left /
  std::right with setw(13) pad to 13 characters.
* ``ybus_from_param``, ``xyce_text`` and ``spef_elements`` follow
  computeYBusFromParam (src/solnoutclass.hpp:1662-1748), makeCSym/makeGSym
  (:1319-1390), toXyce (:2094-2225) and toSPEF (:1972-2091), dense-matrix
  build.  Eigen's row sums and isApprox norms are taken in plain index
  order; Eigen's own reduction order is not pinned (it changes the printed
  six digits only in the last place, if at all).

Pinning: the reference's versions need Eigen, which is not available, so
they cannot be compiled here, and the reference ships no network-parameter
file.  ``convert_param`` is pinned against closed-form two-port results
(series and shunt impedances, matched, open and short terminations; see
tests/test_network_cpu.py); the writers' text is pinned only by the reading
of the source cited above.  The reference prints SPEF through Parser-SPEF
(OpenTimer, cloned from its master branch, no version pinned), which is not
present; only the element choices and values of the SPEF file are checked.
"""
from __future__ import annotations

import numpy as np


def convert_param(frm: str, to: str, p: np.ndarray, z_source) -> np.ndarray:
    """p: (nfreq, P, P) complex.  Returns the converted matrices."""
    p = np.asarray(p, np.complex128)
    if frm == to:
        return p.copy()
    n = p.shape[-1]
    eye = np.eye(n, dtype=np.complex128)
    zs = np.asarray(z_source, np.float64)
    out = np.empty_like(p)
    for f in range(p.shape[0]):
        m = p[f]
        if {frm, to} == {"Z", "Y"}:                       # solnoutclass.hpp:1466-1474, 1512-1520
            out[f] = np.linalg.inv(m)
        elif frm == "Y":                                  # Y -> S, solnoutclass.hpp:1476-1496
            d = np.diag(np.sqrt(zs))
            out[f] = (eye - d @ m @ d) @ np.linalg.inv(eye + d @ m @ d)
        elif frm == "Z":                                  # Z -> S, solnoutclass.hpp:1526-1546
            d = np.diag(np.sqrt(1.0 / zs))
            out[f] = (d @ m @ d - eye) @ np.linalg.inv(d @ m @ d + eye)
        elif to == "Y":                                   # S -> Y, solnoutclass.hpp:1558-1578
            d = np.diag(np.sqrt(1.0 / zs))
            out[f] = d @ (eye - m) @ np.linalg.inv(eye + m) @ d
        else:                                             # S -> Z, solnoutclass.hpp:1580-1600
            d = np.diag(np.sqrt(zs))
            out[f] = d @ (eye + m) @ np.linalg.inv(eye - m) @ d
    return out


def _g(x: float, prec: int = 7) -> str:
    return "%.*g" % (prec, x)


def touchstone_text(param: str, freqs, z_source, p, design: str, stamp: str) -> str:
    """The file dumpTouchstone writes; p: (nfreq, P, P) complex."""
    n = len(z_source)
    o = ["[Version] 2.0\n", "# Hz %s RI R %s\n" % (param, _g(z_source[0], 6)), "[Number of Ports] %d\n" % n]
    if n == 2:
        o.append("[Two-Port Data Order] 12_21\n")
    o.append("[Number of Frequencies] %d\n" % len(freqs))
    o.append("[Reference]\n")
    o.append("".join(_g(z, 6) + " " for z in z_source))
    o.append("\n[Matrix Format] Full\n")
    o.append("! Date/Time %s\n! Name %s\n" % (stamp, design))
    o.append("! Provider: DARPA ERI IDEA/POSH Contributors\n! Program: Xyce Writer from DARPA ERI\n"
             "! Author: Purdue University\n[Network Data] \n")
    o.append("!freq         ")
    for i in range(n):
        for j in range(n):
            w = max(0, 8 - i // 10 - j // 10)
            if n > 2 and i > 0 and j == 0:
                o.append("!Re%s%d,%d%s" % (param, i + 1, j + 1, " " * max(0, w - 1)))
            else:
                o.append("Re%s%d,%d%s" % (param, i + 1, j + 1, " " * w))
            o.append("Im%s%d,%d%s" % (param, i + 1, j + 1, " " * w))
            if (j + 1) % 4 == 0 and j + 1 != n and n > 2:
                o.append("\n!" + " " * 13)
        if n > 2:
            o.append("\n")
    o.append("\n")
    for f in range(len(freqs)):
        o.append(_g(freqs[f]).ljust(13) + " ")
        for i in range(n):
            for j in range(n):
                v = p[f][i][j]
                o.append(_g(v.real).ljust(13) + " " + _g(v.imag).ljust(13) + " ")
                if (j + 1) % 4 == 0 and j + 1 != n and n > 2:
                    o.append("\n" + " " * 14)
            if n > 2:
                o.append(" ! row %d\n" % (i + 1))
        if n <= 2:
            o.append("\n")
    o.append("[End]\n")
    return "".join(o)


def citi_text(param: str, freqs, p, design: str, stamp: str) -> str:
    """The file dumpCITI writes; p: (nfreq, P, P) complex."""
    n = p.shape[-1]
    o = ["CITIFILE A.01.01\n", "CONSTANT TIME %s\n" % stamp, "NAME %s\n" % design.upper(),
         "VAR FREQ MAG %d\n" % len(freqs)]
    for i in range(n):
        for j in range(n):
            o.append("DATA %s[%d,%d] RI\n" % (param, i + 1, j + 1))
    o.append("VAR_LIST_BEGIN\n")
    for f in freqs:
        o.append(_g(f).ljust(13) + "\n")
    o.append("VAR_LIST_END\n")
    for i in range(n):
        for j in range(n):
            o.append("BEGIN\n")
            for f in range(len(freqs)):
                v = p[f][i][j]
                o.append(_g(v.real).rjust(13) + "," + _g(v.imag).ljust(13) + "\n")
            o.append("END\n")
    return "".join(o)


def ybus_from_param(param: str, p0: np.ndarray, freq0: float):
    """computeYBusFromParam (src/solnoutclass.hpp:1662-1748, dense build):
    'Z' takes the matrix itself as Y, 'Y' its inverse; returns (G, C)."""
    y = np.asarray(p0, np.complex128) if param == "Z" else np.linalg.inv(p0)
    w = 2.0 * np.pi * freq0
    return y.real.copy(), -1 / (y.imag * w)


def _symmetrise(a: np.ndarray) -> np.ndarray:
    """makeCSym / makeGSym (src/solnoutclass.hpp:1319-1390) with Eigen's
    isApprox test at its default precision 1e-12."""
    n = a.shape[0]
    d2 = na = nt = 0.0
    for j in range(n):
        for i in range(n):
            x, y = a[i, j], a[j, i]
            d2 += (x - y) * (x - y)
            na += x * x
            nt += y * y
    if d2 <= 1e-24 * min(na, nt):
        return a.copy()
    return (a + a.T) * 0.5


def _nodal(g, c):
    c = _symmetrise(np.asarray(c, np.float64))
    g = _symmetrise(np.asarray(g, np.float64))
    n = g.shape[0]
    gg, cg = [], []
    gt = ct = 0.0
    for i in range(n):
        sg = sc = 0.0
        for j in range(n):
            sg += g[i, j]
            sc += c[i, j]
        gg.append(sg)
        cg.append(sc)
        for j in range(i, n):
            gt += g[i, j]
            ct += c[i, j]
    return g, c, gg, cg, gt, ct


def _elements(g, c, thresh):
    """The capacitor and resistor choices toXyce / toSPEF make
    (src/solnoutclass.hpp:2062-2085, 2166-2200): (kind, i, j or -1, value)."""
    g, c, gg, cg, gt, ct = _nodal(g, c)
    n = g.shape[0]
    out = []
    for i in range(n):
        for j in range(n):
            if i == j and abs(cg[i]) >= thresh * ct:
                out.append(("C", i, -1, cg[i]))
            elif j > i and abs(-c[i, j]) >= thresh * ct:
                out.append(("C", i, j, -1.0 * c[i, j]))
        for j in range(n):
            if i == j and abs(gg[i]) >= thresh * gt:
                out.append(("R", i, -1, abs(1.0 / gg[i])))
            elif j > i and abs(-1.0 / g[i, j]) >= thresh * gt:
                out.append(("R", i, j, abs(-1.0 / g[i, j])))
    return out, ct


def xyce_text(path: str, design: str, names, freq0: float, g, c, thresh: float, stamp: str) -> str:
    """The file toXyce writes (src/solnoutclass.hpp:2094-2225)."""
    o = ["* File: %s\n* Design: %s\n" % (path, design), "* Vendor: DARPA ERI Contributors\n",
         "* Program: Xyce Writer from DARPA ERI\n* Author: Purdue University\n", "* Date: %s\n\n" % stamp,
         ".subckt " + design + "".join(" " + nm for nm in names) + "\n"]
    w2 = (2.0 * np.pi * freq0) ** 2.0
    k = {"C": 1, "L": 1, "R": 1}
    els, _ = _elements(g, c, thresh)
    for kind, i, j, v in els:
        other = "0" if j < 0 else names[j]
        if kind == "C" and v <= 0.0:
            kind, v = "L", -1.0 / (v * w2)
        o.append("%s%d %s %s %s\n" % (kind, k[kind], names[i], other, _g(v, 6)))
        k[kind] += 1
    o.append(".ends\n")
    return "".join(o)


def spef_elements(g, c, thresh):
    """(caps, ress, total capacitance) as toSPEF fills its net
    (src/solnoutclass.hpp:2027-2087); nodes as 1-based port numbers, 0 for
    ground."""
    els, ct = _elements(g, c, thresh)
    caps = [(i + 1, j + 1, v) for kind, i, j, v in els if kind == "C"]
    ress = [(i + 1, j + 1, v) for kind, i, j, v in els if kind == "R"]
    return caps, ress, ct
