"""CPU restatement of the reference's network-parameter stage -- test
infrastructure only (the checker for g2p_convert_param and the two writers).

* ``convert_param`` follows convertParam (src/solnoutclass.hpp:1456-1610)
  with numpy's LAPACK inverse in place of Eigen's.
* ``touchstone_text`` and ``citi_text`` follow dumpTouchstone
  (src/solnoutclass.hpp:6118-6226) and dumpCITI
  (src/solnoutclass.hpp:6040-6115); C++ iostream output of a double at
  precision p in the default float field is printf's %.{p}g, std::left /
  std::right with setw(13) pad to 13 characters.

Pinning: the reference's versions need Eigen, which is not available, so
they cannot be compiled here, and the reference ships no network-parameter
file.  ``convert_param`` is pinned against closed-form two-port results
(series and shunt impedances, matched, open and short terminations; see
tests/test_network_cpu.py); the writers' text is pinned only by the reading
of the source cited above.
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
