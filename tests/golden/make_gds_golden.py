"""Makes tests/golden/gdsii_cases.npz: synthetic GDSII files (written here,
not taken from any design) and, for each, the conductor polygons that the
reference's own AsciiDataBase + saveToMesh (limboint.hpp) produce when run by
oracle/_ref/ref_gds (oracle/build_ref.sh builds it from the reference
sources with a project-written stand-in for Limbo's stream reader).

The cases exercise every branch of the flattening: boundaries in both
orientations and with or without a closing point, boxes of BOXTYPE 0 and 1,
paths of PATHTYPE 0, 1, 2 and 4 with begin and end extensions, segments along
x and y in both directions and a diagonal one, references with mirroring,
rotation, magnification and the absolute flags, nested references, and array
references.

When the reference's example designs are present (argument: their folder),
the library's reader is also compared with the reference on each of them.

usage: python tests/golden/make_gds_golden.py [examples_dir]
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_GDS = os.path.join(ROOT, "oracle", "_ref", "ref_gds")


def rec(rt, dt, payload=b""):
    return struct.pack(">HBB", 4 + len(payload), rt, dt) + payload


def i2(*v):
    return struct.pack(">%dh" % len(v), *v)


def i4(*v):
    return struct.pack(">%di" % len(v), *v)


def s(text):
    b = text.encode()
    return b + (b"\0" if len(b) % 2 else b"")


def r8(v):
    """8-byte GDSII real (excess-64, base 16)."""
    if v == 0:
        return b"\0" * 8
    sign = 0x80 if v < 0 else 0
    v, e = abs(v), 64
    while v >= 1:
        v /= 16
        e += 1
    while v < 1 / 16:
        v *= 16
        e -= 1
    return bytes([sign | e]) + int(round(v * 2 ** 56)).to_bytes(7, "big")


DATE = i2(*([2021, 3, 4, 5, 6, 7] * 2))


def lib(cells, dbu=1e-9):
    out = rec(0x00, 2, i2(600)) + rec(0x01, 2, DATE) + rec(0x02, 6, s("LIB")) + rec(0x03, 5, r8(1e-3) + r8(dbu))
    for name, els in cells:
        out += rec(0x05, 2, DATE) + rec(0x06, 6, s(name)) + b"".join(els) + rec(0x07, 0)
    return out + rec(0x04, 0)


def xy(pts):
    return rec(0x10, 3, i4(*[c for p in pts for c in p]))


def boundary(layer, pts, datatype=0):
    return rec(0x08, 0) + rec(0x0D, 2, i2(layer)) + rec(0x0E, 2, i2(datatype)) + xy(pts) + rec(0x11, 0)


def box(layer, pts, boxtype=0):
    return rec(0x2D, 0) + rec(0x0D, 2, i2(layer)) + rec(0x2E, 2, i2(boxtype)) + xy(pts) + rec(0x11, 0)


def path(layer, pts, width, ptype=None, bext=None, eext=None):
    out = rec(0x09, 0) + rec(0x0D, 2, i2(layer)) + rec(0x0E, 2, i2(0))
    if ptype is not None:
        out += rec(0x21, 2, i2(ptype))
    out += rec(0x0F, 3, i4(width))
    if bext is not None:
        out += rec(0x30, 3, i4(bext))
    if eext is not None:
        out += rec(0x31, 3, i4(eext))
    return out + xy(pts) + rec(0x11, 0)


def strans(mirror=False, abs_mag=False, abs_rot=False, mag=None, angle=None):
    bits = (0x8000 if mirror else 0) | (0x4 if abs_mag else 0) | (0x2 if abs_rot else 0)
    out = rec(0x1A, 1, struct.pack(">H", bits))
    if mag is not None:
        out += rec(0x1B, 5, r8(mag))
    if angle is not None:
        out += rec(0x1C, 5, r8(angle))
    return out


def sref(name, at, tr=b""):
    return rec(0x0A, 0) + rec(0x12, 6, s(name)) + tr + xy([at]) + rec(0x11, 0)


def aref(name, cols, rows, p0, pc, pr, tr=b""):
    return (rec(0x0B, 0) + rec(0x12, 6, s(name)) + tr + rec(0x13, 2, i2(cols, rows)) + xy([p0, pc, pr])
            + rec(0x11, 0))


def cases():
    shapes = [
        boundary(1, [(0, 0), (4000, 0), (4000, 2000), (0, 2000), (0, 0)]),
        boundary(1, [(0, 0), (0, 3000), (5000, 3000), (5000, 0)]),            # clockwise, not closed
        boundary(2, [(1000, 1000), (6000, 1000), (6000, 2000), (3000, 2000), (3000, 5000), (1000, 5000), (1000, 1000)],
                 datatype=7),                                                 # L shape, datatype kept
        box(3, [(0, 0), (2000, 0), (2000, 1000), (0, 1000), (0, 0)]),
        box(3, [(0, 0), (2000, 0), (2000, 1000), (0, 1000), (0, 0)], boxtype=1),   # skipped
        path(4, [(0, 0), (0, 5000), (6000, 5000)], 400, ptype=0),
        path(4, [(6000, 0), (0, 0)], 400, ptype=1),
        path(4, [(0, 8000), (0, 3000)], 300),                                 # default PATHTYPE 2
        path(5, [(1000, 1000), (5000, 1000), (5000, 6000), (1000, 6000)], 200, ptype=4, bext=150, eext=90),
        path(5, [(0, 0), (3000, 2000)], 200, ptype=2),                        # diagonal: taken along x
    ]
    flat = lib([("TOP", shapes)])
    leaf = [boundary(10, [(0, 0), (1000, 0), (1000, 500), (0, 500), (0, 0)]),
            path(11, [(0, 0), (0, 2000)], 100, ptype=0)]
    mid = [boundary(12, [(0, 0), (300, 0), (300, 300), (0, 300), (0, 0)]),
           sref("LEAF", (1000, 0), strans(angle=90)),
           sref("LEAF", (0, 3000), strans(mirror=True, mag=2.0)),
           sref("LEAF", (5000, 5000), strans(mirror=True, angle=270)),
           sref("LEAF", (-4000, 0), strans(abs_rot=True, abs_mag=True, mag=0.5, angle=180))]
    top = [sref("MID", (20000, 10000), strans(angle=90)),
           sref("MID", (-20000, 0), strans(mirror=True, angle=45, mag=1.5)),
           sref("MID", (0, -30000)),
           aref("LEAF", 4, 3, (0, 0), (8000, 0), (0, 6000)),
           aref("LEAF", 3, 2, (1000, 1000), (7000, 4000), (1000, 9000), strans(mirror=True, angle=90)),
           aref("LEAF", 1, 4, (0, 0), (0, 0), (0, 9000)),
           sref("NOSUCH", (0, 0)),
           boundary(13, [(0, 0), (100, 0), (100, 100), (0, 100), (0, 0)])]
    hier = lib([("LEAF", leaf), ("MID", mid), ("TOP", top)], dbu=1e-8)
    return {"flat": (flat, []), "hier": (hier, []), "hier_ignore": (hier, [11, 13])}


def run_ref(gds_bytes, ignore):
    with tempfile.NamedTemporaryFile(suffix=".gds", delete=False) as f:
        f.write(gds_bytes)
        name = f.name
    try:
        out = subprocess.run([REF_GDS, name] + [str(i) for i in ignore], check=True, capture_output=True,
                             text=True).stdout
    finally:
        os.unlink(name)
    return parse_ref(out)


def parse_ref(text):
    layer, vptr, xs, ys = [], [0], [], []
    for line in text.splitlines():
        t = line.split()
        if not t or t[0] != "P":       # the reference's own messages
            continue
        layer.append(int(t[1]))
        n = int(t[2])
        xs += [float(v) for v in t[3:3 + 2 * n:2]]
        ys += [float(v) for v in t[4:4 + 2 * n:2]]
        vptr.append(len(xs))
    return (np.array(layer, np.int32), np.array(vptr, np.int64), np.array(xs), np.array(ys))


def main():
    if not os.path.exists(REF_GDS):
        sys.exit("build oracle/_ref first: sh oracle/build_ref.sh")
    arrays = {}
    for name, (gds, ignore) in cases().items():
        layer, vptr, x, y = run_ref(gds, ignore)
        arrays[f"{name}_gds"] = np.frombuffer(gds, np.uint8)
        arrays[f"{name}_ignore"] = np.array(ignore, np.int32)
        arrays[f"{name}_layer"], arrays[f"{name}_vptr"] = layer, vptr
        arrays[f"{name}_x"], arrays[f"{name}_y"] = x, y
        print(f"{name}: {len(layer)} polygons")
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "gdsii_cases.npz"), **arrays)
    if len(sys.argv) > 1:
        sys.path.insert(0, ROOT)
        from gds2para_gb300 import api
        folder = sys.argv[1]
        for fn in sorted(os.listdir(folder)):
            if not fn.endswith(".gds"):
                continue
            path = os.path.join(folder, fn)
            want = parse_ref(subprocess.run([REF_GDS, path], check=True, capture_output=True, text=True).stdout)
            got = api.readGDSII(path)
            same = all(np.array_equal(a, b) for a, b in zip(got, want))
            print(f"{fn}: {len(want[0])} polygons, library {'identical' if same else 'DIFFERS'}")


if __name__ == "__main__":
    main()
