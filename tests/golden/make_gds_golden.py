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

It also runs the reference's meshAndMark on two of the layouts with made-up
limits, layer stacks and port sides (GRID_CASES) and stores its grid lines
and per-layer constants.

When the reference's example designs are present (argument: their folder),
the library's reader and grid are also compared with the reference on each
of them (the grid where the .sim_input names its layers by GDSII number).

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


# Grid cases: limits, stack layers (z begin, z end, eps_r, sigma, GDSII layer)
# and port sides (x1 y1 z1 x2 y2 z2 direction), in metres, for the layouts
# above; run through the reference's meshAndMark by ref_gds --grid.
GRID_CASES = {
    "flat": ((-1e-6, 9e-6, -1e-6, 1e-5, 0.0, 6e-6),
             [(0.0, 1e-6, 3.9, 0.0, 100), (1e-6, 2e-6, 3.9, 5.8e7, 1), (2e-6, 2.5e-6, 2.5, 5.8e7, 2),
              (2.5e-6, 3e-6, 2.5, 5.8e7, 3), (3e-6, 3.2e-6, 2.5, 5.8e7, 4), (3.2e-6, 4e-6, 4.2, 5.8e7, 5),
              (4e-6, 6e-6, 3.9, 0.0, 101)],
             [(2e-6, 1e-6, 2e-6, 2e-6, 1e-6, 1e-6, -1), (3e-6, 5e-6, 3.2e-6, 3e-6, 5e-6, 3e-6, 1)]),
    "hier": ((-4e-4, 4e-4, -4e-4, 4e-4, 0.0, 5e-6),
             [(0.0, 1e-6, 3.9, 0.0, 100), (1e-6, 1.5e-6, 3.2, 5.8e7, 10), (1.5e-6, 2e-6, 3.2, 5.8e7, 11),
              (2e-6, 3e-6, 2.7, 5.8e7, 12), (3e-6, 3.5e-6, 2.7, 5.8e7, 13), (3.5e-6, 5e-6, 3.9, 0.0, 101)],
             [(5e-6, 2e-6, 1.5e-6, 5e-6, 2e-6, 0.0, 1)]),
}


def grid_settings(lim, stack, sides):
    out = " ".join(repr(v) for v in lim) + "\n%d\n" % len(stack)
    out += "".join("%r %r %r %r %d\n" % layer for layer in stack)
    return out + "%d\n" % len(sides) + "".join(" ".join(repr(v) for v in sd[:6]) + " %d\n" % sd[6] for sd in sides)


def run_ref_grid(gds_bytes, settings):
    with tempfile.TemporaryDirectory() as d:
        gp, sp = os.path.join(d, "in.gds"), os.path.join(d, "in.txt")
        with open(gp, "wb") as f:
            f.write(gds_bytes)
        with open(sp, "w") as f:
            f.write(settings)
        # the reference's meshAndMark writes debug dumps (x.txt, cond.txt, ...)
        # into its working directory: keep them in the temporary one
        out = subprocess.run([REF_GDS, gp, "--grid", sp], check=True, capture_output=True, text=True,
                             cwd=d).stdout
    lines = {t[0]: np.array([float(v) for v in t[1:]]) for t in (l.split() for l in out.splitlines())
             if t and t[0] in ("X", "Y", "Z", "E", "S")}
    return [lines[k] for k in "XYZES"]


def mark_settings(sim):
    """ref_gds --mark settings from the library's readSimInput result: the
    limits, the valid stack layers with their GDSII numbers, and every port
    with its sides and directions."""
    out = " ".join(repr(float(v)) for v in sim["lim"]) + "\n%d\n" % len(sim["layers"])
    for (zb, ze, eps, sig), g in zip(sim["layers"], sim["layer_gdsii"]):
        out += "%r %r %r %r %d\n" % (float(zb), float(ze), float(eps), float(sig), int(g))
    sptr = sim["port_side_ptr"]
    out += "%d\n" % (len(sptr) - 1)
    for p in range(len(sptr) - 1):
        out += "%d\n" % (sptr[p + 1] - sptr[p])
        for k in range(sptr[p], sptr[p + 1]):
            out += " ".join(repr(float(v)) for v in sim["side_coords"][k]) + " %d\n" % int(sim["side_dir"][k])
    return out


def run_ref_mark(gds_path, settings):
    """The reference's meshAndMark + portSet on a GDSII file (ref_gds
    --mark): grid, marks, conductor ports and port sides."""
    with tempfile.TemporaryDirectory() as d:
        sp, dd = os.path.join(d, "in.txt"), os.path.join(d, "dump")
        os.makedirs(dd)
        with open(sp, "w") as f:
            f.write(settings)
        subprocess.run([REF_GDS, gds_path, "--mark", sp, dd], check=True, capture_output=True, text=True, cwd=d)
        meta = open(os.path.join(dd, "meta.txt")).read().split()
        out = {"meta": np.array([int(v) for v in meta], np.int64)}
        ext = {"i64": np.int64, "f64": np.float64, "i32": np.int32}
        for fn in os.listdir(dd):
            stem, _, e = fn.rpartition(".")
            if e in ext:
                out[stem] = np.fromfile(os.path.join(dd, fn), ext[e])
    return out


def sim_input_settings(path):
    """Limits, stack and port sides of a .sim_input file in metres (stack
    layers must be named by GDSII number); None when the file does not fit."""
    import re
    t = [line.split("#")[0].strip() for line in open(path)]
    t = [line for line in t if line]
    try:
        i = t.index("TOTAL SIZE")
        lu = float(t[i + 2].split("=")[1])
        lim = [float(v) * lu for v in t[i + 1].split()]
        j = t.index("DIELECTRIC STACK")
        stack = []
        for line in t[j + 2:j + 2 + int(t[j + 1].split("=")[1])]:
            kv = dict(re.findall(r"(\w+)\s*=\s*([-+.\deE]+)", line))
            z, h = float(kv["z"]), float(kv["h"])
            stack.append((z * lu, (z + h) * lu, float(kv["e"]), float(kv.get("sigma", 0.0)),
                          int(line.split()[0].lstrip("M"))))
        k = t.index("PORT")
        sides = [[float(v) * lu for v in line.split()[1:7]] + [int(line.split()[7])]
                 for line in t[k + 2:k + 2 + int(t[k + 1].split("=")[1])]]
    except (ValueError, IndexError, KeyError):
        return None
    return lim, stack, sides


def run_ref(gds_bytes, ignore):
    with tempfile.NamedTemporaryFile(suffix=".gds", delete=False) as f:
        f.write(gds_bytes)
        name = f.name
    try:
        out = subprocess.run([REF_GDS, name] + [str(i) for i in ignore], check=True, capture_output=True,
                             text=True, cwd=tempfile.gettempdir()).stdout
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
    all_cases = cases()
    for name, (lim, stack, sides) in GRID_CASES.items():
        grid = run_ref_grid(all_cases[name][0], grid_settings(lim, stack, sides))
        arrays[f"{name}_grid_lim"] = np.array(lim)
        arrays[f"{name}_grid_stack"] = np.array([layer[:4] for layer in stack])
        arrays[f"{name}_grid_sides"] = np.array([sd[:6] for sd in sides])
        for key, v in zip("XYZES", grid):
            arrays[f"{name}_grid_{key}"] = v
        print(f"{name} grid: {len(grid[0])} x {len(grid[1])} x {len(grid[2])} lines")
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "gdsii_cases.npz"), **arrays)
    if len(sys.argv) > 1:
        sys.path.insert(0, ROOT)
        from gds2para_gb300 import api
        folder = sys.argv[1]
        for fn in sorted(os.listdir(folder)):
            if not fn.endswith(".gds"):
                continue
            path = os.path.join(folder, fn)
            want = parse_ref(subprocess.run([REF_GDS, path], check=True, capture_output=True, text=True,
                                            cwd=tempfile.gettempdir()).stdout)
            got = api.readGDSII(path)
            same = all(np.array_equal(a, b) for a, b in zip(got, want))
            msg = f"{fn}: {len(want[0])} polygons, library {'identical' if same else 'DIFFERS'}"
            sim = path[:-4] + ".sim_input"
            st = sim_input_settings(sim) if os.path.exists(sim) else None
            if st:
                lim, stack, sides = st
                with open(path, "rb") as f:
                    ref_grid = run_ref_grid(f.read(), grid_settings(lim, stack, sides))
                grid = api.meshGrid(lim, got, [sd[:6] for sd in sides], [layer[:4] for layer in stack])
                same = all(np.array_equal(a, b) for a, b in zip(grid, ref_grid))
                msg += f"; grid {len(grid[0])} x {len(grid[1])} x {len(grid[2])}, {'identical' if same else 'DIFFERS'}"
            print(msg)


if __name__ == "__main__":
    main()
