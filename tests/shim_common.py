"""Helpers for the reference-signature shim tests: compile tests/shim_driver.cpp
against include/ and the in-tree library, and write a layout's fdtdMesh fields
in the driver's input format."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "gds2para_gb300", "_build")


def build_driver(out_dir: str) -> str:
    from gds2para_gb300 import build
    build.build()
    exe = os.path.join(out_dir, "shim_driver")
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "shim_driver.cpp"), "-o", exe, "-L", LIBDIR, "-lgds2para_gb300",
                    f"-Wl,-rpath,{LIBDIR}"], check=True, capture_output=True, text=True)
    return exe


def write_mesh(d, path: str) -> None:
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "meta.txt"), "w") as f:
        f.write(f"{d.nx} {d.ny} {d.nz} {d.num_cdt} {d.num_ports} {d.nfreq} {d.freq_start!r} {d.freq_end!r} "
                f"{d.freq_unit!r} {d.freq_scale}\n")
    for name, a, dt in (("xn.f64", d.xn, np.float64), ("yn.f64", d.yn, np.float64), ("zn.f64", d.zn, np.float64),
                        ("stack_epsn.f64", d.stack_epsn, np.float64), ("stack_sign.f64", d.stack_sign, np.float64),
                        ("mark_node.i64", d.mark_node, np.int64), ("mark_edge.i64", d.mark_edge, np.int64),
                        ("mark_port.i32", d.mark_port, np.int32), ("port_side_ptr.i32", d.port_side_ptr, np.int32),
                        ("side_edge_ptr.i64", d.side_edge_ptr, np.int64), ("side_edges.i64", d.side_edges, np.int64),
                        ("side_area.f64", d.side_area, np.float64), ("side_dir.i32", d.side_dir, np.int32)):
        np.ascontiguousarray(a, dtype=dt).tofile(os.path.join(path, name))
