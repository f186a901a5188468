"""The C-ABI library builds for sm_103a, loads without a GPU and exports every
symbol the public header declares (no compute calls here)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "gds2para_gb300.h")).read()
    return sorted(set(re.findall(r"\b(g2p_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_header_symbols():
    from gds2para_gb300 import build, _lib
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = header_symbols()
    assert len(syms) >= 17
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_lib.EXPORTS) == set(syms)


def test_build_targets_sm103a_only():
    from gds2para_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_default_params_are_the_reference_settings():
    import ctypes as C
    from gds2para_gb300 import _lib
    L = _lib.load()
    p = _lib.SolverParams()
    L.g2p_default_params(C.byref(p), 1)
    assert (p.restart, p.maxit, p.rtol) == (10, 100, 1e-4)      # hypreSolver.h:7-11
    L.g2p_default_params(C.byref(p), 0)
    assert p.rtol == 1e-10 and p.precision == _lib.G2P_PREC_FP64


def test_version_and_error_strings_without_gpu():
    from gds2para_gb300 import _lib
    L = _lib.load()
    assert b"sm_103a" in L.g2p_version()
    assert isinstance(L.g2p_last_error(), bytes)


def test_ctypes_structs_match_the_header(tmp_path):
    """Sizes and field offsets of the ctypes mirrors equal the C compiler's
    for every struct the header declares (a host C program, no GPU)."""
    import ctypes as C
    import subprocess
    from gds2para_gb300 import _lib
    structs = {
        "g2p_solver_params": (_lib.SolverParams, [f[0] for f in _lib.SolverParams._fields_]),
        "g2p_solve_stats": (_lib.SolveStats, [f[0] for f in _lib.SolveStats._fields_]),
        "g2p_sizes": (_lib.Sizes, [f[0] for f in _lib.Sizes._fields_]),
        "g2p_extract_stats": (_lib.ExtractStats, [f[0] for f in _lib.ExtractStats._fields_]),
        "g2p_mesh_desc": (_lib.MeshDescC, [f[0] for f in _lib.MeshDescC._fields_]),
        "g2p_job_times": (_lib.JobTimes, [f[0] for f in _lib.JobTimes._fields_]),
        "g2p_box": (_lib.BoxC, [f[0] for f in _lib.BoxC._fields_]),
        "g2p_port_side": (_lib.PortSideC, [f[0] for f in _lib.PortSideC._fields_]),
    }
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "gds2para_gb300.h"', "int main(void) {"]
    for name, (_, fields) in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for f in fields:
            lines.append(f'printf("{name}.{f} %zu\\n", offsetof({name}, {f}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines())
    for name, (cls, fields) in structs.items():
        assert int(got[name]) == C.sizeof(cls), name
        for f in fields:
            assert int(got[f"{name}.{f}"]) == getattr(cls, f).offset, f"{name}.{f}"
