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
