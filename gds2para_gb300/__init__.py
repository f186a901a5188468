"""gds2para_gb300: the gds2Para full-wave extraction hot path on GB300 (sm_103a).

Index maps, curl-curl stiffness, V0 bases and node Laplacians, the
AMG-preconditioned FGMRES that replaces hypreSolve, and the paraGenerator
Z-parameter pipeline, all as hand-written CUDA behind a C ABI
(include/gds2para_gb300.h).  ``api`` mirrors the reference's entry points;
``layout`` builds synthetic layouts.
"""
from . import layout  # noqa: F401

__version__ = "0.1.0"
