"""The reference-signature shim (include/gds2para_gb300_shim.hpp) without a
GPU: it compiles and links against the library, and, where the reference
checkout was present for build(), the reference's own harness linked with
oracle/gb300_path.cpp in place of its generateStiff.cpp, hypreSolve and
matrixCon.cpp reaches the library through all of them."""
import os
import subprocess

import numpy as np
import pytest

from conftest import check_golden_array, golden_layout, have_gpu
from shim_common import ROOT, build_driver


def test_shim_driver_compiles_and_links(tmp_path):
    try:
        exe = build_driver(str(tmp_path))
    except subprocess.CalledProcessError as e:
        pytest.fail(f"shim driver failed to build:\n{e.stderr[-3000:]}")
    assert os.access(exe, os.X_OK)


def test_reference_harness_runs_through_the_shim(tmp_path):
    """oracle/_ref/ref_pipeline_gb300: the reference's mesh code and
    fdtdMesh members with generateStiff, hypreSolve and paraGenerator from
    the shim.  With no GPU, both entry points the harness calls report the
    library's CUDA error and return (the reference's own V0 exports, made by
    its unmodified members, are unaffected)."""
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_pipeline_gb300")
    if not os.path.exists(exe):
        pytest.skip("oracle/_ref/ref_pipeline_gb300 is built only where the reference checkout exists")
    if have_gpu():
        pytest.skip("with a GPU the shim computes; tests/test_gpu_shim.py covers that")
    import oracle.harness as h
    d, A, M = golden_layout("strip_tiny")
    old = h.REF_BIN
    h.REF_BIN = exe
    try:
        R = h.run_reference(d, workdir=str(tmp_path))
    finally:
        h.REF_BIN = old
    log = R["_log"]
    assert "gds2para_gb300: generateStiff" in log and "gds2para_gb300: paraGenerator" in log
    for k in ("v0d_val", "Ad_val", "Ac_val", "map_edge"):
        check_golden_array(A, M, k, R[k])
    assert R["solves"] == 0          # nothing went through the CPU hypreSolve stand-in
