"""The reference-signature shim on the GPU.  tests/shim_driver.cpp
instantiates generateStiff / paraGenerator / hypreSolve of
include/gds2para_gb300_shim.hpp with a mesh type carrying fdtdMesh's member
names and types, fills it as meshAndMark and portSet leave an fdtdMesh,
and calls them in TestMain's order.  Its S must be the reference's, bit for
bit; its Z the reference's within the GPU parity bound; paraGenerator must
free what the reference frees; hypreSolve must meet hypreSolve's own
tolerance."""
import os
import subprocess

import numpy as np
import pytest

from conftest import check_golden_array, golden_layout
from shim_common import build_driver, write_mesh

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(tmp_path_factory, g2p):
    return build_driver(str(tmp_path_factory.mktemp("shim")))


@pytest.mark.parametrize("name", ["strip_tiny", "manhattan_small", "manhattan_sweep"])
def test_gpu_shim_generate_stiff_and_para_generator(name, driver, tmp_path):
    d, A, M = golden_layout(name)
    src, out = tmp_path / "in", tmp_path / "out"
    write_mesh(d, str(src))
    out.mkdir()
    r = subprocess.run([driver, "extract", str(src), str(out), "0", "1e-10"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    check_golden_array(A, M, "S_row", np.fromfile(out / "S_row.i64", np.int64))
    check_golden_array(A, M, "S_col", np.fromfile(out / "S_col.i64", np.int64))
    check_golden_array(A, M, "S_val", np.fromfile(out / "S_val.f64", np.float64))
    z = np.fromfile(out / "Z.f64", np.float64)
    Z = z[0::2] + 1j * z[1::2]
    Zr = A["Z"]
    assert Z.shape == Zr.shape
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < 1e-7
    assert (out / "freed.txt").read_text().strip() == "1"


def test_gpu_shim_hypre_solve(driver, tmp_path):
    d, A, M = golden_layout("strip_tiny")
    rows, cols, vals = A["Ad_row"], A["Ad_col"], A["Ad_val"]
    b, xr = A["solve0_b"], A["solve0_x"]
    src, out = tmp_path / "in", tmp_path / "out"
    src.mkdir()
    out.mkdir()
    for nm, a in (("A_row.i64", rows), ("A_col.i64", cols), ("A_val.f64", vals), ("b.f64", b)):
        np.ascontiguousarray(a).tofile(src / nm)
    r = subprocess.run([driver, "hypre", str(src), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    x = np.fromfile(out / "x.f64", np.float64)
    import scipy.sparse as sp
    n = len(b)
    Ad = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    assert np.linalg.norm(b - Ad @ x) <= 1e-4 * np.linalg.norm(b) * 1.0001
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-2
