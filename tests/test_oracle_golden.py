"""The C restatement (oracle/) and the layout generator against fixtures made
by the reference's own sources (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import BENCH_CASES, GOLDEN_CASES, check_golden_array, golden_layout

# the assembly pins also cover the bench configurations (c2: 231M S entries,
# about 5 s of oracle time on one thread); the CPU Z checks stay on the small
# layouts, the bench configurations' Z is checked on the GPU
ASSEMBLY_CASES = GOLDEN_CASES + BENCH_CASES


@pytest.mark.parametrize("name", ASSEMBLY_CASES)
def test_generator_matches_reference_meshing(name):
    # conductor labelling, recolouring, ports (mesh.cpp:683-1020, portSet)
    d, A, M = golden_layout(name)
    check_golden_array(A, M, "mark_node", d.mark_node)
    check_golden_array(A, M, "mark_edge", d.mark_edge)
    check_golden_array(A, M, "mark_port", d.mark_port)
    check_golden_array(A, M, "cdt_return", d.cdt_return)
    check_golden_array(A, M, "side_edges", d.side_edges)
    check_golden_array(A, M, "side_area", d.side_area)
    check_golden_array(A, M, "side_dir", d.side_dir)
    assert M["numCdt"] == d.num_cdt


@pytest.mark.parametrize("name", ASSEMBLY_CASES)
def test_oracle_index_maps_and_stiffness(name, coracle):
    d, A, M = golden_layout(name)
    me, pe, pn, bden = coracle.index_maps(d)
    assert bden == M["bden"]
    check_golden_array(A, M, "map_edge", me)
    ptr, col, val = coracle.stiffness(d)
    rows = np.repeat(np.arange(len(ptr) - 1, dtype=np.int64), np.diff(ptr))
    assert len(col) == M["leng_S"]
    check_golden_array(A, M, "S_row", rows)
    check_golden_array(A, M, "S_col", col)
    check_golden_array(A, M, "S_val", val)       # bit-exact


@pytest.mark.parametrize("name", ASSEMBLY_CASES)
def test_oracle_v0_and_laplacians(name, coracle):
    d, A, M = golden_layout(name)
    V = coracle.v0_and_laplacians(d)
    for t in "dc":
        v = V["v0" + t]
        for k in ("row", "col", "val", "aval", "map"):
            check_golden_array(A, M, f"v0{t}_{k}", v[k])
        ptr, col, val = V["A" + t]
        rows = np.repeat(np.arange(len(ptr) - 1, dtype=np.int64), np.diff(ptr))
        check_golden_array(A, M, f"A{t}_row", rows)
        check_golden_array(A, M, f"A{t}_col", col)
        check_golden_array(A, M, f"A{t}_val", val)
    assert V["v0d"]["ncol"] == M["leng_v0d"] and V["v0c"]["ncol"] == M["leng_v0c"]


@pytest.mark.parametrize("name", [c for c in GOLDEN_CASES if c != "strip_c1"])
def test_oracle_z_matches_reference(name, coracle):
    d, A, M = golden_layout(name)
    Z, st = coracle.para_generator(d)
    Zr = A["Z"].reshape(Z.shape)
    err = np.abs(Z - Zr).max() / np.abs(Zr).max()
    assert err < 1e-9, err
    assert st.max_rel_residual < 1e-11


def test_oracle_solver_matches_direct_solve(coracle):
    # the CPU solver against a sparse direct solve on a reference-assembled Ad
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    d, A, M = golden_layout("manhattan_small")
    V = coracle.v0_and_laplacians(d)
    ptr, col, val = V["Ad"]
    n = len(ptr) - 1
    Ad = sp.csr_matrix((val, col, ptr), shape=(n, n))
    b = np.random.default_rng(3).standard_normal(n)
    x, st = coracle.solve_csr(ptr, col, val, b)
    xd = spl.spsolve(Ad.tocsc(), b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8
    assert st.rel_residual < 1e-11


@pytest.mark.parametrize("name", ["manhattan_small", "multistrip_small"])
def test_oracle_job_on_threads_matches_reference(name, coracle):
    """The job form the CPU baseline times (ports spread over host threads,
    a fresh AMG setup per solve as hypreSolve does) gives the reference's Z."""
    d, A, M = golden_layout(name)
    job = coracle.job(d)
    o = coracle.default_opts(rtol=1e-12, maxit=3000, restart=50, reuse_setup=0)
    for k in range(3):
        job.stage(k, o, threads=3)
    Z = job.z()
    job.close()
    Zr = A["Z"].reshape(Z.shape)
    assert np.abs(Z - Zr).max() / np.abs(Zr).max() < 1e-9
