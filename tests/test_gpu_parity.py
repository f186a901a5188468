"""GPU path (libgds2para_gb300.so through the C ABI) against fixtures made by
the reference's own sources and against the C oracle."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, check_golden_array, golden_layout

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_index_maps_and_stiffness_bit_exact(name, g2p):
    d, A, M = golden_layout(name)
    with g2p.FdtdMesh(d) as m:
        me, bden = m.index_maps()
        assert bden == M["bden"]
        check_golden_array(A, M, "map_edge", me)
        assert g2p.generateStiff(m) == M["leng_S"]
        r, c, v = m.export_stiff()
        check_golden_array(A, M, "S_row", r)
        check_golden_array(A, M, "S_col", c)
        check_golden_array(A, M, "S_val", v)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_v0_and_laplacians_bit_exact(name, g2p):
    d, A, M = golden_layout(name)
    with g2p.FdtdMesh(d) as m:
        s = m.assemble_v0()
        assert s.leng_v0d == M["leng_v0d"] and s.leng_v0c == M["leng_v0c"]
        for t in "dc":
            v = m.export_v0(t)
            for k in ("row", "col", "val", "aval", "map"):
                check_golden_array(A, M, f"v0{t}_{k}", v[k])
            r, c, val = m.export_laplacian(t)
            check_golden_array(A, M, f"A{t}_row", r)
            check_golden_array(A, M, f"A{t}_col", c)
            check_golden_array(A, M, f"A{t}_val", val)


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("precision,batch", [("fp64", 0), ("fp64", 1), ("mixed", 1)])
def test_gpu_z_matches_reference(name, precision, batch, g2p):
    # tolerance: the GPU solves stop at ||r|| <= 1e-10 ||b||; the fixture's
    # solves were taken to 1e-13, so Z may differ at the 1e-8 level
    d, A, M = golden_layout(name)
    with g2p.FdtdMesh(d) as m:
        Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, batch=batch, rtol=1e-10))
    Zr = A["Z"].reshape(Z.shape)
    err = np.abs(Z - Zr).max() / np.abs(Zr).max()
    assert err < 1e-7, (err, st.total_iterations)
    assert st.max_rel_residual <= 1e-10
    assert st.solves == 3 * d.num_ports


def test_gpu_hypre_solve_dropin_matches_reference_solution(g2p):
    # hypreSolve's own settings (rtol 1e-4) on the reference's Ad and rhs
    d, A, M = golden_layout("strip_tiny")
    rows, cols, vals = A["Ad_row"], A["Ad_col"], A["Ad_val"]
    b, xr = A["solve0_b"], A["solve0_x"]
    n = len(b)
    x = np.zeros(n)
    assert g2p.hypreSolve(None, rows, cols, vals, len(vals), b, n, x) == 0
    import scipy.sparse as sp
    Ad = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    assert np.linalg.norm(b - Ad @ x) <= 1e-4 * np.linalg.norm(b) * 1.0001
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-2


@pytest.mark.parametrize("precision", ["fp64", "mixed", "fp64_pc32"])
def test_gpu_solver_multi_rhs_against_direct(precision, g2p, coracle):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    d, A, M = golden_layout("manhattan_small")
    V = coracle.v0_and_laplacians(d)
    for t in "dc":
        ptr, col, val = V["A" + t]
        n = len(ptr) - 1
        rows = np.repeat(np.arange(n), np.diff(ptr))
        B = np.random.default_rng(7).standard_normal((n, 5))
        S = g2p.Solver(rows, col, val, n, g2p.default_params(precision=precision, rtol=1e-10))
        X, st = S.solve(B)
        S.close()
        Am = sp.csr_matrix((val, col, ptr), shape=(n, n))
        Xd = spl.spsolve(Am.tocsc(), B)
        res = np.linalg.norm(B - Am @ X, axis=0) / np.linalg.norm(B, axis=0)
        assert res.max() <= 1e-10 * 1.0001, res
        assert np.linalg.norm(X - Xd) / np.linalg.norm(Xd) < 1e-7


def test_gpu_solver_rejects_unknown_precision(g2p):
    rows = np.array([0, 1]); col = np.array([0, 1]); val = np.array([2.0, 3.0])
    with pytest.raises(g2p.G2PError):
        g2p.Solver(rows, col, val, 2, g2p.default_params(precision=7))


def test_gpu_rejects_bad_coo(g2p):
    with pytest.raises(g2p.G2PError):
        g2p.Solver(np.array([1, 0]), np.array([0, 1]), np.array([1.0, 1.0]), 2)   # not row-sorted
    with pytest.raises(g2p.G2PError):
        g2p.Solver(np.array([0, 1]), np.array([0, 5]), np.array([1.0, 1.0]), 2)   # column out of range


@pytest.mark.parametrize("name,precision", [("strip_c1", "mixed"), ("manhattan_sweep", "fp64"), ("multistrip_small", "mixed")])
def test_gpu_graph_replay_gives_identical_z(name, precision, g2p):
    """Arnoldi steps replayed from CUDA graphs give the same Z, bit for bit,
    as the same steps launched one kernel at a time."""
    d, A, M = golden_layout(name)
    out = []
    for graphs in (0, 1):
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10, use_graphs=graphs))
        out.append((Z, st.total_iterations))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])


def test_gpu_autotune_picks_a_candidate_and_keeps_it(g2p):
    """The autotuner's block width, degree, Ac strength and Ac precision mode
    come from its candidate sets, are kept for later jobs of the same shape,
    and give Z within the solve tolerance of the untuned run."""
    from gds2para_gb300 import layout as lay
    d = lay.build(lay.multistrip(nx=40, ny=64, nz=8, n_strips=16, freq_start=1e8, freq_end=1e10, nfreq=3))
    res = []
    for tune in (0, 1, 1):
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision="mixed", rtol=1e-10, autotune=tune))
        res.append((Z, st.rhs_block, st.ad_degree, st.ac_strength, st.ac_precision))
    assert res[0][1] == 16 and res[0][2] == 2 and res[0][3] == 0.08 and res[0][4] == 2
    assert res[1][1] in (16, 8) and res[1][2] in (2, 3, 4) and res[1][3] in (0.02, 0.04, 0.08)
    assert res[1][4] in (1, 2)        # mixed refinement or FP64 Krylov with the FP32 V-cycle
    assert res[2][1:] == res[1][1:]
    assert np.array_equal(res[1][0], res[2][0])
    err = np.abs(res[1][0] - res[0][0]).max() / np.abs(res[0][0]).max()
    assert err < 1e-7, err


@pytest.mark.parametrize("name,precision", [("strip_c1", "mixed"), ("manhattan_sweep", "fp64"), ("multistrip_small", "mixed")])
def test_gpu_galerkin_hash_path_matches_sort_path(name, precision, g2p, monkeypatch):
    """The per-row shared-memory Galerkin product sums in the same member and
    column order as the global expand-sort-compress product (sums of more
    than 32 terms excepted), and it is deterministic: Z agrees to solver
    tolerance and repeats bit for bit."""
    d, A, M = golden_layout(name)
    out = []
    for esc in (False, False, True):
        if esc:
            monkeypatch.setenv("G2P_RAP_ESC", "1")
        else:
            monkeypatch.delenv("G2P_RAP_ESC", raising=False)
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10))
        out.append(Z)
    assert np.array_equal(out[0], out[1])
    assert np.abs(out[0] - out[2]).max() / np.abs(out[2]).max() < 1e-8


@pytest.mark.parametrize("name,precision", [("strip_c1", "mixed"), ("manhattan_sweep", "fp64")])
def test_gpu_coarse_inverse_one_launch_matches_per_pivot(name, precision, g2p, monkeypatch):
    """The coarsest level's dense inverse from one cooperative launch (a grid
    barrier between pivots) does the per-pivot launches' arithmetic: Z is
    bit-identical either way."""
    d, A, M = golden_layout(name)
    out = []
    for steps in (False, True):
        if steps:
            monkeypatch.setenv("G2P_GJ_STEPS", "1")
        else:
            monkeypatch.delenv("G2P_GJ_STEPS", raising=False)
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10))
        out.append(Z)
    assert np.array_equal(out[0], out[1])


def test_gpu_coarse_inverse_barrier_give_up_recomputes_the_same(g2p, monkeypatch, capfd):
    """The cooperative inverse's grid barrier gives up after a bounded number
    of polls; with that bound cut to one poll it does give up, the host
    recomputes with one launch per pivot, and Z is bit-identical to the
    normal path's."""
    d, A, M = golden_layout("strip_c1")
    out = []
    for limit in (None, "1"):
        if limit:
            monkeypatch.setenv("G2P_GJ_SPIN_LIMIT", limit)
            monkeypatch.setenv("G2P_DEBUG", "1")
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision="fp64", rtol=1e-10))
        out.append(Z)
    monkeypatch.delenv("G2P_GJ_SPIN_LIMIT")
    monkeypatch.delenv("G2P_DEBUG")
    assert "barrier gave up; recomputed with one launch per pivot" in capfd.readouterr().err
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("name,precision", [("strip_c1", "mixed"), ("multistrip_small", "mixed"), ("strip_c1", "fp64")])
def test_gpu_extraction_leaves_exact_ad_and_repattern_path_agrees(name, precision, g2p, monkeypatch):
    """Ad's preconditioner is built from tree-summed stand-ins for its longest
    conductor segments while their ordered sums run; the Ad an extraction
    leaves behind, and multiplies by, is still the reference's bit for bit.
    Forcing the reassembly taken when a stand-in's kept/dropped status
    differs gives the same Ad and the same Z."""
    d, A, M = golden_layout(name)
    out = []
    for force in (False, True):
        if force:
            monkeypatch.setenv("G2P_AD_REPATTERN", "1")
        else:
            monkeypatch.delenv("G2P_AD_REPATTERN", raising=False)
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10))
            r, c, v = m.export_laplacian("d")
        check_golden_array(A, M, "Ad_row", r)
        check_golden_array(A, M, "Ad_col", c)
        check_golden_array(A, M, "Ad_val", v)
        assert st.max_rel_residual <= 1e-10
        out.append(Z)
    assert np.array_equal(out[0], out[1])


def _extract(g2p, d, precision):
    from gds2para_gb300 import _lib
    L = _lib.load()
    n0 = L.g2p_launch_count()
    with g2p.FdtdMesh(d) as m:
        g2p.generateStiff(m)
        Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10))
    return Z, st, L.g2p_launch_count() - n0


@pytest.mark.parametrize("mode", ["1", "2"])
@pytest.mark.parametrize("name,precision", [("strip_c1", "mixed"), ("manhattan_sweep", "fp64"),
                                            ("multistrip_small", "mixed")])
def test_gpu_fused_coarse_cycle_matches_launch_per_kernel(name, precision, mode, g2p, monkeypatch):
    """The coarse tail of the V-cycle in one launch (k_coarse_cycle: G2P_FUSE=1
    cooperative over the grid, G2P_FUSE=2 one thread-block cluster with the
    hardware cluster barrier) against the same levels launched kernel by
    kernel: the same arithmetic up to summation order, so Z agrees to the
    solves' tolerance, with far fewer launches."""
    d, A, M = golden_layout(name)
    monkeypatch.setenv("G2P_FUSE", "0")
    Z0, st0, n0 = _extract(g2p, d, precision)
    monkeypatch.setenv("G2P_FUSE", mode)
    Z1, st1, n1 = _extract(g2p, d, precision)
    monkeypatch.delenv("G2P_FUSE")
    assert np.abs(Z1 - Z0).max() / np.abs(Z0).max() < 1e-8
    assert st1.max_rel_residual <= 1e-10
    assert n1 < n0, (n1, n0)
    Zr = A["Z"].reshape(Z1.shape)
    assert np.abs(Z1 - Zr).max() / np.abs(Zr).max() < 1e-7


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_gpu_fused_coarse_cycle_give_up_repeats_the_solve_unfused(precision, g2p, monkeypatch, capfd):
    """The fused cycle's grid barrier gives up after a bounded number of
    polls; with the bound cut to one poll it does, the solver notices at the
    end of the solve and repeats it with the launch-per-kernel V-cycle, and Z
    is bit-identical to a run that never fused."""
    d, A, M = golden_layout("strip_c1")
    monkeypatch.setenv("G2P_FUSE", "0")
    Z0, _, _ = _extract(g2p, d, precision)
    monkeypatch.setenv("G2P_FUSE", "1")
    monkeypatch.setenv("G2P_FUSE_SPIN_LIMIT", "1")
    monkeypatch.setenv("G2P_DEBUG", "1")
    capfd.readouterr()
    Z1, _, _ = _extract(g2p, d, precision)
    monkeypatch.delenv("G2P_FUSE")
    monkeypatch.delenv("G2P_FUSE_SPIN_LIMIT")
    monkeypatch.delenv("G2P_DEBUG")
    assert "fused coarse cycle gave up; solve repeated unfused" in capfd.readouterr().err
    assert np.array_equal(Z0, Z1)


@pytest.mark.parametrize("name,precision", [("multistrip_small", "mixed"), ("manhattan_sweep", "fp64"),
                                            ("strip_c1", "mixed")])
def test_gpu_long_rows_beside_short_rows_give_identical_z(name, precision, g2p, monkeypatch):
    """The long-row kernels of coarse sliced-ELL operators on a side stream
    beside the short-row kernel (the default) write other rows than it does:
    Z is bit-identical to the serial order (G2P_LONG_FORK=0), graphs on."""
    d, A, M = golden_layout(name)
    out = []
    for fork in ("0", "1"):
        monkeypatch.setenv("G2P_LONG_FORK", fork)
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10))
        out.append((Z, st.total_iterations))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])


@pytest.mark.parametrize("name", ["multistrip_small", "manhattan_small"])
def test_gpu_unnormalised_basis_matches_normalised(name, g2p, monkeypatch):
    """The FP32 solves' unnormalised Arnoldi basis (the default) against the
    normalised one (G2P_UNNORM_BASIS=0): the same Krylov spaces in another
    scaling, so Z agrees to the solves' tolerance, and both match the
    reference."""
    d, A, M = golden_layout(name)
    out = []
    for un in ("0", "1"):
        monkeypatch.setenv("G2P_UNNORM_BASIS", un)
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision="mixed", rtol=1e-10))
        assert st.max_rel_residual <= 1e-10
        out.append(Z)
    assert np.abs(out[1] - out[0]).max() / np.abs(out[0]).max() < 1e-8
    Zr = A["Z"].reshape(out[1].shape)
    assert np.abs(out[1] - Zr).max() / np.abs(Zr).max() < 1e-7
