"""Block FGMRES (csrc/block_krylov.cu, switched on by G2P_BLOCK_KRYLOV=1):
the k right-hand sides share one block Krylov space.  Checked against a
direct solve, on rank-deficient blocks, against the lock-step solver's Z on
a two-port layout, and for bit-identical graph replays."""
import numpy as np
import pytest

from conftest import golden_layout

pytestmark = pytest.mark.gpu


def _ad(coracle, name="manhattan_small", t="d"):
    d, A, M = golden_layout(name)
    V = coracle.v0_and_laplacians(d)
    ptr, col, val = V["A" + t]
    n = len(ptr) - 1
    return n, np.repeat(np.arange(n), np.diff(ptr)), col, val, ptr


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("k", [2, 4, 8, 16, 32])
def test_gpu_block_krylov_against_direct(precision, k, g2p, coracle, monkeypatch):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    monkeypatch.setenv("G2P_BLOCK_KRYLOV", "1")
    for t in "dc":
        n, rows, col, val, ptr = _ad(coracle, t=t)
        B = np.random.default_rng(11 + k).standard_normal((n, k))
        S = g2p.Solver(rows, col, val, n, g2p.default_params(precision=precision, rtol=1e-10))
        X, st = S.solve(B)
        S.close()
        Am = sp.csr_matrix((val, col, ptr), shape=(n, n))
        res = np.linalg.norm(B - Am @ X, axis=0) / np.linalg.norm(B, axis=0)
        assert res.max() <= 1e-10 * 1.0001, res
        Xd = spl.spsolve(Am.tocsc(), B)
        assert np.linalg.norm(X - Xd) / np.linalg.norm(Xd) < 1e-7


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_block_krylov_rank_deficient_block(precision, g2p, coracle, monkeypatch):
    """Repeated, scaled and zero right-hand sides: their dependent basis
    columns are dropped and every column still converges."""
    import scipy.sparse as sp
    monkeypatch.setenv("G2P_BLOCK_KRYLOV", "1")
    n, rows, col, val, ptr = _ad(coracle)
    r = np.random.default_rng(3)
    B = r.standard_normal((n, 8))
    B[:, 3] = B[:, 1]
    B[:, 5] = -2.0 * B[:, 0]
    B[:, 6] = 0.0
    B[:, 7] = B[:, 2] + B[:, 4]
    S = g2p.Solver(rows, col, val, n, g2p.default_params(precision=precision, rtol=1e-10))
    X, st = S.solve(B)
    S.close()
    Am = sp.csr_matrix((val, col, ptr), shape=(n, n))
    nz = [c for c in range(8) if c != 6]
    res = np.linalg.norm(B[:, nz] - Am @ X[:, nz], axis=0) / np.linalg.norm(B[:, nz], axis=0)
    assert res.max() <= 1e-10 * 1.0001, res
    assert np.all(X[:, 6] == 0.0)
    # same tolerance as against the direct solve
    assert np.linalg.norm(X[:, 3] - X[:, 1]) <= 1e-7 * np.linalg.norm(X[:, 1])
    assert np.linalg.norm(X[:, 5] + 2.0 * X[:, 0]) <= 1e-7 * np.linalg.norm(X[:, 5])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_block_krylov_z_matches_lock_step(precision, g2p, monkeypatch):
    """Both ports of manhattan_sweep as one block (k = 2): Z agrees with the
    lock-step solver's to the solve tolerance."""
    d, A, M = golden_layout("manhattan_sweep")
    out = []
    for block in ("0", "1"):
        monkeypatch.setenv("G2P_BLOCK_KRYLOV", block)
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            Z, st = g2p.paraGenerator(m, g2p.default_params(precision=precision, rtol=1e-10, batch=2))
        out.append(Z)
    rel = np.abs(out[1] - out[0]).max() / np.abs(out[0]).max()
    assert rel < 1e-7, rel
    Zr = A["Z"].reshape(out[1].shape)
    assert np.abs(out[1] - Zr).max() / np.abs(Zr).max() < 1e-7


def test_gpu_block_krylov_graph_replay_identical(g2p, coracle, monkeypatch):
    """Block Arnoldi steps replayed from CUDA graphs give the same solution,
    bit for bit, as the same steps launched one kernel at a time."""
    monkeypatch.setenv("G2P_BLOCK_KRYLOV", "1")
    n, rows, col, val, ptr = _ad(coracle, name="multistrip_small")
    B = np.random.default_rng(5).standard_normal((n, 8))
    out = []
    for graphs in (0, 1):
        S = g2p.Solver(rows, col, val, n, g2p.default_params(precision="mixed", rtol=1e-10, use_graphs=graphs))
        X1, st1 = S.solve(B)
        X2, st2 = S.solve(B)      # second solve replays the captured steps
        S.close()
        assert np.array_equal(X1, X2)
        out.append((X2, st2.iterations))
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])
