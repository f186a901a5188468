"""The matrix-free curl-curl stencil (g2p_stiff_apply with matrix_free = 1:
TMA-tiled face circulations then edge sums) against the assembled S: the
oracle's CSR product on the golden layouts and the library's own CSR product
at the c2 bench size.  Equal to rounding (the stencil sums each row face by
face instead of entry by entry)."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_layout

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_stencil_matches_oracle_stiffness_product(name, g2p, coracle):
    d, A, M = golden_layout(name)
    ptr, col, val = coracle.stiffness(d)
    n = len(ptr) - 1
    x = np.random.default_rng(1).normal(size=n)
    rows = np.repeat(np.arange(n), np.diff(ptr))
    want = np.bincount(rows, weights=val * x[col], minlength=n)
    with g2p.FdtdMesh(d) as m:
        g2p.generateStiff(m)
        y, _ = g2p.stiffApply(m, x, matrix_free=True)
        y_csr, _ = g2p.stiffApply(m, x, matrix_free=False)
    scale = np.abs(want).max()
    assert np.abs(y - want).max() / scale < 1e-13
    assert np.abs(y_csr - want).max() / scale < 1e-13


def test_gpu_stencil_matches_csr_at_bench_size(g2p):
    from gds2para_gb300 import layout as lay
    d = lay.build(lay.config("c2"))
    with g2p.FdtdMesh(d) as m:
        g2p.generateStiff(m)
        n = d.N_edge - m.sizes().bden
        x = np.random.default_rng(2).normal(size=n)
        y, t_mf = g2p.stiffApply(m, x, matrix_free=True, reps=5)
        y_csr, t_csr = g2p.stiffApply(m, x, matrix_free=False, reps=5)
    assert np.abs(y - y_csr).max() / np.abs(y_csr).max() < 1e-13
    assert t_mf > 0 and t_csr > 0


def test_gpu_full_wave_arnoldi_same_with_csr_or_stencil(g2p, monkeypatch):
    d, A, M = golden_layout("strip_tiny_vh")
    out = []
    for stencil in (False, True):
        if stencil:
            monkeypatch.setenv("G2P_FW_STENCIL", "1")
        with g2p.FdtdMesh(d) as m:
            g2p.generateStiff(m)
            out.append(g2p.findVh(m, 40))
    monkeypatch.delenv("G2P_FW_STENCIL")
    assert out[0].shape == out[1].shape
    qa, _ = np.linalg.qr(out[0])
    qb, _ = np.linalg.qr(out[1])
    assert np.linalg.svd(qa.conj().T @ qb, compute_uv=False).min() > 1 - 1e-10


def test_gpu_full_wave_reference_setting_with_stencil(g2p, monkeypatch):
    """k = 1000 with S applied by the stencil: the rounding the Arnoldi
    basis amplifies moves a few eigenvalues across the |Im| > 1e-6 filter,
    and Z stays within the spread the reference setting allows."""
    d, A, M = golden_layout("strip_tiny_vh")
    monkeypatch.setenv("G2P_FW_STENCIL", "1")
    with g2p.FdtdMesh(d) as m:
        g2p.generateStiff(m)
        vh = g2p.findVh(m, 1000)
        z_vh, z_v0, _ = g2p.paraGeneratorVh(m, g2p.default_params(rtol=1e-12), 1000)
    monkeypatch.delenv("G2P_FW_STENCIL")
    assert abs(vh.shape[1] - M["leng_Vh"]) <= 8
    zf = A["Z"].reshape(z_vh.shape)
    assert np.abs(z_vh[1:] - zf[1:]).max() / np.abs(zf[1:]).max() < 2e-2
