"""Host-side parts of the full-wave (Vh) path, no GPU needed: the library's
Hessenberg eigenvalue routine (its dhseqr stand-in, called by g2p_find_vh on
the k x k Arnoldi matrix) and the oracle's dhseqr/dhsein stand-ins, both
against numpy's general eigensolver on seeded Hessenberg matrices."""
import ctypes as C

import numpy as np
import pytest

from gds2para_gb300 import api


def _hessenberg(n, seed, scale=1.0):
    r = np.random.default_rng(seed)
    h = np.triu(r.standard_normal((n, n)) * scale, -1)
    return h


def _backward_error(h, lam):
    """min singular value of h - lam I relative to |h|: ~ ulp for an
    eigenvalue computed by a backward-stable method."""
    n = h.shape[0]
    s = np.linalg.svd(h - lam * np.eye(n), compute_uv=False)
    return s[-1] / np.linalg.norm(h, 2)


@pytest.mark.parametrize("n", [1, 2, 7, 40, 250])
def test_library_hessenberg_eigenvalues(n):
    h = _hessenberg(n, 100 + n)
    lam = api.hessenbergEigenvalues(h)
    assert lam.shape == (n,)
    ref = np.linalg.eigvals(h)
    # same multiset (matched by sorting on real then imaginary parts)
    a = np.sort_complex(lam)
    b = np.sort_complex(ref)
    assert np.max(np.abs(a - b)) < 1e-8 * max(1.0, np.max(np.abs(b)))
    for v in lam:
        assert _backward_error(h, v) < 1e-14
    # conjugate pairs adjacent, positive imaginary part first
    i = 0
    while i < n:
        if lam[i].imag != 0:
            assert lam[i].imag > 0 and lam[i + 1] == np.conj(lam[i])
            i += 2
        else:
            i += 1


def test_library_hessenberg_eigenvalues_scaled():
    """The Arnoldi matrices of find_Vh carry entries of order 1e0..1e2 after
    the 1e14 operator scaling; a wide dynamic range must not lose pairs."""
    h = _hessenberg(120, 7)
    h[np.arange(1, 120), np.arange(119)] *= 1e-3
    lam = api.hessenbergEigenvalues(h)
    for v in lam:
        assert _backward_error(h, v) < 1e-13


def test_library_hessenberg_rejects_bad_size():
    with pytest.raises(api.G2PError):
        api.hessenbergEigenvalues(np.zeros((0, 0)))


def test_oracle_standins_eigenpairs():
    """oracle/lapacke_shim.cpp: LAPACKE_dhseqr eigenvalues and
    LAPACKE_dhsein right eigenvectors (a complex pair as two real columns,
    re and im) satisfy h v = lam v."""
    import oracle.harness as hh
    L = C.CDLL(hh.build_coracle())
    lint = C.c_longlong
    n = 60
    h = np.asfortranarray(_hessenberg(n, 3))
    hq = h.copy(order="F")
    wr, wi = np.zeros(n), np.zeros(n)
    L.LAPACKE_dhseqr.restype = lint
    L.LAPACKE_dhseqr.argtypes = [C.c_int, C.c_char, C.c_char, lint, lint, lint, C.c_void_p, lint, C.c_void_p,
                                 C.c_void_p, C.c_void_p, lint]
    assert L.LAPACKE_dhseqr(102, b"E", b"N", n, 1, n, hq.ctypes.data, n, wr.ctypes.data, wi.ctypes.data, None, n) == 0
    lam = wr + 1j * wi
    assert np.max(np.abs(np.sort_complex(lam) - np.sort_complex(np.linalg.eigvals(h)))) < 1e-8
    sel = (np.abs(wi) > 1e-6).astype(np.int64)
    mm = int(sel.sum())
    vr = np.zeros((n, mm), order="F")
    m = lint()
    ifl = np.zeros(max(mm, 1), np.int64)
    L.LAPACKE_dhsein.restype = lint
    L.LAPACKE_dhsein.argtypes = [C.c_int, C.c_char, C.c_char, C.c_char, C.c_void_p, lint, C.c_void_p, lint,
                                 C.c_void_p, C.c_void_p, C.c_void_p, lint, C.c_void_p, lint, lint, C.POINTER(lint),
                                 C.c_void_p, C.c_void_p]
    assert L.LAPACKE_dhsein(102, b"R", b"Q", b"N", sel.ctypes.data, n, h.ctypes.data, n, wr.ctypes.data,
                            wi.ctypes.data, None, n, vr.ctypes.data, n, mm, C.byref(m), ifl.ctypes.data,
                            ifl.ctypes.data) == 0
    col = 0
    for j in range(n):
        if wi[j] > 1e-6:
            v = vr[:, col] + 1j * vr[:, col + 1]
            res = np.linalg.norm(h @ v - lam[j] * v) / (np.linalg.norm(h, 2) * np.linalg.norm(v))
            assert res < 1e-12
            col += 2
    assert col == m.value == mm
