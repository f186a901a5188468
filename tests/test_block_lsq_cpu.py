"""The block FGMRES least-squares solver (gds2para_gb300/csrc/block_lsq.h,
host C++) against numpy's lstsq on random block upper-Hessenberg problems,
with and without dead indices (basis columns the Cholesky QR dropped as
dependent: a zero row and a zero column of Hbar, a zero row of the
right-hand side).  No GPU: a small driver compiled with g++."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "block_lsq.h"
int main(int argc, char **argv) {
    FILE *f = fopen(argv[1], "r");
    int K, m, J;
    if (fscanf(f, "%d %d %d", &K, &m, &J) != 3) return 2;
    std::vector<double> B0((size_t)K * K);
    for (auto &v : B0) if (fscanf(f, "%lf", &v) != 1) return 2;
    g2p::BlockLSQ ls;
    ls.reset(K, m, B0.data());
    std::vector<double> res(K);
    for (int j = 0; j < J; j++) {
        std::vector<double> h((size_t)(j + 2) * K * K);
        for (auto &v : h) if (fscanf(f, "%lf", &v) != 1) return 2;
        ls.add_block(j, h.data(), res.data());
        for (int r = 0; r < K; r++) printf("%.17g ", res[r]);
        printf("\n");
    }
    std::vector<double> Y((size_t)J * K * K);
    ls.solve(J * K, Y.data());
    for (double v : Y) printf("%.17g ", v);
    printf("\n");
    return 0;
}
"""


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    d = tmp_path_factory.mktemp("lsq")
    src = d / "lsq.cpp"
    src.write_text(DRIVER)
    exe = d / "lsq"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "gds2para_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    return exe


def _problem(K, J, seed, dead=()):
    """A random (J+1)K x JK block upper-Hessenberg Hbar (subdiagonal blocks
    upper triangular) and B0 (upper triangular); raw indices in dead have
    zero rows and columns, and a zero row in B0 if below K.  As in the block
    Arnoldi process, a dead index i makes i + K dead too (its basis vector is
    zero, so is its preconditioned vector and the next block's column)."""
    dead = sorted({i + t * K for i in dead for t in range(J + 1) if i + t * K < (J + 1) * K})
    r = np.random.default_rng(seed)
    H = np.zeros(((J + 1) * K, J * K))
    for j in range(J):
        H[: (j + 1) * K, j * K:(j + 1) * K] = r.standard_normal(((j + 1) * K, K))
        R = np.triu(r.standard_normal((K, K)))
        R[np.diag_indices(K)] = np.abs(R[np.diag_indices(K)]) + 0.5
        H[(j + 1) * K:(j + 2) * K, j * K:(j + 1) * K] = R
    B0 = np.triu(r.standard_normal((K, K)))
    B0[np.diag_indices(K)] = np.abs(B0[np.diag_indices(K)]) + 0.5
    for i in dead:
        H[i, :] = 0.0
        if i < J * K:
            H[:, i] = 0.0
        if i < K:
            B0[i, :] = 0.0
    return H, B0


def _run(driver, tmp_path, H, B0, K, J, m):
    lines = [f"{K} {m} {J}", " ".join(repr(float(v)) for v in B0.ravel())]
    for j in range(J):
        lines.append(" ".join(repr(float(v)) for v in H[: (j + 2) * K, j * K:(j + 1) * K].ravel()))
    p = tmp_path / "in.txt"
    p.write_text("\n".join(lines) + "\n")
    out = subprocess.run([str(driver), str(p)], check=True, capture_output=True, text=True).stdout.split("\n")
    res = [np.array([float(v) for v in out[j].split()]) for j in range(J)]
    Y = np.array([float(v) for v in out[J].split()]).reshape(J * K, K)
    return res, Y


@pytest.mark.parametrize("K,J,dead", [(2, 4, ()), (4, 5, ()), (8, 3, ()), (4, 5, (3, 6, 13)), (8, 4, (1, 9, 10, 30))])
def test_block_lsq_matches_lstsq(K, J, dead, driver, tmp_path):
    H, B0 = _problem(K, J, 100 + K + J + len(dead), dead)
    dead = sorted({i + t * K for i in dead for t in range(J + 1) if i + t * K < (J + 1) * K})
    res, Y = _run(driver, tmp_path, H, B0, K, J, m=J + 1)
    rhs = np.zeros(((J + 1) * K, K))
    rhs[:K] = B0
    for j in range(J):
        Hj = H[: (j + 2) * K, : (j + 1) * K]
        bj = rhs[: (j + 2) * K]
        Yj = np.linalg.lstsq(Hj, bj, rcond=None)[0]
        rj = np.linalg.norm(bj - Hj @ Yj, axis=0)
        np.testing.assert_allclose(res[j], rj, rtol=1e-9, atol=1e-12 * np.linalg.norm(bj))
    Yr = np.linalg.lstsq(H, rhs, rcond=None)[0]
    np.testing.assert_allclose(Y, Yr, rtol=1e-8, atol=1e-10 * np.abs(Yr).max())
    for i in dead:
        if i < J * K:
            assert np.all(Y[i] == 0.0)
