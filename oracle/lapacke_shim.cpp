/* Dense stand-ins for the LAPACKE and PARDISO routines on the reference's
 * full-wave (Vh) path, for compiling the reference's own find_Vh
 * (src/fdtd.hpp:3577-3859), Vh products (src/matrixCon.cpp:609-805) and
 * reference1 (src/fdtd.hpp:3963-4071) as a CPU oracle.  TEST INFRASTRUCTURE
 * ONLY.  LAPACK and MKL are not in this image; these restate the published
 * algorithms the reference calls them for, in plain double and complex
 * arithmetic, for the small systems the oracle runs:
 *   LAPACKE_dhseqr  eigenvalues of an upper Hessenberg matrix: Francis
 *                   double-shift QR iteration (Francis 1961) with deflation
 *                   on negligible subdiagonal entries;
 *   LAPACKE_dhsein  right eigenvectors of selected eigenvalues by inverse
 *                   iteration on H - lambda I (complex pairs as two real
 *                   columns, real part then imaginary part; each vector
 *                   scaled so that its largest |re| + |im| is 1);
 *   LAPACKE_zgesv, LAPACKE_zcgesv   complex LU with partial pivoting;
 *   pardiso         phase 13 on a complex unsymmetric CSR (mtype 13) by a
 *                   dense complex LU; phase -1 releases nothing.
 * The calls come from sites declared variadic in mkl.h; on x86-64 and
 * AArch64 Linux a variadic call passes these arguments as a prototyped one
 * does, and this file gives the prototypes.  They override the aborting
 * weak definitions of mkl_sparse_shim.cpp. */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <vector>

typedef long long lint;
typedef std::complex<double> cd;

namespace {

// ---------------------------------------------------------- eigenvalues
// Eigenvalues of the upper Hessenberg matrix a (column-major, n x n, leading
// dimension lda), destroyed.  Complex conjugate pairs are stored at
// consecutive positions with the positive imaginary part first.
int hessenberg_eigenvalues(lint n, double *a, lint lda, double *wr, double *wi) {
    auto A = [&](lint i, lint j) -> double & { return a[i + j * lda]; };
    double anorm = 0;
    for (lint j = 0; j < n; j++)
        for (lint i = 0; i <= std::min(j + 1, n - 1); i++) anorm += std::fabs(A(i, j));
    const double eps = 2.220446049250313e-16;
    lint hi = n - 1;
    double shift_acc = 0;          // exceptional shifts applied to the diagonal
    int its = 0;
    while (hi >= 0) {
        // smallest l such that the subdiagonal entries l..hi are not negligible
        lint l = hi;
        for (; l >= 1; l--) {
            double s = std::fabs(A(l - 1, l - 1)) + std::fabs(A(l, l));
            if (s == 0) s = anorm;
            if (std::fabs(A(l, l - 1)) <= eps * s) {
                A(l, l - 1) = 0;
                break;
            }
        }
        const double x = A(hi, hi);
        if (l == hi) {                      // a 1 x 1 block splits off
            wr[hi] = x + shift_acc;
            wi[hi] = 0;
            hi--;
            its = 0;
            continue;
        }
        const double y = A(hi - 1, hi - 1), w = A(hi, hi - 1) * A(hi - 1, hi);
        if (l == hi - 1) {                  // a 2 x 2 block splits off
            const double p = 0.5 * (y - x), q = p * p + w, z = std::sqrt(std::fabs(q));
            if (q >= 0) {
                const double zz = p + (p >= 0 ? z : -z);
                wr[hi - 1] = wr[hi] = x + zz + shift_acc;
                if (zz != 0) wr[hi] = x - w / zz + shift_acc;
                wi[hi - 1] = wi[hi] = 0;
            } else {
                wr[hi - 1] = wr[hi] = x + p + shift_acc;
                wi[hi - 1] = z;
                wi[hi] = -z;
            }
            hi -= 2;
            its = 0;
            continue;
        }
        if (its >= 60 * n) return (int)(hi + 1);
        double sx = x, sy = y, sw = w;
        if (its > 0 && its % 10 == 0) {     // exceptional shift
            shift_acc += x;
            for (lint i = 0; i <= hi; i++) A(i, i) -= x;
            const double s = std::fabs(A(hi, hi - 1)) + std::fabs(A(hi - 1, hi - 2));
            sx = sy = 0.75 * s;
            sw = -0.4375 * s * s;
        }
        its++;
        // first column of (H - s1 I)(H - s2 I) from rows m..m+2, looking for
        // a start row m >= l where the bulge stays small
        lint m = hi - 2;
        double p = 0, q = 0, r = 0;
        for (; m >= l; m--) {
            const double z = A(m, m), rr = sx - z, ss = sy - z;
            p = (rr * ss - sw) / A(m + 1, m) + A(m, m + 1);
            q = A(m + 1, m + 1) - z - rr - ss;
            r = A(m + 2, m + 1);
            const double s = std::fabs(p) + std::fabs(q) + std::fabs(r);
            p /= s; q /= s; r /= s;
            if (m == l) break;
            const double u = std::fabs(A(m, m - 1)) * (std::fabs(q) + std::fabs(r));
            const double v = std::fabs(p) * (std::fabs(A(m - 1, m - 1)) + std::fabs(z) + std::fabs(A(m + 1, m + 1)));
            if (u <= eps * v) break;
        }
        for (lint i = m + 2; i <= hi; i++) {
            A(i, i - 2) = 0;
            if (i != m + 2) A(i, i - 3) = 0;
        }
        // chase the bulge with 3 x 3 (last: 2 x 2) Householder reflectors
        for (lint kk = m; kk <= hi - 1; kk++) {
            if (kk != m) {
                p = A(kk, kk - 1);
                q = A(kk + 1, kk - 1);
                r = kk != hi - 1 ? A(kk + 2, kk - 1) : 0;
                const double xs = std::fabs(p) + std::fabs(q) + std::fabs(r);
                if (xs == 0) continue;
                p /= xs; q /= xs; r /= xs;
            }
            double s = std::sqrt(p * p + q * q + r * r);
            if (p < 0) s = -s;
            if (kk == m) {
                if (l != m) A(kk, kk - 1) = -A(kk, kk - 1);
            } else {
                const double xs = std::fabs(A(kk, kk - 1)) + std::fabs(A(kk + 1, kk - 1)) +
                                  (kk != hi - 1 ? std::fabs(A(kk + 2, kk - 1)) : 0.0);
                A(kk, kk - 1) = -s * xs;
            }
            p += s;
            const double vx = p / s, vy = q / s, vz = r / s;
            q /= p;
            r /= p;
            for (lint j = kk; j < n; j++) {             // rows kk..kk+2 from the left
                double t = A(kk, j) + q * A(kk + 1, j);
                if (kk != hi - 1) {
                    t += r * A(kk + 2, j);
                    A(kk + 2, j) -= t * vz;
                }
                A(kk + 1, j) -= t * vy;
                A(kk, j) -= t * vx;
            }
            const lint imax = std::min(hi, kk + 3);
            for (lint i = 0; i <= imax; i++) {           // columns kk..kk+2 from the right
                double t = vx * A(i, kk) + vy * A(i, kk + 1);
                if (kk != hi - 1) {
                    t += vz * A(i, kk + 2);
                    A(i, kk + 2) -= t * r;
                }
                A(i, kk + 1) -= t * q;
                A(i, kk) -= t;
            }
        }
    }
    return 0;
}

// ----------------------------------------------------------- dense LU
// Solves a x = b in place for nrhs columns (column-major), partial pivoting.
int complex_lu_solve(lint n, std::vector<cd> &a, lint nrhs, cd *b, lint ldb) {
    auto A = [&](lint i, lint j) -> cd & { return a[(size_t)(i + j * n)]; };
    std::vector<lint> piv((size_t)n);
    int info = 0;
    for (lint k = 0; k < n; k++) {
        lint p = k;
        double mv = std::abs(A(k, k));
        for (lint i = k + 1; i < n; i++)
            if (std::abs(A(i, k)) > mv) { mv = std::abs(A(i, k)); p = i; }
        piv[(size_t)k] = p;
        if (mv == 0) { info = (int)(k + 1); continue; }
        if (p != k)
            for (lint j = 0; j < n; j++) std::swap(A(k, j), A(p, j));
        const cd d = A(k, k);
        for (lint i = k + 1; i < n; i++) A(i, k) /= d;
        for (lint j = k + 1; j < n; j++) {
            const cd f = A(k, j);
            if (f == cd(0)) continue;
            for (lint i = k + 1; i < n; i++) A(i, j) -= A(i, k) * f;
        }
    }
    for (lint c = 0; c < nrhs; c++) {
        cd *x = b + c * ldb;
        for (lint k = 0; k < n; k++) std::swap(x[k], x[piv[(size_t)k]]);
        for (lint k = 0; k < n; k++)
            for (lint i = k + 1; i < n; i++) x[i] -= A(i, k) * x[k];
        for (lint k = n - 1; k >= 0; k--) {
            x[k] /= A(k, k);
            for (lint i = 0; i < k; i++) x[i] -= A(i, k) * x[k];
        }
    }
    return info;
}

// Eigenvector of the real upper Hessenberg h (column-major) for the
// eigenvalue lambda: inverse iteration on h - lambda I (LU of a Hessenberg
// matrix: one row interchange and one multiplier per column, O(n^2)), scaled
// so that the largest |re| + |im| of its entries is 1.
std::vector<cd> hessenberg_eigenvector(lint n, const double *h, lint ldh, cd lambda, double hnorm) {
    std::vector<cd> a((size_t)(n * n), cd(0));
    auto A = [&](lint i, lint j) -> cd & { return a[(size_t)(i + j * n)]; };
    for (lint j = 0; j < n; j++)
        for (lint i = 0; i <= std::min(j + 1, n - 1); i++) A(i, j) = cd(h[i + j * ldh]);
    // a tiny shift away from the computed eigenvalue keeps the LU finite
    const double tiny = 1e-13 * std::max(hnorm, 1e-300);
    for (lint i = 0; i < n; i++) A(i, i) -= lambda + cd(tiny, 0);
    std::vector<char> swp((size_t)n, 0);
    std::vector<cd> mul((size_t)n, cd(0));
    for (lint k = 0; k + 1 < n; k++) {
        if (std::abs(A(k + 1, k)) > std::abs(A(k, k))) {
            swp[(size_t)k] = 1;
            for (lint j = k; j < n; j++) std::swap(A(k, j), A(k + 1, j));
        }
        if (A(k, k) == cd(0)) A(k, k) = cd(tiny, 0);
        const cd m = A(k + 1, k) / A(k, k);
        mul[(size_t)k] = m;
        for (lint j = k + 1; j < n; j++) A(k + 1, j) -= m * A(k, j);
    }
    if (A(n - 1, n - 1) == cd(0)) A(n - 1, n - 1) = cd(tiny, 0);
    std::vector<cd> x((size_t)n, cd(1.0 / std::sqrt((double)n), 0));
    for (int it = 0; it < 3; it++) {
        for (lint k = 0; k + 1 < n; k++) {
            if (swp[(size_t)k]) std::swap(x[(size_t)k], x[(size_t)k + 1]);
            x[(size_t)k + 1] -= mul[(size_t)k] * x[(size_t)k];
        }
        for (lint k = n - 1; k >= 0; k--) {
            x[(size_t)k] /= A(k, k);
            const cd xk = x[(size_t)k];
            for (lint i = 0; i < k; i++) x[(size_t)i] -= A(i, k) * xk;
        }
        double mx = 0;
        for (lint i = 0; i < n; i++) mx = std::max(mx, std::abs(x[(size_t)i]));
        if (mx == 0 || !std::isfinite(mx)) break;
        for (auto &v : x) v /= mx;
    }
    double big = 0;
    for (auto &v : x) big = std::max(big, std::fabs(v.real()) + std::fabs(v.imag()));
    if (big > 0)
        for (auto &v : x) v /= big;
    return x;
}

}  // namespace

extern "C" {

lint LAPACKE_dhseqr(int layout, char job, char compz, lint n, lint ilo, lint ihi, double *h, lint ldh, double *wr,
                    double *wi, double *z, lint ldz) {
    (void)layout; (void)job; (void)compz; (void)ilo; (void)ihi; (void)z; (void)ldz;
    return hessenberg_eigenvalues(n, h, ldh, wr, wi);
}

lint LAPACKE_dhsein(int layout, char side, char eigsrc, char initv, lint *select, lint n, const double *h, lint ldh,
                    double *wr, const double *wi, double *vl, lint ldvl, double *vr, lint ldvr, lint mm, lint *m,
                    lint *ifaill, lint *ifailr) {
    (void)layout; (void)side; (void)eigsrc; (void)initv; (void)vl; (void)ldvl; (void)ifaill;
    double hnorm = 0;
    for (lint j = 0; j < n; j++)
        for (lint i = 0; i <= std::min(j + 1, n - 1); i++) hnorm += std::fabs(h[i + j * ldh]);
    lint col = 0, nf = 0;
    for (lint j = 0; j < n; j++) {
        const bool pair = wi[j] != 0 && j + 1 < n && wi[j] > 0;
        if (pair) {
            if (!select[j] && !select[j + 1]) { j++; continue; }
            select[j] = 1;
            select[j + 1] = 0;
            if (col + 2 > mm) return -1;
            const std::vector<cd> x = hessenberg_eigenvector(n, h, ldh, cd(wr[j], wi[j]), hnorm);
            for (lint i = 0; i < n; i++) {
                vr[i + col * ldvr] = x[(size_t)i].real();
                vr[i + (col + 1) * ldvr] = x[(size_t)i].imag();
            }
            ifailr[nf++] = 0;
            ifailr[nf++] = 0;
            col += 2;
            j++;
        } else if (select[j]) {
            if (col + 1 > mm) return -1;
            const std::vector<cd> x = hessenberg_eigenvector(n, h, ldh, cd(wr[j], 0), hnorm);
            for (lint i = 0; i < n; i++) vr[i + col * ldvr] = x[(size_t)i].real();
            ifailr[nf++] = 0;
            col++;
        }
    }
    *m = col;
    return 0;
}

lint LAPACKE_zgesv(int layout, lint n, lint nrhs, cd *a, lint lda, lint *ipiv, cd *b, lint ldb) {
    (void)layout;
    std::vector<cd> m((size_t)(n * n));
    for (lint j = 0; j < n; j++)
        for (lint i = 0; i < n; i++) m[(size_t)(i + j * n)] = a[i + j * lda];
    for (lint i = 0; i < n; i++) ipiv[i] = i + 1;
    return complex_lu_solve(n, m, nrhs, b, ldb);
}

lint LAPACKE_zcgesv(int layout, lint n, lint nrhs, cd *a, lint lda, lint *ipiv, cd *b, lint ldb, cd *x, lint ldx,
                    lint *iter) {
    for (lint c = 0; c < nrhs; c++)
        for (lint i = 0; i < n; i++) x[i + c * ldx] = b[i + c * ldb];
    *iter = 0;
    return LAPACKE_zgesv(layout, n, nrhs, a, lda, ipiv, x, ldx);
}

void pardisoinit(void *pt, const lint *mtype, lint *iparm) {
    (void)pt; (void)mtype;
    for (int i = 0; i < 64; i++) iparm[i] = 0;
}

void pardiso(void *pt, const lint *maxfct, const lint *mnum, const lint *mtype, const lint *phase, const lint *n,
             const void *a, const lint *ia, const lint *ja, lint *perm, const lint *nrhs, lint *iparm,
             const lint *msglvl, void *b, void *x, lint *error) {
    (void)pt; (void)maxfct; (void)mnum; (void)perm; (void)msglvl;
    *error = 0;
    if (*phase < 0) return;
    if (*mtype != 13 || *phase != 13) {
        std::fprintf(stderr, "pardiso stand-in: only mtype 13, phase 13\n");
        std::abort();
    }
    const lint nn = *n, base = iparm[34] ? 0 : 1;
    const cd *av = static_cast<const cd *>(a);
    std::vector<cd> m((size_t)(nn * nn), cd(0));
    for (lint i = 0; i < nn; i++)
        for (lint q = ia[i] - base; q < ia[i + 1] - base; q++) m[(size_t)(i + (ja[q] - base) * nn)] += av[q];
    cd *xv = static_cast<cd *>(x);
    const cd *bv = static_cast<const cd *>(b);
    for (lint c = 0; c < *nrhs; c++)
        for (lint i = 0; i < nn; i++) xv[i + c * nn] = bv[i + c * nn];
    if (complex_lu_solve(nn, m, *nrhs, xv, nn) != 0) *error = -4;
}

}  // extern "C"
