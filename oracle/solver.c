/* CPU oracle: FP64 flexible GMRES preconditioned by aggregation AMG.
 * TEST INFRASTRUCTURE ONLY -- the checker, never the product.
 *
 * Stand-in for hypreSolve (reference hypreSolve.cpp:9-283).  HYPRE is not
 * vendored by the reference and has no pinned version (purdue_install.md:
 * 178-192); the published algorithm it is configured for is FlexGMRES(KDim=10,
 * MaxIter=100, Tol=1e-4) with one BoomerAMG V-cycle per iteration, hybrid
 * symmetric Gauss-Seidel relaxation (relax type 6, one sweep, ten while the
 * relative residual exceeds 0.1; hypreSolve.cpp:206-253,285-293).  This file
 * keeps the outer method, the relaxation and the sweep rule, and replaces
 * BoomerAMG's Falgout coarsening by smoothed-aggregation coarsening (Vanek,
 * Mandel, Brezina 1996), which is simpler to restate and converges to the
 * same solution: only the solve's residual, not its path, is compared. */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <stdio.h>
#include "oracle.h"

void g2po_csr_free(g2po_csr *A) {
    if (!A) return;
    free(A->ptr); free(A->col); free(A->val);
    A->ptr = NULL; A->col = NULL; A->val = NULL;
}

static g2po_csr csr_alloc(int64_t n, int64_t m, int64_t nnz) {
    g2po_csr A;
    A.n = n; A.m = m;
    A.ptr = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
    A.col = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnz > 0 ? nnz : 1));
    A.val = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    return A;
}

static g2po_csr csr_transpose(const g2po_csr *A) {
    int64_t nnz = A->ptr[A->n];
    g2po_csr T = csr_alloc(A->m, A->n, nnz);
    for (int64_t k = 0; k < nnz; k++) T.ptr[A->col[k] + 1]++;
    for (int64_t i = 0; i < A->m; i++) T.ptr[i + 1] += T.ptr[i];
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(A->m + 1));
    memcpy(fill, T.ptr, sizeof(int64_t) * (size_t)(A->m + 1));
    for (int64_t i = 0; i < A->n; i++)
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++) {
            int64_t p = fill[A->col[k]]++;
            T.col[p] = i;
            T.val[p] = A->val[k];
        }
    free(fill);
    return T;
}

static int cmp_i64(const void *a, const void *b) {
    int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
    return (x > y) - (x < y);
}

/* C = A*B (Gustavson, sorted columns, structural pattern kept). */
static g2po_csr csr_matmul(const g2po_csr *A, const g2po_csr *B) {
    int64_t *mark = (int64_t *)malloc(sizeof(int64_t) * (size_t)B->m);
    double *acc = (double *)calloc((size_t)B->m, sizeof(double));
    for (int64_t j = 0; j < B->m; j++) mark[j] = -1;
    int64_t cap = A->ptr[A->n] + B->ptr[B->n] + 16;
    g2po_csr C = csr_alloc(A->n, B->m, cap);
    int64_t *rowcols = (int64_t *)malloc(sizeof(int64_t) * (size_t)(B->m + 1));
    int64_t nnz = 0;
    for (int64_t i = 0; i < A->n; i++) {
        int64_t nr = 0;
        for (int64_t ka = A->ptr[i]; ka < A->ptr[i + 1]; ka++) {
            int64_t k = A->col[ka];
            double a = A->val[ka];
            for (int64_t kb = B->ptr[k]; kb < B->ptr[k + 1]; kb++) {
                int64_t j = B->col[kb];
                if (mark[j] != i) { mark[j] = i; acc[j] = 0.0; rowcols[nr++] = j; }
                acc[j] += a * B->val[kb];
            }
        }
        qsort(rowcols, (size_t)nr, sizeof(int64_t), cmp_i64);
        if (nnz + nr > cap) {
            cap = (nnz + nr) * 2;
            C.col = (int64_t *)realloc(C.col, sizeof(int64_t) * (size_t)cap);
            C.val = (double *)realloc(C.val, sizeof(double) * (size_t)cap);
        }
        for (int64_t t = 0; t < nr; t++) { C.col[nnz] = rowcols[t]; C.val[nnz] = acc[rowcols[t]]; nnz++; }
        C.ptr[i + 1] = nnz;
    }
    free(mark); free(acc); free(rowcols);
    return C;
}

static void csr_spmv(const g2po_csr *A, const double *x, double *y) {
    for (int64_t i = 0; i < A->n; i++) {
        double s = 0.0;
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++) s += A->val[k] * x[A->col[k]];
        y[i] = s;
    }
}

/* ------------------------------------------------------------------ AMG */
#define MAX_LEVELS 30
#define DENSE_ROW 32

typedef struct {
    g2po_csr A, P, R;
    double *diag;
    double *x, *b, *r;
} amg_level;

typedef struct {
    int nlev;
    amg_level lev[MAX_LEVELS];
    double *lu;          /* coarsest dense LU (row-major) */
    int64_t *piv;
    int64_t nc;
} amg_t;

static void amg_free(amg_t *h) {
    for (int l = 0; l < h->nlev; l++) {
        amg_level *L = &h->lev[l];
        g2po_csr_free(&L->A);
        if (l + 1 < h->nlev) { g2po_csr_free(&L->P); g2po_csr_free(&L->R); }
        free(L->diag); free(L->x); free(L->b); free(L->r);
    }
    free(h->lu); free(h->piv);
}

static double row_diag(const g2po_csr *A, int64_t i) {
    for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++)
        if (A->col[k] == i) return A->val[k];
    return 0.0;
}

/* Aggregates from the symmetric strength measure |a_ij| >= theta*sqrt(|a_ii a_jj|).
 * Rows with more than DENSE_ROW entries (a conductor's lumped potential in Ad)
 * are kept as singleton aggregates and ignored as neighbours. */
static int64_t dense_limit(const g2po_csr *A) {
    return DENSE_ROW + 4 * (A->ptr[A->n] / (A->n > 0 ? A->n : 1));
}

static int64_t aggregate(const g2po_csr *A, const double *diag, double theta, int64_t *agg) {
    int64_t n = A->n;
    int64_t lim = dense_limit(A);
    uint8_t *dense = (uint8_t *)calloc((size_t)n, 1);
    for (int64_t i = 0; i < n; i++) {
        dense[i] = (A->ptr[i + 1] - A->ptr[i]) > lim;
        agg[i] = -1;
    }
#define STRONG(i, k) (A->col[k] != (i) && !dense[A->col[k]] && \
    fabs(A->val[k]) >= theta * sqrt(fabs(diag[i] * diag[A->col[k]])))
    int64_t na = 0;
    for (int64_t i = 0; i < n; i++) if (dense[i]) agg[i] = na++;
    /* pass 1: roots whose strong neighbourhood is still free */
    for (int64_t i = 0; i < n; i++) {
        if (agg[i] >= 0) continue;
        int ok = 1, has = 0;
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++)
            if (STRONG(i, k)) { has = 1; if (agg[A->col[k]] >= 0) { ok = 0; break; } }
        if (!ok || !has) continue;
        agg[i] = na;
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++)
            if (STRONG(i, k)) agg[A->col[k]] = na;
        na++;
    }
    /* pass 2: attach to the aggregate of the strongest aggregated neighbour */
    int64_t *snap = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
    memcpy(snap, agg, sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < n; i++) {
        if (snap[i] >= 0) continue;
        double best = -1.0; int64_t ba = -1;
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++)
            if (STRONG(i, k) && snap[A->col[k]] >= 0 && !dense[A->col[k]] && fabs(A->val[k]) > best) {
                best = fabs(A->val[k]); ba = snap[A->col[k]];
            }
        if (ba >= 0) agg[i] = ba;
    }
    /* pass 3: the rest form aggregates with their free strong neighbours;
       rows with no strong connection get no coarse representative (their
       error is removed by the smoother alone) */
    for (int64_t i = 0; i < n; i++) {
        if (agg[i] >= 0) continue;
        int has = 0;
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++) if (STRONG(i, k)) { has = 1; break; }
        if (!has) continue;
        agg[i] = na;
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++)
            if (STRONG(i, k) && agg[A->col[k]] < 0) agg[A->col[k]] = na;
        na++;
    }
#undef STRONG
    free(snap); free(dense);
    return na;
}

static void lu_factor(double *a, int64_t n, int64_t *piv) {
    for (int64_t k = 0; k < n; k++) {
        int64_t p = k; double mx = fabs(a[k * n + k]);
        for (int64_t i = k + 1; i < n; i++) if (fabs(a[i * n + k]) > mx) { mx = fabs(a[i * n + k]); p = i; }
        piv[k] = p;
        if (p != k) for (int64_t j = 0; j < n; j++) { double t = a[k * n + j]; a[k * n + j] = a[p * n + j]; a[p * n + j] = t; }
        double d = a[k * n + k];
        if (d == 0.0) { a[k * n + k] = d = 1e-300; }
        for (int64_t i = k + 1; i < n; i++) {
            double f = a[i * n + k] / d;
            a[i * n + k] = f;
            if (f != 0.0) for (int64_t j = k + 1; j < n; j++) a[i * n + j] -= f * a[k * n + j];
        }
    }
}

static void lu_solve(const double *a, int64_t n, const int64_t *piv, double *b) {
    for (int64_t k = 0; k < n; k++) { int64_t p = piv[k]; if (p != k) { double t = b[k]; b[k] = b[p]; b[p] = t; } }
    for (int64_t i = 0; i < n; i++) for (int64_t j = 0; j < i; j++) b[i] -= a[i * n + j] * b[j];
    for (int64_t i = n - 1; i >= 0; i--) {
        for (int64_t j = i + 1; j < n; j++) b[i] -= a[i * n + j] * b[j];
        b[i] /= a[i * n + i];
    }
}

static void amg_setup(amg_t *h, const g2po_csr *A0, const g2po_solver_opts *o) {
    memset(h, 0, sizeof(*h));
    h->lev[0].A = *A0;           /* borrowed; copied below so amg_free may release it */
    h->lev[0].A = csr_alloc(A0->n, A0->m, A0->ptr[A0->n]);
    memcpy(h->lev[0].A.ptr, A0->ptr, sizeof(int64_t) * (size_t)(A0->n + 1));
    memcpy(h->lev[0].A.col, A0->col, sizeof(int64_t) * (size_t)A0->ptr[A0->n]);
    memcpy(h->lev[0].A.val, A0->val, sizeof(double) * (size_t)A0->ptr[A0->n]);
    int l = 0;
    for (;;) {
        amg_level *L = &h->lev[l];
        int64_t n = L->A.n;
        L->diag = (double *)malloc(sizeof(double) * (size_t)n);
        for (int64_t i = 0; i < n; i++) { double d = row_diag(&L->A, i); L->diag[i] = d != 0.0 ? d : 1.0; }
        L->x = (double *)calloc((size_t)n, sizeof(double));
        L->b = (double *)calloc((size_t)n, sizeof(double));
        L->r = (double *)calloc((size_t)n, sizeof(double));
        if (n <= o->coarse_size || l == MAX_LEVELS - 1) break;
        int64_t *agg = (int64_t *)malloc(sizeof(int64_t) * (size_t)n);
        int64_t na = aggregate(&L->A, L->diag, o->strength, agg);
        if (na == 0 || na > (n * 4) / 5) { free(agg); break; }
        /* tentative P, then one damped-Jacobi smoothing step P = (I - w D^-1 A) T */
        g2po_csr T = csr_alloc(n, na, n);
        int64_t tn = 0;
        for (int64_t i = 0; i < n; i++) {
            if (agg[i] >= 0) { T.col[tn] = agg[i]; T.val[tn] = 1.0; tn++; }
            T.ptr[i + 1] = tn;
        }
        double lmax = 0.0;
        for (int64_t i = 0; i < n; i++) {
            double s = 0.0;
            for (int64_t k = L->A.ptr[i]; k < L->A.ptr[i + 1]; k++) s += fabs(L->A.val[k]);
            s /= fabs(L->diag[i]);
            if (s > lmax) lmax = s;
        }
        double w = 4.0 / (3.0 * lmax);
        /* dense rows keep their tentative (unsmoothed) prolongation */
        g2po_csr DA = csr_alloc(n, n, L->A.ptr[n]);
        int64_t lim = dense_limit(&L->A), dn = 0;
        for (int64_t i = 0; i < n; i++) {
            if ((L->A.ptr[i + 1] - L->A.ptr[i]) <= lim)
                for (int64_t k = L->A.ptr[i]; k < L->A.ptr[i + 1]; k++) {
                    DA.col[dn] = L->A.col[k];
                    DA.val[dn] = -w * L->A.val[k] / L->diag[i];
                    dn++;
                }
            DA.ptr[i + 1] = dn;
        }
        g2po_csr DAT = csr_matmul(&DA, &T);
        /* P = T + DAT (same row order; merge) */
        g2po_csr P = csr_alloc(n, na, DAT.ptr[n] + n);
        int64_t nnz = 0;
        for (int64_t i = 0; i < n; i++) {
            int placed = agg[i] < 0;
            for (int64_t k = DAT.ptr[i]; k < DAT.ptr[i + 1]; k++) {
                int64_t j = DAT.col[k]; double v = DAT.val[k];
                if (!placed && j >= agg[i]) {
                    if (j == agg[i]) { v += 1.0; placed = 1; }
                    else { P.col[nnz] = agg[i]; P.val[nnz] = 1.0; nnz++; placed = 1; }
                }
                P.col[nnz] = j; P.val[nnz] = v; nnz++;
            }
            if (!placed) { P.col[nnz] = agg[i]; P.val[nnz] = 1.0; nnz++; }
            P.ptr[i + 1] = nnz;
        }
        g2po_csr_free(&DA); g2po_csr_free(&DAT); g2po_csr_free(&T); free(agg);
        if (getenv("G2PO_DEBUG")) {
            int64_t mx = 0, mxr = -1;
            for (int64_t i = 0; i < n; i++) if (P.ptr[i + 1] - P.ptr[i] > mx) { mx = P.ptr[i + 1] - P.ptr[i]; mxr = i; }
            fprintf(stderr, "[amg] P n=%lld na=%lld nnz=%lld maxrow=%lld at %lld lim=%lld\n", (long long)n, (long long)na,
                    (long long)P.ptr[n], (long long)mx, (long long)mxr, (long long)dense_limit(&L->A));
        }
        g2po_csr R = csr_transpose(&P);
        g2po_csr AP = csr_matmul(&L->A, &P);
        g2po_csr Ac = csr_matmul(&R, &AP);
        g2po_csr_free(&AP);
        L->P = P; L->R = R;
        h->lev[l + 1].A = Ac;
        l++;
    }
    h->nlev = l + 1;
    if (getenv("G2PO_DEBUG"))
        for (int q = 0; q <= l; q++)
            fprintf(stderr, "[amg] level %d n=%lld nnz=%lld\n", q, (long long)h->lev[q].A.n, (long long)h->lev[q].A.ptr[h->lev[q].A.n]);
    amg_level *C = &h->lev[l];
    h->nc = C->A.n;
    if (h->nc > 1500) { h->lu = NULL; h->piv = NULL; return; }   /* coarsest by relaxation */
    h->lu = (double *)calloc((size_t)(h->nc * h->nc), sizeof(double));
    h->piv = (int64_t *)malloc(sizeof(int64_t) * (size_t)(h->nc + 1));
    for (int64_t i = 0; i < h->nc; i++)
        for (int64_t k = C->A.ptr[i]; k < C->A.ptr[i + 1]; k++) h->lu[i * h->nc + C->A.col[k]] += C->A.val[k];
    lu_factor(h->lu, h->nc, h->piv);
}

static void gs_sweep(const g2po_csr *A, const double *diag, const double *b, double *x, int backward) {
    int64_t n = A->n;
    for (int64_t t = 0; t < n; t++) {
        int64_t i = backward ? n - 1 - t : t;
        double s = b[i];
        for (int64_t k = A->ptr[i]; k < A->ptr[i + 1]; k++)
            if (A->col[k] != i) s -= A->val[k] * x[A->col[k]];
        x[i] = s / diag[i];
    }
}

static void vcycle(amg_t *h, int l, int sweeps) {
    amg_level *L = &h->lev[l];
    if (l == h->nlev - 1) {
        if (h->lu) {
            memcpy(L->x, L->b, sizeof(double) * (size_t)L->A.n);
            lu_solve(h->lu, h->nc, h->piv, L->x);
        } else {
            for (int s = 0; s < 20; s++) { gs_sweep(&L->A, L->diag, L->b, L->x, 0); gs_sweep(&L->A, L->diag, L->b, L->x, 1); }
        }
        return;
    }
    for (int s = 0; s < sweeps; s++) gs_sweep(&L->A, L->diag, L->b, L->x, 0);
    csr_spmv(&L->A, L->x, L->r);
    for (int64_t i = 0; i < L->A.n; i++) L->r[i] = L->b[i] - L->r[i];
    amg_level *N = &h->lev[l + 1];
    csr_spmv(&L->R, L->r, N->b);
    memset(N->x, 0, sizeof(double) * (size_t)N->A.n);
    vcycle(h, l + 1, sweeps);
    for (int64_t i = 0; i < L->A.n; i++) {
        double s = 0.0;
        for (int64_t k = L->P.ptr[i]; k < L->P.ptr[i + 1]; k++) s += L->P.val[k] * N->x[L->P.col[k]];
        L->x[i] += s;
    }
    for (int s = 0; s < sweeps; s++) gs_sweep(&L->A, L->diag, L->b, L->x, 1);
}

static double dot(const double *a, const double *b, int64_t n) {
    double s = 0.0;
    for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

void g2po_solver_default_opts(g2po_solver_opts *o) {
    o->restart = 10; o->maxit = 100; o->rtol = 1e-4;
    o->pc_tol = 0.1; o->pc_mod_sweeps = 10;
    o->coarse_size = 400; o->strength = 0.08; o->reuse_setup = 0;
    o->stop_after_solves = 0;
}

static int fgmres(const g2po_csr *A, amg_t *h, const double *b, double *x,
                  const g2po_solver_opts *o, g2po_solve_stats *st) {
    int64_t n = A->n;
    int m = o->restart;
    double *V = (double *)malloc(sizeof(double) * (size_t)(n * (m + 1)));
    double *Z = (double *)malloc(sizeof(double) * (size_t)(n * m));
    double *H = (double *)calloc((size_t)((m + 1) * m), sizeof(double));
    double *cs = (double *)calloc((size_t)m, sizeof(double)), *sn = (double *)calloc((size_t)m, sizeof(double));
    double *g = (double *)calloc((size_t)(m + 1), sizeof(double)), *y = (double *)calloc((size_t)m, sizeof(double));
    double *w = (double *)malloc(sizeof(double) * (size_t)n);
    double bn = sqrt(dot(b, b, n));
    int it = 0;
    double rel = 0.0;
    if (bn == 0.0) { memset(x, 0, sizeof(double) * (size_t)n); st->iterations = 0; st->rel_residual = 0; st->converged = 1; goto done; }
    for (;;) {
        csr_spmv(A, x, w);
        for (int64_t i = 0; i < n; i++) V[i] = b[i] - w[i];
        double beta = sqrt(dot(V, V, n));
        rel = beta / bn;
        if (rel <= o->rtol || it >= o->maxit) break;
        for (int64_t i = 0; i < n; i++) V[i] /= beta;
        memset(g, 0, sizeof(double) * (size_t)(m + 1));
        g[0] = beta;
        int j;
        for (j = 0; j < m && it < o->maxit; j++, it++) {
            int sweeps = rel > o->pc_tol ? o->pc_mod_sweeps : 1;
            amg_level *L0 = &h->lev[0];
            memcpy(L0->b, V + (size_t)j * n, sizeof(double) * (size_t)n);
            memset(L0->x, 0, sizeof(double) * (size_t)n);
            vcycle(h, 0, sweeps);
            memcpy(Z + (size_t)j * n, L0->x, sizeof(double) * (size_t)n);
            csr_spmv(A, Z + (size_t)j * n, w);
            for (int i = 0; i <= j; i++) {
                double hij = dot(w, V + (size_t)i * n, n);
                H[i * m + j] = hij;
                for (int64_t k = 0; k < n; k++) w[k] -= hij * V[(size_t)i * n + k];
            }
            double hn = sqrt(dot(w, w, n));
            H[(j + 1) * m + j] = hn;
            if (hn != 0.0) for (int64_t k = 0; k < n; k++) V[(size_t)(j + 1) * n + k] = w[k] / hn;
            for (int i = 0; i < j; i++) {
                double t = cs[i] * H[i * m + j] + sn[i] * H[(i + 1) * m + j];
                H[(i + 1) * m + j] = -sn[i] * H[i * m + j] + cs[i] * H[(i + 1) * m + j];
                H[i * m + j] = t;
            }
            double a = H[j * m + j], c = H[(j + 1) * m + j];
            double r = sqrt(a * a + c * c);
            cs[j] = r != 0.0 ? a / r : 1.0; sn[j] = r != 0.0 ? c / r : 0.0;
            H[j * m + j] = r; H[(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            rel = fabs(g[j + 1]) / bn;
            if (rel <= o->rtol || hn == 0.0) { j++; it++; break; }
        }
        for (int i = j - 1; i >= 0; i--) {
            double s = g[i];
            for (int k = i + 1; k < j; k++) s -= H[i * m + k] * y[k];
            y[i] = s / H[i * m + i];
        }
        for (int i = 0; i < j; i++)
            for (int64_t k = 0; k < n; k++) x[k] += y[i] * Z[(size_t)i * n + k];
    }
    st->iterations = it;
    st->rel_residual = rel;
    st->converged = rel <= o->rtol;
done:
    free(V); free(Z); free(H); free(cs); free(sn); free(g); free(y); free(w);
    return 0;
}

/* Solve with a prebuilt hierarchy (used by the pipeline to reuse setups). */
typedef struct g2po_amg_handle { g2po_csr A; amg_t h; } g2po_amg_handle;

g2po_amg_handle *g2po_amg_create(const g2po_csr *A, const g2po_solver_opts *o) {
    g2po_amg_handle *H = (g2po_amg_handle *)calloc(1, sizeof(*H));
    H->A = *A;
    amg_setup(&H->h, A, o);
    return H;
}

int g2po_amg_solve(g2po_amg_handle *H, const double *b, double *x, const g2po_solver_opts *o,
                   g2po_solve_stats *st) {
    memset(x, 0, sizeof(double) * (size_t)H->A.n);
    int rc = fgmres(&H->A, &H->h, b, x, o, st);
    st->levels = H->h.nlev;
    return rc;
}

void g2po_amg_destroy(g2po_amg_handle *H) {
    if (!H) return;
    amg_free(&H->h);
    free(H);
}

int g2po_solve_coo(const int64_t *rows, const int64_t *cols, const double *vals, int64_t nnz,
                   const double *b, int64_t n, double *x, const g2po_solver_opts *o,
                   g2po_solve_stats *st) {
    g2po_csr A = csr_alloc(n, n, nnz);
    for (int64_t k = 0; k < nnz; k++) {
        if (rows[k] < 0 || rows[k] >= n || cols[k] < 0 || cols[k] >= n) { g2po_csr_free(&A); return -1; }
        A.ptr[rows[k] + 1]++;
    }
    for (int64_t i = 0; i < n; i++) A.ptr[i + 1] += A.ptr[i];
    memcpy(A.col, cols, sizeof(int64_t) * (size_t)nnz);   /* row-sorted COO: order kept */
    memcpy(A.val, vals, sizeof(double) * (size_t)nnz);
    g2po_amg_handle *H = g2po_amg_create(&A, o);
    int rc = g2po_amg_solve(H, b, x, o, st);
    g2po_amg_destroy(H);
    g2po_csr_free(&A);
    return rc;
}
