/* Minimal implementation of the MKL sparse-BLAS calls made by the reference's
 * hot path, so that its own sources can run unmodified as a CPU oracle.
 *
 *   mkl_sparse_d_create_csr  generateStiff.cpp:918-921, matrixCon.cpp:109-113,313-317
 *   mkl_sparse_d_mv          matrixCon.cpp:384,411-412,436,451,528-529,540,553-554
 *   mkl_sparse_spmm          generateStiff.cpp:926 (op = TRANSPOSE: C = A^T * B)
 *   mkl_sparse_d_export_csr  generateStiff.cpp:931
 *   mkl_sparse_destroy       generateStiff.cpp:976-978, matrixCon.cpp:903-906
 *
 * The product keeps the structural pattern (no zero filtering) and emits each
 * row's columns in increasing order; each entry is summed over the shared
 * inner index in increasing order.  Test infrastructure only. */
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include "mkl.h"

struct g2p_shim_csr {
    MKL_INT rows, cols;
    MKL_INT *rs, *re, *ci;
    double *v;
    bool owned;
};

extern "C" sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, sparse_index_base_t base,
                                                   MKL_INT rows, MKL_INT cols, MKL_INT *rows_start,
                                                   MKL_INT *rows_end, MKL_INT *col_indx, double *values) {
    if (base != SPARSE_INDEX_BASE_ZERO) return SPARSE_STATUS_NOT_SUPPORTED;
    g2p_shim_csr *m = new g2p_shim_csr{rows, cols, rows_start, rows_end, col_indx, values, false};
    *A = m;
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_d_mv(sparse_operation_t op, double alpha, const sparse_matrix_t A,
                                           struct matrix_descr, const double *x, double beta, double *y) {
    if (op == SPARSE_OPERATION_NON_TRANSPOSE) {
        for (MKL_INT i = 0; i < A->rows; i++) {
            double s = 0.0;
            for (MKL_INT k = A->rs[i]; k < A->re[i]; k++) s += A->v[k] * x[A->ci[k]];
            y[i] = (beta == 0.0 ? 0.0 : beta * y[i]) + alpha * s;
        }
    } else {
        for (MKL_INT j = 0; j < A->cols; j++) y[j] = (beta == 0.0 ? 0.0 : beta * y[j]);
        for (MKL_INT i = 0; i < A->rows; i++) {
            double xi = alpha * x[i];
            for (MKL_INT k = A->rs[i]; k < A->re[i]; k++) y[A->ci[k]] += A->v[k] * xi;
        }
    }
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_spmm(sparse_operation_t op, const sparse_matrix_t A,
                                           const sparse_matrix_t B, sparse_matrix_t *C) {
    if (op != SPARSE_OPERATION_TRANSPOSE || A->rows != B->rows) return SPARSE_STATUS_NOT_SUPPORTED;
    /* C = A^T B: row i of C gathers, over inner index f in increasing order,
       A(f,i) * B(f,:).  Build A^T (CSR) with inner indices ascending. */
    MKL_INT nr = A->cols, ni = A->rows, nc = B->cols;
    std::vector<MKL_INT> tptr(nr + 1, 0);
    for (MKL_INT f = 0; f < ni; f++)
        for (MKL_INT k = A->rs[f]; k < A->re[f]; k++) tptr[A->ci[k] + 1]++;
    for (MKL_INT i = 0; i < nr; i++) tptr[i + 1] += tptr[i];
    std::vector<MKL_INT> tcol(tptr[nr]);
    std::vector<double> tval(tptr[nr]);
    std::vector<MKL_INT> fill(tptr.begin(), tptr.end() - 1);
    for (MKL_INT f = 0; f < ni; f++)
        for (MKL_INT k = A->rs[f]; k < A->re[f]; k++) {
            MKL_INT p = fill[A->ci[k]]++;
            tcol[p] = f;
            tval[p] = A->v[k];
        }
    std::vector<MKL_INT> rptr(nr + 1, 0);
    std::vector<MKL_INT> cols;
    std::vector<double> vals;
    std::vector<MKL_INT> mark(nc, -1);
    std::vector<double> acc(nc, 0.0);
    std::vector<MKL_INT> rowcols;
    for (MKL_INT i = 0; i < nr; i++) {
        rowcols.clear();
        for (MKL_INT p = tptr[i]; p < tptr[i + 1]; p++) {
            MKL_INT f = tcol[p];
            double a = tval[p];
            for (MKL_INT k = B->rs[f]; k < B->re[f]; k++) {
                MKL_INT j = B->ci[k];
                if (mark[j] != i) { mark[j] = i; acc[j] = 0.0; rowcols.push_back(j); }
                acc[j] += a * B->v[k];
            }
        }
        std::sort(rowcols.begin(), rowcols.end());
        for (MKL_INT j : rowcols) { cols.push_back(j); vals.push_back(acc[j]); }
        rptr[i + 1] = (MKL_INT)cols.size();
    }
    g2p_shim_csr *m = new g2p_shim_csr;
    m->rows = nr; m->cols = nc; m->owned = true;
    m->rs = (MKL_INT *)malloc(sizeof(MKL_INT) * (nr + 1));
    memcpy(m->rs, rptr.data(), sizeof(MKL_INT) * (nr + 1));
    m->re = m->rs + 1;
    m->ci = (MKL_INT *)malloc(sizeof(MKL_INT) * (cols.size() + 1));
    memcpy(m->ci, cols.data(), sizeof(MKL_INT) * cols.size());
    m->v = (double *)malloc(sizeof(double) * (vals.size() + 1));
    memcpy(m->v, vals.data(), sizeof(double) * vals.size());
    *C = m;
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_d_export_csr(const sparse_matrix_t A, sparse_index_base_t *base,
                                                   MKL_INT *rows, MKL_INT *cols, MKL_INT **rows_start,
                                                   MKL_INT **rows_end, MKL_INT **col_indx, double **values) {
    *base = SPARSE_INDEX_BASE_ZERO;
    *rows = A->rows; *cols = A->cols;
    *rows_start = A->rs; *rows_end = A->re; *col_indx = A->ci; *values = A->v;
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
    if (A && A->owned) { free(A->rs); free(A->ci); free(A->v); }
    delete A;
    return SPARSE_STATUS_SUCCESS;
}

extern "C" sparse_status_t mkl_sparse_d_mm(...) { abort(); }
// Weak: oracle/ref_shims/lapacke_shim.cpp defines the dense routines of the
// full-wave path for the build that compiles it in.
#define G2P_WEAK __attribute__((weak))
extern "C" G2P_WEAK lapack_int LAPACKE_dgeev(...) { abort(); }
extern "C" G2P_WEAK lapack_int LAPACKE_dggev(...) { abort(); }
extern "C" G2P_WEAK lapack_int LAPACKE_dhsein(...) { abort(); }
extern "C" G2P_WEAK lapack_int LAPACKE_dhseqr(...) { abort(); }
extern "C" G2P_WEAK lapack_int LAPACKE_zcgesv(...) { abort(); }
extern "C" G2P_WEAK lapack_int LAPACKE_zgesv(...) { abort(); }
extern "C" G2P_WEAK void pardiso(...) { abort(); }
extern "C" G2P_WEAK void pardisoinit(...) { abort(); }

/* MPI as a single rank (the reference only ever ran with one). */
extern "C" int MPI_Init(int *, char ***) { return 0; }
extern "C" int MPI_Finalize(void) { return 0; }
extern "C" int MPI_Comm_size(int, int *n) { *n = 1; return 0; }
extern "C" int MPI_Comm_rank(int, int *r) { *r = 0; return 0; }
