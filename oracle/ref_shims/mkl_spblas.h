/* Sparse-BLAS subset of the MKL inspector-executor API, declared for the
 * reference-compiled oracle.  Semantics follow MKL's documentation for the
 * calls made at generateStiff.cpp:920-931 and matrixCon.cpp:109-113,384-554.
 * Test infrastructure only. */
#ifndef G2P_ORACLE_MKL_SPBLAS_SHIM_H
#define G2P_ORACLE_MKL_SPBLAS_SHIM_H

typedef enum { SPARSE_STATUS_SUCCESS = 0, SPARSE_STATUS_NOT_INITIALIZED = 1,
               SPARSE_STATUS_ALLOC_FAILED = 2, SPARSE_STATUS_INVALID_VALUE = 3,
               SPARSE_STATUS_EXECUTION_FAILED = 4, SPARSE_STATUS_INTERNAL_ERROR = 5,
               SPARSE_STATUS_NOT_SUPPORTED = 6 } sparse_status_t;
typedef enum { SPARSE_OPERATION_NON_TRANSPOSE = 10, SPARSE_OPERATION_TRANSPOSE = 11,
               SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12 } sparse_operation_t;
typedef enum { SPARSE_MATRIX_TYPE_GENERAL = 20, SPARSE_MATRIX_TYPE_SYMMETRIC = 21 } sparse_matrix_type_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;
typedef enum { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41, SPARSE_FILL_MODE_FULL = 42 } sparse_fill_mode_t;
typedef enum { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 } sparse_diag_type_t;
typedef enum { SPARSE_LAYOUT_ROW_MAJOR = 101, SPARSE_LAYOUT_COLUMN_MAJOR = 102 } sparse_layout_t;

struct matrix_descr {
    sparse_matrix_type_t type;
    sparse_fill_mode_t mode;
    sparse_diag_type_t diag;
};

struct g2p_shim_csr;
typedef struct g2p_shim_csr *sparse_matrix_t;

extern "C" {
sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, sparse_index_base_t base,
                                        MKL_INT rows, MKL_INT cols, MKL_INT *rows_start,
                                        MKL_INT *rows_end, MKL_INT *col_indx, double *values);
sparse_status_t mkl_sparse_d_mv(sparse_operation_t op, double alpha, const sparse_matrix_t A,
                                struct matrix_descr descr, const double *x, double beta, double *y);
sparse_status_t mkl_sparse_spmm(sparse_operation_t op, const sparse_matrix_t A,
                                const sparse_matrix_t B, sparse_matrix_t *C);
sparse_status_t mkl_sparse_d_export_csr(const sparse_matrix_t A, sparse_index_base_t *base,
                                        MKL_INT *rows, MKL_INT *cols, MKL_INT **rows_start,
                                        MKL_INT **rows_end, MKL_INT **col_indx, double **values);
sparse_status_t mkl_sparse_destroy(sparse_matrix_t A);
sparse_status_t mkl_sparse_d_mm(...);
}

#endif
