/* Declaration shim standing in for Intel MKL when the reference's own sources
 * are compiled as a CPU oracle.  Only the names the hot-path files use are
 * declared.  The sparse subset is implemented in mkl_sparse_shim.cpp; the
 * dense LAPACKE and PARDISO routines sit on code paths the reference compiles
 * out (SKIP_VH, SKIP_PARDISO) and are declared variadic so the in-class
 * member functions that mention them still parse.  Test infrastructure only. */
#ifndef G2P_ORACLE_MKL_SHIM_H
#define G2P_ORACLE_MKL_SHIM_H

typedef long long MKL_INT;          /* MKL_ILP64 is defined by fdtd.hpp */
typedef long long lapack_int;
typedef lapack_int lapack_logical;
typedef struct _MKL_Complex16 { double real; double imag; } MKL_Complex16;
#define lapack_complex_double MKL_Complex16
typedef struct _MKL_Complex8 { float real; float imag; } MKL_Complex8;
#define lapack_complex_float MKL_Complex8

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

extern "C" {
lapack_int LAPACKE_dgeev(...);
lapack_int LAPACKE_dggev(...);
lapack_int LAPACKE_dhsein(...);
lapack_int LAPACKE_dhseqr(...);
lapack_int LAPACKE_zcgesv(...);
lapack_int LAPACKE_zgesv(...);
void pardiso(...);
void pardisoinit(...);
}

#include "mkl_spblas.h"

#endif
