/* Test-infrastructure shim: maps the three LAPACKE calls made by the reference
 * (zgetrf/zgetri in solve_bieq2.c, zgesv in mo_solve.c) onto the ILP64
 * symbols exported by numpy's bundled OpenBLAS (scipy_LAPACKE_*64_). */
#ifndef ORACLE_SHIM_MKL_LAPACKE_H
#define ORACLE_SHIM_MKL_LAPACKE_H
#include "mkl_types.h"
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
MKL_INT scipy_LAPACKE_zgetrf64_(int layout, MKL_INT m, MKL_INT n, MKL_Complex16 *a, MKL_INT lda, MKL_INT *ipiv);
MKL_INT scipy_LAPACKE_zgetri64_(int layout, MKL_INT n, MKL_Complex16 *a, MKL_INT lda, const MKL_INT *ipiv);
MKL_INT scipy_LAPACKE_zgesv64_(int layout, MKL_INT n, MKL_INT nrhs, MKL_Complex16 *a, MKL_INT lda, MKL_INT *ipiv, MKL_Complex16 *b, MKL_INT ldb);
#define LAPACKE_zgetrf scipy_LAPACKE_zgetrf64_
#define LAPACKE_zgetri scipy_LAPACKE_zgetri64_
#define LAPACKE_zgesv  scipy_LAPACKE_zgesv64_
#endif
