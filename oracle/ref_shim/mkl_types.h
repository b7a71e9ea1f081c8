/* Test-infrastructure shim: lets the reference C sources compile against the
 * ILP64 OpenBLAS that numpy bundles instead of Intel MKL (the reference's
 * d3b1_const.h includes these four MKL headers).  Only the two MKL types the
 * reference uses are provided. */
#ifndef ORACLE_SHIM_MKL_TYPES_H
#define ORACLE_SHIM_MKL_TYPES_H
typedef long long MKL_INT;
typedef struct { double real, imag; } MKL_Complex16;
#endif
