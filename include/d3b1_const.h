/*
 * d3b1_const.h -- compile-time constants of the BEM hot path.
 *
 * Same macro names and values as the reference's d3b2_src/d3b1_const.h:27-88
 * (quadrature orders, switching thresholds, Gmsh element codes, Gauss point
 * tables).  They must be identical because they fix the numerical method; the
 * MKL includes of the reference (d3b1_const.h:20-23) are gone: the dense
 * linear algebra runs in this library's own CUDA kernels.
 */
#ifndef D3B1_CONST_H_
#define D3B1_CONST_H_

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <complex.h>
#include <time.h>
#include "multi_fbeam.h"

/* tolerances */
#define MEPS   1.0e-15 /* machine epsilon */
#define GEPS   1.0e-15 /* geometric tolerance (planarity tests) */
#define IEPS   1.0e-12 /* tolerance of the DE rule (not on the default path) */
#define DEPS   0.1     /* radius of the principal-value disc D_eps */
#define CDFH   1.0e-3  /* finite-difference step of the DV variant */

/* numeric constants */
#define I_TH    3.333333333333333333333e-1 /* 1/3 */
#define I_FP    7.957747154594766788444e-2 /* 1/(4 pi) */
#define I_EP    3.978873577297383394222e-2 /* 1/(8 pi) */
#define SQ3     1.732050807568877293528e+0 /* sqrt(3) */
#define I_SPSQ3 3.062938307898844719507e-2 /* 1/(6 pi sqrt(3)) */

/* Gmsh 2.2 ASCII conventions */
#define MSHVER  2.2
#define MSHASCI 0
#define MSHPREC 8
#define ELT3    2   /* 3-node triangle: linear triangular element */
#define ELT4    3   /* 4-node quadrangle: bilinear element */
#define OPENDID 99  /* physical tag of the open (host) region */

/* 4- and 9-point rules on the bilinear element */
#define P44_N  0.5773502691896257645091
#define P44_W  1.0
#define P49_N  0.7745966692414833770359
#define P49_W0 0.3086419753086419753086
#define P49_W1 0.4938271604938271604938
#define P49_W2 0.7901234567901234567901
/* 4- and 7-point rules on the linear triangle */
#define P34_N0 0.2
#define P34_N1 0.3464101615137754587055
#define P34_W0 0.5208333333333333333333
#define P34_W1 0.5625
#define P37_N0 0.3480702390148154917985
#define P37_N1 0.2052130961576726346557
#define P37_N2 0.6028753385763033130539
#define P37_N3 0.3554395089236065568357
#define P37_W0 0.1259391805448271525957
#define P37_W1 0.1323941527885061807376
#define P37_W2 0.225

/* Gauss-Legendre orders: regular rule and the near-singular fallback rule */
#define GLN 12
#define GHN 64

/* switches of the reference kept at their default (0) values */
#define SW_BDR_BIEQ 0
#define SW_BDT_BIEQ 0
#define CBD_CDF   100.0 /* far-field cutoff on |dF/dv| (EH_mEMP_s) */
#define CBD_SDF     0.5 /* |Re dF/dv| above which the GHN rule replaces GLN */
#define SW_DBIEQ      0
#define SW_DBDR_BDE   0
#define SW_DBDR_DE    0
#define SW_DBDT_BDE   0
#define SW_DBDT_DE    0

#endif
