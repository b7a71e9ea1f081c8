// gb_fieldobj.cuh -- the view of one object that the point kernels read.
#pragma once
#include "gb_common.cuh"
#include "gb_internal.h"

struct FieldObj {
  const double* cr;
  const double* cw;
  const double* corner;  // (Ne+1)*12 corner coordinates
  const int* etype;
  const int* sd;
  const int* sid;        // concatenated lists
  int sb_Ne[GB_MAXDOM];
  int sb_off[GB_MAXDOM + 1];
  double kn[2 * GB_MAXDOM];
  int MN;
  // boundary values per domain (device), reference layout [s][node][comp]
  const cplx* U[GB_MAXDOM];
  const cplx* dU[GB_MAXDOM];
  const cplx* E[GB_MAXDOM];
  const cplx* dE[GB_MAXDOM];
  const cplx* H[GB_MAXDOM];
  const cplx* dH[GB_MAXDOM];
  double lambda0;
  int prec;  // 2: regular GLN pairs in double-float (gb_quad_df.cuh); 3: the same with the
             // distance-adaptive order of reg_order; else FP64
  int ntri, nquad;  // elements of each type
};

