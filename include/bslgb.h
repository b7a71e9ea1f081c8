/*
 * bslgb.h -- Bessel beam with a spiral phase (reference mfb_src/bslgb.h:14-39).
 *
 * Member order and types follow the reference's mfb_src/bslgb.h:14-39: .obj and .dat files
 * store these structs as raw bytes.  The fields are evaluated on the GPU
 * (gb_beam.cu) by the angular-spectrum sum that the reference integrates:
 * Gauss-Legendre nodes over the polar angle of the plane-wave spectrum,
 * adaptive composite trapezoidal rule over its azimuth.
 */
#if !defined BSLGB_H
#define BSLGB_H

#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <complex.h>
#include <string.h>
#include "mfb_const.h"
#include "gauleg.h"
#include "osu_mksa.h"
#include "my_utils.h"

typedef struct bslgb_data{
  double ki;
  double E0;
  double complex ex,ey;
  double complex hx,hy;
  double cos_t,sin_t;
  double cos_p,sin_p;
  double ct,st;
  double *cp,*sp;
  double complex *ph_p;
}BsLGbD;

typedef struct bslgb{
  double lambda0;
  double ni;
  double d_angle;
  double power;
  double complex e0x;
  double complex e0y;
  double fx,fy,fz;
  double theta,phi;
  int    lg_m;
  BsLGbD data;
}BsLGb;

void print_data_bslgb(BsLGb *bsb);
void print_data_bslgb_mksa(BsLGb *bsb);
void setup_BsLGb(BsLGb *bsb);
void free_BsLGb(BsLGb *bsb);
void calc_bslgb_EH(double complex *e,double complex *h,double *x,BsLGb *bsb);
void calc_bslgb_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,BsLGb *bsb);

#endif
