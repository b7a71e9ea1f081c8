/*
 * bsb.h -- Bessel beam: one cone of plane waves (reference mfb_src/bsb.h:14-38).
 *
 * Member order and types follow the reference's mfb_src/bsb.h:14-38: .obj and .dat files
 * store these structs as raw bytes.  The fields are evaluated on the GPU
 * (gb_beam.cu) by the angular-spectrum sum that the reference integrates:
 * Gauss-Legendre nodes over the polar angle of the plane-wave spectrum,
 * adaptive composite trapezoidal rule over its azimuth.
 */
#if !defined BSB_H
#define BSB_H

#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <complex.h>
#include <string.h>
#include "mfb_const.h"
#include "gauleg.h"
#include "osu_mksa.h"
#include "my_utils.h"

typedef struct bsb_data{
  double ki;
  double E0;
  double complex ex,ey;
  double complex hx,hy;
  double cos_t,sin_t;
  double cos_p,sin_p;
  double ct,st;           /* cos, sin of the cone (deflection) angle */
  double *cp;
  double *sp;
}BsbD;

typedef struct bsb{
  double lambda0;
  double ni;
  double d_angle;         /* cone (deflection) angle */
  double power;           /* power per unit area */
  double complex e0x;
  double complex e0y;
  double fx,fy,fz;
  double theta,phi;
  BsbD data;
}Bsb;

void print_data_bsb(Bsb *bsb);
void print_data_bsb_mksa(Bsb *bsb);
void setup_Bsb(Bsb *bsb);
void free_Bsb(Bsb *bsb);
void calc_bsb_EH(double complex *e,double complex *h,double *x,Bsb *bsb);
void calc_bsb_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Bsb *bsb);

#endif
