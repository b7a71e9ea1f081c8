/*
 * rab.h -- focused beam with radial/azimuthal pupil polarisation (reference mfb_src/rab.h:14-44).
 *
 * Member order and types follow the reference's mfb_src/rab.h:14-44: .obj and .dat files
 * store these structs as raw bytes.  The fields are evaluated on the GPU
 * (gb_beam.cu) by the angular-spectrum sum that the reference integrates:
 * Gauss-Legendre nodes over the polar angle of the plane-wave spectrum,
 * adaptive composite trapezoidal rule over its azimuth.
 */
#if !defined RAB_H
#define RAB_H

#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <complex.h>
#include <string.h>
#include "mfb_const.h"
#include "gauleg.h"
#include "osu_mksa.h"
#include "my_utils.h"

typedef struct rab_data{
  double ki;
  double E0;
  double complex er,ea;   /* normalised radial and azimuthal polarisation, electric */
  double complex hr,ha;   /* and magnetic */
  double cos_t,sin_t;
  double cos_p,sin_p;
  int nt;
  double *wt;
  double *ct;
  double *st;
  double *cp;
  double *sp;
}RAbD;

typedef struct rab{
  double lambda0;
  double ni;
  double NA;
  double power;
  double complex e0r;     /* radial polarisation coefficient (with phase) */
  double complex e0a;     /* azimuthal polarisation coefficient */
  double fx,fy,fz;
  double theta,phi;
  int    nn;
  RAbD data;
}RAb;

void print_data_rab(RAb *rab);
void print_data_rab_mksa(RAb *rab);
void setup_rab(RAb *rab);
void free_rab(RAb *rab);
void calc_rab_EH(double complex *e,double complex *h,double *x,RAb *rab);
void calc_rab_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,RAb *rab);

#endif
