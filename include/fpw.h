/*
 * fpw.h -- focused plane wave (reference mfb_src/fpw.h:15-44).
 *
 * Member order and types follow the reference's mfb_src/fpw.h:15-44: .obj and .dat files
 * store these structs as raw bytes.  The fields are evaluated on the GPU
 * (gb_beam.cu) by the angular-spectrum sum that the reference integrates:
 * Gauss-Legendre nodes over the polar angle of the plane-wave spectrum,
 * adaptive composite trapezoidal rule over its azimuth.
 */
#if !defined FPW_H
#define FPW_H

#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <complex.h>
#include <string.h>
#include "mfb_const.h"
#include "gauleg.h"
#include "osu_mksa.h"
#include "my_utils.h"

typedef struct fpw_data{
  double ki;              /* wave number in the host medium */
  double E0;              /* power coefficient */
  double complex ex,ey;   /* normalised pupil polarisation, electric */
  double complex hx,hy;   /* and magnetic */
  double cos_t,sin_t;     /* rotation angle theta */
  double cos_p,sin_p;     /* rotation angle phi */
  int nt;                 /* Gauss-Legendre nodes over the polar angle */
  double *wt,*ct,*st;     /* weights (times sin), cos and sin of the nodes */
  double *cp,*sp;         /* cos, sin of the trapezoidal azimuths, in refinement order */
}FpwD;

typedef struct fpw{
  double lambda0;         /* vacuum wavelength */
  double ni;              /* refractive index of the host medium */
  double NA;              /* numerical aperture */
  double power;           /* beam power through the pupil */
  double complex e0x;     /* polarisation coefficients (with phase) */
  double complex e0y;
  double fx,fy,fz;        /* focus position */
  double theta,phi;       /* rotation of the beam axis */
  int    nn;              /* Gauss-Legendre nodes */
  FpwD data;
}Fpw;

void print_data_fpw(Fpw *fpw);
void print_data_fpw_mksa(Fpw *fpw);
void setup_Fpw(Fpw *fpw);
void free_Fpw(Fpw *fpw);
void calc_fpw_EH(double complex *e,double complex *h,double *x,Fpw *fpw);
void calc_fpw_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Fpw *fpw);

#endif
