/*
 * lgb.h -- Laguerre-Gaussian (spiral-phase) focused beam (reference mfb_src/lgb.h:14-46).
 *
 * Member order and types follow the reference's mfb_src/lgb.h:14-46: .obj and .dat files
 * store these structs as raw bytes.  The fields are evaluated on the GPU
 * (gb_beam.cu) by the angular-spectrum sum that the reference integrates:
 * Gauss-Legendre nodes over the polar angle of the plane-wave spectrum,
 * adaptive composite trapezoidal rule over its azimuth.
 */
#if !defined LGB_H
#define LGB_H

#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <complex.h>
#include <string.h>
#include "mfb_const.h"
#include "gauleg.h"
#include "osu_mksa.h"
#include "my_utils.h"

typedef struct lgb_data{
  double ki;
  double E0;
  double complex ex,ey;
  double complex hx,hy;
  double cos_t,sin_t;
  double cos_p,sin_p;
  int nt;                 /* Gauss-Legendre nodes over the polar angle */
  double *wt,*ct,*st;     /* weights (times sin), cos and sin of the nodes */
  double *cp,*sp;         /* cos, sin of the trapezoidal azimuths, in refinement order */
  double complex *ph_p;   /* exp(i m phi) at the trapezoidal azimuths */
}LGbD;

typedef struct lgb{
  double lambda0;
  double ni;
  double NA;
  double power;
  double complex e0x;
  double complex e0y;
  double fx,fy,fz;
  double theta,phi;
  int    lg_m;            /* topological charge m of the spiral phase */
  int    nn;
  LGbD data;
}LGb;

void print_data_lgb(LGb *lgb);
void print_data_lgb_mksa(LGb *lgb);
void setup_LGb(LGb *lgb);
void free_LGb(LGb *lgb);
void calc_lgb_EH(double complex *e,double complex *h,double *x,LGb *lgb);
void calc_lgb_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,LGb *lgb);

#endif
