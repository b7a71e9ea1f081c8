/*
 * ipw.h -- incident plane wave (the only incident beam of the BEM hot path).
 *
 * The two structs keep the member order and types of the reference's
 * mfb_src/ipw.h:11-33, because .obj/.dat files store them as raw bytes
 * (solve_bieq2.c:459-465, mo_setup.c:170-176).
 */
#ifndef IPW_H
#define IPW_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <complex.h>
#include "osu_mksa.h"

typedef struct incident_planewave_data{
  double E0;                 /* amplitude sqrt(2 power / n) */
  double ki;                 /* wave number in the host medium */
  double cos_t,sin_t;        /* direction angles theta */
  double cos_p,sin_p;        /* and phi */
  double complex ex,ey,ez;   /* unit electric field vector */
  double complex hx,hy,hz;   /* unit magnetic field vector */
}IpwD;

typedef struct incident_planewave{
  double lambda0;            /* vacuum wavelength */
  double ni;                 /* refractive index of the host medium */
  double power;              /* power per unit area */
  double complex e0x;        /* polarisation coefficients (with phase) */
  double complex e0y;
  double fx,fy,fz;           /* translation of the phase origin */
  double theta;              /* propagation direction: (sin t cos p, sin t sin p, cos t) */
  double phi;
  IpwD data;                 /* derived by setup_ipw() */
}Ipw;

void print_data_ipw(Ipw *ipw);
void print_data_ipw_mksa(Ipw *ipw);
void setup_ipw(Ipw *ipw);
void calc_ipw_EH(double complex *e,double complex *h,double *x,Ipw *ipw);
void calc_ipw_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Ipw *ipw);

#endif
