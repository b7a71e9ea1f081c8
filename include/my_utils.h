/*
 * my_utils.h -- small 3-vector and allocation helpers with the reference's
 * names (com_src/my_utils.h), so that callers of the reference compile
 * unchanged.
 */
#ifndef MY_UTILS_H_
#define MY_UTILS_H_
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <complex.h>
void vadd_d(double *r,double *v0,double *v1);
void vsub_d(double *r,double *v0,double *v1);
int vuni_d(double *r);
double vabs_d(double *v);
double vabs_2dm(double *v0,double *v1);
double vdot_d(double *v0,double *v1);
void vcrs_d(double *r,double *v0,double *v1);
void prt_z_en(double complex z);
void prt_z_fen(char *txt,int n,double complex z);
void *m_alloc2(size_t num,size_t size, char *txt);
void continue_message(void);
#endif
