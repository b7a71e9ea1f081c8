/*
 * multi_fbeam.h -- incident-field container of the reference
 * (mfb_src/multi_fbeam.h): plane waves and the five angular-spectrum beam
 * families, read from ipw.txt, fpw.txt, lgb.txt, bsb.txt, blg.txt and
 * rab.txt and summed in that order.  Bobj keeps the reference's exact layout
 * (it is stored as raw bytes in .obj/.dat files).
 */
#if !defined MULTI_FBEAM_H
#define MULTI_FBEAM_H

#include "ipw.h"
#include "fpw.h"
#include "lgb.h"
#include "bsb.h"
#include "bslgb.h"
#include "rab.h"

#define fn_ipw "ipw.txt"
#define fn_fpw "fpw.txt"
#define fn_lgb "lgb.txt"
#define fn_bsb "bsb.txt"
#define fn_blg "blg.txt"
#define fn_rab "rab.txt"

typedef struct beam_data{
  Ipw *ipw;
  Fpw *fpw;
  LGb *lgb;
  Bsb *bsb;
  BsLGb *blg;
  RAb *rab;
}Bdata;

typedef struct beam_object{
  int n_ipw;  char fname_ipw[28];
  int n_fpw;  char fname_fpw[28];
  int n_lgb;  char fname_lgb[28];
  int n_bsb;  char fname_bsb[28];
  int n_blg;  char fname_blg[28];
  int n_rab;  char fname_rab[28];
  double n_0;       /* host refractive index */
  double lambda_0;  /* vacuum wavelength */
  double omega;     /* angular frequency 2 pi / lambda_0 */
  Bdata bd;
}Bobj;

void init_mfb(Bobj *obj);
void read_data_mfb(Bobj *obj);
void print_data_mfb(Bobj *obj);
void print_data_mfb_mksa(Bobj *obj);
void setup_mfb(Bobj *obj);
void free_mfb(Bobj *obj);
void calc_mfb_EH(double complex *e,double complex *h,double *x,Bobj *obj);
void calc_mfb_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Bobj *obj);
int read_data_mfb_ipw(char *fname,Bobj *obj);
int read_data_mfb_fpw(char *fname,Bobj *obj);
int read_data_mfb_lgb(char *fname,Bobj *obj);
int read_data_mfb_bsb(char *fname,Bobj *obj);
int read_data_mfb_blg(char *fname,Bobj *obj);
int read_data_mfb_rab(char *fname,Bobj *obj);

/* Batched forms of calc_mfb_EH / calc_mfb_EH_dv: n points x[n][3] (and
 * directions v[n][3]) at once, outputs [n][3].  The angular-spectrum beams
 * are evaluated on the GPU in one launch set per call. */
void calc_mfb_EH_points(Bobj *obj,int n,const double *x,double complex *e,double complex *h);
void calc_mfb_EH_dv_points(Bobj *obj,int n,const double *x,const double *v,double complex *e,double complex *h,
                           double complex *dedv,double complex *dhdv);
/* the beam part of .obj/.dat files: raw Bobj, then the six beam arrays */
void gb_mfb_write(FILE *fp,Bobj *obj);
void gb_mfb_read(FILE *fp,Bobj *obj);

#endif
