/*
 * multi_fbeam.h -- incident-field container of the reference (mfb_src/multi_fbeam.h).
 *
 * The BEM hot path supports the plane-wave member (ipw).  The other five beam
 * families of the reference (focused, Laguerre-Gaussian, Bessel, Bessel-LG,
 * radial/azimuthal) are outside this library's scope; their struct types are
 * left incomplete so that Bobj keeps the reference's exact layout (it is
 * stored as raw bytes in .obj/.dat files), and a file that defines such a
 * beam is rejected with a message.
 */
#if !defined MULTI_FBEAM_H
#define MULTI_FBEAM_H

#include "ipw.h"

#define fn_ipw "ipw.txt"
#define fn_fpw "fpw.txt"
#define fn_lgb "lgb.txt"
#define fn_bsb "bsb.txt"
#define fn_blg "blg.txt"
#define fn_rab "rab.txt"

typedef struct focused_planewave Fpw;
typedef struct lg_beam LGb;
typedef struct bessel_beam Bsb;
typedef struct bessel_lg_beam BsLGb;
typedef struct ra_beam RAb;

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

#endif
