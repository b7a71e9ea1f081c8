/* Test infrastructure: incident field of the beam files in the current
 * directory (ipw.txt, fpw.txt, lgb.txt, bsb.txt, blg.txt, rab.txt, whichever
 * exist) through the beam API of the library it is linked against
 * (init_mfb, read_data_mfb, setup_mfb, calc_mfb_EH_dv; reference
 * mfb_src/multi_fbeam.c).  Reads lines "x y z vx vy vz" from standard input
 * and prints per point E, H, dE/dv, dH/dv as 24 numbers (re, im). */
#include <stdio.h>
#include "multi_fbeam.h"
int main(void)
{
  Bobj bm;
  double x[3],v[3];
  double complex e[3],h[3],de[3],dh[3];
  init_mfb(&bm);
  read_data_mfb(&bm);
  setup_mfb(&bm);
  while(scanf("%lf %lf %lf %lf %lf %lf",x,x+1,x+2,v,v+1,v+2)==6){
    calc_mfb_EH_dv(e,h,de,dh,x,v,&bm);
    double complex *o[4]={e,h,de,dh};
    for(int g=0;g<4;g++) for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(o[g][i]),cimag(o[g][i]));
    printf("\n");
  }
  free_mfb(&bm);
  return 0;
}
