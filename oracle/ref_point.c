/* Test infrastructure: prints the total field of a solved scene at one point
 * (mo_EH_t, quadrature types 0 and 1) through the API of whichever library
 * it is linked against; used to pin oracle/_ref to the reference's shipped
 * example1.log.  Usage: ref_point result.dat x y z */
#include "bem3_emf_b2.h"
int main(int argc,char **argv)
{
  MOBJ mo;
  double complex E[3],H[3];
  double r[3];
  if(argc!=5) return 1;
  r[0]=atof(argv[2]); r[1]=atof(argv[3]); r[2]=atof(argv[4]);
  mo_dat_read(argv[1],&mo);
  for(int type=0;type<=1;type++){
    mo_EH_t(E,H,r,type,&mo);
    printf("type %d",type);
    for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(E[i]),cimag(E[i]));
    for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(H[i]),cimag(H[i]));
    printf("\n");
  }
  mo_finalize(&mo);
  return 0;
}
