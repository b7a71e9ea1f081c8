/* bem3_analysis: fields, radiation force/torque and absorbed power of a
 * solved scene, printed with full precision.
 * Usage: bem3_analysis result.dat x y z */
#include "bem3_emf_b2.h"

int main(int argc,char **argv)
{
  MOBJ mo;
  double complex E[3],H[3];
  double r[3]={0.3,0.0,1.1},rc[3]={0.0,0.0,0.0},F[3],N[3],P;
  if(argc!=2 && argc!=5){ printf("Usage : %s datafile_name [x y z]\n",argv[0]); return 0; }
  if(argc==5){ r[0]=atof(argv[2]); r[1]=atof(argv[3]); r[2]=atof(argv[4]); }
  mo_dat_read(argv[1],&mo);
  for(int type=0;type<=2;type++){
    int oid=mo_EH_t(E,H,r,type,&mo);
    printf("EH_t type %d oid %d",type,oid);
    for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(E[i]),cimag(E[i]));
    for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(H[i]),cimag(H[i]));
    printf("\n");
  }
  for(int type=0;type<=2;type++){
    int oid=mo_EH_mEMP_t(E,H,r,type,&mo);
    printf("EH_mEMP_t type %d oid %d",type,oid);
    for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(E[i]),cimag(E[i]));
    for(int i=0;i<3;i++) printf(" %.17e %.17e",creal(H[i]),cimag(H[i]));
    printf("\n");
  }
  for(int m=0;m<mo.N;m++){
    for(int type=0;type<=1;type++){
      int ret=mo_force_FN(F,N,rc,m,type,&mo);
      printf("force obj %d type %d ret %d %.17e %.17e %.17e %.17e %.17e %.17e\n",m,type,ret,F[0],F[1],F[2],N[0],N[1],N[2]);
      ret=mo_absorb_P(&P,m,type,&mo);
      printf("absorb obj %d type %d ret %d %.17e\n",m,type,ret,P);
    }
  }
  mo_finalize(&mo);
  return 0;
}
