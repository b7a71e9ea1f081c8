/*
 * util.c -- 3-vector helpers, checked allocation, Gauss-Legendre rule and the
 * unit conversion used for printing.  Same names and behaviour as the
 * reference's com_src/my_utils.c, com_src/gauleg.c and com_src/osu_mksa.c,
 * which callers of the reference API link against.
 */
#include "bem3_emf_b2.h"
#include "osu_mksa.h"

void vadd_d(double *r,double *v0,double *v1){ for(int i=0;i<3;i++) r[i]=v0[i]+v1[i]; }
void vsub_d(double *r,double *v0,double *v1){ for(int i=0;i<3;i++) r[i]=v0[i]-v1[i]; }
double vabs_d(double *v){ return sqrt(v[0]*v[0]+v[1]*v[1]+v[2]*v[2]); }
double vdot_d(double *a,double *b){ return a[0]*b[0]+a[1]*b[1]+a[2]*b[2]; }
double vabs_2dm(double *a,double *b)
{
  double d0=a[0]-b[0],d1=a[1]-b[1],d2=a[2]-b[2];
  return sqrt(d0*d0+d1*d1+d2*d2);
}
int vuni_d(double *r)
{
  double a=vabs_d(r);
  if(a==0.0) return -1;
  r[0]/=a; r[1]/=a; r[2]/=a;
  return 0;
}
void vcrs_d(double *r,double *a,double *b)
{
  r[0]=a[1]*b[2]-a[2]*b[1];
  r[1]=a[2]*b[0]-a[0]*b[2];
  r[2]=a[0]*b[1]-a[1]*b[0];
}
void prt_z_en(double complex z){ printf("% 15.14e %+15.14eI\n",creal(z),cimag(z)); }
void prt_z_fen(char *txt,int n,double complex z)
{
  if(n>=0) printf("%s[%3d] = % 15.14e %+15.14eI\n",txt,n,creal(z),cimag(z));
  else printf("%s = % 15.14e %+15.14eI\n",txt,creal(z),cimag(z));
}
/* zero-filled allocation; a failure ends the program like the reference */
void *m_alloc2(size_t num,size_t size,char *txt)
{
  void *p=calloc(num,size);
  if(p==NULL){
    printf("memory allocation error!\n%s. Exit..\n",txt);
    exit(1);
  }
  return p;
}
void continue_message(void)
{
  printf("continue? (y/n) : ");
  if(getchar()!='y'){ printf("Exit\n"); exit(0); }
}

/* Gauss-Legendre nodes x[] and weights w[] on [x1,x2]: Newton iteration on
 * P_n from the Chebyshev-like initial guess cos(pi (i-1/4)/(n+1/2)),
 * tolerance 3e-16 -- the textbook method the reference uses (gauleg.c:3-36),
 * so the tables agree to the last bit. */
void gauleg(double x1,double x2,double x[],double w[],int n)
{
  int m=(n+1)/2;
  double xm=0.5*(x2+x1), xl=0.5*(x2-x1);
  for(int i=1;i<=m;i++){
    double z=cos(M_PI*((double)i-0.25)/((double)n+0.5)),z1,pp,p1,p2,p3;
    for(;;){
      p1=1.0; p2=0.0;
      for(int j=1;j<=n;j++){
        p3=p2; p2=p1;
        p1=((double)(2*j-1)*z*p2-(double)(j-1)*p3)/(double)j;
      }
      pp=(double)n*(z*p1-p2)/(z*z-1.0);
      z1=z;
      z=z1-p1/pp;
      if(fabs(z-z1)<=3.0e-16) break;
    }
    x[i-1]=xm-xl*z;
    x[n-i]=xm+xl*z;
    w[i-1]=2.0*xl/((1.0-z*z)*pp*pp);
    w[n-i]=w[i-1];
  }
  if(x1==-x2 && n%2==1) x[n/2]=0.0;
}

/* normalised units (c0 = mu0 = 1) to MKSA: unit length 1 um, unit power
 * 1 mW (the reference's osu_mksa.h convention); printing only */
#define GB_UL 1.0e-6
#define GB_UP 1.0e-3
#define GB_C0 299792458.0
double OSUtoMKSA_length(double l){ return l*GB_UL; }
double OSUtoMKSA_Power_per_unit_area(double p){ return p*GB_UP/(GB_UL*GB_UL); }
double OSUtoMKSA_Force(double f){ return f*GB_UP/GB_C0; }
double OSUtoMKSA_Torque(double n){ return n*GB_UL*GB_UP/GB_C0; }
double OSUtoMKSA_Power(double p){ return p*GB_UP; }
double OSUtoMKSA_power(double p){ return p*GB_UP; }
