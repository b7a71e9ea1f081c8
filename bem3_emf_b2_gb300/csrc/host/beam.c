/*
 * beam.c -- incident fields of the BEM path (reference mfb_src/): plane waves
 * (ipw.c) and the five angular-spectrum families -- focused plane wave (fpw),
 * Laguerre-Gaussian (lgb), Bessel (bsb), Bessel with spiral phase (blg) and
 * radially/azimuthally polarised (rab) -- read from the reference's data
 * files, summed in the reference's order (multi_fbeam.c:764-876).
 *
 * Plane waves cost one phase per point and are summed here.  The
 * angular-spectrum beams are evaluated on the GPU (gb_beam.cu): per point,
 * Gauss-Legendre nodes over the polar angle times an adaptive trapezoidal
 * rule over the azimuth, up to 8,192 plane waves per node.  The batched
 * entry points (calc_mfb_EH_points, calc_mfb_EH_dv_points) take all points
 * of a call at once; the reference's single-point functions call them with
 * one point.
 */
#include "bem3_emf_b2.h"
#include "../gb_beam.h"
#include <pthread.h>

int gbi_beam_points(int nb,const GbBeamDesc *beams,int T,const int *item_beam,const double *nodes,const double *phi,
                    int nphase,const double *phase,int n,const double *x,const double *v,double *E,double *H,
                    double *dE,double *dH);
const char *gb_last_error(void);

/* ------------------------------------------------------------ containers */

void init_mfb(Bobj *obj)
{
  memset(obj,0,sizeof(Bobj));
  snprintf(obj->fname_ipw,28,"null"); snprintf(obj->fname_fpw,28,"null");
  snprintf(obj->fname_lgb,28,"null"); snprintf(obj->fname_bsb,28,"null");
  snprintf(obj->fname_blg,28,"null"); snprintf(obj->fname_rab,28,"null");
}

void read_data_mfb(Bobj *obj)
{
  int wn=0;
  wn+=read_data_mfb_ipw(fn_ipw,obj);
  wn+=read_data_mfb_fpw(fn_fpw,obj);
  wn+=read_data_mfb_lgb(fn_lgb,obj);
  wn+=read_data_mfb_bsb(fn_bsb,obj);
  wn+=read_data_mfb_blg(fn_blg,obj);
  wn+=read_data_mfb_rab(fn_rab,obj);
  if(wn==0){
    printf("read_data_mfb() No beam defined, check beam data file : %s, %s, %s, %s, %s, %s.\n",fn_ipw,fn_fpw,fn_lgb,
           fn_bsb,fn_blg,fn_rab);
    exit(1);
  }
}

/* ------------------------------------------------------------ file input */

static void gb_fail_read(const char *fn,const char *what)
{
  printf("beam.c, read_data_mfb_%s(), failed to read the %s. exit...\n",fn,what);
  exit(1);
}

/* Header of every beam file: two comment lines, the number of beams, one
 * comment line.  Returns the count (0 and no file: 0); fname is recorded. */
static FILE *gb_open_beam_file(const char *fname,const char *tag,char *dst,int *nn)
{
  FILE *fp=fopen(fname,"rt");
  char buf[256];
  *nn=0;
  if(fp==NULL) return NULL;
  if(fgets(buf,256,fp)==NULL || fgets(buf,256,fp)==NULL) gb_fail_read(tag,"line");
  snprintf(dst,28,"%s",fname);
  if(fscanf(fp,"%d\n",nn)!=1) gb_fail_read(tag,"nn");
  if(fgets(buf,256,fp)==NULL) gb_fail_read(tag,"line");
  if(*nn<=0){ fclose(fp); *nn=0; return NULL; }
  return fp;
}

static void gb_read_values(FILE *fp,const char *tag,double *v,int n)
{
  for(int j=0;j<n;j++) if(fscanf(fp,"%lf",&v[j])!=1) gb_fail_read(tag,"beam parameters");
}

static int gb_read_int(FILE *fp,const char *tag)
{
  int k;
  if(fscanf(fp,"%d",&k)!=1) gb_fail_read(tag,"integer parameter");
  return k;
}

/* ipw.txt, per wave: lambda0 ni power Re(e0x) Im(e0x) Re(e0y) Im(e0y) fx fy fz theta phi */
int read_data_mfb_ipw(char *fname,Bobj *obj)
{
  int nn;
  FILE *fp=gb_open_beam_file(fname,"ipw",obj->fname_ipw,&nn);
  if(fp==NULL) return 0;
  free(obj->bd.ipw);
  obj->n_ipw=nn;
  obj->bd.ipw=(Ipw *)m_alloc2(nn,sizeof(Ipw),"beam.c, read_data_mfb_ipw(), ipw");
  for(int i=0;i<nn;i++){
    double v[12];
    gb_read_values(fp,"ipw",v,12);
    Ipw *p=&obj->bd.ipw[i];
    p->lambda0=v[0]; p->ni=v[1]; p->power=v[2];
    p->e0x=v[3]+I*v[4]; p->e0y=v[5]+I*v[6];
    p->fx=v[7]; p->fy=v[8]; p->fz=v[9]; p->theta=v[10]; p->phi=v[11];
  }
  fclose(fp);
  return nn;
}

/* fpw.txt: lambda0 ni NA power Re(e0x) Im(e0x) Re(e0y) Im(e0y) fx fy fz theta phi nn */
int read_data_mfb_fpw(char *fname,Bobj *obj)
{
  int nn;
  FILE *fp=gb_open_beam_file(fname,"fpw",obj->fname_fpw,&nn);
  if(fp==NULL) return 0;
  free(obj->bd.fpw);
  obj->n_fpw=nn;
  obj->bd.fpw=(Fpw *)m_alloc2(nn,sizeof(Fpw),"beam.c, read_data_mfb_fpw(), fpw");
  for(int i=0;i<nn;i++){
    double v[13];
    gb_read_values(fp,"fpw",v,13);
    Fpw *p=&obj->bd.fpw[i];
    p->lambda0=v[0]; p->ni=v[1]; p->NA=v[2]; p->power=v[3];
    p->e0x=v[4]+I*v[5]; p->e0y=v[6]+I*v[7];
    p->fx=v[8]; p->fy=v[9]; p->fz=v[10]; p->theta=v[11]; p->phi=v[12];
    p->nn=gb_read_int(fp,"fpw");
  }
  fclose(fp);
  return nn;
}

/* lgb.txt: as fpw.txt with lg_m before nn */
int read_data_mfb_lgb(char *fname,Bobj *obj)
{
  int nn;
  FILE *fp=gb_open_beam_file(fname,"lgb",obj->fname_lgb,&nn);
  if(fp==NULL) return 0;
  free(obj->bd.lgb);
  obj->n_lgb=nn;
  obj->bd.lgb=(LGb *)m_alloc2(nn,sizeof(LGb),"beam.c, read_data_mfb_lgb(), lgb");
  for(int i=0;i<nn;i++){
    double v[13];
    gb_read_values(fp,"lgb",v,13);
    LGb *p=&obj->bd.lgb[i];
    p->lambda0=v[0]; p->ni=v[1]; p->NA=v[2]; p->power=v[3];
    p->e0x=v[4]+I*v[5]; p->e0y=v[6]+I*v[7];
    p->fx=v[8]; p->fy=v[9]; p->fz=v[10]; p->theta=v[11]; p->phi=v[12];
    p->lg_m=gb_read_int(fp,"lgb");
    p->nn=gb_read_int(fp,"lgb");
  }
  fclose(fp);
  return nn;
}

/* bsb.txt: lambda0 ni d_angle power Re(e0x) Im(e0x) Re(e0y) Im(e0y) fx fy fz theta phi */
int read_data_mfb_bsb(char *fname,Bobj *obj)
{
  int nn;
  FILE *fp=gb_open_beam_file(fname,"bsb",obj->fname_bsb,&nn);
  if(fp==NULL) return 0;
  free(obj->bd.bsb);
  obj->n_bsb=nn;
  obj->bd.bsb=(Bsb *)m_alloc2(nn,sizeof(Bsb),"beam.c, read_data_mfb_bsb(), bsb");
  for(int i=0;i<nn;i++){
    double v[13];
    gb_read_values(fp,"bsb",v,13);
    Bsb *p=&obj->bd.bsb[i];
    p->lambda0=v[0]; p->ni=v[1]; p->d_angle=v[2]; p->power=v[3];
    p->e0x=v[4]+I*v[5]; p->e0y=v[6]+I*v[7];
    p->fx=v[8]; p->fy=v[9]; p->fz=v[10]; p->theta=v[11]; p->phi=v[12];
  }
  fclose(fp);
  return nn;
}

/* blg.txt: as bsb.txt with lg_m at the end */
int read_data_mfb_blg(char *fname,Bobj *obj)
{
  int nn;
  FILE *fp=gb_open_beam_file(fname,"blg",obj->fname_blg,&nn);
  if(fp==NULL) return 0;
  free(obj->bd.blg);
  obj->n_blg=nn;
  obj->bd.blg=(BsLGb *)m_alloc2(nn,sizeof(BsLGb),"beam.c, read_data_mfb_blg(), blg");
  for(int i=0;i<nn;i++){
    double v[13];
    gb_read_values(fp,"blg",v,13);
    BsLGb *p=&obj->bd.blg[i];
    p->lambda0=v[0]; p->ni=v[1]; p->d_angle=v[2]; p->power=v[3];
    p->e0x=v[4]+I*v[5]; p->e0y=v[6]+I*v[7];
    p->fx=v[8]; p->fy=v[9]; p->fz=v[10]; p->theta=v[11]; p->phi=v[12];
    p->lg_m=gb_read_int(fp,"blg");
  }
  fclose(fp);
  return nn;
}

/* rab.txt: lambda0 ni NA power Re(e0r) Im(e0r) Re(e0a) Im(e0a) fx fy fz theta phi nn */
int read_data_mfb_rab(char *fname,Bobj *obj)
{
  int nn;
  FILE *fp=gb_open_beam_file(fname,"rab",obj->fname_rab,&nn);
  if(fp==NULL) return 0;
  free(obj->bd.rab);
  obj->n_rab=nn;
  obj->bd.rab=(RAb *)m_alloc2(nn,sizeof(RAb),"beam.c, read_data_mfb_rab(), rab");
  for(int i=0;i<nn;i++){
    double v[13];
    gb_read_values(fp,"rab",v,13);
    RAb *p=&obj->bd.rab[i];
    p->lambda0=v[0]; p->ni=v[1]; p->NA=v[2]; p->power=v[3];
    p->e0r=v[4]+I*v[5]; p->e0a=v[6]+I*v[7];
    p->fx=v[8]; p->fy=v[9]; p->fz=v[10]; p->theta=v[11]; p->phi=v[12];
    p->nn=gb_read_int(fp,"rab");
  }
  fclose(fp);
  return nn;
}

/* ------------------------------------------------------------ printing */

/* The reference's parameter listing (the log format is kept). */
typedef struct {
  const char *title;
  double lambda0,ni;
  int third;                  /* 0 numerical aperture, 1 deflection angle */
  double third_v;
  int per_area;               /* power per unit area (Bessel beams) */
  double power;
  int radial;                 /* radial/azimuthal polarisation labels */
  double complex p0,p1;
  double fx,fy,fz,theta,phi;
  int lg_m,has_m,nn,has_nn;
} GbBeamPrint;

static void gb_print_beam(const GbBeamPrint *b,int mksa)
{
  if(mksa) printf("-- %s, MKSA system --\n",b->title); else printf("-- %s --\n",b->title);
  if(mksa) printf("wave length of incident beam in vacuum   [m]: %15.14g\n",OSUtoMKSA_length(b->lambda0));
  else     printf("wave length of incident beam in vacuum      : %15.14g\n",b->lambda0);
  printf("refractive index of surrounding             : %15.14g\n",b->ni);
  if(b->third==0) printf("numerical aperture                          : %15.14g\n",b->third_v);
  else            printf("deflection angle                       [rad]: %15.14g\n",b->third_v);
  if(b->per_area){
    if(mksa) printf("incident beam power per unit area    [W/m^2]: %15.14g\n",OSUtoMKSA_Power_per_unit_area(b->power));
    else     printf("incident beam power per unit area           : %15.14g\n",b->power);
  }
  else {
    if(mksa) printf("incident beam power                      [W]: %15.14g\n",OSUtoMKSA_power(b->power));
    else     printf("incident beam power                         : %15.14g\n",b->power);
  }
  if(b->radial){
    printf("radial-component of polarization coefficient:%7.6g+%7.6gi\n",creal(b->p0),cimag(b->p0));
    printf("azimuthal-component of polarization coef    :%7.6g+%7.6gi\n",creal(b->p1),cimag(b->p1));
  }
  else {
    printf("x-component of polarization coefficient     :%7.6g+%7.6gi\n",creal(b->p0),cimag(b->p0));
    printf("y-component of polarization coefficient     :%7.6g+%7.6gi\n",creal(b->p1),cimag(b->p1));
  }
  double f[3]={b->fx,b->fy,b->fz};
  const char *ax="xyz";
  for(int i=0;i<3;i++){
    if(mksa) printf("%c-component of translation vector        [m]: %15.14g\n",ax[i],OSUtoMKSA_length(f[i]));
    else     printf("%c-component of translation vector           : %15.14g\n",ax[i],f[i]);
  }
  printf("rotation parameter theta               [rad]: %15.14g\n",b->theta);
  printf("rotation parameter phi                 [rad]: %15.14g\n",b->phi);
  if(b->has_m)  printf("mode number for spiral phase modulation     : %15d\n",b->lg_m);
  if(b->has_nn) printf("gauss-legendre integration sampling number  : %15d\n",b->nn);
}

#define GB_PRINT_XY(P,TITLE,THIRD,THIRDV,AREA,HASM,M,HASNN,NN) \
  { GbBeamPrint b={TITLE,(P)->lambda0,(P)->ni,THIRD,THIRDV,AREA,(P)->power,0,(P)->e0x,(P)->e0y,(P)->fx,(P)->fy,(P)->fz, \
                   (P)->theta,(P)->phi,M,HASM,NN,HASNN}; gb_print_beam(&b,mksa); }

static void gb_print_fpw(Fpw *p,int mksa){ GB_PRINT_XY(p,"focused plane wave",0,p->NA,0,0,0,1,p->nn) }
static void gb_print_lgb(LGb *p,int mksa)
{ GB_PRINT_XY(p,"focused plane wave with spiral phase modulation",0,p->NA,0,1,p->lg_m,1,p->nn) }
static void gb_print_bsb(Bsb *p,int mksa){ GB_PRINT_XY(p,"Bessel beam",1,p->d_angle,1,0,0,0,0) }
static void gb_print_blg(BsLGb *p,int mksa)
{ GB_PRINT_XY(p,"Bessel beam with spiral phase modulation",1,p->d_angle,1,1,p->lg_m,0,0) }
static void gb_print_rab(RAb *p,int mksa)
{
  GbBeamPrint b={"focused radially and azimuthally polarized beam",p->lambda0,p->ni,0,p->NA,0,p->power,1,p->e0r,p->e0a,
                 p->fx,p->fy,p->fz,p->theta,p->phi,0,0,p->nn,1};
  gb_print_beam(&b,mksa);
}

void print_data_fpw(Fpw *p){ gb_print_fpw(p,0); }
void print_data_fpw_mksa(Fpw *p){ gb_print_fpw(p,1); }
void print_data_lgb(LGb *p){ gb_print_lgb(p,0); }
void print_data_lgb_mksa(LGb *p){ gb_print_lgb(p,1); }
void print_data_bsb(Bsb *p){ gb_print_bsb(p,0); }
void print_data_bsb_mksa(Bsb *p){ gb_print_bsb(p,1); }
void print_data_bslgb(BsLGb *p){ gb_print_blg(p,0); }
void print_data_bslgb_mksa(BsLGb *p){ gb_print_blg(p,1); }
void print_data_rab(RAb *p){ gb_print_rab(p,0); }
void print_data_rab_mksa(RAb *p){ gb_print_rab(p,1); }

void print_data_ipw(Ipw *ipw)
{
  printf("-- plane wave --\n");
  printf("wave length of incident beam in vacuum      : %15.14g\n",ipw->lambda0);
  printf("refractive index of surrounding             : %15.14g\n",ipw->ni);
  printf("incident beam power per unit area           : %15.14g\n",ipw->power);
  printf("x-component of polarization coefficient     :%7.6g+%7.6gi\n",creal(ipw->e0x),cimag(ipw->e0x));
  printf("y-component of polarization coefficient     :%7.6g+%7.6gi\n",creal(ipw->e0y),cimag(ipw->e0y));
  printf("x-component of translation vector           : %15.14g\n",ipw->fx);
  printf("y-component of translation vector           : %15.14g\n",ipw->fy);
  printf("z-component of translation vector           : %15.14g\n",ipw->fz);
  printf("rotation parameter theta               [rad]: %15.14g\n",ipw->theta);
  printf("rotation parameter phi                 [rad]: %15.14g\n",ipw->phi);
}

void print_data_ipw_mksa(Ipw *ipw)
{
  printf("-- plane wave, MKSA system --\n");
  printf("wave length of incident beam in vacuum   [m]: %15.14g\n",OSUtoMKSA_length(ipw->lambda0));
  printf("refractive index of surrounding             : %15.14g\n",ipw->ni);
  printf("incident beam power per unit area    [W/m^2]: %15.14g\n",OSUtoMKSA_Power_per_unit_area(ipw->power));
  printf("x-component of polarization coefficient     :%7.6g+%7.6gi\n",creal(ipw->e0x),cimag(ipw->e0x));
  printf("y-component of polarization coefficient     :%7.6g+%7.6gi\n",creal(ipw->e0y),cimag(ipw->e0y));
  printf("x-component of translation vector        [m]: %15.14g\n",OSUtoMKSA_length(ipw->fx));
  printf("y-component of translation vector        [m]: %15.14g\n",OSUtoMKSA_length(ipw->fy));
  printf("z-component of translation vector        [m]: %15.14g\n",OSUtoMKSA_length(ipw->fz));
  printf("rotation parameter theta               [rad]: %15.14g\n",ipw->theta);
  printf("rotation parameter phi                 [rad]: %15.14g\n",ipw->phi);
}

static void gb_print_mfb(Bobj *obj,int mksa)
{
  for(int i=0;i<obj->n_ipw;i++){
    printf(" \"%s\" No.%02d ",obj->fname_ipw,i);
    if(mksa) print_data_ipw_mksa(&obj->bd.ipw[i]); else print_data_ipw(&obj->bd.ipw[i]);
  }
  for(int i=0;i<obj->n_fpw;i++){ printf(" \"%s\" No.%02d ",obj->fname_fpw,i); gb_print_fpw(&obj->bd.fpw[i],mksa); }
  for(int i=0;i<obj->n_lgb;i++){ printf(" \"%s\" No.%02d ",obj->fname_lgb,i); gb_print_lgb(&obj->bd.lgb[i],mksa); }
  for(int i=0;i<obj->n_bsb;i++){ printf(" \"%s\" No.%02d ",obj->fname_bsb,i); gb_print_bsb(&obj->bd.bsb[i],mksa); }
  for(int i=0;i<obj->n_blg;i++){ printf(" \"%s\" No.%02d ",obj->fname_blg,i); gb_print_blg(&obj->bd.blg[i],mksa); }
  for(int i=0;i<obj->n_rab;i++){ printf(" \"%s\" No.%02d ",obj->fname_rab,i); gb_print_rab(&obj->bd.rab[i],mksa); }
  printf("\n");
}

void print_data_mfb(Bobj *obj){ gb_print_mfb(obj,0); }
void print_data_mfb_mksa(Bobj *obj){ gb_print_mfb(obj,1); }

/* ------------------------------------------------------------ setup */

/* Unit polarisation e = (e0x,e0y,0)/|.|, h = n z x e, rotated so that the
 * wave travels along (sin t cos p, sin t sin p, cos t) (reference ipw.c:65-89). */
void setup_ipw(Ipw *ipw)
{
  double cs=1.0/sqrt(pow(cabs(ipw->e0x),2)+pow(cabs(ipw->e0y),2));
  double complex ex=ipw->e0x*cs, ey=ipw->e0y*cs;
  double complex hx=-ey*ipw->ni, hy=ex*ipw->ni;
  double st=sin(ipw->theta), ct=cos(ipw->theta), sp=sin(ipw->phi), cp=cos(ipw->phi);
  IpwD *d=&ipw->data;
  d->E0=sqrt(ipw->power*2.0/ipw->ni);
  d->ki=2.0*M_PI*ipw->ni/ipw->lambda0;
  d->sin_t=st; d->cos_t=ct; d->sin_p=sp; d->cos_p=cp;
  double a=sp*sp+cp*cp*ct, b=sp*cp*ct-sp*cp, c=sp*sp*ct+cp*cp;
  d->ex=ex*a+ey*b;  d->ey=ex*b+ey*c;  d->ez=-(ex*cp+ey*sp)*st;
  d->hx=hx*a+hy*b;  d->hy=hx*b+hy*c;  d->hz=-(hx*cp+hy*sp)*st;
}

/* Trapezoidal azimuths in refinement order: -pi first, then level l adds the
 * 2^l midpoints -pi + (2s-1) 2 pi / 2^(l+1), s = 1 .. 2^l (the order in which
 * the adaptive rule consumes them). */
static double gb_azimuth(int j)
{
  if(j==0) return -M_PI;
  int l=0;
  while((2<<l)-1<j) l++;           /* level l holds j = 2^l .. 2^(l+1)-1 */
  int s=j-(1<<l)+1;
  double h=2.0*M_PI/(double)(2<<l);
  return -M_PI+(double)(2*s-1)*h;
}

static void gb_azimuth_tables(double **cp,double **sp,const char *who)
{
  *cp=(double *)m_alloc2(GB_BEAM_NPHI,sizeof(double),(char *)who);
  *sp=(double *)m_alloc2(GB_BEAM_NPHI,sizeof(double),(char *)who);
  for(int j=0;j<GB_BEAM_NPHI;j++){
    if(j==0){ (*cp)[0]=-1.0; (*sp)[0]=0.0; continue; }
    double a=gb_azimuth(j);
    (*cp)[j]=cos(a); (*sp)[j]=sin(a);
  }
}

/* exp(i m a) at the azimuths, with m a reduced modulo 2 pi from a in [0, 2 pi)
 * (reference lgb.c:177-187) */
static double complex *gb_spiral_phase(int m,const char *who)
{
  double complex *ph=(double complex *)m_alloc2(GB_BEAM_NPHI,sizeof(double complex),(char *)who);
  for(int j=0;j<GB_BEAM_NPHI;j++){
    if(m==0){ ph[j]=1.0; continue; }
    double a=gb_azimuth(j);
    if(a<0.0) a+=2.0*M_PI;
    double t=fmod((double)m*a,2.0*M_PI);
    ph[j]=cos(t)+I*sin(t);
  }
  return ph;
}

/* Gauss-Legendre nodes in sin t on [0, NA/n]; weights times sin t */
static void gb_polar_nodes(int nt,double kr,double **wt,double **ct,double **st,const char *who)
{
  *wt=(double *)m_alloc2(nt,sizeof(double),(char *)who);
  *ct=(double *)m_alloc2(nt,sizeof(double),(char *)who);
  *st=(double *)m_alloc2(nt,sizeof(double),(char *)who);
  double *xt=(double *)m_alloc2(nt,sizeof(double),(char *)who);
  gauleg(0.0,kr,xt,*wt,nt);
  for(int i=0;i<nt;i++){ (*st)[i]=xt[i]; (*ct)[i]=sqrt(1.0-xt[i]*xt[i]); (*wt)[i]*=xt[i]; }
  free(xt);
}

void setup_Fpw(Fpw *p)
{
  FpwD *d=&p->data;
  double kr=p->NA/p->ni;
  double ce=sqrt(1.0/M_PI)/(kr*sqrt(pow(cabs(p->e0x),2)+pow(cabs(p->e0y),2)));
  d->ki=2.0*M_PI*p->ni/p->lambda0;
  d->ex=p->e0x*ce; d->ey=p->e0y*ce;
  d->hx=-d->ey*p->ni; d->hy=d->ex*p->ni;
  d->E0=sqrt(2.0*p->power*p->ni)/p->lambda0;
  d->cos_t=cos(p->theta); d->sin_t=sin(p->theta); d->cos_p=cos(p->phi); d->sin_p=sin(p->phi);
  d->nt=p->nn;
  gb_polar_nodes(d->nt,kr,&d->wt,&d->ct,&d->st,"beam.c, setup_Fpw()");
  gb_azimuth_tables(&d->cp,&d->sp,"beam.c, setup_Fpw()");
}

void setup_LGb(LGb *p)
{
  LGbD *d=&p->data;
  double kr=p->NA/p->ni;
  double ce=sqrt(1.0/M_PI)/(kr*sqrt(pow(cabs(p->e0x),2)+pow(cabs(p->e0y),2)));
  d->ki=2.0*M_PI*p->ni/p->lambda0;
  d->ex=p->e0x*ce; d->ey=p->e0y*ce;
  d->hx=-d->ey*p->ni; d->hy=d->ex*p->ni;
  d->E0=sqrt(2.0*p->power*p->ni)/p->lambda0;
  d->cos_t=cos(p->theta); d->sin_t=sin(p->theta); d->cos_p=cos(p->phi); d->sin_p=sin(p->phi);
  d->nt=p->nn;
  gb_polar_nodes(d->nt,kr,&d->wt,&d->ct,&d->st,"beam.c, setup_LGb()");
  gb_azimuth_tables(&d->cp,&d->sp,"beam.c, setup_LGb()");
  d->ph_p=gb_spiral_phase(p->lg_m,"beam.c, setup_LGb()");
}

void setup_Bsb(Bsb *p)
{
  BsbD *d=&p->data;
  double ce=1.0/sqrt(pow(cabs(p->e0x),2)+pow(cabs(p->e0y),2));
  d->st=sin(p->d_angle); d->ct=cos(p->d_angle);
  d->ki=2.0*M_PI*p->ni/p->lambda0;
  d->ex=p->e0x*ce; d->ey=p->e0y*ce;
  d->hx=-d->ey*p->ni; d->hy=d->ex*p->ni;
  d->E0=sqrt(2.0*p->power/p->ni);
  d->cos_t=cos(p->theta); d->sin_t=sin(p->theta); d->cos_p=cos(p->phi); d->sin_p=sin(p->phi);
  gb_azimuth_tables(&d->cp,&d->sp,"beam.c, setup_Bsb()");
}

void setup_BsLGb(BsLGb *p)
{
  BsLGbD *d=&p->data;
  double ce=1.0/sqrt(pow(cabs(p->e0x),2)+pow(cabs(p->e0y),2));
  d->st=sin(p->d_angle); d->ct=cos(p->d_angle);
  d->ki=2.0*M_PI*p->ni/p->lambda0;
  d->ex=p->e0x*ce; d->ey=p->e0y*ce;
  d->hx=-d->ey*p->ni; d->hy=d->ex*p->ni;
  d->E0=sqrt(2.0*p->power/p->ni);
  d->cos_t=cos(p->theta); d->sin_t=sin(p->theta); d->cos_p=cos(p->phi); d->sin_p=sin(p->phi);
  gb_azimuth_tables(&d->cp,&d->sp,"beam.c, setup_BsLGb()");
  d->ph_p=gb_spiral_phase(p->lg_m,"beam.c, setup_BsLGb()");
}

void setup_rab(RAb *p)
{
  RAbD *d=&p->data;
  double kr=p->NA/p->ni;
  double ce=sqrt(1.0/M_PI)/(kr*sqrt(pow(cabs(p->e0r),2)+pow(cabs(p->e0a),2)));
  d->ki=2.0*M_PI*p->ni/p->lambda0;
  d->er=p->e0r*ce; d->ea=p->e0a*ce;
  d->hr=-d->ea*p->ni; d->ha=d->er*p->ni;
  d->E0=sqrt(2.0*p->power*p->ni)/p->lambda0;
  d->cos_t=cos(p->theta); d->sin_t=sin(p->theta); d->cos_p=cos(p->phi); d->sin_p=sin(p->phi);
  d->nt=p->nn;
  gb_polar_nodes(d->nt,kr,&d->wt,&d->ct,&d->st,"beam.c, setup_rab()");
  gb_azimuth_tables(&d->cp,&d->sp,"beam.c, setup_rab()");
}

void free_Fpw(Fpw *p){ free(p->data.ct); free(p->data.st); free(p->data.wt); free(p->data.cp); free(p->data.sp); }
void free_LGb(LGb *p)
{
  free(p->data.ct); free(p->data.st); free(p->data.wt); free(p->data.cp); free(p->data.sp); free(p->data.ph_p);
}
void free_Bsb(Bsb *p){ free(p->data.cp); free(p->data.sp); }
void free_BsLGb(BsLGb *p){ free(p->data.cp); free(p->data.sp); free(p->data.ph_p); }
void free_rab(RAb *p){ free(p->data.ct); free(p->data.st); free(p->data.wt); free(p->data.cp); free(p->data.sp); }

/* one wavelength and host index for all beams (reference multi_fbeam.c:878-961) */
static void gb_check_beam(Bobj *obj,int *st,double ni,double lambda0,const char *tag)
{
  if(*st==0){ obj->n_0=ni; obj->lambda_0=lambda0; (*st)++; return; }
  if(obj->n_0!=ni){ printf("data error %s ni, exit\n",tag); exit(1); }
  if(obj->lambda_0!=lambda0){ printf("data error %s lambda0, exit\n",tag); exit(1); }
}

void setup_mfb(Bobj *obj)
{
  int st=0;
  obj->n_0=0.0; obj->lambda_0=0.0;
  for(int i=0;i<obj->n_ipw;i++) gb_check_beam(obj,&st,obj->bd.ipw[i].ni,obj->bd.ipw[i].lambda0,"ipw");
  for(int i=0;i<obj->n_fpw;i++) gb_check_beam(obj,&st,obj->bd.fpw[i].ni,obj->bd.fpw[i].lambda0,"fpw");
  for(int i=0;i<obj->n_lgb;i++) gb_check_beam(obj,&st,obj->bd.lgb[i].ni,obj->bd.lgb[i].lambda0,"lgb");
  for(int i=0;i<obj->n_bsb;i++) gb_check_beam(obj,&st,obj->bd.bsb[i].ni,obj->bd.bsb[i].lambda0,"bsb");
  for(int i=0;i<obj->n_blg;i++) gb_check_beam(obj,&st,obj->bd.blg[i].ni,obj->bd.blg[i].lambda0,"blg");
  for(int i=0;i<obj->n_rab;i++) gb_check_beam(obj,&st,obj->bd.rab[i].ni,obj->bd.rab[i].lambda0,"rab");
  if(st==0){
    printf("no beams defined. check datafile name. Exit...\n");
    exit(0);
  }
  obj->omega=2.0*M_PI/obj->lambda_0;
  for(int i=0;i<obj->n_ipw;i++) setup_ipw(&obj->bd.ipw[i]);
  for(int i=0;i<obj->n_fpw;i++) setup_Fpw(&obj->bd.fpw[i]);
  for(int i=0;i<obj->n_lgb;i++) setup_LGb(&obj->bd.lgb[i]);
  for(int i=0;i<obj->n_bsb;i++) setup_Bsb(&obj->bd.bsb[i]);
  for(int i=0;i<obj->n_blg;i++) setup_BsLGb(&obj->bd.blg[i]);
  for(int i=0;i<obj->n_rab;i++) setup_rab(&obj->bd.rab[i]);
}

void free_mfb(Bobj *obj)
{
  for(int i=0;i<obj->n_fpw;i++) free_Fpw(&obj->bd.fpw[i]);
  for(int i=0;i<obj->n_lgb;i++) free_LGb(&obj->bd.lgb[i]);
  for(int i=0;i<obj->n_bsb;i++) free_Bsb(&obj->bd.bsb[i]);
  for(int i=0;i<obj->n_blg;i++) free_BsLGb(&obj->bd.blg[i]);
  for(int i=0;i<obj->n_rab;i++) free_rab(&obj->bd.rab[i]);
  free(obj->bd.ipw); free(obj->bd.fpw); free(obj->bd.lgb); free(obj->bd.bsb); free(obj->bd.blg); free(obj->bd.rab);
  memset(&obj->bd,0,sizeof(Bdata));
  obj->n_ipw=obj->n_fpw=obj->n_lgb=obj->n_bsb=obj->n_blg=obj->n_rab=0;
}

/* ------------------------------------------------------------ .obj / .dat */

/* raw Bobj, then the six beam arrays (reference mo_setup.c:170-176) */
void gb_mfb_write(FILE *fp,Bobj *obj)
{
  size_t ok=fwrite(obj,sizeof(Bobj),1,fp);
  ok+=fwrite(obj->bd.ipw,sizeof(Ipw),obj->n_ipw,fp);
  ok+=fwrite(obj->bd.fpw,sizeof(Fpw),obj->n_fpw,fp);
  ok+=fwrite(obj->bd.lgb,sizeof(LGb),obj->n_lgb,fp);
  ok+=fwrite(obj->bd.bsb,sizeof(Bsb),obj->n_bsb,fp);
  ok+=fwrite(obj->bd.blg,sizeof(BsLGb),obj->n_blg,fp);
  ok+=fwrite(obj->bd.rab,sizeof(RAb),obj->n_rab,fp);
  if(ok!=(size_t)(1+obj->n_ipw+obj->n_fpw+obj->n_lgb+obj->n_bsb+obj->n_blg+obj->n_rab)){
    printf("beam.c, gb_mfb_write(), failed to write the beam data. exit...\n");
    exit(1);
  }
}

static void *gb_read_array(FILE *fp,int n,size_t sz,const char *what)
{
  void *p=m_alloc2(n>0?n:1,sz,(char *)what);
  if(n>0 && fread(p,sz,n,fp)!=(size_t)n){
    printf("beam.c, gb_mfb_read(), failed to read the %s. exit...\n",what);
    exit(1);
  }
  return p;
}

/* the counterpart of gb_mfb_write; the stored table pointers are rebuilt by setup_mfb */
void gb_mfb_read(FILE *fp,Bobj *obj)
{
  if(fread(obj,sizeof(Bobj),1,fp)!=1){ printf("beam.c, gb_mfb_read(), failed to read the mw. exit...\n"); exit(1); }
  memset(&obj->bd,0,sizeof(Bdata));
  obj->bd.ipw=(Ipw *)gb_read_array(fp,obj->n_ipw,sizeof(Ipw),"ipw");
  obj->bd.fpw=(Fpw *)gb_read_array(fp,obj->n_fpw,sizeof(Fpw),"fpw");
  obj->bd.lgb=(LGb *)gb_read_array(fp,obj->n_lgb,sizeof(LGb),"lgb");
  obj->bd.bsb=(Bsb *)gb_read_array(fp,obj->n_bsb,sizeof(Bsb),"bsb");
  obj->bd.blg=(BsLGb *)gb_read_array(fp,obj->n_blg,sizeof(BsLGb),"blg");
  obj->bd.rab=(RAb *)gb_read_array(fp,obj->n_rab,sizeof(RAb),"rab");
  setup_mfb(obj);
}

/* ------------------------------------------------------------ evaluation */

static double gb_phi_tab[2*GB_BEAM_NPHI];
static pthread_once_t gb_phi_once=PTHREAD_ONCE_INIT;
static void gb_phi_init(void)
{
  double *cp,*sp;
  gb_azimuth_tables(&cp,&sp,"beam.c, azimuths");
  for(int j=0;j<GB_BEAM_NPHI;j++){ gb_phi_tab[2*j]=cp[j]; gb_phi_tab[2*j+1]=sp[j]; }
  free(cp); free(sp);
}

/* descriptors of the spectrum beams of obj (or of the one beam given) */
typedef struct {
  int nb,T,nphase;
  GbBeamDesc *d;
  int *item;
  double *nodes;
  double *phase;
} GbBeamSet;

static void gb_desc_common(GbBeamDesc *b,int kind,double ki,double E0,double ni,double fx,double fy,double fz,
                           double ct,double st,double cp,double sp,double complex p0,double complex p1,
                           double complex q0,double complex q1)
{
  memset(b,0,sizeof(*b));
  b->kind=kind; b->ki=ki; b->E0=E0; b->cep=ni*ni; b->phase=-1;
  b->f[0]=fx; b->f[1]=fy; b->f[2]=fz;
  double M[9]={ct*cp*cp+sp*sp, sp*cp*(ct-1.0), -st*cp,
               sp*cp*(ct-1.0), ct*sp*sp+cp*cp, -st*sp,
               st*cp,          st*sp,          ct};
  memcpy(b->M,M,sizeof(M));
  b->ex[0]=creal(p0); b->ex[1]=cimag(p0); b->ey[0]=creal(p1); b->ey[1]=cimag(p1);
  b->hx[0]=creal(q0); b->hx[1]=cimag(q0); b->hy[0]=creal(q1); b->hy[1]=cimag(q1);
}

static void gb_set_add(GbBeamSet *s,GbBeamDesc *b,int nt,const double *ct,const double *st,const double *wt,
                       const double complex *ph)
{
  b->t0=s->T; b->nt=nt;
  s->d=(GbBeamDesc *)realloc(s->d,(s->nb+1)*sizeof(GbBeamDesc));
  s->item=(int *)realloc(s->item,(s->T+nt)*sizeof(int));
  s->nodes=(double *)realloc(s->nodes,(size_t)(s->T+nt)*3*sizeof(double));
  if(ph){
    b->phase=s->nphase;
    s->phase=(double *)realloc(s->phase,(size_t)(s->nphase+1)*GB_BEAM_NPHI*2*sizeof(double));
    memcpy(s->phase+(size_t)s->nphase*GB_BEAM_NPHI*2,ph,GB_BEAM_NPHI*sizeof(double complex));
    s->nphase++;
  }
  if(!s->d || !s->item || !s->nodes || (ph && !s->phase)){ printf("beam.c: memory allocation failed. exit...\n"); exit(1); }
  for(int t=0;t<nt;t++){
    s->item[s->T+t]=s->nb;
    s->nodes[3*(s->T+t)]=ct[t]; s->nodes[3*(s->T+t)+1]=st[t]; s->nodes[3*(s->T+t)+2]=wt[t];
  }
  s->d[s->nb++]=*b;
  s->T+=nt;
}

static void gb_add_fpw(GbBeamSet *s,Fpw *p)
{
  FpwD *d=&p->data; GbBeamDesc b;
  gb_desc_common(&b,0,d->ki,d->E0,p->ni,p->fx,p->fy,p->fz,d->cos_t,d->sin_t,d->cos_p,d->sin_p,d->ex,d->ey,d->hx,d->hy);
  gb_set_add(s,&b,d->nt,d->ct,d->st,d->wt,NULL);
}
static void gb_add_lgb(GbBeamSet *s,LGb *p)
{
  LGbD *d=&p->data; GbBeamDesc b;
  gb_desc_common(&b,0,d->ki,d->E0,p->ni,p->fx,p->fy,p->fz,d->cos_t,d->sin_t,d->cos_p,d->sin_p,d->ex,d->ey,d->hx,d->hy);
  gb_set_add(s,&b,d->nt,d->ct,d->st,d->wt,p->lg_m?d->ph_p:NULL);
}
static void gb_add_bsb(GbBeamSet *s,Bsb *p)
{
  BsbD *d=&p->data; GbBeamDesc b;
  gb_desc_common(&b,0,d->ki,d->E0,p->ni,p->fx,p->fy,p->fz,d->cos_t,d->sin_t,d->cos_p,d->sin_p,d->ex,d->ey,d->hx,d->hy);
  gb_set_add(s,&b,1,&d->ct,&d->st,&d->st,NULL);
}
static void gb_add_blg(GbBeamSet *s,BsLGb *p)
{
  BsLGbD *d=&p->data; GbBeamDesc b;
  gb_desc_common(&b,0,d->ki,d->E0,p->ni,p->fx,p->fy,p->fz,d->cos_t,d->sin_t,d->cos_p,d->sin_p,d->ex,d->ey,d->hx,d->hy);
  gb_set_add(s,&b,1,&d->ct,&d->st,&d->st,p->lg_m?d->ph_p:NULL);
}
static void gb_add_rab(GbBeamSet *s,RAb *p)
{
  RAbD *d=&p->data; GbBeamDesc b;
  gb_desc_common(&b,1,d->ki,d->E0,p->ni,p->fx,p->fy,p->fz,d->cos_t,d->sin_t,d->cos_p,d->sin_p,d->er,d->ea,d->hr,d->ha);
  gb_set_add(s,&b,d->nt,d->ct,d->st,d->wt,NULL);
}

static void gb_set_free(GbBeamSet *s){ free(s->d); free(s->item); free(s->nodes); free(s->phase); }

/* E, H (and dE/dv, dH/dv when v is given) of the set at n points, added to
 * the outputs; a failure stops the program like the reference's integrator */
static void gb_set_eval(GbBeamSet *s,int n,const double *x,const double *v,double complex *e,double complex *h,
                        double complex *de,double complex *dh)
{
  if(s->nb==0 || n<=0) return;
  pthread_once(&gb_phi_once,gb_phi_init);
  double complex *buf=(double complex *)m_alloc2((size_t)n*12,sizeof(double complex),"beam.c, gb_set_eval()");
  double complex *E=buf,*H=buf+(size_t)3*n,*dE=buf+(size_t)6*n,*dH=buf+(size_t)9*n;
  int rc=gbi_beam_points(s->nb,s->d,s->T,s->item,s->nodes,gb_phi_tab,s->nphase,s->phase,n,x,v,(double *)E,(double *)H,
                         v?(double *)dE:NULL,v?(double *)dH:NULL);
  if(rc==1){ printf("phi integration limit over! Exit...\n"); exit(1); }
  if(rc!=0){ printf("beam.c: GPU evaluation of the incident beams failed: %s. Exit...\n",gb_last_error()); exit(1); }
  for(size_t i=0;i<(size_t)3*n;i++){
    e[i]+=E[i]; h[i]+=H[i];
    if(v){ de[i]+=dE[i]; dh[i]+=dH[i]; }
  }
  free(buf);
}

static void gb_set_build(GbBeamSet *s,Bobj *obj)
{
  memset(s,0,sizeof(*s));
  for(int i=0;i<obj->n_fpw;i++) gb_add_fpw(s,&obj->bd.fpw[i]);
  for(int i=0;i<obj->n_lgb;i++) gb_add_lgb(s,&obj->bd.lgb[i]);
  for(int i=0;i<obj->n_bsb;i++) gb_add_bsb(s,&obj->bd.bsb[i]);
  for(int i=0;i<obj->n_blg;i++) gb_add_blg(s,&obj->bd.blg[i]);
  for(int i=0;i<obj->n_rab;i++) gb_add_rab(s,&obj->bd.rab[i]);
}

static double complex gb_ipw_phase(const double *x,Ipw *p)
{
  IpwD *d=&p->data;
  double te=d->ki*((x[0]-p->fx)*d->sin_t*d->cos_p+(x[1]-p->fy)*d->sin_t*d->sin_p+(x[2]-p->fz)*d->cos_t);
  return cos(te)+I*sin(te);
}

void calc_ipw_EH(double complex *e,double complex *h,double *x,Ipw *ipw)
{
  IpwD *d=&ipw->data;
  double complex Ee=gb_ipw_phase(x,ipw);
  e[0]=d->ex*Ee*d->E0; e[1]=d->ey*Ee*d->E0; e[2]=d->ez*Ee*d->E0;
  h[0]=d->hx*Ee*d->E0; h[1]=d->hy*Ee*d->E0; h[2]=d->hz*Ee*d->E0;
}

void calc_ipw_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Ipw *ipw)
{
  IpwD *d=&ipw->data;
  double complex g=I*d->ki*(d->sin_t*d->cos_p*v[0]+d->sin_t*d->sin_p*v[1]+d->cos_t*v[2]);
  calc_ipw_EH(e,h,x,ipw);
  for(int i=0;i<3;i++){ dedv[i]=e[i]*g; dhdv[i]=h[i]*g; }
}

/* Incident E, H at n points x[n][3] (all beams of obj), into e, h [n][3]. */
void calc_mfb_EH_points(Bobj *obj,int n,const double *x,double complex *e,double complex *h)
{
  for(int p=0;p<n;p++){
    double complex te[3],th[3];
    for(int j=0;j<3;j++){ e[3*p+j]=0.0; h[3*p+j]=0.0; }
    for(int i=0;i<obj->n_ipw;i++){
      calc_ipw_EH(te,th,(double *)x+3*p,&obj->bd.ipw[i]);
      for(int j=0;j<3;j++){ e[3*p+j]+=te[j]; h[3*p+j]+=th[j]; }
    }
  }
  GbBeamSet s;
  gb_set_build(&s,obj);
  gb_set_eval(&s,n,x,NULL,e,h,NULL,NULL);
  gb_set_free(&s);
}

/* The same with the derivatives along v[n][3]: dedv, dhdv [n][3]. */
void calc_mfb_EH_dv_points(Bobj *obj,int n,const double *x,const double *v,double complex *e,double complex *h,
                           double complex *dedv,double complex *dhdv)
{
  for(int p=0;p<n;p++){
    double complex te[3],th[3],tde[3],tdh[3];
    for(int j=0;j<3;j++){ e[3*p+j]=h[3*p+j]=dedv[3*p+j]=dhdv[3*p+j]=0.0; }
    for(int i=0;i<obj->n_ipw;i++){
      calc_ipw_EH_dv(te,th,tde,tdh,(double *)x+3*p,(double *)v+3*p,&obj->bd.ipw[i]);
      for(int j=0;j<3;j++){ e[3*p+j]+=te[j]; h[3*p+j]+=th[j]; dedv[3*p+j]+=tde[j]; dhdv[3*p+j]+=tdh[j]; }
    }
  }
  GbBeamSet s;
  gb_set_build(&s,obj);
  gb_set_eval(&s,n,x,v,e,h,dedv,dhdv);
  gb_set_free(&s);
}

void calc_mfb_EH(double complex *e,double complex *h,double *x,Bobj *obj){ calc_mfb_EH_points(obj,1,x,e,h); }

void calc_mfb_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Bobj *obj)
{
  calc_mfb_EH_dv_points(obj,1,x,v,e,h,dedv,dhdv);
}

/* the reference's per-family single-point functions */
#define GB_ONE_BEAM(NAME,TYPE,ADD)                                                                     \
  void calc_##NAME##_EH(double complex *e,double complex *h,double *x,TYPE *p)                        \
  {                                                                                                    \
    GbBeamSet s; memset(&s,0,sizeof(s)); ADD(&s,p);                                                    \
    for(int j=0;j<3;j++){ e[j]=0.0; h[j]=0.0; }                                                        \
    gb_set_eval(&s,1,x,NULL,e,h,NULL,NULL); gb_set_free(&s);                                           \
  }                                                                                                    \
  void calc_##NAME##_EH_dv(double complex *e,double complex *h,double complex *de,double complex *dh, \
                           double *x,double *v,TYPE *p)                                                \
  {                                                                                                    \
    GbBeamSet s; memset(&s,0,sizeof(s)); ADD(&s,p);                                                    \
    for(int j=0;j<3;j++){ e[j]=h[j]=de[j]=dh[j]=0.0; }                                                 \
    gb_set_eval(&s,1,x,v,e,h,de,dh); gb_set_free(&s);                                                  \
  }
GB_ONE_BEAM(fpw,Fpw,gb_add_fpw)
GB_ONE_BEAM(lgb,LGb,gb_add_lgb)
GB_ONE_BEAM(bsb,Bsb,gb_add_bsb)
GB_ONE_BEAM(bslgb,BsLGb,gb_add_blg)
GB_ONE_BEAM(rab,RAb,gb_add_rab)
