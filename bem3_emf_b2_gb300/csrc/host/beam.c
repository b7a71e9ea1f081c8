/*
 * beam.c -- incident field of the BEM hot path: plane waves (reference
 * mfb_src/ipw.c and the plane-wave part of mfb_src/multi_fbeam.c).
 *
 * Several plane waves listed in ipw.txt are summed into one incident field,
 * as in the reference.  The other beam families of the reference are outside
 * this library's scope: if their data files are present (or a stored object
 * carries them) the program stops with a message instead of silently
 * ignoring them.
 */
#include "bem3_emf_b2.h"

void init_mfb(Bobj *obj)
{
  memset(obj,0,sizeof(Bobj));
  snprintf(obj->fname_ipw,28,"null"); snprintf(obj->fname_fpw,28,"null");
  snprintf(obj->fname_lgb,28,"null"); snprintf(obj->fname_bsb,28,"null");
  snprintf(obj->fname_blg,28,"null"); snprintf(obj->fname_rab,28,"null");
  obj->bd.ipw=(Ipw *)m_alloc2(1,sizeof(Ipw),"beam.c, init_mfb(), ipw");
}

static void gb_reject_other_beams(Bobj *obj)
{
  const char *fn[5]={fn_fpw,fn_lgb,fn_bsb,fn_blg,fn_rab};
  int n[5]={obj->n_fpw,obj->n_lgb,obj->n_bsb,obj->n_blg,obj->n_rab};
  for(int i=0;i<5;i++){
    if(n[i]!=0){
      printf("beam.c: beam data '%s' is not supported by this library (plane waves only). Exit...\n",fn[i]);
      exit(1);
    }
  }
}

void read_data_mfb(Bobj *obj)
{
  const char *other[5]={fn_fpw,fn_lgb,fn_bsb,fn_blg,fn_rab};
  int wn=read_data_mfb_ipw(fn_ipw,obj);
  for(int i=0;i<5;i++){
    FILE *fp=fopen(other[i],"rt");
    if(fp!=NULL){
      fclose(fp);
      printf("read_data_mfb(): beam data file '%s' found; only plane waves (%s) are supported. Exit...\n",other[i],fn_ipw);
      exit(1);
    }
  }
  if(wn==0){
    printf("read_data_mfb() No beam defined, check beam data file : %s, %s, %s, %s, %s, %s.\n",fn_ipw,other[0],other[1],
           other[2],other[3],other[4]);
    exit(1);
  }
}

static void gb_fail_read(const char *what)
{
  printf("beam.c, read_data_mfb_ipw(), failed to read the %s. exit...\n",what);
  exit(1);
}

/* ipw.txt: two comment lines, the number of waves, a comment line, then per
 * wave: lambda0 ni power Re(e0x) Im(e0x) Re(e0y) Im(e0y) fx fy fz theta phi */
int read_data_mfb_ipw(char *fname,Bobj *obj)
{
  FILE *fp=fopen(fname,"rt");
  char buf[256];
  int nn;
  if(fp==NULL) return 0;
  if(fgets(buf,256,fp)==NULL || fgets(buf,256,fp)==NULL) gb_fail_read("line");
  snprintf(obj->fname_ipw,28,"%s",fname);
  if(fscanf(fp,"%d\n",&nn)!=1) gb_fail_read("nn");
  if(fgets(buf,256,fp)==NULL) gb_fail_read("line");
  if(nn==0){ fclose(fp); return 0; }
  free(obj->bd.ipw);
  obj->n_ipw=nn;
  obj->bd.ipw=(Ipw *)m_alloc2(nn,sizeof(Ipw),"beam.c, read_data_mfb_ipw(), ipw");
  for(int i=0;i<nn;i++){
    double v[12];
    for(int j=0;j<12;j++) if(fscanf(fp,"%lf",&v[j])!=1) gb_fail_read("plane wave parameters");
    Ipw *p=&obj->bd.ipw[i];
    p->lambda0=v[0]; p->ni=v[1]; p->power=v[2];
    p->e0x=v[3]+I*v[4]; p->e0y=v[5]+I*v[6];
    p->fx=v[7]; p->fy=v[8]; p->fz=v[9];
    p->theta=v[10]; p->phi=v[11];
  }
  fclose(fp);
  return nn;
}

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

void print_data_mfb(Bobj *obj)
{
  for(int i=0;i<obj->n_ipw;i++){
    printf(" \"%s\" No.%02d ",obj->fname_ipw,i);
    print_data_ipw(&obj->bd.ipw[i]);
  }
  printf("\n");
}

void print_data_mfb_mksa(Bobj *obj)
{
  for(int i=0;i<obj->n_ipw;i++){
    printf(" \"%s\" No.%02d ",obj->fname_ipw,i);
    print_data_ipw_mksa(&obj->bd.ipw[i]);
  }
  printf("\n");
}

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

static double complex gb_ipw_phase(double *x,Ipw *p)
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

void setup_mfb(Bobj *obj)
{
  gb_reject_other_beams(obj);
  if(obj->n_ipw<=0){
    printf("no beams defined. check datafile name. Exit...\n");
    exit(0);
  }
  obj->n_0=obj->bd.ipw[0].ni;
  obj->lambda_0=obj->bd.ipw[0].lambda0;
  for(int i=1;i<obj->n_ipw;i++){
    if(obj->bd.ipw[i].ni!=obj->n_0){ printf("data error ipw ni, exit\n"); exit(1); }
    if(obj->bd.ipw[i].lambda0!=obj->lambda_0){ printf("data error ipw lambda0, exit\n"); exit(1); }
  }
  obj->omega=2.0*M_PI/obj->lambda_0;
  for(int i=0;i<obj->n_ipw;i++) setup_ipw(&obj->bd.ipw[i]);
}

void free_mfb(Bobj *obj)
{
  free(obj->bd.ipw);
  obj->bd.ipw=NULL;
  obj->n_ipw=0;
}

void calc_mfb_EH(double complex *e,double complex *h,double *x,Bobj *obj)
{
  double complex te[3],th[3];
  for(int i=0;i<3;i++){ e[i]=0.0; h[i]=0.0; }
  for(int i=0;i<obj->n_ipw;i++){
    calc_ipw_EH(te,th,x,&obj->bd.ipw[i]);
    for(int j=0;j<3;j++){ e[j]+=te[j]; h[j]+=th[j]; }
  }
}

void calc_mfb_EH_dv(double complex *e,double complex *h,double complex *dedv,double complex *dhdv,double *x,double *v,Bobj *obj)
{
  double complex te[3],th[3],tde[3],tdh[3];
  for(int i=0;i<3;i++){ e[i]=0.0; h[i]=0.0; dedv[i]=0.0; dhdv[i]=0.0; }
  for(int i=0;i<obj->n_ipw;i++){
    calc_ipw_EH_dv(te,th,tde,tdh,x,v,&obj->bd.ipw[i]);
    for(int j=0;j<3;j++){ e[j]+=te[j]; h[j]+=th[j]; dedv[j]+=tde[j]; dhdv[j]+=tdh[j]; }
  }
}
