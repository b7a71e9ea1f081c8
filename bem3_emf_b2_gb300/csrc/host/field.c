/*
 * field.c -- potentials and fields at points (reference d3b1_field.c,
 * mo_field.c, setup2.c:944-978).  Every call evaluates on the GPU; the
 * per-point entry points keep the reference's signatures and may be called
 * from several host threads at once, as the reference's examples do from
 * OpenMP loops (example2.c:45, example4.c:53): only the one-time setup of an
 * object's device copy is serialised; the evaluations run concurrently, each
 * thread on its own stream (gb_field_points).  gb_mo_EH_points() evaluates
 * many points in one launch per object.
 */
#include "gb_host.h"

/* the object's device copy with its boundary values uploaded (once) */
static gb_obj *gb_ready(DOMD *md)
{
  gb_call_lock();
  gb_obj *o=gb_dev(md);
  gb_bv_to_device(md);
  gb_call_unlock();
  return o;
}

static gb_obj *gb_dev_locked(DOMD *md)
{
  gb_call_lock();
  gb_obj *o=gb_dev(md);
  gb_call_unlock();
  return o;
}

int domain_id(double *rt,DOMD *md)
{
  int did;
  if(gb_domain_id(gb_dev_locked(md),1,rt,&did)) gb_die("field.c, domain_id()");
  return did;
}

/* mode: 0 potentials (4 values), 1 E,H from E/H boundary values (6),
 * 2 E,H from potential derivatives (6) */
static int gb_obj_field(double complex *out,double *rt,int type,DOMD *md,int mode)
{
  int did,flag=0;
  gb_obj *o=gb_ready(md);
  if(gb_domain_id(o,1,rt,&did)) gb_die("field.c, domain_id()");
  if(did<0){
    int n=(mode==0)?4:6;
    for(int i=0;i<n;i++) out[i]=0.0;
    return did;
  }
  if(gb_field_points(o,mode,type,1,rt,NULL,&did,out,&flag)) gb_die("field.c, gb_field_points()");
  if(mode==2) return flag;
  return did;
}

int gb_mEMP_s(double complex *U,double *rt,int type,DOMD *md){ return gb_obj_field(U,rt,type,md,0); }
int gb_EH_s(double complex *E,double complex *H,double *rt,int type,DOMD *md)
{
  double complex o[6];
  int did=gb_obj_field(o,rt,type,md,1);
  for(int i=0;i<3;i++){ E[i]=o[i]; H[i]=o[3+i]; }
  return did;
}
int gb_EH_mEMP_s(double complex *E,double complex *H,double *rt,int type,DOMD *md)
{
  double complex o[6];
  int did=gb_obj_field(o,rt,type,md,2);
  for(int i=0;i<3;i++){ E[i]=o[i]; H[i]=o[3+i]; }
  return did;
}

void mo_object_domain_id(int *oid,int *did,double *rt,MOBJ *mo)
{
  for(int o=0;o<mo->N;o++){
    *did=domain_id(rt,&mo->md[o]);
    if(*did!=0){ *oid=o; return; }
  }
  *oid=-1;
}

int mo_mEMP_s(double complex *U,double *rt,int type,MOBJ *mo)
{
  int oid,did;
  mo_object_domain_id(&oid,&did,rt,mo);
  if(oid<0){
    double complex tu[4];
    for(int i=0;i<4;i++) U[i]=0.0;
    for(int m=0;m<mo->N;m++){ gb_mEMP_s(tu,rt,type,&mo->md[m]); for(int i=0;i<4;i++) U[i]+=tu[i]; }
  }
  else gb_mEMP_s(U,rt,type,&mo->md[oid]);
  return oid;
}

int mo_mEMP_t(double complex *U,double *rt,int type,MOBJ *mo)
{
  int oid,did;
  mo_object_domain_id(&oid,&did,rt,mo);
  if(oid<0){
    double complex te[3],th[3],tu[4];
    calc_mfb_EH(te,th,rt,&mo->md[0].mw);
    for(int i=0;i<3;i++) U[i]=te[i];
    U[3]=0.0;
    for(int m=0;m<mo->N;m++){ gb_mEMP_s(tu,rt,type,&mo->md[m]); for(int i=0;i<4;i++) U[i]+=tu[i]; }
  }
  else gb_mEMP_s(U,rt,type,&mo->md[oid]);
  return oid;
}

int mo_mEMP_i(double complex *U,double *rt,int type,MOBJ *mo)
{
  int oid,did;
  double complex e[3],h[3];
  mo_object_domain_id(&oid,&did,rt,mo);
  calc_mfb_EH(e,h,rt,&mo->md[0].mw);
  for(int i=0;i<3;i++) U[i]=e[i];
  U[3]=0.0;
  return oid;
}

static int gb_mo_EH_any(double complex *E,double complex *H,double *rt,int type,MOBJ *mo,int total,int memp)
{
  int oid,did;
  double complex te[3],th[3];
  mo_object_domain_id(&oid,&did,rt,mo);
  if(oid<0){
    if(total) calc_mfb_EH(E,H,rt,&mo->md[0].mw);
    else for(int i=0;i<3;i++){ E[i]=0.0; H[i]=0.0; }
    for(int m=0;m<mo->N;m++){
      if(memp) gb_EH_mEMP_s(te,th,rt,type,&mo->md[m]); else gb_EH_s(te,th,rt,type,&mo->md[m]);
      for(int i=0;i<3;i++){ E[i]+=te[i]; H[i]+=th[i]; }
    }
  }
  else {
    if(memp) gb_EH_mEMP_s(E,H,rt,type,&mo->md[oid]); else gb_EH_s(E,H,rt,type,&mo->md[oid]);
  }
  return oid;
}

int mo_EH_s(double complex *E,double complex *H,double *rt,int type,MOBJ *mo){ return gb_mo_EH_any(E,H,rt,type,mo,0,0); }
int mo_EH_t(double complex *E,double complex *H,double *rt,int type,MOBJ *mo){ return gb_mo_EH_any(E,H,rt,type,mo,1,0); }
int mo_EH_mEMP_s(double complex *E,double complex *H,double *rt,int type,MOBJ *mo){ return gb_mo_EH_any(E,H,rt,type,mo,0,1); }
int mo_EH_mEMP_t(double complex *E,double complex *H,double *rt,int type,MOBJ *mo){ return gb_mo_EH_any(E,H,rt,type,mo,1,1); }

int mo_EH_i(double complex *E,double complex *H,double *rt,int type,MOBJ *mo)
{
  int oid,did;
  mo_object_domain_id(&oid,&did,rt,mo);
  calc_mfb_EH(E,H,rt,&mo->md[0].mw);
  return oid;
}
int mo_EH_mEMP_i(double complex *E,double complex *H,double *rt,int type,MOBJ *mo){ return mo_EH_i(E,H,rt,type,mo); }

/* ---- on the boundary ---- */
void gb_EH_s_bd(double complex *E,double complex *H,int did,int t,double zt,double et,int type,DOMD *md)
{
  double z[2]={zt,et};
  double complex o[6];
  gb_obj *ob=gb_ready(md);
  if(gb_field_bd(ob,type,1,&did,&t,z,o)) gb_die("field.c, EH_s_bd()");
  for(int i=0;i<3;i++){ E[i]=o[i]; H[i]=o[3+i]; }
}

void mo_EH_s_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo)
{
  gb_EH_s_bd(E,H,did,t,zeta_t,eta_t,type,&mo->md[oid]);
}

static void gb_add_others(double complex *E,double complex *H,double *rt,int oid,int type,MOBJ *mo)
{
  double complex te[3],th[3];
  for(int m=0;m<mo->N;m++){
    if(m==oid) continue;
    gb_EH_s(te,th,rt,type,&mo->md[m]);
    for(int i=0;i<3;i++){ E[i]+=te[i]; H[i]+=th[i]; }
  }
}

void mo_EH_t_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo)
{
  gb_EH_s_bd(E,H,did,t,zeta_t,eta_t,type,&mo->md[oid]);
  if(did==0){
    double rt[3];
    double complex te[3],th[3];
    r_bd(rt,mo->md[oid].bd.sb[did].sid[t],zeta_t,eta_t,&mo->md[oid].bd);
    gb_add_others(E,H,rt,oid,type,mo);
    calc_mfb_EH(te,th,rt,&mo->md[0].mw);
    for(int i=0;i<3;i++){ E[i]+=te[i]; H[i]+=th[i]; }
  }
}

void mo_EH_i_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo)
{
  if(did==0){
    double rt[3];
    r_bd(rt,mo->md[oid].bd.sb[did].sid[t],zeta_t,eta_t,&mo->md[oid].bd);
    calc_mfb_EH(E,H,rt,&mo->md[0].mw);
    gb_add_others(E,H,rt,oid,type,mo);
  }
  else for(int i=0;i<3;i++){ E[i]=0.0; H[i]=0.0; }
}

void mo_EH_a_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo)
{
  gb_EH_s_bd(E,H,did,t,zeta_t,eta_t,type,&mo->md[oid]);
  if(did==0){
    double rt[3];
    r_bd(rt,mo->md[oid].bd.sb[did].sid[t],zeta_t,eta_t,&mo->md[oid].bd);
    gb_add_others(E,H,rt,oid,type,mo);
  }
}

/* Batched field map: total (which = 1), scattered (0) or incident (2) field
 * at n points, through the boundary-value formula (memp = 0, mo_EH_*) or the
 * potential-derivative formula (memp = 1, mo_EH_mEMP_*).  One domain-id and
 * one field launch per object instead of one per point; results equal n
 * calls of the per-point functions.  oid may be NULL. */
int gb_mo_EH_points(MOBJ *mo,int n,const double *rt,int type,int which,int memp,double complex *E,double complex *H,int *oid)
{
  if(n<=0) return 0;
  int *own=(int *)m_alloc2(n,sizeof(int),"field.c own");
  int *did=(int *)m_alloc2((size_t)n*mo->N,sizeof(int),"field.c did");
  double complex *buf=(double complex *)m_alloc2((size_t)n*6,sizeof(double complex),"field.c buf");
  int *flag=(int *)m_alloc2(n,sizeof(int),"field.c flag");
  for(int m=0;m<mo->N;m++){
    gb_obj *o=gb_ready(&mo->md[m]);
    if(gb_domain_id(o,n,rt,did+(size_t)m*n)) gb_die("field.c, gb_mo_EH_points()");
  }
  /* the incident field where it is wanted, all such points in one call */
  double *ip=(double *)m_alloc2((size_t)n*3,sizeof(double),"field.c ip");
  int *ix=(int *)m_alloc2(n,sizeof(int),"field.c ix");
  int ni=0;
  for(int p=0;p<n;p++){
    own[p]=-1;
    for(int m=0;m<mo->N;m++) if(did[(size_t)m*n+p]!=0){ own[p]=m; break; }
    for(int i=0;i<3;i++){ E[3*p+i]=0.0; H[3*p+i]=0.0; }
    if(which==2 || (which==1 && own[p]<0)){
      for(int i=0;i<3;i++) ip[3*ni+i]=rt[3*p+i];
      ix[ni++]=p;
    }
  }
  if(ni>0){
    double complex *ti=(double complex *)m_alloc2((size_t)6*ni,sizeof(double complex),"field.c ti");
    calc_mfb_EH_points(&mo->md[0].mw,ni,ip,ti,ti+(size_t)3*ni);
    for(int k=0;k<ni;k++) for(int i=0;i<3;i++){ E[3*ix[k]+i]=ti[3*k+i]; H[3*ix[k]+i]=ti[(size_t)3*ni+3*k+i]; }
    free(ti);
  }
  free(ip); free(ix);
  if(which!=2){
    double *pr=(double *)m_alloc2((size_t)n*3,sizeof(double),"field.c pr");
    int *pd=(int *)m_alloc2(n,sizeof(int),"field.c pd");
    int *pi=(int *)m_alloc2(n,sizeof(int),"field.c pi");
    for(int m=0;m<mo->N;m++){
      int k=0;
      for(int p=0;p<n;p++){
        int d=did[(size_t)m*n+p];
        if(d<0) continue;
        if(own[p]>=0 && own[p]!=m) continue;   /* inside another object: only that object contributes */
        pr[3*k]=rt[3*p]; pr[3*k+1]=rt[3*p+1]; pr[3*k+2]=rt[3*p+2];
        pd[k]=d; pi[k]=p; k++;
      }
      if(k==0) continue;
      if(gb_field_points(gb_dev(&mo->md[m]),memp?2:1,type,k,pr,NULL,pd,buf,flag)) gb_die("field.c, gb_mo_EH_points()");
      for(int q=0;q<k;q++){
        int p=pi[q];
        for(int i=0;i<3;i++){ E[3*p+i]+=buf[6*q+i]; H[3*p+i]+=buf[6*q+3+i]; }
      }
    }
    free(pr); free(pd); free(pi);
  }
  if(oid) for(int p=0;p<n;p++) oid[p]=own[p];
  free(own); free(did); free(buf); free(flag);
  return 0;
}
