/*
 * force.c -- radiation force and torque (Maxwell stress tensor) and absorbed
 * power (Poynting flux) over the exterior surface of one object (reference
 * d3b2_src/mo_force.c, mo_absorb.c).
 *
 * All evaluation points of the object are gathered first; the fields there
 * come from three batched GPU calls (own object on the boundary with the
 * singular self-element rule, every other object's scattered field, and the
 * plane wave on the host), then the surface sums are formed on the host in
 * FP64 in element order.
 */
#include "gb_host.h"

int gb_mo_EH_points(MOBJ *mo,int n,const double *rt,int type,int which,int memp,double complex *E,double complex *H,int *oid);

typedef struct {
  int n;
  int *t;          /* element index in domain 0's list */
  double *zt;      /* (zeta, eta) */
  double *r;       /* point (torque arm and field point) */
  double *w;       /* non-unit normal */
  double *wt;      /* rule weight */
  int *node;       /* stored node value index (0..3) or -1: evaluate on the boundary */
  double complex *E,*H;
} gb_pts;

static void gb_pts_alloc(gb_pts *p,int n)
{
  p->n=0;
  p->t=(int *)m_alloc2(n,sizeof(int),"force.c");
  p->zt=(double *)m_alloc2(2*n,sizeof(double),"force.c");
  p->r=(double *)m_alloc2(3*n,sizeof(double),"force.c");
  p->w=(double *)m_alloc2(3*n,sizeof(double),"force.c");
  p->wt=(double *)m_alloc2(n,sizeof(double),"force.c");
  p->node=(int *)m_alloc2(n,sizeof(int),"force.c");
  p->E=(double complex *)m_alloc2(3*n,sizeof(double complex),"force.c");
  p->H=(double complex *)m_alloc2(3*n,sizeof(double complex),"force.c");
}
static void gb_pts_free(gb_pts *p)
{
  free(p->t); free(p->zt); free(p->r); free(p->w); free(p->wt); free(p->node); free(p->E); free(p->H);
}

/* evaluation points of the surface rules (reference mo_force.c:56-240):
 * type 0: the 4 (3) collocation nodes with their stored fields, plus the
 * centroid of triangles; type != 0: the 9-point (7-point) rule */
static void gb_surface_points(gb_pts *p,int oid,int type,MOBJ *mo)
{
  DOMD *md=&mo->md[oid];
  BOUD *bd=&md->bd;
  SUBD *sb=&bd->sb[0];
  gb_pts_alloc(p,9*(sb->Ne+1));
  for(int t=1;t<=sb->Ne;t++){
    int asd=abs(sb->sid[t]);
    int quad=(check_element_type(sb->sid[t],bd)==ELT4);
    double cr[3][4],cw[3][3];
    if(quad) bil_copy_elem_const_rw(cr,cw,asd,bd); else lit_copy_elem_const_rw(cr,cw,asd,bd);
    int np; const double *zt,*et,*wt;
    if(type==0){ np=4; if(quad){ zt=bd->zt_44; et=bd->et_44; wt=bd->wt_44; } else { zt=bd->zt_34; et=bd->et_34; wt=bd->wt_34; } }
    else if(quad){ np=9; zt=bd->zt_49; et=bd->et_49; wt=bd->wt_49; }
    else { np=7; zt=bd->zt_37; et=bd->et_37; wt=bd->wt_37; }
    for(int i=0;i<np;i++){
      int k=p->n++;
      p->t[k]=t; p->zt[2*k]=zt[i]; p->zt[2*k+1]=et[i]; p->wt[k]=wt[i];
      if(type==0 && (quad || i<3)){
        p->node[k]=i;
        for(int j=0;j<3;j++){ p->r[3*k+j]=bd->ren[asd][i][j]; p->w[3*k+j]=bd->wen[asd][i][j]; }
      }
      else {
        double r[3],w[3];
        p->node[k]=-1;
        if(quad) bil_rw_zeta_eta(r,w,zt[i],et[i],cr,cw); else lit_rw_zeta_eta(r,w,zt[i],et[i],cr,cw);
        for(int j=0;j<3;j++){ p->r[3*k+j]=r[j]; p->w[3*k+j]=w[j]; }
      }
    }
  }
}

/* total field at the points: stored node values or the own object's
 * boundary integral (EH_s_bd), plus the other objects' scattered fields and
 * the incident wave (reference mo_EH_i_bd / mo_EH_t_bd, mo_field.c:227-282) */
static void gb_point_fields(gb_pts *p,int oid,MOBJ *mo)
{
  DOMD *md=&mo->md[oid];
  SUBD *sb=&md->bd.sb[0];
  int n=p->n;
  double *fr=(double *)m_alloc2(3*n+3,sizeof(double),"force.c");
  for(int k=0;k<n;k++) r_bd(fr+3*k,sb->sid[p->t[k]],p->zt[2*k],p->zt[2*k+1],&md->bd);
  /* own object on the boundary */
  int nb=0;
  for(int k=0;k<n;k++) if(p->node[k]<0) nb++;
  int *bt=(int *)m_alloc2(nb+1,sizeof(int),"force.c");
  int *bdid=(int *)m_alloc2(nb+1,sizeof(int),"force.c");
  double *bz=(double *)m_alloc2(2*nb+2,sizeof(double),"force.c");
  double complex *bo=(double complex *)m_alloc2(6*nb+6,sizeof(double complex),"force.c");
  int q=0;
  for(int k=0;k<n;k++) if(p->node[k]<0){ bt[q]=p->t[k]; bdid[q]=0; bz[2*q]=p->zt[2*k]; bz[2*q+1]=p->zt[2*k+1]; q++; }
  gb_call_lock();
  gb_obj *o=gb_dev(md);
  gb_bv_to_device(md);
  gb_call_unlock();
  if(nb>0 && gb_field_bd(o,PREC_DEF,nb,bdid,bt,bz,bo)) gb_die("force.c, EH_s_bd()");
  q=0;
  for(int k=0;k<n;k++){
    if(p->node[k]>=0){
      for(int j=0;j<3;j++){ p->E[3*k+j]=sb->E[p->t[k]][p->node[k]][j]; p->H[3*k+j]=sb->H[p->t[k]][p->node[k]][j]; }
    }
    else {
      for(int j=0;j<3;j++){ p->E[3*k+j]=bo[6*q+j]; p->H[3*k+j]=bo[6*q+3+j]; }
      q++;
    }
  }
  /* other objects' scattered fields (EH_s, domain chosen per object) */
  double complex *buf=(double complex *)m_alloc2(6*n+6,sizeof(double complex),"force.c");
  int *did=(int *)m_alloc2(n+1,sizeof(int),"force.c");
  for(int m=0;m<mo->N;m++){
    if(m==oid) continue;
    gb_call_lock();
    gb_obj *om=gb_dev(&mo->md[m]);
    gb_bv_to_device(&mo->md[m]);
    gb_call_unlock();
    if(gb_domain_id(om,n,fr,did)) gb_die("force.c, domain_id()");
    if(gb_field_points(om,1,PREC_DEF,n,fr,NULL,did,buf,NULL)) gb_die("force.c, EH_s()");
    for(int k=0;k<n;k++) for(int j=0;j<3;j++){ p->E[3*k+j]+=buf[6*k+j]; p->H[3*k+j]+=buf[6*k+3+j]; }
  }
  /* incident field, all points in one call */
  {
    double complex *ti=(double complex *)m_alloc2((size_t)6*n+6,sizeof(double complex),"force.c");
    calc_mfb_EH_points(&mo->md[0].mw,n,fr,ti,ti+(size_t)3*n);
    for(int k=0;k<n;k++) for(int j=0;j<3;j++){ p->E[3*k+j]+=ti[3*k+j]; p->H[3*k+j]+=ti[(size_t)3*n+3*k+j]; }
    free(ti);
  }
  free(buf); free(did); free(bt); free(bdid); free(bz); free(bo); free(fr);
}

int mo_force_FN(double *F,double *N,double *rc,int oid,int type,MOBJ *mo)
{
  gb_pts p;
  DOMD *md=&mo->md[oid];
  BOUD *bd=&md->bd;
  SUBD *sb=&bd->sb[0];
  double epd=creal(md->n[0])*creal(md->n[0]);
  gb_surface_points(&p,oid,type,mo);
  gb_point_fields(&p,oid,mo);
  double Fs[3]={0,0,0},Ns[3]={0,0,0};
  int k=0;
  for(int t=1;t<=sb->Ne;t++){
    int quad=(check_element_type(sb->sid[t],bd)==ELT4);
    double f[3]={0,0,0},nq[3]={0,0,0};
    while(k<p.n && p.t[k]==t){
      double complex *e=p.E+3*k,*h=p.H+3*k;
      double *r=p.r+3*k,*w=p.w+3*k,T[9];
      double aE2=creal(e[0]*conj(e[0])+e[1]*conj(e[1])+e[2]*conj(e[2]));
      double aH2=creal(h[0]*conj(h[0])+h[1]*conj(h[1])+h[2]*conj(h[2]));
      double Tc=0.25*(epd*aE2+aH2);
      for(int j=0;j<3;j++) for(int l=0;l<3;l++) T[3*j+l]=0.5*(epd*creal(e[j]*conj(e[l]))+creal(h[j]*conj(h[l])));
      T[0]-=Tc; T[4]-=Tc; T[8]-=Tc;
      for(int j=0;j<3;j++){
        f[j]+=(T[3*j]*w[0]+T[3*j+1]*w[1]+T[3*j+2]*w[2])*p.wt[k];
        nq[j]+=(((r[1]-rc[1])*T[3*j+2]-(r[2]-rc[2])*T[3*j+1])*w[0]
               +((r[2]-rc[2])*T[3*j+0]-(r[0]-rc[0])*T[3*j+2])*w[1]
               +((r[0]-rc[0])*T[3*j+1]-(r[1]-rc[1])*T[3*j+0])*w[2])*p.wt[k];
      }
      k++;
    }
    double sc=quad?-1.0:-0.5;
    for(int j=0;j<3;j++){ Fs[j]+=f[j]*sc; Ns[j]+=nq[j]*sc; }
  }
  for(int j=0;j<3;j++){ F[j]=Fs[j]; N[j]=Ns[j]; }
  int nc=sb->Ne;
  gb_pts_free(&p);
  return (nc!=0)?0:-1;
}

int mo_absorb_P(double *P,int oid,int type,MOBJ *mo)
{
  gb_pts p;
  DOMD *md=&mo->md[oid];
  BOUD *bd=&md->bd;
  SUBD *sb=&bd->sb[0];
  gb_surface_points(&p,oid,type,mo);
  gb_point_fields(&p,oid,mo);
  double ps=0.0;
  int k=0;
  for(int t=1;t<=sb->Ne;t++){
    int quad=(check_element_type(sb->sid[t],bd)==ELT4);
    double pe=0.0;
    while(k<p.n && p.t[k]==t){
      double complex *e=p.E+3*k,*h=p.H+3*k;
      double *w=p.w+3*k,vp[3];
      vp[0]=creal(e[1]*conj(h[2])-e[2]*conj(h[1]));
      vp[1]=creal(e[2]*conj(h[0])-e[0]*conj(h[2]));
      vp[2]=creal(e[0]*conj(h[1])-e[1]*conj(h[0]));
      pe+=(vp[0]*w[0]+vp[1]*w[1]+vp[2]*w[2])*p.wt[k];
      k++;
    }
    ps+=pe*(quad?-0.5:-0.25);
  }
  gb_pts_free(&p);
  *P=-ps;
  if(*P<0.0){ *P*=-1.0; return -2; }
  return (sb->Ne!=0)?0:-1;
}
