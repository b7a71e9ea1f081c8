/*
 * dev.c -- binding of host objects (DOMD) to device-resident gb_obj handles.
 *
 * The reference's structs are stored as raw bytes and sized by callers, so the
 * device handle is not a member of DOMD: a small table keyed by the DOMD
 * address holds it.  Calls from several host threads (the examples call the
 * field API from OpenMP loops) are serialised by a mutex.
 */
#include <pthread.h>
#include "gb_host.h"

typedef struct { DOMD *md; gb_obj *o; int flags; } gb_bind;
static gb_bind *g_tab=NULL;
static int g_n=0,g_cap=0;
static pthread_mutex_t g_mu=PTHREAD_MUTEX_INITIALIZER;

void gb_die(const char *where)
{
  printf("%s: %s. Exit...\n",where,gb_last_error());
  exit(1);
}

gb_obj *gb_dev_peek(DOMD *md)
{
  gb_obj *o=NULL;
  pthread_mutex_lock(&g_mu);
  for(int i=0;i<g_n;i++) if(g_tab[i].md==md){ o=g_tab[i].o; break; }
  pthread_mutex_unlock(&g_mu);
  return o;
}

static gb_obj *gb_make(DOMD *md)
{
  BOUD *bd=&md->bd;
  int Ne=bd->Ne,MN=md->MN;
  size_t n1=(size_t)Ne+1;
  double *cr=(double *)m_alloc2(n1*12,sizeof(double),"dev.c cr");
  double *cw=(double *)m_alloc2(n1*9,sizeof(double),"dev.c cw");
  double *ren=(double *)m_alloc2(n1*12,sizeof(double),"dev.c ren");
  double *wen=(double *)m_alloc2(n1*12,sizeof(double),"dev.c wen");
  double *cor=(double *)m_alloc2(n1*12,sizeof(double),"dev.c corner");
  int *et=(int *)m_alloc2(n1,sizeof(int),"dev.c etype");
  int *eni=(int *)m_alloc2(n1*4,sizeof(int),"dev.c eni");
  int *mdd=(int *)m_alloc2(n1,sizeof(int),"dev.c md");
  int *sdd=(int *)m_alloc2(n1,sizeof(int),"dev.c sd");
  double *kn=(double *)m_alloc2(2*(MN+1),sizeof(double),"dev.c kn");
  int *sbn=(int *)m_alloc2(MN+1,sizeof(int),"dev.c sbn");
  int tot=0;
  for(int d=0;d<=MN;d++) tot+=bd->sb[d].Ne+1;
  int *sid=(int *)m_alloc2(tot,sizeof(int),"dev.c sid");
  for(size_t e=0;e<n1;e++){
    for(int a=0;a<3;a++){
      for(int c=0;c<4;c++) cr[e*12+a*4+c]=bd->cr[e][a][c];
      for(int c=0;c<3;c++) cw[e*9+a*3+c]=bd->cw[e][a][c];
    }
    for(int j=0;j<4;j++) for(int a=0;a<3;a++){
      ren[e*12+j*3+a]=bd->ren[e][j][a];
      wen[e*12+j*3+a]=bd->wen[e][j][a];
      cor[e*12+j*3+a]=bd->rn[bd->ed[e][j]][a];
    }
    et[e]=(e==0)?1:(bd->ed[e][3]!=0);
    for(int j=0;j<4;j++) eni[e*4+j]=bd->eni[e][j];
    mdd[e]=bd->md[e]; sdd[e]=bd->sd[e];
  }
  for(int d=0;d<=MN;d++){ kn[2*d]=creal(md->kn[d]); kn[2*d+1]=cimag(md->kn[d]); sbn[d]=bd->sb[d].Ne; }
  int off=0;
  for(int d=0;d<=MN;d++){ for(int i=0;i<=bd->sb[d].Ne;i++) sid[off+i]=bd->sb[d].sid[i]; off+=bd->sb[d].Ne+1; }
  gb_mesh_desc m;
  m.Ne=Ne; m.NN=bd->NN; m.MN=MN;
  m.cr=cr; m.cw=cw; m.ren=ren; m.wen=wen; m.etype=et; m.eni=eni; m.md=mdd; m.sd=sdd;
  m.kn=kn; m.sb_Ne=sbn; m.sid=sid; m.corner=cor; m.lambda0=md->mw.lambda_0;
  gb_obj *o=NULL;
  int rc=gb_obj_create(&m,&o);
  free(cr); free(cw); free(ren); free(wen); free(cor); free(et); free(eni); free(mdd); free(sdd); free(kn); free(sbn); free(sid);
  if(rc) gb_die("dev.c, gb_obj_create()");
  return o;
}

gb_obj *gb_dev(DOMD *md)
{
  gb_obj *o=gb_dev_peek(md);
  if(o) return o;
  o=gb_make(md);
  pthread_mutex_lock(&g_mu);
  if(g_n==g_cap){
    g_cap=g_cap?2*g_cap:8;
    g_tab=(gb_bind *)realloc(g_tab,g_cap*sizeof(gb_bind));
    if(!g_tab){ printf("dev.c: out of memory. Exit...\n"); exit(1); }
  }
  g_tab[g_n].md=md; g_tab[g_n].o=o; g_tab[g_n].flags=0; g_n++;
  pthread_mutex_unlock(&g_mu);
  return o;
}

void gb_dev_release(DOMD *md)
{
  gb_obj *o=NULL;
  pthread_mutex_lock(&g_mu);
  for(int i=0;i<g_n;i++) if(g_tab[i].md==md){ o=g_tab[i].o; g_tab[i]=g_tab[g_n-1]; g_n--; break; }
  pthread_mutex_unlock(&g_mu);
  if(o) gb_obj_destroy(o);
}

int gb_dev_flags(DOMD *md)
{
  int f=0;
  pthread_mutex_lock(&g_mu);
  for(int i=0;i<g_n;i++) if(g_tab[i].md==md){ f=g_tab[i].flags; break; }
  pthread_mutex_unlock(&g_mu);
  return f;
}

void gb_dev_set_flags(DOMD *md,int set,int clear)
{
  pthread_mutex_lock(&g_mu);
  for(int i=0;i<g_n;i++) if(g_tab[i].md==md){ g_tab[i].flags=(g_tab[i].flags|set)&~clear; break; }
  pthread_mutex_unlock(&g_mu);
}

/* serialises the per-point analysis calls made from several host threads */
static pthread_mutex_t g_call_mu=PTHREAD_MUTEX_INITIALIZER;
void gb_call_lock(void){ pthread_mutex_lock(&g_call_mu); }
void gb_call_unlock(void){ pthread_mutex_unlock(&g_call_mu); }
