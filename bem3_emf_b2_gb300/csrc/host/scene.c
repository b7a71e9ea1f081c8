/*
 * scene.c -- single- and multi-object scenes without intermediate files
 * (gb_scene.h).
 */
#include <time.h>
#include <pthread.h>
#include "gb_host.h"
#include "gb_scene.h"

void gbi_set_error(const char *fmt, ...);

/* host setup of one object in md (rotation th about rv, then translation tv,
 * as d3b2_create_matrix's optional arguments); 0 on success */
static int gbh_setup_object(DOMD *md,const char *medium_file,const char *mesh_file,const char *ipw_file,
                            const double *rv,double th,const double *tv)
{
  memset(md,0,sizeof(DOMD));
  init_mfb(&md->mw);
  if(read_data_mfb_ipw((char *)ipw_file,&md->mw)==0){ printf("scene.c: no plane wave in %s\n",ipw_file); return -1; }
  gb_read_medium_data((char *)medium_file,md);
  gb_read_mesh_data((char *)mesh_file,md);
  md->rv[0]=1.0;
  if(rv){ md->rv[0]=rv[0]; md->rv[1]=rv[1]; md->rv[2]=rv[2]; }
  md->th=th;
  if(tv){ md->tv[0]=tv[0]; md->tv[1]=tv[1]; md->tv[2]=tv[2]; }
  initialize_domd2(md);
  md->cm.MN=md->MN;
  md->cm.nn=(size_t)md->bd.NN;
  md->cm.na=8*md->cm.nn;
  gb_initalize_cmd2(&md->cm);
  gb_init_boundary_data_u2(md);
  return 0;
}

DOMD *gbh_scene_open(const char *medium_file,const char *mesh_file,const char *ipw_file)
{
  DOMD *md=(DOMD *)m_alloc2(1,sizeof(DOMD),"scene.c md");
  if(gbh_setup_object(md,medium_file,mesh_file,ipw_file,NULL,0.0,NULL)){ free(md); return NULL; }
  return md;
}

static void gb_upload_incident_now(DOMD *md)
{
  BOUD *bd=&md->bd;
  size_t n=((size_t)bd->Ne+1)*16;
  double complex *u=(double complex *)m_alloc2(n,sizeof(double complex),"scene.c u");
  double complex *du=(double complex *)m_alloc2(n,sizeof(double complex),"scene.c du");
  for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) for(int l=0;l<4;l++){
    u[(i*4+j)*4+l]=bd->Ui0[i][j][l];
    du[(i*4+j)*4+l]=bd->dUi0[i][j][l];
  }
  if(gb_incident_upload(gb_dev(md),u,du)) gb_die("scene.c, gb_incident_upload()");
  free(u); free(du);
}

int gbh_scene_step(DOMD *md,int form,int type,const double *rc,double *F,double *N)
{
  gb_obj *o=gb_dev(md);
  if(!(gb_dev_flags(md)&GB_F_INC)){
    gb_upload_incident_now(md);
    gb_dev_set_flags(md,GB_F_INC,0);
  }
  if(gb_scene_step(o,form,type)){ printf("gbh_scene_step: %s\n",gb_last_error()); return -1; }
  gb_bv_to_host(md);
  gb_dev_set_flags(md,GB_F_BV,0);
  MOBJ mo;
  memset(&mo,0,sizeof(mo));
  mo.N=1;
  mo.md=md;
  double c[3]={rc[0],rc[1],rc[2]};
  return mo_force_FN(F,N,c,0,0,&mo);
}

void gbh_scene_drop_device(DOMD *md){ gb_dev_release(md); }

size_t gbh_scene_h2d_bytes(DOMD *md)
{
  size_t n1=(size_t)md->bd.Ne+1,tot=0;
  for(int d=0;d<=md->MN;d++) tot+=(size_t)md->bd.sb[d].Ne+1;
  /* cr, cw, ren, wen, corner (doubles), etype, eni, md, sd (ints), sid, kn, incident Ui0/dUi0 */
  return n1*(12+9+12+12+12)*8+n1*(1+4+1+1)*4+tot*4+(size_t)(md->MN+1)*16+2*n1*16*16;
}

size_t gbh_scene_d2h_bytes(DOMD *md)
{
  size_t tot=0;
  for(int d=0;d<=md->MN;d++) tot+=((size_t)md->bd.sb[d].Ne+1)*(16+16+12*4)*16;
  return tot+3*((size_t)md->bd.Ne+1)*16*16;
}

void gbh_scene_close(DOMD *md)
{
  gb_finalize_cmd2(&md->cm);
  finalize_domd2(md);
  free(md);
}

void *gbh_scene_stream(DOMD *md){ return gb_obj_stream(gb_dev(md)); }

void *gbh_scene_obj(DOMD *md)
{
  gb_obj *o=gb_dev(md);
  if(!(gb_dev_flags(md)&GB_F_INC)){
    gb_upload_incident_now(md);
    gb_dev_set_flags(md,GB_F_INC,0);
  }
  return o;
}

/* ------------------------------------------------------------ multi-object */
MOBJ *gbh_mscene_open(int n,const char *const *medium_files,const char *const *mesh_files,const char *ipw_file,
                      const double *rv,const double *th,const double *tv)
{
  if(n<1){ printf("gbh_mscene_open: no objects\n"); return NULL; }
  MOBJ *mo=(MOBJ *)m_alloc2(1,sizeof(MOBJ),"scene.c mo");
  mo->N=n;
  gb_mo_malloc(mo);
  for(int m=0;m<n;m++){
    if(gbh_setup_object(&mo->md[m],medium_files[m],mesh_files[m],ipw_file,rv?rv+3*m:NULL,th?th[m]:0.0,tv?tv+3*m:NULL)){
      printf("gbh_mscene_open: object %d failed\n",m);
      return NULL;
    }
    snprintf(mo->mod_fn[m],FNLGTH,"object_%02d",m);
  }
  return mo;
}

static double g_phase[4];
static double gbh_now(void){ struct timespec t; clock_gettime(CLOCK_MONOTONIC,&t); return t.tv_sec+1e-9*t.tv_nsec; }

/* factorisation of one object (its own gb_obj and streams), run for all
 * objects at once from one host thread each: the objects are independent
 * until the multiple-scattering iteration, and their LU panel chains leave
 * most SMs idle one by one */
struct mscene_job { gb_obj *o; int MN,form,type,dev,rc; double tf; char err[256]; };

static void *mscene_worker(void *p)
{
  struct mscene_job *j=(struct mscene_job *)p;
  if(gb_use_device(j->dev)){ j->rc=-1; snprintf(j->err,sizeof(j->err),"%s",gb_last_error()); return NULL; }
  double t2=gbh_now();
  if(j->form==0 ? gb_factor_fp64(j->o) : gb_factor_mixed(j->o)) j->rc=-1;
  if(j->rc) snprintf(j->err,sizeof(j->err),"%s",gb_last_error());
  j->tf=gbh_now()-t2;
  return NULL;
}

/* assembly of every object (one work list) and the objects' factorisations
 * (concurrently); *ta, *tf: their wall times */
static int mscene_factor(MOBJ *mo,int form,int type,double *ta_out,double *tf_out)
{
  double ta=0.0,tf=0.0;
  struct mscene_job *jobs=(struct mscene_job *)calloc(mo->N,sizeof(struct mscene_job));
  pthread_t *th=(pthread_t *)calloc(mo->N,sizeof(pthread_t));
  gb_obj **objs=(gb_obj **)calloc(mo->N,sizeof(gb_obj *));
  int dev=gb_current_device();
  for(int m=0;m<mo->N;m++){  /* device copies first (host tables, sequential) */
    jobs[m].o=objs[m]=gb_dev(&mo->md[m]);
    jobs[m].MN=mo->md[m].MN; jobs[m].form=form; jobs[m].type=type; jobs[m].dev=dev;
  }
  /* every domain of every object: one launch per assembly phase */
  double ta0=gbh_now();
  if(gb_assemble_objects(objs,mo->N,type,gb_form_precision(form))){
    printf("gbh_mscene_step: %s\n",gb_last_error()); free(jobs); free(th); free(objs); return -1;
  }
  ta=gbh_now()-ta0;
  free(objs);
  double tw=gbh_now();
  for(int m=0;m<mo->N;m++)
    if(pthread_create(&th[m],NULL,mscene_worker,&jobs[m])){ jobs[m].rc=-2; }
  int bad=-1;
  for(int m=0;m<mo->N;m++){
    if(jobs[m].rc!=-2) pthread_join(th[m],NULL);
    else { jobs[m].rc=0; mscene_worker(&jobs[m]); }  /* no thread available: run here */
    if(jobs[m].rc && bad<0) bad=m;
  }
  double tw2=gbh_now();
  if(bad>=0){
    printf("gbh_mscene_step: %s\n",jobs[bad].err);
    gbi_set_error("%s",jobs[bad].err);  /* the worker's message, for this thread's gb_last_error() */
    free(jobs); free(th); return -1;
  }
  free(jobs); free(th);
  tf=tw2-tw;
  /* matrices and the factors are resident: the iteration reads no .cmat file */
  for(int m=0;m<mo->N;m++) gb_dev_set_flags(&mo->md[m],GB_F_CMAT|GB_F_INV,GB_F_BV);
  *ta_out=ta; *tf_out=tf;
  return 0;
}

/* force and torque of every object at once (mo_force_FN per object, one
 * host thread each, at most 16): the objects' sums are independent, their
 * field evaluations run on each thread's own stream */
struct force_pool { MOBJ *mo; const double *rc; double *F,*N; int dev,next,bad; pthread_mutex_t mu; };

static void *force_worker(void *p)
{
  struct force_pool *q=(struct force_pool *)p;
  if(gb_use_device(q->dev)){ q->bad=1; return NULL; }
  for(;;){
    pthread_mutex_lock(&q->mu);
    int m=q->next++;
    pthread_mutex_unlock(&q->mu);
    if(m>=q->mo->N) break;
    double c[3];
    for(int i=0;i<3;i++) c[i]=q->rc?q->rc[3*m+i]:q->mo->md[m].tv[i];
    if(mo_force_FN(q->F+3*m,q->N+3*m,c,m,0,q->mo)<0){ pthread_mutex_lock(&q->mu); q->bad=1; pthread_mutex_unlock(&q->mu); }
  }
  return NULL;
}

static int mscene_forces(MOBJ *mo,const double *rc,double *F,double *N)
{
  struct force_pool q;
  q.mo=mo; q.rc=rc; q.F=F; q.N=N; q.dev=gb_current_device(); q.next=0; q.bad=0;
  pthread_mutex_init(&q.mu,NULL);
  int nt=mo->N<16?mo->N:16,started=0;
  pthread_t th[16];
  for(int i=0;i<nt;i++){ if(pthread_create(&th[i],NULL,force_worker,&q)) break; started++; }
  if(started==0) force_worker(&q);
  for(int i=0;i<started;i++) pthread_join(th[i],NULL);
  pthread_mutex_destroy(&q.mu);
  return q.bad?-1:0;
}

int gbh_mscene_step(MOBJ *mo,int form,int type,const double *rc,double *F,double *N)
{
  double ta=0.0,tf=0.0;
  if(mscene_factor(mo,form,type,&ta,&tf)) return -1;
  double t3=gbh_now();
  mo_solve_bv(mo);
  double t4=gbh_now();
  if(mscene_forces(mo,rc,F,N)) return -1;
  g_phase[0]=ta; g_phase[1]=tf; g_phase[2]=t4-t3; g_phase[3]=gbh_now()-t4;
  return 0;
}

/* Many incident beams as right-hand sides of one scene (the reference sums
 * every wave of ipw.txt into one field, multi_fbeam.c:817-833, so beam b
 * alone is what a reference run with an ipw.txt holding only wave b
 * computes).  The coefficient matrices, the factors and the
 * multiple-scattering operators do not depend on the beam: they are built
 * once -- assembly (one work list over every domain of every object),
 * factorisations, and the cross operators (by the first beam's iteration,
 * then kept) -- and each beam costs its incident potential, the iteration,
 * E/H and the force.  Beam b is wave b of beams_file (ipw.txt layout); its
 * force and torque on object m about rc[3m..] (NULL: the object's
 * translation point) go to F, N [b][m][3]; *nbeam the number of waves read.
 * The phases' wall times are those of gbh_mscene_phase_times, the iteration
 * and force summed over the beams. */
int gbh_mscene_beams(MOBJ *mo,int form,int type,const char *beams_file,const double *rc,double *F,double *N,
                     int *nbeam)
{
  Bobj all;
  memset(&all,0,sizeof(all));
  init_mfb(&all);
  int nb=read_data_mfb_ipw((char *)beams_file,&all);
  if(nb<=0){ printf("gbh_mscene_beams: no plane wave in %s\n",beams_file); return -1; }
  setup_mfb(&all);
  *nbeam=nb;
  double ta=0.0,tf=0.0;
  if(mscene_factor(mo,form,type,&ta,&tf)){ free_mfb(&all); return -1; }
  double tit=0.0,tfo=0.0;
  Ipw **keep=(Ipw **)calloc(mo->N,sizeof(Ipw *));
  int *keepn=(int *)calloc(mo->N,sizeof(int));
  for(int m=0;m<mo->N;m++){ keep[m]=mo->md[m].mw.bd.ipw; keepn[m]=mo->md[m].mw.n_ipw; }
  int rcode=0;
  for(int b=0;b<nb && !rcode;b++){
    for(int m=0;m<mo->N;m++){  /* this beam alone, as the objects' incident field */
      DOMD *md=&mo->md[m];
      md->mw.n_ipw=1;
      md->mw.bd.ipw=all.bd.ipw+b;
      gb_init_boundary_data_u2(md);
      gb_dev_set_flags(md,0,GB_F_INC|GB_F_BV);
    }
    double t3=gbh_now();
    mo_solve_bv(mo);
    double t4=gbh_now();
    if(mscene_forces(mo,rc,F+3*(size_t)b*mo->N,N+3*(size_t)b*mo->N)) rcode=-1;
    tit+=t4-t3; tfo+=gbh_now()-t4;
  }
  for(int m=0;m<mo->N;m++){ mo->md[m].mw.bd.ipw=keep[m]; mo->md[m].mw.n_ipw=keepn[m]; }
  /* the objects' own incident field again (their beams were replaced above) */
  for(int m=0;m<mo->N;m++){ gb_init_boundary_data_u2(&mo->md[m]); gb_dev_set_flags(&mo->md[m],0,GB_F_INC|GB_F_BV); }
  free(keep); free(keepn);
  free_mfb(&all);
  g_phase[0]=ta; g_phase[1]=tf; g_phase[2]=tit; g_phase[3]=tfo;
  return rcode;
}

void gbh_mscene_phase_times(double *t){ for(int i=0;i<4;i++) t[i]=g_phase[i]; }

void gbh_mscene_drop_device(MOBJ *mo){ for(int m=0;m<mo->N;m++) gb_dev_release(&mo->md[m]); }

size_t gbh_mscene_h2d_bytes(MOBJ *mo)
{
  size_t t=0;
  for(int m=0;m<mo->N;m++) t+=gbh_scene_h2d_bytes(&mo->md[m]);
  return t;
}

size_t gbh_mscene_d2h_bytes(MOBJ *mo)
{
  size_t t=0;
  for(int m=0;m<mo->N;m++) t+=gbh_scene_d2h_bytes(&mo->md[m]);
  return t;
}

void gbh_mscene_close(MOBJ *mo)
{
  mo_finalize(mo);  /* releases the device copies too */
  free(mo);
}
