/*
 * solve.c -- multi-object iteration (reference d3b2_src/mo_solve.c:10-120).
 *
 * The coefficient matrices and the inverse of A of every object are read
 * from their .cmat files once and stay in the GPU's memory; the iteration
 * (incident-field update from the other objects' scattered fields, RHS,
 * invA * B, boundary values, convergence measure) runs on the device.  Only
 * the convergence sums cross to the host per iteration.  Messages and the
 * stopping rule (cc < CCD after more than ITER_MIN iterations, at most
 * ITER_MAX) are the reference's.
 */
#include "gb_host.h"
#include <pthread.h>

/* progress messages of mo_solve_bv (the reference's); off with gbh_set_quiet(1) */
static int g_quiet=0;
void gbh_set_quiet(int q){ g_quiet=q; }
/* iteration count and convergence measure of the last mo_solve_bv */
static int g_last_iter=0;
static double g_last_cc=0.0;
void gbh_last_iteration(int *iter,double *cc){ *iter=g_last_iter; *cc=g_last_cc; }
#define MSG(...) do{ if(!g_quiet){ printf(__VA_ARGS__); fflush(stdout); } }while(0)

static double complex *gb_read_cmat_file(const char *fn,size_t n)
{
  FILE *fp=fopen(fn,"rb");
  if(fp==NULL){ printf("solve.c, Failed to open %s file.\n",fn); exit(1); }
  double complex *b=(double complex *)malloc(n*sizeof(double complex)+16);
  if(b==NULL){ printf("solve.c, memory allocation error for %s. Exit..\n",fn); exit(1); }
  if(fread(b,sizeof(double complex),n,fp)!=n){ printf("solve.c, failed to read %s. exit...\n",fn); exit(1); }
  fclose(fp);
  return b;
}

/* the object's factors from a block-factor file (GB_BLK_MAGIC); 0 if the
 * file is the reference's dense inverse instead, 1 when loaded */
static int gb_read_block_file(DOMD *md,gb_obj *o)
{
  FILE *fp=fopen(md->cm.lupfn,"rb");
  if(fp==NULL){ printf("solve.c, failed to open %s. exit...\n",md->cm.lupfn); exit(1); }
  unsigned char hdr[GB_BLK_HEADER];
  size_t got=fread(hdr,1,GB_BLK_HEADER,fp);
  if(got!=GB_BLK_HEADER || memcmp(hdr,GB_BLK_MAGIC,8)!=0){ fclose(fp); return 0; }
  int meta[4];
  memcpy(meta,hdr+8,sizeof(meta));
  size_t nn=(size_t)md->bd.NN;
  if(meta[0]!=GB_BLK_VERSION || meta[1]!=(int)nn || meta[2]!=5 || meta[3]!=(int)sizeof(double complex)){
    printf("solve.c, %s: block factors version %d for %d nodes, expected version %d for %zu nodes. exit...\n",
           md->cm.lupfn,meta[0],meta[1],GB_BLK_VERSION,nn);
    exit(1);
  }
  double complex *m=(double complex *)m_alloc2(5*nn*nn,sizeof(double complex),"solve.c blk");
  if(fread(m,sizeof(double complex),5*nn*nn,fp)!=5*nn*nn){ printf("solve.c, failed to read %s. exit...\n",md->cm.lupfn); exit(1); }
  fclose(fp);
  if(gb_block_factors_upload(o,m,m+nn*nn,m+2*nn*nn,m+3*nn*nn,m+4*nn*nn)) gb_die("solve.c, gb_block_factors_upload()");
  free(m);
  return 1;
}

void gb_cmat_read(DOMD *md,int with_inverse)
{
  gb_obj *o=gb_dev(md);
  int f=gb_dev_flags(md);
  if(!(f&GB_F_CMAT)){
    for(int d=0;d<=md->MN;d++){
      size_t N=4*(size_t)md->bd.sb[d].Ne;
      double complex *G=gb_read_cmat_file(md->cm.tgfn[d],N*N);
      double complex *H=gb_read_cmat_file(md->cm.thfn[d],N*N);
      if(gb_cmatrix_upload(o,d,G,H,NULL,NULL,NULL)) gb_die("solve.c, gb_cmatrix_upload()");
      free(G); free(H);
      double complex *dG=gb_read_cmat_file(md->cm.tdgfn[d],2*N*N);
      double complex *dH=gb_read_cmat_file(md->cm.tdhfn[d],2*N*N);
      FILE *fp=fopen(md->cm.tdffn[d],"rb");
      double *dFe=(double *)malloc(3*N*sizeof(double)+8);
      if(fp==NULL || fread(dFe,sizeof(double),3*N,fp)!=3*N){ printf("solve.c, failed to read %s. exit...\n",md->cm.tdffn[d]); exit(1); }
      fclose(fp);
      if(gb_cmatrix_upload(o,d,NULL,NULL,dG,dH,dFe)) gb_die("solve.c, gb_cmatrix_upload()");
      free(dG); free(dH); free(dFe);
    }
    gb_dev_set_flags(md,GB_F_CMAT,0);
  }
  if(with_inverse && !(gb_dev_flags(md)&GB_F_INV)){
    if(gb_read_block_file(md,o)==0){
      size_t na=8*(size_t)md->bd.NN;
      double complex *A=gb_read_cmat_file(md->cm.lupfn,na*na);
      if(gb_invA_upload(o,A)) gb_die("solve.c, gb_invA_upload()");
      free(A);
    }
    gb_dev_set_flags(md,GB_F_INV,0);
  }
}

static void gb_flat_incident(DOMD *md,double complex *u,double complex *du)
{
  BOUD *bd=&md->bd;
  for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) for(int l=0;l<4;l++){
    u[(i*4+j)*4+l]=bd->Ui0[i][j][l];
    du[(i*4+j)*4+l]=bd->dUi0[i][j][l];
  }
}

static void gb_upload_incident(DOMD *md)
{
  size_t n=((size_t)md->bd.Ne+1)*16;
  double complex *u=(double complex *)m_alloc2(n,sizeof(double complex),"solve.c u");
  double complex *du=(double complex *)m_alloc2(n,sizeof(double complex),"solve.c du");
  gb_flat_incident(md,u,du);
  if(gb_incident_upload(gb_dev(md),u,du)) gb_die("solve.c, gb_incident_upload()");
  free(u); free(du);
  gb_dev_set_flags(md,GB_F_INC,0);
}

/* device boundary values and incident potential -> host structs */
void gb_bv_to_host(DOMD *md)
{
  gb_obj *o=gb_dev(md);
  BOUD *bd=&md->bd;
  for(int d=0;d<=md->MN;d++){
    SUBD *sb=&bd->sb[d];
    size_t n1=(size_t)sb->Ne+1;
    double complex *U=(double complex *)m_alloc2(n1*16,sizeof(double complex),"solve.c U");
    double complex *dU=(double complex *)m_alloc2(n1*16,sizeof(double complex),"solve.c dU");
    double complex *E=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c E");
    double complex *dE=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c dE");
    double complex *H=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c H");
    double complex *dH=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c dH");
    if(gb_bv_download(o,d,U,dU,E,dE,H,dH)) gb_die("solve.c, gb_bv_download()");
    for(size_t s=1;s<n1;s++) for(int j=0;j<4;j++){
      for(int l=0;l<4;l++){ sb->U[s][j][l]=U[(s*4+j)*4+l]; sb->dU[s][j][l]=dU[(s*4+j)*4+l]; }
      for(int l=0;l<3;l++){
        sb->E[s][j][l]=E[(s*4+j)*3+l]; sb->dE[s][j][l]=dE[(s*4+j)*3+l];
        sb->H[s][j][l]=H[(s*4+j)*3+l]; sb->dH[s][j][l]=dH[(s*4+j)*3+l];
      }
    }
    free(U); free(dU); free(E); free(dE); free(H); free(dH);
  }
  size_t n=((size_t)bd->Ne+1)*16;
  double complex *u=(double complex *)m_alloc2(n,sizeof(double complex),"solve.c ui");
  double complex *du=(double complex *)m_alloc2(n,sizeof(double complex),"solve.c dui");
  double complex *up=(double complex *)m_alloc2(n,sizeof(double complex),"solve.c uip");
  if(gb_incident_download(o,u,du,up)) gb_die("solve.c, gb_incident_download()");
  for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) for(int l=0;l<4;l++){
    bd->Ui[i][j][l]=u[(i*4+j)*4+l]; bd->dUi[i][j][l]=du[(i*4+j)*4+l]; bd->Uip[i][j][l]=up[(i*4+j)*4+l];
  }
  free(u); free(du); free(up);
}

/* host boundary values (e.g. from mo_dat_read) -> device, once */
void gb_bv_to_device(DOMD *md)
{
  if(gb_dev_flags(md)&GB_F_BV) return;
  gb_obj *o=gb_dev(md);
  BOUD *bd=&md->bd;
  for(int d=0;d<=md->MN;d++){
    SUBD *sb=&bd->sb[d];
    size_t n1=(size_t)sb->Ne+1;
    double complex *U=(double complex *)m_alloc2(n1*16,sizeof(double complex),"solve.c U");
    double complex *dU=(double complex *)m_alloc2(n1*16,sizeof(double complex),"solve.c dU");
    double complex *E=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c E");
    double complex *dE=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c dE");
    double complex *H=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c H");
    double complex *dH=(double complex *)m_alloc2(n1*12,sizeof(double complex),"solve.c dH");
    for(size_t s=0;s<n1;s++) for(int j=0;j<4;j++){
      for(int l=0;l<4;l++){ U[(s*4+j)*4+l]=sb->U[s][j][l]; dU[(s*4+j)*4+l]=sb->dU[s][j][l]; }
      for(int l=0;l<3;l++){
        E[(s*4+j)*3+l]=sb->E[s][j][l]; dE[(s*4+j)*3+l]=sb->dE[s][j][l];
        H[(s*4+j)*3+l]=sb->H[s][j][l]; dH[(s*4+j)*3+l]=sb->dH[s][j][l];
      }
    }
    if(gb_bv_upload(o,d,U,dU,E,dE,H,dH)) gb_die("solve.c, gb_bv_upload()");
    free(U); free(dU); free(E); free(dE); free(H); free(dH);
  }
  gb_dev_set_flags(md,GB_F_BV,0);
}

static void gb_solve_coefficient_mEMP(int flg,DOMD *md)
{
  time_t ms,me;
  if(flg==1){ MSG("  solve mEMP boundary value ");  }
  time(&ms);
  if(gb_solve_mEMP(gb_dev(md))) gb_die("mo_solve.c, solve_coefficient_mEMP()");
  time(&me);
  if(flg==1) MSG("finished. Elapsed time : %5g (sec)\n",difftime(me,ms));
}

static void gb_solve_coefficient_EH(int flg,DOMD *md)
{
  time_t ms,me;
  if(flg==1){ MSG("  solve EH boundary value   ");  }
  time(&ms);
  if(gb_solve_EH(gb_dev(md))) gb_die("mo_solve.c, solve_coefficient_EH()");
  time(&me);
  if(flg==1) MSG("finished. Elapsed time : %5g (sec)\n",difftime(me,ms));
}

/* One phase of an iteration for every object at once, one host thread per
 * object (at most 16 at a time).  The iteration is a Jacobi sweep: every
 * object's incident field takes the other objects' boundary values of the
 * previous sweep (add_scattered_mEMP, mo_solve.c:296-349, reads them before
 * any object solves again), so within a phase the objects are independent;
 * each object's kernels run on its own stream, and the results are those of
 * the sequential order bit for bit.  phase 0: the incident field plus the
 * other objects' scattered potentials; 1: the boundary values; 2: E, H. */
typedef struct { MOBJ *mo; int phase,dev; int *next; pthread_mutex_t *mu; } gb_phase_pool;

static void gb_phase_object(MOBJ *mo,int m,int phase)
{
  if(phase==0){
    /* object m alone is written: its incident field is reset and receives
     * the other objects' scattered potentials in object order (their
     * boundary values are not written in this phase) */
    if(gb_reset_incident(gb_dev(&mo->md[m]))) gb_die("mo_solve.c, reset_incident_bd()");
    for(int d=0;d<mo->N;d++){
      if(d==m) continue;
      if(gb_add_scattered(gb_dev(&mo->md[m]),gb_dev(&mo->md[d]),PREC_DEF)) gb_die("mo_solve.c, add_scattered_mEMP()");
    }
  }
  else if(phase==1){ if(gb_solve_mEMP(gb_dev(&mo->md[m]))) gb_die("mo_solve.c, solve_coefficient_mEMP()"); }
  else { if(gb_solve_EH(gb_dev(&mo->md[m]))) gb_die("mo_solve.c, solve_coefficient_EH()"); }
}

static void *gb_phase_worker(void *p)
{
  gb_phase_pool *q=(gb_phase_pool *)p;
  if(gb_use_device(q->dev)) gb_die("mo_solve.c, worker device");
  for(;;){
    pthread_mutex_lock(q->mu);
    int m=(*q->next)++;
    pthread_mutex_unlock(q->mu);
    if(m>=q->mo->N) break;
    gb_phase_object(q->mo,m,q->phase);
  }
  return NULL;
}

static void gb_phase_all(MOBJ *mo,int phase)
{
  int nt=mo->N<16?mo->N:16,next=0;
  pthread_mutex_t mu=PTHREAD_MUTEX_INITIALIZER;
  gb_phase_pool q={mo,phase,gb_current_device(),&next,&mu};
  pthread_t th[16];
  int started=0;
  for(int i=0;i<nt;i++){
    if(pthread_create(&th[i],NULL,gb_phase_worker,&q)) break;
    started++;
  }
  if(started==0) gb_phase_worker(&q);  /* no thread available: here */
  for(int i=0;i<started;i++) pthread_join(th[i],NULL);
}

static double gb_ccd_f(MOBJ *mo)
{
  double us=0.0,ps=0.0,sc=0.0,out[3];
  for(int i=0;i<mo->N;i++){
    if(gb_ccd_sums(gb_dev(&mo->md[i]),out)) gb_die("mo_solve.c, ccd_f()");
    us+=out[0]; ps+=out[1]; sc+=out[2];
  }
  return (us>ps)?us/sc:ps/sc;
}

void mo_solve_bv(MOBJ *mo)
{
  time_t start,end,ms,me;
  int iter,itermax=ITER_MAX;
  for(int m=0;m<mo->N;m++){
    gb_cmat_read(&mo->md[m],1);
    gb_upload_incident(&mo->md[m]);
  }
  g_last_iter=1;
  g_last_cc=0.0;
  if(mo->N==1){
    MSG("\nsingle object\n");
    gb_solve_coefficient_mEMP(1,&mo->md[0]);
    gb_solve_coefficient_EH(1,&mo->md[0]);
  }
  else {
    MSG("\ninitialize boundary value\n");
    for(int m=0;m<mo->N;m++){
      MSG("object % 2d\n",m);
      gb_solve_coefficient_mEMP(1,&mo->md[m]);
    }
    MSG("\nthe first iterative operation\n");
    time(&start);
    for(int m=0;m<mo->N;m++) if(gb_reset_incident(gb_dev(&mo->md[m]))) gb_die("mo_solve.c, reset_incident_bd()");
    for(int m=0;m<mo->N;m++){
      MSG("object % 2d\n",m);
      MSG("  add scattered field       "); 
      time(&ms);
      for(int d=0;d<mo->N;d++){
        if(d==m) continue;
        if(gb_add_scattered(gb_dev(&mo->md[m]),gb_dev(&mo->md[d]),PREC_DEF)) gb_die("mo_solve.c, add_scattered_mEMP()");
      }
      time(&me);
      MSG("finished. Elapsed time : %5g (sec)\n",difftime(me,ms));
    }
    for(int m=0;m<mo->N;m++){
      MSG("object % 2d\n",m);
      gb_solve_coefficient_mEMP(1,&mo->md[m]);
    }
    time(&end);
    MSG("Estimated time per one iteration : %5g (sec)\n\n",difftime(end,start));
    MSG("iterative operation start. convergence criterion cc < %g and count > %d\n",CCD,ITER_MIN);
    time(&start);
    for(iter=2;iter<itermax;iter++){
      MSG("count =% 3d",iter);
      gb_phase_all(mo,0);
      gb_phase_all(mo,1);
      double cc=gb_ccd_f(mo);
      g_last_iter=iter;
      g_last_cc=cc;
      MSG(", cc = %g\n",cc);
      
      if(cc<CCD && iter>ITER_MIN) break;
    }
    if(iter==itermax) MSG("The maximum number of iterations has been reached (The result has not converged).\n");
    gb_phase_all(mo,2);
    time(&end);
    MSG("finished. Elapsed time : %5g (sec)\n",difftime(end,start));
  }
  for(int m=0;m<mo->N;m++){
    gb_bv_to_host(&mo->md[m]);
    gb_dev_set_flags(&mo->md[m],GB_F_BV,0);
  }
}
