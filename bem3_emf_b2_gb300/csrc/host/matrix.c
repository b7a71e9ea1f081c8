/*
 * matrix.c -- create_matrix (reference solve_bieq2.c:10-47 and 439-502).
 *
 * The coefficient matrices of every domain are assembled on the GPU, the
 * coupled matrix A is built and inverted on the GPU, and everything is
 * written in the reference's formats: headerless row-major .cmat files and
 * the .obj object file that d3b2_bv_solver reads.
 */
#include "gb_host.h"

void gb_initalize_cmd2(CMD *cm)
{
  int MN=cm->MN;
  cm->tgfn=(char **)m_alloc2(MN+1,sizeof(char *),"matrix.c tgfn");
  cm->thfn=(char **)m_alloc2(MN+1,sizeof(char *),"matrix.c thfn");
  cm->tdgfn=(char **)m_alloc2(MN+1,sizeof(char *),"matrix.c tdgfn");
  cm->tdhfn=(char **)m_alloc2(MN+1,sizeof(char *),"matrix.c tdhfn");
  cm->tdffn=(char **)m_alloc2(MN+1,sizeof(char *),"matrix.c tdffn");
  for(int i=0;i<=MN;i++){
    cm->tgfn[i]=(char *)m_alloc2(128,1,"matrix.c"); snprintf(cm->tgfn[i],128,"tmpG_%05d.cmat",i);
    cm->thfn[i]=(char *)m_alloc2(128,1,"matrix.c"); snprintf(cm->thfn[i],128,"tmpH_%05d.cmat",i);
    cm->tdgfn[i]=(char *)m_alloc2(128,1,"matrix.c"); snprintf(cm->tdgfn[i],128,"tmpdG_%05d.cmat",i);
    cm->tdhfn[i]=(char *)m_alloc2(128,1,"matrix.c"); snprintf(cm->tdhfn[i],128,"tmpdH_%05d.cmat",i);
    cm->tdffn[i]=(char *)m_alloc2(128,1,"matrix.c"); snprintf(cm->tdffn[i],128,"tmpdF_%05d.cmat",i);
  }
  cm->lupfn=(char *)m_alloc2(128,1,"matrix.c"); snprintf(cm->lupfn,128,"tmpinvA.cmat");
  /* names of the reference's CSR scratch files; nothing is written to them here */
  cm->aval=(char *)m_alloc2(16,1,"matrix.c"); snprintf(cm->aval,16,"tmpAval.dat");
  cm->aptr=(char *)m_alloc2(16,1,"matrix.c"); snprintf(cm->aptr,16,"tmpAprt.dat");
  cm->aidx=(char *)m_alloc2(16,1,"matrix.c"); snprintf(cm->aidx,16,"tmpAidx.dat");
  cm->b=(char *)m_alloc2(16,1,"matrix.c"); snprintf(cm->b,16,"tmpB.dat");
}

void gb_finalize_cmd2(CMD *cm)
{
  if(cm->tgfn==NULL) return;
  for(int i=0;i<=cm->MN;i++){ free(cm->tgfn[i]); free(cm->thfn[i]); free(cm->tdgfn[i]); free(cm->tdhfn[i]); free(cm->tdffn[i]); }
  free(cm->tgfn); free(cm->thfn); free(cm->tdgfn); free(cm->tdhfn); free(cm->tdffn);
  free(cm->lupfn);
  free(cm->aval); free(cm->aptr); free(cm->aidx); free(cm->b);
  cm->tgfn=NULL;
  cm->MN=0; cm->nn=0; cm->na=0; cm->nnz=0;
}

static void gb_fwrite(const void *p,size_t sz,size_t n,FILE *fp,const char *fn)
{
  if(n>0 && fwrite(p,sz,n,fp)!=n){ printf("matrix.c, failed to write %s. Exit...\n",fn); exit(1); }
}

static FILE *gb_fopen_w(const char *fn)
{
  FILE *fp=fopen(fn,"wb");
  if(fp==NULL){ printf("matrix.c, Failed to create %s file.\n",fn); exit(1); }
  return fp;
}

/* G, H, dG, dH, dF of every domain: assembled on the GPU, written to the
 * temporary .cmat files named in cm */
static void gb_create_cmatrix(CMD *cm,DOMD *md)
{
  gb_obj *o=gb_dev(md);
  for(int d=0;d<=md->MN;d++){
    size_t N=4*(size_t)md->bd.sb[d].Ne;
    if(gb_assemble(o,d,cm->type)) gb_die("matrix.c, create_cmatrix()");
    double complex *buf=(double complex *)m_alloc2(2*N*N+1,sizeof(double complex),"matrix.c buf");
    double *df=(double *)m_alloc2(3*N+1,sizeof(double),"matrix.c df");
    FILE *fp;
    if(gb_cmatrix_download(o,d,buf,NULL,NULL,NULL,NULL)) gb_die("matrix.c G");
    fp=gb_fopen_w(cm->tgfn[d]); gb_fwrite(buf,sizeof(double complex),N*N,fp,cm->tgfn[d]); fclose(fp);
    if(gb_cmatrix_download(o,d,NULL,buf,NULL,NULL,NULL)) gb_die("matrix.c H");
    fp=gb_fopen_w(cm->thfn[d]); gb_fwrite(buf,sizeof(double complex),N*N,fp,cm->thfn[d]); fclose(fp);
    if(gb_cmatrix_download(o,d,NULL,NULL,buf,NULL,NULL)) gb_die("matrix.c dG");
    fp=gb_fopen_w(cm->tdgfn[d]); gb_fwrite(buf,sizeof(double complex),2*N*N,fp,cm->tdgfn[d]); fclose(fp);
    if(gb_cmatrix_download(o,d,NULL,NULL,NULL,buf,NULL)) gb_die("matrix.c dH");
    fp=gb_fopen_w(cm->tdhfn[d]); gb_fwrite(buf,sizeof(double complex),2*N*N,fp,cm->tdhfn[d]); fclose(fp);
    if(gb_cmatrix_download(o,d,NULL,NULL,NULL,NULL,df)) gb_die("matrix.c dF");
    fp=gb_fopen_w(cm->tdffn[d]); gb_fwrite(df,sizeof(double),3*N,fp,cm->tdffn[d]); fclose(fp);
    free(buf); free(df);
  }
}

/* block factors in place of the dense inverse? (GB_CMAT_FORMAT = block or
 * dense; by default dense, as the reference, unless the inverse would take
 * more than half the device memory) */
static int gb_use_block(DOMD *md,gb_obj *o)
{
  if(!gb_obj_one_interface(o)) return 0;
  const char *e=getenv("GB_CMAT_FORMAT");
  if(e && strcmp(e,"block")==0) return 1;
  if(e && strcmp(e,"dense")==0) return 0;
  size_t fr=0,tot=0;
  if(gb_device_memory(&fr,&tot)) return 0;
  size_t na=8*(size_t)md->bd.NN;
  return na*na*sizeof(double complex)>tot/2;
}

static void gb_write_block(CMD *cm,DOMD *md,gb_obj *o)
{
  if(gb_factor_fp64(o)) gb_die("matrix.c, block factors");
  size_t nn=(size_t)md->bd.NN;
  snprintf(cm->lupfn,128,"tmpblk.cmat");
  FILE *fp=gb_fopen_w(cm->lupfn);
  unsigned char hdr[GB_BLK_HEADER];
  memset(hdr,0,sizeof(hdr));
  memcpy(hdr,GB_BLK_MAGIC,8);
  int meta[4]={GB_BLK_VERSION,(int)nn,5,(int)sizeof(double complex)};
  memcpy(hdr+8,meta,sizeof(meta));
  gb_fwrite(hdr,1,GB_BLK_HEADER,fp,cm->lupfn);
  double complex *buf=(double complex *)m_alloc2(nn*nn,sizeof(double complex),"matrix.c blk");
  for(int i=0;i<5;i++){
    void *p[5]={NULL,NULL,NULL,NULL,NULL};
    p[i]=buf;
    if(gb_block_factors_download(o,p[0],p[1],p[2],p[3],p[4])) gb_die("matrix.c, block factors");
    gb_fwrite(buf,sizeof(double complex),nn*nn,fp,cm->lupfn);
  }
  free(buf);
  fclose(fp);
}

static void gb_lu_dec_A(CMD *cm,DOMD *md)
{
  gb_obj *o=gb_dev(md);
  if(gb_use_block(md,o)){ gb_write_block(cm,md,o); return; }
  if(gb_invA_compute(o)) gb_die("matrix.c, lu_dec_A()");
  double complex *buf=(double complex *)m_alloc2(cm->na*cm->na,sizeof(double complex),"matrix.c invA");
  if(gb_invA_download(o,buf)) gb_die("matrix.c, lu_dec_A()");
  FILE *fp=gb_fopen_w(cm->lupfn);
  gb_fwrite(buf,sizeof(double complex),cm->na*cm->na,fp,cm->lupfn);
  fclose(fp);
  free(buf);
}

/* .obj object file (reference dat_write2, solve_bieq2.c:439-502); the
 * temporary .cmat files are renamed to <prefix>_<name>, prefix being the
 * output name up to its first '.', and those names are recorded */
static void gb_dat_write2(char *fname,DOMD *md)
{
  FILE *fp=gb_fopen_w(fname);
  BOUD *bd=&md->bd;
  char pfn[128],tfn[256],rec[128];
  int i;
  gb_fwrite(md->med_fn,1,128,fp,fname);
  gb_fwrite(md->msh_fn,1,128,fp,fname);
  gb_fwrite(md->rv,sizeof(double),3,fp,fname);
  gb_fwrite(&md->th,sizeof(double),1,fp,fname);
  gb_fwrite(md->tv,sizeof(double),3,fp,fname);
  gb_fwrite(&md->MN,sizeof(int),1,fp,fname);
  gb_fwrite(md->n,sizeof(double complex),md->MN+1,fp,fname);
  gb_fwrite(md->kn,sizeof(double complex),md->MN+1,fp,fname);
  gb_mfb_write(fp,&md->mw);
  gb_fwrite(&bd->Nn,sizeof(int),1,fp,fname);
  gb_fwrite(&bd->Ne,sizeof(int),1,fp,fname);
  for(i=0;i<=bd->Nn;i++) gb_fwrite(bd->rn[i],sizeof(double),3,fp,fname);
  for(i=0;i<=bd->Ne;i++) gb_fwrite(bd->ed[i],sizeof(int),4,fp,fname);
  gb_fwrite(&bd->NN,sizeof(int),1,fp,fname);
  for(i=0;i<=bd->Ne;i++) gb_fwrite(bd->eni[i],sizeof(int),4,fp,fname);
  gb_fwrite(bd->md,sizeof(int),bd->Ne+1,fp,fname);
  gb_fwrite(bd->sd,sizeof(int),bd->Ne+1,fp,fname);
  gb_fwrite(bd->gd,sizeof(int),bd->Ne+1,fp,fname);
  for(i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) gb_fwrite(bd->ren[i][j],sizeof(double),3,fp,fname);
  for(i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) gb_fwrite(bd->wen[i][j],sizeof(double),3,fp,fname);
  for(int d=0;d<=md->MN;d++){
    gb_fwrite(&bd->sb[d].Ne,sizeof(int),1,fp,fname);
    gb_fwrite(bd->sb[d].sid,sizeof(int),bd->sb[d].Ne+1,fp,fname);
  }
  for(i=0;i<127 && fname[i]!='\0' && fname[i]!='.';i++) pfn[i]=fname[i];
  pfn[i]='\0';
  CMD *cm=&md->cm;
  char **lists[5]={cm->tgfn,cm->thfn,cm->tdgfn,cm->tdhfn,cm->tdffn};
  for(int d=0;d<=md->MN;d++){
    for(int l=0;l<5;l++){
      snprintf(tfn,256,"%s_%s",pfn,lists[l][d]+3);
      rename(lists[l][d],tfn);
      memset(rec,0,128); snprintf(rec,128,"%s",tfn);
      gb_fwrite(rec,1,128,fp,fname);
    }
  }
  snprintf(tfn,256,"%s_%s",pfn,cm->lupfn+3);
  rename(cm->lupfn,tfn);
  memset(rec,0,128); snprintf(rec,128,"%s",tfn);
  gb_fwrite(rec,1,128,fp,fname);
  fclose(fp);
}

void create_matrix(DOMD *md,char *ofn)
{
  time_t start,end,ms,me;
  printf("\ncreate matrix data \n");
  time(&start);
  printf("  coefficient matrix          "); fflush(stdout);
  time(&ms);
  md->cm.type=PREC_DEF;
  md->cm.MN=md->MN;
  gb_initalize_cmd2(&md->cm);
  gb_create_cmatrix(&md->cm,md);
  time(&me);
  printf("finished. Elapsed time : %5g (sec)\n",difftime(me,ms));
  printf("  inverse matrix              "); fflush(stdout);
  time(&ms);
  md->cm.nn=(size_t)md->bd.NN;
  md->cm.na=md->cm.nn*8;
  gb_lu_dec_A(&md->cm,md);
  time(&me);
  printf("finished. Elapsed time : %5g (sec)\n",difftime(me,ms));
  gb_dat_write2(ofn,md);
  gb_finalize_cmd2(&md->cm);
  time(&end);
  printf("Total elapsed time : %g (sec)\n",difftime(end,start));
}
