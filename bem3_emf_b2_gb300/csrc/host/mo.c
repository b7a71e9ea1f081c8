/*
 * mo.c -- multiple objects: object-settings input, .obj and .dat files,
 * incident field at the collocation nodes (reference d3b2_src/mo_setup.c).
 */
#include "gb_host.h"

static void gb_rfail(const char *where,const char *what)
{
  printf("%s, failed to read the %s. exit...\n",where,what);
  exit(1);
}
static void gb_fread(void *p,size_t sz,size_t n,FILE *fp,const char *what)
{
  if(n>0 && fread(p,sz,n,fp)!=n) gb_rfail("mo.c",what);
}
static void gb_fwr(const void *p,size_t sz,size_t n,FILE *fp)
{
  if(n>0 && fwrite(p,sz,n,fp)!=n){ printf("mo.c, failed to write the data file. Exit...\n"); exit(1); }
}

void gb_mo_malloc(MOBJ *mo)
{
  int N=mo->N;
  mo->md=(DOMD *)m_alloc2(N,sizeof(DOMD),"mo.c md");
  mo->mod_fn=(char **)m_alloc2(N,sizeof(char *),"mo.c mod_fn");
  mo->rs=(double **)m_alloc2(N,sizeof(double *),"mo.c rs");
  for(int i=0;i<N;i++){
    mo->mod_fn[i]=(char *)m_alloc2(FNLGTH,sizeof(char),"mo.c mod_fn[i]");
    mo->rs[i]=(double *)m_alloc2(3,sizeof(double),"mo.c rs[i]");
  }
}

/* raw Bobj plus its beam arrays; the stored pointers are replaced */
static void gb_read_beam(FILE *fp,Bobj *mw)
{
  gb_mfb_read(fp,mw);
}

/* mesh part common to .obj and .dat (reference dat_read2 / mo_dat_read) */
static void gb_read_mesh_part(FILE *fp,DOMD *md)
{
  BOUD *bd=&md->bd;
  gb_fread(md->med_fn,1,128,fp,"med_fn");
  gb_fread(md->msh_fn,1,128,fp,"msh_fn");
  gb_fread(md->rv,sizeof(double),3,fp,"rv");
  gb_fread(&md->th,sizeof(double),1,fp,"th");
  gb_fread(md->tv,sizeof(double),3,fp,"tv");
  gb_fread(&md->MN,sizeof(int),1,fp,"MN");
  md->n=(double complex *)m_alloc2(md->MN+1,sizeof(double complex),"mo.c n");
  md->kn=(double complex *)m_alloc2(md->MN+1,sizeof(double complex),"mo.c kn");
  gb_fread(md->n,sizeof(double complex),md->MN+1,fp,"n");
  gb_fread(md->kn,sizeof(double complex),md->MN+1,fp,"kn");
  gb_read_beam(fp,&md->mw);
  gb_fread(&bd->Nn,sizeof(int),1,fp,"Nn");
  gb_fread(&bd->Ne,sizeof(int),1,fp,"Ne");
  gb_malloc_node(bd);
  gb_malloc_elem(bd);
  for(int i=0;i<=bd->Nn;i++) gb_fread(bd->rn[i],sizeof(double),3,fp,"rn");
  for(int i=0;i<=bd->Ne;i++) gb_fread(bd->ed[i],sizeof(int),4,fp,"ed");
  gb_fread(&bd->NN,sizeof(int),1,fp,"NN");
  for(int i=0;i<=bd->Ne;i++) gb_fread(bd->eni[i],sizeof(int),4,fp,"eni");
  gb_fread(bd->md,sizeof(int),bd->Ne+1,fp,"md");
  gb_fread(bd->sd,sizeof(int),bd->Ne+1,fp,"sd");
  gb_fread(bd->gd,sizeof(int),bd->Ne+1,fp,"gd");
  for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) gb_fread(bd->ren[i][j],sizeof(double),3,fp,"ren");
  for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) gb_fread(bd->wen[i][j],sizeof(double),3,fp,"wen");
  gb_init_elem_const(bd);
  gb_malloc_sub_domain(md);
}

static void gb_dat_read2(char *fname,DOMD *md)
{
  FILE *fp=fopen(fname,"rb");
  if(fp==NULL){ printf("dat_read(), Failed to open the %s file.\n",fname); exit(1); }
  memset(md,0,sizeof(DOMD));
  gb_read_mesh_part(fp,md);
  for(int d=0;d<=md->MN;d++){
    int tmp;
    gb_fread(&tmp,sizeof(int),1,fp,"sub domain Ne");
    gb_fread(md->bd.sb[d].sid,sizeof(int),md->bd.sb[d].Ne+1,fp,"sid");
  }
  md->cm.MN=md->MN;
  md->cm.na=8*(size_t)md->bd.NN;
  md->cm.nn=(size_t)md->bd.NN;
  gb_initalize_cmd2(&md->cm);
  for(int i=0;i<=md->MN;i++){
    gb_fread(md->cm.tgfn[i],1,128,fp,"G file name");
    gb_fread(md->cm.thfn[i],1,128,fp,"H file name");
    gb_fread(md->cm.tdgfn[i],1,128,fp,"dG file name");
    gb_fread(md->cm.tdhfn[i],1,128,fp,"dH file name");
    gb_fread(md->cm.tdffn[i],1,128,fp,"dF file name");
  }
  gb_fread(md->cm.lupfn,1,128,fp,"invA file name");
  fclose(fp);
}

static void gb_renew_beam_data(DOMD *md)
{
  double l0=md->mw.lambda_0,n0=md->mw.n_0;
  free_mfb(&md->mw);
  init_mfb(&md->mw);
  read_data_mfb(&md->mw);
  setup_mfb(&md->mw);
  if(l0!=md->mw.lambda_0 || n0!=md->mw.n_0){
    printf("mo.c, renew_beam_data(), wave number check error!\n");
    printf("multi wave old data lambda0=%g, n_0=%g\n",l0,n0);
    printf("multi wave new data lambda0=%g, n_0=%g\n",md->mw.lambda_0,md->mw.n_0);
    printf("Exit...\n");
    exit(1);
  }
}

/* collocation points, normals and the incident potential (A = E_incident,
 * phi = 0) with its normal derivative at the exterior nodes
 * (reference init_boundary_data_u2, mo_setup.c:704-758) */
void gb_init_boundary_data_u2(DOMD *md)
{
  BOUD *bd=&md->bd;
  /* collocation points and normals; the exterior ones are gathered for one
   * batched evaluation of the incident field */
  double *xr=(double *)m_alloc2((size_t)4*bd->Ne+1,3*sizeof(double),"mo.c xr");
  double *xw=(double *)m_alloc2((size_t)4*bd->Ne+1,3*sizeof(double),"mo.c xw");
  int *xi=(int *)m_alloc2((size_t)4*bd->Ne+1,sizeof(int),"mo.c xi");
  int nx=0;
  for(int i=1;i<=bd->Ne;i++){
    double cr[3][4],cw[3][3],r[3],w[3];
    for(int l=0;l<3;l++){ for(int m=0;m<4;m++) cr[l][m]=bd->cr[i][l][m]; for(int m=0;m<3;m++) cw[l][m]=bd->cw[i][l][m]; }
    for(int j=0;j<4;j++){
      if(bd->ed[i][3]==0) lit_rw_zeta_eta(r,w,bd->zt_34[j],bd->et_34[j],cr,cw);
      else bil_rw_zeta_eta(r,w,bd->zt_44[j],bd->et_44[j],cr,cw);
      for(int l=0;l<3;l++){ bd->ren[i][j][l]=r[l]; bd->wen[i][j][l]=w[l]; }
      if(bd->md[i]==0){
        vuni_d(w);
        for(int l=0;l<3;l++){ xr[3*nx+l]=r[l]; xw[3*nx+l]=w[l]; }
        xi[nx++]=4*i+j;
      }
    }
  }
  if(nx>0){
    double complex *f=(double complex *)m_alloc2((size_t)12*nx,sizeof(double complex),"mo.c f");
    double complex *e=f,*h=f+(size_t)3*nx,*de=f+(size_t)6*nx,*dh=f+(size_t)9*nx;
    calc_mfb_EH_dv_points(&md->mw,nx,xr,xw,e,h,de,dh);
    for(int k=0;k<nx;k++){
      int i=xi[k]/4,j=xi[k]%4;
      for(int l=0;l<3;l++){ bd->Ui[i][j][l]=e[3*k+l]; bd->dUi[i][j][l]=de[3*k+l]; }
      bd->Ui[i][j][3]=0.0;
      bd->dUi[i][j][3]=0.0;
      for(int l=0;l<4;l++){
        bd->Ui0[i][j][l]=bd->Ui[i][j][l];
        bd->dUi0[i][j][l]=bd->dUi[i][j][l];
        bd->Uip[i][j][l]=bd->Ui[i][j][l];
      }
    }
    free(f);
  }
  free(xr); free(xw); free(xi);
}

void mo_initialize(int argc,char **argv,MOBJ *mo)
{
  FILE *fp;
  char tmp[FNLGTH];
  int n,flg;
  if(argc!=3){
    printf("This program needs command line argument as follows.\n");
    printf("%s object_setting_file output_data_file_name\n",argv[0]);
    exit(0);
  }
  if((fp=fopen(argv[1],"rt"))==NULL){ printf("mo_read_data(),Can not open the %s file.\n",argv[1]); exit(1); }
  if(fgets(tmp,FNLGTH,fp)==NULL) gb_rfail("mo.c, mo_initialize()","line");
  if(fscanf(fp,"%d %d\n",&n,&flg)!=2) gb_rfail("mo.c, mo_initialize()","number of objects and incident field renew flag");
  mo->N=n;
  gb_mo_malloc(mo);
  if(fgets(tmp,256,fp)==NULL) gb_rfail("mo.c, mo_initialize()","line");
  for(int i=0;i<mo->N;i++){
    if(fscanf(fp,"%255s %lf %lf %lf",mo->mod_fn[i],&mo->rs[i][0],&mo->rs[i][1],&mo->rs[i][2])!=4)
      gb_rfail("mo.c, mo_initialize()","mod_fn,rs");
    gb_dat_read2(mo->mod_fn[i],&mo->md[i]);
    if(flg==1) gb_renew_beam_data(&mo->md[i]);
    gb_rotation_translation_obj(mo->md[i].rv,0.0,mo->rs[i],&mo->md[i]);
    gb_init_elem_const(&mo->md[i].bd);
    gb_init_boundary_data2(&mo->md[i]);
    gb_init_boundary_data_u2(&mo->md[i]);
  }
  fclose(fp);
}

static void gb_mo_print(MOBJ *mo,int mksa)
{
  printf("-- multi_fbeam --\n");
  if(mksa) print_data_mfb_mksa(&mo->md[0].mw); else print_data_mfb(&mo->md[0].mw);
  for(int i=0;i<mo->N;i++){
    DOMD *md=&mo->md[i];
    printf("********** object %d **********\n",i);
    printf("data file name                : %s\n",mo->mod_fn[i]);
    if(mksa) printf("additional translation vector [m]: (% 8.7g,% 8.7g,% 8.7g)\n",OSUtoMKSA_length(mo->rs[i][0]),OSUtoMKSA_length(mo->rs[i][1]),OSUtoMKSA_length(mo->rs[i][2]));
    else printf("additional translation vector : (% 8.7g,% 8.7g,% 8.7g)\n",mo->rs[i][0],mo->rs[i][1],mo->rs[i][2]);
    gb_print_medium_data(md);
    gb_print_mesh_data(md);
    if(md->th!=0.0 || vabs_d(md->tv)!=0.0){
      printf("-- rotation and translation settings --\n");
      if(md->th!=0.0){
        printf("vector defining rotation axis :(% 8.7g,% 8.7g,% 8.7g)\n",md->rv[0],md->rv[1],md->rv[2]);
        printf("rotation angle           [rad]: % 8.7g\n",md->th);
      }
      if(vabs_d(md->tv)!=0.0) printf("translation vector            :(% 8.7g,% 8.7g,% 8.7g)\n",md->tv[0],md->tv[1],md->tv[2]);
    }
  }
  printf("\n");
}
void mo_print_data(MOBJ *mo){ gb_mo_print(mo,0); }
void mo_print_data_mksa(MOBJ *mo){ gb_mo_print(mo,1); }

void mo_finalize(MOBJ *mo)
{
  for(int i=0;i<mo->N;i++){
    gb_finalize_cmd2(&mo->md[i].cm);
    finalize_domd2(&mo->md[i]);
    free(mo->mod_fn[i]);
    free(mo->rs[i]);
  }
  free(mo->md);
  free(mo->mod_fn);
  free(mo->rs);
}

/* .dat result file (reference mo_dat_write, mo_setup.c:147-203) */
void mo_dat_write(char *fname,MOBJ *mo)
{
  FILE *fp=fopen(fname,"wb");
  if(fp==NULL){ printf("mo_dat_write(), Failed to create the %s file.\n",fname); exit(1); }
  gb_fwr(&mo->N,sizeof(int),1,fp);
  for(int m=0;m<mo->N;m++){
    DOMD *md=&mo->md[m];
    BOUD *bd=&md->bd;
    char name[FNLGTH];
    memset(name,0,FNLGTH);
    snprintf(name,FNLGTH,"%s",mo->mod_fn[m]);
    gb_fwr(name,1,FNLGTH,fp);
    gb_fwr(mo->rs[m],sizeof(double),3,fp);
    gb_fwr(md->med_fn,1,128,fp);
    gb_fwr(md->msh_fn,1,128,fp);
    gb_fwr(md->rv,sizeof(double),3,fp);
    gb_fwr(&md->th,sizeof(double),1,fp);
    gb_fwr(md->tv,sizeof(double),3,fp);
    gb_fwr(&md->MN,sizeof(int),1,fp);
    gb_fwr(md->n,sizeof(double complex),md->MN+1,fp);
    gb_fwr(md->kn,sizeof(double complex),md->MN+1,fp);
    gb_mfb_write(fp,&md->mw);
    gb_fwr(&bd->Nn,sizeof(int),1,fp);
    gb_fwr(&bd->Ne,sizeof(int),1,fp);
    for(int i=0;i<=bd->Nn;i++) gb_fwr(bd->rn[i],sizeof(double),3,fp);
    for(int i=0;i<=bd->Ne;i++) gb_fwr(bd->ed[i],sizeof(int),4,fp);
    gb_fwr(&bd->NN,sizeof(int),1,fp);
    for(int i=0;i<=bd->Ne;i++) gb_fwr(bd->eni[i],sizeof(int),4,fp);
    gb_fwr(bd->md,sizeof(int),bd->Ne+1,fp);
    gb_fwr(bd->sd,sizeof(int),bd->Ne+1,fp);
    gb_fwr(bd->gd,sizeof(int),bd->Ne+1,fp);
    for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) gb_fwr(bd->ren[i][j],sizeof(double),3,fp);
    for(int i=0;i<=bd->Ne;i++) for(int j=0;j<4;j++) gb_fwr(bd->wen[i][j],sizeof(double),3,fp);
    for(int d=0;d<=md->MN;d++){
      SUBD *sb=&bd->sb[d];
      gb_fwr(&sb->Ne,sizeof(int),1,fp);
      gb_fwr(sb->sid,sizeof(int),sb->Ne+1,fp);
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fwr(sb->U[i][j],sizeof(double complex),4,fp);
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fwr(sb->dU[i][j],sizeof(double complex),4,fp);
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fwr(sb->E[i][j],sizeof(double complex),3,fp);
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fwr(sb->dE[i][j],sizeof(double complex),3,fp);
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fwr(sb->H[i][j],sizeof(double complex),3,fp);
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fwr(sb->dH[i][j],sizeof(double complex),3,fp);
    }
  }
  fclose(fp);
}

void mo_dat_read(char *fname,MOBJ *mo)
{
  FILE *fp=fopen(fname,"rb");
  if(fp==NULL){ printf("mo_dat_read(), Failed to open the %s file.\n",fname); exit(1); }
  gb_fread(&mo->N,sizeof(int),1,fp,"N");
  gb_mo_malloc(mo);
  for(int m=0;m<mo->N;m++){
    DOMD *md=&mo->md[m];
    memset(md,0,sizeof(DOMD));
    gb_fread(mo->mod_fn[m],1,FNLGTH,fp,"mod_fn");
    gb_fread(mo->rs[m],sizeof(double),3,fp,"rs");
    gb_read_mesh_part(fp,md);
    for(int d=0;d<=md->MN;d++){
      SUBD *sb=&md->bd.sb[d];
      int tmp;
      gb_fread(&tmp,sizeof(int),1,fp,"sub domain Ne");
      gb_fread(sb->sid,sizeof(int),sb->Ne+1,fp,"sid");
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fread(sb->U[i][j],sizeof(double complex),4,fp,"U");
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fread(sb->dU[i][j],sizeof(double complex),4,fp,"dU");
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fread(sb->E[i][j],sizeof(double complex),3,fp,"E");
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fread(sb->dE[i][j],sizeof(double complex),3,fp,"dE");
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fread(sb->H[i][j],sizeof(double complex),3,fp,"H");
      for(int i=0;i<=sb->Ne;i++) for(int j=0;j<4;j++) gb_fread(sb->dH[i][j],sizeof(double complex),3,fp,"dH");
    }
    md->cm.MN=md->MN;
    md->cm.na=8*(size_t)md->bd.NN;
    gb_initalize_cmd2(&md->cm);
  }
  fclose(fp);
}

void mo_output_node_particles(char *fname,MOBJ *mo)
{
  char fo[256]={0},tf[200]={0};
  size_t s1=strlen(fname);
  if(s1>200){ printf("mo_output_node_particles(), file name is too long. exit...\n"); exit(1); }
  snprintf(fo,256,"%s",fname);
  char *sd=strrchr(fo,'.');
  if(sd!=NULL){
    size_t s2=strlen(sd);
    strncpy(tf,fname,s1-s2);
    snprintf(fo,256,"%s.particles",tf);
  }
  FILE *fp=fopen(fo,"wt");
  if(fp==NULL){ printf("Can not open the %s file.\n",fo); exit(1); }
  fprintf(fp,"# x y z object_id\n");
  for(int oid=0;oid<mo->N;oid++)
    for(int i=1;i<=mo->md[oid].bd.Ne;i++)
      for(int j=0;j<4;j++)
        fprintf(fp,"%15.14e %15.14e %15.14e %d\n",mo->md[oid].bd.ren[i][j][0],mo->md[oid].bd.ren[i][j][1],mo->md[oid].bd.ren[i][j][2],oid);
  fclose(fp);
}
