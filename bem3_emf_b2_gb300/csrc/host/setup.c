/*
 * setup.c -- one BEM object on the host: medium and Gmsh 2.2 mesh input,
 * element geometry coefficients, collocation nodes, sub-domain element lists
 * (reference d3b2_src/setup2.c) and the host-side element geometry helpers
 * (reference d3b1_elem.c:11-143, 556-711).  Arrays are 1-based in the element
 * index, as in the reference, because callers index them directly.
 */
#include "bem3_emf_b2.h"
#include "gb_host.h"

static void gb_fail(const char *where,const char *what)
{
  printf("%s, failed to read the %s. exit...\n",where,what);
  exit(1);
}

void gb_filename_chk(int argc,char **argv)
{
  if(argc!=4 && argc!=11){
    printf("This program needs command line arguments as follows.\n");
    printf("%s medium_datafile_name mesh_datafile_name output_datafile_name [rv_x rv_y rv_z theta tr_x tr_y tr_z ](optional)\n",argv[0]);
    printf("rv : vector defining rotation axis, theta : rotation angle ( using Rodrigues' rotation formula ), tr : translation vector\n");
    printf("Exit...\n");
    exit(0);
  }
}

/* medium file: two comment lines, MN, a comment line, then MN lines
 * "Re(n) Im(n)" for domains 1..MN (reference setup2.c:153-193) */
void gb_read_medium_data(char *fn,DOMD *md)
{
  FILE *fp=fopen(fn,"rt");
  char buf[256];
  int mn;
  if(fp==NULL){ printf("Can not open the '%s' file. Exit...\n",fn); exit(1); }
  snprintf(md->med_fn,128,"%s",fn);
  if(fgets(buf,256,fp)==NULL || fgets(buf,256,fp)==NULL) gb_fail("setup.c, read_medium_data()","line");
  if(fscanf(fp,"%d\n",&mn)!=1) gb_fail("setup.c, read_medium_data()","MN");
  md->MN=mn;
  md->n=(double complex *)m_alloc2(mn+1,sizeof(double complex),"setup.c, n");
  md->kn=(double complex *)m_alloc2(mn+1,sizeof(double complex),"setup.c, kn");
  if(fgets(buf,256,fp)==NULL) gb_fail("setup.c, read_medium_data()","line");
  for(int i=1;i<=mn;i++){
    double re,im;
    if(fscanf(fp,"%lf",&re)!=1) gb_fail("setup.c, read_medium_data()","real(n)");
    if(fscanf(fp,"%lf",&im)!=1) gb_fail("setup.c, read_medium_data()","imag(n)");
    md->n[i]=re+im*I;
  }
  fclose(fp);
}

void gb_malloc_node(BOUD *bd)
{
  bd->rn=(double **)m_alloc2(bd->Nn+1,sizeof(double *),"setup.c, rn");
  for(int i=0;i<=bd->Nn;i++) bd->rn[i]=(double *)m_alloc2(3,sizeof(double),"setup.c, rn[i]");
}

void gb_mfree_node(BOUD *bd)
{
  for(int i=0;i<=bd->Nn;i++) free(bd->rn[i]);
  free(bd->rn);
  bd->Nn=0;
}

static double complex ***gb_alloc_c3(int n,int m,int l)
{
  double complex ***p=(double complex ***)m_alloc2(n,sizeof(double complex **),"setup.c, c3");
  for(int i=0;i<n;i++){
    p[i]=(double complex **)m_alloc2(m,sizeof(double complex *),"setup.c, c3[i]");
    for(int j=0;j<m;j++) p[i][j]=(double complex *)m_alloc2(l,sizeof(double complex),"setup.c, c3[i][j]");
  }
  return p;
}
static double ***gb_alloc_d3(int n,int m,int l)
{
  double ***p=(double ***)m_alloc2(n,sizeof(double **),"setup.c, d3");
  for(int i=0;i<n;i++){
    p[i]=(double **)m_alloc2(m,sizeof(double *),"setup.c, d3[i]");
    for(int j=0;j<m;j++) p[i][j]=(double *)m_alloc2(l,sizeof(double),"setup.c, d3[i][j]");
  }
  return p;
}
static void gb_free_c3(double complex ***p,int n,int m)
{
  for(int i=0;i<n;i++){ for(int j=0;j<m;j++) free(p[i][j]); free(p[i]); }
  free(p);
}
static void gb_free_d3(double ***p,int n,int m)
{
  for(int i=0;i<n;i++){ for(int j=0;j<m;j++) free(p[i][j]); free(p[i]); }
  free(p);
}

void gb_malloc_elem(BOUD *bd)
{
  int n=bd->Ne+1;
  bd->ed=(int **)m_alloc2(n,sizeof(int *),"setup.c, ed");
  bd->eni=(int **)m_alloc2(n,sizeof(int *),"setup.c, eni");
  for(int i=0;i<n;i++){
    bd->ed[i]=(int *)m_alloc2(4,sizeof(int),"setup.c, ed[i]");
    bd->eni[i]=(int *)m_alloc2(4,sizeof(int),"setup.c, eni[i]");
  }
  bd->md=(int *)m_alloc2(n,sizeof(int),"setup.c, md");
  bd->sd=(int *)m_alloc2(n,sizeof(int),"setup.c, sd");
  bd->gd=(int *)m_alloc2(n,sizeof(int),"setup.c, gd");
  bd->cr=gb_alloc_d3(n,3,4);
  bd->cw=gb_alloc_d3(n,3,3);
  bd->ren=gb_alloc_d3(n,4,3);
  bd->wen=gb_alloc_d3(n,4,3);
  bd->Ui=gb_alloc_c3(n,4,4);
  bd->dUi=gb_alloc_c3(n,4,4);
  bd->Ui0=gb_alloc_c3(n,4,4);
  bd->dUi0=gb_alloc_c3(n,4,4);
  bd->Uip=gb_alloc_c3(n,4,4);
}

void gb_mfree_elem(BOUD *bd)
{
  int n=bd->Ne+1;
  for(int i=0;i<n;i++){ free(bd->ed[i]); free(bd->eni[i]); }
  free(bd->ed); free(bd->eni);
  free(bd->md); free(bd->sd); free(bd->gd);
  gb_free_d3(bd->cr,n,3); gb_free_d3(bd->cw,n,3);
  gb_free_d3(bd->ren,n,4); gb_free_d3(bd->wen,n,4);
  gb_free_c3(bd->Ui,n,4); gb_free_c3(bd->dUi,n,4);
  gb_free_c3(bd->Ui0,n,4); gb_free_c3(bd->dUi0,n,4); gb_free_c3(bd->Uip,n,4);
  bd->Ne=0;
}

/* Gmsh 2.2 ASCII mesh.  Every surface element is listed twice: id 2i-1 with
 * the physical tag of one side and id 2i with the other side's tag and the
 * reversed node order; tag 99 is the open region (domain 0).  When one side
 * is the open region it becomes the main domain and the node order is
 * reversed accordingly (reference setup2.c:205-503). */
void gb_read_mesh_data(char *fn,DOMD *md)
{
  const char *W="setup.c, read_mesh_data()";
  FILE *fp=fopen(fn,"rt");
  char buf[256];
  double ver;
  int ti,fmt,prec,nc=0;
  if(fp==NULL){ printf("Can not open the '%s' file. Exit...\n",fn); exit(1); }
  snprintf(md->msh_fn,128,"%s",fn);
  if(fgets(buf,256,fp)==NULL) gb_fail(W,"line");
  if(fscanf(fp,"%lf",&ver)!=1) gb_fail(W,"msh version");
  if(ver!=MSHVER){ printf("This program supports mesh file version %g. Reading file version is %g. Exit...\n",MSHVER,ver); exit(1); }
  if(fscanf(fp,"%d",&fmt)!=1) gb_fail(W,"msh format");
  if(fmt!=MSHASCI){ printf("This program supports 'ASCII' data format mesh file. Exit...\n"); exit(1); }
  if(fscanf(fp,"%d\n",&prec)!=1) gb_fail(W,"data precision");
  if(prec!=MSHPREC){ printf("This program supports double precision mesh data. Exit...\n"); exit(1); }
  if(fgets(buf,256,fp)==NULL || fgets(buf,256,fp)==NULL) gb_fail(W,"line");
  if(fscanf(fp,"%d\n",&ti)!=1) gb_fail(W,"Nn");
  md->bd.Nn=ti;
  gb_malloc_node(&md->bd);
  for(int i=1;i<=md->bd.Nn;i++){
    double x,y,z;
    if(fscanf(fp,"%d",&ti)!=1) gb_fail(W,"node id");
    if(ti!=i) printf("bad id %d\n",ti);
    if(fscanf(fp,"%lf %lf %lf\n",&x,&y,&z)!=3) gb_fail(W,"node coordinates");
    md->bd.rn[i][0]=x; md->bd.rn[i][1]=y; md->bd.rn[i][2]=z;
  }
  if(fgets(buf,256,fp)==NULL || fgets(buf,256,fp)==NULL) gb_fail(W,"line");
  if(fscanf(fp,"%d",&ti)!=1) gb_fail(W,"Ne");
  md->bd.Ne=ti/2;
  gb_malloc_elem(&md->bd);
  BOUD *bd=&md->bd;
  for(int i=1;i<=bd->Ne;i++){
    int id,et,nt,tag,nod[4],chk[4];
    /* first copy: main-side tags and node order */
    if(fscanf(fp,"%d %d %d",&id,&et,&nt)!=3) gb_fail(W,"element header");
    if(id!=2*i-1){ printf("bad id :%d. Exit...\n",id); exit(1); }
    if(et!=ELT3 && et!=ELT4){ printf("bad element type. element type must be %d or %d. Exit...\n",ELT3,ELT4); exit(1); }
    for(int j=0;j<nt;j++){
      if(fscanf(fp,"%d",&tag)!=1) gb_fail(W,"physical entity");
      if(j==0){
        if(tag==OPENDID) tag=0;
        if(tag>md->MN){ printf("domain id %d is not defined medium data. check domain and medium data. exit..\n",tag); exit(1); }
        bd->md[i]=tag;
      }
      else if(j==1) bd->gd[i]=tag;
    }
    int nv=(et==ELT3)?3:4;
    for(int j=0;j<nv;j++) if(fscanf(fp,"%d",&nod[j])!=1) gb_fail(W,"element node");
    if(nv==3) nod[3]=0;
    for(int j=0;j<4;j++) bd->ed[i][j]=nod[j];
    for(int j=0;j<4;j++) bd->eni[i][j]=(j<nv)?nc++:-1;
    /* second copy: opposite side, reversed order */
    if(fscanf(fp,"%d %d %d",&id,&et,&nt)!=3) gb_fail(W,"element header");
    if(id!=2*i){ printf("bad id :%d. Exit...\n",id); exit(1); }
    if(et!=ELT3 && et!=ELT4){ printf("bad element type. element type must be %d or %d. Exit...\n",ELT3,ELT4); exit(1); }
    for(int j=0;j<nt;j++){
      if(fscanf(fp,"%d",&tag)!=1) gb_fail(W,"domain id");
      if(j==0){
        if(tag==OPENDID) tag=0;
        if(tag>md->MN){ printf("domain id %d is not defined medium data. check domain and medium data! exit..\n",tag); exit(1); }
        bd->sd[i]=tag;
      }
    }
    for(int j=0;j<nv;j++) if(fscanf(fp,"%d",&chk[j])!=1) gb_fail(W,"element node");
    /* reversed order of the first copy: (n0, n_last, ..., n1) */
    for(int j=0;j<nv;j++){
      int expect=(j==0)?nod[0]:nod[nv-j];
      if(chk[j]!=expect){ printf("node id miss matched. check element id %d. Exit...\n",2*i); exit(1); }
    }
    if(bd->sd[i]==0){ /* the open region becomes the main domain */
      bd->sd[i]=bd->md[i];
      bd->md[i]=0;
      if(nv==3){ int tmp=bd->ed[i][1]; bd->ed[i][1]=bd->ed[i][2]; bd->ed[i][2]=tmp; }
      else { int tmp=bd->ed[i][3]; bd->ed[i][3]=bd->ed[i][1]; bd->ed[i][1]=tmp; }
    }
  }
  fclose(fp);
  bd->NN=nc;
}

void read_domd2(int argc,char **argv,DOMD *md)
{
  gb_filename_chk(argc,argv);
  memset(md,0,sizeof(DOMD));
  init_mfb(&md->mw);
  read_data_mfb(&md->mw);
  gb_read_medium_data(argv[1],md);
  gb_read_mesh_data(argv[2],md);
  if(argc==11){
    for(int i=0;i<3;i++) md->rv[i]=atof(argv[4+i]);
    md->th=atof(argv[7]);
    for(int i=0;i<3;i++) md->tv[i]=atof(argv[8+i]);
  }
  else {
    md->rv[0]=1.0; md->rv[1]=0.0; md->rv[2]=0.0;
    md->th=0.0;
    md->tv[0]=md->tv[1]=md->tv[2]=0.0;
  }
}

void gb_print_medium_data(DOMD *md)
{
  printf("-- medium data --\n");
  printf("medium data file name                  : %s\n",md->med_fn);
  for(int i=1;i<=md->MN;i++)
    printf("medium (domain) id %2d refractive index :%8.7g + %8.7gI\n",i,creal(md->n[i]),cimag(md->n[i]));
}

void gb_print_mesh_data(DOMD *md)
{
  printf("-- mesh data --\n");
  printf("mesh data file name    : %s\n",md->msh_fn);
  printf("node number            : %8d\n",md->bd.Nn);
  printf("defined element number : %8d\n",md->bd.Ne*2);
}

static void gb_print_domd_common(DOMD *md)
{
  gb_print_medium_data(md);
  printf("\n");
  gb_print_mesh_data(md);
  printf("\n");
  if(md->th!=0.0 || vabs_d(md->tv)!=0.0){
    printf("-- rotation and translation settings --\n");
    if(md->th!=0.0){
      printf("vector defining rotation axis :(% 8.7g,% 8.7g,% 8.7g)\n",md->rv[0],md->rv[1],md->rv[2]);
      printf("rotation angle           [rad]: %8.7g\n",md->th);
    }
    if(vabs_d(md->tv)!=0.0) printf("translation vector            :(%8.7g,%8.7g,%8.7g)\n",md->tv[0],md->tv[1],md->tv[2]);
    printf("\n");
  }
}

void print_domd2(DOMD *md)
{
  printf("-- multi_fbeam data --\n");
  print_data_mfb(&md->mw);
  gb_print_domd_common(md);
}

void print_domd2_mksa(DOMD *md)
{
  printf("-- multi_fbeam data --\n");
  print_data_mfb_mksa(&md->mw);
  gb_print_domd_common(md);
}

/* Rodrigues rotation about rv by th, then translation by tv, applied to the
 * mesh nodes (reference setup2.c:637-664) */
void gb_rotation_translation_obj(double *rv,double th,double *tv,DOMD *md)
{
  double nv[3]={rv[0],rv[1],rv[2]},M[9],r[3];
  vuni_d(nv);
  double s=sin(th),c=cos(th),oc=1.0-c;
  M[0]=c+nv[0]*nv[0]*oc;        M[1]=nv[0]*nv[1]*oc-nv[2]*s;  M[2]=nv[2]*nv[0]*oc+nv[1]*s;
  M[3]=nv[0]*nv[1]*oc+nv[2]*s;  M[4]=c+nv[1]*nv[1]*oc;        M[5]=nv[1]*nv[2]*oc-nv[0]*s;
  M[6]=nv[2]*nv[0]*oc-nv[1]*s;  M[7]=nv[1]*nv[2]*oc+nv[0]*s;  M[8]=c+nv[2]*nv[2]*oc;
  for(int i=1;i<=md->bd.Nn;i++){
    double *p=md->bd.rn[i];
    for(int d=0;d<3;d++) r[d]=M[3*d]*p[0]+M[3*d+1]*p[1]+M[3*d+2]*p[2]+tv[d];
    for(int d=0;d<3;d++) p[d]=r[d];
  }
}

/* Geometry coefficients of every element and the quadrature tables.
 * Bilinear: r(z,e) = a + b z + c e + d z e from the 4 corners, W = dr/dz x dr/de
 * = A + B z + C e.  Linear triangle on the reference triangle with corners
 * (-1/2,-sqrt3/2), (1,0), (-1/2,sqrt3/2): r = a + b z + c e, W constant
 * (reference setup2.c:666-749). */
void gb_init_elem_const(BOUD *bd)
{
  for(int i=1;i<=bd->Ne;i++){
    double rc[3][4];
    for(int d=0;d<3;d++) for(int j=0;j<4;j++) rc[d][j]=bd->rn[bd->ed[i][j]][d];
    if(bd->ed[i][3]!=0){
      for(int d=0;d<3;d++){
        bd->cr[i][d][0]=0.25*( rc[d][0]+rc[d][1]+rc[d][2]+rc[d][3]);
        bd->cr[i][d][1]=0.25*(-rc[d][0]+rc[d][1]+rc[d][2]-rc[d][3]);
        bd->cr[i][d][2]=0.25*(-rc[d][0]-rc[d][1]+rc[d][2]+rc[d][3]);
        bd->cr[i][d][3]=0.25*( rc[d][0]-rc[d][1]+rc[d][2]-rc[d][3]);
      }
      for(int d=0;d<3;d++){
        int a=(d+1)%3,b=(d+2)%3;
        bd->cw[i][d][0]=0.125*((rc[a][0]-rc[a][2])*(rc[b][1]-rc[b][3])-(rc[a][1]-rc[a][3])*(rc[b][0]-rc[b][2]));
        bd->cw[i][d][1]=0.125*((rc[a][2]-rc[a][3])*(rc[b][0]-rc[b][1])-(rc[a][0]-rc[a][1])*(rc[b][2]-rc[b][3]));
        bd->cw[i][d][2]=0.125*((rc[a][1]-rc[a][2])*(rc[b][0]-rc[b][3])-(rc[a][0]-rc[a][3])*(rc[b][1]-rc[b][2]));
      }
    }
    else {
      for(int d=0;d<3;d++){
        bd->cr[i][d][0]=1.0/3.0*( rc[d][0]+rc[d][1]+rc[d][2]);
        bd->cr[i][d][1]=1.0/3.0*(-rc[d][0]+2.0*rc[d][1]-rc[d][2]);
        bd->cr[i][d][2]=1.0/sqrt(3.0)*(rc[d][2]-rc[d][0]);
        bd->cr[i][d][3]=0.0;
      }
      for(int d=0;d<3;d++){
        int a=(d+1)%3,b=(d+2)%3;
        bd->cw[i][d][0]=(rc[a][1]-rc[a][0])*(rc[b][2]-rc[b][0])-(rc[b][1]-rc[b][0])*(rc[a][2]-rc[a][0]);
        bd->cw[i][d][1]=0.0;
        bd->cw[i][d][2]=0.0;
      }
    }
  }
  const double z44[4]={-P44_N,P44_N,P44_N,-P44_N}, e44[4]={-P44_N,-P44_N,P44_N,P44_N};
  const double z49[9]={-P49_N,P49_N,P49_N,-P49_N,0.0,P49_N,0.0,-P49_N,0.0};
  const double e49[9]={-P49_N,-P49_N,P49_N,P49_N,-P49_N,0.0,P49_N,0.0,0.0};
  const double w49[9]={P49_W0,P49_W0,P49_W0,P49_W0,P49_W1,P49_W1,P49_W1,P49_W1,P49_W2};
  const double z34[4]={-P34_N0,2.0*P34_N0,-P34_N0,0.0}, e34[4]={-P34_N1,0.0,P34_N1,0.0};
  const double w34[4]={P34_W0,P34_W0,P34_W0,-P34_W1};
  const double z37[7]={-P37_N0,2.0*P37_N0,-P37_N0,P37_N1,-2.0*P37_N1,P37_N1,0.0};
  const double e37[7]={-P37_N2,0.0,P37_N2,P37_N3,0.0,-P37_N3,0.0};
  const double w37[7]={P37_W0,P37_W0,P37_W0,P37_W1,P37_W1,P37_W1,P37_W2};
  for(int j=0;j<4;j++){ bd->zt_44[j]=z44[j]; bd->et_44[j]=e44[j]; bd->wt_44[j]=P44_W;
                        bd->zt_34[j]=z34[j]; bd->et_34[j]=e34[j]; bd->wt_34[j]=w34[j]; }
  for(int j=0;j<9;j++){ bd->zt_49[j]=z49[j]; bd->et_49[j]=e49[j]; bd->wt_49[j]=w49[j]; }
  for(int j=0;j<7;j++){ bd->zt_37[j]=z37[j]; bd->et_37[j]=e37[j]; bd->wt_37[j]=w37[j]; }
  gauleg(-1.0,1.0,bd->xli,bd->wli,GLN);
  gauleg(-1.0,1.0,bd->xhi,bd->whi,GHN);
}

void gb_malloc_sub_domain(DOMD *md)
{
  int *nc=(int *)m_alloc2(md->MN+1,sizeof(int),"setup.c, Nc");
  for(int i=1;i<=md->bd.Ne;i++){ nc[md->bd.md[i]]++; nc[md->bd.sd[i]]++; }
  md->bd.sb=(SUBD *)m_alloc2(md->MN+1,sizeof(SUBD),"setup.c, sb");
  for(int d=0;d<=md->MN;d++){
    SUBD *s=&md->bd.sb[d];
    s->Ne=nc[d];
    s->sid=(int *)m_alloc2(nc[d]+1,sizeof(int),"setup.c, sid");
    s->U=gb_alloc_c3(nc[d]+1,4,4);  s->dU=gb_alloc_c3(nc[d]+1,4,4);
    s->E=gb_alloc_c3(nc[d]+1,4,3);  s->dE=gb_alloc_c3(nc[d]+1,4,3);
    s->H=gb_alloc_c3(nc[d]+1,4,3);  s->dH=gb_alloc_c3(nc[d]+1,4,3);
  }
  free(nc);
}

void gb_mfree_sub_domain(DOMD *md)
{
  for(int d=0;d<=md->MN;d++){
    SUBD *s=&md->bd.sb[d];
    int n=s->Ne+1;
    gb_free_c3(s->U,n,4); gb_free_c3(s->dU,n,4);
    gb_free_c3(s->E,n,4); gb_free_c3(s->dE,n,4);
    gb_free_c3(s->H,n,4); gb_free_c3(s->dH,n,4);
    free(s->sid);
  }
  free(md->bd.sb);
}

/* sid lists: element i enters the list of its main domain as +i and the list
 * of its sub domain as -i, in element order (reference setup2.c:817-835) */
void gb_init_sub_domain(DOMD *md)
{
  for(int d=0;d<=md->MN;d++){
    int c=1;
    for(int i=1;i<=md->bd.Ne;i++){
      if(md->bd.md[i]==d) md->bd.sb[d].sid[c++]=i;
      else if(md->bd.sd[i]==d) md->bd.sb[d].sid[c++]=-i;
    }
  }
}

/* collocation points and normals at the 4 (3) interior Gauss points */
void gb_init_boundary_data2(DOMD *md)
{
  BOUD *bd=&md->bd;
  for(int i=1;i<=bd->Ne;i++){
    double cr[3][4],cw[3][3],r[3],w[3];
    for(int l=0;l<3;l++){ for(int m=0;m<4;m++) cr[l][m]=bd->cr[i][l][m]; for(int m=0;m<3;m++) cw[l][m]=bd->cw[i][l][m]; }
    for(int j=0;j<4;j++){
      if(bd->ed[i][3]==0) lit_rw_zeta_eta(r,w,bd->zt_34[j],bd->et_34[j],cr,cw);
      else bil_rw_zeta_eta(r,w,bd->zt_44[j],bd->et_44[j],cr,cw);
      for(int l=0;l<3;l++){ bd->ren[i][j][l]=r[l]; bd->wen[i][j][l]=w[l]; }
    }
  }
}

void initialize_domd2(DOMD *md)
{
  setup_mfb(&md->mw);
  md->n[0]=md->mw.n_0;
  for(int i=0;i<=md->MN;i++) md->kn[i]=2.0*M_PI/md->mw.lambda_0*md->n[i];
  if(md->th!=0.0 || vabs_d(md->tv)!=0.0) gb_rotation_translation_obj(md->rv,md->th,md->tv,md);
  gb_init_elem_const(&md->bd);
  gb_init_boundary_data2(md);
  gb_malloc_sub_domain(md);
  gb_init_sub_domain(md);
}

void finalize_domd2(DOMD *md)
{
  gb_dev_release(md);
  gb_mfree_sub_domain(md);
  gb_mfree_elem(&md->bd);
  gb_mfree_node(&md->bd);
  free(md->n);
  free(md->kn);
  free_mfb(&md->mw);
}

/* ---- element geometry helpers ---- */
int check_element_type(int seid,BOUD *bd){ return (bd->ed[abs(seid)][3]==0)?ELT3:ELT4; }

void r_bd(double *r,int seid,double zeta,double eta,BOUD *bd)
{
  int s=abs(seid);
  for(int i=0;i<3;i++){
    if(check_element_type(seid,bd)==ELT4) r[i]=bd->cr[s][i][0]+bd->cr[s][i][1]*zeta+bd->cr[s][i][2]*eta+bd->cr[s][i][3]*zeta*eta;
    else r[i]=bd->cr[s][i][0]+bd->cr[s][i][1]*zeta+bd->cr[s][i][2]*eta;
  }
}
void r_bd_node(double *r,int seid,int nid,BOUD *bd){ for(int l=0;l<3;l++) r[l]=bd->ren[abs(seid)][nid][l]; }
void n_bd_node(double *n,int seid,int nid,BOUD *bd)
{
  for(int l=0;l<3;l++) n[l]=bd->wen[abs(seid)][nid][l];
  vuni_d(n);
}
void tz_te_bd_node(double *vtz,double *vte,int seid,int nid,BOUD *bd)
{
  int s=abs(seid);
  for(int i=0;i<3;i++){
    if(check_element_type(seid,bd)==ELT4){
      vtz[i]=bd->cr[s][i][1]+bd->cr[s][i][3]*bd->et_44[nid];
      vte[i]=bd->cr[s][i][2]+bd->cr[s][i][3]*bd->zt_44[nid];
    }
    else { vtz[i]=bd->cr[s][i][1]; vte[i]=bd->cr[s][i][2]; }
  }
  vuni_d(vtz);
  vuni_d(vte);
}
double bil_Nn(int n,double z,double e)
{
  double ia=1.0/P44_N;
  switch(n){
  case 0: return 0.25*(1.0-z*ia)*(1.0-e*ia);
  case 1: return 0.25*(1.0+z*ia)*(1.0-e*ia);
  case 2: return 0.25*(1.0+z*ia)*(1.0+e*ia);
  case 3: return 0.25*(1.0-z*ia)*(1.0+e*ia);
  }
  printf("setup.c, bil_Nn(), mode number error! n=%d. Exit...\n",n);
  exit(1);
}
double lit_Nn(int n,double z,double e)
{
  double ia=0.5/P34_N0;
  switch(n){
  case 0: return 1.0/3.0*(1.0-ia*(z+sqrt(3.0)*e));
  case 1: return 1.0/3.0*(1.0+2.0*ia*z);
  case 2: return 1.0/3.0*(1.0-ia*(z-sqrt(3.0)*e));
  }
  printf("setup.c, lit_Nn(), mode number error! n=%d. Exit...\n",n);
  exit(1);
}
void bil_copy_elem_const_rw(double cr[][4],double cw[][3],int s,BOUD *bd)
{
  for(int l=0;l<3;l++){ for(int m=0;m<4;m++) cr[l][m]=bd->cr[s][l][m]; for(int m=0;m<3;m++) cw[l][m]=bd->cw[s][l][m]; }
}
void lit_copy_elem_const_rw(double cr[][4],double cw[][3],int s,BOUD *bd)
{
  for(int l=0;l<3;l++){
    cr[l][0]=bd->cr[s][l][0]; cr[l][1]=bd->cr[s][l][1]; cr[l][2]=bd->cr[s][l][2]; cr[l][3]=0.0;
    cw[l][0]=bd->cw[s][l][0]; cw[l][1]=0.0; cw[l][2]=0.0;
  }
}
void bil_rw_zeta_eta(double *r,double *w,double z,double e,double cr[][4],double cw[][3])
{
  for(int i=0;i<3;i++){
    r[i]=cr[i][0]+cr[i][1]*z+cr[i][2]*e+cr[i][3]*z*e;
    w[i]=cw[i][0]+cw[i][1]*z+cw[i][2]*e;
  }
}
void lit_rw_zeta_eta(double *r,double *w,double z,double e,double cr[][4],double cw[][3])
{
  for(int i=0;i<3;i++){
    r[i]=cr[i][0]+cr[i][1]*z+cr[i][2]*e;
    w[i]=cw[i][0];
  }
}
