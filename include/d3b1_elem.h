/*
 * d3b1_elem.h -- data model of one BEM object and the element-level API.
 *
 * CMD, SUBD, BOUD, DOMD and TDATA keep the member order and types of the
 * reference's d3b2_src/d3b1_elem.h:13-97 (callers index them directly and the
 * .obj/.dat formats are defined through them).  Arrays are 1-based in the
 * element index ([Ne+1], slot 0 unused), exactly as in the reference.
 *
 * Element-level quadrature (coef_rt, dcoef_rt, dcoef_bd_node_t2, ...) runs on
 * the GPU in this library; the host-side helpers below are geometry only.
 */
#ifndef BEM1_ELEM_H_
#define BEM1_ELEM_H_

#include "d3b1_const.h"

typedef struct coef_matrix{
  int type;      /* quadrature type of the coefficient matrices */
  int MN;        /* number of media (domains 0..MN) */
  char **tgfn;   /* .cmat file name of G, per domain */
  char **thfn;   /* H */
  char **tdgfn;  /* dG (two tangential directions) */
  char **tdhfn;  /* dH */
  char **tdffn;  /* dF (F, dF/dt_zeta, dF/dt_eta) */
  char *lupfn;   /* inverse of the coupled matrix A */
  size_t nn;     /* collocation nodes NN */
  size_t na;     /* order of A: 8 NN */
  size_t nnz;    /* non-zeros of A (kept for layout compatibility) */
  char *aval;    /* scratch file names of the reference's CSR stage (unused here) */
  char *aptr;
  char *aidx;
  char *b;
}CMD;

typedef struct sub_domain_data{
  int Ne;        /* elements bounding this domain */
  int *sid;      /* signed element ids, sid[1..Ne]; negative: seen from the sub-domain side */
  double complex ***U,***dU;  /* potentials (Ax,Ay,Az,phi) and normal derivatives [s][node][4] */
  double complex ***E,***dE;  /* electric field and normal derivative [s][node][3] */
  double complex ***H,***dH;  /* magnetic field and normal derivative [s][node][3] */
}SUBD;

typedef struct boundary_data{
  int Nn;        /* mesh nodes */
  int Ne;        /* elements (each listed twice in the mesh file) */
  double **rn;   /* rn[node][xyz] */
  int **ed;      /* ed[element][0..3] node ids; ed[e][3]==0 for triangles */
  int NN;        /* collocation nodes: 4 per quad, 3 per triangle */
  int **eni;     /* eni[element][0..3] collocation node ids (-1 unused) */
  int *md;       /* main-domain id of each element */
  int *sd;       /* sub-domain id of each element */
  int *gd;       /* Gmsh elementary entity */
  double ***cr,***cw;    /* geometry coefficients cr[e][xyz][a,b,c,d], cw[e][xyz][3] */
  double ***ren,***wen;  /* collocation points and (non-unit) normals [e][node][xyz] */
  double complex ***Ui,***dUi;   /* incident potential at collocation points */
  double complex ***Ui0,***dUi0; /* initial incident potential */
  double complex ***Uip;         /* previous iterate (convergence test) */
  double zt_44[4],et_44[4],wt_44[4],zt_49[9],et_49[9],wt_49[9];
  double zt_34[4],et_34[4],wt_34[4],zt_37[7],et_37[7],wt_37[7];
  double xli[GLN],wli[GLN];
  double xhi[GHN],whi[GHN];
  SUBD *sb;
}BOUD;

typedef struct domain_data {
  char med_fn[128], msh_fn[128];
  double rv[3],th;     /* rotation axis and angle (Rodrigues) */
  double tv[3];        /* translation applied after the rotation */
  int MN;
  double complex *n;   /* refractive index per medium */
  double complex *kn;  /* wave number per medium */
  Bobj mw;
  BOUD bd;
  CMD cm;
} DOMD;

typedef struct tmp_data{
  double complex k;
  double zeta,eta;
  double zeta_t,eta_t;
  double r0,r1,th0,th1;
  double sth,cth;
  double rt[3],vt[3],vu[3],aW;
  double cr[3][4],cw[3][3];
  double *xi,*wi,*xhi,*whi;
  int nid,gn,ghn;
}TDATA;

/* geometry helpers (reference d3b1_elem.c:11-143) */
int check_element_type(int seid,BOUD *bd);
void r_bd(double *r,int seid,double zeta,double eta,BOUD *bd);
void r_bd_node(double *r,int seid,int nid,BOUD *bd);
void n_bd_node(double *n,int seid,int nid,BOUD *bd);
void tz_te_bd_node(double *vtz,double *vte,int seid,int nid,BOUD *bd);
double bil_Nn(int n,double zeta,double eta);
double lit_Nn(int n,double zeta,double eta);
void bil_copy_elem_const_rw(double cr[][4],double cw[][3],int s,BOUD *bd);
void lit_copy_elem_const_rw(double cr[][4],double cw[][3],int s,BOUD *bd);
void bil_rw_zeta_eta(double *r,double *w,double zeta,double eta,double cr[][4],double cw[][3]);
void lit_rw_zeta_eta(double *r,double *w,double zeta,double eta,double cr[][4],double cw[][3]);

#endif
