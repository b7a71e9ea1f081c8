/*
 * bem3_emf_b2.h -- public API of the GB300 BEM hot path.
 *
 * Drop-in for the reference's d3b2_src/bem3_emf_b2.h:31-124: same types,
 * names, argument meaning and return conventions, so d3b2_create_matrix,
 * d3b2_bv_solver and example1-4 compile unchanged against it.  Every
 * compute-heavy call runs in this library's sm_103a kernels through the
 * C ABI declared in gb_bem.h.
 */
#ifndef BEM3_EMF_B2_H_
#define BEM3_EMF_B2_H_

#include "d3b1_const.h"
#include "d3b1_elem.h"
#include "my_utils.h"
#include "gauleg.h"

#define FNLGTH   256
#define ITER_MIN  10     /* minimum iterations of mo_solve_bv */
#define ITER_MAX 100     /* maximum iterations of mo_solve_bv */
#define PREC_DEF   2     /* quadrature of the coefficient matrices: GLN x GLN with GHN fallback */
#define CCD   1.0e-6     /* convergence threshold of mo_solve_bv */

typedef struct multi_object_data{
  int N;          /* number of objects */
  char **mod_fn;  /* object (.obj) file names */
  double **rs;    /* translation of each object */
  DOMD *md;       /* objects */
} MOBJ;

/* single object: setup, assembly, inverse (reference setup2.c, solve_bieq2.c) */
void read_domd2(int argc,char **argv,DOMD *md);
void print_domd2(DOMD *md);
void print_domd2_mksa(DOMD *md);
void initialize_domd2(DOMD *md);
void finalize_domd2(DOMD *md);
int domain_id(double *rt,DOMD *md);
void create_matrix(DOMD *md,char *ofn);

/* multiple objects (reference mo_setup.c, mo_solve.c) */
void mo_initialize(int argc,char **argv,MOBJ *mo);
void mo_print_data(MOBJ *mo);
void mo_print_data_mksa(MOBJ *mo);
void mo_finalize(MOBJ *mo);
void mo_dat_write(char *fname,MOBJ *mo);
void mo_dat_read(char *fname,MOBJ *mo);
void mo_output_node_particles(char *fname,MOBJ *mo);
void mo_solve_bv(MOBJ *mo);

/* analysis (reference mo_field.c, mo_force.c, mo_absorb.c) */
void mo_object_domain_id(int *oid,int *did,double *rt,MOBJ *mo);
int mo_mEMP_s(double complex *U,double *rt,int type,MOBJ *mo);
int mo_mEMP_t(double complex *U,double *rt,int type,MOBJ *mo);
int mo_mEMP_i(double complex *U,double *rt,int type,MOBJ *mo);
int mo_EH_s(double complex *E,double complex *H,double *rt,int type,MOBJ *mo);
int mo_EH_t(double complex *E,double complex *H,double *rt,int type,MOBJ *mo);
int mo_EH_i(double complex *E,double complex *H,double *rt,int type,MOBJ *mo);
int mo_EH_mEMP_s(double complex *E,double complex *H,double *rt,int type,MOBJ *mo);
int mo_EH_mEMP_t(double complex *E,double complex *H,double *rt,int type,MOBJ *mo);
int mo_EH_mEMP_i(double complex *E,double complex *H,double *rt,int type,MOBJ *mo);
void mo_EH_s_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo);
void mo_EH_t_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo);
void mo_EH_i_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo);
void mo_EH_a_bd(double complex *E,double complex *H,int oid,int did,int t,double zeta_t,double eta_t,int type,MOBJ *mo);
int mo_force_FN(double *F,double *N,double *rc,int oid,int type,MOBJ *mo);
int mo_absorb_P(double *P,int oid,int type,MOBJ *mo);

#endif
