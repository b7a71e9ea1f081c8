/*
 * gb_host.h -- internal declarations of the host library (not part of the API).
 */
#ifndef GB_HOST_H
#define GB_HOST_H
#include "bem3_emf_b2.h"
#include "gb_bem.h"

/* setup.c */
void gb_filename_chk(int argc,char **argv);
void gb_read_medium_data(char *fn,DOMD *md);
void gb_read_mesh_data(char *fn,DOMD *md);
void gb_print_medium_data(DOMD *md);
void gb_print_mesh_data(DOMD *md);
void gb_malloc_node(BOUD *bd);
void gb_mfree_node(BOUD *bd);
void gb_malloc_elem(BOUD *bd);
void gb_mfree_elem(BOUD *bd);
void gb_rotation_translation_obj(double *rv,double th,double *tv,DOMD *md);
void gb_init_elem_const(BOUD *bd);
void gb_malloc_sub_domain(DOMD *md);
void gb_mfree_sub_domain(DOMD *md);
void gb_init_sub_domain(DOMD *md);
void gb_init_boundary_data2(DOMD *md);

/* dev.c: the device object of a DOMD, kept in a side table so that
 * sizeof(DOMD) stays the reference's */
gb_obj *gb_dev(DOMD *md);          /* create on first use; exits with a message on failure */
gb_obj *gb_dev_peek(DOMD *md);     /* NULL if none */
void gb_dev_release(DOMD *md);
void gb_die(const char *where);    /* print gb_last_error() and exit(1) (the reference's error convention) */
#define GB_F_CMAT 1   /* coefficient matrices of every domain on the device */
#define GB_F_INV  2   /* inverse of A on the device */
#define GB_F_BV   4   /* device boundary values are current */
#define GB_F_INC  8   /* incident potential uploaded */
int gb_dev_flags(DOMD *md);
void gb_dev_set_flags(DOMD *md,int set,int clear);
void gb_call_lock(void);
void gb_call_unlock(void);
void gb_bv_to_device(DOMD *md);    /* host SUBD boundary values -> device (once) */
void gb_bv_to_host(DOMD *md);      /* device boundary values -> host SUBD */

/* Versioned .cmat of the FP64 block factors, written in place of the dense
 * inverse for objects with one interface (GB_CMAT_FORMAT=block, or when the
 * dense inverse would take more than half the device memory): a 64-byte
 * header -- the 8 bytes "GBBLKF64", int32 version 1, int32 NN, int32 number
 * of matrices 5, int32 bytes per element 16, zeros -- then G0^-1, G1^-1,
 * -G0^-1 H0, M^-1, S^-1, each NN x NN complex128 row-major.  The dense
 * inverse stays the reference's headerless file. */
#define GB_BLK_MAGIC "GBBLKF64"
#define GB_BLK_HEADER 64
#define GB_BLK_VERSION 1

/* matrix.c */
void gb_initalize_cmd2(CMD *cm);
void gb_finalize_cmd2(CMD *cm);
void gb_cmat_read(DOMD *md,int with_inverse);   /* .cmat files named in md->cm -> device */
/* mo.c */
void gb_mo_malloc(MOBJ *mo);
void gb_init_boundary_data_u2(DOMD *md);
#endif
