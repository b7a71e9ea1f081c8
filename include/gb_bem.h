/*
 * gb_bem.h -- C ABI of the GB300 BEM kernels (sm_103a).
 *
 * Plain pointers and sizes only.  Complex numbers are interleaved
 * (real, imaginary) doubles, the memory layout of C99 `double complex`.
 * Every entry point returns 0 on success and -1 on failure; gb_last_error()
 * then describes the failure.  A gb_obj is one BEM object (one mesh with its
 * media) resident in the GPU's memory: mesh, coefficient matrices, the
 * inverse or LU factors of the coupled matrix A, and the boundary values.
 *
 * Each entry point replaces one stage of the reference (akohta/bem3_emf_b2);
 * the file:line of the replaced code is given beside it.  The reference API
 * (bem3_emf_b2.h) is implemented on top of these calls.
 */
#ifndef GB_BEM_H
#define GB_BEM_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_obj gb_obj;

/* Host description of one object, 1-based in the element index like the
 * reference's BOUD (d3b1_elem.h:50-75): arrays have Ne+1 entries, slot 0
 * unused. */
typedef struct gb_mesh_desc {
  int Ne;              /* elements */
  int NN;              /* collocation nodes */
  int MN;              /* media; domains are 0..MN */
  const double *cr;    /* (Ne+1)*12: cr[e][xyz][a,b,c,d] */
  const double *cw;    /* (Ne+1)*9:  cw[e][xyz][A,B,C] */
  const double *ren;   /* (Ne+1)*12: collocation points ren[e][node][xyz] */
  const double *wen;   /* (Ne+1)*12: normals at the collocation points */
  const int *etype;    /* (Ne+1): 1 bilinear quadrangle, 0 linear triangle */
  const int *eni;      /* (Ne+1)*4: collocation node ids (-1 unused) */
  const int *md;       /* (Ne+1): main domain */
  const int *sd;       /* (Ne+1): sub domain */
  const double *kn;    /* 2*(MN+1): wave number of each domain (re, im) */
  const int *sb_Ne;    /* MN+1: elements bounding each domain */
  const int *sid;      /* sum_d (sb_Ne[d]+1): signed element ids, domain after domain, each list 1-based */
  const double *corner;/* (Ne+1)*12: corner node coordinates rn[ed[e][j]] (solid angles) */
  double lambda0;      /* vacuum wavelength */
} gb_mesh_desc;

const char *gb_last_error(void);
int gb_device_count(void);
/* free and total memory of the current device, bytes */
int gb_device_memory(size_t *free_bytes, size_t *total_bytes);
/* kernel launches made by this library so far (all threads) */
unsigned long long gb_launch_count(void);
/* the CUDA stream (cudaStream_t) the object's work runs on */
void *gb_obj_stream(gb_obj *o);
/* the calling host thread's current device, and setting it (for host
 * threads that drive objects created on another thread) */
int gb_current_device(void);
int gb_use_device(int dev);
/* live timing of the tensor-core trailing-update kernel (roofline figures):
 * enable(1) starts recording (CUDA events around every launch on its stream),
 * read() returns total device ms, launches, complex-equivalent flops (8 M N K)
 * and algorithmic HBM bytes since then and clears the record */
void gb_ktime_enable(int on);
int gb_ktime_read(double *ms, long *launches, double *flops, double *bytes);
/* the recorded launches one by one, without clearing: rec[4i..4i+3] = device
 * ms, M, N, K of launch i (i < cap); returns the number recorded, -1 on error */
int gb_ktime_list(int cap, double *rec);
/* the double-float regular assembly launches recorded while timing was on:
 * total device ms, (collocation node, element) pairs they covered, launches */
int gb_ktime_asm(double *ms, double *pairs, long *launches);

int gb_obj_create(const gb_mesh_desc *m, gb_obj **out);
void gb_obj_destroy(gb_obj *o);

/* Coefficient matrices G, H (N x N), dG, dH (2N x N), dF (N x 3) of domain did,
 * N = 4 sb_Ne[did], quadrature type 0..3 (4-point, 9/7-point, GLN, GHN; the
 * reference uses 2).  Replaces create_cmatrix_domain, solve_bieq2.c:98-184. */
int gb_assemble(gb_obj *o, int did, int type);
/* as gb_assemble (precision 0: all in FP64) with another arithmetic for the
 * regular pairs of the GLN x GLN rule.
 * precision 2: regular pairs in double-float (two FP32 numbers, ~48 bits),
 * pairs that need the GHN fallback and the singular elements in FP64.  The
 * matrices agree with precision 0 to ~1e-14 relative Frobenius (rounding
 * level); the chosen scene form uses it.  The object's field kernels
 * (gb_field_points, gb_field_bd, gb_add_scattered) then integrate their
 * regular GLN pairs in double-float too; any other precision sets them back
 * to FP64.
 * precision 3 (the chosen scene form): as precision 2, with the regular
 * pairs' Gauss order adapted to the pair: n x n points, n = max(n_D, n_k),
 * n_D = 12, 9, 6, 5 for distances below 2, 3, 5 and beyond (in units of the
 * element's parameter-map size a), n_k = 5, 7, 8, 12 for |k| a up to 0.75,
 * 2.4, 4.5 and beyond; pairs that keep n = 12 are integrated exactly as in
 * precision 2.  Each far pair's integrals stay within ~1e-12 of their
 * natural scale; the field kernels then use the same rule.
 * precision 1: regular pairs farther than three element radii in FP32
 * relative to the source element's centre (FP64 phase at the centre).
 * Matrix entries then carry ~1e-7 relative error (measured: G 9e-8, dH 2e-7,
 * radiation force up to 8e-7 on the 384-element sphere): an opt-in only. */
int gb_assemble2(gb_obj *o, int did, int type, int precision);
/* Rows row0 .. row0 + nrow - 1 of domain did's G, H, dG, dH, dF (the rows
 * that create_cmatrix_domain writes, solve_bieq2.c:98-184, free term on the
 * diagonal included) into caller DEVICE buffers: G, H nrow x N, dG, dH
 * 2 nrow x N, dF nrow x 3 (N = 4 sb_Ne[did]); precision as gb_assemble2.
 * The object's own matrices are neither allocated nor touched, so a domain
 * too large to store (the 38,400-element cube: 377 GB per matrix) can be
 * assembled block by block and streamed to a consumer.  Asynchronous on the
 * object's stream (gb_obj_stream); its small scratch is stream-ordered. */
int gb_assemble_rows(gb_obj *o, int did, int row0, int nrow, int type, int precision, void *G, void *H, void *dG,
                     void *dH, double *dF);
/* every domain of every object of a scene (objects of uneven sizes, on the
 * current device), as gb_assemble2, with one launch per phase over a work
 * list of (object, domain) items instead of a launch sequence per domain */
int gb_assemble_objects(gb_obj **objs, int n, int type, int precision);
/* every domain of the object, as gb_assemble2, the domains at once (one host
 * thread and stream each) */
int gb_assemble_all(gb_obj *o, int type, int precision);
/* assembly precision of scene form `form` (1 -> 3, 2 -> 1, 0 and 3 -> 0) */
int gb_form_precision(int form);
/* copy the resident matrices of domain did to/from host buffers in the
 * reference's .cmat layout (any pointer may be NULL to skip that matrix) */
int gb_cmatrix_download(gb_obj *o, int did, void *G, void *H, void *dG, void *dH, double *dF);
int gb_cmatrix_upload(gb_obj *o, int did, const void *G, const void *H, const void *dG, const void *dH, const double *dF);
/* selected rows of the resident matrices of domain did (rows[i] in 0..N-1):
 * row i of G and H (N complex each), rows 2 i, 2 i + 1 of dG and dH, row i
 * of dF, packed in the order given (any output may be NULL) */
int gb_cmatrix_rows(gb_obj *o, int did, int nrows, const int *rows, void *G, void *H, void *dG, void *dH, double *dF);

/* Coupled matrix A (na x na, na = 8 NN) from the resident G, H of all domains,
 * LU-factorised with partial pivoting, and its explicit inverse.
 * Replaces create_Amatrix_csr + lu_dec_A, solve_bieq2.c:186-408. */
int gb_invA_compute(gb_obj *o);
int gb_invA_download(gb_obj *o, void *invA);
int gb_invA_upload(gb_obj *o, const void *invA);
/* A alone (for tests): built from the resident G, H; not factorised */
int gb_A_download(gb_obj *o, void *A);

/* x <- invA b for host vectors of length na.  Replaces solve_ABmatrix,
 * mo_solve.c:246-274. */
int gb_solve_AB(gb_obj *o, const void *b, void *x);

/* ---- boundary values and the multi-object iteration (reference mo_solve.c) ----
 * Boundary values of domain did, reference layout: U, dU [(Ne_d+1)][4][4],
 * E, dE, H, dH [(Ne_d+1)][4][3] (complex).  Incident potential per element:
 * [(Ne+1)][4][4].  NULL pointers are skipped. */
int gb_bv_upload(gb_obj *o, int did, const void *U, const void *dU, const void *E, const void *dE, const void *H, const void *dH);
int gb_bv_download(gb_obj *o, int did, void *U, void *dU, void *E, void *dE, void *H, void *dH);
int gb_incident_upload(gb_obj *o, const void *Ui0, const void *dUi0);      /* also sets Ui = Uip = Ui0, dUi = dUi0 */
int gb_incident_download(gb_obj *o, void *Ui, void *dUi, void *Uip);
/* B from the incident potential, X = invA B, U and dU of every domain
 * (create_Bmatrix + solve_ABmatrix + tmatrix_bd_store, mo_solve.c:137-274,457) */
int gb_solve_mEMP(gb_obj *o);
/* Uip <- Ui, Ui <- Ui0, dUi <- dUi0 (reset_incident_bd, mo_solve.c:398-411) */
int gb_reset_incident(gb_obj *o);
/* dst.Ui, dst.dUi += potential scattered by src at dst's exterior nodes
 * (add_scattered_mEMP, mo_solve.c:296-396); fails if a node lies inside src.
 * The first call for a (src, type) pair fixes the nodes' domains and, when
 * they fit in a quarter of the free device memory, integrates the
 * coefficients of src's potential at dst's nodes once; later calls are a
 * product with src's current boundary values, until dst is assembled again
 * (an assembly drops the operators dst holds).  Concurrent calls must not
 * share dst. */
int gb_add_scattered(gb_obj *dst, gb_obj *src, int type);
/* sums of the convergence measure over the exterior nodes (ccd_f, mo_solve.c:413-455):
 * out[0] sum of potential changes, out[1] sum of phi changes, out[2] node count */
int gb_ccd_sums(gb_obj *o, double *out);
/* E, H and dE/dn, dH/dn of every domain (solve_eh_bv, solve_deh_bv, mo_solve.c:547-789) */
int gb_solve_EH(gb_obj *o);

/* ---- points (reference setup2.c:944-978, d3b1_field.c, mo_field.c) ----
 * rt: [n][3].  gb_domain_id: domain of each point (-1: none).
 * gb_field_points, mode 0: potentials U[4] (mEMP_s); 1: E[3],H[3] (EH_s);
 * 2: E[3],H[3] from potential derivatives (EH_mEMP_s; flag = -did where the
 * near-boundary cutoff applied); 3: U[4], dU/dv[4] along v[n][3] (mEMP2_s).
 * did: domain of each point (from gb_domain_id); type: quadrature 0..3.
 * gb_field_bd: E[3],H[3] on the boundary (EH_s_bd) at element t (1-based in
 * domain did's list), parameters zt[n][2]. */
int gb_domain_id(gb_obj *o, int n, const double *rt, int *did);
int gb_field_points(gb_obj *o, int mode, int type, int n, const double *rt, const double *v, const int *did, void *out, int *flag);
int gb_field_bd(gb_obj *o, int type, int n, const int *did, const int *t, const double *zt, void *out);

/* Allocation-free domain assembly.  No counterpart in the reference.
 * For callers that cannot allocate device memory -- their device memory is
 * owned by another allocator (e.g. a framework's caching pool), they cannot
 * accept cudaFree's implicit device synchronisation, or they must allocate
 * nothing after start-up -- this computes the same G, H, dG, dH, dF of one
 * domain as gb_assemble with every buffer supplied by the caller (all device
 * pointers): mesh arrays as in gb_mesh_desc (cr, cw, ren, etype, 1-based),
 * sid = the domain's signed element list (Ne+1 ints, slot 0 unused), wave
 * number k, domain id did (0: the open region, which takes the free term
 * 1 + F), quadrature type; outputs in the .cmat layout (N = 4 Ne); stream is a
 * cudaStream_t (NULL: the default stream); the call is asynchronous.
 * It calls no cudaMalloc, cudaFree or allocating routine: its scratch is a
 * fixed 16 MiB static device array that every GPU loading the library holds
 * until exit, so a domain may have at most 418 elements (larger: error).  The
 * array's device address is looked up on the first call on each device, so
 * make that first call before any stream capture.  All calls share the array
 * (cleared at the start of each call): calls that overlap on the GPU race and
 * must be serialised by the caller. */
int gb_assemble_domain_noalloc(const double *cr, const double *cw, const int *etype, const double *ren, const int *sid,
                               int Ne, double k_re, double k_im, int did, int type,
                               void *G, void *H, void *dG, void *dH, double *dF, void *stream);

/* ---- mixed-precision form ----
 * gb_factor_mixed: A from the resident G, H, kept in FP64, and its complex
 * FP32 LU factors; later gb_solve_mEMP calls solve A x = b by FP64 GMRES
 * preconditioned by those factors (gb_set_refinement; residual b - A x in
 * FP64, relative residual <= 1e-13) instead of applying an explicit inverse.
 * gb_ir_info: corrections and final relative residual of the last solve.
 * gb_scene_step: assembly of every domain + factorisation + U, dU + E, H,
 * dE, dH.  form 0: FP64 assembly and FP64 factorisation (gb_factor_fp64);
 * form 1 (chosen): double-float regular pairs with the adaptive order
 * (gb_assemble2 precision 3) and the mixed factorisation; form 2: FP32 far pairs
 * (precision 1) and mixed; form 3: FP64 assembly and mixed. */
int gb_factor_mixed(gb_obj *o);
int gb_ir_info(gb_obj *o, int *iters, double *relres);
/* Refinement of the solves that use lower-precision or block factors.
 * mode 0 (default): FP64 flexible GMRES(20), right-preconditioned by the factors
 * (residual b - A x in FP64 from G, H; converged at ||b - A x|| <= 1e-13 ||b||;
 * a run that does not converge with butterfly or block factors refactorises
 * with tournament pivoting and continues).  mode 1 (diagnostic): classical
 * refinement x += M^-1 (b - A x) with the same fallback rules.
 * gb_ir_info reports the preconditioner solves of the last solve. */
int gb_set_refinement(gb_obj *o, int mode);
/* tensor-core passes of every complex-FP32 factorisation started afterwards
 * (process-wide): 1 (default; plain TF32 products, ~1e-3 relative error in
 * the factors -- they only precondition the FP64 GMRES, which absorbs it in
 * a few more iterations) or 3 (split TF32: FP32-accurate products, for
 * callers that use the FP32 factors directly) */
int gb_set_tc_passes(int passes);
int gb_get_tc_passes(void);
/* Row interchanges of the FP32 factorisation.  mode 0 (default): A is
 * randomised by two-sided recursive butterfly transforms of depth 2
 * (U^T A V, random diagonal entries e^{rho/10}, fixed seed; Parker 1995,
 * Baboulin et al. 2013) and factorised without interchanges, when na is
 * divisible by 4; a zero pivot, or a refinement that does not contract the
 * residual 10x per correction, makes the object factorise again with
 * tournament pivoting.  mode 1: tournament pivoting always.  mode 2
 * (diagnostic): as mode 0, but the first refinement check takes the
 * fallback, so that the refactorisation path can be exercised.  mode 3 (the
 * default): block elimination for an object whose elements all separate
 * domain 0 (outside) from domain 1 (inside): the corrections go through
 * complex-FP32 inverses of order NN (G0^-1, G1^-1, G0^-1 H0, and those of the
 * two Schur complements; each node matrix randomised by butterflies and
 * factorised without interchanges) instead of factors of the 8 NN x 8 NN
 * matrix A -- about 43x fewer flop and 5 NN^2 instead of 64 NN^2 elements;
 * the FP64 refinement on A is unchanged.  Other objects are factorised as in
 * mode 0; a zero pivot or a stalled refinement falls back to
 * tournament-pivoted dense factors.  The environment variable GB_LU_MODE
 * (0..3) sets the mode objects are created with (default 3).
 * gb_lu_info: rbt = 1 if the current factors are of the randomised matrix,
 * 2 if they are the FP32 block factors of mode 3, 3 if they are the FP64
 * block factors of gb_factor_fp64; fallbacks = refactorisations after a zero
 * pivot or a stalled refinement so far.
 * gb_factor_fp64: the plain FP64 form's factorisation.  For an object with
 * one interface in mode 3 the same block elimination in complex FP64 (node
 * LUs with tournament pivoting, FP64 inverses and products; later solves
 * take one FP64 correction and confirm the residual from G, H); otherwise
 * the dense LU and explicit inverse of A as the reference's lu_dec_A
 * (gb_invA_compute). */
int gb_set_lu_pivoting(gb_obj *o, int mode);
/* Outer block of the blocked LUs and inverses (process-wide; the K of the
 * trailing tensor-core updates, inner 64-column panels update only inside
 * it): 256 by default, a multiple of 64 up to 2048.  gb_tune_lu_outer_block
 * times the complex-FP32 LU and inverse of an n x n test matrix with 128,
 * 256, 512 and 1024 (ms[4], CUDA events, second of two runs), keeps the
 * fastest and returns it in *best. */
int gb_set_lu_outer_block(int nbo);
int gb_lu_outer_block(void);
int gb_tune_lu_outer_block(int n, int *best, double *ms);
int gb_lu_info(gb_obj *o, int *rbt, int *fallbacks);
int gb_factor_fp64(gb_obj *o);
/* 1 if every element of the object separates domain 0 (outside) from domain
 * 1 (inside): the block elimination applies */
int gb_obj_one_interface(gb_obj *o);
/* the FP64 block factors of gb_factor_fp64 (each NN x NN complex, row-major):
 * G0^-1, G1^-1, -G0^-1 H0, M^-1, S^-1 -- to and from host memory (upload
 * makes them the object's factors for later gb_solve_mEMP calls).  The
 * tools keep them in the versioned <prefix>_blk.cmat file in place of the
 * dense inverse. */
int gb_block_factors_download(gb_obj *o, void *G0i, void *G1i, void *nX0, void *Minv, void *Si);
int gb_block_factors_upload(gb_obj *o, const void *G0i, const void *G1i, const void *nX0, const void *Minv,
                            const void *Si);
int gb_scene_step(gb_obj *o, int form, int type);

/* ---- learned near-singular quadrature (quadrangles) ----
 * The reference integrates a (node, element) pair with |Re dF| > CBD_SDF by
 * its 64 x 64 fallback rule (d3b1_elem.c:503-504, bil_dcoef_v2.c:235-326).
 * With a trained network enabled, a precision >= 2 assembly keeps such a
 * quadrangle pair's 12 x 12 values and adds the network's prediction of the
 * difference between the two rules (G, H, dG, dH, F, dF); every assembly
 * then checks a sample of its corrected pairs (every 16th, at least 64, at
 * most 2,048) against the 64 x 64 rule and, if the sample's RMS error
 * (largest output error over
 * the pair's largest output, in size-scaled units) exceeds tol, integrates
 * all of them by that rule.  FP64 (precision 0) assemblies never use it.
 * gb_lq_collect(1): later precision >= 2 assemblies list their fallback
 * quadrangle pairs and keep features and targets for training (their
 * matrices then hold the 12 x 12 values of those pairs); (0) stops.
 * gb_lq_train: trains the process-wide network (20 -> 256 x 3 -> 51, GELU)
 * on everything collected: seeded shuffle, 1/20 held out, standardised
 * inputs and targets, Adam with a cosine schedule from lr; info[5]: pairs
 * trained on, held out, final training loss, held-out loss, held-out loss of
 * a zero prediction (standardised units).
 * gb_lq_enable(on, tol): use it in later assemblies (default off).
 * gb_lq_stats(out[8]) of the last assembly that listed pairs: pairs
 * corrected, pairs beyond the list's capacity (64 x 64 rule), pairs judged,
 * RMS error of the corrected sample, RMS error of the 12 x 12 rule alone on
 * the same sample, largest corrected error, 1 if the assembly reverted to
 * the 64 x 64 rule, milliseconds of the stage. */
int gb_lq_collect(int on);
int gb_lq_train(int epochs, int batch, float lr, unsigned seed, double *info);
int gb_lq_enable(int on, double tol);
int gb_lq_stats(double *out);

/* Dense complex FP64 LU solve of a host system: A (n x n, row-major) X = B
 * (n x nrhs, row-major), B overwritten by X.  The kernel behind the dE/dn,
 * dH/dn solve (LAPACKE_zgesv, mo_solve.c:751). */
int gb_zgesv(int n, int nrhs, void *A, void *B);

#ifdef __cplusplus
}
#endif
#endif
