/*
 * gb_scene.h -- one-call entry points for a single-object scene (no files
 * written), for callers that want the whole hot path -- assembly, the
 * coupled system, boundary values, fields and radiation force -- without the
 * reference's .cmat/.obj/.dat round trips.  The setup reads the reference's
 * input files (medium data, Gmsh 2.2 mesh, ipw.txt) like read_domd2 +
 * initialize_domd2 (reference setup2.c:11-121).
 */
#ifndef GB_SCENE_H
#define GB_SCENE_H
#include "bem3_emf_b2.h"
#ifdef __cplusplus
extern "C" {
#endif

/* host setup of one object and its device copy; NULL on failure (message printed) */
DOMD *gbh_scene_open(const char *medium_file, const char *mesh_file, const char *ipw_file);
/* device step: assembly (quadrature type), factorisation, boundary values,
 * E/H, then the radiation force and torque about rc (type-0 surface rule,
 * mo_force_FN).  form 0: FP64 assembly and FP64 factorisation (block
 * elimination for one-interface objects, else LU + explicit inverse as the
 * reference); form 1 (chosen): double-float regular-pair assembly with the
 * distance-adaptive order, complex FP32 factors + FP64 iterative refinement; form 2: FP32 far-pair assembly (opt-in,
 * ~1e-7 relative error), mixed LU; form 3: FP64 assembly, mixed LU
 * (gb_scene_step in gb_bem.h) */
int gbh_scene_step(DOMD *md, int form, int type, const double *rc, double *F, double *N);
/* drop the device copy; the next step re-uploads the mesh from host memory */
void gbh_scene_drop_device(DOMD *md);
/* bytes moved host->device to (re)create the device copy, and device->host per step */
size_t gbh_scene_h2d_bytes(DOMD *md);
size_t gbh_scene_d2h_bytes(DOMD *md);
void gbh_scene_close(DOMD *md);
/* the cudaStream_t of the scene's device copy (created if needed) */
void *gbh_scene_stream(DOMD *md);
/* the device object (gb_obj *) of the scene, for phase-by-phase calls of gb_bem.h;
 * the incident potential is uploaded on first use */
void *gbh_scene_obj(DOMD *md);

/* Multi-object scene (reference d3b2_create_matrix per object + mo_solve_bv
 * + mo_force_FN, mo_solve.c:10-88): object m is read from medium_files[m] and
 * mesh_files[m], rotated by th[m] about the axis rv[3m..3m+2] and then
 * translated by tv[3m..3m+2] (d3b2_create_matrix's optional arguments; rv, th,
 * tv may be NULL), all lit by the plane waves of ipw_file.  NULL on failure. */
MOBJ *gbh_mscene_open(int n, const char *const *medium_files, const char *const *mesh_files, const char *ipw_file,
                      const double *rv, const double *th, const double *tv);
/* device step of the whole scene: assembly and factorisation (form as in
 * gbh_scene_step) of every object, the multiple-scattering iteration, then
 * force and torque of each object (type-0 surface rule) about rc[3m..3m+2]
 * (rc NULL: the object's translation point); F, N: 3 n */
int gbh_mscene_step(MOBJ *mo, int form, int type, const double *rc, double *F, double *N);
/* Many incident beams as right-hand sides: beam b is wave b of beams_file
 * (ipw.txt layout) on its own -- what a reference run with an ipw.txt that
 * holds only that wave computes (the reference sums all waves of ipw.txt
 * into one field, multi_fbeam.c:817-833).  Assembly, factorisations and the
 * multiple-scattering operators are built once for all beams; each beam
 * then takes the iteration, E/H and force and torque of every object,
 * F, N [nbeam][n][3] (rc as in gbh_mscene_step).  *nbeam: waves read. */
int gbh_mscene_beams(MOBJ *mo, int form, int type, const char *beams_file, const double *rc, double *F, double *N,
                     int *nbeam);
void gbh_mscene_drop_device(MOBJ *mo);
size_t gbh_mscene_h2d_bytes(MOBJ *mo);
size_t gbh_mscene_d2h_bytes(MOBJ *mo);
void gbh_mscene_close(MOBJ *mo);
/* Batched field map of a solved multi-object scene (the examples' per-point
 * loops, reference example2.c:43-50, example4.c:53-66, in one call): the
 * total (which = 1), scattered (0) or incident (2) field E[3 n], H[3 n] at the
 * points rt[3 n], through the boundary-value formula (memp = 0, as mo_EH_t /
 * mo_EH_s) or the potential-derivative formula (memp = 1, as mo_EH_mEMP_t /
 * mo_EH_mEMP_s, the far-field form of example4.c); quadrature type as the
 * reference's.  One domain-id and one field launch per object instead of one
 * per point; each point's value equals the per-point function's.  oid[n]
 * (may be NULL): the object containing the point, -1 outside all.  Returns 0.
 * The per-point functions (mo_EH_*, mo_mEMP_*, domain_id) may also be called
 * from several host threads at once: each thread evaluates on its own stream. */
int gb_mo_EH_points(MOBJ *mo, int n, const double *rt, int type, int which, int memp, double complex *E,
                    double complex *H, int *oid);
/* suppress (1) or restore (0) the progress messages of mo_solve_bv */
void gbh_set_quiet(int q);
/* iteration count and convergence measure cc of the last mo_solve_bv */
void gbh_last_iteration(int *iter, double *cc);
/* host wall-clock seconds of the last gbh_mscene_step: assembly, factorisation,
 * multiple-scattering iteration with E/H (mo_solve_bv), force and torque */
void gbh_mscene_phase_times(double *t);

#ifdef __cplusplus
}
#endif
#endif
