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
/* device step: assembly (quadrature type), factorisation (form 0: FP64 LU +
 * explicit inverse, as the reference; form 1: complex FP32 LU + FP64
 * iterative refinement), boundary values, E/H, then the radiation force and
 * torque about rc (type-0 surface rule, mo_force_FN) */
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

#ifdef __cplusplus
}
#endif
#endif
