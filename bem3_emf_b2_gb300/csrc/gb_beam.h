/* gb_beam.h -- descriptor of one angular-spectrum beam for the GPU field
 * evaluation (gb_beam.cu), filled by the host beam code (host/beam.c). */
#ifndef GB_BEAM_H
#define GB_BEAM_H

typedef struct GbBeamDesc {
  int kind;         /* 0: xy-polarised pupil (fpw, lgb, bsb, blg); 1: radial/azimuthal (rab) */
  int t0, nt;       /* its polar nodes in the node table */
  int phase;        /* index of its spiral-phase table, -1 for none */
  double ki;        /* wave number in the host medium */
  double E0;        /* power coefficient */
  double cep;       /* n^2: weight of the electric energy in the stopping rule */
  double f[3];      /* focus */
  double M[9];      /* rotation into the beam frame, row-major: y = M (x - f) */
  double ex[2], ey[2], hx[2], hy[2]; /* pupil polarisation (re, im); er, ea, hr, ha for kind 1 */
} GbBeamDesc;

#define GB_BEAM_NPHI 8193  /* (2 << TRAP_MNUM) + 1 trapezoidal azimuths */

#ifdef __cplusplus
extern "C" {
#endif
/* Fields of nb beams summed at n points; x, v [n][3] (v may be NULL: no
 * derivative); E, H, dE, dH [n][3] complex as (re, im) pairs (dE, dH only
 * with v).  T polar nodes in total: item_beam[T] names each node's beam,
 * nodes[T][3] its (cos t, sin t, weight); phi[GB_BEAM_NPHI][2] the azimuths'
 * (cos, sin) in refinement order; phase[nphase][GB_BEAM_NPHI][2] spiral
 * phases.  Returns 0, 1 when an azimuthal integral did not converge within
 * the rule's halvings, -1 on a CUDA error (gb_last_error()). */
int gbi_beam_points(int nb, const GbBeamDesc* beams, int T, const int* item_beam, const double* nodes,
                    const double* phi, int nphase, const double* phase, int n, const double* x, const double* v,
                    double* E, double* H, double* dE, double* dH);
#ifdef __cplusplus
}
#endif
#endif
