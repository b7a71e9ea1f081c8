// gb_internal.h -- declarations shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#define GB_MAXDOM 16

// Device copy of one object's mesh (pointers are device addresses; the small
// per-domain tables are host copies passed to kernels by value).
typedef struct GbMeshDev {
  int Ne, NN, MN;
  double* cr;   // (Ne+1)*12
  double* cw;   // (Ne+1)*9
  double* ren;  // (Ne+1)*12
  double* wen;  // (Ne+1)*12
  int* etype;   // (Ne+1): 1 quadrangle, 0 triangle
  int* eni;     // (Ne+1)*4
  int* md;      // (Ne+1)
  int* sd;      // (Ne+1)
  int* sid;     // concatenated sid lists, domain d at sb_off[d] (1-based inside)
  double* corner; // (Ne+1)*12 corner coordinates
  int sb_Ne[GB_MAXDOM];
  int sb_off[GB_MAXDOM + 1];
  double kn[2 * GB_MAXDOM];
  int ntri, nquad;  // elements of each type (host count)
} GbMeshDev;

// one item of a work-list assembly: rows row0 .. row0 + nrow - 1 of domain did
// of the object with mesh m, into the given outputs (nrow rows each)
struct cplx;
typedef struct GbAsmItem {
  const GbMeshDev* m;
  int did, row0, nrow;
  struct cplx *G, *H, *dG, *dH;
  double* dF;
} GbAsmItem;

// one near-singular quadrangle pair handed to the learned quadrature: the
// source element, the observation node with its two tangents, the wave
// number, the sub-domain sign, and where its matrix entries and solid-angle
// terms live (G, H, dG0, dG1, dH0, dH1 rows of 4 entries; F, dF0, dF1)
typedef struct GbLqPair {
  double cr[12], cw[9];
  double rt[3], vt[6];
  double k[2];
  struct cplx* out[6];
  double* f;
  int neg;
  int gh_df;  // the pair certainly takes the GHN rule: without the network it is integrated in double-float
} GbLqPair;
typedef struct GbLqList {
  GbLqPair* p;       // null: the assembly integrates every fallback pair by the 64 x 64 rule
  unsigned* count;   // pairs offered (may exceed cap: the surplus took the 64 x 64 rule)
  unsigned cap;
  int pad;
} GbLqList;

#ifdef __cplusplus
extern "C" {
#endif
void gbi_set_error(const char* fmt, ...);
void gbi_count_launch(void);
int gbi_kt_asm_start(cudaStream_t st, void** h);
void gbi_kt_asm_stop(void* h, cudaStream_t st, double pairs);
#ifdef __cplusplus
}
#endif

#define GB_CUDA(x)                                                                         \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) {                                                               \
      gbi_set_error("%s:%d %s: %s", __FILE__, __LINE__, #x, cudaGetErrorString(e_));       \
      return -1;                                                                           \
    }                                                                                      \
  } while (0)
