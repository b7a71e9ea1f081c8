// gb_assemble.cu -- coefficient-matrix assembly of one domain on the GPU.
//
// Replaces create_cmatrix_domain (reference solve_bieq2.c:98-184) and the
// element dispatch dcoef_bd_node_t2 (d3b1_elem.c:482-539):
//   rows  (t,tn): collocation node tn of element t of the domain
//   cols  (s,n) : shape function n of source element s
//   G,H   [N][N], dG,dH [2N][N] (t_zeta, t_eta), dF [N][3], N = 4 Ne,
// all in the reference's row-major .cmat layout, written straight into HBM.
//
// Kernels
//   k_asm_regular   one thread per (row, source) pair, GLN x GLN rule; pairs
//                   whose |Re dF/dt| exceeds CBD_SDF are re-integrated with the
//                   GHN x GHN rule by the whole warp cooperatively (4096 points
//                   spread over 32 lanes) instead of stalling one lane.
//   k_asm_singular  one block per row for the pair s == t (polar / principal
//                   value integrals, ~45k points split over the block).
//   k_asm_rows      per row: solid-angle sums F, dF in source order
//                   s = 1..Ne (the reference's summation order), free term
//                   1 + F (domain 0) or F on the diagonal of H.
// Per-pair solid-angle terms go through a scratch array Fs[N][Ne][3] so the
// row sums are deterministic.
//
// Precision 0: the kernels above in FP64.  Precision 2 (the chosen form):
//   k_asm_regular_df     the GLN x GLN rule of the regular pairs in
//                        double-float on the FP32 pipes (gb_quad_df.cuh);
//                        pairs near the CBD_SDF switch are flagged and
//                        integrated by k_asm_regular (FP64)
//   k_asm_singular<1>    all point sets of the singular integrals in
//                        double-float, the directions from per-row
//                        double-float constants
// with matrices that agree with precision 0 to ~1e-14.
//
// Opt-in FP32 regular pairs (precision 1, not used by the scene forms that
// are measured, because the per-pair FP32 constants -- wave number, scale,
// weights -- bias every far entry alike by ~1e-7, which moves the radiation
// force by up to ~1e-6): k_asm_regular_f32 integrates the GLN x GLN rule
// of every regular pair in FP32, relative to the source element's centre
// (the phase e^{ikR} = e^{ik|R0|} e^{ik(|R|-|R0|)}, the first factor in FP64
// once per pair, the second from the stably computed difference
// (2 R0.d + |d|^2) / (|R| + |R0|), so the phase error does not grow with the
// distance).  Pairs closer than GB_F32_NEAR element radii, and pairs whose
// FP32 |Re dF/dt| exceeds 0.45 (the CBD_SDF = 0.5 decision and its
// neighbourhood) or is not finite, are flagged and integrated by the FP64
// kernel, which makes the GLN/GHN decision exactly as the reference.
// Singular pairs stay FP64.
#include "gb_quad.cuh"
#include "gb_reduce.cuh"
#include "gb_internal.h"
#include "gb_quad_df.cuh"
#include <algorithm>
#include <mutex>
#include <vector>

#include "gb_mlp.h"



struct AsmArgs {
  const double* cr;
  const double* cw;
  const int* etype;
  const double* ren;
  const int* sid;  // signed element ids of the domain, 1-based (sid[0] unused)
  int Ne;          // elements of the domain
  cplx k;
  int type;
  int did;
  cplx* G;
  cplx* H;
  cplx* dG;
  cplx* dH;
  double* dF;
  double* Fs;      // scratch [N][Ne][3]
  const uint8_t* only;  // non-null: k_asm_regular integrates only the pairs flagged here
  int adapt;       // k_asm_regular_df: the distance-adaptive order (precision 3)
  int row0, nrow;  // the rows row0 .. row0 + nrow - 1 of the domain; outputs hold nrow rows
  uint8_t* redo;   // work-list launches: the item's flags of pairs for the FP64 pass
  GbLqList lq;     // learned quadrature: quadrangle fallback pairs listed instead of integrated
  // pairs that certainly take the GHN fallback rule, listed by the
  // double-float pass for k_asm_gh_df (null: they go to the FP64 pass)
  struct GbGhPair* gh;
  unsigned* ghn;
  unsigned ghcap;
  int item;        // this item's index in the launch's item array
};

// one pair of the GHN list: item, row (in the domain), source element index, sign
struct GbGhPair {
  int item, row, sidx, neg;
};

// unit tangents at collocation node tn of element |td| (reference tz_te_bd_node d3b1_elem.c:122-143)
__device__ __forceinline__ void node_tangents(const Elem& T, int tn, double vt[2][3]) {
  for (int d = 0; d < 3; d++) {
    if (T.quad) {
      vt[0][d] = T.cr[d][1] + T.cr[d][3] * c_tab.et_44[tn];
      vt[1][d] = T.cr[d][2] + T.cr[d][3] * c_tab.zt_44[tn];
    } else {
      vt[0][d] = T.cr[d][1];
      vt[1][d] = T.cr[d][2];
    }
  }
  for (int i = 0; i < 2; i++) {
    double a = norm3(vt[i]);
    if (a != 0.0) { vt[i][0] /= a; vt[i][1] /= a; vt[i][2] /= a; }
  }
}

__device__ __forceinline__ void store_pair(const AsmArgs& a, size_t N, int grow, int sidx, const RegAcc<2>& A) {
  const int row = grow - a.row0;  // row of the output block
  size_t col = (size_t)sidx * 4;
  cplx* g = a.G + (size_t)row * N + col;
  cplx* h = a.H + (size_t)row * N + col;
  cplx* dg0 = a.dG + ((size_t)row * 2 + 0) * N + col;
  cplx* dg1 = a.dG + ((size_t)row * 2 + 1) * N + col;
  cplx* dh0 = a.dH + ((size_t)row * 2 + 0) * N + col;
  cplx* dh1 = a.dH + ((size_t)row * 2 + 1) * N + col;
#pragma unroll
  for (int n = 0; n < 4; n++) {
    g[n] = A.G[n];
    h[n] = A.H[n];
    dg0[n] = A.dG[0][n];
    dg1[n] = A.dG[1][n];
    dh0[n] = A.dH[0][n];
    dh1[n] = A.dH[1][n];
  }
  double* f = a.Fs + ((size_t)row * a.Ne + sidx) * 3;
  f[0] = A.F;
  f[1] = A.dF[0];
  f[2] = A.dF[1];
}

// ------------------------------------------------------------------ FP32 regular pairs
#define GB_F32_NEAR 3.0  // pairs closer than this many element radii are integrated in FP64

struct GbTablesF {
  float xli[GB_GLN], wli[GB_GLN];
};
static __constant__ GbTablesF c_tabf;

// per-pair constants in FP32, relative to the source element's point (0, 0)
struct PairF {
  float R0[3];   // r_s(0,0) - r_t
  float a0;      // |R0| (FP64, rounded)
  float c1[3], c2[3], c3[3];  // r_s(z,e) - r_s(0,0) = c1 z + c2 e + c3 z e
  float w0[3], w1[3], w2[3];  // W(z,e) = w0 + w1 z + w2 e
  float vt[2][3];
  cplxf k, klo;  // k = k + klo exactly (the FP32 rounding of k would bias every far entry alike)
};

struct RegAccF {
  cplxf G[4], H[4];
  float F;
  cplxf dG[2][4], dH[2][4];
  float dF[2];
};

__device__ __forceinline__ float dot3f(const float a[3], const float b[3]) {
  return fmaf(a[0], b[0], fmaf(a[1], b[1], a[2] * b[2]));
}

// FP32 point evaluation relative to the source element's point (0,0).  The
// common factor e^{ik|R0|} of all phased sums is left out (applied in FP64 to
// the sums), the triangle's shape functions are accumulated times 3 (the 1/3
// applied in FP64), and k and sqrt(3) carry a low part: constants that would
// otherwise round alike for every pair do not bias the matrix.
__device__ __forceinline__ void reg_point_f32(const PairF& P, bool quad, float z, float e, float w, RegAccF& A) {
  float d[3], R[3], W[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    d[i] = fmaf(P.c3[i] * z, e, fmaf(P.c2[i], e, P.c1[i] * z));
    R[i] = P.R0[i] + d[i];
    W[i] = fmaf(P.w2[i], e, fmaf(P.w1[i], z, P.w0[i]));
  }
  const float aR = sqrtf(dot3f(R, R));
  const float iR = 1.0f / aR;
  const float aW = sqrtf(dot3f(W, W));
  const float dl = (2.0f * dot3f(P.R0, d) + dot3f(d, d)) / (aR + P.a0);  // |R| - |R0|
  float sn, cs;
  sincosf(P.k.x * dl, &sn, &cs);
  const float ex = (P.k.y == 0.0f) ? 1.0f : expf(-P.k.y * dl);
  const cplxf ce = cmkf(cs * ex, sn * ex);  // e^{ik(|R| - |R0|)}
  const cplxf kR = cmkf(fmaf(P.k.x, aR, P.klo.x * aR), fmaf(P.k.y, aR, P.klo.y * aR));
  const cplxf cb = cmkf(-kR.y - 1.0f, kR.x);  // i k R - 1
  const float rdW = dot3f(R, W) * iR;
  const float tD = rdW * iR * iR;
  float N[4];
  if (quad) {
    const float ia = 1.7320508f, ial = 3.1087249e-08f;  // 1 / GB_P44_N = sqrt(3), high + low
    const float za = fmaf(z, ia, z * ial), ea = fmaf(e, ia, e * ial);
    const float zm = 1.0f - za, zp = 1.0f + za, em = 1.0f - ea, ep = 1.0f + ea;
    N[0] = 0.25f * zm * em; N[1] = 0.25f * zp * em; N[2] = 0.25f * zp * ep; N[3] = 0.25f * zm * ep;
  } else {  // 3 x the shape functions (ia = 0.5 / GB_P34_N0 = 2.5 exactly)
    const float ia = 2.5f, s3 = 1.7320508f, s3l = 3.1087249e-08f;
    const float se = fmaf(s3, e, s3l * e);
    N[0] = 1.0f - ia * (z + se); N[1] = 1.0f + 2.0f * ia * z; N[2] = 1.0f - ia * (z - se);
    N[3] = 0.0f;
  }
  const cplxf g = ce * (iR * aW * w);
  const cplxf cbe = cb * ce;
  const cplxf h = cbe * (tD * w);
#pragma unroll
  for (int n = 0; n < 4; n++) { A.G[n] += g * N[n]; A.H[n] += h * N[n]; }
  A.F += w * tD;
  const cplxf t1 = kR * kR + cb * 3.0f;
  const float iR3 = iR * iR * iR;
#pragma unroll
  for (int q = 0; q < 2; q++) {
    const float rdv = dot3f(R, P.vt[q]) * iR;
    const float Wdv = dot3f(W, P.vt[q]);
    const cplxf dg = cbe * (iR * iR * rdv * aW * w);
    const cplxf dh = (ce * (t1 * (rdv * rdW) - cb * Wdv)) * (iR3 * w);
#pragma unroll
    for (int n = 0; n < 4; n++) { A.dG[q][n] += dg * N[n]; A.dH[q][n] += dh * N[n]; }
    A.dF[q] += w * iR3 * (3.0f * rdv * rdW - Wdv);
  }
}

// one thread per (row, source) pair, FP32 GLN x GLN rule; flags the pairs the
// FP64 kernel must redo
__global__ void __launch_bounds__(128) k_asm_regular_f32(AsmArgs a, uint8_t* redo) {
  const size_t N = (size_t)a.Ne * 4;
  const size_t npair = (size_t)a.nrow * (size_t)a.Ne;
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int row = a.row0 + (int)(p / a.Ne), sidx = (int)(p % a.Ne);
  const int t = row / 4 + 1, tn = row % 4;
  const int td = __ldg(a.sid + t), sd = __ldg(a.sid + sidx + 1);
  const int atd = abs(td);
  Elem T;
  load_elem(T, a.cr, a.cw, a.etype, atd);
  redo[p] = 0;
  if (!(T.quad || tn < 3) || sd == td) return;
  Elem S;
  load_elem(S, a.cr, a.cw, a.etype, abs(sd));
  double rt[3], vt[2][3];
  for (int d = 0; d < 3; d++) rt[d] = __ldg(a.ren + (size_t)atd * 12 + tn * 3 + d);
  node_tangents(T, tn, vt);
  PairF P;
  double R0[3];
  for (int d = 0; d < 3; d++) {
    R0[d] = S.cr[d][0] - rt[d];
    P.R0[d] = (float)R0[d];
    P.c1[d] = (float)S.cr[d][1]; P.c2[d] = (float)S.cr[d][2]; P.c3[d] = (float)S.cr[d][3];
    P.w0[d] = (float)S.cw[d][0]; P.w1[d] = (float)S.cw[d][1]; P.w2[d] = (float)S.cw[d][2];
    P.vt[0][d] = (float)vt[0][d]; P.vt[1][d] = (float)vt[1][d];
  }
  const double a0 = norm3(R0);
  // near pairs stay FP64: their entries are the row's largest, so their
  // relative rounding would dominate the matrix error (hs bounds |r - r(0,0)|
  // over the element)
  double hs = 0.0;
  for (int d = 0; d < 3; d++) hs += S.cr[d][1] * S.cr[d][1] + S.cr[d][2] * S.cr[d][2] + S.cr[d][3] * S.cr[d][3];
  hs = (S.quad ? 1.8 : 3.0) * sqrt(hs);
  if (a0 < GB_F32_NEAR * hs) {
    redo[p] = 1;
    return;
  }
  P.a0 = (float)a0;
  const cplx E0 = cexpik(a.k, a0);
  P.k = cmkf((float)a.k.x, (float)a.k.y);
  P.klo = cmkf((float)(a.k.x - (double)P.k.x), (float)(a.k.y - (double)P.k.y));
  RegAccF A;
#pragma unroll
  for (int n = 0; n < 4; n++) {
    A.G[n] = cmkf(0, 0); A.H[n] = cmkf(0, 0);
    A.dG[0][n] = cmkf(0, 0); A.dG[1][n] = cmkf(0, 0); A.dH[0][n] = cmkf(0, 0); A.dH[1][n] = cmkf(0, 0);
  }
  A.F = 0.f; A.dF[0] = 0.f; A.dF[1] = 0.f;
  double S0;  // scale in FP64, with the 1/3 of the triangle's shape functions
  if (S.quad) {
    S0 = GB_I_FP;
    for (int i = 0; i < GB_GLN; i++)
      for (int j = 0; j < GB_GLN; j++)
        reg_point_f32(P, true, c_tabf.xli[i], c_tabf.xli[j], c_tabf.wli[i] * c_tabf.wli[j], A);
  } else {
    S0 = 0.0625 * GB_SQ3 * GB_I_SPSQ3;
    const float s3 = 1.7320508f, s3l = 3.1087249e-08f;
    for (int i = 0; i < GB_GLN; i++) {
      const float x = c_tabf.xli[i];
      for (int j = 0; j < GB_GLN; j++) {
        const float y = c_tabf.xli[j];
        const float w = c_tabf.wli[i] * c_tabf.wli[j] * (1.0f + 0.25f * x + 0.25f * y);
        const float q1 = -x + y, q2 = 3.0f + 3.0f * x + y + x * y, q3 = -3.0f - x - 3.0f * y - x * y;
        reg_point_f32(P, false, 0.125f * (3.0f + 2.0f * x + 2.0f * y + x * y), 0.125f * fmaf(s3, q1, s3l * q1), w, A);
        reg_point_f32(P, false, 0.0625f * (-3.0f + x - 5.0f * y - x * y), 0.0625f * fmaf(s3, q2, s3l * q2), w, A);
        reg_point_f32(P, false, 0.0625f * (-3.0f - 5.0f * x + y - x * y), 0.0625f * fmaf(s3, q3, s3l * q3), w, A);
      }
    }
  }
  const double sh = sd < 0 ? -S0 : S0;
  const double s3n = S.quad ? 1.0 : 1.0 / 3.0;  // the triangle's shape functions were accumulated times 3
  const double dF0 = (double)A.dF[0] * sh, dF1 = (double)A.dF[1] * sh;
  if (!(fabs(dF0) <= 0.45 && fabs(dF1) <= 0.45)) {  // near the GLN/GHN decision (or not finite): FP64
    redo[p] = 1;
    return;
  }
  RegAcc<2> D;
  const cplx eS = E0 * (S0 * s3n), eH = E0 * (sh * s3n), eDG = E0 * (-S0 * s3n);
#pragma unroll
  for (int n = 0; n < 4; n++) {
    D.G[n] = cmk(A.G[n].x, A.G[n].y) * eS;
    D.H[n] = cmk(A.H[n].x, A.H[n].y) * eH;
    for (int q = 0; q < 2; q++) {
      D.dG[q][n] = cmk(A.dG[q][n].x, A.dG[q][n].y) * eDG;
      D.dH[q][n] = cmk(A.dH[q][n].x, A.dH[q][n].y) * eH;
    }
  }
  D.F = (double)A.F * sh;
  D.dF[0] = dF0;
  D.dF[1] = dF1;
  store_pair(a, N, row, sidx, D);
}

// ------------------------------------------------------------------ double-float regular pairs
// Precision 2: the GLN x GLN rule of the regular pairs in double-float
// (reg_integrate_dn, gb_quad_df.cuh); pairs whose |Re dF/dt| is within 0.05
// of the CBD_SDF decision (or not finite) are flagged and redone by the FP64
// kernel, which decides GLN/GHN exactly as the reference.
// TSEL: 0 every pair; 1 only pairs whose source element is a triangle
// (compiled with three shape functions' sums: fewer registers), 2 only
// quadrangle sources.  A launch of TSEL 1 or 2 writes nothing for the other
// type's pairs, so the two launches together cover each pair once.
template <int TSEL>
__device__ __forceinline__ void asm_regular_df_body(const AsmArgs& a, uint8_t* redo, unsigned bx) {
  const size_t N = (size_t)a.Ne * 4;
  const size_t npair = (size_t)a.nrow * (size_t)a.Ne;
  size_t p = (size_t)bx * blockDim.x + threadIdx.x;
  if (p >= npair) return;
  const int row = a.row0 + (int)(p / a.Ne), sidx = (int)(p % a.Ne);
  const int t = row / 4 + 1, tn = row % 4;
  const int td = __ldg(a.sid + t), sd = __ldg(a.sid + sidx + 1);
  if (TSEL != 0 && (__ldg(a.etype + abs(sd)) != 0) != (TSEL == 2)) return;
  const int atd = abs(td);
  Elem T;
  load_elem(T, a.cr, a.cw, a.etype, atd);
  redo[p] = 0;
  if (!(T.quad || tn < 3) || sd == td) return;
  Elem S;
  load_elem(S, a.cr, a.cw, a.etype, abs(sd));
  double rt[3], vt[2][3];
  for (int d = 0; d < 3; d++) rt[d] = __ldg(a.ren + (size_t)atd * 12 + tn * 3 + d);
  node_tangents(T, tn, vt);
  RegAcc<2> D;
  int why = 0;
  if (!reg_integrate_dn<2, TSEL == 1 ? 3 : 4>(S, rt, vt, a.k, sd < 0, D, a.adapt != 0, &why)) {
    // certainly the GHN rule (the FP64 decision cannot differ): listed for
    // the double-float GHN kernel instead of the FP64 pass (the learned
    // quadrature, when on, takes these pairs in the FP64 pass, flagged 2 so
    // that a reverted correction integrates them as this path does)
    redo[p] = why == 2 ? 2 : 1;
    if (why == 2 && a.gh != nullptr && a.lq.p == nullptr) {
      const unsigned slot = atomicAdd(a.ghn, 1u);
      if (slot < a.ghcap) {
        GbGhPair e;
        e.item = a.item; e.row = row; e.sidx = sidx; e.neg = sd < 0 ? 1 : 0;
        a.gh[slot] = e;
        redo[p] = 0;
      }
    }
    return;
  }
  store_pair(a, N, row, sidx, D);
}

// The listed GHN pairs in double-float: one warp per pair, the GHN x GHN
// points shared by the lanes, the sums reduced across the warp in FP64 and
// finished as reg_finish does (the FP64 pass integrates the same pairs with
// the same rule in FP64)
__global__ void __launch_bounds__(128) k_asm_gh_df(const AsmArgs* __restrict__ items, const GbGhPair* __restrict__ L,
                                                   unsigned n) {
  const unsigned w = (unsigned)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= n) return;
  const GbGhPair e = L[w];
  const AsmArgs& a = items[e.item];
  const int t = e.row / 4 + 1, tn = e.row % 4;
  const int td = __ldg(a.sid + t), sd = __ldg(a.sid + e.sidx + 1);
  const int atd = abs(td);
  Elem T, S;
  load_elem(T, a.cr, a.cw, a.etype, atd);
  load_elem(S, a.cr, a.cw, a.etype, abs(sd));
  double rt[3], vt[2][3];
  for (int d = 0; d < 3; d++) rt[d] = __ldg(a.ren + (size_t)atd * 12 + tn * 3 + d);
  node_tangents(T, tn, vt);
  RegAcc<2> R;
  cplx E0;
  reg_gh_part_dn<2>(S, rt, vt, a.k, lane, 32, R, E0);
  warp_allreduce<sizeof(RegAcc<2>) / sizeof(double)>((double*)&R);
  if (lane != 0) return;
  RegAcc<2> D;
  finish_dn<2>(R, S, e.neg != 0, E0, D);
  store_pair(a, (size_t)a.Ne * 4, e.row, e.sidx, D);
}
__global__ void __launch_bounds__(128) k_asm_regular_df(AsmArgs a, uint8_t* redo) {
  asm_regular_df_body<0>(a, redo, blockIdx.x);
}

// FP64 regular pairs (all, or those flagged in only); the whole warp
// integrates each pair that needs the GHN fallback
__device__ __forceinline__ void asm_regular_body(const AsmArgs& a, const uint8_t* only, unsigned bx) {
  const size_t N = (size_t)a.Ne * 4;
  const size_t npair = (size_t)a.nrow * (size_t)a.Ne;
  size_t p = (size_t)bx * blockDim.x + threadIdx.x;
  // a pair the flags leave out reads nothing else (the pass over the pairs a
  // double-float pass declined touches a few of them)
  bool active = p < npair && (only == nullptr || only[p] != 0);
  int row = 0, sidx = 0;
  bool work = false, fb = false;
  Elem S;
  double rt[3], vt[2][3];
  RegAcc<2> A;
  bool neg = false;
  if (active) {
    row = a.row0 + (int)(p / a.Ne);
    sidx = (int)(p % a.Ne);
    int t = row / 4 + 1, tn = row % 4;
    int td = __ldg(a.sid + t);
    int s = sidx + 1;
    int sd = __ldg(a.sid + s);
    int atd = abs(td);
    Elem T;
    load_elem(T, a.cr, a.cw, a.etype, atd);
    bool rowok = T.quad || tn < 3;
    if (rowok && sd != td) {
      work = true;
      for (int d = 0; d < 3; d++) rt[d] = __ldg(a.ren + (size_t)atd * 12 + tn * 3 + d);
      node_tangents(T, tn, vt);
      load_elem(S, a.cr, a.cw, a.etype, abs(sd));
      neg = sd < 0;
      reg_integrate<2>(S, a.type, rt, vt, a.k, neg, A);
      if (a.type < 3 && (fabs(A.dF[0]) > GB_CBD_SDF || fabs(A.dF[1]) > GB_CBD_SDF)) fb = true;
    }
  }
  // near-singular fallback: the warp integrates each flagged pair together
  unsigned mask = __ballot_sync(0xffffffffu, fb);
  const int lane = threadIdx.x & 31;
  while (mask) {
    int src = __ffs(mask) - 1;
    mask &= mask - 1;
    // learned quadrature: a quadrangle pair keeps its GLN x GLN values and is
    // listed for the network's correction (when the list has room)
    int listed = 0;
    if (lane == src && a.lq.p != nullptr && S.quad) {
      const unsigned slot = atomicAdd(a.lq.count, 1u);
      if (slot < a.lq.cap) {
        GbLqPair& q = a.lq.p[slot];
        for (int i = 0; i < 12; i++) q.cr[i] = (&S.cr[0][0])[i];
        for (int i = 0; i < 9; i++) q.cw[i] = (&S.cw[0][0])[i];
        for (int i = 0; i < 3; i++) q.rt[i] = rt[i];
        for (int i = 0; i < 6; i++) q.vt[i] = (&vt[0][0])[i];
        q.k[0] = a.k.x;
        q.k[1] = a.k.y;
        const size_t lr = (size_t)(row - a.row0), col = (size_t)sidx * 4;
        q.out[0] = (struct cplx*)(a.G + lr * N + col);
        q.out[1] = (struct cplx*)(a.H + lr * N + col);
        q.out[2] = (struct cplx*)(a.dG + (lr * 2 + 0) * N + col);
        q.out[3] = (struct cplx*)(a.dG + (lr * 2 + 1) * N + col);
        q.out[4] = (struct cplx*)(a.dH + (lr * 2 + 0) * N + col);
        q.out[5] = (struct cplx*)(a.dH + (lr * 2 + 1) * N + col);
        q.f = a.Fs + (lr * a.Ne + sidx) * 3;
        q.neg = neg ? 1 : 0;
        q.gh_df = (only != nullptr && only[p] == 2) ? 1 : 0;
        listed = 1;
      }
    }
    if (__shfl_sync(0xffffffffu, listed, src)) continue;
    // broadcast the flagged pair's geometry
    Elem Sb;
    double rtb[3], vtb[2][3];
    for (int i = 0; i < 12; i++) (&Sb.cr[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cr[0][0])[i], src);
    for (int i = 0; i < 9; i++) (&Sb.cw[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cw[0][0])[i], src);
    Sb.quad = __shfl_sync(0xffffffffu, S.quad, src);
    for (int i = 0; i < 3; i++) rtb[i] = __shfl_sync(0xffffffffu, rt[i], src);
    for (int i = 0; i < 6; i++) (&vtb[0][0])[i] = __shfl_sync(0xffffffffu, (&vt[0][0])[i], src);
    bool negb = __shfl_sync(0xffffffffu, (int)neg, src) != 0;
    RegAcc<2> B;
    reg_integrate_gh_part<2>(Sb, lane, 32, rtb, vtb, a.k, B);
    warp_allreduce<sizeof(RegAcc<2>) / sizeof(double)>((double*)&B);
    reg_finish<2>(B, reg_scale_gh(Sb), negb);
    if (lane == src) A = B;
  }
  if (work) store_pair(a, N, row, sidx, A);
}
__global__ void __launch_bounds__(128) k_asm_regular(AsmArgs a) { asm_regular_body(a, a.only, blockIdx.x); }

// ---- double-float set B of the singular pairs (precision 2)
// The derivative integrals on [DEPS, rm] with the GHN rule (sing_bil_setB /
// sing_lit_setB of gb_quad.cuh, reference bil_dcoef.c / lit_dcoef.c D-bar_eps
// parts) take 64 of every ~88 points of a singular row; here they run in
// double-float.  The geometry along the ray is affine in r (K = Ka + Kb r,
// W = Wa + Wb r, per direction in FP64), each direction's sums are kept in
// double-float and added to the FP64 accumulators.
struct SingAccB {
  dfc dG[2][4], dH[2][4];
  df dF[2];
};

__device__ __forceinline__ void singb_add(const SingAccB& B, SingAcc& A, int nsh, double scale) {
#pragma unroll
  for (int d = 0; d < 2; d++) {
#pragma unroll
    for (int n = 0; n < 4; n++) {
      if (n >= nsh) break;
      A.dG[d][n] += cmk(df_to(B.dG[d][n].re), df_to(B.dG[d][n].im)) * scale;
      A.dH[d][n] += cmk(df_to(B.dH[d][n].re), df_to(B.dH[d][n].im)) * scale;
    }
    A.dF[d] += df_to(B.dF[d]);
  }
}

__device__ __forceinline__ void singb_zero(SingAccB& B) {
  const df z = dfmk(0.0f, 0.0f);
#pragma unroll
  for (int d = 0; d < 2; d++) {
#pragma unroll
    for (int n = 0; n < 4; n++) { B.dG[d][n] = dfcmk(z, z); B.dH[d][n] = dfcmk(z, z); }
    B.dF[d] = z;
  }
}

// Per-row constants in double-float, set once per block from the FP64
// polar decomposition (sing_setup): along a ray in direction (c, s) from
// (zt, et), K = Ka + Kb r with Ka = a1 c + a2 s (a1 = cr1 + cr3 et,
// a2 = cr2 + cr3 zt; triangles: cr1, cr2) and Kb = cr3 c s, and
// W = Wa + (w1 c + w2 s) r; per edge j the end angles t0, t1 with their
// cosines and sines, the end radii r0, r1 and sin(t1 - t0), so that the
// distance to the edge along theta, r0 r1 sin(t1 - t0) / (r0 sin(theta - t0)
// - r1 sin(theta - t1)), needs no further transcendental.
struct RowD {
  df a1[3], a2[3], c3[3], Wa[3], w1[3], w2[3], vt[2][3];
  df zt, et, kr, ki;
  df t0[4], dt[4], ct0[4], st0[4], ct1[4], st1[4], r0[4], r1[4], sdt[4];
};
__device__ void row_setup_df(const SingCtx& c, RowD& R) {
  const Elem& E = c.E;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (E.quad) {
      R.a1[d] = df_from(E.cr[d][1] + E.cr[d][3] * c.et);
      R.a2[d] = df_from(E.cr[d][2] + E.cr[d][3] * c.zt);
      R.c3[d] = df_from(E.cr[d][3]);
    } else {
      R.a1[d] = df_from(E.cr[d][1]);
      R.a2[d] = df_from(E.cr[d][2]);
      R.c3[d] = dfmk(0.0f, 0.0f);
    }
    R.Wa[d] = df_from(E.cw[d][0] + E.cw[d][1] * c.zt + E.cw[d][2] * c.et);
    R.w1[d] = df_from(E.cw[d][1]);
    R.w2[d] = df_from(E.cw[d][2]);
    R.vt[0][d] = df_from(c.vt[0][d]);
    R.vt[1][d] = df_from(c.vt[1][d]);
  }
  R.zt = df_from(c.zt);
  R.et = df_from(c.et);
  R.kr = df_from(c.k.x);
  R.ki = df_from(c.k.y);
  for (int j = 0; j < c.nedge; j++) {
    const double t0 = c.th[j], t1 = c.th[j + 1];
    R.t0[j] = df_from(t0);
    R.dt[j] = df_from(t1 - t0);
    R.ct0[j] = df_from(cos(t0));
    R.st0[j] = df_from(sin(t0));
    R.ct1[j] = df_from(cos(t1));
    R.st1[j] = df_from(sin(t1));
    R.r0[j] = df_from(c.r[j]);
    R.r1[j] = df_from(c.r[j + 1]);
    R.sdt[j] = df_from(sin(t1 - t0));
  }
}

// per-direction geometry of a ray from (zt, et) in direction (c, s) of a
// bilinear element, affine in the distance r: K = Ka + Kb r, W = Wa + Wb r
struct RayD {
  df Ka[3], Kb[3], Wa[3], Wb[3], vt[2][3];
  df zt, et, c, s, kr, ki;
};
__device__ __forceinline__ void ray_geom_df(const RowD& R, df cth, df sth, RayD& g) {
  const df cs = df_mul(cth, sth);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    g.Ka[d] = df_fma(df_mul(R.a1[d], cth), R.a2[d], sth);
    g.Kb[d] = df_mul(R.c3[d], cs);
    g.Wa[d] = R.Wa[d];
    g.Wb[d] = df_fma(df_mul(R.w1[d], cth), R.w2[d], sth);
    g.vt[0][d] = R.vt[0][d];
    g.vt[1][d] = R.vt[1][d];
  }
  g.zt = R.zt;
  g.et = R.et;
  g.c = cth;
  g.s = sth;
  g.kr = R.kr;
  g.ki = R.ki;
}
// point at signed distance rr (sg = -1: the opposite ray, whose K keeps the
// +direction terms except the r-term, as the reference's principal-value
// pairing): K, W and the bilinear shape functions
__device__ __forceinline__ void ray_point_df(const RayD& g, df rr, float sg, df K[3], df W[3], df N[4]) {
  const df r = df_mul_f(rr, sg);
#pragma unroll
  for (int d = 0; d < 3; d++) {
    K[d] = df_fma(g.Ka[d], g.Kb[d], r);
    W[d] = df_fma(g.Wa[d], g.Wb[d], r);
  }
  const df ia = dfmk(1.7320507764816284f, 3.1087250107475484e-08f);  // 1 / GB_P44_N = sqrt(3)
  const df za = df_mul(df_fma(g.zt, r, g.c), ia), ea = df_mul(df_fma(g.et, r, g.s), ia);
  const df zm = df_add_f(df_neg(za), 1.0f), zp = df_add_f(za, 1.0f);
  const df em = df_add_f(df_neg(ea), 1.0f), ep = df_add_f(ea, 1.0f);
  N[0] = df_mul_f(df_mul(zm, em), 0.25f);
  N[1] = df_mul_f(df_mul(zp, em), 0.25f);
  N[2] = df_mul_f(df_mul(zp, ep), 0.25f);
  N[3] = df_mul_f(df_mul(zm, ep), 0.25f);
}

static __device__ void sing_bil_setB_df(const SingCtx& c, const RowD& R, df cth, df sth, df rm, df wth,
                                        SingAcc& A) {
  RayD g;
  ray_geom_df(R, cth, sth, g);
  const df deps = dfmk(0.1f, -1.4901161415892261e-09f);  // GB_DEPS = 0.1 in double-float
  const df hr = df_mul_f(df_sub(rm, deps), 0.5f), r0 = df_mul_f(df_add(rm, deps), 0.5f);
  const df w0 = df_mul(wth, hr);
  const df cs[2] = {g.c, g.s}, outer[2] = {g.s, g.c};
  SingAccB B;
  singb_zero(B);
  for (int i = 0; i < GB_GHN; i++) {
    const df rr = df_fma(r0, hr, dfmk(c_tabd.xh[i].x, c_tabd.xh[i].y));
    const df w = df_mul(w0, dfmk(c_tabd.wh[i].x, c_tabd.wh[i].y));
    df K[3], W[3], N[4];
    ray_point_df(g, rr, 1.0f, K, W, N);
    const df aK2 = dot3d(K, K);
    const df aK = df_sqrt(aK2), aW = df_sqrt(dot3d(W, W));
    const df iK = df_rcp(aK), irr = df_rcp(rr);
    const df x = df_mul(aK, rr);
    const dfc kR = dfcmk(df_mul(g.kr, x), df_mul(g.ki, x));
    const dfc ce = dfc_expik(g.kr, g.ki, x);
    const dfc cb = dfcmk(df_add_f(df_neg(kR.im), -1.0f), kR.re);
    const dfc cbce = dfc_mul(cb, ce);
    const df iK2 = df_sqr(iK);
    const df gs = df_mul(df_mul(df_mul(w, iK2), df_mul(irr, iK)), aW);
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const df KdT = dot3d(K, g.vt[d]);
      const dfc gg = dfc_scale(cbce, df_mul(gs, KdT));
#pragma unroll
      for (int n = 0; n < 4; n++) B.dG[d][n] = dfc_fma_re(B.dG[d][n], gg, N[n]);
    }
    if (!c.planar) {
      const dfc t1 = dfc_add(dfc_mul(kR, kR), dfcmk(df_mul_f(cb.re, 3.0f), df_mul_f(cb.im, 3.0f)));
      const df iK5r = df_mul(df_mul(df_sqr(iK2), iK), irr);
#pragma unroll
      for (int d = 0; d < 2; d++) {
        const df KdT = dot3d(K, g.vt[d]);
        const df wo = df_mul(df_mul(w, outer[d]), iK5r);
        const df kc = df_mul(KdT, cs[d]);
        const dfc u = dfc_add(dfc_scale(t1, kc), dfc_scale(cb, df_neg(aK2)));
        const dfc h = dfc_scale(dfc_mul(ce, u), wo);
#pragma unroll
        for (int n = 0; n < 4; n++) B.dH[d][n] = dfc_fma_re(B.dH[d][n], h, N[n]);
        B.dF[d] = df_fma(B.dF[d], wo, df_sub(df_mul_f(kc, 3.0f), aK2));
      }
    }
  }
  singb_add(B, A, 4, 1.0);
}

// set A: G, H, F on [0, rm] with the GLN rule (sing_bil_setA)
static __device__ void sing_bil_setA_df(const SingCtx& c, const RowD& R, df cth, df sth, df rm, df wth,
                                        SingAcc& A) {
  RayD g;
  ray_geom_df(R, cth, sth, g);
  const df hr = df_mul_f(rm, 0.5f), w0 = df_mul(wth, hr), csn = df_mul(cth, sth);
  const df zero = dfmk(0.0f, 0.0f);
  dfc Gs[4], Hs[4];
  df Fs = zero;
#pragma unroll
  for (int n = 0; n < 4; n++) { Gs[n] = dfcmk(zero, zero); Hs[n] = dfcmk(zero, zero); }
  for (int i = 0; i < GB_GLN; i++) {
    const df rr = df_mul(hr, df_add_f(dfmk(c_tabd.x[i].x, c_tabd.x[i].y), 1.0f));
    const df w = df_mul(w0, dfmk(c_tabd.w[i].x, c_tabd.w[i].y));
    df K[3], W[3], N[4];
    ray_point_df(g, rr, 1.0f, K, W, N);
    const df aK = df_sqrt(dot3d(K, K)), aW = df_sqrt(dot3d(W, W));
    const df iK = df_rcp(aK);
    const df x = df_mul(aK, rr);
    const dfc ce = dfc_expik(g.kr, g.ki, x);
    const dfc gg = dfc_scale(ce, df_mul(df_mul(w, aW), iK));
#pragma unroll
    for (int n = 0; n < 4; n++) Gs[n] = dfc_fma_re(Gs[n], gg, N[n]);
    if (!c.planar) {
      const df wk = df_mul(df_mul(w, df_mul(df_sqr(iK), iK)), csn);
      const dfc kR = dfcmk(df_mul(g.kr, x), df_mul(g.ki, x));
      const dfc cb = dfcmk(df_add_f(df_neg(kR.im), -1.0f), kR.re);
      const dfc h = dfc_scale(dfc_mul(cb, ce), wk);
#pragma unroll
      for (int n = 0; n < 4; n++) Hs[n] = dfc_fma_re(Hs[n], h, N[n]);
      Fs = df_add(Fs, wk);
    }
  }
#pragma unroll
  for (int n = 0; n < 4; n++) {
    A.G[n] += cmk(df_to(Gs[n].re), df_to(Gs[n].im));
    A.H[n] += cmk(df_to(Hs[n].re), df_to(Hs[n].im));
  }
  A.F += df_to(Fs);
}

// set C: the disc D_eps, r in [0, DEPS] with the GLN rule (sing_bil_setC)
static __device__ void sing_bil_setC_df(const SingCtx& c, const RowD& R, df cth, df sth, df wth, SingAcc& A) {
  RayD g;
  ray_geom_df(R, cth, sth, g);
  const df hr = df_from(0.5 * GB_DEPS), w0 = df_mul(wth, hr);
  const df cs[2] = {g.c, g.s}, outer[2] = {g.s, g.c};
  const dfc k = dfcmk(g.kr, g.ki), ik = dfcmk(df_neg(g.ki), g.kr);
  const dfc ik3 = dfcmk(df_mul_f(ik.re, 3.0f), df_mul_f(ik.im, 3.0f));
  SingAccB B;
  singb_zero(B);
  for (int i = 0; i < GB_GLN; i++) {
    const df rr = df_mul(hr, df_add_f(dfmk(c_tabd.x[i].x, c_tabd.x[i].y), 1.0f));
    const df w = df_mul(w0, dfmk(c_tabd.w[i].x, c_tabd.w[i].y));
    df K[3], W[3], N[4];
    ray_point_df(g, rr, 1.0f, K, W, N);
    const df aK2 = dot3d(K, K);
    const df aK = df_sqrt(aK2), aW = df_sqrt(dot3d(W, W));
    const df iK = df_rcp(aK), irr = df_rcp(rr);
    const df x = df_mul(aK, rr);
    const dfc kR = dfcmk(df_mul(g.kr, x), df_mul(g.ki, x));
    const dfc cb = dfcmk(df_add_f(df_neg(kR.im), -1.0f), kR.re);
    dfc cc, sn;
    dfc_cossin(kR, &cc, &sn);
    const dfc ce = dfc_expik(g.kr, g.ki, x);
    const dfc gbase = dfc_muli(dfc_add(dfc_mul(cb, sn), dfc_mul(kR, cc)));
    const df gs = df_mul(df_mul(df_mul(w, df_sqr(iK)), df_mul(irr, iK)), aW);
    const df iK4 = df_sqr(df_sqr(iK));
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const df KdT = dot3d(K, g.vt[d]);
      const dfc gg = dfc_scale(gbase, df_mul(gs, KdT));
#pragma unroll
      for (int n = 0; n < 4; n++) B.dG[d][n] = dfc_fma_re(B.dG[d][n], gg, N[n]);
      if (!c.planar) {
        const df wo = df_mul(w, outer[d]);
        const df kc = df_mul(KdT, cs[d]);
        const dfc u = dfc_sub(dfc_scale(dfc_add(dfc_mul(k, kR), ik3), kc), dfc_scale(ik, aK2));
        const dfc v0 = dfc_scale(dfc_mul(ce, u), iK4);
        const dfc v1 = dfc_scale(sn, df_mul(df_mul(df_sub(df_mul_f(kc, 3.0f), aK2), df_mul(iK4, iK)), irr));
        const dfc h = dfc_scale(dfc_sub(v0, dfc_muli(v1)), wo);
#pragma unroll
        for (int n = 0; n < 4; n++) B.dH[d][n] = dfc_fma_re(B.dH[d][n], h, N[n]);
      }
    }
  }
  singb_add(B, A, 4, 1.0);
}

// set D: principal-value pairing of +r and -r, r in [0, DEPS] (sing_bil_setD)
static __device__ void sing_bil_setD_df(const SingCtx& c, const RowD& R, df cth, df sth, df wth, SingAcc& A) {
  RayD g;
  ray_geom_df(R, cth, sth, g);
  const df hr = df_from(0.5 * GB_DEPS), w0 = df_mul(wth, hr);
  const df cs[2] = {g.c, g.s}, outer[2] = {g.s, g.c};
  SingAccB B;
  singb_zero(B);
  for (int i = 0; i < GB_GLN; i++) {
    const df rr = df_mul(hr, df_add_f(dfmk(c_tabd.x[i].x, c_tabd.x[i].y), 1.0f));
    const df w = df_mul(w0, dfmk(c_tabd.w[i].x, c_tabd.w[i].y));
    df Kp[3], Wp[3], Np[4], Km[3], Wm[3], Nm[4];
    ray_point_df(g, rr, 1.0f, Kp, Wp, Np);
    ray_point_df(g, rr, -1.0f, Km, Wm, Nm);
    const df aKp2 = dot3d(Kp, Kp), aKm2 = dot3d(Km, Km);
    const df aKp = df_sqrt(aKp2), aWp = df_sqrt(dot3d(Wp, Wp));
    const df aKm = df_sqrt(aKm2), aWm = df_sqrt(dot3d(Wm, Wm));
    const df iKp = df_rcp(aKp), iKm = df_rcp(aKm), ir = df_rcp(rr);
    const df xp = df_mul(aKp, rr), xm = df_neg(df_mul(aKm, rr));
    dfc ccp, snp, ccm, snm;
    dfc_cossin(dfcmk(df_mul(g.kr, xp), df_mul(g.ki, xp)), &ccp, &snp);
    dfc_cossin(dfcmk(df_mul(g.kr, xm), df_mul(g.ki, xm)), &ccm, &snm);
    const df iKp2 = df_sqr(iKp), iKm2 = df_sqr(iKm);
    const df iKp5 = df_mul(df_sqr(iKp2), iKp), iKm5 = df_mul(df_sqr(iKm2), iKm);
    const df gsp = df_mul(df_mul(df_mul(w, ir), df_mul(iKp2, iKp)), aWp);
    const df gsm = df_mul(df_mul(df_mul(w, ir), df_mul(iKm2, iKm)), aWm);
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const df KpdT = dot3d(Kp, g.vt[d]), KmdT = dot3d(Km, g.vt[d]);
      const dfc gp = dfc_scale(ccp, df_mul(gsp, KpdT));
      const dfc gm = dfc_scale(ccm, df_mul(gsm, KmdT));
#pragma unroll
      for (int n = 0; n < 4; n++) {
        const dfc t = dfc_sub(dfcmk(df_mul(gp.re, Np[n]), df_mul(gp.im, Np[n])),
                              dfcmk(df_mul(gm.re, Nm[n]), df_mul(gm.im, Nm[n])));
        B.dG[d][n] = dfc_sub(B.dG[d][n], t);
      }
      if (!c.planar) {
        const df wo = df_mul(df_mul(w, outer[d]), ir);
        const df fp = df_mul(iKp5, df_sub(df_mul_f(df_mul(KpdT, cs[d]), 3.0f), aKp2));
        const df fm = df_mul(iKm5, df_sub(df_mul_f(df_mul(KmdT, cs[d]), 3.0f), aKm2));
        const dfc hp = dfc_scale(ccp, df_mul(wo, fp)), hm = dfc_scale(ccm, df_mul(wo, fm));
#pragma unroll
        for (int n = 0; n < 4; n++) {
          const dfc t = dfc_sub(dfcmk(df_mul(hp.re, Np[n]), df_mul(hp.im, Np[n])),
                                dfcmk(df_mul(hm.re, Nm[n]), df_mul(hm.im, Nm[n])));
          B.dH[d][n] = dfc_sub(B.dH[d][n], t);
        }
        B.dF[d] = df_fma(B.dF[d], wo, df_sub(fp, fm));
      }
    }
  }
  singb_add(B, A, 4, 1.0);
}

// triangle set A: G on [0, rm] with the GLN rule; K is constant along the
// ray; 3 x the shape functions, the 1/3 applied in FP64
static __device__ void sing_lit_setA_df(const SingCtx& c, const RowD& R, df dc, df ds, df rm, df wth,
                                        SingAcc& A) {
  df K[3];
#pragma unroll
  for (int d = 0; d < 3; d++) K[d] = df_fma(df_mul(R.a1[d], dc), R.a2[d], ds);
  const df daK = df_sqrt(dot3d(K, K)), iaK = df_rcp(daK);
  const df hr = df_mul_f(rm, 0.5f), w0 = df_mul(wth, hr);
  const df dzt = R.zt, det = R.et;
  const df kr = R.kr, ki = R.ki;
  const df s3 = dfmk(1.7320507764816284f, 3.1087250107475484e-08f);
  const df zero = dfmk(0.0f, 0.0f);
  dfc Gs[3];
#pragma unroll
  for (int n = 0; n < 3; n++) Gs[n] = dfcmk(zero, zero);
  for (int i = 0; i < GB_GLN; i++) {
    const df rr = df_mul(hr, df_add_f(dfmk(c_tabd.x[i].x, c_tabd.x[i].y), 1.0f));
    const df w = df_mul(w0, dfmk(c_tabd.w[i].x, c_tabd.w[i].y));
    const dfc ce = dfc_expik(kr, ki, df_mul(daK, rr));
    const df z = df_fma(dzt, rr, dc), e = df_fma(det, rr, ds);
    const df se = df_mul(s3, e);
    df N[3];
    N[0] = df_add_f(df_mul_f(df_add(z, se), -2.5f), 1.0f);
    N[1] = df_add_f(df_mul_f(z, 5.0f), 1.0f);
    N[2] = df_add_f(df_mul_f(df_sub(z, se), -2.5f), 1.0f);
    const dfc gg = dfc_scale(ce, df_mul(w, iaK));
#pragma unroll
    for (int n = 0; n < 3; n++) Gs[n] = dfc_fma_re(Gs[n], gg, N[n]);
  }
#pragma unroll
  for (int n = 0; n < 3; n++) A.G[n] += cmk(df_to(Gs[n].re), df_to(Gs[n].im)) * (1.0 / 3.0);
}

// triangle: K is constant along the ray; 3 x the shape functions in
// double-float, the 1/3 applied in FP64
static __device__ void sing_lit_setB_df(const SingCtx& c, const RowD& R, df dc, df ds, df rm, df wth,
                                        SingAcc& A) {
  df K[3];
#pragma unroll
  for (int d = 0; d < 3; d++) K[d] = df_fma(df_mul(R.a1[d], dc), R.a2[d], ds);
  const df daK = df_sqrt(dot3d(K, K)), iK = df_rcp(daK);
  const df kv[2] = {df_mul(dot3d(K, R.vt[0]), iK), df_mul(dot3d(K, R.vt[1]), iK)};
  const df iK2 = df_sqr(iK);
  const df deps = dfmk(0.1f, -1.4901161415892261e-09f);  // GB_DEPS = 0.1 in double-float
  const df hr = df_mul_f(df_sub(rm, deps), 0.5f), r0 = df_mul_f(df_add(rm, deps), 0.5f);
  const df w0 = df_mul(wth, hr);
  const df dzt = R.zt, det = R.et;
  const df kr = R.kr, ki = R.ki;
  const df s3 = dfmk(1.7320507764816284f, 3.1087250107475484e-08f);
  SingAccB B;
  singb_zero(B);
  for (int i = 0; i < GB_GHN; i++) {
    const df rr = df_fma(r0, hr, dfmk(c_tabd.xh[i].x, c_tabd.xh[i].y));
    const df w = df_mul(w0, dfmk(c_tabd.wh[i].x, c_tabd.wh[i].y));
    const df x = df_mul(daK, rr);
    const dfc kR = dfcmk(df_mul(kr, x), df_mul(ki, x));
    df sn, co;
    df_sincos(kR.re, &sn, &co);
    dfc ce = dfcmk(co, sn);
    if (ki.hi != 0.0f) ce = dfc_scale(ce, df_exp(df_neg(kR.im)));
    const dfc cb = dfcmk(df_add_f(df_neg(kR.im), -1.0f), kR.re);
    const df z = df_fma(dzt, rr, dc), e = df_fma(det, rr, ds);
    const df se = df_mul(s3, e);
    df N[3];
    N[0] = df_add_f(df_mul_f(df_add(z, se), -2.5f), 1.0f);
    N[1] = df_add_f(df_mul_f(z, 5.0f), 1.0f);
    N[2] = df_add_f(df_mul_f(df_sub(z, se), -2.5f), 1.0f);
    const dfc base = dfc_scale(dfc_mul(cb, ce), df_mul(df_mul(w, df_rcp(rr)), iK2));
#pragma unroll
    for (int d = 0; d < 2; d++) {
      const dfc g = dfc_scale(base, kv[d]);
#pragma unroll
      for (int n = 0; n < 3; n++) B.dG[d][n] = dfc_fma_re(B.dG[d][n], g, N[n]);
    }
  }
  singb_add(B, A, 3, 1.0 / 3.0);
}

// sing_item with the point sets in double-float, the directions too: theta,
// its weight, cos and sin and the distance to the edge from the row's
// double-float constants (the triangle's analytic sets C and D stay FP64:
// one evaluation per direction)
static __device__ void sing_item_df(const SingCtx& c, const RowD& R, int q, SingAcc& A) {
  const int nA = c.nedge * 2 * GB_GHN;
  if (q < 2 * nA) {
    const int setB = q >= nA;
    const int qq = setB ? q - nA : q;
    const int j = qq / (2 * GB_GHN), rem = qq % (2 * GB_GHN);
    const int h = rem / GB_GHN, m = rem % GB_GHN;
    const df x = dfmk(c_tabd.xh[m].x, c_tabd.xh[m].y), wx = dfmk(c_tabd.wh[m].x, c_tabd.wh[m].y);
    // theta = t0 + dt (x/4 + 1/4) (first half of the edge) or + dt (x/4 + 3/4)
    const df th = df_fma(R.t0[j], R.dt[j], df_add_f(df_mul_f(x, 0.25f), h == 0 ? 0.25f : 0.75f));
    const df wth = df_mul_f(df_mul(R.dt[j], wx), 0.25f);
    df sn, cs;
    df_sincos(th, &sn, &cs);
    const df den = df_sub(df_mul(R.r0[j], df_fma(df_mul(sn, R.ct0[j]), df_neg(cs), R.st0[j])),
                          df_mul(R.r1[j], df_fma(df_mul(sn, R.ct1[j]), df_neg(cs), R.st1[j])));
    const df rm = df_div(df_mul(df_mul(R.r0[j], R.r1[j]), R.sdt[j]), den);
    if (c.E.quad) {
      if (setB) sing_bil_setB_df(c, R, cs, sn, rm, wth, A);
      else sing_bil_setA_df(c, R, cs, sn, rm, wth, A);
    } else {
      if (setB) sing_lit_setB_df(c, R, cs, sn, rm, wth, A);
      else sing_lit_setA_df(c, R, cs, sn, rm, wth, A);
    }
    return;
  }
  if (!c.E.quad) {
    sing_item(c, q, A);
    return;
  }
  q -= 2 * nA;
  const df qpi = dfmk(0.7853981852531433f, -2.1855694143368964e-08f);  // pi / 4
  if (q < 4 * GB_GHN) {  // set C: theta over (-pi, pi] in four quarters, centres -3pi/4 .. 3pi/4
    const int quarter = q / GB_GHN, m = q % GB_GHN;
    const df x = dfmk(c_tabd.xh[m].x, c_tabd.xh[m].y), wx = dfmk(c_tabd.wh[m].x, c_tabd.wh[m].y);
    const df th = df_mul(qpi, df_add_f(x, (float)(2 * quarter - 3)));
    df sn, cs;
    df_sincos(th, &sn, &cs);
    sing_bil_setC_df(c, R, cs, sn, df_mul(qpi, wx), A);
    return;
  }
  q -= 4 * GB_GHN;
  {  // set D: theta over (0, pi) in two halves, centres pi/4 and 3pi/4
    const int half = q / GB_GHN, m = q % GB_GHN;
    const df x = dfmk(c_tabd.xh[m].x, c_tabd.xh[m].y), wx = dfmk(c_tabd.wh[m].x, c_tabd.wh[m].y);
    const df th = df_mul(qpi, df_add_f(x, half == 0 ? 1.0f : 3.0f));
    df sn, cs;
    df_sincos(th, &sn, &cs);
    sing_bil_setD_df(c, R, cs, sn, df_mul(qpi, wx), A);
  }
}

template <bool DF>
__device__ __forceinline__ void asm_singular_body(const AsmArgs& a, unsigned bx) {
  __shared__ double red[51 * 8];
  const int row = a.row0 + (int)bx;
  const int t = row / 4 + 1, tn = row % 4;
  const int td = __ldg(a.sid + t);
  const int atd = abs(td);
  SingCtx c;
  load_elem(c.E, a.cr, a.cw, a.etype, atd);
  if (!c.E.quad && tn == 3) return;
  c.zt = c.E.quad ? c_tab.zt_44[tn] : c_tab.zt_34[tn];
  c.et = c.E.quad ? c_tab.et_44[tn] : c_tab.et_34[tn];
  c.k = a.k;
  sing_setup(c);
  SingAcc A;
  singacc_zero(A);
  int nit = sing_items(c, 1);
  if (DF) {
    __shared__ RowD R;
    if (threadIdx.x == 0) row_setup_df(c, R);
    __syncthreads();
    for (int q = threadIdx.x; q < nit; q += blockDim.x) sing_item_df(c, R, q, A);
  } else {
    for (int q = threadIdx.x; q < nit; q += blockDim.x) sing_item(c, q, A);
  }
  static_assert(sizeof(SingAcc) == 51 * sizeof(double), "SingAcc layout");
  block_reduce<51>((double*)&A, red);
  if (threadIdx.x == 0) {
    sing_finish(c, A, td < 0);
    RegAcc<2> R;
    for (int n = 0; n < 4; n++) {
      R.G[n] = A.G[n];
      R.H[n] = A.H[n];
      R.dG[0][n] = A.dG[0][n];
      R.dG[1][n] = A.dG[1][n];
      R.dH[0][n] = A.dH[0][n];
      R.dH[1][n] = A.dH[1][n];
    }
    R.F = A.F;
    R.dF[0] = A.dF[0];
    R.dF[1] = A.dF[1];
    store_pair(a, (size_t)a.Ne * 4, row, t - 1, R);
  }
}
template <bool DF>
__global__ void __launch_bounds__(256) k_asm_singular(AsmArgs a) { asm_singular_body<DF>(a, blockIdx.x); }

__device__ __forceinline__ void asm_rows_body(const AsmArgs& a, unsigned bx) {
  const size_t N = (size_t)a.Ne * 4;
  const int lr = (int)bx * blockDim.x + threadIdx.x;  // row of the output block
  if (lr >= a.nrow) return;
  const int row = a.row0 + lr;
  int t = row / 4 + 1, tn = row % 4;
  int td = __ldg(a.sid + t);
  if (__ldg(a.etype + abs(td)) == 0 && tn == 3) return;
  const double* f = a.Fs + (size_t)lr * a.Ne * 3;
  double F = 0.0, Fz = 0.0, Fe = 0.0;
  for (int s = 0; s < a.Ne; s++) {
    F += f[3 * s + 0];
    Fz += f[3 * s + 1];
    Fe += f[3 * s + 2];
  }
  double diag = (a.did == 0) ? 1.0 + F : F;
  cplx* h = a.H + (size_t)lr * N + (size_t)(t - 1) * 4 + tn;
  h->x += diag;
  a.dF[(size_t)lr * 3 + 0] = diag;
  a.dF[(size_t)lr * 3 + 1] = Fz;
  a.dF[(size_t)lr * 3 + 2] = Fe;
}
__global__ void k_asm_rows(AsmArgs a) { asm_rows_body(a, blockIdx.x); }

// ---- work-list launches: one launch per phase over items of uneven size
// (every domain of every object of a scene).  Item i owns the blocks
// blk0[i] .. blk0[i + 1] - 1 of the launch; a block finds its item by binary
// search and runs the single-domain body with its local block index.
__device__ __forceinline__ int find_item(const unsigned* __restrict__ blk0, int nitems, unsigned b) {
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (blk0[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
// resident blocks of 128 threads per SM the list kernel is compiled for
// (quadrangle sources; GB_ASM_TRI_MINB for the triangle-only variant)
#ifndef GB_ASM_MINB
#define GB_ASM_MINB 3
#endif
#ifndef GB_ASM_TRI_MINB
#define GB_ASM_TRI_MINB 4
#endif
template <int TSEL>
__global__ void __launch_bounds__(128, TSEL == 1 ? GB_ASM_TRI_MINB : GB_ASM_MINB) k_asm_regular_df_list(const AsmArgs* __restrict__ items,
                                                             const unsigned* __restrict__ blk0, int nitems) {
  const int i = find_item(blk0, nitems, blockIdx.x);
  asm_regular_df_body<TSEL>(items[i], items[i].redo, blockIdx.x - blk0[i]);
}
__global__ void __launch_bounds__(128) k_asm_regular_list(const AsmArgs* __restrict__ items,
                                                          const unsigned* __restrict__ blk0, int nitems, int flagged) {
  const int i = find_item(blk0, nitems, blockIdx.x);
  asm_regular_body(items[i], flagged ? items[i].redo : nullptr, blockIdx.x - blk0[i]);
}
template <bool DF>
__global__ void __launch_bounds__(256) k_asm_singular_list(const AsmArgs* __restrict__ items,
                                                           const unsigned* __restrict__ blk0, int nitems) {
  const int i = find_item(blk0, nitems, blockIdx.x);
  asm_singular_body<DF>(items[i], blockIdx.x - blk0[i]);
}
__global__ void k_asm_rows_list(const AsmArgs* __restrict__ items, const unsigned* __restrict__ blk0, int nitems) {
  const int i = find_item(blk0, nitems, blockIdx.x);
  asm_rows_body(items[i], blockIdx.x - blk0[i]);
}

// ------------------------------------------------------------------ learned quadrature
// A near-singular quadrangle pair that needs the reference's fallback rule
// (|Re dF| > CBD_SDF: the 64 x 64 rule, d3b1_elem.c:503-504,
// bil_dcoef_v2.c:235-326) keeps its 12 x 12 values and is listed; a network
// then predicts the difference between the two rules.  Inputs (20, invariant
// under rigid motions and scaling): the element's corners in a frame at the
// observation node (z along the normal at the element's centre, x along the
// first edge) divided by the element size h = 2 sqrt|W(0,0)|, the node's two
// tangents in that frame, and k h.  Outputs (51): the 64 x 64 minus 12 x 12
// difference of G/h, H, dG, dH h, F and dF h (G, H, dG, dH complex, four
// shape functions, two tangents) for the element's own orientation; the
// sub-domain sign flips H, F, dH, dF as reg_finish does.  Every assembly
// checks the corrected values of a sample of its listed pairs against the
// 64 x 64 rule and integrates all listed pairs by that rule if the sample's
// RMS error exceeds the tolerance.
#define GB_LQ_NIN 20
#define GB_LQ_NOUT 51

__device__ __forceinline__ void lq_elem(const GbLqPair& q, Elem& S, double& h) {
  for (int i = 0; i < 12; i++) (&S.cr[0][0])[i] = q.cr[i];
  for (int i = 0; i < 9; i++) (&S.cw[0][0])[i] = q.cw[i];
  S.quad = 1;
  h = 2.0 * sqrt(sqrt(q.cw[0] * q.cw[0] + q.cw[3] * q.cw[3] + q.cw[6] * q.cw[6]));
}

// the 27 values of a pair as 51 reals in the network's units
__device__ __forceinline__ void lq_scaled(const RegAcc<2>& A, double h, double* o) {
  for (int n = 0; n < 4; n++) {
    o[2 * n] = A.G[n].x / h;
    o[2 * n + 1] = A.G[n].y / h;
    o[8 + 2 * n] = A.H[n].x;
    o[9 + 2 * n] = A.H[n].y;
    for (int d = 0; d < 2; d++) {
      o[16 + 8 * d + 2 * n] = A.dG[d][n].x;
      o[17 + 8 * d + 2 * n] = A.dG[d][n].y;
      o[32 + 8 * d + 2 * n] = A.dH[d][n].x * h;
      o[33 + 8 * d + 2 * n] = A.dH[d][n].y * h;
    }
  }
  o[48] = A.F;
  o[49] = A.dF[0] * h;
  o[50] = A.dF[1] * h;
}

// the pair's GLN x GLN (GL) and GHN x GHN (GH) integrals by the whole warp,
// finished with the given sign
__device__ void lq_rules(const GbLqPair& q, int lane, bool neg, bool want_gl, RegAcc<2>& GL, RegAcc<2>& GH) {
  Elem S;
  double h;
  lq_elem(q, S, h);
  const double vt[2][3] = {{q.vt[0], q.vt[1], q.vt[2]}, {q.vt[3], q.vt[4], q.vt[5]}};
  const cplx k = cmk(q.k[0], q.k[1]);
  reg_integrate_gh_part<2>(S, lane, 32, q.rt, vt, k, GH);
  warp_allreduce<sizeof(RegAcc<2>) / sizeof(double)>((double*)&GH);
  reg_finish<2>(GH, GB_I_FP, neg);
  if (want_gl) {
    regacc_zero(GL);
    for (int p = lane; p < GB_GLN * GB_GLN; p += 32) {
      const int i = p / GB_GLN, j = p % GB_GLN;
      reg_point<2>(S, c_tab.xli[i], c_tab.xli[j], c_tab.wli[i] * c_tab.wli[j], q.rt, vt, k, GL);
    }
    warp_allreduce<sizeof(RegAcc<2>) / sizeof(double)>((double*)&GL);
    reg_finish<2>(GL, GB_I_FP, neg);
  }
}

// network inputs, standardised by (mu, sd)
__global__ void k_lq_features(int n, const GbLqPair* __restrict__ P, const float* __restrict__ mu,
                              const float* __restrict__ sd, float* X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const GbLqPair& q = P[i];
  Elem S;
  double h;
  lq_elem(q, S, h);
  double z[3] = {q.cw[0], q.cw[3], q.cw[6]};
  const double zn = norm3(z);
  for (int d = 0; d < 3; d++) z[d] /= zn;
  double c[4][3];
  const double sz[4] = {-1.0, 1.0, 1.0, -1.0}, se[4] = {-1.0, -1.0, 1.0, 1.0};
  for (int j = 0; j < 4; j++)
    for (int d = 0; d < 3; d++)
      c[j][d] = S.cr[d][0] + S.cr[d][1] * sz[j] + S.cr[d][2] * se[j] + S.cr[d][3] * sz[j] * se[j];
  double x[3] = {c[1][0] - c[0][0], c[1][1] - c[0][1], c[1][2] - c[0][2]};
  const double xz = x[0] * z[0] + x[1] * z[1] + x[2] * z[2];
  for (int d = 0; d < 3; d++) x[d] -= xz * z[d];
  const double xn = norm3(x);
  for (int d = 0; d < 3; d++) x[d] /= xn;
  const double y[3] = {z[1] * x[2] - z[2] * x[1], z[2] * x[0] - z[0] * x[2], z[0] * x[1] - z[1] * x[0]};
  double f[GB_LQ_NIN];
  for (int j = 0; j < 4; j++) {
    const double r[3] = {c[j][0] - q.rt[0], c[j][1] - q.rt[1], c[j][2] - q.rt[2]};
    f[3 * j] = (r[0] * x[0] + r[1] * x[1] + r[2] * x[2]) / h;
    f[3 * j + 1] = (r[0] * y[0] + r[1] * y[1] + r[2] * y[2]) / h;
    f[3 * j + 2] = (r[0] * z[0] + r[1] * z[1] + r[2] * z[2]) / h;
  }
  for (int t = 0; t < 2; t++) {
    const double* v = q.vt + 3 * t;
    f[12 + 3 * t] = v[0] * x[0] + v[1] * x[1] + v[2] * x[2];
    f[13 + 3 * t] = v[0] * y[0] + v[1] * y[1] + v[2] * y[2];
    f[14 + 3 * t] = v[0] * z[0] + v[1] * z[1] + v[2] * z[2];
  }
  f[18] = q.k[0] * h;
  f[19] = q.k[1] * h;
  for (int j = 0; j < GB_LQ_NIN; j++) X[(size_t)i * GB_LQ_NIN + j] = (float)((f[j] - mu[j]) / sd[j]);
}

// training targets: GH minus GL in the network's units (element's own orientation)
__global__ void __launch_bounds__(128) k_lq_label(int n, const GbLqPair* __restrict__ P, float* T) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= n) return;
  RegAcc<2> GL, GH;
  lq_rules(P[w], lane, false, true, GL, GH);
  if (lane != 0) return;
  double h, a[GB_LQ_NOUT], b[GB_LQ_NOUT];
  Elem S;
  lq_elem(P[w], S, h);
  lq_scaled(GH, h, a);
  lq_scaled(GL, h, b);
  for (int j = 0; j < GB_LQ_NOUT; j++) T[(size_t)w * GB_LQ_NOUT + j] = (float)(a[j] - b[j]);
}

// the network's corrections (standardised outputs Y, scales mu, sd) added to
// the listed pairs' matrix entries and solid-angle terms
__global__ void k_lq_apply(int n, const GbLqPair* __restrict__ P, const float* __restrict__ Y,
                           const float* __restrict__ mu, const float* __restrict__ sd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const GbLqPair& q = P[i];
  Elem S;
  double h;
  lq_elem(q, S, h);
  double d[GB_LQ_NOUT];
  for (int j = 0; j < GB_LQ_NOUT; j++) d[j] = (double)Y[(size_t)i * GB_LQ_NOUT + j] * sd[j] + mu[j];
  const double sh = q.neg ? -1.0 : 1.0;
  cplx* g = q.out[0];
  cplx* hh = q.out[1];
  for (int nn = 0; nn < 4; nn++) {
    g[nn] = g[nn] + cmk(d[2 * nn] * h, d[2 * nn + 1] * h);
    hh[nn] = hh[nn] + cmk(d[8 + 2 * nn] * sh, d[9 + 2 * nn] * sh);
    for (int t = 0; t < 2; t++) {
      cplx* dg = q.out[2 + t];
      cplx* dh = q.out[4 + t];
      dg[nn] = dg[nn] + cmk(d[16 + 8 * t + 2 * nn], d[17 + 8 * t + 2 * nn]);
      dh[nn] = dh[nn] + cmk(d[32 + 8 * t + 2 * nn] * sh / h, d[33 + 8 * t + 2 * nn] * sh / h);
    }
  }
  q.f[0] += d[48] * sh;
  q.f[1] += d[49] * sh / h;
  q.f[2] += d[50] * sh / h;
}

// the current (corrected) values of sampled pairs against the GH rule: per
// pair the largest error over the 51 outputs in the network's units, over the
// largest GH output; also the plain GL rule's error
__global__ void __launch_bounds__(128) k_lq_judge(int m, const int* __restrict__ idx, const GbLqPair* __restrict__ P,
                                                  double* err) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= m) return;
  const GbLqPair& q = P[idx[w]];
  RegAcc<2> GL, GH, C;
  lq_rules(q, lane, q.neg != 0, true, GL, GH);
  if (lane != 0) return;
  for (int nn = 0; nn < 4; nn++) {
    C.G[nn] = q.out[0][nn];
    C.H[nn] = q.out[1][nn];
    for (int t = 0; t < 2; t++) {
      C.dG[t][nn] = q.out[2 + t][nn];
      C.dH[t][nn] = q.out[4 + t][nn];
    }
  }
  C.F = q.f[0];
  C.dF[0] = q.f[1];
  C.dF[1] = q.f[2];
  Elem S;
  double h, a[GB_LQ_NOUT], b[GB_LQ_NOUT], c[GB_LQ_NOUT];
  lq_elem(q, S, h);
  lq_scaled(GH, h, a);
  lq_scaled(GL, h, b);
  lq_scaled(C, h, c);
  double sc = 0.0, ec = 0.0, eg = 0.0;
  for (int j = 0; j < GB_LQ_NOUT; j++) {
    sc = fmax(sc, fabs(a[j]));
    ec = fmax(ec, fabs(c[j] - a[j]));
    eg = fmax(eg, fabs(b[j] - a[j]));
  }
  err[2 * w] = ec / sc;
  err[2 * w + 1] = eg / sc;
}

// the GH rule written for every listed pair (the judge's fallback)
__global__ void __launch_bounds__(128) k_lq_exact(int n, const GbLqPair* __restrict__ P) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= n) return;
  const GbLqPair& q = P[w];
  RegAcc<2> GL, GH;
  if (q.gh_df) {
    // as k_asm_gh_df integrates the pair when the network is off
    Elem S;
    double h;
    lq_elem(q, S, h);
    const double vt[2][3] = {{q.vt[0], q.vt[1], q.vt[2]}, {q.vt[3], q.vt[4], q.vt[5]}};
    RegAcc<2> R;
    cplx E0;
    reg_gh_part_dn<2>(S, q.rt, vt, cmk(q.k[0], q.k[1]), lane, 32, R, E0);
    warp_allreduce<sizeof(RegAcc<2>) / sizeof(double)>((double*)&R);
    finish_dn<2>(R, S, q.neg != 0, E0, GH);
  } else {
    lq_rules(q, lane, q.neg != 0, false, GL, GH);
  }
  if (lane != 0) return;
  for (int nn = 0; nn < 4; nn++) {
    q.out[0][nn] = GH.G[nn];
    q.out[1][nn] = GH.H[nn];
    for (int t = 0; t < 2; t++) {
      q.out[2 + t][nn] = GH.dG[t][nn];
      q.out[4 + t][nn] = GH.dH[t][nn];
    }
  }
  q.f[0] = GH.F;
  q.f[1] = GH.dF[0];
  q.f[2] = GH.dF[1];
}

__global__ void k_lq_gather(size_t n, int w, const int* __restrict__ perm, const float* __restrict__ src, float* dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * w) return;
  const size_t r = i / w, c = i % w;
  dst[i] = src[(size_t)perm[r] * w + c];
}

// ---- model state (process-wide)
struct LqState {
  gb_mlp* net = nullptr;
  float xmu[GB_LQ_NIN], xsd[GB_LQ_NIN], ymu[GB_LQ_NOUT], ysd[GB_LQ_NOUT];
  int enabled = 0;
  int collect = 0;
  double tol = 1e-7;
  double stats[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  std::vector<float*> cx, ct;      // collected raw features / targets, per assembly
  std::vector<size_t> cn;
};
static LqState g_lq;
static std::mutex g_lq_mu;

static bool lq_active(int precision, int type) {
  std::lock_guard<std::mutex> lk(g_lq_mu);
  return precision >= 2 && type == 2 && (g_lq.collect || (g_lq.enabled && g_lq.net));
}

static int lq_alloc(GbLqList& L, size_t npair, cudaStream_t st) {
  L.cap = (unsigned)std::min<size_t>(npair / 32 + 4096, (size_t)4 << 20);
  GB_CUDA(cudaMallocAsync((void**)&L.p, (size_t)L.cap * sizeof(GbLqPair), st));
  GB_CUDA(cudaMallocAsync((void**)&L.count, sizeof(unsigned), st));
  GB_CUDA(cudaMemsetAsync(L.count, 0, sizeof(unsigned), st));
  return 0;
}

static void lq_free(GbLqList& L, cudaStream_t st) {
  if (L.p) cudaFreeAsync(L.p, st);
  if (L.count) cudaFreeAsync(L.count, st);
  L.p = nullptr;
  L.count = nullptr;
}

// After the regular passes: correct the listed pairs (or, collecting, keep
// their features and targets); synchronises st.
static int lq_stage(GbLqList& L, cudaStream_t st) {
  unsigned cnt = 0;
  GB_CUDA(cudaMemcpyAsync(&cnt, L.count, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  const int n = (int)std::min(cnt, L.cap);
  std::lock_guard<std::mutex> lk(g_lq_mu);
  if (n == 0) {
    for (int i = 0; i < 8; i++) g_lq.stats[i] = 0.0;
    return 0;
  }
  if (g_lq.collect) {
    float *X = nullptr, *T = nullptr, *mu = nullptr, *sd = nullptr;
    GB_CUDA(cudaMalloc((void**)&X, (size_t)n * GB_LQ_NIN * sizeof(float)));
    GB_CUDA(cudaMalloc((void**)&T, (size_t)n * GB_LQ_NOUT * sizeof(float)));
    GB_CUDA(cudaMallocAsync((void**)&mu, 2 * GB_LQ_NIN * sizeof(float), st));
    sd = mu + GB_LQ_NIN;
    std::vector<float> id(2 * GB_LQ_NIN, 0.0f);
    for (int j = 0; j < GB_LQ_NIN; j++) id[GB_LQ_NIN + j] = 1.0f;
    GB_CUDA(cudaMemcpyAsync(mu, id.data(), id.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    k_lq_features<<<(n + 127) / 128, 128, 0, st>>>(n, L.p, mu, sd, X);
    k_lq_label<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, st>>>(n, L.p, T);
    gbi_count_launch();
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
    cudaFreeAsync(mu, st);
    GB_CUDA(cudaStreamSynchronize(st));
    g_lq.cx.push_back(X);
    g_lq.ct.push_back(T);
    g_lq.cn.push_back((size_t)n);
    g_lq.stats[0] = n;
    return 0;
  }
  cudaEvent_t e0, e1;
  GB_CUDA(cudaEventCreate(&e0));
  GB_CUDA(cudaEventCreate(&e1));
  GB_CUDA(cudaEventRecord(e0, st));
  float *X = nullptr, *Y = nullptr, *nrm = nullptr;
  int* idx = nullptr;
  double* err = nullptr;
  // the judged sample: every 16th pair (at least 64, at most 2,048)
  const int m = std::min(n, std::min(2048, std::max(64, n / 16)));
  GB_CUDA(cudaMallocAsync((void**)&X, (size_t)n * GB_LQ_NIN * sizeof(float), st));
  GB_CUDA(cudaMallocAsync((void**)&Y, (size_t)n * GB_LQ_NOUT * sizeof(float), st));
  GB_CUDA(cudaMallocAsync((void**)&nrm, 2 * (GB_LQ_NIN + GB_LQ_NOUT) * sizeof(float), st));
  GB_CUDA(cudaMallocAsync((void**)&idx, (size_t)m * sizeof(int), st));
  GB_CUDA(cudaMallocAsync((void**)&err, (size_t)m * 2 * sizeof(double), st));
  std::vector<float> h(2 * (GB_LQ_NIN + GB_LQ_NOUT));
  memcpy(h.data(), g_lq.xmu, sizeof(g_lq.xmu));
  memcpy(h.data() + GB_LQ_NIN, g_lq.xsd, sizeof(g_lq.xsd));
  memcpy(h.data() + 2 * GB_LQ_NIN, g_lq.ymu, sizeof(g_lq.ymu));
  memcpy(h.data() + 2 * GB_LQ_NIN + GB_LQ_NOUT, g_lq.ysd, sizeof(g_lq.ysd));
  std::vector<int> hi(m);
  for (int i = 0; i < m; i++) hi[i] = (int)(((long long)i * n) / m);
  GB_CUDA(cudaMemcpyAsync(nrm, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(idx, hi.data(), (size_t)m * sizeof(int), cudaMemcpyHostToDevice, st));
  k_lq_features<<<(n + 127) / 128, 128, 0, st>>>(n, L.p, nrm, nrm + GB_LQ_NIN, X);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  for (int r0 = 0; r0 < n; r0 += 65536) {
    const int b = std::min(65536, n - r0);
    if (gb_mlp_forward(g_lq.net, b, X + (size_t)r0 * GB_LQ_NIN, Y + (size_t)r0 * GB_LQ_NOUT)) return -1;
  }
  k_lq_apply<<<(n + 127) / 128, 128, 0, st>>>(n, L.p, Y, nrm + 2 * GB_LQ_NIN, nrm + 2 * GB_LQ_NIN + GB_LQ_NOUT);
  k_lq_judge<<<(unsigned)(((size_t)m * 32 + 127) / 128), 128, 0, st>>>(m, idx, L.p, err);
  gbi_count_launch();
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  std::vector<double> he((size_t)m * 2);
  GB_CUDA(cudaMemcpyAsync(he.data(), err, he.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  double sc = 0.0, sg = 0.0, mc = 0.0;
  for (int i = 0; i < m; i++) {
    sc += he[2 * i] * he[2 * i];
    sg += he[2 * i + 1] * he[2 * i + 1];
    mc = std::max(mc, he[2 * i]);
  }
  const double rc = sqrt(sc / m), rg = sqrt(sg / m);
  const bool revert = !(rc <= g_lq.tol);
  if (revert) {
    k_lq_exact<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, st>>>(n, L.p);
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
  }
  GB_CUDA(cudaEventRecord(e1, st));
  GB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  for (void* p : {(void*)X, (void*)Y, (void*)nrm, (void*)idx, (void*)err}) cudaFreeAsync(p, st);
  const double s[8] = {(double)n, (double)(cnt - (unsigned)n), (double)m, rc, rg, mc, revert ? 1.0 : 0.0, ms};
  for (int i = 0; i < 8; i++) g_lq.stats[i] = s[i];
  return 0;
}

extern "C" int gb_lq_collect(int on) {
  std::lock_guard<std::mutex> lk(g_lq_mu);
  g_lq.collect = on ? 1 : 0;
  if (on) {
    for (float* p : g_lq.cx) cudaFree(p);
    for (float* p : g_lq.ct) cudaFree(p);
    g_lq.cx.clear();
    g_lq.ct.clear();
    g_lq.cn.clear();
  }
  return 0;
}

extern "C" int gb_lq_enable(int on, double tol) {
  std::lock_guard<std::mutex> lk(g_lq_mu);
  if (on && !g_lq.net) {
    gbi_set_error("gb_lq_enable: no trained network (gb_lq_train)");
    return -1;
  }
  if (!(tol > 0.0)) {
    gbi_set_error("gb_lq_enable: tolerance %g must be positive", tol);
    return -1;
  }
  g_lq.enabled = on ? 1 : 0;
  g_lq.tol = tol;
  return 0;
}

extern "C" int gb_lq_stats(double* out) {
  std::lock_guard<std::mutex> lk(g_lq_mu);
  for (int i = 0; i < 8; i++) out[i] = g_lq.stats[i];
  return 0;
}

// Training on the collected pairs: a seeded shuffle, 1/20 held out, inputs
// and targets standardised per component, Adam with a cosine learning rate.
// info: samples trained on, held out, last 100 steps' mean training loss,
// held-out loss (standardised units), the held-out loss of predicting zero.
extern "C" int gb_lq_train(int epochs, int batch, float lr, unsigned seed, double* info) {
  std::lock_guard<std::mutex> lk(g_lq_mu);
  size_t n = 0;
  for (size_t c : g_lq.cn) n += c;
  if (n < (size_t)4 * batch || batch < 1 || epochs < 1) {
    gbi_set_error("gb_lq_train: %zu collected pairs for batches of %d (collect with gb_lq_collect(1) and a "
                  "precision >= 2 assembly of quadrangle meshes first)", n, batch);
    return -1;
  }
  // host copies: raw features and targets, concatenated
  std::vector<float> X(n * GB_LQ_NIN), T(n * GB_LQ_NOUT);
  size_t off = 0;
  for (size_t i = 0; i < g_lq.cn.size(); i++) {
    GB_CUDA(cudaMemcpy(X.data() + off * GB_LQ_NIN, g_lq.cx[i], g_lq.cn[i] * GB_LQ_NIN * sizeof(float),
                       cudaMemcpyDeviceToHost));
    GB_CUDA(cudaMemcpy(T.data() + off * GB_LQ_NOUT, g_lq.ct[i], g_lq.cn[i] * GB_LQ_NOUT * sizeof(float),
                       cudaMemcpyDeviceToHost));
    off += g_lq.cn[i];
  }
  // seeded shuffle (64-bit LCG, Fisher-Yates)
  std::vector<int> perm(n);
  for (size_t i = 0; i < n; i++) perm[i] = (int)i;
  unsigned long long s = 0x9E3779B97F4A7C15ull ^ seed;
  for (size_t i = n - 1; i > 0; i--) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    const size_t j = (size_t)((s >> 33) % (i + 1));
    std::swap(perm[i], perm[j]);
  }
  const size_t nval = std::max<size_t>(n / 20, 1), ntr = n - nval;
  // standardisation from the training part
  double mx[GB_LQ_NIN] = {0}, sx[GB_LQ_NIN] = {0}, my[GB_LQ_NOUT] = {0}, sy[GB_LQ_NOUT] = {0};
  for (size_t r = 0; r < ntr; r++) {
    const size_t p = perm[r];
    for (int j = 0; j < GB_LQ_NIN; j++) { const double v = X[p * GB_LQ_NIN + j]; mx[j] += v; sx[j] += v * v; }
    for (int j = 0; j < GB_LQ_NOUT; j++) { const double v = T[p * GB_LQ_NOUT + j]; my[j] += v; sy[j] += v * v; }
  }
  for (int j = 0; j < GB_LQ_NIN; j++) {
    mx[j] /= ntr;
    const double v = sx[j] / ntr - mx[j] * mx[j];
    g_lq.xmu[j] = (float)mx[j];
    g_lq.xsd[j] = (float)(v > 1e-24 ? sqrt(v) : 1.0);
  }
  for (int j = 0; j < GB_LQ_NOUT; j++) {
    my[j] /= ntr;
    const double v = sy[j] / ntr - my[j] * my[j];
    g_lq.ymu[j] = (float)my[j];
    g_lq.ysd[j] = (float)(v > 1e-36 ? sqrt(v) : 1.0);
  }
  std::vector<float> Xs(n * GB_LQ_NIN), Ts(n * GB_LQ_NOUT);
  for (size_t r = 0; r < n; r++) {
    const size_t p = perm[r];
    for (int j = 0; j < GB_LQ_NIN; j++) Xs[r * GB_LQ_NIN + j] = (X[p * GB_LQ_NIN + j] - g_lq.xmu[j]) / g_lq.xsd[j];
    for (int j = 0; j < GB_LQ_NOUT; j++) Ts[r * GB_LQ_NOUT + j] = (T[p * GB_LQ_NOUT + j] - g_lq.ymu[j]) / g_lq.ysd[j];
  }
  float *dX = nullptr, *dT = nullptr, *dY = nullptr;
  GB_CUDA(cudaMalloc((void**)&dX, Xs.size() * sizeof(float)));
  GB_CUDA(cudaMalloc((void**)&dT, Ts.size() * sizeof(float)));
  GB_CUDA(cudaMalloc((void**)&dY, nval * GB_LQ_NOUT * sizeof(float)));
  GB_CUDA(cudaMemcpy(dX, Xs.data(), Xs.size() * sizeof(float), cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(dT, Ts.data(), Ts.size() * sizeof(float), cudaMemcpyHostToDevice));
  // network 20 -> 256 -> 256 -> 256 -> 51, He-scaled seeded initialisation
  if (g_lq.net) { gb_mlp_destroy(g_lq.net); g_lq.net = nullptr; }
  const int widths[5] = {GB_LQ_NIN, 256, 256, 256, GB_LQ_NOUT};
  if (gb_mlp_create(4, widths, &g_lq.net)) return -1;
  std::vector<float> par(gb_mlp_param_count(g_lq.net));
  size_t o = 0;
  for (int l = 0; l < 4; l++) {
    const double sc = sqrt(2.0 / widths[l]);
    for (int i = 0; i < widths[l] * widths[l + 1]; i++) {
      s = s * 6364136223846793005ull + 1442695040888963407ull;
      const double u1 = ((s >> 11) + 0.5) / 9007199254740992.0;
      s = s * 6364136223846793005ull + 1442695040888963407ull;
      const double u2 = ((s >> 11) + 0.5) / 9007199254740992.0;
      par[o++] = (float)(sc * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2));
    }
    for (int i = 0; i < widths[l + 1]; i++) par[o++] = 0.0f;
  }
  int rc = gb_mlp_set_params(g_lq.net, par.data());
  const long steps = (long)epochs * (long)(ntr / batch);
  double tail = 0.0;
  int ntail = 0;
  for (long st = 0; st < steps && !rc; st++) {
    const size_t r0 = (size_t)(st % (long)(ntr / batch)) * batch;
    const float a = (float)(lr * 0.5 * (1.0 + cos(3.141592653589793 * (double)st / (double)steps)));
    double loss = 0.0;
    rc = gb_mlp_train_step(g_lq.net, batch, dX + r0 * GB_LQ_NIN, dT + r0 * GB_LQ_NOUT, a, &loss);
    if (st >= steps - 100) { tail += loss; ntail++; }
  }
  double val = 0.0, zero = 0.0;
  if (!rc) rc = gb_mlp_forward(g_lq.net, (int)nval, dX + ntr * GB_LQ_NIN, dY);
  if (!rc) {
    std::vector<float> hy(nval * GB_LQ_NOUT);
    cudaMemcpy(hy.data(), dY, hy.size() * sizeof(float), cudaMemcpyDeviceToHost);
    for (size_t r = 0; r < nval; r++)
      for (int j = 0; j < GB_LQ_NOUT; j++) {
        const double t = Ts[(ntr + r) * GB_LQ_NOUT + j], d = hy[r * GB_LQ_NOUT + j] - t;
        val += d * d;
        zero += t * t;
      }
    val /= nval;
    zero /= nval;
  }
  cudaFree(dX);
  cudaFree(dT);
  cudaFree(dY);
  if (rc) return -1;
  info[0] = (double)ntr;
  info[1] = (double)nval;
  info[2] = ntail ? tail / ntail : 0.0;
  info[3] = val;
  info[4] = zero;
  return 0;
}

extern "C" int gbi_assemble_domain2(const GbMeshDev* m, int did, int type, int precision, cplx* G, cplx* H, cplx* dG,
                                    cplx* dH, double* dF, double* Fs, cudaStream_t st);

// Assemble G,H,dG,dH,dF of one domain into device buffers.  Fs is scratch of
// 3 N Ne doubles.  Buffers are cleared here (rows of the unused fourth node of
// triangles and columns of the fourth shape function of triangles stay zero).
extern "C" int gbi_assemble_domain(const GbMeshDev* m, int did, int type, cplx* G, cplx* H, cplx* dG, cplx* dH,
                                   double* dF, double* Fs, cudaStream_t st) {
  return gbi_assemble_domain2(m, did, type, 0, G, H, dG, dH, dF, Fs, st);
}

// Rows row0 .. row0 + nrow - 1 of domain did into G, H (nrow x N), dG, dH
// (2 nrow x N), dF (nrow x 3); Fs: scratch of 3 nrow Ne doubles.  The full
// domain is row0 = 0, nrow = N.
extern "C" int gbi_assemble_rows(const GbMeshDev* m, int did, int type, int precision, int row0, int nrow, cplx* G,
                                 cplx* H, cplx* dG, cplx* dH, double* dF, double* Fs, cudaStream_t st) {
  int Ne = m->sb_Ne[did];
  if (Ne <= 0 || nrow <= 0) return 0;
  size_t N = (size_t)Ne * 4;
  if (row0 < 0 || (size_t)row0 + (size_t)nrow > N) {
    gbi_set_error("assembly: rows %d..%d outside 0..%zu", row0, row0 + nrow - 1, N - 1);
    return -1;
  }
  const size_t nr = (size_t)nrow;
  AsmArgs a;
  a.cr = m->cr;
  a.cw = m->cw;
  a.etype = m->etype;
  a.ren = m->ren;
  a.sid = m->sid + m->sb_off[did];
  a.Ne = Ne;
  a.k = cmk(m->kn[2 * did], m->kn[2 * did + 1]);
  a.type = type;
  a.did = did;
  a.G = G;
  a.H = H;
  a.dG = dG;
  a.dH = dH;
  a.dF = dF;
  a.Fs = Fs;
  a.only = nullptr;
  a.adapt = precision == 3;
  a.row0 = row0;
  a.nrow = nrow;
  a.redo = nullptr;
  memset(&a.lq, 0, sizeof(a.lq));
  a.gh = nullptr; a.ghn = nullptr; a.ghcap = 0; a.item = 0;
  GB_CUDA(cudaMemsetAsync(G, 0, nr * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(H, 0, nr * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(dG, 0, 2 * nr * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(dH, 0, 2 * nr * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(dF, 0, 3 * nr * sizeof(double), st));
  GB_CUDA(cudaMemsetAsync(Fs, 0, 3 * nr * (size_t)Ne * sizeof(double), st));
  size_t npair = nr * (size_t)Ne;
  unsigned nb = (unsigned)((npair + 127) / 128);
  uint8_t* redo = nullptr;
  const bool lq = lq_active(precision, type);
  if (lq && lq_alloc(a.lq, npair, st)) return -1;
  if (precision >= 2 && type == 2) {
    GB_CUDA(cudaMallocAsync((void**)&redo, npair, st));
    a.ghcap = (unsigned)std::min<size_t>(npair / 16 + 4096, (size_t)1 << 26);
    GB_CUDA(cudaMallocAsync((void**)&a.gh, (size_t)a.ghcap * sizeof(GbGhPair), st));
    GB_CUDA(cudaMallocAsync((void**)&a.ghn, sizeof(unsigned), st));
    GB_CUDA(cudaMemsetAsync(a.ghn, 0, sizeof(unsigned), st));
    k_asm_regular_df<<<nb, 128, 0, st>>>(a, redo);
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
    unsigned ng = 0;
    GB_CUDA(cudaMemcpyAsync(&ng, a.ghn, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    GB_CUDA(cudaStreamSynchronize(st));
    ng = std::min(ng, a.ghcap);
    if (ng > 0) {
      AsmArgs* da = nullptr;
      GB_CUDA(cudaMallocAsync((void**)&da, sizeof(AsmArgs), st));
      GB_CUDA(cudaMemcpyAsync(da, &a, sizeof(AsmArgs), cudaMemcpyHostToDevice, st));
      k_asm_gh_df<<<(unsigned)(((size_t)ng * 32 + 127) / 128), 128, 0, st>>>(da, a.gh, ng);
      gbi_count_launch();
      GB_CUDA(cudaGetLastError());
      cudaFreeAsync(da, st);
      GB_CUDA(cudaStreamSynchronize(st));  // a (host) was the copy's source
    }
    cudaFreeAsync(a.gh, st);
    cudaFreeAsync(a.ghn, st);
    a.gh = nullptr; a.ghn = nullptr; a.ghcap = 0;
    a.only = redo;
  } else if (precision == 1 && type == 2) {
    GB_CUDA(cudaMallocAsync((void**)&redo, npair, st));
    k_asm_regular_f32<<<nb, 128, 0, st>>>(a, redo);
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
    a.only = redo;
  }
  k_asm_regular<<<nb, 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  if (redo) GB_CUDA(cudaFreeAsync(redo, st));
  if (lq) {
    const int r = lq_stage(a.lq, st);
    lq_free(a.lq, st);
    memset(&a.lq, 0, sizeof(a.lq));
    if (r) return -1;
  }
  if (precision >= 2) k_asm_singular<true><<<(unsigned)nr, 256, 0, st>>>(a);
  else k_asm_singular<false><<<(unsigned)nr, 256, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  k_asm_rows<<<(unsigned)((nr + 127) / 128), 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// Work-list assembly: every item (rows of one domain of one object) with one
// launch per phase -- double-float regular pairs (precision >= 2), FP64
// regular pairs (the flagged ones after a double-float pass), singular
// pairs, row sums -- instead of a launch sequence per domain.  Items of
// uneven size share the GPU without tails of their own.  Synchronises st.
extern "C" int gbi_assemble_list(const GbAsmItem* d, int n, int type, int precision, cudaStream_t st) {
  if (n <= 0) return 0;
  std::vector<AsmArgs> it((size_t)n);
  std::vector<unsigned> breg((size_t)n + 1, 0), bsing((size_t)n + 1, 0), brows((size_t)n + 1, 0);
  std::vector<void*> tmp;
  int rc = 0;
  GbLqList lql;
  memset(&lql, 0, sizeof(lql));
  const bool lq = lq_active(precision, type);
  size_t tot = 0;
  for (int i = 0; i < n; i++) tot += (size_t)d[i].nrow * (size_t)d[i].m->sb_Ne[d[i].did];
  if (lq && lq_alloc(lql, tot, st)) return -1;
  // the certain-GHN pairs of the double-float pass (k_asm_gh_df)
  GbGhPair* ghl = nullptr;
  unsigned* ghn = nullptr;
  unsigned ghcap = 0;
  if (precision >= 2 && type == 2) {
    ghcap = (unsigned)std::min<size_t>(tot / 16 + 4096, (size_t)1 << 26);
    if (cudaMallocAsync((void**)&ghl, (size_t)ghcap * sizeof(GbGhPair), st) != cudaSuccess ||
        cudaMallocAsync((void**)&ghn, sizeof(unsigned), st) != cudaSuccess ||
        cudaMemsetAsync(ghn, 0, sizeof(unsigned), st) != cudaSuccess) {
      gbi_set_error("work-list assembly: out of device memory");
      return -1;
    }
  }
  for (int i = 0; i < n && !rc; i++) {
    const GbMeshDev* m = d[i].m;
    const int did = d[i].did, Ne = m->sb_Ne[did];
    const size_t N = (size_t)Ne * 4, nr = (size_t)d[i].nrow;
    AsmArgs& a = it[i];
    memset(&a, 0, sizeof(a));
    a.cr = m->cr; a.cw = m->cw; a.etype = m->etype; a.ren = m->ren;
    a.sid = m->sid + m->sb_off[did];
    a.Ne = Ne;
    a.k = cmk(m->kn[2 * did], m->kn[2 * did + 1]);
    a.type = type; a.did = did;
    a.G = d[i].G; a.H = d[i].H; a.dG = d[i].dG; a.dH = d[i].dH; a.dF = d[i].dF;
    a.adapt = precision == 3;
    a.row0 = d[i].row0; a.nrow = d[i].nrow;
    a.lq = lql;
    a.gh = ghl; a.ghn = ghn; a.ghcap = ghcap; a.item = i;
    const size_t npair = nr * (size_t)Ne;
    if (cudaMallocAsync((void**)&a.Fs, 3 * nr * (size_t)Ne * sizeof(double), st) != cudaSuccess ||
        cudaMallocAsync((void**)&a.redo, npair + 16, st) != cudaSuccess) {
      gbi_set_error("work-list assembly: out of device memory");
      rc = -1;
      break;
    }
    tmp.push_back(a.Fs);
    tmp.push_back(a.redo);
    if (cudaMemsetAsync(a.G, 0, nr * N * sizeof(cplx), st) != cudaSuccess ||
        cudaMemsetAsync(a.H, 0, nr * N * sizeof(cplx), st) != cudaSuccess ||
        cudaMemsetAsync(a.dG, 0, 2 * nr * N * sizeof(cplx), st) != cudaSuccess ||
        cudaMemsetAsync(a.dH, 0, 2 * nr * N * sizeof(cplx), st) != cudaSuccess ||
        cudaMemsetAsync(a.dF, 0, 3 * nr * sizeof(double), st) != cudaSuccess ||
        cudaMemsetAsync(a.Fs, 0, 3 * nr * (size_t)Ne * sizeof(double), st) != cudaSuccess) {
      gbi_set_error("work-list assembly: memset");
      rc = -1;
    }
    breg[i + 1] = breg[i] + (unsigned)((npair + 127) / 128);
    bsing[i + 1] = bsing[i] + (unsigned)nr;
    brows[i + 1] = brows[i] + (unsigned)((nr + 127) / 128);
  }
  AsmArgs* dit = nullptr;
  unsigned* db = nullptr;
  if (!rc && (cudaMallocAsync((void**)&dit, (size_t)n * sizeof(AsmArgs), st) != cudaSuccess ||
              cudaMallocAsync((void**)&db, 3 * ((size_t)n + 1) * sizeof(unsigned), st) != cudaSuccess ||
              cudaMemcpyAsync(dit, it.data(), (size_t)n * sizeof(AsmArgs), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemcpyAsync(db, breg.data(), ((size_t)n + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemcpyAsync(db + n + 1, bsing.data(), ((size_t)n + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemcpyAsync(db + 2 * (n + 1), brows.data(), ((size_t)n + 1) * sizeof(unsigned), cudaMemcpyHostToDevice, st) != cudaSuccess)) {
    gbi_set_error("work-list assembly: upload");
    rc = -1;
  }
  if (!rc) {
    const bool df = precision >= 2 && type == 2;
    if (df) {
      void* kt = nullptr;
      const int timed = gbi_kt_asm_start(st, &kt);
      // triangle sources by the three-shape-function variant, quadrangles by
      // the general one (one launch when the meshes hold one type)
      bool tri = false, quad = false;
      for (int i = 0; i < n; i++) {
        tri = tri || d[i].m->ntri > 0;
        quad = quad || d[i].m->nquad > 0;
      }
      if (!tri && !quad) quad = true;  // counts not known: the general variant
      if (tri) {
        k_asm_regular_df_list<1><<<breg[n], 128, 0, st>>>(dit, db, n);
        gbi_count_launch();
      }
      if (quad) {
        if (tri) k_asm_regular_df_list<2><<<breg[n], 128, 0, st>>>(dit, db, n);
        else k_asm_regular_df_list<0><<<breg[n], 128, 0, st>>>(dit, db, n);
        gbi_count_launch();
      }
      if (timed) {
        double pairs = 0.0;
        for (int i = 0; i < n; i++) pairs += (double)d[i].nrow * (double)d[i].m->sb_Ne[d[i].did];
        gbi_kt_asm_stop(kt, st, pairs);
      }
      unsigned ng = 0;
      if (cudaMemcpyAsync(&ng, ghn, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) {
        gbi_set_error("work-list assembly: %s", cudaGetErrorString(cudaGetLastError()));
        rc = -1;
      }
      ng = std::min(ng, ghcap);
      if (!rc && ng > 0) {
        k_asm_gh_df<<<(unsigned)(((size_t)ng * 32 + 127) / 128), 128, 0, st>>>(dit, ghl, ng);
        gbi_count_launch();
      }
    }
    k_asm_regular_list<<<breg[n], 128, 0, st>>>(dit, db, n, df ? 1 : 0);
    gbi_count_launch();
    if (lq && lq_stage(lql, st)) rc = -1;
  }
  if (!rc) {
    if (precision >= 2) k_asm_singular_list<true><<<bsing[n], 256, 0, st>>>(dit, db + n + 1, n);
    else k_asm_singular_list<false><<<bsing[n], 256, 0, st>>>(dit, db + n + 1, n);
    gbi_count_launch();
    k_asm_rows_list<<<brows[n], 128, 0, st>>>(dit, db + 2 * (n + 1), n);
    gbi_count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { gbi_set_error("work-list assembly launch: %s", cudaGetErrorString(e)); rc = -1; }
  }
  if (dit) cudaFreeAsync(dit, st);
  if (db) cudaFreeAsync(db, st);
  for (void* t : tmp) cudaFreeAsync(t, st);
  lq_free(lql, st);
  if (ghl) cudaFreeAsync(ghl, st);
  if (ghn) cudaFreeAsync(ghn, st);
  const cudaError_t e = cudaStreamSynchronize(st);  // the host arrays above are read by the copies
  if (!rc && e != cudaSuccess) { gbi_set_error("work-list assembly: %s", cudaGetErrorString(e)); rc = -1; }
  return rc;
}

// precision 0: FP64 throughout (the reference's arithmetic); 1: regular pairs
// of the GLN x GLN rule in FP32 with FP64 near pairs; 2: regular pairs and
// singular point sets in double-float; 3 (the chosen form): as 2 with the
// regular pairs' order adapted to their distance (reg_order)
extern "C" int gbi_assemble_domain2(const GbMeshDev* m, int did, int type, int precision, cplx* G, cplx* H, cplx* dG,
                                    cplx* dH, double* dF, double* Fs, cudaStream_t st) {
  return gbi_assemble_rows(m, did, type, precision, 0, 4 * m->sb_Ne[did], G, H, dG, dH, dF, Fs, st);
}

extern "C" int gbi_upload_tables_asm(const void* t) {
  GB_CUDA(cudaMemcpyToSymbol(c_tab, t, sizeof(GbTables)));
  const GbTables* d = (const GbTables*)t;
  GbTablesF f;
  for (int i = 0; i < GB_GLN; i++) { f.xli[i] = (float)d->xli[i]; f.wli[i] = (float)d->wli[i]; }
  GB_CUDA(cudaMemcpyToSymbol(c_tabf, &f, sizeof(GbTablesF)));
  return gbi_upload_tabd(d);
}
// ==================================================================== no allocation
// Allocation-free variant of the domain assembly (gb_assemble_domain_noalloc
// in gb_bem.h).  Some callers cannot allocate device memory: an application
// whose device memory is entirely owned by another allocator (a framework's
// caching pool holds the free memory, so a library cudaMalloc fails or
// fragments it), a latency-critical loop that cannot afford cudaFree's
// implicit device-wide synchronisation, or a code certified to allocate
// nothing after start-up.  This entry point takes every input and output from
// the caller and keeps its only scratch -- the per-pair solid-angle terms
// Fs[4 Ne][Ne][3] -- in the fixed array below, so it never calls cudaMalloc,
// cudaFree or an allocating library routine.
//
// The array is GB_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB) of static device
// memory: every GPU that loads this library holds it until the process exits.
// It limits a domain to GB_NOALLOC_MAX_NE elements (12 Ne^2 <= 2^21).
// All calls share the one array; it keeps the last call's contents and is
// cleared at the start of every call.  Calls that overlap on the GPU (two
// streams, or two host threads on one device) race on it and must be
// serialised by the caller.
#define GB_NOALLOC_SCRATCH_DOUBLES (2u * 1024u * 1024u)
#define GB_NOALLOC_MAX_NE 418
static __device__ __align__(256) double g_noalloc_scratch[GB_NOALLOC_SCRATCH_DOUBLES];

// Host code may not use g_noalloc_scratch's name as a device address: the
// device address is looked up once per device (with that device current) by
// cudaGetSymbolAddress and cached here.
static double* g_noalloc_dev_ptr[64];
static std::mutex g_noalloc_mu;

static int noalloc_scratch_ptr(double** out) {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { gbi_set_error("gb_assemble_domain_noalloc: device ordinal %d not supported", dev); return -1; }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_dev_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      gbi_set_error("gb_assemble_domain_noalloc: cudaGetSymbolAddress of the scratch failed: %s", cudaGetErrorString(e));
      return -1;
    }
    g_noalloc_dev_ptr[dev] = (double*)p;
  }
  *out = g_noalloc_dev_ptr[dev];
  return 0;
}

extern "C" int gbi_ensure_tables(void);

extern "C" int gb_assemble_domain_noalloc(const double* cr, const double* cw, const int* etype, const double* ren,
                                          const int* sid, int Ne, double k_re, double k_im, int did, int type, void* G,
                                          void* H, void* dG, void* dH, double* dF, void* stream) {
  if (Ne < 1 || Ne > GB_NOALLOC_MAX_NE) {
    gbi_set_error("gb_assemble_domain_noalloc: %d elements in the domain; this entry point supports 1..%d "
                  "(fixed 16 MiB scratch); use gb_assemble for larger domains", Ne, GB_NOALLOC_MAX_NE);
    return -1;
  }
  if (type < 0 || type > 3) { gbi_set_error("gb_assemble_domain_noalloc: quadrature type %d not in 0..3", type); return -1; }
  if (did < 0 || did >= GB_MAXDOM) { gbi_set_error("gb_assemble_domain_noalloc: domain id %d not in 0..%d", did, GB_MAXDOM - 1); return -1; }
  if (!cr || !cw || !etype || !ren || !sid || !G || !H || !dG || !dH || !dF) {
    gbi_set_error("gb_assemble_domain_noalloc: null input or output pointer");
    return -1;
  }
  double* scratch = nullptr;
  if (noalloc_scratch_ptr(&scratch)) return -1;
  if (gbi_ensure_tables()) return -1;
  GbMeshDev m;
  memset(&m, 0, sizeof(m));
  m.cr = (double*)cr;
  m.cw = (double*)cw;
  m.ren = (double*)ren;
  m.etype = (int*)etype;
  m.sid = (int*)sid;
  m.sb_Ne[did] = Ne;
  m.sb_off[did] = 0;
  m.kn[2 * did] = k_re;
  m.kn[2 * did + 1] = k_im;
  return gbi_assemble_domain(&m, did, type, (cplx*)G, (cplx*)H, (cplx*)dG, (cplx*)dH, dF, scratch, (cudaStream_t)stream);
}
