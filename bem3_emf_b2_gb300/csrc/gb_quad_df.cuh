// gb_quad_df.cuh -- the regular-pair rule of gb_quad.cuh in double-float
// (gb_df64.cuh) on the FP32 pipes, for the assembly (k_asm_regular_df) and
// the field kernels (gb_field.cu).
//
// Same points, weights, shape functions and scalings as reg_integrate
// (reference bil_dcoef_v2_GL, lit_dcoef_v2_GL) for the GLN x GLN rule, the
// geometry relative to the source element's point (0, 0): R = R0 + d with
// d = c1 z + c2 e + c3 z e (for a quadrangle's tensor rule evaluated row by
// row: affine in e with per-row constants); the common factor e^{ik|R0|} is
// taken out of the sums and applied in FP64, so the double-float phase is
// e^{ik(|R| - |R0|)}.
// The GLN/GHN decision of the reference (|Re dF/dv| > CBD_SDF) belongs to the
// FP64 path: reg_integrate_dn declines (returns false) when a |dF| lies
// within 0.05 of CBD_SDF or is not finite, and the caller integrates the pair
// in FP64.  Each translation unit that includes this header holds its own
// copy of the tables (c_tabd) and uploads it with gbi_upload_tabd.
// Adaptive order (precision 3): far pairs take an n x n Gauss-Legendre rule
// with n < GLN chosen from the pair's distance and the element's phase
// variation (reg_order); the GLN rule and its tables are unchanged for the
// pairs that keep it.
#pragma once
#include "gb_quad.cuh"
#include "gb_df64.cuh"
#include "gb_internal.h"
#include "gb_rules.h"

// Conical product rules over a triangle for n = 5..8 points per direction
// (n^2 points, rule n at gb_con_off(n)): the element's reference triangle,
// vertices (1, 0), (-1/2, +-sqrt(3)/2) in (z, e), as the image of the unit
// square under (s, t) -> V0 + s (V1 - V0) + s t (V2 - V1) with Jacobian
// proportional to s; Gauss-Jacobi nodes for the weight s in s, Gauss-Legendre
// in t (Stroud's conical product; exact for polynomials of degree 2n - 1 in
// z, e).  Weights scaled to the sub-quadrangle rule's total (12).
#define GB_NCON (25 + 36 + 49 + 64)
__host__ __device__ __forceinline__ int gb_con_off(int n) { return n == 5 ? 0 : (n == 6 ? 25 : (n == 7 ? 61 : 110)); }

struct GbTablesD {  // GL nodes and weights in double-float (hi, lo)
  float2 x[GB_GLN], w[GB_GLN];
  float2 xh[GB_GHN], wh[GB_GHN];
  float2 xn[GB_NTAB], wn[GB_NTAB];  // the rules of 1..GLN points, rule n at n (n - 1) / 2
  float2 cz[GB_NCON], ce[GB_NCON], cwt[GB_NCON];  // conical rules: z, e, weight per point
};
static __constant__ GbTablesD c_tabd;

static int gbi_upload_tabd(const GbTables* d) {
  GbTablesD g;
  for (int i = 0; i < GB_GLN; i++) {
    g.x[i].x = (float)d->xli[i];
    g.x[i].y = (float)(d->xli[i] - (double)g.x[i].x);
    g.w[i].x = (float)d->wli[i];
    g.w[i].y = (float)(d->wli[i] - (double)g.w[i].x);
  }
  for (int i = 0; i < GB_NTAB; i++) {
    g.xn[i].x = (float)d->xn[i];
    g.xn[i].y = (float)(d->xn[i] - (double)g.xn[i].x);
    g.wn[i].x = (float)d->wn[i];
    g.wn[i].y = (float)(d->wn[i] - (double)g.wn[i].x);
  }
  for (int i = 0; i < GB_GHN; i++) {
    g.xh[i].x = (float)d->xhi[i];
    g.xh[i].y = (float)(d->xhi[i] - (double)g.xh[i].x);
    g.wh[i].x = (float)d->whi[i];
    g.wh[i].y = (float)(d->whi[i] - (double)g.wh[i].x);
  }
  auto split = [](double v, float2& f) {
    f.x = (float)v;
    f.y = (float)(v - (double)f.x);
  };
  for (int n = 5; n <= 8; n++) {
    double z[64], e[64], w[64];
    const int o = gb_con_off(n), ol = n * (n - 1) / 2;
    gb_conical_rule(n, d->xn + ol, d->wn + ol, z, e, w);
    for (int q = 0; q < n * n; q++) {
      split(z[q], g.cz[o + q]);
      split(e[q], g.ce[o + q]);
      split(w[q], g.cwt[o + q]);
    }
  }
  GB_CUDA(cudaMemcpyToSymbol(c_tabd, &g, sizeof(GbTablesD)));
  return 0;
}

__device__ __forceinline__ df dot3d(const df a[3], const df b[3]) {
  return df_fma(df_fma(df_mul(a[0], b[0]), a[1], b[1]), a[2], b[2]);
}
__device__ __forceinline__ dfc dfc_fma_re(dfc acc, dfc v, df s) {  // acc + v s
  return dfcmk(df_fma(acc.re, v.re, s), df_fma(acc.im, v.im, s));
}
__device__ __forceinline__ dfc dfc_acc_re(dfc acc, dfc v, df s) {  // acc + v s (accumulators: df_acc)
  return dfcmk(df_acc(acc.re, v.re, s), df_acc(acc.im, v.im, s));
}

#define GB_ND(n) ((n) > 0 ? (n) : 1)
// sums of one pair; NS = the shape functions held: 4, or 3 where the
// source element is known to be a triangle (its fourth shape function is zero)
template <int NDIR, int NS = 4>
struct AccDN {
  dfc G[NS], H[NS];
  df F;
  dfc dG[GB_ND(NDIR)][NS], dH[GB_ND(NDIR)][NS];
  df dF[GB_ND(NDIR)];
};

template <int NDIR>
struct PairDN {
  df R0[3], a0;
  df c1[3], c2[3], c3[3];
  df w0[3], w1[3], w2[3];
  df vt[GB_ND(NDIR)][3];
  df kr, ki;
  // a flat triangle's surface vector is w0 everywhere: |w0| and w0 . vt[q]
  // once per pair instead of at every point
  df aW, Wv[GB_ND(NDIR)];
};

// the integrand at one point (R = r - rt, W = the surface vector, shape
// functions N, weight w) added to the sums
template <int NDIR, int NS = 4>
__device__ __forceinline__ void reg_kernel_dn(const PairDN<NDIR>& P, const df R[3], const df W[3], const df N[4], df w,
                                              AccDN<NDIR, NS>& A, int ns = NS) {
  const bool tri = ns == 3;  // flat triangle: W = w0, |W| and W . vt[q] from the pair
  const df aR = df_sqrt(dot3d(R, R));
  const df iR = df_rcp(aR);
  const df aW = tri ? P.aW : df_sqrt(dot3d(W, W));
  const df dl = df_sub(aR, P.a0);
  df sn, cs;
  df_sincos(df_mul(P.kr, dl), &sn, &cs);
  dfc ph = dfcmk(cs, sn);  // e^{ik(|R| - |R0|)}
  if (P.ki.hi != 0.0f) ph = dfc_scale(ph, df_exp(df_neg(df_mul(P.ki, dl))));
  const dfc kR = dfcmk(df_mul(P.kr, aR), df_mul(P.ki, aR));
  const dfc cb = dfcmk(df_add_f(df_neg(kR.im), -1.0f), kR.re);  // i k R - 1
  const df iR2 = df_sqr(iR);
  const df rdW = df_mul(dot3d(R, W), iR);
  const df tD = df_mul(rdW, iR2);
  const dfc g = dfc_scale(ph, df_mul(df_mul(iR, aW), w));
  const dfc cbe = dfc_mul(cb, ph);
  const dfc h = dfc_scale(cbe, df_mul(tD, w));
  // ns = 3 for a triangle, whose fourth shape function is zero: skipped
#pragma unroll
  for (int n = 0; n < NS; n++) {
    if (n < ns) {
      A.G[n] = dfc_acc_re(A.G[n], g, N[n]);
      A.H[n] = dfc_acc_re(A.H[n], h, N[n]);
    }
  }
  A.F = df_acc(A.F, w, tD);
  if (NDIR > 0) {
    const dfc t1 = dfc_add(dfc_mul(kR, kR), dfcmk(df_mul_f(cb.re, 3.0f), df_mul_f(cb.im, 3.0f)));
    const df iR3w = df_mul(df_mul(iR2, iR), w);
#pragma unroll
    for (int q = 0; q < NDIR; q++) {
      const df rdv = df_mul(dot3d(R, P.vt[q]), iR);
      const df Wdv = tri ? P.Wv[q] : dot3d(W, P.vt[q]);
      const dfc dg = dfc_scale(cbe, df_mul(df_mul(iR2, rdv), df_mul(aW, w)));
      const dfc u = dfc_add(dfc_scale(t1, df_mul(rdv, rdW)), dfc_scale(cb, df_neg(Wdv)));
      const dfc dh = dfc_scale(dfc_mul(ph, u), iR3w);
#pragma unroll
      for (int n = 0; n < NS; n++) {
        if (n < ns) {
          A.dG[q][n] = dfc_acc_re(A.dG[q][n], dg, N[n]);
          A.dH[q][n] = dfc_acc_re(A.dH[q][n], dh, N[n]);
        }
      }
      A.dF[q] = df_acc(A.dF[q], iR3w, df_sub(df_mul_f(df_mul(rdv, rdW), 3.0f), Wdv));
    }
  }
}


// Points per direction of the regular rule of a pair in the adaptive form.
// With a = |c1| + |c2| (+ |c3| for a quadrangle) the size of the source
// element's parameter map and D = |R0| / a the distance of the observation
// point from the element's point (0, 0) in those units:
//   n_D = GLN for D < 2, 9 for D < 3, 6 for D < 5, 5 beyond (the integrand's
//         nearest complex singularity bounds the Gauss error);
//   n_k = 5, 7, 8 for |k| a <= 0.75, 2.4, 4.5, else GLN (the phase
//         e^{ik|R|} varies by up to |k| a over the element); a triangle,
//         whose three sub-quadrangles each span about half of a, takes
//         5, 6 for |k| a <= 1.2, 2.4 (largest error over random triangles
//         at D >= 3 against a 40-point rule: 5e-13 of the natural scale);
// n = max(n_D, n_k).  Calibrated against a 24-point rule on cubed-sphere
// quadrangles (4 and 8 per face) and cone triangles (the reference's three
// sub-quadrangle map): every output of a pair (G, H, F and the two
// derivative sets) is within ~1e-12 of its natural scale (area / R^p with
// the (1 + |k| R) factors of the kernel).
__device__ __forceinline__ int reg_order(const Elem& S, double a0, cplx k) {
  double a = 0.0;
#pragma unroll
  for (int j = 1; j < 4; j++) {
    if (j == 3 && !S.quad) break;
    a += sqrt(S.cr[0][j] * S.cr[0][j] + S.cr[1][j] * S.cr[1][j] + S.cr[2][j] * S.cr[2][j]);
  }
  const double D = a0 / a, ka = sqrt(k.x * k.x + k.y * k.y) * a;
  const int nD = D < 2.0 ? GB_GLN : (D < 3.0 ? 9 : (D < 5.0 ? 6 : 5));
  const int nk = S.quad ? (ka <= 0.75 ? 5 : (ka <= 2.4 ? 7 : (ka <= 4.5 ? 8 : GB_GLN)))
                        : (ka <= 1.2 ? 5 : (ka <= 2.4 ? 6 : (ka <= 4.5 ? 8 : GB_GLN)));
  // a triangle at D >= 3 with ka <= 3.6: the conical product rule over the
  // whole triangle, returned as -n (n^2 points instead of 3 n^2; largest
  // error over random triangles against a 40-point sub-quadrangle rule:
  // 7e-13 of the natural scale for n = 5, ka <= 0.6, D >= 8; 1e-13 for n = 6,
  // ka <= 1.2, D >= 5; 2e-13 for n = 7, ka <= 2.4; 1e-13 for n = 8, ka <= 3.6)
  if (!S.quad && D >= 3.0 && ka <= 3.6)
    return (ka <= 0.6 && D >= 8.0) ? -5 : ((ka <= 1.2 && D >= 5.0) ? -6 : (ka <= 2.4 ? -7 : -8));
  const int n = nD > nk ? nD : nk;
  return n < GB_GLN ? n : GB_GLN;
}

// Points q0, q0 + qstep, ... of the n x n Gauss-Legendre rule over source
// element S -- the tensor rule on a quadrangle, the same on each of the
// three sub-quadrangles of a triangle (the reference's maps) -- added to A.
// GH: the GHN rule (n = GHN), else the rule of nq points (tables at off).
// con > 0 (a triangle): the conical rule of con^2 points instead (tables at
// gb_con_off(con)).
template <int NDIR, bool GH, int NS = 4>
__device__ __forceinline__ void reg_points_dn(const Elem& S, const PairDN<NDIR>& P, int nq, int off, int q0, int qstep,
                                              AccDN<NDIR, NS>& A, int con = 0) {
  const bool quad = NS == 4 && S.quad;  // NS = 3: the source is a triangle
  const int npts = con ? con * con : (quad ? 1 : 3) * nq * nq;
  const int coff = con ? gb_con_off(con) : 0;
  const df s3 = dfmk(1.7320507764816284f, 3.1087250107475484e-08f);  // sqrt(3)
#pragma unroll 1
  for (int q = q0; q < npts; q += qstep) {
    df z, e, w, N[4];
    if (!GH && con) {
      const float2 cz = c_tabd.cz[coff + q], ce = c_tabd.ce[coff + q], cw = c_tabd.cwt[coff + q];
      z = dfmk(cz.x, cz.y);
      e = dfmk(ce.x, ce.y);
      w = dfmk(cw.x, cw.y);
      const df se = df_mul(s3, e);  // 3 x the shape functions, as below
      N[0] = df_add_f(df_mul_f(df_add(z, se), -2.5f), 1.0f);
      N[1] = df_add_f(df_mul_f(z, 5.0f), 1.0f);
      N[2] = df_add_f(df_mul_f(df_sub(z, se), -2.5f), 1.0f);
      N[3] = dfmk(0.0f, 0.0f);
    } else {
    int sub = 0, ij = q;
    if (!quad) { sub = q % 3; ij = q / 3; }
    const int i = ij / nq, j = ij - i * nq;
    const float2 xi = GH ? c_tabd.xh[i] : c_tabd.xn[off + i], wi = GH ? c_tabd.wh[i] : c_tabd.wn[off + i];
    const float2 xj = GH ? c_tabd.xh[j] : c_tabd.xn[off + j], wj = GH ? c_tabd.wh[j] : c_tabd.wn[off + j];
    const df x = dfmk(xi.x, xi.y), wx = dfmk(wi.x, wi.y);
    const df y = dfmk(xj.x, xj.y), wy = dfmk(wj.x, wj.y);
    if (quad) {
      z = x;
      e = y;
      w = df_mul(wx, wy);
      const df za = df_mul(z, s3), ea = df_mul(e, s3);  // 1 / GB_P44_N = sqrt(3)
      const df zm = df_add_f(df_neg(za), 1.0f), zp = df_add_f(za, 1.0f);
      const df em = df_add_f(df_neg(ea), 1.0f), ep = df_add_f(ea, 1.0f);
      N[0] = df_mul_f(df_mul(zm, em), 0.25f);
      N[1] = df_mul_f(df_mul(zp, em), 0.25f);
      N[2] = df_mul_f(df_mul(zp, ep), 0.25f);
      N[3] = df_mul_f(df_mul(zm, ep), 0.25f);
    } else {
      // w = wx wy (1 + x/4 + y/4); the three sub-quadrangle maps of the reference
      w = df_mul(df_mul(wx, wy), df_add_f(df_mul_f(df_add(x, y), 0.25f), 1.0f));
      const df xy = df_mul(x, y);
      if (sub == 0) {
        z = df_mul_f(df_add(df_add_f(df_mul_f(df_add(x, y), 2.0f), 3.0f), xy), 0.125f);
        e = df_mul_f(df_mul(s3, df_sub(y, x)), 0.125f);
      } else if (sub == 1) {
        z = df_mul_f(df_sub(df_add_f(df_sub(x, df_mul_f(y, 5.0f)), -3.0f), xy), 0.0625f);
        e = df_mul_f(df_mul(s3, df_add(df_add_f(df_add(df_mul_f(x, 3.0f), y), 3.0f), xy)), 0.0625f);
      } else {
        z = df_mul_f(df_sub(df_add_f(df_sub(y, df_mul_f(x, 5.0f)), -3.0f), xy), 0.0625f);
        e = df_mul_f(df_mul(s3, df_sub(df_add_f(df_neg(df_add(x, df_mul_f(y, 3.0f))), -3.0f), xy)), 0.0625f);
      }
      // 3 x the shape functions (0.5 / GB_P34_N0 = 2.5 exactly); the 1/3 is applied in FP64
      const df se = df_mul(s3, e);
      N[0] = df_add_f(df_mul_f(df_add(z, se), -2.5f), 1.0f);
      N[1] = df_add_f(df_mul_f(z, 5.0f), 1.0f);
      N[2] = df_add_f(df_mul_f(df_sub(z, se), -2.5f), 1.0f);
      N[3] = dfmk(0.0f, 0.0f);
    }
    }
    df R[3], W[3];
    // a triangle's map has no z e term (c3 = 0) and a constant surface vector
    const df ze = quad ? df_mul(z, e) : dfmk(0.0f, 0.0f);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const df lin = df_fma(df_mul(P.c1[d], z), P.c2[d], e);
      R[d] = df_add(P.R0[d], quad ? df_fma(lin, P.c3[d], ze) : lin);
      W[d] = quad ? df_fma(df_fma(P.w0[d], P.w1[d], z), P.w2[d], e) : P.w0[d];
    }
    reg_kernel_dn<NDIR, NS>(P, R, W, N, w, A, quad ? 4 : 3);
  }
}

// the pair's constants in double-float (source element S, observation point
// rt, directions vt, wave number k); returns |R0|, the distance to the
// element's point (0, 0)
template <int NDIR>
__device__ __forceinline__ double pair_setup_dn(const Elem& S, const double rt[3], const double (*vt)[3], cplx k,
                                                PairDN<NDIR>& P) {
  double R0[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    R0[d] = S.cr[d][0] - rt[d];
    P.R0[d] = df_from(R0[d]);
    P.c1[d] = df_from(S.cr[d][1]); P.c2[d] = df_from(S.cr[d][2]); P.c3[d] = df_from(S.cr[d][3]);
    P.w0[d] = df_from(S.cw[d][0]); P.w1[d] = df_from(S.cw[d][1]); P.w2[d] = df_from(S.cw[d][2]);
#pragma unroll
    for (int q = 0; q < NDIR; q++) P.vt[q][d] = df_from(vt[q][d]);
  }
  const double a0 = norm3(R0);
  P.a0 = df_from(a0);
  P.kr = df_from(k.x);
  P.ki = df_from(k.y);
  if (!S.quad) {
    P.aW = df_sqrt(dot3d(P.w0, P.w0));
#pragma unroll
    for (int q = 0; q < NDIR; q++) P.Wv[q] = dot3d(P.w0, P.vt[q]);
  }
  return a0;
}

template <int NDIR, int NS = 4>
__device__ __forceinline__ void acc_zero_dn(AccDN<NDIR, NS>& A) {
  const df zero = dfmk(0.0f, 0.0f);
#pragma unroll
  for (int n = 0; n < NS; n++) {
    A.G[n] = dfcmk(zero, zero);
    A.H[n] = dfcmk(zero, zero);
#pragma unroll
    for (int q = 0; q < GB_ND(NDIR); q++) { A.dG[q][n] = dfcmk(zero, zero); A.dH[q][n] = dfcmk(zero, zero); }
  }
  A.F = zero;
#pragma unroll
  for (int q = 0; q < GB_ND(NDIR); q++) A.dF[q] = zero;
}

// the sums of A as doubles (unscaled), for reductions across threads
template <int NDIR, int NS = 4>
__device__ __forceinline__ void acc_to_double(const AccDN<NDIR, NS>& A, RegAcc<NDIR>& R) {
#pragma unroll
  for (int n = 0; n < 4; n++) {
    if (n >= NS) {  // the triangle's zero fourth shape function
      R.G[n] = R.H[n] = cmk(0.0, 0.0);
#pragma unroll
      for (int q = 0; q < NDIR; q++) R.dG[q][n] = R.dH[q][n] = cmk(0.0, 0.0);
      continue;
    }
    R.G[n] = cmk(df_to(A.G[n].re), df_to(A.G[n].im));
    R.H[n] = cmk(df_to(A.H[n].re), df_to(A.H[n].im));
#pragma unroll
    for (int q = 0; q < NDIR; q++) {
      R.dG[q][n] = cmk(df_to(A.dG[q][n].re), df_to(A.dG[q][n].im));
      R.dH[q][n] = cmk(df_to(A.dH[q][n].re), df_to(A.dH[q][n].im));
    }
  }
  R.F = df_to(A.F);
#pragma unroll
  for (int q = 0; q < NDIR; q++) R.dF[q] = df_to(A.dF[q]);
}

// raw sums R (as acc_to_double gives them) finished into D: the phase
// e^{ik|R0|}, the rule's scale (1/3 of the triangle's tripled shape
// functions) and the sub-domain sign, as reg_finish does in FP64
template <int NDIR>
__device__ __forceinline__ void finish_dn(const RegAcc<NDIR>& R, const Elem& S, bool neg, cplx E0, RegAcc<NDIR>& D) {
  const double S0 = S.quad ? GB_I_FP : 0.0625 * GB_SQ3 * GB_I_SPSQ3;
  const double sh = neg ? -S0 : S0;
  const double s3n = S.quad ? 1.0 : 1.0 / 3.0;
  const cplx eS = E0 * (S0 * s3n), eH = E0 * (sh * s3n), eDG = E0 * (-S0 * s3n);
#pragma unroll
  for (int n = 0; n < 4; n++) {
    D.G[n] = R.G[n] * eS;
    D.H[n] = R.H[n] * eH;
#pragma unroll
    for (int q = 0; q < NDIR; q++) {
      D.dG[q][n] = R.dG[q][n] * eDG;
      D.dH[q][n] = R.dH[q][n] * eH;
    }
  }
  D.F = R.F * sh;
#pragma unroll
  for (int q = 0; q < NDIR; q++) D.dF[q] = R.dF[q] * sh;
}

// GLN x GLN integrals of source element S at the observation point rt (with
// NDIR directions vt) in double-float, finished (scaled, sub-domain sign) into
// D as reg_integrate<NDIR>(S, 2, ...) would; false if the pair must be
// integrated in FP64 (a |dF| within 0.05 of CBD_SDF, or not finite).  why
// (may be null) then tells which: 2 when every dF is finite and one exceeds
// CBD_SDF + 0.05 (the pair certainly takes the GHN fallback rule), else 1.
// adapt: the n x n rule of reg_order instead (n = GLN for near pairs).
template <int NDIR, int NS = 4>
__device__ bool reg_integrate_dn(const Elem& S, const double rt[3], const double (*vt)[3], cplx k, bool neg,
                                 RegAcc<NDIR>& D, bool adapt = false, int* why = nullptr) {
  PairDN<NDIR> P;
  const double a0 = pair_setup_dn<NDIR>(S, rt, vt, k, P);
  int nq = adapt ? reg_order(S, a0, k) : GB_GLN;
  const int con = nq < 0 ? -nq : 0;  // a triangle's conical rule
  if (con) nq = 1;
  const int off = nq * (nq - 1) / 2;
  const cplx E0 = cexpik(k, a0);
  AccDN<NDIR, NS> A;
  acc_zero_dn<NDIR, NS>(A);
  // one loop over every point of the rule, so that the integrand is inlined
  // at one site (the kernel is instruction-fetch bound otherwise)
  reg_points_dn<NDIR, false, NS>(S, P, nq, off, 0, 1, A, con);
  RegAcc<NDIR> R;
  acc_to_double<NDIR, NS>(A, R);
  finish_dn<NDIR>(R, S, neg, E0, D);
  bool fin = true;
  double mx = 0.0;
#pragma unroll
  for (int q = 0; q < NDIR; q++) {
    if (!(fabs(D.dF[q]) <= 1e300)) fin = false;
    else mx = fmax(mx, fabs(D.dF[q]));
  }
  if (!fin || mx > GB_CBD_SDF - 0.05) {
    if (why) *why = (fin && mx > GB_CBD_SDF + 0.05) ? 2 : 1;
    return false;
  }
  return true;
}

// This thread's part (points lane, lane + nthr, ...) of the GHN x GHN rule
// of the pair in double-float, as raw sums (acc_to_double) for a reduction
// across the threads; E0 = e^{ik|R0|} for finish_dn.
template <int NDIR>
__device__ void reg_gh_part_dn(const Elem& S, const double rt[3], const double (*vt)[3], cplx k, int lane, int nthr,
                               RegAcc<NDIR>& R, cplx& E0) {
  PairDN<NDIR> P;
  const double a0 = pair_setup_dn<NDIR>(S, rt, vt, k, P);
  E0 = cexpik(k, a0);
  AccDN<NDIR> A;
  acc_zero_dn<NDIR>(A);
  reg_points_dn<NDIR, true>(S, P, GB_GHN, 0, lane, nthr, A);
  acc_to_double<NDIR>(A, R);
}
