// gb_quad.cuh -- FP64 element quadrature of the Helmholtz boundary integrals.
//
// GPU-first restatement of the reference's element kernels:
//   regular pairs   bil_dcoef_v2_GL/_GH (bil_dcoef_v2.c:142-326), lit_dcoef_v2_GL/_GH
//                   (lit_dcoef_v2.c:185-357), the 4p/9p/7p point rules (bil_coef.c:25-100,
//                   lit_coef.c:25-120) and the single-direction dcoef variants (bil_dcoef.c:50-300);
//   singular pairs  bil_coef_bd (bil_coef.c:244-342), bil_dcoef_bd_tz0_PV/_te0_PV
//                   (bil_dcoef.c:369-739), lit_coef_bd (lit_coef.c:290-349),
//                   lit_dcoef_bd_tz0_PV/_te0_PV (lit_dcoef.c:460-636).
// The reference recomputes the geometry once per shape function and once per
// tangential direction; here each quadrature point is evaluated once and its
// kernel value is scattered to all shape functions and all directions.  The
// rules, nodes, weights, scalings and the sign convention of the sub-domain
// side (negative element id: H, F and their derivatives change sign) are the
// reference's.
#pragma once
#include "gb_common.cuh"

// ------------------------------------------------------------------ regular
// Accumulated integrals of one (observation point, source element) pair.
//  G[n], H[n]  single/double layer coefficients for shape function n
//  F           solid-angle coefficient
//  dG,dH,dF    directional derivatives along NDIR observation directions
template <int NDIR>
struct RegAcc {
  cplx G[4], H[4];
  double F;
  cplx dG[NDIR > 0 ? NDIR : 1][4], dH[NDIR > 0 ? NDIR : 1][4];
  double dF[NDIR > 0 ? NDIR : 1];
};

template <int NDIR>
__device__ __forceinline__ void regacc_zero(RegAcc<NDIR>& A) {
#pragma unroll
  for (int n = 0; n < 4; n++) { A.G[n] = cmk(0, 0); A.H[n] = cmk(0, 0); }
  A.F = 0.0;
#pragma unroll
  for (int d = 0; d < (NDIR > 0 ? NDIR : 1); d++) {
#pragma unroll
    for (int n = 0; n < 4; n++) { A.dG[d][n] = cmk(0, 0); A.dH[d][n] = cmk(0, 0); }
    A.dF[d] = 0.0;
  }
}

// one quadrature point (z,e) with weight w
template <int NDIR>
__device__ __forceinline__ void reg_point(const Elem& E, double z, double e, double w, const double rt[3],
                                          const double (*vt)[3], cplx k, RegAcc<NDIR>& A) {
  double r[3], W[3];
  elem_rw(E, z, e, r, W);
  double R[3] = {r[0] - rt[0], r[1] - rt[1], r[2] - rt[2]};
  double aR = norm3(R);
  double iR = 1.0 / aR;
  double aW = norm3(W);
  cplx ce = cexpik(k, aR);
  cplx cb = cmk(-k.y * aR - 1.0, k.x * aR);  // i k R - 1
  double rdW = dot3(R, W) * iR;
  double tD = rdW * iR * iR;
  double N[4];
  shape_fn(E, z, e, N);
  cplx g = ce * (iR * aW * w);
  cplx h = (cb * ce) * (tD * w);
  // a triangle's fourth shape function is zero: its sums are skipped
  const int ns = E.quad ? 4 : 3;
#pragma unroll
  for (int n = 0; n < 4; n++)
    if (n < ns) { A.G[n] += g * N[n]; A.H[n] += h * N[n]; }
  A.F += w * tD;
  if (NDIR > 0) {
    cplx kR = k * aR;
    cplx t1 = kR * kR + 3.0 * cb;
    double iR3 = iR * iR * iR;
#pragma unroll
    for (int d = 0; d < NDIR; d++) {
      double rdv = dot3(R, vt[d]) * iR;
      double Wdv = dot3(W, vt[d]);
      cplx dg = (cb * ce) * (iR * iR * rdv * aW * w);
      cplx dh = (ce * (t1 * (rdv * rdW) - cb * Wdv)) * (iR3 * w);
#pragma unroll
      for (int n = 0; n < 4; n++)
        if (n < ns) { A.dG[d][n] += dg * N[n]; A.dH[d][n] += dh * N[n]; }
      A.dF[d] += w * iR3 * (3.0 * rdv * rdW - Wdv);
    }
  }
}

// scale factors and the sub-domain sign flip
template <int NDIR>
__device__ __forceinline__ void reg_finish(RegAcc<NDIR>& A, double S, bool neg) {
  double sh = neg ? -S : S;
#pragma unroll
  for (int n = 0; n < 4; n++) { A.G[n] = A.G[n] * S; A.H[n] = A.H[n] * sh; }
  A.F *= sh;
#pragma unroll
  for (int d = 0; d < NDIR; d++) {
#pragma unroll
    for (int n = 0; n < 4; n++) { A.dG[d][n] = A.dG[d][n] * (-S); A.dH[d][n] = A.dH[d][n] * sh; }
    A.dF[d] *= sh;
  }
}

// Quadrature types of the reference: 0 4-point, 1 9-point (quad) / 7-point
// (triangle), 2 GLN x GLN, 3 GHN x GHN.  Triangles use the reference's
// three-quadrangle split of the GL rules.
template <int NDIR>
static __device__ void reg_integrate(const Elem& E, int type, const double rt[3], const double (*vt)[3], cplx k, bool neg,
                              RegAcc<NDIR>& A) {
  regacc_zero(A);
  double S;
  if (E.quad) {
    S = GB_I_FP;
    if (type == 0) {
      for (int j = 0; j < 4; j++) reg_point<NDIR>(E, c_tab.zt_44[j], c_tab.et_44[j], c_tab.wt_44[j], rt, vt, k, A);
    } else if (type == 1) {
      for (int j = 0; j < 9; j++) reg_point<NDIR>(E, c_tab.zt_49[j], c_tab.et_49[j], c_tab.wt_49[j], rt, vt, k, A);
    } else if (type == 2) {
      for (int i = 0; i < GB_GLN; i++)
        for (int j = 0; j < GB_GLN; j++)
          reg_point<NDIR>(E, c_tab.xli[i], c_tab.xli[j], c_tab.wli[i] * c_tab.wli[j], rt, vt, k, A);
    } else {
      for (int i = 0; i < GB_GHN; i++)
        for (int j = 0; j < GB_GHN; j++)
          reg_point<NDIR>(E, c_tab.xhi[i], c_tab.xhi[j], c_tab.whi[i] * c_tab.whi[j], rt, vt, k, A);
    }
  } else {
    if (type == 0 || type == 1) {
      S = GB_I_EP;
      if (type == 0)
        for (int j = 0; j < 4; j++) reg_point<NDIR>(E, c_tab.zt_34[j], c_tab.et_34[j], c_tab.wt_34[j], rt, vt, k, A);
      else
        for (int j = 0; j < 7; j++) reg_point<NDIR>(E, c_tab.zt_37[j], c_tab.et_37[j], c_tab.wt_37[j], rt, vt, k, A);
    } else {
      S = 0.0625 * GB_SQ3 * GB_I_SPSQ3;
      const int n = (type == 2) ? GB_GLN : GB_GHN;
      const double* x = (type == 2) ? c_tab.xli : c_tab.xhi;
      const double* wq = (type == 2) ? c_tab.wli : c_tab.whi;
      for (int i = 0; i < n; i++) {
        double a = x[i];
        for (int j = 0; j < n; j++) {
          double b = x[j];
          double w = wq[i] * wq[j] * (1.0 + 0.25 * a + 0.25 * b);
          reg_point<NDIR>(E, 0.125 * (3.0 + 2.0 * a + 2.0 * b + a * b), 0.125 * GB_SQ3 * (-a + b), w, rt, vt, k, A);
          reg_point<NDIR>(E, 0.0625 * (-3.0 + a - 5.0 * b - a * b), 0.0625 * GB_SQ3 * (3.0 + 3.0 * a + b + a * b), w, rt,
                          vt, k, A);
          reg_point<NDIR>(E, 0.0625 * (-3.0 - 5.0 * a + b - a * b), 0.0625 * GB_SQ3 * (-3.0 - a - 3.0 * b - a * b), w,
                          rt, vt, k, A);
        }
      }
    }
  }
  reg_finish<NDIR>(A, S, neg);
}

// Partial integral over a strided subset of the points of the GHN rule: used
// by the block-cooperative fallback kernels (one block per pair); the caller
// reduces the partial sums and then calls reg_finish.
template <int NDIR>
static __device__ void reg_integrate_gh_part(const Elem& E, int tid, int nthr, const double rt[3], const double (*vt)[3],
                                      cplx k, RegAcc<NDIR>& A) {
  regacc_zero(A);
  for (int p = tid; p < GB_GHN * GB_GHN; p += nthr) {
    int i = p / GB_GHN, j = p % GB_GHN;
    if (E.quad) {
      reg_point<NDIR>(E, c_tab.xhi[i], c_tab.xhi[j], c_tab.whi[i] * c_tab.whi[j], rt, vt, k, A);
    } else {
      double a = c_tab.xhi[i], b = c_tab.xhi[j];
      double w = c_tab.whi[i] * c_tab.whi[j] * (1.0 + 0.25 * a + 0.25 * b);
      reg_point<NDIR>(E, 0.125 * (3.0 + 2.0 * a + 2.0 * b + a * b), 0.125 * GB_SQ3 * (-a + b), w, rt, vt, k, A);
      reg_point<NDIR>(E, 0.0625 * (-3.0 + a - 5.0 * b - a * b), 0.0625 * GB_SQ3 * (3.0 + 3.0 * a + b + a * b), w, rt, vt,
                      k, A);
      reg_point<NDIR>(E, 0.0625 * (-3.0 - 5.0 * a + b - a * b), 0.0625 * GB_SQ3 * (-3.0 - a - 3.0 * b - a * b), w, rt,
                      vt, k, A);
    }
  }
}
__device__ __forceinline__ double reg_scale_gh(const Elem& E) { return E.quad ? GB_I_FP : 0.0625 * GB_SQ3 * GB_I_SPSQ3; }

// ------------------------------------------------------------------ singular
// Observation point on its own element at parameter (zt,et).  The element is
// cut into triangles from the point to each edge (polar coordinates r,theta);
// the derivative integrals are split into the disc D_eps (r < DEPS, principal
// value) and its complement.  All shape functions and both tangential
// directions (t_zeta, t_eta) are accumulated together.
struct SingAcc {
  cplx G[4], H[4];
  double F;
  cplx dG[2][4], dH[2][4];
  double dF[2];
};

__device__ __forceinline__ void singacc_zero(SingAcc& A) {
  for (int n = 0; n < 4; n++) { A.G[n] = cmk(0, 0); A.H[n] = cmk(0, 0); }
  A.F = 0.0;
  for (int d = 0; d < 2; d++) {
    for (int n = 0; n < 4; n++) { A.dG[d][n] = cmk(0, 0); A.dH[d][n] = cmk(0, 0); }
    A.dF[d] = 0.0;
  }
}

// polar decomposition of the element around (zt,et): radii and angles of the
// corners (reference bil_calc_node_r_th d3b1_elem.c:667, lit_calc_node_r_th :700)
__device__ __forceinline__ int node_r_th(int quad, double zt, double et, double r[5], double th[5]) {
  if (quad) {
    double ztp = 1.0 - zt, ztm = -1.0 - zt, etp = 1.0 - et, etm = -1.0 - et;
    r[0] = sqrt(ztm * ztm + etm * etm);
    r[1] = sqrt(ztp * ztp + etm * etm);
    r[2] = sqrt(ztp * ztp + etp * etp);
    r[3] = sqrt(ztm * ztm + etp * etp);
    r[4] = r[0];
    th[0] = atan2(etm, ztm);
    th[1] = atan2(etm, ztp);
    th[2] = atan2(etp, ztp);
    th[3] = atan2(etp, ztm);
    th[4] = th[0] + 2.0 * GB_PI;
    return 4;
  } else {
    double ztp = 1.0 - zt, ztm = -0.5 - zt, etp = 0.5 * GB_SQ3 - et, etm = -0.5 * GB_SQ3 - et;
    r[0] = sqrt(ztm * ztm + etm * etm);
    r[1] = sqrt(ztp * ztp + et * et);
    r[2] = sqrt(ztm * ztm + etp * etp);
    r[3] = r[0];
    th[0] = atan2(etm, ztm);
    th[1] = atan2(-et, ztp);
    th[2] = atan2(etp, ztm);
    th[3] = th[0] + 2.0 * GB_PI;
    r[4] = 0.0;
    th[4] = 0.0;
    return 3;
  }
}

struct SingCtx {
  Elem E;
  double zt, et;
  cplx k;
  double vt[2][3];   // non-unit tangents T_zeta, T_eta at (zt,et)
  double iaT[2];     // 1/|T|
  int planar;        // bilinear element lies in a plane: H, F and their derivatives vanish
  double bdC;        // b . C of the bilinear element
  int nedge;
  double r[5], th[5];
};

__device__ __forceinline__ void sing_setup(SingCtx& c) {
  const Elem& E = c.E;
  for (int d = 0; d < 3; d++) {
    c.vt[0][d] = E.cr[d][1] + E.cr[d][3] * c.et;
    c.vt[1][d] = E.cr[d][2] + E.cr[d][3] * c.zt;
  }
  c.iaT[0] = 1.0 / norm3(c.vt[0]);
  c.iaT[1] = 1.0 / norm3(c.vt[1]);
  if (E.quad) {
    double bdc = E.cr[0][1] * E.cw[0][2] + E.cr[1][1] * E.cw[1][2] + E.cr[2][1] * E.cw[2][2];
    double ab = sqrt(E.cr[0][1] * E.cr[0][1] + E.cr[1][1] * E.cr[1][1] + E.cr[2][1] * E.cr[2][1]);
    double aC = sqrt(E.cw[0][2] * E.cw[0][2] + E.cw[1][2] * E.cw[1][2] + E.cw[2][2] * E.cw[2][2]);
    c.planar = (fabs(bdc / (ab * aC)) < 1.0e-15) ? 1 : 0;  // NaN (C = 0) compares false, as in the reference
    c.bdC = bdc;
  } else {
    c.planar = 1;
    c.bdC = 0.0;
  }
  c.nedge = node_r_th(E.quad, c.zt, c.et, c.r, c.th);
}

// theta of point m (0..GHN-1) of half h (0,1) of edge j, its weight and the
// distance rm to the edge along that direction
__device__ __forceinline__ void sing_edge_theta(const SingCtx& c, int j, int h, int m, double* th, double* wth,
                                                double* rm) {
  double t0 = c.th[j], t1 = c.th[j + 1];
  double dt = t1 - t0;
  double x = c_tab.xhi[m];
  *th = (h == 0) ? 0.25 * dt * x + 0.25 * (t1 + 3.0 * t0) : 0.25 * dt * x + 0.25 * (3.0 * t1 + t0);
  *wth = 0.25 * dt * c_tab.whi[m];
  double r0 = c.r[j], r1 = c.r[j + 1];
  *rm = r0 * r1 * sin(t1 - t0) / (r0 * sin(*th - t0) - r1 * sin(*th - t1));
}

// geometry along a ray: K = d r / d rho, W(zeta,eta)
__device__ __forceinline__ void sing_ray(const Elem& E, double zt, double et, double cth, double sth, double rr,
                                         double K[3], double W[3], double* zeta, double* eta) {
  *zeta = rr * cth + zt;
  *eta = rr * sth + et;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    K[d] = E.cr[d][1] * cth + E.cr[d][2] * sth + E.cr[d][3] * (rr * cth * sth + zt * sth + et * cth);
    W[d] = E.cw[d][0] + E.cw[d][1] * (*zeta) + E.cw[d][2] * (*eta);
  }
}

// ---- bilinear element: work items
// set A: G,H,F on [0,rm] with GLN points          (bil_coef_bd)
static __device__ void sing_bil_setA(const SingCtx& c, double cth, double sth, double rm, double wth, SingAcc& A) {
  const Elem& E = c.E;
  for (int i = 0; i < GB_GLN; i++) {
    double rr = 0.5 * rm * (c_tab.xli[i] + 1.0);
    double w = wth * 0.5 * rm * c_tab.wli[i];
    double K[3], W[3], z, e;
    sing_ray(E, c.zt, c.et, cth, sth, rr, K, W, &z, &e);
    double aK = norm3(K), aW = norm3(W);
    cplx ce = cexpik(c.k, aK * rr);
    double N[4];
    shape_bil(z, e, N);
    cplx g = ce * (w * aW / aK);
    for (int n = 0; n < 4; n++) A.G[n] += g * N[n];
    if (!c.planar) {
      double iK3 = 1.0 / (aK * aK * aK);
      cplx kR = c.k * (rr * aK);
      cplx h = (cmk(-kR.y - 1.0, kR.x) * ce) * (w * iK3 * cth * sth);
      for (int n = 0; n < 4; n++) A.H[n] += h * N[n];
      A.F += w * iK3 * cth * sth;
    }
  }
}
// set B: derivative integrals on [DEPS,rm] with GHN points (D-bar_eps part)
static __device__ void sing_bil_setB(const SingCtx& c, double cth, double sth, double rm, double wth, SingAcc& A) {
  const Elem& E = c.E;
  const double cs[2] = {cth, sth}, outer[2] = {sth, cth};
  for (int i = 0; i < GB_GHN; i++) {
    double rr = 0.5 * (rm - GB_DEPS) * c_tab.xhi[i] + 0.5 * (rm + GB_DEPS);
    double w = wth * 0.5 * (rm - GB_DEPS) * c_tab.whi[i];
    double K[3], W[3], z, e;
    sing_ray(E, c.zt, c.et, cth, sth, rr, K, W, &z, &e);
    double aK = norm3(K), aW = norm3(W);
    double iK = 1.0 / aK;
    cplx kR = c.k * (rr * aK);
    cplx ce = cexpik(c.k, aK * rr);
    cplx cb = cmk(-kR.y - 1.0, kR.x);
    double N[4];
    shape_bil(z, e, N);
    cplx cbce = cb * ce;
    cplx t1 = kR * kR + 3.0 * cb;
    double iK5r = 1.0 / (rr * aK * aK * aK * aK * aK);
    for (int d = 0; d < 2; d++) {
      double KdT = dot3(K, c.vt[d]);
      cplx g = cbce * (w * iK * iK / rr * KdT * iK * aW);
      for (int n = 0; n < 4; n++) A.dG[d][n] += g * N[n];
      if (!c.planar) {
        double wo = w * outer[d];
        cplx h = (ce * (t1 * (KdT * cs[d]) - cb * (aK * aK))) * (wo * iK5r);
        for (int n = 0; n < 4; n++) A.dH[d][n] += h * N[n];
        A.dF[d] += wo * iK5r * (3.0 * KdT * cs[d] - aK * aK);
      }
    }
  }
}
// set C: D_eps disc, r in [0,DEPS] with GLN points; the reference multiplies
// the dG part by i (bil_dcoef.c:425) and splits the dH part into De0 - i De1
static __device__ void sing_bil_setC(const SingCtx& c, double cth, double sth, double wth, SingAcc& A) {
  const Elem& E = c.E;
  const double cs[2] = {cth, sth}, outer[2] = {sth, cth};
  cplx ik = cmuli(c.k);
  for (int i = 0; i < GB_GLN; i++) {
    double rr = 0.5 * GB_DEPS * (c_tab.xli[i] + 1.0);
    double w = wth * 0.5 * GB_DEPS * c_tab.wli[i];
    double K[3], W[3], z, e;
    sing_ray(E, c.zt, c.et, cth, sth, rr, K, W, &z, &e);
    double aK = norm3(K), aW = norm3(W);
    double iK = 1.0 / aK;
    cplx kR = c.k * (aK * rr);
    cplx cb = cmk(-kR.y - 1.0, kR.x);
    cplx cc, sn;
    ccossin(kR, &cc, &sn);
    cplx ce = cexpik(c.k, aK * rr);
    double N[4];
    shape_bil(z, e, N);
    cplx gbase = cb * sn + kR * cc;
    double aK2 = aK * aK;
    for (int d = 0; d < 2; d++) {
      double KdT = dot3(K, c.vt[d]);
      cplx g = cmuli(gbase) * (w * iK * iK / rr * (KdT * iK) * aW);
      for (int n = 0; n < 4; n++) A.dG[d][n] += g * N[n];
      if (!c.planar) {
        double wo = w * outer[d];
        cplx v0 = (ce * ((c.k * kR + 3.0 * ik) * (KdT * cs[d]) - ik * aK2)) * (1.0 / (aK2 * aK2));
        cplx v1 = sn * ((3.0 * KdT * cs[d] - aK2) / (aK2 * aK2 * aK * rr));
        cplx h = (v0 - cmuli(v1)) * wo;
        for (int n = 0; n < 4; n++) A.dH[d][n] += h * N[n];
      }
    }
  }
}
// set D: principal-value pairing of +r and -r, r in [0,DEPS] with GLN points
static __device__ void sing_bil_setD(const SingCtx& c, double cth, double sth, double wth, SingAcc& A) {
  const Elem& E = c.E;
  const double cs[2] = {cth, sth}, outer[2] = {sth, cth};
  for (int i = 0; i < GB_GLN; i++) {
    double rr = 0.5 * GB_DEPS * (c_tab.xli[i] + 1.0);
    double w = wth * 0.5 * GB_DEPS * c_tab.wli[i];
    double Kp[3], Wp[3], zp, ep, Km[3], Wm[3], zm, em;
    sing_ray(E, c.zt, c.et, cth, sth, rr, Kp, Wp, &zp, &ep);
    sing_ray(E, c.zt, c.et, -cth, -sth, rr, Km, Wm, &zm, &em);
    // K for the minus point keeps +cth,+sth directions (reference bil_sdG_DP_r)
    for (int d = 0; d < 3; d++) {
      Km[d] = E.cr[d][1] * cth + E.cr[d][2] * sth + E.cr[d][3] * (-rr * cth * sth + c.zt * sth + c.et * cth);
    }
    double aKp = norm3(Kp), aWp = norm3(Wp), aKm = norm3(Km), aWm = norm3(Wm);
    cplx kRp = c.k * (aKp * rr), kRm = -(c.k * (aKm * rr));
    cplx ccp, snp, ccm, snm;
    ccossin(kRp, &ccp, &snp);
    ccossin(kRm, &ccm, &snm);
    double Np[4], Nm[4];
    shape_bil(zp, ep, Np);
    shape_bil(zm, em, Nm);
    double ir = 1.0 / rr;
    double aKp2 = aKp * aKp, aKm2 = aKm * aKm;
    double iKp5 = 1.0 / (aKp2 * aKp2 * aKp), iKm5 = 1.0 / (aKm2 * aKm2 * aKm);
    for (int d = 0; d < 2; d++) {
      double KpdT = dot3(Kp, c.vt[d]), KmdT = dot3(Km, c.vt[d]);
      // dG: subtract
      cplx gp = ccp * (w * ir / aKp2 * (KpdT / aKp) * aWp);
      cplx gm = ccm * (w * ir / aKm2 * (KmdT / aKm) * aWm);
      for (int n = 0; n < 4; n++) A.dG[d][n] -= gp * Np[n] - gm * Nm[n];
      if (!c.planar) {
        double wo = w * outer[d] * ir;
        double fp = iKp5 * (3.0 * KpdT * cs[d] - aKp2), fm = iKm5 * (3.0 * KmdT * cs[d] - aKm2);
        cplx hp = ccp * (wo * fp), hm = ccm * (wo * fm);
        for (int n = 0; n < 4; n++) A.dH[d][n] -= hp * Np[n] - hm * Nm[n];
        A.dF[d] += wo * (fp - fm);
      }
    }
  }
}

// ---- linear triangle: work items (H, F and their derivatives vanish on the
// own planar element)
static __device__ void sing_lit_setA(const SingCtx& c, double cth, double sth, double rm, double wth, SingAcc& A) {
  const Elem& E = c.E;
  double K[3];
  for (int d = 0; d < 3; d++) K[d] = E.cr[d][1] * cth + E.cr[d][2] * sth;
  double aK = norm3(K);
  for (int i = 0; i < GB_GLN; i++) {
    double rr = 0.5 * rm * (c_tab.xli[i] + 1.0);
    double w = wth * 0.5 * rm * c_tab.wli[i];
    cplx ce = cexpik(c.k, aK * rr);
    double N[4];
    shape_lit(rr * cth + c.zt, rr * sth + c.et, N);
    cplx g = ce * (w / aK);
    for (int n = 0; n < 3; n++) A.G[n] += g * N[n];
  }
}
static __device__ void sing_lit_setB(const SingCtx& c, double cth, double sth, double rm, double wth, SingAcc& A) {
  const Elem& E = c.E;
  double K[3];
  for (int d = 0; d < 3; d++) K[d] = E.cr[d][1] * cth + E.cr[d][2] * sth;
  double aK = norm3(K), iK = 1.0 / aK;
  double Kdv[2] = {dot3(K, c.vt[0]) * iK, dot3(K, c.vt[1]) * iK};
  for (int i = 0; i < GB_GHN; i++) {
    double rr = 0.5 * (rm - GB_DEPS) * c_tab.xhi[i] + 0.5 * (rm + GB_DEPS);
    double w = wth * 0.5 * (rm - GB_DEPS) * c_tab.whi[i];
    cplx kR = c.k * (aK * rr);
    cplx ce = cexpik(c.k, aK * rr);
    cplx cb = cmk(-kR.y - 1.0, kR.x);
    double N[4];
    shape_lit(rr * cth + c.zt, rr * sth + c.et, N);
    cplx base = (cb * ce) * (w / rr * iK * iK);
    for (int d = 0; d < 2; d++) {
      cplx g = base * Kdv[d];
      for (int n = 0; n < 3; n++) A.dG[d][n] += g * N[n];
    }
  }
}
// derivative of the triangle shape functions along the ray (lit_dNn_pr_cs)
__device__ __forceinline__ void lit_dN_ray(double cth, double sth, double dN[3]) {
  const double ia = 0.5 / GB_P34_N0;
  dN[0] = -2.0 / 3.0 * ia * (cth + GB_SQ3 * sth);
  dN[1] = 4.0 / 3.0 * ia * cth;
  dN[2] = -2.0 / 3.0 * ia * (cth - GB_SQ3 * sth);
}
// set C (analytic disc integral) and set D (principal value); both carry the
// reference's 1/k factor (lit_dcoef.c:500-520)
static __device__ void sing_lit_setCD(const SingCtx& c, double cth, double sth, double wth, int setC, SingAcc& A) {
  const Elem& E = c.E;
  double K[3];
  for (int d = 0; d < 3; d++) K[d] = E.cr[d][1] * cth + E.cr[d][2] * sth;
  double aK = norm3(K), iK = 1.0 / aK;
  double iK3 = iK * iK * iK;
  double dN[3];
  lit_dN_ray(cth, sth, dN);
  cplx keK = c.k * (GB_DEPS * aK);
  cplx cc, sn;
  ccossin(keK, &cc, &sn);
  cplx val;
  if (setC) {
    // i/k * ((keK + i) sin + (2 - i keK) cos - 2)
    cplx t = (keK + cmk(0.0, 1.0)) * sn + (cmk(2.0, 0.0) - cmuli(keK)) * cc - cmk(2.0, 0.0);
    val = cdivc(cmuli(t), c.k);
  } else {
    val = -cdivc(sn, c.k);
  }
  for (int d = 0; d < 2; d++) {
    double Kdv = dot3(K, c.vt[d]) * iK;
    cplx g = val * (wth * iK3 * Kdv);
    for (int n = 0; n < 3; n++) A.dG[d][n] += g * dN[n];
  }
}

// final scalings of the singular integrals and the sub-domain sign flip
static __device__ void sing_finish(const SingCtx& c, SingAcc& A, bool neg) {
  double sh = neg ? -1.0 : 1.0;
  if (c.E.quad) {
    for (int n = 0; n < 4; n++) {
      A.G[n] = A.G[n] * GB_I_FP;
      A.H[n] = c.planar ? cmk(0, 0) : A.H[n] * (GB_I_FP * c.bdC * sh);
    }
    A.F = c.planar ? 0.0 : A.F * GB_I_FP * c.bdC * sh;
    for (int d = 0; d < 2; d++) {
      for (int n = 0; n < 4; n++) {
        A.dG[d][n] = A.dG[d][n] * (-GB_I_FP * c.iaT[d]);
        A.dH[d][n] = c.planar ? cmk(0, 0) : A.dH[d][n] * (c.bdC * GB_I_FP * c.iaT[d] * sh);
      }
      A.dF[d] = c.planar ? 0.0 : A.dF[d] * c.bdC * GB_I_FP * c.iaT[d] * sh;
    }
  } else {
    double aW = sqrt(c.E.cw[0][0] * c.E.cw[0][0] + c.E.cw[1][0] * c.E.cw[1][0] + c.E.cw[2][0] * c.E.cw[2][0]);
    for (int n = 0; n < 4; n++) {
      A.G[n] = (n < 3) ? A.G[n] * (GB_I_SPSQ3 * aW) : cmk(0, 0);
      A.H[n] = cmk(0, 0);
    }
    A.F = 0.0;
    for (int d = 0; d < 2; d++) {
      for (int n = 0; n < 4; n++) {
        A.dG[d][n] = (n < 3) ? A.dG[d][n] * (-GB_I_SPSQ3 * aW * c.iaT[d]) : cmk(0, 0);
        A.dH[d][n] = cmk(0, 0);
      }
      A.dF[d] = 0.0;
    }
  }
}

// Work decomposition of one singular pair into independent items, so that a
// block of threads can share it: returns the number of items; item q runs one
// theta direction of one of the sets A-D.  want_d == 0 evaluates G, H, F only
// (coef_bd), want_d == 1 also the derivatives (dcoef_bd_*_PV).
__device__ __forceinline__ int sing_items(const SingCtx& c, int want_d) {
  int ne = c.nedge;
  int nA = ne * 2 * GB_GHN;                 // edge x half x theta
  if (!want_d) return nA;
  return 2 * nA + 4 * GB_GHN + 2 * GB_GHN;  // + set B + set C (4 quarters) + set D (2 halves)
}
static __device__ void sing_item(const SingCtx& c, int q, SingAcc& A) {
  int ne = c.nedge;
  int nA = ne * 2 * GB_GHN;
  if (q < 2 * nA) {
    int setB = q >= nA;
    int qq = setB ? q - nA : q;
    int j = qq / (2 * GB_GHN), rem = qq % (2 * GB_GHN);
    int h = rem / GB_GHN, m = rem % GB_GHN;
    double th, wth, rm;
    sing_edge_theta(c, j, h, m, &th, &wth, &rm);
    double sth, cth;
    sincos(th, &sth, &cth);
    if (c.E.quad) {
      if (setB) sing_bil_setB(c, cth, sth, rm, wth, A); else sing_bil_setA(c, cth, sth, rm, wth, A);
    } else {
      if (setB) sing_lit_setB(c, cth, sth, rm, wth, A); else sing_lit_setA(c, cth, sth, rm, wth, A);
    }
    return;
  }
  q -= 2 * nA;
  if (q < 4 * GB_GHN) {  // set C: theta over (-pi, pi] in four quarters
    int quarter = q / GB_GHN, m = q % GB_GHN;
    const double off[4] = {-0.75 * GB_PI, -0.25 * GB_PI, 0.25 * GB_PI, 0.75 * GB_PI};
    double th = 0.25 * GB_PI * c_tab.xhi[m] + off[quarter];
    double wth = 0.25 * GB_PI * c_tab.whi[m];
    double sth, cth;
    sincos(th, &sth, &cth);
    if (c.E.quad) sing_bil_setC(c, cth, sth, wth, A); else sing_lit_setCD(c, cth, sth, wth, 1, A);
    return;
  }
  q -= 4 * GB_GHN;
  {  // set D: theta over (0, pi) in two halves
    int half = q / GB_GHN, m = q % GB_GHN;
    double th = 0.25 * GB_PI * c_tab.xhi[m] + (half == 0 ? 0.25 * GB_PI : 0.75 * GB_PI);
    double wth = 0.25 * GB_PI * c_tab.whi[m];
    double sth, cth;
    sincos(th, &sth, &cth);
    if (c.E.quad) sing_bil_setD(c, cth, sth, wth, A); else sing_lit_setCD(c, cth, sth, wth, 0, A);
  }
}
