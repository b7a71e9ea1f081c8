/*
 * bem_port.c -- CPU restatement of the reference's BEM element quadrature,
 * coefficient-matrix assembly, solid-angle domain test and field sums.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py as the checker; the product never calls it.
 *
 * It follows the reference (akohta/bem3_emf_b2) function by function, in its
 * loop order (shape function outermost, as the reference does), so that it is
 * an independent restatement of the GPU kernels' arithmetic:
 *   port_reg       bil_dcoef_v2_GL/GH bil_dcoef_v2.c:142-326, bil_coef_4p/9p/GL/GH
 *                  bil_coef.c:25-200, lit_dcoef_v2_GL/GH lit_dcoef_v2.c:185-357,
 *                  lit_coef_4p/7p/GL/GH lit_coef.c:25-250, single-direction dcoef
 *                  bil_dcoef.c:50-300, lit_dcoef.c:25-300
 *   port_sing_bil  bil_coef_bd bil_coef.c:244-342 + bil_dcoef_bd_tz0_PV/te0_PV
 *                  bil_dcoef.c:369-739 (integrands :824-1631)
 *   port_sing_lit  lit_coef_bd lit_coef.c:290-349 + lit_dcoef_bd_tz0_PV/te0_PV
 *                  lit_dcoef.c:460-636 (integrands :638-955)
 *   port_pair      dcoef_bd_node_t2 d3b1_elem.c:482-539 (GHN fallback on |Re dF| > 0.5)
 *   port_rows      create_cmatrix_domain solve_bieq2.c:98-184 for a subset of rows
 *   port_domain_id domain_id / fid_calc_solid_angle setup2.c:871-978
 *   port_field     mEMP_s / EH_s / EH_mEMP_s / mEMP2_s d3b1_field.c:12-139, mo_solve.c:351-396
 *   port_field_bd  EH_s_bd d3b1_field.c:238-279
 * Parity pinned against the reference's own outputs (tests/golden).
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cd;

#define P_GLN 12
#define P_GHN 64
#define P_IFP 7.957747154594766788444e-2
#define P_IEP 3.978873577297383394222e-2
#define P_SQ3 1.732050807568877293528e+0
#define P_ISPSQ3 3.062938307898844719507e-2
#define P_DEPS 0.1
#define P_PI 3.14159265358979323846

static double xl[P_GLN], wl[P_GLN], xh[P_GHN], wh[P_GHN];
static int tab_ready = 0;

/* Newton iteration for the Gauss-Legendre nodes (same method as the
 * reference's gauleg.c:3-36) */
static void port_gauleg(double *x, double *w, int n) {
  int m = (n + 1) / 2;
  for (int i = 1; i <= m; i++) {
    double z = cos(P_PI * ((double)i - 0.25) / ((double)n + 0.5)), z1, pp, p1, p2, p3;
    do {
      p1 = 1.0; p2 = 0.0;
      for (int j = 1; j <= n; j++) { p3 = p2; p2 = p1; p1 = ((double)(2 * j - 1) * z * p2 - (double)(j - 1) * p3) / (double)j; }
      pp = (double)n * (z * p1 - p2) / (z * z - 1.0);
      z1 = z;
      z = z1 - p1 / pp;
    } while (fabs(z - z1) > 3.0e-16);
    x[i - 1] = -z; x[n - i] = z;
    w[i - 1] = 2.0 / ((1.0 - z * z) * pp * pp); w[n - i] = w[i - 1];
  }
}
static void tables(void) {
  if (tab_ready) return;
  port_gauleg(xl, wl, P_GLN);
  port_gauleg(xh, wh, P_GHN);
  tab_ready = 1;
}

static const double A44 = 0.5773502691896257645091;
static const double Z44[4] = {-0.5773502691896257645091, 0.5773502691896257645091, 0.5773502691896257645091, -0.5773502691896257645091};
static const double E44[4] = {-0.5773502691896257645091, -0.5773502691896257645091, 0.5773502691896257645091, 0.5773502691896257645091};
static const double N9 = 0.7745966692414833770359;
static const double Z34[4] = {-0.2, 0.4, -0.2, 0.0}, E34[4] = {-0.3464101615137754587055, 0.0, 0.3464101615137754587055, 0.0};
static const double W34[4] = {0.5208333333333333333333, 0.5208333333333333333333, 0.5208333333333333333333, -0.5625};

typedef struct { double cr[3][4], cw[3][3]; int quad; } pelem;

static double Nbil(int n, double z, double e) {
  double ia = 1.0 / A44;
  switch (n) {
    case 0: return 0.25 * (1.0 - z * ia) * (1.0 - e * ia);
    case 1: return 0.25 * (1.0 + z * ia) * (1.0 - e * ia);
    case 2: return 0.25 * (1.0 + z * ia) * (1.0 + e * ia);
    default: return 0.25 * (1.0 - z * ia) * (1.0 + e * ia);
  }
}
static double Nlit(int n, double z, double e) {
  double ia = 0.5 / 0.2;
  switch (n) {
    case 0: return (1.0 - ia * (z + sqrt(3.0) * e)) / 3.0;
    case 1: return (1.0 + 2.0 * ia * z) / 3.0;
    default: return (1.0 - ia * (z - sqrt(3.0) * e)) / 3.0;
  }
}
static double Nsh(const pelem *E, int n, double z, double e) { return E->quad ? Nbil(n, z, e) : Nlit(n, z, e); }
static double dot(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static double nrm(const double *a) { return sqrt(dot(a, a)); }
static cd ceik(cd k, double a) { return (cimag(k) == 0.0) ? cos(creal(k) * a) + I * sin(creal(k) * a) : cexp(I * k * a); }

/* ---- regular integrals --------------------------------------------------
 * quadrature point list of a rule: (zeta, eta, weight) */
static int rule_points(const pelem *E, int type, double *z, double *e, double *w, double *scale) {
  int n = 0;
  if (E->quad) {
    *scale = P_IFP;
    if (type == 0) { for (int i = 0; i < 4; i++) { z[n] = Z44[i]; e[n] = E44[i]; w[n++] = 1.0; } }
    else if (type == 1) {
      const double zz[9] = {-N9, N9, N9, -N9, 0.0, N9, 0.0, -N9, 0.0}, ee[9] = {-N9, -N9, N9, N9, -N9, 0.0, N9, 0.0, 0.0};
      const double ww[9] = {0.3086419753086419753086, 0.3086419753086419753086, 0.3086419753086419753086, 0.3086419753086419753086,
                            0.4938271604938271604938, 0.4938271604938271604938, 0.4938271604938271604938, 0.4938271604938271604938,
                            0.7901234567901234567901};
      for (int i = 0; i < 9; i++) { z[n] = zz[i]; e[n] = ee[i]; w[n++] = ww[i]; }
    } else {
      int m = (type == 2) ? P_GLN : P_GHN;
      const double *x = (type == 2) ? xl : xh, *wq = (type == 2) ? wl : wh;
      for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) { z[n] = x[i]; e[n] = x[j]; w[n++] = wq[i] * wq[j]; }
    }
  } else {
    if (type == 0) { *scale = P_IEP; for (int i = 0; i < 4; i++) { z[n] = Z34[i]; e[n] = E34[i]; w[n++] = W34[i]; } }
    else if (type == 1) {
      *scale = P_IEP;
      const double q0 = 0.3480702390148154917985, q1 = 0.2052130961576726346557, q2 = 0.6028753385763033130539, q3 = 0.3554395089236065568357;
      const double zz[7] = {-q0, 2 * q0, -q0, q1, -2 * q1, q1, 0.0}, ee[7] = {-q2, 0.0, q2, q3, 0.0, -q3, 0.0};
      const double ww[7] = {0.1259391805448271525957, 0.1259391805448271525957, 0.1259391805448271525957, 0.1323941527885061807376,
                            0.1323941527885061807376, 0.1323941527885061807376, 0.225};
      for (int i = 0; i < 7; i++) { z[n] = zz[i]; e[n] = ee[i]; w[n++] = ww[i]; }
    } else {
      *scale = 0.0625 * P_SQ3 * P_ISPSQ3;
      int m = (type == 2) ? P_GLN : P_GHN;
      const double *x = (type == 2) ? xl : xh, *wq = (type == 2) ? wl : wh;
      for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) {
        double a = x[i], b = x[j], ww = wq[i] * wq[j] * (1.0 + 0.25 * a + 0.25 * b);
        z[n] = 0.125 * (3.0 + 2.0 * a + 2.0 * b + a * b); e[n] = 0.125 * P_SQ3 * (-a + b); w[n++] = ww;
        z[n] = 0.0625 * (-3.0 + a - 5.0 * b - a * b); e[n] = 0.0625 * P_SQ3 * (3.0 + 3.0 * a + b + a * b); w[n++] = ww;
        z[n] = 0.0625 * (-3.0 - 5.0 * a + b - a * b); e[n] = 0.0625 * P_SQ3 * (-3.0 - a - 3.0 * b - a * b); w[n++] = ww;
      }
    }
  }
  return n;
}

/* CC[0..3] G, CC[4..7] H, CC[8] F; dC[d][..] along vt[d] */
void port_reg(const pelem *E, int type, const double *rt, int ndir, const double (*vt)[3], cd k, int neg, cd *CC, cd (*dC)[9]) {
  tables();
  static __thread double z[3 * P_GHN * P_GHN], e[3 * P_GHN * P_GHN], w[3 * P_GHN * P_GHN];
  double S;
  int np = rule_points(E, type, z, e, w, &S);
  for (int l = 0; l < 9; l++) { CC[l] = 0.0; for (int d = 0; d < ndir; d++) dC[d][l] = 0.0; }
  int nsf = E->quad ? 4 : 3;
  for (int ep = 0; ep < nsf; ep++) {
    for (int p = 0; p < np; p++) {
      double r[3], W[3], R[3];
      for (int i = 0; i < 3; i++) {
        r[i] = E->cr[i][0] + E->cr[i][1] * z[p] + E->cr[i][2] * e[p] + E->cr[i][3] * z[p] * e[p];
        W[i] = E->cw[i][0] + E->cw[i][1] * z[p] + E->cw[i][2] * e[p];
        R[i] = r[i] - rt[i];
      }
      double aR = nrm(R), iR = 1.0 / aR, aW = nrm(W);
      cd ca = I * k * aR, cb = ca - 1.0, ce = ceik(k, aR);
      double rdW = dot(R, W) * iR, tD = rdW * iR * iR;
      double Np = Nsh(E, ep, z[p], e[p]);
      CC[ep] += w[p] * ce * iR * aW * Np;
      CC[ep + 4] += w[p] * cb * ce * tD * Np;
      if (ep == 0) CC[8] += w[p] * tD;
      for (int d = 0; d < ndir; d++) {
        double rdv = dot(R, vt[d]) * iR, Wdv = dot(W, vt[d]);
        dC[d][ep] += w[p] * cb * ce * iR * iR * rdv * aW * Np;
        dC[d][ep + 4] += w[p] * ce * iR * iR * iR * ((k * k * aR * aR + 3.0 * cb) * rdv * rdW - cb * Wdv) * Np;
        if (ep == 0) dC[d][8] += w[p] * iR * iR * iR * (3.0 * rdv * rdW - Wdv);
      }
    }
  }
  double sh = neg ? -S : S;
  for (int l = 0; l < 4; l++) { CC[l] *= S; CC[l + 4] *= sh; }
  CC[8] *= sh;
  for (int d = 0; d < ndir; d++) {
    for (int l = 0; l < 4; l++) { dC[d][l] *= -S; dC[d][l + 4] *= sh; }
    dC[d][8] *= sh;
  }
}

/* ---- singular integrals (observation point on its own element) ---------- */
typedef struct { const pelem *E; double zt, et; cd k; double vt[3]; double cth, sth; } sctx;

static void Kvec(const sctx *c, double r, double *K, double *W, double *z, double *e) {
  const pelem *E = c->E;
  *z = r * c->cth + c->zt;
  *e = r * c->sth + c->et;
  for (int i = 0; i < 3; i++) {
    K[i] = E->cr[i][1] * c->cth + E->cr[i][2] * c->sth + E->cr[i][3] * (r * c->cth * c->sth + c->zt * c->sth + c->et * c->cth);
    W[i] = E->cw[i][0] + E->cw[i][1] * (*z) + E->cw[i][2] * (*e);
  }
}
static void Kminus(const sctx *c, double r, double *K, double *W, double *z, double *e) {
  const pelem *E = c->E;
  *z = -r * c->cth + c->zt;
  *e = -r * c->sth + c->et;
  for (int i = 0; i < 3; i++) {
    K[i] = E->cr[i][1] * c->cth + E->cr[i][2] * c->sth + E->cr[i][3] * (-r * c->cth * c->sth + c->zt * c->sth + c->et * c->cth);
    W[i] = E->cw[i][0] + E->cw[i][1] * (*z) + E->cw[i][2] * (*e);
  }
}

/* which integrand: 0 G, 1 H, 2 F (coef part, set A); derivatives (sets B-D)
 * selected by kind codes below; nid shape function; dir 0: zeta (outer sth,
 * inner cth), 1: eta (outer cth, inner sth) */
static cd bil_A_r(const sctx *c, int what, int nid, double r) {
  double K[3], W[3], z, e;
  Kvec(c, r, K, W, &z, &e);
  double aK = nrm(K), aW = nrm(W);
  cd kr = c->k * aK * r, ce = ceik(c->k, aK * r);
  if (what == 0) return ce / aK * aW * Nbil(nid, z, e);
  if (what == 1) return (I * kr - 1.0) * ce / (aK * aK * aK) * c->cth * c->sth * Nbil(nid, z, e);
  return 1.0 / (aK * aK * aK) * c->cth * c->sth;
}
static cd bil_B_r(const sctx *c, int what, int nid, int dir, double r) {
  double K[3], W[3], z, e;
  Kvec(c, r, K, W, &z, &e);
  double aK = nrm(K), aW = nrm(W);
  cd kr = c->k * r * aK, cb = I * kr - 1.0, ce = ceik(c->k, aK * r);
  double inner = dir == 0 ? c->cth : c->sth;
  if (what == 0) return cb * ce / (aK * aK) / r * (dot(K, c->vt) / aK) * Nbil(nid, z, e) * aW;
  double KdT = dot(K, c->vt), aK5 = aK * aK * aK * aK * aK;
  if (what == 1) return ce / (r * aK5) * ((kr * kr + 3.0 * cb) * KdT * inner - cb * aK * aK) * Nbil(nid, z, e);
  return 1.0 / (r * aK5) * (3.0 * KdT * inner - aK * aK);
}
static cd bil_C_r(const sctx *c, int what, int nid, int dir, double r) {
  double K[3], W[3], z, e;
  Kvec(c, r, K, W, &z, &e);
  double aK = nrm(K), aW = nrm(W);
  cd kr = c->k * aK * r;
  double inner = dir == 0 ? c->cth : c->sth;
  if (what == 0) {
    cd cc = ccos(kr), cs = csin(kr);
    if (cimag(c->k) == 0.0) { cc = cos(creal(kr)); cs = sin(creal(kr)); }
    return ((I * kr - 1.0) * cs + kr * cc) / (aK * aK) / r * (dot(K, c->vt) / aK) * aW * Nbil(nid, z, e);
  }
  double KdT = dot(K, c->vt);
  if (what == 1) {  /* De0 */
    cd ce = ceik(c->k, aK * r), cb = I * c->k;
    return ce / (aK * aK * aK * aK) * ((c->k * kr + 3.0 * cb) * KdT * inner - cb * aK * aK) * Nbil(nid, z, e);
  }
  cd cs = (cimag(c->k) == 0.0) ? sin(creal(kr)) : csin(kr); /* De1 */
  return cs / (aK * aK * aK * aK * aK * r) * (3.0 * KdT * inner - aK * aK) * Nbil(nid, z, e);
}
static cd bil_D_r(const sctx *c, int what, int nid, int dir, double r) {
  double Kp[3], Wp[3], zp, ep, Km[3], Wm[3], zm, em;
  Kvec(c, r, Kp, Wp, &zp, &ep);
  Kminus(c, r, Km, Wm, &zm, &em);
  double aKp = nrm(Kp), aKm = nrm(Km), aWp = nrm(Wp), aWm = nrm(Wm);
  cd kRp = c->k * aKp * r, kRm = -c->k * aKm * r;
  cd ccp = (cimag(c->k) == 0.0) ? cos(creal(kRp)) : ccos(kRp), ccm = (cimag(c->k) == 0.0) ? cos(creal(kRm)) : ccos(kRm);
  double inner = dir == 0 ? c->cth : c->sth;
  if (what == 0)
    return 1.0 / r * (ccp / (aKp * aKp) * (dot(Kp, c->vt) / aKp) * Nbil(nid, zp, ep) * aWp -
                      ccm / (aKm * aKm) * (dot(Km, c->vt) / aKm) * Nbil(nid, zm, em) * aWm);
  double p5 = pow(aKp, 5), m5 = pow(aKm, 5);
  double fp = (3.0 * dot(Kp, c->vt) * inner - aKp * aKp) / p5, fm = (3.0 * dot(Km, c->vt) * inner - aKm * aKm) / m5;
  if (what == 1) return 1.0 / r * (ccp * fp * Nbil(nid, zp, ep) - ccm * fm * Nbil(nid, zm, em));
  return 1.0 / r * (fp - fm);
}

static void node_r_th(int quad, double zt, double et, double *r, double *th) {
  if (quad) {
    double ztp = 1.0 - zt, ztm = -1.0 - zt, etp = 1.0 - et, etm = -1.0 - et;
    r[0] = sqrt(ztm * ztm + etm * etm); r[1] = sqrt(ztp * ztp + etm * etm);
    r[2] = sqrt(ztp * ztp + etp * etp); r[3] = sqrt(ztm * ztm + etp * etp); r[4] = r[0];
    th[0] = atan2(etm, ztm); th[1] = atan2(etm, ztp); th[2] = atan2(etp, ztp); th[3] = atan2(etp, ztm);
    th[4] = th[0] + 2.0 * P_PI;
  } else {
    double ztp = 1.0 - zt, ztm = -0.5 - zt, etp = 0.5 * P_SQ3 - et, etm = -0.5 * P_SQ3 - et;
    r[0] = sqrt(ztm * ztm + etm * etm); r[1] = sqrt(ztp * ztp + et * et); r[2] = sqrt(ztm * ztm + etp * etp); r[3] = r[0];
    th[0] = atan2(etm, ztm); th[1] = atan2(-et, ztp); th[2] = atan2(etp, ztm); th[3] = th[0] + 2.0 * P_PI;
  }
}
static double rmax(double r0, double r1, double t0, double t1, double th) {
  return r0 * r1 * sin(t1 - t0) / (r0 * sin(th - t0) - r1 * sin(th - t1));
}

/* bilinear element, observation node (zt, et): CC (G,H,F) and the two
 * tangential derivatives (reference bil_dcoef_bd_vt2_PV) */
void port_sing_bil(const pelem *E, double zt, double et, cd k, int neg, cd *CC, cd *dCz, cd *dCe) {
  tables();
  sctx c;
  c.E = E; c.zt = zt; c.et = et; c.k = k;
  double r[5], th[5];
  node_r_th(1, zt, et, r, th);
  double bdc = E->cr[0][1] * E->cw[0][2] + E->cr[1][1] * E->cw[1][2] + E->cr[2][1] * E->cw[2][2];
  double ab = sqrt(E->cr[0][1] * E->cr[0][1] + E->cr[1][1] * E->cr[1][1] + E->cr[2][1] * E->cr[2][1]);
  double aC = sqrt(E->cw[0][2] * E->cw[0][2] + E->cw[1][2] * E->cw[1][2] + E->cw[2][2] * E->cw[2][2]);
  int planar = fabs(bdc / (ab * aC)) < 1.0e-15;
  for (int l = 0; l < 9; l++) { CC[l] = 0.0; dCz[l] = 0.0; dCe[l] = 0.0; }
  /* coefficients: per shape function, per edge, two theta halves x GHN, r on [0, rm] with GLN */
  for (int what = 0; what < 3; what++) {
    if (what > 0 && planar) break;
    for (int i = 0; i < (what == 2 ? 1 : 4); i++) {
      cd acc = 0.0;
      for (int j = 0; j < 4; j++) {
        cd tC = 0.0;
        for (int m = 0; m < P_GHN; m++)
          for (int h = 0; h < 2; h++) {
            double t = (h == 0) ? 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (th[j + 1] + 3.0 * th[j])
                                : 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (3.0 * th[j + 1] + th[j]);
            double rm = rmax(r[j], r[j + 1], th[j], th[j + 1], t);
            c.cth = cos(t); c.sth = sin(t);
            cd s = 0.0;
            for (int q = 0; q < P_GLN; q++) s += bil_A_r(&c, what, i, 0.5 * rm * (xl[q] + 1.0)) * wl[q];
            tC += s * 0.5 * rm * wh[m];
          }
        acc += tC * 0.25 * (th[j + 1] - th[j]);
      }
      if (what == 0) CC[i] = acc * P_IFP;
      else if (what == 1) CC[i + 4] = acc * P_IFP * bdc;
      else CC[8] = acc * P_IFP * bdc;
    }
  }
  /* derivatives */
  for (int dir = 0; dir < 2; dir++) {
    cd *dC = dir == 0 ? dCz : dCe;
    for (int l = 0; l < 3; l++) c.vt[l] = dir == 0 ? E->cr[l][1] + E->cr[l][3] * et : E->cr[l][2] + E->cr[l][3] * zt;
    double iaT = 1.0 / nrm(c.vt);
    for (int what = 0; what < 3; what++) {
      if (what > 0 && planar) break;
      for (int i = 0; i < (what == 2 ? 1 : 4); i++) {
        cd acc = 0.0;
        /* D-bar_eps: r on [DEPS, rm] with GHN */
        for (int j = 0; j < 4; j++) {
          cd tC = 0.0;
          for (int m = 0; m < P_GHN; m++)
            for (int h = 0; h < 2; h++) {
              double t = (h == 0) ? 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (th[j + 1] + 3.0 * th[j])
                                  : 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (3.0 * th[j + 1] + th[j]);
              double rm = rmax(r[j], r[j + 1], th[j], th[j + 1], t);
              c.cth = cos(t); c.sth = sin(t);
              cd s = 0.0;
              for (int q = 0; q < P_GHN; q++) s += bil_B_r(&c, what, i, dir, 0.5 * (rm - P_DEPS) * xh[q] + 0.5 * (rm + P_DEPS)) * wh[q];
              s *= 0.5 * (rm - P_DEPS);
              if (what > 0) s *= (dir == 0 ? c.sth : c.cth);
              tC += s * wh[m];
            }
          acc += tC * 0.25 * (th[j + 1] - th[j]);
        }
        /* D_eps disc (G and H only) */
        if (what < 2) {
          const double off[4] = {-0.75 * P_PI, -0.25 * P_PI, 0.25 * P_PI, 0.75 * P_PI};
          cd tC = 0.0;
          for (int m = 0; m < P_GHN; m++)
            for (int qq = 0; qq < 4; qq++) {
              double t = 0.25 * P_PI * xh[m] + off[qq];
              c.cth = cos(t); c.sth = sin(t);
              cd s = 0.0;
              if (what == 0) {
                for (int q = 0; q < P_GLN; q++) s += bil_C_r(&c, 0, i, dir, 0.5 * P_DEPS * (xl[q] + 1.0)) * wl[q];
                s *= 0.5 * P_DEPS;
              } else {
                cd s0 = 0.0, s1 = 0.0;
                for (int q = 0; q < P_GLN; q++) {
                  double rr = 0.5 * P_DEPS * (xl[q] + 1.0);
                  s0 += bil_C_r(&c, 1, i, dir, rr) * wl[q];
                  s1 += bil_C_r(&c, 2, i, dir, rr) * wl[q];
                }
                s = (s0 - I * s1) * 0.5 * P_DEPS * (dir == 0 ? c.sth : c.cth);
              }
              tC += s * wh[m];
            }
          tC *= 0.25 * P_PI;
          acc += (what == 0) ? I * tC : tC;
        }
        /* principal value pairing */
        {
          cd tC = 0.0;
          for (int m = 0; m < P_GHN; m++)
            for (int hh = 0; hh < 2; hh++) {
              double t = 0.25 * P_PI * xh[m] + (hh == 0 ? 0.25 : 0.75) * P_PI;
              c.cth = cos(t); c.sth = sin(t);
              cd s = 0.0;
              for (int q = 0; q < P_GLN; q++) s += bil_D_r(&c, what, i, dir, 0.5 * P_DEPS * (xl[q] + 1.0)) * wl[q];
              s *= 0.5 * P_DEPS;
              if (what > 0) s *= (dir == 0 ? c.sth : c.cth);
              tC += s * wh[m];
            }
          tC *= 0.25 * P_PI;
          acc += (what == 2) ? tC : -tC;
        }
        if (what == 0) dC[i] = acc * (-P_IFP * iaT);
        else if (what == 1) dC[i + 4] = acc * bdc * P_IFP * iaT;
        else dC[8] = acc * bdc * P_IFP * iaT;
      }
    }
  }
  if (neg) {
    for (int l = 4; l < 9; l++) { CC[l] = -CC[l]; dCz[l] = -dCz[l]; dCe[l] = -dCe[l]; }
  }
}

static double dN_ray(int n, double cth, double sth) {
  double ia = 0.5 / 0.2;
  if (n == 0) return -2.0 / 3.0 * ia * (cth + P_SQ3 * sth);
  if (n == 1) return 4.0 / 3.0 * ia * cth;
  return -2.0 / 3.0 * ia * (cth - P_SQ3 * sth);
}

/* linear triangle, observation node (zt, et): G and the tangential
 * derivatives of G (H, F vanish on the own planar element) */
void port_sing_lit(const pelem *E, double zt, double et, cd k, int neg, cd *CC, cd *dCz, cd *dCe) {
  tables();
  double r[4], th[4];
  node_r_th(0, zt, et, r, th);
  double aW = sqrt(E->cw[0][0] * E->cw[0][0] + E->cw[1][0] * E->cw[1][0] + E->cw[2][0] * E->cw[2][0]);
  for (int l = 0; l < 9; l++) { CC[l] = 0.0; dCz[l] = 0.0; dCe[l] = 0.0; }
  for (int i = 0; i < 3; i++) {
    cd acc = 0.0;
    for (int j = 0; j < 3; j++) {
      cd tC = 0.0;
      for (int m = 0; m < P_GHN; m++)
        for (int h = 0; h < 2; h++) {
          double t = (h == 0) ? 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (th[j + 1] + 3.0 * th[j])
                              : 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (3.0 * th[j + 1] + th[j]);
          double rm = rmax(r[j], r[j + 1], th[j], th[j + 1], t), cth = cos(t), sth = sin(t), K[3];
          for (int l = 0; l < 3; l++) K[l] = E->cr[l][1] * cth + E->cr[l][2] * sth;
          double aK = nrm(K);
          cd s = 0.0;
          for (int q = 0; q < P_GLN; q++) {
            double rr = 0.5 * rm * (xl[q] + 1.0);
            s += ceik(k, aK * rr) / aK * Nlit(i, rr * cth + zt, rr * sth + et) * wl[q];
          }
          tC += s * 0.5 * rm * wh[m];
        }
      acc += tC * 0.25 * (th[j + 1] - th[j]);
    }
    CC[i] = acc * P_ISPSQ3 * aW;
  }
  for (int dir = 0; dir < 2; dir++) {
    cd *dC = dir == 0 ? dCz : dCe;
    double vt[3];
    for (int l = 0; l < 3; l++) vt[l] = dir == 0 ? E->cr[l][1] : E->cr[l][2];
    double iaT = 1.0 / nrm(vt);
    for (int i = 0; i < 3; i++) {
      cd acc = 0.0;
      for (int j = 0; j < 3; j++) {
        cd tC = 0.0;
        for (int m = 0; m < P_GHN; m++)
          for (int h = 0; h < 2; h++) {
            double t = (h == 0) ? 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (th[j + 1] + 3.0 * th[j])
                                : 0.25 * (th[j + 1] - th[j]) * xh[m] + 0.25 * (3.0 * th[j + 1] + th[j]);
            double rm = rmax(r[j], r[j + 1], th[j], th[j + 1], t), cth = cos(t), sth = sin(t), K[3];
            for (int l = 0; l < 3; l++) K[l] = E->cr[l][1] * cth + E->cr[l][2] * sth;
            double aK = nrm(K), Kdv = dot(K, vt) / aK;
            cd s = 0.0;
            for (int q = 0; q < P_GHN; q++) {
              double rr = 0.5 * (rm - P_DEPS) * xh[q] + 0.5 * (rm + P_DEPS);
              cd kr = k * aK * rr;
              s += (I * kr - 1.0) * ceik(k, aK * rr) / rr / (aK * aK) * Kdv * Nlit(i, rr * cth + zt, rr * sth + et) * wh[q];
            }
            tC += s * 0.5 * (rm - P_DEPS) * wh[m];
          }
        acc += tC * 0.25 * (th[j + 1] - th[j]);
      }
      const double off[4] = {-0.75 * P_PI, -0.25 * P_PI, 0.25 * P_PI, 0.75 * P_PI};
      cd tC = 0.0;
      for (int m = 0; m < P_GHN; m++)
        for (int qq = 0; qq < 4; qq++) {
          double t = 0.25 * P_PI * xh[m] + off[qq], cth = cos(t), sth = sin(t), K[3];
          for (int l = 0; l < 3; l++) K[l] = E->cr[l][1] * cth + E->cr[l][2] * sth;
          double aK = nrm(K), Kdv = dot(K, vt) / aK;
          cd keK = k * P_DEPS * aK;
          cd cc = (cimag(k) == 0.0) ? cos(creal(keK)) : ccos(keK), cs = (cimag(k) == 0.0) ? sin(creal(keK)) : csin(keK);
          tC += dN_ray(i, cth, sth) / (aK * aK * aK) * Kdv * ((keK + I) * cs + (2.0 - I * keK) * cc - 2.0) * wh[m];
        }
      acc += I * tC * 0.25 * P_PI / k;
      tC = 0.0;
      for (int m = 0; m < P_GHN; m++)
        for (int hh = 0; hh < 2; hh++) {
          double t = 0.25 * P_PI * xh[m] + (hh == 0 ? 0.25 : 0.75) * P_PI, cth = cos(t), sth = sin(t), K[3];
          for (int l = 0; l < 3; l++) K[l] = E->cr[l][1] * cth + E->cr[l][2] * sth;
          double aK = nrm(K), Kdv = dot(K, vt) / aK;
          cd cs = (cimag(k) == 0.0) ? sin(creal(k) * aK * P_DEPS) : csin(k * aK * P_DEPS);
          tC += dN_ray(i, cth, sth) * cs / (aK * aK * aK) * Kdv * wh[m];
        }
      acc -= tC * 0.25 * P_PI / k;
      dC[i] = acc * (-P_ISPSQ3 * aW * iaT);
    }
  }
  if (neg) {
    for (int l = 4; l < 9; l++) { CC[l] = -CC[l]; dCz[l] = -dCz[l]; dCe[l] = -dCe[l]; }
  }
}

/* ---- mesh view ------------------------------------------------------------ */
typedef struct {
  int Ne, MN;
  const double *cr, *cw, *ren, *corner;
  const int *etype, *sd;
  const int *sid, *sb_Ne, *sb_off;
  const double *kn;
} pmesh;

static void pload(const pmesh *m, int s, pelem *E) {
  for (int i = 0; i < 12; i++) (&E->cr[0][0])[i] = m->cr[(size_t)s * 12 + i];
  for (int i = 0; i < 9; i++) (&E->cw[0][0])[i] = m->cw[(size_t)s * 9 + i];
  E->quad = m->etype[s];
  if (!E->quad)
    for (int d = 0; d < 3; d++) { E->cr[d][3] = 0.0; E->cw[d][1] = 0.0; E->cw[d][2] = 0.0; }
}

/* one (node, element) pair of the assembly, reference dispatch rules */
static void port_pair(const pmesh *m, int td, int tn, int sd, cd k, int type, cd *CC, cd *dCz, cd *dCe) {
  pelem T, S;
  pload(m, abs(td), &T);
  pload(m, abs(sd), &S);
  if (td == sd) {
    double zt = T.quad ? Z44[tn] : Z34[tn], et = T.quad ? E44[tn] : E34[tn];
    if (S.quad) port_sing_bil(&S, zt, et, k, sd < 0, CC, dCz, dCe);
    else port_sing_lit(&S, zt, et, k, sd < 0, CC, dCz, dCe);
    return;
  }
  double vt[2][3], rt[3];
  for (int d = 0; d < 3; d++) {
    rt[d] = m->ren[(size_t)abs(td) * 12 + tn * 3 + d];
    if (T.quad) { vt[0][d] = T.cr[d][1] + T.cr[d][3] * E44[tn]; vt[1][d] = T.cr[d][2] + T.cr[d][3] * Z44[tn]; }
    else { vt[0][d] = T.cr[d][1]; vt[1][d] = T.cr[d][2]; }
  }
  for (int i = 0; i < 2; i++) { double a = nrm(vt[i]); for (int d = 0; d < 3; d++) vt[i][d] /= a; }
  cd dC[2][9];
  port_reg(&S, type, rt, 2, (const double(*)[3])vt, k, sd < 0, CC, dC);
  if (type < 3 && (fabs(creal(dC[0][8])) > 0.5 || fabs(creal(dC[1][8])) > 0.5)) port_reg(&S, 3, rt, 2, (const double(*)[3])vt, k, sd < 0, CC, dC);
  memcpy(dCz, dC[0], sizeof(cd) * 9);
  memcpy(dCe, dC[1], sizeof(cd) * 9);
}

/* rows rows[0..nr-1] (row = (t-1)*4+tn) of G, H (each N), dG, dH (2N), dF (3)
 * of domain did (reference create_cmatrix_domain, solve_bieq2.c:124-166) */
void port_rows(const pmesh *m, int did, int type, int nr, const int *rows, cd *G, cd *H, cd *dG, cd *dH, double *dF) {
  const int *sid = m->sid + m->sb_off[did];
  int Ne = m->sb_Ne[did];
  size_t N = 4 * (size_t)Ne;
  cd k = m->kn[2 * did] + I * m->kn[2 * did + 1];
#pragma omp parallel for schedule(dynamic)
  for (int q = 0; q < nr; q++) {
    int row = rows[q], t = row / 4 + 1, tn = row % 4, td = sid[t];
    cd *g = G + (size_t)q * N, *h = H + (size_t)q * N, *dg = dG + (size_t)q * 2 * N, *dh = dH + (size_t)q * 2 * N;
    for (size_t c = 0; c < N; c++) { g[c] = 0.0; h[c] = 0.0; dg[c] = 0.0; dg[N + c] = 0.0; dh[c] = 0.0; dh[N + c] = 0.0; }
    dF[3 * q] = dF[3 * q + 1] = dF[3 * q + 2] = 0.0;
    if (!m->etype[abs(td)] && tn == 3) continue;
    double F = 0.0, Fz = 0.0, Fe = 0.0;
    for (int s = 1; s <= Ne; s++) {
      cd CC[9], dCz[9], dCe[9];
      port_pair(m, td, tn, sid[s], k, type, CC, dCz, dCe);
      for (int i = 0; i < 4; i++) {
        g[(s - 1) * 4 + i] = CC[i];
        h[(s - 1) * 4 + i] = CC[i + 4];
        dg[(s - 1) * 4 + i] = dCz[i];
        dg[N + (s - 1) * 4 + i] = dCe[i];
        dh[(s - 1) * 4 + i] = dCz[i + 4];
        dh[N + (s - 1) * 4 + i] = dCe[i + 4];
      }
      F += creal(CC[8]);
      Fz += creal(dCz[8]);
      Fe += creal(dCe[8]);
    }
    double diag = (did == 0) ? 1.0 + F : F;
    h[(t - 1) * 4 + tn] += diag;
    dF[3 * q] = diag;
    dF[3 * q + 1] = Fz;
    dF[3 * q + 2] = Fe;
  }
}

/* ---- domain id ------------------------------------------------------------ */
static int vuni(double *r) {
  double a = nrm(r);
  if (a == 0.0) return -1;
  r[0] /= a; r[1] /= a; r[2] /= a;
  return 0;
}
static void cross(const double *a, const double *b, double *r) {
  r[0] = a[1] * b[2] - a[2] * b[1]; r[1] = a[2] * b[0] - a[0] * b[2]; r[2] = a[0] * b[1] - a[1] * b[0];
}
static double tri_angle(const double *r0, const double *r1, const double *r2, int *flg) {
  double n01[3], n12[3], n20[3], nt[3];
  cross(r0, r1, n01); cross(r1, r2, n12); cross(r2, r0, n20);
  cross(n01, n20, nt); double a0 = atan2(nrm(nt), -dot(n01, n20));
  cross(n12, n01, nt); double a1 = atan2(nrm(nt), -dot(n12, n01));
  cross(n20, n12, nt); double a2 = atan2(nrm(nt), -dot(n20, n12));
  double D = dot(r0, n12);
  if (D > 0.0) return a0 + a1 + a2 - P_PI;
  if (D < 0.0) return -(a0 + a1 + a2 - P_PI);
  *flg = -1;
  return 0.0;
}
int port_domain_id(const pmesh *m, const double *rt) {
  double Og[32] = {0};
  for (int d = 0; d <= m->MN; d++) {
    const int *sid = m->sid + m->sb_off[d];
    for (int i = 1; i <= m->sb_Ne[d]; i++) {
      int s = sid[i];
      if (s <= 0) continue;
      double r[4][3];
      for (int j = 0; j < 4; j++) for (int l = 0; l < 3; l++) r[j][l] = m->corner[(size_t)s * 12 + j * 3 + l] - rt[l];
      int nv = m->etype[s] ? 4 : 3, st = 0, flg = 0;
      for (int j = 0; j < nv; j++) st += vuni(r[j]);
      if (st < 0) return d;
      double om = tri_angle(r[0], r[1], r[2], &flg);
      if (flg < 0) return d;
      if (nv == 4) { om += tri_angle(r[0], r[2], r[3], &flg); if (flg < 0) return d; }
      Og[d] += om;
      Og[m->sd[s]] -= om;
    }
    if (d == 0 && fabs(Og[0]) < 2.0 * P_PI) return 0;
    if (Og[d] > 2.0 * P_PI) return d;
  }
  return -1;
}

/* ---- field sums ------------------------------------------------------------
 * mode 0: U[4] (mEMP_s); 1: E[3],H[3] (EH_s); 2: E,H from potential
 * derivatives (EH_mEMP_s, returns -did at the cutoff); 3: U[4], dU[4] along v
 * (mEMP2_s).  Boundary values bv_*[d] in the reference layout [s][node][comp]. */
int port_field(const pmesh *m, int mode, int type, const double *rt, const double *v, double lambda0, const cd *const *bU,
               const cd *const *bdU, const cd *const *bE, const cd *const *bdE, const cd *const *bH, const cd *const *bdH,
               cd *out) {
  int did = port_domain_id(m, rt);
  if (did < 0) return did;
  const int *sid = m->sid + m->sb_off[did];
  cd k = m->kn[2 * did] + I * m->kn[2 * did + 1];
  double F = 0.0, dF[3] = {0, 0, 0};
  cd acc[40];
  for (int i = 0; i < 40; i++) acc[i] = 0.0;
  const double ax[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int s = 1; s <= m->sb_Ne[did]; s++) {
    pelem S;
    int sd = sid[s];
    pload(m, abs(sd), &S);
    cd CC[9], dC[3][9];
    if (mode <= 1) {
      port_reg(&S, type, rt, 0, NULL, k, sd < 0, CC, dC);
    } else if (mode == 3) {
      double vt[1][3] = {{v[0], v[1], v[2]}};
      port_reg(&S, type, rt, 1, (const double(*)[3])vt, k, sd < 0, CC, dC);
      if (type < 3 && fabs(creal(dC[0][8])) > 0.5) port_reg(&S, 3, rt, 1, (const double(*)[3])vt, k, sd < 0, CC, dC);
    } else {
      for (int d = 0; d < 3; d++) {  /* one call per direction; CC of the last one kept */
        cd c1[9], d1[1][9];
        port_reg(&S, type, rt, 1, (const double(*)[3])ax[d], k, sd < 0, c1, d1);
        if (type < 3 && fabs(creal(d1[0][8])) > 0.5) port_reg(&S, 3, rt, 1, (const double(*)[3])ax[d], k, sd < 0, c1, d1);
        memcpy(dC[d], d1[0], sizeof(cd) * 9);
        memcpy(CC, c1, sizeof(cd) * 9);
      }
    }
    F += creal(CC[8]);
    for (int n = 0; n < 4; n++) {
      if (mode == 1) {
        for (int l = 0; l < 3; l++) {
          size_t q = ((size_t)s * 4 + n) * 3 + l;
          acc[l] += CC[n] * bdE[did][q] - CC[n + 4] * bE[did][q];
          acc[3 + l] += CC[n] * bdH[did][q] - CC[n + 4] * bH[did][q];
        }
      } else {
        for (int l = 0; l < 4; l++) {
          size_t q = ((size_t)s * 4 + n) * 4 + l;
          acc[l] += CC[n] * bdU[did][q] - CC[n + 4] * bU[did][q];
          int nd = (mode == 3) ? 1 : (mode == 2 ? 3 : 0);
          for (int d = 0; d < nd; d++) acc[4 + 4 * d + l] += dC[d][n] * bdU[did][q] - dC[d][n + 4] * bU[did][q];
        }
      }
    }
    int nd = (mode == 3) ? 1 : (mode == 2 ? 3 : 0);
    for (int d = 0; d < nd; d++) dF[d] += creal(dC[d][8]);
  }
  double den = (did == 0) ? 1.0 + F : F;
  if (mode == 0) { for (int l = 0; l < 4; l++) out[l] = acc[l] / den; return did; }
  if (mode == 1) { for (int l = 0; l < 6; l++) out[l] = acc[l] / den; return did; }
  cd U[4];
  for (int l = 0; l < 4; l++) U[l] = acc[l] / den;
  if (mode == 3) {
    for (int l = 0; l < 4; l++) { out[l] = U[l]; out[4 + l] = (acc[4 + l] - U[l] * dF[0]) / den; }
    return did;
  }
  cd dU[3][4];
  for (int d = 0; d < 3; d++) for (int l = 0; l < 4; l++) dU[d][l] = (acc[4 + 4 * d + l] - U[l] * dF[d]) / den;
  if (fabs(dF[0]) > 100.0 || fabs(dF[1]) > 100.0 || fabs(dF[2]) > 100.0) {
    for (int i = 0; i < 6; i++) out[i] = 0.0;
    return -did;
  }
  cd ch = lambda0 / (2.0 * P_PI * I);
  for (int i = 0; i < 3; i++) out[i] = -dU[i][3] + U[i];
  out[3] = ch * (dU[1][2] - dU[2][1]);
  out[4] = ch * (dU[2][0] - dU[0][2]);
  out[5] = ch * (dU[0][1] - dU[1][0]);
  return did;
}

/* exported with plain pointers for ctypes */
typedef struct {
  int Ne, MN;
  const double *cr, *cw, *ren, *corner;
  const int *etype, *sd, *sid, *sb_Ne, *sb_off;
  const double *kn;
} port_mesh_args;

void port_rows_c(const port_mesh_args *a, int did, int type, int nr, const int *rows, double *G, double *H, double *dG,
                 double *dH, double *dF) {
  pmesh m = {a->Ne, a->MN, a->cr, a->cw, a->ren, a->corner, a->etype, a->sd, a->sid, a->sb_Ne, a->sb_off, a->kn};
  port_rows(&m, did, type, nr, rows, (cd *)G, (cd *)H, (cd *)dG, (cd *)dH, dF);
}

int port_domain_id_c(const port_mesh_args *a, int n, const double *rt, int *did) {
  pmesh m = {a->Ne, a->MN, a->cr, a->cw, a->ren, a->corner, a->etype, a->sd, a->sid, a->sb_Ne, a->sb_off, a->kn};
  for (int p = 0; p < n; p++) did[p] = port_domain_id(&m, rt + 3 * p);
  return 0;
}

/* bv: per domain d pointers U,dU,E,dE,H,dH (6 * (MN+1) entries) */
void port_field_c(const port_mesh_args *a, int mode, int type, int n, const double *rt, const double *v, double lambda0,
                  const double *const *bv, double *out, int *ret) {
  pmesh m = {a->Ne, a->MN, a->cr, a->cw, a->ren, a->corner, a->etype, a->sd, a->sid, a->sb_Ne, a->sb_off, a->kn};
  const cd *bU[32], *bdU[32], *bE[32], *bdE[32], *bH[32], *bdH[32];
  for (int d = 0; d <= a->MN; d++) {
    bU[d] = (const cd *)bv[6 * d]; bdU[d] = (const cd *)bv[6 * d + 1]; bE[d] = (const cd *)bv[6 * d + 2];
    bdE[d] = (const cd *)bv[6 * d + 3]; bH[d] = (const cd *)bv[6 * d + 4]; bdH[d] = (const cd *)bv[6 * d + 5];
  }
  int nout = (mode == 0) ? 4 : (mode == 3 ? 8 : 6);
#pragma omp parallel for schedule(dynamic)
  for (int p = 0; p < n; p++)
    ret[p] = port_field(&m, mode, type, rt + 3 * p, v ? v + 3 * p : NULL, lambda0, bU, bdU, bE, bdE, bH, bdH, (cd *)out + (size_t)nout * p);
}

/* ---- labels of the learned near-singular quadrature -------------------------
 * G (CC[0..3]) and H (CC[4..7]) of bilinear elements given by their corners
 * (corner[p][4][3], the mesh's corner order) at observation points rt[p], by
 * the rule `type` (3: the GHN 64 x 64 Gauss-Legendre rule that the reference's
 * fallback bil_dcoef_v2_GH, bil_dcoef_v2.c:235-326, integrates with).  The
 * element coefficients cr, cw are the reference's (setup2.c:666-745).
 * out[p][16]: re, im of G_0..G_3 then of H_0..H_3. */
void port_quad_labels_c(int n, const double *corner, const double *rt, const double *k, int type, double *out) {
  tables();
#pragma omp parallel for schedule(dynamic, 16)
  for (int p = 0; p < n; p++) {
    const double *c = corner + (size_t)p * 12;
    double rc[3][4];
    for (int j = 0; j < 4; j++)
      for (int d = 0; d < 3; d++) rc[d][j] = c[j * 3 + d];
    pelem E;
    E.quad = 1;
    for (int d = 0; d < 3; d++) {
      E.cr[d][0] = 0.25 * (rc[d][0] + rc[d][1] + rc[d][2] + rc[d][3]);
      E.cr[d][1] = 0.25 * (-rc[d][0] + rc[d][1] + rc[d][2] - rc[d][3]);
      E.cr[d][2] = 0.25 * (-rc[d][0] - rc[d][1] + rc[d][2] + rc[d][3]);
      E.cr[d][3] = 0.25 * (rc[d][0] - rc[d][1] + rc[d][2] - rc[d][3]);
      const int a = (d + 1) % 3, b = (d + 2) % 3;
      E.cw[d][0] = 0.125 * ((rc[a][0] - rc[a][2]) * (rc[b][1] - rc[b][3]) - (rc[a][1] - rc[a][3]) * (rc[b][0] - rc[b][2]));
      E.cw[d][1] = 0.125 * ((rc[a][2] - rc[a][3]) * (rc[b][0] - rc[b][1]) - (rc[a][0] - rc[a][1]) * (rc[b][2] - rc[b][3]));
      E.cw[d][2] = 0.125 * ((rc[a][1] - rc[a][2]) * (rc[b][0] - rc[b][3]) - (rc[a][0] - rc[a][3]) * (rc[b][1] - rc[b][2]));
    }
    cd CC[9], dC[1][9];
    port_reg(&E, type, rt + (size_t)p * 3, 0, NULL, k[2 * (size_t)p] + I * k[2 * (size_t)p + 1], 0, CC, dC);
    for (int i = 0; i < 8; i++) {
      out[(size_t)p * 16 + 2 * i] = creal(CC[i]);
      out[(size_t)p * 16 + 2 * i + 1] = cimag(CC[i]);
    }
  }
}
