// gb_common.cuh -- shared device definitions of the GB300 BEM hot path.
//
// Complex FP64 arithmetic, the quadrature tables held in constant memory and
// the element record the kernels read.  All quadrature runs in FP64: the
// coefficient matrices must agree with the reference's double-complex
// arithmetic to <= 1e-10 relative Frobenius error.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#ifndef GB_GLN
#define GB_GLN 12   // regular Gauss-Legendre order (reference d3b1_const.h GLN)
#define GB_GHN 64   // fallback / singular order (reference d3b1_const.h GHN)
#endif

#define GB_PI 3.14159265358979323846
#define GB_I_FP 7.957747154594766788444e-2   // 1/(4 pi)
#define GB_I_EP 3.978873577297383394222e-2   // 1/(8 pi)
#define GB_SQ3 1.732050807568877293528e+0
#define GB_I_SPSQ3 3.062938307898844719507e-2 // 1/(6 pi sqrt 3)
#define GB_P44_N 0.5773502691896257645091
#define GB_P34_N0 0.2
#define GB_DEPS 0.1
#define GB_CBD_SDF 0.5
#define GB_CBD_CDF 100.0

// ---------------------------------------------------------------- complex
struct cplx {
  double x, y;
};
__host__ __device__ __forceinline__ cplx cmk(double a, double b) { cplx r; r.x = a; r.y = b; return r; }
__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return cmk(-a.x, -a.y); }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__host__ __device__ __forceinline__ cplx operator*(cplx a, double s) { return cmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ cplx operator*(double s, cplx a) { return cmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ cplx& operator+=(cplx& a, cplx b) { a.x += b.x; a.y += b.y; return a; }
__host__ __device__ __forceinline__ cplx& operator-=(cplx& a, cplx b) { a.x -= b.x; a.y -= b.y; return a; }
__host__ __device__ __forceinline__ cplx cconjg(cplx a) { return cmk(a.x, -a.y); }
__host__ __device__ __forceinline__ cplx cdivc(cplx a, cplx b) {
  double d = b.x * b.x + b.y * b.y;
  return cmk((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__host__ __device__ __forceinline__ cplx cdivr(cplx a, double s) { return cmk(a.x / s, a.y / s); }
// i * a
__host__ __device__ __forceinline__ cplx cmuli(cplx a) { return cmk(-a.y, a.x); }
__host__ __device__ __forceinline__ double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }

// single-precision complex (the LU factors of the mixed-precision form)
struct cplxf {
  float x, y;
};
__host__ __device__ __forceinline__ cplxf cmkf(float a, float b) { cplxf r; r.x = a; r.y = b; return r; }
__host__ __device__ __forceinline__ cplxf operator+(cplxf a, cplxf b) { return cmkf(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cplxf operator*(cplxf a, float s) { return cmkf(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a, cplxf b) { return cmkf(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cplxf operator*(cplxf a, cplxf b) { return cmkf(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__host__ __device__ __forceinline__ cplxf& operator+=(cplxf& a, cplxf b) { a.x += b.x; a.y += b.y; return a; }
__host__ __device__ __forceinline__ cplxf& operator-=(cplxf& a, cplxf b) { a.x -= b.x; a.y -= b.y; return a; }
__host__ __device__ __forceinline__ cplxf cdivc(cplxf a, cplxf b) {
  float d = b.x * b.x + b.y * b.y;
  return cmkf((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__host__ __device__ __forceinline__ cplxf to_c64f(cplx a) { return cmkf((float)a.x, (float)a.y); }
template <class T> __host__ __device__ __forceinline__ T czero();
template <> __host__ __device__ __forceinline__ cplx czero<cplx>() { return cmk(0.0, 0.0); }
template <> __host__ __device__ __forceinline__ cplxf czero<cplxf>() { return cmkf(0.0f, 0.0f); }

// e^{i k a} for complex k and real a >= 0
__device__ __forceinline__ cplx cexpik(cplx k, double a) {
  double s, c;
  sincos(k.x * a, &s, &c);
  if (k.y == 0.0) return cmk(c, s);
  double e = exp(-k.y * a);
  return cmk(c * e, s * e);
}
// cos(z), sin(z) of a complex argument
__device__ __forceinline__ void ccossin(cplx z, cplx* cz, cplx* sz) {
  double s, c;
  sincos(z.x, &s, &c);
  if (z.y == 0.0) { *cz = cmk(c, 0.0); *sz = cmk(s, 0.0); return; }
  double ch = cosh(z.y), sh = sinh(z.y);
  *cz = cmk(c * ch, -s * sh);
  *sz = cmk(s * ch, c * sh);
}

// ---------------------------------------------------------------- tables
// Gauss-Legendre nodes/weights (computed on the host by the same Newton
// iteration the reference uses, gauleg.c:3-36) and the small point rules of
// the reference's init_elem_const (setup2.c:704-745).
#define GB_NTAB (GB_GLN * (GB_GLN + 1) / 2)  // GL rules of 1..GLN points, rule n at n (n - 1) / 2
struct GbTables {
  double xli[GB_GLN], wli[GB_GLN];
  double xhi[GB_GHN], whi[GB_GHN];
  double xn[GB_NTAB], wn[GB_NTAB];
  double zt_44[4], et_44[4], wt_44[4];
  double zt_49[9], et_49[9], wt_49[9];
  double zt_34[4], et_34[4], wt_34[4];
  double zt_37[7], et_37[7], wt_37[7];
};
static __constant__ GbTables c_tab;

// ---------------------------------------------------------------- elements
// One boundary element as the kernels see it: the bilinear/linear geometry
// coefficients cr (r = a + b zeta + c eta + d zeta eta) and cw (normal
// W = A + B zeta + C eta), in the reference's [xyz][coef] order.
struct Elem {
  double cr[3][4];
  double cw[3][3];
  int quad;  // 1: bilinear quadrangle (ELT4), 0: linear triangle (ELT3)
};

__device__ __forceinline__ void load_elem(Elem& e, const double* __restrict__ cr, const double* __restrict__ cw,
                                          const int* __restrict__ etype, int s) {
#pragma unroll
  for (int i = 0; i < 12; i++) (&e.cr[0][0])[i] = __ldg(cr + (size_t)s * 12 + i);
#pragma unroll
  for (int i = 0; i < 9; i++) (&e.cw[0][0])[i] = __ldg(cw + (size_t)s * 9 + i);
  e.quad = __ldg(etype + s);
  if (!e.quad) {  // the reference zeroes the unused coefficients (lit_copy_elem_const_rw)
#pragma unroll
    for (int d = 0; d < 3; d++) { e.cr[d][3] = 0.0; e.cw[d][1] = 0.0; e.cw[d][2] = 0.0; }
  }
}

// interpolation (shape) functions at the collocation nodes
__device__ __forceinline__ void shape_bil(double z, double e, double N[4]) {
  const double ia = 1.0 / GB_P44_N;
  double zm = 1.0 - z * ia, zp = 1.0 + z * ia, em = 1.0 - e * ia, ep = 1.0 + e * ia;
  N[0] = 0.25 * zm * em;
  N[1] = 0.25 * zp * em;
  N[2] = 0.25 * zp * ep;
  N[3] = 0.25 * zm * ep;
}
__device__ __forceinline__ void shape_lit(double z, double e, double N[4]) {
  const double ia = 0.5 / GB_P34_N0;
  const double s3 = 1.7320508075688772;  // sqrt(3)
  N[0] = 1.0 / 3.0 * (1.0 - ia * (z + s3 * e));
  N[1] = 1.0 / 3.0 * (1.0 + 2.0 * ia * z);
  N[2] = 1.0 / 3.0 * (1.0 - ia * (z - s3 * e));
  N[3] = 0.0;
}
__device__ __forceinline__ void shape_fn(const Elem& E, double z, double e, double N[4]) {
  if (E.quad) shape_bil(z, e, N); else shape_lit(z, e, N);
}

__device__ __forceinline__ double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ double norm3(const double a[3]) { return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

__device__ __forceinline__ void elem_rw(const Elem& E, double z, double e, double r[3], double w[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    r[d] = E.cr[d][0] + E.cr[d][1] * z + E.cr[d][2] * e + E.cr[d][3] * z * e;
    w[d] = E.cw[d][0] + E.cw[d][1] * z + E.cw[d][2] * e;
  }
}

// status codes written by kernels into a device word (host reads them)
enum { GB_DEV_OK = 0, GB_DEV_ERR_REGION = 1, GB_DEV_ERR_OVERLAP = 2, GB_DEV_ERR_QUEUE = 3 };
