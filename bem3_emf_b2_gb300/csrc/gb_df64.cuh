// gb_df64.cuh -- double-float arithmetic: a value is an unevaluated sum of two
// FP32 numbers hi + lo (|lo| <= ulp(hi) / 2), about 48 significant bits.
// The error-free transformations are the classical ones (Dekker 1971, Knuth
// TAOCP vol. 2 sec. 4.2.2; with a fused multiply-add the exact product error
// is fma(a, b, -a b)), as used in double-double libraries (Hida, Li and
// Bailey, "Library for double-double and quad-double arithmetic", 2000).
// GB300's FP32 pipes are 64 times wider than its FP64 pipe, so quadrature that
// needs FP64-level accuracy runs faster in double-float than in FP64.
//
// The compiler may fuse a multiply and a following add into one fused
// multiply-add, which is exact where the algorithms rely on the rounded
// product: inside the error-free transformations every sum and every product
// that feeds a sum goes through __fadd_rn / __fsub_rn / __fmul_rn, which are
// never fused, so the results do not depend on the surrounding code's shape.
#pragma once
#include <cuda_runtime.h>

struct df {
  float hi, lo;
};

__device__ __forceinline__ df dfmk(float h, float l) { df r; r.hi = h; r.lo = l; return r; }
__device__ __forceinline__ df df_from(double d) {
  const float h = (float)d;
  return dfmk(h, (float)(d - (double)h));
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

// s + e = a + b exactly
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dfmk(s, e);
}
// |a| >= |b|
__device__ __forceinline__ df quick_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dfmk(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return dfmk(p, fmaf(a, b, -p));
}

__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = quick_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return dfmk(-a.hi, -a.lo); }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo));
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
// c + a b with one rounding error of the double-float format: the product's
// error terms folded into the sum's (two_sum of the high parts, then one
// renormalisation); about half the instructions of df_add(c, df_mul(a, b))
__device__ __forceinline__ df df_fma(df c, df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, pe));
  const float s = __fadd_rn(c.hi, p);
  const float bb = __fsub_rn(s, c.hi);
  const float e = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  return quick_two_sum(s, __fadd_rn(e, __fadd_rn(c.lo, pe)));
}
// Accumulator step c + a b for sums that are only read through df_to: the
// high parts are added exactly (two_sum) and every error term goes to the
// low part, which is never renormalised (compensated summation).  The low
// part stays within a few ulps of the high part over the short sums of a
// quadrature rule, so hi + lo still holds the sum to the format's rounding
// and converts to double exactly; three instructions fewer than df_fma.
__device__ __forceinline__ df df_acc(df c, df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float pe = fmaf(a.hi, b.hi, -p);
  pe = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, pe));
  const float s = __fadd_rn(c.hi, p);
  const float bb = __fsub_rn(s, c.hi);
  const float e = __fadd_rn(__fsub_rn(c.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  return dfmk(s, __fadd_rn(c.lo, __fadd_rn(e, pe)));
}
__device__ __forceinline__ df df_sqr(df a) {
  df p = two_prod(a.hi, a.hi);
  p.lo = fmaf(2.0f * a.hi, a.lo, p.lo);
  return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ float rcp_approx(float x) {  // hardware reciprocal estimate (about 1 ulp)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
// 1 / b: the FP32 estimate q1 and one Newton correction with the residual
// 1 - b q1 formed exactly enough by fused multiply-adds (relative error
// about 2^-46; b normal, not zero)
__device__ __forceinline__ df df_rcp(df b) {
  const float q1 = rcp_approx(b.hi);
  float r = fmaf(-b.hi, q1, 1.0f);
  r = fmaf(-b.lo, q1, r);
  return quick_two_sum(q1, __fmul_rn(r, q1));
}
// a / b: a first quotient, its remainder, a correction
__device__ __forceinline__ df df_div(df a, df b) {
  const float ib = rcp_approx(b.hi);
  const float q1 = __fmul_rn(a.hi, ib);
  const df r = df_sub(a, df_mul_f(b, q1));
  return quick_two_sum(q1, __fmul_rn(r.hi, ib));
}
// sqrt(a), a > 0: the FP32 root corrected by one Newton step in double-float
__device__ __forceinline__ df df_sqrt(df a) {
  const float s = sqrtf(a.hi);
  const df e = df_sub(a, two_prod(s, s));
  return quick_two_sum(s, __fmul_rn(e.hi, 0.5f * rsqrt_approx(a.hi)));
}

// complex double-float
struct dfc {
  df re, im;
};
__device__ __forceinline__ dfc dfcmk(df r, df i) { dfc c; c.re = r; c.im = i; return c; }
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return dfcmk(df_add(a.re, b.re), df_add(a.im, b.im)); }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
  return dfcmk(df_fma(df_mul(a.re, b.re), df_neg(a.im), b.im), df_fma(df_mul(a.re, b.im), a.im, b.re));
}
__device__ __forceinline__ dfc dfc_scale(dfc a, df s) { return dfcmk(df_mul(a.re, s), df_mul(a.im, s)); }

// cos and sin of x in double-float, |x| < 1000: x = j pi/8 + t with
// |t| <= pi/16 (pi/8 carried to about 70 bits in three floats), Taylor
// polynomials of t to t^11 / t^10 (truncation below 1e-17 for |t| <= pi/16,
// under the double-float rounding of ~4e-15), then the
// rotation by j pi/8 with cos, sin (j pi/8) from a double-float table.
// Coefficients: 1/n! in double-float (hi, lo).
static __device__ const float2 g_df_sin_c[8] = {
    {1.0f, 0.0f}, {0.1666666716337204f, -4.967053879312289e-09f}, {0.008333333767950535f, -4.34617203337595e-10f},
    {0.00019841270113829523f, -2.725596874933456e-12f}, {2.7557318844628753e-06f, 3.793571224297229e-14f},
    {2.5052107943679403e-08f, 4.4176230446483665e-16f}, {1.6059044372074283e-10f, -5.352526511562726e-18f},
    {7.647163609812713e-13f, 1.2200710471178288e-20f}};  // 1/(2m+1)!
static __device__ const float2 g_df_cos_c[8] = {
    {1.0f, 0.0f}, {0.5f, 0.0f}, {0.0416666679084301f, -1.2417634698280722e-09f},
    {0.0013888889225199819f, -3.3631094437103215e-11f}, {2.4801587642286904e-05f, -3.40699609366682e-13f},
    {2.755731998149713e-07f, -7.575112209051195e-15f}, {2.0876755879584152e-09f, 1.1082839147459852e-16f},
    {1.147074536050896e-11f, 2.372207689231238e-19f}};  // 1/(2m)!
static __device__ const float2 g_df_cos_j[16] = {
    {1.0f, 0.0f}, {0.9238795042037964f, 2.830748968563057e-08f}, {0.7071067690849304f, 1.2101617485882343e-08f},
    {0.3826834261417389f, 6.2233507236442165e-09f}, {0.0f, 0.0f}, {-0.3826834261417389f, -6.2233507236442165e-09f},
    {-0.7071067690849304f, -1.2101617485882343e-08f}, {-0.9238795042037964f, -2.830748968563057e-08f},
    {-1.0f, 0.0f}, {-0.9238795042037964f, -2.830748968563057e-08f}, {-0.7071067690849304f, -1.2101617485882343e-08f},
    {-0.3826834261417389f, -6.2233507236442165e-09f}, {0.0f, 0.0f}, {0.3826834261417389f, 6.2233507236442165e-09f},
    {0.7071067690849304f, 1.2101617485882343e-08f}, {0.9238795042037964f, 2.830748968563057e-08f}};  // cos(j pi/8)

__device__ __forceinline__ df df_ld(const float2* t, int i) {
  const float2 v = t[i];
  return dfmk(v.x, v.y);
}

__device__ __forceinline__ void df_sincos(df x, df* s, df* c) {
  const float P1 = 0.39269909262657166f, P2 = -1.0927847071684482e-08f, P3 = -4.2878112750147047e-16f;  // pi/8
  const float jf = rintf(x.hi * 2.5464789867401123f);                                                  // x 8/pi
  df t = df_sub(x, two_prod(jf, P1));
  t = df_sub(t, two_prod(jf, P2));
  t = df_add_f(t, __fmul_rn(-jf, P3));
  const df mu = df_neg(df_sqr(t));  // -t^2
  df sp = df_ld(g_df_sin_c, 5), cp = df_ld(g_df_cos_c, 5);
#pragma unroll
  for (int m = 4; m >= 0; m--) {
    sp = df_fma(df_ld(g_df_sin_c, m), sp, mu);
    cp = df_fma(df_ld(g_df_cos_c, m), cp, mu);
  }
  const df st = df_mul(sp, t), ct = cp;
  const int j = ((int)jf) & 15;
  const df ca = df_ld(g_df_cos_j, j), sa = df_ld(g_df_cos_j, (j + 12) & 15);  // sin(a) = cos(a - pi/2)
  *s = df_fma(df_mul(st, ca), ct, sa);
  *c = df_fma(df_mul(ct, ca), df_neg(st), sa);
}

// exp(y) in double-float, |y| < 80: y = n ln2 + r, |r| <= ln2 / 2 (ln 2 in
// three floats), Taylor polynomial of r to r^15 (truncation below 1e-18), then
// the exact scaling by 2^n
static __device__ const float2 g_df_exp_c[16] = {
    {1.0f, 0.0f}, {1.0f, 0.0f}, {0.5f, 0.0f}, {0.1666666716337204f, -4.967053879312289e-09f},
    {0.0416666679084301f, -1.2417634698280722e-09f}, {0.008333333767950535f, -4.34617203337595e-10f},
    {0.0013888889225199819f, -3.3631094437103215e-11f}, {0.00019841270113829523f, -2.725596874933456e-12f},
    {2.4801587642286904e-05f, -3.40699609366682e-13f}, {2.7557318844628753e-06f, 3.793571224297229e-14f},
    {2.755731998149713e-07f, -7.575112209051195e-15f}, {2.5052107943679403e-08f, 4.4176230446483665e-16f},
    {2.0876755879584152e-09f, 1.1082839147459852e-16f}, {1.6059044372074283e-10f, -5.352526511562726e-18f},
    {1.147074536050896e-11f, 2.372207689231238e-19f}, {7.647163609812713e-13f, 1.2200710471178288e-20f}};  // 1/k!

__device__ __forceinline__ df df_exp(df y) {
  const float L1 = 0.6931471824645996f, L2 = -1.9046542121259336e-09f, L3 = -8.78318373858934e-17f;  // ln 2
  const float nf = rintf(y.hi * 1.4426950216293335f);
  df r = df_sub(y, two_prod(nf, L1));
  r = df_sub(r, two_prod(nf, L2));
  r = df_add_f(r, __fmul_rn(-nf, L3));
  df e = df_ld(g_df_exp_c, 15);
#pragma unroll
  for (int k = 14; k >= 0; k--) e = df_fma(df_ld(g_df_exp_c, k), e, r);
  const float sc = ldexpf(1.0f, (int)nf);
  return dfmk(e.hi * sc, e.lo * sc);
}

// e^{i k x} for k = kr + i ki
__device__ __forceinline__ dfc dfc_expik(df kr, df ki, df x) {
  df sn, cs;
  df_sincos(df_mul(kr, x), &sn, &cs);
  dfc r = dfcmk(cs, sn);
  if (ki.hi != 0.0f) r = dfc_scale(r, df_exp(df_neg(df_mul(ki, x))));
  return r;
}

// cosh and sinh of b: Taylor polynomials to b^15 for |b| < 1/2 (truncation
// below 1e-22), exponentials otherwise
__device__ __forceinline__ void df_coshsinh(df b, df* ch, df* sh) {
  if (fabsf(b.hi) < 0.5f) {
    const df t = df_sqr(b);
    df sp = df_ld(g_df_sin_c, 7), cp = df_ld(g_df_cos_c, 7);
#pragma unroll
    for (int m = 6; m >= 0; m--) {
      sp = df_fma(df_ld(g_df_sin_c, m), sp, t);
      cp = df_fma(df_ld(g_df_cos_c, m), cp, t);
    }
    *sh = df_mul(sp, b);
    *ch = cp;
  } else {
    const df e = df_exp(b), ei = df_rcp(e);
    *ch = df_mul_f(df_add(e, ei), 0.5f);
    *sh = df_mul_f(df_sub(e, ei), 0.5f);
  }
}

// cos z and sin z of a complex argument
__device__ __forceinline__ void dfc_cossin(dfc z, dfc* cz, dfc* sz) {
  df s, c;
  df_sincos(z.re, &s, &c);
  if (z.im.hi == 0.0f) {
    const df zero = dfmk(0.0f, 0.0f);
    *cz = dfcmk(c, zero);
    *sz = dfcmk(s, zero);
    return;
  }
  df ch, sh;
  df_coshsinh(z.im, &ch, &sh);
  *cz = dfcmk(df_mul(c, ch), df_neg(df_mul(s, sh)));
  *sz = dfcmk(df_mul(s, ch), df_mul(c, sh));
}

__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return dfcmk(df_sub(a.re, b.re), df_sub(a.im, b.im)); }
__device__ __forceinline__ dfc dfc_muli(dfc a) { return dfcmk(df_neg(a.im), a.re); }  // i a
