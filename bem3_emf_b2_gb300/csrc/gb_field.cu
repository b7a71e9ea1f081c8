// gb_field.cu -- potentials and fields at arbitrary points (batched).
//
// Replaces, on the GPU:
//   domain_id / fid_calc_solid_angle  reference setup2.c:871-978
//   mEMP_s, EH_s, EH_mEMP_s           d3b1_field.c:12-209
//   mEMP2_s (scattered potential and its directional derivative at the
//            nodes of another object)  mo_solve.c:351-396
//   EH_s_bd (fields on the boundary, own element integrated singularly)
//                                     d3b1_field.c:238-279
// One warp per point for the domain id (solid-angle sums over each domain's
// element list, boundary and region decisions as the reference's) and for the
// boundary-integral sums (lanes over source elements).  A lane whose pair needs the GHN fallback
// (|Re dF/dv| > CBD_SDF, d3b1_elem.c:296,314) gets it integrated by the whole
// warp.
#include "gb_quad_df.cuh"
#include "gb_reduce.cuh"
#include "gb_internal.h"
#include "gb_fieldobj.cuh"

extern "C" int gbi_upload_tables_field(const void* t) {
  GB_CUDA(cudaMemcpyToSymbol(c_tab, t, sizeof(GbTables)));
  return gbi_upload_tabd((const GbTables*)t);
}

// the regular integral of one (point, source element) pair: in double-float
// when DF and the rule is GLN (falling back to FP64 near the CBD_SDF
// decision), else FP64 -- the same values to ~1e-14; adapt: the double-float
// rule with the distance-adaptive order (reg_order)
// the FP64 rule as a called function: in the double-float kernels it serves
// only the declined pairs, and its registers then do not count against the
// double-float path's
template <int NDIR>
__device__ __noinline__ void reg_integrate_cold(const Elem& S, int type, const double* rt, const double (*vt)[3], cplx k,
                                                bool neg, RegAcc<NDIR>& A) {
  reg_integrate<NDIR>(S, type, rt, vt, k, neg, A);
}

// NS = 3: every source element is a triangle (the double-float sums then hold
// three shape functions)
template <bool DF, int NDIR, int NS = 4>
__device__ __forceinline__ void reg_pair(const Elem& S, int type, const double rt[3], const double (*vt)[3], cplx k,
                                         bool neg, RegAcc<NDIR>& A, bool adapt) {
  if (DF && type == 2) {
    if (reg_integrate_dn<NDIR, NS>(S, rt, vt, k, neg, A, adapt)) return;
    reg_integrate_cold<NDIR>(S, type, rt, vt, k, neg, A);
    return;
  }
  reg_integrate<NDIR>(S, type, rt, vt, k, neg, A);
}

// ------------------------------------------------------------------ domain id
__device__ __forceinline__ void cross3(const double a[3], const double b[3], double r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ int unit3(double a[3]) {
  double n = norm3(a);
  if (n == 0.0) return -1;
  a[0] /= n; a[1] /= n; a[2] /= n;
  return 0;
}
// solid angle of a triangle (r0,r1,r2) seen from the origin via its three
// spherical angles; *onb = 1 if the origin lies on the triangle's plane
__device__ __forceinline__ double tri_solid(const double r0[3], const double r1[3], const double r2[3], int* onb) {
  double n01[3], n12[3], n20[3], nt[3];
  cross3(r0, r1, n01);
  cross3(r1, r2, n12);
  cross3(r2, r0, n20);
  cross3(n01, n20, nt);
  double a0 = atan2(norm3(nt), -dot3(n01, n20));
  cross3(n12, n01, nt);
  double a1 = atan2(norm3(nt), -dot3(n12, n01));
  cross3(n20, n12, nt);
  double a2 = atan2(norm3(nt), -dot3(n20, n12));
  double D = dot3(r0, n12);
  if (D > 0.0) return a0 + a1 + a2 - GB_PI;
  if (D < 0.0) return -(a0 + a1 + a2 - GB_PI);
  *onb = 1;
  return 0.0;
}
// element solid angle (reference fid_calc_solid_angle, setup2.c:871-942): the
// quadrangle is split into (0,1,2) and (0,2,3) with unit corner vectors
__device__ double elem_solid_angle(int quad, double r[4][3], int* onb) {
  int nv = quad ? 4 : 3;
  int st = 0;
  for (int j = 0; j < nv; j++) st += unit3(r[j]);
  if (st < 0) { *onb = 1; return 0.0; }
  double om = tri_solid(r[0], r[1], r[2], onb);
  if (*onb) return 0.0;
  if (quad) {
    om += tri_solid(r[0], r[2], r[3], onb);
    if (*onb) return 0.0;
  }
  return om;
}

// Domain of a point (reference domain_id, setup2.c:944-978): per domain d in
// order, accumulate the solid angles of its positively listed elements into
// Og[d] and subtract them from Og[sd]; a point on an element of domain d's list
// belongs to d; after domain d's list, |Og[0]| < 2 pi (d = 0) or Og[d] > 2 pi
// decides d; no decision: -1.
// One warp per point, lanes over the elements of each domain's list: a
// boundary hit anywhere in domain d's list returns d (the sequential loop
// returns d at its first hit), and the region tests after domain d read the
// warp-reduced sums Og (their summation order differs from the sequential
// loop only by rounding).
// FP32 screen of the same decision: unit vectors, spherical angles and sums
// in FP32; a point is decided here only when no element's plane passes within
// a relative 1e-4 of it, no corner coincides with it and every decision sum
// is farther than 0.01 from 2 pi (FP32 sums of up to ~1e5 solid angles err
// by far less); otherwise (and for a boundary hit) the FP64 path below
// decides, so the result is the FP64 path's.
__device__ __forceinline__ void cross3f(const float a[3], const float b[3], float r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ float dot3f(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
__device__ __forceinline__ float norm3f(const float a[3]) { return sqrtf(dot3f(a, a)); }
// solid angle of the triangle of unit vectors (r0, r1, r2); *unsure when the
// point lies within a relative 1e-4 of the triangle's plane
__device__ __forceinline__ float tri_solid_f(const float r0[3], const float r1[3], const float r2[3], bool* unsure) {
  float n01[3], n12[3], n20[3], nt[3];
  cross3f(r0, r1, n01);
  cross3f(r1, r2, n12);
  cross3f(r2, r0, n20);
  cross3f(n01, n20, nt);
  const float a0 = atan2f(norm3f(nt), -dot3f(n01, n20));
  cross3f(n12, n01, nt);
  const float a1 = atan2f(norm3f(nt), -dot3f(n12, n01));
  cross3f(n20, n12, nt);
  const float a2 = atan2f(norm3f(nt), -dot3f(n20, n12));
  const float D = dot3f(r0, n12);
  if (!(fabsf(D) > 1e-4f * norm3f(n12))) { *unsure = true; return 0.0f; }
  return D > 0.0f ? a0 + a1 + a2 - (float)GB_PI : -(a0 + a1 + a2 - (float)GB_PI);
}
// the FP32 decision of k_domain_id for the warp's point: the domain id, or -2
// when the FP64 path must decide
__device__ int domain_id_f32(const FieldObj& o, const double r0[3], int lane) {
  float Og[GB_MAXDOM];
  for (int d = 0; d <= o.MN; d++) Og[d] = 0.0f;
  for (int d = 0; d <= o.MN; d++) {
    const int* sid = o.sid + o.sb_off[d];
    bool unsure = false;
    for (int i = 1 + lane; i <= o.sb_Ne[d]; i += 32) {
      const int s = sid[i];
      if (s <= 0) continue;
      float r[4][3];
      const int nv = o.etype[s] ? 4 : 3;
      for (int j = 0; j < nv; j++) {
        for (int k = 0; k < 3; k++) r[j][k] = (float)(o.corner[(size_t)s * 12 + j * 3 + k] - r0[k]);
        const float nr = norm3f(r[j]);
        if (!(nr > 0.0f)) { unsure = true; break; }
        for (int k = 0; k < 3; k++) r[j][k] /= nr;
      }
      if (unsure) break;
      float om = tri_solid_f(r[0], r[1], r[2], &unsure);
      if (nv == 4 && !unsure) om += tri_solid_f(r[0], r[2], r[3], &unsure);
      if (unsure) break;
      Og[d] += om;
      Og[o.sd[s]] -= om;
    }
    if (__any_sync(0xffffffffu, unsure)) return -2;
    float od = Og[d];
    for (int off = 16; off > 0; off >>= 1) od += __shfl_xor_sync(0xffffffffu, od, off);
    const float tp = 2.0f * (float)GB_PI;
    if (fabsf(fabsf(od) - tp) < 0.01f || fabsf(od - tp) < 0.01f) return -2;
    if (d == 0 && fabsf(od) < tp) return 0;
    if (od > tp) return d;
  }
  return -1;
}

__global__ void __launch_bounds__(128) k_domain_id(FieldObj o, int n, const double* rt, int* did) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= n) return;
  const double r0[3] = {rt[3 * p], rt[3 * p + 1], rt[3 * p + 2]};
  const int fast = domain_id_f32(o, r0, lane);
  if (fast != -2) {
    if (lane == 0) did[p] = fast;
    return;
  }
  double Og[GB_MAXDOM];
  for (int d = 0; d <= o.MN; d++) Og[d] = 0.0;
  int res = -1;
  for (int d = 0; d <= o.MN; d++) {
    const int* sid = o.sid + o.sb_off[d];
    int hit = 0;
    for (int i = 1 + lane; i <= o.sb_Ne[d]; i += 32) {
      const int s = sid[i];
      if (s <= 0) continue;
      double r[4][3];
      for (int j = 0; j < 4; j++)
        for (int k = 0; k < 3; k++) r[j][k] = o.corner[(size_t)s * 12 + j * 3 + k] - r0[k];
      int onb = 0;
      const double om = elem_solid_angle(o.etype[s], r, &onb);
      if (onb) { hit = 1; continue; }
      Og[d] += om;
      Og[o.sd[s]] -= om;
    }
    if (__any_sync(0xffffffffu, hit)) { res = d; break; }
    double od = Og[d];
    for (int off = 16; off > 0; off >>= 1) od += __shfl_xor_sync(0xffffffffu, od, off);
    if (d == 0 && fabs(od) < 2.0 * GB_PI) { res = 0; break; }
    if (od > 2.0 * GB_PI) { res = d; break; }
  }
  if (lane == 0) did[p] = res;
}

// Resident blocks of 128 threads per SM the point-sum kernels are compiled
// for (register cap 65536 / (128 x blocks)): the double-float sums are
// latency-bound chains, so more resident warps can outweigh spilled registers
#ifndef GB_FIELD_MINB
#define GB_FIELD_MINB 1
#endif
#ifndef GB_CROSS_MINB
#define GB_CROSS_MINB 3
#endif

// ------------------------------------------------------------------ field sums
enum { FM_MEMP = 0, FM_EH = 1, FM_EH_MEMP = 2, FM_MEMP2 = 3 };

// Per-lane GHN fallback of flagged pairs, integrated by the whole warp.
template <int NDIR>
__device__ void warp_fallback(bool fb, const Elem& S, const double rt[3], const double (*vt)[3], cplx k, bool neg,
                              RegAcc<NDIR>& A) {
  unsigned mask = __ballot_sync(0xffffffffu, fb);
  const int lane = threadIdx.x & 31;
  while (mask) {
    int src = __ffs(mask) - 1;
    mask &= mask - 1;
    Elem Sb;
    for (int i = 0; i < 12; i++) (&Sb.cr[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cr[0][0])[i], src);
    for (int i = 0; i < 9; i++) (&Sb.cw[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cw[0][0])[i], src);
    Sb.quad = __shfl_sync(0xffffffffu, S.quad, src);
    bool negb = __shfl_sync(0xffffffffu, (int)neg, src) != 0;
    RegAcc<NDIR> B;
    reg_integrate_gh_part<NDIR>(Sb, lane, 32, rt, vt, k, B);
    warp_allreduce<sizeof(RegAcc<NDIR>) / sizeof(double)>((double*)&B);
    reg_finish<NDIR>(B, reg_scale_gh(Sb), negb);
    if (lane == src) A = B;
  }
}

struct FieldArgs {
  FieldObj o;
  int mode, type, n;
  const double* rt;   // [n][3]
  const double* v;    // [n][3] (FM_MEMP2)
  const int* did;     // [n]
  cplx* out;          // per point: FM_MEMP 4, FM_EH 6, FM_EH_MEMP 6, FM_MEMP2 8
  int* flag;          // FM_EH_MEMP: -did where the near-boundary cutoff applies, else did
};

// one warp per point; the point's domain (and therefore its source list and
// wave number) is uniform across the warp
// MODE: FM_MEMP, FM_EH or FM_MEMP2, fixed at compile time so that each
// variant holds only its own accumulators
template <bool DF, int MODE, int NS = 4>
__global__ void __launch_bounds__(128, GB_FIELD_MINB) k_field(FieldArgs a) {
  constexpr int NACC = MODE == FM_MEMP ? 9 : (MODE == FM_EH ? 13 : 18);
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= a.n) return;
  const FieldObj& o = a.o;
  int did = a.did[p];
  if (did < 0 || did > o.MN) return;
  double rt[3] = {a.rt[3 * p], a.rt[3 * p + 1], a.rt[3 * p + 2]};
  cplx k = cmk(o.kn[2 * did], o.kn[2 * did + 1]);
  const int* sid = o.sid + o.sb_off[did];
  const int Ne = o.sb_Ne[did];
  const cplx* U = o.U[did];
  const cplx* dU = o.dU[did];
  const cplx* Eb = o.E[did];
  const cplx* dEb = o.dE[did];
  const cplx* Hb = o.H[did];
  const cplx* dHb = o.dH[did];
  // accumulators (per lane), then reduced
  double acc[NACC];
  for (int i = 0; i < NACC; i++) acc[i] = 0.0;
  int niter = (Ne + 31) / 32;
  for (int it = 0; it < niter; it++) {
    int s = 1 + it * 32 + lane;
    bool act = s <= Ne;
    int sd = act ? sid[s] : sid[1];
    Elem S;
    load_elem(S, o.cr, o.cw, o.etype, abs(sd));
    bool neg = sd < 0;
    if (MODE == FM_MEMP || MODE == FM_EH) {
      if (!act) continue;
      RegAcc<0> A;
      reg_pair<DF, 0, NS>(S, a.type, rt, nullptr, k, neg, A, o.prec == 3);
      acc[0] += A.F;
      if (MODE == FM_MEMP) {
        for (int n = 0; n < 4; n++)
          for (int l = 0; l < 4; l++) {
            cplx t = A.G[n] * dU[((size_t)s * 4 + n) * 4 + l] - A.H[n] * U[((size_t)s * 4 + n) * 4 + l];
            acc[1 + 2 * l] += t.x;
            acc[2 + 2 * l] += t.y;
          }
      } else {
        for (int n = 0; n < 4; n++)
          for (int l = 0; l < 3; l++) {
            size_t q = ((size_t)s * 4 + n) * 3 + l;
            cplx te = A.G[n] * dEb[q] - A.H[n] * Eb[q];
            cplx th = A.G[n] * dHb[q] - A.H[n] * Hb[q];
            acc[1 + 2 * l] += te.x;
            acc[2 + 2 * l] += te.y;
            acc[7 + 2 * l] += th.x;
            acc[8 + 2 * l] += th.y;
          }
      }
    } else if (MODE == FM_MEMP2) {
      double vt[1][3] = {{a.v[3 * p], a.v[3 * p + 1], a.v[3 * p + 2]}};
      RegAcc<1> A;
      bool fb = false;
      if (act) {
        reg_pair<DF, 1, NS>(S, a.type, rt, vt, k, neg, A, o.prec == 3);
        fb = a.type < 3 && fabs(A.dF[0]) > GB_CBD_SDF;
      }
      warp_fallback<1>(fb, S, rt, vt, k, neg, A);
      if (!act) continue;
      acc[0] += A.F;
      acc[1] += A.dF[0];
      for (int n = 0; n < 4; n++)
        for (int l = 0; l < 4; l++) {
          size_t q = ((size_t)s * 4 + n) * 4 + l;
          cplx u = A.G[n] * dU[q] - A.H[n] * U[q];
          cplx du = A.dG[0][n] * dU[q] - A.dH[0][n] * U[q];
          acc[2 + 2 * l] += u.x;
          acc[3 + 2 * l] += u.y;
          acc[10 + 2 * l] += du.x;
          acc[11 + 2 * l] += du.y;
        }
    }
  }
  warp_allreduce<NACC>(acc);
  if (lane != 0) return;
  double F = acc[0];
  double den = (did == 0) ? 1.0 + F : F;
  cplx* out = a.out;
  if (MODE == FM_MEMP) {
    for (int l = 0; l < 4; l++) out[(size_t)p * 4 + l] = cdivr(cmk(acc[1 + 2 * l], acc[2 + 2 * l]), den);
  } else if (MODE == FM_EH) {
    for (int l = 0; l < 6; l++) out[(size_t)p * 6 + l] = cdivr(cmk(acc[1 + 2 * l], acc[2 + 2 * l]), den);
  } else if (MODE == FM_MEMP2) {
    double dF = acc[1];
    for (int l = 0; l < 4; l++) {
      cplx u = cdivr(cmk(acc[2 + 2 * l], acc[3 + 2 * l]), den);
      cplx du = cdivr(cmk(acc[10 + 2 * l], acc[11 + 2 * l]) - u * dF, den);
      out[(size_t)p * 8 + l] = u;
      out[(size_t)p * 8 + 4 + l] = du;
    }
  }
}

// Adds pair s's share to the FM_EH_MEMP accumulators: `take` bit d (d < 3)
// selects the derivative terms of direction d, bit 3 the potential terms.
__device__ __forceinline__ void eh_memp_add(double* acc, const RegAcc<3>& A, unsigned take, const cplx* U,
                                            const cplx* dU, int s) {
  if (take & 8u) acc[0] += A.F;
  for (int d = 0; d < 3; d++)
    if (take & (1u << d)) acc[1 + d] += A.dF[d];
  for (int n = 0; n < 4; n++)
    for (int l = 0; l < 4; l++) {
      size_t q = ((size_t)s * 4 + n) * 4 + l;
      if (take & 8u) {
        cplx u = A.G[n] * dU[q] - A.H[n] * U[q];
        acc[4 + 2 * l] += u.x;
        acc[5 + 2 * l] += u.y;
      }
      for (int d = 0; d < 3; d++)
        if (take & (1u << d)) {
          cplx du = A.dG[d][n] * dU[q] - A.dH[d][n] * U[q];
          acc[12 + d * 8 + 2 * l] += du.x;
          acc[13 + d * 8 + 2 * l] += du.y;
        }
    }
}

// FM_EH_MEMP (reference EH_mEMP_s): U and the x,y,z derivatives of all four
// potential components; separate kernel because it needs 2 + 3 + 8 + 24
// accumulators.
template <bool DF>
__global__ void __launch_bounds__(128) k_field_eh_memp(FieldArgs a) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= a.n) return;
  const FieldObj& o = a.o;
  int did = a.did[p];
  if (did < 0 || did > o.MN) return;
  double rt[3] = {a.rt[3 * p], a.rt[3 * p + 1], a.rt[3 * p + 2]};
  cplx k = cmk(o.kn[2 * did], o.kn[2 * did + 1]);
  const int* sid = o.sid + o.sb_off[did];
  const int Ne = o.sb_Ne[did];
  const cplx* U = o.U[did];
  const cplx* dU = o.dU[did];
  double acc[36];  // F, dF[3], U[4] (8), dU[3][4] (24)
  for (int i = 0; i < 36; i++) acc[i] = 0.0;
  const double vt[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  int niter = (Ne + 31) / 32;
  for (int it = 0; it < niter; it++) {
    int s = 1 + it * 32 + lane;
    bool act = s <= Ne;
    int sd = act ? sid[s] : sid[1];
    Elem S;
    load_elem(S, o.cr, o.cw, o.etype, abs(sd));
    bool neg = sd < 0;
    // fm: bit d = direction d needs the GHN rule, bit 3 = the potential
    // terms do (they follow the z direction); the regular values of the
    // other parts are added at once, so no copy of them is held while the
    // warp integrates flagged pairs
    unsigned fm = 0;
    if (act) {
      RegAcc<3> A;
      reg_pair<DF, 3>(S, a.type, rt, vt, k, neg, A, o.prec == 3);
      if (a.type < 3)
        for (int d = 0; d < 3; d++)
          if (fabs(A.dF[d]) > GB_CBD_SDF) fm |= 1u << d;
      if (fm & 4u) fm |= 8u;
      eh_memp_add(acc, A, ~fm & 15u, U, dU, s);
    }
    unsigned mask = __ballot_sync(0xffffffffu, fm != 0);
    while (mask) {
      int src = __ffs(mask) - 1;
      mask &= mask - 1;
      Elem Sb;
      for (int i = 0; i < 12; i++) (&Sb.cr[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cr[0][0])[i], src);
      for (int i = 0; i < 9; i++) (&Sb.cw[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cw[0][0])[i], src);
      Sb.quad = __shfl_sync(0xffffffffu, S.quad, src);
      bool negb = __shfl_sync(0xffffffffu, (int)neg, src) != 0;
      RegAcc<3> B;
      reg_integrate_gh_part<3>(Sb, lane, 32, rt, vt, k, B);
      warp_allreduce<sizeof(RegAcc<3>) / sizeof(double)>((double*)&B);
      reg_finish<3>(B, reg_scale_gh(Sb), negb);
      if (lane == src) eh_memp_add(acc, B, fm, U, dU, s);
    }
  }
  warp_allreduce<36>(acc);
  if (lane != 0) return;
  double F = acc[0];
  double den = (did == 0) ? 1.0 + F : F;
  cplx Uv[4], dUv[3][4];
  for (int l = 0; l < 4; l++) Uv[l] = cdivr(cmk(acc[4 + 2 * l], acc[5 + 2 * l]), den);
  for (int d = 0; d < 3; d++)
    for (int l = 0; l < 4; l++) dUv[d][l] = cdivr(cmk(acc[12 + d * 8 + 2 * l], acc[13 + d * 8 + 2 * l]) - Uv[l] * acc[1 + d], den);
  cplx* out = a.out + (size_t)p * 6;
  if (fabs(acc[1]) > GB_CBD_CDF || fabs(acc[2]) > GB_CBD_CDF || fabs(acc[3]) > GB_CBD_CDF) {
    for (int i = 0; i < 6; i++) out[i] = cmk(0, 0);
    a.flag[p] = -did;
    return;
  }
  a.flag[p] = did;
  for (int i = 0; i < 3; i++) out[i] = Uv[i] - dUv[i][3];
  // ch = lambda0 / (2 pi i) = -i lambda0 / (2 pi)
  cplx ch = cmk(0.0, -o.lambda0 / (2.0 * GB_PI));
  out[3] = ch * (dUv[1][2] - dUv[2][1]);
  out[4] = ch * (dUv[2][0] - dUv[0][2]);
  out[5] = ch * (dUv[0][1] - dUv[1][0]);
}

// ------------------------------------------------------------------ on-boundary
// Fields on the boundary of the own object (reference EH_s_bd): point on
// element t (1-based index in domain did's list) at (zt, et); the pair s == t
// is integrated singularly (coef_bd) by the whole warp.
struct BdArgs {
  FieldObj o;
  int type, n;
  const int* did;
  const int* t;
  const double* zt;  // [n][2]
  cplx* out;         // [n][6]: E, H
};

template <bool DF, int NS = 4>
__global__ void __launch_bounds__(128, GB_FIELD_MINB) k_field_bd(BdArgs a) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= a.n) return;
  const FieldObj& o = a.o;
  int did = a.did[p];
  const int* sid = o.sid + o.sb_off[did];
  const int Ne = o.sb_Ne[did];
  int t = a.t[p];
  int td = sid[t];
  double zt = a.zt[2 * p], et = a.zt[2 * p + 1];
  Elem T;
  load_elem(T, o.cr, o.cw, o.etype, abs(td));
  double rt[3];
  for (int d = 0; d < 3; d++) {
    rt[d] = T.cr[d][0] + T.cr[d][1] * zt + T.cr[d][2] * et;
    if (T.quad) rt[d] += T.cr[d][3] * zt * et;
  }
  cplx k = cmk(o.kn[2 * did], o.kn[2 * did + 1]);
  const cplx* Eb = o.E[did];
  const cplx* dEb = o.dE[did];
  const cplx* Hb = o.H[did];
  const cplx* dHb = o.dH[did];
  double acc[13];
  for (int i = 0; i < 13; i++) acc[i] = 0.0;
  for (int s = 1 + lane; s <= Ne; s += 32) {
    int sd = sid[s];
    if (sd == td) continue;
    Elem S;
    load_elem(S, o.cr, o.cw, o.etype, abs(sd));
    RegAcc<0> A;
    reg_pair<DF, 0, NS>(S, a.type, rt, nullptr, k, sd < 0, A, o.prec == 3);
    acc[0] += A.F;
    for (int n = 0; n < 4; n++)
      for (int l = 0; l < 3; l++) {
        size_t q = ((size_t)s * 4 + n) * 3 + l;
        cplx te = A.G[n] * dEb[q] - A.H[n] * Eb[q];
        cplx th = A.G[n] * dHb[q] - A.H[n] * Hb[q];
        acc[1 + 2 * l] += te.x;
        acc[2 + 2 * l] += te.y;
        acc[7 + 2 * l] += th.x;
        acc[8 + 2 * l] += th.y;
      }
  }
  // singular self term
  SingCtx c;
  c.E = T;
  c.zt = zt;
  c.et = et;
  c.k = k;
  sing_setup(c);
  SingAcc A;
  singacc_zero(A);
  int nit = sing_items(c, 0);
  for (int q = lane; q < nit; q += 32) sing_item(c, q, A);
  warp_allreduce<51>((double*)&A);
  sing_finish(c, A, td < 0);
  if (lane == 0) {
    acc[0] += A.F;
    for (int n = 0; n < 4; n++)
      for (int l = 0; l < 3; l++) {
        size_t q = ((size_t)t * 4 + n) * 3 + l;
        cplx te = A.G[n] * dEb[q] - A.H[n] * Eb[q];
        cplx th = A.G[n] * dHb[q] - A.H[n] * Hb[q];
        acc[1 + 2 * l] += te.x;
        acc[2 + 2 * l] += te.y;
        acc[7 + 2 * l] += th.x;
        acc[8 + 2 * l] += th.y;
      }
  }
  warp_allreduce<13>(acc);
  if (lane != 0) return;
  double den = (did == 0) ? 1.0 + acc[0] : acc[0];
  for (int l = 0; l < 6; l++) a.out[(size_t)p * 6 + l] = cdivr(cmk(acc[1 + 2 * l], acc[2 + 2 * l]), den);
}

// ------------------------------------------------------------------ cross operators
// The potential scattered by object src at fixed points (the exterior nodes
// of another object, mEMP2_s of add_scattered_mEMP, reference mo_solve.c:351-396)
// is linear in src's boundary values of domain 0:
//   u_l(p)  = (sum_c G[p][c] dU[c][l] - H[p][c] U[c][l]) / den_p
//   du_l(p) = (sum_c dG[p][c] dU[c][l] - dH[p][c] U[c][l] - u_l(p) dF_p) / den_p
// with c = (element s, shape function n) of src's domain-0 list and
// den_p = 1 + F_p.  k_cross_build integrates these coefficients once, with
// the quadrature and GHN fallback of k_field's mode 3, and stores them with
// F_p and dF_p; k_cross_apply evaluates the sums at every iteration of the
// multiple-scattering loop (a matrix-vector product instead of a quadrature).
struct CrossArgs {
  FieldObj o;
  int type, n, C;
  const double* rt;  // [n][3]
  const double* v;   // [n][3]
  cplx* Gm;          // [n][C]
  cplx* Hm;
  cplx* dGm;
  cplx* dHm;
  double* Fp;        // [n][2]: F, dF
  // two-pass build (double-float first): only the pairs flagged in `only`
  // ([n][Ne]) are integrated, and their F, dF go to Fs ([n][Ne][2]) instead
  // of the per-point sums
  const uint8_t* only;
  double* Fs;
  // coefficients stored in double-float (float4: re.hi, re.lo, im.hi, im.lo
  // in the 16 bytes of a complex FP64 entry), for k_cross_apply_df
  int dfout;
};

// one coefficient into a cross-operator matrix, complex FP64 or double-float
__device__ __forceinline__ void store_coef(cplx* M, size_t i, cplx v, int dfout) {
  if (!dfout) { M[i] = v; return; }
  const float rh = (float)v.x, ih = (float)v.y;
  ((float4*)M)[i] = make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
}

template <bool DF>
__global__ void __launch_bounds__(128) k_cross_build(CrossArgs a) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= a.n) return;
  const FieldObj& o = a.o;
  const double rt[3] = {a.rt[3 * p], a.rt[3 * p + 1], a.rt[3 * p + 2]};
  const double vt[1][3] = {{a.v[3 * p], a.v[3 * p + 1], a.v[3 * p + 2]}};
  const cplx k = cmk(o.kn[0], o.kn[1]);
  const int* sid = o.sid + o.sb_off[0];
  const int Ne = o.sb_Ne[0];
  double F = 0.0, dF = 0.0;
  const size_t row = (size_t)p * a.C;
  const int niter = (Ne + 31) / 32;
  for (int it = 0; it < niter; it++) {
    const int s = 1 + it * 32 + lane;
    const bool act = s <= Ne;
    const int sd = act ? sid[s] : sid[1];
    Elem S;
    load_elem(S, o.cr, o.cw, o.etype, abs(sd));
    const bool neg = sd < 0;
    const bool todo = act && (!a.only || a.only[(size_t)p * Ne + s - 1]);
    RegAcc<1> A;
    bool fb = false;
    if (todo) {
      reg_pair<DF, 1>(S, a.type, rt, vt, k, neg, A, o.prec == 3);
      fb = a.type < 3 && fabs(A.dF[0]) > GB_CBD_SDF;
    }
    warp_fallback<1>(fb, S, rt, vt, k, neg, A);
    if (!todo) continue;
    if (a.Fs) {
      a.Fs[((size_t)p * Ne + s - 1) * 2] = A.F;
      a.Fs[((size_t)p * Ne + s - 1) * 2 + 1] = A.dF[0];
    }
    F += A.F;
    dF += A.dF[0];
    const size_t c = row + (size_t)(s - 1) * 4;
    for (int nn = 0; nn < 4; nn++) {
      store_coef(a.Gm, c + nn, A.G[nn], a.dfout);
      store_coef(a.Hm, c + nn, A.H[nn], a.dfout);
      store_coef(a.dGm, c + nn, A.dG[0][nn], a.dfout);
      store_coef(a.dHm, c + nn, A.dH[0][nn], a.dfout);
    }
  }
  for (int o2 = 16; o2 > 0; o2 >>= 1) {
    F += __shfl_down_sync(0xffffffffu, F, o2);
    dF += __shfl_down_sync(0xffffffffu, dF, o2);
  }
  if (lane == 0 && !a.Fs) { a.Fp[2 * p] = F; a.Fp[2 * p + 1] = dF; }
}

// double-float pass of the two-pass build: one thread per (point, source
// element) pair, the GLN rule in double-float (reg_integrate_dn); pairs it
// declines (near the CBD_SDF decision) are flagged for the FP64 pass
// TSEL as for the assembly: 0 every pair, 1 triangle sources only (three
// shape functions' sums), 2 quadrangle sources only
template <int TSEL>
__global__ void __launch_bounds__(128, GB_CROSS_MINB) k_cross_build_df(CrossArgs a, uint8_t* redo) {
  const FieldObj& o = a.o;
  const int Ne = o.sb_Ne[0];
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)a.n * Ne) return;
  const int p = (int)(q / Ne), s = 1 + (int)(q % Ne);
  const int sd = o.sid[o.sb_off[0] + s];
  if (TSEL != 0 && (o.etype[abs(sd)] != 0) != (TSEL == 2)) return;
  const double rt[3] = {a.rt[3 * p], a.rt[3 * p + 1], a.rt[3 * p + 2]};
  const double vt[1][3] = {{a.v[3 * p], a.v[3 * p + 1], a.v[3 * p + 2]}};
  const cplx k = cmk(o.kn[0], o.kn[1]);
  Elem S;
  load_elem(S, o.cr, o.cw, o.etype, abs(sd));
  RegAcc<1> A;
  if (!reg_integrate_dn<1, TSEL == 1 ? 3 : 4>(S, rt, vt, k, sd < 0, A, o.prec == 3)) {
    redo[q] = 1;
    return;
  }
  redo[q] = 0;
  const size_t c = (size_t)p * a.C + (size_t)(s - 1) * 4;
#pragma unroll
  for (int nn = 0; nn < 4; nn++) {
    store_coef(a.Gm, c + nn, A.G[nn], a.dfout);
    store_coef(a.Hm, c + nn, A.H[nn], a.dfout);
    store_coef(a.dGm, c + nn, A.dG[0][nn], a.dfout);
    store_coef(a.dHm, c + nn, A.dH[0][nn], a.dfout);
  }
  a.Fs[2 * q] = A.F;
  a.Fs[2 * q + 1] = A.dF[0];
}

// per point: F, dF summed over the source elements in their order
__global__ void k_cross_fsum(int n, int Ne, const double* Fs, double* Fp) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  double F = 0.0, dF = 0.0;
  for (int s = 0; s < Ne; s++) {
    F += Fs[((size_t)p * Ne + s) * 2];
    dF += Fs[((size_t)p * Ne + s) * 2 + 1];
  }
  Fp[2 * p] = F;
  Fp[2 * p + 1] = dF;
}

// one warp per point: out[p][0..3] = u, out[p][4..7] = du (layout of k_field's mode 3)
__global__ void __launch_bounds__(128) k_cross_apply(int n, int C, const cplx* __restrict__ Gm, const cplx* __restrict__ Hm,
                                                     const cplx* __restrict__ dGm, const cplx* __restrict__ dHm,
                                                     const double* __restrict__ Fp, const cplx* __restrict__ U,
                                                     const cplx* __restrict__ dU, cplx* out) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= n) return;
  double acc[16];
#pragma unroll
  for (int i = 0; i < 16; i++) acc[i] = 0.0;
  const size_t row = (size_t)p * C;
  for (int c = lane; c < C; c += 32) {
    const cplx g = Gm[row + c], h = Hm[row + c], dg = dGm[row + c], dh = dHm[row + c];
    const cplx* u = U + (size_t)(c + 4) * 4;    // element c / 4 + 1 (1-based), node c % 4
    const cplx* du = dU + (size_t)(c + 4) * 4;
#pragma unroll
    for (int l = 0; l < 4; l++) {
      const cplx t = g * du[l] - h * u[l];
      const cplx td = dg * du[l] - dh * u[l];
      acc[2 * l] += t.x;
      acc[2 * l + 1] += t.y;
      acc[8 + 2 * l] += td.x;
      acc[9 + 2 * l] += td.y;
    }
  }
  warp_allreduce<16>(acc);
  if (lane != 0) return;
  const double den = 1.0 + Fp[2 * p], dF = Fp[2 * p + 1];
  for (int l = 0; l < 4; l++) {
    const cplx uu = cdivr(cmk(acc[2 * l], acc[2 * l + 1]), den);
    const cplx dd = cdivr(cmk(acc[8 + 2 * l], acc[9 + 2 * l]) - uu * dF, den);
    out[(size_t)p * 8 + l] = uu;
    out[(size_t)p * 8 + 4 + l] = dd;
  }
}

extern "C" int gbi_cross_build(const FieldObj* o, int type, int n, const double* rt, const double* v, int C, cplx* Gm,
                               cplx* Hm, cplx* dGm, cplx* dHm, double* Fp, int dfout, cudaStream_t st) {
  if (n <= 0) return 0;
  CrossArgs a;
  a.o = *o; a.type = type; a.n = n; a.C = C; a.rt = rt; a.v = v;
  a.Gm = Gm; a.Hm = Hm; a.dGm = dGm; a.dHm = dHm; a.Fp = Fp;
  a.only = nullptr; a.Fs = nullptr; a.dfout = dfout;
  const unsigned nbw = (unsigned)(((size_t)n * 32 + 127) / 128);
  const int Ne = o->sb_Ne[0];
  if (o->prec >= 2 && type == 2 && Ne > 0 && !dfout) {
    gbi_set_error("gbi_cross_build: the double-float build stores double-float coefficients");
    return -1;
  }
  if (o->prec >= 2 && type == 2 && Ne > 0) {
    // double-float pass over all pairs, FP64 pass over the declined ones,
    // then the per-point sums in element order
    const size_t np = (size_t)n * Ne;
    uint8_t* redo = nullptr;
    double* Fs = nullptr;
    GB_CUDA(cudaMallocAsync((void**)&redo, np, st));
    GB_CUDA(cudaMallocAsync((void**)&Fs, np * 2 * sizeof(double), st));
    a.Fs = Fs;
    const unsigned nb = (unsigned)((np + 127) / 128);
    if (o->ntri > 0) {
      k_cross_build_df<1><<<nb, 128, 0, st>>>(a, redo);
      gbi_count_launch();
    }
    if (o->nquad > 0 || o->ntri <= 0) {  // counts not known: the general variant
      if (o->ntri > 0) k_cross_build_df<2><<<nb, 128, 0, st>>>(a, redo);
      else k_cross_build_df<0><<<nb, 128, 0, st>>>(a, redo);
      gbi_count_launch();
    }
    a.only = redo;
    k_cross_build<false><<<nbw, 128, 0, st>>>(a);
    gbi_count_launch();
    k_cross_fsum<<<(n + 127) / 128, 128, 0, st>>>(n, Ne, Fs, Fp);
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
    cudaFreeAsync(redo, st);
    cudaFreeAsync(Fs, st);
    return 0;
  }
  k_cross_build<false><<<nbw, 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// the source's boundary values U, dU (elements 1..C/4, nodes, components)
// in double-float, for k_cross_apply_df
__global__ void k_bv_to_df(int C, const cplx* __restrict__ U, const cplx* __restrict__ dU, float4* Ud, float4* dUd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 4 * C) return;
  const cplx u = U[16 + i], du = dU[16 + i];  // skip element 0
  const float a = (float)u.x, b = (float)u.y, c = (float)du.x, d = (float)du.y;
  Ud[i] = make_float4(a, (float)(u.x - (double)a), b, (float)(u.y - (double)b));
  dUd[i] = make_float4(c, (float)(du.x - (double)c), d, (float)(du.y - (double)d));
}

__device__ __forceinline__ dfc dfc_ld(const float4& f) { return dfcmk(dfmk(f.x, f.y), dfmk(f.z, f.w)); }
// acc + a b (complex double-float) for accumulators read only through df_to
// (compensated steps)
__device__ __forceinline__ dfc dfc_fma(dfc acc, dfc a, dfc b) {
  dfc r;
  r.re = df_acc(df_acc(acc.re, a.re, b.re), df_neg(a.im), b.im);
  r.im = df_acc(df_acc(acc.im, a.re, b.im), a.im, b.re);
  return r;
}

// k_cross_apply with double-float coefficients and boundary values: the
// same sums on the FP32 pipes (the FP64 version is bound by the DFMA rate);
// the division by 1 + F in FP64
__global__ void __launch_bounds__(128) k_cross_apply_df(int n, int C, const float4* __restrict__ Gm,
                                                        const float4* __restrict__ Hm, const float4* __restrict__ dGm,
                                                        const float4* __restrict__ dHm, const double* __restrict__ Fp,
                                                        const float4* __restrict__ Ud, const float4* __restrict__ dUd,
                                                        cplx* out) {
  const int lane = threadIdx.x & 31;
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (p >= n) return;
  const df z = dfmk(0.0f, 0.0f);
  dfc u[4], du[4];
#pragma unroll
  for (int l = 0; l < 4; l++) { u[l] = dfcmk(z, z); du[l] = dfcmk(z, z); }
  const size_t row = (size_t)p * C;
  // software-pipelined: the next column's coefficients and boundary values
  // are loaded before this column's products
  const float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 mn[4] = {f0, f0, f0, f0}, an[4], bn[4];
  if (lane < C) {
    mn[0] = Gm[row + lane]; mn[1] = Hm[row + lane]; mn[2] = dGm[row + lane]; mn[3] = dHm[row + lane];
#pragma unroll
    for (int l = 0; l < 4; l++) { an[l] = dUd[(size_t)lane * 4 + l]; bn[l] = Ud[(size_t)lane * 4 + l]; }
  }
  for (int c = lane; c < C; c += 32) {
    const dfc g = dfc_ld(mn[0]), h = dfc_ld(mn[1]), dg = dfc_ld(mn[2]), dh = dfc_ld(mn[3]);
    float4 ac[4], bc[4];
#pragma unroll
    for (int l = 0; l < 4; l++) { ac[l] = an[l]; bc[l] = bn[l]; }
    const int cn = c + 32;
    if (cn < C) {
      mn[0] = Gm[row + cn]; mn[1] = Hm[row + cn]; mn[2] = dGm[row + cn]; mn[3] = dHm[row + cn];
#pragma unroll
      for (int l = 0; l < 4; l++) { an[l] = dUd[(size_t)cn * 4 + l]; bn[l] = Ud[(size_t)cn * 4 + l]; }
    }
    const dfc mh = dfcmk(df_neg(h.re), df_neg(h.im)), mdh = dfcmk(df_neg(dh.re), df_neg(dh.im));
#pragma unroll
    for (int l = 0; l < 4; l++) {
      const dfc a = dfc_ld(ac[l]), b = dfc_ld(bc[l]);
      u[l] = dfc_fma(dfc_fma(u[l], g, a), mh, b);
      du[l] = dfc_fma(dfc_fma(du[l], dg, a), mdh, b);
    }
  }
  double acc[16];
#pragma unroll
  for (int l = 0; l < 4; l++) {
    acc[2 * l] = df_to(u[l].re);
    acc[2 * l + 1] = df_to(u[l].im);
    acc[8 + 2 * l] = df_to(du[l].re);
    acc[9 + 2 * l] = df_to(du[l].im);
  }
  warp_allreduce<16>(acc);
  if (lane != 0) return;
  const double den = 1.0 + Fp[2 * p], dF = Fp[2 * p + 1];
  for (int l = 0; l < 4; l++) {
    const cplx uu = cdivr(cmk(acc[2 * l], acc[2 * l + 1]), den);
    const cplx dd = cdivr(cmk(acc[8 + 2 * l], acc[9 + 2 * l]) - uu * dF, den);
    out[(size_t)p * 8 + l] = uu;
    out[(size_t)p * 8 + 4 + l] = dd;
  }
}

// dfin: the coefficients are in double-float (gbi_cross_build with dfout)
extern "C" int gbi_cross_apply(int n, int C, const cplx* Gm, const cplx* Hm, const cplx* dGm, const cplx* dHm,
                               const double* Fp, const cplx* U, const cplx* dU, cplx* out, int dfin, cudaStream_t st) {
  if (n <= 0) return 0;
  if (!dfin) {
    k_cross_apply<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, st>>>(n, C, Gm, Hm, dGm, dHm, Fp, U, dU, out);
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
    return 0;
  }
  float4 *Ud = nullptr, *dUd = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&Ud, (size_t)4 * C * sizeof(float4), st));
  GB_CUDA(cudaMallocAsync((void**)&dUd, (size_t)4 * C * sizeof(float4), st));
  k_bv_to_df<<<(unsigned)((4 * (size_t)C + 255) / 256), 256, 0, st>>>(C, U, dU, Ud, dUd);
  k_cross_apply_df<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, st>>>(
      n, C, (const float4*)Gm, (const float4*)Hm, (const float4*)dGm, (const float4*)dHm, Fp, Ud, dUd, out);
  gbi_count_launch();
  gbi_count_launch();
  cudaFreeAsync(Ud, st);
  cudaFreeAsync(dUd, st);
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------ launchers
extern "C" int gbi_domain_id(const FieldObj* o, int n, const double* rt, int* did, cudaStream_t st) {
  if (n <= 0) return 0;
  k_domain_id<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, st>>>(*o, n, rt, did);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbi_field(const FieldObj* o, int mode, int type, int n, const double* rt, const double* v, const int* did,
                         cplx* out, int* flag, cudaStream_t st) {
  if (n <= 0) return 0;
  FieldArgs a;
  a.o = *o;
  a.mode = mode;
  a.type = type;
  a.n = n;
  a.rt = rt;
  a.v = v;
  a.did = did;
  a.out = out;
  a.flag = flag;
  unsigned nb = (unsigned)(((size_t)n * 32 + 127) / 128);
  const bool dfp = o->prec >= 2;
  const bool tri = dfp && o->ntri > 0 && o->nquad == 0;  // only triangles: three shape functions' sums
  if (mode == FM_EH_MEMP) {
    if (dfp) k_field_eh_memp<true><<<nb, 128, 0, st>>>(a);
    else k_field_eh_memp<false><<<nb, 128, 0, st>>>(a);
  } else {
    if (a.mode == FM_MEMP) {
      if (tri) k_field<true, FM_MEMP, 3><<<nb, 128, 0, st>>>(a);
      else if (dfp) k_field<true, FM_MEMP><<<nb, 128, 0, st>>>(a);
      else k_field<false, FM_MEMP><<<nb, 128, 0, st>>>(a);
    } else if (a.mode == FM_EH) {
      if (tri) k_field<true, FM_EH, 3><<<nb, 128, 0, st>>>(a);
      else if (dfp) k_field<true, FM_EH><<<nb, 128, 0, st>>>(a);
      else k_field<false, FM_EH><<<nb, 128, 0, st>>>(a);
    } else {
      if (tri) k_field<true, FM_MEMP2, 3><<<nb, 128, 0, st>>>(a);
      else if (dfp) k_field<true, FM_MEMP2><<<nb, 128, 0, st>>>(a);
      else k_field<false, FM_MEMP2><<<nb, 128, 0, st>>>(a);
    }
  }
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbi_field_bd(const FieldObj* o, int type, int n, const int* did, const int* t, const double* zt, cplx* out,
                            cudaStream_t st) {
  if (n <= 0) return 0;
  BdArgs a;
  a.o = *o;
  a.type = type;
  a.n = n;
  a.did = did;
  a.t = t;
  a.zt = zt;
  a.out = out;
  unsigned nb = (unsigned)(((size_t)n * 32 + 127) / 128);
  if (o->prec >= 2 && o->ntri > 0 && o->nquad == 0) k_field_bd<true, 3><<<nb, 128, 0, st>>>(a);
  else if (o->prec >= 2) k_field_bd<true><<<nb, 128, 0, st>>>(a);
  else k_field_bd<false><<<nb, 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}
