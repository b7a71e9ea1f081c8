// gb_linalg.cu -- dense complex linear algebra of the BEM hot path (FP64 and
// the chosen form's complex FP32 with FP64 refinement).
//
// Replaces, on the GPU:
//   create_Amatrix_csr(_dac)  reference solve_bieq2.c:186-341 (coupled matrix A;
//                             built dense in HBM directly from G,H: no CSR files)
//   lu_dec_A                  solve_bieq2.c:343-408 (MKL zgetrf + zgetri)
//   solve_ABmatrix            mo_solve.c:246-274 (invA * B, streamed from disk there)
//   LAPACKE_zgesv             mo_solve.c:751 (dE/dn, dH/dn with 6 right-hand sides)
// All matrices are row-major, as in the reference's files.
//
// LU: right-looking blocked factorisation with tournament pivoting
// (communication-avoiding LU, "CALU": Grigori, Demmel and Xiang, SIAM J.
// Matrix Anal. Appl. 32 (2011) 1317-1350).  Per panel of nb <= LU_NB columns
// starting at row and column k:
//   k_tslu_leaf    one block per set of TS_ROWS panel rows: partial-pivoting
//                  elimination in shared memory picks nb candidate rows
//   k_tslu_merge   4-ary tree: four candidate sets (their original rows read
//                  back from A) -> nb winners, until one set is left; the last
//                  block writes the winners, in their pivot order, as
//                  LAPACK-style sequential interchanges ipiv[k..k+nb)
//   k_laswp_rows   the interchanges applied across the full row width
//   k_diag_lu      L11 U11 of the (now leading) winner rows
//   k_trsm_right   L21 = A21 U11^-1
//   k_trsm_rows    U12 = L11^-1 A12 (L11 unit lower, staged in shared memory)
//   GEMM           A22 -= L21 U12 (FP64: k_zgemm_nn, DFMA; FP32: tensor
//                  cores, gb_tc.cu)
// Every elimination uses LAPACK's pivot rule (first maximum of |Re|+|Im|);
// the tournament keeps the backward stability of partial pivoting in practice
// while a panel needs about log4(n / TS_ROWS) + 1 dependent launches instead
// of two per column.  The pivot sequence may differ from zgetrf's; the factors
// solve the same system to rounding.
// The inverse solves A X = I through the factors: X = U^-1 (L^-1 (P I)),
// two blocked triangular solves whose updates use the same GEMM kernel.
// The chosen form's FP32 factors are of the butterfly-randomised matrix
// U^T A V (k_rbt_matrix) without interchanges (lu_factor with pivot =
// false: the tournament kernels are skipped); the tournament is its fallback.
// Panels are blocked two-level: 64-column panels update only their
// 256-column outer block, the trailing matrix is updated once per outer
// block with K = 256.
#include "gb_common.cuh"
#include "gb_df64.cuh"
#include "gb_internal.h"
#include <atomic>
#include <vector>

#define LU_NB 64
// outer block: the trailing update's K (256 unless set or tuned: gb_set_lu_outer_block, gb_tune_lu_outer_block)
static std::atomic<int> g_lu_nbo{256};
#define LU_NBO (g_lu_nbo.load(std::memory_order_relaxed))

// ------------------------------------------------------------------ A build
struct ABuildArgs {
  const cplx* G;      // domain matrix [N][N]
  const cplx* H;
  const int* sid;     // domain sid list (1-based)
  const int* rowk;    // [N]: row index within the domain block (-1: unused 4th node)
  const int* eni;
  const int* md;
  const int* sd;
  const int* etype;
  const double* wen;
  const double* kn;   // device copy, 2*(MN+1)
  int Ne, did, nrows;
  size_t base;        // first row of this domain in A
  size_t nn, na;
  cplx* A;
};

// one thread per (cid, row, source element): the coupling rules of the
// reference (solve_bieq2.c:241-316): U block (cid < 3), phi block (cid == 3),
// main-domain rows take (H, -G); sub-domain rows take the interface terms
// with delta = k1^2-k2^2, beta = k1^2/k2^2, sigma = 1-beta.
__global__ void k_build_A(ABuildArgs a) {
  size_t N = (size_t)a.Ne * 4;
  size_t tot = 4 * N * (size_t)a.Ne;
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= tot) return;
  int sidx = (int)(p % a.Ne);
  size_t q = p / a.Ne;
  int row = (int)(q % N);
  int cid = (int)(q / N);
  int k = a.rowk[row];
  if (k < 0) return;
  size_t j = a.base + (size_t)cid * a.nrows + k;
  int sd = a.sid[sidx + 1];
  int asd = abs(sd);
  int mdid = a.md[asd], sdid = a.sd[asd];
  int nl = a.etype[asd] ? 4 : 3;
  const cplx* g = a.G + (size_t)row * N + (size_t)sidx * 4;
  const cplx* h = a.H + (size_t)row * N + (size_t)sidx * 4;
  cplx* Aj = a.A + j * a.na;
  const size_t nn = a.nn;
  if (a.did == mdid) {
    for (int l = 0; l < nl; l++) {
      size_t c = (size_t)a.eni[asd * 4 + l];
      Aj[nn * (cid + 0) + c] = h[l];
      Aj[nn * (cid + 4) + c] = -g[l];
    }
    return;
  }
  cplx k1 = cmk(a.kn[2 * mdid], a.kn[2 * mdid + 1]);
  cplx k2 = cmk(a.kn[2 * sdid], a.kn[2 * sdid + 1]);
  cplx k12 = k1 * k1, k22 = k2 * k2;
  cplx delt = k12 - k22;
  cplx beps = cdivc(k12, k22);
  cplx sigm = cmk(1.0, 0.0) - beps;
  for (int l = 0; l < nl; l++) {
    size_t c = (size_t)a.eni[asd * 4 + l];
    double vn[3];
    for (int d = 0; d < 3; d++) vn[d] = a.wen[(size_t)asd * 12 + l * 3 + d];
    double an = sqrt(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
    if (an != 0.0) { vn[0] /= an; vn[1] /= an; vn[2] /= an; }
    if (cid < 3) {
      Aj[nn * (cid + 0) + c] = h[l];
      Aj[nn * 3 + c] = (delt * vn[cid]) * g[l];
      Aj[nn * (cid + 4) + c] = g[l];
    } else {
      Aj[nn * 0 + c] = (sigm * vn[0]) * g[l];
      Aj[nn * 1 + c] = (sigm * vn[1]) * g[l];
      Aj[nn * 2 + c] = (sigm * vn[2]) * g[l];
      Aj[nn * 3 + c] = h[l];
      Aj[nn * 7 + c] = beps * g[l];
    }
  }
}

extern "C" int gbi_build_A_domain(const cplx* G, const cplx* H, const int* sid, const int* rowk, const GbMeshDev* m,
                                  const double* kn_dev, int did, int nrows, size_t base, size_t na, cplx* A,
                                  cudaStream_t st) {
  ABuildArgs a;
  a.G = G; a.H = H; a.sid = sid; a.rowk = rowk;
  a.eni = m->eni; a.md = m->md; a.sd = m->sd; a.etype = m->etype; a.wen = m->wen; a.kn = kn_dev;
  a.Ne = m->sb_Ne[did]; a.did = did; a.nrows = nrows; a.base = base; a.nn = (size_t)m->NN; a.na = na; a.A = A;
  size_t tot = 16 * (size_t)a.Ne * a.Ne;
  if (tot == 0) return 0;
  k_build_A<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// A built directly in complex FP32 (chosen form: the FP32 factors start from
// it; no FP64 copy of A is kept)
__global__ void k_build_A32(ABuildArgs a, cplxf* A32) {
  size_t N = (size_t)a.Ne * 4;
  size_t tot = 4 * N * (size_t)a.Ne;
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= tot) return;
  int sidx = (int)(p % a.Ne);
  size_t q = p / a.Ne;
  int row = (int)(q % N);
  int cid = (int)(q / N);
  int k = a.rowk[row];
  if (k < 0) return;
  size_t j = a.base + (size_t)cid * a.nrows + k;
  int sd = a.sid[sidx + 1];
  int asd = abs(sd);
  int mdid = a.md[asd], sdid = a.sd[asd];
  int nl = a.etype[asd] ? 4 : 3;
  const cplx* g = a.G + (size_t)row * N + (size_t)sidx * 4;
  const cplx* h = a.H + (size_t)row * N + (size_t)sidx * 4;
  cplxf* Aj = A32 + j * a.na;
  const size_t nn = a.nn;
  if (a.did == mdid) {
    for (int l = 0; l < nl; l++) {
      size_t c = (size_t)a.eni[asd * 4 + l];
      Aj[nn * (cid + 0) + c] = to_c64f(h[l]);
      Aj[nn * (cid + 4) + c] = to_c64f(-g[l]);
    }
    return;
  }
  cplx k1 = cmk(a.kn[2 * mdid], a.kn[2 * mdid + 1]);
  cplx k2 = cmk(a.kn[2 * sdid], a.kn[2 * sdid + 1]);
  cplx k12 = k1 * k1, k22 = k2 * k2;
  cplx delt = k12 - k22;
  cplx beps = cdivc(k12, k22);
  cplx sigm = cmk(1.0, 0.0) - beps;
  for (int l = 0; l < nl; l++) {
    size_t c = (size_t)a.eni[asd * 4 + l];
    double vn[3];
    for (int d = 0; d < 3; d++) vn[d] = a.wen[(size_t)asd * 12 + l * 3 + d];
    double an = sqrt(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
    if (an != 0.0) { vn[0] /= an; vn[1] /= an; vn[2] /= an; }
    if (cid < 3) {
      Aj[nn * (cid + 0) + c] = to_c64f(h[l]);
      Aj[nn * 3 + c] = to_c64f((delt * vn[cid]) * g[l]);
      Aj[nn * (cid + 4) + c] = to_c64f(g[l]);
    } else {
      Aj[nn * 0 + c] = to_c64f((sigm * vn[0]) * g[l]);
      Aj[nn * 1 + c] = to_c64f((sigm * vn[1]) * g[l]);
      Aj[nn * 2 + c] = to_c64f((sigm * vn[2]) * g[l]);
      Aj[nn * 3 + c] = to_c64f(h[l]);
      Aj[nn * 7 + c] = to_c64f(beps * g[l]);
    }
  }
}

extern "C" int gbi_build_A32_domain(const cplx* G, const cplx* H, const int* sid, const int* rowk, const GbMeshDev* m,
                                    const double* kn_dev, int did, int nrows, size_t base, size_t na, cplxf* A32,
                                    cudaStream_t st) {
  ABuildArgs a;
  a.G = G; a.H = H; a.sid = sid; a.rowk = rowk;
  a.eni = m->eni; a.md = m->md; a.sd = m->sd; a.etype = m->etype; a.wen = m->wen; a.kn = kn_dev;
  a.Ne = m->sb_Ne[did]; a.did = did; a.nrows = nrows; a.base = base; a.nn = (size_t)m->NN; a.na = na; a.A = nullptr;
  size_t tot = 16 * (size_t)a.Ne * a.Ne;
  if (tot == 0) return 0;
  k_build_A32<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(a, A32);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---- y = A x without forming A (FP64), for the refinement residual.
// Row (domain d, collocation row, block cid) of A holds, for each column
// (source element s, node l), h_l at x-component cid and g_l-terms at other
// components (the coupling rules of k_build_A).  Per column they collapse to
// two numbers per cid, P_cid (multiplies H) and Q_cid (multiplies G), so the
// four rows of a collocation node are H P + G Q: one pass over G and H with
// four right-hand sides.
struct PQArgs {
  const int* sid;
  const int* eni;
  const int* md;
  const int* sd;
  const int* etype;
  const double* wen;
  const double* kn;
  int Ne, did;
  size_t nn;
  const cplx* x;
  cplx* PQ;  // [8][N]: P_0..P_3, Q_0..Q_3
};

__global__ void k_pq_gather(PQArgs a) {
  const size_t N = (size_t)a.Ne * 4;
  size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= N) return;
  int sidx = (int)(col / 4), l = (int)(col % 4);
  int asd = abs(a.sid[sidx + 1]);
  int nl = a.etype[asd] ? 4 : 3;
  cplx P[4], Q[4];
  for (int c = 0; c < 4; c++) { P[c] = cmk(0, 0); Q[c] = cmk(0, 0); }
  if (l < nl) {
    size_t c = (size_t)a.eni[asd * 4 + l];
    cplx xv[8];
    for (int q = 0; q < 8; q++) xv[q] = a.x[a.nn * q + c];
    int mdid = a.md[asd], sdid = a.sd[asd];
    if (a.did == mdid) {
      for (int q = 0; q < 4; q++) { P[q] = xv[q]; Q[q] = -xv[q + 4]; }
    } else {
      cplx k1 = cmk(a.kn[2 * mdid], a.kn[2 * mdid + 1]);
      cplx k2 = cmk(a.kn[2 * sdid], a.kn[2 * sdid + 1]);
      cplx k12 = k1 * k1, k22 = k2 * k2;
      cplx delt = k12 - k22;
      cplx beps = cdivc(k12, k22);
      cplx sigm = cmk(1.0, 0.0) - beps;
      double vn[3];
      for (int d = 0; d < 3; d++) vn[d] = a.wen[(size_t)asd * 12 + l * 3 + d];
      double an = sqrt(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
      if (an != 0.0) { vn[0] /= an; vn[1] /= an; vn[2] /= an; }
      for (int q = 0; q < 3; q++) { P[q] = xv[q]; Q[q] = (delt * vn[q]) * xv[3] + xv[q + 4]; }
      P[3] = xv[3];
      Q[3] = sigm * (xv[0] * vn[0] + xv[1] * vn[1] + xv[2] * vn[2]) + beps * xv[7];
    }
  }
  for (int q = 0; q < 4; q++) { a.PQ[(size_t)q * N + col] = P[q]; a.PQ[(size_t)(4 + q) * N + col] = Q[q]; }
}

// one warp per collocation row: y[base + cid nrows + k] = (H P_cid + G Q_cid)[row]
__global__ void k_apply_rows(const cplx* __restrict__ G, const cplx* __restrict__ H, const int* rowk, int Ne, int nrows,
                             size_t base, const cplx* __restrict__ PQ, cplx* y) {
  const int lane = threadIdx.x & 31;
  const size_t N = (size_t)Ne * 4;
  size_t row = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (row >= N) return;
  int k = rowk[row];
  if (k < 0) return;
  const cplx* g = G + row * N;
  const cplx* h = H + row * N;
  double acc[8];
  for (int i = 0; i < 8; i++) acc[i] = 0.0;
  for (size_t c = lane; c < N; c += 32) {
    cplx gv = g[c], hv = h[c];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      cplx p = PQ[(size_t)q * N + c], qq = PQ[(size_t)(4 + q) * N + c];
      acc[2 * q] = fma(hv.x, p.x, acc[2 * q]);
      acc[2 * q] = fma(-hv.y, p.y, acc[2 * q]);
      acc[2 * q] = fma(gv.x, qq.x, acc[2 * q]);
      acc[2 * q] = fma(-gv.y, qq.y, acc[2 * q]);
      acc[2 * q + 1] = fma(hv.x, p.y, acc[2 * q + 1]);
      acc[2 * q + 1] = fma(hv.y, p.x, acc[2 * q + 1]);
      acc[2 * q + 1] = fma(gv.x, qq.y, acc[2 * q + 1]);
      acc[2 * q + 1] = fma(gv.y, qq.x, acc[2 * q + 1]);
    }
  }
  for (int i = 0; i < 8; i++)
    for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
  if (lane == 0)
    for (int q = 0; q < 4; q++) y[base + (size_t)q * nrows + k] = cmk(acc[2 * q], acc[2 * q + 1]);
}

// complex FP64 to double-float (float4: re.hi, re.lo, im.hi, im.lo)
__global__ void k_to_df(size_t n, const cplx* __restrict__ src, float4* dst) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cplx v = src[i];
  const float a = (float)v.x, b = (float)v.y;
  dst[i] = make_float4(a, (float)(v.x - (double)a), b, (float)(v.y - (double)b));
}

extern "C" int gbi_to_df(size_t n, const cplx* src, void* dst, cudaStream_t st) {
  if (n == 0) return 0;
  k_to_df<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, src, (float4*)dst);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

__device__ __forceinline__ dfc dfc_ld4(const float4 f) { return dfcmk(dfmk(f.x, f.y), dfmk(f.z, f.w)); }
// acc + a b, complex double-float, for accumulators read only through
// df_to (compensated steps, df_acc)
__device__ __forceinline__ dfc dfc_mac(dfc acc, dfc a, dfc b) {
  dfc r;
  r.re = df_acc(df_acc(acc.re, a.re, b.re), df_neg(a.im), b.im);
  r.im = df_acc(df_acc(acc.im, a.re, b.im), a.im, b.re);
  return r;
}

// k_apply_rows with the matrices and node vectors in double-float: the
// products of the GMRES iterations on the FP32 pipes (the FP64 version is
// bound by the DFMA rate); sums finished in FP64.  Two rows per warp: each
// node-vector load serves both rows (half the L1 traffic per product) and
// the two rows' sums are independent chains; the next column's matrix
// entries are loaded before this column's products (the loop was bound by
// load latency).  Each lane sums its columns in order and the warp reduces
// the lanes in a fixed pattern.
__global__ void __launch_bounds__(128) k_apply_rows_df2(const float4* __restrict__ G, const float4* __restrict__ H,
                                                        const int* rowk, int Ne, int nrows, size_t base,
                                                        const float4* __restrict__ PQ, cplx* y) {
  const int lane = threadIdx.x & 31;
  const size_t N = (size_t)Ne * 4;
  const size_t r0 = (((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2;
  if (r0 >= N) return;
  const bool two = r0 + 1 < N;
  const int k0 = rowk[r0], k1 = two ? rowk[r0 + 1] : -1;
  if (k0 < 0 && k1 < 0) return;
  const size_t r1 = two ? r0 + 1 : r0;
  const float4* g0 = G + r0 * N;
  const float4* h0 = H + r0 * N;
  const float4* g1 = G + r1 * N;
  const float4* h1 = H + r1 * N;
  const df z = dfmk(0.0f, 0.0f);
  dfc a0[4], a1[4];
#pragma unroll
  for (int q = 0; q < 4; q++) { a0[q] = dfcmk(z, z); a1[q] = dfcmk(z, z); }
  const float4 f0 = make_float4(0.f, 0.f, 0.f, 0.f);
  float4 gn0 = f0, hn0 = f0, gn1 = f0, hn1 = f0;
  if ((size_t)lane < N) { gn0 = g0[lane]; hn0 = h0[lane]; gn1 = g1[lane]; hn1 = h1[lane]; }
  for (size_t c = lane; c < N; c += 32) {
    const dfc gv0 = dfc_ld4(gn0), hv0 = dfc_ld4(hn0), gv1 = dfc_ld4(gn1), hv1 = dfc_ld4(hn1);
    float4 v[8];
#pragma unroll
    for (int q = 0; q < 8; q++) v[q] = PQ[(size_t)q * N + c];
    const size_t cn = c + 32;
    if (cn < N) { gn0 = g0[cn]; hn0 = h0[cn]; gn1 = g1[cn]; hn1 = h1[cn]; }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const dfc p = dfc_ld4(v[q]), qq = dfc_ld4(v[4 + q]);
      a0[q] = dfc_mac(dfc_mac(a0[q], hv0, p), gv0, qq);
      a1[q] = dfc_mac(dfc_mac(a1[q], hv1, p), gv1, qq);
    }
  }
  double s[16];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    s[2 * q] = df_to(a0[q].re); s[2 * q + 1] = df_to(a0[q].im);
    s[8 + 2 * q] = df_to(a1[q].re); s[9 + 2 * q] = df_to(a1[q].im);
  }
  for (int i = 0; i < 16; i++)
    for (int o = 16; o > 0; o >>= 1) s[i] += __shfl_down_sync(0xffffffffu, s[i], o);
  if (lane != 0) return;
  if (k0 >= 0)
    for (int q = 0; q < 4; q++) y[base + (size_t)q * nrows + k0] = cmk(s[2 * q], s[2 * q + 1]);
  if (k1 >= 0)
    for (int q = 0; q < 4; q++) y[base + (size_t)q * nrows + k1] = cmk(s[8 + 2 * q], s[9 + 2 * q]);
}

extern "C" int gbi_apply_A_domain_df(const void* Gd, const void* Hd, const int* sid, const int* rowk,
                                     const GbMeshDev* m, const double* kn_dev, int did, int nrows, size_t base,
                                     const cplx* x, cplx* PQ, void* PQd, cplx* y, cudaStream_t st) {
  const int Ne = m->sb_Ne[did];
  const size_t N = (size_t)Ne * 4;
  if (N == 0) return 0;
  PQArgs a;
  a.sid = sid; a.eni = m->eni; a.md = m->md; a.sd = m->sd; a.etype = m->etype; a.wen = m->wen; a.kn = kn_dev;
  a.Ne = Ne; a.did = did; a.nn = (size_t)m->NN; a.x = x; a.PQ = PQ;
  k_pq_gather<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(a);
  gbi_count_launch();
  k_to_df<<<(unsigned)((8 * N + 255) / 256), 256, 0, st>>>(8 * N, PQ, (float4*)PQd);
  gbi_count_launch();
  k_apply_rows_df2<<<(unsigned)(((N + 1) / 2 * 32 + 127) / 128), 128, 0, st>>>((const float4*)Gd, (const float4*)Hd, rowk,
                                                                                Ne, nrows, base, (const float4*)PQd, y);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// y rows of H P + G Q for a gathered PQ [8][N]: FP64, or with Gd, Hd
// (double-float copies of G, H) on the FP32 pipes (PQd: scratch of 8 N float4)
extern "C" int gbi_rows_apply(const cplx* G, const cplx* H, const void* Gd, const void* Hd, const int* rowk, int Ne,
                              int nrows, size_t base, cplx* PQ, void* PQd, cplx* y, cudaStream_t st) {
  const size_t N = (size_t)Ne * 4;
  if (N == 0) return 0;
  if (Gd && Hd) {
    k_to_df<<<(unsigned)((8 * N + 255) / 256), 256, 0, st>>>(8 * N, PQ, (float4*)PQd);
    gbi_count_launch();
    k_apply_rows_df2<<<(unsigned)(((N + 1) / 2 * 32 + 127) / 128), 128, 0, st>>>((const float4*)Gd, (const float4*)Hd,
                                                                                  rowk, Ne, nrows, base,
                                                                                  (const float4*)PQd, y);
  } else {
    k_apply_rows<<<(unsigned)((N * 32 + 255) / 256), 256, 0, st>>>(G, H, rowk, Ne, nrows, base, PQ, y);
  }
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbi_apply_A_domain(const cplx* G, const cplx* H, const int* sid, const int* rowk, const GbMeshDev* m,
                                  const double* kn_dev, int did, int nrows, size_t base, const cplx* x, cplx* PQ, cplx* y,
                                  cudaStream_t st) {
  const int Ne = m->sb_Ne[did];
  const size_t N = (size_t)Ne * 4;
  if (N == 0) return 0;
  PQArgs a;
  a.sid = sid; a.eni = m->eni; a.md = m->md; a.sd = m->sd; a.etype = m->etype; a.wen = m->wen; a.kn = kn_dev;
  a.Ne = Ne; a.did = did; a.nn = (size_t)m->NN; a.x = x; a.PQ = PQ;
  k_pq_gather<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(a);
  gbi_count_launch();
  k_apply_rows<<<(unsigned)((N * 32 + 255) / 256), 256, 0, st>>>(G, H, rowk, Ne, nrows, base, PQ, y);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// r = b - y and the squared norms of r and b accumulated into nrm[0], nrm[1]
__global__ void k_resid_finish(const cplx* b, const cplx* y, cplx* r, size_t n, double* nrm) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double rr = 0.0, bb = 0.0;
  if (i < n) {
    cplx t = cmk(b[i].x - y[i].x, b[i].y - y[i].y);
    r[i] = t;
    rr = t.x * t.x + t.y * t.y;
    bb = b[i].x * b[i].x + b[i].y * b[i].y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_down_sync(0xffffffffu, rr, o);
    bb += __shfl_down_sync(0xffffffffu, bb, o);
  }
  if ((threadIdx.x & 31) == 0) { atomicAdd(nrm, rr); atomicAdd(nrm + 1, bb); }
}
extern "C" int gbi_resid_finish(const cplx* b, const cplx* y, cplx* r, size_t n, double* nrm, cudaStream_t st) {
  GB_CUDA(cudaMemsetAsync(nrm, 0, 2 * sizeof(double), st));
  k_resid_finish<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(b, y, r, n, nrm);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------ LU
__device__ __forceinline__ double cabs1(cplx a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ float cabs1(cplxf a) { return fabsf(a.x) + fabsf(a.y); }

// real type of a complex element type (sums of FP32 solves stay in FP32: a
// GB300 SM has a narrow FP64 pipe, and the FP64 refinement corrects them)
template <class T> struct RealOf { typedef double type; };
template <> struct RealOf<cplxf> { typedef float type; };

// Rows k..k+nb-1 (nb <= LU_NB), columns [c0, c1): X <- L11^-1 X with L11 the
// unit lower triangle of A[k:k+nb][k:k+nb] (or, with UPPER = 1, X <- U11^-1 X
// with the non-unit upper triangle).  Lsrc gives the triangle's storage
// (row-major, leading dimension ldl).  A block takes 32 columns: the triangle
// is staged transposed in shared memory (with the inverted diagonal), the
// nb x 32 tile of X is loaded and stored coalesced, and each warp solves four
// columns with the column in registers (lane l: rows l and l + 32) by
// substitution with warp shuffles.
#define TRSM_COLS 32
template <class T, int UPPER>
__global__ void __launch_bounds__(256) k_trsm_rows(const T* Lsrc, size_t ldl, T* X, size_t ldx, int nb, int c0,
                                                   int c1) {
  extern __shared__ __align__(16) unsigned char sLraw[];
  // lower: the strictly lower triangle zero-padded to LU_NB x LU_NB (no
  // predicates in the substitution); upper: the nb x nb triangle
  const int ld = UPPER ? nb + 1 : LU_NB + 1;
  T* sT = (T*)sLraw;           // sT[j * ld + i] = triangle[i][j]
  T* dinv = sT + (UPPER ? nb : LU_NB) * ld;  // LU_NB
  T* Xs = dinv + LU_NB;        // LU_NB x (TRSM_COLS + 1)
  constexpr int XL = TRSM_COLS + 1;
  if (UPPER) {
    for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
      int i = t / nb, j = t % nb;
      sT[j * ld + i] = Lsrc[(size_t)i * ldl + j];
    }
  } else {
    for (int t = threadIdx.x; t < LU_NB * LU_NB; t += blockDim.x) {
      const int i = t / LU_NB, j = t % LU_NB;
      T v;
      v.x = 0;
      v.y = 0;
      if (i > j && i < nb) v = Lsrc[(size_t)i * ldl + j];
      sT[j * ld + i] = v;
    }
  }
  const int cb = c0 + blockIdx.x * TRSM_COLS;
  for (int t = threadIdx.x; t < nb * TRSM_COLS; t += blockDim.x) {
    int i = t / TRSM_COLS, c = t % TRSM_COLS;
    if (cb + c < c1) Xs[i * XL + c] = X[(size_t)i * ldx + cb + c];
  }
  __syncthreads();
  if (UPPER)
    for (int j = threadIdx.x; j < nb; j += blockDim.x) {
      T one;
      one.x = 1; one.y = 0;
      dinv[j] = cdivc(one, sT[j * ld + j]);
    }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int i0 = lane, i1 = lane + 32;
  if (!UPPER) {
    // two columns per warp (two independent chains); the second half of the
    // steps touches only rows 32..63
    for (int c = w; c < TRSM_COLS; c += 2 * nw) {
      const int cB = c + nw;
      if (cb + c >= c1) break;  // warp-uniform
      const bool okB = cB < TRSM_COLS && cb + cB < c1;
      T zero;
      zero.x = 0;
      zero.y = 0;
      T xa0 = i0 < nb ? Xs[i0 * XL + c] : zero, xa1 = i1 < nb ? Xs[i1 * XL + c] : zero;
      T xb0 = (okB && i0 < nb) ? Xs[i0 * XL + cB] : zero, xb1 = (okB && i1 < nb) ? Xs[i1 * XL + cB] : zero;
#pragma unroll 8
      for (int j = 0; j < 32; j++) {
        T va, vb;
        va.x = __shfl_sync(0xffffffffu, xa0.x, j);
        va.y = __shfl_sync(0xffffffffu, xa0.y, j);
        vb.x = __shfl_sync(0xffffffffu, xb0.x, j);
        vb.y = __shfl_sync(0xffffffffu, xb0.y, j);
        const T l0 = sT[j * ld + i0], l1 = sT[j * ld + i1];
        xa0 -= l0 * va;
        xa1 -= l1 * va;
        xb0 -= l0 * vb;
        xb1 -= l1 * vb;
      }
#pragma unroll 8
      for (int j = 32; j < LU_NB; j++) {
        T va, vb;
        va.x = __shfl_sync(0xffffffffu, xa1.x, j - 32);
        va.y = __shfl_sync(0xffffffffu, xa1.y, j - 32);
        vb.x = __shfl_sync(0xffffffffu, xb1.x, j - 32);
        vb.y = __shfl_sync(0xffffffffu, xb1.y, j - 32);
        const T l1 = sT[j * ld + i1];
        xa1 -= l1 * va;
        xb1 -= l1 * vb;
      }
      if (i0 < nb) Xs[i0 * XL + c] = xa0;
      if (i1 < nb) Xs[i1 * XL + c] = xa1;
      if (okB && i0 < nb) Xs[i0 * XL + cB] = xb0;
      if (okB && i1 < nb) Xs[i1 * XL + cB] = xb1;
    }
  }
  for (int c = w; c < TRSM_COLS && UPPER; c += nw) {
    if (cb + c >= c1) break;  // warp-uniform
    T x0, x1;
    x0.x = 0; x0.y = 0; x1 = x0;
    if (i0 < nb) x0 = Xs[i0 * XL + c];
    if (i1 < nb) x1 = Xs[i1 * XL + c];
    if (!UPPER) {
      for (int j = 0; j < nb; j++) {
        T v = (j < 32) ? x0 : x1;
        T xj;
        xj.x = __shfl_sync(0xffffffffu, v.x, j & 31);
        xj.y = __shfl_sync(0xffffffffu, v.y, j & 31);
        const T* col = sT + j * ld;
        if (i0 > j && i0 < nb) x0 -= col[i0] * xj;
        if (i1 > j && i1 < nb) x1 -= col[i1] * xj;
      }
    } else {
      for (int j = nb - 1; j >= 0; j--) {
        T v = (j < 32) ? x0 : x1;
        T xj;
        xj.x = __shfl_sync(0xffffffffu, v.x, j & 31);
        xj.y = __shfl_sync(0xffffffffu, v.y, j & 31);
        xj = xj * dinv[j];
        if (lane == (j & 31)) { if (j < 32) x0 = xj; else x1 = xj; }
        const T* col = sT + j * ld;
        if (i0 < j) x0 -= col[i0] * xj;
        if (i1 < j) x1 -= col[i1] * xj;
      }
    }
    if (i0 < nb) Xs[i0 * XL + c] = x0;
    if (i1 < nb) Xs[i1 * XL + c] = x1;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nb * TRSM_COLS; t += blockDim.x) {
    int i = t / TRSM_COLS, c = t % TRSM_COLS;
    if (cb + c < c1) X[(size_t)i * ldx + cb + c] = Xs[i * XL + c];
  }
}

// C[M][N] -= A[M][K] B[K][N], complex FP64, row-major with leading dims.
// 64x64 output tile per 256-thread block, each thread a 4x4 complex sub-tile,
// K staged through shared memory in slices of 16.
#define GT_BM 64
#define GT_BN 64
#define GT_BK 16
__global__ void __launch_bounds__(256) k_zgemm_nn(int M, int N, int K, const cplx* __restrict__ A, size_t lda,
                                                  const cplx* __restrict__ B, size_t ldb, cplx* C, size_t ldc) {
  __shared__ cplx As[GT_BK][GT_BM];
  __shared__ cplx Bs[GT_BK][GT_BN];
  int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  int m0 = blockIdx.y * GT_BM, n0 = blockIdx.x * GT_BN;
  double accr[4][4], acci[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) { accr[i][j] = 0.0; acci[i][j] = 0.0; }
  for (int k0 = 0; k0 < K; k0 += GT_BK) {
    for (int t = threadIdx.x; t < GT_BK * GT_BM; t += 256) {
      int kk = t % GT_BK, mm = t / GT_BK;
      int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(size_t)gm * lda + gk] : cmk(0, 0);
    }
    for (int t = threadIdx.x; t < GT_BK * GT_BN; t += 256) {
      int nn = t % GT_BN, kk = t / GT_BN;
      int gn = n0 + nn, gk = k0 + kk;
      Bs[kk][nn] = (gn < N && gk < K) ? B[(size_t)gk * ldb + gn] : cmk(0, 0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GT_BK; kk++) {
      cplx a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
          accr[i][j] = fma(a[i].x, b[j].x, accr[i][j]);
          accr[i][j] = fma(-a[i].y, b[j].y, accr[i][j]);
          acci[i][j] = fma(a[i].x, b[j].y, acci[i][j]);
          acci[i][j] = fma(a[i].y, b[j].x, acci[i][j]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      cplx* c = C + (size_t)gm * ldc + gn;
      c->x -= accr[i][j];
      c->y -= acci[i][j];
    }
  }
}

static int gemm_sub(int M, int N, int K, const cplx* A, size_t lda, const cplx* B, size_t ldb, cplx* C, size_t ldc,
                    cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  dim3 grid((N + GT_BN - 1) / GT_BN, (M + GT_BM - 1) / GT_BM);
  k_zgemm_nn<<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

template <class T>
static int trsm_rows(int upper, const T* L, size_t ldl, T* X, size_t ldx, int nb, int c0, int c1, cudaStream_t st) {
  if (c1 <= c0) return 0;
  const size_t tri = upper ? (size_t)nb * (nb + 1) : (size_t)LU_NB * (LU_NB + 1);
  size_t sm = (tri + LU_NB + (size_t)LU_NB * (TRSM_COLS + 1)) * sizeof(T);
  // the function attribute is process-wide and host threads factorise
  // objects at once: it is always set to the largest request (nb = LU_NB),
  // never to this call's, so that no thread lowers it under another's launch
  const int sm_max = (int)(((size_t)LU_NB * (LU_NB + 1) + LU_NB + (size_t)LU_NB * (TRSM_COLS + 1)) * sizeof(T));
  unsigned nblk = (unsigned)((c1 - c0 + TRSM_COLS - 1) / TRSM_COLS);
  if (upper) {
    GB_CUDA(cudaFuncSetAttribute(k_trsm_rows<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_max));
    k_trsm_rows<T, 1><<<nblk, 256, sm, st>>>(L, ldl, X, ldx, nb, c0, c1);
    gbi_count_launch();
  } else {
    GB_CUDA(cudaFuncSetAttribute(k_trsm_rows<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_max));
    k_trsm_rows<T, 0><<<nblk, 256, sm, st>>>(L, ldl, X, ldx, nb, c0, c1);
    gbi_count_launch();
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---- tournament-pivoting panel (CALU)
#define TS_ARITY 4                   // candidate sets merged per tree node
#define TS_ROWS (TS_ARITY * LU_NB)   // rows of a leaf set and of a merge
#define TS_THREADS 1024              // elimination blocks: 32 warps, 8 rows each
#define PANEL_THREADS 256
#define DIAG_THREADS 1024            // k_diag_lu: 32 warps, two rows of the block each

__device__ __forceinline__ cplxf to_c64(cplx a) { return cmkf((float)a.x, (float)a.y); }
__device__ __forceinline__ cplxf to_c64(cplxf a) { return a; }

// Partial-pivoting elimination of the R <= TS_ROWS panel rows idx[0..R) of A
// (columns k..k+nb-1, nb <= LU_NB): only the choice of rows is kept -- on
// return win[0..min(R, nb)) holds the selected rows (global indices) in pivot
// order.  The selection runs in complex FP32 for both LU types: it only ranks
// candidate rows, and a block's FP64 pipe is too narrow for it (the FP64
// factors themselves are computed in FP64 by k_diag_lu / k_trsm_right).
// The rows live in registers: warp w holds rows w + 32 i (i < TS_ROWS / 32),
// lane l columns l and l + 32.  Rows are never moved: a chosen pivot row is
// retired from its warp's active mask (the interchange of partial pivoting
// only reorders, and the order is kept in win[]).  Per column: a block
// reduction for the pivot (one REDUX per warp on a 32-bit key), the pivot row
// and its reciprocal published through shared memory by its owner warp, and a
// register-only rank-1 update of the active rows that also ranks the next
// column; two block barriers.
template <class T>
__device__ void ts_select(const T* A, size_t lda, int k, int nb, const int* idx, int R, int* win) {
  constexpr int NW = TS_THREADS / 32;
  constexpr int RPW = TS_ROWS / NW;  // rows per warp
  static_assert(TS_ROWS <= 256, "pivot keys hold 9-bit row numbers");
  __shared__ uint32_t skey[NW];
  __shared__ cplxf sP[LU_NB];
  __shared__ cplxf sPinv;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int c0 = lane, c1 = lane + 32;
  const cplxf z = cmkf(0.f, 0.f);
  cplxf v0[RPW], v1[RPW];
  uint32_t active = 0u;  // warp-uniform: bit i = row w + NW i still a candidate
#pragma unroll
  for (int i = 0; i < RPW; i++) {
    const int r = w + NW * i;
    v0[i] = z;
    v1[i] = z;
    if (r < R) {
      active |= 1u << i;
      const T* src = A + (size_t)idx[r] * lda + k;
      if (c0 < nb) v0[i] = to_c64(src[c0]);
      if (c1 < nb) v1[i] = to_c64(src[c1]);
    }
  }
  // pivot keys: |Re|+|Im| with its 9 low mantissa bits replaced by 511 - row,
  // so one unsigned maximum picks the largest magnitude and, among magnitudes
  // within 2^-14 relative, the first row (any of them is as good a pivot);
  // every active row has a non-zero key, so a zero column still yields a row
  const int steps = R < nb ? R : nb;
  uint32_t key = 0u;
  if (lane == 0) {  // column 0
#pragma unroll
    for (int i = 0; i < RPW; i++)
      if ((active >> i) & 1u) key = max(key, (__float_as_uint(cabs1(v0[i])) & ~0x1FFu) | (uint32_t)(511 - (w + NW * i)));
  }
  for (int j = 0; j < steps; j++) {
    key = __reduce_max_sync(0xffffffffu, key);
    if (lane == 0) skey[w] = key;
    __syncthreads();
    key = __reduce_max_sync(0xffffffffu, lane < NW ? skey[lane] : 0u);
    const int p = 511 - (int)(key & 0x1FFu);
    // the owner warp publishes the pivot row and its reciprocal and retires it
    // (register slots are picked with bit masks: an indexed access, or a select
    // chain the compiler turns into one, would move the row arrays to local
    // memory)
    if (w == (p % NW)) {
      uint32_t t[4] = {0u, 0u, 0u, 0u};
#pragma unroll
      for (int i = 0; i < RPW; i++) {
        const uint32_t msk = 0u - (uint32_t)(i == p / NW);
        t[0] |= __float_as_uint(v0[i].x) & msk; t[1] |= __float_as_uint(v0[i].y) & msk;
        t[2] |= __float_as_uint(v1[i].x) & msk; t[3] |= __float_as_uint(v1[i].y) & msk;
      }
      const cplxf q0 = cmkf(__uint_as_float(t[0]), __uint_as_float(t[1]));
      const cplxf q1 = cmkf(__uint_as_float(t[2]), __uint_as_float(t[3]));
      sP[c0] = q0;
      sP[c1] = q1;
      if (lane == (j & 31)) {
        const cplxf piv = (j < 32) ? q0 : q1;
        sPinv = (piv.x == 0.f && piv.y == 0.f) ? z : cdivc(cmkf(1.f, 0.f), piv);
      }
      active &= ~(1u << (p / NW));
      if (lane == 0) win[j] = idx[p];
    }
    __syncthreads();
    const cplxf pinv = sPinv;
    const int cn = j + 1;
    const bool own_next = lane == (cn & 31) && cn < nb;
    key = 0u;
    if (j < 31) {  // both column halves still have entries to the right of j
      const cplxf p0 = (c0 > j && c0 < nb) ? sP[c0] : z;
      const cplxf p1 = (c1 < nb) ? sP[c1] : z;
#pragma unroll
      for (int i = 0; i < RPW; i++) {
        if (!((active >> i) & 1u)) continue;  // warp-uniform
        cplxf l;
        l.x = __shfl_sync(0xffffffffu, v0[i].x, j);
        l.y = __shfl_sync(0xffffffffu, v0[i].y, j);
        l = l * pinv;
        v0[i] -= l * p0;
        v1[i] -= l * p1;
        if (own_next)
          key = max(key, (__float_as_uint(cabs1(cn < 32 ? v0[i] : v1[i])) & ~0x1FFu) | (uint32_t)(511 - (w + NW * i)));
      }
    } else {  // only the upper half (columns 32..63) is still to the right of j
      const cplxf p1 = (c1 > j && c1 < nb) ? sP[c1] : z;
      const int src = (j < 32) ? j : j - 32;
#pragma unroll
      for (int i = 0; i < RPW; i++) {
        if (!((active >> i) & 1u)) continue;  // warp-uniform
        const cplxf xv = (j < 32) ? v0[i] : v1[i];
        cplxf l;
        l.x = __shfl_sync(0xffffffffu, xv.x, src);
        l.y = __shfl_sync(0xffffffffu, xv.y, src);
        l = l * pinv;
        v1[i] -= l * p1;
        if (own_next) key = max(key, (__float_as_uint(cabs1(v1[i])) & ~0x1FFu) | (uint32_t)(511 - (w + NW * i)));
      }
    }
    // the next step's reductions start only after every thread passed the
    // barrier above, and its first barrier orders these updates before use
  }
  __syncthreads();
}

// the winners idx[0..nb) (global rows, pivot order) as LAPACK-style
// interchanges: ipiv[k + j] = the row swapped with row k + j when the swaps
// are applied in sequence.  Only rows of the block [k, k + nb) can move
// before their turn, so two small tables suffice: where[] (current position
// of each row of the block) and cont[] (current row at each block position).
// One thread; where/cont: nb ints of shared memory each.
__device__ void calu_ipiv(const int* win, int k, int nb, int64_t* ipiv, int* where, int* cont) {
  for (int i = 0; i < nb; i++) { where[i] = k + i; cont[i] = k + i; }
  for (int j = 0; j < nb; j++) {
    const int wr = win[j];
    const bool win_in = wr >= k && wr < k + nb;
    const int pos = win_in ? where[wr - k] : wr;
    ipiv[k + j] = pos;
    const int c = cont[j];  // a row of the block
    cont[j] = wr;
    if (win_in) where[wr - k] = k + j;
    if (pos >= k && pos < k + nb) cont[pos - k] = c;
    where[c - k] = pos;
  }
}

// one block per set of TS_ROWS rows of the panel: nb candidate rows (and the
// interchanges, when the panel has a single set)
template <class T>
__global__ void __launch_bounds__(TS_THREADS) k_tslu_leaf(const T* A, size_t lda, int n, int k, int nb, int* cand,
                                                         int64_t* ipiv) {
  __shared__ int idx[TS_ROWS + 2 * LU_NB];
  const int r0 = k + blockIdx.x * TS_ROWS;
  const int R = (n - r0 < TS_ROWS) ? n - r0 : TS_ROWS;
  __shared__ int win[LU_NB];
  for (int r = threadIdx.x; r < R; r += TS_THREADS) idx[r] = r0 + r;
  __syncthreads();
  ts_select<T>(A, lda, k, nb, idx, R, win);
  const int steps = R < nb ? R : nb;
  for (int j = threadIdx.x; j < nb; j += TS_THREADS) cand[(size_t)blockIdx.x * nb + j] = j < steps ? win[j] : -1;
  if (gridDim.x == 1 && threadIdx.x == 0) calu_ipiv(win, k, nb, ipiv, idx + TS_ROWS, idx + TS_ROWS + LU_NB);
}

// sets TS_ARITY b .. TS_ARITY b + TS_ARITY - 1 of cin (nin sets of nb entries;
// the valid entries of a set are a prefix) -> set b of cout; the last level
// (one block) also writes the interchanges
template <class T>
__global__ void __launch_bounds__(TS_THREADS) k_tslu_merge(const T* A, size_t lda, int k, int nb, const int* cin, int nin,
                                                          int* cout, int64_t* ipiv) {
  __shared__ int idx[TS_ROWS + 2 * LU_NB];
  __shared__ int cnt[TS_ARITY];
  const int b = blockIdx.x;
  if (threadIdx.x < TS_ARITY) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int q = threadIdx.x / LU_NB, e = threadIdx.x % LU_NB;  // set q, entry e
  const int set = TS_ARITY * b + q;
  int v = -1;
  if (q < TS_ARITY && set < nin && e < nb) v = cin[(size_t)set * nb + e];
  if (v >= 0) atomicAdd(&cnt[q], 1);
  __syncthreads();
  if (v >= 0) {
    int off = 0;
    for (int u = 0; u < q; u++) off += cnt[u];
    idx[off + e] = v;
  }
  int R = 0;
  for (int u = 0; u < TS_ARITY; u++) R += cnt[u];
  __shared__ int win[LU_NB];
  __syncthreads();
  ts_select<T>(A, lda, k, nb, idx, R, win);
  const int steps = R < nb ? R : nb;
  for (int j = threadIdx.x; j < nb; j += TS_THREADS) cout[(size_t)b * nb + j] = j < steps ? win[j] : -1;
  if (gridDim.x == 1 && threadIdx.x == 0) calu_ipiv(win, k, nb, ipiv, idx + TS_ROWS, idx + TS_ROWS + LU_NB);
}

// interchanges ipiv[k..k+nb) applied in sequence to columns [0, ncol)
template <class T>
__global__ void k_laswp_rows(T* A, size_t lda, int ncol, int k, int nb, const int64_t* ipiv) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  for (int j = k; j < k + nb; j++) {
    int p = (int)ipiv[j];
    if (p != j) {
      T t = A[(size_t)j * lda + c];
      A[(size_t)j * lda + c] = A[(size_t)p * lda + c];
      A[(size_t)p * lda + c] = t;
    }
  }
}

// L11 U11 = A[k:k+nb][k:k+nb] in place, without interchanges; info[0] = k + j + 1
// at the first exactly zero pivot (LAPACK's convention)
template <class T>
__global__ void __launch_bounds__(DIAG_THREADS) k_diag_lu(T* A, size_t lda, int k, int nb, int* info) {
  extern __shared__ __align__(16) unsigned char tsraw[];
  T* M = (T*)tsraw;
  const int ld = nb + 1;
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) M[(t / nb) * ld + t % nb] = A[(size_t)(k + t / nb) * lda + k + t % nb];
  __syncthreads();
  T one, zero;
  one.x = 1; one.y = 0; zero.x = 0; zero.y = 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = DIAG_THREADS / 32;
  const int c0 = lane, c1 = lane + 32;
  for (int j = 0; j < nb; j++) {
    const T piv = M[j * ld + j];
    const bool nz = !(piv.x == 0 && piv.y == 0);
    if (!nz && threadIdx.x == 0 && info[0] == 0) info[0] = k + j + 1;
    // 1 / piv through one real division
    typedef typename RealOf<T>::type Rt;
    const Rt d2 = piv.x * piv.x + piv.y * piv.y;
    const Rt id = nz ? (Rt)1 / d2 : (Rt)0;
    T pinv;
    pinv.x = piv.x * id;
    pinv.y = -piv.y * id;
    // warp w: rows j + 1 + ((w - j - 1) mod nw) + nw i; lanes: columns c0, c1 > j
    const bool u0 = c0 > j && c0 < nb, u1 = c1 > j && c1 < nb;
    const T p0 = u0 ? M[j * ld + c0] : zero;
    const T p1 = u1 ? M[j * ld + c1] : zero;
    for (int r = j + 1 + ((w - (j + 1)) % nw + nw) % nw; r < nb; r += nw) {
      T* row = M + r * ld;
      const T l = row[j] * pinv;
      __syncwarp();
      if (lane == (j & 31)) row[j] = l;
      if (u0) row[c0] -= l * p0;
      if (u1) row[c1] -= l * p1;
    }
    __syncthreads();
  }
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) A[(size_t)(k + t / nb) * lda + k + t % nb] = M[(t / nb) * ld + t % nb];
}

// rows [r0, r1), columns k..k+nb-1: X <- X U11^-1 (U11 non-unit upper of
// A[k:k+nb][k:k+nb]).  Column-oriented substitution per row with the rows of
// U11 pre-divided by their diagonal and zero-padded to 64 x 64 in shared
// memory (W[j][c] = U[j][c] / U[j][j] for j < c < nb, else 0): at step j every
// lane subtracts a_j W[j][c] from its columns without a predicate, and a_j
// stays untouched from step j on, so x_j = a_j / U[j][j] is applied once at
// the end.  A warp holds two rows (lanes: columns l and l + 32), two
// independent chains; the second half of the steps touches only the upper
// 32 columns.
template <class T>
__global__ void __launch_bounds__(PANEL_THREADS) k_trsm_right(T* A, size_t lda, int k, int nb, int r0, int r1) {
  extern __shared__ __align__(16) unsigned char tsraw[];
  T* W = (T*)tsraw;  // LU_NB x LU_NB
  T* dinv = W + LU_NB * LU_NB;
  T zero;
  zero.x = 0;
  zero.y = 0;
  for (int t = threadIdx.x; t < LU_NB * LU_NB; t += blockDim.x) {
    const int j = t / LU_NB, c = t % LU_NB;
    W[t] = (j < nb && c < nb) ? A[(size_t)(k + j) * lda + k + c] : zero;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < LU_NB; j += blockDim.x) {
    const T d = W[j * LU_NB + j];
    T one;
    one.x = 1;
    one.y = 0;
    dinv[j] = (j >= nb || (d.x == 0 && d.y == 0)) ? zero : cdivc(one, d);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < LU_NB * LU_NB; t += blockDim.x) {
    const int j = t / LU_NB, c = t % LU_NB;
    W[t] = (c > j) ? W[t] * dinv[j] : zero;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  const int stride = 2 * gridDim.x * wpb;
  for (int r = r0 + 2 * (blockIdx.x * wpb + (threadIdx.x >> 5)); r < r1; r += stride) {
    const bool hasB = r + 1 < r1;
    T* rowA = A + (size_t)r * lda + k;
    T* rowB = rowA + lda;
    T a0 = zero, a1 = zero, b0 = zero, b1 = zero;
    if (lane < nb) { a0 = rowA[lane]; if (hasB) b0 = rowB[lane]; }
    if (lane + 32 < nb) { a1 = rowA[lane + 32]; if (hasB) b1 = rowB[lane + 32]; }
#pragma unroll 8
    for (int j = 0; j < 32; j++) {
      T va, vb;
      va.x = __shfl_sync(0xffffffffu, a0.x, j);
      va.y = __shfl_sync(0xffffffffu, a0.y, j);
      vb.x = __shfl_sync(0xffffffffu, b0.x, j);
      vb.y = __shfl_sync(0xffffffffu, b0.y, j);
      const T w0 = W[j * LU_NB + lane], w1 = W[j * LU_NB + lane + 32];
      a0 -= va * w0;
      a1 -= va * w1;
      b0 -= vb * w0;
      b1 -= vb * w1;
    }
#pragma unroll 8
    for (int j = 32; j < LU_NB; j++) {
      T va, vb;
      va.x = __shfl_sync(0xffffffffu, a1.x, j - 32);
      va.y = __shfl_sync(0xffffffffu, a1.y, j - 32);
      vb.x = __shfl_sync(0xffffffffu, b1.x, j - 32);
      vb.y = __shfl_sync(0xffffffffu, b1.y, j - 32);
      const T w1 = W[j * LU_NB + lane + 32];
      a1 -= va * w1;
      b1 -= vb * w1;
    }
    const T d0 = dinv[lane], d1 = dinv[lane + 32];
    if (lane < nb) { rowA[lane] = a0 * d0; if (hasB) rowB[lane] = b0 * d0; }
    if (lane + 32 < nb) { rowA[lane + 32] = a1 * d1; if (hasB) rowB[lane + 32] = b1 * d1; }
  }
}

// In-place LU of the n x n row-major matrix A (lda) with tournament pivoting;
// ipiv[j] = 0-based row interchanged with row j (interchanges applied in
// sequence across the full row width, as LAPACK's); info (device int)
// receives LAPACK's info (0: success).  gemm(M, N, K, A, lda, B, ldb, C, ldc,
// st) performs C -= A B.
__global__ void k_iota_i64(int64_t* v, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

// pivot == false: no row interchanges at all (ipiv = identity): for a matrix
// randomised by butterfly transforms (k_rbt_matrix), where the refinement
// that follows checks the factors
template <class T, class GEMM>
static int lu_factor(T* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st, GEMM gemm, bool pivot = true) {
  if (n <= 0) return 0;
  if (!pivot) {
    k_iota_i64<<<(n + 255) / 256, 256, 0, st>>>(ipiv, n);
    gbi_count_launch();
  }
  const int nsets0 = (n + TS_ROWS - 1) / TS_ROWS;
  int* cand = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&cand, sizeof(int) * (size_t)2 * nsets0 * LU_NB, st));
  GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), st));
  const size_t sm_diag = (size_t)LU_NB * (LU_NB + 1) * sizeof(T);
  const size_t sm_right = (size_t)LU_NB * LU_NB * sizeof(T) + LU_NB * sizeof(T);  // W, dinv
  int rc = 0;
  int dev = 0, nsm = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GB_CUDA(cudaFuncSetAttribute(k_diag_lu<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_diag));
  GB_CUDA(cudaFuncSetAttribute(k_trsm_right<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_right));
  for (int k = 0; k < n && !rc; k += LU_NB) {
    const int nb = (n - k < LU_NB) ? n - k : LU_NB;
    const int kend = k + nb;
    int nsets = (n - k + TS_ROWS - 1) / TS_ROWS;
    int* cin = cand;
    int* cout = cand + (size_t)nsets0 * LU_NB;
    if (pivot) {
      k_tslu_leaf<T><<<nsets, TS_THREADS, 0, st>>>(A, lda, n, k, nb, cin, ipiv);
      gbi_count_launch();
      while (nsets > 1) {
        int nout = (nsets + TS_ARITY - 1) / TS_ARITY;
        k_tslu_merge<T><<<nout, TS_THREADS, 0, st>>>(A, lda, k, nb, cin, nsets, cout, ipiv);
        gbi_count_launch();
        int* t = cin;
        cin = cout;
        cout = t;
        nsets = nout;
      }
      k_laswp_rows<T><<<(n + 255) / 256, 256, 0, st>>>(A, lda, n, k, nb, ipiv);
      gbi_count_launch();
    }
    k_diag_lu<T><<<1, DIAG_THREADS, sm_diag, st>>>(A, lda, k, nb, info);
    gbi_count_launch();
    if (kend < n) {
      int rows = n - kend;
      int wpb = PANEL_THREADS / 32;
      int nblk = (rows + 2 * wpb - 1) / (2 * wpb);
      if (nblk > 2 * nsm) nblk = 2 * nsm;
      k_trsm_right<T><<<nblk, PANEL_THREADS, sm_right, st>>>(A, lda, k, nb, kend, n);
      gbi_count_launch();
      if (cudaGetLastError() != cudaSuccess) { gbi_set_error("LU panel launch failed"); rc = -1; break; }
    }
    // updates: inside the outer block of LU_NBO columns only, until its last
    // panel; then the block's columns of U and one trailing update with
    // K = LU_NBO (a quarter of the C traffic of per-panel updates)
    const int K0 = (k / LU_NBO) * LU_NBO;
    const int Kend = (K0 + LU_NBO < n) ? K0 + LU_NBO : n;
    if (kend < Kend) {
      if (trsm_rows<T>(0, A + (size_t)k * lda + k, lda, A + (size_t)k * lda, lda, nb, kend, Kend, st)) { rc = -1; break; }
      if (gemm(n - kend, Kend - kend, nb, A + (size_t)kend * lda + k, lda, A + (size_t)k * lda + kend, lda,
               A + (size_t)kend * lda + kend, lda, st)) { rc = -1; break; }
    } else if (Kend < n) {
      // U12 of the outer block: X <- L^-1 X for rows K0..Kend, columns Kend..n,
      // L the block's unit lower triangle, by its 64-row diagonal blocks
      for (int i0 = K0; i0 < Kend && !rc; i0 += LU_NB) {
        const int ib = (Kend - i0 < LU_NB) ? Kend - i0 : LU_NB;
        if (trsm_rows<T>(0, A + (size_t)i0 * lda + i0, lda, A + (size_t)i0 * lda, lda, ib, Kend, n, st)) rc = -1;
        else if (i0 + ib < Kend &&
                 gemm(Kend - i0 - ib, n - Kend, ib, A + (size_t)(i0 + ib) * lda + i0, lda, A + (size_t)i0 * lda + Kend,
                      lda, A + (size_t)(i0 + ib) * lda + Kend, lda, st))
          rc = -1;
      }
      if (rc) break;
      if (gemm(n - Kend, n - Kend, Kend - K0, A + (size_t)Kend * lda + K0, lda, A + (size_t)K0 * lda + Kend, lda,
               A + (size_t)Kend * lda + Kend, lda, st)) { rc = -1; break; }
    }
  }
  cudaFreeAsync(cand, st);
  if (!rc) GB_CUDA(cudaGetLastError());
  return rc;
}

extern "C" int gbi_zgetrf(cplx* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st) {
  return lu_factor<cplx>(A, lda, n, ipiv, info, st, gemm_sub);
}

// apply the row interchanges of zgetrf to X (n rows, ncol columns)
template <class T>
__global__ void k_laswp(T* X, size_t ldx, int n, int ncol, const int64_t* ipiv) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  for (int j = 0; j < n; j++) {
    int p = (int)ipiv[j];
    if (p != j) {
      T t = X[(size_t)j * ldx + c];
      X[(size_t)j * ldx + c] = X[(size_t)p * ldx + c];
      X[(size_t)p * ldx + c] = t;
    }
  }
}

// Solve (LU) X = P B in place for X (n x nrhs, row-major ldx), given the
// factors of gbi_zgetrf.  Blocked: triangular solve of a block row, then a
// GEMM update of the remaining rows.
extern "C" int gbi_zgetrs(const cplx* LU, size_t lda, int n, const int64_t* ipiv, cplx* X, size_t ldx, int nrhs,
                          cudaStream_t st) {
  k_laswp<cplx><<<(nrhs + 127) / 128, 128, 0, st>>>(X, ldx, n, nrhs, ipiv);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  for (int k = 0; k < n; k += LU_NB) {  // forward: L Y = P B
    int nb = (n - k < LU_NB) ? n - k : LU_NB;
    if (trsm_rows<cplx>(0, LU + (size_t)k * lda + k, lda, X + (size_t)k * ldx, ldx, nb, 0, nrhs, st)) return -1;
    if (gemm_sub(n - k - nb, nrhs, nb, LU + (size_t)(k + nb) * lda + k, lda, X + (size_t)k * ldx, ldx,
                 X + (size_t)(k + nb) * ldx, ldx, st))
      return -1;
  }
  int last = ((n - 1) / LU_NB) * LU_NB;
  for (int k = last; k >= 0; k -= LU_NB) {  // backward: U X = Y
    int nb = (n - k < LU_NB) ? n - k : LU_NB;
    if (trsm_rows<cplx>(1, LU + (size_t)k * lda + k, lda, X + (size_t)k * ldx, ldx, nb, 0, nrhs, st)) return -1;
    if (gemm_sub(k, nrhs, nb, LU + k, lda, X + (size_t)k * ldx, ldx, X, ldx, st)) return -1;
  }
  return 0;
}

__global__ void k_set_identity(cplx* X, size_t ldx, int n) {
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n * n) return;
  int i = (int)(p / n), j = (int)(p % n);
  X[(size_t)i * ldx + j] = cmk(i == j ? 1.0 : 0.0, 0.0);
}

// X = A^{-1} from the factors of gbi_zgetrf
extern "C" int gbi_zinverse(const cplx* LU, size_t lda, int n, const int64_t* ipiv, cplx* X, size_t ldx,
                            cudaStream_t st) {
  size_t nn = (size_t)n * n;
  k_set_identity<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(X, ldx, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return gbi_zgetrs(LU, lda, n, ipiv, X, ldx, n, st);
}

// y[i] = sum_j M[i][j] x[j]  (complex FP64 GEMV; one warp per row)
__global__ void k_zgemv(const cplx* __restrict__ M, size_t ldm, int n, int ncol, const cplx* __restrict__ x, cplx* y) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= n) return;
  const cplx* r = M + (size_t)warp * ldm;
  double sr = 0.0, si = 0.0;
  for (int j = lane; j < ncol; j += 32) {
    cplx a = r[j], b = x[j];
    sr = fma(a.x, b.x, sr);
    sr = fma(-a.y, b.y, sr);
    si = fma(a.x, b.y, si);
    si = fma(a.y, b.x, si);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (lane == 0) y[warp] = cmk(sr, si);
}

extern "C" int gbi_zgemv(const cplx* M, size_t ldm, int n, int ncol, const cplx* x, cplx* y, cudaStream_t st) {
  unsigned nb = (unsigned)(((size_t)n * 32 + 255) / 256);
  k_zgemv<<<nb, 256, 0, st>>>(M, ldm, n, ncol, x, y);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// C -= A B (exported for the tests of the GEMM kernel)
extern "C" int gbi_zgemm_sub(int M, int N, int K, const cplx* A, size_t lda, const cplx* B, size_t ldb, cplx* C,
                             size_t ldc, cudaStream_t st) {
  return gemm_sub(M, N, K, A, lda, B, ldb, C, ldc, st);
}

// ==================================================================== FP32
// Mixed-precision form: complex FP32 factors of A, refined in FP64 against
// the FP64 matrix (the residual b - A x is always formed in FP64).

// C[M][N] -= A[M][K] B[K][N], complex FP32, row-major.  64 x 128 output tile
// per 256-thread block, each thread a 4 x 8 complex sub-tile.
#define CG_BM 64
#define CG_BN 128
#define CG_BK 16
__global__ void __launch_bounds__(256) k_cgemm_nn(int M, int N, int K, const cplxf* __restrict__ A, size_t lda,
                                                  const cplxf* __restrict__ B, size_t ldb, cplxf* C, size_t ldc) {
  __shared__ cplxf As[CG_BK][CG_BM];
  __shared__ cplxf Bs[CG_BK][CG_BN];
  int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  int m0 = blockIdx.y * CG_BM, n0 = blockIdx.x * CG_BN;
  float accr[4][8], acci[4][8];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) { accr[i][j] = 0.f; acci[i][j] = 0.f; }
  for (int k0 = 0; k0 < K; k0 += CG_BK) {
    for (int t = threadIdx.x; t < CG_BK * CG_BM; t += 256) {
      int kk = t % CG_BK, mm = t / CG_BK;
      int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(size_t)gm * lda + gk] : cmkf(0.f, 0.f);
    }
    for (int t = threadIdx.x; t < CG_BK * CG_BN; t += 256) {
      int nn = t % CG_BN, kk = t / CG_BN;
      int gn = n0 + nn, gk = k0 + kk;
      Bs[kk][nn] = (gn < N && gk < K) ? B[(size_t)gk * ldb + gn] : cmkf(0.f, 0.f);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < CG_BK; kk++) {
      cplxf a[4], b[8];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 8; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) {
          accr[i][j] = fmaf(a[i].x, b[j].x, accr[i][j]);
          accr[i][j] = fmaf(-a[i].y, b[j].y, accr[i][j]);
          acci[i][j] = fmaf(a[i].x, b[j].y, acci[i][j]);
          acci[i][j] = fmaf(a[i].y, b[j].x, acci[i][j]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      cplxf* c = C + (size_t)gm * ldc + gn;
      c->x -= accr[i][j];
      c->y -= acci[i][j];
    }
  }
}

static int cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C, size_t ldc,
                     cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  dim3 grid((N + CG_BN - 1) / CG_BN, (M + CG_BM - 1) / CG_BM);
  k_cgemm_nn<<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" size_t gbi_tc_scratch_floats(int M, int N, int K);
extern "C" int gbi_tc_cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C,
                                size_t ldc, int passes, float* scratch, int* err, cudaStream_t st);
extern "C" int gbi_tc_passes(void);

// Complex-FP32 LU: the trailing updates on the tensor cores (split TF32, three
// passes: FP32-level products), scratch and the time-out flag shared by all
// panels; the flag is read back once at the end.
static int cgetrf_tc(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st, bool pivot);
extern "C" int gbi_cgetrf(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st) {
  return cgetrf_tc(A, lda, n, ipiv, info, st, true);
}
// as gbi_cgetrf without row interchanges (ipiv = identity)
extern "C" int gbi_cgetrf_nopiv(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st) {
  return cgetrf_tc(A, lda, n, ipiv, info, st, false);
}
static int cgetrf_tc(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st, bool pivot) {
  if (n <= 0) return 0;
  float* scratch = nullptr;
  int* err = nullptr;
  size_t need = gbi_tc_scratch_floats(n, n, LU_NBO);
  GB_CUDA(cudaMallocAsync((void**)&scratch, need * sizeof(float), st));
  GB_CUDA(cudaMallocAsync((void**)&err, 16, st));
  GB_CUDA(cudaMemsetAsync(err, 0, 4, st));
  auto tc = [scratch, err](int M, int N, int K, const cplxf* a, size_t la, const cplxf* b, size_t lb, cplxf* c, size_t lc,
                           cudaStream_t s) { return gbi_tc_cgemm_sub(M, N, K, a, la, b, lb, c, lc, gbi_tc_passes(), scratch, err, s); };
  int rc = lu_factor<cplxf>(A, lda, n, ipiv, info, st, tc, pivot);
  int h = 0;
  if (!rc && (cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("FP32 LU: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  cudaFreeAsync(scratch, st);
  cudaFreeAsync(err, st);
  if (!rc && h) {
    gbi_set_error("FP32 LU: a tensor-core pipeline wait timed out");
    rc = -1;
  }
  return rc;
}

// the previous FP32 path (SIMT GEMM), kept for comparison in tests and benches
extern "C" int gbi_cgetrf_simt(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st) {
  return lu_factor<cplxf>(A, lda, n, ipiv, info, st, cgemm_sub);
}

extern "C" int gbi_cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C,
                             size_t ldc, cudaStream_t st) {
  return cgemm_sub(M, N, K, A, lda, B, ldb, C, ldc, st);
}

// complex FP64 -> complex FP32 (n elements)
__global__ void k_to_c64(const cplx* __restrict__ a, cplxf* __restrict__ b, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) b[i] = cmkf((float)a[i].x, (float)a[i].y);
}
extern "C" int gbi_to_c64(const cplx* a, cplxf* b, size_t n, cudaStream_t st) {
  k_to_c64<<<152 * 8, 256, 0, st>>>(a, b, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// out[0] += sum |a_i|^2
__global__ void k_sqnorm(const cplx* a, size_t n, double* out) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (i < n) v = a[i].x * a[i].x + a[i].y * a[i].y;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}

// Solve A X = B (A n x n FP64, B n x nrhs, nrhs <= 8, packed) with complex-FP32
// factors of A (tensor-core LU) and FP64 iterative refinement on the FP64 A:
// X += LU32^-1 (B - A X) until ||B - A X||_F <= 1e-13 ||B||_F (at most 30
// corrections).  *iters, *relres report the refinement.
extern "C" int gbi_zgesv_mixed(const cplx* A, int n, const cplx* B, int nrhs, cplx* X, int* iters, double* relres,
                               cudaStream_t st);
// x += d (FP32 correction) and r -> d (FP64 residual rounded to FP32)
__global__ void k_axpy_c64(cplx* x, const cplxf* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { x[i].x += (double)d[i].x; x[i].y += (double)d[i].y; }
}
__global__ void k_c128_to_c64_scaled(const cplx* r, cplxf* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = cmkf((float)r[i].x, (float)r[i].y);
}
template <class T>
static int lu_solve_multi(const T* LU, size_t lda, int n, const int* perm, const T* X, size_t ldx, int nrhs, T* Y,
                          cudaStream_t st);
// ---- random butterfly transforms (RBT)
// Parker's recursive butterflies of depth 2 as used to avoid pivoting
// (D. S. Parker, UCLA tech. report CSD-950023, 1995; M. Baboulin, J.
// Dongarra, J. Herrmann, S. Tomov, ACM TOMS 39 (2013) 16): A_r = U^T A V with
// U, V = diag(B', B'') B, B = [R0 R1; R0 -R1] / sqrt 2 of size n (R0, R1
// random diagonal, entries e^{rho/10}, rho uniform in [-1/2, 1/2)), B', B''
// the same of size n/2.  A_r is factorised without interchanges; then
// A^-1 b = V A_r^-1 U^T b.  With q = n/4, indices i + a q (a = 0..3) mix only
// among themselves.  Parameters p[2][n] per side, level 1 (pairs a, a+2) then
// level 2 (pairs (0,1), (2,3)): for the pair (a, b) the diagonal entries are
// p[i + a q] and p[i + b q].
//   transposed butterfly (U^T from the left, V from the right, in the order
//   level 2 then level 1): x_a' = r_a (x_a + x_b) / sqrt 2,
//                          x_b' = r_b (x_a - x_b) / sqrt 2
//   butterfly (V y, level 1 then level 2): x_a' = (r_a x_a + r_b x_b) / sqrt 2,
//                                          x_b' = (r_a x_a - r_b x_b) / sqrt 2
template <class C, class R>
__device__ __forceinline__ void bfly_t(C& xa, C& xb, R ra, R rb) {
  const R s = (R)0.70710678118654752440;
  const C u = xa + xb, v = xa - xb;
  xa = u * (ra * s);
  xb = v * (rb * s);
}
template <class C, class R>
__device__ __forceinline__ void bfly_f(C& xa, C& xb, R ra, R rb) {
  const R s = (R)0.70710678118654752440;
  const C u = xa * (ra * s), v = xb * (rb * s);
  xa = u + v;
  xb = u - v;
}
template <class C, class R>
__device__ __forceinline__ void rbt4_t(C x[4], const float* p, int i, int q) {  // U^T x (or the columns of A V)
  const float* p1 = p;
  const float* p2 = p + 4 * (size_t)q;
  bfly_t<C, R>(x[0], x[1], (R)p2[i], (R)p2[i + q]);
  bfly_t<C, R>(x[2], x[3], (R)p2[i + 2 * q], (R)p2[i + 3 * q]);
  bfly_t<C, R>(x[0], x[2], (R)p1[i], (R)p1[i + 2 * q]);
  bfly_t<C, R>(x[1], x[3], (R)p1[i + q], (R)p1[i + 3 * q]);
}
template <class C, class R>
__device__ __forceinline__ void rbt4_f(C x[4], const float* p, int i, int q) {  // V y
  const float* p1 = p;
  const float* p2 = p + 4 * (size_t)q;
  bfly_f<C, R>(x[0], x[2], (R)p1[i], (R)p1[i + 2 * q]);
  bfly_f<C, R>(x[1], x[3], (R)p1[i + q], (R)p1[i + 3 * q]);
  bfly_f<C, R>(x[0], x[1], (R)p2[i], (R)p2[i + q]);
  bfly_f<C, R>(x[2], x[3], (R)p2[i + 2 * q], (R)p2[i + 3 * q]);
}

// A <- U^T A V in place (n divisible by 4); thread per index pair (i, j) of
// [0, n/4)^2: the 16 entries A[i + a q][j + b q]
__global__ void k_rbt_matrix(cplxf* A, size_t lda, int n, const float* pu, const float* pv) {
  const int q = n / 4;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)q * q) return;
  const int i = (int)(t / q), j = (int)(t % q);
  cplxf x[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) x[a][b] = A[(size_t)(i + a * q) * lda + j + b * q];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    cplxf c[4] = {x[0][b], x[1][b], x[2][b], x[3][b]};
    rbt4_t<cplxf, float>(c, pu, i, q);
#pragma unroll
    for (int a = 0; a < 4; a++) x[a][b] = c[a];
  }
#pragma unroll
  for (int a = 0; a < 4; a++) rbt4_t<cplxf, float>(x[a], pv, j, q);
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) A[(size_t)(i + a * q) * lda + j + b * q] = x[a][b];
}
// d = U^T r in FP64, rounded to FP32 (n x nrhs, packed rows)
__global__ void k_rbt_ut(const cplx* r, cplxf* d, int n, int nrhs, const float* pu) {
  const int q = n / 4;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q * nrhs) return;
  const int i = t / nrhs, c = t % nrhs;
  cplx x[4];
#pragma unroll
  for (int a = 0; a < 4; a++) x[a] = r[(size_t)(i + a * q) * nrhs + c];
  rbt4_t<cplx, double>(x, pu, i, q);
#pragma unroll
  for (int a = 0; a < 4; a++) d[(size_t)(i + a * q) * nrhs + c] = cmkf((float)x[a].x, (float)x[a].y);
}
// x += V y in FP64 (n x nrhs, packed rows)
__global__ void k_rbt_axpy_v(cplx* x, const cplxf* y, int n, int nrhs, const float* pv) {
  const int q = n / 4;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= q * nrhs) return;
  const int i = t / nrhs, c = t % nrhs;
  cplx v[4];
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const cplxf w = y[(size_t)(i + a * q) * nrhs + c];
    v[a] = cmk((double)w.x, (double)w.y);
  }
  rbt4_f<cplx, double>(v, pv, i, q);
#pragma unroll
  for (int a = 0; a < 4; a++) x[(size_t)(i + a * q) * nrhs + c] += v[a];
}

// butterfly parameters for order n: 4 n floats (U's two levels, then V's),
// e^{rho/10} with rho uniform in [-1/2, 1/2) from splitmix64 with a fixed
// seed, so that a factorisation is reproducible
extern "C" void gbi_rbt_params(int n, float* h) {
  const size_t n4 = 4 * (size_t)n;
  uint64_t z = 0x243F6A8885A308D3ull ^ (uint64_t)n;
  for (size_t i = 0; i < n4; i++) {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    const double rho = (double)(x >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    h[i] = (float)exp(rho / 10.0);
  }
}
extern "C" int gbi_rbt_matrix(cplxf* A, size_t lda, int n, const float* pu, const float* pv, cudaStream_t st) {
  if (n % 4) { gbi_set_error("gbi_rbt_matrix: n = %d not divisible by 4", n); return -1; }
  const size_t qq = (size_t)(n / 4) * (n / 4);
  if (qq == 0) return 0;
  k_rbt_matrix<<<(unsigned)((qq + 255) / 256), 256, 0, st>>>(A, lda, n, pu, pv);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// X <- V X U^T in place: the inverse of A from the inverse X of the
// randomised U^T A V.  Column groups take the butterfly V (rbt4_f, pv), row
// groups the butterfly U (row . U^T = (U row^T)^T: rbt4_f, pu).
__global__ void k_rbt_inverse(cplxf* X, size_t ldx, int n, const float* pu, const float* pv) {
  const int q = n / 4;
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)q * q) return;
  const int i = (int)(t / q), j = (int)(t % q);
  cplxf x[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) x[a][b] = X[(size_t)(i + a * q) * ldx + j + b * q];
#pragma unroll
  for (int b = 0; b < 4; b++) {
    cplxf c[4] = {x[0][b], x[1][b], x[2][b], x[3][b]};
    rbt4_f<cplxf, float>(c, pv, i, q);
#pragma unroll
    for (int a = 0; a < 4; a++) x[a][b] = c[a];
  }
#pragma unroll
  for (int a = 0; a < 4; a++) rbt4_f<cplxf, float>(x[a], pu, j, q);
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) X[(size_t)(i + a * q) * ldx + j + b * q] = x[a][b];
}
extern "C" int gbi_rbt_inverse(cplxf* X, size_t ldx, int n, const float* pu, const float* pv, cudaStream_t st) {
  if (n % 4) { gbi_set_error("gbi_rbt_inverse: n = %d not divisible by 4", n); return -1; }
  const size_t qq = (size_t)(n / 4) * (n / 4);
  if (qq == 0) return 0;
  k_rbt_inverse<<<(unsigned)((qq + 255) / 256), 256, 0, st>>>(X, ldx, n, pu, pv);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

template <class T>
static int lu_solve_multi(const T* LU, size_t lda, int n, const int* perm, const T* X, size_t ldx, int nrhs, T* Y,
                          cudaStream_t st);
// x += V LU32^-1 U^T r for the factors of the randomised matrix (no
// interchanges; perm = identity)
extern "C" int gbi_ir_step_rbt(cplx* x, const cplx* r, cplxf* d, cplxf* d2, const cplxf* LU32, size_t lda, int n,
                               const int* perm, const float* pu, const float* pv, cudaStream_t st) {
  const int q = n / 4;
  k_rbt_ut<<<(q + 255) / 256, 256, 0, st>>>(r, d, n, 1, pu);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  if (lu_solve_multi<cplxf>(LU32, lda, n, perm, d, 1, 1, d2, st)) return -1;
  k_rbt_axpy_v<<<(q + 255) / 256, 256, 0, st>>>(x, d2, n, 1, pv);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// x += LU32^-1 P r (r converted to FP32; d, d2: n-element FP32 work vectors)
extern "C" int gbi_ir_step(cplx* x, const cplx* r, cplxf* d, cplxf* d2, const cplxf* LU32, size_t lda, int n,
                           const int* perm, cudaStream_t st) {
  k_c128_to_c64_scaled<<<(n + 255) / 256, 256, 0, st>>>(r, d, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  if (lu_solve_multi<cplxf>(LU32, lda, n, perm, d, 1, 1, d2, st)) return -1;
  k_axpy_c64<<<(n + 255) / 256, 256, 0, st>>>(x, d2, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---- permutation and multi-RHS triangular solves (nrhs <= 8)
// perm[i] = original row at position i after the interchanges ipiv[0..n)
// (sequential by nature: one block, the vector in shared memory when it fits)
#define PERM_SMEM_MAX 49152
__global__ void k_make_perm(const int64_t* ipiv, int n, int* perm) {
  extern __shared__ int sperm[];
  int* v = (n <= PERM_SMEM_MAX) ? sperm : perm;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = i;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int j = 0; j < n; j++) {
      int p = (int)ipiv[j];
      if (p != j) { int t = v[j]; v[j] = v[p]; v[p] = t; }
    }
  __syncthreads();
  if (v != perm)
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = v[i];
}
__global__ void k_iota_i32(int* v, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}
// the identity permutation (factors without interchanges)
extern "C" int gbi_perm_identity(int n, int* perm, cudaStream_t st) {
  if (n <= 0) return 0;
  k_iota_i32<<<(n + 255) / 256, 256, 0, st>>>(perm, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}
extern "C" int gbi_make_perm(const int64_t* ipiv, int n, int* perm, cudaStream_t st) {
  size_t sm = (n <= PERM_SMEM_MAX) ? (size_t)n * sizeof(int) : 0;
  GB_CUDA(cudaFuncSetAttribute(k_make_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, PERM_SMEM_MAX * (int)sizeof(int)));
  k_make_perm<<<1, 1024, sm, st>>>(ipiv, n, perm);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}
template <class T>
__global__ void k_gather_rows(const T* X, size_t ldx, int n, int nrhs, const int* perm, T* Y) {
  size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)n * nrhs) return;
  int i = (int)(q / nrhs), c = (int)(q % nrhs);
  Y[(size_t)i * nrhs + c] = X[(size_t)perm[i] * ldx + c];
}
// One cooperative launch per triangular solve.  Row blocks of LU_NB rows are
// owned by the CTAs (block q by CTA q mod gridDim, in increasing q).  A CTA
// streams its block's strip of the factor, LU_NB x LU_NB tiles of block
// pairs (q, j < q), into shared memory ahead of need (cp.async, two stages:
// the tiles do not depend on the other blocks), and folds in tile j as soon
// as block j's flag is set: thread (row i, quarter kq) keeps its partial sums
// of the block's right-hand sides in registers across all tiles, reduced once
// at the end.  Then the diagonal block is solved (warp per right-hand side,
// substitution with shuffles), the block's rows of Y published and its flag
// set.  All CTAs are co-resident (cooperative launch) and every block waits
// only on blocks of smaller q, so the waits end; each wait is also bounded
// (TRSV_SPIN_LIMIT polls): on time-out *err is raised and every CTA returns.
// Tile layout in shared memory: row i of a tile is 512 B (FP32 complex) or
// 1 KB (FP64 complex) of 16-byte chunks; chunk c of row i is stored at
// position c ^ (i & 7), so that 32 lanes reading one chunk of 32 consecutive
// rows hit every bank once per 8 rows.
#define TRSV_SPIN_LIMIT (1 << 22)
#define TRSV_THREADS 256
__device__ __forceinline__ cplx ldcg_c(const cplx* p) { return cmk(__ldcg(&p->x), __ldcg(&p->y)); }
__device__ __forceinline__ cplxf ldcg_c(const cplxf* p) { return cmkf(__ldcg(&p->x), __ldcg(&p->y)); }

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <class T>
struct TrsvLayout {
  static constexpr int CPC = 16 / (int)sizeof(T);      // complex per 16-byte chunk
  static constexpr int CHUNKS = LU_NB / CPC;           // chunks per tile row
  static constexpr int TILE = LU_NB * LU_NB;           // complex per tile
  static constexpr int LDT = LU_NB + 1;                // transposed diagonal block
  static constexpr size_t SMEM = (size_t)(2 * TILE + LU_NB * LDT + LU_NB + 2 * LU_NB * 8) * sizeof(T);
};

// stage tile (rows r0.., columns c0..) of the factor into buf (swizzled
// chunks); rows >= rows_, columns >= cols_ are zero.  vec: 16-byte copies
// are legal (aligned base and leading dimension)
template <class T>
__device__ __forceinline__ void trsv_stage(const T* LU, size_t lda, int r0, int rows_, int c0, int cols_, T* buf,
                                           bool vec) {
  typedef TrsvLayout<T> Ly;
  for (int t = threadIdx.x; t < LU_NB * Ly::CHUNKS; t += blockDim.x) {
    const int i = t / Ly::CHUNKS, c = t % Ly::CHUNKS;
    T* dst = buf + i * LU_NB + ((c ^ (i & 7)) * Ly::CPC);
    const int col = c * Ly::CPC;
    const T* src = LU + (size_t)(r0 + i) * lda + c0 + col;
    if (i < rows_ && col + Ly::CPC <= cols_ && vec) {
      cp_async16(dst, src);
    } else {
#pragma unroll
      for (int e = 0; e < Ly::CPC; e++) {
        T v;
        v.x = 0;
        v.y = 0;
        if (i < rows_ && col + e < cols_) v = src[e];
        dst[e] = v;
      }
    }
  }
}

template <class T, int UPPER>
__global__ void __launch_bounds__(TRSV_THREADS) k_trsv_flags(const T* __restrict__ LU, size_t lda, int n, T* Y,
                                                             int nrhs, int* flags, int* err, int vec) {
  typedef typename RealOf<T>::type Rt;
  typedef TrsvLayout<T> Ly;
  extern __shared__ __align__(16) unsigned char tfraw[];
  T* sL = (T*)tfraw;                     // two tile stages
  T* sT = sL + 2 * Ly::TILE;             // diagonal block, transposed: sT[j * LDT + i] = block[i][j]
  T* sdinv = sT + LU_NB * Ly::LDT;       // inverted diagonal (UPPER)
  T* sy = sdinv + LU_NB;                 // right-hand sides of the tile's column block, LU_NB x 8
  T* sx = sy + LU_NB * 8;                // the block's right-hand sides, LU_NB x 8
  __shared__ int s_abort;
  const int nbk = (n + LU_NB - 1) / LU_NB;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int mi = threadIdx.x & (LU_NB - 1), kq = threadIdx.x / LU_NB;  // row, quarter of the chunks
  constexpr int QCH = Ly::CHUNKS / 4;
  for (int q = blockIdx.x; q < nbk; q += gridDim.x) {
    const int b = UPPER ? nbk - 1 - q : q;
    const int r0 = b * LU_NB, rows = min(LU_NB, n - r0);
    for (int t = threadIdx.x; t < rows * nrhs; t += blockDim.x) sx[t] = Y[(size_t)r0 * nrhs + t];
    for (int t = threadIdx.x; t < rows * rows; t += blockDim.x) {
      const int i = t / rows, j = t % rows;
      sT[j * Ly::LDT + i] = LU[(size_t)(r0 + i) * lda + r0 + j];
    }
    if (threadIdx.x == 0) s_abort = 0;
    Rt ar[8], ai[8];
#pragma unroll
    for (int c = 0; c < 8; c++) { ar[c] = 0; ai[c] = 0; }
    // tiles of the blocks this one depends on, in the order their flags are set
    if (q > 0) {
      const int jb0 = UPPER ? nbk - 1 : 0;
      trsv_stage<T>(LU, lda, r0, rows, jb0 * LU_NB, min(LU_NB, n - jb0 * LU_NB), sL, vec != 0);
    }
    cp_async_commit();
    for (int jq = 0; jq < q; jq++) {
      const int jb = UPPER ? nbk - 1 - jq : jq;
      const int c0 = jb * LU_NB, cols = min(LU_NB, n - c0);
      if (jq + 1 < q) {
        const int jn = UPPER ? nbk - 2 - jq : jq + 1;
        trsv_stage<T>(LU, lda, r0, rows, jn * LU_NB, min(LU_NB, n - jn * LU_NB), sL + ((jq + 1) & 1) * Ly::TILE,
                      vec != 0);
      }
      cp_async_commit();
      if (threadIdx.x == 0) {
        int it = 0;
        while (*(volatile int*)(flags + jb) == 0) {
          if (*(volatile int*)err != 0 || ++it > TRSV_SPIN_LIMIT) { atomicExch(err, 1); s_abort = 1; break; }
          __nanosleep(32);
        }
        __threadfence();
      }
      __syncthreads();
      if (s_abort) {
        cp_async_wait0();
        return;
      }
      for (int t = threadIdx.x; t < LU_NB * 8; t += blockDim.x) {
        const int k = t >> 3, c = t & 7;
        T v;
        v.x = 0;
        v.y = 0;
        if (k < cols && c < nrhs) v = ldcg_c(Y + (size_t)(c0 + k) * nrhs + c);
        sy[t] = v;
      }
      cp_async_wait1();
      __syncthreads();
      const T* tile = sL + (jq & 1) * Ly::TILE + mi * LU_NB;
#pragma unroll 2
      for (int cc = 0; cc < QCH; cc++) {
        const int ch = kq * QCH + cc;
        const T* src = tile + ((ch ^ (mi & 7)) * Ly::CPC);
#pragma unroll
        for (int e = 0; e < Ly::CPC; e++) {
          const T av = src[e];
          const T* yv = sy + (ch * Ly::CPC + e) * 8;
#pragma unroll
          for (int c = 0; c < 8; c++) {
            if (c < nrhs) {
              const T y = yv[c];
              ar[c] += av.x * y.x - av.y * y.y;
              ai[c] += av.x * y.y + av.y * y.x;
            }
          }
        }
      }
      __syncthreads();  // the stage and sy are rewritten next
    }
    cp_async_wait0();
    // reduce the four quarters (the tile stages are free now)
    if (q > 0) {
      T* red = sL;  // [4][LU_NB][8]
#pragma unroll
      for (int c = 0; c < 8; c++) {
        T v;
        v.x = ar[c];
        v.y = ai[c];
        red[(kq * LU_NB + mi) * 8 + c] = v;
      }
      __syncthreads();
      for (int t = threadIdx.x; t < rows * nrhs; t += blockDim.x) {
        const int i = t / nrhs, c = t % nrhs;
        T sum = red[i * 8 + c];
        for (int u = 1; u < 4; u++) sum += red[(u * LU_NB + i) * 8 + c];
        sx[t] -= sum;
      }
    }
    __syncthreads();  // sT, sx complete (no tile loop when q == 0)
    if (UPPER) {
      for (int j = threadIdx.x; j < rows; j += blockDim.x) {
        T one;
        one.x = 1; one.y = 0;
        sdinv[j] = cdivc(one, sT[j * Ly::LDT + j]);
      }
    }
    __syncthreads();
    if (w < nrhs) {  // diagonal block: warp w solves right-hand side w
      const int i0 = lane, i1 = lane + 32;
      T x0, x1;
      x0.x = 0; x0.y = 0; x1 = x0;
      if (i0 < rows) x0 = sx[i0 * nrhs + w];
      if (i1 < rows) x1 = sx[i1 * nrhs + w];
      if (!UPPER) {
        for (int j = 0; j < rows; j++) {
          T v = (j < 32) ? x0 : x1;
          T xj;
          xj.x = __shfl_sync(0xffffffffu, v.x, j & 31);
          xj.y = __shfl_sync(0xffffffffu, v.y, j & 31);
          const T* col = sT + j * Ly::LDT;
          if (i0 > j && i0 < rows) x0 -= col[i0] * xj;
          if (i1 > j && i1 < rows) x1 -= col[i1] * xj;
        }
      } else {
        for (int j = rows - 1; j >= 0; j--) {
          T v = (j < 32) ? x0 : x1;
          T xj;
          xj.x = __shfl_sync(0xffffffffu, v.x, j & 31);
          xj.y = __shfl_sync(0xffffffffu, v.y, j & 31);
          xj = xj * sdinv[j];
          if (lane == (j & 31)) { if (j < 32) x0 = xj; else x1 = xj; }
          const T* col = sT + j * Ly::LDT;
          if (i0 < j) x0 -= col[i0] * xj;
          if (i1 < j) x1 -= col[i1] * xj;
        }
      }
      if (i0 < rows) Y[(size_t)(r0 + i0) * nrhs + w] = x0;
      if (i1 < rows) Y[(size_t)(r0 + i1) * nrhs + w] = x1;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicExch(flags + b, 1);
  }
}

template <class T, int UPPER>
static int trsv_flags(const T* LU, size_t lda, int n, T* Y, int nrhs, int* flags, int* err, cudaStream_t st) {
  const size_t sm = TrsvLayout<T>::SMEM;
  GB_CUDA(cudaFuncSetAttribute(k_trsv_flags<T, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int dev = 0, nsm = 0, occ = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_trsv_flags<T, UPPER>, TRSV_THREADS, sm));
  const int nbk = (n + LU_NB - 1) / LU_NB;
  int grid = nsm * (occ > 0 ? occ : 1);
  if (grid > nbk) grid = nbk;
  const int vec = ((((uintptr_t)LU) & 15) == 0 && ((lda * sizeof(T)) & 15) == 0) ? 1 : 0;
  GB_CUDA(cudaMemsetAsync(flags, 0, (size_t)nbk * sizeof(int), st));
  void* args[] = {(void*)&LU, (void*)&lda, (void*)&n, (void*)&Y, (void*)&nrhs, (void*)&flags, (void*)&err, (void*)&vec};
  GB_CUDA(cudaLaunchCooperativeKernel((const void*)k_trsv_flags<T, UPPER>, dim3(grid), dim3(TRSV_THREADS), args, sm, st));
  gbi_count_launch();
  return 0;
}

// Y <- (LU)^-1 P X for nrhs <= 8 columns; X (ldx) is read, Y (n x nrhs, packed)
// written; a forward and a backward cooperative launch (k_trsv_flags).  The
// time-out flag is checked once at the end (one host synchronisation).
template <class T>
static int lu_solve_multi(const T* LU, size_t lda, int n, const int* perm, const T* X, size_t ldx, int nrhs, T* Y,
                          cudaStream_t st) {
  if (nrhs < 1 || nrhs > 8) { gbi_set_error("lu_solve_multi: nrhs %d not in 1..8", nrhs); return -1; }
  size_t tot = (size_t)n * nrhs;
  const int nbk = (n + LU_NB - 1) / LU_NB;
  int* flags = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&flags, ((size_t)nbk + 1) * sizeof(int), st));
  int* err = flags + nbk;
  GB_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  k_gather_rows<T><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(X, ldx, n, nrhs, perm, Y);
  gbi_count_launch();
  int rc = trsv_flags<T, 0>(LU, lda, n, Y, nrhs, flags, err, st);
  if (!rc) rc = trsv_flags<T, 1>(LU, lda, n, Y, nrhs, flags, err, st);
  int herr = 0;
  if (!rc && (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("lu_solve_multi: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  cudaFreeAsync(flags, st);
  if (!rc && herr) { gbi_set_error("lu_solve_multi: a block wait timed out"); rc = -1; }
  if (!rc) GB_CUDA(cudaGetLastError());
  return rc;
}
extern "C" int gbi_zsolve_multi(const cplx* LU, size_t lda, int n, const int* perm, const cplx* X, size_t ldx, int nrhs,
                                cplx* Y, cudaStream_t st) {
  return lu_solve_multi<cplx>(LU, lda, n, perm, X, ldx, nrhs, Y, st);
}
extern "C" int gbi_csolve_multi(const cplxf* LU, size_t lda, int n, const int* perm, const cplxf* X, size_t ldx, int nrhs,
                                cplxf* Y, cudaStream_t st) {
  return lu_solve_multi<cplxf>(LU, lda, n, perm, X, ldx, nrhs, Y, st);
}

extern "C" int gbi_cgetrf(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
extern "C" int gbi_make_perm(const int64_t* ipiv, int n, int* perm, cudaStream_t st);

// R = B - A X for A n x n, X and B n x nrhs packed (nrhs <= 8); one warp per row
__global__ void k_resid_multi(const cplx* __restrict__ A, int n, const cplx* __restrict__ X, const cplx* __restrict__ B,
                              int nrhs, cplx* R) {
  const int lane = threadIdx.x & 31;
  const int row = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (row >= n) return;
  const cplx* a = A + (size_t)row * n;
  double sr[8], si[8];
  for (int c = 0; c < 8; c++) { sr[c] = 0.0; si[c] = 0.0; }
  for (int j = lane; j < n; j += 32) {
    const cplx av = a[j];
    for (int c = 0; c < nrhs; c++) {
      const cplx xv = X[(size_t)j * nrhs + c];
      sr[c] = fma(av.x, xv.x, fma(-av.y, xv.y, sr[c]));
      si[c] = fma(av.x, xv.y, fma(av.y, xv.x, si[c]));
    }
  }
  for (int c = 0; c < nrhs; c++)
    for (int o = 16; o > 0; o >>= 1) {
      sr[c] += __shfl_down_sync(0xffffffffu, sr[c], o);
      si[c] += __shfl_down_sync(0xffffffffu, si[c], o);
    }
  if (lane == 0)
    for (int c = 0; c < nrhs; c++) {
      const cplx b = B[(size_t)row * nrhs + c];
      R[(size_t)row * nrhs + c] = cmk(b.x - sr[c], b.y - si[c]);
    }
}

// FP32 factors of A (n x n, FP64 input) into A32: randomised without
// interchanges (rbt: butterfly parameters on the device) or with tournament
// pivoting; *hinfo: first zero pivot (0: none)
static int factor32_dense(const cplx* A, int n, cplxf* A32, int64_t* ipiv, int* perm, int* info, const float* rbt,
                          int* hinfo, cudaStream_t st) {
  const size_t nn = (size_t)n * n;
  int rc = gbi_to_c64(A, A32, nn, st);
  if (rbt) {
    if (!rc) rc = gbi_rbt_matrix(A32, n, n, rbt, rbt + 2 * (size_t)n, st);
    if (!rc) rc = gbi_cgetrf_nopiv(A32, n, n, ipiv, info, st);
  } else if (!rc) {
    rc = gbi_cgetrf(A32, n, n, ipiv, info, st);
  }
  if (!rc) rc = rbt ? gbi_perm_identity(n, perm, st) : gbi_make_perm(ipiv, n, perm, st);
  *hinfo = 0;
  if (!rc && (cudaMemcpyAsync(hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("gbi_zgesv_mixed: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  return rc;
}

// A X = B (FP64, n x n, nrhs <= 8 packed columns) by FP32 factors and FP64
// refinement to a relative residual of 1e-13; the factors are of the
// butterfly-randomised matrix without interchanges when n is divisible by 4,
// with tournament pivoting after a zero pivot or a refinement that does not
// contract the residual 10x per correction (and when n is not)
extern "C" int gbi_zgesv_mixed(const cplx* A, int n, const cplx* B, int nrhs, cplx* X, int* iters, double* relres,
                               cudaStream_t st) {
  if (nrhs < 1 || nrhs > 8) { gbi_set_error("gbi_zgesv_mixed: nrhs %d not in 1..8", nrhs); return -1; }
  const size_t nn = (size_t)n * n, nb = (size_t)n * nrhs;
  cplxf *A32 = nullptr, *D = nullptr, *Y = nullptr;
  cplx* R = nullptr;
  int64_t* ipiv = nullptr;
  int *perm = nullptr, *info = nullptr;
  double* nrm = nullptr;
  float* rbt = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&A32, nn * sizeof(cplxf), st));
  GB_CUDA(cudaMallocAsync((void**)&D, nb * sizeof(cplxf), st));
  GB_CUDA(cudaMallocAsync((void**)&Y, nb * sizeof(cplxf), st));
  GB_CUDA(cudaMallocAsync((void**)&R, nb * sizeof(cplx), st));
  GB_CUDA(cudaMallocAsync((void**)&ipiv, (size_t)n * sizeof(int64_t), st));
  GB_CUDA(cudaMallocAsync((void**)&perm, (size_t)n * sizeof(int), st));
  GB_CUDA(cudaMallocAsync((void**)&info, sizeof(int), st));
  GB_CUDA(cudaMallocAsync((void**)&nrm, 2 * sizeof(double), st));
  int rc = 0;
  if (n % 4 == 0 && n >= 4) {
    std::vector<float> h(4 * (size_t)n);
    gbi_rbt_params(n, h.data());
    GB_CUDA(cudaMallocAsync((void**)&rbt, h.size() * sizeof(float), st));
    if (cudaMemcpyAsync(rbt, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
  }
  int hinfo = 0;
  if (!rc) rc = factor32_dense(A, n, A32, ipiv, perm, info, rbt, &hinfo, st);
  if (!rc && rbt && hinfo) {
    cudaFreeAsync(rbt, st);
    rbt = nullptr;
    rc = factor32_dense(A, n, A32, ipiv, perm, info, nullptr, &hinfo, st);
  }
  if (!rc && hinfo) { gbi_set_error("mixed solve: FP32 factor singular (info=%d)", hinfo); rc = -1; }
  if (!rc && (cudaMemsetAsync(X, 0, nb * sizeof(cplx), st) != cudaSuccess ||
              cudaMemcpyAsync(R, B, nb * sizeof(cplx), cudaMemcpyDeviceToDevice, st) != cudaSuccess))
    rc = -1;
  double rel = 1.0, prev = 1.0;
  int it = 0, since = 0;
  const unsigned gb = (unsigned)((nb + 255) / 256);
  for (; !rc && it < 31; it++, since++) {
    if (it > 0) {
      // R = B - A X (FP64)
      k_resid_multi<<<(unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, st>>>(A, n, X, B, nrhs, R);
      gbi_count_launch();
      if (cudaMemsetAsync(nrm, 0, 2 * sizeof(double), st) != cudaSuccess) { rc = -1; break; }
      k_sqnorm<<<gb, 256, 0, st>>>(R, nb, nrm);
      k_sqnorm<<<gb, 256, 0, st>>>(B, nb, nrm + 1);
      gbi_count_launch();
      gbi_count_launch();
      double h[2];
      if (cudaMemcpyAsync(h, nrm, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) { rc = -1; break; }
      prev = rel;
      rel = (h[1] > 0.0) ? sqrt(h[0] / h[1]) : 0.0;
      if (rel <= 1e-13) break;
      if (rbt && ((since >= 2 && rel > 0.1 * prev && rel > 1e-11) || since >= 12 || !(rel < 1e3))) {
        cudaFreeAsync(rbt, st);
        rbt = nullptr;
        rc = factor32_dense(A, n, A32, ipiv, perm, info, nullptr, &hinfo, st);
        if (!rc && hinfo) { gbi_set_error("mixed solve: FP32 factor singular (info=%d)", hinfo); rc = -1; }
        if (rc) break;
        if (!(rel < 1.0) &&
            (cudaMemsetAsync(X, 0, nb * sizeof(cplx), st) != cudaSuccess ||
             cudaMemcpyAsync(R, B, nb * sizeof(cplx), cudaMemcpyDeviceToDevice, st) != cudaSuccess)) { rc = -1; break; }
        since = 0;
      }
    }
    const int q = n / 4;
    if (rbt) {
      k_rbt_ut<<<(unsigned)(((size_t)q * nrhs + 255) / 256), 256, 0, st>>>(R, D, n, nrhs, rbt);
      gbi_count_launch();
      if (lu_solve_multi<cplxf>(A32, n, n, perm, D, nrhs, nrhs, Y, st)) { rc = -1; break; }
      k_rbt_axpy_v<<<(unsigned)(((size_t)q * nrhs + 255) / 256), 256, 0, st>>>(X, Y, n, nrhs, rbt + 2 * (size_t)n);
      gbi_count_launch();
    } else {
      k_c128_to_c64_scaled<<<gb, 256, 0, st>>>(R, D, (int)nb);
      gbi_count_launch();
      if (lu_solve_multi<cplxf>(A32, n, n, perm, D, nrhs, nrhs, Y, st)) { rc = -1; break; }
      k_axpy_c64<<<gb, 256, 0, st>>>(X, Y, (int)nb);
      gbi_count_launch();
    }
  }
  cudaFreeAsync(rbt, st);
  if (iters) *iters = it;
  if (relres) *relres = rel;
  if (!rc && rel > 1e-10) { gbi_set_error("mixed solve: refinement stalled at relative residual %g", rel); rc = -1; }
  cudaFreeAsync(A32, st); cudaFreeAsync(D, st); cudaFreeAsync(Y, st); cudaFreeAsync(R, st);
  cudaFreeAsync(ipiv, st); cudaFreeAsync(perm, st); cudaFreeAsync(info, st); cudaFreeAsync(nrm, st);
  if (!rc) GB_CUDA(cudaGetLastError());
  return rc;
}

// ------------------------------------------------------------------ FP32 inverse
// X = P I for the permutation of gbi_make_perm: row i of X is e_perm[i]
__global__ void k_perm_identity_c64(cplxf* X, size_t ldx, int n, const int* perm) {
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n * n) return;
  const int i = (int)(p / n), j = (int)(p % n);
  X[(size_t)i * ldx + j] = cmkf(j == perm[i] ? 1.0f : 0.0f, 0.0f);
}

// X <- U^-1 L^-1 X (X n x nrhs, row-major) with the factors of an LU in LU;
// two-level blocking as in lu_factor: inside an outer block of LU_NBO rows the
// LU_NB-row diagonal blocks are solved by k_trsm_rows and update only the
// outer block (K = LU_NB), the rows beyond it are updated once per outer block
// (K = LU_NBO).  gemm(M, N, K, A, lda, B, ldb, C, ldc, st): C -= A B.
template <class T, class GEMM>
static int lu_solve_blocked(const T* LU, size_t lda, int n, T* X, size_t ldx, int nrhs, cudaStream_t st, GEMM gemm) {
  for (int K0 = 0; K0 < n; K0 += LU_NBO) {  // forward: L Y = X
    const int Kend = (K0 + LU_NBO < n) ? K0 + LU_NBO : n;
    for (int i0 = K0; i0 < Kend; i0 += LU_NB) {
      const int ib = (Kend - i0 < LU_NB) ? Kend - i0 : LU_NB;
      if (trsm_rows<T>(0, LU + (size_t)i0 * lda + i0, lda, X + (size_t)i0 * ldx, ldx, ib, 0, nrhs, st)) return -1;
      if (i0 + ib < Kend && gemm(Kend - i0 - ib, nrhs, ib, LU + (size_t)(i0 + ib) * lda + i0, lda, X + (size_t)i0 * ldx,
                                 ldx, X + (size_t)(i0 + ib) * ldx, ldx, st))
        return -1;
    }
    if (Kend < n && gemm(n - Kend, nrhs, Kend - K0, LU + (size_t)Kend * lda + K0, lda, X + (size_t)K0 * ldx, ldx,
                         X + (size_t)Kend * ldx, ldx, st))
      return -1;
  }
  for (int K0 = ((n - 1) / LU_NBO) * LU_NBO; K0 >= 0; K0 -= LU_NBO) {  // backward: U X = Y
    const int Kend = (K0 + LU_NBO < n) ? K0 + LU_NBO : n;
    for (int i0 = K0 + ((Kend - 1 - K0) / LU_NB) * LU_NB; i0 >= K0; i0 -= LU_NB) {
      const int ib = (Kend - i0 < LU_NB) ? Kend - i0 : LU_NB;
      if (trsm_rows<T>(1, LU + (size_t)i0 * lda + i0, lda, X + (size_t)i0 * ldx, ldx, ib, 0, nrhs, st)) return -1;
      if (i0 > K0 && gemm(i0 - K0, nrhs, ib, LU + (size_t)K0 * lda + i0, lda, X + (size_t)i0 * ldx, ldx,
                          X + (size_t)K0 * ldx, ldx, st))
        return -1;
    }
    if (K0 > 0 && gemm(K0, nrhs, Kend - K0, LU + K0, lda, X + (size_t)K0 * ldx, ldx, X, ldx, st)) return -1;
  }
  return 0;
}

// X = A^-1 (complex FP32, n x n) from the factors of gbi_cgetrf (LU, perm of
// gbi_make_perm), the updates on the tensor cores (split TF32, three passes)
extern "C" int gbi_cinverse_tc(const cplxf* LU, size_t lda, int n, const int* perm, cplxf* X, size_t ldx,
                               cudaStream_t st) {
  if (n <= 0) return 0;
  const size_t nn = (size_t)n * n;
  k_perm_identity_c64<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(X, ldx, n, perm);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  float* scratch = nullptr;
  int* err = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&scratch, gbi_tc_scratch_floats(n, n, LU_NBO) * sizeof(float), st));
  GB_CUDA(cudaMallocAsync((void**)&err, 16, st));
  GB_CUDA(cudaMemsetAsync(err, 0, 4, st));
  auto tc = [scratch, err](int M, int N, int K, const cplxf* a, size_t la, const cplxf* b, size_t lb, cplxf* c, size_t lc,
                           cudaStream_t s) { return gbi_tc_cgemm_sub(M, N, K, a, la, b, lb, c, lc, gbi_tc_passes(), scratch, err, s); };
  int rc = lu_solve_blocked<cplxf>(LU, lda, n, X, ldx, n, st, tc);
  int h = 0;
  if (!rc && (cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("FP32 inverse: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  cudaFreeAsync(scratch, st);
  cudaFreeAsync(err, st);
  if (!rc && h) {
    gbi_set_error("FP32 inverse: a tensor-core pipeline wait timed out");
    rc = -1;
  }
  return rc;
}

// ---- outer block size of the blocked LU / inverse, and its tuner
extern "C" int gb_set_lu_outer_block(int nbo) {
  if (nbo < LU_NB || nbo > 2048 || nbo % LU_NB) {
    gbi_set_error("gb_set_lu_outer_block: %d is not a multiple of %d in %d..2048", nbo, LU_NB, LU_NB);
    return -1;
  }
  g_lu_nbo.store(nbo);
  return 0;
}
extern "C" int gb_lu_outer_block(void) { return g_lu_nbo.load(); }

// seeded diagonally dominant complex test matrix (an integer hash per entry)
__global__ void k_tune_matrix(cplxf* A, int n) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n * n) return;
  unsigned h = (unsigned)p * 2654435761u + 12345u;
  h ^= h >> 15; h *= 2246822519u; h ^= h >> 13;
  const float a = (float)(h & 0xffff) / 65536.0f - 0.5f, b = (float)(h >> 16) / 65536.0f - 0.5f;
  const int i = (int)(p / n), j = (int)(p % n);
  A[p] = cmkf(a + (i == j ? (float)n * 0.05f : 0.0f), b);
}

// Times the FP32 LU (without interchanges) and inverse of an n x n test
// matrix with outer blocks of 128, 256, 512 and 1024 columns (second of two
// runs each, CUDA events), sets the fastest (gb_set_lu_outer_block) and
// returns it in *best, the four times (ms) in ms[4].
extern "C" int gb_tune_lu_outer_block(int n, int* best, double* ms) {
  if (n < 2 * LU_NB) { gbi_set_error("gb_tune_lu_outer_block: order %d below %d", n, 2 * LU_NB); return -1; }
  const int cand[4] = {128, 256, 512, 1024};
  const size_t nn = (size_t)n * n;
  cudaStream_t st = nullptr;
  GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  cplxf *A = nullptr, *LU = nullptr, *X = nullptr;
  int64_t* ipiv = nullptr;
  int *perm = nullptr, *info = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = 0;
  if (cudaMalloc((void**)&A, nn * sizeof(cplxf)) != cudaSuccess || cudaMalloc((void**)&LU, nn * sizeof(cplxf)) != cudaSuccess ||
      cudaMalloc((void**)&X, nn * sizeof(cplxf)) != cudaSuccess || cudaMalloc((void**)&ipiv, (size_t)n * sizeof(int64_t)) != cudaSuccess ||
      cudaMalloc((void**)&perm, (size_t)n * sizeof(int)) != cudaSuccess || cudaMalloc((void**)&info, sizeof(int)) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    gbi_set_error("gb_tune_lu_outer_block: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  const int keep = g_lu_nbo.load();
  double bestms = 1e300;
  int bestc = keep;
  if (!rc) {
    k_tune_matrix<<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(A, n);
    gbi_count_launch();
  }
  for (int c = 0; c < 4 && !rc; c++) {
    g_lu_nbo.store(cand[c]);
    float t = 0.0f;
    for (int rep = 0; rep < 2 && !rc; rep++) {
      if (cudaMemcpyAsync(LU, A, nn * sizeof(cplxf), cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
          cudaEventRecord(e0, st) != cudaSuccess) { rc = -1; break; }
      rc = gbi_cgetrf_nopiv(LU, (size_t)n, n, ipiv, info, st);
      if (!rc) rc = gbi_make_perm(ipiv, n, perm, st);
      if (!rc) rc = gbi_cinverse_tc(LU, (size_t)n, n, perm, X, (size_t)n, st);
      if (!rc && (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                  cudaEventElapsedTime(&t, e0, e1) != cudaSuccess)) rc = -1;
    }
    ms[c] = t;
    if (!rc && t < bestms) { bestms = t; bestc = cand[c]; }
  }
  g_lu_nbo.store(rc ? keep : bestc);
  *best = g_lu_nbo.load();
  if (st) cudaStreamSynchronize(st);
  cudaFree(A); cudaFree(LU); cudaFree(X); cudaFree(ipiv); cudaFree(perm); cudaFree(info);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return rc;
}
