// gb_linalg.cu -- dense complex linear algebra of the BEM hot path (FP64).
//
// Replaces, on the GPU:
//   create_Amatrix_csr(_dac)  reference solve_bieq2.c:186-341 (coupled matrix A;
//                             built dense in HBM directly from G,H: no CSR files)
//   lu_dec_A                  solve_bieq2.c:343-408 (MKL zgetrf + zgetri)
//   solve_ABmatrix            mo_solve.c:246-274 (invA * B, streamed from disk there)
//   LAPACKE_zgesv             mo_solve.c:751 (dE/dn, dH/dn with 6 right-hand sides)
// All matrices are row-major, as in the reference's files.
//
// LU: right-looking blocked factorisation with partial pivoting (LAPACK's
// pivot rule: first index of max |Re|+|Im|).  Per panel of NB columns:
//   k_pivot_swap   one block: pivot search in column j, full-row interchange
//   k_panel_update warp per row: scale column j, rank-1 update of the panel
//   k_trsm_rows    U12 = L11^-1 A12 (L11 unit lower, staged in shared memory)
//   k_zgemm_nn     A22 -= L21 U12 (complex FP64 GEMM, 64x64 tiles, DFMA)
// The inverse solves A X = I through the factors: X = U^-1 (L^-1 (P I)),
// two blocked triangular solves whose updates use the same GEMM kernel.
#include "gb_common.cuh"
#include "gb_internal.h"

#define LU_NB 64

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

// ------------------------------------------------------------------ LU
__device__ __forceinline__ double cabs1(cplx a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double cabs1(cplxf a) { return (double)(fabsf(a.x) + fabsf(a.y)); }

// pivot search in column j over rows j..n-1, then the full-row interchange;
// info[0] receives j+1 on an exactly zero pivot (LAPACK's info convention)
template <class T>
__global__ void __launch_bounds__(1024) k_pivot_swap(T* A, size_t lda, int n, int j, int64_t* ipiv, int* info) {
  __shared__ double sv[32];
  __shared__ int si[32];
  double best = -1.0;
  int bi = n;
  for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
    double v = cabs1(A[(size_t)i * lda + j]);
    if (v > best) { best = v; bi = i; }
  }
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, best, o);
    int oi = __shfl_down_sync(0xffffffffu, bi, o);
    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { sv[w] = best; si[w] = bi; }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    best = lane < nw ? sv[lane] : -1.0;
    bi = lane < nw ? si[lane] : n;
    for (int o = 16; o > 0; o >>= 1) {
      double ov = __shfl_down_sync(0xffffffffu, best, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if (lane == 0) { si[0] = bi; sv[0] = best; }
  }
  __syncthreads();
  int p = si[0];
  if (threadIdx.x == 0) {
    ipiv[j] = p;
    if (!(sv[0] > 0.0) && info[0] == 0) info[0] = j + 1;
  }
  if (p != j) {
    T* rj = A + (size_t)j * lda;
    T* rp = A + (size_t)p * lda;
    for (int c = threadIdx.x; c < n; c += blockDim.x) {
      T t = rj[c];
      rj[c] = rp[c];
      rp[c] = t;
    }
  }
}

// rows i > j: l = A[i][j] / A[j][j]; A[i][c] -= l A[j][c] for c in (j, kend)
template <class T>
__global__ void k_panel_update(T* A, size_t lda, int n, int j, int kend) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  int i = j + 1 + warp;
  if (i >= n) return;
  T piv = A[(size_t)j * lda + j];
  T* ri = A + (size_t)i * lda;
  const T* rj = A + (size_t)j * lda;
  T l = (piv.x == 0 && piv.y == 0) ? ri[j] : cdivc(ri[j], piv);
  for (int c = j + 1 + lane; c < kend; c += 32) ri[c] -= l * rj[c];
  if (lane == 0) ri[j] = l;
}

// Rows k..k+nb-1, columns [c0, c1): X <- L11^-1 X with L11 the unit lower
// triangle of A[k:k+nb][k:k+nb] (or, with upper = 1, X <- U11^-1 X with the
// non-unit upper triangle), one thread per column.  Lsrc gives the triangle's
// storage (row-major, leading dimension ldl).
template <class T, int UPPER>
__global__ void __launch_bounds__(128) k_trsm_rows(const T* Lsrc, size_t ldl, T* X, size_t ldx, int nb, int c0,
                                                   int c1) {
  extern __shared__ __align__(16) unsigned char sLraw[];
  T* sL = (T*)sLraw;  // nb*nb
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) sL[t] = Lsrc[(size_t)(t / nb) * ldl + (t % nb)];
  __syncthreads();
  int c = c0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= c1) return;
  T x[LU_NB];
#pragma unroll
  for (int i = 0; i < LU_NB; i++)
    if (i < nb) x[i] = X[(size_t)i * ldx + c];
  if (!UPPER) {
#pragma unroll
    for (int i = 0; i < LU_NB; i++) {
      if (i >= nb) break;
      T s = x[i];
#pragma unroll
      for (int jj = 0; jj < LU_NB; jj++) {
        if (jj >= i) break;
        s -= sL[i * nb + jj] * x[jj];
      }
      x[i] = s;
    }
  } else {
#pragma unroll
    for (int i = LU_NB - 1; i >= 0; i--) {
      if (i >= nb) continue;
      T s = x[i];
#pragma unroll
      for (int jj = LU_NB - 1; jj >= 0; jj--) {
        if (jj <= i) break;
        if (jj < nb) s -= sL[i * nb + jj] * x[jj];
      }
      x[i] = cdivc(s, sL[i * nb + i]);
    }
  }
#pragma unroll
  for (int i = 0; i < LU_NB; i++)
    if (i < nb) X[(size_t)i * ldx + c] = x[i];
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
  size_t sm = (size_t)nb * nb * sizeof(T);
  unsigned nblk = (unsigned)((c1 - c0 + 127) / 128);
  if (upper) {
    GB_CUDA(cudaFuncSetAttribute(k_trsm_rows<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_trsm_rows<T, 1><<<nblk, 128, sm, st>>>(L, ldl, X, ldx, nb, c0, c1);
    gbi_count_launch();
  } else {
    GB_CUDA(cudaFuncSetAttribute(k_trsm_rows<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_trsm_rows<T, 0><<<nblk, 128, sm, st>>>(L, ldl, X, ldx, nb, c0, c1);
    gbi_count_launch();
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

// In-place LU of the n x n row-major matrix A (lda); ipiv[j] = 0-based row
// interchanged with row j (rows are swapped across the full width).
// info (device int) receives LAPACK's info (0: success).
template <class T, class GEMM>
static int lu_factor(T* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st, GEMM gemm) {
  GB_CUDA(cudaMemsetAsync(info, 0, sizeof(int), st));
  for (int k = 0; k < n; k += LU_NB) {
    int nb = (n - k < LU_NB) ? n - k : LU_NB;
    int kend = k + nb;
    for (int j = k; j < kend; j++) {
      k_pivot_swap<T><<<1, 1024, 0, st>>>(A, lda, n, j, ipiv, info);
      gbi_count_launch();
      GB_CUDA(cudaGetLastError());
      int rows = n - j - 1;
      if (rows > 0) {
        unsigned nbk = (unsigned)((rows * 32 + 255) / 256);
        k_panel_update<T><<<nbk, 256, 0, st>>>(A, lda, n, j, kend);
        gbi_count_launch();
        GB_CUDA(cudaGetLastError());
      }
    }
    if (kend < n) {
      if (trsm_rows<T>(0, A + (size_t)k * lda + k, lda, A + (size_t)k * lda, lda, nb, kend, n, st)) return -1;
      if (gemm(n - kend, n - kend, nb, A + (size_t)kend * lda + k, lda, A + (size_t)k * lda + kend, lda,
               A + (size_t)kend * lda + kend, lda, st))
        return -1;
    }
  }
  return 0;
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

extern "C" int gbi_cgetrf(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st) {
  return lu_factor<cplxf>(A, lda, n, ipiv, info, st, cgemm_sub);
}

extern "C" int gbi_cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C,
                             size_t ldc, cudaStream_t st) {
  return cgemm_sub(M, N, K, A, lda, B, ldb, C, ldc, st);
}

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

// ---- single right-hand side solve with LU factors (row-major, in place on x)
// x <- P x (interchanges in order)
template <class T>
__global__ void k_perm1(T* x, int n, const int64_t* ipiv) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int j = 0; j < n; j++) {
    int p = (int)ipiv[j];
    if (p != j) { T t = x[j]; x[j] = x[p]; x[p] = t; }
  }
}
// diagonal block k0..k0+nb-1: unit lower (UPPER = 0) or non-unit upper solve,
// column-oriented sweep, one thread per row of the block
template <class T, int UPPER>
__global__ void k_trsv_diag(const T* LU, size_t lda, int k0, int nb, T* x) {
  __shared__ T xs[LU_NB];
  int i = threadIdx.x;
  if (i < nb) xs[i] = x[k0 + i];
  __syncthreads();
  if (!UPPER) {
    for (int j = 0; j < nb; j++) {
      T xj = xs[j];
      __syncthreads();
      if (i > j && i < nb) xs[i] -= LU[(size_t)(k0 + i) * lda + k0 + j] * xj;
      __syncthreads();
    }
  } else {
    for (int j = nb - 1; j >= 0; j--) {
      if (i == j) xs[j] = cdivc(xs[j], LU[(size_t)(k0 + j) * lda + k0 + j]);
      __syncthreads();
      T xj = xs[j];
      if (i < j) xs[i] -= LU[(size_t)(k0 + i) * lda + k0 + j] * xj;
      __syncthreads();
    }
  }
  if (i < nb) x[k0 + i] = xs[i];
}
// rows r in [r0, r1): x[r] -= sum_j LU[r][k0+j] x[k0+j], j < nb (warp per row)
template <class T>
__global__ void k_trsv_update(const T* LU, size_t lda, int r0, int r1, int k0, int nb, T* x) {
  int w = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  int lane = threadIdx.x & 31;
  int r = r0 + w;
  if (r >= r1) return;
  const T* row = LU + (size_t)r * lda + k0;
  double sr = 0.0, si = 0.0;
  for (int j = lane; j < nb; j += 32) {
    T a = row[j], b = x[k0 + j];
    sr += (double)a.x * (double)b.x - (double)a.y * (double)b.y;
    si += (double)a.x * (double)b.y + (double)a.y * (double)b.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (lane == 0) { x[r].x -= sr; x[r].y -= si; }
}

template <class T>
static int lu_solve1(const T* LU, size_t lda, int n, const int64_t* ipiv, T* x, cudaStream_t st) {
  k_perm1<T><<<1, 32, 0, st>>>(x, n, ipiv);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  for (int k = 0; k < n; k += LU_NB) {
    int nb = (n - k < LU_NB) ? n - k : LU_NB;
    k_trsv_diag<T, 0><<<1, LU_NB, 0, st>>>(LU, lda, k, nb, x);
    gbi_count_launch();
    int rows = n - k - nb;
    if (rows > 0) {
      k_trsv_update<T><<<(unsigned)(((size_t)rows * 32 + 255) / 256), 256, 0, st>>>(LU, lda, k + nb, n, k, nb, x);
      gbi_count_launch();
    }
  }
  int last = ((n - 1) / LU_NB) * LU_NB;
  for (int k = last; k >= 0; k -= LU_NB) {
    int nb = (n - k < LU_NB) ? n - k : LU_NB;
    k_trsv_diag<T, 1><<<1, LU_NB, 0, st>>>(LU, lda, k, nb, x);
    gbi_count_launch();
    if (k > 0) {
      k_trsv_update<T><<<(unsigned)(((size_t)k * 32 + 255) / 256), 256, 0, st>>>(LU, lda, 0, k, k, nb, x);
      gbi_count_launch();
    }
  }
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbi_csolve1(const cplxf* LU, size_t lda, int n, const int64_t* ipiv, cplxf* x, cudaStream_t st) {
  return lu_solve1<cplxf>(LU, lda, n, ipiv, x, st);
}
extern "C" int gbi_zsolve1(const cplx* LU, size_t lda, int n, const int64_t* ipiv, cplx* x, cudaStream_t st) {
  return lu_solve1<cplx>(LU, lda, n, ipiv, x, st);
}

// r = b - A x (FP64), and the squared norms of r and b accumulated into nrm[0], nrm[1]
__global__ void k_residual(const cplx* __restrict__ A, size_t lda, int n, const cplx* __restrict__ x,
                           const cplx* __restrict__ b, cplx* r, double* nrm) {
  int w = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  int lane = threadIdx.x & 31;
  if (w >= n) return;
  const cplx* row = A + (size_t)w * lda;
  double sr = 0.0, si = 0.0;
  for (int j = lane; j < n; j += 32) {
    cplx a = row[j], v = x[j];
    sr = fma(a.x, v.x, sr);
    sr = fma(-a.y, v.y, sr);
    si = fma(a.x, v.y, si);
    si = fma(a.y, v.x, si);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (lane == 0) {
    cplx rr = cmk(b[w].x - sr, b[w].y - si);
    r[w] = rr;
    atomicAdd(nrm, rr.x * rr.x + rr.y * rr.y);
    atomicAdd(nrm + 1, b[w].x * b[w].x + b[w].y * b[w].y);
  }
}
extern "C" int gbi_residual(const cplx* A, size_t lda, int n, const cplx* x, const cplx* b, cplx* r, double* nrm,
                            cudaStream_t st) {
  GB_CUDA(cudaMemsetAsync(nrm, 0, 2 * sizeof(double), st));
  k_residual<<<(unsigned)(((size_t)n * 32 + 255) / 256), 256, 0, st>>>(A, lda, n, x, b, r, nrm);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// x += (cplx) d ; also converts: d64 -> d32 helper
__global__ void k_axpy_c64(cplx* x, const cplxf* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { x[i].x += (double)d[i].x; x[i].y += (double)d[i].y; }
}
__global__ void k_c128_to_c64_scaled(const cplx* r, cplxf* d, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = cmkf((float)r[i].x, (float)r[i].y);
}
extern "C" int gbi_ir_step(cplx* x, const cplx* r, cplxf* d, const cplxf* LU32, size_t lda, int n, const int64_t* ipiv,
                           cudaStream_t st) {
  k_c128_to_c64_scaled<<<(n + 255) / 256, 256, 0, st>>>(r, d, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  if (lu_solve1<cplxf>(LU32, lda, n, ipiv, d, st)) return -1;
  k_axpy_c64<<<(n + 255) / 256, 256, 0, st>>>(x, d, n);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}
