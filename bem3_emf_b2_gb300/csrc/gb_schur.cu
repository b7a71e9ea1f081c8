// gb_schur.cu -- block elimination of the coupled system of an object whose
// elements all lie on one interface (exterior domain 0 outside, domain 1
// inside): the correction solve through node-sized inverses instead of the
// dense factors of the 8 NN x 8 NN coupled matrix.  Two arithmetics share the
// code: complex FP32 (the chosen form: tensor-core LUs and inverses, FP64
// refinement around the corrections) and complex FP64 (the plain FP64 form
// for objects whose dense inverse does not fit: one correction reaches the
// rounding level).
//
// The coupled matrix of such an object (reference solve_bieq2.c:241-316, built
// densely by k_build_A) with G_d, H_d the domain-d coefficient matrices
// gathered to node columns (rows: the domain's collocation rows in order),
// D_c the diagonal of the c-th component of the nodes' unit normals, unknown
// node vectors U_0..U_3, dU_0..dU_3 and right-hand sides re_c (domain-0 rows),
// ri_c (domain-1 rows):
//   H0 U_c - G0 dU_c                               = re_c     c = 0..3
//   H1 U_c + delta G1 D_c U_3 + G1 dU_c            = ri_c     c = 0..2
//   sigma G1 sum_c D_c U_c + H1 U_3 + beta G1 dU_3 = ri_3
// with delta = k0^2 - k1^2, beta = k0^2 / k1^2, sigma = 1 - beta.  With
// X_d = G_d^-1 H_d, the exterior rows give dU_c = X0 U_c - G0^-1 re_c;
// substituted into the interior rows multiplied by G1^-1:
//   M U_c + delta D_c U_3 = y_c,      y_c = G1^-1 ri_c + G0^-1 re_c   (c < 3)
//   sigma sum_c D_c U_c + M3 U_3 = y_3,  y_3 = G1^-1 ri_3 + beta G0^-1 re_3
// with M = X0 + X1 and M3 = X1 + beta X0; eliminating U_c (c < 3):
//   S U_3 = y_3 - sigma sum_c D_c M^-1 y_c,
//   S = M3 - sigma delta sum_c D_c M^-1 D_c,
//   U_c = M^-1 (y_c - delta D_c U_3),   dU_c = X0 U_c - G0^-1 re_c.
// Factorisation: G0^-1, G1^-1, X0, M^-1, S^-1 -- about 32 NN^3
// complex-equivalent flop against (8/3) (8 NN)^3 = 1365 NN^3 for the dense
// LU, and five NN x NN matrices instead of one (8 NN)^2.  The G0 chain
// (G0^-1, X0) and the G1 chain (G1^-1, X1) are independent and run at once on
// two streams from two host threads.  FP32 node LUs: the matrix is randomised
// by two-sided recursive butterflies (U^T A V) and factorised without row
// interchanges, the inverse of A is V (U^T A V)^-1 U^T; a zero pivot makes the
// caller fall back to the dense tournament factors.  FP64 node LUs use the
// tournament-pivoted FP64 LU of gb_linalg.cu.  A correction is six products
// of those matrices with at most four node vectors.
#include "gb_common.cuh"
#include "gb_internal.h"

#include <complex>
#include <string>
#include <thread>
#include <vector>

extern "C" {
int gbi_cgetrf(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
int gbi_cgetrf_nopiv(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
int gbi_make_perm(const int64_t* ipiv, int n, int* perm, cudaStream_t st);
int gbi_perm_identity(int n, int* perm, cudaStream_t st);
int gbi_cinverse_tc(const cplxf* LU, size_t lda, int n, const int* perm, cplxf* X, size_t ldx, cudaStream_t st);
int gbi_tc_cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C, size_t ldc,
                     int passes, float* scratch, int* err, cudaStream_t st);
int gbi_tc_passes(void);
void gbi_rbt_params(int n, float* h);
const char* gb_last_error(void);
int gbi_rbt_matrix(cplxf* A, size_t lda, int n, const float* pu, const float* pv, cudaStream_t st);
int gbi_rbt_inverse(cplxf* X, size_t ldx, int n, const float* pu, const float* pv, cudaStream_t st);
int gbi_zgetrf(cplx* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
int gbi_zinverse(const cplx* LU, size_t lda, int n, const int64_t* ipiv, cplx* X, size_t ldx, cudaStream_t st);
int gbi_zgemm_sub(int M, int N, int K, const cplx* A, size_t lda, const cplx* B, size_t ldb, cplx* C, size_t ldc,
                  cudaStream_t st);
}

// node vectors of the correction are kept four to a row: V[i * 4 + c]
#define SC_W 4

template <class T> struct SchurTy;
template <> struct SchurTy<cplx> {
  typedef double R;
  static __host__ __device__ __forceinline__ cplx from(cplx v) { return v; }
};
template <> struct SchurTy<cplxf> {
  typedef float R;
  static __host__ __device__ __forceinline__ cplxf from(cplx v) { return cmkf((float)v.x, (float)v.y); }
};
__device__ __forceinline__ float sfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double sfma(double a, double b, double c) { return fma(a, b, c); }

struct GbSchur {
  int n;
  int fp64;             // 1: complex FP64 matrices, 0: complex FP32
  size_t esz;           // bytes per matrix element
  void *G0i, *G1i, *nX0, *Minv, *Si;  // n x n each; nX0 = -X0
  void* vn;             // n x 3 unit normals of the nodes (double / float)
  void* work;           // 7 blocks of n x SC_W: R0 R1 T0 Y MY W U
  float* rbt;           // butterfly parameters of order n (FP32 node LUs), 4 n floats
  cplx beta, sigma, delta, sigdel;  // sigdel = sigma * delta
  cudaStream_t st2;     // second stream of the factorisation (the G1 chain)
  cudaEvent_t ev0, ev1;
};

// ---------------------------------------------------------------- factorisation
// Gather the domain matrices (N x N, rows (t-1)*4+tn, columns (s-1)*4+l) to
// node columns: out[rowk[row]][eni[|sid[s]|][l]]
template <class T>
__global__ void k_schur_gather(const cplx* __restrict__ G, const cplx* __restrict__ H, int N, const int* sid,
                               const int* rowk, const int* eni, const int* etype, int n, T* Gh, T* Hh) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)N * N) return;
  const int row = (int)(p / N), col = (int)(p % N);
  const int k = rowk[row];
  if (k < 0) return;
  const int e = abs(sid[(col >> 2) + 1]), l = col & 3;
  if (l == 3 && etype[e] == 0) return;
  const int c = eni[e * 4 + l];
  const size_t q = (size_t)k * n + c;
  Gh[q] = SchurTy<T>::from(G[p]);
  Hh[q] = SchurTy<T>::from(H[p]);
}

// unit normals of the nodes (the A build's vn: wen normalised)
template <class R>
__global__ void k_schur_normals(const double* wen, const int* eni, const int* etype, int Ne, R* vn) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= 4 * Ne) return;
  const int e = 1 + p / 4, l = p % 4;
  if (l == 3 && etype[e] == 0) return;
  const int c = eni[e * 4 + l];
  double w[3], a = 0.0;
  for (int d = 0; d < 3; d++) { w[d] = wen[(size_t)e * 12 + l * 3 + d]; a += w[d] * w[d]; }
  a = sqrt(a);
  for (int d = 0; d < 3; d++) vn[(size_t)c * 3 + d] = (R)(a != 0.0 ? w[d] / a : w[d]);
}

// M = -(nX0 + nX1) = X0 + X1 and M3 = -(nX1 + beta nX0) = X1 + beta X0
template <class T>
__global__ void k_schur_combine(const T* __restrict__ nX0, const T* __restrict__ nX1, size_t nn, T beta, T* M, T* M3) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nn) return;
  const T a = nX0[p], b = nX1[p];
  M[p] = czero<T>() - (a + b);
  M3[p] = czero<T>() - (b + beta * a);
}

// S = M3 - sigma delta (vn_i . vn_j) M^-1_ij
template <class T, class R>
__global__ void k_schur_s(T* S, const T* __restrict__ Minv, const R* __restrict__ vn, int n, T sigdel) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n * n) return;
  const int i = (int)(p / n), j = (int)(p % n);
  const R w = vn[i * 3] * vn[j * 3] + vn[i * 3 + 1] * vn[j * 3 + 1] + vn[i * 3 + 2] * vn[j * 3 + 2];
  S[p] -= (sigdel * Minv[p]) * w;
}

// ---------------------------------------------------------------- correction
// r (FP64, A's row order: domain-0 rows c*n + k, domain-1 rows 4n + c*n + k)
// -> R0[k][c] = re_c[k], R1[k][c] = ri_c[k]
template <class T>
__global__ void k_schur_in(const cplx* __restrict__ r, int n, T* R0, T* R1) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= 8 * (size_t)n) return;
  const int blk = (int)(p / n), k = (int)(p % n);
  const T f = SchurTy<T>::from(r[p]);
  if (blk < 4) R0[(size_t)k * SC_W + blk] = f;
  else R1[(size_t)k * SC_W + blk - 4] = f;
}

enum { SC_T0 = 0, SC_Y = 1, SC_MY = 2, SC_U3 = 3, SC_U = 4, SC_DU = 5 };

template <class T>
struct SchurMv {
  typedef typename SchurTy<T>::R R;
  const T* Mat;  // n x n
  int n;
  const T* X;    // n x SC_W; columns xoff .. xoff + NC - 1 are multiplied
  int xoff;
  T* out;        // n x SC_W
  const T* aux;  // n x SC_W (mode-dependent)
  const R* vn;
  T c0;          // beta (SC_Y), sigma (SC_MY), delta (SC_U)
  cplx* x;       // FP64 solution (SC_DU)
};

// acc_c = sum_j Mat[i][j] X[j][xoff + c] for row i (one warp), then the
// mode's epilogue by lane 0:
//   SC_T0  out = acc                                   (T0 = G0^-1 re)
//   SC_Y   out_c = acc_c + T0_c (c < 3), acc_3 + beta T0_3   (aux = T0)
//   SC_MY  out_c = acc_c (c < 3), out_3 = Y_3 - sigma sum_c vn_c acc_c   (X = Y)
//   SC_U3  out_c = vn_c acc_0 (c < 3), out_3 = acc_0   (X = MY, column 3)
//   SC_U   out_c = MY_c - delta acc_c (c < 3), out_3 = X_3   (X = W, aux = MY)
//   SC_DU  x[c n + i] += U_c, x[(4 + c) n + i] += -acc_c - T0_c   (Mat = -X0,
//          X = U, aux = T0)
// this lane's part of row i's sums, one matrix entry per lane and step
template <class T, int NC>
__device__ __forceinline__ void schur_row(const SchurMv<T>& a, int i, int lane, typename SchurTy<T>::R* sr,
                                          typename SchurTy<T>::R* si) {
  const T* m = a.Mat + (size_t)i * a.n;
  for (int j = lane; j < a.n; j += 32) {
    const T mv = m[j];
    const T* xv = a.X + (size_t)j * SC_W + a.xoff;
#pragma unroll
    for (int c = 0; c < NC; c++) {
      const T v = xv[c];
      sr[c] = sfma(mv.x, v.x, sfma(-mv.y, v.y, sr[c]));
      si[c] = sfma(mv.x, v.y, sfma(mv.y, v.x, si[c]));
    }
  }
}

template <class T, int NC>
__global__ void __launch_bounds__(256) k_schur_mv(SchurMv<T> a, int mode) {
  typedef typename SchurTy<T>::R R;
  const int lane = threadIdx.x & 31;
  const int i = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= a.n) return;
  R sr[NC], si[NC];
#pragma unroll
  for (int c = 0; c < NC; c++) { sr[c] = (R)0; si[c] = (R)0; }
  schur_row<T, NC>(a, i, lane, sr, si);
#pragma unroll
  for (int c = 0; c < NC; c++)
    for (int o = 16; o > 0; o >>= 1) {
      sr[c] += __shfl_down_sync(0xffffffffu, sr[c], o);
      si[c] += __shfl_down_sync(0xffffffffu, si[c], o);
    }
  if (lane != 0) return;
  const size_t r4 = (size_t)i * SC_W;
  T acc[NC];
#pragma unroll
  for (int c = 0; c < NC; c++) { acc[c].x = sr[c]; acc[c].y = si[c]; }
  if (mode == SC_T0) {
#pragma unroll
    for (int c = 0; c < NC; c++) a.out[r4 + c] = acc[c];
  } else if (mode == SC_Y) {
#pragma unroll
    for (int c = 0; c < NC; c++) a.out[r4 + c] = acc[c] + (c < 3 ? a.aux[r4 + c] : a.c0 * a.aux[r4 + c]);
  } else if (mode == SC_MY) {
    T t = a.X[r4 + 3];
#pragma unroll
    for (int c = 0; c < NC && c < 3; c++) {
      a.out[r4 + c] = acc[c];
      t -= (a.c0 * acc[c]) * a.vn[(size_t)i * 3 + c];
    }
    a.out[r4 + 3] = t;
  } else if (mode == SC_U3) {
    for (int c = 0; c < 3; c++) a.out[r4 + c] = acc[0] * a.vn[(size_t)i * 3 + c];
    a.out[r4 + 3] = acc[0];
  } else if (mode == SC_U) {
#pragma unroll
    for (int c = 0; c < NC && c < 3; c++) a.out[r4 + c] = a.aux[r4 + c] - a.c0 * acc[c];
    a.out[r4 + 3] = a.X[r4 + 3];
  } else {  // SC_DU
    const size_t n = (size_t)a.n;
#pragma unroll
    for (int c = 0; c < NC; c++) {
      const T u = a.X[r4 + c], t0 = a.aux[r4 + c];
      cplx& xu = a.x[c * n + i];
      cplx& xd = a.x[(4 + c) * n + i];
      xu.x += (double)u.x;
      xu.y += (double)u.y;
      xd.x += (double)(-acc[c].x - t0.x);
      xd.y += (double)(-acc[c].y - t0.y);
    }
  }
}

template <class T, int NC>
static int schur_mv(const SchurMv<T>& a, int mode, cudaStream_t st) {
  const unsigned grid = (unsigned)(((size_t)a.n * 32 + 255) / 256);
  k_schur_mv<T, NC><<<grid, 256, 0, st>>>(a, mode);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------- C ABI (internal)
extern "C" void gbi_schur_destroy(GbSchur* s) {
  if (!s) return;
  cudaFree(s->G0i); cudaFree(s->G1i); cudaFree(s->nX0); cudaFree(s->Minv); cudaFree(s->Si);
  cudaFree(s->vn); cudaFree(s->work); cudaFree(s->rbt);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->st2) cudaStreamDestroy(s->st2);
  delete s;
}

// fp64: 1 complex FP64 matrices (plain FP64 form), 0 complex FP32
extern "C" int gbi_schur_create(int n, int fp64, GbSchur** out) {
  *out = nullptr;
  GbSchur* s = new GbSchur();
  s->n = n;
  s->fp64 = fp64 ? 1 : 0;
  s->esz = fp64 ? sizeof(cplx) : sizeof(cplxf);
  s->G0i = s->G1i = s->nX0 = s->Minv = s->Si = s->work = s->vn = nullptr;
  s->rbt = nullptr;
  s->st2 = nullptr;
  s->ev0 = s->ev1 = nullptr;
  const size_t nn = (size_t)n * n;
  void** mats[5] = {&s->G0i, &s->G1i, &s->nX0, &s->Minv, &s->Si};
  for (auto p : mats)
    if (cudaMalloc(p, nn * s->esz) != cudaSuccess) {
      gbi_set_error("block elimination: out of device memory (%zu bytes)", nn * s->esz);
      gbi_schur_destroy(s);
      return -1;
    }
  if (cudaMalloc(&s->vn, (size_t)n * 3 * (fp64 ? sizeof(double) : sizeof(float))) != cudaSuccess ||
      cudaMalloc(&s->work, 7 * (size_t)n * SC_W * s->esz) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->st2, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev0, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&s->ev1, cudaEventDisableTiming) != cudaSuccess) {
    gbi_set_error("block elimination: out of device memory");
    gbi_schur_destroy(s);
    return -1;
  }
  if (!fp64 && n % 4 == 0) {
    std::vector<float> h(4 * (size_t)n);
    gbi_rbt_params(n, h.data());
    if (cudaMalloc((void**)&s->rbt, h.size() * sizeof(float)) != cudaSuccess ||
        cudaMemcpy(s->rbt, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
      gbi_set_error("block elimination: butterfly parameters");
      gbi_schur_destroy(s);
      return -1;
    }
  }
  *out = s;
  return 0;
}

// per-chain work of a factorisation (stream-ordered on that chain's stream)
struct ChainWs {
  int64_t* ipiv;
  int* perm;
  int* info;  // [1]
  int* err;   // [4]: tensor-core wait time-out flag
};

static int ws_alloc(ChainWs& w, int n, cudaStream_t st) {
  w.ipiv = nullptr; w.perm = nullptr; w.info = nullptr; w.err = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&w.ipiv, (size_t)n * sizeof(int64_t), st));
  GB_CUDA(cudaMallocAsync((void**)&w.perm, (size_t)n * sizeof(int), st));
  GB_CUDA(cudaMallocAsync((void**)&w.info, 16, st));
  GB_CUDA(cudaMallocAsync((void**)&w.err, 16, st));
  GB_CUDA(cudaMemsetAsync(w.info, 0, 16, st));
  GB_CUDA(cudaMemsetAsync(w.err, 0, 16, st));
  return 0;
}
static void ws_free(ChainWs& w, cudaStream_t st) {
  if (w.ipiv) cudaFreeAsync(w.ipiv, st);
  if (w.perm) cudaFreeAsync(w.perm, st);
  if (w.info) cudaFreeAsync(w.info, st);
  if (w.err) cudaFreeAsync(w.err, st);
}

// X = A^-1 (A overwritten by factors); a zero pivot is reported in w.info
static int lu_inverse(GbSchur* s, void* A, void* X, ChainWs& w, cudaStream_t st) {
  const int n = s->n;
  if (s->fp64) {
    if (gbi_zgetrf((cplx*)A, n, n, w.ipiv, w.info, st)) return -1;
    return gbi_zinverse((const cplx*)A, n, n, w.ipiv, (cplx*)X, n, st);
  }
  cplxf* a = (cplxf*)A;
  cplxf* x = (cplxf*)X;
  if (s->rbt) {  // butterflies, no interchanges: A^-1 = V (U^T A V)^-1 U^T
    const float* pu = s->rbt;
    const float* pv = s->rbt + 2 * (size_t)n;
    if (gbi_rbt_matrix(a, n, n, pu, pv, st)) return -1;
    if (gbi_cgetrf_nopiv(a, n, n, w.ipiv, w.info, st)) return -1;
    if (gbi_perm_identity(n, w.perm, st)) return -1;
    if (gbi_cinverse_tc(a, n, n, w.perm, x, n, st)) return -1;
    return gbi_rbt_inverse(x, n, n, pu, pv, st);
  }
  if (gbi_cgetrf(a, n, n, w.ipiv, w.info, st)) return -1;
  if (gbi_make_perm(w.ipiv, n, w.perm, st)) return -1;
  return gbi_cinverse_tc(a, n, n, w.perm, x, n, st);
}

// C = -A B (n x n)
static int neg_product(GbSchur* s, const void* A, const void* B, void* C, ChainWs& w, cudaStream_t st) {
  const int n = s->n;
  GB_CUDA(cudaMemsetAsync(C, 0, (size_t)n * n * s->esz, st));
  if (s->fp64) return gbi_zgemm_sub(n, n, n, (const cplx*)A, n, (const cplx*)B, n, (cplx*)C, n, st);
  return gbi_tc_cgemm_sub(n, n, n, (const cplxf*)A, n, (const cplxf*)B, n, (cplxf*)C, n, gbi_tc_passes(), nullptr, w.err,
                          st);
}

// one chain: X_inv = P^-1 (P overwritten), then out = -X_inv Q
static int chain(GbSchur* s, void* P, void* Xinv, const void* Q, void* out, ChainWs& w, cudaStream_t st) {
  if (lu_inverse(s, P, Xinv, w, st)) return -1;
  return neg_product(s, Xinv, Q, out, w, st);
}

template <class T>
static int launch_gathers(GbSchur* s, const GbMeshDev* m, const cplx* G0, const cplx* H0, const cplx* G1,
                          const cplx* H1, const int* sid0, const int* sid1, const int* rowk0, const int* rowk1, void* P0,
                          void* Q0, void* P1, void* Q1, cudaStream_t st) {
  typedef typename SchurTy<T>::R R;
  const int N = 4 * m->Ne;
  const unsigned gq = (unsigned)(((size_t)N * N + 255) / 256);
  k_schur_gather<T><<<gq, 256, 0, st>>>(G0, H0, N, sid0, rowk0, m->eni, m->etype, s->n, (T*)P0, (T*)Q0);
  k_schur_gather<T><<<gq, 256, 0, st>>>(G1, H1, N, sid1, rowk1, m->eni, m->etype, s->n, (T*)P1, (T*)Q1);
  k_schur_normals<R><<<(unsigned)((4 * m->Ne + 255) / 256), 256, 0, st>>>(m->wen, m->eni, m->etype, m->Ne, (R*)s->vn);
  gbi_count_launch();
  gbi_count_launch();
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

template <class T>
static int launch_combine(GbSchur* s, void* P1, void* P0, void* Q0, cudaStream_t st) {
  const size_t nn = (size_t)s->n * s->n;
  k_schur_combine<T><<<(unsigned)((nn + 255) / 256), 256, 0, st>>>((const T*)s->nX0, (const T*)P1, nn,
                                                                     SchurTy<T>::from(s->beta), (T*)P0, (T*)Q0);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

template <class T>
static int launch_s(GbSchur* s, void* Q0, cudaStream_t st) {
  typedef typename SchurTy<T>::R R;
  const size_t nn = (size_t)s->n * s->n;
  k_schur_s<T, R><<<(unsigned)((nn + 255) / 256), 256, 0, st>>>((T*)Q0, (const T*)s->Minv, (const R*)s->vn, s->n,
                                                                SchurTy<T>::from(s->sigdel));
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// Block factors of an object with one interface (domain 0 outside, 1
// inside): G[d], H[d] its FP64 domain matrices, sid[d] / rowk[d] the domain
// lists (device, 1-based) and row maps, m the mesh (device arrays, host kn).
// Returns 0, 1 when an LU met a zero pivot (the caller factorises densely),
// -1 on error.  Synchronises st.
extern "C" int gbi_schur_factor(GbSchur* s, const GbMeshDev* m, const cplx* G0, const cplx* H0, const cplx* G1,
                                const cplx* H1, const int* sid0, const int* sid1, const int* rowk0, const int* rowk1,
                                cudaStream_t st) {
  const int n = s->n;
  const size_t nn = (size_t)n * n;
  {
    const std::complex<double> k0(m->kn[0], m->kn[1]), k1(m->kn[2], m->kn[3]);
    const std::complex<double> delt = k0 * k0 - k1 * k1, beps = (k0 * k0) / (k1 * k1), sigm = 1.0 - beps;
    const std::complex<double> sd = sigm * delt;
    s->beta = cmk(beps.real(), beps.imag());
    s->sigma = cmk(sigm.real(), sigm.imag());
    s->delta = cmk(delt.real(), delt.imag());
    s->sigdel = cmk(sd.real(), sd.imag());
  }
  void *P0 = nullptr, *P1 = nullptr, *Q0 = nullptr, *Q1 = nullptr;
  ChainWs w0, w1;
  memset(&w0, 0, sizeof(w0));
  memset(&w1, 0, sizeof(w1));
  int rc = 0;
  // temporaries (freed on every path below; a failed allocation leaves null)
  if (cudaMallocAsync(&P0, nn * s->esz, st) != cudaSuccess || cudaMallocAsync(&P1, nn * s->esz, st) != cudaSuccess ||
      cudaMallocAsync(&Q0, nn * s->esz, st) != cudaSuccess || cudaMallocAsync(&Q1, nn * s->esz, st) != cudaSuccess ||
      ws_alloc(w0, n, st) || ws_alloc(w1, n, st)) {
    gbi_set_error("block elimination: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  if (!rc && (cudaMemsetAsync(P0, 0, nn * s->esz, st) != cudaSuccess ||
              cudaMemsetAsync(P1, 0, nn * s->esz, st) != cudaSuccess ||
              cudaMemsetAsync(Q0, 0, nn * s->esz, st) != cudaSuccess ||
              cudaMemsetAsync(Q1, 0, nn * s->esz, st) != cudaSuccess)) {
    gbi_set_error("block elimination: memset");
    rc = -1;
  }
  if (!rc)
    rc = s->fp64 ? launch_gathers<cplx>(s, m, G0, H0, G1, H1, sid0, sid1, rowk0, rowk1, P0, Q0, P1, Q1, st)
                 : launch_gathers<cplxf>(s, m, G0, H0, G1, H1, sid0, sid1, rowk0, rowk1, P0, Q0, P1, Q1, st);
  // the G0 chain (G0^-1, nX0 = -G0^-1 H0) here on st, the G1 chain
  // (G1^-1, P1 = -G1^-1 H1) on st2 from a second host thread
  if (!rc && (cudaEventRecord(s->ev0, st) != cudaSuccess || cudaStreamWaitEvent(s->st2, s->ev0, 0) != cudaSuccess)) {
    gbi_set_error("block elimination: stream order");
    rc = -1;
  }
  if (!rc) {
    int dev = 0;
    cudaGetDevice(&dev);
    int rc1 = 0;
    std::string msg1;
    auto job1 = [&]() {
      if (cudaSetDevice(dev) != cudaSuccess) { rc1 = -1; msg1 = "cudaSetDevice failed"; return; }
      rc1 = chain(s, P1, s->G1i, Q1, P1, w1, s->st2);
      if (!rc1 && cudaEventRecord(s->ev1, s->st2) != cudaSuccess) { rc1 = -1; gbi_set_error("event record"); }
      if (rc1) msg1 = gb_last_error();
    };
    std::thread th;
    bool threaded = true;
    try {
      th = std::thread(job1);
    } catch (...) {
      threaded = false;
    }
    if (!threaded) job1();  // no thread available: run the G1 chain first, here
    rc = chain(s, P0, s->G0i, Q0, s->nX0, w0, st);
    if (threaded) th.join();
    if (!rc && rc1) { gbi_set_error("%s", msg1.c_str()); rc = -1; }
    if (!rc && cudaStreamWaitEvent(st, s->ev1, 0) != cudaSuccess) { gbi_set_error("block elimination: join"); rc = -1; }
  }
  // P0 = M, Q0 = M3
  if (!rc) rc = s->fp64 ? launch_combine<cplx>(s, P1, P0, Q0, st) : launch_combine<cplxf>(s, P1, P0, Q0, st);
  if (!rc) rc = lu_inverse(s, P0, s->Minv, w0, st);
  if (!rc) rc = s->fp64 ? launch_s<cplx>(s, Q0, st) : launch_s<cplxf>(s, Q0, st);
  int h[4] = {0, 0, 0, 0};
  if (!rc && (cudaMemcpyAsync(h, w1.info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(h + 1, w1.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)) {
    gbi_set_error("block elimination: status copy");
    rc = -1;
  }
  // S^-1 (w1's status is read above; reuse it for this last LU)
  if (!rc) rc = lu_inverse(s, Q0, s->Si, w1, st);
  int g[2] = {0, 0};
  if (!rc && (cudaMemcpyAsync(h + 2, w0.info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(h + 3, w0.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(g, w1.info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(g + 1, w1.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("block elimination: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  void* tmp[4] = {P0, P1, Q0, Q1};
  for (void* t : tmp)
    if (t) cudaFreeAsync(t, st);
  ws_free(w0, st);
  ws_free(w1, st);
  if (!rc && (h[1] || h[3] || g[1])) { gbi_set_error("block elimination: a tensor-core pipeline wait timed out"); rc = -1; }
  if (!rc && (h[0] || h[2] || g[0])) rc = 1;
  return rc;
}

// x += P^-1 r: one correction of the refinement (r, x FP64 of A's order)
template <class T>
static int schur_apply(GbSchur* s, const cplx* r, cplx* x, cudaStream_t st) {
  typedef typename SchurTy<T>::R R;
  const int n = s->n;
  const size_t b = (size_t)n * SC_W;
  T *R0 = (T*)s->work, *R1 = R0 + b, *T0 = R1 + b, *Y = T0 + b, *MY = Y + b, *W = MY + b, *U = W + b;
  k_schur_in<T><<<(unsigned)((8 * (size_t)n + 255) / 256), 256, 0, st>>>(r, n, R0, R1);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  SchurMv<T> a;
  a.n = n;
  a.vn = (const R*)s->vn;
  a.x = x;
  a.aux = nullptr;
  a.c0 = czero<T>();
  // T0 = G0^-1 R0
  a.Mat = (const T*)s->G0i; a.X = R0; a.xoff = 0; a.out = T0;
  if (schur_mv<T, 4>(a, SC_T0, st)) return -1;
  // Y = G1^-1 R1 + (1, 1, 1, beta) T0
  a.Mat = (const T*)s->G1i; a.X = R1; a.out = Y; a.aux = T0; a.c0 = SchurTy<T>::from(s->beta);
  if (schur_mv<T, 4>(a, SC_Y, st)) return -1;
  // MY_c = M^-1 y_c (c < 3), MY_3 = y_3 - sigma sum_c vn_c MY_c
  a.Mat = (const T*)s->Minv; a.X = Y; a.out = MY; a.aux = nullptr; a.c0 = SchurTy<T>::from(s->sigma);
  if (schur_mv<T, 3>(a, SC_MY, st)) return -1;
  // U3 = S^-1 MY_3; W_c = vn_c U3, W_3 = U3
  a.Mat = (const T*)s->Si; a.X = MY; a.xoff = 3; a.out = W;
  if (schur_mv<T, 1>(a, SC_U3, st)) return -1;
  // U_c = MY_c - delta M^-1 W_c (c < 3), U_3 = U3
  a.Mat = (const T*)s->Minv; a.X = W; a.xoff = 0; a.out = U; a.aux = MY; a.c0 = SchurTy<T>::from(s->delta);
  if (schur_mv<T, 3>(a, SC_U, st)) return -1;
  // x += (U, -nX0 U ... ) : dU = X0 U - T0
  a.Mat = (const T*)s->nX0; a.X = U; a.out = nullptr; a.aux = T0;
  if (schur_mv<T, 4>(a, SC_DU, st)) return -1;
  return 0;
}

extern "C" int gbi_schur_apply(GbSchur* s, const cplx* r, cplx* x, cudaStream_t st) {
  return s->fp64 ? schur_apply<cplx>(s, r, x, st) : schur_apply<cplxf>(s, r, x, st);
}

extern "C" int gbi_schur_is_fp64(const GbSchur* s) { return s ? s->fp64 : -1; }

// device addresses of the five factors (G0^-1, G1^-1, -X0, M^-1, S^-1)
extern "C" void gbi_schur_mats(GbSchur* s, void** out) {
  out[0] = s->G0i; out[1] = s->G1i; out[2] = s->nX0; out[3] = s->Minv; out[4] = s->Si;
}

// after the five factors were loaded from a file: the node normals and the
// interface constants, as gbi_schur_factor sets them
extern "C" int gbi_schur_prepare(GbSchur* s, const GbMeshDev* m, cudaStream_t st) {
  const std::complex<double> k0(m->kn[0], m->kn[1]), k1(m->kn[2], m->kn[3]);
  const std::complex<double> delt = k0 * k0 - k1 * k1, beps = (k0 * k0) / (k1 * k1), sigm = 1.0 - beps;
  const std::complex<double> sd = sigm * delt;
  s->beta = cmk(beps.real(), beps.imag());
  s->sigma = cmk(sigm.real(), sigm.imag());
  s->delta = cmk(delt.real(), delt.imag());
  s->sigdel = cmk(sd.real(), sd.imag());
  const unsigned g = (unsigned)((4 * m->Ne + 255) / 256);
  if (s->fp64) k_schur_normals<double><<<g, 256, 0, st>>>(m->wen, m->eni, m->etype, m->Ne, (double*)s->vn);
  else k_schur_normals<float><<<g, 256, 0, st>>>(m->wen, m->eni, m->etype, m->Ne, (float*)s->vn);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  GB_CUDA(cudaStreamSynchronize(st));
  return 0;
}
