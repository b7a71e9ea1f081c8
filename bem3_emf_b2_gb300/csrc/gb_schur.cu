// gb_schur.cu -- block elimination of the coupled system of an object whose
// elements all lie on one interface (exterior domain 0 outside, domain 1
// inside): the chosen form's correction solve through node-sized complex-FP32
// inverses instead of the dense factors of the 8 NN x 8 NN coupled matrix.
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
// Factorisation (complex FP32, tournament-pivoted LUs with tensor-core
// updates, explicit inverses): G0^-1, G1^-1, X0, M^-1, S^-1 -- about 32 NN^3
// complex-equivalent flop against (8/3) (8 NN)^3 = 1365 NN^3 for the dense
// LU, and five NN x NN matrices instead of one (8 NN)^2.  A correction is six
// products of those matrices with at most four node vectors.  The FP64
// refinement around it (residual b - A x from the FP64 G, H) is unchanged:
// the solution is the same to the refinement's tolerance.
#include "gb_common.cuh"
#include "gb_internal.h"

#include <complex>

extern "C" {
int gbi_cgetrf(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
int gbi_make_perm(const int64_t* ipiv, int n, int* perm, cudaStream_t st);
int gbi_cinverse_tc(const cplxf* LU, size_t lda, int n, const int* perm, cplxf* X, size_t ldx, cudaStream_t st);
size_t gbi_tc_scratch_floats(int M, int N, int K);
int gbi_tc_cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C, size_t ldc,
                     int passes, float* scratch, int* err, cudaStream_t st);
}

// node vectors of the correction are kept four to a row: V[i * 4 + c]
#define SC_W 4

struct GbSchur {
  int n;                                // NN
  cplxf *G0i, *G1i, *nX0, *Minv, *Si;   // n x n each; nX0 = -X0
  float* vn;                            // n x 3 unit normals of the nodes
  cplxf* work;                          // 7 blocks of n x SC_W: R0 R1 T0 Y MY W U
  cplxf beta, sigma, delta, sigdel;     // sigdel = sigma * delta
};

// ---------------------------------------------------------------- factorisation
// Gather the domain matrices (N x N, rows (t-1)*4+tn, columns (s-1)*4+l) to
// node columns: out[rowk[row]][eni[|sid[s]|][l]], in complex FP32
__global__ void k_schur_gather(const cplx* __restrict__ G, const cplx* __restrict__ H, int N, const int* sid,
                               const int* rowk, const int* eni, const int* etype, int n, cplxf* Gh, cplxf* Hh) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)N * N) return;
  const int row = (int)(p / N), col = (int)(p % N);
  const int k = rowk[row];
  if (k < 0) return;
  const int e = abs(sid[(col >> 2) + 1]), l = col & 3;
  if (l == 3 && etype[e] == 0) return;
  const int c = eni[e * 4 + l];
  const size_t q = (size_t)k * n + c;
  const cplx g = G[p], h = H[p];
  Gh[q] = cmkf((float)g.x, (float)g.y);
  Hh[q] = cmkf((float)h.x, (float)h.y);
}

// unit normals of the nodes (the A build's vn: wen normalised)
__global__ void k_schur_normals(const double* wen, const int* eni, const int* etype, int Ne, float* vn) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= 4 * Ne) return;
  const int e = 1 + p / 4, l = p % 4;
  if (l == 3 && etype[e] == 0) return;
  const int c = eni[e * 4 + l];
  double w[3], a = 0.0;
  for (int d = 0; d < 3; d++) { w[d] = wen[(size_t)e * 12 + l * 3 + d]; a += w[d] * w[d]; }
  a = sqrt(a);
  for (int d = 0; d < 3; d++) vn[(size_t)c * 3 + d] = (float)(a != 0.0 ? w[d] / a : w[d]);
}

// M = -(nX0 + nX1) = X0 + X1 and M3 = -(nX1 + beta nX0) = X1 + beta X0
__global__ void k_schur_combine(const cplxf* __restrict__ nX0, const cplxf* __restrict__ nX1, size_t nn, cplxf beta,
                                cplxf* M, cplxf* M3) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nn) return;
  const cplxf a = nX0[p], b = nX1[p];
  M[p] = cmkf(-(a.x + b.x), -(a.y + b.y));
  const cplxf ba = beta * a;
  M3[p] = cmkf(-(b.x + ba.x), -(b.y + ba.y));
}

// S = M3 - sigma delta (vn_i . vn_j) M^-1_ij
__global__ void k_schur_s(cplxf* S, const cplxf* __restrict__ Minv, const float* __restrict__ vn, int n, cplxf sigdel) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= (size_t)n * n) return;
  const int i = (int)(p / n), j = (int)(p % n);
  const float w = vn[i * 3] * vn[j * 3] + vn[i * 3 + 1] * vn[j * 3 + 1] + vn[i * 3 + 2] * vn[j * 3 + 2];
  S[p] -= (sigdel * Minv[p]) * w;
}

// ---------------------------------------------------------------- correction
// r (FP64, A's row order: domain-0 rows c*n + k, domain-1 rows 4n + c*n + k)
// -> R0[k][c] = re_c[k], R1[k][c] = ri_c[k] in complex FP32
__global__ void k_schur_in(const cplx* __restrict__ r, int n, cplxf* R0, cplxf* R1) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= 8 * (size_t)n) return;
  const int blk = (int)(p / n), k = (int)(p % n);
  const cplx v = r[p];
  const cplxf f = cmkf((float)v.x, (float)v.y);
  if (blk < 4) R0[(size_t)k * SC_W + blk] = f;
  else R1[(size_t)k * SC_W + blk - 4] = f;
}

enum { SC_T0 = 0, SC_Y = 1, SC_MY = 2, SC_U3 = 3, SC_U = 4, SC_DU = 5 };

struct SchurMv {
  const cplxf* Mat;  // n x n
  int n;
  const cplxf* X;    // n x SC_W; columns xoff .. xoff + NC - 1 are multiplied
  int xoff;
  cplxf* out;        // n x SC_W
  const cplxf* aux;  // n x SC_W (mode-dependent)
  const float* vn;
  cplxf c0;          // beta (SC_Y), sigma (SC_MY), delta (SC_U)
  cplx* x;           // FP64 solution (SC_DU)
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
template <int NC>
__global__ void __launch_bounds__(256) k_schur_mv(SchurMv a, int mode) {
  const int lane = threadIdx.x & 31;
  const int i = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (i >= a.n) return;
  const cplxf* m = a.Mat + (size_t)i * a.n;
  float sr[NC], si[NC];
#pragma unroll
  for (int c = 0; c < NC; c++) { sr[c] = 0.f; si[c] = 0.f; }
  for (int j = lane; j < a.n; j += 32) {
    const cplxf mv = m[j];
    const cplxf* xv = a.X + (size_t)j * SC_W + a.xoff;
#pragma unroll
    for (int c = 0; c < NC; c++) {
      const cplxf v = xv[c];
      sr[c] = fmaf(mv.x, v.x, fmaf(-mv.y, v.y, sr[c]));
      si[c] = fmaf(mv.x, v.y, fmaf(mv.y, v.x, si[c]));
    }
  }
#pragma unroll
  for (int c = 0; c < NC; c++)
    for (int o = 16; o > 0; o >>= 1) {
      sr[c] += __shfl_down_sync(0xffffffffu, sr[c], o);
      si[c] += __shfl_down_sync(0xffffffffu, si[c], o);
    }
  if (lane != 0) return;
  const size_t r4 = (size_t)i * SC_W;
  cplxf acc[NC];
#pragma unroll
  for (int c = 0; c < NC; c++) acc[c] = cmkf(sr[c], si[c]);
  if (mode == SC_T0) {
#pragma unroll
    for (int c = 0; c < NC; c++) a.out[r4 + c] = acc[c];
  } else if (mode == SC_Y) {
#pragma unroll
    for (int c = 0; c < NC; c++) a.out[r4 + c] = acc[c] + (c < 3 ? a.aux[r4 + c] : a.c0 * a.aux[r4 + c]);
  } else if (mode == SC_MY) {
    cplxf t = a.X[r4 + 3];
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
      const cplxf u = a.X[r4 + c], t0 = a.aux[r4 + c];
      cplx& xu = a.x[c * n + i];
      cplx& xd = a.x[(4 + c) * n + i];
      xu.x += (double)u.x;
      xu.y += (double)u.y;
      xd.x += (double)(-acc[c].x - t0.x);
      xd.y += (double)(-acc[c].y - t0.y);
    }
  }
}

template <int NC>
static int schur_mv(const SchurMv& a, int mode, cudaStream_t st) {
  const unsigned grid = (unsigned)(((size_t)a.n * 32 + 255) / 256);
  k_schur_mv<NC><<<grid, 256, 0, st>>>(a, mode);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ---------------------------------------------------------------- C ABI (internal)
extern "C" void gbi_schur_destroy(GbSchur* s) {
  if (!s) return;
  cudaFree(s->G0i); cudaFree(s->G1i); cudaFree(s->nX0); cudaFree(s->Minv); cudaFree(s->Si);
  cudaFree(s->vn); cudaFree(s->work);
  delete s;
}

extern "C" int gbi_schur_create(int n, GbSchur** out) {
  *out = nullptr;
  GbSchur* s = new GbSchur();
  s->n = n;
  s->G0i = s->G1i = s->nX0 = s->Minv = s->Si = s->work = nullptr;
  s->vn = nullptr;
  const size_t nn = (size_t)n * n;
  cplxf** mats[5] = {&s->G0i, &s->G1i, &s->nX0, &s->Minv, &s->Si};
  for (auto p : mats)
    if (cudaMalloc((void**)p, nn * sizeof(cplxf)) != cudaSuccess) {
      gbi_set_error("block elimination: out of device memory (%zu bytes)", nn * sizeof(cplxf));
      gbi_schur_destroy(s);
      return -1;
    }
  if (cudaMalloc((void**)&s->vn, (size_t)n * 3 * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void**)&s->work, 7 * (size_t)n * SC_W * sizeof(cplxf)) != cudaSuccess) {
    gbi_set_error("block elimination: out of device memory");
    gbi_schur_destroy(s);
    return -1;
  }
  *out = s;
  return 0;
}

// LU of A (n x n, tournament pivoting) and X = A^-1; info: device int of the LU
static int lu_inverse(cplxf* A, int n, int64_t* ipiv, int* perm, int* info, cplxf* X, cudaStream_t st) {
  if (gbi_cgetrf(A, n, n, ipiv, info, st)) return -1;
  if (gbi_make_perm(ipiv, n, perm, st)) return -1;
  return gbi_cinverse_tc(A, n, n, perm, X, n, st);
}

// C = -A B (n x n complex FP32, tensor cores)
static int neg_product(const cplxf* A, const cplxf* B, int n, cplxf* C, float* scratch, int* err, cudaStream_t st) {
  GB_CUDA(cudaMemsetAsync(C, 0, (size_t)n * n * sizeof(cplxf), st));
  return gbi_tc_cgemm_sub(n, n, n, A, n, B, n, C, n, 3, scratch, err, st);
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
  const int N = 4 * m->Ne;
  {
    const std::complex<double> k0(m->kn[0], m->kn[1]), k1(m->kn[2], m->kn[3]);
    const std::complex<double> delt = k0 * k0 - k1 * k1, beps = (k0 * k0) / (k1 * k1), sigm = 1.0 - beps;
    const std::complex<double> sd = sigm * delt;
    s->beta = cmkf((float)beps.real(), (float)beps.imag());
    s->sigma = cmkf((float)sigm.real(), (float)sigm.imag());
    s->delta = cmkf((float)delt.real(), (float)delt.imag());
    s->sigdel = cmkf((float)sd.real(), (float)sd.imag());
  }
  cplxf *P0 = nullptr, *P1 = nullptr, *Q0 = nullptr, *Q1 = nullptr;
  int64_t* ipiv = nullptr;
  int *perm = nullptr, *info = nullptr, *err = nullptr;
  float* scratch = nullptr;
  int rc = 0;
  // temporaries (freed on every path below; a failed allocation leaves null)
  if (cudaMallocAsync((void**)&P0, nn * sizeof(cplxf), st) != cudaSuccess ||
      cudaMallocAsync((void**)&P1, nn * sizeof(cplxf), st) != cudaSuccess ||
      cudaMallocAsync((void**)&Q0, nn * sizeof(cplxf), st) != cudaSuccess ||
      cudaMallocAsync((void**)&Q1, nn * sizeof(cplxf), st) != cudaSuccess ||
      cudaMallocAsync((void**)&ipiv, (size_t)n * sizeof(int64_t), st) != cudaSuccess ||
      cudaMallocAsync((void**)&perm, (size_t)n * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync((void**)&info, 4 * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync((void**)&err, 16, st) != cudaSuccess ||
      cudaMallocAsync((void**)&scratch, gbi_tc_scratch_floats(n, n, n) * sizeof(float), st) != cudaSuccess ||
      cudaMemsetAsync(err, 0, 16, st) != cudaSuccess) {
    gbi_set_error("block elimination: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  const unsigned gq = (unsigned)(((size_t)N * N + 255) / 256), gn = (unsigned)((nn + 255) / 256);
  if (!rc && (cudaMemsetAsync(P0, 0, nn * sizeof(cplxf), st) != cudaSuccess ||
              cudaMemsetAsync(P1, 0, nn * sizeof(cplxf), st) != cudaSuccess ||
              cudaMemsetAsync(Q0, 0, nn * sizeof(cplxf), st) != cudaSuccess ||
              cudaMemsetAsync(Q1, 0, nn * sizeof(cplxf), st) != cudaSuccess)) {
    gbi_set_error("block elimination: memset");
    rc = -1;
  }
  if (!rc) {
    k_schur_gather<<<gq, 256, 0, st>>>(G0, H0, N, sid0, rowk0, m->eni, m->etype, n, P0, Q0);
    k_schur_gather<<<gq, 256, 0, st>>>(G1, H1, N, sid1, rowk1, m->eni, m->etype, n, P1, Q1);
    k_schur_normals<<<(unsigned)((4 * m->Ne + 255) / 256), 256, 0, st>>>(m->wen, m->eni, m->etype, m->Ne, s->vn);
    gbi_count_launch();
    gbi_count_launch();
    gbi_count_launch();
    if (cudaGetLastError() != cudaSuccess) { gbi_set_error("block elimination: gather launch"); rc = -1; }
  }
  // G0^-1, G1^-1 (P0, P1 hold the factors afterwards)
  if (!rc) rc = lu_inverse(P0, n, ipiv, perm, info + 0, s->G0i, st);
  if (!rc) rc = lu_inverse(P1, n, ipiv, perm, info + 1, s->G1i, st);
  // nX0 = -G0^-1 H0, P1 = -G1^-1 H1
  if (!rc) rc = neg_product(s->G0i, Q0, n, s->nX0, scratch, err, st);
  if (!rc) rc = neg_product(s->G1i, Q1, n, P1, scratch, err, st);
  // P0 = M, Q0 = M3
  if (!rc) {
    k_schur_combine<<<gn, 256, 0, st>>>(s->nX0, P1, nn, s->beta, P0, Q0);
    gbi_count_launch();
    if (cudaGetLastError() != cudaSuccess) { gbi_set_error("block elimination: combine launch"); rc = -1; }
  }
  if (!rc) rc = lu_inverse(P0, n, ipiv, perm, info + 2, s->Minv, st);
  if (!rc) {
    k_schur_s<<<gn, 256, 0, st>>>(Q0, s->Minv, s->vn, n, s->sigdel);
    gbi_count_launch();
    if (cudaGetLastError() != cudaSuccess) { gbi_set_error("block elimination: S launch"); rc = -1; }
  }
  if (!rc) rc = lu_inverse(Q0, n, ipiv, perm, info + 3, s->Si, st);
  int h[5] = {0, 0, 0, 0, 0};
  if (!rc && (cudaMemcpyAsync(h, info, 4 * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaMemcpyAsync(h + 4, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("block elimination: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  void* tmp[9] = {P0, P1, Q0, Q1, ipiv, perm, info, err, scratch};
  for (void* t : tmp)
    if (t) cudaFreeAsync(t, st);
  if (!rc && h[4]) { gbi_set_error("block elimination: a tensor-core pipeline wait timed out"); rc = -1; }
  if (!rc && (h[0] || h[1] || h[2] || h[3])) rc = 1;
  return rc;
}

// x += P^-1 r: one correction of the refinement (r, x FP64 of A's order)
extern "C" int gbi_schur_apply(GbSchur* s, const cplx* r, cplx* x, cudaStream_t st) {
  const int n = s->n;
  const size_t b = (size_t)n * SC_W;
  cplxf *R0 = s->work, *R1 = R0 + b, *T0 = R1 + b, *Y = T0 + b, *MY = Y + b, *W = MY + b, *U = W + b;
  k_schur_in<<<(unsigned)((8 * (size_t)n + 255) / 256), 256, 0, st>>>(r, n, R0, R1);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  SchurMv a;
  a.n = n;
  a.vn = s->vn;
  a.x = x;
  a.aux = nullptr;
  a.c0 = cmkf(0.f, 0.f);
  // T0 = G0^-1 R0
  a.Mat = s->G0i; a.X = R0; a.xoff = 0; a.out = T0;
  if (schur_mv<4>(a, SC_T0, st)) return -1;
  // Y = G1^-1 R1 + (1, 1, 1, beta) T0
  a.Mat = s->G1i; a.X = R1; a.out = Y; a.aux = T0; a.c0 = s->beta;
  if (schur_mv<4>(a, SC_Y, st)) return -1;
  // MY_c = M^-1 y_c (c < 3), MY_3 = y_3 - sigma sum_c vn_c MY_c
  a.Mat = s->Minv; a.X = Y; a.out = MY; a.aux = nullptr; a.c0 = s->sigma;
  if (schur_mv<3>(a, SC_MY, st)) return -1;
  // U3 = S^-1 MY_3; W_c = vn_c U3, W_3 = U3
  a.Mat = s->Si; a.X = MY; a.xoff = 3; a.out = W;
  if (schur_mv<1>(a, SC_U3, st)) return -1;
  // U_c = MY_c - delta M^-1 W_c (c < 3), U_3 = U3
  a.Mat = s->Minv; a.X = W; a.xoff = 0; a.out = U; a.aux = MY; a.c0 = s->delta;
  if (schur_mv<3>(a, SC_U, st)) return -1;
  // x += (U, -nX0 U ... ) : dU = X0 U - T0
  a.Mat = s->nX0; a.X = U; a.out = nullptr; a.aux = T0;
  if (schur_mv<4>(a, SC_DU, st)) return -1;
  return 0;
}
