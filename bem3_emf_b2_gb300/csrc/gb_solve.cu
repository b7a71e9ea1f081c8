// gb_solve.cu -- kernels of the multi-object iteration (reference mo_solve.c).
//
//   k_build_B_prep + k_b_gather  right-hand side B of the coupled system
//               from the incident potential at the exterior nodes
//               (create_Bmatrix_dac, mo_solve.c:150-244) as rows of H P + G Q
//               (the row product of gb_linalg.cu)
//   k_store_bv  unpack X = invA B into U, dU of every domain (tmatrix_bd_store :457-545)
//   k_eh_bv     E, H at the nodes from U, dU and the tangential derivative
//               matrices dG, dH, dF (solve_eh_bv :547-661)
//   k_deh_build compressed G and the 6 right-hand sides H [E H] of the
//               normal-derivative solve (solve_deh_bv :663-789)
//   k_ccd       convergence measure (ccd_f :413-455), one block, fixed order
// One warp per matrix row for the row sums (lanes over columns).
#include "gb_common.cuh"
#include "gb_internal.h"

__device__ __forceinline__ void unit_normal(const double* wen, int asd, int l, double vn[3]) {
  for (int d = 0; d < 3; d++) vn[d] = wen[(size_t)asd * 12 + l * 3 + d];
  double a = sqrt(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
  if (a != 0.0) { vn[0] /= a; vn[1] /= a; vn[2] /= a; }
}

struct BArgs {
  const cplx* G;
  const cplx* H;
  const int* sid;
  const int* rowk;
  const int* md;
  const int* sd;
  const int* etype;
  const double* wen;
  const double* kn;
  const cplx* Ui;   // [(Ne+1)][4][4]
  const cplx* dUi;
  int Ne, did, nrows;
  size_t base;
  cplx* B;
};

// per source element of the domain, the constants of the right-hand side: the
// interface factors of its (main, sub) media and the unit normals at its
// nodes (the same operations as before, done once per element instead of
// once per row and component)
struct BElem {
  cplx delt, beps, sigm;
  double vn[4][3];
  int asd, nl, active;
};
__global__ void k_build_B_prep(BArgs a, BElem* E) {
  const int s = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  if (s > a.Ne) return;
  BElem e;
  const int sd = a.sid[s], asd = abs(sd);
  const int mdid = a.md[asd], sdid = a.sd[asd];
  e.asd = asd;
  e.nl = a.etype[asd] ? 4 : 3;
  e.active = !(a.did == mdid || mdid != 0);
  const cplx k1 = cmk(a.kn[2 * mdid], a.kn[2 * mdid + 1]), k2 = cmk(a.kn[2 * sdid], a.kn[2 * sdid + 1]);
  const cplx k12 = k1 * k1, k22 = k2 * k2;
  e.delt = k12 - k22;
  e.beps = cdivc(k12, k22);
  e.sigm = cmk(1.0, 0.0) - e.beps;
  for (int l = 0; l < 4; l++) {
    double vn[3] = {0.0, 0.0, 0.0};
    if (l < e.nl) unit_normal(a.wen, asd, l, vn);
    for (int d = 0; d < 3; d++) e.vn[l][d] = vn[d];
  }
  E[s - 1] = e;
}


// The same right-hand side as the rows of H P + G Q: per column (source
// element s, node l) the four components of P = -Ui and of Q = -(dUi + the
// interface terms) -- the column form of the reference's row sum, so that B is
// one product of G and H with four vectors (k_apply_rows / _df)
__global__ void k_b_gather(BArgs a, const BElem* __restrict__ E, cplx* PQ) {
  const size_t N = (size_t)a.Ne * 4;
  const size_t col = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= N) return;
  const int s = (int)(col / 4) + 1, l = (int)(col % 4);
  const BElem& e = E[s - 1];
  cplx P[4], Q[4];
  for (int q = 0; q < 4; q++) { P[q] = cmk(0.0, 0.0); Q[q] = cmk(0.0, 0.0); }
  if (e.active && l < e.nl) {
    const cplx* ui = a.Ui + ((size_t)e.asd * 4 + l) * 4;
    const cplx* dui = a.dUi + ((size_t)e.asd * 4 + l) * 4;
    const double* vn = e.vn[l];
    for (int c = 0; c < 3; c++) {
      P[c] = -ui[c];
      Q[c] = -(dui[c] + ui[3] * (e.delt * vn[c]));
    }
    const cplx un = ui[0] * vn[0] + ui[1] * vn[1] + ui[2] * vn[2];
    P[3] = -ui[3];
    Q[3] = -(e.sigm * un + e.beps * dui[3]);
  }
  for (int q = 0; q < 4; q++) { PQ[(size_t)q * N + col] = P[q]; PQ[(size_t)(4 + q) * N + col] = Q[q]; }
}

extern "C" int gbi_rows_apply(const cplx* G, const cplx* H, const void* Gd, const void* Hd, const int* rowk, int Ne,
                              int nrows, size_t base, cplx* PQ, void* PQd, cplx* y, cudaStream_t st);

// B of one domain; Gd, Hd (may be null): double-float copies of G, H, which
// take the products onto the FP32 pipes (the chosen form)
extern "C" int gbi_build_B(const cplx* G, const cplx* H, const void* Gd, const void* Hd, const int* sid,
                           const int* rowk, const GbMeshDev* m, const double* kn_dev, const cplx* Ui, const cplx* dUi,
                           int did, int nrows, size_t base, cplx* B, cudaStream_t st) {
  BArgs a;
  a.G = G; a.H = H; a.sid = sid; a.rowk = rowk; a.md = m->md; a.sd = m->sd; a.etype = m->etype; a.wen = m->wen;
  a.kn = kn_dev; a.Ui = Ui; a.dUi = dUi; a.Ne = m->sb_Ne[did]; a.did = did; a.nrows = nrows; a.base = base; a.B = B;
  const size_t N = 4 * (size_t)a.Ne;
  if (N == 0) return 0;
  BElem* E = nullptr;
  cplx* PQ = nullptr;
  void* PQd = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&E, (size_t)a.Ne * sizeof(BElem), st));
  GB_CUDA(cudaMallocAsync((void**)&PQ, 8 * N * sizeof(cplx), st));
  if (Gd) GB_CUDA(cudaMallocAsync(&PQd, 8 * N * 16, st));
  k_build_B_prep<<<(unsigned)((a.Ne + 127) / 128), 128, 0, st>>>(a, E);
  gbi_count_launch();
  k_b_gather<<<(unsigned)((N + 255) / 256), 256, 0, st>>>(a, E, PQ);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  const int rc = gbi_rows_apply(G, H, Gd, Hd, rowk, a.Ne, nrows, base, PQ, PQd, B, st);
  cudaFreeAsync(E, st);
  cudaFreeAsync(PQ, st);
  if (PQd) cudaFreeAsync(PQd, st);
  return rc;
}

struct StoreArgs {
  const cplx* X;
  const int* sid;
  const int* eni;
  const int* md;
  const int* sd;
  const int* etype;
  const double* wen;
  const double* kn;
  const cplx* Ui;
  const cplx* dUi;
  int Ne, did;
  size_t nn;
  cplx* U;   // domain boundary values [(Ne_d+1)][4][4]
  cplx* dU;
};

__global__ void k_store_bv(StoreArgs a) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.Ne * 4) return;
  int s = p / 4 + 1, l = p % 4;
  int sd = a.sid[s], asd = abs(sd);
  int mdid = a.md[asd], sdid = a.sd[asd];
  if (l == 3 && a.etype[asd] == 0) return;
  size_t c = (size_t)a.eni[asd * 4 + l];
  const size_t nn = a.nn;
  cplx* U = a.U + ((size_t)s * 4 + l) * 4;
  cplx* dU = a.dU + ((size_t)s * 4 + l) * 4;
  if (a.did == mdid) {
    for (int i = 0; i < 4; i++) {
      U[i] = a.X[nn * (i + 0) + c];
      dU[i] = a.X[nn * (i + 4) + c];
    }
    return;
  }
  cplx k1 = cmk(a.kn[2 * mdid], a.kn[2 * mdid + 1]), k2 = cmk(a.kn[2 * sdid], a.kn[2 * sdid + 1]);
  cplx k12 = k1 * k1, k22 = k2 * k2;
  cplx delt = k12 - k22, beps = cdivc(k12, k22), sigm = cmk(1.0, 0.0) - beps;
  double n[3];
  unit_normal(a.wen, asd, l, n);
  cplx tU[4], tUi[3];
  tU[3] = a.X[nn * 3 + c];
  const cplx* ui = a.Ui + ((size_t)asd * 4 + l) * 4;
  const cplx* dui = a.dUi + ((size_t)asd * 4 + l) * 4;
  for (int i = 0; i < 3; i++) {
    tU[i] = a.X[nn * (i + 0) + c];
    U[i] = tU[i];
    dU[i] = -(a.X[nn * (i + 4) + c] + (delt * tU[3]) * n[i]);
    if (mdid == 0) {
      tUi[i] = ui[i];
      U[i] += tUi[i];
      dU[i] -= dui[i];
    }
  }
  U[3] = tU[3];
  dU[3] = -(beps * a.X[nn * 7 + c] + sigm * (tU[0] * n[0] + tU[1] * n[1] + tU[2] * n[2]));
  if (mdid == 0) dU[3] -= sigm * (tUi[0] * n[0] + tUi[1] * n[1] + tUi[2] * n[2]);
}

extern "C" int gbi_store_bv(const cplx* X, const GbMeshDev* m, const double* kn_dev, const cplx* Ui, const cplx* dUi,
                            int did, cplx* U, cplx* dU, cudaStream_t st) {
  StoreArgs a;
  a.X = X; a.sid = m->sid + m->sb_off[did]; a.eni = m->eni; a.md = m->md; a.sd = m->sd; a.etype = m->etype;
  a.wen = m->wen; a.kn = kn_dev; a.Ui = Ui; a.dUi = dUi; a.Ne = m->sb_Ne[did]; a.did = did; a.nn = (size_t)m->NN;
  a.U = U; a.dU = dU;
  int n = a.Ne * 4;
  if (n == 0) return 0;
  k_store_bv<<<(n + 127) / 128, 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------ E, H
struct EHArgs {
  const cplx* dG;  // [2N][N]
  const cplx* dH;
  const double* dF;  // [N][3]
  const int* sid;
  const int* etype;
  const double* cr;
  const double* wen;
  const cplx* U;
  const cplx* dU;
  int Ne;
  double lambda0;
  cplx* E;
  cplx* H;
};

__global__ void k_eh_bv(EHArgs a) {
  const int lane = threadIdx.x & 31;
  int row = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  size_t N = (size_t)a.Ne * 4;
  if (row >= (int)N) return;
  int t = row / 4 + 1, tn = row % 4;
  int at = a.sid[t], atd = abs(at);
  int quad = a.etype[atd];
  if (tn == 3 && !quad) return;
  const cplx* g0 = a.dG + ((size_t)row * 2 + 0) * N;
  const cplx* g1 = a.dG + ((size_t)row * 2 + 1) * N;
  const cplx* h0 = a.dH + ((size_t)row * 2 + 0) * N;
  const cplx* h1 = a.dH + ((size_t)row * 2 + 1) * N;
  double acc[16];
  for (int i = 0; i < 16; i++) acc[i] = 0.0;
  for (size_t col = lane; col < N; col += 32) {
    size_t s = col / 4 + 1, sn = col % 4;
    const cplx* U = a.U + (s * 4 + sn) * 4;
    const cplx* dU = a.dU + (s * 4 + sn) * 4;
    cplx G0 = g0[col], G1 = g1[col], H0 = h0[col], H1 = h1[col];
    for (int i = 0; i < 4; i++) {
      cplx z = G0 * dU[i] - H0 * U[i];
      cplx e = G1 * dU[i] - H1 * U[i];
      acc[2 * i] += z.x;
      acc[2 * i + 1] += z.y;
      acc[8 + 2 * i] += e.x;
      acc[9 + 2 * i] += e.y;
    }
  }
  for (int i = 0; i < 16; i++)
    for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
  if (lane != 0) return;
  // tangents, normal (with the side's sign), inverse of [n tz te]
  double vtz[3], vte[3], vn[3];
  const double P = 0.5773502691896257645091;
  const double zt44[4] = {-P, P, P, -P}, et44[4] = {-P, -P, P, P};
  for (int d = 0; d < 3; d++) {
    const double* c = a.cr + (size_t)atd * 12 + d * 4;
    if (quad) { vtz[d] = c[1] + c[3] * et44[tn]; vte[d] = c[2] + c[3] * zt44[tn]; }
    else { vtz[d] = c[1]; vte[d] = c[2]; }
    vn[d] = (at < 0 ? -1.0 : 1.0) * a.wen[(size_t)atd * 12 + tn * 3 + d];
  }
  double nz = norm3(vtz), ne = norm3(vte), nv = norm3(vn);
  for (int d = 0; d < 3; d++) { vtz[d] /= nz; vte[d] /= ne; vn[d] /= nv; }
  double m[9];
  double idet = 1.0 / (vn[0] * vtz[1] * vte[2] + vn[1] * vtz[2] * vte[0] + vn[2] * vtz[0] * vte[1] -
                       (vn[2] * vtz[1] * vte[0] + vn[1] * vtz[0] * vte[2] + vn[0] * vtz[2] * vte[1]));
  m[0] = vtz[1] * vte[2] - vtz[2] * vte[1];
  m[1] = -vn[1] * vte[2] + vn[2] * vte[1];
  m[2] = vn[1] * vtz[2] - vn[2] * vtz[1];
  m[3] = -vtz[0] * vte[2] + vtz[2] * vte[0];
  m[4] = vn[0] * vte[2] - vn[2] * vte[0];
  m[5] = -vn[0] * vtz[2] + vn[2] * vtz[0];
  m[6] = vtz[0] * vte[1] - vtz[1] * vte[0];
  m[7] = -vn[0] * vte[1] + vn[1] * vte[0];
  m[8] = vn[0] * vtz[1] - vn[1] * vtz[0];
  for (int i = 0; i < 9; i++) m[i] *= idet;
  const double* df = a.dF + (size_t)row * 3;
  const cplx* U = a.U + ((size_t)t * 4 + tn) * 4;
  const cplx* dU = a.dU + ((size_t)t * 4 + tn) * 4;
  cplx dUz[4], dUe[4];
  for (int i = 0; i < 4; i++) {
    dUz[i] = cdivr(cmk(acc[2 * i], acc[2 * i + 1]) - U[i] * df[1], df[0]);
    dUe[i] = cdivr(cmk(acc[8 + 2 * i], acc[9 + 2 * i]) - U[i] * df[2], df[0]);
  }
  // gradient component i of potential l: dU_n m[i][0] + dU_tz m[i][1] + dU_te m[i][2]
  auto grad = [&](int i, int l) { return dU[l] * m[i * 3 + 0] + dUz[l] * m[i * 3 + 1] + dUe[l] * m[i * 3 + 2]; };
  cplx* E = a.E + ((size_t)t * 4 + tn) * 3;
  cplx* H = a.H + ((size_t)t * 4 + tn) * 3;
  for (int i = 0; i < 3; i++) E[i] = U[i] - grad(i, 3);
  cplx ch = cmk(0.0, -a.lambda0 / (2.0 * GB_PI));
  H[0] = ch * (grad(1, 2) - grad(2, 1));
  H[1] = ch * (grad(2, 0) - grad(0, 2));
  H[2] = ch * (grad(0, 1) - grad(1, 0));
}

extern "C" int gbi_eh_bv(const cplx* dG, const cplx* dH, const double* dF, const GbMeshDev* m, int did, double lambda0,
                         const cplx* U, const cplx* dU, cplx* E, cplx* H, cudaStream_t st) {
  EHArgs a;
  a.dG = dG; a.dH = dH; a.dF = dF; a.sid = m->sid + m->sb_off[did]; a.etype = m->etype; a.cr = m->cr; a.wen = m->wen;
  a.U = U; a.dU = dU; a.Ne = m->sb_Ne[did]; a.lambda0 = lambda0; a.E = E; a.H = H;
  size_t warps = 4 * (size_t)a.Ne;
  if (!warps) return 0;
  k_eh_bv<<<(unsigned)((warps * 32 + 127) / 128), 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// compressed row rk of G (columns of unused fourth nodes dropped) and
// B = H_row [E H] (6 right-hand sides)
__global__ void k_deh_build(const cplx* G, const cplx* H, const int* rowk, int Ne, int nn, const cplx* E, const cplx* Hf,
                            cplx* Ac, cplx* Bc) {
  const int lane = threadIdx.x & 31;
  int row = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  size_t N = (size_t)Ne * 4;
  if (row >= (int)N) return;
  int k = rowk[row];
  if (k < 0) return;
  const cplx* g = G + (size_t)row * N;
  const cplx* h = H + (size_t)row * N;
  double acc[12];
  for (int i = 0; i < 12; i++) acc[i] = 0.0;
  for (size_t col = lane; col < N; col += 32) {
    int kc = rowk[col];
    if (kc < 0) continue;
    Ac[(size_t)k * nn + kc] = g[col];
    size_t s = col / 4 + 1, sn = col % 4;
    cplx hv = h[col];
    for (int i = 0; i < 3; i++) {
      cplx e = hv * E[(s * 4 + sn) * 3 + i];
      cplx f = hv * Hf[(s * 4 + sn) * 3 + i];
      acc[2 * i] += e.x;
      acc[2 * i + 1] += e.y;
      acc[6 + 2 * i] += f.x;
      acc[7 + 2 * i] += f.y;
    }
  }
  for (int i = 0; i < 12; i++)
    for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_down_sync(0xffffffffu, acc[i], o);
  if (lane == 0)
    for (int i = 0; i < 6; i++) Bc[(size_t)k * 6 + i] = cmk(acc[2 * i], acc[2 * i + 1]);
}

__global__ void k_deh_scatter(const cplx* Bc, const int* rowk, int Ne, cplx* dE, cplx* dHf) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= Ne * 4) return;
  int k = rowk[p];
  if (k < 0) return;
  size_t s = p / 4 + 1, sn = p % 4;
  for (int i = 0; i < 3; i++) {
    dE[(s * 4 + sn) * 3 + i] = Bc[(size_t)k * 6 + i];
    dHf[(s * 4 + sn) * 3 + i] = Bc[(size_t)k * 6 + 3 + i];
  }
}

extern "C" int gbi_deh_build(const cplx* G, const cplx* H, const int* rowk, int Ne, int nn, const cplx* E, const cplx* Hf,
                             cplx* Ac, cplx* Bc, cudaStream_t st) {
  size_t warps = 4 * (size_t)Ne;
  if (!warps) return 0;
  GB_CUDA(cudaMemsetAsync(Ac, 0, (size_t)nn * nn * sizeof(cplx), st));
  k_deh_build<<<(unsigned)((warps * 32 + 127) / 128), 128, 0, st>>>(G, H, rowk, Ne, nn, E, Hf, Ac, Bc);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbi_deh_scatter(const cplx* Bc, const int* rowk, int Ne, cplx* dE, cplx* dHf, cudaStream_t st) {
  if (!Ne) return 0;
  k_deh_scatter<<<(Ne * 4 + 127) / 128, 128, 0, st>>>(Bc, rowk, Ne, dE, dHf);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------------ incident field
// Ui[idx] += out[0..3], dUi[idx] += out[4..7] for the exterior nodes of an object
__global__ void k_add_incident(int n, const int* idx, const cplx* out, cplx* Ui, cplx* dUi, const int* did, int* bad) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (did[p] != 0) { atomicExch(bad, 1000 + did[p]); return; }
  size_t q = (size_t)idx[p] * 4;
  for (int l = 0; l < 4; l++) {
    Ui[q + l] += out[(size_t)p * 8 + l];
    dUi[q + l] += out[(size_t)p * 8 + 4 + l];
  }
}

extern "C" int gbi_add_incident(int n, const int* idx, const cplx* out, cplx* Ui, cplx* dUi, const int* did, int* bad,
                                cudaStream_t st) {
  if (n <= 0) return 0;
  k_add_incident<<<(n + 127) / 128, 128, 0, st>>>(n, idx, out, Ui, dUi, did, bad);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// convergence sums over the exterior element nodes (fixed order, one block)
__global__ void k_ccd(int Ne, const int* md, const cplx* Ui, const cplx* Uip, double* out) {
  __shared__ double su[256], sp[256];
  __shared__ int sc[256];
  double us = 0.0, ps = 0.0;
  int c = 0;
  for (int q = threadIdx.x; q < Ne * 4; q += blockDim.x) {
    int s = q / 4 + 1, p = q % 4;
    if (md[s] != 0) continue;
    const cplx* tc = Ui + ((size_t)s * 4 + p) * 4;
    const cplx* tp = Uip + ((size_t)s * 4 + p) * 4;
    double ac = cabs2(tc[0]) + cabs2(tc[1]) + cabs2(tc[2]);
    double ap = cabs2(tp[0]) + cabs2(tp[1]) + cabs2(tp[2]);
    double dcp = cabs2(tc[0] - tp[0]) + cabs2(tc[1] - tp[1]) + cabs2(tc[2] - tp[2]);
    us += 2.0 * dcp / (ac + ap);
    double bc = cabs2(tc[3]), bp = cabs2(tp[3]), db = cabs2(tc[3] - tp[3]);
    ps += 2.0 * db / (bc + bp);
    c++;
  }
  su[threadIdx.x] = us;
  sp[threadIdx.x] = ps;
  sc[threadIdx.x] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    int n = 0;
    for (int i = 0; i < blockDim.x; i++) { a += su[i]; b += sp[i]; n += sc[i]; }
    out[0] = a;
    out[1] = b;
    out[2] = (double)n;
  }
}

extern "C" int gbi_ccd(int Ne, const int* md, const cplx* Ui, const cplx* Uip, double* out, cudaStream_t st) {
  k_ccd<<<1, 256, 0, st>>>(Ne, md, Ui, Uip, out);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}
