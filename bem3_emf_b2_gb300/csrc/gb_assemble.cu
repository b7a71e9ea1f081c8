// gb_assemble.cu -- coefficient-matrix assembly of one domain on the GPU.
//
// Replaces create_cmatrix_domain (reference solve_bieq2.c:98-184) and the
// element dispatch dcoef_bd_node_t2 (d3b1_elem.c:482-539):
//   rows  (t,tn): collocation node tn of element t of the domain
//   cols  (s,n) : shape function n of source element s
//   G,H   [N][N], dG,dH [2N][N] (t_zeta, t_eta), dF [N][3], N = 4 Ne,
// all in the reference's row-major .cmat layout, written straight into HBM.
//
// Kernels
//   k_asm_regular   one thread per (row, source) pair, GLN x GLN rule; pairs
//                   whose |Re dF/dt| exceeds CBD_SDF are re-integrated with the
//                   GHN x GHN rule by the whole warp cooperatively (4096 points
//                   spread over 32 lanes) instead of stalling one lane.
//   k_asm_singular  one block per row for the pair s == t (polar / principal
//                   value integrals, ~45k points split over the block).
//   k_asm_rows      per row: solid-angle sums F, dF in source order
//                   s = 1..Ne (the reference's summation order), free term
//                   1 + F (domain 0) or F on the diagonal of H.
// Per-pair solid-angle terms go through a scratch array Fs[N][Ne][3] so the
// row sums are deterministic.
#include "gb_quad.cuh"
#include "gb_reduce.cuh"
#include "gb_internal.h"
#include <mutex>



struct AsmArgs {
  const double* cr;
  const double* cw;
  const int* etype;
  const double* ren;
  const int* sid;  // signed element ids of the domain, 1-based (sid[0] unused)
  int Ne;          // elements of the domain
  cplx k;
  int type;
  int did;
  cplx* G;
  cplx* H;
  cplx* dG;
  cplx* dH;
  double* dF;
  double* Fs;      // scratch [N][Ne][3]
};

// unit tangents at collocation node tn of element |td| (reference tz_te_bd_node d3b1_elem.c:122-143)
__device__ __forceinline__ void node_tangents(const Elem& T, int tn, double vt[2][3]) {
  for (int d = 0; d < 3; d++) {
    if (T.quad) {
      vt[0][d] = T.cr[d][1] + T.cr[d][3] * c_tab.et_44[tn];
      vt[1][d] = T.cr[d][2] + T.cr[d][3] * c_tab.zt_44[tn];
    } else {
      vt[0][d] = T.cr[d][1];
      vt[1][d] = T.cr[d][2];
    }
  }
  for (int i = 0; i < 2; i++) {
    double a = norm3(vt[i]);
    if (a != 0.0) { vt[i][0] /= a; vt[i][1] /= a; vt[i][2] /= a; }
  }
}

__device__ __forceinline__ void store_pair(const AsmArgs& a, size_t N, int row, int sidx, const RegAcc<2>& A) {
  size_t col = (size_t)sidx * 4;
  cplx* g = a.G + (size_t)row * N + col;
  cplx* h = a.H + (size_t)row * N + col;
  cplx* dg0 = a.dG + ((size_t)row * 2 + 0) * N + col;
  cplx* dg1 = a.dG + ((size_t)row * 2 + 1) * N + col;
  cplx* dh0 = a.dH + ((size_t)row * 2 + 0) * N + col;
  cplx* dh1 = a.dH + ((size_t)row * 2 + 1) * N + col;
#pragma unroll
  for (int n = 0; n < 4; n++) {
    g[n] = A.G[n];
    h[n] = A.H[n];
    dg0[n] = A.dG[0][n];
    dg1[n] = A.dG[1][n];
    dh0[n] = A.dH[0][n];
    dh1[n] = A.dH[1][n];
  }
  double* f = a.Fs + ((size_t)row * a.Ne + sidx) * 3;
  f[0] = A.F;
  f[1] = A.dF[0];
  f[2] = A.dF[1];
}

__global__ void __launch_bounds__(128) k_asm_regular(AsmArgs a) {
  const size_t N = (size_t)a.Ne * 4;
  const size_t npair = N * (size_t)a.Ne;
  size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  bool active = p < npair;
  int row = 0, sidx = 0;
  bool work = false, fb = false;
  Elem S;
  double rt[3], vt[2][3];
  RegAcc<2> A;
  bool neg = false;
  if (active) {
    row = (int)(p / a.Ne);
    sidx = (int)(p % a.Ne);
    int t = row / 4 + 1, tn = row % 4;
    int td = __ldg(a.sid + t);
    int s = sidx + 1;
    int sd = __ldg(a.sid + s);
    int atd = abs(td);
    Elem T;
    load_elem(T, a.cr, a.cw, a.etype, atd);
    bool rowok = T.quad || tn < 3;
    if (rowok && sd != td) {
      work = true;
      for (int d = 0; d < 3; d++) rt[d] = __ldg(a.ren + (size_t)atd * 12 + tn * 3 + d);
      node_tangents(T, tn, vt);
      load_elem(S, a.cr, a.cw, a.etype, abs(sd));
      neg = sd < 0;
      reg_integrate<2>(S, a.type, rt, vt, a.k, neg, A);
      if (a.type < 3 && (fabs(A.dF[0]) > GB_CBD_SDF || fabs(A.dF[1]) > GB_CBD_SDF)) fb = true;
    }
  }
  // near-singular fallback: the warp integrates each flagged pair together
  unsigned mask = __ballot_sync(0xffffffffu, fb);
  const int lane = threadIdx.x & 31;
  while (mask) {
    int src = __ffs(mask) - 1;
    mask &= mask - 1;
    // broadcast the flagged pair's geometry
    Elem Sb;
    double rtb[3], vtb[2][3];
    for (int i = 0; i < 12; i++) (&Sb.cr[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cr[0][0])[i], src);
    for (int i = 0; i < 9; i++) (&Sb.cw[0][0])[i] = __shfl_sync(0xffffffffu, (&S.cw[0][0])[i], src);
    Sb.quad = __shfl_sync(0xffffffffu, S.quad, src);
    for (int i = 0; i < 3; i++) rtb[i] = __shfl_sync(0xffffffffu, rt[i], src);
    for (int i = 0; i < 6; i++) (&vtb[0][0])[i] = __shfl_sync(0xffffffffu, (&vt[0][0])[i], src);
    bool negb = __shfl_sync(0xffffffffu, (int)neg, src) != 0;
    RegAcc<2> B;
    reg_integrate_gh_part<2>(Sb, lane, 32, rtb, vtb, a.k, B);
    warp_allreduce<sizeof(RegAcc<2>) / sizeof(double)>((double*)&B);
    reg_finish<2>(B, reg_scale_gh(Sb), negb);
    if (lane == src) A = B;
  }
  if (work) store_pair(a, N, row, sidx, A);
}

__global__ void __launch_bounds__(256) k_asm_singular(AsmArgs a) {
  __shared__ double red[51 * 8];
  const int row = blockIdx.x;
  const int t = row / 4 + 1, tn = row % 4;
  const int td = __ldg(a.sid + t);
  const int atd = abs(td);
  SingCtx c;
  load_elem(c.E, a.cr, a.cw, a.etype, atd);
  if (!c.E.quad && tn == 3) return;
  c.zt = c.E.quad ? c_tab.zt_44[tn] : c_tab.zt_34[tn];
  c.et = c.E.quad ? c_tab.et_44[tn] : c_tab.et_34[tn];
  c.k = a.k;
  sing_setup(c);
  SingAcc A;
  singacc_zero(A);
  int nit = sing_items(c, 1);
  for (int q = threadIdx.x; q < nit; q += blockDim.x) sing_item(c, q, A);
  static_assert(sizeof(SingAcc) == 51 * sizeof(double), "SingAcc layout");
  block_reduce<51>((double*)&A, red);
  if (threadIdx.x == 0) {
    sing_finish(c, A, td < 0);
    RegAcc<2> R;
    for (int n = 0; n < 4; n++) {
      R.G[n] = A.G[n];
      R.H[n] = A.H[n];
      R.dG[0][n] = A.dG[0][n];
      R.dG[1][n] = A.dG[1][n];
      R.dH[0][n] = A.dH[0][n];
      R.dH[1][n] = A.dH[1][n];
    }
    R.F = A.F;
    R.dF[0] = A.dF[0];
    R.dF[1] = A.dF[1];
    store_pair(a, (size_t)a.Ne * 4, row, t - 1, R);
  }
}

__global__ void k_asm_rows(AsmArgs a) {
  const size_t N = (size_t)a.Ne * 4;
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= (int)N) return;
  int t = row / 4 + 1, tn = row % 4;
  int td = __ldg(a.sid + t);
  if (__ldg(a.etype + abs(td)) == 0 && tn == 3) return;
  const double* f = a.Fs + (size_t)row * a.Ne * 3;
  double F = 0.0, Fz = 0.0, Fe = 0.0;
  for (int s = 0; s < a.Ne; s++) {
    F += f[3 * s + 0];
    Fz += f[3 * s + 1];
    Fe += f[3 * s + 2];
  }
  double diag = (a.did == 0) ? 1.0 + F : F;
  cplx* h = a.H + (size_t)row * N + (size_t)(t - 1) * 4 + tn;
  h->x += diag;
  a.dF[(size_t)row * 3 + 0] = diag;
  a.dF[(size_t)row * 3 + 1] = Fz;
  a.dF[(size_t)row * 3 + 2] = Fe;
}

// Assemble G,H,dG,dH,dF of one domain into device buffers.  Fs is scratch of
// 3 N Ne doubles.  Buffers are cleared here (rows of the unused fourth node of
// triangles and columns of the fourth shape function of triangles stay zero).
extern "C" int gbi_assemble_domain(const GbMeshDev* m, int did, int type, cplx* G, cplx* H, cplx* dG, cplx* dH,
                                   double* dF, double* Fs, cudaStream_t st) {
  int Ne = m->sb_Ne[did];
  if (Ne <= 0) return 0;
  size_t N = (size_t)Ne * 4;
  AsmArgs a;
  a.cr = m->cr;
  a.cw = m->cw;
  a.etype = m->etype;
  a.ren = m->ren;
  a.sid = m->sid + m->sb_off[did];
  a.Ne = Ne;
  a.k = cmk(m->kn[2 * did], m->kn[2 * did + 1]);
  a.type = type;
  a.did = did;
  a.G = G;
  a.H = H;
  a.dG = dG;
  a.dH = dH;
  a.dF = dF;
  a.Fs = Fs;
  GB_CUDA(cudaMemsetAsync(G, 0, N * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(H, 0, N * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(dG, 0, 2 * N * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(dH, 0, 2 * N * N * sizeof(cplx), st));
  GB_CUDA(cudaMemsetAsync(dF, 0, 3 * N * sizeof(double), st));
  GB_CUDA(cudaMemsetAsync(Fs, 0, 3 * N * (size_t)Ne * sizeof(double), st));
  size_t npair = N * (size_t)Ne;
  unsigned nb = (unsigned)((npair + 127) / 128);
  k_asm_regular<<<nb, 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  k_asm_singular<<<(unsigned)N, 256, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  k_asm_rows<<<(unsigned)((N + 127) / 128), 128, 0, st>>>(a);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

extern "C" int gbi_upload_tables_asm(const void* t) {
  GB_CUDA(cudaMemcpyToSymbol(c_tab, t, sizeof(GbTables)));
  return 0;
}

// ==================================================================== no allocation
// Allocation-free variant of the domain assembly (gb_assemble_domain_noalloc
// in gb_bem.h).  Some callers cannot allocate device memory: an application
// whose device memory is entirely owned by another allocator (a framework's
// caching pool holds the free memory, so a library cudaMalloc fails or
// fragments it), a latency-critical loop that cannot afford cudaFree's
// implicit device-wide synchronisation, or a code certified to allocate
// nothing after start-up.  This entry point takes every input and output from
// the caller and keeps its only scratch -- the per-pair solid-angle terms
// Fs[4 Ne][Ne][3] -- in the fixed array below, so it never calls cudaMalloc,
// cudaFree or an allocating library routine.
//
// The array is GB_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB) of static device
// memory: every GPU that loads this library holds it until the process exits.
// It limits a domain to GB_NOALLOC_MAX_NE elements (12 Ne^2 <= 2^21).
// All calls share the one array; it keeps the last call's contents and is
// cleared at the start of every call.  Calls that overlap on the GPU (two
// streams, or two host threads on one device) race on it and must be
// serialised by the caller.
#define GB_NOALLOC_SCRATCH_DOUBLES (2u * 1024u * 1024u)
#define GB_NOALLOC_MAX_NE 418
static __device__ __align__(256) double g_noalloc_scratch[GB_NOALLOC_SCRATCH_DOUBLES];

// Host code may not use g_noalloc_scratch's name as a device address: the
// device address is looked up once per device (with that device current) by
// cudaGetSymbolAddress and cached here.
static double* g_noalloc_dev_ptr[64];
static std::mutex g_noalloc_mu;

static int noalloc_scratch_ptr(double** out) {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { gbi_set_error("gb_assemble_domain_noalloc: device ordinal %d not supported", dev); return -1; }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_dev_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      gbi_set_error("gb_assemble_domain_noalloc: cudaGetSymbolAddress of the scratch failed: %s", cudaGetErrorString(e));
      return -1;
    }
    g_noalloc_dev_ptr[dev] = (double*)p;
  }
  *out = g_noalloc_dev_ptr[dev];
  return 0;
}

extern "C" int gbi_ensure_tables(void);

extern "C" int gb_assemble_domain_noalloc(const double* cr, const double* cw, const int* etype, const double* ren,
                                          const int* sid, int Ne, double k_re, double k_im, int did, int type, void* G,
                                          void* H, void* dG, void* dH, double* dF, void* stream) {
  if (Ne < 1 || Ne > GB_NOALLOC_MAX_NE) {
    gbi_set_error("gb_assemble_domain_noalloc: %d elements in the domain; this entry point supports 1..%d "
                  "(fixed 16 MiB scratch); use gb_assemble for larger domains", Ne, GB_NOALLOC_MAX_NE);
    return -1;
  }
  if (type < 0 || type > 3) { gbi_set_error("gb_assemble_domain_noalloc: quadrature type %d not in 0..3", type); return -1; }
  if (did < 0 || did >= GB_MAXDOM) { gbi_set_error("gb_assemble_domain_noalloc: domain id %d not in 0..%d", did, GB_MAXDOM - 1); return -1; }
  if (!cr || !cw || !etype || !ren || !sid || !G || !H || !dG || !dH || !dF) {
    gbi_set_error("gb_assemble_domain_noalloc: null input or output pointer");
    return -1;
  }
  double* scratch = nullptr;
  if (noalloc_scratch_ptr(&scratch)) return -1;
  if (gbi_ensure_tables()) return -1;
  GbMeshDev m;
  memset(&m, 0, sizeof(m));
  m.cr = (double*)cr;
  m.cw = (double*)cw;
  m.ren = (double*)ren;
  m.etype = (int*)etype;
  m.sid = (int*)sid;
  m.sb_Ne[did] = Ne;
  m.sb_off[did] = 0;
  m.kn[2 * did] = k_re;
  m.kn[2 * did + 1] = k_im;
  return gbi_assemble_domain(&m, did, type, (cplx*)G, (cplx*)H, (cplx*)dG, (cplx*)dH, dF, scratch, (cudaStream_t)stream);
}
