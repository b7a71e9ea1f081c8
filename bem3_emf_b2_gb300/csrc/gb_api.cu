// gb_api.cu -- the C ABI (gb_bem.h): device-resident BEM objects.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <mutex>
#include <vector>
#include <thread>
#include <string>
#include "gb_common.cuh"
#include "gb_internal.h"
#include "gb_bem.h"
#include "gb_fieldobj.cuh"

extern "C" {
void gauleg(double x1, double x2, double x[], double w[], int n);
int gbi_upload_tables_asm(const void* t);
int gbi_upload_tables_field(const void* t);
int gbi_assemble_domain(const GbMeshDev* m, int did, int type, cplx* G, cplx* H, cplx* dG, cplx* dH, double* dF,
                        double* Fs, cudaStream_t st);
int gbi_assemble_domain2(const GbMeshDev* m, int did, int type, int precision, cplx* G, cplx* H, cplx* dG, cplx* dH,
                         double* dF, double* Fs, cudaStream_t st);
int gbi_assemble_rows(const GbMeshDev* m, int did, int type, int precision, int row0, int nrow, cplx* G, cplx* H,
                      cplx* dG, cplx* dH, double* dF, double* Fs, cudaStream_t st);
int gbi_assemble_list(const GbAsmItem* d, int n, int type, int precision, cudaStream_t st);
int gbi_build_A_domain(const cplx* G, const cplx* H, const int* sid, const int* rowk, const GbMeshDev* m,
                       const double* kn_dev, int did, int nrows, size_t base, size_t na, cplx* A, cudaStream_t st);
int gbi_zgetrf(cplx* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
int gbi_zgetrs(const cplx* LU, size_t lda, int n, const int64_t* ipiv, cplx* X, size_t ldx, int nrhs, cudaStream_t st);
int gbi_zinverse(const cplx* LU, size_t lda, int n, const int64_t* ipiv, cplx* X, size_t ldx, cudaStream_t st);
int gbi_zgemv(const cplx* M, size_t ldm, int n, int ncol, const cplx* x, cplx* y, cudaStream_t st);
int gbi_build_B(const cplx* G, const cplx* H, const void* Gd, const void* Hd, const int* sid, const int* rowk,
                const GbMeshDev* m, const double* kn_dev, const cplx* Ui, const cplx* dUi, int did, int nrows, size_t base,
                cplx* B, cudaStream_t st);
int gbi_store_bv(const cplx* X, const GbMeshDev* m, const double* kn_dev, const cplx* Ui, const cplx* dUi, int did,
                 cplx* U, cplx* dU, cudaStream_t st);
int gbi_eh_bv(const cplx* dG, const cplx* dH, const double* dF, const GbMeshDev* m, int did, double lambda0,
              const cplx* U, const cplx* dU, cplx* E, cplx* H, cudaStream_t st);
int gbi_deh_build(const cplx* G, const cplx* H, const int* rowk, int Ne, int nn, const cplx* E, const cplx* Hf, cplx* Ac,
                  cplx* Bc, cudaStream_t st);
int gbi_deh_scatter(const cplx* Bc, const int* rowk, int Ne, cplx* dE, cplx* dHf, cudaStream_t st);
int gbi_add_incident(int n, const int* idx, const cplx* out, cplx* Ui, cplx* dUi, const int* did, int* bad,
                     cudaStream_t st);
int gbi_ccd(int Ne, const int* md, const cplx* Ui, const cplx* Uip, double* out, cudaStream_t st);
int gbi_domain_id(const FieldObj* o, int n, const double* rt, int* did, cudaStream_t st);
int gbi_field(const FieldObj* o, int mode, int type, int n, const double* rt, const double* v, const int* did, cplx* out,
              int* flag, cudaStream_t st);
int gbi_field_bd(const FieldObj* o, int type, int n, const int* did, const int* t, const double* zt, cplx* out,
                 cudaStream_t st);
int gbi_cross_build(const FieldObj* o, int type, int n, const double* rt, const double* v, int C, cplx* Gm, cplx* Hm,
                    cplx* dGm, cplx* dHm, double* Fp, int dfout, cudaStream_t st);
int gbi_cross_apply(int n, int C, const cplx* Gm, const cplx* Hm, const cplx* dGm, const cplx* dHm, const double* Fp,
                    const cplx* U, const cplx* dU, cplx* out, int dfin, cudaStream_t st);
int gbi_cgetrf(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
int gbi_build_A32_domain(const cplx* G, const cplx* H, const int* sid, const int* rowk, const GbMeshDev* m,
                         const double* kn_dev, int did, int nrows, size_t base, size_t na, cplxf* A32, cudaStream_t st);
int gbi_apply_A_domain(const cplx* G, const cplx* H, const int* sid, const int* rowk, const GbMeshDev* m,
                       const double* kn_dev, int did, int nrows, size_t base, const cplx* x, cplx* PQ, cplx* y,
                       cudaStream_t st);
int gbi_resid_finish(const cplx* b, const cplx* y, cplx* r, size_t n, double* nrm, cudaStream_t st);
int gbi_zgesv_mixed(const cplx* A, int n, const cplx* B, int nrhs, cplx* X, int* iters, double* relres, cudaStream_t st);
int gbi_ir_step(cplx* x, const cplx* r, cplxf* d, cplxf* d2, const cplxf* LU32, size_t lda, int n, const int* perm,
                cudaStream_t st);
int gbi_ir_step_rbt(cplx* x, const cplx* r, cplxf* d, cplxf* d2, const cplxf* LU32, size_t lda, int n, const int* perm,
                    const float* pu, const float* pv, cudaStream_t st);
int gbi_rbt_matrix(cplxf* A, size_t lda, int n, const float* pu, const float* pv, cudaStream_t st);
int gbi_cgetrf_nopiv(cplxf* A, size_t lda, int n, int64_t* ipiv, int* info, cudaStream_t st);
void gbi_rbt_params(int n, float* h);
int gbi_make_perm(const int64_t* ipiv, int n, int* perm, cudaStream_t st);
int gbi_perm_identity(int n, int* perm, cudaStream_t st);
int gbi_zsolve_multi(const cplx* LU, size_t lda, int n, const int* perm, const cplx* X, size_t ldx, int nrhs, cplx* Y,
                     cudaStream_t st);
struct GbSchur;
int gbi_schur_create(int n, int fp64, GbSchur** out);
void gbi_schur_destroy(GbSchur* s);
int gbi_schur_factor(GbSchur* s, const GbMeshDev* m, const cplx* G0, const cplx* H0, const cplx* G1, const cplx* H1,
                     const int* sid0, const int* sid1, const int* rowk0, const int* rowk1, cudaStream_t st);
int gbi_schur_apply(GbSchur* s, const cplx* r, cplx* x, cudaStream_t st);
void gbi_schur_mats(GbSchur* s, void** out);
int gbi_schur_prepare(GbSchur* s, const GbMeshDev* m, cudaStream_t st);
}
#include <functional>
typedef std::function<int(const cplx* x, cplx* y, cudaStream_t st)> GbOp;
extern "C" int gbi_gmres(size_t n, const cplx* b, cplx* x, bool x_zero, const GbOp& A, const GbOp* Af, const GbOp& M,
                         int m, double tol, int maxit, cudaStream_t st, const cplx* Ax0, cplx* Ax_out, int* ax_ok,
                         int* iters, double* relres);
extern "C" int gbi_to_df(size_t n, const cplx* src, void* dst, cudaStream_t st);
extern "C" int gbi_apply_A_domain_df(const void* Gd, const void* Hd, const int* sid, const int* rowk, const GbMeshDev* m,
                          const double* kn_dev, int did, int nrows, size_t base, const cplx* x, cplx* PQ, void* PQd,
                          cplx* y, cudaStream_t st);

// ------------------------------------------------------------------ errors
static thread_local char g_err[1024];
extern "C" void gbi_set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
extern "C" const char* gb_last_error(void) { return g_err; }

// number of kernel launches made by this library (all threads)
#include <atomic>
static std::atomic<unsigned long long> g_launches{0};
extern "C" void gbi_count_launch(void) { g_launches.fetch_add(1, std::memory_order_relaxed); }
extern "C" unsigned long long gb_launch_count(void) { return g_launches.load(); }
extern "C" void* gb_obj_stream(gb_obj* o);

// ------------------------------------------------------------------ tables
// The quadrature tables live in __constant__ memory, which every device holds
// separately: they are uploaded once per device (a blocking copy), so that a
// process that moves between devices uploads nothing on later calls.
static std::mutex g_init_mu;
static bool g_tables_done[64];

static int ensure_tables() {
  int dev;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { gbi_set_error("device ordinal %d not supported", dev); return -1; }
  std::lock_guard<std::mutex> lk(g_init_mu);
  if (g_tables_done[dev]) return 0;
  GbTables t;
  memset(&t, 0, sizeof(t));
  gauleg(-1.0, 1.0, t.xli, t.wli, GB_GLN);
  gauleg(-1.0, 1.0, t.xhi, t.whi, GB_GHN);
  for (int n = 1; n < GB_GLN; n++) gauleg(-1.0, 1.0, t.xn + n * (n - 1) / 2, t.wn + n * (n - 1) / 2, n);
  for (int i = 0; i < GB_GLN; i++) {  // the GLN rule itself: the reference's table
    t.xn[GB_GLN * (GB_GLN - 1) / 2 + i] = t.xli[i];
    t.wn[GB_GLN * (GB_GLN - 1) / 2 + i] = t.wli[i];
  }
  const double a = GB_P44_N;
  const double z44[4] = {-a, a, a, -a}, e44[4] = {-a, -a, a, a};
  const double n9 = 0.7745966692414833770359;
  const double w0 = 0.3086419753086419753086, w1 = 0.4938271604938271604938, w2 = 0.7901234567901234567901;
  const double z49[9] = {-n9, n9, n9, -n9, 0.0, n9, 0.0, -n9, 0.0};
  const double e49[9] = {-n9, -n9, n9, n9, -n9, 0.0, n9, 0.0, 0.0};
  const double w49[9] = {w0, w0, w0, w0, w1, w1, w1, w1, w2};
  const double p0 = 0.2, p1 = 0.3464101615137754587055;
  const double z34[4] = {-p0, 2.0 * p0, -p0, 0.0}, e34[4] = {-p1, 0.0, p1, 0.0};
  const double w34[4] = {0.5208333333333333333333, 0.5208333333333333333333, 0.5208333333333333333333, -0.5625};
  const double q0 = 0.3480702390148154917985, q1 = 0.2052130961576726346557, q2 = 0.6028753385763033130539,
               q3 = 0.3554395089236065568357;
  const double v0 = 0.1259391805448271525957, v1 = 0.1323941527885061807376, v2 = 0.225;
  const double z37[7] = {-q0, 2.0 * q0, -q0, q1, -2.0 * q1, q1, 0.0};
  const double e37[7] = {-q2, 0.0, q2, q3, 0.0, -q3, 0.0};
  const double w37[7] = {v0, v0, v0, v1, v1, v1, v2};
  for (int i = 0; i < 4; i++) {
    t.zt_44[i] = z44[i]; t.et_44[i] = e44[i]; t.wt_44[i] = 1.0;
    t.zt_34[i] = z34[i]; t.et_34[i] = e34[i]; t.wt_34[i] = w34[i];
  }
  for (int i = 0; i < 9; i++) { t.zt_49[i] = z49[i]; t.et_49[i] = e49[i]; t.wt_49[i] = w49[i]; }
  for (int i = 0; i < 7; i++) { t.zt_37[i] = z37[i]; t.et_37[i] = e37[i]; t.wt_37[i] = w37[i]; }
  if (gbi_upload_tables_asm(&t)) return -1;
  if (gbi_upload_tables_field(&t)) return -1;
  g_tables_done[dev] = true;
  return 0;
}

extern "C" int gbi_ensure_tables(void) { return ensure_tables(); }

extern "C" int gb_device_memory(size_t* free_bytes, size_t* total_bytes) {
  GB_CUDA(cudaMemGetInfo(free_bytes, total_bytes));
  return 0;
}

extern "C" int gb_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

// ------------------------------------------------------------------ object
// Cached pieces of add_scattered for one (destination, source, quadrature
// type): the domain of each destination node with respect to the source (a
// sequential solid-angle sum per node, fixed by the geometry) and, when they
// fit, the coefficients of the source's scattered potential at those nodes
// (k_cross_build), so that every later iteration is a product with the
// source's current boundary values.
struct CrossCache {
  unsigned long long src_uid;
  int type;
  int prec;  // field_prec of the source when built
  int n, C;
  int* did;
  int bad;  // first invalid domain id (+1000), 0 if all nodes are outside the source
  int df;   // coefficients in double-float (the source's fields are): applied on the FP32 pipes
  cplx *Gm, *Hm, *dGm, *dHm;
  double* Fp;
};

struct gb_obj {
  unsigned long long uid;
  std::vector<CrossCache> xc;
  GbMeshDev m;
  double lambda0;
  cudaStream_t st;
  double* kn_dev;
  // per-domain coefficient matrices
  cplx* G[GB_MAXDOM];
  cplx* H[GB_MAXDOM];
  cplx* dG[GB_MAXDOM];
  cplx* dH[GB_MAXDOM];
  double* dF[GB_MAXDOM];
  int* rowk[GB_MAXDOM];   // device: row index inside the domain block of A (-1: unused node)
  int nrows[GB_MAXDOM];
  size_t na;
  cplx* invA;             // na x na
  int have_invA;
  // mixed-precision form: complex FP32 LU factors of A; the FP64 residuals
  // are formed from G and H (A itself is never stored in FP64)
  cplxf* LU32;
  int64_t* ipiv32;
  int* perm32;
  int have_lu32;
  int ir_iters;
  double ir_relres;
  // the FP32 factors are of U^T A V (random butterflies, no interchanges)
  // when lu_rbt; lu_mode 1 forces tournament pivoting
  float* rbt;        // [4][na]: U's two levels, then V's
  int lu_rbt;
  int lu_mode;
  int lu_fallbacks;  // refactorisations with interchanges after a stalled refinement
  // block elimination (lu_mode 3) for an object with one interface: the
  // correction solve through node-sized FP32 inverses (gb_schur.cu)
  GbSchur* schur;
  int schur_ok;  // every element between domain 0 (outside) and 1 (inside)
  int lu_schur;  // the current factors are the block ones
  // plain FP64 form of such an object (lu_mode 3): complex FP64 block
  // factors; solves refine in FP64 with them (one correction reaches the
  // rounding level) -- the FP64 form of objects whose dense inverse does not fit
  GbSchur* schur64;
  int have_blk64;
  int refine_mode;  // 0: FP64 GMRES (default), 1: classical refinement (diagnostic)
  // right-hand side and solution of the last gb_solve_mEMP, kept between
  // calls: the next solve with the same factors starts from that solution
  // (the multiple-scattering iteration changes the right-hand side less and
  // less); invalidated by an assembly or a factorisation
  cplx *Bw, *Xw;
  int have_xw;
  // A Xw from the last solve's final FP64 residual (valid with have_xw):
  // the next warm-started solve's first residual needs no product
  cplx* Axw;
  int have_axw;
  // double-float copies of G, H for the GMRES iterations' products (chosen
  // form), rebuilt after an assembly or upload
  void* GHdf[GB_MAXDOM][2];
  int have_ghdf;
  // arithmetic of the regular pairs of the field kernels (potentials at
  // points, fields on the boundary, cross operators): 2 double-float after a
  // precision-2 assembly, else FP64
  int field_prec;
  cudaStream_t st_dom[GB_MAXDOM];  // per-domain streams (concurrent assembly and dE/dn solves)
  // boundary values per domain, [(Ne_d+1)][4][4] (U, dU) and [(Ne_d+1)][4][3] (E, dE, H, dH)
  cplx* bU[GB_MAXDOM];
  cplx* bdU[GB_MAXDOM];
  cplx* bE[GB_MAXDOM];
  cplx* bdE[GB_MAXDOM];
  cplx* bH[GB_MAXDOM];
  cplx* bdH[GB_MAXDOM];
  // incident potential per element [(Ne+1)][4][4]
  cplx *Ui, *dUi, *Ui0, *dUi0, *Uip;
  // exterior nodes (md == 0) as field points: position, unit normal, flat index e*4+j
  int next;
  double* ext_r;
  double* ext_v;
  int* ext_idx;
  std::vector<int> h_etype, h_sid;
  std::mutex bv_mu;  // first allocation of the boundary-value buffers
};

static int dalloc(void** p, size_t bytes) {
  GB_CUDA(cudaMalloc(p, bytes > 0 ? bytes : 16));
  return 0;
}
template <class T>
static int dup(T** dst, const T* src, size_t n) {
  if (dalloc((void**)dst, n * sizeof(T))) return -1;
  GB_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

extern "C" void gb_obj_destroy(gb_obj* o) {
  if (!o) return;
  for (auto& e : o->xc) {
    cudaFree(e.did); cudaFree(e.Gm); cudaFree(e.Hm); cudaFree(e.dGm); cudaFree(e.dHm); cudaFree(e.Fp);
  }
  cudaFree(o->m.cr); cudaFree(o->m.cw); cudaFree(o->m.ren); cudaFree(o->m.wen);
  cudaFree(o->m.etype); cudaFree(o->m.eni); cudaFree(o->m.md); cudaFree(o->m.sd); cudaFree(o->m.sid);
  cudaFree(o->kn_dev);
  for (int d = 0; d < GB_MAXDOM; d++) {
    cudaFree(o->G[d]); cudaFree(o->H[d]); cudaFree(o->dG[d]); cudaFree(o->dH[d]); cudaFree(o->dF[d]);
    cudaFree(o->rowk[d]);
  }
  cudaFree(o->invA);
  cudaFree(o->LU32); cudaFree(o->ipiv32); cudaFree(o->perm32); cudaFree(o->rbt);
  gbi_schur_destroy(o->schur);
  gbi_schur_destroy(o->schur64);
  cudaFree(o->Bw); cudaFree(o->Xw); cudaFree(o->Axw);
  for (int d = 0; d < GB_MAXDOM; d++) { cudaFree(o->GHdf[d][0]); cudaFree(o->GHdf[d][1]); }
  for (int d = 0; d < GB_MAXDOM; d++) {
    cudaFree(o->bU[d]); cudaFree(o->bdU[d]); cudaFree(o->bE[d]); cudaFree(o->bdE[d]); cudaFree(o->bH[d]); cudaFree(o->bdH[d]);
  }
  cudaFree(o->Ui); cudaFree(o->dUi); cudaFree(o->Ui0); cudaFree(o->dUi0); cudaFree(o->Uip);
  cudaFree(o->m.corner); cudaFree(o->ext_r); cudaFree(o->ext_v); cudaFree(o->ext_idx);
  for (int d = 0; d < GB_MAXDOM; d++)
    if (o->st_dom[d]) cudaStreamDestroy(o->st_dom[d]);
  if (o->st) cudaStreamDestroy(o->st);
  delete o;
}

extern "C" int gb_obj_create(const gb_mesh_desc* md, gb_obj** out) {
  *out = nullptr;
  if (md->MN + 1 > GB_MAXDOM) { gbi_set_error("gb_obj_create: %d media exceed the limit %d", md->MN, GB_MAXDOM - 1); return -1; }
  if (md->Ne <= 0) { gbi_set_error("gb_obj_create: no elements"); return -1; }
  if (ensure_tables()) return -1;
  gb_obj* o = new gb_obj();
  static std::atomic<unsigned long long> s_uid{1};
  o->uid = s_uid.fetch_add(1);
  memset(&o->m, 0, sizeof(o->m));
  for (int d = 0; d < GB_MAXDOM; d++) { o->G[d] = o->H[d] = o->dG[d] = o->dH[d] = nullptr; o->dF[d] = nullptr; o->rowk[d] = nullptr; }
  o->invA = nullptr;
  o->have_invA = 0;
  o->LU32 = nullptr; o->ipiv32 = nullptr; o->perm32 = nullptr; o->have_lu32 = 0; o->ir_iters = 0; o->ir_relres = 0.0;
  o->rbt = nullptr; o->lu_rbt = 0; o->lu_mode = 0; o->lu_fallbacks = 0; o->field_prec = 0;
  o->schur = nullptr; o->schur_ok = 0; o->lu_schur = 0;
  o->schur64 = nullptr; o->have_blk64 = 0; o->refine_mode = 0;
  o->Bw = o->Xw = nullptr; o->have_xw = 0;
  o->Axw = nullptr; o->have_axw = 0;
  for (int d = 0; d < GB_MAXDOM; d++) o->GHdf[d][0] = o->GHdf[d][1] = nullptr;
  o->have_ghdf = 0;
  o->lu_mode = 3;  // block elimination where the object allows it
  {  // GB_LU_MODE: the objects' initial gb_set_lu_pivoting mode (0..3)
    const char* e = getenv("GB_LU_MODE");
    if (e && e[0] >= '0' && e[0] <= '3' && e[1] == 0) o->lu_mode = e[0] - '0';
  }
  for (int d = 0; d < GB_MAXDOM; d++) o->st_dom[d] = nullptr;
  for (int d = 0; d < GB_MAXDOM; d++) o->bU[d] = o->bdU[d] = o->bE[d] = o->bdE[d] = o->bH[d] = o->bdH[d] = nullptr;
  o->Ui = o->dUi = o->Ui0 = o->dUi0 = o->Uip = nullptr;
  o->next = 0;
  o->ext_r = o->ext_v = nullptr;
  o->ext_idx = nullptr;
  o->kn_dev = nullptr;
  o->st = nullptr;
  GbMeshDev& m = o->m;
  m.Ne = md->Ne; m.NN = md->NN; m.MN = md->MN;
  size_t ne1 = (size_t)md->Ne + 1;
  m.ntri = m.nquad = 0;
  for (int e = 1; e <= md->Ne; e++) (md->etype[e] ? m.nquad : m.ntri)++;
  int tot = 0;
  for (int d = 0; d <= md->MN; d++) { m.sb_Ne[d] = md->sb_Ne[d]; m.sb_off[d] = tot; tot += md->sb_Ne[d] + 1; }
  m.sb_off[md->MN + 1] = tot;
  for (int d = 0; d <= md->MN; d++) { m.kn[2 * d] = md->kn[2 * d]; m.kn[2 * d + 1] = md->kn[2 * d + 1]; }
  o->lambda0 = md->lambda0;
  if (cudaStreamCreateWithFlags(&o->st, cudaStreamNonBlocking) != cudaSuccess) { gbi_set_error("stream"); gb_obj_destroy(o); return -1; }
  if (dup(&m.cr, md->cr, ne1 * 12) || dup(&m.cw, md->cw, ne1 * 9) || dup(&m.ren, md->ren, ne1 * 12) ||
      dup(&m.wen, md->wen, ne1 * 12) || dup(&m.etype, md->etype, ne1) || dup(&m.eni, md->eni, ne1 * 4) ||
      dup(&m.md, md->md, ne1) || dup(&m.sd, md->sd, ne1) || dup(&m.sid, md->sid, (size_t)tot) ||
      dup(&o->kn_dev, md->kn, (size_t)2 * (md->MN + 1)) || dup(&m.corner, md->corner, ne1 * 12)) {
    gb_obj_destroy(o);
    return -1;
  }
  o->h_etype.assign(md->etype, md->etype + ne1);
  o->h_sid.assign(md->sid, md->sid + tot);
  // rows of A: per domain, collocation nodes (t,tn) in order, skipping the
  // fourth node of triangles (reference solve_bieq2.c:228-239)
  size_t na = 0;
  for (int d = 0; d <= md->MN; d++) {
    int Ne = md->sb_Ne[d];
    std::vector<int> rk((size_t)Ne * 4, -1);
    int k = 0;
    for (int t = 1; t <= Ne; t++) {
      int td = abs(o->h_sid[m.sb_off[d] + t]);
      for (int tn = 0; tn < 4; tn++) {
        if (tn == 3 && o->h_etype[td] == 0) continue;
        rk[(size_t)(t - 1) * 4 + tn] = k++;
      }
    }
    o->nrows[d] = k;
    na += 4 * (size_t)k;
    if (dup(&o->rowk[d], rk.data(), rk.size())) { gb_obj_destroy(o); return -1; }
  }
  o->na = na;
  {  // exterior collocation points of the object (reference add_scattered_mEMP loop, mo_solve.c:306-346)
    std::vector<double> er, ev;
    std::vector<int> ei;
    for (int e = 1; e <= md->Ne; e++) {
      if (md->md[e] != 0) continue;
      for (int j = 0; j < 4; j++) {
        double w[3], a = 0.0;
        for (int d = 0; d < 3; d++) { er.push_back(md->ren[(size_t)e * 12 + j * 3 + d]); w[d] = md->wen[(size_t)e * 12 + j * 3 + d]; a += w[d] * w[d]; }
        a = sqrt(a);
        for (int d = 0; d < 3; d++) ev.push_back(a != 0.0 ? w[d] / a : w[d]);
        ei.push_back(e * 4 + j);
      }
    }
    o->next = (int)ei.size();
    if (dup(&o->ext_r, er.data(), er.size()) || dup(&o->ext_v, ev.data(), ev.size()) || dup(&o->ext_idx, ei.data(), ei.size())) {
      gb_obj_destroy(o);
      return -1;
    }
  }
  if (na != 8 * (size_t)md->NN) {
    gbi_set_error("gb_obj_create: inconsistent mesh (rows %zu != 8 NN = %zu)", na, 8 * (size_t)md->NN);
    gb_obj_destroy(o);
    return -1;
  }
  if (md->MN == 1 && md->sb_Ne[0] == md->Ne && md->sb_Ne[1] == md->Ne && o->nrows[0] == md->NN &&
      o->nrows[1] == md->NN) {
    o->schur_ok = 1;
    for (int e = 1; e <= md->Ne && o->schur_ok; e++)
      if (md->md[e] != 0 || md->sd[e] != 1) o->schur_ok = 0;
  }
  *out = o;
  return 0;
}

static int ensure_cmatrix(gb_obj* o, int did) {
  size_t N = (size_t)o->m.sb_Ne[did] * 4;
  if (!o->G[did]) {
    if (dalloc((void**)&o->G[did], N * N * sizeof(cplx)) || dalloc((void**)&o->H[did], N * N * sizeof(cplx)) ||
        dalloc((void**)&o->dG[did], 2 * N * N * sizeof(cplx)) || dalloc((void**)&o->dH[did], 2 * N * N * sizeof(cplx)) ||
        dalloc((void**)&o->dF[did], 3 * N * sizeof(double)))
      return -1;
  }
  return 0;
}

static int check_did(gb_obj* o, int did) {
  if (did < 0 || did > o->m.MN) { gbi_set_error("domain id %d out of range 0..%d", did, o->m.MN); return -1; }
  return 0;
}

extern "C" int gb_assemble(gb_obj* o, int did, int type) { return gb_assemble2(o, did, type, 0); }

// domain did into its (allocated) matrices on stream st, scratch
// stream-ordered; synchronises st
static int assemble_on(gb_obj* o, int did, int type, int precision, cudaStream_t st) {
  const size_t Ne = (size_t)o->m.sb_Ne[did];
  double* Fs = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&Fs, 3 * 4 * Ne * Ne * sizeof(double), st));
  const int rc = gbi_assemble_domain2(&o->m, did, type, precision, o->G[did], o->H[did], o->dG[did], o->dH[did],
                                      o->dF[did], Fs, st);
  cudaFreeAsync(Fs, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (rc) return -1;
  if (e != cudaSuccess) { gbi_set_error("gb_assemble: %s", cudaGetErrorString(e)); return -1; }
  return 0;
}

static int check_asm_args(int type, int precision) {
  if (type < 0 || type > 3) { gbi_set_error("gb_assemble: quadrature type %d not in 0..3", type); return -1; }
  if (precision < 0 || precision > 3) { gbi_set_error("gb_assemble: precision %d not in 0..3", precision); return -1; }
  return 0;
}

// Newly assembled matrices: every factor, warm start and scattering operator
// derived from the previous ones is dropped, so that a scene step after an
// assembly repeats all of the scene's work (the scattering operators this
// object holds are rebuilt by the next iteration that needs them)
static void assembled(gb_obj* o, int precision) {
  for (auto& e : o->xc) {
    cudaFree(e.did); cudaFree(e.Gm); cudaFree(e.Hm); cudaFree(e.dGm); cudaFree(e.dHm); cudaFree(e.Fp);
  }
  o->xc.clear();
  o->have_invA = 0;
  o->have_lu32 = 0;
  o->have_blk64 = 0;
  o->have_xw = 0;
  o->have_ghdf = 0;
  o->field_prec = precision >= 2 ? precision : 0;
}

extern "C" int gb_assemble2(gb_obj* o, int did, int type, int precision) {
  if (check_did(o, did) || check_asm_args(type, precision)) return -1;
  if (ensure_cmatrix(o, did)) return -1;
  if (assemble_on(o, did, type, precision, o->st)) return -1;
  assembled(o, precision);
  return 0;
}

extern "C" int gb_assemble_all(gb_obj* o, int type, int precision) {
  if (check_asm_args(type, precision)) return -1;
  for (int d = 0; d <= o->m.MN; d++)
    if (ensure_cmatrix(o, d)) return -1;
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  for (int d = 0; d <= o->m.MN; d++)
    if (!o->st_dom[d]) GB_CUDA(cudaStreamCreateWithFlags(&o->st_dom[d], cudaStreamNonBlocking));
  // o->st may hold earlier work on these matrices: the domain streams start after it
  GB_CUDA(cudaStreamSynchronize(o->st));
  std::vector<int> rcs((size_t)o->m.MN + 1, 0);
  std::vector<std::string> msg((size_t)o->m.MN + 1);
  std::vector<std::thread> th;
  for (int d = 0; d <= o->m.MN; d++) {
    if (o->m.sb_Ne[d] == 0) continue;
    auto job = [o, d, dev, type, precision, &rcs, &msg]() {
      if (cudaSetDevice(dev) != cudaSuccess) { rcs[d] = -1; msg[d] = "cudaSetDevice failed"; return; }
      rcs[d] = assemble_on(o, d, type, precision, o->st_dom[d]);
      if (rcs[d]) msg[d] = gb_last_error();
    };
    try {
      th.emplace_back(job);
    } catch (...) {
      job();  // no thread available: assemble this domain here
    }
  }
  for (auto& t : th) t.join();
  for (int d = 0; d <= o->m.MN; d++)
    if (rcs[d]) { gbi_set_error("%s", msg[d].c_str()); return -1; }
  assembled(o, precision);
  return 0;
}

extern "C" int gb_assemble_rows(gb_obj* o, int did, int row0, int nrow, int type, int precision, void* G, void* H,
                                void* dG, void* dH, double* dF) {
  if (check_did(o, did) || check_asm_args(type, precision)) return -1;
  if (!G || !H || !dG || !dH || !dF) { gbi_set_error("gb_assemble_rows: null output"); return -1; }
  const size_t Ne = (size_t)o->m.sb_Ne[did];
  if (nrow <= 0 || row0 < 0 || (size_t)row0 + (size_t)nrow > 4 * Ne) {
    gbi_set_error("gb_assemble_rows: rows %d..%d outside 0..%zu", row0, row0 + nrow - 1, 4 * Ne - 1);
    return -1;
  }
  if (ensure_tables()) return -1;
  double* Fs = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&Fs, 3 * (size_t)nrow * Ne * sizeof(double), o->st));
  const int rc = gbi_assemble_rows(&o->m, did, type, precision, row0, nrow, (cplx*)G, (cplx*)H, (cplx*)dG, (cplx*)dH,
                                   dF, Fs, o->st);
  cudaFreeAsync(Fs, o->st);
  return rc;
}

extern "C" int gb_assemble_objects(gb_obj** objs, int n, int type, int precision) {
  if (n <= 0) return 0;
  if (check_asm_args(type, precision)) return -1;
  std::vector<GbAsmItem> items;
  for (int i = 0; i < n; i++) {
    gb_obj* o = objs[i];
    for (int d = 0; d <= o->m.MN; d++) {
      if (ensure_cmatrix(o, d)) return -1;
      if (o->m.sb_Ne[d] == 0) continue;
      GbAsmItem it;
      it.m = &o->m; it.did = d; it.row0 = 0; it.nrow = 4 * o->m.sb_Ne[d];
      it.G = o->G[d]; it.H = o->H[d]; it.dG = o->dG[d]; it.dH = o->dH[d]; it.dF = o->dF[d];
      items.push_back(it);
    }
    GB_CUDA(cudaStreamSynchronize(o->st));  // earlier work on these matrices
  }
  if (gbi_assemble_list(items.data(), (int)items.size(), type, precision, objs[0]->st)) return -1;
  for (int i = 0; i < n; i++) assembled(objs[i], precision);
  return 0;
}

extern "C" int gb_cmatrix_download(gb_obj* o, int did, void* G, void* H, void* dG, void* dH, double* dF) {
  if (check_did(o, did)) return -1;
  if (!o->G[did]) { gbi_set_error("gb_cmatrix_download: domain %d not assembled", did); return -1; }
  size_t N = (size_t)o->m.sb_Ne[did] * 4;
  if (G) GB_CUDA(cudaMemcpy(G, o->G[did], N * N * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (H) GB_CUDA(cudaMemcpy(H, o->H[did], N * N * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (dG) GB_CUDA(cudaMemcpy(dG, o->dG[did], 2 * N * N * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (dH) GB_CUDA(cudaMemcpy(dH, o->dH[did], 2 * N * N * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (dF) GB_CUDA(cudaMemcpy(dF, o->dF[did], 3 * N * sizeof(double), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gb_cmatrix_rows(gb_obj* o, int did, int nrows, const int* rows, void* G, void* H, void* dG, void* dH,
                               double* dF) {
  if (check_did(o, did)) return -1;
  if (!o->G[did]) { gbi_set_error("gb_cmatrix_rows: domain %d not assembled", did); return -1; }
  const size_t N = (size_t)o->m.sb_Ne[did] * 4;
  for (int i = 0; i < nrows; i++)
    if (rows[i] < 0 || (size_t)rows[i] >= N) { gbi_set_error("gb_cmatrix_rows: row %d out of range", rows[i]); return -1; }
  for (int i = 0; i < nrows; i++) {
    const size_t r = (size_t)rows[i];
    cplx* g = (cplx*)G;
    cplx* h = (cplx*)H;
    cplx* dg = (cplx*)dG;
    cplx* dh = (cplx*)dH;
    if (G) GB_CUDA(cudaMemcpy(g + i * N, o->G[did] + r * N, N * sizeof(cplx), cudaMemcpyDeviceToHost));
    if (H) GB_CUDA(cudaMemcpy(h + i * N, o->H[did] + r * N, N * sizeof(cplx), cudaMemcpyDeviceToHost));
    if (dG) GB_CUDA(cudaMemcpy(dg + 2 * i * N, o->dG[did] + 2 * r * N, 2 * N * sizeof(cplx), cudaMemcpyDeviceToHost));
    if (dH) GB_CUDA(cudaMemcpy(dh + 2 * i * N, o->dH[did] + 2 * r * N, 2 * N * sizeof(cplx), cudaMemcpyDeviceToHost));
    if (dF) GB_CUDA(cudaMemcpy(dF + 3 * i, o->dF[did] + 3 * r, 3 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return 0;
}

extern "C" int gb_cmatrix_upload(gb_obj* o, int did, const void* G, const void* H, const void* dG, const void* dH,
                                 const double* dF) {
  if (check_did(o, did)) return -1;
  if (ensure_cmatrix(o, did)) return -1;
  size_t N = (size_t)o->m.sb_Ne[did] * 4;
  if (G) GB_CUDA(cudaMemcpy(o->G[did], G, N * N * sizeof(cplx), cudaMemcpyHostToDevice));
  if (H) GB_CUDA(cudaMemcpy(o->H[did], H, N * N * sizeof(cplx), cudaMemcpyHostToDevice));
  if (dG) GB_CUDA(cudaMemcpy(o->dG[did], dG, 2 * N * N * sizeof(cplx), cudaMemcpyHostToDevice));
  if (dH) GB_CUDA(cudaMemcpy(o->dH[did], dH, 2 * N * N * sizeof(cplx), cudaMemcpyHostToDevice));
  if (dF) GB_CUDA(cudaMemcpy(o->dF[did], dF, 3 * N * sizeof(double), cudaMemcpyHostToDevice));
  o->have_invA = 0;
  o->have_xw = 0;
  o->have_ghdf = 0;
  return 0;
}

static int build_A(gb_obj* o, cplx* A) {
  size_t na = o->na;
  GB_CUDA(cudaMemsetAsync(A, 0, na * na * sizeof(cplx), o->st));
  size_t base = 0;
  for (int d = 0; d <= o->m.MN; d++) {
    if (!o->G[d]) { gbi_set_error("coupled matrix: domain %d has no coefficient matrices", d); return -1; }
    if (gbi_build_A_domain(o->G[d], o->H[d], o->m.sid + o->m.sb_off[d], o->rowk[d], &o->m, o->kn_dev, d, o->nrows[d],
                           base, na, A, o->st))
      return -1;
    base += 4 * (size_t)o->nrows[d];
  }
  return 0;
}

extern "C" int gb_A_download(gb_obj* o, void* Ah) {
  size_t na = o->na;
  cplx* A = nullptr;
  if (dalloc((void**)&A, na * na * sizeof(cplx))) return -1;
  int rc = build_A(o, A);
  if (!rc) {
    if (cudaMemcpyAsync(Ah, A, na * na * sizeof(cplx), cudaMemcpyDeviceToHost, o->st) != cudaSuccess ||
        cudaStreamSynchronize(o->st) != cudaSuccess) {
      gbi_set_error("gb_A_download: copy failed");
      rc = -1;
    }
  }
  cudaFree(A);
  return rc;
}

extern "C" int gb_invA_compute(gb_obj* o) {
  size_t na = o->na;
  cplx* A = nullptr;
  int64_t* ipiv = nullptr;
  int* info = nullptr;
  if (!o->invA && dalloc((void**)&o->invA, na * na * sizeof(cplx))) return -1;
  if (dalloc((void**)&A, na * na * sizeof(cplx)) || dalloc((void**)&ipiv, na * sizeof(int64_t)) ||
      dalloc((void**)&info, sizeof(int))) {
    cudaFree(A); cudaFree(ipiv);
    return -1;
  }
  int rc = build_A(o, A);
  if (!rc) rc = gbi_zgetrf(A, na, (int)na, ipiv, info, o->st);
  int hinfo = 0;
  if (!rc) {
    if (cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, o->st) != cudaSuccess ||
        cudaStreamSynchronize(o->st) != cudaSuccess) {
      gbi_set_error("gb_invA_compute: LU failed: %s", cudaGetErrorString(cudaGetLastError()));
      rc = -1;
    } else if (hinfo != 0) {
      gbi_set_error("gb_invA_compute: matrix is singular (zgetrf info=%d)", hinfo);
      rc = -1;
    }
  }
  if (!rc) rc = gbi_zinverse(A, na, (int)na, ipiv, o->invA, na, o->st);
  if (!rc && cudaStreamSynchronize(o->st) != cudaSuccess) {
    gbi_set_error("gb_invA_compute: inverse failed: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  cudaFree(A); cudaFree(ipiv); cudaFree(info);
  if (!rc) { o->have_invA = 1; o->have_lu32 = 0; o->have_blk64 = 0; }
  return rc;
}

extern "C" int gb_invA_download(gb_obj* o, void* invA) {
  if (!o->have_invA) { gbi_set_error("gb_invA_download: no inverse"); return -1; }
  GB_CUDA(cudaMemcpy(invA, o->invA, o->na * o->na * sizeof(cplx), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gb_invA_upload(gb_obj* o, const void* invA) {
  if (!o->invA && dalloc((void**)&o->invA, o->na * o->na * sizeof(cplx))) return -1;
  GB_CUDA(cudaMemcpy(o->invA, invA, o->na * o->na * sizeof(cplx), cudaMemcpyHostToDevice));
  o->have_invA = 1;
  o->have_lu32 = 0;
  o->have_blk64 = 0;
  return 0;
}

extern "C" int gb_solve_AB(gb_obj* o, const void* b, void* x) {
  if (!o->have_invA) { gbi_set_error("gb_solve_AB: no inverse"); return -1; }
  size_t na = o->na;
  cplx *db = nullptr, *dx = nullptr;
  if (dalloc((void**)&db, na * sizeof(cplx)) || dalloc((void**)&dx, na * sizeof(cplx))) { cudaFree(db); return -1; }
  int rc = 0;
  if (cudaMemcpyAsync(db, b, na * sizeof(cplx), cudaMemcpyHostToDevice, o->st) != cudaSuccess) rc = -1;
  if (!rc) rc = gbi_zgemv(o->invA, na, (int)na, (int)na, db, dx, o->st);
  if (!rc && (cudaMemcpyAsync(x, dx, na * sizeof(cplx), cudaMemcpyDeviceToHost, o->st) != cudaSuccess ||
              cudaStreamSynchronize(o->st) != cudaSuccess)) {
    gbi_set_error("gb_solve_AB failed");
    rc = -1;
  }
  cudaFree(db); cudaFree(dx);
  return rc;
}

extern "C" int gb_zgesv(int n, int nrhs, void* Ah, void* Bh) {
  if (n <= 0 || nrhs <= 0) { gbi_set_error("gb_zgesv: bad size n=%d nrhs=%d", n, nrhs); return -1; }
  cplx *A = nullptr, *B = nullptr;
  int64_t* ipiv = nullptr;
  int* info = nullptr;
  cudaStream_t st;
  GB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int rc = 0;
  if (dalloc((void**)&A, (size_t)n * n * sizeof(cplx)) || dalloc((void**)&B, (size_t)n * nrhs * sizeof(cplx)) ||
      dalloc((void**)&ipiv, (size_t)n * sizeof(int64_t)) || dalloc((void**)&info, sizeof(int)))
    rc = -1;
  if (!rc && (cudaMemcpyAsync(A, Ah, (size_t)n * n * sizeof(cplx), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemcpyAsync(B, Bh, (size_t)n * nrhs * sizeof(cplx), cudaMemcpyHostToDevice, st) != cudaSuccess)) {
    gbi_set_error("gb_zgesv: upload failed");
    rc = -1;
  }
  if (!rc) rc = gbi_zgetrf(A, n, n, ipiv, info, st);
  int hinfo = 0;
  if (!rc && (cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("gb_zgesv: LU failed");
    rc = -1;
  }
  if (!rc && hinfo) { gbi_set_error("gb_zgesv: singular matrix (info=%d)", hinfo); rc = -1; }
  if (!rc) rc = gbi_zgetrs(A, n, n, ipiv, B, nrhs, nrhs, st);
  if (!rc && (cudaMemcpyAsync(Bh, B, (size_t)n * nrhs * sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("gb_zgesv: solve failed");
    rc = -1;
  }
  cudaFree(A); cudaFree(B); cudaFree(ipiv); cudaFree(info);
  cudaStreamDestroy(st);
  return rc;
}

// ------------------------------------------------------------------ boundary values
static int ensure_bv_locked(gb_obj* o);
// allocates the boundary-value buffers on first use; safe against concurrent
// first calls from several host threads
static int ensure_bv(gb_obj* o) {
  std::lock_guard<std::mutex> lk(o->bv_mu);
  return ensure_bv_locked(o);
}
static int ensure_bv_locked(gb_obj* o) {
  for (int d = 0; d <= o->m.MN; d++) {
    if (o->bU[d]) continue;
    size_t n1 = (size_t)o->m.sb_Ne[d] + 1;
    if (dalloc((void**)&o->bU[d], n1 * 16 * sizeof(cplx)) || dalloc((void**)&o->bdU[d], n1 * 16 * sizeof(cplx)) ||
        dalloc((void**)&o->bE[d], n1 * 12 * sizeof(cplx)) || dalloc((void**)&o->bdE[d], n1 * 12 * sizeof(cplx)) ||
        dalloc((void**)&o->bH[d], n1 * 12 * sizeof(cplx)) || dalloc((void**)&o->bdH[d], n1 * 12 * sizeof(cplx)))
      return -1;
    GB_CUDA(cudaMemset(o->bU[d], 0, n1 * 16 * sizeof(cplx)));
    GB_CUDA(cudaMemset(o->bdU[d], 0, n1 * 16 * sizeof(cplx)));
    GB_CUDA(cudaMemset(o->bE[d], 0, n1 * 12 * sizeof(cplx)));
    GB_CUDA(cudaMemset(o->bdE[d], 0, n1 * 12 * sizeof(cplx)));
    GB_CUDA(cudaMemset(o->bH[d], 0, n1 * 12 * sizeof(cplx)));
    GB_CUDA(cudaMemset(o->bdH[d], 0, n1 * 12 * sizeof(cplx)));
  }
  if (!o->Ui) {
    size_t n = ((size_t)o->m.Ne + 1) * 16 * sizeof(cplx);
    if (dalloc((void**)&o->Ui, n) || dalloc((void**)&o->dUi, n) || dalloc((void**)&o->Ui0, n) ||
        dalloc((void**)&o->dUi0, n) || dalloc((void**)&o->Uip, n))
      return -1;
    GB_CUDA(cudaMemset(o->Ui, 0, n)); GB_CUDA(cudaMemset(o->dUi, 0, n)); GB_CUDA(cudaMemset(o->Ui0, 0, n));
    GB_CUDA(cudaMemset(o->dUi0, 0, n)); GB_CUDA(cudaMemset(o->Uip, 0, n));
  }
  return 0;
}

extern "C" int gb_bv_upload(gb_obj* o, int did, const void* U, const void* dU, const void* E, const void* dE,
                            const void* H, const void* dH) {
  if (check_did(o, did) || ensure_bv(o)) return -1;
  size_t n1 = (size_t)o->m.sb_Ne[did] + 1;
  if (U) GB_CUDA(cudaMemcpy(o->bU[did], U, n1 * 16 * sizeof(cplx), cudaMemcpyHostToDevice));
  if (dU) GB_CUDA(cudaMemcpy(o->bdU[did], dU, n1 * 16 * sizeof(cplx), cudaMemcpyHostToDevice));
  if (E) GB_CUDA(cudaMemcpy(o->bE[did], E, n1 * 12 * sizeof(cplx), cudaMemcpyHostToDevice));
  if (dE) GB_CUDA(cudaMemcpy(o->bdE[did], dE, n1 * 12 * sizeof(cplx), cudaMemcpyHostToDevice));
  if (H) GB_CUDA(cudaMemcpy(o->bH[did], H, n1 * 12 * sizeof(cplx), cudaMemcpyHostToDevice));
  if (dH) GB_CUDA(cudaMemcpy(o->bdH[did], dH, n1 * 12 * sizeof(cplx), cudaMemcpyHostToDevice));
  return 0;
}

extern "C" int gb_bv_download(gb_obj* o, int did, void* U, void* dU, void* E, void* dE, void* H, void* dH) {
  if (check_did(o, did) || ensure_bv(o)) return -1;
  size_t n1 = (size_t)o->m.sb_Ne[did] + 1;
  if (U) GB_CUDA(cudaMemcpy(U, o->bU[did], n1 * 16 * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (dU) GB_CUDA(cudaMemcpy(dU, o->bdU[did], n1 * 16 * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (E) GB_CUDA(cudaMemcpy(E, o->bE[did], n1 * 12 * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (dE) GB_CUDA(cudaMemcpy(dE, o->bdE[did], n1 * 12 * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (H) GB_CUDA(cudaMemcpy(H, o->bH[did], n1 * 12 * sizeof(cplx), cudaMemcpyDeviceToHost));
  if (dH) GB_CUDA(cudaMemcpy(dH, o->bdH[did], n1 * 12 * sizeof(cplx), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gb_incident_upload(gb_obj* o, const void* Ui0, const void* dUi0) {
  if (ensure_bv(o)) return -1;
  size_t n = ((size_t)o->m.Ne + 1) * 16 * sizeof(cplx);
  GB_CUDA(cudaMemcpy(o->Ui0, Ui0, n, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(o->dUi0, dUi0, n, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(o->Ui, o->Ui0, n, cudaMemcpyDeviceToDevice));
  GB_CUDA(cudaMemcpy(o->Uip, o->Ui0, n, cudaMemcpyDeviceToDevice));
  GB_CUDA(cudaMemcpy(o->dUi, o->dUi0, n, cudaMemcpyDeviceToDevice));
  return 0;
}

extern "C" int gb_incident_download(gb_obj* o, void* Ui, void* dUi, void* Uip) {
  if (ensure_bv(o)) return -1;
  size_t n = ((size_t)o->m.Ne + 1) * 16 * sizeof(cplx);
  if (Ui) GB_CUDA(cudaMemcpy(Ui, o->Ui, n, cudaMemcpyDeviceToHost));
  if (dUi) GB_CUDA(cudaMemcpy(dUi, o->dUi, n, cudaMemcpyDeviceToHost));
  if (Uip) GB_CUDA(cudaMemcpy(Uip, o->Uip, n, cudaMemcpyDeviceToHost));
  return 0;
}

static int sync_obj(gb_obj* o, const char* what) {
  cudaError_t e = cudaStreamSynchronize(o->st);
  if (e != cudaSuccess) { gbi_set_error("%s: %s", what, cudaGetErrorString(e)); return -1; }
  return 0;
}

static int ir_solve(gb_obj* o, const cplx* B, cplx* X, bool warm);
static int ensure_ghdf(gb_obj* o);

extern "C" int gb_solve_mEMP(gb_obj* o) {
  if (!o->have_invA && !o->have_lu32 && !o->have_blk64) {
    gbi_set_error("gb_solve_mEMP: A is neither inverted nor factorised");
    return -1;
  }
  if (ensure_bv(o)) return -1;
  size_t na = o->na;
  if (!o->Bw && (dalloc((void**)&o->Bw, na * sizeof(cplx)) || dalloc((void**)&o->Xw, na * sizeof(cplx)))) {
    cudaFree(o->Bw);
    o->Bw = nullptr;
    return -1;
  }
  cplx *B = o->Bw, *X = o->Xw;
  int rc = 0;
  size_t base = 0;
  // lower-precision factors (the chosen form): B's products in double-float
  bool df = false;
  if (!o->have_invA && !o->have_blk64) {
    const int e = ensure_ghdf(o);
    if (e < 0) return -1;
    df = e == 0;
  }
  for (int d = 0; d <= o->m.MN && !rc; d++) {
    if (!o->G[d]) { gbi_set_error("gb_solve_mEMP: domain %d has no coefficient matrices", d); rc = -1; break; }
    rc = gbi_build_B(o->G[d], o->H[d], df ? o->GHdf[d][0] : nullptr, df ? o->GHdf[d][1] : nullptr,
                     o->m.sid + o->m.sb_off[d], o->rowk[d], &o->m, o->kn_dev, o->Ui, o->dUi, d, o->nrows[d], base, B,
                     o->st);
    base += 4 * (size_t)o->nrows[d];
  }
  const bool warm = o->have_xw != 0;
  o->have_xw = 0;
  if (!o->have_invA && !o->Axw && dalloc((void**)&o->Axw, na * sizeof(cplx))) return -1;
  if (!rc) rc = o->have_invA ? gbi_zgemv(o->invA, na, (int)na, (int)na, B, X, o->st) : ir_solve(o, B, X, warm);
  for (int d = 0; d <= o->m.MN && !rc; d++) rc = gbi_store_bv(X, &o->m, o->kn_dev, o->Ui, o->dUi, d, o->bU[d], o->bdU[d], o->st);
  if (!rc) rc = sync_obj(o, "gb_solve_mEMP");
  if (!rc) o->have_xw = 1;
  return rc;
}


extern "C" int gb_reset_incident(gb_obj* o) {
  if (ensure_bv(o)) return -1;
  size_t n = ((size_t)o->m.Ne + 1) * 16 * sizeof(cplx);
  GB_CUDA(cudaMemcpyAsync(o->Uip, o->Ui, n, cudaMemcpyDeviceToDevice, o->st));
  GB_CUDA(cudaMemcpyAsync(o->Ui, o->Ui0, n, cudaMemcpyDeviceToDevice, o->st));
  GB_CUDA(cudaMemcpyAsync(o->dUi, o->dUi0, n, cudaMemcpyDeviceToDevice, o->st));
  return sync_obj(o, "gb_reset_incident");
}

static FieldObj field_view(gb_obj* o) {
  FieldObj f;
  memset(&f, 0, sizeof(f));
  f.cr = o->m.cr; f.cw = o->m.cw; f.corner = o->m.corner; f.etype = o->m.etype; f.sd = o->m.sd; f.sid = o->m.sid;
  for (int d = 0; d <= o->m.MN; d++) {
    f.sb_Ne[d] = o->m.sb_Ne[d];
    f.sb_off[d] = o->m.sb_off[d];
    f.kn[2 * d] = o->m.kn[2 * d];
    f.kn[2 * d + 1] = o->m.kn[2 * d + 1];
    f.U[d] = o->bU[d]; f.dU[d] = o->bdU[d]; f.E[d] = o->bE[d]; f.dE[d] = o->bdE[d]; f.H[d] = o->bH[d]; f.dH[d] = o->bdH[d];
  }
  f.sb_off[o->m.MN + 1] = o->m.sb_off[o->m.MN + 1];
  f.MN = o->m.MN;
  f.lambda0 = o->lambda0;
  f.prec = o->field_prec;
  f.ntri = o->m.ntri;
  f.nquad = o->m.nquad;
  return f;
}

// cross operators are kept while they need at most this share of the free device memory
#define GB_CROSS_MEM_SHARE 0.25

static CrossCache* cross_entry(gb_obj* dst, gb_obj* src, int type) {
  for (auto& e : dst->xc)
    if (e.src_uid == src->uid && e.type == type && e.prec == src->field_prec) return &e;
  CrossCache e;
  memset(&e, 0, sizeof(e));
  e.src_uid = src->uid;
  e.type = type;
  e.prec = src->field_prec;
  e.n = dst->next;
  e.C = 4 * src->m.sb_Ne[0];
  e.df = (src->field_prec >= 2 && type == 2) ? 1 : 0;
  if (dalloc((void**)&e.did, (size_t)e.n * sizeof(int))) return nullptr;
  FieldObj f = field_view(src);
  int* bad = nullptr;
  if (dalloc((void**)&bad, sizeof(int))) { cudaFree(e.did); return nullptr; }
  int rc = 0;
  if (cudaMemsetAsync(bad, 0, sizeof(int), dst->st) != cudaSuccess) rc = -1;
  if (!rc) rc = gbi_domain_id(&f, e.n, dst->ext_r, e.did, dst->st);
  // the validity of every node is fixed by the geometry: checked once, here
  std::vector<int> hd((size_t)e.n);
  if (!rc && (cudaMemcpyAsync(hd.data(), e.did, (size_t)e.n * sizeof(int), cudaMemcpyDeviceToHost, dst->st) != cudaSuccess ||
              cudaStreamSynchronize(dst->st) != cudaSuccess))
    rc = -1;
  cudaFree(bad);
  if (rc) { cudaFree(e.did); if (!gb_last_error()[0]) gbi_set_error("add_scattered: domain id failed"); return nullptr; }
  for (int i = 0; i < e.n && !e.bad; i++)
    if (hd[i] != 0) e.bad = 1000 + hd[i];
  size_t bytes = (size_t)e.n * e.C * 4 * sizeof(cplx);
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  if (!e.bad && e.n > 0 && e.C > 0 && bytes <= (size_t)(GB_CROSS_MEM_SHARE * (double)fr)) {
    size_t nc = (size_t)e.n * e.C;
    if (cudaMalloc((void**)&e.Gm, nc * sizeof(cplx)) == cudaSuccess &&
        cudaMalloc((void**)&e.Hm, nc * sizeof(cplx)) == cudaSuccess &&
        cudaMalloc((void**)&e.dGm, nc * sizeof(cplx)) == cudaSuccess &&
        cudaMalloc((void**)&e.dHm, nc * sizeof(cplx)) == cudaSuccess &&
        cudaMalloc((void**)&e.Fp, (size_t)e.n * 2 * sizeof(double)) == cudaSuccess &&
        gbi_cross_build(&f, type, e.n, dst->ext_r, dst->ext_v, e.C, e.Gm, e.Hm, e.dGm, e.dHm, e.Fp, e.df, dst->st) == 0 &&
        cudaStreamSynchronize(dst->st) == cudaSuccess) {
      // kept
    } else {
      cudaGetLastError();  // an allocation failure is not an error here: the direct path serves
      cudaFree(e.Gm); cudaFree(e.Hm); cudaFree(e.dGm); cudaFree(e.dHm); cudaFree(e.Fp);
      e.Gm = e.Hm = e.dGm = e.dHm = nullptr;
      e.Fp = nullptr;
    }
  }
  dst->xc.push_back(e);
  return &dst->xc.back();
}

extern "C" int gb_add_scattered(gb_obj* dst, gb_obj* src, int type) {
  if (ensure_bv(dst) || ensure_bv(src)) return -1;
  int n = dst->next;
  if (n == 0) return 0;
  CrossCache* e = cross_entry(dst, src, type);
  if (!e) return -1;
  if (e->bad) {
    gbi_set_error("scattered field domain id error!(overlapped). domain id=%d", e->bad - 1000);
    return -1;
  }
  // stream-ordered scratch: no device-wide synchronisation (objects of a
  // multiple-scattering sweep run concurrently)
  cplx* out = nullptr;
  int* bad = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&out, (size_t)n * 8 * sizeof(cplx), dst->st));
  GB_CUDA(cudaMallocAsync((void**)&bad, sizeof(int), dst->st));
  int rc = 0;
  if (e->Gm) {
    rc = gbi_cross_apply(n, e->C, e->Gm, e->Hm, e->dGm, e->dHm, e->Fp, src->bU[0], src->bdU[0], out, e->df, dst->st);
  } else {
    FieldObj f = field_view(src);
    rc = gbi_field(&f, 3, type, n, dst->ext_r, dst->ext_v, e->did, out, nullptr, dst->st);
  }
  if (!rc && cudaMemsetAsync(bad, 0, sizeof(int), dst->st) != cudaSuccess) rc = -1;
  if (!rc) rc = gbi_add_incident(n, dst->ext_idx, out, dst->Ui, dst->dUi, e->did, bad, dst->st);
  cudaFreeAsync(out, dst->st);
  cudaFreeAsync(bad, dst->st);
  if (!rc && cudaStreamSynchronize(dst->st) != cudaSuccess) {
    gbi_set_error("gb_add_scattered: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  return rc;
}

extern "C" int gb_ccd_sums(gb_obj* o, double* hout) {
  if (ensure_bv(o)) return -1;
  double* out = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&out, 3 * sizeof(double), o->st));
  int rc = gbi_ccd(o->m.Ne, o->m.md, o->Ui, o->Uip, out, o->st);
  if (!rc && cudaMemcpyAsync(hout, out, 3 * sizeof(double), cudaMemcpyDeviceToHost, o->st) != cudaSuccess) rc = -1;
  cudaFreeAsync(out, o->st);
  if (!rc && cudaStreamSynchronize(o->st) != cudaSuccess) rc = -1;
  if (rc) gbi_set_error("gb_ccd_sums failed");
  return rc;
}

// dE/dn, dH/dn of domain d in the chosen form on stream st: the system of
// solve_deh_bv built from G, H, E, H, solved by FP32 factors + FP64
// refinement, scattered back; synchronises st
static int deh_mixed(gb_obj* o, int d, cudaStream_t st) {
  const int Ne = o->m.sb_Ne[d], nn = o->nrows[d];
  cplx *Ac = nullptr, *Bc = nullptr, *Yc = nullptr;
  GB_CUDA(cudaMallocAsync((void**)&Ac, (size_t)nn * nn * sizeof(cplx), st));
  GB_CUDA(cudaMallocAsync((void**)&Bc, (size_t)nn * 6 * sizeof(cplx), st));
  GB_CUDA(cudaMallocAsync((void**)&Yc, (size_t)nn * 6 * sizeof(cplx), st));
  int rc = gbi_deh_build(o->G[d], o->H[d], o->rowk[d], Ne, nn, o->bE[d], o->bH[d], Ac, Bc, st);
  if (!rc) rc = gbi_zgesv_mixed(Ac, nn, Bc, 6, Yc, nullptr, nullptr, st);
  if (!rc) rc = gbi_deh_scatter(Yc, o->rowk[d], Ne, o->bdE[d], o->bdH[d], st);
  cudaFreeAsync(Ac, st);
  cudaFreeAsync(Bc, st);
  cudaFreeAsync(Yc, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (!rc && e != cudaSuccess) { gbi_set_error("gb_solve_EH: %s", cudaGetErrorString(e)); rc = -1; }
  return rc;
}

extern "C" int gb_solve_EH(gb_obj* o) {
  if (ensure_bv(o)) return -1;
  int rc = 0;
  if (o->have_lu32) {
    // chosen form: E, H of every domain, then the domains' dE/dn systems at
    // once, one host thread and stream each (each solve is a chain of small
    // dependent launches that leaves most SMs idle)
    for (int d = 0; d <= o->m.MN; d++) {
      if (o->m.sb_Ne[d] == 0) continue;
      if (!o->G[d]) { gbi_set_error("gb_solve_EH: domain %d has no coefficient matrices", d); return -1; }
      if (gbi_eh_bv(o->dG[d], o->dH[d], o->dF[d], &o->m, d, o->lambda0, o->bU[d], o->bdU[d], o->bE[d], o->bH[d], o->st))
        return -1;
    }
    if (sync_obj(o, "gb_solve_EH")) return -1;
    int dev = 0;
    GB_CUDA(cudaGetDevice(&dev));
    for (int d = 0; d <= o->m.MN; d++)
      if (!o->st_dom[d]) GB_CUDA(cudaStreamCreateWithFlags(&o->st_dom[d], cudaStreamNonBlocking));
    std::vector<int> rcs((size_t)o->m.MN + 1, 0);
    std::vector<std::string> msg((size_t)o->m.MN + 1);
    std::vector<std::thread> th;
    for (int d = 0; d <= o->m.MN; d++) {
      if (o->m.sb_Ne[d] == 0) continue;
      auto job = [o, d, dev, &rcs, &msg]() {
        if (cudaSetDevice(dev) != cudaSuccess) { rcs[d] = -1; msg[d] = "cudaSetDevice failed"; return; }
        rcs[d] = deh_mixed(o, d, o->st_dom[d]);
        if (rcs[d]) msg[d] = gb_last_error();
      };
      try {
        th.emplace_back(job);
      } catch (...) {
        job();  // no thread available: solve this domain here
      }
    }
    for (auto& t : th) t.join();
    for (int d = 0; d <= o->m.MN; d++)
      if (rcs[d]) { gbi_set_error("%s", msg[d].c_str()); return -1; }
    return 0;
  }
  for (int d = 0; d <= o->m.MN && !rc; d++) {
    int Ne = o->m.sb_Ne[d];
    if (Ne == 0) continue;
    if (!o->G[d]) { gbi_set_error("gb_solve_EH: domain %d has no coefficient matrices", d); return -1; }
    rc = gbi_eh_bv(o->dG[d], o->dH[d], o->dF[d], &o->m, d, o->lambda0, o->bU[d], o->bdU[d], o->bE[d], o->bH[d], o->st);
    if (rc) break;
    int nn = o->nrows[d];
    cplx *Ac = nullptr, *Bc = nullptr, *Yc = nullptr;
    int64_t* ipiv = nullptr;
    int *info = nullptr, *perm = nullptr;
    if (dalloc((void**)&Ac, (size_t)nn * nn * sizeof(cplx)) || dalloc((void**)&Bc, (size_t)nn * 6 * sizeof(cplx)) ||
        dalloc((void**)&Yc, (size_t)nn * 6 * sizeof(cplx)) || dalloc((void**)&perm, (size_t)nn * sizeof(int)) ||
        dalloc((void**)&ipiv, (size_t)nn * sizeof(int64_t)) || dalloc((void**)&info, sizeof(int))) {
      cudaFree(Ac); cudaFree(Bc); cudaFree(Yc); cudaFree(perm); cudaFree(ipiv);
      return -1;
    }
    rc = gbi_deh_build(o->G[d], o->H[d], o->rowk[d], Ne, nn, o->bE[d], o->bH[d], Ac, Bc, o->st);
    if (!rc) rc = gbi_zgetrf(Ac, nn, nn, ipiv, info, o->st);
    int hinfo = 0;
    if (!rc && (cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, o->st) != cudaSuccess ||
                cudaStreamSynchronize(o->st) != cudaSuccess)) {
      gbi_set_error("gb_solve_EH: LU failed");
      rc = -1;
    }
    if (!rc && hinfo) { gbi_set_error("mo_solve.c, solve_deh_bv(), zgesv info=%d error", hinfo); rc = -1; }
    if (!rc) rc = gbi_make_perm(ipiv, nn, perm, o->st);
    if (!rc) rc = gbi_zsolve_multi(Ac, nn, nn, perm, Bc, 6, 6, Yc, o->st);
    if (!rc) rc = gbi_deh_scatter(Yc, o->rowk[d], Ne, o->bdE[d], o->bdH[d], o->st);
    if (!rc) rc = sync_obj(o, "gb_solve_EH");
    cudaFree(Ac); cudaFree(Bc); cudaFree(Yc); cudaFree(perm); cudaFree(ipiv); cudaFree(info);
  }
  return rc;
}

// ------------------------------------------------------------------ points
// The point entry points are synchronous and may be called from several host
// threads at once (the reference's examples call the per-point field functions
// from OpenMP loops): each calling thread runs them on its own stream, with
// stream-ordered temporaries (no cudaFree and its device-wide synchronisation),
// after the object's own stream has drained.
// the calling thread's stream per device for point evaluations, destroyed
// when the thread ends (worker threads come and go)
struct ThreadStreams {
  cudaStream_t s[64] = {};
  ~ThreadStreams() {
    for (int d = 0; d < 64; d++)
      if (s[d] && cudaSetDevice(d) == cudaSuccess) cudaStreamDestroy(s[d]);
  }
};
static thread_local ThreadStreams t_point_stream;
static int point_stream(gb_obj* o, cudaStream_t* st) {
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { gbi_set_error("device ordinal %d not supported", dev); return -1; }
  if (!t_point_stream.s[dev]) GB_CUDA(cudaStreamCreateWithFlags(&t_point_stream.s[dev], cudaStreamNonBlocking));
  GB_CUDA(cudaStreamSynchronize(o->st));
  *st = t_point_stream.s[dev];
  return 0;
}

extern "C" int gb_domain_id(gb_obj* o, int n, const double* rt, int* did) {
  if (n <= 0) return 0;
  cudaStream_t st;
  if (point_stream(o, &st)) return -1;
  double* drt = nullptr;
  int* dd = nullptr;
  if (cudaMallocAsync((void**)&drt, (size_t)n * 3 * sizeof(double), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dd, (size_t)n * sizeof(int), st) != cudaSuccess) {
    gbi_set_error("gb_domain_id: out of device memory");
    if (drt) cudaFreeAsync(drt, st);
    return -1;
  }
  FieldObj f = field_view(o);
  int rc = 0;
  if (cudaMemcpyAsync(drt, rt, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess) rc = -1;
  if (!rc) rc = gbi_domain_id(&f, n, drt, dd, st);
  if (!rc && cudaMemcpyAsync(did, dd, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = -1;
  cudaFreeAsync(drt, st);
  cudaFreeAsync(dd, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
  if (rc) gbi_set_error("gb_domain_id failed");
  return rc;
}

extern "C" int gb_field_points(gb_obj* o, int mode, int type, int n, const double* rt, const double* v, const int* did,
                               void* out, int* flag) {
  if (n <= 0) return 0;
  if (mode < 0 || mode > 3 || type < 0 || type > 3) { gbi_set_error("gb_field_points: mode %d type %d", mode, type); return -1; }
  if (ensure_bv(o)) return -1;
  cudaStream_t st;
  if (point_stream(o, &st)) return -1;
  int nout = (mode == 0) ? 4 : (mode == 3 ? 8 : 6);
  double *drt = nullptr, *dv = nullptr;
  int *dd = nullptr, *df = nullptr;
  cplx* dout = nullptr;
  int rc = 0;
  if (cudaMallocAsync((void**)&drt, (size_t)n * 3 * sizeof(double), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dv, (size_t)n * 3 * sizeof(double), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dd, (size_t)n * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync((void**)&df, (size_t)n * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dout, (size_t)n * nout * sizeof(cplx), st) != cudaSuccess) {
    gbi_set_error("gb_field_points: out of device memory");
    rc = -1;
  }
  FieldObj f = field_view(o);
  if (!rc && (cudaMemcpyAsync(drt, rt, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              (v && cudaMemcpyAsync(dv, v, (size_t)n * 3 * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess) ||
              cudaMemcpyAsync(dd, did, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemsetAsync(dout, 0, (size_t)n * nout * sizeof(cplx), st) != cudaSuccess)) {
    gbi_set_error("gb_field_points: upload failed");
    rc = -1;
  }
  if (!rc) rc = gbi_field(&f, mode, type, n, drt, dv, dd, dout, df, st);
  if (!rc && cudaMemcpyAsync(out, dout, (size_t)n * nout * sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = -1;
  if (!rc && flag && mode == 2 && cudaMemcpyAsync(flag, df, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = -1;
  void* tmp[5] = {drt, dv, dd, df, dout};
  for (void* t : tmp)
    if (t) cudaFreeAsync(t, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
  if (rc && !gb_last_error()[0]) gbi_set_error("gb_field_points failed");
  return rc;
}

extern "C" int gb_field_bd(gb_obj* o, int type, int n, const int* did, const int* t, const double* zt, void* out) {
  if (n <= 0) return 0;
  if (ensure_bv(o)) return -1;
  for (int i = 0; i < n; i++) {
    if (did[i] < 0 || did[i] > o->m.MN || t[i] < 1 || t[i] > o->m.sb_Ne[did[i]]) {
      gbi_set_error("gb_field_bd: point %d: domain %d element %d out of range", i, did[i], t[i]);
      return -1;
    }
  }
  cudaStream_t st;
  if (point_stream(o, &st)) return -1;
  int *dd = nullptr, *dt = nullptr;
  double* dz = nullptr;
  cplx* dout = nullptr;
  int rc = 0;
  if (cudaMallocAsync((void**)&dd, (size_t)n * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dt, (size_t)n * sizeof(int), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dz, (size_t)n * 2 * sizeof(double), st) != cudaSuccess ||
      cudaMallocAsync((void**)&dout, (size_t)n * 6 * sizeof(cplx), st) != cudaSuccess) {
    gbi_set_error("gb_field_bd: out of device memory");
    rc = -1;
  }
  FieldObj f = field_view(o);
  if (!rc && (cudaMemcpyAsync(dd, did, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemcpyAsync(dt, t, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st) != cudaSuccess ||
              cudaMemcpyAsync(dz, zt, (size_t)n * 2 * sizeof(double), cudaMemcpyHostToDevice, st) != cudaSuccess))
    rc = -1;
  if (!rc) rc = gbi_field_bd(&f, type, n, dd, dt, dz, dout, st);
  if (!rc && cudaMemcpyAsync(out, dout, (size_t)n * 6 * sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess) rc = -1;
  void* tmp[4] = {dd, dt, dz, dout};
  for (void* p : tmp)
    if (p) cudaFreeAsync(p, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) rc = -1;
  if (rc && !gb_last_error()[0]) gbi_set_error("gb_field_bd failed");
  return rc;
}

// ------------------------------------------------------------------ mixed precision
// Complex FP32 LU of A (tournament pivoting, tensor-core trailing updates);
// A is built directly in FP32 into the factor's buffer.
// butterfly parameters of the object's order (gbi_rbt_params)
static int ensure_rbt(gb_obj* o) {
  if (o->rbt) return 0;
  const size_t n4 = 4 * o->na;
  std::vector<float> h(n4);
  gbi_rbt_params((int)o->na, h.data());
  if (dalloc((void**)&o->rbt, n4 * sizeof(float))) return -1;
  GB_CUDA(cudaMemcpy(o->rbt, h.data(), n4 * sizeof(float), cudaMemcpyHostToDevice));
  return 0;
}

// A (complex FP32) from the resident G, H into LU32 and its factors:
// randomised (U^T A V) without interchanges when rbt, else tournament
// pivoting; *hinfo: the first zero pivot (0: none)
static int factor32(gb_obj* o, bool rbt, int* hinfo) {
  size_t na = o->na;
  int* info = nullptr;
  if (dalloc((void**)&info, sizeof(int))) return -1;
  int rc = 0;
  if (cudaMemsetAsync(o->LU32, 0, na * na * sizeof(cplxf), o->st) != cudaSuccess) { gbi_set_error("memset"); rc = -1; }
  size_t base = 0;
  for (int d = 0; d <= o->m.MN && !rc; d++) {
    if (!o->G[d]) { gbi_set_error("coupled matrix: domain %d has no coefficient matrices", d); rc = -1; break; }
    rc = gbi_build_A32_domain(o->G[d], o->H[d], o->m.sid + o->m.sb_off[d], o->rowk[d], &o->m, o->kn_dev, d,
                              o->nrows[d], base, na, o->LU32, o->st);
    base += 4 * (size_t)o->nrows[d];
  }
  if (rbt) {
    if (!rc) rc = gbi_rbt_matrix(o->LU32, na, (int)na, o->rbt, o->rbt + 2 * na, o->st);
    if (!rc) rc = gbi_cgetrf_nopiv(o->LU32, na, (int)na, o->ipiv32, info, o->st);
  } else if (!rc) {
    rc = gbi_cgetrf(o->LU32, na, (int)na, o->ipiv32, info, o->st);
  }
  if (!rc) rc = rbt ? gbi_perm_identity((int)na, o->perm32, o->st) : gbi_make_perm(o->ipiv32, (int)na, o->perm32, o->st);
  *hinfo = 0;
  if (!rc && (cudaMemcpyAsync(hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, o->st) != cudaSuccess ||
              cudaStreamSynchronize(o->st) != cudaSuccess)) {
    gbi_set_error("gb_factor_mixed: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  cudaFree(info);
  if (!rc) o->lu_rbt = rbt ? 1 : 0;
  return rc;
}

static int alloc_lu32(gb_obj* o) {
  size_t na = o->na;
  if (!o->LU32 && dalloc((void**)&o->LU32, na * na * sizeof(cplxf))) return -1;
  if (!o->ipiv32 && dalloc((void**)&o->ipiv32, na * sizeof(int64_t))) return -1;
  if (!o->perm32 && dalloc((void**)&o->perm32, na * sizeof(int))) return -1;
  return 0;
}

// block factors (gb_schur.cu): 0, 1 after a zero pivot, -1 on error
static int factor_schur(gb_obj* o) {
  if (!o->G[0] || !o->G[1]) { gbi_set_error("coupled matrix: a domain has no coefficient matrices"); return -1; }
  if (!o->schur && gbi_schur_create(o->m.NN, 0, &o->schur)) return -1;
  return gbi_schur_factor(o->schur, &o->m, o->G[0], o->H[0], o->G[1], o->H[1], o->m.sid + o->m.sb_off[0],
                          o->m.sid + o->m.sb_off[1], o->rowk[0], o->rowk[1], o->st);
}

extern "C" int gb_factor_mixed(gb_obj* o) {
  size_t na = o->na;
  o->have_lu32 = 0;
  o->have_xw = 0;
  o->have_blk64 = 0;
  if (o->lu_mode == 3 && o->schur_ok) {
    const int r = factor_schur(o);
    if (r < 0) return -1;
    if (r == 0) {
      o->lu_schur = 1;
      o->have_lu32 = 1;
      o->have_invA = 0;
      return 0;
    }
    o->lu_fallbacks++;  // a zero pivot in the block factors: the dense factors instead
  }
  o->lu_schur = 0;
  if (alloc_lu32(o)) return -1;
  const bool rbt = (o->lu_mode == 0 || o->lu_mode == 2 || o->lu_mode == 3) && na % 4 == 0;
  if (rbt && ensure_rbt(o)) return -1;
  int hinfo = 0;
  int rc = factor32(o, rbt, &hinfo);
  if (!rc && rbt && hinfo) {  // a zero pivot without interchanges: factorise with them
    o->lu_fallbacks++;
    rc = factor32(o, false, &hinfo);
  }
  if (!rc && hinfo) { gbi_set_error("gb_factor_mixed: FP32 factor singular (info=%d)", hinfo); rc = -1; }
  if (!rc) { o->have_lu32 = 1; o->have_invA = 0; }
  return rc;
}

extern "C" int gb_set_lu_pivoting(gb_obj* o, int mode) {
  if (mode < 0 || mode > 3) { gbi_set_error("gb_set_lu_pivoting: mode %d not in 0..3", mode); return -1; }
  o->lu_mode = mode;
  return 0;
}

extern "C" int gb_lu_info(gb_obj* o, int* rbt, int* fallbacks) {
  *rbt = o->have_blk64 ? 3 : (o->lu_schur ? 2 : o->lu_rbt);
  *fallbacks = o->lu_fallbacks;
  return 0;
}

// double-float copies of G and H (for the GMRES products); 0 when present
static int ensure_ghdf(gb_obj* o) {
  if (o->have_ghdf) return 0;
  for (int d = 0; d <= o->m.MN; d++) {
    const size_t N = 4 * (size_t)o->m.sb_Ne[d];
    if (N == 0) continue;
    for (int i = 0; i < 2; i++) {
      if (!o->GHdf[d][i] && cudaMalloc(&o->GHdf[d][i], N * N * 16) != cudaSuccess) {
        cudaGetLastError();
        o->GHdf[d][i] = nullptr;
        return 1;  // no room: the products stay in FP64
      }
      if (gbi_to_df(N * N, i ? o->H[d] : o->G[d], o->GHdf[d][i], o->st)) return -1;
    }
  }
  o->have_ghdf = 1;
  return 0;
}

// y = A x with G and H in double-float (PQ, PQd: scratch of 8 N_max entries)
static int apply_A_df(gb_obj* o, const cplx* x, cplx* PQ, void* PQd, cplx* y) {
  size_t base = 0;
  for (int d = 0; d <= o->m.MN; d++) {
    if (gbi_apply_A_domain_df(o->GHdf[d][0], o->GHdf[d][1], o->m.sid + o->m.sb_off[d], o->rowk[d], &o->m, o->kn_dev,
                              d, o->nrows[d], base, x, PQ, PQd, y, o->st))
      return -1;
    base += 4 * (size_t)o->nrows[d];
  }
  return 0;
}

// y = A x in FP64 from G and H (PQ: scratch of 8 N_max complex)
static int apply_A(gb_obj* o, const cplx* x, cplx* PQ, cplx* y) {
  size_t base = 0;
  for (int d = 0; d <= o->m.MN; d++) {
    if (gbi_apply_A_domain(o->G[d], o->H[d], o->m.sid + o->m.sb_off[d], o->rowk[d], &o->m, o->kn_dev, d, o->nrows[d],
                           base, x, PQ, y, o->st))
      return -1;
    base += 4 * (size_t)o->nrows[d];
  }
  return 0;
}

// Classical FP64 iterative refinement with the FP32 factors (refinement mode
// 1, a diagnostic): x <- x + LU32^-1 (b - A x) until ||b - A x|| <= 1e-13 ||b||
// (at most 30 corrections); b - A x is formed in FP64 from G and H
static int ir_classical(gb_obj* o, const cplx* B, cplx* X) {
  size_t na = o->na;
  size_t nmax = 0;
  for (int d = 0; d <= o->m.MN; d++) nmax = std::max(nmax, 4 * (size_t)o->m.sb_Ne[d]);
  cplx *r = nullptr, *y = nullptr, *PQ = nullptr;
  cplxf *d = nullptr, *d2 = nullptr;
  double* nrm = nullptr;
  if (dalloc((void**)&r, na * sizeof(cplx)) || dalloc((void**)&y, na * sizeof(cplx)) ||
      dalloc((void**)&PQ, 8 * nmax * sizeof(cplx)) || dalloc((void**)&d, na * sizeof(cplxf)) ||
      dalloc((void**)&d2, na * sizeof(cplxf)) || dalloc((void**)&nrm, 2 * sizeof(double))) {
    cudaFree(r); cudaFree(y); cudaFree(PQ); cudaFree(d); cudaFree(d2);
    return -1;
  }
  int rc = 0;
  if (cudaMemsetAsync(X, 0, na * sizeof(cplx), o->st) != cudaSuccess ||
      cudaMemcpyAsync(r, B, na * sizeof(cplx), cudaMemcpyDeviceToDevice, o->st) != cudaSuccess)
    rc = -1;
  double h[2] = {0.0, 1.0}, rel = 1.0, prev = 1.0;
  int it = 0, since = 0;  // corrections, corrections with the current factors
  for (; !rc && it < 31; it++, since++) {
    if (it > 0) {
      rc = apply_A(o, X, PQ, y);
      if (!rc) rc = gbi_resid_finish(B, y, r, na, nrm, o->st);
      if (rc) break;
      if (cudaMemcpyAsync(h, nrm, 2 * sizeof(double), cudaMemcpyDeviceToHost, o->st) != cudaSuccess ||
          cudaStreamSynchronize(o->st) != cudaSuccess) { rc = -1; break; }
      prev = rel;
      rel = (h[1] > 0.0) ? sqrt(h[0] / h[1]) : 0.0;
      if (rel <= 1e-13) break;
      // factors without interchanges that do not contract the residual by
      // 10x per correction (far from the rounding floor), or not within 12
      // corrections: factorise again with tournament pivoting and go on
      // from the current x (from x = 0 if it diverged)
      const bool forced = o->lu_mode == 2 && o->lu_rbt;  // diagnostic mode: take the fallback at the first check
      if (!o->have_blk64 && (o->lu_rbt || o->lu_schur) &&
          (forced || (since >= 2 && rel > 0.1 * prev && rel > 1e-11) || since >= 12 || !(rel < 1e3))) {
        int hinfo = 0;
        o->lu_fallbacks++;
        o->lu_schur = 0;
        rc = alloc_lu32(o);
        if (!rc) rc = factor32(o, false, &hinfo);
        if (!rc && hinfo) { gbi_set_error("ir_solve: FP32 factor singular (info=%d)", hinfo); rc = -1; }
        if (rc) break;
        if (!(rel < 1.0) &&
            (cudaMemsetAsync(X, 0, na * sizeof(cplx), o->st) != cudaSuccess ||
             cudaMemcpyAsync(r, B, na * sizeof(cplx), cudaMemcpyDeviceToDevice, o->st) != cudaSuccess)) { rc = -1; break; }
        since = 0;
      }
    }
    if (o->have_blk64)
      rc = gbi_schur_apply(o->schur64, r, X, o->st);
    else if (o->lu_schur)
      rc = gbi_schur_apply(o->schur, r, X, o->st);
    else
      rc = o->lu_rbt ? gbi_ir_step_rbt(X, r, d, d2, o->LU32, na, (int)na, o->perm32, o->rbt, o->rbt + 2 * na, o->st)
                     : gbi_ir_step(X, r, d, d2, o->LU32, na, (int)na, o->perm32, o->st);
  }
  o->ir_iters = it;
  o->ir_relres = rel;
  if (!rc && rel > 1e-10) { gbi_set_error("iterative refinement stalled at relative residual %g", rel); rc = -1; }
  cudaFree(r); cudaFree(y); cudaFree(PQ); cudaFree(d); cudaFree(d2); cudaFree(nrm);
  return rc;
}

// refactorisation with tournament pivoting after the butterfly or block
// factors failed to refine
static int refactor_pivoted(gb_obj* o) {
  int hinfo = 0;
  o->lu_fallbacks++;
  o->lu_schur = 0;
  if (alloc_lu32(o)) return -1;
  if (factor32(o, false, &hinfo)) return -1;
  if (hinfo) { gbi_set_error("ir_solve: FP32 factor singular (info=%d)", hinfo); return -1; }
  return 0;
}

// z = M^-1 v with the object's current factors (FP32 dense butterfly or
// tournament LU, FP32 or FP64 block elimination); d, d2: FP32 work vectors
static int precond(gb_obj* o, const cplx* v, cplx* z, cplxf* d, cplxf* d2, cudaStream_t st) {
  const size_t na = o->na;
  GB_CUDA(cudaMemsetAsync(z, 0, na * sizeof(cplx), st));
  if (o->have_blk64) return gbi_schur_apply(o->schur64, v, z, st);
  if (o->lu_schur) return gbi_schur_apply(o->schur, v, z, st);
  if (o->lu_rbt)
    return gbi_ir_step_rbt(z, v, d, d2, o->LU32, na, (int)na, o->perm32, o->rbt, o->rbt + 2 * na, st);
  return gbi_ir_step(z, v, d, d2, o->LU32, na, (int)na, o->perm32, st);
}

// FP64 flexible GMRES(20) refinement, right-preconditioned by the current factors, to
// ||b - A x|| <= 1e-13 ||b||; A applied in FP64 from G and H.  A run that
// does not converge with butterfly or block factors (or, in the diagnostic
// LU mode 2, after its first iteration) refactorises with tournament
// pivoting and continues from the current x.
static int ir_solve(gb_obj* o, const cplx* B, cplx* X, bool warm) {
  if (o->refine_mode == 1) {
    o->have_axw = 0;
    return ir_classical(o, B, X);
  }
  const size_t na = o->na;
  size_t nmax = 0;
  for (int d = 0; d <= o->m.MN; d++) nmax = std::max(nmax, 4 * (size_t)o->m.sb_Ne[d]);
  cplx* PQ = nullptr;
  void* PQd = nullptr;
  cplxf *d = nullptr, *d2 = nullptr;
  // stream-ordered scratch (no device-wide synchronisation)
  GB_CUDA(cudaMallocAsync((void**)&PQ, 8 * nmax * sizeof(cplx), o->st));
  GB_CUDA(cudaMallocAsync(&PQd, 8 * nmax * 16, o->st));
  GB_CUDA(cudaMallocAsync((void**)&d, na * sizeof(cplxf), o->st));
  GB_CUDA(cudaMallocAsync((void**)&d2, na * sizeof(cplxf), o->st));
  GbOp A = [o, PQ](const cplx* x, cplx* y, cudaStream_t) { return apply_A(o, x, PQ, y); };
  GbOp Adf = [o, PQ, PQd](const cplx* x, cplx* y, cudaStream_t) { return apply_A_df(o, x, PQ, PQd, y); };
  GbOp M = [o, d, d2](const cplx* v, cplx* z, cudaStream_t st) { return precond(o, v, z, d, d2, st); };
  int rc = 0;
  // lower-precision factors: the iterations' products in double-float
  // (every true residual, the convergence test, stays FP64); the FP64 block
  // factors of the plain FP64 form keep FP64 products
  const GbOp* Af = nullptr;
  if (!o->have_blk64) {
    const int e = ensure_ghdf(o);
    if (e < 0) rc = -1;
    else if (e == 0) Af = &Adf;
  }
  // from the previous solution with the same factors (warm), else from zero;
  // warm, the previous solve's last FP64 product A x gives the first residual
  if (!warm && cudaMemsetAsync(X, 0, na * sizeof(cplx), o->st) != cudaSuccess) { gbi_set_error("ir_solve: memset"); rc = -1; }
  const cplx* ax0 = (warm && o->have_axw) ? o->Axw : nullptr;
  o->have_axw = 0;
  int it = 0, tot = 0, axok = 0;
  double rel = 1.0;
  const bool forced = o->lu_mode == 2 && o->lu_rbt;  // diagnostic: the fallback after one iteration
  int r = rc ? -1
             : gbi_gmres(na, B, X, !warm, A, Af, M, 20, 1e-13, forced ? 1 : 60, o->st, ax0, o->Axw, &axok, &it, &rel);
  tot += it;
  if (r == 1 && !o->have_blk64 && (o->lu_rbt || o->lu_schur)) {
    if (!(rel < 1.0) && cudaMemsetAsync(X, 0, na * sizeof(cplx), o->st) != cudaSuccess) r = -1;
    if (r == 1 && refactor_pivoted(o)) r = -1;
    if (r == 1) {
      r = gbi_gmres(na, B, X, !(rel < 1.0), A, Af, M, 20, 1e-13, 60, o->st, nullptr, o->Axw, &axok, &it, &rel);
      tot += it;
    }
  }
  o->have_axw = (r == 0 && axok) ? 1 : 0;
  o->ir_iters = tot;
  o->ir_relres = rel;
  if (r < 0) rc = -1;
  else if (r == 1 || rel > 1e-10) { gbi_set_error("iterative refinement stalled at relative residual %g", rel); rc = -1; }
  cudaFreeAsync(PQ, o->st); cudaFreeAsync(PQd, o->st); cudaFreeAsync(d, o->st); cudaFreeAsync(d2, o->st);
  return rc;
}

extern "C" int gb_set_refinement(gb_obj* o, int mode) {
  if (mode < 0 || mode > 1) { gbi_set_error("gb_set_refinement: mode %d not in 0..1", mode); return -1; }
  o->refine_mode = mode;
  return 0;
}

extern "C" int gb_ir_info(gb_obj* o, int* iters, double* relres) {
  *iters = o->ir_iters;
  *relres = o->ir_relres;
  return 0;
}

// Assembly precision of each scene form: form 1 (the chosen form) integrates
// the regular pairs in double-float with the distance-adaptive order
// (precision 3), form 2 the far pairs in FP32, forms 0 and 3 everything in
// FP64.
extern "C" int gb_form_precision(int form) { return form == 1 ? 3 : (form == 2 ? 1 : 0); }

// One scene step on the device for a single object: assembly of every
// domain (quadrature type, precision gb_form_precision(form)), factorisation
// of A (form 0: FP64 LU and explicit inverse; forms 1-3: complex FP32 LU +
// FP64 refinement), boundary values U,dU, then E, H and their normal
// derivatives.
// Plain FP64 factorisation: the FP64 block factors for an object with one
// interface in LU mode 3 (the default), else the dense LU and explicit
// inverse of A as the reference (gb_invA_compute).
extern "C" int gb_factor_fp64(gb_obj* o) {
  o->have_lu32 = 0;
  o->have_xw = 0;
  o->have_blk64 = 0;
  if (o->lu_mode == 3 && o->schur_ok) {
    if (!o->G[0] || !o->G[1]) { gbi_set_error("coupled matrix: a domain has no coefficient matrices"); return -1; }
    if (!o->schur64 && gbi_schur_create(o->m.NN, 1, &o->schur64)) return -1;
    const int r = gbi_schur_factor(o->schur64, &o->m, o->G[0], o->H[0], o->G[1], o->H[1], o->m.sid + o->m.sb_off[0],
                                   o->m.sid + o->m.sb_off[1], o->rowk[0], o->rowk[1], o->st);
    if (r < 0) return -1;
    if (r > 0) { gbi_set_error("gb_factor_fp64: a node matrix is singular"); return -1; }
    o->have_blk64 = 1;
    o->have_invA = 0;
    return 0;
  }
  return gb_invA_compute(o);
}

extern "C" int gb_obj_one_interface(gb_obj* o) { return o->schur_ok; }

extern "C" int gb_block_factors_download(gb_obj* o, void* G0i, void* G1i, void* nX0, void* Minv, void* Si) {
  if (!o->have_blk64) { gbi_set_error("gb_block_factors_download: no FP64 block factors"); return -1; }
  void* d[5];
  gbi_schur_mats(o->schur64, d);
  void* h[5] = {G0i, G1i, nX0, Minv, Si};
  const size_t bytes = (size_t)o->m.NN * o->m.NN * sizeof(cplx);
  for (int i = 0; i < 5; i++)
    if (h[i]) GB_CUDA(cudaMemcpy(h[i], d[i], bytes, cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int gb_block_factors_upload(gb_obj* o, const void* G0i, const void* G1i, const void* nX0, const void* Minv,
                                       const void* Si) {
  if (!o->schur_ok) { gbi_set_error("gb_block_factors_upload: the object does not have one interface"); return -1; }
  if (!o->schur64 && gbi_schur_create(o->m.NN, 1, &o->schur64)) return -1;
  void* d[5];
  gbi_schur_mats(o->schur64, d);
  const void* h[5] = {G0i, G1i, nX0, Minv, Si};
  const size_t bytes = (size_t)o->m.NN * o->m.NN * sizeof(cplx);
  for (int i = 0; i < 5; i++) GB_CUDA(cudaMemcpy(d[i], h[i], bytes, cudaMemcpyHostToDevice));
  if (gbi_schur_prepare(o->schur64, &o->m, o->st)) return -1;
  o->have_xw = 0;
  o->have_blk64 = 1;
  o->have_invA = 0;
  o->have_lu32 = 0;
  return 0;
}

extern "C" int gb_scene_step(gb_obj* o, int form, int type) {
  if (form < 0 || form > 3) { gbi_set_error("gb_scene_step: form %d not in 0..3", form); return -1; }
  if (gb_assemble_objects(&o, 1, type, gb_form_precision(form))) return -1;
  if (form == 0) { if (gb_factor_fp64(o)) return -1; }
  else if (gb_factor_mixed(o)) return -1;
  if (gb_solve_mEMP(o)) return -1;
  return gb_solve_EH(o);
}

extern "C" void* gb_obj_stream(gb_obj* o) { return (void*)o->st; }

extern "C" int gb_current_device(void) {
  int d = 0;
  return cudaGetDevice(&d) == cudaSuccess ? d : -1;
}
extern "C" int gb_use_device(int dev) {
  if (cudaSetDevice(dev) != cudaSuccess) { gbi_set_error("cudaSetDevice(%d) failed", dev); return -1; }
  return 0;
}
