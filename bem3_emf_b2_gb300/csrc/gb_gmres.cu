// gb_gmres.cu -- restarted GMRES in FP64, right-preconditioned by the
// lower-precision factors: the refinement of the chosen form's solves
// (A x = b with A applied in FP64 from the coefficient matrices, the
// preconditioner a solve with the complex-FP32 factors -- dense butterfly LU,
// tournament LU or the block elimination's node inverses -- or with the FP64
// block factors).
//
// Flexible GMRES(m) (Saad 1993) on A M^-1 u = b: per iteration one
// preconditioner solve z_j = M^-1 v_j, kept, and one FP64 product w = A z_j,
// classical Gram-Schmidt against v_0..v_j done twice (Giraud, Langou and
// Rozloznik 2005: "twice is enough"), complex Givens rotations on the host
// for the (m+1) x m Hessenberg least-squares problem; the update is
// x += Z y with the stored z_j (the lower-precision solve is not exactly
// linear, so x = M^-1 (V y) would reintroduce its rounding: a second cycle
// per solve).  The recurrence's residual estimate ends a cycle; the true
// residual b - A x is formed in FP64 at the start of every cycle and decides
// convergence.  Against classical
// refinement (x += M^-1 (b - A x)) it costs the same per step but converges
// whenever the preconditioned operator's spectrum stays away from zero,
// which tolerates much less accurate factors (Carson and Higham 2017).
//
// Dot products are reduced deterministically: fixed chunks per block, block
// partials summed in order by one thread per vector.
#include "gb_common.cuh"
#include "gb_internal.h"

#include <complex>
#include <functional>
#include <vector>

typedef std::function<int(const cplx* x, cplx* y, cudaStream_t st)> GbOp;

#define GS_THREADS 256
#define GS_CHUNK 8192

// partial[i * nchunk + c] = sum over chunk c of conj(V_i[k]) w[k]
__global__ void __launch_bounds__(GS_THREADS) k_gs_dot(const cplx* __restrict__ V, size_t ldv, size_t n,
                                                       const cplx* __restrict__ w, cplx* partial, int nchunk) {
  const int c = blockIdx.x, i = blockIdx.y;
  const cplx* v = V + (size_t)i * ldv;
  const size_t k0 = (size_t)c * GS_CHUNK;
  const size_t k1 = (k0 + GS_CHUNK < n) ? k0 + GS_CHUNK : n;
  double sr = 0.0, si = 0.0;
  for (size_t k = k0 + threadIdx.x; k < k1; k += GS_THREADS) {
    const cplx a = v[k], b = w[k];
    sr = fma(a.x, b.x, fma(a.y, b.y, sr));
    si = fma(a.x, b.y, fma(-a.y, b.x, si));
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  __shared__ double s[2][GS_THREADS / 32];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { s[0][wid] = sr; s[1][wid] = si; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int q = 0; q < GS_THREADS / 32; q++) { a += s[0][q]; b += s[1][q]; }
    partial[(size_t)i * nchunk + c] = cmk(a, b);
  }
}

// h[i] = sum_c partial[i][c] (in chunk order)
__global__ void k_gs_sum(const cplx* partial, int nvec, int nchunk, cplx* h) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nvec) return;
  double a = 0.0, b = 0.0;
  for (int c = 0; c < nchunk; c++) {
    const cplx p = partial[(size_t)i * nchunk + c];
    a += p.x;
    b += p.y;
  }
  h[i] = cmk(a, b);
}

// w -= sum_i h_i V_i
__global__ void k_gs_update(const cplx* __restrict__ V, size_t ldv, int nvec, size_t n, const cplx* __restrict__ h,
                            cplx* w) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  cplx acc = w[k];
  for (int i = 0; i < nvec; i++) acc -= h[i] * V[(size_t)i * ldv + k];
  w[k] = acc;
}

// u = sum_i y_i V_i
__global__ void k_gs_combine(const cplx* __restrict__ V, size_t ldv, int nvec, size_t n, const cplx* __restrict__ y,
                             cplx* u) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  cplx acc = cmk(0.0, 0.0);
  for (int i = 0; i < nvec; i++) acc += y[i] * V[(size_t)i * ldv + k];
  u[k] = acc;
}

__global__ void k_gs_scale(const cplx* x, size_t n, double s, cplx* y) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) y[k] = x[k] * s;
}
__global__ void k_gs_sub(const cplx* b, const cplx* y, size_t n, cplx* r) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) r[k] = b[k] - y[k];
}
__global__ void k_gs_add(cplx* x, const cplx* z, size_t n) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) x[k] += z[k];
}

namespace {
struct Work {
  size_t n;
  int nchunk;
  cplx *partial, *h;
  cudaStream_t st;
  unsigned grid() const { return (unsigned)((n + 255) / 256); }
  // h[0..nvec) = V^H w (device)
  int dots(const cplx* V, size_t ldv, int nvec, const cplx* w, cplx* out) {
    dim3 g((unsigned)nchunk, (unsigned)nvec);
    k_gs_dot<<<g, GS_THREADS, 0, st>>>(V, ldv, n, w, partial, nchunk);
    k_gs_sum<<<(nvec + 63) / 64, 64, 0, st>>>(partial, nvec, nchunk, out);
    gbi_count_launch();
    gbi_count_launch();
    GB_CUDA(cudaGetLastError());
    return 0;
  }
};
}  // namespace

// Solves A x = b to ||b - A x|| <= tol ||b|| by flexible GMRES(m) right-preconditioned
// by M (z = M^-1 v), from the initial guess in x (x_zero: x is zero, so the
// first residual is b without a product).  At most maxit iterations.
// Returns 0 when converged, 1 when not (maxit reached, or a cycle that did not
// reduce the true residual 10x while far from the target), -1 on error.
// *iters: iterations (preconditioner solves) done, *relres: the last true
// relative residual.  Synchronises st.
// Af (may be null): the operator of the Arnoldi products (a lower-precision
// application of A); every true residual still uses A.  Ax0 (may be null,
// only with !x_zero): A x for the initial x, so the first residual takes no
// product.  Ax_out (may be null): on convergence, A x of the returned x;
// *ax_ok (with Ax_out) 1 when it was written.
extern "C" int gbi_gmres(size_t n, const cplx* b, cplx* x, bool x_zero, const GbOp& A, const GbOp* Af, const GbOp& M,
                         int m, double tol, int maxit, cudaStream_t st, const cplx* Ax0, cplx* Ax_out, int* ax_ok,
                         int* iters, double* relres) {
  *iters = 0;
  *relres = 1.0;
  if (ax_ok) *ax_ok = 0;
  if (n == 0) return 0;
  if (m < 1) m = 1;
  Work W;
  W.n = n;
  W.nchunk = (int)((n + GS_CHUNK - 1) / GS_CHUNK);
  W.st = st;
  cplx *V = nullptr, *Z = nullptr, *w = nullptr, *z = nullptr, *r = nullptr, *yd = nullptr, *h2 = nullptr;
  W.partial = nullptr;
  W.h = nullptr;
  int rc = 0;
  if (cudaMallocAsync((void**)&V, (size_t)(m + 1) * n * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&Z, (size_t)m * n * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&w, n * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&z, n * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&r, n * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&yd, (size_t)(m + 2) * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&h2, (size_t)2 * (m + 2) * sizeof(cplx), st) != cudaSuccess ||
      cudaMallocAsync((void**)&W.partial, (size_t)(m + 2) * W.nchunk * sizeof(cplx), st) != cudaSuccess) {
    gbi_set_error("gmres: out of device memory: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  typedef std::complex<double> C;
  double bnorm = 0.0;
  if (!rc) rc = W.dots(b, n, 1, b, yd);
  cplx hb = cmk(0.0, 0.0);
  if (!rc && (cudaMemcpyAsync(&hb, yd, sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
              cudaStreamSynchronize(st) != cudaSuccess)) {
    gbi_set_error("gmres: %s", cudaGetErrorString(cudaGetLastError()));
    rc = -1;
  }
  bnorm = sqrt(hb.x);
  std::vector<C> H((size_t)(m + 1) * m), g((size_t)m + 1), cs((size_t)m), sn((size_t)m), y((size_t)m);
  std::vector<cplx> hh((size_t)2 * (m + 2));
  int it = 0, status = 1;
  double prev_cycle = -1.0;
  bool first = true;
  const cplx* ax = nullptr;  // where A x of the current x is, if known
  while (!rc) {
    // true residual r = b - A x
    if (first && x_zero) {
      if (cudaMemcpyAsync(r, b, n * sizeof(cplx), cudaMemcpyDeviceToDevice, st) != cudaSuccess) { rc = -1; break; }
      ax = nullptr;
    } else if (first && Ax0) {
      k_gs_sub<<<W.grid(), 256, 0, st>>>(b, Ax0, n, r);
      gbi_count_launch();
      ax = Ax0;
    } else {
      if (A(x, w, st)) { rc = -1; break; }
      k_gs_sub<<<W.grid(), 256, 0, st>>>(b, w, n, r);
      gbi_count_launch();
      ax = w;
    }
    first = false;
    if (W.dots(r, n, 1, r, yd)) { rc = -1; break; }
    cplx hr;
    if (cudaMemcpyAsync(&hr, yd, sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) { rc = -1; break; }
    const double beta = sqrt(hr.x);
    const double rel = bnorm > 0.0 ? beta / bnorm : 0.0;
    *relres = rel;
    if (!(rel > tol)) {
      status = (rel == rel) ? 0 : 1;
      if (status == 0 && Ax_out && ax) {
        if (ax != Ax_out &&
            cudaMemcpyAsync(Ax_out, ax, n * sizeof(cplx), cudaMemcpyDeviceToDevice, st) != cudaSuccess) { rc = -1; break; }
        if (ax_ok) *ax_ok = 1;
      }
      break;
    }
    if (it >= maxit) break;
    // a cycle that did not reduce the residual 10x (far from the target) stalls
    if (prev_cycle > 0.0 && rel > 0.1 * prev_cycle && rel > 1e3 * tol) break;
    prev_cycle = rel;
    k_gs_scale<<<W.grid(), 256, 0, st>>>(r, n, 1.0 / beta, V);
    gbi_count_launch();
    std::fill(H.begin(), H.end(), C(0.0, 0.0));
    std::fill(g.begin(), g.end(), C(0.0, 0.0));
    g[0] = C(beta, 0.0);
    int jend = 0;
    for (int j = 0; j < m && it < maxit; j++) {
      cplx* vj = V + (size_t)j * n;
      cplx* zj = Z + (size_t)j * n;
      if (M(vj, zj, st)) { rc = -1; break; }
      if ((Af ? (*Af)(zj, w, st) : A(zj, w, st))) { rc = -1; break; }
      it++;
      // classical Gram-Schmidt, twice
      if (W.dots(V, n, j + 1, w, h2)) { rc = -1; break; }
      k_gs_update<<<W.grid(), 256, 0, st>>>(V, n, j + 1, n, h2, w);
      gbi_count_launch();
      if (W.dots(V, n, j + 1, w, h2 + (m + 2))) { rc = -1; break; }
      k_gs_update<<<W.grid(), 256, 0, st>>>(V, n, j + 1, n, h2 + (m + 2), w);
      gbi_count_launch();
      if (W.dots(w, n, 1, w, yd)) { rc = -1; break; }
      if (cudaMemcpyAsync(hh.data(), h2, (size_t)2 * (m + 2) * sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaMemcpyAsync(&hr, yd, sizeof(cplx), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess) { rc = -1; break; }
      const double hn = sqrt(hr.x);
      for (int i = 0; i <= j; i++)
        H[(size_t)i * m + j] = C(hh[i].x + hh[m + 2 + i].x, hh[i].y + hh[m + 2 + i].y);
      H[(size_t)(j + 1) * m + j] = C(hn, 0.0);
      if (hn > 0.0) {
        k_gs_scale<<<W.grid(), 256, 0, st>>>(w, n, 1.0 / hn, V + (size_t)(j + 1) * n);
        gbi_count_launch();
      }
      // previous rotations, then the one that zeroes H[j+1][j]
      for (int i = 0; i < j; i++) {
        const C a = H[(size_t)i * m + j], c2 = H[(size_t)(i + 1) * m + j];
        H[(size_t)i * m + j] = std::conj(cs[i]) * a + std::conj(sn[i]) * c2;
        H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * c2;
      }
      const C a = H[(size_t)j * m + j], c2 = H[(size_t)(j + 1) * m + j];
      const double den = std::sqrt(std::norm(a) + std::norm(c2));
      if (den == 0.0) { cs[j] = C(1.0, 0.0); sn[j] = C(0.0, 0.0); }
      else { cs[j] = a / den; sn[j] = c2 / den; }
      H[(size_t)j * m + j] = std::conj(cs[j]) * a + std::conj(sn[j]) * c2;
      H[(size_t)(j + 1) * m + j] = C(0.0, 0.0);
      g[j + 1] = -sn[j] * g[j];
      g[j] = std::conj(cs[j]) * g[j];
      jend = j + 1;
      if (!(std::abs(g[j + 1]) > 0.5 * tol * bnorm) || hn == 0.0) break;
    }
    if (rc || jend == 0) break;
    // y = H^-1 g (upper triangular), x += Z y
    for (int i = jend - 1; i >= 0; i--) {
      C s = g[i];
      for (int k = i + 1; k < jend; k++) s -= H[(size_t)i * m + k] * y[k];
      const C d = H[(size_t)i * m + i];
      y[i] = (std::abs(d) > 0.0) ? s / d : C(0.0, 0.0);
    }
    std::vector<cplx> yh((size_t)jend);
    for (int i = 0; i < jend; i++) yh[i] = cmk(y[i].real(), y[i].imag());
    if (cudaMemcpyAsync(yd, yh.data(), (size_t)jend * sizeof(cplx), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = -1;
      break;
    }
    k_gs_combine<<<W.grid(), 256, 0, st>>>(Z, n, jend, n, yd, z);
    gbi_count_launch();
    k_gs_add<<<W.grid(), 256, 0, st>>>(x, z, n);
    gbi_count_launch();
    if (cudaStreamSynchronize(st) != cudaSuccess) { rc = -1; break; }  // yh is host memory
  }
  if (rc) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) gbi_set_error("gmres: %s", cudaGetErrorString(e));
  }
  void* tmp[8] = {V, Z, w, z, r, yd, h2, W.partial};
  for (void* t : tmp)
    if (t) cudaFreeAsync(t, st);
  cudaStreamSynchronize(st);
  *iters = it;
  if (rc) return -1;
  return status;
}
