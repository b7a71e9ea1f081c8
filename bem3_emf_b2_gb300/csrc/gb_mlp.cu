// gb_mlp.cu -- training and inference of the fully connected network of the
// learned near-singular quadrature (include/gb_mlp.h).
//
// The network is small (widths <= a few hundred) and its batches are large
// (up to the near-singular pairs of an assembly, or a training batch), so
// every layer is one tiled SIMT GEMM with its epilogue fused:
//   forward      Z = A W + b, A' = GELU(Z)             (MLP_FWD)
//   data grad    dA = dZ W^T, dZ' = dA * GELU'(Z')     (MLP_BWD)
//   weight grad  dW += A^T dZ over a slice of the batch (MLP_WGRAD, the batch
//                split over gridDim.z, partial sums added with atomics)
// W is read in bfloat16 (the quantised weights), everything else in FP32;
// FP32 accumulation.  The bias gradient is a column sum, the loss an FP64
// reduction, the optimiser Adam on the FP32 master copy, which then refreshes
// the bfloat16 copy.  GELU is the erf form: GELU(z) = z (1 + erf(z / sqrt 2)) / 2.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"
#include "gb_mlp.h"

#define MLP_BM 64
#define MLP_BN 64
#define MLP_BK 16
#define MLP_THREADS 256
#define MLP_WG_ROWS 1024  // batch rows per weight-gradient block

enum { MLP_FWD = 0, MLP_FWD_LAST = 1, MLP_BWD = 2, MLP_WGRAD = 3 };

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad_f(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

struct MlpGemm {
  int M, N, K;
  const float* A;           // FWD/BWD: [M][K]; WGRAD: activations [K = batch][M]
  int lda;
  const __nv_bfloat16* Wb;  // FWD: [K][N]; BWD: [N][K] (read transposed)
  const float* Bf;          // WGRAD: dZ [K = batch][N]
  int ldb;
  const float* bias;        // FWD: [N]
  float* C;                 // FWD: Z [M][N]; BWD: dZ' [M][N]; WGRAD: dW [M][N] (+=)
  float* Act;               // FWD: GELU(Z) [M][N] (MLP_FWD only)
  const float* Zp;          // BWD: Z' [M][N] of the layer below
  int ldc;
  int kchunk;               // WGRAD: batch rows per block
};

// C tile 64 x 64 per block, 4 x 4 per thread, K in slices of 16 staged in
// shared memory (A slice as [k][m], B slice as [k][n])
template <int MODE>
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_gemm(MlpGemm g) {
  __shared__ float As[MLP_BK][MLP_BM + 4];
  __shared__ float Bs[MLP_BK][MLP_BN + 4];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * MLP_BM, n0 = blockIdx.x * MLP_BN;
  int k0 = 0, k1 = g.K;
  if (MODE == MLP_WGRAD) {
    k0 = blockIdx.z * g.kchunk;
    k1 = min(g.K, k0 + g.kchunk);
  }
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  for (int kb = k0; kb < k1; kb += MLP_BK) {
    // A slice: 64 rows x 16 k = 1024 values, 4 per thread
    for (int t = threadIdx.x; t < MLP_BM * MLP_BK; t += MLP_THREADS) {
      int mm, kk;
      if (MODE == MLP_WGRAD) { mm = t % MLP_BM; kk = t / MLP_BM; }  // consecutive threads along m (contiguous)
      else { kk = t % MLP_BK; mm = t / MLP_BK; }                    // along k (contiguous)
      const int m = m0 + mm, k = kb + kk;
      float v = 0.f;
      if (m < g.M && k < k1) v = (MODE == MLP_WGRAD) ? g.A[(size_t)k * g.lda + m] : g.A[(size_t)m * g.lda + k];
      As[kk][mm] = v;
    }
    // B slice: 16 k x 64 cols
    for (int t = threadIdx.x; t < MLP_BK * MLP_BN; t += MLP_THREADS) {
      int nn, kk;
      if (MODE == MLP_BWD) { kk = t % MLP_BK; nn = t / MLP_BK; }  // W[n][k]: along k
      else { nn = t % MLP_BN; kk = t / MLP_BN; }                   // along n
      const int n = n0 + nn, k = kb + kk;
      float v = 0.f;
      if (n < g.N && k < k1) {
        if (MODE == MLP_WGRAD) v = g.Bf[(size_t)k * g.ldb + n];
        else if (MODE == MLP_BWD) v = __bfloat162float(g.Wb[(size_t)n * g.ldb + k]);
        else v = __bfloat162float(g.Wb[(size_t)k * g.ldb + n]);
      }
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < MLP_BK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int m = m0 + ty + 16 * i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int n = n0 + tx + 16 * j;
      if (n >= g.N) continue;
      const size_t q = (size_t)m * g.ldc + n;
      if (MODE == MLP_FWD || MODE == MLP_FWD_LAST) {
        const float z = acc[i][j] + g.bias[n];
        g.C[q] = z;
        if (MODE == MLP_FWD) g.Act[q] = gelu_f(z);
      } else if (MODE == MLP_BWD) {
        g.C[q] = acc[i][j] * gelu_grad_f(g.Zp[q]);
      } else {
        atomicAdd(&g.C[q], acc[i][j]);
      }
    }
  }
}

// D = Y - T: dZ = 2 D / B and loss += sum D^2 / B
__global__ void k_mlp_loss(const float* Y, const float* T, size_t n, float scale, float* dZ, double* loss) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (i < n) {
    const float d = Y[i] - T[i];
    dZ[i] = 2.0f * d * scale;
    s = (double)d * (double)d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s != 0.0) atomicAdd(loss, s * (double)scale);
}

// db[n] += sum over a slice of rows of dZ[r][n]
__global__ void k_mlp_colsum(const float* dZ, int B, int N, int rows, float* db) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int r0 = blockIdx.y * rows, r1 = min(B, r0 + rows);
  float s = 0.f;
  for (int r = r0; r < r1; r++) s += dZ[(size_t)r * N + n];
  atomicAdd(&db[n], s);
}

__global__ void k_mlp_to_bf16(const float* w, __nv_bfloat16* wb, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) wb[i] = __float2bfloat16_rn(w[i]);
}

// Adam on the packed parameters (bias correction c1 = 1 - beta1^t, c2 = 1 - beta2^t)
__global__ void k_mlp_adam(float* p, const float* g, float* m1, float* m2, size_t n, float lr, float c1, float c2) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = 0.9f * m1[i] + 0.1f * gi, b = 0.999f * m2[i] + 0.001f * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
}

// ---------------------------------------------------------------- host side
struct gb_mlp {
  int nl;
  std::vector<int> w;         // widths[0..nl]
  std::vector<size_t> woff;   // offset of W_l in the packed parameters (b_l follows)
  size_t np;                  // parameter count
  float *p, *g, *m1, *m2;     // packed FP32: master, gradient, Adam moments
  __nv_bfloat16* wb;          // bfloat16 copies of the W_l, packed like p (biases unused)
  long step;
  int cap;                    // batch rows the work buffers hold
  std::vector<float*> Z, A;   // Z[l] and, for l < nl - 1, A[l] = GELU(Z[l]) (layer l + 1's input): [cap][w[l + 1]]
  float *dZa, *dZb;           // [cap][max width] each
  double* loss;
  cudaStream_t st;
};

static void mlp_free_work(gb_mlp* m) {
  for (float* z : m->Z) cudaFree(z);
  for (float* a : m->A) cudaFree(a);
  m->Z.assign(m->nl, nullptr);
  m->A.assign(m->nl, nullptr);
  cudaFree(m->dZa); cudaFree(m->dZb);
  m->dZa = m->dZb = nullptr;
  m->cap = 0;
}

static int mlp_work(gb_mlp* m, int B) {
  if (B <= m->cap) return 0;
  mlp_free_work(m);
  int wmax = 0;
  for (int x : m->w) wmax = std::max(wmax, x);
  for (int l = 0; l < m->nl; l++) {
    GB_CUDA(cudaMalloc((void**)&m->Z[l], (size_t)B * m->w[l + 1] * sizeof(float)));
    if (l + 1 < m->nl) GB_CUDA(cudaMalloc((void**)&m->A[l], (size_t)B * m->w[l + 1] * sizeof(float)));
  }
  GB_CUDA(cudaMalloc((void**)&m->dZa, (size_t)B * wmax * sizeof(float)));
  GB_CUDA(cudaMalloc((void**)&m->dZb, (size_t)B * wmax * sizeof(float)));
  m->cap = B;
  return 0;
}

extern "C" void gb_mlp_destroy(gb_mlp* m) {
  if (!m) return;
  mlp_free_work(m);
  cudaFree(m->p); cudaFree(m->g); cudaFree(m->m1); cudaFree(m->m2); cudaFree(m->wb); cudaFree(m->loss);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
}

extern "C" int gb_mlp_create(int nl, const int* widths, gb_mlp** out) {
  *out = nullptr;
  if (nl < 1 || nl > 16) { gbi_set_error("gb_mlp_create: %d layers not in 1..16", nl); return -1; }
  for (int l = 0; l <= nl; l++)
    if (widths[l] < 1 || widths[l] > 4096) { gbi_set_error("gb_mlp_create: width %d not in 1..4096", widths[l]); return -1; }
  gb_mlp* m = new gb_mlp();
  m->nl = nl;
  m->w.assign(widths, widths + nl + 1);
  m->np = 0;
  for (int l = 0; l < nl; l++) {
    m->woff.push_back(m->np);
    m->np += (size_t)widths[l] * widths[l + 1] + widths[l + 1];
  }
  m->p = m->g = m->m1 = m->m2 = nullptr;
  m->wb = nullptr;
  m->loss = nullptr;
  m->st = nullptr;
  m->dZa = m->dZb = nullptr;
  m->Z.assign(nl, nullptr);
  m->A.assign(nl, nullptr);
  m->cap = 0;
  m->step = 0;
  const size_t by = m->np * sizeof(float);
  if (cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc((void**)&m->p, by) != cudaSuccess || cudaMalloc((void**)&m->g, by) != cudaSuccess ||
      cudaMalloc((void**)&m->m1, by) != cudaSuccess || cudaMalloc((void**)&m->m2, by) != cudaSuccess ||
      cudaMalloc((void**)&m->wb, m->np * sizeof(__nv_bfloat16)) != cudaSuccess ||
      cudaMalloc((void**)&m->loss, sizeof(double)) != cudaSuccess) {
    gbi_set_error("gb_mlp_create: %s", cudaGetErrorString(cudaGetLastError()));
    gb_mlp_destroy(m);
    return -1;
  }
  if (cudaMemset(m->p, 0, by) != cudaSuccess || cudaMemset(m->m1, 0, by) != cudaSuccess ||
      cudaMemset(m->m2, 0, by) != cudaSuccess || cudaMemset(m->wb, 0, m->np * sizeof(__nv_bfloat16)) != cudaSuccess) {
    gbi_set_error("gb_mlp_create: memset");
    gb_mlp_destroy(m);
    return -1;
  }
  *out = m;
  return 0;
}

extern "C" size_t gb_mlp_param_count(const gb_mlp* m) { return m->np; }

static int mlp_refresh_bf16(gb_mlp* m) {
  k_mlp_to_bf16<<<(unsigned)((m->np + 255) / 256), 256, 0, m->st>>>(m->p, m->wb, m->np);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

static int mlp_sync(gb_mlp* m, const char* what) {
  cudaError_t e = cudaStreamSynchronize(m->st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) { gbi_set_error("%s: %s", what, cudaGetErrorString(e)); return -1; }
  return 0;
}

extern "C" int gb_mlp_set_params(gb_mlp* m, const float* params) {
  const size_t by = m->np * sizeof(float);
  GB_CUDA(cudaMemcpyAsync(m->p, params, by, cudaMemcpyHostToDevice, m->st));
  GB_CUDA(cudaMemsetAsync(m->m1, 0, by, m->st));
  GB_CUDA(cudaMemsetAsync(m->m2, 0, by, m->st));
  m->step = 0;
  if (mlp_refresh_bf16(m)) return -1;
  return mlp_sync(m, "gb_mlp_set_params");
}

extern "C" int gb_mlp_get_params(gb_mlp* m, float* params) {
  GB_CUDA(cudaMemcpyAsync(params, m->p, m->np * sizeof(float), cudaMemcpyDeviceToHost, m->st));
  return mlp_sync(m, "gb_mlp_get_params");
}

template <int MODE>
static int mlp_gemm(const MlpGemm& g, int zsplit, cudaStream_t st) {
  dim3 grid((unsigned)((g.N + MLP_BN - 1) / MLP_BN), (unsigned)((g.M + MLP_BM - 1) / MLP_BM), (unsigned)zsplit);
  k_mlp_gemm<MODE><<<grid, MLP_THREADS, 0, st>>>(g);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  return 0;
}

// forward of B rows; the output layer's Z is Z[nl - 1]
static int mlp_fwd(gb_mlp* m, int B, const float* X) {
  const float* in = X;
  for (int l = 0; l < m->nl; l++) {
    MlpGemm g;
    memset(&g, 0, sizeof(g));
    g.M = B; g.N = m->w[l + 1]; g.K = m->w[l];
    g.A = in; g.lda = m->w[l];
    g.Wb = m->wb + m->woff[l]; g.ldb = m->w[l + 1];
    g.bias = m->p + m->woff[l] + (size_t)m->w[l] * m->w[l + 1];
    g.C = m->Z[l]; g.Act = m->A[l]; g.ldc = m->w[l + 1];
    const bool last = l + 1 == m->nl;
    if (last ? mlp_gemm<MLP_FWD_LAST>(g, 1, m->st) : mlp_gemm<MLP_FWD>(g, 1, m->st)) return -1;
    in = m->A[l];
  }
  return 0;
}

static int check_batch(gb_mlp* m, int B, const char* what) {
  if (B < 1) { gbi_set_error("%s: batch %d < 1", what, B); return -1; }
  return mlp_work(m, B);
}

extern "C" int gb_mlp_forward(gb_mlp* m, int B, const float* X, float* Y) {
  if (check_batch(m, B, "gb_mlp_forward") || mlp_fwd(m, B, X)) return -1;
  GB_CUDA(cudaMemcpyAsync(Y, m->Z[m->nl - 1], (size_t)B * m->w[m->nl] * sizeof(float), cudaMemcpyDeviceToDevice, m->st));
  return mlp_sync(m, "gb_mlp_forward");
}

// loss and gradient into m->g (and *loss)
static int mlp_grad(gb_mlp* m, int B, const float* X, const float* T, double* loss) {
  if (check_batch(m, B, "gb_mlp_loss_grad") || mlp_fwd(m, B, X)) return -1;
  GB_CUDA(cudaMemsetAsync(m->g, 0, m->np * sizeof(float), m->st));
  GB_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(double), m->st));
  const int L = m->nl;
  const size_t no = (size_t)B * m->w[L];
  k_mlp_loss<<<(unsigned)((no + 255) / 256), 256, 0, m->st>>>(m->Z[L - 1], T, no, 1.0f / (float)B, m->dZa, m->loss);
  gbi_count_launch();
  float* dZ = m->dZa;   // gradient of the current layer's Z
  float* dZn = m->dZb;  // of the layer below
  const int zs = (B + MLP_WG_ROWS - 1) / MLP_WG_ROWS;
  for (int l = L - 1; l >= 0; l--) {
    const float* Ain = l ? m->A[l - 1] : X;
    float* gW = m->g + m->woff[l];
    float* gb = gW + (size_t)m->w[l] * m->w[l + 1];
    MlpGemm g;
    memset(&g, 0, sizeof(g));
    g.M = m->w[l]; g.N = m->w[l + 1]; g.K = B;
    g.A = Ain; g.lda = m->w[l];
    g.Bf = dZ; g.ldb = m->w[l + 1];
    g.C = gW; g.ldc = m->w[l + 1];
    g.kchunk = MLP_WG_ROWS;
    if (mlp_gemm<MLP_WGRAD>(g, zs, m->st)) return -1;
    dim3 cg((unsigned)((m->w[l + 1] + 255) / 256), (unsigned)zs);
    k_mlp_colsum<<<cg, 256, 0, m->st>>>(dZ, B, m->w[l + 1], MLP_WG_ROWS, gb);
    gbi_count_launch();
    if (l > 0) {
      MlpGemm d;
      memset(&d, 0, sizeof(d));
      d.M = B; d.N = m->w[l]; d.K = m->w[l + 1];
      d.A = dZ; d.lda = m->w[l + 1];
      d.Wb = m->wb + m->woff[l]; d.ldb = m->w[l + 1];
      d.C = dZn; d.Zp = m->Z[l - 1]; d.ldc = m->w[l];
      if (mlp_gemm<MLP_BWD>(d, 1, m->st)) return -1;
      float* t = dZ;
      dZ = dZn;
      dZn = t;
    }
  }
  GB_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(double), cudaMemcpyDeviceToHost, m->st));
  return 0;
}

extern "C" int gb_mlp_loss_grad(gb_mlp* m, int B, const float* X, const float* T, double* loss, float* grad) {
  double h = 0.0;
  if (mlp_grad(m, B, X, T, &h)) return -1;
  GB_CUDA(cudaMemcpyAsync(grad, m->g, m->np * sizeof(float), cudaMemcpyDeviceToDevice, m->st));
  if (mlp_sync(m, "gb_mlp_loss_grad")) return -1;
  *loss = h;
  return 0;
}

extern "C" int gb_mlp_train_step(gb_mlp* m, int B, const float* X, const float* T, float lr, double* loss) {
  double h = 0.0;
  if (mlp_grad(m, B, X, T, &h)) return -1;
  m->step++;
  const float c1 = 1.0f - powf(0.9f, (float)m->step), c2 = 1.0f - powf(0.999f, (float)m->step);
  k_mlp_adam<<<(unsigned)((m->np + 255) / 256), 256, 0, m->st>>>(m->p, m->g, m->m1, m->m2, m->np, lr, c1, c2);
  gbi_count_launch();
  if (mlp_refresh_bf16(m) || mlp_sync(m, "gb_mlp_train_step")) return -1;
  *loss = h;
  return 0;
}

// ---------------------------------------------------------------- host arrays
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() { cudaFree(p); }
};

static int upload(DevBuf& b, const float* h, size_t n, cudaStream_t st) {
  GB_CUDA(cudaMalloc(&b.p, n * sizeof(float)));
  GB_CUDA(cudaMemcpyAsync(b.p, h, n * sizeof(float), cudaMemcpyHostToDevice, st));
  return 0;
}

extern "C" int gb_mlp_forward_host(gb_mlp* m, int B, const float* X, float* Y) {
  if (B < 1) { gbi_set_error("gb_mlp_forward_host: batch %d < 1", B); return -1; }
  DevBuf x, y;
  if (upload(x, X, (size_t)B * m->w[0], m->st)) return -1;
  GB_CUDA(cudaMalloc(&y.p, (size_t)B * m->w[m->nl] * sizeof(float)));
  if (gb_mlp_forward(m, B, (const float*)x.p, (float*)y.p)) return -1;
  GB_CUDA(cudaMemcpyAsync(Y, y.p, (size_t)B * m->w[m->nl] * sizeof(float), cudaMemcpyDeviceToHost, m->st));
  return mlp_sync(m, "gb_mlp_forward_host");
}

extern "C" int gb_mlp_loss_grad_host(gb_mlp* m, int B, const float* X, const float* T, double* loss, float* grad) {
  if (B < 1) { gbi_set_error("gb_mlp_loss_grad_host: batch %d < 1", B); return -1; }
  DevBuf x, t, g;
  if (upload(x, X, (size_t)B * m->w[0], m->st) || upload(t, T, (size_t)B * m->w[m->nl], m->st)) return -1;
  GB_CUDA(cudaMalloc(&g.p, m->np * sizeof(float)));
  if (gb_mlp_loss_grad(m, B, (const float*)x.p, (const float*)t.p, loss, (float*)g.p)) return -1;
  GB_CUDA(cudaMemcpyAsync(grad, g.p, m->np * sizeof(float), cudaMemcpyDeviceToHost, m->st));
  return mlp_sync(m, "gb_mlp_loss_grad_host");
}

// steps Adam steps over the n samples (X [n][w0], T [n][w_nl], host), held on
// the device for the call, in consecutive batches of B rows (wrapping round);
// losses[s] (host, may be NULL): the loss of step s's batch before the step
extern "C" int gb_mlp_train_host(gb_mlp* m, int n, const float* X, const float* T, int B, int steps, float lr,
                                 double* losses) {
  if (n < 1 || B < 1 || B > n || steps < 0) {
    gbi_set_error("gb_mlp_train_host: need 1 <= batch %d <= samples %d, steps %d >= 0", B, n, steps);
    return -1;
  }
  DevBuf x, t;
  if (upload(x, X, (size_t)n * m->w[0], m->st) || upload(t, T, (size_t)n * m->w[m->nl], m->st)) return -1;
  const int nb = n / B;  // whole batches per pass
  for (int s = 0; s < steps; s++) {
    const size_t r0 = (size_t)(s % nb) * B;
    double l = 0.0;
    if (gb_mlp_train_step(m, B, (const float*)x.p + r0 * m->w[0], (const float*)t.p + r0 * m->w[m->nl], lr, &l))
      return -1;
    if (losses) losses[s] = l;
  }
  return 0;
}
