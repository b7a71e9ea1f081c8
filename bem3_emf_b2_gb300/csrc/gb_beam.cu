// gb_beam.cu -- incident fields of the focused-beam families on the GPU.
//
// The reference evaluates every beam except the plane wave as an angular
// spectrum of plane waves (mfb_src/fpw.c:170-383, lgb.c:189-397,
// bsb.c:157-343, bslgb.c:178-365, rab.c:170-375):
//
//   e(x) = E0 M^T sum_t w_t  I_t(M (x - f)),
//   I_t(y) = integral over the azimuth a in [-pi, pi) of
//            P(t, a) exp(i ki s(t, a) . y) [exp(i m a)] da,
//
// s = (sin t cos a, sin t sin a, cos t), P the pupil polarisation carried to
// direction s (xy-polarised pupils: fpw, lgb, bsb, blg; radial/azimuthal:
// rab), M the beam's rotation, f its focus.  The polar angle takes
// Gauss-Legendre nodes in sin t on [0, NA/n] (fpw, lgb, rab) or the single
// cone angle of a Bessel beam (bsb, blg, weight sin t).  The azimuthal
// integral is the composite trapezoidal rule refined by halving until the
// electric+magnetic energy of the running sum changes by less than
// TRAP_EPS sqrt(points) times its largest value (after at least two
// halvings): the reference's stopping rule, so the same number of azimuths
// is taken for every node.  The directional derivative d/dv multiplies each
// plane wave by i ki s . (M v).
//
// Work decomposition: one thread per (point, polar node) runs the adaptive
// azimuthal rule for its node; a second kernel sums each point's nodes in
// node order, beams in the reference's order (fpw, lgb, bsb, blg, rab),
// rotates back and scales.  FP64 throughout, as the reference.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <mutex>

#include "gb_beam.h"
#include "gb_internal.h"

#define TRAP_MNUM 12
#define TRAP_LNUM 1
#define TRAP_EPS 1.0e-15
#define GB_NPHI GB_BEAM_NPHI

namespace {

struct z2 {
  double x, y;
};
__device__ __forceinline__ z2 zmk(double a, double b) { return {a, b}; }
__device__ __forceinline__ z2 zadd(z2 a, z2 b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ z2 zmul(z2 a, z2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ z2 zscale(z2 a, double s) { return {a.x * s, a.y * s}; }

// the six field components (E, H) of one plane wave of the spectrum, and
// their derivative along v (the plane wave times i ki s.v)
__device__ __forceinline__ void spectrum_wave(const GbBeamDesc& b, double ct, double st, double cpa, double spa, z2 ph,
                                              const double* y, const double* v, z2* eh, z2* deh) {
  const double sx = st * cpa, sy = st * spa;
  double sn, cs;
  sincos(b.ki * (sx * y[0] + sy * y[1] + ct * y[2]), &sn, &cs);
  const z2 ce = zmul(ph, zmk(cs, sn));
  z2 p[6];
  if (b.kind == 0) {
    const double a = spa * spa + ct * cpa * cpa, bb = spa * cpa * (ct - 1.0), c = ct * spa * spa + cpa * cpa;
    const z2 ex = zmk(b.ex[0], b.ex[1]), ey = zmk(b.ey[0], b.ey[1]);
    const z2 hx = zmk(b.hx[0], b.hx[1]), hy = zmk(b.hy[0], b.hy[1]);
    p[0] = zadd(zscale(ex, a), zscale(ey, bb));
    p[1] = zadd(zscale(ex, bb), zscale(ey, c));
    p[2] = zadd(zscale(ex, -sx), zscale(ey, -sy));
    p[3] = zadd(zscale(hx, a), zscale(hy, bb));
    p[4] = zadd(zscale(hx, bb), zscale(hy, c));
    p[5] = zadd(zscale(hx, -sx), zscale(hy, -sy));
  } else {
    const z2 er = zmk(b.ex[0], b.ex[1]), ea = zmk(b.ey[0], b.ey[1]);
    const z2 hr = zmk(b.hx[0], b.hx[1]), ha = zmk(b.hy[0], b.hy[1]);
    p[0] = zadd(zscale(er, ct * cpa), zscale(ea, -spa));
    p[1] = zadd(zscale(er, ct * spa), zscale(ea, cpa));
    p[2] = zscale(er, -st);
    p[3] = zadd(zscale(hr, ct * cpa), zscale(ha, -spa));
    p[4] = zadd(zscale(hr, ct * spa), zscale(ha, cpa));
    p[5] = zscale(hr, -st);
  }
#pragma unroll
  for (int i = 0; i < 6; i++) eh[i] = zmul(p[i], ce);
  if (v) {
    const z2 g = zmk(0.0, b.ki * (sx * v[0] + sy * v[1] + ct * v[2]));
#pragma unroll
    for (int i = 0; i < 6; i++) deh[i] = zmul(eh[i], g);
  }
}

__device__ __forceinline__ double energy(const z2* It, double cep) {
  double e = 0.0;
#pragma unroll
  for (int i = 0; i < 6; i++) e += (i < 3 ? cep : 1.0) * (It[i].x * It[i].x + It[i].y * It[i].y);
  return e;
}

struct BeamArgs {
  int n, T;
  const double* x;      // [n][3]
  const double* v;      // [n][3] or null
  const GbBeamDesc* beams;
  const int* item_beam;  // [T]
  const double* node;    // [T][3]: cos t, sin t, weight
  const double* phi;     // [GB_NPHI][2]: cos, sin of the azimuths in refinement order
  const double* phase;   // [nphase][GB_NPHI][2]
  double* out;           // [n][T][24]: weighted I (6) and dI (6), complex
  int* err;
};

__global__ void __launch_bounds__(128) k_beam_nodes(BeamArgs a) {
  const size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (size_t)a.n * a.T) return;
  const int p = (int)(q / a.T), it = (int)(q % a.T);
  const GbBeamDesc& b = a.beams[a.item_beam[it]];
  const double ct = a.node[3 * it], st = a.node[3 * it + 1], w = a.node[3 * it + 2];
  // point and direction in the beam's frame
  double y[3], vv[3];
  const double xb[3] = {a.x[3 * p] - b.f[0], a.x[3 * p + 1] - b.f[1], a.x[3 * p + 2] - b.f[2]};
  const bool dv = a.v != nullptr;
  for (int r = 0; r < 3; r++) {
    y[r] = b.M[3 * r] * xb[0] + b.M[3 * r + 1] * xb[1] + b.M[3 * r + 2] * xb[2];
    if (dv) vv[r] = b.M[3 * r] * a.v[3 * p] + b.M[3 * r + 1] * a.v[3 * p + 1] + b.M[3 * r + 2] * a.v[3 * p + 2];
  }
  const double* vp = dv ? vv : nullptr;
  const double2* ph = b.phase >= 0 ? (const double2*)(a.phase + (size_t)b.phase * GB_NPHI * 2) : nullptr;
  const double2* cs = (const double2*)a.phi;
  z2 Ia[6], dIa[6], It[6], dIt[6], Is[6], dIs[6];
  double h = 2.0 * 3.14159265358979323846;
  {
    const double2 c0 = cs[0];
    const z2 p0 = ph ? zmk(ph[0].x, ph[0].y) : zmk(1.0, 0.0);
    spectrum_wave(b, ct, st, c0.x, c0.y, p0, y, vp, Ia, dIa);
  }
#pragma unroll
  for (int i = 0; i < 6; i++) {
    It[i] = zscale(Ia[i], h);
    dIt[i] = dv ? zscale(dIa[i], h) : zmk(0.0, 0.0);
  }
  double abst = energy(It, b.cep), f_order = abst;
  int j = 1, sc = 1, cc = 0;
  while (cc <= TRAP_MNUM) {
    h *= 0.5;
#pragma unroll
    for (int i = 0; i < 6; i++) Is[i] = dIs[i] = zmk(0.0, 0.0);
    for (int s = 1; s <= sc; s++, j++) {
      const double2 c = cs[j];
      const z2 pj = ph ? zmk(ph[j].x, ph[j].y) : zmk(1.0, 0.0);
      spectrum_wave(b, ct, st, c.x, c.y, pj, y, vp, Ia, dIa);
#pragma unroll
      for (int i = 0; i < 6; i++) {
        Is[i] = zadd(Is[i], Ia[i]);
        if (dv) dIs[i] = zadd(dIs[i], dIa[i]);
      }
    }
#pragma unroll
    for (int i = 0; i < 6; i++) {
      It[i] = zadd(zscale(It[i], 0.5), zscale(Is[i], h));
      if (dv) dIt[i] = zadd(zscale(dIt[i], 0.5), zscale(dIs[i], h));
    }
    const double abss = energy(It, b.cep);
    const double cr = sqrt((double)sc) * f_order;
    if ((cc > TRAP_LNUM && fabs(abst - abss) < TRAP_EPS * cr) || (abss == 0.0 && abst == 0.0)) break;
    abst = abss;
    if (abst > f_order) f_order = abst;
    sc *= 2;
    cc++;
  }
  if (cc >= TRAP_MNUM) atomicExch(a.err, 1);
  double* o = a.out + q * 24;
#pragma unroll
  for (int i = 0; i < 6; i++) {
    o[2 * i] = It[i].x * w;
    o[2 * i + 1] = It[i].y * w;
    o[12 + 2 * i] = dIt[i].x * w;
    o[13 + 2 * i] = dIt[i].y * w;
  }
}

// per point: node sums in node order, beam by beam in the given order,
// rotated back (M^T) and scaled by E0; E, H, dE, dH [n][3] complex
__global__ void k_beam_sum(int n, int T, int nb, const GbBeamDesc* beams, const double* nodes_out, double* E,
                           double* H, double* dE, double* dH) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  double acc[24];
  for (int i = 0; i < 24; i++) acc[i] = 0.0;
  const double* base = nodes_out + (size_t)p * T * 24;
  for (int bi = 0; bi < nb; bi++) {
    const GbBeamDesc& b = beams[bi];
    double s[24];
    for (int i = 0; i < 24; i++) s[i] = 0.0;
    for (int t = b.t0; t < b.t0 + b.nt; t++)
      for (int i = 0; i < 24; i++) s[i] += base[(size_t)t * 24 + i];
    // groups of three complex components: e, h, de, dh
    for (int g = 0; g < 4; g++) {
      const double* c = s + 6 * g;
      for (int r = 0; r < 3; r++) {
        const double re = b.M[r] * c[0] + b.M[3 + r] * c[2] + b.M[6 + r] * c[4];
        const double im = b.M[r] * c[1] + b.M[3 + r] * c[3] + b.M[6 + r] * c[5];
        acc[6 * g + 2 * r] += re * b.E0;
        acc[6 * g + 2 * r + 1] += im * b.E0;
      }
    }
  }
  double* outs[4] = {E, H, dE, dH};
  for (int g = 0; g < 4; g++)
    if (outs[g])
      for (int i = 0; i < 6; i++) outs[g][(size_t)p * 6 + i] = acc[6 * g + i];
}

// the calling thread's stream per device, destroyed when the thread ends
struct BeamStreams {
  cudaStream_t s[64] = {};
  ~BeamStreams() {
    for (int d = 0; d < 64; d++)
      if (s[d] && cudaSetDevice(d) == cudaSuccess) cudaStreamDestroy(s[d]);
  }
};
thread_local BeamStreams t_beam_stream;

}  // namespace

// Fields of a set of spectrum beams at n points (host arrays in and out).
extern "C" int gbi_beam_points(int nb, const GbBeamDesc* beams, int T, const int* item_beam, const double* nodes,
                               const double* phi, int nphase, const double* phase, int n, const double* x,
                               const double* v, double* E, double* H, double* dE, double* dH) {
  if (n <= 0 || nb <= 0) return 0;
  if (T <= 0 || !beams || !item_beam || !nodes || !phi || !x) {
    gbi_set_error("gbi_beam_points: invalid arguments");
    return -1;
  }
  int dev = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    gbi_set_error("gbi_beam_points: device %d", dev);
    return -1;
  }
  if (!t_beam_stream.s[dev]) GB_CUDA(cudaStreamCreateWithFlags(&t_beam_stream.s[dev], cudaStreamNonBlocking));
  cudaStream_t st = t_beam_stream.s[dev];
  // points in chunks: at most 256 MiB of node partial sums at a time
  const size_t per_point = (size_t)T * 24 * sizeof(double);
  int chunk = (int)(((size_t)256 << 20) / per_point);
  if (chunk < 1) chunk = 1;
  if (chunk > n) chunk = n;
  GbBeamDesc* d_beams = nullptr;
  int *d_item = nullptr, *d_err = nullptr;
  double *d_nodes = nullptr, *d_phi = nullptr, *d_phase = nullptr, *d_x = nullptr, *d_v = nullptr, *d_out = nullptr,
         *d_res = nullptr;
  int rc = -1;
  int herr = 0;
  auto fail = [&](cudaError_t e, const char* what) {
    gbi_set_error("gbi_beam_points: %s: %s", what, cudaGetErrorString(e));
  };
  cudaError_t e;
#define GB_BEAM_TRY(call, what) \
  if ((e = (call)) != cudaSuccess) { fail(e, what); goto done; }
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_beams, nb * sizeof(GbBeamDesc), st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_item, T * sizeof(int), st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_err, sizeof(int), st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_nodes, (size_t)T * 3 * sizeof(double), st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_phi, (size_t)GB_NPHI * 2 * sizeof(double), st), "alloc");
  if (nphase > 0) GB_BEAM_TRY(cudaMallocAsync((void**)&d_phase, (size_t)nphase * GB_NPHI * 2 * sizeof(double), st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_x, (size_t)chunk * 3 * sizeof(double), st), "alloc");
  if (v) GB_BEAM_TRY(cudaMallocAsync((void**)&d_v, (size_t)chunk * 3 * sizeof(double), st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_out, (size_t)chunk * per_point, st), "alloc");
  GB_BEAM_TRY(cudaMallocAsync((void**)&d_res, (size_t)chunk * 24 * sizeof(double), st), "alloc");
  GB_BEAM_TRY(cudaMemcpyAsync(d_beams, beams, nb * sizeof(GbBeamDesc), cudaMemcpyHostToDevice, st), "copy");
  GB_BEAM_TRY(cudaMemcpyAsync(d_item, item_beam, T * sizeof(int), cudaMemcpyHostToDevice, st), "copy");
  GB_BEAM_TRY(cudaMemcpyAsync(d_nodes, nodes, (size_t)T * 3 * sizeof(double), cudaMemcpyHostToDevice, st), "copy");
  GB_BEAM_TRY(cudaMemcpyAsync(d_phi, phi, (size_t)GB_NPHI * 2 * sizeof(double), cudaMemcpyHostToDevice, st), "copy");
  if (nphase > 0)
    GB_BEAM_TRY(cudaMemcpyAsync(d_phase, phase, (size_t)nphase * GB_NPHI * 2 * sizeof(double), cudaMemcpyHostToDevice, st),
                "copy");
  GB_BEAM_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st), "memset");
  for (int p0 = 0; p0 < n; p0 += chunk) {
    const int m = n - p0 < chunk ? n - p0 : chunk;
    GB_BEAM_TRY(cudaMemcpyAsync(d_x, x + (size_t)p0 * 3, (size_t)m * 3 * sizeof(double), cudaMemcpyHostToDevice, st),
                "copy");
    if (v)
      GB_BEAM_TRY(cudaMemcpyAsync(d_v, v + (size_t)p0 * 3, (size_t)m * 3 * sizeof(double), cudaMemcpyHostToDevice, st),
                  "copy");
    BeamArgs a;
    a.n = m; a.T = T; a.x = d_x; a.v = v ? d_v : nullptr; a.beams = d_beams; a.item_beam = d_item;
    a.node = d_nodes; a.phi = d_phi; a.phase = d_phase; a.out = d_out; a.err = d_err;
    const size_t nq = (size_t)m * T;
    k_beam_nodes<<<(unsigned)((nq + 127) / 128), 128, 0, st>>>(a);
    gbi_count_launch();
    double* r = d_res;
    k_beam_sum<<<(m + 127) / 128, 128, 0, st>>>(m, T, nb, d_beams, d_out, r, r + (size_t)m * 6,
                                                v ? r + (size_t)m * 12 : nullptr, v ? r + (size_t)m * 18 : nullptr);
    gbi_count_launch();
    GB_BEAM_TRY(cudaGetLastError(), "launch");
    double* hosts[4] = {E, H, dE, dH};
    for (int g = 0; g < (v ? 4 : 2); g++)
      if (hosts[g])
        GB_BEAM_TRY(cudaMemcpyAsync(hosts[g] + (size_t)p0 * 6, r + (size_t)m * 6 * g, (size_t)m * 6 * sizeof(double),
                                    cudaMemcpyDeviceToHost, st),
                    "copy");
  }
  GB_BEAM_TRY(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st), "copy");
  GB_BEAM_TRY(cudaStreamSynchronize(st), "sync");
  rc = herr ? 1 : 0;
  if (herr) gbi_set_error("phi integration limit over!");
done:
#undef GB_BEAM_TRY
  void* bufs[] = {d_beams, d_item, d_err, d_nodes, d_phi, d_phase, d_x, d_v, d_out, d_res};
  for (void* b : bufs)
    if (b) cudaFreeAsync(b, st);
  if (rc < 0) cudaStreamSynchronize(st);
  return rc;
}
