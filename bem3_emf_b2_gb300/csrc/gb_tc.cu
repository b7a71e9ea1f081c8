// gb_tc.cu -- complex-FP32 GEMM update C -= A B on the 5th-generation tensor
// cores (tcgen05.mma kind::tf32, TMA, TMEM): the trailing update of the
// complex-FP32 LU of the chosen form.
//
// A complex product is a real GEMM on interleaved (re, im) storage.  With C, A,
// B row-major complex64,
//     Cr[m][2n] -= Ar[m][2k] * Bt[2n][2k]^T,
//     Bt[2j+e][2l+f] = f == 0 ? (e == 0 ? Re b :  Im b)
//                             : (e == 0 ? -Im b : Re b),      b = B[l][j],
// and Ar is A itself read as floats (row i: re a_i0, im a_i0, re a_i1, ...).
// TF32 keeps 10 mantissa bits.  With PASSES = 3 every operand x is split as
// x = hi + lo (hi = x rounded to TF32, lo = x - hi exact in FP32) and the
// tile accumulates hi*hi + hi*lo + lo*hi in FP32: products then carry about
// 2^-21 relative error, close to FP32 arithmetic (the standard 3xTF32
// emulation).  PASSES = 1 is plain TF32.
//
// Kernel: persistent, one CTA per SM, 128 x 256 tiles of Cr, 320 threads.
//   warp 0     streams K-slices of 32 floats (one 128-byte swizzle atom) of
//              the operands into a ring of shared-memory stages with TMA
//              (SWIZZLE_128B), running ahead across tiles;
//   warp 1     allocates 512 TMEM columns (two FP32 accumulators) and issues
//              tcgen05.mma.cta_group::1.kind::tf32 (M = 128, N = 256, K = 8),
//              committing each stage back to the producer and each finished
//              accumulator to the epilogue;
//   warps 2-9  read an accumulator (tcgen05.ld 32x32b: TMEM lane = tile row,
//              two warps per lane quarter, one per half of the columns),
//              transpose it through shared memory and subtract it from C
//              (lanes on consecutive columns) while the next tile accumulates
//              in the other buffer.
// Every mbarrier wait is bounded in time (TC_WAIT_NS); on time-out the CTA
// raises *err, stops issuing work, frees its TMEM and returns.
#include <cuda.h>

#include <cstring>
#include <mutex>
#include <atomic>
#include <vector>

#include "gb_common.cuh"
#include "gb_internal.h"

#define TC_BM 128
#define TC_BN 256
#define TC_BK 32  // floats per K-slice: 128 bytes, one swizzle atom
#define TC_THREADS 320
#define TC_WAIT_NS 2000000000ull  // 2 s

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// wait for the phase of the given parity to complete; false after TC_WAIT_NS
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_test(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  while (!mbar_test(bar, parity)) {
    if (globaltimer() - t0 > TC_WAIT_NS) return false;
  }
  return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, rows of
// 128 bytes, 8-row atoms 1024 bytes apart (stride byte offset); the leading
// byte offset is unused for this layout.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // bits 0-13: start address >> 4
  d |= (uint64_t)(1024u >> 4) << 32;          // bits 32-45: stride byte offset >> 4
  d |= (uint64_t)1 << 46;                     // bits 46-47: descriptor version
  d |= (uint64_t)2 << 61;                     // bits 61-63: SWIZZLE_128B
  return d;
}

// instruction descriptor, kind::tf32: D = F32, A = B = TF32, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                            // bits 4-5: D format F32
         | (2u << 7)                          // bits 7-9: A format TF32
         | (2u << 10)                         // bits 10-12: B format TF32
         | ((uint32_t)(N >> 3) << 17)         // bits 17-22: N >> 3
         | ((uint32_t)(M >> 4) << 24);        // bits 24-28: M >> 4
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

template <int PASSES>
struct TcLayout {
  static constexpr int A_BYTES = TC_BM * TC_BK * 4;  // 16 KB
  static constexpr int B_BYTES = TC_BN * TC_BK * 4;  // 32 KB
  static constexpr int NOPS = PASSES == 3 ? 2 : 1;
  static constexpr int STAGE = NOPS * (A_BYTES + B_BYTES);
  static constexpr int STAGES = PASSES == 3 ? 2 : 4;  // 192 KB either way: one CTA per SM owns all of TMEM
  static constexpr int EPI = 8 * 32 * 32 * 4;  // per epilogue warp a 32 x 32 float chunk (128-byte swizzle)
  static constexpr int SMEM = STAGES * STAGE + 1024 /* alignment */ + 1024 /* barriers */ + EPI;
};

// Persistent: CTA b takes tiles b, b + gridDim.x, ...; tile t covers rows
// 128 (t / ntn) and real columns 256 (t % ntn) of Cr.  Warp roles:
//   warp 0     (one lane) TMA producer, ring of STAGES K-slices across tiles
//   warp 1     allocates TMEM (two 256-column accumulators); one lane issues
//              the MMAs of a tile into accumulator (local tile index & 1)
//   warps 2-9  epilogue: warp w reads TMEM lanes 32 (w & 3) .. + 31 (tile
//              rows) for one half of the tile's columns, transposes 32 x 32
//              chunks through shared memory and subtracts them from C with
//              coalesced accesses, while the MMAs of the next tile fill the
//              other accumulator
template <int PASSES>
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_tc_cgemm_sub(const __grid_constant__ CUtensorMap mAhi, const __grid_constant__ CUtensorMap mAlo,
                   const __grid_constant__ CUtensorMap mBhi, const __grid_constant__ CUtensorMap mBlo,
                   const __grid_constant__ CUtensorMap mC, int use_tma_c, int m, int n2, int nkb, float* C, size_t ldcf,
                   int* err) {
  using L = TcLayout<PASSES>;
  constexpr int S = L::STAGES;
  extern __shared__ uint8_t smraw[];
  const uint32_t raw_u32 = smem_u32(smraw);
  uint8_t* sm = smraw + ((1024u - (raw_u32 & 1023u)) & 1023u);  // 1024-byte aligned (swizzle atoms)
  const uint32_t sbase = smem_u32(sm);
  // barriers: full[s] bar0 + 8 s, empty[s] bar0 + 64 + 8 s, tfull[b] bar0 + 128 + 8 b, tempty[b] bar0 + 144 + 8 b
  const uint32_t bar0 = sbase + S * L::STAGE;
  uint32_t* tslot = (uint32_t*)(sm + S * L::STAGE + 192);
  volatile int* s_fail = (volatile int*)(sm + S * L::STAGE + 200);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntn = (n2 + TC_BN - 1) / TC_BN;
  const int ntiles = ((m + TC_BM - 1) / TC_BM) * ntn;

  if (threadIdx.x == 0) {
    *s_fail = 0;
    for (int s = 0; s < S; s++) {
      mbar_init(bar0 + 8 * s, 1);
      mbar_init(bar0 + 64 + 8 * s, 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(bar0 + 128 + 8 * b, 1);
      mbar_init(bar0 + 144 + 8 * b, 8);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(2 * TC_BN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      uint32_t g = 0;
      for (int t = blockIdx.x; t < ntiles && !*s_fail; t += gridDim.x) {
        const int i0 = (t / ntn) * TC_BM, c0 = (t % ntn) * TC_BN;
        for (int kb = 0; kb < nkb; kb++, g++) {
          const uint32_t s = g % S, u = g / S;
          if (u >= 1 && !mbar_wait(bar0 + 64 + 8 * s, (u - 1) & 1)) { *s_fail = 1; break; }
          const uint32_t st = sbase + s * L::STAGE;
          const uint32_t fb = bar0 + 8 * s;
          mbar_expect_tx(fb, L::STAGE);
          tma_load_2d(st, &mAhi, fb, kb * TC_BK, i0);
          tma_load_2d(st + L::A_BYTES, &mBhi, fb, kb * TC_BK, c0);
          if (PASSES == 3) {
            tma_load_2d(st + L::A_BYTES + L::B_BYTES, &mAlo, fb, kb * TC_BK, i0);
            tma_load_2d(st + 2 * L::A_BYTES + L::B_BYTES, &mBlo, fb, kb * TC_BK, c0);
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      constexpr uint32_t idesc = idesc_tf32(TC_BM, TC_BN);
      uint32_t g = 0, lt = 0;
      for (int t = blockIdx.x; t < ntiles && !*s_fail; t += gridDim.x, lt++) {
        const uint32_t b = lt & 1, u = lt >> 1;
        if (u >= 1 && !mbar_wait(bar0 + 144 + 8 * b, (u - 1) & 1)) { *s_fail = 1; break; }
        tc_fence_after();
        const uint32_t d = tmem + b * TC_BN;
        bool ok = true;
        for (int kb = 0; kb < nkb; kb++, g++) {
          const uint32_t s = g % S;
          if (!mbar_wait(bar0 + 8 * s, (g / S) & 1)) { *s_fail = 1; ok = false; break; }
          tc_fence_after();
          const uint32_t ahi = sbase + s * L::STAGE, bhi = ahi + L::A_BYTES;
          const uint32_t alo = bhi + L::B_BYTES, blo = alo + L::A_BYTES;
#pragma unroll
          for (int kk = 0; kk < TC_BK / 8; kk++) {
            const uint32_t off = kk * 32;  // 8 TF32 = 32 bytes along K inside the swizzle atom
            mma_tf32(d, sdesc_sw128(ahi + off), sdesc_sw128(bhi + off), idesc, (kb | kk) != 0);
            if (PASSES == 3) {
              mma_tf32(d, sdesc_sw128(ahi + off), sdesc_sw128(blo + off), idesc, 1);
              mma_tf32(d, sdesc_sw128(alo + off), sdesc_sw128(bhi + off), idesc, 1);
            }
          }
          mma_commit(bar0 + 64 + 8 * s);  // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        mma_commit(bar0 + 128 + 8 * b);  // accumulator b complete
      }
    }
  } else {  // epilogue warps 2..9: warp w reads TMEM lanes 32 (w & 3).. (tile rows), columns 128 h.. (h = (w-2) / 4)
    const int q = warp & 3, h = (warp - 2) >> 2;
    // Accumulator rows arrive one per lane.  With use_tma_c each 32 x 32 chunk
    // is negated into a 128-byte-swizzled shared-memory tile and added to C by
    // a TMA reduction (cp.reduce.async.bulk.tensor ... .add: the L2 does the
    // read-modify-write, the SM never loads C); otherwise the chunk is
    // transposed through the same buffer and C is read and written with lanes
    // on consecutive columns.
    uint8_t* tbb = sm + S * L::STAGE + 1024 + (warp - 2) * 4096;  // 1024-byte aligned, 4 KB
    float* tb = (float*)tbb;
    const uint32_t tb_s = smem_u32(tbb);
    uint32_t lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, lt++) {
      const uint32_t b = lt & 1, u = lt >> 1;
      const int i0 = (t / ntn) * TC_BM + q * 32, c0 = (t % ntn) * TC_BN + h * (TC_BN / 2);
      int ok = 1;
      if (lane == 0) ok = mbar_wait(bar0 + 128 + 8 * b, u & 1) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (!ok || *s_fail) { *s_fail = 1; break; }
      __syncwarp();
      tc_fence_after();
      const uint32_t ta = tmem + b * TC_BN + (uint32_t)(h * (TC_BN / 2)) + ((uint32_t)(q * 32) << 16);
#pragma unroll 1
      for (int cc = 0; cc < TC_BN / 2; cc += 32) {
        if (use_tma_c) {
          float v[32];
          tmem_ld16(ta + cc, v);
          tmem_ld16(ta + cc + 16, v + 16);
          if (cc + 32 == TC_BN / 2) {  // this warp's part of accumulator b is read: signal the MMA warp
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar0 + 144 + 8 * b) : "memory");
          }
          if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");  // the buffer is free
          __syncwarp();
          // row lane: 16-byte chunk c4 sits at chunk position c4 ^ (lane & 7)
#pragma unroll
          for (int c4 = 0; c4 < 8; c4++) {
            float4 t4 = make_float4(-v[4 * c4], -v[4 * c4 + 1], -v[4 * c4 + 2], -v[4 * c4 + 3]);
            *(float4*)(tbb + lane * 128 + ((c4 ^ (lane & 7)) << 4)) = t4;
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          __syncwarp();
          if (lane == 0) {
            asm volatile(
                "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                    (uint64_t)&mC),
                "r"(c0 + cc), "r"(i0), "r"(tb_s)
                : "memory");
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
          }
        } else {
          const int col = c0 + cc + lane;
          const bool colok = col < n2;
          float cv[32];
#pragma unroll
          for (int r = 0; r < 32; r++) cv[r] = (colok && i0 + r < m) ? C[(size_t)(i0 + r) * ldcf + col] : 0.f;
          float v[32];
          tmem_ld16(ta + cc, v);
          tmem_ld16(ta + cc + 16, v + 16);
          if (cc + 32 == TC_BN / 2) {
            tc_fence_before();
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar0 + 144 + 8 * b) : "memory");
          }
#pragma unroll
          for (int c = 0; c < 32; c++) tb[lane * 32 + (c ^ lane)] = v[c];  // XOR layout: conflict-free both ways
          __syncwarp();
#pragma unroll
          for (int r = 0; r < 32; r++)
            if (colok && i0 + r < m) C[(size_t)(i0 + r) * ldcf + col] = cv[r] - tb[r * 32 + (lane ^ r)];
          __syncwarp();
        }
      }
    }
    if (use_tma_c && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_BN) : "memory");
  }
  if (threadIdx.x == 0 && *s_fail) atomicExch(err, 1);
}

// The operands as TF32 hi (and lo) parts in the layouts the TMA loads:
//   A (m x kc complex, lda) -> [m][Kp] floats, row i = (re, im) of A[i][*]
//   B (kc x n complex, ldb) -> Bt [2n][Kp]: Bt[2j+e][2l+f] = re, im, -im, re
//     of B[l][j] for (e, f) = (0,0), (1,0), (0,1), (1,1), so that the real
//     GEMM on interleaved storage gives re and im of the complex product
// (columns >= 2 kc zero).  Both in one launch: blocks [0, nba) split A, the
// rest build Bt (independent; one launch instead of two per update).
__global__ void k_tc_prep(const cplxf* __restrict__ A, size_t lda, int m, const cplxf* __restrict__ B, size_t ldb,
                          int n, int kc, int Kp, unsigned nba, float* ahi, float* alo, float* bhi, float* blo) {
  if (blockIdx.x < nba) {
    const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (size_t)m * Kp) return;
    const int i = (int)(t / Kp), q = (int)(t % Kp);
    float v = 0.f;
    if (q < 2 * kc) {
      const cplxf a = A[(size_t)i * lda + (q >> 1)];
      v = (q & 1) ? a.y : a.x;
    }
    const float h = tf32_round(v);
    ahi[t] = h;
    if (alo) alo[t] = v - h;
  } else {
    const size_t t = (size_t)(blockIdx.x - nba) * blockDim.x + threadIdx.x;
    if (t >= (size_t)2 * n * Kp) return;
    const int cp = (int)(t / Kp), q = (int)(t % Kp);
    float v = 0.f;
    if (q < 2 * kc) {
      const cplxf b = B[(size_t)(q >> 1) * ldb + (cp >> 1)];
      const int e = cp & 1, f = q & 1;
      v = f == 0 ? (e == 0 ? b.x : b.y) : (e == 0 ? -b.y : b.x);
    }
    const float h = tf32_round(v);
    bhi[t] = h;
    if (blo) blo[t] = v - h;
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  // looked up once; the initialisation of a function-local static is
  // thread-safe (callers may run on several host threads)
  static const EncodeTiledFn fn = []() -> EncodeTiledFn {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return (EncodeTiledFn)p;
    return nullptr;
  }();
  return fn;
}

// 2-D FP32 tensor map over rows x Kp floats (row stride Kp), box 32 x box_rows
int make_map(CUtensorMap* map, const float* base, int rows, int Kp, int box_rows) {
  EncodeTiledFn enc = encode_fn();
  if (!enc) {
    gbi_set_error("tensor-core GEMM: cuTensorMapEncodeTiled unavailable");
    return -1;
  }
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 4};
  cuuint32_t box[2] = {TC_BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    gbi_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
    return -1;
  }
  return 0;
}

}  // namespace

// Optional live timing of the tensor-core kernel (for roofline figures): while
// enabled, every launch is bracketed by two CUDA events on its own stream and
// its algorithmic work is recorded; gb_ktime_read() sums after the caller
// synchronised.  Algorithmic HBM bytes of one launch: C read and written
// (16 M N), the split operands read once (2 passes x 4 bytes x (M + 2N) Kp).
namespace {
struct KtRec {
  cudaEvent_t a, b;
  double flops, bytes;
  int M, N, K;
};
std::mutex g_kt_mu;
bool g_kt_on = false;
std::vector<KtRec> g_kt;
// launches of the double-float regular assembly (k_asm_regular_df_list):
// events and the (collocation node, element) pairs each one covers
struct KaRec {
  cudaEvent_t a, b;
  double pairs;
};
std::vector<KaRec> g_ka;
}  // namespace

// While timing is enabled: records an event on st before an assembly launch;
// returns 1 if it did (the caller then calls gbi_kt_asm_stop after the launch)
extern "C" int gbi_kt_asm_start(cudaStream_t st, void** h) {
  std::lock_guard<std::mutex> lk(g_kt_mu);
  if (!g_kt_on) return 0;
  KaRec* r = new KaRec;
  if (cudaEventCreate(&r->a) != cudaSuccess || cudaEventCreate(&r->b) != cudaSuccess ||
      cudaEventRecord(r->a, st) != cudaSuccess) {
    delete r;
    return 0;
  }
  *h = r;
  return 1;
}

extern "C" void gbi_kt_asm_stop(void* h, cudaStream_t st, double pairs) {
  KaRec* r = (KaRec*)h;
  r->pairs = pairs;
  cudaEventRecord(r->b, st);
  std::lock_guard<std::mutex> lk(g_kt_mu);
  g_ka.push_back(*r);
  delete r;
}

// recorded double-float assembly launches: total device ms, pairs, launches
// (not cleared; gb_ktime_enable clears)
extern "C" int gb_ktime_asm(double* ms, double* pairs, long* launches) {
  std::lock_guard<std::mutex> lk(g_kt_mu);
  double t = 0.0, p = 0.0;
  for (auto& r : g_ka) {
    float x = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&x, r.a, r.b) != cudaSuccess) {
      gbi_set_error("gb_ktime_asm: event query failed");
      return -1;
    }
    t += x;
    p += r.pairs;
  }
  *ms = t;
  *pairs = p;
  *launches = (long)g_ka.size();
  return 0;
}

extern "C" void gb_ktime_enable(int on) {
  std::lock_guard<std::mutex> lk(g_kt_mu);
  for (auto& r : g_kt) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  g_kt.clear();
  for (auto& r : g_ka) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  g_ka.clear();
  g_kt_on = on != 0;
}

// total device milliseconds, launches, algorithmic complex-equivalent flops
// (8 M N K) and HBM bytes of the recorded launches; clears the record
extern "C" int gb_ktime_read(double* ms, long* launches, double* flops, double* bytes) {
  std::lock_guard<std::mutex> lk(g_kt_mu);
  double t = 0.0, f = 0.0, b = 0.0;
  int rc = 0;
  for (auto& r : g_kt) {
    float x = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&x, r.a, r.b) != cudaSuccess) rc = -1;
    t += x;
    f += r.flops;
    b += r.bytes;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  *ms = t;
  *launches = (long)g_kt.size();
  *flops = f;
  *bytes = b;
  g_kt.clear();
  if (rc) gbi_set_error("gb_ktime_read: event query failed");
  return rc;
}

// the recorded launches one by one (not cleared): rec[4 i .. 4 i + 3] = device
// ms, M, N, K of launch i for i < min(cap, count); returns the count or -1
extern "C" int gb_ktime_list(int cap, double* rec) {
  std::lock_guard<std::mutex> lk(g_kt_mu);
  int i = 0;
  for (auto& r : g_kt) {
    if (i >= cap) break;
    float x = 0.f;
    if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&x, r.a, r.b) != cudaSuccess) {
      gbi_set_error("gb_ktime_list: event query failed");
      return -1;
    }
    rec[4 * i] = x;
    rec[4 * i + 1] = r.M;
    rec[4 * i + 2] = r.N;
    rec[4 * i + 3] = r.K;
    i++;
  }
  return (int)g_kt.size();
}

// Tensor-core passes of the complex-FP32 factorisations (LU updates, inverses,
// block-elimination products): 3 (split TF32 hi/lo: FP32-level products, the
// default) or 1 (plain TF32, ~1e-3 relative error in the factors; the FP64
// GMRES refinement tolerates it).  Process-wide: it applies to factorisations
// started after the call.
static std::atomic<int> g_tc_passes{1};
extern "C" int gb_set_tc_passes(int passes) {
  if (passes != 1 && passes != 3) { gbi_set_error("gb_set_tc_passes: passes must be 1 or 3"); return -1; }
  g_tc_passes.store(passes);
  return 0;
}
extern "C" int gbi_tc_passes(void) { return g_tc_passes.load(); }
extern "C" int gb_get_tc_passes(void) { return g_tc_passes.load(); }

// floats of scratch that gbi_tc_cgemm_sub needs for an M x N x K update
extern "C" size_t gbi_tc_scratch_floats(int M, int N, int K) {
  size_t Kp = (size_t)((2 * K + TC_BK - 1) / TC_BK) * TC_BK;
  return 2 * Kp * ((size_t)M + 2 * (size_t)N) + 64;
}

// C[M][N] -= A[M][K] B[K][N], complex FP32, row-major with leading dimensions
// (in complex elements).  passes: 3 (split TF32, FP32-level accuracy) or 1
// (plain TF32).  scratch: gbi_tc_scratch_floats(M, N, K) floats of device
// memory (16-byte aligned), or NULL to allocate on the stream.  err: device
// int raised to 1 if a CTA timed out (may be NULL when the caller does not
// check).
extern "C" int gbi_tc_cgemm_sub(int M, int N, int K, const cplxf* A, size_t lda, const cplxf* B, size_t ldb, cplxf* C,
                                size_t ldc, int passes, float* scratch, int* err, cudaStream_t st) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  if (passes != 1 && passes != 3) {
    gbi_set_error("gbi_tc_cgemm_sub: passes must be 1 or 3");
    return -1;
  }
  const int Kp = ((2 * K + TC_BK - 1) / TC_BK) * TC_BK;
  const size_t need = gbi_tc_scratch_floats(M, N, K);
  float* buf = scratch;
  if (!buf) GB_CUDA(cudaMallocAsync((void**)&buf, need * sizeof(float), st));
  int* e = err;
  if (!e) GB_CUDA(cudaMallocAsync((void**)&e, 16, st));
  if (!err) GB_CUDA(cudaMemsetAsync(e, 0, 4, st));
  float* ahi = buf;
  float* alo = ahi + (size_t)M * Kp;
  float* bhi = alo + (size_t)M * Kp;
  float* blo = bhi + (size_t)2 * N * Kp;
  const bool three = passes == 3;
  size_t ta = (size_t)M * Kp, tb = (size_t)2 * N * Kp;
  const unsigned nba = (unsigned)((ta + 255) / 256), nbb = (unsigned)((tb + 255) / 256);
  k_tc_prep<<<nba + nbb, 256, 0, st>>>(A, lda, M, B, ldb, N, K, Kp, nba, ahi, three ? alo : nullptr, bhi,
                                       three ? blo : nullptr);
  gbi_count_launch();
  GB_CUDA(cudaGetLastError());
  CUtensorMap mAhi, mAlo, mBhi, mBlo;
  int rc = make_map(&mAhi, ahi, M, Kp, TC_BM);
  if (!rc) rc = make_map(&mAlo, alo, M, Kp, TC_BM);
  if (!rc) rc = make_map(&mBhi, bhi, 2 * N, Kp, TC_BN);
  if (!rc) rc = make_map(&mBlo, blo, 2 * N, Kp, TC_BN);
  // C as a 2-D FP32 tensor (rows M, 2N floats each, row stride 2 ldc floats)
  // for the TMA reduce-add epilogue: needs a 16-byte aligned base and stride
  CUtensorMap mC;
  memset(&mC, 0, sizeof(mC));
  int use_tma_c = ((((uintptr_t)C) & 15) == 0) && ((ldc * 8) % 16 == 0);
  if (!rc && use_tma_c) {
    EncodeTiledFn enc = encode_fn();
    cuuint64_t dims[2] = {(cuuint64_t)2 * N, (cuuint64_t)M};
    cuuint64_t strides[1] = {(cuuint64_t)ldc * 8};
    cuuint32_t box[2] = {32, 32};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc ? enc(&mC, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)C, dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE)
                     : CUDA_ERROR_NOT_SUPPORTED;
    if (r != CUDA_SUCCESS) use_tma_c = 0;  // the register epilogue handles it
  }
  if (!rc) {
    int dev = 0, nsm = 0;
    GB_CUDA(cudaGetDevice(&dev));
    GB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long ntiles = (long)((2 * N + TC_BN - 1) / TC_BN) * ((M + TC_BM - 1) / TC_BM);
    dim3 grid((unsigned)(ntiles < nsm ? ntiles : nsm));
    const int nkb = Kp / TC_BK;
    cudaError_t ce;
    KtRec rec;
    bool timing = false;
    {
      std::lock_guard<std::mutex> lk(g_kt_mu);
      timing = g_kt_on;
    }
    if (timing) {
      GB_CUDA(cudaEventCreate(&rec.a));
      GB_CUDA(cudaEventCreate(&rec.b));
      rec.M = M;
      rec.N = N;
      rec.K = K;
      rec.flops = 8.0 * M * (double)N * K;
      rec.bytes = 16.0 * M * (double)N + (three ? 2.0 : 1.0) * 4.0 * ((double)M + 2.0 * N) * Kp;
      GB_CUDA(cudaEventRecord(rec.a, st));
    }
    if (three) {
      GB_CUDA(cudaFuncSetAttribute(k_tc_cgemm_sub<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcLayout<3>::SMEM));
      k_tc_cgemm_sub<3><<<grid, TC_THREADS, TcLayout<3>::SMEM, st>>>(mAhi, mAlo, mBhi, mBlo, mC, use_tma_c, M, 2 * N, nkb, (float*)C,
                                                                      2 * ldc, e);
    } else {
      GB_CUDA(cudaFuncSetAttribute(k_tc_cgemm_sub<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TcLayout<1>::SMEM));
      k_tc_cgemm_sub<1><<<grid, TC_THREADS, TcLayout<1>::SMEM, st>>>(mAhi, mAlo, mBhi, mBlo, mC, use_tma_c, M, 2 * N, nkb, (float*)C,
                                                                      2 * ldc, e);
    }
    gbi_count_launch();
    if (timing) {
      GB_CUDA(cudaEventRecord(rec.b, st));
      std::lock_guard<std::mutex> lk(g_kt_mu);
      g_kt.push_back(rec);
    }
    ce = cudaGetLastError();
    if (ce != cudaSuccess) {
      gbi_set_error("tensor-core GEMM launch: %s", cudaGetErrorString(ce));
      rc = -1;
    }
  }
  if (!scratch) cudaFreeAsync(buf, st);
  if (!err) {
    int h = 0;
    if (!rc && (cudaMemcpyAsync(&h, e, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess)) {
      gbi_set_error("tensor-core GEMM: %s", cudaGetErrorString(cudaGetLastError()));
      rc = -1;
    }
    cudaFreeAsync(e, st);
    if (!rc && h) {
      gbi_set_error("tensor-core GEMM: a pipeline wait timed out");
      rc = -1;
    }
  }
  return rc;
}
