// Complex FP32 products on the fifth-generation tensor cores (tcgen05, kind::tf32), with FP32
// accuracy by the split (3xTF32) product, for sm_103a.
//
// C = alpha A B + beta C, A (m x k), B (k x n), C (m x n) complex64, batched, each addressed by
// (row stride, column stride, batch stride). A complex product is one real product of twice
// the size:
//   [Re C]   [Re A  -Im A] [Re B]
//   [Im C] = [Im A   Re A] [Im B]
// so a CTA's output tile of 64 complex rows by 128 complex columns is one 128 x 128 real MMA
// tile, Re C in accumulator rows 0..63 and Im C in rows 64..127, with K = 16 real per block of
// 8 complex k. Each real operand x is split into x_hi = tf32(x) (round to nearest) and
// x_lo = x - x_hi (exact in FP32), and A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi: three MMAs per
// K chunk into the same FP32 accumulator in tensor memory. The result has an error of a few
// FP32 ulps of sum |a||b|, like an FP32 SIMT product.
//
// Data path per CTA (128 threads): every thread loads its share of the A and B tiles from global
// memory one block ahead into registers, then splits and de-interleaves them into the canonical
// no-swizzle K-major layout in shared memory (double-buffered); one thread issues the MMAs and
// commits them to an mbarrier. The accumulator (128 lanes x 128 columns of tensor memory) is
// read back with tcgen05.ld; with real alpha and beta every lane writes its row's real or
// imaginary parts directly, otherwise the tile goes through shared memory to be combined. Every
// mbarrier wait is bounded: on a timeout the CTA raises g_tc_error, waits (bounded) for its own
// MMAs, frees its tensor memory and returns.
#pragma once
#include <stdint.h>
#include "wb_common.cuh"
#include "wb_num.cuh"

namespace wb {
namespace tc {

constexpr int kThreads = 128;
constexpr int kTileM = 64;          // complex rows per CTA (128 real accumulator rows)
constexpr int kTileN = 128;         // complex columns per CTA (128 accumulator columns)
constexpr int kKb = 8;              // complex k per block (K = 16 real)
constexpr int kPlane = 8192;        // bytes of one 128 x 16 tf32 operand plane
constexpr int kStage = 4 * kPlane;  // A_hi, A_lo, B_hi, B_lo
constexpr int kTmemCols = 128;
constexpr unsigned kSpinLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (row, kk) of a 128 x 16 operand plane: 8-row x 16-byte core matrices,
// K-adjacent cores 128 B apart (LBO), 8-row groups 512 B apart (SBO)
__device__ __forceinline__ uint32_t plane_off(int row, int kk) {
  return (uint32_t)((row & 7) * 16 + (row >> 3) * 512 + (kk & 3) * 4 + (kk >> 2) * 128);
}

// shared-memory matrix descriptor: start address, leading (K) and stride (M/N) byte offsets,
// the fixed version bits of tcgen05 descriptors, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(128u >> 4) << 16;
  d |= (uint64_t)(512u >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: D FP32, A and B TF32, both K-major, N = 128, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTileN >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (unsigned it = 0; it < kSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ unsigned int g_tc_error;

// One CTA: 64 x 128 complex outputs of batch entry blockIdx.z.
__global__ void __launch_bounds__(kThreads) cgemm_kernel(int m, int n, int k, float2 alpha, float2 beta,
                                                         const Cx<float>* __restrict__ A, long long a_rs,
                                                         long long a_cs, long long a_bs,
                                                         const Cx<float>* __restrict__ B, long long b_rs,
                                                         long long b_cs, long long b_bs, Cx<float>* __restrict__ C,
                                                         long long c_rs, long long c_cs, long long c_bs) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int row0 = blockIdx.x * kTileM, col0 = blockIdx.y * kTileN;
  A += blockIdx.z * a_bs;
  B += blockIdx.z * b_bs;
  C += blockIdx.z * c_bs;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    mbar_init(&bars[0]);
    mbar_init(&bars[1]);
    asm volatile("fence.mbarrier_init.release.cluster;");
    s_fail = 0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const int nkb = (k + kKb - 1) / kKb;
  uint32_t issued[2] = {0, 0};        // commits made on each barrier
  bool ok = true;
  // this thread's share of a block: 4 complex of A (64 x 8) and 8 of B (8 x 128), loaded into
  // registers one block ahead so that the global latency overlaps the staging and the MMAs
  constexpr int kAp = kTileM * kKb / kThreads, kBp = kKb * kTileN / kThreads;
  Cx<float> ra[kAp], rb[kBp];
  auto load_block = [&](int k0) {
#pragma unroll
    for (int u = 0; u < kAp; ++u) {
      const int e = tid + u * kThreads, r = e % kTileM, q = e / kTileM;
      ra[u].x = 0.f; ra[u].y = 0.f;
      if (row0 + r < m && k0 + q < k) ra[u] = A[(row0 + r) * a_rs + (k0 + q) * a_cs];
    }
#pragma unroll
    for (int u = 0; u < kBp; ++u) {
      const int e = tid + u * kThreads, q = e % kKb, c = e / kKb;
      rb[u].x = 0.f; rb[u].y = 0.f;
      if (k0 + q < k && col0 + c < n) rb[u] = B[(k0 + q) * b_rs + (col0 + c) * b_cs];
    }
  };
  if (nkb > 0) load_block(0);
  for (int kb = 0; kb < nkb && ok; ++kb) {
    const int buf = kb & 1;
    unsigned char* st = smem + buf * kStage;
    if (kb >= 2 && tid == 0) {        // the MMAs of block kb-2 have read this buffer
      if (!mbar_wait(&bars[buf], (issued[buf] - 1) & 1)) s_fail = 1;
    }
    __syncthreads();
    if (s_fail) { ok = false; break; }
    float* ah = reinterpret_cast<float*>(st);
    float* al = reinterpret_cast<float*>(st + kPlane);
    float* bh = reinterpret_cast<float*>(st + 2 * kPlane);
    float* bl = reinterpret_cast<float*>(st + 3 * kPlane);
    // A: 64 x 8 complex -> the 128 x 16 real expansion, hi and lo planes
#pragma unroll
    for (int u = 0; u < kAp; ++u) {
      const int e = tid + u * kThreads, r = e % kTileM, q = e / kTileM;
      const float re = ra[u].x, im = ra[u].y;
      const float rh = tf32_hi(re), ih = tf32_hi(im);
      const float rl = re - rh, il = im - ih;
      ah[plane_off(r, q) >> 2] = rh;           al[plane_off(r, q) >> 2] = rl;
      ah[plane_off(r, q + 8) >> 2] = -ih;      al[plane_off(r, q + 8) >> 2] = -il;
      ah[plane_off(r + 64, q) >> 2] = ih;      al[plane_off(r + 64, q) >> 2] = il;
      ah[plane_off(r + 64, q + 8) >> 2] = rh;  al[plane_off(r + 64, q + 8) >> 2] = rl;
    }
    // B: 8 x 128 complex -> 16 x 128 real, K-major by column
#pragma unroll
    for (int u = 0; u < kBp; ++u) {
      const int e = tid + u * kThreads, q = e % kKb, c = e / kKb;
      const float re = rb[u].x, im = rb[u].y;
      const float rh = tf32_hi(re), ih = tf32_hi(im);
      bh[plane_off(c, q) >> 2] = rh;      bl[plane_off(c, q) >> 2] = re - rh;
      bh[plane_off(c, q + 8) >> 2] = ih;  bl[plane_off(c, q + 8) >> 2] = im - ih;
    }
    if (kb + 1 < nkb) load_block((kb + 1) * kKb);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t base = smem_u32(st);
#pragma unroll
      for (int j = 0; j < 2; ++j) {                  // the two K = 8 chunks of the block
        const uint64_t dah = sdesc(base + 256 * j), dal = sdesc(base + kPlane + 256 * j);
        const uint64_t dbh = sdesc(base + 2 * kPlane + 256 * j), dbl = sdesc(base + 3 * kPlane + 256 * j);
        mma_tf32(tmem, dah, dbh, (kb > 0 || j > 0) ? 1u : 0u);
        mma_tf32(tmem, dah, dbl, 1u);
        mma_tf32(tmem, dal, dbh, 1u);
      }
      mma_commit(&bars[buf]);
    }
    ++issued[buf];
  }
  // wait for every committed group (bounded), then read the accumulator
  if (tid == 0) {
    for (int b = 0; b < 2; ++b)
      if (issued[b] && !mbar_wait(&bars[b], (issued[b] - 1) & 1)) s_fail = 1;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const bool good = ok && !s_fail && nkb > 0;
  // Real alpha and beta (every use in this library): each lane writes its own row's component
  // straight from tensor memory -- lanes 0..63 the real parts, 64..127 the imaginary parts.
  const bool real_ab = (alpha.y == 0.f && beta.y == 0.f);
  float* Dsm = reinterpret_cast<float*>(smem);      // 128 rows x (kTileN + 1), complex alpha/beta only
  if (good) {
    const int lane_row = warp * 32 + (tid & 31);
    const int gr = row0 + (lane_row & 63), comp = lane_row >> 6;
    const bool zero_beta = (beta.x == 0.f && beta.y == 0.f);
#pragma unroll 1
    for (int c0 = 0; c0 < kTileN; c0 += 16) {
      uint32_t v[16];
      const uint32_t addr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(addr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (real_ab) {
        if (gr < m) {
          float* p0 = reinterpret_cast<float*>(C + gr * c_rs + (col0 + c0) * c_cs) + comp;
          const long long step = 2 * c_cs;           // floats between consecutive columns
          float old[16];
          if (!zero_beta) {                          // all loads first: one latency per 16 outputs
#pragma unroll
            for (int j = 0; j < 16; ++j) old[j] = (col0 + c0 + j < n) ? p0[j * step] : 0.f;
          }
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            if (col0 + c0 + j >= n) break;
            const float d = alpha.x * __uint_as_float(v[j]);
            p0[j * step] = zero_beta ? d : d + beta.x * old[j];
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) Dsm[lane_row * (kTileN + 1) + c0 + j] = __uint_as_float(v[j]);
      }
    }
  } else if (tid == 0) {
    atomicAdd(&g_tc_error, 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  if (!good || real_ab) return;
  const bool zero_beta = (beta.x == 0.f && beta.y == 0.f);
  constexpr int kPer = kTileM * kTileN / kThreads;
  for (int u0 = 0; u0 < kPer; u0 += 8) {              // 8 outputs a thread: loads, then stores
    Cx<float> cv[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + (u0 + u) * kThreads, r = e % kTileM, c = e / kTileM;
      cv[u].x = 0.f; cv[u].y = 0.f;
      if (!zero_beta && row0 + r < m && col0 + c < n) cv[u] = C[(row0 + r) * c_rs + (col0 + c) * c_cs];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int e = tid + (u0 + u) * kThreads, r = e % kTileM, c = e / kTileM;
      const int gr = row0 + r, gc = col0 + c;
      if (gr >= m || gc >= n) continue;
      const float dr = Dsm[r * (kTileN + 1) + c], di = Dsm[(r + 64) * (kTileN + 1) + c];
      Cx<float> o;
      o.x = alpha.x * dr - alpha.y * di + beta.x * cv[u].x - beta.y * cv[u].y;
      o.y = alpha.x * di + alpha.y * dr + beta.x * cv[u].y + beta.y * cv[u].x;
      C[gr * c_rs + gc * c_cs] = o;
    }
  }
}

// dynamic shared memory of a launch: two operand stages, also holding the epilogue's accumulator
// copy (128 x 129 floats)
constexpr size_t kSmemBytes = 2 * kStage > 128 * (kTileN + 1) * 4 ? 2 * kStage : 128 * (kTileN + 1) * 4;

}  // namespace tc
}  // namespace wb
