// Batched dense complex linear algebra for the RCWA path: GEMM, LU with partial pivoting,
// triangular solves with many right-hand sides, transposes, conversions. Every kernel is a
// template over the real type R in {double, float, df64} (wb_num.cuh).
//
// On GB300 the FP64 pipe delivers about 1 TFLOP/s (measured: DFMA 1.0, DMMA m8n8k4 1.05,
// DGEMM 1.05), so the FP64 instantiations are written to keep the FP64 units busy rather than
// to save bandwidth: a 64x64 CTA tile with 4x4 register blocking is far above the arithmetic
// intensity HBM needs. FP64 mma.sync runs at the same rate as DFMA on this part, so plain
// fused multiply-adds are used. The float and df64 instantiations run on the FP32 pipes.
#include <type_traits>
#include "wb_common.cuh"
#include "wb_num.cuh"
#include "wb_kernels.h"

namespace wb {

// ------------------------------------------------------------------------------------- GEMM
// C = alpha * A * B + beta * C for a batch; A (m x k), B (k x n), C (m x n), each addressed by
// (row stride, column stride) so that transposed views need no copies.
constexpr int GT = 64;   // CTA tile
constexpr int GK = 8;    // K step

// CA / CB: the operand's elements are conjugated on load (op(A) = conj(A) under the given
// strides, so a (rs, cs) swap with CA gives A^H).
template <class R, bool CA = false, bool CB = false>
__global__ void __launch_bounds__(256) gemm_kernel(
    int m, int n, int k, double2 alpha_d,
    const Cx<R>* __restrict__ A, long long a_rs, long long a_cs, long long a_bs,
    const Cx<R>* __restrict__ B, long long b_rs, long long b_cs, long long b_bs,
    double2 beta_d, Cx<R>* __restrict__ C, long long c_rs, long long c_cs, long long c_bs,
    const int* __restrict__ a_idx) {
  using C_ = Cx<R>;
  __shared__ C_ sA[GK][GT + 1];
  __shared__ C_ sB[GK][GT + 1];
  const int bz = blockIdx.z;
  A += (a_idx ? (long long)a_idx[bz] : (long long)bz) * a_bs; B += bz * b_bs; C += bz * c_bs;
  const int row0 = blockIdx.x * GT, col0 = blockIdx.y * GT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  C_ acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cxzero<R>();
  for (int k0 = 0; k0 < k; k0 += GK) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % GT, c = idx / GT;
      int gr = row0 + r, gc = k0 + c;
      C_ v = (gr < m && gc < k) ? A[gr * a_rs + gc * a_cs] : cxzero<R>();
      sA[c][r] = CA ? cxconj(v) : v;
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % GK, c = idx / GK;
      int gr = k0 + r, gc = col0 + c;
      C_ v = (gr < k && gc < n) ? B[gr * b_rs + gc * b_cs] : cxzero<R>();
      sB[r][c] = CB ? cxconj(v) : v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      C_ a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cxfma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const C_ alpha = cxfrom<R>(alpha_d), beta = cxfrom<R>(beta_d);
  const bool zero_beta = (beta_d.x == 0.0 && beta_d.y == 0.0);
  C_ old[4][4];
  if (!zero_beta) {                 // every load before any store: one latency, not sixteen
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int gr = row0 + tx + 16 * i, gc = col0 + ty + 16 * j;
        old[i][j] = (gr < m && gc < n) ? C[gr * c_rs + gc * c_cs] : cxzero<R>();
      }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gr = row0 + tx + 16 * i;
    if (gr >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gc = col0 + ty + 16 * j;
      if (gc >= n) continue;
      C_ v = alpha * acc[i][j];
      if (!zero_beta) v = cxfma(beta, old[i][j], v);
      C[gr * c_rs + gc * c_cs] = v;
    }
  }
}

// Narrow products (C with at most 8 columns: right-hand-side blocks, residual products). One
// output row per thread: every A element is loaded once, coalesced down its column, and used for
// all NC columns of B, which sit in shared memory. The square-tile kernel above would spend most
// of its 64-column tile on zeros here.
constexpr int NW_ROWS = 128;
template <class R, int NC>
__global__ void __launch_bounds__(NW_ROWS) gemm_narrow_kernel(
    int m, int nc, int k, double2 alpha_d, const Cx<R>* __restrict__ A, long long lda, long long a_bs,
    const Cx<R>* __restrict__ B, long long ldb, long long b_bs, double2 beta_d, Cx<R>* __restrict__ C,
    long long ldc, long long c_bs) {
  using C_ = Cx<R>;
  __shared__ C_ sB[32][NC];
  const long long bz = blockIdx.y;
  A += bz * a_bs; B += bz * b_bs; C += bz * c_bs;
  const int row = blockIdx.x * NW_ROWS + threadIdx.x;
  C_ acc[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc[c] = cxzero<R>();
  for (int k0 = 0; k0 < k; k0 += 32) {
    __syncthreads();
    for (int e = threadIdx.x; e < 32 * NC; e += NW_ROWS) {
      const int kk = e % 32, c = e / 32;
      sB[kk][c] = (k0 + kk < k && c < nc) ? B[(k0 + kk) + (long long)c * ldb] : cxzero<R>();
    }
    __syncthreads();
    if (row < m) {
      const int kend = min(32, k - k0);
      for (int kk = 0; kk < kend; ++kk) {
        const C_ a = A[row + (long long)(k0 + kk) * lda];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = cxfma(a, sB[kk][c], acc[c]);
      }
    }
  }
  if (row >= m) return;
  const C_ alpha = cxfrom<R>(alpha_d), beta = cxfrom<R>(beta_d);
  const bool zero_beta = (beta_d.x == 0.0 && beta_d.y == 0.0);
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    if (c >= nc) break;
    C_* p = C + row + (long long)c * ldc;
    *p = zero_beta ? alpha * acc[c] : alpha * acc[c] + beta * *p;
  }
}

template <class R>
void gemm(cudaStream_t s, int batch, int m, int n, int k, double2 alpha,
          const Cx<R>* A, long long a_rs, long long a_cs, long long a_bs,
          const Cx<R>* B, long long b_rs, long long b_cs, long long b_bs,
          double2 beta, Cx<R>* C, long long c_rs, long long c_cs, long long c_bs) {
  if (batch <= 0 || m <= 0 || n <= 0) return;
  if constexpr (sizeof(R) == 4) {      // FP32: the tensor cores (3xTF32) for all but small products
    if (tc_cgemm(s, batch, m, n, k, alpha, (const Cx<float>*)A, a_rs, a_cs, a_bs, (const Cx<float>*)B, b_rs, b_cs,
                 b_bs, beta, (Cx<float>*)C, c_rs, c_cs, c_bs))
      return;
  }
  if (n <= 8 && k > 0 && a_rs == 1 && b_rs == 1 && c_rs == 1) {
    dim3 g((m + NW_ROWS - 1) / NW_ROWS, batch);
    if (n <= 3)
      gemm_narrow_kernel<R, 3><<<g, NW_ROWS, 0, s>>>(m, n, k, alpha, A, a_cs, a_bs, B, b_cs, b_bs, beta, C, c_cs, c_bs);
    else if (n <= 6)
      gemm_narrow_kernel<R, 6><<<g, NW_ROWS, 0, s>>>(m, n, k, alpha, A, a_cs, a_bs, B, b_cs, b_bs, beta, C, c_cs, c_bs);
    else
      gemm_narrow_kernel<R, 8><<<g, NW_ROWS, 0, s>>>(m, n, k, alpha, A, a_cs, a_bs, B, b_cs, b_bs, beta, C, c_cs, c_bs);
    note_launch();
    return;
  }
  dim3 grid((m + GT - 1) / GT, (n + GT - 1) / GT, batch);
  gemm_kernel<R><<<grid, 256, 0, s>>>(m, n, k, alpha, A, a_rs, a_cs, a_bs, B, b_rs, b_cs, b_bs, beta, C, c_rs,
                                      c_cs, c_bs, nullptr); note_launch();
}

// As gemm, with the A operand of batch entry z at A + a_idx[z] * a_bs (a table of operands
// shared by several entries, e.g. one convolution slot per layer for every solve).
template <class R>
void gemm_idx(cudaStream_t s, int batch, int m, int n, int k, double2 alpha,
              const Cx<R>* A, long long a_rs, long long a_cs, long long a_bs, const int* a_idx,
              const Cx<R>* B, long long b_rs, long long b_cs, long long b_bs,
              double2 beta, Cx<R>* C, long long c_rs, long long c_cs, long long c_bs) {
  if (batch <= 0 || m <= 0 || n <= 0) return;
  dim3 grid((m + GT - 1) / GT, (n + GT - 1) / GT, batch);
  gemm_kernel<R><<<grid, 256, 0, s>>>(m, n, k, alpha, A, a_rs, a_cs, a_bs, B, b_rs, b_cs, b_bs, beta, C, c_rs,
                                      c_cs, c_bs, a_idx); note_launch();
}

// ------------------------------------------------- FP64 products accumulated in double-float
// C = alpha A B + beta C for FP64 (complex128) operands, with the products and sums carried in
// double-float arithmetic on the FP32 pipes instead of the FP64 ones: each operand is split on
// load into hi + lo FP32 words (48 significant bits), and each real product-accumulate is
//   p = ah bh (rounded), e = fma(ah, bh, -p) + ah bl + al bh       (Dekker's product; al bl dropped)
//   hi + err = hi + p exactly (Knuth's two-sum),  lo += err + e
// with one renormalisation of (hi, lo) per K tile. About 12 FP32 instructions per real
// multiply-add against one FP64 instruction, on pipes 64x wider on GB300: about 5x the DFMA rate
// at a unit roundoff of about 2^-48 (the error grows like K 2^-48 of sum |a||b| in the worst case).
// Used by the mixed form for the products whose results must be FP64-accurate (the Newton
// residual Omega^2 W and V = Omega_R W), never by the plain FP64 form.
namespace {
struct DD { float hi, lo; };
__device__ __forceinline__ void dd_mac(DD& acc, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  const float s = __fadd_rn(acc.hi, p);
  const float bb = __fsub_rn(s, acc.hi);
  const float err = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(err, e));
}
__device__ __forceinline__ void dd_norm(DD& a) {
  const float s = __fadd_rn(a.hi, a.lo);
  a.lo = __fsub_rn(a.lo, __fsub_rn(s, a.hi));
  a.hi = s;
}
// (re.hi, re.lo, im.hi, im.lo) of an FP64 complex value
__device__ __forceinline__ float4 dd_split(double2 v) {
  const float rh = (float)v.x, ih = (float)v.y;
  return make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
}
}  // namespace

__global__ void __launch_bounds__(256) gemm_dd_kernel(
    int m, int n, int k, double2 alpha, const double2* __restrict__ A, long long a_rs, long long a_cs,
    long long a_bs, const int* __restrict__ a_idx, const double2* __restrict__ B, long long b_rs, long long b_cs,
    long long b_bs, double2 beta, double2* __restrict__ C, long long c_rs, long long c_cs, long long c_bs) {
  __shared__ float4 sA[GK][GT + 1];
  __shared__ float4 sB[GK][GT + 1];
  const int bz = blockIdx.z;
  A += (a_idx ? (long long)a_idx[bz] : (long long)bz) * a_bs; B += bz * b_bs; C += bz * c_bs;
  const int row0 = blockIdx.x * GT, col0 = blockIdx.y * GT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  DD re[4][4], im[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { re[i][j] = DD{0.f, 0.f}; im[i][j] = DD{0.f, 0.f}; }
  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int k0 = 0; k0 < k; k0 += GK) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int idx = tid + e * 256;
      const int r = idx % GT, c = idx / GT;
      const int gr = row0 + r, gc = k0 + c;
      sA[c][r] = (gr < m && gc < k) ? dd_split(A[gr * a_rs + gc * a_cs]) : zero4;
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int idx = tid + e * 256;
      const int r = idx % GK, c = idx / GK;
      const int gr = k0 + r, gc = col0 + c;
      sB[r][c] = (gr < k && gc < n) ? dd_split(B[gr * b_rs + gc * b_cs]) : zero4;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float4 a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // (ar + i ai)(br + i bi): re += ar br - ai bi, im += ar bi + ai br
          dd_mac(re[i][j], a[i].x, a[i].y, b[j].x, b[j].y);
          dd_mac(re[i][j], -a[i].z, -a[i].w, b[j].z, b[j].w);
          dd_mac(im[i][j], a[i].x, a[i].y, b[j].z, b[j].w);
          dd_mac(im[i][j], a[i].z, a[i].w, b[j].x, b[j].y);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) { dd_norm(re[i][j]); dd_norm(im[i][j]); }
    __syncthreads();
  }
  const bool zero_beta = (beta.x == 0.0 && beta.y == 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = row0 + tx + 16 * i;
    if (gr >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gc = col0 + ty + 16 * j;
      if (gc >= n) continue;
      double2* p = C + gr * c_rs + gc * c_cs;
      const double2 v = make_double2((double)re[i][j].hi + (double)re[i][j].lo,
                                     (double)im[i][j].hi + (double)im[i][j].lo);
      double2 o = make_double2(alpha.x * v.x - alpha.y * v.y, alpha.x * v.y + alpha.y * v.x);
      if (!zero_beta) {
        const double2 c = *p;
        o.x += beta.x * c.x - beta.y * c.y;
        o.y += beta.x * c.y + beta.y * c.x;
      }
      *p = o;
    }
  }
}

void zgemm_dd_idx(cudaStream_t s, int batch, int m, int n, int k, double2 alpha, const cplx* A, long long a_rs,
                  long long a_cs, long long a_bs, const int* a_idx, const cplx* B, long long b_rs, long long b_cs,
                  long long b_bs, double2 beta, cplx* C, long long c_rs, long long c_cs, long long c_bs) {
  if (batch <= 0 || m <= 0 || n <= 0) return;
  dim3 grid((m + GT - 1) / GT, (n + GT - 1) / GT, batch);
  gemm_dd_kernel<<<grid, 256, 0, s>>>(m, n, k, alpha, A, a_rs, a_cs, a_bs, a_idx, B, b_rs, b_cs, b_bs, beta, C,
                                      c_rs, c_cs, c_bs);
  note_launch();
}

// ----------------------------------------------------------------------- LU factorisation
// One CTA per matrix, right-looking, panel width LU_NB. Pivot choice is the largest |re|+|im|
// in the column (the LAPACK izamax measure). Row swaps are applied across the full width.
constexpr int LU_NB = 16;
constexpr int LU_THREADS = 256;

template <class R>
__device__ void block_argmax(R v, int idx, R* sval, int* sidx, R& out_v, int& out_i) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  // warp stage through shared memory (R may be a two-word type)
  __shared__ int s_lane_idx[LU_THREADS];
  sval[threadIdx.x] = v;
  s_lane_idx[threadIdx.x] = idx;
  __syncthreads();
  if (lane == 0) {
    R bv = sval[threadIdx.x]; int bi = s_lane_idx[threadIdx.x];
    for (int l = 1; l < 32; ++l) {
      R ov = sval[threadIdx.x + l]; int oi = s_lane_idx[threadIdx.x + l];
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    sval[threadIdx.x] = bv; s_lane_idx[threadIdx.x] = bi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    R bv = sval[0]; int bi = s_lane_idx[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      R ov = sval[w * 32]; int oi = s_lane_idx[w * 32];
      if (ov > bv || (ov == bv && oi < bi)) { bv = ov; bi = oi; }
    }
    sval[0] = bv; sidx[0] = bi;
  }
  __syncthreads();
  out_v = sval[0]; out_i = sidx[0];
  __syncthreads();
  (void)warp;
}

template <class R>
__global__ void __launch_bounds__(LU_THREADS) getrf_kernel(
    Cx<R>* __restrict__ Aall, int n, int lda, long long a_bs, int* __restrict__ ipiv_all, long long piv_bs,
    int32_t* __restrict__ status, int st_div) {
  using C_ = Cx<R>;
  __shared__ R sval[LU_THREADS];
  __shared__ int sidx[1];
  __shared__ C_ sL[GT][LU_NB + 1];
  __shared__ C_ sU[LU_NB][GT + 1];
  C_* A = Aall + blockIdx.x * a_bs;
  int* ipiv = ipiv_all + (long long)blockIdx.x * piv_bs;
  int32_t* st = status ? status + blockIdx.x / st_div : nullptr;
  const int tid = threadIdx.x;
  for (int k0 = 0; k0 < n; k0 += LU_NB) {
    const int kb = min(LU_NB, n - k0);
    for (int j = k0; j < k0 + kb; ++j) {
      R best = R(-1.0); int bi = j;
      for (int i = j + tid; i < n; i += blockDim.x) {
        R v = cxabs1(A[i + (long long)j * lda]);
        if (v > best) { best = v; bi = i; }
      }
      R pv; int p;
      block_argmax<R>(best, bi, sval, sidx, pv, p);
      if (tid == 0) ipiv[j] = p;
      if (p != j) {
        for (int c = tid; c < n; c += blockDim.x) {
          C_ t = A[j + (long long)c * lda];
          A[j + (long long)c * lda] = A[p + (long long)c * lda];
          A[p + (long long)c * lda] = t;
        }
      }
      __syncthreads();
      C_ piv = A[j + (long long)j * lda];
      if (piv.x == R(0.0) && piv.y == R(0.0)) {
        if (tid == 0) wb_flag(st, WB_ST_SINGULAR);
        __syncthreads();
        continue;
      }
      C_ rp = cxinv(piv);
      for (int i = j + 1 + tid; i < n; i += blockDim.x) {
        C_ l = A[i + (long long)j * lda] * rp;
        A[i + (long long)j * lda] = l;
        for (int c = j + 1; c < k0 + kb; ++c)
          A[i + (long long)c * lda] = A[i + (long long)c * lda] - l * A[j + (long long)c * lda];
      }
      __syncthreads();
    }
    const int c0 = k0 + kb;
    if (c0 >= n) break;
    for (int c = c0 + tid; c < n; c += blockDim.x) {
      for (int r = k0 + 1; r < k0 + kb; ++r) {
        C_ acc = A[r + (long long)c * lda];
        for (int t = k0; t < r; ++t) acc = acc - A[r + (long long)t * lda] * A[t + (long long)c * lda];
        A[r + (long long)c * lda] = acc;
      }
    }
    __syncthreads();
    const int tx = tid & 15, ty = tid >> 4;
    for (int cc = c0; cc < n; cc += GT) {
      for (int e = tid; e < LU_NB * GT; e += blockDim.x) {
        int r = e % LU_NB, c = e / LU_NB;
        sU[r][c] = (r < kb && cc + c < n) ? A[k0 + r + (long long)(cc + c) * lda] : cxzero<R>();
      }
      for (int rr = c0; rr < n; rr += GT) {
        for (int e = tid; e < LU_NB * GT; e += blockDim.x) {
          int r = e % GT, c = e / GT;
          sL[r][c] = (c < kb && rr + r < n) ? A[rr + r + (long long)(k0 + c) * lda] : cxzero<R>();
        }
        __syncthreads();
        C_ acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[i][q] = cxzero<R>();
        for (int kk = 0; kk < kb; ++kk) {
          C_ a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = sL[tx + 16 * i][kk];
#pragma unroll
          for (int q = 0; q < 4; ++q) b[q] = sU[kk][ty + 16 * q];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = cxfma(a[i], b[q], acc[i][q]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          int gr = rr + tx + 16 * i;
          if (gr >= n) continue;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int gc = cc + ty + 16 * q;
            if (gc >= n) continue;
            C_* p = A + gr + (long long)gc * lda;
            *p = *p - acc[i][q];
          }
        }
        __syncthreads();
      }
    }
  }
}

// ------------------------------------------------ LU across the GPU for small batches
// When a batch holds fewer matrices than the GPU has room for (the cascade factors one layer of
// every solve at a time), one CTA per matrix leaves most SMs idle. The blocked right-looking LU
// then runs as three launches per panel of LU_PB columns:
//   lu_panel_kernel      one CTA per matrix: partial pivoting down the panel, swaps inside it
//   lu_swap_trsm_kernel  one thread per column outside the panel: the panel's row swaps, then
//                        U12 = L11^-1 A12 for the trailing columns
//   lu_update_kernel     A22 -= L21 U12 in 64 x 64 tiles over every SM
// The pivots are the single-CTA kernel's (largest |re| + |im|, first index on ties).
constexpr int LU_PB = 32;            // panel width
constexpr int LU_PANEL_THREADS = 1024;

namespace {
__device__ __forceinline__ double lu_shfl_down(double v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ float lu_shfl_down(float v, int o) { return __shfl_down_sync(0xffffffffu, v, o); }
__device__ __forceinline__ df64 lu_shfl_down(df64 v, int o) {
  return df64(__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o));
}
__device__ __forceinline__ double lu_shfl(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float lu_shfl(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ df64 lu_shfl(df64 v, int src) {
  return df64(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
// (value, index) maximum over the block; ties go to the smaller index
template <class R>
__device__ void lu_block_argmax(R v, int idx, R* wv, int* wi, R& out_v, int& out_i) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R ov = lu_shfl_down(v, o);
    int oi = __shfl_down_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  if (lane == 0) { wv[warp] = v; wi[warp] = idx; }
  __syncthreads();
  if (warp == 0) {
    v = lane < nw ? wv[lane] : R(-1.0);
    idx = lane < nw ? wi[lane] : 0x7fffffff;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      R ov = lu_shfl_down(v, o);
      int oi = __shfl_down_sync(0xffffffffu, idx, o);
      if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
    }
    if (lane == 0) { wv[0] = v; wi[0] = idx; }
  }
  __syncthreads();
  out_v = wv[0]; out_i = wi[0];
  __syncthreads();
}
}  // namespace

template <class R>
__global__ void __launch_bounds__(LU_PANEL_THREADS) lu_panel_kernel(
    Cx<R>* __restrict__ Aall, int n, int lda, long long a_bs, int* __restrict__ ipiv_all, long long piv_bs,
    int32_t* __restrict__ status, int st_div, int k0, int kb) {
  using C_ = Cx<R>;
  __shared__ R wv[32];
  __shared__ int wi[32];
  __shared__ C_ prow[LU_PB];
  C_* A = Aall + blockIdx.x * a_bs;
  int* ipiv = ipiv_all + (long long)blockIdx.x * piv_bs;
  int32_t* st = status ? status + blockIdx.x / st_div : nullptr;
  const int tid = threadIdx.x;
  auto a = [&](int i, int j) -> C_& { return A[i + (long long)j * lda]; };
  for (int j = k0; j < k0 + kb; ++j) {
    R best = R(-1.0); int bi = j;
    for (int i = j + tid; i < n; i += blockDim.x) {
      const R v = cxabs1(a(i, j));
      if (v > best) { best = v; bi = i; }
    }
    R pv; int p;
    lu_block_argmax<R>(best, bi, wv, wi, pv, p);
    if (tid == 0) ipiv[j] = p;
    // swap rows j, p inside the panel; the pivot row to shared memory
    if (tid < kb) {
      const int c = k0 + tid;
      C_ x = a(j, c), y = a(p, c);
      if (p != j) { a(j, c) = y; a(p, c) = x; }
      prow[tid] = (p != j) ? y : x;
    }
    __syncthreads();
    const C_ piv = prow[j - k0];
    if (piv.x == R(0.0) && piv.y == R(0.0)) {
      if (tid == 0) wb_flag(st, WB_ST_SINGULAR);
      continue;
    }
    const C_ rp = cxinv(piv);
    const int ce = k0 + kb;
    for (int i = j + 1 + tid; i < n; i += blockDim.x) {
      const C_ l = a(i, j) * rp;
      a(i, j) = l;
      for (int c0 = j + 1; c0 < ce; c0 += 8) {
        C_ v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (c0 + u < ce) v[u] = a(i, c0 + u);
#pragma unroll
        for (int u = 0; u < 8; ++u)
          if (c0 + u < ce) a(i, c0 + u) = v[u] - l * prow[c0 + u - k0];
      }
    }
    __syncthreads();
  }
}

// One thread per column c outside the panel [k0, k0 + kb): the panel's row swaps in order, and
// for trailing columns U12 = L11^-1 A12 (L11 unit lower, from shared memory).
template <class R>
__global__ void __launch_bounds__(256) lu_swap_trsm_kernel(Cx<R>* __restrict__ Aall, int n, int lda, long long a_bs,
                                                           const int* __restrict__ ipiv_all, long long piv_bs, int k0,
                                                           int kb) {
  using C_ = Cx<R>;
  __shared__ C_ sL[LU_PB][LU_PB + 1];
  __shared__ int sp[LU_PB];
  C_* A = Aall + blockIdx.y * a_bs;
  const int* ipiv = ipiv_all + (long long)blockIdx.y * piv_bs;
  const int tid = threadIdx.x;
  for (int e = tid; e < kb * kb; e += blockDim.x) {
    const int r = e % kb, c = e / kb;
    sL[r][c] = A[k0 + r + (long long)(k0 + c) * lda];
  }
  if (tid < kb) sp[tid] = ipiv[k0 + tid];
  __syncthreads();
  int c = blockIdx.x * blockDim.x + tid;
  if (c >= n - kb) return;
  if (c >= k0) c += kb;                      // skip the panel
  C_* col = A + (long long)c * lda;
  for (int j = 0; j < kb; ++j) {
    const int p = sp[j];
    if (p != k0 + j) {
      const C_ x = col[k0 + j], y = col[p];
      col[k0 + j] = y; col[p] = x;
    }
  }
  if (c < k0) return;
  C_ x[LU_PB];
#pragma unroll
  for (int r = 0; r < LU_PB; ++r)
    if (r < kb) x[r] = col[k0 + r];
#pragma unroll
  for (int r = 1; r < LU_PB; ++r) {
    if (r >= kb) break;
    C_ acc = x[r];
#pragma unroll
    for (int t = 0; t < LU_PB; ++t)
      if (t < r) acc = acc - sL[r][t] * x[t];
    x[r] = acc;
  }
#pragma unroll
  for (int r = 1; r < LU_PB; ++r)
    if (r < kb) col[k0 + r] = x[r];
}

// A22 -= L21 U12 on rows and columns [c0, n), K = kb <= LU_PB
template <class R>
__global__ void __launch_bounds__(256) lu_update_kernel(Cx<R>* __restrict__ Aall, int n, int lda, long long a_bs,
                                                        int k0, int kb) {
  using C_ = Cx<R>;
  constexpr int KC = 16;                       // K chunk held in shared memory
  __shared__ C_ sL[KC][GT + 1];
  __shared__ C_ sU[KC][GT + 1];
  C_* A = Aall + blockIdx.z * a_bs;
  const int c0 = k0 + kb;
  const int row0 = c0 + blockIdx.x * GT, col0 = c0 + blockIdx.y * GT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  C_ acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cxzero<R>();
  for (int q0 = 0; q0 < kb; q0 += KC) {
    if (q0 > 0) __syncthreads();
    for (int e = tid; e < GT * KC; e += blockDim.x) {
      const int r = e % GT, k = e / GT;
      sL[k][r] = (q0 + k < kb && row0 + r < n) ? A[row0 + r + (long long)(k0 + q0 + k) * lda] : cxzero<R>();
    }
    for (int e = tid; e < GT * KC; e += blockDim.x) {
      const int k = e % KC, c = e / KC;
      sU[k][c] = (q0 + k < kb && col0 + c < n) ? A[k0 + q0 + k + (long long)(col0 + c) * lda] : cxzero<R>();
    }
    __syncthreads();
    const int kend = min(KC, kb - q0);
    for (int kk = 0; kk < kend; ++kk) {
      C_ a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sL[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sU[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cxfma(a[i], b[j], acc[i][j]);
    }
  }
  C_ old[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gr = row0 + tx + 16 * i, gc = col0 + ty + 16 * j;
      if (gr < n && gc < n) old[i][j] = A[gr + (long long)gc * lda];
    }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gr = row0 + tx + 16 * i, gc = col0 + ty + 16 * j;
      if (gr < n && gc < n) A[gr + (long long)gc * lda] = old[i][j] - acc[i][j];
    }
}

template <class R>
void getrf(cudaStream_t s, int batch, int n, Cx<R>* A, int lda, long long a_bs, int* ipiv, long long piv_bs,
           int32_t* status, int st_div) {
  if (batch <= 0 || n <= 0) return;
  st_div = st_div < 1 ? 1 : st_div;
  if (batch >= 2 * sm_count() || n < 2 * LU_PB) {
    getrf_kernel<R><<<batch, LU_THREADS, 0, s>>>(A, n, lda, a_bs, ipiv, piv_bs, status, st_div);
    note_launch();
    return;
  }
  for (int k0 = 0; k0 < n; k0 += LU_PB) {
    const int kb = min(LU_PB, n - k0);
    lu_panel_kernel<R><<<batch, LU_PANEL_THREADS, 0, s>>>(A, n, lda, a_bs, ipiv, piv_bs, status, st_div, k0, kb);
    note_launch();
    if (n - kb > 0) {
      dim3 g2((n - kb + 255) / 256, batch);
      lu_swap_trsm_kernel<R><<<g2, 256, 0, s>>>(A, n, lda, a_bs, ipiv, piv_bs, k0, kb);
      note_launch();
    }
    const int m = n - k0 - kb;
    if (m > 0) {
      dim3 g3((m + GT - 1) / GT, (m + GT - 1) / GT, batch);
      lu_update_kernel<R><<<g3, 256, 0, s>>>(A, n, lda, a_bs, k0, kb);
      note_launch();
    }
  }
}

// --------------------------------------------------------------------- triangular solves
// X = op(A)^{-1} B with A = P L U from getrf; B (n x nrhs, column-major, ldb) is overwritten.
// trans = 0: A X = B.  trans = 1: A^T X = B.  Each CTA owns SV_W right-hand sides of one
// matrix and runs blocked substitution with K = SV_NB register-tiled updates.
constexpr int SV_W = 64;
constexpr int SV_NB = 16;

template <class R>
__global__ void __launch_bounds__(256) getrs_kernel(
    const Cx<R>* __restrict__ LUall, int n, int lda, long long a_bs, const int* __restrict__ ipiv_all,
    long long piv_bs, Cx<R>* __restrict__ Ball, int nrhs, int ldb, long long b_bs, int trans) {
  using C_ = Cx<R>;
  __shared__ C_ sT[SV_NB][SV_NB + 1];
  __shared__ C_ sX[SV_NB][SV_W + 1];
  __shared__ C_ sM[GT][SV_NB + 1];
  const C_* LU = LUall + blockIdx.y * a_bs;
  const int* ipiv = ipiv_all + (long long)blockIdx.y * piv_bs;
  C_* B = Ball + blockIdx.y * b_bs;
  const int r0 = blockIdx.x * SV_W;
  const int w = min(SV_W, nrhs - r0);
  if (w <= 0) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  auto Bat = [&](int i, int c) -> C_& { return B[i + (long long)(r0 + c) * ldb]; };
  auto Lat = [&](int i, int j) -> C_ { return LU[i + (long long)j * lda]; };
  if (trans == 0) {
    for (int j = 0; j < n; ++j) {
      int p = ipiv[j];
      if (p != j)
        for (int c = tid; c < w; c += blockDim.x) { C_ t = Bat(j, c); Bat(j, c) = Bat(p, c); Bat(p, c) = t; }
      __syncthreads();
    }
  }
  for (int sweep = 0; sweep < 2; ++sweep) {
    const bool forward = (sweep == 0);
    // trans 0: fwd uses L (unit, A(i,j) i>j), bwd uses U (A(i,j) i<=j)
    // trans 1: fwd uses U^T: (i,j) i>=j is A(j,i), non-unit; bwd uses L^T: (i,j) i<j is A(j,i), unit
    const bool unit = (trans == 0) ? forward : !forward;
    const int nblk = (n + SV_NB - 1) / SV_NB;
    for (int bi = 0; bi < nblk; ++bi) {
      const int blk = forward ? bi : (nblk - 1 - bi);
      const int i0 = blk * SV_NB, ib = min(SV_NB, n - i0);
      for (int e = tid; e < SV_NB * SV_NB; e += blockDim.x) {
        int r = e % SV_NB, c = e / SV_NB;
        C_ v = cxzero<R>();
        if (r < ib && c < ib) v = (trans == 0) ? Lat(i0 + r, i0 + c) : Lat(i0 + c, i0 + r);
        sT[r][c] = v;
      }
      for (int e = tid; e < SV_NB * SV_W; e += blockDim.x) {
        int r = e % SV_NB, c = e / SV_NB;
        sX[r][c] = (r < ib && c < w) ? Bat(i0 + r, c) : cxzero<R>();
      }
      __syncthreads();
      if (tid < w) {
        const int c = tid;
        if (forward) {
          for (int r = 0; r < ib; ++r) {
            C_ acc = sX[r][c];
            for (int t = 0; t < r; ++t) acc = acc - sT[r][t] * sX[t][c];
            if (!unit) acc = cxdiv(acc, sT[r][r]);
            sX[r][c] = acc;
          }
        } else {
          for (int r = ib - 1; r >= 0; --r) {
            C_ acc = sX[r][c];
            for (int t = r + 1; t < ib; ++t) acc = acc - sT[r][t] * sX[t][c];
            if (!unit) acc = cxdiv(acc, sT[r][r]);
            sX[r][c] = acc;
          }
        }
      }
      __syncthreads();
      for (int e = tid; e < SV_NB * SV_W; e += blockDim.x) {
        int r = e % SV_NB, c = e / SV_NB;
        if (r < ib && c < w) Bat(i0 + r, c) = sX[r][c];
      }
      const int rs = forward ? i0 + ib : 0;
      const int re = forward ? n : i0;
      for (int rr = rs; rr < re; rr += GT) {
        for (int e = tid; e < GT * SV_NB; e += blockDim.x) {
          int r = e % GT, c = e / GT;
          int gr = rr + r;
          C_ v = cxzero<R>();
          if (gr < re && c < ib) v = (trans == 0) ? Lat(gr, i0 + c) : Lat(i0 + c, gr);
          sM[r][c] = v;
        }
        __syncthreads();
        C_ acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[i][q] = cxzero<R>();
        for (int kk = 0; kk < ib; ++kk) {
          C_ a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = sM[tx + 16 * i][kk];
#pragma unroll
          for (int q = 0; q < 4; ++q) b[q] = sX[kk][ty + 16 * q];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = cxfma(a[i], b[q], acc[i][q]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          int gr = rr + tx + 16 * i;
          if (gr >= re) continue;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int c = ty + 16 * q;
            if (c >= w) continue;
            Bat(gr, c) = Bat(gr, c) - acc[i][q];
          }
        }
        __syncthreads();
      }
      __syncthreads();
    }
  }
  if (trans == 1) {
    for (int j = n - 1; j >= 0; --j) {
      int p = ipiv[j];
      if (p != j)
        for (int c = tid; c < w; c += blockDim.x) { C_ t = Bat(j, c); Bat(j, c) = Bat(p, c); Bat(p, c) = t; }
      __syncthreads();
    }
  }
}

// Few right-hand sides (the cascade's incidence columns): one CTA per matrix holds X = B
// (n x NC) in shared memory and substitutes 32 rows at a time. Per block: the 32 x 32 diagonal
// block is staged in shared memory, warp 0 solves it with the block's rows in its lanes
// (shuffles carry each solved row to the others), then every thread takes rows below (above,
// going back) and subtracts the block's contribution, reading L (U) down its columns, coalesced.
constexpr int NS_B = 32;
constexpr int NS_THREADS = 1024;

template <class R, int NC>
__global__ void __launch_bounds__(NS_THREADS) getrs_narrow_kernel(
    const Cx<R>* __restrict__ LUall, int n, int lda, long long a_bs, const int* __restrict__ ipiv_all,
    long long piv_bs, Cx<R>* __restrict__ Ball, int nrhs, int ldb, long long b_bs) {
  using C_ = Cx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C_* X = reinterpret_cast<C_*>(smraw);            // (n, NC), row-major
  __shared__ C_ sD[NS_B][NS_B + 1];
  const C_* LU = LUall + blockIdx.x * a_bs;
  const int* ipiv = ipiv_all + (long long)blockIdx.x * piv_bs;
  C_* B = Ball + blockIdx.x * b_bs;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < n * NC; e += blockDim.x) {
    const int r = e % n, c = e / n;
    X[r * NC + c] = (c < nrhs) ? B[r + (long long)c * ldb] : cxzero<R>();
  }
  __syncthreads();
  if (tid < nrhs) {                                // the row swaps, in order, one column each
    for (int j = 0; j < n; ++j) {
      const int p = ipiv[j];
      if (p != j) { const C_ t = X[j * NC + tid]; X[j * NC + tid] = X[p * NC + tid]; X[p * NC + tid] = t; }
    }
  }
  for (int sweep = 0; sweep < 2; ++sweep) {
    const bool fwd = sweep == 0;                   // L (unit lower), then U (upper)
    const int nblk = (n + NS_B - 1) / NS_B;
    for (int bi = 0; bi < nblk; ++bi) {
      const int i0 = fwd ? bi * NS_B : max(0, n - (bi + 1) * NS_B);
      const int ib = fwd ? min(NS_B, n - i0) : (n - bi * NS_B) - i0;
      __syncthreads();
      for (int e = tid; e < NS_B * NS_B; e += blockDim.x) {
        const int r = e % NS_B, c = e / NS_B;
        sD[r][c] = (r < ib && c < ib) ? LU[i0 + r + (long long)(i0 + c) * lda] : cxzero<R>();
      }
      __syncthreads();
      if (warp == 0) {
        C_ x[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) x[c] = lane < ib ? X[(i0 + lane) * NC + c] : cxzero<R>();
        if (fwd) {
          for (int t = 0; t < ib; ++t) {
            const C_ l = sD[lane][t];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
              C_ xt;
              xt.x = lu_shfl(x[c].x, t);
              xt.y = lu_shfl(x[c].y, t);
              if (lane > t) x[c] = x[c] - l * xt;
            }
          }
        } else {
          for (int t = ib - 1; t >= 0; --t) {
            if (lane == t) {
              const C_ d = sD[t][t];
#pragma unroll
              for (int c = 0; c < NC; ++c) x[c] = cxdiv(x[c], d);
            }
            const C_ u = sD[lane][t];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
              C_ xt;
              xt.x = lu_shfl(x[c].x, t);
              xt.y = lu_shfl(x[c].y, t);
              if (lane < t) x[c] = x[c] - u * xt;
            }
          }
        }
        if (lane < ib) {
#pragma unroll
          for (int c = 0; c < NC; ++c) X[(i0 + lane) * NC + c] = x[c];
        }
      }
      __syncthreads();
      // the block's contribution to the rows still to solve
      const int rs = fwd ? i0 + ib : 0, re = fwd ? n : i0;
      for (int i = rs + tid; i < re; i += blockDim.x) {
        C_ acc[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) acc[c] = X[i * NC + c];
        const C_* li = LU + i + (long long)i0 * lda;
        for (int t = 0; t < ib; ++t) {
          const C_ l = li[(long long)t * lda];
#pragma unroll
          for (int c = 0; c < NC; ++c) acc[c] = acc[c] - l * X[(i0 + t) * NC + c];
        }
#pragma unroll
        for (int c = 0; c < NC; ++c) X[i * NC + c] = acc[c];
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < n * nrhs; e += blockDim.x) {
    const int r = e % n, c = e / n;
    B[r + (long long)c * ldb] = X[r * NC + c];
  }
}

template <class R, int NC>
static bool getrs_narrow(cudaStream_t s, int batch, int n, const Cx<R>* LU, int lda, long long a_bs, const int* ipiv,
                         long long piv_bs, Cx<R>* B, int nrhs, int ldb, long long b_bs) {
  const size_t sm = (size_t)n * NC * sizeof(Cx<R>);
  if (sm > (size_t)200 * 1024) return false;
  cudaFuncSetAttribute(getrs_narrow_kernel<R, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  getrs_narrow_kernel<R, NC><<<batch, NS_THREADS, sm, s>>>(LU, n, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs);
  note_launch();
  return true;
}

// Many right-hand sides: a blocked substitution across the GPU. The FP32 form's cascade always
// takes it; FP64 takes it only for batches too small to fill the GPU with getrs_kernel's CTAs
// (stage A's outer inverses: a few N x N systems with N right-hand sides), since a large FP64
// batch is bound by FP64 issue either way.
// The row interchanges are applied first (trans 0) or last (trans 1), one thread per column;
// then, per block of TB_NB rows, trsm_diag_kernel solves the diagonal block for every column
// (the block and 64 columns in shared memory, one thread per column) and the batched GEMM
// subtracts the block's contribution from the rows still to solve (K = TB_NB). The
// substitution order and pivots are those of getrs_kernel; only the summation order differs.
constexpr int TB_NB = 64;
constexpr int TB_W = 64;

template <class R>
__global__ void laswp_kernel(Cx<R>* __restrict__ Ball, int n, int nrhs, int ldb, long long b_bs,
                             const int* __restrict__ ipiv_all, long long piv_bs, int forward) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nrhs) return;
  Cx<R>* col = Ball + blockIdx.y * b_bs + (long long)c * ldb;
  const int* ipiv = ipiv_all + (long long)blockIdx.y * piv_bs;
  if (forward) {
    for (int j = 0; j < n; ++j) {
      const int p = ipiv[j];
      if (p != j) { const Cx<R> t = col[j]; col[j] = col[p]; col[p] = t; }
    }
  } else {
    for (int j = n - 1; j >= 0; --j) {
      const int p = ipiv[j];
      if (p != j) { const Cx<R> t = col[j]; col[j] = col[p]; col[p] = t; }
    }
  }
}

// op(A)'s diagonal block [i0, i0 + ib) solved for TB_W columns: lower (forward) or upper
// (backward) triangle, unit or stored diagonal; op(A) = A (trans 0) or A^T (trans 1).
template <class R>
__global__ void __launch_bounds__(TB_W) trsm_diag_kernel(const Cx<R>* __restrict__ LUall, int lda, long long a_bs,
                                                         Cx<R>* __restrict__ Ball, int nrhs, int ldb, long long b_bs,
                                                         int i0, int ib, int lower, int unit, int trans) {
  using C_ = Cx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C_* sL = reinterpret_cast<C_*>(smraw);                 // (TB_NB, TB_NB + 1)
  C_* sX = sL + TB_NB * (TB_NB + 1);                     // (TB_NB, TB_W + 1)
  const C_* LU = LUall + blockIdx.y * a_bs;
  C_* B = Ball + blockIdx.y * b_bs;
  const int c0 = blockIdx.x * TB_W, tid = threadIdx.x;
  const int w = min(TB_W, nrhs - c0);
  for (int e = tid; e < TB_NB * TB_NB; e += blockDim.x) {
    const int r = e % TB_NB, t = e / TB_NB;
    C_ v = cxzero<R>();
    if (r < ib && t < ib) v = trans ? LU[i0 + t + (long long)(i0 + r) * lda] : LU[i0 + r + (long long)(i0 + t) * lda];
    sL[r * (TB_NB + 1) + t] = v;
  }
  for (int e = tid; e < TB_NB * TB_W; e += blockDim.x) {
    const int r = e % TB_NB, c = e / TB_NB;
    sX[r * (TB_W + 1) + c] = (r < ib && c < w) ? B[i0 + r + (long long)(c0 + c) * ldb] : cxzero<R>();
  }
  __syncthreads();
  if (tid < w) {
    auto L = [&](int r, int t) -> C_ { return sL[r * (TB_NB + 1) + t]; };
    auto X = [&](int r) -> C_& { return sX[r * (TB_W + 1) + tid]; };
    if (lower) {
      for (int r = 0; r < ib; ++r) {
        C_ acc = X(r);
        for (int t = 0; t < r; ++t) acc = acc - L(r, t) * X(t);
        if (!unit) acc = cxdiv(acc, L(r, r));
        X(r) = acc;
      }
    } else {
      for (int r = ib - 1; r >= 0; --r) {
        C_ acc = X(r);
        for (int t = r + 1; t < ib; ++t) acc = acc - L(r, t) * X(t);
        if (!unit) acc = cxdiv(acc, L(r, r));
        X(r) = acc;
      }
    }
  }
  __syncthreads();
  for (int e = tid; e < TB_NB * TB_W; e += blockDim.x) {
    const int r = e % TB_NB, c = e / TB_NB;
    if (r < ib && c < w) B[i0 + r + (long long)(c0 + c) * ldb] = sX[r * (TB_W + 1) + c];
  }
}

template <class R>
static void getrs_blocked(cudaStream_t s, int batch, int n, const Cx<R>* LU, int lda, long long a_bs, const int* ipiv,
                          long long piv_bs, Cx<R>* B, int nrhs, int ldb, long long b_bs, int trans) {
  const dim3 gs((nrhs + 127) / 128, batch);
  if (trans == 0) { laswp_kernel<R><<<gs, 128, 0, s>>>(B, n, nrhs, ldb, b_bs, ipiv, piv_bs, 1); note_launch(); }
  const size_t sm = sizeof(Cx<R>) * ((size_t)TB_NB * (TB_NB + 1) + (size_t)TB_NB * (TB_W + 1));
  cudaFuncSetAttribute(trsm_diag_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  const dim3 gd((nrhs + TB_W - 1) / TB_W, batch);
  const double2 m1 = make_double2(-1.0, 0.0), p1 = make_double2(1.0, 0.0);
  // forward: L (unit lower) for trans 0, U^T (lower, stored diagonal) for trans 1
  for (int i0 = 0; i0 < n; i0 += TB_NB) {
    const int ib = min(TB_NB, n - i0), i1 = i0 + ib, m = n - i1;
    trsm_diag_kernel<R><<<gd, TB_W, sm, s>>>(LU, lda, a_bs, B, nrhs, ldb, b_bs, i0, ib, 1, trans == 0, trans);
    note_launch();
    if (m > 0) {
      if (trans == 0)
        gemm<R>(s, batch, m, nrhs, ib, m1, LU + i1 + (long long)i0 * lda, 1, lda, a_bs, B + i0, 1, ldb, b_bs, p1,
                B + i1, 1, ldb, b_bs);
      else
        gemm<R>(s, batch, m, nrhs, ib, m1, LU + i0 + (long long)i1 * lda, lda, 1, a_bs, B + i0, 1, ldb, b_bs, p1,
                B + i1, 1, ldb, b_bs);
    }
  }
  // backward: U (upper, stored diagonal) for trans 0, L^T (unit upper) for trans 1
  for (int i1 = n; i1 > 0; i1 -= TB_NB) {
    const int i0 = max(0, i1 - TB_NB), ib = i1 - i0;
    trsm_diag_kernel<R><<<gd, TB_W, sm, s>>>(LU, lda, a_bs, B, nrhs, ldb, b_bs, i0, ib, 0, trans == 1, trans);
    note_launch();
    if (i0 > 0) {
      if (trans == 0)
        gemm<R>(s, batch, i0, nrhs, ib, m1, LU + (long long)i0 * lda, 1, lda, a_bs, B + i0, 1, ldb, b_bs, p1, B, 1,
                ldb, b_bs);
      else
        gemm<R>(s, batch, i0, nrhs, ib, m1, LU + i0, lda, 1, a_bs, B + i0, 1, ldb, b_bs, p1, B, 1, ldb, b_bs);
    }
  }
  if (trans == 1) { laswp_kernel<R><<<gs, 128, 0, s>>>(B, n, nrhs, ldb, b_bs, ipiv, piv_bs, 0); note_launch(); }
}

template <class R>
void getrs(cudaStream_t s, int batch, int n, const Cx<R>* LU, int lda, long long a_bs, const int* ipiv,
           long long piv_bs, Cx<R>* B, int nrhs, int ldb, long long b_bs, int trans) {
  if (batch <= 0 || n <= 0 || nrhs <= 0) return;
  if (sizeof(R) == 4 && nrhs >= 32 && n >= 2 * TB_NB) {     // FP32: the cascade of the mixed form
    getrs_blocked<R>(s, batch, n, LU, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs, trans);
    return;
  }
  if (std::is_same<R, double>::value && nrhs >= 2 * SV_W && n >= 2 * TB_NB &&
      (long long)batch * ((nrhs + SV_W - 1) / SV_W) < sm_count()) {
    getrs_blocked<R>(s, batch, n, LU, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs, trans);
    return;
  }
  if (trans == 0 && n >= 64 && batch < 4 * sm_count()) {
    if (nrhs <= 3 && getrs_narrow<R, 3>(s, batch, n, LU, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs)) return;
    if (nrhs > 3 && nrhs <= 6 && getrs_narrow<R, 6>(s, batch, n, LU, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs))
      return;
  }
  dim3 grid((nrhs + SV_W - 1) / SV_W, batch);
  getrs_kernel<R><<<grid, 256, 0, s>>>(LU, n, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs, trans); note_launch();
}

// ---------------------------------------------------------------------- small helpers
template <class R>
__global__ void set_identity_kernel(Cx<R>* A, int n, int lda, long long a_bs, long long total) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  long long per = (long long)n * n;
  long long b = idx / per, r = idx % per;
  int i = (int)(r % n), j = (int)(r / n);
  A[b * a_bs + i + (long long)j * lda] = (i == j) ? cxone<R>() : cxzero<R>();
}

template <class R>
void set_identity(cudaStream_t s, int batch, int n, Cx<R>* A, int lda, long long a_bs) {
  long long total = (long long)batch * n * n;
  if (total <= 0) return;
  set_identity_kernel<R><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(A, n, lda, a_bs, total); note_launch();
}

// dst (Cx<R2>) <- src (Cx<R1>), elementwise over `count` entries
template <class R1, class R2>
__global__ void convert_kernel(const Cx<R1>* __restrict__ src, Cx<R2>* __restrict__ dst, long long count) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  Cx<R1> v = src[i];
  dst[i] = cxmk<R2>(R2(rto(v.x)), R2(rto(v.y)));
}
template <>
__global__ void convert_kernel<double, df64>(const Cx<double>* __restrict__ src, Cx<df64>* __restrict__ dst,
                                            long long count) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  Cx<double> v = src[i];
  dst[i] = cxmk<df64>(df64(v.x), df64(v.y));
}

template <class R1, class R2>
void convert(cudaStream_t s, const Cx<R1>* src, Cx<R2>* dst, long long count) {
  if (count <= 0) return;
  convert_kernel<R1, R2><<<(unsigned)((count + 255) / 256), 256, 0, s>>>(src, dst, count); note_launch();
}

// ---------------------------------------------------------- double2 (plain FP64) wrappers
void zgemm(cudaStream_t s, int batch, int m, int n, int k, cplx alpha,
           const cplx* A, long long a_rs, long long a_cs, long long a_bs,
           const cplx* B, long long b_rs, long long b_cs, long long b_bs,
           cplx beta, cplx* C, long long c_rs, long long c_cs, long long c_bs) {
  gemm<double>(s, batch, m, n, k, alpha, (const Cx<double>*)A, a_rs, a_cs, a_bs, (const Cx<double>*)B, b_rs, b_cs,
               b_bs, beta, (Cx<double>*)C, c_rs, c_cs, c_bs);
}
void zgemm_conj(cudaStream_t s, int batch, int m, int n, int k, cplx alpha, const cplx* A, long long a_rs,
                long long a_cs, long long a_bs, bool conj_a, const cplx* B, long long b_rs, long long b_cs,
                long long b_bs, bool conj_b, cplx beta, cplx* C, long long c_rs, long long c_cs, long long c_bs) {
  if (batch <= 0 || m <= 0 || n <= 0) return;
  if (!conj_a && !conj_b) {
    zgemm(s, batch, m, n, k, alpha, A, a_rs, a_cs, a_bs, B, b_rs, b_cs, b_bs, beta, C, c_rs, c_cs, c_bs);
    return;
  }
  using D = Cx<double>;
  const D* a = (const D*)A;
  const D* b = (const D*)B;
  D* c = (D*)C;
  dim3 grid((m + GT - 1) / GT, (n + GT - 1) / GT, batch);
  if (conj_a && conj_b)
    gemm_kernel<double, true, true><<<grid, 256, 0, s>>>(m, n, k, alpha, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs,
                                                         beta, c, c_rs, c_cs, c_bs, nullptr);
  else if (conj_a)
    gemm_kernel<double, true, false><<<grid, 256, 0, s>>>(m, n, k, alpha, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs,
                                                          beta, c, c_rs, c_cs, c_bs, nullptr);
  else
    gemm_kernel<double, false, true><<<grid, 256, 0, s>>>(m, n, k, alpha, a, a_rs, a_cs, a_bs, b, b_rs, b_cs, b_bs,
                                                          beta, c, c_rs, c_cs, c_bs, nullptr);
  note_launch();
}
void zgetrf(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs, int* ipiv, long long piv_bs,
            int32_t* status, int st_div) {
  getrf<double>(s, batch, n, (Cx<double>*)A, lda, a_bs, ipiv, piv_bs, status, st_div);
}
void zgetrs(cudaStream_t s, int batch, int n, const cplx* LU, int lda, long long a_bs,
            const int* ipiv, long long piv_bs, cplx* B, int nrhs, int ldb, long long b_bs, int trans) {
  getrs<double>(s, batch, n, (const Cx<double>*)LU, lda, a_bs, ipiv, piv_bs, (Cx<double>*)B, nrhs, ldb, b_bs, trans);
}
void zset_identity(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs) {
  set_identity<double>(s, batch, n, (Cx<double>*)A, lda, a_bs);
}

#define WB_INST(R)                                                                                       \
  template void gemm<R>(cudaStream_t, int, int, int, int, double2, const Cx<R>*, long long, long long,     \
                        long long, const Cx<R>*, long long, long long, long long, double2, Cx<R>*,         \
                        long long, long long, long long);                                                 \
  template void gemm_idx<R>(cudaStream_t, int, int, int, int, double2, const Cx<R>*, long long, long long, \
                            long long, const int*, const Cx<R>*, long long, long long, long long, double2,  \
                            Cx<R>*, long long, long long, long long);                                     \
  template void getrf<R>(cudaStream_t, int, int, Cx<R>*, int, long long, int*, long long, int32_t*, int); \
  template void getrs<R>(cudaStream_t, int, int, const Cx<R>*, int, long long, const int*, long long,      \
                         Cx<R>*, int, int, long long, int);                                               \
  template void set_identity<R>(cudaStream_t, int, int, Cx<R>*, int, long long);
WB_INST(double)
WB_INST(float)
WB_INST(df64)
template void convert<double, float>(cudaStream_t, const Cx<double>*, Cx<float>*, long long);
template void convert<double, double>(cudaStream_t, const Cx<double>*, Cx<double>*, long long);
template void convert<float, double>(cudaStream_t, const Cx<float>*, Cx<double>*, long long);
template void convert<double, df64>(cudaStream_t, const Cx<double>*, Cx<df64>*, long long);
template void convert<df64, double>(cudaStream_t, const Cx<df64>*, Cx<double>*, long long);
template void convert<df64, float>(cudaStream_t, const Cx<df64>*, Cx<float>*, long long);

}  // namespace wb
