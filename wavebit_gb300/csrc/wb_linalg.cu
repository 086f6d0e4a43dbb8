// Batched dense complex FP64 linear algebra for the RCWA path: GEMM, LU with partial pivoting,
// triangular solves with many right-hand sides, transposes and diagonal scalings.
//
// On GB300 the FP64 pipe delivers about 1 TFLOP/s (measured: DFMA 1.0, DMMA m8n8k4 1.05,
// DGEMM 1.05), so every kernel here is written to keep the FP64 units busy rather than to
// save bandwidth: a 64x64 CTA tile with 4x4 register blocking reaches the FP64 rate at an
// arithmetic intensity far above what HBM needs. FP64 mma.sync runs at the same rate as DFMA
// on this part, so plain fused multiply-adds are used.
#include "wb_common.cuh"
#include "wb_kernels.h"

namespace wb {

// ------------------------------------------------------------------------------------- GEMM
// C = alpha * A * B + beta * C for a batch; A (m x k), B (k x n), C (m x n), each addressed by
// (row stride, column stride) so that transposed views need no copies.
constexpr int GT = 64;   // CTA tile
constexpr int GK = 8;    // K step

__global__ void __launch_bounds__(256) zgemm_kernel(
    int m, int n, int k, cplx alpha,
    const cplx* __restrict__ A, long long a_rs, long long a_cs, long long a_bs,
    const cplx* __restrict__ B, long long b_rs, long long b_cs, long long b_bs,
    cplx beta, cplx* __restrict__ C, long long c_rs, long long c_cs, long long c_bs) {
  __shared__ cplx sA[GK][GT + 1];
  __shared__ cplx sB[GK][GT + 1];
  const int bz = blockIdx.z;
  A += bz * a_bs; B += bz * b_bs; C += bz * c_bs;
  const int row0 = blockIdx.x * GT, col0 = blockIdx.y * GT;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  cplx acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cmk(0.0, 0.0);
  for (int k0 = 0; k0 < k; k0 += GK) {
    // A tile: GT rows x GK cols; 512 elements, 2 per thread; rows fastest for column-major A
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % GT, c = idx / GT;
      int gr = row0 + r, gc = k0 + c;
      sA[c][r] = (gr < m && gc < k) ? A[gr * a_rs + gc * a_cs] : cmk(0.0, 0.0);
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % GK, c = idx / GK;
      int gr = k0 + r, gc = col0 + c;
      sB[r][c] = (gr < k && gc < n) ? B[gr * b_rs + gc * b_cs] : cmk(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      cplx a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = cfma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  const bool zero_beta = (beta.x == 0.0 && beta.y == 0.0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gr = row0 + tx + 16 * i;
    if (gr >= m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gc = col0 + ty + 16 * j;
      if (gc >= n) continue;
      cplx* p = C + gr * c_rs + gc * c_cs;
      cplx v = cmul(alpha, acc[i][j]);
      if (!zero_beta) v = cfma(beta, *p, v);
      *p = v;
    }
  }
}

void zgemm(cudaStream_t s, int batch, int m, int n, int k, cplx alpha,
           const cplx* A, long long a_rs, long long a_cs, long long a_bs,
           const cplx* B, long long b_rs, long long b_cs, long long b_bs,
           cplx beta, cplx* C, long long c_rs, long long c_cs, long long c_bs) {
  if (batch <= 0 || m <= 0 || n <= 0) return;
  dim3 grid((m + GT - 1) / GT, (n + GT - 1) / GT, batch);
  zgemm_kernel<<<grid, 256, 0, s>>>(m, n, k, alpha, A, a_rs, a_cs, a_bs, B, b_rs, b_cs, b_bs,
                                    beta, C, c_rs, c_cs, c_bs); note_launch();
}

// ----------------------------------------------------------------------- LU factorisation
// One CTA per matrix, right-looking, panel width LU_NB. Pivot choice is the largest |re|+|im|
// in the column (the LAPACK izamax measure). Row swaps are applied across the full width.
constexpr int LU_NB = 16;
constexpr int LU_THREADS = 256;

__device__ void block_argmax(double v, int idx, double* sval, int* sidx, double& out_v, int& out_i) {
  // reduce (value, index) to the largest value, ties to the smallest index
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    double ov = __shfl_down_sync(0xffffffffu, v, off);
    int oi = __shfl_down_sync(0xffffffffu, idx, off);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
  if (lane == 0) { sval[warp] = v; sidx[warp] = idx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double bv = sval[0]; int bi = sidx[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (sval[w] > bv || (sval[w] == bv && sidx[w] < bi)) { bv = sval[w]; bi = sidx[w]; }
    sval[0] = bv; sidx[0] = bi;
  }
  __syncthreads();
  out_v = sval[0]; out_i = sidx[0];
  __syncthreads();
}

__global__ void __launch_bounds__(LU_THREADS) zgetrf_kernel(
    cplx* __restrict__ Aall, int n, int lda, long long a_bs, int* __restrict__ ipiv_all, long long piv_bs,
    int32_t* __restrict__ status, int st_div) {
  __shared__ double sval[32];
  __shared__ int sidx[32];
  __shared__ cplx sL[GT][LU_NB + 1];
  __shared__ cplx sU[LU_NB][GT + 1];
  cplx* A = Aall + blockIdx.x * a_bs;
  int* ipiv = ipiv_all + (long long)blockIdx.x * piv_bs;
  int32_t* st = status ? status + blockIdx.x / st_div : nullptr;
  const int tid = threadIdx.x;
  for (int k0 = 0; k0 < n; k0 += LU_NB) {
    const int kb = min(LU_NB, n - k0);
    // ---- panel factorisation, unblocked
    for (int j = k0; j < k0 + kb; ++j) {
      double best = -1.0; int bi = j;
      for (int i = j + tid; i < n; i += blockDim.x) {
        double v = cabs1(A[i + (long long)j * lda]);
        if (v > best) { best = v; bi = i; }
      }
      double pv; int p;
      block_argmax(best, bi, sval, sidx, pv, p);
      if (tid == 0) ipiv[j] = p;
      if (p != j) {
        for (int c = tid; c < n; c += blockDim.x) {
          cplx t = A[j + (long long)c * lda];
          A[j + (long long)c * lda] = A[p + (long long)c * lda];
          A[p + (long long)c * lda] = t;
        }
      }
      __syncthreads();
      cplx piv = A[j + (long long)j * lda];
      if (piv.x == 0.0 && piv.y == 0.0) {
        if (tid == 0) wb_flag(st, WB_ST_SINGULAR);
        __syncthreads();
        continue;
      }
      cplx rp = cinv(piv);
      for (int i = j + 1 + tid; i < n; i += blockDim.x) {
        cplx l = cmul(A[i + (long long)j * lda], rp);
        A[i + (long long)j * lda] = l;
        for (int c = j + 1; c < k0 + kb; ++c)
          A[i + (long long)c * lda] = csub(A[i + (long long)c * lda], cmul(l, A[j + (long long)c * lda]));
      }
      __syncthreads();
    }
    const int c0 = k0 + kb;
    if (c0 >= n) break;
    // ---- U12 = L11^{-1} A12 (unit lower triangular), columns independent
    for (int c = c0 + tid; c < n; c += blockDim.x) {
      for (int r = k0 + 1; r < k0 + kb; ++r) {
        cplx acc = A[r + (long long)c * lda];
        for (int t = k0; t < r; ++t)
          acc = csub(acc, cmul(A[r + (long long)t * lda], A[t + (long long)c * lda]));
        A[r + (long long)c * lda] = acc;
      }
    }
    __syncthreads();
    // ---- A22 -= L21 * U12, 64x64 tiles, K = kb
    const int tx = tid & 15, ty = tid >> 4;
    for (int cc = c0; cc < n; cc += GT) {
      for (int e = tid; e < LU_NB * GT; e += blockDim.x) {
        int r = e % LU_NB, c = e / LU_NB;
        sU[r][c] = (r < kb && cc + c < n) ? A[k0 + r + (long long)(cc + c) * lda] : cmk(0.0, 0.0);
      }
      for (int rr = c0; rr < n; rr += GT) {
        for (int e = tid; e < LU_NB * GT; e += blockDim.x) {
          int r = e % GT, c = e / GT;
          sL[r][c] = (c < kb && rr + r < n) ? A[rr + r + (long long)(k0 + c) * lda] : cmk(0.0, 0.0);
        }
        __syncthreads();
        cplx acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[i][q] = cmk(0.0, 0.0);
        for (int kk = 0; kk < kb; ++kk) {
          cplx a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = sL[tx + 16 * i][kk];
#pragma unroll
          for (int q = 0; q < 4; ++q) b[q] = sU[kk][ty + 16 * q];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = cfma(a[i], b[q], acc[i][q]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          int gr = rr + tx + 16 * i;
          if (gr >= n) continue;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int gc = cc + ty + 16 * q;
            if (gc >= n) continue;
            cplx* p = A + gr + (long long)gc * lda;
            *p = csub(*p, acc[i][q]);
          }
        }
        __syncthreads();
      }
    }
  }
}

void zgetrf(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs, int* ipiv, long long piv_bs,
            int32_t* status, int st_div) {
  if (batch <= 0 || n <= 0) return;
  zgetrf_kernel<<<batch, LU_THREADS, 0, s>>>(A, n, lda, a_bs, ipiv, piv_bs, status, st_div < 1 ? 1 : st_div); note_launch();
}

// --------------------------------------------------------------------- triangular solves
// X = op(A)^{-1} B with A = P L U from zgetrf; B (n x nrhs, column-major, ldb) is overwritten.
// trans = 0: A X = B.  trans = 1: A^T X = B.  Each CTA owns SV_W right-hand sides of one
// matrix and runs blocked substitution with K = SV_NB register-tiled updates.
constexpr int SV_W = 64;
constexpr int SV_NB = 16;

__global__ void __launch_bounds__(256) zgetrs_kernel(
    const cplx* __restrict__ LUall, int n, int lda, long long a_bs, const int* __restrict__ ipiv_all,
    long long piv_bs, cplx* __restrict__ Ball, int nrhs, int ldb, long long b_bs, int trans) {
  __shared__ cplx sT[SV_NB][SV_NB + 1];
  __shared__ cplx sX[SV_NB][SV_W + 1];
  __shared__ cplx sM[GT][SV_NB + 1];
  const cplx* LU = LUall + blockIdx.y * a_bs;
  const int* ipiv = ipiv_all + (long long)blockIdx.y * piv_bs;
  cplx* B = Ball + blockIdx.y * b_bs;
  const int r0 = blockIdx.x * SV_W;
  const int w = min(SV_W, nrhs - r0);
  if (w <= 0) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  auto Bat = [&](int i, int c) -> cplx& { return B[i + (long long)(r0 + c) * ldb]; };
  auto Lat = [&](int i, int j) -> cplx { return LU[i + (long long)j * lda]; };
  // op(A) = L_eff * U_eff after the permutation; for trans = 0 first P^T B, forward with L
  // (unit), backward with U.  For trans = 1: forward with U^T (non-unit), backward with L^T
  // (unit), then the inverse permutation.
  if (trans == 0) {
    for (int j = 0; j < n; ++j) {
      int p = ipiv[j];
      if (p != j)
        for (int c = tid; c < w; c += blockDim.x) { cplx t = Bat(j, c); Bat(j, c) = Bat(p, c); Bat(p, c) = t; }
      __syncthreads();
    }
  }
  // two sweeps: sweep 0 = forward (lower), sweep 1 = backward (upper)
  for (int sweep = 0; sweep < 2; ++sweep) {
    const bool forward = (sweep == 0);
    // which triangle and diagonal handling
    // trans 0: fwd uses L (unit, A(i,j) i>j), bwd uses U (A(i,j) i<=j)
    // trans 1: fwd uses U^T: element (i,j) i>=j is A(j,i), non-unit; bwd uses L^T: (i,j) i<j is A(j,i), unit
    const bool unit = (trans == 0) ? forward : !forward;
    const int nblk = (n + SV_NB - 1) / SV_NB;
    for (int bi = 0; bi < nblk; ++bi) {
      const int blk = forward ? bi : (nblk - 1 - bi);
      const int i0 = blk * SV_NB, ib = min(SV_NB, n - i0);
      // load the diagonal block of op-triangle into sT[r][c] (row r, col c of the effective matrix)
      for (int e = tid; e < SV_NB * SV_NB; e += blockDim.x) {
        int r = e % SV_NB, c = e / SV_NB;
        cplx v = cmk(0.0, 0.0);
        if (r < ib && c < ib) v = (trans == 0) ? Lat(i0 + r, i0 + c) : Lat(i0 + c, i0 + r);
        sT[r][c] = v;
      }
      for (int e = tid; e < SV_NB * SV_W; e += blockDim.x) {
        int r = e % SV_NB, c = e / SV_NB;
        sX[r][c] = (r < ib && c < w) ? Bat(i0 + r, c) : cmk(0.0, 0.0);
      }
      __syncthreads();
      // small triangular solve, one thread per right-hand side column
      if (tid < w) {
        const int c = tid;
        if (forward) {
          for (int r = 0; r < ib; ++r) {
            cplx acc = sX[r][c];
            for (int t = 0; t < r; ++t) acc = csub(acc, cmul(sT[r][t], sX[t][c]));
            if (!unit) acc = cdiv(acc, sT[r][r]);
            sX[r][c] = acc;
          }
        } else {
          for (int r = ib - 1; r >= 0; --r) {
            cplx acc = sX[r][c];
            for (int t = r + 1; t < ib; ++t) acc = csub(acc, cmul(sT[r][t], sX[t][c]));
            if (!unit) acc = cdiv(acc, sT[r][r]);
            sX[r][c] = acc;
          }
        }
      }
      __syncthreads();
      for (int e = tid; e < SV_NB * SV_W; e += blockDim.x) {
        int r = e % SV_NB, c = e / SV_NB;
        if (r < ib && c < w) Bat(i0 + r, c) = sX[r][c];
      }
      // update the remaining rows: B[rest] -= M[rest, block] * X[block]
      const int rs = forward ? i0 + ib : 0;
      const int re = forward ? n : i0;
      for (int rr = rs; rr < re; rr += GT) {
        for (int e = tid; e < GT * SV_NB; e += blockDim.x) {
          int r = e % GT, c = e / GT;
          int gr = rr + r;
          cplx v = cmk(0.0, 0.0);
          if (gr < re && c < ib) v = (trans == 0) ? Lat(gr, i0 + c) : Lat(i0 + c, gr);
          sM[r][c] = v;
        }
        __syncthreads();
        cplx acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int q = 0; q < 4; ++q) acc[i][q] = cmk(0.0, 0.0);
        for (int kk = 0; kk < ib; ++kk) {
          cplx a[4], b[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) a[i] = sM[tx + 16 * i][kk];
#pragma unroll
          for (int q = 0; q < 4; ++q) b[q] = sX[kk][ty + 16 * q];
#pragma unroll
          for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[i][q] = cfma(a[i], b[q], acc[i][q]);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          int gr = rr + tx + 16 * i;
          if (gr >= re) continue;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            int c = ty + 16 * q;
            if (c >= w) continue;
            Bat(gr, c) = csub(Bat(gr, c), acc[i][q]);
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
        for (int c = tid; c < w; c += blockDim.x) { cplx t = Bat(j, c); Bat(j, c) = Bat(p, c); Bat(p, c) = t; }
      __syncthreads();
    }
  }
}

void zgetrs(cudaStream_t s, int batch, int n, const cplx* LU, int lda, long long a_bs,
            const int* ipiv, long long piv_bs, cplx* B, int nrhs, int ldb, long long b_bs, int trans) {
  if (batch <= 0 || n <= 0 || nrhs <= 0) return;
  dim3 grid((nrhs + SV_W - 1) / SV_W, batch);
  zgetrs_kernel<<<grid, 256, 0, s>>>(LU, n, lda, a_bs, ipiv, piv_bs, B, nrhs, ldb, b_bs, trans); note_launch();
}

// ---------------------------------------------------------------------- small helpers
__global__ void ztranspose_kernel(const cplx* __restrict__ A, int m, int n, int lda, long long a_bs,
                                  cplx* __restrict__ B, int ldb, long long b_bs) {
  // B (n x m) = A^T, A (m x n); 32x32 tiles through shared memory
  __shared__ cplx t[32][33];
  A += blockIdx.z * a_bs; B += blockIdx.z * b_bs;
  int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int e = threadIdx.y; e < 32; e += blockDim.y) {
    int i = i0 + threadIdx.x, j = j0 + e;
    if (i < m && j < n) t[e][threadIdx.x] = A[i + (long long)j * lda];
  }
  __syncthreads();
  for (int e = threadIdx.y; e < 32; e += blockDim.y) {
    int j = j0 + threadIdx.x, i = i0 + e;
    if (i < m && j < n) B[j + (long long)i * ldb] = t[threadIdx.x][e];
  }
}

void ztranspose(cudaStream_t s, int batch, int m, int n, const cplx* A, int lda, long long a_bs,
                cplx* B, int ldb, long long b_bs) {
  if (batch <= 0 || m <= 0 || n <= 0) return;
  dim3 grid((m + 31) / 32, (n + 31) / 32, batch);
  ztranspose_kernel<<<grid, dim3(32, 8), 0, s>>>(A, m, n, lda, a_bs, B, ldb, b_bs); note_launch();
}

__global__ void zset_identity_kernel(cplx* A, int n, int lda, long long a_bs, long long total) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  long long per = (long long)n * n;
  long long b = idx / per, r = idx % per;
  int i = (int)(r % n), j = (int)(r / n);
  A[b * a_bs + i + (long long)j * lda] = cmk(i == j ? 1.0 : 0.0, 0.0);
}

void zset_identity(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs) {
  long long total = (long long)batch * n * n;
  if (total <= 0) return;
  zset_identity_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(A, n, lda, a_bs, total); note_launch();
}

}  // namespace wb
