// Batched complex non-Hermitian eigen-decomposition, one CTA per matrix, templated over the
// real type R in {double, float, df64} (wb_num.cuh).
//
// The layer operator Omega^2 of every (solve, layer) pair is decomposed as
//   Omega^2 = Z T Z^H  (Hessenberg reduction, then Francis single-shift QR to Schur form)
//   Omega^2 W = W diag(w),  W = Z X  (X: eigenvectors of the triangular T by back-substitution)
// which is the factorisation LAPACK's zgeev performs for numpy.linalg.eig (right vectors only).
//
// GB300 note: FP64 runs at ~1 TFLOP/s, about 2 FP64 FMAs per clock per SM. A rotation applied
// across a row/column of a few hundred elements costs more in FP64 issue than in latency, so a
// one-CTA-per-matrix layout with the matrix resident in L2/HBM keeps the FP64 pipe busy. The
// df64 instantiation (mixed form) runs the same algorithm on the FP32 pipes.
//
// Every iteration is capped; a matrix that hits the cap gets WB_ST_NOCONV in its status word
// and NaN eigenvalues, and the kernel returns normally.
#include <mutex>
#include <utility>
#include <vector>
#include "wb_common.cuh"
#include "wb_num.cuh"
#include "wb_kernels.h"

namespace wb {


__device__ __forceinline__ double shfl_xor(double v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ float shfl_xor(float v, int off) { return __shfl_xor_sync(0xffffffffu, v, off); }
__device__ __forceinline__ df64 shfl_xor(df64 v, int off) {
  return df64(__shfl_xor_sync(0xffffffffu, v.hi, off), __shfl_xor_sync(0xffffffffu, v.lo, off));
}
__device__ __forceinline__ double shfl_idx(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float shfl_idx(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ df64 shfl_idx(df64 v, int src) {
  return df64(__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src));
}
template <class R> __device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = v + shfl_xor(v, off);
  return v;
}

template <class R> __device__ R block_sum(R v, R* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    R s = R(0.0);
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s = s + red[w];
    red[0] = s;
  }
  __syncthreads();
  R r = red[0];
  __syncthreads();
  return r;
}

__device__ int block_max_int(int v, int* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, off));
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) s = max(s, red[w]);
    red[0] = s;
  }
  __syncthreads();
  int r = red[0];
  __syncthreads();
  return r;
}

// Householder reflector for (alpha, x): returns beta (real), tau and the scale of x so that
// (I - tau v v^H)^H (alpha; x) = (beta; 0), v = (1; x * scale).
template <class R> struct Refl { R beta; Cx<R> tau; Cx<R> scale; bool identity; };
template <class R> __device__ __forceinline__ Refl<R> make_reflector(Cx<R> alpha, R xnorm) {
  Refl<R> r;
  if (xnorm == R(0.0) && alpha.y == R(0.0)) {
    r.identity = true; r.beta = alpha.x; r.tau = cxzero<R>(); r.scale = cxzero<R>();
    return r;
  }
  R ax = rabs(alpha.x), ay = rabs(alpha.y);
  R m = rmax(rmax(ax, ay), xnorm);
  R u = ax / m, v = ay / m, w = xnorm / m;
  R nrm = m * rsqrt_(u * u + v * v + w * w);
  R beta = (alpha.x >= R(0.0)) ? -nrm : nrm;
  r.identity = false;
  r.beta = beta;
  r.tau = cxmk<R>((beta - alpha.x) / beta, -alpha.y / beta);
  r.scale = cxinv(cxmk<R>(alpha.x - beta, alpha.y));
  return r;
}

// ------------------------------------------------------------- 1. Hessenberg reduction
// H := Q^H A Q, reflectors stored below the subdiagonal (v_0 = 1 implicit), tau[k].
//
// Both sides of reflector k are applied in one pass over the trailing columns. With y = A v
// (all rows) and c = v^H y, the right update A' = A - t y v^H and the left update
// A'' = A' - conj(t) v (v^H A') combine, column by column, into
//   A''[:, j] = A[:, j] - t y conj(v_j) - conj(t) v z_j,   z_j = v^H A[:, j] - t c conj(v_j),
// so each step reads the trailing matrix twice (y, then each column's z_j and its update) and
// writes it once. Every load-modify-store sweep issues kUnroll loads before its stores, so one
// memory latency serves kUnroll elements per lane.
constexpr int kUnroll = 4;

template <class R>
__device__ __forceinline__ Cx<R> block_sum_cx(Cx<R> v, R* red) {
  Cx<R> r;
  r.x = block_sum(v.x, red);
  r.y = block_sum(v.y, red);
  return r;
}

// sum_i conj(v_i) c_i over i < m by one warp, the total in every lane. The FP32 form issues four
// loads per lane before it accumulates (four partial sums), the other forms one.
template <class R>
__device__ __forceinline__ Cx<R> column_dot(const Cx<R>* v, const Cx<R>* c, int m, int lane) {
  Cx<R> acc = cxzero<R>();
  int i = lane;
  if constexpr (sizeof(R) == 4) {
    Cx<R> acc1 = cxzero<R>(), acc2 = cxzero<R>(), acc3 = cxzero<R>();
    for (; i + 96 < m; i += 128) {
      const Cx<R> c0 = c[i], c1 = c[i + 32], c2 = c[i + 64], c3 = c[i + 96];
      acc = cxfma_conj(v[i], c0, acc);
      acc1 = cxfma_conj(v[i + 32], c1, acc1);
      acc2 = cxfma_conj(v[i + 64], c2, acc2);
      acc3 = cxfma_conj(v[i + 96], c3, acc3);
    }
    acc = (acc + acc2) + (acc1 + acc3);
  }
  for (; i < m; i += 32) acc = cxfma_conj(v[i], c[i], acc);
  acc.x = warp_sum(acc.x);
  acc.y = warp_sum(acc.y);
  return acc;
}

template <class R>
__global__ void __launch_bounds__(1024) gehrd_kernel(Cx<R>* __restrict__ Aall, int n, int lda,
                                                     long long a_bs, Cx<R>* __restrict__ tau_all) {
  using C_ = Cx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C_* sv = reinterpret_cast<C_*>(smraw);          // v (n), then y = A v (n)
  __shared__ R red[32];
  __shared__ C_ s_tau;
  C_* A = Aall + blockIdx.x * a_bs;
  C_* tau = tau_all + (long long)blockIdx.x * n;
  C_* sy = sv + n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;
    C_* col = A + (long long)k * lda;
    R part = R(0.0);
    for (int i = k + 2 + tid; i < n; i += blockDim.x) part = part + cxabs2(col[i]);
    R xn2 = block_sum(part, red);
    C_ alpha = col[k + 1];
    Refl<R> r = make_reflector(alpha, rsqrt_(xn2));
    if (r.identity) {
      if (tid == 0) tau[k] = cxzero<R>();
      __syncthreads();
      continue;
    }
    for (int i = k + 2 + tid; i < n; i += blockDim.x) {
      C_ v = col[i] * r.scale;
      col[i] = v;
      sv[i - k - 1] = v;
    }
    if (tid == 0) {
      sv[0] = cxone<R>();
      tau[k] = r.tau;
      s_tau = r.tau;
    }
    __syncthreads();
    // every thread has read alpha = A(k+1, k) by now; column k is not touched again in this step
    if (tid == 0) col[k + 1] = cxmk<R>(r.beta, R(0.0));
    const C_ t = s_tau, tc = cxconj(t);
    // y = A[:, k+1:n] v, one row per thread (loads only: they pipeline). The FP32 form keeps four
    // loads in flight per thread (its registers allow it; the FP64-sized forms are at the limit).
    for (int i = tid; i < n; i += blockDim.x) {
      const C_* ai = A + i + (long long)(k + 1) * lda;
      C_ acc0 = cxzero<R>(), acc1 = cxzero<R>();
      int j = 0;
      if constexpr (sizeof(R) == 4) {
        C_ acc2 = cxzero<R>(), acc3 = cxzero<R>();
        for (; j + 3 < m; j += 4) {
          const C_ a0 = ai[(long long)j * lda], a1 = ai[(long long)(j + 1) * lda];
          const C_ a2 = ai[(long long)(j + 2) * lda], a3 = ai[(long long)(j + 3) * lda];
          acc0 = cxfma(a0, sv[j], acc0);
          acc1 = cxfma(a1, sv[j + 1], acc1);
          acc2 = cxfma(a2, sv[j + 2], acc2);
          acc3 = cxfma(a3, sv[j + 3], acc3);
        }
        acc0 = acc0 + acc2;
        acc1 = acc1 + acc3;
      }
      for (; j + 1 < m; j += 2) {
        acc0 = cxfma(ai[(long long)j * lda], sv[j], acc0);
        acc1 = cxfma(ai[(long long)(j + 1) * lda], sv[j + 1], acc1);
      }
      if (j < m) acc0 = cxfma(ai[(long long)j * lda], sv[j], acc0);
      sy[i] = acc0 + acc1;
    }
    __syncthreads();
    C_ cp = cxzero<R>();
    for (int i = tid; i < m; i += blockDim.x) cp = cxfma_conj(sv[i], sy[k + 1 + i], cp);
    const C_ c = block_sum_cx(cp, red);
    const C_ tcoef = t * c;
    // both sides, one warp per trailing column
    for (int jj = warp; jj < m; jj += nw) {
      C_* cj = A + (long long)(k + 1 + jj) * lda;
      const C_ acc = column_dot<R>(sv, cj + k + 1, m, lane);
      const C_ vjc = cxconj(sv[jj]);
      const C_ z = acc - tcoef * vjc;
      const C_ a1 = t * vjc, a2 = tc * z;
      for (int i0 = lane; i0 < n; i0 += 32 * kUnroll) {
        C_ val[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
          const int i = i0 + 32 * u;
          if (i < n) val[u] = cj[i];
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
          const int i = i0 + 32 * u;
          if (i >= n) continue;
          C_ nv = val[u] - sy[i] * a1;
          if (i > k) nv = nv - sv[i - k - 1] * a2;
          cj[i] = nv;
        }
      }
    }
    __syncthreads();
  }
}

// --------------------------------------- 1b. blocked Hessenberg reduction (FP32 form)
// The same reflectors and storage as gehrd_kernel, kHrdPanel columns at a time in WY form. With
// the panel's reflectors so far Q_j = I - V_j T_j V_j^H and Y_j = A V_j T_j (A as at the panel's
// start), column c = k + j of Q_j^H A Q_j is
//   b = a_c - Y_j V_j(c, :)^H,   then   b <- b - V_j T_j^H (V_j^H b)   (rows below k),
// its reflector (tau_j, v_j) extends T (T[:j, j] = -tau_j T_j V_j^H v_j, T[j, j] = tau_j) and Y
// (Y[:, j] = tau_j (A v_j - Y_j V_j^H v_j)); a_c and A v_j read columns the panel has not yet
// written, so the panel makes one pass over the trailing columns per column. After the panel,
// A <- Q^H (A - Y V^H) on the columns right of it, as batched products (geev_schur). Scratch per
// matrix (column-major, ld n): V, conj(V), Y (n x kHrdPanel), W, X (kHrdPanel x n), T^H.
constexpr int kHrdPanel = 32;

template <class R>
__global__ void __launch_bounds__(1024) gehrd_panel_kernel(Cx<R>* __restrict__ Aall, int n, int lda, long long a_bs,
                                                           Cx<R>* __restrict__ tau_all, int k, int bb,
                                                           Cx<R>* __restrict__ Wsall, long long ws_bs) {
  using C_ = Cx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C_* sb = reinterpret_cast<C_*>(smraw);          // (n) the column being reduced
  C_* sv = sb + n;                                 // (n) its reflector
  __shared__ C_ T[kHrdPanel][kHrdPanel + 1];
  __shared__ C_ s_vc[kHrdPanel], s_w[kHrdPanel], s_u[kHrdPanel];
  __shared__ R red[32];
  __shared__ C_ s_tau, s_scale;
  __shared__ R s_beta;
  __shared__ int s_id;
  C_* A = Aall + blockIdx.x * a_bs;
  C_* tau = tau_all + (long long)blockIdx.x * n;
  C_* ws = Wsall + blockIdx.x * ws_bs;
  const long long nB = (long long)n * kHrdPanel;
  C_* V = ws;
  C_* Vc = ws + nB;
  C_* Y = ws + 2 * nB;
  C_* TH = ws + 5 * nB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x, nw = nt >> 5;
  for (int e = tid; e < kHrdPanel * (kHrdPanel + 1); e += nt) T[e / (kHrdPanel + 1)][e % (kHrdPanel + 1)] = cxzero<R>();
  __syncthreads();
  for (int j = 0; j < bb; ++j) {
    const int c = k + j;
    if (tid < j) s_vc[tid] = cxconj(V[c + (long long)tid * n]);
    __syncthreads();
    // b = a_c - Y_j conj(V_j(c, :))
    for (int r = tid; r < n; r += nt) {
      C_ acc = A[r + (long long)c * lda];
      for (int l = 0; l < j; ++l) acc = acc - Y[r + (long long)l * n] * s_vc[l];
      sb[r] = acc;
    }
    __syncthreads();
    if (j > 0) {
      // w = V_j^H b (rows below k), u = T_j^H w, b <- b - V_j u
      for (int l = warp; l < j; l += nw) {
        C_ acc = cxzero<R>();
        for (int r = k + 1 + lane; r < n; r += 32) acc = cxfma_conj(V[r + (long long)l * n], sb[r], acc);
        acc.x = warp_sum(acc.x);
        acc.y = warp_sum(acc.y);
        if (lane == 0) s_w[l] = acc;
      }
      __syncthreads();
      if (tid < j) {
        C_ acc = cxzero<R>();
        for (int lp = 0; lp <= tid; ++lp) acc = cxfma_conj(T[lp][tid], s_w[lp], acc);
        s_u[tid] = acc;
      }
      __syncthreads();
      for (int r = k + 1 + tid; r < n; r += nt) {
        C_ acc = sb[r];
        for (int l = 0; l < j; ++l) acc = acc - V[r + (long long)l * n] * s_u[l];
        sb[r] = acc;
      }
      __syncthreads();
    }
    // the reflector of (b[c+1]; b[c+2:])
    R part = R(0.0);
    for (int r = c + 2 + tid; r < n; r += nt) part = part + cxabs2(sb[r]);
    const R xn2 = block_sum(part, red);
    if (tid == 0) {
      const Refl<R> rf = make_reflector(sb[c + 1], rsqrt_(xn2));
      s_id = rf.identity ? 1 : 0;
      s_tau = rf.identity ? cxzero<R>() : rf.tau;
      s_scale = rf.scale;
      s_beta = rf.beta;
      tau[c] = s_tau;
    }
    __syncthreads();
    const bool ident = s_id != 0;
    const C_ tj = s_tau, scl = s_scale;
    // v, V[:, j] and conj(V[:, j]), and column c in its final form
    for (int r = tid; r < n; r += nt) {
      C_ v = cxzero<R>();
      if (!ident) {
        if (r == c + 1) v = cxone<R>();
        else if (r > c + 1) v = sb[r] * scl;
      }
      sv[r] = v;
      V[r + (long long)j * n] = v;
      Vc[r + (long long)j * n] = cxconj(v);
      C_ a = sb[r];
      if (!ident && r == c + 1) a = cxmk<R>(s_beta, R(0.0));
      else if (!ident && r > c + 1) a = v;
      A[r + (long long)c * lda] = a;
    }
    __syncthreads();
    // w2 = V_j^H v, T[:j, j] = -tau T_j w2, T[j, j] = tau
    if (j > 0) {
      for (int l = warp; l < j; l += nw) {
        C_ acc = cxzero<R>();
        for (int r = c + 1 + lane; r < n; r += 32) acc = cxfma_conj(V[r + (long long)l * n], sv[r], acc);
        acc.x = warp_sum(acc.x);
        acc.y = warp_sum(acc.y);
        if (lane == 0) s_w[l] = acc;
      }
      __syncthreads();
      if (tid < j) {
        C_ acc = cxzero<R>();
        for (int lp = tid; lp < j; ++lp) acc = acc + T[tid][lp] * s_w[lp];
        T[tid][j] = -(tj * acc);
      }
    }
    if (tid == 0) T[j][j] = tj;
    __syncthreads();
    // Y[:, j] = tau (A[:, c+1:] v[c+1:] - Y_j w2), one row per thread, four loads in flight
    const int m = n - c - 1;
    for (int r = tid; r < n; r += nt) {
      const C_* ar = A + r + (long long)(c + 1) * lda;
      const C_* vv = sv + c + 1;
      C_ acc0 = cxzero<R>(), acc1 = cxzero<R>(), acc2 = cxzero<R>(), acc3 = cxzero<R>();
      int q = 0;
      for (; q + 3 < m; q += 4) {
        const C_ a0 = ar[(long long)q * lda], a1 = ar[(long long)(q + 1) * lda];
        const C_ a2 = ar[(long long)(q + 2) * lda], a3 = ar[(long long)(q + 3) * lda];
        acc0 = cxfma(a0, vv[q], acc0);
        acc1 = cxfma(a1, vv[q + 1], acc1);
        acc2 = cxfma(a2, vv[q + 2], acc2);
        acc3 = cxfma(a3, vv[q + 3], acc3);
      }
      for (; q < m; ++q) acc0 = cxfma(ar[(long long)q * lda], vv[q], acc0);
      C_ y = (acc0 + acc2) + (acc1 + acc3);
      for (int l = 0; l < j; ++l) y = y - Y[r + (long long)l * n] * s_w[l];
      Y[r + (long long)j * n] = ident ? cxzero<R>() : tj * y;
    }
    __syncthreads();
  }
  // T^H, column-major kHrdPanel x kHrdPanel, for the trailing update's X = T^H W
  for (int e = tid; e < kHrdPanel * kHrdPanel; e += nt) {
    const int r = e % kHrdPanel, cc = e / kHrdPanel;
    TH[e] = (r < bb && cc < bb) ? cxconj(T[cc][r]) : cxzero<R>();
  }
}

// --------------------------------------------- 2b. Q from the reflectors in panels (FP32 form)
// Q = H_0 H_1 ... H_{n-3} is formed as unghr_kernel forms it, last reflectors first, but
// kHrdPanel reflectors at a time: their product is I - V T V^H (T upper triangular, built
// forward: T[:j, j] = -tau_j T_j V_j^H v_j, T[j, j] = tau_j), and Z's trailing block gets
// Z <- Z - V (T (V^H Z)) as batched products. This kernel writes the panel's V, conj(V) (n x
// kHrdPanel) and T (column-major kHrdPanel x kHrdPanel) into the scratch.
template <class R>
__global__ void __launch_bounds__(1024) unghr_panel_kernel(const Cx<R>* __restrict__ Aall, int n, int lda,
                                                           long long a_bs, const Cx<R>* __restrict__ tau_all, int k0,
                                                           int bb, Cx<R>* __restrict__ Wsall, long long ws_bs) {
  using C_ = Cx<R>;
  __shared__ C_ T[kHrdPanel][kHrdPanel + 1];
  __shared__ C_ s_w[kHrdPanel];
  const C_* A = Aall + blockIdx.x * a_bs;
  const C_* tau = tau_all + (long long)blockIdx.x * n;
  C_* ws = Wsall + blockIdx.x * ws_bs;
  const long long nB = (long long)n * kHrdPanel;
  C_* V = ws;
  C_* Vc = ws + nB;
  C_* Tm = ws + 4 * nB;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x, nw = nt >> 5;
  for (int e = tid; e < kHrdPanel * (kHrdPanel + 1); e += nt) T[e / (kHrdPanel + 1)][e % (kHrdPanel + 1)] = cxzero<R>();
  for (long long e = tid; e < nB; e += nt) {
    const int r = (int)(e % n), j = (int)(e / n), c = k0 + j;
    C_ v = cxzero<R>();
    if (j < bb) {
      const C_ t = tau[c];
      if (!(t.x == R(0.0) && t.y == R(0.0))) {
        if (r == c + 1) v = cxone<R>();
        else if (r > c + 1) v = A[r + (long long)c * lda];
      }
    }
    V[e] = v;
    Vc[e] = cxconj(v);
  }
  __syncthreads();
  for (int j = 0; j < bb; ++j) {
    const int c = k0 + j;
    const C_ tj = tau[c];
    for (int l = warp; l < j; l += nw) {
      C_ acc = cxzero<R>();
      for (int r = c + 1 + lane; r < n; r += 32) acc = cxfma_conj(V[r + (long long)l * n], V[r + (long long)j * n], acc);
      acc.x = warp_sum(acc.x);
      acc.y = warp_sum(acc.y);
      if (lane == 0) s_w[l] = acc;
    }
    __syncthreads();
    if (tid < j) {
      C_ acc = cxzero<R>();
      for (int lp = tid; lp < j; ++lp) acc = acc + T[tid][lp] * s_w[lp];
      T[tid][j] = -(tj * acc);
    }
    if (tid == 0) T[j][j] = tj;
    __syncthreads();
  }
  for (int e = tid; e < kHrdPanel * kHrdPanel; e += nt) {
    const int r = e % kHrdPanel, cc = e / kHrdPanel;
    Tm[e] = (r < bb && cc < bb) ? T[r][cc] : cxzero<R>();
  }
}

// the reflectors' storage below the subdiagonal cleared, leaving H
template <class R>
__global__ void clear_below_subdiag_kernel(Cx<R>* __restrict__ Aall, int n, int lda, long long a_bs) {
  Cx<R>* A = Aall + blockIdx.y * a_bs;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * n;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    if (i > j + 1) A[i + (long long)j * lda] = cxzero<R>();
  }
}

// ------------------------------------------------------------------ 2. form Q = Z
template <class R>
__global__ void __launch_bounds__(1024) unghr_kernel(Cx<R>* __restrict__ Aall, int n, int lda,
                                                            long long a_bs, const Cx<R>* __restrict__ tau_all,
                                                            Cx<R>* __restrict__ Zall, int ldz, long long z_bs) {
  using C_ = Cx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C_* sv = reinterpret_cast<C_*>(smraw);
  C_* A = Aall + blockIdx.x * a_bs;
  C_* Z = Zall + blockIdx.x * z_bs;
  const C_* tau = tau_all + (long long)blockIdx.x * n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (long long e = tid; e < (long long)n * n; e += blockDim.x) {
    int i = (int)(e % n), j = (int)(e / n);
    Z[i + (long long)j * ldz] = (i == j) ? cxone<R>() : cxzero<R>();
  }
  __syncthreads();
  for (int k = n - 3; k >= 0; --k) {
    const int m = n - k - 1;
    const C_ t = tau[k];
    if (t.x == R(0.0) && t.y == R(0.0)) continue;
    for (int i = tid; i < m; i += blockDim.x) sv[i] = (i == 0) ? cxone<R>() : A[k + 1 + i + (long long)k * lda];
    __syncthreads();
    for (int j = warp; j < m; j += nw) {
      C_* cj = Z + (long long)(k + 1 + j) * ldz;
      const C_ acc = column_dot<R>(sv, cj + k + 1, m, lane);
      const C_ f = t * acc;
      for (int i0 = lane; i0 < m; i0 += 32 * kUnroll) {
        C_ val[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
          if (i0 + 32 * u < m) val[u] = cj[k + 1 + i0 + 32 * u];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
          if (i0 + 32 * u < m) cj[k + 1 + i0 + 32 * u] = val[u] - sv[i0 + 32 * u] * f;
      }
    }
    __syncthreads();
  }
  for (long long e = tid; e < (long long)n * n; e += blockDim.x) {
    int i = (int)(e % n), j = (int)(e / n);
    if (i > j + 1) A[i + (long long)j * lda] = cxzero<R>();
  }
}

// ---------------------------------------------------------- 3. Schur form by shifted QR
// Francis single-shift implicit QR on the Hessenberg H (complex), full Schur form: T in H,
// Schur vectors accumulated into Z. The subdiagonal is kept real so that every 2-element
// reflector has a real second coefficient. Deflation uses the standard small-subdiagonal test
// with the Ahues-Tisseur refinement; shifts are Wilkinson shifts with exceptional shifts after
// 10 and 20 stalled iterations.
//
// One bulge step = lane 0 builds the 2x2 reflector, then the CTA applies it to rows (k, k+1),
// to columns (k, k+1) and to Z. The step is latency bound (three barriers and a serial
// reflector), so the kernel is sized to run several matrices per SM: their steps interleave
// and keep the FP64 (or, for df64, FP32) pipes busy.
//
// Reflector of (alpha, x) with x real, as used by the chase: beta = -sign(Re alpha)|(alpha, x)|,
// tau = (beta - alpha)/beta, v2 = x/(alpha - beta); one square root and two reciprocals.
template <class R> struct Rot { Cx<R> t1, v2; R t2, beta; bool identity; };
template <class R> __device__ __forceinline__ Rot<R> chase_reflector(Cx<R> alpha, R x) {
  Rot<R> r;
  // scaled by m = max(|Re a|, |Im a|, |x|) so that squares stay in range (the double-float form
  // has FP32's exponent range, where a nearly converged bulge of 1e-25 would square to zero)
  const R m = rmax(rmax(rabs(alpha.x), rabs(alpha.y)), rabs(x));
  if ((x == R(0.0) && alpha.y == R(0.0)) || !(m > RealT<R>::tiny())) {
    r.identity = true; r.t1 = cxzero<R>(); r.v2 = cxzero<R>(); r.t2 = R(0.0); r.beta = alpha.x;
    return r;
  }
  const R im = R(1.0) / m;
  const R ax = alpha.x * im, ay = alpha.y * im, xs = x * im;
  R nrm = rsqrt_(ax * ax + ay * ay + xs * xs);
  R bs = (ax >= R(0.0)) ? -nrm : nrm;                         // beta / m
  R ib = R(1.0) / bs;
  Cx<R> d = cxmk<R>(ax - bs, ay);                              // (alpha - beta) / m
  R idd = R(1.0) / (d.x * d.x + d.y * d.y);
  r.identity = false;
  r.beta = bs * m;
  r.t1 = cxmk<R>((bs - ax) * ib, -(ay * ib));
  r.v2 = cxmk<R>(xs * d.x * idd, -(xs * d.y * idd));            // x / (alpha - beta)
  r.t2 = -(xs * ib);                                           // Re(t1 v2) = -x / beta
  return r;
}

// One sweep of the bulge chase with the workers' operands carried in registers (FP32 form).
// Every worker owns up to kCarry element pairs for the whole sweep, with a step-invariant map:
// item e < n is row e of Z; item e = n + q is, while q >= k, column q + 2 of H (rows k, k+1:
// the left update) and, from step q + 1 on, row q of H (columns k, k+1: the right update).
// An item keeps the value it pairs with this step (cy) and the next one (n1, loaded one step
// ahead), so a step's critical path holds no memory read: it updates (cy, n1), stores the
// finished element, keeps the other and issues the load for the next step (an element no step
// touches in between). The two values that cross between threads go through shared memory,
// double buffered by step parity: H(k+1, k+2) from column k+2's item to the core lane, and
// H(k, k+1) from the core to the item of row k as it joins the right update. Results are those of
// the chunked loop in hseqr_kernel, operation for operation.
constexpr int kCarry = 4;
// largest QR-sweep CTA: 85 registers a thread, room for the carried pairs without spills
constexpr int kQrMaxThreads = 768;

// Algorithmic bytes of the QR sweeps, per real type (0 double, 1 float, 2 df64): every bulge step
// reads and writes each of its 2n - 2 element pairs' moving element once (the minimum of the
// single-shift sweep: Z's row, H's row or column carries the other element), so a step moves
// 2 (2n - 2) complex values. Each CTA adds its steps' bytes at the end.
__device__ unsigned long long g_qr_bytes[3];
template <class R> struct QrSlot;
template <> struct QrSlot<double> { static constexpr int v = 0; };
template <> struct QrSlot<float> { static constexpr int v = 1; };
template <> struct QrSlot<df64> { static constexpr int v = 2; };

template <class R>
__device__ void chase_sweep_carry(Cx<R>* __restrict__ H, int ldh, Cx<R>* __restrict__ Z, int ldz, int n, int l,
                                  int i, Cx<R>* s_t1, Cx<R>* s_v2, R* s_t2, Cx<R>* s_c01, Cx<R>* s_h01) {
  using C_ = Cx<R>;
  const int tid = threadIdx.x, warp = tid >> 5;
  auto h = [&](int r, int c) -> C_& { return H[r + (long long)c * ldh]; };
  const int wt = blockDim.x - 32, wid = tid - 32;
  const int nitems = 2 * n - 2;
  const C_ zero = cxzero<R>();
  C_ cy[kCarry], n1[kCarry];
  // core lane state: the 2 x 2 block at (k, k) and H(k+2, k+1) in shared memory (so that the
  // workers' registers are not spent on it); the elements two steps ahead, whose loads are in
  // flight across a step, in registers
  __shared__ C_ cs[5];
  enum { C00, C01, C10, C11, C21 };
  C_ p22 = zero, p32 = zero;
  if (warp > 0) {
#pragma unroll
    for (int u = 0; u < kCarry; ++u) {
      const int e = wid + u * wt;
      cy[u] = zero; n1[u] = zero;
      if (e >= nitems) continue;
      if (e < n) {
        cy[u] = Z[e + (long long)l * ldz]; n1[u] = Z[e + (long long)(l + 1) * ldz];
      } else {
        const int q = e - n;
        if (q < l) { cy[u] = h(q, l); n1[u] = h(q, l + 1); }
        else { cy[u] = h(l, q + 2); n1[u] = h(l + 1, q + 2); }
      }
    }
  } else if (tid == 0) {
    cs[C00] = h(l, l); cs[C01] = h(l, l + 1); cs[C10] = h(l + 1, l); cs[C11] = h(l + 1, l + 1);
    cs[C21] = (l + 2 <= i) ? h(l + 2, l + 1) : zero;
    if (l + 2 <= i) p22 = h(l + 2, l + 2);
    if (l + 3 <= i) p32 = h(l + 3, l + 2);
  }
  for (int k = l; k < i; ++k) {
    const int sl = k & 1, sn = sl ^ 1;
    const C_ t1 = s_t1[sl], v2 = s_v2[sl];
    const R t2 = s_t2[sl];
    const C_ t1c = cxconj(t1), v2c = cxconj(v2);
    if (warp == 0) {
      if (tid == 0) {
        const C_ c00 = cs[C00], c10 = cs[C10], c11 = cs[C11], c21 = cs[C21];
        const C_ c01 = (k > l) ? s_c01[sl] : cs[C01];
        const bool has2 = (k + 2 <= i);
        C_ sum = t1c * c00 + c10 * t2;             // left on columns k, k+1
        C_ h00 = c00 - sum, h10 = c10 - sum * v2;
        sum = t1c * c01 + c11 * t2;
        C_ h01 = c01 - sum, h11 = c11 - sum * v2;
        sum = t1 * h00 + h01 * t2;                 // right on rows k, k+1, k+2
        h00 = h00 - sum; h01 = h01 - sum * v2c;
        sum = t1 * h10 + h11 * t2;
        h10 = h10 - sum; h11 = h11 - sum * v2c;
        C_ h21 = has2 ? c21 : zero;
        sum = h21 * t2;
        const C_ h20 = -sum;
        h21 = h21 - sum * v2c;
        h(k, k) = h00; h(k, k + 1) = h01;
        s_h01[sn] = h01;
        if (k + 1 < i) {
          Rot<R> rn = chase_reflector(h10, h20.x);
          h(k + 1, k) = rn.identity ? h10 : cxmk<R>(rn.beta, R(0.0));
          h(k + 2, k) = zero;
          s_t1[sn] = rn.t1; s_v2[sn] = rn.v2; s_t2[sn] = rn.t2;
          cs[C00] = h11; cs[C10] = h21; cs[C11] = p22; cs[C21] = p32;
          p22 = (k + 3 <= i) ? h(k + 3, k + 3) : zero;
          p32 = (k + 4 <= i) ? h(k + 4, k + 3) : zero;
        } else {
          h(k + 1, k) = h10; h(k + 1, k + 1) = h11;
        }
      }
    } else {
#pragma unroll
      for (int u = 0; u < kCarry; ++u) {
        const int e = wid + u * wt;
        if (e >= nitems) continue;
        if (e < n) {                                                   // Z row e
          const C_ sum = t1 * cy[u] + n1[u] * t2;
          Z[e + (long long)k * ldz] = cy[u] - sum;
          cy[u] = n1[u] - sum * v2c;
          n1[u] = (k + 2 < n) ? Z[e + (long long)(k + 2) * ldz] : zero;
          continue;
        }
        const int q = e - n;
        if (q < k) {                                                   // H row q, right update
          if (q == k - 1 && k > l) cy[u] = s_h01[sl];                  // joins: n1 is its own
          const C_ sum = t1 * cy[u] + n1[u] * t2;
          h(q, k) = cy[u] - sum;
          cy[u] = n1[u] - sum * v2c;
          n1[u] = (k + 2 < n) ? h(q, k + 2) : zero;
        } else {                                                       // H column q + 2, left update
          const int j = q + 2;
          const C_ sum = t1c * cy[u] + n1[u] * t2;
          const C_ a = cy[u] - sum, b = n1[u] - sum * v2;
          h(k, j) = a;
          if (q == k) {              // last left step: H(k+1, k+2) to the core, then rows join
            h(k + 1, j) = b;
            s_c01[sn] = b;
            n1[u] = a;
          } else {
            cy[u] = b;
            n1[u] = (k + 2 < n) ? h(k + 2, j) : zero;
          }
        }
      }
    }
    __syncthreads();
  }
  // the carried elements of the last step
  if (warp > 0) {
#pragma unroll
    for (int u = 0; u < kCarry; ++u) {
      const int e = wid + u * wt;
      if (e >= nitems) continue;
      if (e < n) { Z[e + (long long)i * ldz] = cy[u]; continue; }
      const int q = e - n;
      if (q < i - 1) h(q, i) = cy[u];
      else if (q > i - 1) h(i, q + 2) = cy[u];
    }
  }
  __syncthreads();
}

template <class R>
__global__ void __launch_bounds__(kQrMaxThreads) hseqr_kernel(Cx<R>* __restrict__ Hall, int n, int ldh,
                                                            long long h_bs, Cx<R>* __restrict__ Zall, int ldz,
                                                            long long z_bs, Cx<R>* __restrict__ w_all,
                                                            int32_t* __restrict__ status, int st_div, int itmax) {
  using C_ = Cx<R>;
  extern __shared__ __align__(16) unsigned char smraw[];
  C_* sphase = reinterpret_cast<C_*>(smraw);
  __shared__ int ired[32];
  __shared__ C_ s_t1[2], s_v2[2], s_sc, s_c01[2], s_h01[2];
  __shared__ R s_t2[2];
  __shared__ int s_done;
  constexpr int kChunk = sizeof(R) <= 4 ? 4 : 2;   // worker items whose loads are issued together
  C_* H = Hall + blockIdx.x * h_bs;
  C_* Z = Zall + blockIdx.x * z_bs;
  C_* w = w_all + (long long)blockIdx.x * n;
  int32_t* st = status ? status + blockIdx.x / st_div : nullptr;
  const int tid = threadIdx.x, warp = tid >> 5;
  const R ulp = RealT<R>::eps();
  const R smlnum = RealT<R>::tiny() * (R((double)n) / ulp);
  auto h = [&](int i, int j) -> C_& { return H[i + (long long)j * ldh]; };
  // subdiagonal made real by a diagonal similarity D^-1 H D, |d_i| = 1, d_i = d_{i-1} sd_i/|sd_i|
  if (tid == 0) {
    C_ d = cxone<R>();
    sphase[0] = d;
    for (int r = 1; r < n; ++r) {
      C_ sd = h(r, r - 1);
      R a = cxabs(sd);
      // a subdiagonal below the safe range keeps a unit phase (its imaginary part is dropped)
      if (a > RealT<R>::tiny() && sd.y != R(0.0)) d = d * (sd * (R(1.0) / a));
      sphase[r] = d;
    }
  }
  __syncthreads();
  for (long long e = tid; e < (long long)n * n; e += blockDim.x) {
    int r = (int)(e % n), c = (int)(e / n);
    if (r <= c + 1) h(r, c) = (cxconj(sphase[r]) * h(r, c)) * sphase[c];
    Z[r + (long long)c * ldz] = Z[r + (long long)c * ldz] * sphase[c];
  }
  __syncthreads();
  for (int r = 1 + tid; r < n; r += blockDim.x) h(r, r - 1) = cxmk<R>(h(r, r - 1).x, R(0.0));
  __syncthreads();
  int i = n - 1;
  int total = 0;
  long long steps = 0;
  bool failed = false;
  while (i >= 0 && !failed) {
    int its = 0;
    for (;;) {
      // --- deflation: largest k in [1, i] with a negligible subdiagonal H(k, k-1)
      int cand = 0;
      for (int k = 1 + tid; k <= i; k += blockDim.x) {
        C_ sub = h(k, k - 1);
        bool small = false;
        if (cxabs1(sub) <= smlnum) {
          small = true;
        } else {
          R tst = cxabs1(h(k - 1, k - 1)) + cxabs1(h(k, k));
          if (tst == R(0.0)) {
            if (k - 2 >= 0) tst = tst + rabs(h(k - 1, k - 2).x);
            if (k + 1 <= i) tst = tst + rabs(h(k + 1, k).x);
          }
          if (rabs(sub.x) <= ulp * tst) {
            R ab = rmax(cxabs1(sub), cxabs1(h(k - 1, k)));
            R ba = rmin(cxabs1(sub), cxabs1(h(k - 1, k)));
            C_ dd = h(k - 1, k - 1) - h(k, k);
            R aa = rmax(cxabs1(h(k, k)), cxabs1(dd));
            R bb = rmin(cxabs1(h(k, k)), cxabs1(dd));
            R sx = aa + ab;
            if (ba * (ab / sx) <= rmax(smlnum, ulp * (bb * (aa / sx)))) small = true;
          }
        }
        if (small) cand = max(cand, k);
      }
      const int l = block_max_int(cand, ired);
      if (l >= i) break;
      if (tid == 0 && l > 0) h(l, l - 1) = cxzero<R>();
      if (its >= 60 || total >= itmax) { failed = true; break; }
      ++its; ++total;
      steps += i - l;
      // --- shift and first reflector vector (thread 0)
      if (tid == 0) {
        C_ t;
        if (its % 20 == 10) {
          R sx = R(0.75) * rabs(h(l + 1, l).x);
          t = cxmk<R>(sx, R(0.0)) + h(l, l);
        } else if (its % 20 == 0) {
          R sx = R(0.75) * rabs(h(i, i - 1).x);
          t = cxmk<R>(sx, R(0.0)) + h(i, i);
        } else {
          t = h(i, i);
          C_ u = cxsqrt(h(i - 1, i)) * cxsqrt(h(i, i - 1));
          R sx = cxabs1(u);
          if (sx != R(0.0)) {
            C_ x = (h(i - 1, i - 1) - t) * R(0.5);
            R sxx = cxabs1(x);
            sx = rmax(sx, cxabs1(x));
            C_ xs = x * (R(1.0) / sx), us = u * (R(1.0) / sx);
            C_ y = cxsqrt(xs * xs + us * us) * sx;
            if (sxx > R(0.0)) {
              C_ xn = x * (R(1.0) / sxx);
              if (xn.x * y.x + xn.y * y.y < R(0.0)) y = -y;
            }
            t = t - u * cxdiv(u, x + y);
          }
        }
        C_ h11s = h(l, l) - t;
        R h21 = h(l + 1, l).x;
        R sc = cxabs1(h11s) + rabs(h21);
        if (sc == R(0.0)) sc = R(1.0);
        R isc = R(1.0) / sc;
        // the first reflector of the sweep, from the shifted first column
        Rot<R> rf = chase_reflector(h11s * isc, h21 * isc);
        s_t1[l & 1] = rf.t1; s_v2[l & 1] = rf.v2; s_t2[l & 1] = rf.t2;
      }
      __syncthreads();
      // Bulge chase, one CTA barrier per step. Reflector k acts on rows/columns (k, k+1). The core
      // lane (thread 0) owns the elements where its left and right applications meet -- rows
      // k..min(k+2, i) of columns k, k+1 -- and, having updated them, builds reflector k+1 from
      // its own (k+1, k), (k+2, k) and publishes it (double-buffered in shared memory). The worker
      // warps (all but warp 0) apply reflector k everywhere else, in one phase, since those
      // elements are disjoint: rows k, k+1 of columns k+2..n-1 (left), rows 0..k-1 of columns
      // k, k+1 (right) and Z's columns k, k+1. Each worker issues the loads of up to kChunk items
      // before it updates any, so that one memory latency serves the chunk.
      const bool carry = sizeof(R) == 4 && 2 * n - 2 <= kCarry * ((int)blockDim.x - 32);
      if (carry) chase_sweep_carry<R>(H, ldh, Z, ldz, n, l, i, s_t1, s_v2, s_t2, s_c01, s_h01);
      for (int k = carry ? i : l; k < i; ++k) {
        const int sl = k & 1;
        const C_ t1 = s_t1[sl], v2 = s_v2[sl];
        const R t2 = s_t2[sl];
        const C_ t1c = cxconj(t1), v2c = cxconj(v2);
        if (warp == 0) {
          if (tid == 0) {
            const bool has2 = (k + 2 <= i);
            C_ h00 = h(k, k), h01 = h(k, k + 1), h10 = h(k + 1, k), h11 = h(k + 1, k + 1);
            C_ h21 = has2 ? h(k + 2, k + 1) : cxzero<R>();
            C_ sum = t1c * h00 + h10 * t2;             // left on columns k, k+1
            h00 = h00 - sum; h10 = h10 - sum * v2;
            sum = t1c * h01 + h11 * t2;
            h01 = h01 - sum; h11 = h11 - sum * v2;
            sum = t1 * h00 + h01 * t2;                 // right on rows k, k+1, k+2
            h00 = h00 - sum; h01 = h01 - sum * v2c;
            sum = t1 * h10 + h11 * t2;
            h10 = h10 - sum; h11 = h11 - sum * v2c;
            sum = h21 * t2;                            // (k+2, k) is zero before this step
            C_ h20 = -sum;
            h21 = h21 - sum * v2c;
            h(k, k) = h00; h(k, k + 1) = h01; h(k + 1, k + 1) = h11;
            if (has2) h(k + 2, k + 1) = h21;
            if (k + 1 < i) {
              Rot<R> rn = chase_reflector(h10, h20.x);
              h(k + 1, k) = rn.identity ? h10 : cxmk<R>(rn.beta, R(0.0));
              h(k + 2, k) = cxzero<R>();
              s_t1[sl ^ 1] = rn.t1; s_v2[sl ^ 1] = rn.v2; s_t2[sl ^ 1] = rn.t2;
            } else {
              h(k + 1, k) = h10;
              if (has2) h(k + 2, k) = h20;
            }
          }
        } else {
          const int wt = blockDim.x - 32, wid = tid - 32;
          const int nL = max(0, n - (k + 2)), nR = k, total = nL + nR + n;
          for (int base = wid; base < total; base += kChunk * wt) {
            C_* pa[kChunk];
            C_* pb[kChunk];
            C_ a[kChunk], b[kChunk];
#pragma unroll
            for (int u = 0; u < kChunk; ++u) {
              int e = base + u * wt;
              if (e < nL) { pa[u] = &h(k, k + 2 + e); pb[u] = pa[u] + 1; }
              else if (e < nL + nR) { e -= nL; pa[u] = &h(e, k); pb[u] = &h(e, k + 1); }
              else if (e < total) { e -= nL + nR; pa[u] = Z + e + (long long)k * ldz; pb[u] = pa[u] + ldz; }
              else { pa[u] = nullptr; pb[u] = nullptr; }
            }
#pragma unroll
            for (int u = 0; u < kChunk; ++u)
              if (pa[u]) { a[u] = *pa[u]; b[u] = *pb[u]; }
#pragma unroll
            for (int u = 0; u < kChunk; ++u) {
              if (!pa[u]) continue;
              if (base + u * wt < nL) {
                const C_ sum = t1c * a[u] + b[u] * t2;
                *pa[u] = a[u] - sum; *pb[u] = b[u] - sum * v2;
              } else {
                const C_ sum = t1 * a[u] + b[u] * t2;
                *pa[u] = a[u] - sum; *pb[u] = b[u] - sum * v2c;
              }
            }
          }
        }
        __syncthreads();
      }
      // make H(i, i-1) real again
      if (tid == 0) {
        C_ sd = h(i, i - 1);
        s_done = 0;
        if (sd.y != R(0.0)) {
          R a = cxabs(sd);
          if (a > RealT<R>::tiny()) {
            h(i, i - 1) = cxmk<R>(a, R(0.0));
            s_sc = sd * (R(1.0) / a);
            s_done = 1;
          } else {
            h(i, i - 1) = cxmk<R>(sd.x, R(0.0));      // below the safe range: negligible
          }
        }
      }
      __syncthreads();
      if (s_done) {
        const C_ sc = s_sc;
        for (int j = i + 1 + tid; j < n; j += blockDim.x) h(i, j) = cxconj(sc) * h(i, j);
        for (int j = tid; j < i; j += blockDim.x) h(j, i) = sc * h(j, i);
        for (int j = tid; j < n; j += blockDim.x) Z[j + (long long)i * ldz] = sc * Z[j + (long long)i * ldz];
      }
      __syncthreads();
    }
    if (failed) break;
    if (tid == 0) w[i] = h(i, i);
    __syncthreads();
    i -= 1;
  }
  if (failed) {
    for (int j = tid; j <= i; j += blockDim.x) w[j] = cxmk<R>(R(NAN), R(NAN));
    if (tid == 0) wb_flag(st, WB_ST_NOCONV);
  }
  if (tid == 0)
    atomicAdd(&g_qr_bytes[QrSlot<R>::v],
              (unsigned long long)steps * (unsigned long long)(2 * n - 2) * 2ULL * sizeof(C_));
}

// -------------------------------------------------- 4. eigenvectors of the triangular T
// X[:, k] solves (T[0:k,0:k] - T(k,k) I) x = -T[0:k, k] with x_k = 1, x_j = 0 for j > k.
// One warp per column; tiny pivots are replaced by max(ulp |T(k,k)|, smlnum).
template <class R>
__global__ void __launch_bounds__(256) trevc_kernel(const Cx<R>* __restrict__ Tall, int n, int ldt,
                                                    long long t_bs, Cx<R>* __restrict__ Xall, int ldx,
                                                    long long x_bs, int batch) {
  using C_ = Cx<R>;
  const int warps_per_block = blockDim.x >> 5;
  long long gw = (long long)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), k = (int)(gw % n);
  const C_* T = Tall + b * t_bs;
  C_* x = Xall + b * x_bs + (long long)k * ldx;
  const R ulp = RealT<R>::eps();
  const R smlnum = RealT<R>::tiny() * (R((double)n) / ulp);
  const C_ lam = T[k + (long long)k * ldt];
  const R smin = rmax(ulp * cxabs1(lam), smlnum);
  for (int r = lane; r < n; r += 32) {
    C_ v;
    if (r < k) v = -T[r + (long long)k * ldt];
    else v = (r == k) ? cxone<R>() : cxzero<R>();
    x[r] = v;
  }
  __syncwarp();
  // back-substitution with rescaling: whenever a component exceeds `big`, the whole column (the
  // solved part and the remaining right-hand side) is scaled down, since an eigenvector is only
  // defined up to scale. This keeps the double-float form (FP32 exponent range) finite where
  // nearly equal eigenvalues make the triangular solve grow.
  const R big = RealT<R>::big();
  for (int j = k - 1; j >= 0; --j) {
    C_ xj = cxzero<R>();
    if (lane == (j & 31)) {
      C_ d = T[j + (long long)j * ldt] - lam;
      if (cxabs1(d) < smin) d = cxmk<R>(smin, R(0.0));
      xj = cxdiv(x[j], d);
      x[j] = xj;
    }
    xj.x = shfl_idx(xj.x, j & 31);
    xj.y = shfl_idx(xj.y, j & 31);
    R mag = cxabs1(xj);
    if (mag > big) {
      const R sc = R(1.0) / mag;
      __syncwarp();
      for (int r = lane; r <= k; r += 32) x[r] = x[r] * sc;
      xj = xj * sc;
      __syncwarp();
    }
    const C_* tc = T + (long long)j * ldt;
    for (int r = lane; r < j; r += 32) x[r] = x[r] - xj * tc[r];
    __syncwarp();
  }
}

// ------------------------------------------------------------- 5. column normalisation
template <class R>
__global__ void normalize_columns_kernel(Cx<R>* __restrict__ Wall, int n, int ldw, long long w_bs, int batch) {
  using C_ = Cx<R>;
  const int warps_per_block = blockDim.x >> 5;
  long long gw = (long long)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), k = (int)(gw % n);
  C_* c = Wall + b * w_bs + (long long)k * ldw;
  R s = R(0.0);
  for (int r = lane; r < n; r += 32) s = s + cxabs2(c[r]);
  s = warp_sum(s);
  R inv = (s > R(0.0)) ? R(1.0) / rsqrt_(s) : R(1.0);
  for (int r = lane; r < n; r += 32) c[r] = c[r] * inv;
}

// Live timing of the QR-sweep launches (per real type), for the benchmark's roofline: CUDA
// events recorded on the launching stream around every hseqr launch while profiling is on.
namespace {
struct QrProfile {
  bool on = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[3];
};
QrProfile g_qrp;
std::mutex g_qrp_mutex;
}  // namespace

void qr_profile(bool on) {
  std::lock_guard<std::mutex> lock(g_qrp_mutex);
  for (auto& v : g_qrp.ev)
    for (auto& e : v) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto& v : g_qrp.ev) v.clear();
  unsigned long long zero[3] = {0, 0, 0};
  cudaMemcpyToSymbol(g_qr_bytes, zero, sizeof(zero));
  g_qrp.on = on;
}

int qr_profile_read(int slot, double* ms, long long* launches, double* bytes) {
  if (slot < 0 || slot > 2) return 1;
  std::lock_guard<std::mutex> lock(g_qrp_mutex);
  double t = 0.0;
  for (auto& e : g_qrp.ev[slot]) {
    float x = 0.f;
    if (cudaEventSynchronize(e.second) != cudaSuccess || cudaEventElapsedTime(&x, e.first, e.second) != cudaSuccess) {
      cudaGetLastError();
      return 2;
    }
    t += x;
  }
  unsigned long long b[3] = {0, 0, 0};
  if (cudaMemcpyFromSymbol(b, g_qr_bytes, sizeof(b)) != cudaSuccess) { cudaGetLastError(); return 2; }
  *ms = t;
  *launches = (long long)g_qrp.ev[slot].size();
  *bytes = (double)b[slot];
  return 0;
}

// Threads of one QR-sweep CTA. A bulge step has about 2n independent element pairs to update,
// one memory latency deep; the fewer matrices share an SM, the more threads each needs to keep
// enough loads in flight. The tunable WB_TUNE_QR_THREADS overrides the choice (the autotuner sets it).
int qr_threads(int batch, int n, bool carried) {
  const int forced = tuning(kTuneQrThreads);
  if (forced >= 64 && forced <= kQrMaxThreads && forced % 32 == 0) return forced;
  const int per_sm = (batch + sm_count() - 1) / sm_count();
  int t = per_sm <= 1 ? kQrMaxThreads : per_sm <= 2 ? 512 : 256;
  while (t > 128 && t / 2 >= 2 * n) t /= 2;       // small matrices: no idle warps
  if (carried) {                                  // enough workers to hold every pair in registers
    const int need = ((2 * n - 2 + kCarry - 1) / kCarry + 31) / 32 * 32 + 32;
    if (need <= kQrMaxThreads && need > t) t = need;
  }
  return t;
}

// Threads of one Hessenberg-reduction (and Q-forming) CTA: one warp per trailing column, so as
// many warps as fit when few matrices share an SM. WB_TUNE_HRD_THREADS overrides the choice.
int hrd_threads(int batch, int n) {
  const int forced = tuning(kTuneHrdThreads);
  if (forced >= 64 && forced <= 1024 && forced % 32 == 0) return forced;
  const int per_sm = (batch + sm_count() - 1) / sm_count();
  int t = per_sm <= 1 ? 1024 : per_sm <= 2 ? 512 : 256;
  while (t > 128 && t / 32 > n) t /= 2;
  return t;
}

template <class R>
void geev_schur(cudaStream_t s, int batch, int n, Cx<R>* A, int lda, long long a_bs, Cx<R>* Z, int ldz,
                long long z_bs, Cx<R>* w, Cx<R>* tau, int32_t* status, int st_div, Cx<R>* ws, long long ws_bs) {
  if (batch <= 0 || n <= 0) return;
  size_t sm = 2 * (size_t)n * sizeof(Cx<R>);
  cudaFuncSetAttribute(gehrd_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  cudaFuncSetAttribute(unghr_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  const int th = hrd_threads(batch, n);
  // the FP32 form at n >= 192 reduces in panels (Z, not yet formed, holds the panels' scratch:
  // 5 n kHrdPanel + kHrdPanel^2 elements, within n * ldz from n = 161 on)
  const bool blocked = sizeof(R) == 4 && n >= 192 && ldz >= n && tuning(kTuneHrdBlocked) != 1;
  if (blocked) {
    cudaFuncSetAttribute(gehrd_panel_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    const int BB = kHrdPanel;
    const long long nB = (long long)n * BB;
    Cx<R>* V = Z;
    Cx<R>* Vc = Z + nB;
    Cx<R>* Y = Z + 2 * nB;
    Cx<R>* Wm = Z + 3 * nB;
    Cx<R>* Xm = Z + 4 * nB;
    Cx<R>* TH = Z + 5 * nB;
    const double2 one = make_double2(1.0, 0.0), mone = make_double2(-1.0, 0.0), zero = make_double2(0.0, 0.0);
    for (int k = 0; k + 2 < n; k += BB) {
      const int bb = min(BB, n - 2 - k);
      gehrd_panel_kernel<R><<<batch, th, sm, s>>>(A, n, lda, a_bs, tau, k, bb, Z, z_bs); note_launch();
      const int c0 = k + bb, m = n - c0, rows = n - k - 1;
      if (m <= 0) continue;
      Cx<R>* Ac = A + (long long)c0 * lda;
      // A[:, c0:] -= Y conj(V[c0:, :])^T
      gemm<R>(s, batch, n, m, bb, mone, Y, 1, n, z_bs, Vc + c0, n, 1, z_bs, one, Ac, 1, lda, a_bs);
      // W = V[k+1:, :]^H A[k+1:, c0:];  X = T^H W;  A[k+1:, c0:] -= V[k+1:, :] X
      gemm<R>(s, batch, bb, m, rows, one, Vc + (k + 1), n, 1, z_bs, Ac + (k + 1), 1, lda, a_bs, zero, Wm, 1, BB, z_bs);
      gemm<R>(s, batch, bb, m, bb, one, TH, 1, BB, z_bs, Wm, 1, BB, z_bs, zero, Xm, 1, BB, z_bs);
      gemm<R>(s, batch, rows, m, bb, mone, V + (k + 1), 1, n, z_bs, Xm, 1, BB, z_bs, one, Ac + (k + 1), 1, lda, a_bs);
    }
  } else {
    gehrd_kernel<R><<<batch, th, sm, s>>>(A, n, lda, a_bs, tau); note_launch();
  }
  // Q in panels when the caller lends scratch (5 n kHrdPanel + kHrdPanel^2 elements a matrix)
  if (blocked && ws && ws_bs >= 5LL * n * kHrdPanel + kHrdPanel * kHrdPanel) {
    const int BB = kHrdPanel;
    const long long nB = (long long)n * BB;
    Cx<R>* V = ws;
    Cx<R>* Vc = ws + nB;
    Cx<R>* Wm = ws + 2 * nB;
    Cx<R>* Xm = ws + 3 * nB;
    Cx<R>* Tm = ws + 4 * nB;
    const double2 one = make_double2(1.0, 0.0), mone = make_double2(-1.0, 0.0), zero = make_double2(0.0, 0.0);
    set_identity<R>(s, batch, n, Z, ldz, z_bs);
    const int nk = n - 2;                                  // reflectors 0 .. n - 3
    for (int k0 = ((nk - 1) / BB) * BB; k0 >= 0; k0 -= BB) {
      const int bb = min(BB, nk - k0), rows = n - k0 - 1;
      unghr_panel_kernel<R><<<batch, th, 0, s>>>(A, n, lda, a_bs, tau, k0, bb, ws, ws_bs); note_launch();
      Cx<R>* Zb = Z + (k0 + 1) + (long long)(k0 + 1) * ldz;
      // W = V[k0+1:, :]^H Z_blk;  X = T W;  Z_blk -= V[k0+1:, :] X
      gemm<R>(s, batch, bb, rows, rows, one, Vc + (k0 + 1), n, 1, ws_bs, Zb, 1, ldz, z_bs, zero, Wm, 1, BB, ws_bs);
      gemm<R>(s, batch, bb, rows, bb, one, Tm, 1, BB, ws_bs, Wm, 1, BB, ws_bs, zero, Xm, 1, BB, ws_bs);
      gemm<R>(s, batch, rows, rows, bb, mone, V + (k0 + 1), 1, n, ws_bs, Xm, 1, BB, ws_bs, one, Zb, 1, ldz, z_bs);
    }
    const unsigned gx = (unsigned)min((long long)sm_count(), ((long long)n * n + 255) / 256);
    clear_below_subdiag_kernel<R><<<dim3(gx, batch), 256, 0, s>>>(A, n, lda, a_bs); note_launch();
  } else {
    unghr_kernel<R><<<batch, th, sm, s>>>(A, n, lda, a_bs, tau, Z, ldz, z_bs); note_launch();
  }
  int itmax = 30 * (n > 10 ? n : 10);
  size_t sm2 = (size_t)n * sizeof(Cx<R>);
  cudaFuncSetAttribute(hseqr_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  bool timed = false;
  {
    std::lock_guard<std::mutex> lock(g_qrp_mutex);
    if (g_qrp.on && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
      timed = true;
      g_qrp.ev[QrSlot<R>::v].push_back({e0, e1});
    }
  }
  if (timed) cudaEventRecord(e0, s);
  hseqr_kernel<R><<<batch, qr_threads(batch, n, sizeof(R) == 4), sm2, s>>>(A, n, lda, a_bs, Z, ldz, z_bs, w, status,
                                                           st_div < 1 ? 1 : st_div, itmax); note_launch();
  if (timed) cudaEventRecord(e1, s);
}

template <class R>
void trevc(cudaStream_t s, int batch, int n, const Cx<R>* T, int ldt, long long t_bs, Cx<R>* X, int ldx,
           long long x_bs) {
  long long warps = (long long)batch * n;
  if (warps <= 0) return;
  trevc_kernel<R><<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(T, n, ldt, t_bs, X, ldx, x_bs, batch); note_launch();
}

template <class R>
void normalize_columns(cudaStream_t s, int batch, int n, Cx<R>* W, int ldw, long long w_bs) {
  long long warps = (long long)batch * n;
  if (warps <= 0) return;
  normalize_columns_kernel<R><<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(W, n, ldw, w_bs, batch); note_launch();
}

// double2 wrappers of the plain FP64 path
void zgeev_schur(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs, cplx* Z, int ldz,
                 long long z_bs, cplx* w, cplx* tau, int32_t* status, int st_div) {
  geev_schur<double>(s, batch, n, (Cx<double>*)A, lda, a_bs, (Cx<double>*)Z, ldz, z_bs, (Cx<double>*)w,
                     (Cx<double>*)tau, status, st_div);
}
void ztrevc(cudaStream_t s, int batch, int n, const cplx* T, int ldt, long long t_bs, cplx* X, int ldx,
            long long x_bs) {
  trevc<double>(s, batch, n, (const Cx<double>*)T, ldt, t_bs, (Cx<double>*)X, ldx, x_bs);
}
void znormalize_columns(cudaStream_t s, int batch, int n, cplx* W, int ldw, long long w_bs) {
  normalize_columns<double>(s, batch, n, (Cx<double>*)W, ldw, w_bs);
}

#define WB_EIG_INST(R)                                                                                   \
  template void geev_schur<R>(cudaStream_t, int, int, Cx<R>*, int, long long, Cx<R>*, int, long long,     \
                              Cx<R>*, Cx<R>*, int32_t*, int, Cx<R>*, long long);                          \
  template void trevc<R>(cudaStream_t, int, int, const Cx<R>*, int, long long, Cx<R>*, int, long long);  \
  template void normalize_columns<R>(cudaStream_t, int, int, Cx<R>*, int, long long);
WB_EIG_INST(double)
WB_EIG_INST(float)
WB_EIG_INST(df64)

}  // namespace wb
