// Batched complex non-Hermitian eigen-decomposition, FP64, one CTA per matrix.
//
// The layer operator Omega^2 of every (solve, layer) pair is decomposed as
//   Omega^2 = Z T Z^H  (Hessenberg reduction, then Francis single-shift QR to Schur form)
//   Omega^2 W = W diag(w),  W = Z X  (X: eigenvectors of the triangular T by back-substitution)
// which is the factorisation LAPACK's zgeev performs for numpy.linalg.eig (right vectors only).
//
// GB300 note: FP64 runs at ~1 TFLOP/s, i.e. about 2 FP64 FMAs per clock per SM. A rotation
// applied across a row/column of a few hundred elements costs more in FP64 issue than in
// latency, so a plain one-CTA-per-matrix layout with the matrix resident in L2/HBM keeps the
// FP64 pipe busy; several CTAs per SM overlap each other's synchronisation latency.
//
// Every iteration is capped; a matrix that hits the cap gets WB_ST_NOCONV in its status word
// and NaN eigenvalues, and the kernel returns normally.
#include "wb_common.cuh"
#include "wb_kernels.h"

namespace wb {

constexpr int EIG_THREADS = 256;

__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    red[0] = s;
  }
  __syncthreads();
  double r = red[0];
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

// Householder reflector for (alpha, x): returns beta (real), tau and scales x in place so
// that (I - tau v v^H)^H (alpha; x) = (beta; 0), v = (1; x_scaled).
struct Refl { double beta; cplx tau; cplx scale; bool identity; };
__device__ __forceinline__ Refl make_reflector(cplx alpha, double xnorm) {
  Refl r;
  if (xnorm == 0.0 && alpha.y == 0.0) {
    r.identity = true; r.beta = alpha.x; r.tau = cmk(0.0, 0.0); r.scale = cmk(0.0, 0.0);
    return r;
  }
  double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
  double beta = (alpha.x >= 0.0) ? -nrm : nrm;
  r.identity = false;
  r.beta = beta;
  r.tau = cmk((beta - alpha.x) / beta, -alpha.y / beta);
  r.scale = cinv(cmk(alpha.x - beta, alpha.y));
  return r;
}

// ------------------------------------------------------------- 1. Hessenberg reduction
// H := Q^H A Q, reflectors stored below the subdiagonal (v_0 = 1 implicit), tau[k].
__global__ void __launch_bounds__(EIG_THREADS) zgehrd_kernel(cplx* __restrict__ Aall, int n, int lda,
                                                             long long a_bs, cplx* __restrict__ tau_all,
                                                             cplx* __restrict__ work_all) {
  extern __shared__ cplx sv[];         // v (n), then y/z (n)
  __shared__ double red[32];
  __shared__ cplx s_tau;
  cplx* A = Aall + blockIdx.x * a_bs;
  cplx* tau = tau_all + (long long)blockIdx.x * n;
  cplx* sy = sv + n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;           // reflector length
    cplx* col = A + (long long)k * lda;
    double part = 0.0;
    for (int i = k + 2 + tid; i < n; i += blockDim.x) part += cabs2(col[i]);
    double xn2 = block_sum(part, red);
    cplx alpha = col[k + 1];
    Refl r = make_reflector(alpha, sqrt(xn2));
    if (r.identity) {
      if (tid == 0) tau[k] = cmk(0.0, 0.0);
      __syncthreads();
      continue;
    }
    for (int i = k + 2 + tid; i < n; i += blockDim.x) {
      cplx v = cmul(col[i], r.scale);
      col[i] = v;
      sv[i - k - 1] = v;
    }
    if (tid == 0) {
      sv[0] = cmk(1.0, 0.0);
      col[k + 1] = cmk(r.beta, 0.0);
      tau[k] = r.tau;
      s_tau = r.tau;
    }
    __syncthreads();
    const cplx t = s_tau;
    // right: y = A[:, k+1:n] v ; A[:, k+1:n] -= t y v^H  (all rows)
    for (int i = tid; i < n; i += blockDim.x) {
      cplx acc = cmk(0.0, 0.0);
      for (int j = 0; j < m; ++j) acc = cfma(A[i + (long long)(k + 1 + j) * lda], sv[j], acc);
      sy[i] = cmul(t, acc);
    }
    __syncthreads();
    for (int j = warp; j < m; j += nw) {
      cplx* cj = A + (long long)(k + 1 + j) * lda;
      cplx vjc = cconj(sv[j]);
      for (int i = lane; i < n; i += 32) cj[i] = csub(cj[i], cmul(sy[i], vjc));
    }
    __syncthreads();
    // left: z_j = v^H A[k+1:n, j] ; A[k+1:n, j] -= conj(t) v z_j   for j = k+1 .. n-1
    const cplx tc = cconj(t);
    for (int j = warp; j < m; j += nw) {
      cplx* cj = A + (long long)(k + 1 + j) * lda;
      cplx acc = cmk(0.0, 0.0);
      for (int i = lane; i < m; i += 32) acc = cfma_conj(sv[i], cj[k + 1 + i], acc);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
      }
      cplx f = cmul(tc, acc);
      for (int i = lane; i < m; i += 32) cj[k + 1 + i] = csub(cj[k + 1 + i], cmul(sv[i], f));
    }
    __syncthreads();
  }
  (void)work_all;
}

// ------------------------------------------------------------------ 2. form Q = Z
// Z = H_0 H_1 ... H_{n-3} by backward accumulation; then clears the reflectors from A so that
// A holds the Hessenberg matrix only.
__global__ void __launch_bounds__(EIG_THREADS) zunghr_kernel(cplx* __restrict__ Aall, int n, int lda,
                                                             long long a_bs, const cplx* __restrict__ tau_all,
                                                             cplx* __restrict__ Zall, int ldz, long long z_bs) {
  extern __shared__ cplx sv[];
  cplx* A = Aall + blockIdx.x * a_bs;
  cplx* Z = Zall + blockIdx.x * z_bs;
  const cplx* tau = tau_all + (long long)blockIdx.x * n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (long long e = tid; e < (long long)n * n; e += blockDim.x) {
    int i = (int)(e % n), j = (int)(e / n);
    Z[i + (long long)j * ldz] = cmk(i == j ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int k = n - 3; k >= 0; --k) {
    const int m = n - k - 1;
    const cplx t = tau[k];
    if (t.x == 0.0 && t.y == 0.0) continue;
    for (int i = tid; i < m; i += blockDim.x)
      sv[i] = (i == 0) ? cmk(1.0, 0.0) : A[k + 1 + i + (long long)k * lda];
    __syncthreads();
    // Z[k+1:n, k+1:n] -= t v (v^H Z[k+1:n, k+1:n]); columns j <= k untouched (identity there)
    for (int j = warp; j < m; j += nw) {
      cplx* cj = Z + (long long)(k + 1 + j) * ldz;
      cplx acc = cmk(0.0, 0.0);
      for (int i = lane; i < m; i += 32) acc = cfma_conj(sv[i], cj[k + 1 + i], acc);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, off);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, off);
      }
      cplx f = cmul(t, acc);
      for (int i = lane; i < m; i += 32) cj[k + 1 + i] = csub(cj[k + 1 + i], cmul(sv[i], f));
    }
    __syncthreads();
  }
  // clear the reflector storage below the subdiagonal
  for (long long e = tid; e < (long long)n * n; e += blockDim.x) {
    int i = (int)(e % n), j = (int)(e / n);
    if (i > j + 1) A[i + (long long)j * lda] = cmk(0.0, 0.0);
  }
}

// ---------------------------------------------------------- 3. Schur form by shifted QR
// Francis single-shift implicit QR on the Hessenberg H (complex), full Schur form: T in H,
// Schur vectors accumulated into Z. The subdiagonal is kept real so that each 2-element
// reflector has a real second coefficient. Deflation uses the standard small-subdiagonal test
// with the Ahues-Tisseur refinement; shifts are Wilkinson shifts with exceptional shifts after
// 10 and 20 stalled iterations.
__global__ void __launch_bounds__(EIG_THREADS) zhseqr_kernel(cplx* __restrict__ Hall, int n, int ldh,
                                                             long long h_bs, cplx* __restrict__ Zall, int ldz,
                                                             long long z_bs, cplx* __restrict__ w_all,
                                                             int32_t* __restrict__ status, int st_div,
                                                             int itmax) {
  __shared__ int ired[32];
  __shared__ cplx s_t1, s_v2;
  __shared__ double s_t2;
  __shared__ int s_l, s_m, s_done;
  __shared__ cplx s_v0, s_v1;
  cplx* H = Hall + blockIdx.x * h_bs;
  cplx* Z = Zall + blockIdx.x * z_bs;
  cplx* w = w_all + (long long)blockIdx.x * n;
  int32_t* st = status ? status + blockIdx.x / st_div : nullptr;
  const int tid = threadIdx.x;
  const double ulp = 2.220446049250313e-16;        // DBL_EPSILON
  const double safmin = 2.2250738585072014e-308;   // DBL_MIN
  const double smlnum = safmin * ((double)n / ulp);
  auto h = [&](int i, int j) -> cplx& { return H[i + (long long)j * ldh]; };
  // make every subdiagonal real with a diagonal similarity D^-1 H D, |d_i| = 1:
  // d_0 = 1, d_i = d_{i-1} * sd_i / |sd_i| (a prefix product of phases, computed by one thread)
  extern __shared__ cplx sphase[];
  if (tid == 0) {
    cplx d = cmk(1.0, 0.0);
    sphase[0] = d;
    for (int r = 1; r < n; ++r) {
      cplx sd = h(r, r - 1);
      double a = cabsv(sd);
      if (a > 0.0 && sd.y != 0.0) d = cmul(d, cscale(sd, 1.0 / a));
      sphase[r] = d;
    }
  }
  __syncthreads();
  for (long long e = tid; e < (long long)n * n; e += blockDim.x) {
    int r = (int)(e % n), c = (int)(e / n);
    if (r <= c + 1) h(r, c) = cmul(cmul(cconj(sphase[r]), h(r, c)), sphase[c]);
    Z[r + (long long)c * ldz] = cmul(Z[r + (long long)c * ldz], sphase[c]);
  }
  __syncthreads();
  for (int r = 1 + tid; r < n; r += blockDim.x) h(r, r - 1) = cmk(h(r, r - 1).x, 0.0);
  __syncthreads();
  int i = n - 1;
  int total = 0;
  bool failed = false;
  while (i >= 0 && !failed) {
    int its = 0;
    for (;;) {
      // --- deflation: largest k in [1, i] with a negligible subdiagonal H(k, k-1)
      int cand = 0;
      for (int k = 1 + tid; k <= i; k += blockDim.x) {
        cplx sub = h(k, k - 1);
        bool small = false;
        if (cabs1(sub) <= smlnum) {
          small = true;
        } else {
          double tst = cabs1(h(k - 1, k - 1)) + cabs1(h(k, k));
          if (tst == 0.0) {
            if (k - 2 >= 0) tst += fabs(h(k - 1, k - 2).x);
            if (k + 1 <= i) tst += fabs(h(k + 1, k).x);
          }
          if (fabs(sub.x) <= ulp * tst) {
            double ab = fmax(cabs1(sub), cabs1(h(k - 1, k)));
            double ba = fmin(cabs1(sub), cabs1(h(k - 1, k)));
            cplx dd = csub(h(k - 1, k - 1), h(k, k));
            double aa = fmax(cabs1(h(k, k)), cabs1(dd));
            double bb = fmin(cabs1(h(k, k)), cabs1(dd));
            double s = aa + ab;
            if (ba * (ab / s) <= fmax(smlnum, ulp * (bb * (aa / s)))) small = true;
          }
        }
        if (small) cand = max(cand, k);
      }
      const int l = block_max_int(cand, ired);
      if (l >= i) break;                          // H(i,i) isolated: converged
      if (tid == 0 && l > 0) h(l, l - 1) = cmk(0.0, 0.0);
      if (its >= 60 || total >= itmax) { failed = true; break; }
      ++its; ++total;
      // --- shift (thread 0)
      if (tid == 0) {
        cplx t;
        if (its % 20 == 10) {
          double s = 0.75 * fabs(h(l + 1, l).x);
          t = cadd(cmk(s, 0.0), h(l, l));
        } else if (its % 20 == 0) {
          double s = 0.75 * fabs(h(i, i - 1).x);
          t = cadd(cmk(s, 0.0), h(i, i));
        } else {
          // Wilkinson: eigenvalue of the trailing 2x2 block closer to H(i,i)
          t = h(i, i);
          cplx u = cmul(csqrt_p(h(i - 1, i)), csqrt_p(h(i, i - 1)));
          double s = cabs1(u);
          if (s != 0.0) {
            cplx x = cscale(csub(h(i - 1, i - 1), t), 0.5);
            double sx = cabs1(x);
            s = fmax(s, cabs1(x));
            cplx xs = cscale(x, 1.0 / s), us = cscale(u, 1.0 / s);
            cplx y = cscale(csqrt_p(cadd(cmul(xs, xs), cmul(us, us))), s);
            if (sx > 0.0) {
              cplx xn = cscale(x, 1.0 / sx);
              if (xn.x * y.x + xn.y * y.y < 0.0) y = cneg(y);
            }
            t = csub(t, cmul(u, cdiv(u, cadd(x, y))));
          }
        }
        // --- the bulge starts at the top of the active block
        const int m = l;
        cplx h11s = csub(h(l, l), t);
        double h21 = h(l + 1, l).x;
        double sc = cabs1(h11s) + fabs(h21);
        cplx v0 = cscale(h11s, 1.0 / sc);
        cplx v1 = cmk(h21 / sc, 0.0);
        s_m = m; s_l = l; s_v0 = v0; s_v1 = v1;
      }
      __syncthreads();
      const int m = s_m;
      // --- single-shift sweep from m to i-1
      for (int k = m; k < i; ++k) {
        if (tid == 0) {
          cplx a0, a1;
          if (k > m) { a0 = h(k, k - 1); a1 = h(k + 1, k - 1); } else { a0 = s_v0; a1 = s_v1; }
          Refl r = make_reflector(a0, cabsv(a1));
          cplx v2, t1;
          if (r.identity) { t1 = cmk(0.0, 0.0); v2 = cmk(0.0, 0.0); }
          else { t1 = r.tau; v2 = cmul(a1, r.scale); }
          if (k > m) { h(k, k - 1) = cmk(r.identity ? a0.x : r.beta, r.identity ? a0.y : 0.0); h(k + 1, k - 1) = cmk(0.0, 0.0); }
          s_t1 = t1; s_v2 = v2; s_t2 = cmul(t1, v2).x;
        }
        __syncthreads();
        const cplx t1 = s_t1, v2 = s_v2;
        const double t2 = s_t2;
        const cplx t1c = cconj(t1), v2c = cconj(v2);
        // left: rows k, k+1, columns k..n-1
        for (int j = k + tid; j < n; j += blockDim.x) {
          cplx a = h(k, j), b = h(k + 1, j);
          cplx sum = cadd(cmul(t1c, a), cscale(b, t2));
          h(k, j) = csub(a, sum);
          h(k + 1, j) = csub(b, cmul(sum, v2));
        }
        __syncthreads();
        // right: columns k, k+1, rows 0..min(k+2, i); and Z rows 0..n-1
        const int rlast = min(k + 2, i);
        for (int e = tid; e <= rlast + n; e += blockDim.x) {
          cplx* pa; cplx* pb;
          if (e <= rlast) { pa = &h(e, k); pb = &h(e, k + 1); }
          else { int j = e - rlast - 1; pa = Z + j + (long long)k * ldz; pb = Z + j + (long long)(k + 1) * ldz; }
          cplx a = *pa, b = *pb;
          cplx sum = cadd(cmul(t1, a), cscale(b, t2));
          *pa = csub(a, sum);
          *pb = csub(b, cmul(sum, v2c));
        }
        __syncthreads();
      }
      // make H(i, i-1) real again
      if (tid == 0) {
        cplx sd = h(i, i - 1);
        s_done = 0;
        if (sd.y != 0.0) {
          double a = cabsv(sd);
          h(i, i - 1) = cmk(a, 0.0);
          s_v0 = cdiv(sd, cmk(a, 0.0));
          s_done = 1;
        }
      }
      __syncthreads();
      if (s_done) {
        const cplx sc = s_v0;
        for (int j = i + 1 + tid; j < n; j += blockDim.x) h(i, j) = cmul(cconj(sc), h(i, j));
        for (int j = tid; j < i; j += blockDim.x) h(j, i) = cmul(sc, h(j, i));
        for (int j = tid; j < n; j += blockDim.x) Z[j + (long long)i * ldz] = cmul(sc, Z[j + (long long)i * ldz]);
      }
      __syncthreads();
    }
    if (failed) break;
    if (tid == 0) w[i] = h(i, i);
    __syncthreads();
    i -= 1;
  }
  if (failed) {
    for (int j = tid; j <= i; j += blockDim.x) w[j] = cmk(NAN, NAN);
    if (tid == 0) wb_flag(st, WB_ST_NOCONV);
  }
}

// -------------------------------------------------- 4. eigenvectors of the triangular T
// X[:, k] solves (T[0:k,0:k] - T(k,k) I) x = -T[0:k, k] with x_k = 1, x_j = 0 for j > k.
// One warp per column; tiny pivots are replaced by max(ulp |T(k,k)|, smlnum).
__global__ void __launch_bounds__(256) ztrevc_kernel(const cplx* __restrict__ Tall, int n, int ldt,
                                                     long long t_bs, cplx* __restrict__ Xall, int ldx,
                                                     long long x_bs, int batch) {
  const int warps_per_block = blockDim.x >> 5;
  long long gw = (long long)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), k = (int)(gw % n);
  const cplx* T = Tall + b * t_bs;
  cplx* x = Xall + b * x_bs + (long long)k * ldx;
  const double ulp = 2.220446049250313e-16;
  const double smlnum = 2.2250738585072014e-308 * ((double)n / ulp);
  const cplx lam = T[k + (long long)k * ldt];
  const double smin = fmax(ulp * cabs1(lam), smlnum);
  for (int r = lane; r < n; r += 32) {
    cplx v;
    if (r < k) v = cneg(T[r + (long long)k * ldt]);
    else v = cmk(r == k ? 1.0 : 0.0, 0.0);
    x[r] = v;
  }
  __syncwarp();
  for (int j = k - 1; j >= 0; --j) {
    cplx xj = cmk(0.0, 0.0);
    if (lane == (j & 31)) {
      cplx d = csub(T[j + (long long)j * ldt], lam);
      if (cabs1(d) < smin) d = cmk(smin, 0.0);
      xj = cdiv(x[j], d);
      x[j] = xj;
    }
    xj.x = __shfl_sync(0xffffffffu, xj.x, j & 31);
    xj.y = __shfl_sync(0xffffffffu, xj.y, j & 31);
    const cplx* tc = T + (long long)j * ldt;
    for (int r = lane; r < j; r += 32) x[r] = csub(x[r], cmul(xj, tc[r]));
    __syncwarp();
  }
}

// ------------------------------------------------------------- 5. column normalisation
__global__ void znormalize_columns_kernel(cplx* __restrict__ Wall, int n, int ldw, long long w_bs, int batch) {
  const int warps_per_block = blockDim.x >> 5;
  long long gw = (long long)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (gw >= (long long)batch * n) return;
  const int b = (int)(gw / n), k = (int)(gw % n);
  cplx* c = Wall + b * w_bs + (long long)k * ldw;
  double s = 0.0;
  for (int r = lane; r < n; r += 32) s += cabs2(c[r]);
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  double inv = (s > 0.0) ? 1.0 / sqrt(s) : 1.0;
  for (int r = lane; r < n; r += 32) c[r] = cscale(c[r], inv);
}

void zgeev_schur(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs, cplx* Z, int ldz,
                 long long z_bs, cplx* w, cplx* tau, int32_t* status, int st_div) {
  if (batch <= 0 || n <= 0) return;
  size_t sm = 2 * (size_t)n * sizeof(cplx);
  if (sm > 48 * 1024) {
    cudaFuncSetAttribute(zgehrd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    cudaFuncSetAttribute(zunghr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  }
  zgehrd_kernel<<<batch, EIG_THREADS, sm, s>>>(A, n, lda, a_bs, tau, nullptr); note_launch();
  zunghr_kernel<<<batch, EIG_THREADS, sm, s>>>(A, n, lda, a_bs, tau, Z, ldz, z_bs); note_launch();
  int itmax = 30 * (n > 10 ? n : 10);
  zhseqr_kernel<<<batch, EIG_THREADS, (size_t)n * sizeof(cplx), s>>>(A, n, lda, a_bs, Z, ldz, z_bs, w, status, st_div < 1 ? 1 : st_div, itmax); note_launch();
}

void ztrevc(cudaStream_t s, int batch, int n, const cplx* T, int ldt, long long t_bs, cplx* X, int ldx,
            long long x_bs) {
  long long warps = (long long)batch * n;
  if (warps <= 0) return;
  ztrevc_kernel<<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(T, n, ldt, t_bs, X, ldx, x_bs, batch); note_launch();
}

void znormalize_columns(cudaStream_t s, int batch, int n, cplx* W, int ldw, long long w_bs) {
  long long warps = (long long)batch * n;
  if (warps <= 0) return;
  znormalize_columns_kernel<<<(unsigned)((warps + 7) / 8), 256, 0, s>>>(W, n, ldw, w_bs, batch); note_launch();
}

}  // namespace wb
