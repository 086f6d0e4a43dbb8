// Stages B and C of the RCWA raster path, and the native orchestration of one batched solve.
//
// Stage B (per (solve, layer) pair): the layer operator Omega^2 (solve_2d.py:2377-2418), its
// eigen-decomposition (wb_eig.cu), q = mode_q(w) (conventions.py:186-249), the H-field modes
// V = Omega_R W / q (solve_2d.py:2445-2448) and the s/p rotation (solve_2d.py:2584-2616).
//
// Stage C (per solve): the reference cascades S-matrices with Redheffer stars
// (scattering.py:163-200, :1272-1293) and reads R and T off the final S11 / S21
// (scattering.py:907-994). Only those two blocks, applied to three incidence columns, are
// ever read, so the stars are evaluated bottom-up keeping the one block the next star needs:
// the reflection R_l seen from the gap above layer l,
//     P1 = bigW^-1 W_g (I + R_l+1),  P2 = bigV^-1 V_g (I - R_l+1),  M = P1 + P2,  N = P1 - P2
//     rho_b = N M^-1,  rho_t = X rho_b X,  X1 = (I - rho_t) bigW^-1,  X2 = (I + rho_t) bigV^-1
//     R_l = A^-1 B,  A = X1 W_g + X2 V_g,  B = -X1 W_g + X2 V_g
// with W_g, V_g the gap modes (scattering.py:128-160) and X = diag(exp(-k0 q d)). The transmitted
// amplitudes follow from one top-down pass with three right-hand sides. This is the same star
// algebra (equal in exact arithmetic; the tests hold it to the reference within 1e-10) at
// ~53 n^3 FP64 flops per layer instead of ~180 n^3.
//
// The mixed form (precision 1) runs stage B as an FP32 eigen-solve brought to FP64 accuracy by
// Newton steps against the FP64 operator (stage_b_newton), and stage C as the FP32 cascade whose
// amplitudes are refined against the stack's interface equations in double-float
// (stage_c_refined). Sections below, in order: ports, Omega^2, q/X, V, the cascade's elementwise
// kernels, the stage-B drivers, the cascade drivers, orchestration (solve_chunk), and the doors of
// wb_smm_solve and wb_layer_modes.
#include <vector>
#include <algorithm>
#include "wb_common.cuh"
#include "wb_kernels.h"
#include "wb_internal.h"
#include "wb_num.cuh"
#include "wb_trace.h"
#include <type_traits>

namespace wb {

static unsigned long long g_launches = 0;
void note_launch() { __atomic_add_fetch(&g_launches, 1ULL, __ATOMIC_RELAXED); }
long long launch_count() { return (long long)__atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

static int g_tuning[kTuneKeys] = {0};
int tuning(int key) { return (key >= 0 && key < kTuneKeys) ? __atomic_load_n(&g_tuning[key], __ATOMIC_RELAXED) : 0; }
void set_tuning(int key, int value) {
  if (key >= 0 && key < kTuneKeys) __atomic_store_n(&g_tuning[key], value, __ATOMIC_RELAXED);
}
int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return 148; }
  if (!cached[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 148;
    }
    cached[dev] = v;
  }
  return cached[dev];
}

// --------------------------------------------------------------------------- ports
// Per solve: order wavevectors, per-order s/p frame, half-space kz, gap waves and the diagonal
// S blocks of the superstrate->gap and gap->substrate interfaces. The incident wavevector is
// fixed by theta and phi in eps_inc (NULL: the superstrate); the mirrored stack of the
// scattering-matrix export keeps the original one while its half-spaces are swapped.
__global__ void ports_kernel(int B, int hu, int hv, const double* __restrict__ wavelength,
                             const double* __restrict__ period, const double* __restrict__ theta,
                             const double* __restrict__ phi, const cplx* __restrict__ eps_top,
                             const cplx* __restrict__ eps_bot, const cplx* __restrict__ eps_inc, PortVectors pv) {
  const int b = blockIdx.x;
  const int nu = 2 * hu + 1, nv = 2 * hv + 1, N = nu * nv, n = 2 * N;
  const double lam = wavelength[b];
  const cplx et = eps_top[b], eb = eps_bot[b];
  // lossless incidence medium: N_phase = sqrt(Re eps), k_inc = N sin(theta) (cos phi, sin phi)
  const double index = sqrt((eps_inc ? eps_inc[b] : et).x);
  const double st = sin(theta[b]);
  const double ph = phi[b];
  const double kix = index * st * cos(ph), kiy = index * st * sin(ph);
  const cplx nt = csqrt_p(et), nb = csqrt_p(eb);
  const cplx nt2 = cmul(nt, nt), nb2 = cmul(nb, nb);
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const int u = i % nu, v = i / nu;
    const double kx = kix + (double)(u - hu) * (lam / period[2 * b + 0]);
    const double ky = kiy + (double)(v - hv) * (lam / period[2 * b + 1]);
    // order_azimuth (conventions.py:1316-1431), real wavevectors
    double vphi;
    if (kx == 0.0) {
      if (ky == 0.0) {
        vphi = atan(sin(ph) / cos(ph)) + (cos(ph) < 0.0 ? 3.141592653589793 : 0.0);
      } else {
        vphi = (ky < 0.0 ? -1.5707963267948966 : 1.5707963267948966) - kx / ky;
      }
    } else {
      vphi = atan(ky / kx) + (kx < 0.0 ? 3.141592653589793 : 0.0);
    }
    double sn, cs;
    sincos(vphi, &sn, &cs);
    const double kpar = kx * kx + ky * ky;
    // boundary_kz (conventions.py:655-760): sqrt(n^2 - kpar^2), flipped where Re+Im < 0
    cplx kzt = csqrt_p(csub(nt2, cmk(kpar, 0.0)));
    if (kzt.x + kzt.y < 0.0) kzt = cneg(kzt);
    cplx kzb = csqrt_p(csub(nb2, cmk(kpar, 0.0)));
    if (kzb.x + kzb.y < 0.0) kzb = cneg(kzb);
    const double y = sqrt(1.0 + kx * kx + ky * ky);      // gap waves (scattering.py:128-160)
    const long long o = (long long)b * N + i, on = (long long)b * n;
    pv.kx[o] = kx; pv.ky[o] = ky; pv.c[o] = cs; pv.s[o] = sn;
    pv.kz_top[o] = kzt; pv.kz_bot[o] = kzb;
    // diagonal W/V of gap, superstrate and substrate in the (E_s, H_p) basis
    const cplx wg_s = cmk(1.0, 0.0), wg_p = cmk(0.0, -y);
    const cplx vg_s = cmk(0.0, -y), vg_p = cmk(1.0, 0.0);
    pv.wg[on + i] = wg_s; pv.wg[on + N + i] = wg_p;
    pv.vg[on + i] = vg_s; pv.vg[on + N + i] = vg_p;
    const cplx mi = cmk(0.0, -1.0);
    const cplx wt_s = cmk(1.0, 0.0), wt_p = cdiv(cmul(mi, kzt), et);
    const cplx vt_s = cmul(mi, kzt), vt_p = cmk(1.0, 0.0);
    const cplx wb_s = cmk(1.0, 0.0), wb_p = cdiv(cmul(mi, kzb), eb);
    const cplx vb_s = cmul(mi, kzb), vb_p = cmk(1.0, 0.0);
    for (int half = 0; half < 2; ++half) {
      const cplx wg = half ? wg_p : wg_s, vg = half ? vg_p : vg_s;
      const cplx wt = half ? wt_p : wt_s, vt = half ? vt_p : vt_s;
      const cplx wbv = half ? wb_p : wb_s, vbv = half ? vb_p : vb_s;
      // _ab_matrices(W_gap, V_gap, W_x, V_x): A = W_gap^-1 W_x + V_gap^-1 V_x, B = difference
      const cplx At = cadd(cdiv(wt, wg), cdiv(vt, vg)), Bt = csub(cdiv(wt, wg), cdiv(vt, vg));
      const cplx Ab = cadd(cdiv(wbv, wg), cdiv(vbv, vg)), Bb = csub(cdiv(wbv, wg), cdiv(vbv, vg));
      const cplx Ati = cinv(At), Abi = cinv(Ab);
      const long long j = on + half * N + i;
      // _s_reflection: (-A^-1 B, 2 A^-1, (A - B A^-1 B)/2, B A^-1)
      pv.r11[j] = cneg(cmul(Ati, Bt));
      pv.r12[j] = cscale(Ati, 2.0);
      pv.r21[j] = cscale(csub(At, cmul(cmul(Bt, Ati), Bt)), 0.5);
      pv.r22[j] = cmul(Bt, Ati);
      // _s_transmission: (B A^-1, (A - B A^-1 B)/2, 2 A^-1, -A^-1 B)
      pv.t11[j] = cmul(Bb, Abi);
      pv.t21[j] = cscale(Abi, 2.0);
    }
  }
  if (threadIdx.x == 0) { pv.nt[b] = nt; pv.nb[b] = nb; }
}


// All kernels below are templates over the working real type R of their stage (wb_num.cuh):
// double for the plain form; df64 (stage B) and float or df64 (stage C) for the mixed form.
// FP64 inputs (convolution matrices, port vectors, exponentials) are converted on load.

template <class R> __device__ __forceinline__ Cx<R> ld(const cplx* p) { return cxfrom<R>(*p); }

// --------------------------------------------------------------- Omega^2 assembly (GEMM)
// Omega2[(rb,cb) quadrant] = (diag(k_rb) epz_i diag(k_cb) - [rb==cb] I) @ (cb ? epy : epx)
//                            + diagonal term, k_0 = kx, k_1 = ky  (solve_2d.py:2377-2418)
template <class R>
__global__ void __launch_bounds__(256) omega2_kernel(int N, const cplx* __restrict__ conv, long long conv_ls,
                                                     const int* __restrict__ pair_layer,
                                                     const int* __restrict__ pair_solve,
                                                     const double* __restrict__ kxa, const double* __restrict__ kya,
                                                     Cx<R>* __restrict__ out, long long out_bs) {
  using C_ = Cx<R>;
  __shared__ C_ sA[8][65];
  __shared__ C_ sB[8][65];
  __shared__ double skr[64], skc_a[8];
  const int pair = blockIdx.z >> 2, quad = blockIdx.z & 3, rb = quad & 1, cb = quad >> 1;
  const int n = 2 * N;
  const cplx* base = conv + (long long)pair_layer[pair] * conv_ls;
  const long long NN = (long long)N * N;
  const cplx* epx = base;
  const cplx* epy = base + NN;
  const cplx* epz = base + 2 * NN;
  const cplx* Bm = cb ? epy : epx;
  const double* kx = kxa + (long long)pair_solve[pair] * N;
  const double* ky = kya + (long long)pair_solve[pair] * N;
  const double* kr = rb ? ky : kx;
  const double* kc = cb ? ky : kx;
  C_* C = out + pair * out_bs;
  const int row0 = blockIdx.x * 64, col0 = blockIdx.y * 64;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  if (tid < 64) skr[tid] = (row0 + tid < N) ? kr[row0 + tid] : 0.0;
  C_ acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cxzero<R>();
  for (int k0 = 0; k0 < N; k0 += 8) {
    if (tid < 8) skc_a[tid] = (k0 + tid < N) ? kc[k0 + tid] : 0.0;
    __syncthreads();
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % 64, c = idx / 64;
      int gr = row0 + r, gc = k0 + c;
      cplx v = cmk(0.0, 0.0);
      if (gr < N && gc < N) {
        v = cscale(cscale(epz[gr + (long long)gc * N], skr[r]), skc_a[c]);
        if (rb == cb && gr == gc) v.x -= 1.0;
      }
      sA[c][r] = cxfrom<R>(v);
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % 8, c = idx / 8;
      int gr = k0 + r, gc = col0 + c;
      sB[r][c] = (gr < N && gc < N) ? ld<R>(Bm + gr + (long long)gc * N) : cxzero<R>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
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
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gr = row0 + tx + 16 * i;
    if (gr >= N) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gc = col0 + ty + 16 * j;
      if (gc >= N) continue;
      C_ v = acc[i][j];
      if (gr == gc) {
        double d;
        if (rb == 0 && cb == 0) d = ky[gr] * ky[gr];
        else if (rb == 1 && cb == 1) d = kx[gr] * kx[gr];
        else d = -kx[gr] * ky[gr];
        v.x = v.x + R(d);
      }
      C[(gr + rb * N) + (long long)(gc + cb * N) * n] = v;
    }
  }
}

// ---------------------------------------------------- q, the grazing screen, X = exp(-k0 d q)
// mode_q (conventions.py:186-249) on the eigenvalues; q and X are kept in FP64.
template <class R>
__global__ void modeq_kernel(int n_pairs, int n, const Cx<R>* __restrict__ w, const int* __restrict__ pair_solve,
                             const double* __restrict__ thick, const double* __restrict__ wavelength,
                             cplx* __restrict__ wout, cplx* __restrict__ q, cplx* __restrict__ X,
                             int32_t* __restrict__ status) {
  __shared__ double smin[32], smax[32];
  const int p = blockIdx.x;
  const Cx<R>* wp = w + (long long)p * n;
  const double k0 = 2.0 * 3.141592653589793 / wavelength[pair_solve[p]];
  const double d = thick[p];
  double lo = INFINITY, hi = 0.0;
  bool bad = false;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    cplx wi = cxto(wp[i]);
    if (wout) wout[(long long)p * n + i] = wi;
    if (!(isfinite(wi.x) && isfinite(wi.y))) bad = true;
    double a = cabsv(wi);
    lo = fmin(lo, a); hi = fmax(hi, a);
    cplx v = csqrt_p(wi);
    bool flip = (fabs(v.x) > 1e-12) ? (v.x < 0.0) : (v.y > 0.0);
    if (flip) v = cneg(v);
    q[(long long)p * n + i] = v;
    X[(long long)p * n + i] = cexp_(cscale(v, -k0 * d));
  }
  for (int off = 16; off > 0; off >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, off));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, off));
  }
  if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = lo; smax[threadIdx.x >> 5] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { lo = fmin(lo, smin[k]); hi = fmax(hi, smax[k]); }
    lo = fmin(lo, smin[0]); hi = fmax(hi, smax[0]);
    if (lo < 1e-9 * hi) wb_flag(status + pair_solve[p], WB_ST_GRAZING);
  }
  if (bad) wb_flag(status + pair_solve[p], WB_ST_NONFINITE);
}

// ------------------------------------------------------------ V = Omega_R W / q
// V_top = -epy W_bot - diag(kx ky) W_top + diag(kx^2) W_bot
// V_bot =  epx W_top - diag(ky^2) W_top + diag(ky kx) W_bot      (solve_2d.py:2393-2448)
template <class R>
__global__ void __launch_bounds__(256) vmodes_kernel(int N, const cplx* __restrict__ conv, long long conv_ls,
                                                     const int* __restrict__ pair_layer,
                                                     const int* __restrict__ pair_solve,
                                                     const double* __restrict__ kxa, const double* __restrict__ kya,
                                                     const Cx<R>* __restrict__ Wall, const cplx* __restrict__ qall,
                                                     Cx<R>* __restrict__ Vall, long long bs) {
  using C_ = Cx<R>;
  __shared__ C_ sA[8][65];
  __shared__ C_ sB[8][65];
  const int pair = blockIdx.z >> 1, half = blockIdx.z & 1;
  const int n = 2 * N;
  const long long NN = (long long)N * N;
  const cplx* base = conv + (long long)pair_layer[pair] * conv_ls;
  const cplx* Am = half ? base : base + NN;
  const double sgn = half ? 1.0 : -1.0;
  const double* kx = kxa + (long long)pair_solve[pair] * N;
  const double* ky = kya + (long long)pair_solve[pair] * N;
  const C_* W = Wall + pair * bs;
  const C_* Wsrc = W + (half ? 0 : N);
  const cplx* q = qall + (long long)pair * n;
  C_* V = Vall + pair * bs;
  const int row0 = blockIdx.x * 64, col0 = blockIdx.y * 64;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  C_ acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = cxzero<R>();
  for (int k0 = 0; k0 < N; k0 += 8) {
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % 64, c = idx / 64;
      int gr = row0 + r, gc = k0 + c;
      sA[c][r] = (gr < N && gc < N) ? cxfrom<R>(cscale(Am[gr + (long long)gc * N], sgn)) : cxzero<R>();
    }
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      int idx = tid + e * 256;
      int r = idx % 8, c = idx / 8;
      int gr = k0 + r, gc = col0 + c;
      sB[r][c] = (gr < N && gc < n) ? Wsrc[gr + (long long)gc * n] : cxzero<R>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
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
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    int gr = row0 + tx + 16 * i;
    if (gr >= N) continue;
    const R kxi = R(kx[gr]), kyi = R(ky[gr]);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int gc = col0 + ty + 16 * j;
      if (gc >= n) continue;
      const C_ wt = W[gr + (long long)gc * n], wb = W[gr + N + (long long)gc * n];
      C_ v = acc[i][j];
      if (half == 0) v = v + wt * (-(kxi * kyi)) + wb * (kxi * kxi);
      else v = v + wt * (-(kyi * kyi)) + wb * (kyi * kxi);
      V[gr + half * N + (long long)gc * n] = cxdiv(v, ld<R>(q + gc));
    }
  }
}

// s/p rotation of W and V in place (solve_2d.py:2584-2616)
template <class R>
__global__ void sp_rotate_kernel(int n_pairs, int N, const int* __restrict__ pair_solve, const double* __restrict__ ca,
                                 const double* __restrict__ sa, Cx<R>* __restrict__ Wall, Cx<R>* __restrict__ Vall,
                                 long long bs) {
  const int n = 2 * N;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)n_pairs * N * n) return;
  const long long pair = idx / ((long long)N * n);
  const long long rem = idx % ((long long)N * n);
  const int i = (int)(rem % N), j = (int)(rem / N);
  const long long o = (long long)pair_solve[pair] * N + i;
  const R c = R(ca[o]), s = R(sa[o]);
  Cx<R>* W = Wall + pair * bs;
  Cx<R>* V = Vall + pair * bs;
  const long long a = i + (long long)j * n, b = a + N;
  const Cx<R> w1 = W[a], w2 = W[b], v1 = V[a], v2 = V[b];
  W[a] = w2 * c - w1 * s;
  W[b] = w1 * c + w2 * s;
  V[a] = v1 * c + v2 * s;
  V[b] = v2 * c - v1 * s;
}

// ------------------------------------------------------------------ cascade elementwise
template <class R>
__global__ void diag_matrix_kernel(int B, int n, const cplx* __restrict__ d, Cx<R>* __restrict__ M, long long bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * n) return;
  const long long b = idx / ((long long)n * n), rem = idx % ((long long)n * n);
  const int i = (int)(rem % n), j = (int)(rem / n);
  M[b * bs + rem] = (i == j) ? ld<R>(d + b * n + i) : cxzero<R>();
}

// U1 = diag(wg)(I + R), U2 = diag(vg)(I - R)
template <class R>
__global__ void u12_kernel(int B, int n, const Cx<R>* __restrict__ Rm, long long r_bs, const cplx* __restrict__ wg,
                           const cplx* __restrict__ vg, Cx<R>* __restrict__ U1, Cx<R>* __restrict__ U2, long long bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * n) return;
  const long long b = idx / ((long long)n * n), rem = idx % ((long long)n * n);
  const int i = (int)(rem % n), j = (int)(rem / n);
  Cx<R> r = Rm[b * r_bs + rem];
  Cx<R> e = (i == j) ? cxone<R>() : cxzero<R>();
  U1[b * bs + rem] = ld<R>(wg + b * n + i) * (e + r);
  U2[b * bs + rem] = ld<R>(vg + b * n + i) * (e - r);
}

// M = P1 + P2 (to Mout, batch stride m_bs), NT = (P1 - P2)^T ; 32x32 tiles
template <class R>
__global__ void mn2_kernel(int n, const Cx<R>* __restrict__ P1, const Cx<R>* __restrict__ P2, long long p_bs,
                           Cx<R>* __restrict__ Mout, long long m_bs, Cx<R>* __restrict__ NT) {
  __shared__ Cx<R> t[32][33];
  const long long b = blockIdx.z;
  const Cx<R>* p1 = P1 + b * p_bs; const Cx<R>* p2 = P2 + b * p_bs;
  Cx<R>* mo = Mout + b * m_bs; Cx<R>* nt = NT + b * p_bs;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int e = threadIdx.y; e < 32; e += blockDim.y) {
    int i = i0 + threadIdx.x, j = j0 + e;
    if (i < n && j < n) {
      long long o = i + (long long)j * n;
      Cx<R> a = p1[o], c = p2[o];
      mo[o] = a + c;
      t[e][threadIdx.x] = a - c;
    }
  }
  __syncthreads();
  for (int e = threadIdx.y; e < 32; e += blockDim.y) {
    int j = j0 + threadIdx.x, i = i0 + e;
    if (i < n && j < n) nt[j + (long long)i * n] = t[threadIdx.x][e];
  }
}

// from rho_b^T: Y1T = (I - X rho_b X)^T into Y1, Y2T = (I + X rho_b X)^T in place
template <class R>
__global__ void rho_kernel(int B, int n, Cx<R>* __restrict__ RT, Cx<R>* __restrict__ Y1, const cplx* __restrict__ X,
                           long long x_ps, long long bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * n) return;
  const long long b = idx / ((long long)n * n), rem = idx % ((long long)n * n);
  const int jr = (int)(rem % n), ic = (int)(rem / n);     // RT(jr, ic) = rho_b(ic, jr)
  const cplx* Xb = X + b * x_ps;
  Cx<R> r = (ld<R>(Xb + ic) * RT[b * bs + rem]) * ld<R>(Xb + jr);
  Cx<R> e = (jr == ic) ? cxone<R>() : cxzero<R>();
  Y1[b * bs + rem] = e - r;
  RT[b * bs + rem] = e + r;
}

// Aterm = X1 diag(wg) + X2 diag(vg) (to Aout), Bterm = -X1 diag(wg) + X2 diag(vg) (to Bout)
template <class R>
__global__ void ab2_kernel(int n, const Cx<R>* __restrict__ X1T, const Cx<R>* __restrict__ X2T, long long x_bs,
                           const cplx* __restrict__ wg, const cplx* __restrict__ vg,
                           Cx<R>* __restrict__ Aout, long long a_bs, Cx<R>* __restrict__ Bout, long long b_bs) {
  __shared__ Cx<R> t1[32][33], t2[32][33];
  const long long b = blockIdx.z;
  const Cx<R>* x1 = X1T + b * x_bs; const Cx<R>* x2 = X2T + b * x_bs;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  for (int e = threadIdx.y; e < 32; e += blockDim.y) {
    int j = j0 + threadIdx.x, i = i0 + e;
    if (i < n && j < n) {
      long long o = j + (long long)i * n;
      t1[e][threadIdx.x] = x1[o];
      t2[e][threadIdx.x] = x2[o];
    }
  }
  __syncthreads();
  for (int e = threadIdx.y; e < 32; e += blockDim.y) {
    int i = i0 + threadIdx.x, j = j0 + e;
    if (i < n && j < n) {
      Cx<R> a1 = t1[threadIdx.x][e] * ld<R>(wg + b * n + j);
      Cx<R> a2 = t2[threadIdx.x][e] * ld<R>(vg + b * n + j);
      long long o = i + (long long)j * n;
      Aout[b * a_bs + o] = a1 + a2;
      Bout[b * b_bs + o] = a2 - a1;
    }
  }
}

// incident columns: [a_s d; -i n_top a_p d], pure s, pure p (d: unit vector on the specular order)
template <class R>
__global__ void incident_kernel(int B, int N, const cplx* __restrict__ pol, const cplx* __restrict__ nt,
                                Cx<R>* __restrict__ C, long long c_bs) {
  const int n = 2 * N;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * 3) return;
  const long long b = idx / (n * 3);
  const int rem = (int)(idx % (n * 3));
  const int i = rem % n, col = rem / n;
  const int spec = N / 2;
  cplx as, ap;
  if (col == 0) { as = pol[2 * b]; ap = pol[2 * b + 1]; }
  else if (col == 1) { as = cmk(1.0, 0.0); ap = cmk(6.123233995736766e-17, 0.0); }   // sin/cos(pi/2)
  else { as = cmk(0.0, 0.0); ap = cmk(1.0, 0.0); }
  cplx v = cmk(0.0, 0.0);
  if (i == spec) v = as;
  else if (i == N + spec) v = cmul(cmul(cmk(0.0, -1.0), nt[b]), ap);
  C[b * c_bs + i + (long long)col * n] = cxfrom<R>(v);
}

// G0 = I - diag(r22) R0
template <class R>
__global__ void top_kernel(int B, int n, const Cx<R>* __restrict__ R1, long long r_bs, const cplx* __restrict__ r22,
                           Cx<R>* __restrict__ G0, long long bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * n) return;
  const long long b = idx / ((long long)n * n), rem = idx % ((long long)n * n);
  const int i = (int)(rem % n), j = (int)(rem / n);
  Cx<R> v = -(ld<R>(r22 + b * n + i) * R1[b * r_bs + rem]);
  if (i == j) v.x = v.x + R(1.0);
  G0[b * bs + rem] = v;
}

// out = diag(d) in (+ diag(e) in2 when e), n x 3 per batch
template <class R>
__global__ void dscale3_kernel(int B, int n, const cplx* __restrict__ d, const Cx<R>* __restrict__ in, long long in_bs,
                               const cplx* __restrict__ e, const Cx<R>* __restrict__ in2, long long in2_bs,
                               Cx<R>* __restrict__ out, long long out_bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * 3) return;
  const long long b = idx / (n * 3);
  const int rem = (int)(idx % (n * 3)), i = rem % n;
  Cx<R> v = ld<R>(d + b * n + i) * in[b * in_bs + rem];
  if (e) v = v + ld<R>(e + b * n + i) * in2[b * in2_bs + rem];
  out[b * out_bs + rem] = v;
}

// rhs1 = wg o (g + h), rhs2 = vg o (g - h)
template <class R>
__global__ void gh_kernel(int B, int n, const Cx<R>* __restrict__ g, const Cx<R>* __restrict__ h,
                          const cplx* __restrict__ wg, const cplx* __restrict__ vg,
                          Cx<R>* __restrict__ r1, Cx<R>* __restrict__ r2, long long bs3) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * 3) return;
  const long long b = idx / (n * 3);
  const int rem = (int)(idx % (n * 3)), i = rem % n;
  Cx<R> gg = g[b * bs3 + rem], hh = h[b * bs3 + rem];
  r1[b * bs3 + rem] = ld<R>(wg + b * n + i) * (gg + hh);
  r2[b * bs3 + rem] = ld<R>(vg + b * n + i) * (gg - hh);
}

// g_next rhs = X o (r1 + r2) (= 2 c+_bottom), written into g
template <class R>
__global__ void ct_kernel(int B, int n, const Cx<R>* __restrict__ r1, const Cx<R>* __restrict__ r2,
                          const cplx* __restrict__ X, long long x_ps, Cx<R>* __restrict__ g, long long bs3) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * 3) return;
  const long long b = idx / (n * 3);
  const int rem = (int)(idx % (n * 3)), i = rem % n;
  g[b * bs3 + rem] = ld<R>(X + b * x_ps + i) * (r1[b * bs3 + rem] + r2[b * bs3 + rem]);
}

// per-order efficiencies (scattering.py:907-994, solve_1d.py:1588-1610, power.py:13-159), in FP64
template <class R>
__global__ void efficiency_kernel(int B, int N, const Cx<R>* __restrict__ cref, const Cx<R>* __restrict__ ctrn,
                                  long long bs3, PortVectors pv, const cplx* __restrict__ eps_top,
                                  const cplx* __restrict__ eps_bot, const cplx* __restrict__ pol,
                                  double* __restrict__ Rout, double* __restrict__ Tout, cplx* __restrict__ amps,
                                  int32_t* __restrict__ status) {
  const int n = 2 * N;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * N * 3) return;
  const long long b = idx / (N * 3);
  const int rem = (int)(idx % (N * 3)), i = rem % N, col = rem / N;
  const cplx et = eps_top[b], eb = eps_bot[b];
  const cplx kzs = pv.kz_top[b * N + N / 2];
  const double s_power = kzs.x;
  const cplx nt = pv.nt[b], nb = pv.nb[b];
  const double p_power = cabs2(nt) * cdiv(kzs, et).x;
  double denom;
  if (col == 0) denom = cabs2(pol[2 * b]) * s_power + cabs2(pol[2 * b + 1]) * p_power;
  else if (col == 1) denom = s_power;
  else denom = p_power;
  const cplx Rs = cxto(cref[b * bs3 + i + (long long)col * n]);
  const cplx Rp = cneg(cxto(cref[b * bs3 + N + i + (long long)col * n]));
  const cplx Ts = cxto(ctrn[b * bs3 + i + (long long)col * n]);
  const cplx Tp = cxto(ctrn[b * bs3 + N + i + (long long)col * n]);
  const cplx kzt = pv.kz_top[b * N + i], kzb = pv.kz_bot[b * N + i];
  const double eRs = cabs2(Rs) * kzt.x / denom;
  const double eRp = cabs2(Rp) * cdiv(kzt, et).x / denom;
  const double eTs = cabs2(Ts) * kzb.x / denom;
  const double eTp = cabs2(Tp) * cdiv(kzb, eb).x / denom;
  const double r = eRs + eRp, t = eTs + eTp;
  Rout[(b * 3 + col) * N + i] = r;
  Tout[(b * 3 + col) * N + i] = t;
  if (amps) {
    const cplx mi_nt = cmul(cmk(0.0, -1.0), nt), mi_nb = cmul(cmk(0.0, -1.0), nb);
    cplx* a = amps + ((b * 3 + col) * 4) * (long long)N;
    a[i] = Rs; a[N + i] = cdiv(Rp, mi_nt); a[2 * N + i] = Ts; a[3 * N + i] = cdiv(Tp, mi_nb);
  }
  if (!(isfinite(r) && isfinite(t))) wb_flag(status + b, WB_ST_NONFINITE);
}

static inline unsigned nblk(long long total, int per) { return (unsigned)((total + per - 1) / per); }

__global__ void pairs_kernel(int B, int L, const int* __restrict__ layer_index, const double* __restrict__ thick,
                             int* __restrict__ pair_layer, int* __restrict__ pair_solve, double* __restrict__ pair_thick) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= B * L) return;
  pair_layer[p] = layer_index ? layer_index[p] : 0;
  pair_solve[p] = p / L;
  pair_thick[p] = thick[p];
}

// ------------------------------------------------------------------- stage B driver
// Omega^2, eigen-decomposition, q/X, V and the s/p rotation for P pairs, in precision RB.
// On return OM holds bigW and Zb holds bigV (both Cx<RB>), w/q/X the FP64 modal data.
template <class RB>
void stage_b(cudaStream_t s, int P, int N, const cplx* conv, const int* pair_layer, const int* pair_solve,
             const double* pair_thick, const double* wavelength, const double* kx, const double* ky,
             Cx<RB>* OM, Cx<RB>* Zb, Cx<RB>* Xv, Cx<RB>* wr, Cx<RB>* tau, cplx* w, cplx* q, cplx* X,
             const double* c, const double* sn, int32_t* st, int st_div, bool rotate) {
  TraceRange trace_("wb:stage_b");
  const int n = 2 * N;
  const long long n2 = (long long)n * n, NN = (long long)N * N;
  {
    dim3 gr((N + 63) / 64, (N + 63) / 64, P * 4);
    omega2_kernel<RB><<<gr, 256, 0, s>>>(N, conv, 3 * NN, pair_layer, pair_solve, kx, ky, OM, n2); note_launch();
  }
  geev_schur<RB>(s, P, n, OM, n, n2, Zb, n, n2, wr, tau, st, st_div);
  trevc<RB>(s, P, n, OM, n, n2, Xv, n, n2);
  gemm<RB>(s, P, n, n, n, make_double2(1, 0), Zb, 1, n, n2, Xv, 1, n, n2, make_double2(0, 0), OM, 1, n, n2);
  normalize_columns<RB>(s, P, n, OM, n, n2);
  modeq_kernel<RB><<<P, 256, 0, s>>>(P, n, wr, pair_solve, pair_thick, wavelength, w, q, X, st); note_launch();
  {
    dim3 gr((N + 63) / 64, (n + 63) / 64, P * 2);
    vmodes_kernel<RB><<<gr, 256, 0, s>>>(N, conv, 3 * NN, pair_layer, pair_solve, kx, ky, OM, q, Zb, n2); note_launch();
  }
  if (rotate) {
    sp_rotate_kernel<RB><<<nblk((long long)P * N * n, 256), 256, 0, s>>>(P, N, pair_solve, c, sn, OM, Zb, n2);
    note_launch();
  }
}

// dst += src over `count` complex entries (FP32 corrections into a wider state)
template <class RS, class RD>
__global__ void accumulate_kernel(long long count, const Cx<RS>* __restrict__ src, Cx<RD>* __restrict__ dst) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const Cx<RS> a = src[i];
  Cx<RD> d = dst[i];
  d.x = d.x + RD((double)a.x);
  d.y = d.y + RD((double)a.y);
  dst[i] = d;
}

// complex128 -> complex double-float in place (both 16 bytes per entry)
__global__ void to_df64_kernel(long long count, cplx* __restrict__ buf) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= count) return;
  const cplx v = buf[i];
  Cx<df64> o;
  o.x = df64(v.x); o.y = df64(v.y);
  reinterpret_cast<Cx<df64>*>(buf)[i] = o;
}

// -------------------------------------- stage B of the mixed form: FP32 Schur + Newton steps
// The eigenpairs are computed in FP32 (the stage_b pipeline on floats) and brought to FP64
// accuracy by Newton steps on the FP64 operator. With W, Lambda the current pairs:
//   R = Omega^2 W - W Lambda                       (FP64 products from the slots)
//   G = W^-1 R                                     (FP32 LU of W rounded to FP32)
//   d_i = lambda_i + G_ii
//   E_ij = G_ij / (d_j - d_i) for i, j in different groups, 0 otherwise
//   W <- W + W E (FP32 product added to the FP64 W); lambda_i <- d_i
// where groups are the connected components of the strong couplings |G_ij| > kCouple |d_j - d_i|
// (near-degenerate modes, for which the first-order formula does not hold). The block
// Lambda + G restricted to each group is diagonalised exactly in FP64 (the stage-B eigen
// pipeline on 32 x 32 blocks padded with distant eigenvalues) and the group's columns of W are
// rotated by its eigenvectors. Each step squares the error; two take FP32 eigenpairs to
// FP64-class ones (|dR,T| ~1e-11 against the FP64 form at (12,12)).
constexpr int kGroupMax = 32;          // largest group diagonalised exactly
constexpr double kCouple = 0.02;
constexpr int kNewtonSteps = 2;
constexpr double kScalarGroup = 1e-10;  // a group whose block is scalar to this (relative) keeps its basis
constexpr double kParallel = 0.99;      // |cos| between eigenvectors above which a group keeps its basis

// Group storage: 2-member groups (the TE/TM pairs of every order of a uniform layer, say) are
// solved in closed form from a compact pool; larger groups go to padded 32 x 32 slots.
struct GroupBufs {
  int cap = 0, cap2 = 0;
  int* count = nullptr;     // (2) slots used: [0] large groups, [1] 2-member groups
  int* pair = nullptr;      // (cap)
  int* size = nullptr;      // (cap)
  int* members = nullptr;   // (cap, 32)
  double* offmax = nullptr; // (cap) largest off-diagonal |B_ab| / scale of the pair
  cplx* A = nullptr;        // (cap, 32, 32) padded blocks -> Schur form -> eigenvectors
  cplx* Z = nullptr;        // (cap, 32, 32) Schur vectors
  cplx* X = nullptr;        // (cap, 32, 32) eigenvectors of the Schur form
  cplx* w = nullptr;        // (cap, 32)
  cplx* tau = nullptr;      // (cap, 32)
  int* pair2 = nullptr;     // (cap2)
  int* mem2 = nullptr;      // (cap2, 2)
  cplx* B2 = nullptr;       // (cap2, 4) blocks, column-major
  double* scale2 = nullptr; // (cap2) scale of the pair
  static int caps(int P, int n, int& cap2) { cap2 = P * (n / 2); return 16 * P + 1024; }
  bool carve(Arena& ar, int P, int n) {
    cap = caps(P, n, cap2);
    const size_t c = (size_t)cap, b2 = (size_t)kGroupMax * kGroupMax, c2 = (size_t)cap2;
    count = ar.get<int>(2); pair = ar.get<int>(c); size = ar.get<int>(c); members = ar.get<int>(c * kGroupMax);
    offmax = ar.get<double>(c);
    A = ar.get<cplx>(c * b2); Z = ar.get<cplx>(c * b2); X = ar.get<cplx>(c * b2);
    w = ar.get<cplx>(c * kGroupMax); tau = ar.get<cplx>(c * kGroupMax);
    pair2 = ar.get<int>(c2); mem2 = ar.get<int>(2 * c2); B2 = ar.get<cplx>(4 * c2); scale2 = ar.get<double>(c2);
    return ar.ok();
  }
  static size_t bytes(int P, int n) {
    int c2i;
    const size_t c = (size_t)caps(P, n, c2i), b2 = (size_t)kGroupMax * kGroupMax, c2 = (size_t)c2i;
    size_t b = 0;
    auto A_ = [&](size_t x) { b += (x + 255) & ~(size_t)255; };
    A_(8); A_(4 * c); A_(4 * c); A_(4 * c * kGroupMax); A_(8 * c);
    A_(16 * c * b2); A_(16 * c * b2); A_(16 * c * b2); A_(16 * c * kGroupMax); A_(16 * c * kGroupMax);
    A_(4 * c2); A_(8 * c2); A_(64 * c2); A_(8 * c2);
    return b;
  }
};

__global__ void widen_kernel(long long count, const Cx<float>* __restrict__ src, cplx* __restrict__ dst) {
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < count) dst[i] = cmk((double)src[i].x, (double)src[i].y);
}

// Omega^2 W without forming Omega^2 (solve_2d.py:2377-2418 with epxy = epyx = 0): with
// T = epx W_top, U = epy W_bot and Y = epz_i (Kx T + Ky U),
//   (Omega^2 W)_top = Kx Y - T + Ky^2 W_top - Kx Ky W_bot
//   (Omega^2 W)_bot = Ky Y - U - Kx Ky W_top + Kx^2 W_bot
// (three N x N by N x n products per pair instead of four to form Omega^2 and one n x n product).
__global__ void omw_s_kernel(long long total, int N, int n, const int* __restrict__ pair_solve,
                             const double* __restrict__ kx, const double* __restrict__ ky, const cplx* __restrict__ T,
                             const cplx* __restrict__ U, cplx* __restrict__ S) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const long long Nn = (long long)N * n;
  const long long p = idx / Nn;
  const int i = (int)((idx % Nn) % N);
  const long long o = (long long)pair_solve[p] * N + i;
  S[idx] = cadd(cscale(T[idx], kx[o]), cscale(U[idx], ky[o]));
}

// R32 = FP32(Omega^2 W - W diag(lambda)) from T, U, Y of omw_s_kernel's products
__global__ void omw_resid_kernel(long long total, int N, int n, const int* __restrict__ pair_solve,
                                 const double* __restrict__ kx, const double* __restrict__ ky,
                                 const cplx* __restrict__ T, const cplx* __restrict__ U, const cplx* __restrict__ Y,
                                 const cplx* __restrict__ W, const cplx* __restrict__ lam, Cx<float>* __restrict__ R) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const long long n2 = (long long)n * n, Nn = (long long)N * n;
  const long long p = idx / n2, rem = idx % n2;
  const int r = (int)(rem % n), j = (int)(rem / n);
  const bool top = r < N;
  const int i = top ? r : r - N;
  const long long o = (long long)pair_solve[p] * N + i;
  const double a = kx[o], b = ky[o];
  const cplx* Wp = W + p * n2;
  const cplx wt = Wp[i + (long long)j * n], wb = Wp[N + i + (long long)j * n];
  const long long h = p * Nn + i + (long long)j * N;
  cplx aw;
  if (top) aw = cadd(csub(cscale(Y[h], a), T[h]), csub(cscale(wt, b * b), cscale(wb, a * b)));
  else aw = cadd(csub(cscale(Y[h], b), U[h]), csub(cscale(wb, a * a), cscale(wt, a * b)));
  const cplx res = csub(aw, cmul(Wp[r + (long long)j * n], lam[p * n + j]));
  R[idx] = cxmk<float>((float)res.x, (float)res.y);
}

// V = Omega_R W / q from the products T = epy W_bot and U = epx W_top (solve_2d.py:2393-2448):
//   V_top = -T - diag(kx ky) W_top + diag(kx^2) W_bot,  V_bot = U - diag(ky^2) W_top + diag(ky kx) W_bot
__global__ void vmodes_epilogue_kernel(long long total, int N, int n, const int* __restrict__ pair_solve,
                                       const double* __restrict__ kx, const double* __restrict__ ky,
                                       const cplx* __restrict__ T, const cplx* __restrict__ U,
                                       const cplx* __restrict__ W, const cplx* __restrict__ q, cplx* __restrict__ V) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const long long n2 = (long long)n * n, Nn = (long long)N * n;
  const long long p = idx / n2, rem = idx % n2;
  const int r = (int)(rem % n), j = (int)(rem / n);
  const bool top = r < N;
  const int i = top ? r : r - N;
  const long long o = (long long)pair_solve[p] * N + i;
  const double a = kx[o], b = ky[o];
  const cplx* Wp = W + p * n2;
  const cplx wt = Wp[i + (long long)j * n], wb = Wp[N + i + (long long)j * n];
  const long long h = p * Nn + i + (long long)j * N;
  cplx v;
  if (top) v = cadd(cneg(T[h]), cadd(cscale(wt, -(a * b)), cscale(wb, a * a)));
  else v = cadd(U[h], cadd(cscale(wt, -(b * b)), cscale(wb, b * a)));
  V[idx] = cdiv(v, q[p * n + j]);
}

// every slot a diagonal 32 x 32 block with distinct entries, so unused slots converge at once
__global__ void group_init_kernel(int cap, cplx* __restrict__ A, int* __restrict__ count) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx == 0) { count[0] = 0; count[1] = 0; }
  if (idx >= (long long)cap * kGroupMax * kGroupMax) return;
  const int rem = (int)(idx % (kGroupMax * kGroupMax)), a = rem % kGroupMax, b = rem / kGroupMax;
  A[idx] = (a == b) ? cmk(1.0 + a, 0.0) : cmk(0.0, 0.0);
}

// One CTA per pair: d, the groups (lock-free union-find over the strong couplings, links always
// from the larger root index to the smaller, retries bounded), the group blocks into slots, E and
// the new lambda. A pair whose groups do not fit (more than kGroupMax members, slots exhausted,
// union retries exhausted) is flagged WB_ST_NOCONV.
__global__ void __launch_bounds__(256) group_kernel(int n, const Cx<float>* __restrict__ Gall, cplx* __restrict__ lam_all,
                                                    Cx<float>* __restrict__ Eall, GroupBufs gb, int32_t* __restrict__ status,
                                                    int st_div) {
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx* d = reinterpret_cast<cplx*>(smraw);
  int* parent = reinterpret_cast<int*>(d + n);
  int* label = parent + n;
  int* cnt = label + n;
  int* slot = cnt + n;
  int* fill = slot + n;
  __shared__ int s_fail;
  __shared__ double s_red[32];
  const int p = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const long long n2 = (long long)n * n;
  const Cx<float>* G = Gall + p * n2;
  Cx<float>* E = Eall + p * n2;
  cplx* lam = lam_all + (long long)p * n;
  if (tid == 0) s_fail = 0;
  double mx = 0.0;
  for (int i = tid; i < n; i += blockDim.x) {
    const Cx<float> g = G[i + (long long)i * n];
    const cplx v = cadd(lam[i], cmk((double)g.x, (double)g.y));
    d[i] = v; parent[i] = i; cnt[i] = 0; slot[i] = -1; fill[i] = 0;
    mx = fmax(mx, cabsv(v));
  }
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if (lane == 0) s_red[warp] = mx;
  __syncthreads();
  double scale = 0.0;
  for (int k = 0; k < nw; ++k) scale = fmax(scale, s_red[k]);
  volatile int* vp = parent;
  for (long long e = tid; e < n2; e += blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    if (i == j) continue;
    const Cx<float> g = G[e];
    const double ga = hypot((double)g.x, (double)g.y);
    if (!(ga > kCouple * cabsv(csub(d[j], d[i])))) continue;
    int a = i, b = j;
    bool linked = false;
    for (int tries = 0; tries < 64 + 4 * n && !linked; ++tries) {
      int ra = a, rb = b;
      for (int h = 0; h < n && vp[ra] != ra; ++h) ra = vp[ra];
      for (int h = 0; h < n && vp[rb] != rb; ++h) rb = vp[rb];
      if (ra == rb) { linked = true; break; }
      if (ra > rb) { const int t = ra; ra = rb; rb = t; }
      if (atomicCAS(&parent[rb], rb, ra) == rb) linked = true;
    }
    if (!linked) s_fail = 1;
  }
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    int r = i;
    for (int h = 0; h < n && vp[r] != r; ++h) r = vp[r];
    label[i] = r;
    atomicAdd(&cnt[r], 1);
  }
  __syncthreads();
  // slots: -1 none; 2-member groups in the compact pool as -2 - index; larger ones padded
  for (int r = tid; r < n; r += blockDim.x) {
    if (label[r] != r || cnt[r] < 2) continue;
    if (cnt[r] == 2) {
      const int sl = atomicAdd(&gb.count[1], 1);
      if (sl < gb.cap2) { slot[r] = -2 - sl; gb.pair2[sl] = p; gb.scale2[sl] = scale; }
      else s_fail = 1;
      continue;
    }
    const int sl = atomicAdd(&gb.count[0], 1);
    if (sl < gb.cap && cnt[r] <= kGroupMax) {
      slot[r] = sl; gb.pair[sl] = p; gb.size[sl] = cnt[r];
    } else {
      s_fail = 1;
    }
  }
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) {
    const int r = label[i];
    if (slot[r] == -1) continue;
    const int pos = atomicAdd(&fill[r], 1);
    if (slot[r] <= -2) gb.mem2[2LL * (-2 - slot[r]) + pos] = i;
    else gb.members[(long long)slot[r] * kGroupMax + pos] = i;
  }
  __syncthreads();
  for (int r = tid; r < n; r += blockDim.x) {
    if (slot[r] > -2) continue;
    const long long sl = -2 - slot[r];
    const int a = gb.mem2[2 * sl], b = gb.mem2[2 * sl + 1];
    const Cx<float> gaa = G[a + (long long)a * n], gba = G[b + (long long)a * n];
    const Cx<float> gab = G[a + (long long)b * n], gbb = G[b + (long long)b * n];
    cplx* B = gb.B2 + 4 * sl;
    B[0] = cadd(lam[a], cmk((double)gaa.x, (double)gaa.y));
    B[1] = cmk((double)gba.x, (double)gba.y);
    B[2] = cmk((double)gab.x, (double)gab.y);
    B[3] = cadd(lam[b], cmk((double)gbb.x, (double)gbb.y));
  }
  // group blocks: B = diag(lambda) + G on the members, padded with distinct distant eigenvalues
  for (int r = warp; r < n; r += nw) {
    const int sl = slot[r];
    if (sl < 0) continue;
    const int sz = cnt[r];
    const int* mem = gb.members + (long long)sl * kGroupMax;
    cplx* B = gb.A + (long long)sl * kGroupMax * kGroupMax;
    double off = 0.0;
    for (int e = lane; e < kGroupMax * kGroupMax; e += 32) {
      const int a = e % kGroupMax, b = e / kGroupMax;
      cplx v = cmk(0.0, 0.0);
      if (a < sz && b < sz) {
        const Cx<float> g = G[mem[a] + (long long)mem[b] * n];
        v = cmk((double)g.x, (double)g.y);
        if (a == b) v = cadd(v, lam[mem[a]]);
        else off = fmax(off, cabsv(v));
      } else if (a == b) {
        v = cmk((3.0 + a) * (scale + 1.0), 0.0);
      }
      B[e] = v;
    }
    for (int o = 16; o > 0; o >>= 1) off = fmax(off, __shfl_xor_sync(0xffffffffu, off, o));
    if (lane == 0) gb.offmax[sl] = off / (scale > 0.0 ? scale : 1.0);
  }
  // first-order corrections between groups, and the new eigenvalues
  for (long long e = tid; e < n2; e += blockDim.x) {
    const int i = (int)(e % n), j = (int)(e / n);
    Cx<float> v = cxzero<float>();
    if (i != j && label[i] != label[j]) {
      const cplx dd = csub(d[j], d[i]);
      if (dd.x != 0.0 || dd.y != 0.0) {
        const Cx<float> g = G[e];
        const cplx q = cdiv(cmk((double)g.x, (double)g.y), dd);
        v = cxmk<float>((float)q.x, (float)q.y);
      }
    }
    E[e] = v;
  }
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) lam[i] = d[i];
  if (tid == 0 && s_fail) wb_flag(status + p / st_div, WB_ST_NOCONV);
}

// One CTA per used slot: rotate the group's columns of W by the block's eigenvectors and set
// its eigenvalues. Eigenvectors of the padded block are told apart by their weight on the
// group's own coordinates (the padding eigenvalues are far away, so the two sets separate).
__global__ void __launch_bounds__(256) group_apply_kernel(int n, long long n2, GroupBufs gb, cplx* __restrict__ W_all,
                                                          cplx* __restrict__ lam_all, int32_t* __restrict__ status,
                                                          int st_div) {
  __shared__ int sel[kGroupMax];
  __shared__ int s_nsel;
  __shared__ cplx S[kGroupMax * kGroupMax];
  const int sl = blockIdx.x;
  const int used = min(gb.count[0], gb.cap);
  if (sl >= used) return;
  if (gb.offmax[sl] <= kScalarGroup) return;               // degenerate group: any basis is an eigenbasis
  const int p = gb.pair[sl], sz = gb.size[sl], tid = threadIdx.x;
  const int* mem = gb.members + (long long)sl * kGroupMax;
  const cplx* V = gb.A + (long long)sl * kGroupMax * kGroupMax;    // normalised eigenvectors
  const cplx* wv = gb.w + (long long)sl * kGroupMax;
  if (tid < 32) {
    double mass = 0.0;
    for (int a = 0; a < sz; ++a) { const cplx v = V[a + tid * kGroupMax]; mass += v.x * v.x + v.y * v.y; }
    const bool take = mass > 0.5 && isfinite(mass) && isfinite(wv[tid].x) && isfinite(wv[tid].y);
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (take) sel[__popc(m & ((1u << tid) - 1u))] = tid;
    if (tid == 0) s_nsel = __popc(m);
  }
  __syncthreads();
  if (s_nsel != sz) {
    if (tid == 0) wb_flag(status + p / st_div, WB_ST_NOCONV);
    return;
  }
  for (int e = tid; e < sz * sz; e += blockDim.x) {
    const int a = e % sz, b = e / sz;
    S[a + b * kGroupMax] = V[a + sel[b] * kGroupMax];
  }
  __syncthreads();
  // an eigenvector set that is nearly dependent (a defective or noise-dominated block) would
  // make W singular: keep the group's basis then
  __shared__ int s_par;
  if (tid == 0) s_par = 0;
  __syncthreads();
  for (int e = tid; e < sz * sz; e += blockDim.x) {
    const int a = e % sz, b = e / sz;
    if (a >= b) continue;
    double na = 0.0, nb2 = 0.0;
    cplx dot = cmk(0.0, 0.0);
    for (int k = 0; k < sz; ++k) {
      const cplx u = S[k + a * kGroupMax], v = S[k + b * kGroupMax];
      na += u.x * u.x + u.y * u.y; nb2 += v.x * v.x + v.y * v.y;
      dot = cadd(dot, cmul(cconj(u), v));
    }
    if (cabsv(dot) > kParallel * sqrt(na * nb2)) s_par = 1;
  }
  __syncthreads();
  if (s_par) return;
  cplx* W = W_all + p * n2;
  for (int r = tid; r < n; r += blockDim.x) {
    cplx row[kGroupMax];
    for (int a = 0; a < sz; ++a) row[a] = W[r + (long long)mem[a] * n];
    for (int b = 0; b < sz; ++b) {
      cplx acc = cmk(0.0, 0.0);
      for (int a = 0; a < sz; ++a) acc = cadd(acc, cmul(row[a], S[a + b * kGroupMax]));
      W[r + (long long)mem[b] * n] = acc;
    }
  }
  if (tid < sz) lam_all[(long long)p * n + mem[tid]] = wv[sel[tid]];
}

// One warp per 2-member group: B = [[a, b], [c, d]] has eigenvalues m +- r, m = (a + d)/2,
// r = sqrt(((a - d)/2)^2 + b c), with the sign of r chosen so that s = (a - d)/2 + r is the larger
// root difference; eigenvectors (s, c) and (b, -s) need no cancelling subtraction.
__global__ void group2_apply_kernel(int n, long long n2, GroupBufs gb, cplx* __restrict__ W_all,
                                    cplx* __restrict__ lam_all) {
  const long long gw = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int used = min(gb.count[1], gb.cap2);
  if (gw >= used) return;
  const int p = gb.pair2[gw];
  const int i = gb.mem2[2 * gw], j = gb.mem2[2 * gw + 1];
  const cplx* B = gb.B2 + 4 * gw;
  const cplx a = B[0], c = B[1], b = B[2], d = B[3];
  const double sc = gb.scale2[gw] > 0.0 ? gb.scale2[gw] : 1.0;
  const cplx m = cscale(cadd(a, d), 0.5), dl = cscale(csub(a, d), 0.5);
  if (fmax(fmax(cabsv(b), cabsv(c)), cabsv(dl)) <= kScalarGroup * sc) return;   // degenerate: keep the basis
  cplx r = csqrt_p(cadd(cmul(dl, dl), cmul(b, c)));
  if (cabsv(cadd(dl, r)) < cabsv(csub(dl, r))) r = cneg(r);
  const cplx sv = cadd(dl, r);
  // v1 = (s, c) for m + r, v2 = (b, -s) for m - r
  const double n1 = sqrt(cabs2(sv) + cabs2(c)), n2v = sqrt(cabs2(b) + cabs2(sv));
  if (!(n1 > 0.0) || !(n2v > 0.0)) return;
  const cplx v11 = cscale(sv, 1.0 / n1), v21 = cscale(c, 1.0 / n1);
  const cplx v12 = cscale(b, 1.0 / n2v), v22 = cscale(cneg(sv), 1.0 / n2v);
  const cplx dot = cadd(cmul(cconj(v11), v12), cmul(cconj(v21), v22));
  if (!(cabsv(dot) <= kParallel)) return;                    // nearly defective: keep the basis
  cplx* W = W_all + p * n2;
  for (int row = lane; row < n; row += 32) {
    const cplx wi = W[row + (long long)i * n], wj = W[row + (long long)j * n];
    W[row + (long long)i * n] = cadd(cmul(wi, v11), cmul(wj, v21));
    W[row + (long long)j * n] = cadd(cmul(wi, v12), cmul(wj, v22));
  }
  if (lane == 0) {
    lam_all[(long long)p * n + i] = cadd(m, r);
    lam_all[(long long)p * n + j] = csub(m, r);
  }
}

// Work buffers of stage_b_newton. The FP32 buffers are the cascade's own (free until stage C).
struct NewtonBufs {
  Cx<float> *F1, *F2, *F3, *F4;   // (P, n, n): Omega^2/T/W32/LU(W), Z/W in FP32, X/E, G/W E
  Cx<float> *wr, *tau;            // (P, n)
  int* piv;                       // (P, n)
  cplx* lam;                      // (P, n)
};

// Outputs as stage_b<df64>: bigW in Wd and bigV in Vd as double-float, w/q/X in FP64.
// Wd, Vd, Om: (P, n, n) complex128-sized buffers (FP64 W; scratch of the Omega^2 W products).
// With for_cascade false the modes stay Cartesian FP64 W and V (wb_layer_modes' outputs): no s/p
// rotation, no double-float conversion; c and sn are not read.
void stage_b_newton(cudaStream_t s, int P, int N, const cplx* conv, const int* pair_layer, const int* pair_solve,
                    const double* pair_thick, const double* wavelength, const double* kx, const double* ky,
                    cplx* Wd, cplx* Vd, cplx* Om, NewtonBufs& nb, GroupBufs& gb, cplx* w, cplx* q, cplx* X,
                    const double* c, const double* sn, int32_t* st, int st_div, bool for_cascade) {
  TraceRange trace_("wb:stage_b.newton");
  const int n = 2 * N;
  const long long n2 = (long long)n * n, NN = (long long)N * N, tot = (long long)P * n2;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  using F = Cx<float>;
  // FP32 eigenpairs
  {
    dim3 gr((N + 63) / 64, (N + 63) / 64, P * 4);
    omega2_kernel<float><<<gr, 256, 0, s>>>(N, conv, 3 * NN, pair_layer, pair_solve, kx, ky, nb.F1, n2); note_launch();
  }
  geev_schur<float>(s, P, n, nb.F1, n, n2, nb.F2, n, n2, nb.wr, nb.tau, st, st_div, nb.F3, n2);   // F3: free here
  trevc<float>(s, P, n, nb.F1, n, n2, nb.F3, n, n2);
  gemm<float>(s, P, n, n, n, one, nb.F2, 1, n, n2, nb.F3, 1, n, n2, zero, nb.F1, 1, n, n2);
  normalize_columns<float>(s, P, n, nb.F1, n, n2);
  widen_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, nb.F1, Wd); note_launch();
  widen_kernel<<<nblk((long long)P * n, 256), 256, 0, s>>>((long long)P * n, nb.wr, nb.lam); note_launch();
  // scratch for Omega^2 W: T, U in Om; S in F3 (as complex128); Y in Vd
  const long long Nn = (long long)N * n, totN = (long long)P * Nn;
  Cx<double>* Tm = (Cx<double>*)Om;
  Cx<double>* Um = Tm + totN;
  Cx<double>* Sm = (Cx<double>*)nb.F3;
  Cx<double>* Ym = (Cx<double>*)Vd;
  const Cx<double>* cv = (const Cx<double>*)conv;
  const size_t gsm = (size_t)n * (sizeof(cplx) + 5 * sizeof(int));
  cudaFuncSetAttribute(group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gsm);
  for (int it = 0; it < kNewtonSteps; ++it) {
    if (it > 0) convert<double, float>(s, (const Cx<double>*)Wd, nb.F1, tot);
    cudaMemcpyAsync(nb.F2, nb.F1, sizeof(F) * tot, cudaMemcpyDeviceToDevice, s);   // W in FP32 for W E
    getrf<float>(s, P, n, nb.F1, n, n2, nb.piv, n, st, st_div);                    // LU of W in FP32
    // the residual's three slot products, FP64 operands accumulated in double-float (FP32 pipes)
    zgemm_dd_idx(s, P, N, n, N, one, conv, 1, N, 3 * NN, pair_layer, Wd, 1, n, n2, zero, (cplx*)Tm, 1, N, Nn);
    zgemm_dd_idx(s, P, N, n, N, one, conv + NN, 1, N, 3 * NN, pair_layer, Wd + N, 1, n, n2, zero, (cplx*)Um, 1, N,
                 Nn);
    omw_s_kernel<<<nblk(totN, 256), 256, 0, s>>>(totN, N, n, pair_solve, kx, ky, (const cplx*)Tm, (const cplx*)Um,
                                                 (cplx*)Sm);
    note_launch();
    zgemm_dd_idx(s, P, N, n, N, one, conv + 2 * NN, 1, N, 3 * NN, pair_layer, (const cplx*)Sm, 1, N, Nn, zero,
                 (cplx*)Ym, 1, N, Nn);
    omw_resid_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, N, n, pair_solve, kx, ky, (const cplx*)Tm, (const cplx*)Um,
                                                    (const cplx*)Ym, Wd, nb.lam, nb.F4);
    note_launch();
    getrs<float>(s, P, n, nb.F1, n, n2, nb.piv, n, nb.F4, n, n, n2, 0);            // G = W32^-1 R
    group_init_kernel<<<nblk((long long)gb.cap * kGroupMax * kGroupMax, 256), 256, 0, s>>>(gb.cap, gb.A, gb.count);
    note_launch();
    group_kernel<<<P, 256, gsm, s>>>(n, nb.F4, nb.lam, nb.F3, gb, st, st_div); note_launch();
    gemm<float>(s, P, n, n, n, one, nb.F2, 1, n, n2, nb.F3, 1, n, n2, zero, nb.F4, 1, n, n2);   // W E
    accumulate_kernel<float, double><<<nblk(tot, 256), 256, 0, s>>>(tot, nb.F4, (Cx<double>*)Wd); note_launch();
    // exact diagonalisation of the groups
    Cx<double>* A = (Cx<double>*)gb.A;
    Cx<double>* Zs = (Cx<double>*)gb.Z;
    Cx<double>* Xs = (Cx<double>*)gb.X;
    const long long b2 = (long long)kGroupMax * kGroupMax;
    geev_schur<double>(s, gb.cap, kGroupMax, A, kGroupMax, b2, Zs, kGroupMax, b2, (Cx<double>*)gb.w,
                       (Cx<double>*)gb.tau, nullptr, 1);
    trevc<double>(s, gb.cap, kGroupMax, A, kGroupMax, b2, Xs, kGroupMax, b2);
    gemm<double>(s, gb.cap, kGroupMax, kGroupMax, kGroupMax, one, Zs, 1, kGroupMax, b2, Xs, 1, kGroupMax, b2, zero,
                 A, 1, kGroupMax, b2);
    normalize_columns<double>(s, gb.cap, kGroupMax, A, kGroupMax, b2);
    group_apply_kernel<<<gb.cap, 256, 0, s>>>(n, n2, gb, Wd, nb.lam, st, st_div); note_launch();
    group2_apply_kernel<<<nblk(32LL * gb.cap2, 256), 256, 0, s>>>(n, n2, gb, Wd, nb.lam); note_launch();
    normalize_columns<double>(s, P, n, (Cx<double>*)Wd, n, n2);
  }
  // q, X, V and the s/p rotation in FP64, then the double-float form the cascade reads
  modeq_kernel<double><<<P, 256, 0, s>>>(P, n, (const Cx<double>*)nb.lam, pair_solve, pair_thick, wavelength, w, q, X, st);
  note_launch();
  // V = Omega_R W / q: the two slot products in double-float (T = epy W_bot, U = epx W_top into
  // the residual's scratch), the diagonal terms and the division by q elementwise
  zgemm_dd_idx(s, P, N, n, N, one, conv + NN, 1, N, 3 * NN, pair_layer, Wd + N, 1, n, n2, zero, (cplx*)Tm, 1, N, Nn);
  zgemm_dd_idx(s, P, N, n, N, one, conv, 1, N, 3 * NN, pair_layer, Wd, 1, n, n2, zero, (cplx*)Um, 1, N, Nn);
  vmodes_epilogue_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, N, n, pair_solve, kx, ky, (const cplx*)Tm, (const cplx*)Um,
                                                        Wd, q, Vd);
  note_launch();
  if (!for_cascade) return;
  sp_rotate_kernel<double><<<nblk((long long)P * N * n, 256), 256, 0, s>>>(P, N, pair_solve, c, sn, (Cx<double>*)Wd,
                                                                          (Cx<double>*)Vd, n2);
  note_launch();
  to_df64_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, Wd); note_launch();
  to_df64_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, Vd); note_launch();
}

// ------------------------------------------------------------------- stage C driver
// Bottom-up reflections, top-down incidence pass and efficiencies, in precision RC.
// bW, bV: (P, n, n) LU-factored bigW / bigV with pivots; X: FP64 (P, n).
// Bottom-up half of the cascade: R_L = diag(t11), then R_l for l = L-1 .. 0, leaving in Mk the
// LU factors of every layer's M and, when Ak is given, those of every layer's A (the matrix
// whose solve yields R_l); otherwise A lives in S1 only for the duration of its layer.
template <class RC>
void cascade_factor(cudaStream_t s, int Bc, int L, int N, Cx<RC>* bW, Cx<RC>* bV, const int* pivW, const int* pivV,
                    const cplx* X, const PortVectors& pv, int32_t* st, Cx<RC>* Mk, int* pivM, Cx<RC>* Rk,
                    Cx<RC>* S1, Cx<RC>* S2, Cx<RC>* S3, int* pivS, Cx<RC>* Ak, int* pivA) {
  const int n = 2 * N;
  const long long n2 = (long long)n * n;
  const long long lay_bs = (long long)L * n2, lay_ps = (long long)L * n, r_bs = (long long)(L + 1) * n2;
  diag_matrix_kernel<RC><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, pv.t11, Rk + (long long)L * n2, r_bs);
  note_launch();
  const dim3 tgrid((n + 31) / 32, (n + 31) / 32, Bc), tblk(32, 8);
  for (int l = L - 1; l >= 0; --l) {
    Cx<RC>* bWl = bW + (long long)l * n2;  const int* pW = pivW + (long long)l * n;
    Cx<RC>* bVl = bV + (long long)l * n2;  const int* pV = pivV + (long long)l * n;
    Cx<RC>* M = Mk + (long long)l * n2;    int* pM = pivM + (long long)l * n;
    const Cx<RC>* Rb = Rk + (long long)(l + 1) * n2;
    u12_kernel<RC><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, Rb, r_bs, pv.wg, pv.vg, S1, S2, n2); note_launch();
    getrs<RC>(s, Bc, n, bWl, n, lay_bs, pW, lay_ps, S1, n, n, n2, 0);            // P1 = bigW^-1 U1
    getrs<RC>(s, Bc, n, bVl, n, lay_bs, pV, lay_ps, S2, n, n, n2, 0);            // P2 = bigV^-1 U2
    mn2_kernel<RC><<<tgrid, tblk, 0, s>>>(n, S1, S2, n2, M, lay_bs, S3); note_launch();   // M, N^T
    getrf<RC>(s, Bc, n, M, n, lay_bs, pM, lay_ps, st, 1);
    getrs<RC>(s, Bc, n, M, n, lay_bs, pM, lay_ps, S3, n, n, n2, 1);             // rho_b^T = M^-T N^T
    rho_kernel<RC><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, S3, S2, X + (long long)l * n, lay_ps, n2);
    note_launch();
    getrs<RC>(s, Bc, n, bWl, n, lay_bs, pW, lay_ps, S2, n, n, n2, 1);            // X1^T
    getrs<RC>(s, Bc, n, bVl, n, lay_bs, pV, lay_ps, S3, n, n, n2, 1);            // X2^T
    Cx<RC>* Rl = Rk + (long long)l * n2;
    Cx<RC>* A = Ak ? Ak + (long long)l * n2 : S1;
    int* pA = Ak ? pivA + (long long)l * n : pivS;
    const long long a_bs = Ak ? lay_bs : n2, pa_bs = Ak ? lay_ps : n;
    ab2_kernel<RC><<<tgrid, tblk, 0, s>>>(n, S2, S3, n2, pv.wg, pv.vg, A, a_bs, Rl, r_bs); note_launch();
    getrf<RC>(s, Bc, n, A, n, a_bs, pA, pa_bs, st, 1);
    getrs<RC>(s, Bc, n, A, n, a_bs, pA, pa_bs, Rl, n, n, r_bs, 0);              // R_l
  }
}

template <class RC>
void stage_c(cudaStream_t s, Arena& ar, int Bc, int L, int N, Cx<RC>* bW, Cx<RC>* bV, const int* pivW,
             const int* pivV, const cplx* X, const PortVectors& pv, const SolveDesc& d, int first,
             const SolveOut& out, int32_t* st, Cx<RC>* Mk, int* pivM, Cx<RC>* Rk, Cx<RC>* S1, Cx<RC>* S2,
             Cx<RC>* S3, int* pivS, Cx<RC>* Cin, Cx<RC>* g, Cx<RC>* h, Cx<RC>* r1, Cx<RC>* r2, Cx<RC>* cref) {
  TraceRange trace_("wb:stage_c");
  const int n = 2 * N;
  const long long n2 = (long long)n * n;
  const long long lay_bs = (long long)L * n2, lay_ps = (long long)L * n, r_bs = (long long)(L + 1) * n2;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  cascade_factor<RC>(s, Bc, L, N, bW, bV, pivW, pivV, X, pv, st, Mk, pivM, Rk, S1, S2, S3, pivS, nullptr, nullptr);
  const long long v3 = (long long)n * 3;
  incident_kernel<RC><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, N, d.pol + 2 * first, pv.nt, Cin, v3); note_launch();
  top_kernel<RC><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, Rk, r_bs, pv.r22, S1, n2); note_launch();
  getrf<RC>(s, Bc, n, S1, n, n2, pivS, n, st, 1);
  dscale3_kernel<RC><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, n, pv.r21, Cin, v3, nullptr, nullptr, 0, g, v3);
  note_launch();
  getrs<RC>(s, Bc, n, S1, n, n2, pivS, n, g, 3, n, v3, 0);                      // g_0
  gemm<RC>(s, Bc, n, 3, n, one, Rk, 1, n, r_bs, g, 1, n, v3, zero, h, 1, n, v3);
  dscale3_kernel<RC><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, n, pv.r11, Cin, v3, pv.r12, h, v3, cref, v3);
  note_launch();
  for (int l = 0; l < L; ++l) {
    Cx<RC>* bWl = bW + (long long)l * n2;  const int* pW = pivW + (long long)l * n;
    Cx<RC>* bVl = bV + (long long)l * n2;  const int* pV = pivV + (long long)l * n;
    Cx<RC>* M = Mk + (long long)l * n2;    const int* pM = pivM + (long long)l * n;
    if (l > 0) gemm<RC>(s, Bc, n, 3, n, one, Rk + (long long)l * n2, 1, n, r_bs, g, 1, n, v3, zero, h, 1, n, v3);
    gh_kernel<RC><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, n, g, h, pv.wg, pv.vg, r1, r2, v3); note_launch();
    getrs<RC>(s, Bc, n, bWl, n, lay_bs, pW, lay_ps, r1, 3, n, v3, 0);
    getrs<RC>(s, Bc, n, bVl, n, lay_bs, pV, lay_ps, r2, 3, n, v3, 0);
    ct_kernel<RC><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, n, r1, r2, X + (long long)l * n, lay_ps, g, v3);
    note_launch();
    getrs<RC>(s, Bc, n, M, n, lay_bs, pM, lay_ps, g, 3, n, v3, 0);              // g_{l+1}
  }
  dscale3_kernel<RC><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, n, pv.t21, g, v3, nullptr, nullptr, 0, h, v3);
  note_launch();
  efficiency_kernel<RC><<<nblk((long long)Bc * N * 3, 256), 256, 0, s>>>(
      Bc, N, cref, h, v3, pv, d.eps_top + first, d.eps_bot + first, d.pol + 2 * first,
      out.R + (long long)first * 3 * N, out.T + (long long)first * 3 * N,
      out.amps ? out.amps + (long long)first * 12 * N : nullptr, st);
  note_launch();
}

// --------------------------------------------------- cascade with FP64-class refinement
// The mixed form factors the cascade in FP32 (cascade_factor<float>) and then solves the
// interface equations of the whole stack by defect correction: the residual of the exact
// equations is evaluated in double-float with the double-float modes of stage B, and the FP32
// factors solve for the correction. Unknowns per solve and incidence column: the gap amplitudes
// g_l (down) and h_l (up) above layer l (l = 0..L, L = the gap above the substrate) and the modal
// amplitudes c+_l (down, at the top of layer l) and c-_l (up, at its bottom). Equations:
//   top     g_0 - r21 C - r22 h_0                      = 0
//   E1      W (c+ + X c-)  - wg (g_l + h_l)            = 0        (tangential E, top of layer l)
//   E2      V (c+ - X c-)  - vg (g_l - h_l)            = 0        (tangential H, top)
//   E3      W (X c+ + c-)  - wg (g_l+1 + h_l+1)        = 0        (tangential E, bottom)
//   E4      V (X c+ - c-)  - vg (g_l+1 - h_l+1)        = 0        (tangential H, bottom)
//   bottom  h_L - t11 g_L                              = 0
// with c_ref = r11 C + r12 h_0 and c_trn = t21 g_L read off the solution (scattering.py:907-994
// reads the same two blocks). Eliminating layer by layer from the bottom with right-hand sides
// f1..f4 on E1..E4 gives h_l = R_l g_l + s_l with the cascade's R_l and
//   a3 = W^-1 (wg s' + f3),  a4 = V^-1 (-vg s' + f4)
//   sigma = ((a3 - a4) - rho_b (a3 + a4)) / 2,   rho_b = N M^-1
//   s_l = A^-1 (2 X sigma - (W^-1 f1 - V^-1 f2) + X rho_b X (W^-1 f1 + V^-1 f2))
// and from the top g_0 = G0^-1 (r22 s_0 + f_top), then per layer
//   c+ = (W^-1 (wg (g + h) + f1) + V^-1 (vg (g - h) + f2)) / 2
//   g' = M^-1 (2 X c+ - (a3 + a4)),   c- = rho_b X c+ + sigma.
// Without sources this is the cascade's own top-down pass. N y = W^-1 wg (y + R' y) -
// V^-1 vg (y - R' y) is applied from R' and the factors of W and V.
//
// Vector layouts: per-solve blocks of k columns of length n (column-major, batch stride given);
// per (solve, layer) arrays (Bc, L, 3, n); gap arrays (Bc, L+1, 3, n).

// WB = [wg s' + f3 | f1], VB = [-vg s' + f4 | f2]
template <class R>
__global__ void bu_rhs_kernel(int Bc, int n, const Cx<R>* __restrict__ sn, long long s_bs, const Cx<R>* __restrict__ f1,
                              const Cx<R>* __restrict__ f2, const Cx<R>* __restrict__ f3, const Cx<R>* __restrict__ f4,
                              long long f_bs, const cplx* __restrict__ wg, const cplx* __restrict__ vg,
                              Cx<R>* __restrict__ WB, Cx<R>* __restrict__ VB) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const Cx<R> sv = sn[b * s_bs + rem];
  const long long o = b * 6LL * n;
  WB[o + rem] = ld<R>(wg + b * n + i) * sv + f3[b * f_bs + rem];
  WB[o + 3LL * n + rem] = f1[b * f_bs + rem];
  VB[o + rem] = f4[b * f_bs + rem] - ld<R>(vg + b * n + i) * sv;
  VB[o + 3LL * n + rem] = f2[b * f_bs + rem];
}

// from WB = [a3 | W^-1 f1], VB = [a4 | V^-1 f2]: Y = [a3 + a4 | X (W^-1 f1 + V^-1 f2)],
// asum = a3 + a4, sig = a3 - a4 (completed later), D = W^-1 f1 - V^-1 f2
template <class R>
__global__ void bu_y_kernel(int Bc, int n, const Cx<R>* __restrict__ WB, const Cx<R>* __restrict__ VB,
                            const cplx* __restrict__ X, long long x_bs, Cx<R>* __restrict__ Y,
                            Cx<R>* __restrict__ asum, Cx<R>* __restrict__ sig, long long f_bs, Cx<R>* __restrict__ D) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const long long o = b * 6LL * n;
  const Cx<R> a3 = WB[o + rem], a4 = VB[o + rem];
  const Cx<R> w1 = WB[o + 3LL * n + rem], v2 = VB[o + 3LL * n + rem];
  const Cx<R> x = ld<R>(X + b * x_bs + i);
  Y[o + rem] = a3 + a4;
  Y[o + 3LL * n + rem] = x * (w1 + v2);
  asum[b * f_bs + rem] = a3 + a4;
  sig[b * f_bs + rem] = a3 - a4;
  D[b * 3LL * n + rem] = w1 - v2;
}

// U1 = wg (Z + Rz), U2 = vg (Z - Rz), k columns, batch stride zs
template <class R>
__global__ void nz_kernel(int Bc, int n, int k, const Cx<R>* __restrict__ Z, long long zs, const Cx<R>* __restrict__ Rz,
                          const cplx* __restrict__ wg, const cplx* __restrict__ vg, Cx<R>* __restrict__ U1,
                          Cx<R>* __restrict__ U2) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * k) return;
  const long long b = idx / ((long long)k * n);
  const int rem = (int)(idx % ((long long)k * n)), i = rem % n;
  const Cx<R> z = Z[b * zs + rem], r = Rz[b * (long long)k * n + rem];
  U1[b * (long long)k * n + rem] = ld<R>(wg + b * n + i) * (z + r);
  U2[b * (long long)k * n + rem] = ld<R>(vg + b * n + i) * (z - r);
}

// NZ = U1 - U2 = rho_b Y:  sigma = (sig - NZ[:, :3]) / 2 ;  rhs = 2 X sigma - D + X NZ[:, 3:]
template <class R>
__global__ void bu_src_kernel(int Bc, int n, const Cx<R>* __restrict__ U1, const Cx<R>* __restrict__ U2,
                              const cplx* __restrict__ X, long long x_bs, Cx<R>* __restrict__ sig, long long f_bs,
                              const Cx<R>* __restrict__ D, Cx<R>* __restrict__ rhs, long long r_bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const long long o = b * 6LL * n;
  const Cx<R> nz0 = U1[o + rem] - U2[o + rem];
  const Cx<R> nz1 = U1[o + 3LL * n + rem] - U2[o + 3LL * n + rem];
  const Cx<R> x = ld<R>(X + b * x_bs + i);
  const Cx<R> sg = (sig[b * f_bs + rem] - nz0) * R(0.5);
  sig[b * f_bs + rem] = sg;
  rhs[b * r_bs + rem] = x * (sg * R(2.0)) - D[b * 3LL * n + rem] + x * nz1;
}

// out = d * a + c  (n x 3 per solve; d per-solve diagonal, FP64)
template <class R>
__global__ void diag_axpy3_kernel(int Bc, int n, const cplx* __restrict__ d, const Cx<R>* __restrict__ a, long long a_bs,
                                  const Cx<R>* __restrict__ c, long long c_bs, Cx<R>* __restrict__ out, long long o_bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  out[b * o_bs + rem] = ld<R>(d + b * n + i) * a[b * a_bs + rem] + c[b * c_bs + rem];
}

// WB = wg (g + h) + f1, VB = vg (g - h) + f2  (3 columns at stride 6n)
template <class R>
__global__ void td_rhs_kernel(int Bc, int n, const Cx<R>* __restrict__ g, const Cx<R>* __restrict__ h, long long g_bs,
                              const Cx<R>* __restrict__ f1, const Cx<R>* __restrict__ f2, long long f_bs,
                              const cplx* __restrict__ wg, const cplx* __restrict__ vg, Cx<R>* __restrict__ WB,
                              Cx<R>* __restrict__ VB) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const Cx<R> gg = g[b * g_bs + rem], hh = h[b * g_bs + rem];
  WB[b * 6LL * n + rem] = ld<R>(wg + b * n + i) * (gg + hh) + f1[b * f_bs + rem];
  VB[b * 6LL * n + rem] = ld<R>(vg + b * n + i) * (gg - hh) + f2[b * f_bs + rem];
}

// c+ = (WB + VB) / 2 ; Y = [X c+ | 2 X c+ - asum]
template <class R>
__global__ void td_cp_kernel(int Bc, int n, const Cx<R>* __restrict__ WB, const Cx<R>* __restrict__ VB,
                             const cplx* __restrict__ X, long long x_bs, const Cx<R>* __restrict__ asum,
                             Cx<R>* __restrict__ cp, long long f_bs, Cx<R>* __restrict__ Y) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const Cx<R> c = (WB[b * 6LL * n + rem] + VB[b * 6LL * n + rem]) * R(0.5);
  cp[b * f_bs + rem] = c;
  const Cx<R> xc = ld<R>(X + b * x_bs + i) * c;
  Y[b * 6LL * n + rem] = xc;
  Y[b * 6LL * n + 3LL * n + rem] = xc * R(2.0) - asum[b * f_bs + rem];
}

// c- = U1 - U2 + sigma ; g_next = Y[:, 3:]
template <class R>
__global__ void td_cm_kernel(int Bc, int n, const Cx<R>* __restrict__ U1, const Cx<R>* __restrict__ U2,
                             const Cx<R>* __restrict__ sig, Cx<R>* __restrict__ cm, long long f_bs,
                             const Cx<R>* __restrict__ Y, Cx<R>* __restrict__ gn, long long g_bs) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n));
  cm[b * f_bs + rem] = U1[b * 3LL * n + rem] - U2[b * 3LL * n + rem] + sig[b * f_bs + rem];
  gn[b * g_bs + rem] = Y[b * 6LL * n + 3LL * n + rem];
}

// per (solve, layer) pair: UW = [c+ + X c- | X c+ + c-], UV = [c+ - X c- | X c+ - c-]
template <class R>
__global__ void res_u_kernel(int P, int n, const Cx<R>* __restrict__ cp, const Cx<R>* __restrict__ cm,
                             const cplx* __restrict__ X, Cx<R>* __restrict__ UW, Cx<R>* __restrict__ UV) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)P * n * 3) return;
  const long long p = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const Cx<R> a = cp[p * 3LL * n + rem], c = cm[p * 3LL * n + rem];
  const Cx<R> x = ld<R>(X + p * n + i);
  const Cx<R> xa = x * a, xc = x * c;
  UW[p * 6LL * n + rem] = a + xc;
  UW[p * 6LL * n + 3LL * n + rem] = xa + c;
  UV[p * 6LL * n + rem] = a - xc;
  UV[p * 6LL * n + 3LL * n + rem] = xa - c;
}

// negated residuals of E1..E4 as FP32 right-hand sides (YW = W UW, YV = V UV)
template <class R>
__global__ void res_f_kernel(int P, int L, int n, const Cx<R>* __restrict__ YW, const Cx<R>* __restrict__ YV,
                             const Cx<R>* __restrict__ g, const Cx<R>* __restrict__ h, const cplx* __restrict__ wg,
                             const cplx* __restrict__ vg, Cx<float>* __restrict__ f1, Cx<float>* __restrict__ f2,
                             Cx<float>* __restrict__ f3, Cx<float>* __restrict__ f4) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)P * n * 3) return;
  const long long p = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const long long b = p / L, l = p % L;
  const long long gt = (b * (L + 1) + l) * 3LL * n + rem, gb = gt + 3LL * n;
  const Cx<R> w = ld<R>(wg + b * n + i), v = ld<R>(vg + b * n + i);
  const Cx<R> g0 = g[gt], h0 = h[gt], g1 = g[gb], h1 = h[gb];
  const Cx<R> e1 = YW[p * 6LL * n + rem] - w * (g0 + h0);
  const Cx<R> e3 = YW[p * 6LL * n + 3LL * n + rem] - w * (g1 + h1);
  const Cx<R> e2 = YV[p * 6LL * n + rem] - v * (g0 - h0);
  const Cx<R> e4 = YV[p * 6LL * n + 3LL * n + rem] - v * (g1 - h1);
  auto neg32 = [](Cx<R> e) { return cxmk<float>((float)(-rto(e.x)), (float)(-rto(e.y))); };
  f1[p * 3LL * n + rem] = neg32(e1);
  f2[p * 3LL * n + rem] = neg32(e2);
  f3[p * 3LL * n + rem] = neg32(e3);
  f4[p * 3LL * n + rem] = neg32(e4);
}

// negated residuals of the top and bottom port equations
template <class R>
__global__ void res_tb_kernel(int Bc, int L, int n, const Cx<R>* __restrict__ g, const Cx<R>* __restrict__ h,
                              const Cx<R>* __restrict__ Cin, const cplx* __restrict__ r21, const cplx* __restrict__ r22,
                              const cplx* __restrict__ t11, Cx<float>* __restrict__ ft, Cx<float>* __restrict__ fb) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)Bc * n * 3) return;
  const long long b = idx / (3LL * n);
  const int rem = (int)(idx % (3LL * n)), i = rem % n;
  const long long top = b * (L + 1) * 3LL * n + rem, bot = top + (long long)L * 3 * n;
  const Cx<R> et = g[top] - ld<R>(r21 + b * n + i) * Cin[b * 3LL * n + rem] - ld<R>(r22 + b * n + i) * h[top];
  const Cx<R> eb = h[bot] - ld<R>(t11 + b * n + i) * g[bot];
  ft[b * 3LL * n + rem] = cxmk<float>((float)(-rto(et.x)), (float)(-rto(et.y)));
  fb[b * 3LL * n + rem] = cxmk<float>((float)(-rto(eb.x)), (float)(-rto(eb.y)));
}

// Work arrays of the refinement (FP32 unless noted), carved from the arena.
struct RefineBufs {
  using F = Cx<float>;
  using D = Cx<df64>;
  F *f1, *f2, *f3, *f4;           // (Bc, L, 3, n) right-hand sides of E1..E4
  F *ft, *fb;                     // (Bc, 3, n)
  F *sv, *asum, *sig;             // s: (Bc, L+1, 3, n); asum, sig: (Bc, L, 3, n)
  F *dg, *dh, *dcp, *dcm;         // corrections
  F *WB, *VB, *Y, *Rz, *U1, *U2;  // (Bc, 6, n) scratch
  F *Dv;                          // (Bc, 3, n)
  D *g, *h, *cp, *cm;             // double-float state
  D *UW, *UV, *YW, *YV;           // (P, 6, n) residual products
  D *Cin, *cref, *ctrn;           // (Bc, 3, n)
  bool carve(Arena& ar, int Bc, int L, int n) {
    const size_t P = (size_t)Bc * L, v = 3 * (size_t)n, G = (size_t)Bc * (L + 1);
    f1 = ar.get<F>(P * v); f2 = ar.get<F>(P * v); f3 = ar.get<F>(P * v); f4 = ar.get<F>(P * v);
    ft = ar.get<F>(Bc * v); fb = ar.get<F>(Bc * v);
    sv = ar.get<F>(G * v); asum = ar.get<F>(P * v); sig = ar.get<F>(P * v);
    dg = ar.get<F>(G * v); dh = ar.get<F>(G * v); dcp = ar.get<F>(P * v); dcm = ar.get<F>(P * v);
    WB = ar.get<F>(2 * Bc * v); VB = ar.get<F>(2 * Bc * v); Y = ar.get<F>(2 * Bc * v);
    Rz = ar.get<F>(2 * Bc * v); U1 = ar.get<F>(2 * Bc * v); U2 = ar.get<F>(2 * Bc * v);
    Dv = ar.get<F>(Bc * v);
    g = ar.get<D>(G * v); h = ar.get<D>(G * v); cp = ar.get<D>(P * v); cm = ar.get<D>(P * v);
    UW = ar.get<D>(2 * P * v); UV = ar.get<D>(2 * P * v); YW = ar.get<D>(2 * P * v); YV = ar.get<D>(2 * P * v);
    Cin = ar.get<D>(Bc * v); cref = ar.get<D>(Bc * v); ctrn = ar.get<D>(Bc * v);
    return ar.ok();
  }
  static size_t bytes(int Bc, int L, int n) {
    const size_t P = (size_t)Bc * L, v = 3 * (size_t)n, G = (size_t)Bc * (L + 1);
    size_t b = 0;
    auto A = [&](size_t x) { b += (x + 255) & ~(size_t)255; };
    for (int k = 0; k < 4; ++k) A(8 * P * v);
    A(8 * Bc * v); A(8 * Bc * v);
    A(8 * G * v); A(8 * P * v); A(8 * P * v);
    A(8 * G * v); A(8 * G * v); A(8 * P * v); A(8 * P * v);
    for (int k = 0; k < 6; ++k) A(8 * 2 * Bc * v);
    A(8 * Bc * v);
    A(16 * G * v); A(16 * G * v); A(16 * P * v); A(16 * P * v);
    for (int k = 0; k < 4; ++k) A(16 * 2 * P * v);
    for (int k = 0; k < 3; ++k) A(16 * Bc * v);
    return b;
  }
};

// One FP32 solve of the interface equations with right-hand sides rb.f*, from the factors left by
// cascade_factor<float> (bW, bV, Mk, Ak with pivots; Rk; G0 in S1 with pivS). Writes the
// solution to rb.dg, rb.dh, rb.dcp, rb.dcm.
static void cascade_sources(cudaStream_t s, int Bc, int L, int n, const Cx<float>* bW, const Cx<float>* bV,
                            const int* pivW, const int* pivV, const Cx<float>* Mk, const int* pivM,
                            const Cx<float>* Ak, const int* pivA, const Cx<float>* Rk, const Cx<float>* G0,
                            const int* pivG, const cplx* X, const PortVectors& pv, RefineBufs& rb) {
  TraceRange trace_("wb:stage_c.sources");
  using F = Cx<float>;
  const long long n2 = (long long)n * n, v3 = 3LL * n, v6 = 6LL * n;
  const long long lay_bs = (long long)L * n2, lay_ps = (long long)L * n, r_bs = (long long)(L + 1) * n2;
  const long long f_bs = (long long)L * v3, g_bs = (long long)(L + 1) * v3;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  const unsigned nb3 = nblk((long long)Bc * v3, 256), nb6 = nblk((long long)Bc * v6, 256);
  // bottom: h_L = t11 g_L + s_L with s_L = f_bottom
  cudaMemcpy2DAsync(rb.sv + (long long)L * v3, g_bs * sizeof(F), rb.fb, v3 * sizeof(F), v3 * sizeof(F), Bc,
                    cudaMemcpyDeviceToDevice, s);
  for (int l = L - 1; l >= 0; --l) {
    const F* Wl = bW + (long long)l * n2;  const int* pW = pivW + (long long)l * n;
    const F* Vl = bV + (long long)l * n2;  const int* pV = pivV + (long long)l * n;
    const F* Ml = Mk + (long long)l * n2;  const int* pM = pivM + (long long)l * n;
    const F* Al = Ak + (long long)l * n2;  const int* pA = pivA + (long long)l * n;
    const F* Rn = Rk + (long long)(l + 1) * n2;
    const long long fo = (long long)l * v3;
    bu_rhs_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, rb.sv + (long long)(l + 1) * v3, g_bs, rb.f1 + fo, rb.f2 + fo,
                                             rb.f3 + fo, rb.f4 + fo, f_bs, pv.wg, pv.vg, rb.WB, rb.VB);
    note_launch();
    getrs<float>(s, Bc, n, Wl, n, lay_bs, pW, lay_ps, rb.WB, 6, n, v6, 0);
    getrs<float>(s, Bc, n, Vl, n, lay_bs, pV, lay_ps, rb.VB, 6, n, v6, 0);
    bu_y_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, rb.WB, rb.VB, X + (long long)l * n, lay_ps, rb.Y, rb.asum + fo,
                                           rb.sig + fo, f_bs, rb.Dv);
    note_launch();
    getrs<float>(s, Bc, n, Ml, n, lay_bs, pM, lay_ps, rb.Y, 6, n, v6, 0);           // Z = M^-1 Y
    gemm<float>(s, Bc, n, 6, n, one, Rn, 1, n, r_bs, rb.Y, 1, n, v6, zero, rb.Rz, 1, n, v6);
    nz_kernel<float><<<nb6, 256, 0, s>>>(Bc, n, 6, rb.Y, v6, rb.Rz, pv.wg, pv.vg, rb.U1, rb.U2); note_launch();
    getrs<float>(s, Bc, n, Wl, n, lay_bs, pW, lay_ps, rb.U1, 6, n, v6, 0);
    getrs<float>(s, Bc, n, Vl, n, lay_bs, pV, lay_ps, rb.U2, 6, n, v6, 0);
    bu_src_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, rb.U1, rb.U2, X + (long long)l * n, lay_ps, rb.sig + fo, f_bs,
                                             rb.Dv, rb.sv + (long long)l * v3, g_bs);
    note_launch();
    getrs<float>(s, Bc, n, Al, n, lay_bs, pA, lay_ps, rb.sv + (long long)l * v3, 3, n, g_bs, 0);   // s_l
  }
  // top: g_0 = G0^-1 (r22 s_0 + f_top)
  diag_axpy3_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, pv.r22, rb.sv, g_bs, rb.ft, v3, rb.dg, g_bs); note_launch();
  getrs<float>(s, Bc, n, G0, n, n2, pivG, n, rb.dg, 3, n, g_bs, 0);
  // h_l = s_l + R_l g_l for every l < L is formed layer by layer below
  for (int l = 0; l < L; ++l) {
    const F* Wl = bW + (long long)l * n2;  const int* pW = pivW + (long long)l * n;
    const F* Vl = bV + (long long)l * n2;  const int* pV = pivV + (long long)l * n;
    const F* Ml = Mk + (long long)l * n2;  const int* pM = pivM + (long long)l * n;
    const long long fo = (long long)l * v3, go = (long long)l * v3;
    cudaMemcpy2DAsync(rb.dh + go, g_bs * sizeof(F), rb.sv + go, g_bs * sizeof(F), v3 * sizeof(F), Bc,
                      cudaMemcpyDeviceToDevice, s);
    gemm<float>(s, Bc, n, 3, n, one, Rk + (long long)l * n2, 1, n, r_bs, rb.dg + go, 1, n, g_bs, one, rb.dh + go, 1, n,
                g_bs);                                                                   // h_l
    td_rhs_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, rb.dg + go, rb.dh + go, g_bs, rb.f1 + fo, rb.f2 + fo, f_bs,
                                             pv.wg, pv.vg, rb.WB, rb.VB);
    note_launch();
    getrs<float>(s, Bc, n, Wl, n, lay_bs, pW, lay_ps, rb.WB, 3, n, v6, 0);
    getrs<float>(s, Bc, n, Vl, n, lay_bs, pV, lay_ps, rb.VB, 3, n, v6, 0);
    td_cp_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, rb.WB, rb.VB, X + (long long)l * n, lay_ps, rb.asum + fo,
                                            rb.dcp + fo, f_bs, rb.Y);
    note_launch();
    getrs<float>(s, Bc, n, Ml, n, lay_bs, pM, lay_ps, rb.Y, 6, n, v6, 0);           // [M^-1 X c+ | g_l+1]
    gemm<float>(s, Bc, n, 3, n, one, Rk + (long long)(l + 1) * n2, 1, n, r_bs, rb.Y, 1, n, v6, zero, rb.Rz, 1, n, v3);
    nz_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, 3, rb.Y, v6, rb.Rz, pv.wg, pv.vg, rb.U1, rb.U2); note_launch();
    getrs<float>(s, Bc, n, Wl, n, lay_bs, pW, lay_ps, rb.U1, 3, n, v3, 0);
    getrs<float>(s, Bc, n, Vl, n, lay_bs, pV, lay_ps, rb.U2, 3, n, v3, 0);
    td_cm_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, rb.U1, rb.U2, rb.sig + fo, rb.dcm + fo, f_bs, rb.Y,
                                            rb.dg + go + v3, g_bs);
    note_launch();
  }
  // h_L = t11 g_L + s_L
  diag_axpy3_kernel<float><<<nb3, 256, 0, s>>>(Bc, n, pv.t11, rb.dg + (long long)L * v3, g_bs,
                                               rb.sv + (long long)L * v3, g_bs, rb.dh + (long long)L * v3, g_bs);
  note_launch();
}

// Stage C of the mixed form: FP32 factorisation, then `passes` solves of the interface equations
// (the first from a zero state), each against the double-float residual of the previous state.
// bWd / bVd: the double-float bigW / bigV of stage B (unfactored); bW / bV: their FP32 LU.
void stage_c_refined(cudaStream_t s, int Bc, int L, int N, const Cx<df64>* bWd, const Cx<df64>* bVd,
                     Cx<float>* bW, Cx<float>* bV, const int* pivW, const int* pivV, const cplx* X,
                     const PortVectors& pv, const SolveDesc& d, int first, const SolveOut& out, int32_t* st,
                     Cx<float>* Mk, int* pivM, Cx<float>* Ak, int* pivA, Cx<float>* Rk, Cx<float>* S1,
                     Cx<float>* S2, Cx<float>* S3, int* pivS, RefineBufs& rb, int passes) {
  TraceRange trace_("wb:stage_c.refined");
  using D = Cx<df64>;
  const int n = 2 * N, P = Bc * L;
  const long long n2 = (long long)n * n, v3 = 3LL * n, v6 = 6LL * n;
  const long long r_bs = (long long)(L + 1) * n2, g_bs = (long long)(L + 1) * v3;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  cascade_factor<float>(s, Bc, L, N, bW, bV, pivW, pivV, X, pv, st, Mk, pivM, Rk, S1, S2, S3, pivS, Ak, pivA);
  top_kernel<float><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, Rk, r_bs, pv.r22, S1, n2); note_launch();
  getrf<float>(s, Bc, n, S1, n, n2, pivS, n, st, 1);
  incident_kernel<df64><<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, N, d.pol + 2 * first, pv.nt, rb.Cin, v3);
  note_launch();
  const size_t gsz = sizeof(D) * (size_t)Bc * g_bs, csz = sizeof(D) * (size_t)P * v3;
  cudaMemsetAsync(rb.g, 0, gsz, s); cudaMemsetAsync(rb.h, 0, gsz, s);
  cudaMemsetAsync(rb.cp, 0, csz, s); cudaMemsetAsync(rb.cm, 0, csz, s);
  const unsigned nbp = nblk((long long)P * v3, 256), nbb = nblk((long long)Bc * v3, 256);
  for (int it = 0; it < passes; ++it) {
    // residual of the current double-float state
    res_u_kernel<df64><<<nbp, 256, 0, s>>>(P, n, rb.cp, rb.cm, X, rb.UW, rb.UV); note_launch();
    gemm<df64>(s, P, n, 6, n, one, bWd, 1, n, n2, rb.UW, 1, n, v6, zero, rb.YW, 1, n, v6);
    gemm<df64>(s, P, n, 6, n, one, bVd, 1, n, n2, rb.UV, 1, n, v6, zero, rb.YV, 1, n, v6);
    res_f_kernel<df64><<<nbp, 256, 0, s>>>(P, L, n, rb.YW, rb.YV, rb.g, rb.h, pv.wg, pv.vg, rb.f1, rb.f2, rb.f3, rb.f4);
    note_launch();
    res_tb_kernel<df64><<<nbb, 256, 0, s>>>(Bc, L, n, rb.g, rb.h, rb.Cin, pv.r21, pv.r22, pv.t11, rb.ft, rb.fb);
    note_launch();
    // FP32 correction, accumulated into the state
    cascade_sources(s, Bc, L, n, bW, bV, pivW, pivV, Mk, pivM, Ak, pivA, Rk, S1, pivS, X, pv, rb);
    const long long gc = (long long)Bc * g_bs, cc = (long long)P * v3;
    accumulate_kernel<float, df64><<<nblk(gc, 256), 256, 0, s>>>(gc, rb.dg, rb.g); note_launch();
    accumulate_kernel<float, df64><<<nblk(gc, 256), 256, 0, s>>>(gc, rb.dh, rb.h); note_launch();
    accumulate_kernel<float, df64><<<nblk(cc, 256), 256, 0, s>>>(cc, rb.dcp, rb.cp); note_launch();
    accumulate_kernel<float, df64><<<nblk(cc, 256), 256, 0, s>>>(cc, rb.dcm, rb.cm); note_launch();
  }
  // c_ref = r11 C + r12 h_0, c_trn = t21 g_L, then the efficiencies
  dscale3_kernel<df64><<<nbb, 256, 0, s>>>(Bc, n, pv.r11, rb.Cin, v3, pv.r12, rb.h, g_bs, rb.cref, v3); note_launch();
  dscale3_kernel<df64><<<nbb, 256, 0, s>>>(Bc, n, pv.t21, rb.g + (long long)L * v3, g_bs, nullptr, nullptr, 0, rb.ctrn, v3);
  note_launch();
  efficiency_kernel<df64><<<nblk((long long)Bc * N * 3, 256), 256, 0, s>>>(
      Bc, N, rb.cref, rb.ctrn, v3, pv, d.eps_top + first, d.eps_bot + first, d.pol + 2 * first,
      out.R + (long long)first * 3 * N, out.T + (long long)first * 3 * N,
      out.amps ? out.amps + (long long)first * 12 * N : nullptr, st);
  note_launch();
}

// ------------------------------------------------------------------------- orchestration
// Solves of the interface equations in the mixed form: the FP32 solve from a zero state and
// one refinement against the double-float residual.
constexpr int kRefinePasses = 2;

// Workspace of one chunk of `chunk` solves with L layers of N orders (n = 2N). All matrices are
// allocated at 16 bytes per complex entry (complex128 or complex df64); the FP32 cascade of the
// mixed form takes its own 8-byte copies.
size_t solve_chunk_bytes(int N, int L, int chunk, int precision) {
  const size_t n = 2 * (size_t)N, n2 = n * n, P = (size_t)chunk * L;
  size_t b = 0;
  auto A = [&](size_t x) { b += (x + 255) & ~(size_t)255; };
  for (int k = 0; k < 4; ++k) A(sizeof(double) * chunk * N);
  A(sizeof(cplx) * chunk * N); A(sizeof(cplx) * chunk * N);
  for (int k = 0; k < 8; ++k) A(sizeof(cplx) * chunk * n);
  A(sizeof(cplx) * chunk); A(sizeof(cplx) * chunk);
  A(sizeof(int) * P); A(sizeof(int) * P); A(sizeof(double) * P);
  A(16 * P * n2); A(16 * P * n2); A(16 * P * n2);                  // OM, Zb, Xv
  for (int k = 0; k < 5; ++k) A(16 * P * n);                        // wr, tau, w, q, X
  A(sizeof(int) * P * n); A(sizeof(int) * P * n); A(sizeof(int) * P * n);
  const bool fp32c = (precision == 1 || precision == 2 || precision == 4);   // FP32 cascade
  const size_t ec = fp32c ? 8 : 16;                                // stage C element size
  if (fp32c) { A(ec * P * n2); A(ec * P * n2); A(ec * P * n2); }   // FP32 bigW, bigV, Mk
  A(ec * (P + chunk) * n2);
  A(ec * chunk * n2); A(ec * chunk * n2); A(ec * chunk * n2);
  A(sizeof(int) * chunk * n);
  if (precision == 1 || precision == 4) {                          // per-layer A factors, refinement
    A(ec * P * n2); A(sizeof(int) * P * n);
    b += RefineBufs::bytes(chunk, L, (int)n);
    if (precision == 1) { A(16 * P * n); b += GroupBufs::bytes((int)P, (int)n); }
  } else {
    for (int k = 0; k < 6; ++k) A(ec * chunk * n * 3);
  }
  return b;
}

// precision: 0 plain FP64; 1 mixed (FP32 eigen-solve with Newton steps against the FP64
// operator, FP32 cascade refined against the double-float interface equations); 2 df64 stage B
// with the unrefined FP32 cascade; 3 df64 stage B and C; 4 df64 stage B with the refined FP32
// cascade
int solve_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, int first, int count, const SolveOut& out,
                int precision) {
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers;
  const long long n2 = (long long)n * n;
  const int Bc = count, P = Bc * L;
  int32_t* st = out.status + first;
  ar.reset();
  PortVectors pv;
  pv.kx = ar.get<double>((size_t)Bc * N); pv.ky = ar.get<double>((size_t)Bc * N);
  pv.c = ar.get<double>((size_t)Bc * N); pv.s = ar.get<double>((size_t)Bc * N);
  pv.kz_top = ar.get<cplx>((size_t)Bc * N); pv.kz_bot = ar.get<cplx>((size_t)Bc * N);
  pv.wg = ar.get<cplx>((size_t)Bc * n); pv.vg = ar.get<cplx>((size_t)Bc * n);
  pv.r11 = ar.get<cplx>((size_t)Bc * n); pv.r12 = ar.get<cplx>((size_t)Bc * n);
  pv.r21 = ar.get<cplx>((size_t)Bc * n); pv.r22 = ar.get<cplx>((size_t)Bc * n);
  pv.t11 = ar.get<cplx>((size_t)Bc * n); pv.t21 = ar.get<cplx>((size_t)Bc * n);
  pv.nt = ar.get<cplx>(Bc); pv.nb = ar.get<cplx>(Bc);
  int* pair_layer = ar.get<int>(P);
  int* pair_solve = ar.get<int>(P);
  double* pair_thick = ar.get<double>(P);
  char* OMr = ar.get<char>((size_t)16 * P * n2);
  char* Zbr = ar.get<char>((size_t)16 * P * n2);
  char* Xvr = ar.get<char>((size_t)16 * P * n2);
  char* wr = ar.get<char>((size_t)16 * P * n);
  char* taur = ar.get<char>((size_t)16 * P * n);
  cplx* w = ar.get<cplx>((size_t)P * n);
  cplx* q = ar.get<cplx>((size_t)P * n);
  cplx* X = ar.get<cplx>((size_t)P * n);
  int* pivW = ar.get<int>((size_t)P * n);
  int* pivV = ar.get<int>((size_t)P * n);
  int* pivM = ar.get<int>((size_t)P * n);
  if (!ar.ok()) return -1;
  ports_kernel<<<Bc, 128, 0, s>>>(Bc, d.hu, d.hv, d.wavelength + first, d.period + 2 * first, d.theta + first,
                                  d.phi + first, d.eps_top + first, d.eps_bot + first, nullptr, pv); note_launch();
  pairs_kernel<<<nblk(P, 128), 128, 0, s>>>(Bc, L, d.layer_index + (long long)first * L,
                                            d.thickness + (long long)first * L, pair_layer, pair_solve, pair_thick);
  note_launch();
  const double* wl = d.wavelength + first;
  if (precision == 0) {
    using R = double;
    Cx<R>* OM = (Cx<R>*)OMr; Cx<R>* Zb = (Cx<R>*)Zbr; Cx<R>* Xv = (Cx<R>*)Xvr;
    stage_b<R>(s, P, N, d.conv, pair_layer, pair_solve, pair_thick, wl, pv.kx, pv.ky, OM, Zb, Xv, (Cx<R>*)wr,
               (Cx<R>*)taur, w, q, X, pv.c, pv.s, st, L, true);
    getrf<R>(s, P, n, OM, n, n2, pivW, n, st, L);
    getrf<R>(s, P, n, Zb, n, n2, pivV, n, st, L);
    Cx<R>* Rk = ar.get<Cx<R>>((size_t)(P + Bc) * n2);
    Cx<R>* S1 = ar.get<Cx<R>>((size_t)Bc * n2); Cx<R>* S2 = ar.get<Cx<R>>((size_t)Bc * n2);
    Cx<R>* S3 = ar.get<Cx<R>>((size_t)Bc * n2);
    int* pivS = ar.get<int>((size_t)Bc * n);
    Cx<R>* v[6];
    for (int k = 0; k < 6; ++k) v[k] = ar.get<Cx<R>>((size_t)Bc * n * 3);
    if (!ar.ok()) return -1;
    stage_c<R>(s, ar, Bc, L, N, OM, Zb, pivW, pivV, X, pv, d, first, out, st, Xv, pivM, Rk, S1, S2, S3, pivS,
               v[0], v[1], v[2], v[3], v[4], v[5]);
    return 0;
  }
  if (precision == 1) {
    // FP32 eigen-solve refined by Newton steps, FP32 cascade refined against the interface equations
    using RC = float;
    Cx<RC>* bW = ar.get<Cx<RC>>((size_t)P * n2);
    Cx<RC>* bV = ar.get<Cx<RC>>((size_t)P * n2);
    Cx<RC>* Mk = ar.get<Cx<RC>>((size_t)P * n2);
    Cx<RC>* Rk = ar.get<Cx<RC>>((size_t)(P + Bc) * n2);
    Cx<RC>* S1 = ar.get<Cx<RC>>((size_t)Bc * n2); Cx<RC>* S2 = ar.get<Cx<RC>>((size_t)Bc * n2);
    Cx<RC>* S3 = ar.get<Cx<RC>>((size_t)Bc * n2);
    int* pivS = ar.get<int>((size_t)Bc * n);
    Cx<RC>* Ak = ar.get<Cx<RC>>((size_t)P * n2);
    int* pivA = ar.get<int>((size_t)P * n);
    RefineBufs rb;
    if (!rb.carve(ar, Bc, L, n)) return -1;
    cplx* lam = ar.get<cplx>((size_t)P * n);
    GroupBufs gb;
    if (!gb.carve(ar, P, n) || !ar.ok()) return -1;
    NewtonBufs nb{bW, bV, Mk, Rk, (Cx<float>*)wr, (Cx<float>*)taur, pivW, lam};
    stage_b_newton(s, P, N, d.conv, pair_layer, pair_solve, pair_thick, wl, pv.kx, pv.ky, (cplx*)OMr, (cplx*)Zbr,
                   (cplx*)Xvr, nb, gb, w, q, X, pv.c, pv.s, st, L, true);
    Cx<df64>* OM = (Cx<df64>*)OMr; Cx<df64>* Zb = (Cx<df64>*)Zbr;
    convert<df64, RC>(s, OM, bW, (long long)P * n2);
    convert<df64, RC>(s, Zb, bV, (long long)P * n2);
    getrf<RC>(s, P, n, bW, n, n2, pivW, n, st, L);
    getrf<RC>(s, P, n, bV, n, n2, pivV, n, st, L);
    stage_c_refined(s, Bc, L, N, OM, Zb, bW, bV, pivW, pivV, X, pv, d, first, out, st, Mk, pivM, Ak, pivA, Rk,
                    S1, S2, S3, pivS, rb, kRefinePasses);
    return 0;
  }
  // mixed: stage B in df64
  {
    using R = df64;
    Cx<R>* OM = (Cx<R>*)OMr; Cx<R>* Zb = (Cx<R>*)Zbr; Cx<R>* Xv = (Cx<R>*)Xvr;
    stage_b<R>(s, P, N, d.conv, pair_layer, pair_solve, pair_thick, wl, pv.kx, pv.ky, OM, Zb, Xv, (Cx<R>*)wr,
               (Cx<R>*)taur, w, q, X, pv.c, pv.s, st, L, true);
    if (precision == 3) {
      getrf<R>(s, P, n, OM, n, n2, pivW, n, st, L);
      getrf<R>(s, P, n, Zb, n, n2, pivV, n, st, L);
      Cx<R>* Rk = ar.get<Cx<R>>((size_t)(P + Bc) * n2);
      Cx<R>* S1 = ar.get<Cx<R>>((size_t)Bc * n2); Cx<R>* S2 = ar.get<Cx<R>>((size_t)Bc * n2);
      Cx<R>* S3 = ar.get<Cx<R>>((size_t)Bc * n2);
      int* pivS = ar.get<int>((size_t)Bc * n);
      Cx<R>* v[6];
      for (int k = 0; k < 6; ++k) v[k] = ar.get<Cx<R>>((size_t)Bc * n * 3);
      if (!ar.ok()) return -1;
      stage_c<R>(s, ar, Bc, L, N, OM, Zb, pivW, pivV, X, pv, d, first, out, st, Xv, pivM, Rk, S1, S2, S3, pivS,
                 v[0], v[1], v[2], v[3], v[4], v[5]);
      return 0;
    }
    using RC = float;
    Cx<RC>* bW = ar.get<Cx<RC>>((size_t)P * n2);
    Cx<RC>* bV = ar.get<Cx<RC>>((size_t)P * n2);
    Cx<RC>* Mk = ar.get<Cx<RC>>((size_t)P * n2);
    Cx<RC>* Rk = ar.get<Cx<RC>>((size_t)(P + Bc) * n2);
    Cx<RC>* S1 = ar.get<Cx<RC>>((size_t)Bc * n2); Cx<RC>* S2 = ar.get<Cx<RC>>((size_t)Bc * n2);
    Cx<RC>* S3 = ar.get<Cx<RC>>((size_t)Bc * n2);
    int* pivS = ar.get<int>((size_t)Bc * n);
    if (!ar.ok()) return -1;
    convert<R, RC>(s, OM, bW, (long long)P * n2);
    convert<R, RC>(s, Zb, bV, (long long)P * n2);
    getrf<RC>(s, P, n, bW, n, n2, pivW, n, st, L);
    getrf<RC>(s, P, n, bV, n, n2, pivV, n, st, L);
    if (precision == 4) {
      Cx<RC>* Ak = ar.get<Cx<RC>>((size_t)P * n2);
      int* pivA = ar.get<int>((size_t)P * n);
      RefineBufs rb;
      if (!rb.carve(ar, Bc, L, n) || !ar.ok()) return -1;
      stage_c_refined(s, Bc, L, N, OM, Zb, bW, bV, pivW, pivV, X, pv, d, first, out, st, Mk, pivM, Ak, pivA, Rk,
                      S1, S2, S3, pivS, rb, kRefinePasses);
      return 0;
    }
    Cx<RC>* v[6];
    for (int k = 0; k < 6; ++k) v[k] = ar.get<Cx<RC>>((size_t)Bc * n * 3);
    if (!ar.ok()) return -1;
    stage_c<RC>(s, ar, Bc, L, N, bW, bV, pivW, pivV, X, pv, d, first, out, st, Mk, pivM, Rk, S1, S2, S3, pivS,
                v[0], v[1], v[2], v[3], v[4], v[5]);
  }
  return 0;
}

// ----------------------------------------------------- stage C door (wb_smm_solve)
// The cascade and the efficiencies of B solves from given modes: W, V (P, n, n) and q (P, n) of
// every (solve, layer) pair as wb_layer_modes returns them (before the s/p rotation).
__global__ void xq_kernel(int P, int n, const cplx* __restrict__ q, const int* __restrict__ pair_solve,
                          const double* __restrict__ thick, const double* __restrict__ wavelength,
                          cplx* __restrict__ X) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)P * n) return;
  const long long p = idx / n;
  const double k0 = 2.0 * 3.141592653589793 / wavelength[pair_solve[p]];
  X[idx] = cexp_(cscale(q[idx], -k0 * thick[p]));
}

// Ports, pairs, the s/p-rotated modes and X for a chunk of solves from given modes (the preamble
// of wb_smm_solve, wb_etm_solve and wb_layer_amplitudes).
static void given_modes(cudaStream_t s, const SolveDesc& d, const cplx* Wm, const cplx* Vm, const cplx* qm, int first,
                        int Bc, const PortVectors& pv, int* pair_layer, int* pair_solve, double* pair_thick,
                        cplx* OM, cplx* Zb, cplx* X) {
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers, P = Bc * L;
  const long long n2 = (long long)n * n;
  ports_kernel<<<Bc, 128, 0, s>>>(Bc, d.hu, d.hv, d.wavelength + first, d.period + 2 * first, d.theta + first,
                                  d.phi + first, d.eps_top + first, d.eps_bot + first, nullptr, pv); note_launch();
  pairs_kernel<<<nblk(P, 128), 128, 0, s>>>(Bc, L, nullptr, d.thickness + (long long)first * L, pair_layer,
                                            pair_solve, pair_thick);
  note_launch();
  const long long off = (long long)first * L;
  cudaMemcpyAsync(OM, Wm + off * n2, sizeof(cplx) * P * n2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(Zb, Vm + off * n2, sizeof(cplx) * P * n2, cudaMemcpyDeviceToDevice, s);
  xq_kernel<<<nblk((long long)P * n, 256), 256, 0, s>>>(P, n, qm + off * n, pair_solve, pair_thick,
                                                        d.wavelength + first, X);
  note_launch();
  sp_rotate_kernel<double><<<nblk((long long)P * N * n, 256), 256, 0, s>>>(P, N, pair_solve, pv.c, pv.s,
                                                                          (Cx<double>*)OM, (Cx<double>*)Zb, n2);
  note_launch();
}

// The port vectors of solves first .. first + Bc - 1 (used by the reverse passes, wb_vjp.cu).
void compute_ports(cudaStream_t s, const SolveDesc& d, int first, int Bc, const PortVectors& pv) {
  ports_kernel<<<Bc, 128, 0, s>>>(Bc, d.hu, d.hv, d.wavelength + first, d.period + 2 * first, d.theta + first,
                                  d.phi + first, d.eps_top + first, d.eps_bot + first, nullptr, pv); note_launch();
}

size_t smm_chunk_bytes(int N, int L, int chunk, int precision) {
  return solve_chunk_bytes(N, L, chunk, precision == 0 ? 0 : 4);
}

// precision: 0 FP64 cascade; otherwise the FP32 cascade refined against the modes (double-float)
int smm_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* Wm, const cplx* Vm, const cplx* qm,
              int first, int count, const SolveOut& out, int precision) {
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers;
  const long long n2 = (long long)n * n;
  const int Bc = count, P = Bc * L;
  int32_t* st = out.status + first;
  ar.reset();
  PortVectors pv;
  pv.kx = ar.get<double>((size_t)Bc * N); pv.ky = ar.get<double>((size_t)Bc * N);
  pv.c = ar.get<double>((size_t)Bc * N); pv.s = ar.get<double>((size_t)Bc * N);
  pv.kz_top = ar.get<cplx>((size_t)Bc * N); pv.kz_bot = ar.get<cplx>((size_t)Bc * N);
  pv.wg = ar.get<cplx>((size_t)Bc * n); pv.vg = ar.get<cplx>((size_t)Bc * n);
  pv.r11 = ar.get<cplx>((size_t)Bc * n); pv.r12 = ar.get<cplx>((size_t)Bc * n);
  pv.r21 = ar.get<cplx>((size_t)Bc * n); pv.r22 = ar.get<cplx>((size_t)Bc * n);
  pv.t11 = ar.get<cplx>((size_t)Bc * n); pv.t21 = ar.get<cplx>((size_t)Bc * n);
  pv.nt = ar.get<cplx>(Bc); pv.nb = ar.get<cplx>(Bc);
  int* pair_layer = ar.get<int>(P);
  int* pair_solve = ar.get<int>(P);
  double* pair_thick = ar.get<double>(P);
  cplx* OM = ar.get<cplx>((size_t)P * n2);
  cplx* Zb = ar.get<cplx>((size_t)P * n2);
  cplx* Xv = ar.get<cplx>((size_t)P * n2);
  cplx* X = ar.get<cplx>((size_t)P * n);
  int* pivW = ar.get<int>((size_t)P * n);
  int* pivV = ar.get<int>((size_t)P * n);
  int* pivM = ar.get<int>((size_t)P * n);
  if (!ar.ok()) return -1;
  given_modes(s, d, Wm, Vm, qm, first, Bc, pv, pair_layer, pair_solve, pair_thick, OM, Zb, X);
  if (precision == 0) {
    using R = double;
    getrf<R>(s, P, n, (Cx<R>*)OM, n, n2, pivW, n, st, L);
    getrf<R>(s, P, n, (Cx<R>*)Zb, n, n2, pivV, n, st, L);
    Cx<R>* Rk = ar.get<Cx<R>>((size_t)(P + Bc) * n2);
    Cx<R>* S1 = ar.get<Cx<R>>((size_t)Bc * n2); Cx<R>* S2 = ar.get<Cx<R>>((size_t)Bc * n2);
    Cx<R>* S3 = ar.get<Cx<R>>((size_t)Bc * n2);
    int* pivS = ar.get<int>((size_t)Bc * n);
    Cx<R>* v[6];
    for (int k = 0; k < 6; ++k) v[k] = ar.get<Cx<R>>((size_t)Bc * n * 3);
    if (!ar.ok()) return -1;
    stage_c<R>(s, ar, Bc, L, N, (Cx<R>*)OM, (Cx<R>*)Zb, pivW, pivV, X, pv, d, first, out, st, (Cx<R>*)Xv, pivM, Rk,
               S1, S2, S3, pivS, v[0], v[1], v[2], v[3], v[4], v[5]);
    return 0;
  }
  using RC = float;
  const long long tot = (long long)P * n2;
  to_df64_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, OM); note_launch();
  to_df64_kernel<<<nblk(tot, 256), 256, 0, s>>>(tot, Zb); note_launch();
  Cx<RC>* bW = ar.get<Cx<RC>>((size_t)P * n2);
  Cx<RC>* bV = ar.get<Cx<RC>>((size_t)P * n2);
  Cx<RC>* Mk = ar.get<Cx<RC>>((size_t)P * n2);
  Cx<RC>* Rk = ar.get<Cx<RC>>((size_t)(P + Bc) * n2);
  Cx<RC>* S1 = ar.get<Cx<RC>>((size_t)Bc * n2); Cx<RC>* S2 = ar.get<Cx<RC>>((size_t)Bc * n2);
  Cx<RC>* S3 = ar.get<Cx<RC>>((size_t)Bc * n2);
  int* pivS = ar.get<int>((size_t)Bc * n);
  Cx<RC>* Ak = ar.get<Cx<RC>>((size_t)P * n2);
  int* pivA = ar.get<int>((size_t)P * n);
  RefineBufs rb;
  if (!rb.carve(ar, Bc, L, n) || !ar.ok()) return -1;
  Cx<df64>* OMd = (Cx<df64>*)OM; Cx<df64>* Zbd = (Cx<df64>*)Zb;
  convert<df64, RC>(s, OMd, bW, tot);
  convert<df64, RC>(s, Zbd, bV, tot);
  getrf<RC>(s, P, n, bW, n, n2, pivW, n, st, L);
  getrf<RC>(s, P, n, bV, n, n2, pivV, n, st, L);
  stage_c_refined(s, Bc, L, N, OMd, Zbd, bW, bV, pivW, pivV, X, pv, d, first, out, st, Mk, pivM, Ak, pivA, Rk,
                  S1, S2, S3, pivS, rb, kRefinePasses);
  return 0;
}

// ------------------------------------------ scattering-matrix export (wb_scattering_matrix)
// The four blocks of the stack's S at the half-space ports, as the reference publishes them
// (Outputs(scattering=True), scattering.py:482-605). The cascade lit in every port column from
// the superstrate gives S11 (the reflected columns) and S21 (the transmitted ones); the mirrored
// stack -- layers in reverse order, half-spaces swapped, the same order wavevectors -- gives S22
// and S12 the same way. Under z -> -z tangential E keeps its sign and tangential H changes it,
// which is the relation between a layer's down- and up-going (W, V) columns, so the rotated,
// factored modes of each layer serve both orientations unchanged. The blocks leave in the
// centre frame, C S C with C = diag((-1)^(m+n)) on both polarization halves.

// out = diag(d) in (+ diag(e) in2 when e): k columns of length n per batch
__global__ void dscale_cols_kernel(int B, int n, int k, const cplx* __restrict__ d, const cplx* __restrict__ in,
                                   long long in_bs, const cplx* __restrict__ e, const cplx* __restrict__ in2,
                                   long long in2_bs, cplx* __restrict__ out, long long out_bs) {
  const long long nk = (long long)n * k;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * nk) return;
  const long long b = idx / nk, rem = idx % nk;
  const int i = (int)(rem % n);
  cplx v = cmul(d[b * n + i], in[b * in_bs + rem]);
  if (e) v = cadd(v, cmul(e[b * n + i], in2[b * in2_bs + rem]));
  out[b * out_bs + rem] = v;
}

// rhs1 = wg o (g + h), rhs2 = vg o (g - h)
__global__ void gh_cols_kernel(int B, int n, int k, const cplx* __restrict__ g, const cplx* __restrict__ h,
                               const cplx* __restrict__ wg, const cplx* __restrict__ vg, cplx* __restrict__ r1,
                               cplx* __restrict__ r2, long long bs) {
  const long long nk = (long long)n * k;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * nk) return;
  const long long b = idx / nk, rem = idx % nk;
  const int i = (int)(rem % n);
  const cplx gg = g[b * bs + rem], hh = h[b * bs + rem];
  r1[b * bs + rem] = cmul(wg[b * n + i], cadd(gg, hh));
  r2[b * bs + rem] = cmul(vg[b * n + i], csub(gg, hh));
}

// g = X o (r1 + r2)  (2 c+ at the bottom of the layer)
__global__ void ct_cols_kernel(int B, int n, int k, const cplx* __restrict__ r1, const cplx* __restrict__ r2,
                               const cplx* __restrict__ X, long long x_ps, cplx* __restrict__ g, long long bs) {
  const long long nk = (long long)n * k;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * nk) return;
  const long long b = idx / nk, rem = idx % nk;
  const int i = (int)(rem % n);
  g[b * bs + rem] = cmul(X[b * x_ps + i], cadd(r1[b * bs + rem], r2[b * bs + rem]));
}

// out[b] = C in[b] C for column-major n x n blocks (n = 2N), C_i = (-1)^(m+n) of order i % N
__global__ void centre_frame_kernel(int B, int hu, int hv, const cplx* __restrict__ in, long long in_bs,
                                    cplx* __restrict__ out) {
  const int nu = 2 * hu + 1, N = nu * (2 * hv + 1), n = 2 * N;
  const long long n2 = (long long)n * n;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n2) return;
  const long long b = idx / n2, rem = idx % n2;
  const int i = (int)(rem % n) % N, j = (int)(rem / n) % N;
  // (u - hu) + (v - hv) has the parity of u + v + hu + hv
  const int par = (i % nu + i / nu + j % nu + j / nu) & 1;
  const cplx v = in[b * in_bs + rem];
  out[b * n2 + rem] = par ? cneg(v) : v;
}

// Top-down pass of the cascade for the k columns of Cin (Bc, n, k), after cascade_factor: the
// reflected columns cref = r11 C + r12 h_0 and the transmitted ctrn = t21 g_L, in the
// half-space port variables (stage_c's three-column pass for any k, FP64).
static void cascade_columns(cudaStream_t s, int Bc, int L, int n, const cplx* bW, const cplx* bV, const int* pivW,
                            const int* pivV, const cplx* X, const PortVectors& pv, int32_t* st, const cplx* Mk,
                            const int* pivM, const cplx* Rk, cplx* G0, int* pivS, const cplx* Cin, int k, cplx* g,
                            cplx* h, cplx* r1, cplx* r2, cplx* cref, cplx* ctrn) {
  typedef Cx<double> C;
  const long long n2 = (long long)n * n, lay_bs = (long long)L * n2, lay_ps = (long long)L * n;
  const long long r_bs = (long long)(L + 1) * n2, vk = (long long)n * k;
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  const unsigned gk = nblk((long long)Bc * vk, 256);
  top_kernel<double><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, (const C*)Rk, r_bs, pv.r22, (C*)G0, n2);
  note_launch();
  getrf<double>(s, Bc, n, (C*)G0, n, n2, pivS, n, st, 1);
  dscale_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, pv.r21, Cin, vk, nullptr, nullptr, 0, g, vk); note_launch();
  getrs<double>(s, Bc, n, (const C*)G0, n, n2, pivS, n, (C*)g, k, n, vk, 0);                      // g_0
  gemm<double>(s, Bc, n, k, n, one, (const C*)Rk, 1, n, r_bs, (const C*)g, 1, n, vk, zero, (C*)h, 1, n, vk);
  dscale_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, pv.r11, Cin, vk, pv.r12, h, vk, cref, vk); note_launch();
  for (int l = 0; l < L; ++l) {
    if (l > 0)
      gemm<double>(s, Bc, n, k, n, one, (const C*)(Rk + l * n2), 1, n, r_bs, (const C*)g, 1, n, vk, zero, (C*)h, 1,
                   n, vk);                                                                        // h_l = R_l g_l
    gh_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, g, h, pv.wg, pv.vg, r1, r2, vk); note_launch();
    getrs<double>(s, Bc, n, (const C*)(bW + l * n2), n, lay_bs, pivW + (long long)l * n, lay_ps, (C*)r1, k, n, vk, 0);
    getrs<double>(s, Bc, n, (const C*)(bV + l * n2), n, lay_bs, pivV + (long long)l * n, lay_ps, (C*)r2, k, n, vk, 0);
    ct_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, r1, r2, X + (long long)l * n, lay_ps, g, vk); note_launch();
    getrs<double>(s, Bc, n, (const C*)(Mk + l * n2), n, lay_bs, pivM + (long long)l * n, lay_ps, (C*)g, k, n, vk,
                  0);                                                                             // g_{l+1}
  }
  dscale_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, pv.t21, g, vk, nullptr, nullptr, 0, ctrn, vk); note_launch();
}

// dst = src with the layers of every solve in reverse order (blocks of `per` elements per layer)
template <class T>
__global__ void mirror_layers_kernel(long long total, int L, long long per, const T* __restrict__ src,
                                     T* __restrict__ dst) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const long long lp = (long long)L * per;
  const long long b = idx / lp, rem = idx % lp;
  const int l = (int)(rem / per);
  dst[idx] = src[b * lp + (long long)(L - 1 - l) * per + rem % per];
}

template <class T>
static void mirror_layers(cudaStream_t s, int Bc, int L, long long per, const T* src, T* dst) {
  const long long total = (long long)Bc * L * per;
  mirror_layers_kernel<T><<<nblk(total, 256), 256, 0, s>>>(total, L, per, src, dst); note_launch();
}

namespace {
struct ByteCount {
  size_t b = 0;
  template <class T> T* get(size_t count) { b += (count * sizeof(T) + 255) & ~(size_t)255; return nullptr; }
  bool ok() const { return true; }
};
}  // namespace

// Scratch of one export chunk; the same carve sizes it (ByteCount) and lays it out (Arena).
struct ScatterBufs {
  PortVectors pv[2];                        // [0] lit from the superstrate, [1] the mirrored stack
  int *pair_layer, *pair_solve;
  double* pair_thick;
  cplx *OM[2], *Zb[2], *X[2];               // factored bigW / bigV and X per (solve, layer), both orders
  int *pivW[2], *pivV[2];
  cplx *Mk, *Rk, *S1, *S2, *S3, *Cin, *g, *h, *r1, *r2, *cref, *ctrn;
  int *pivM, *pivS;
  template <class A> bool carve(A& ar, int Bc, int L, int N) {
    const size_t n = 2 * (size_t)N, n2 = n * n, P = (size_t)Bc * L;
    for (PortVectors& v : pv) {
      v.kx = ar.template get<double>((size_t)Bc * N); v.ky = ar.template get<double>((size_t)Bc * N);
      v.c = ar.template get<double>((size_t)Bc * N); v.s = ar.template get<double>((size_t)Bc * N);
      v.kz_top = ar.template get<cplx>((size_t)Bc * N); v.kz_bot = ar.template get<cplx>((size_t)Bc * N);
      v.wg = ar.template get<cplx>(Bc * n); v.vg = ar.template get<cplx>(Bc * n);
      v.r11 = ar.template get<cplx>(Bc * n); v.r12 = ar.template get<cplx>(Bc * n);
      v.r21 = ar.template get<cplx>(Bc * n); v.r22 = ar.template get<cplx>(Bc * n);
      v.t11 = ar.template get<cplx>(Bc * n); v.t21 = ar.template get<cplx>(Bc * n);
      v.nt = ar.template get<cplx>(Bc); v.nb = ar.template get<cplx>(Bc);
    }
    pair_layer = ar.template get<int>(P); pair_solve = ar.template get<int>(P);
    pair_thick = ar.template get<double>(P);
    for (int o = 0; o < 2; ++o) {
      OM[o] = ar.template get<cplx>(P * n2); Zb[o] = ar.template get<cplx>(P * n2);
      X[o] = ar.template get<cplx>(P * n);
      pivW[o] = ar.template get<int>(P * n); pivV[o] = ar.template get<int>(P * n);
    }
    Mk = ar.template get<cplx>(P * n2); pivM = ar.template get<int>(P * n);
    Rk = ar.template get<cplx>((P + Bc) * n2);
    S1 = ar.template get<cplx>(Bc * n2); S2 = ar.template get<cplx>(Bc * n2); S3 = ar.template get<cplx>(Bc * n2);
    pivS = ar.template get<int>(Bc * n);
    Cin = ar.template get<cplx>(Bc * n2); g = ar.template get<cplx>(Bc * n2); h = ar.template get<cplx>(Bc * n2);
    r1 = ar.template get<cplx>(Bc * n2); r2 = ar.template get<cplx>(Bc * n2);
    cref = ar.template get<cplx>(Bc * n2); ctrn = ar.template get<cplx>(Bc * n2);
    return ar.ok();
  }
};

size_t scattering_chunk_bytes(int N, int L, int chunk) {
  ByteCount c;
  ScatterBufs sb;
  sb.carve(c, chunk, L, N);
  return c.b;
}

int scattering_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* Wm, const cplx* Vm, const cplx* qm,
                     int first, int count, cplx* S11, cplx* S12, cplx* S21, cplx* S22, int32_t* status) {
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers;
  const long long n2 = (long long)n * n;
  const int Bc = count, P = Bc * L;
  int32_t* st = status + first;
  ar.reset();
  ScatterBufs sb;
  if (!sb.carve(ar, Bc, L, N)) return -1;
  const cplx *et = d.eps_top + first, *eb = d.eps_bot + first;
  ports_kernel<<<Bc, 128, 0, s>>>(Bc, d.hu, d.hv, d.wavelength + first, d.period + 2 * first, d.theta + first,
                                  d.phi + first, et, eb, nullptr, sb.pv[0]); note_launch();
  ports_kernel<<<Bc, 128, 0, s>>>(Bc, d.hu, d.hv, d.wavelength + first, d.period + 2 * first, d.theta + first,
                                  d.phi + first, eb, et, et, sb.pv[1]); note_launch();
  pairs_kernel<<<nblk(P, 128), 128, 0, s>>>(Bc, L, nullptr, d.thickness + (long long)first * L, sb.pair_layer,
                                            sb.pair_solve, sb.pair_thick);
  note_launch();
  const long long off = (long long)first * L;
  cudaMemcpyAsync(sb.OM[0], Wm + off * n2, sizeof(cplx) * P * n2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(sb.Zb[0], Vm + off * n2, sizeof(cplx) * P * n2, cudaMemcpyDeviceToDevice, s);
  xq_kernel<<<nblk((long long)P * n, 256), 256, 0, s>>>(P, n, qm + off * n, sb.pair_solve, sb.pair_thick,
                                                        d.wavelength + first, sb.X[0]);
  note_launch();
  sp_rotate_kernel<double><<<nblk((long long)P * N * n, 256), 256, 0, s>>>(
      P, N, sb.pair_solve, sb.pv[0].c, sb.pv[0].s, (Cx<double>*)sb.OM[0], (Cx<double>*)sb.Zb[0], n2);
  note_launch();
  getrf<double>(s, P, n, (Cx<double>*)sb.OM[0], n, n2, sb.pivW[0], n, st, L);
  getrf<double>(s, P, n, (Cx<double>*)sb.Zb[0], n, n2, sb.pivV[0], n, st, L);
  // the mirrored stack's layer l is layer L-1-l: the same factors, X and pivots, reordered
  mirror_layers(s, Bc, L, n2, sb.OM[0], sb.OM[1]);
  mirror_layers(s, Bc, L, n2, sb.Zb[0], sb.Zb[1]);
  mirror_layers(s, Bc, L, (long long)n, sb.X[0], sb.X[1]);
  mirror_layers(s, Bc, L, (long long)n, sb.pivW[0], sb.pivW[1]);
  mirror_layers(s, Bc, L, (long long)n, sb.pivV[0], sb.pivV[1]);
  typedef Cx<double> C;
  for (int o = 0; o < 2; ++o) {
    cascade_factor<double>(s, Bc, L, N, (C*)sb.OM[o], (C*)sb.Zb[o], sb.pivW[o], sb.pivV[o], sb.X[o], sb.pv[o], st,
                           (C*)sb.Mk, sb.pivM, (C*)sb.Rk, (C*)sb.S1, (C*)sb.S2, (C*)sb.S3, sb.pivS, nullptr, nullptr);
    zset_identity(s, Bc, n, sb.Cin, n, n2);
    cascade_columns(s, Bc, L, n, sb.OM[o], sb.Zb[o], sb.pivW[o], sb.pivV[o], sb.X[o], sb.pv[o], st, sb.Mk, sb.pivM,
                    sb.Rk, sb.S1, sb.pivS, sb.Cin, n, sb.g, sb.h, sb.r1, sb.r2, sb.cref, sb.ctrn);
    const unsigned gb = nblk((long long)Bc * n2, 256);
    centre_frame_kernel<<<gb, 256, 0, s>>>(Bc, d.hu, d.hv, sb.cref, n2, (o ? S22 : S11) + (long long)first * n2);
    note_launch();
    centre_frame_kernel<<<gb, 256, 0, s>>>(Bc, d.hu, d.hv, sb.ctrn, n2, (o ? S12 : S21) + (long long)first * n2);
    note_launch();
  }
  return 0;
}

// ---------------------------------------- per-layer field amplitudes (wb_layer_amplitudes)
// The cascade's own state inside the stack, for the field reconstruction (scattering.py:236-350,
// _below_reflections and _field_state): for the k columns of Cin, every layer's mode amplitudes
// at its top face, plus = (b1 + b2)/2 (down-going) and minus_top = (b1 - b2)/2 (up-going), with
// b1 = bW^-1 wg (g + h), b2 = bV^-1 vg (g - h) from the gap above it (g_l, h_l = R_l g_l), and the
// up-going amplitudes read at its bottom face from the gap below, minus_bottom = (b1' - b2')/2 with
// g_{l+1}, h_{l+1} = R_{l+1} g_{l+1} and the same layer's bW, bV. The reflected and transmitted
// columns come out as in cascade_columns. FP64 throughout.

// plus = (r1 + r2)/2 and minus = (r1 - r2)/2 (minus only when plus is null): k columns per batch
__global__ void halves_kernel(int B, int n, int k, const cplx* __restrict__ r1, const cplx* __restrict__ r2,
                              long long bs, cplx* __restrict__ plus, cplx* __restrict__ minus, long long out_bs) {
  const long long nk = (long long)n * k;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * nk) return;
  const long long b = idx / nk, rem = idx % nk;
  const cplx a = r1[b * bs + rem], c = r2[b * bs + rem];
  if (plus) plus[b * out_bs + rem] = cscale(cadd(a, c), 0.5);
  minus[b * out_bs + rem] = cscale(csub(a, c), 0.5);
}

struct AmplitudeBufs {
  PortVectors pv;
  int *pair_layer, *pair_solve;
  double* pair_thick;
  cplx *OM, *Zb, *X, *Mk, *Rk, *S1, *S2, *S3, *g, *h, *r1, *r2;
  int *pivW, *pivV, *pivM, *pivS;
  template <class A> bool carve(A& ar, int Bc, int L, int N, int k) {
    const size_t n = 2 * (size_t)N, n2 = n * n, P = (size_t)Bc * L, vk = n * (size_t)k;
    PortVectors& v = pv;
    v.kx = ar.template get<double>((size_t)Bc * N); v.ky = ar.template get<double>((size_t)Bc * N);
    v.c = ar.template get<double>((size_t)Bc * N); v.s = ar.template get<double>((size_t)Bc * N);
    v.kz_top = ar.template get<cplx>((size_t)Bc * N); v.kz_bot = ar.template get<cplx>((size_t)Bc * N);
    v.wg = ar.template get<cplx>(Bc * n); v.vg = ar.template get<cplx>(Bc * n);
    v.r11 = ar.template get<cplx>(Bc * n); v.r12 = ar.template get<cplx>(Bc * n);
    v.r21 = ar.template get<cplx>(Bc * n); v.r22 = ar.template get<cplx>(Bc * n);
    v.t11 = ar.template get<cplx>(Bc * n); v.t21 = ar.template get<cplx>(Bc * n);
    v.nt = ar.template get<cplx>(Bc); v.nb = ar.template get<cplx>(Bc);
    pair_layer = ar.template get<int>(P); pair_solve = ar.template get<int>(P);
    pair_thick = ar.template get<double>(P);
    OM = ar.template get<cplx>(P * n2); Zb = ar.template get<cplx>(P * n2); X = ar.template get<cplx>(P * n);
    pivW = ar.template get<int>(P * n); pivV = ar.template get<int>(P * n);
    Mk = ar.template get<cplx>(P * n2); pivM = ar.template get<int>(P * n);
    Rk = ar.template get<cplx>((P + Bc) * n2);
    S1 = ar.template get<cplx>(Bc * n2); S2 = ar.template get<cplx>(Bc * n2); S3 = ar.template get<cplx>(Bc * n2);
    pivS = ar.template get<int>(Bc * n);
    g = ar.template get<cplx>(Bc * vk); h = ar.template get<cplx>(Bc * vk);
    r1 = ar.template get<cplx>(Bc * vk); r2 = ar.template get<cplx>(Bc * vk);
    return ar.ok();
  }
};

size_t amplitudes_chunk_bytes(int N, int L, int chunk, int k) {
  ByteCount c;
  AmplitudeBufs ab;
  ab.carve(c, chunk, L, N, k);
  return c.b;
}

int amplitudes_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* Wm, const cplx* Vm, const cplx* qm,
                     const cplx* Cin, int k, int first, int count, cplx* plus, cplx* minus_top, cplx* minus_bottom,
                     cplx* cref, cplx* ctrn, int32_t* status) {
  typedef Cx<double> C;
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers;
  const long long n2 = (long long)n * n, vk = (long long)n * k;
  const long long lay_bs = (long long)L * n2, lay_ps = (long long)L * n, r_bs = (long long)(L + 1) * n2;
  const int Bc = count, P = Bc * L;
  int32_t* st = status + first;
  ar.reset();
  AmplitudeBufs a;
  if (!a.carve(ar, Bc, L, N, k)) return -1;
  given_modes(s, d, Wm, Vm, qm, first, Bc, a.pv, a.pair_layer, a.pair_solve, a.pair_thick, a.OM, a.Zb, a.X);
  getrf<double>(s, P, n, (C*)a.OM, n, n2, a.pivW, n, st, L);
  getrf<double>(s, P, n, (C*)a.Zb, n, n2, a.pivV, n, st, L);
  cascade_factor<double>(s, Bc, L, N, (C*)a.OM, (C*)a.Zb, a.pivW, a.pivV, a.X, a.pv, st, (C*)a.Mk, a.pivM,
                         (C*)a.Rk, (C*)a.S1, (C*)a.S2, (C*)a.S3, a.pivS, nullptr, nullptr);
  const double2 one = make_double2(1, 0), zero = make_double2(0, 0);
  const unsigned gk = nblk((long long)Bc * vk, 256);
  const cplx* Cb = Cin + (long long)first * vk;
  // the reflected columns and g_0, h_0 (cascade_columns' top)
  top_kernel<double><<<nblk((long long)Bc * n2, 256), 256, 0, s>>>(Bc, n, (const C*)a.Rk, r_bs, a.pv.r22, (C*)a.S1,
                                                                   n2);
  note_launch();
  getrf<double>(s, Bc, n, (C*)a.S1, n, n2, a.pivS, n, st, 1);
  dscale_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.pv.r21, Cb, vk, nullptr, nullptr, 0, a.g, vk); note_launch();
  getrs<double>(s, Bc, n, (const C*)a.S1, n, n2, a.pivS, n, (C*)a.g, k, n, vk, 0);
  gemm<double>(s, Bc, n, k, n, one, (const C*)a.Rk, 1, n, r_bs, (const C*)a.g, 1, n, vk, zero, (C*)a.h, 1, n, vk);
  dscale_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.pv.r11, Cb, vk, a.pv.r12, a.h, vk, cref + (long long)first * vk,
                                        vk);
  note_launch();
  const long long o_bs = (long long)L * vk;                 // outputs (B, L, n, k)
  for (int l = 0; l < L; ++l) {
    const C* bWl = (const C*)(a.OM + l * n2);
    const C* bVl = (const C*)(a.Zb + l * n2);
    const long long o = (long long)first * o_bs + (long long)l * vk;
    gh_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.g, a.h, a.pv.wg, a.pv.vg, a.r1, a.r2, vk); note_launch();
    getrs<double>(s, Bc, n, bWl, n, lay_bs, a.pivW + (long long)l * n, lay_ps, (C*)a.r1, k, n, vk, 0);   // b1
    getrs<double>(s, Bc, n, bVl, n, lay_bs, a.pivV + (long long)l * n, lay_ps, (C*)a.r2, k, n, vk, 0);   // b2
    halves_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.r1, a.r2, vk, plus + o, minus_top + o, o_bs); note_launch();
    ct_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.r1, a.r2, a.X + (long long)l * n, lay_ps, a.g, vk); note_launch();
    getrs<double>(s, Bc, n, (const C*)(a.Mk + l * n2), n, lay_bs, a.pivM + (long long)l * n, lay_ps, (C*)a.g, k, n,
                  vk, 0);                                                                         // g_{l+1}
    gemm<double>(s, Bc, n, k, n, one, (const C*)(a.Rk + (l + 1) * n2), 1, n, r_bs, (const C*)a.g, 1, n, vk, zero,
                 (C*)a.h, 1, n, vk);                                                              // h_{l+1}
    gh_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.g, a.h, a.pv.wg, a.pv.vg, a.r1, a.r2, vk); note_launch();
    getrs<double>(s, Bc, n, bWl, n, lay_bs, a.pivW + (long long)l * n, lay_ps, (C*)a.r1, k, n, vk, 0);
    getrs<double>(s, Bc, n, bVl, n, lay_bs, a.pivV + (long long)l * n, lay_ps, (C*)a.r2, k, n, vk, 0);
    halves_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.r1, a.r2, vk, nullptr, minus_bottom + o, o_bs); note_launch();
  }
  dscale_cols_kernel<<<gk, 256, 0, s>>>(Bc, n, k, a.pv.t21, a.g, vk, nullptr, nullptr, 0,
                                        ctrn + (long long)first * vk, vk);
  note_launch();
  return 0;
}

// ------------------------------------------------- ETM connecting algorithm (wb_etm_solve)
// The enhanced transmittance matrix recursion (solve_2d.py:2619-2843, solve_1d.py:1389-1520) on
// given modes, bottom-up from the substrate's field matrices F = diag(1, -i kz_bot/eps_bot),
// G = diag(-i kz_bot, 1):
//   a = (bW^-1 F + bV^-1 G)/2,  b = (bW^-1 F - bV^-1 G)/2,  Y = X b a^-1 X,
//   F <- bW (I + Y),  G <- bV (I - Y),  T <- T a^-1 X,
// then the final matching at the superstrate, [[D1, -F], [D2, -G]] x = c with D1 = diag(1, i kz_top/
// eps_top), D2 = diag(i kz_top, 1), for the three incidence columns; the reflected amplitudes are
// x[:n] (p part with the port sign the efficiency kernel reads) and the transmitted T x[n:].
// T is kept transposed (Tt = X a^-T Tt) so that every solve is a transposed LU solve.

// F = diag(1 (N), -i kz_bot/eps_bot (N)), G = diag(-i kz_bot (N), 1 (N)), Tt = I
__global__ void etm_init_kernel(int B, int N, const cplx* __restrict__ kz_bot, const cplx* __restrict__ eps_bot,
                                cplx* __restrict__ F, cplx* __restrict__ G, cplx* __restrict__ Tt) {
  const int n = 2 * N;
  const long long n2 = (long long)n * n;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n2) return;
  const long long b = idx / n2, rem = idx % n2;
  const int i = (int)(rem % n), j = (int)(rem / n);
  cplx f = cmk(0.0, 0.0), g = cmk(0.0, 0.0), t = cmk(0.0, 0.0);
  if (i == j) {
    const cplx mik = (i < N) ? cmul(cmk(0.0, -1.0), kz_bot[b * N + i]) : cmul(cmk(0.0, -1.0), kz_bot[b * N + i - N]);
    f = (i < N) ? cmk(1.0, 0.0) : cdiv(mik, eps_bot[b]);
    g = (i < N) ? mik : cmk(1.0, 0.0);
    t = cmk(1.0, 0.0);
  }
  F[idx] = f; G[idx] = g; Tt[idx] = t;
}

// A = (S1 + S2)/2 and Bt = ((S1 - S2)/2)^T
__global__ void etm_ab_kernel(int B, int n, const cplx* __restrict__ S1, const cplx* __restrict__ S2,
                              cplx* __restrict__ A, cplx* __restrict__ Bt) {
  const long long n2 = (long long)n * n;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n2) return;
  const long long b = idx / n2, rem = idx % n2;
  const int i = (int)(rem % n), j = (int)(rem / n);
  const cplx s1 = S1[idx], s2 = S2[idx];
  A[idx] = cscale(cadd(s1, s2), 0.5);
  Bt[b * n2 + j + (long long)i * n] = cscale(csub(s1, s2), 0.5);
}

// Y(i, j) = X_i Zt(j, i) X_j (Zt = (b a^-1)^T) into Y, and Tt(i, j) *= X_i
__global__ void etm_y_kernel(int B, int n, const cplx* __restrict__ Zt, const cplx* __restrict__ X, long long x_bs,
                             cplx* __restrict__ Y, cplx* __restrict__ Tt) {
  const long long n2 = (long long)n * n;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n2) return;
  const long long b = idx / n2, rem = idx % n2;
  const int i = (int)(rem % n), j = (int)(rem / n);
  const cplx xi = X[b * x_bs + i];
  Y[idx] = cmul(cmul(xi, Zt[b * n2 + j + (long long)i * n]), X[b * x_bs + j]);
  Tt[idx] = cmul(xi, Tt[idx]);
}

// the final matching matrix [[D1, -F], [D2, -G]] (2n x 2n, column-major) and its three columns
__global__ void etm_final_kernel(int B, int N, const cplx* __restrict__ F, const cplx* __restrict__ G,
                                 const cplx* __restrict__ kz_top, const cplx* __restrict__ eps_top,
                                 const cplx* __restrict__ nt, const cplx* __restrict__ pol, cplx* __restrict__ A,
                                 cplx* __restrict__ cols) {
  const int n = 2 * N, m = 2 * n;
  const long long n2 = (long long)n * n, m2 = (long long)m * m;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * m2) return;
  const long long b = idx / m2, rem = idx % m2;
  const int i = (int)(rem % m), j = (int)(rem / m);
  const cplx I1 = cmk(0.0, 1.0);
  cplx v = cmk(0.0, 0.0);
  if (j >= n) {
    const long long e = b * n2 + (i % n) + (long long)(j - n) * n;
    v = cneg(i < n ? F[e] : G[e]);
  } else if (i == j) {                                          // D1
    v = (i < N) ? cmk(1.0, 0.0) : cdiv(cmul(I1, kz_top[b * N + i - N]), eps_top[b]);
  } else if (i == j + n) {                                      // D2
    v = (j < N) ? cmul(I1, kz_top[b * N + j]) : cmk(1.0, 0.0);
  }
  A[idx] = v;
  if (j < 3) {
    // incidence columns: the given polarization, pure s (sin, cos of pi/2), pure p
    cplx as, ap;
    if (j == 0) { as = pol[2 * b]; ap = pol[2 * b + 1]; }
    else if (j == 1) { as = cmk(1.0, 0.0); ap = cmk(6.123233995736766e-17, 0.0); }
    else { as = cmk(0.0, 0.0); ap = cmk(1.0, 0.0); }
    const int spec = N / 2;
    const cplx kzi = kz_top[b * N + spec], ntb = nt[b];
    cplx c = cmk(0.0, 0.0);
    if (i == spec) c = cneg(as);
    else if (i == N + spec) c = cmul(ap, cdiv(cmul(ntb, kzi), eps_top[b]));
    else if (i == 2 * N + spec) c = cmul(cmul(I1, as), kzi);
    else if (i == 3 * N + spec) c = cmul(cmul(I1, ntb), ap);
    cols[b * 3 * (long long)m + i + (long long)j * m] = c;
  }
}

// cref = [x_s; -x_p] from the final matching's first n unknowns (three columns)
__global__ void etm_cref_kernel(int B, int N, const cplx* __restrict__ x, cplx* __restrict__ cref) {
  const int n = 2 * N;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)B * n * 3) return;
  const long long b = idx / (n * 3);
  const int rem = (int)(idx % (n * 3)), i = rem % n, c = rem / n;
  const cplx v = x[b * 6 * (long long)n + i + (long long)c * 2 * n];
  cref[idx] = i < N ? v : cneg(v);
}

struct EtmBufs {
  PortVectors pv;
  int *pair_layer, *pair_solve;
  double* pair_thick;
  cplx *OM, *Zb, *LW, *LV, *X, *F, *G, *S1, *S2, *A, *Tt, *Fin, *xc, *cref, *ctrn;
  int *pivW, *pivV, *pivA, *pivF;
  template <class Ar> bool carve(Ar& ar, int Bc, int L, int N) {
    const size_t n = 2 * (size_t)N, n2 = n * n, P = (size_t)Bc * L;
    PortVectors& v = pv;
    v.kx = ar.template get<double>((size_t)Bc * N); v.ky = ar.template get<double>((size_t)Bc * N);
    v.c = ar.template get<double>((size_t)Bc * N); v.s = ar.template get<double>((size_t)Bc * N);
    v.kz_top = ar.template get<cplx>((size_t)Bc * N); v.kz_bot = ar.template get<cplx>((size_t)Bc * N);
    v.wg = ar.template get<cplx>(Bc * n); v.vg = ar.template get<cplx>(Bc * n);
    v.r11 = ar.template get<cplx>(Bc * n); v.r12 = ar.template get<cplx>(Bc * n);
    v.r21 = ar.template get<cplx>(Bc * n); v.r22 = ar.template get<cplx>(Bc * n);
    v.t11 = ar.template get<cplx>(Bc * n); v.t21 = ar.template get<cplx>(Bc * n);
    v.nt = ar.template get<cplx>(Bc); v.nb = ar.template get<cplx>(Bc);
    pair_layer = ar.template get<int>(P); pair_solve = ar.template get<int>(P);
    pair_thick = ar.template get<double>(P);
    OM = ar.template get<cplx>(P * n2); Zb = ar.template get<cplx>(P * n2);
    LW = ar.template get<cplx>(P * n2); LV = ar.template get<cplx>(P * n2);
    X = ar.template get<cplx>(P * n);
    pivW = ar.template get<int>(P * n); pivV = ar.template get<int>(P * n);
    F = ar.template get<cplx>(Bc * n2); G = ar.template get<cplx>(Bc * n2);
    S1 = ar.template get<cplx>(Bc * n2); S2 = ar.template get<cplx>(Bc * n2);
    A = ar.template get<cplx>(Bc * n2); Tt = ar.template get<cplx>(Bc * n2);
    pivA = ar.template get<int>(Bc * n);
    Fin = ar.template get<cplx>(Bc * 4 * n2); pivF = ar.template get<int>(Bc * 2 * n);
    xc = ar.template get<cplx>(Bc * 6 * n);
    cref = ar.template get<cplx>(Bc * 3 * n); ctrn = ar.template get<cplx>(Bc * 3 * n);
    return ar.ok();
  }
};

size_t etm_chunk_bytes(int N, int L, int chunk) {
  ByteCount c;
  EtmBufs eb;
  eb.carve(c, chunk, L, N);
  return c.b;
}

int etm_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* Wm, const cplx* Vm, const cplx* qm,
              int first, int count, const SolveOut& out) {
  typedef Cx<double> C;
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers;
  const long long n2 = (long long)n * n, lay_bs = (long long)L * n2, lay_ps = (long long)L * n;
  const int Bc = count, P = Bc * L;
  int32_t* st = out.status + first;
  ar.reset();
  EtmBufs e;
  if (!e.carve(ar, Bc, L, N)) return -1;
  given_modes(s, d, Wm, Vm, qm, first, Bc, e.pv, e.pair_layer, e.pair_solve, e.pair_thick, e.OM, e.Zb, e.X);
  cudaMemcpyAsync(e.LW, e.OM, sizeof(cplx) * P * n2, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(e.LV, e.Zb, sizeof(cplx) * P * n2, cudaMemcpyDeviceToDevice, s);
  getrf<double>(s, P, n, (C*)e.LW, n, n2, e.pivW, n, st, L);
  getrf<double>(s, P, n, (C*)e.LV, n, n2, e.pivV, n, st, L);
  const unsigned gn2 = nblk((long long)Bc * n2, 256);
  etm_init_kernel<<<gn2, 256, 0, s>>>(Bc, N, e.pv.kz_bot, d.eps_bot + first, e.F, e.G, e.Tt); note_launch();
  const double2 one = make_double2(1, 0), mone = make_double2(-1, 0);
  for (int l = L - 1; l >= 0; --l) {
    cudaMemcpyAsync(e.S1, e.F, sizeof(cplx) * Bc * n2, cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(e.S2, e.G, sizeof(cplx) * Bc * n2, cudaMemcpyDeviceToDevice, s);
    getrs<double>(s, Bc, n, (const C*)(e.LW + l * n2), n, lay_bs, e.pivW + (long long)l * n, lay_ps, (C*)e.S1, n, n,
                  n2, 0);                                                                         // bW^-1 F
    getrs<double>(s, Bc, n, (const C*)(e.LV + l * n2), n, lay_bs, e.pivV + (long long)l * n, lay_ps, (C*)e.S2, n, n,
                  n2, 0);                                                                         // bV^-1 G
    etm_ab_kernel<<<gn2, 256, 0, s>>>(Bc, n, e.S1, e.S2, e.A, e.F); note_launch();               // a, b^T
    getrf<double>(s, Bc, n, (C*)e.A, n, n2, e.pivA, n, st, 1);
    getrs<double>(s, Bc, n, (const C*)e.A, n, n2, e.pivA, n, (C*)e.F, n, n, n2, 1);              // (b a^-1)^T
    getrs<double>(s, Bc, n, (const C*)e.A, n, n2, e.pivA, n, (C*)e.Tt, n, n, n2, 1);             // a^-T Tt
    etm_y_kernel<<<gn2, 256, 0, s>>>(Bc, n, e.F, e.X + (long long)l * n, lay_ps, e.S1, e.Tt); note_launch();
    cudaMemcpy2DAsync(e.F, sizeof(cplx) * n2, e.OM + l * n2, sizeof(cplx) * lay_bs, sizeof(cplx) * n2, Bc,
                      cudaMemcpyDeviceToDevice, s);
    cudaMemcpy2DAsync(e.G, sizeof(cplx) * n2, e.Zb + l * n2, sizeof(cplx) * lay_bs, sizeof(cplx) * n2, Bc,
                      cudaMemcpyDeviceToDevice, s);
    gemm<double>(s, Bc, n, n, n, one, (const C*)(e.OM + l * n2), 1, n, lay_bs, (const C*)e.S1, 1, n, n2, one,
                 (C*)e.F, 1, n, n2);                                                              // bW (I + Y)
    gemm<double>(s, Bc, n, n, n, mone, (const C*)(e.Zb + l * n2), 1, n, lay_bs, (const C*)e.S1, 1, n, n2, one,
                 (C*)e.G, 1, n, n2);                                                              // bV (I - Y)
  }
  const long long m2 = 4 * n2;
  etm_final_kernel<<<nblk((long long)Bc * m2, 256), 256, 0, s>>>(Bc, N, e.F, e.G, e.pv.kz_top, d.eps_top + first,
                                                                 e.pv.nt, d.pol + 2 * first, e.Fin, e.xc);
  note_launch();
  getrf<double>(s, Bc, 2 * n, (C*)e.Fin, 2 * n, m2, e.pivF, 2 * n, st, 1);
  getrs<double>(s, Bc, 2 * n, (const C*)e.Fin, 2 * n, m2, e.pivF, 2 * n, (C*)e.xc, 3, 2 * n, 6LL * n, 0);
  const long long v3 = 3LL * n;
  etm_cref_kernel<<<nblk((long long)Bc * v3, 256), 256, 0, s>>>(Bc, N, e.xc, e.cref); note_launch();
  const double2 zero = make_double2(0, 0);
  gemm<double>(s, Bc, n, 3, n, one, (const C*)e.Tt, n, 1, n2, (const C*)(e.xc + n), 1, 2 * n, 6LL * n, zero,
               (C*)e.ctrn, 1, n, v3);                                                             // T x[n:]
  efficiency_kernel<double><<<nblk((long long)Bc * N * 3, 256), 256, 0, s>>>(
      Bc, N, (const C*)e.cref, (const C*)e.ctrn, v3, e.pv, d.eps_top + first, d.eps_bot + first, d.pol + 2 * first,
      out.R + (long long)first * 3 * N, out.T + (long long)first * 3 * N,
      out.amps ? out.amps + (long long)first * 12 * N : nullptr, st);
  note_launch();
  return 0;
}

// ------------------------------------------------------------- stage B door (wb_layer_modes)
__global__ void iota_kernel(int n, int* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}
__global__ void fill_kernel(int n, double v, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = v;
}

size_t layer_modes_bytes(int N, int n_pairs, int precision) {
  const size_t n = 2 * (size_t)N, n2 = n * n, P = n_pairs;
  size_t b = 0;
  auto A = [&](size_t x) { b += (x + 255) & ~(size_t)255; };
  A(sizeof(int) * P); A(sizeof(double) * P); A(sizeof(double) * P);
  if (precision == 1) {                       // FP32 eigen-solve with Newton steps
    A(16 * P * n2);                                                   // Omega^2 W scratch
    for (int k = 0; k < 4; ++k) A(8 * P * n2);                        // F1..F4
    A(8 * P * n); A(8 * P * n);                                       // wr, tau
    A(sizeof(int) * P * n);                                           // pivots
    A(16 * P * n); A(16 * P * n);                                     // lambda, X
    return b + GroupBufs::bytes((int)P, (int)n);
  }
  A(16 * P * n2); A(16 * P * n2); A(16 * P * n2); A(16 * P * n2);
  for (int k = 0; k < 3; ++k) A(16 * P * n);
  return b;
}

// The FP32 eigen-solve refined by Newton steps (the mixed form's stage B), Cartesian FP64 modes
// straight into W and V.
static int layer_modes_newton(cudaStream_t s, Arena& ar, int P, int N, const cplx* conv, const int* pair_layer,
                              const double* kx, const double* ky, cplx* w, cplx* q, cplx* W, cplx* V,
                              int32_t* status) {
  const int n = 2 * N;
  const long long n2 = (long long)n * n;
  ar.reset();
  int* pair_solve = ar.get<int>(P);
  double* zero = ar.get<double>(P);
  double* lam1 = ar.get<double>(P);
  cplx* Om = ar.get<cplx>((size_t)P * n2);
  NewtonBufs nb;
  nb.F1 = ar.get<Cx<float>>((size_t)P * n2); nb.F2 = ar.get<Cx<float>>((size_t)P * n2);
  nb.F3 = ar.get<Cx<float>>((size_t)P * n2); nb.F4 = ar.get<Cx<float>>((size_t)P * n2);
  nb.wr = ar.get<Cx<float>>((size_t)P * n); nb.tau = ar.get<Cx<float>>((size_t)P * n);
  nb.piv = ar.get<int>((size_t)P * n);
  nb.lam = ar.get<cplx>((size_t)P * n);
  cplx* X = ar.get<cplx>((size_t)P * n);
  GroupBufs gb;
  if (!gb.carve(ar, P, n) || !ar.ok()) return -1;
  iota_kernel<<<nblk(P, 128), 128, 0, s>>>(P, pair_solve); note_launch();
  fill_kernel<<<nblk(P, 128), 128, 0, s>>>(P, 0.0, zero); note_launch();
  fill_kernel<<<nblk(P, 128), 128, 0, s>>>(P, 1.0, lam1); note_launch();
  if (status) cudaMemsetAsync(status, 0, sizeof(int32_t) * P, s);
  stage_b_newton(s, P, N, conv, pair_layer, pair_solve, zero, lam1, kx, ky, W, V, Om, nb, gb, w, q, X, nullptr,
                 nullptr, status, 1, false);
  return 0;
}

template <class R>
void layer_modes_t(cudaStream_t s, Arena& ar, int P, int N, const cplx* conv, const int* pair_layer,
                   const double* kx, const double* ky, cplx* w, cplx* q, cplx* W, cplx* V, int32_t* status) {
  const int n = 2 * N;
  const long long n2 = (long long)n * n;
  ar.reset();
  int* pair_solve = ar.get<int>(P);
  double* zero = ar.get<double>(P);
  double* lam = ar.get<double>(P);
  Cx<R>* OM = ar.get<Cx<R>>((size_t)P * n2);
  Cx<R>* Zb = ar.get<Cx<R>>((size_t)P * n2);
  Cx<R>* Xv = ar.get<Cx<R>>((size_t)P * n2);
  Cx<R>* wr = ar.get<Cx<R>>((size_t)P * n);
  Cx<R>* tau = ar.get<Cx<R>>((size_t)P * n);
  cplx* X = ar.get<cplx>((size_t)P * n);
  iota_kernel<<<nblk(P, 128), 128, 0, s>>>(P, pair_solve); note_launch();
  fill_kernel<<<nblk(P, 128), 128, 0, s>>>(P, 0.0, zero); note_launch();
  fill_kernel<<<nblk(P, 128), 128, 0, s>>>(P, 1.0, lam); note_launch();
  if (status) cudaMemsetAsync(status, 0, sizeof(int32_t) * P, s);
  stage_b<R>(s, P, N, conv, pair_layer, pair_solve, zero, lam, kx, ky, OM, Zb, Xv, wr, tau, w, q, X, nullptr, nullptr,
             status, 1, false);
  convert<R, double>(s, OM, (Cx<double>*)W, (long long)P * n2);
  convert<R, double>(s, Zb, (Cx<double>*)V, (long long)P * n2);
}

int layer_modes(cudaStream_t s, Arena& ar, int P, int N, const cplx* conv, const int* pair_layer,
                const double* kx, const double* ky, cplx* w, cplx* q, cplx* W, cplx* V, int32_t* status,
                int precision) {
  if (precision == 1) return layer_modes_newton(s, ar, P, N, conv, pair_layer, kx, ky, w, q, W, V, status);
  if (precision == 0) layer_modes_t<double>(s, ar, P, N, conv, pair_layer, kx, ky, w, q, W, V, status);
  else layer_modes_t<df64>(s, ar, P, N, conv, pair_layer, kx, ky, w, q, W, V, status);
  return ar.ok() ? 0 : -1;
}

__global__ void regroup_kernel(int L, long long NN, const cplx* __restrict__ planes, cplx* __restrict__ out) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= 3LL * L * NN) return;
  const long long slot = idx / ((long long)L * NN), rem = idx % ((long long)L * NN);
  const long long layer = rem / NN, e = rem % NN;
  out[(layer * 3 + slot) * NN + e] = planes[idx];
}

void regroup_slots(cudaStream_t s, int L, int N, const cplx* planes, cplx* out) {
  long long NN = (long long)N * N;
  regroup_kernel<<<nblk(3LL * L * NN, 256), 256, 0, s>>>(L, NN, planes, out); note_launch();
}

}  // namespace wb
