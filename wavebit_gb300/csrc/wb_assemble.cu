// Stage A: Li-rule convolution matrices of permittivity rasters (fixed nesting, sampled
// coefficients). Follows factorization.py of the reference:
//   series:  _raster_series / _row_dft / _pixel_correction   (factorization.py:289-440)
//   epx = ( T_u( [T_v(eps)]^-1 ) )^-1,  epy = T_u( [T_v(1/eps)]^-1 ),  epz_i = ( T_uv(eps) )^-1
//            (_nested_rule :523-567, _li_slot :600-633, _li_conv :636-642)
//   BTTB rows i = n * n_u + m, entry (i, i') = c_{(n-n'), (m-m')}  (_conv_matrix :504-520)
// Only orders -2h..2h of each line are needed, so each coefficient is a direct DFT sum over
// the line's pixels (with exact integer argument reduction) rather than a full FFT.
// Integrated coefficients (to_conv_mat_raster_integrated, factorization.py:3181-3206) run the
// same pipeline on a compressed raster, with the closed-form segment series (wb_series.cuh) in
// place of the staircase series; the compression itself is done once on the host.
// The work is a few tens of MFLOP per 256x256 layer and is cached per layer: it is
// HBM/latency-bound and tiny next to stages B and C.
#include "wb_common.cuh"
#include "wb_kernels.h"
#include "wb_series.cuh"

namespace wb {

// coefficient of order k (|k| <= 2h) of one staircase line a_0..a_{n-1}:
//   sum_j (a_j - a_0)/n exp(-2 pi i k j / n) * sinc(k/n) exp(-i pi k / n)  (+ a_0 at k = 0)
// The twiddles exp(-2 pi i p / n), p = k j mod n, come from a table of the line length built once
// per block in dynamic shared memory (the same sincospi values the sum would compute term by
// term), so a term is one complex multiply-add; lines longer than the table compute them in place.
constexpr int kSeriesTable = 3072;                  // 48 KB of twiddles: no shared-memory opt-in

__global__ void series_kernel(const cplx* __restrict__ in, long long n_lines, int lines_per_group,
                              long long group_stride, long long line_stride, long long pt_stride,
                              int npts, int h, int reciprocal, cplx* __restrict__ out) {
  extern __shared__ cplx tw[];
  const bool table = npts <= kSeriesTable;
  if (table)
    for (int p = threadIdx.x; p < npts; p += blockDim.x) {
      double sn, cs;
      sincospi(-2.0 * (double)p / (double)npts, &sn, &cs);
      tw[p] = cmk(cs, sn);
    }
  __syncthreads();
  const int nk = 4 * h + 1;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n_lines * nk) return;
  const long long line = idx / nk;
  const int kk = (int)(idx % nk);
  const int k = kk - 2 * h;
  const cplx* a = in + (line / lines_per_group) * group_stride + (line % lines_per_group) * line_stride;
  cplx a0 = a[0];
  if (reciprocal) a0 = cinv(a0);
  cplx acc = cmk(0.0, 0.0);
  if (npts > 1) {
    const int kmod = ((k % npts) + npts) % npts;
    int p = kmod;                                     // (kmod * j) mod npts, advanced by kmod
    for (int j = 1; j < npts; ++j) {
      cplx aj = a[j * pt_stride];
      if (reciprocal) aj = cinv(aj);
      const cplx d = csub(aj, a0);
      cplx t;
      if (table) {
        t = tw[p];
      } else {
        double sn, cs;
        sincospi(-2.0 * (double)p / (double)npts, &sn, &cs);
        t = cmk(cs, sn);
      }
      acc = cfma(d, t, acc);
      p += kmod;
      if (p >= npts) p -= npts;
    }
    acc = cscale(acc, 1.0 / (double)npts);
  }
  // pixel correction sinc(k/n) exp(-i pi k/n)
  if (k != 0) {
    const double t = (double)k / (double)npts;
    const double sinc = sinpi(t) / (3.141592653589793 * t);
    double sn, cs;
    sincospi(-t, &sn, &cs);
    acc = cmul(acc, cmk(sinc * cs, sinc * sn));
  } else {
    acc = cadd(acc, a0);
  }
  out[line * nk + kk] = acc;
}

// The integrated counterpart of series_kernel: the same line addressing, and per line the
// right edges of its segments, edges[((line / lines_per_seg) % n_seg_rows) * npts + j].
__global__ void segment_series_kernel(const cplx* __restrict__ in, long long n_lines, int lines_per_group,
                                      long long group_stride, long long line_stride, long long pt_stride,
                                      int npts, int h, int reciprocal, const double* __restrict__ edges,
                                      long long lines_per_seg, int n_seg_rows, cplx* __restrict__ out) {
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= n_lines * (4 * h + 1)) return;
  segment_series_at(idx, in, lines_per_group, group_stride, line_stride, pt_stride, npts, h, reciprocal, edges,
                    lines_per_seg, n_seg_rows, out);
}

// One series launch: the staircase series when `edges` is NULL, else the segment series with
// `lines_per_seg` consecutive lines sharing a row of edges (rows cycle over n_seg_rows layers).
static void launch_series(cudaStream_t s, const cplx* in, long long lines, int lines_per_group,
                          long long group_stride, long long line_stride, long long pt_stride, int npts, int h,
                          int reciprocal, const double* edges, long long lines_per_seg, int n_seg_rows,
                          cplx* out) {
  const long long th = lines * (4 * h + 1);
  const unsigned blocks = (unsigned)((th + 127) / 128);
  if (edges)
    segment_series_kernel<<<blocks, 128, 0, s>>>(in, lines, lines_per_group, group_stride, line_stride, pt_stride,
                                                 npts, h, reciprocal, edges, lines_per_seg, n_seg_rows, out);
  else
    series_kernel<<<blocks, 128, npts <= kSeriesTable ? sizeof(cplx) * npts : 0, s>>>(
        in, lines, lines_per_group, group_stride, line_stride, pt_stride, npts, h, reciprocal, out);
  note_launch();
}

// Inverse of the (2h+1)^2 Toeplitz matrix T[r][c] = coef[r - c + 2h] of each line, by
// Gauss-Jordan elimination with partial pivoting in shared memory. Output layout
// out[((g * nv + r) * nv + c) * n_lines_per_group + x] so that each matrix entry is a
// contiguous line over x for the next series.
__global__ void toeplitz_inverse_kernel(const cplx* __restrict__ coef, int n_lines_per_group, int h,
                                        cplx* __restrict__ out, int32_t* status) {
  extern __shared__ cplx sm[];
  const int nv = 2 * h + 1, nk = 4 * h + 1, w2 = 2 * nv;
  __shared__ int piv;
  const long long line = blockIdx.x;   // g * n_lines_per_group + x
  const long long g = line / n_lines_per_group;
  const int x = (int)(line % n_lines_per_group);
  const cplx* cf = coef + line * nk;
  cplx* M = sm;   // nv x (2 nv), row-major
  for (int e = threadIdx.x; e < nv * w2; e += blockDim.x) {
    int r = e / w2, c = e % w2;
    M[e] = (c < nv) ? cf[r - c + 2 * h] : cmk(c - nv == r ? 1.0 : 0.0, 0.0);
  }
  __syncthreads();
  for (int col = 0; col < nv; ++col) {
    if (threadIdx.x == 0) {
      int p = col; double best = cabs1(M[col * w2 + col]);
      for (int r = col + 1; r < nv; ++r) {
        double v = cabs1(M[r * w2 + col]);
        if (v > best) { best = v; p = r; }
      }
      piv = p;
      if (best == 0.0) wb_flag(status, WB_ST_SINGULAR);
    }
    __syncthreads();
    const int p = piv;
    if (p != col)
      for (int c = threadIdx.x; c < w2; c += blockDim.x) {
        cplx t = M[col * w2 + c]; M[col * w2 + c] = M[p * w2 + c]; M[p * w2 + c] = t;
      }
    __syncthreads();
    const cplx rp = cinv(M[col * w2 + col]);
    __syncthreads();
    for (int c = threadIdx.x; c < w2; c += blockDim.x) M[col * w2 + c] = cmul(M[col * w2 + c], rp);
    __syncthreads();
    for (int e = threadIdx.x; e < nv * w2; e += blockDim.x) {
      int r = e / w2, c = e % w2;
      if (r == col) continue;
      cplx f = M[r * w2 + col];
      if (c == col) continue;
      M[e] = csub(M[e], cmul(f, M[col * w2 + c]));
    }
    __syncthreads();
    for (int r = threadIdx.x; r < nv; r += blockDim.x)
      if (r != col) M[r * w2 + col] = cmk(0.0, 0.0);
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nv * nv; e += blockDim.x) {
    int r = e / nv, c = e % nv;
    out[((g * nv + r) * nv + c) * n_lines_per_group + x] = M[r * w2 + nv + c];
  }
}

// conv (column-major N x N, N = nv * nu) from per-entry u-series:
//   nested: conv[r nu + m, c nu + m'] = cu[((g * nv + r) * nv + c) * nku + (m - m' + 2hu)]
//   direct: conv[r nu + m, c nu + m'] = c2[(g * nkv + (r - c + 2hv)) * nku + (m - m' + 2hu)]
__global__ void bttb_scatter_kernel(const cplx* __restrict__ cu, int L, int hu, int hv, int direct,
                                    cplx* __restrict__ conv) {
  const int nu = 2 * hu + 1, nv = 2 * hv + 1, N = nu * nv, nku = 4 * hu + 1, nkv = 4 * hv + 1;
  long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)L * N * N) return;
  const long long g = idx / ((long long)N * N);
  const long long rem = idx % ((long long)N * N);
  const int i = (int)(rem % N), ip = (int)(rem / N);
  const int r = i / nu, m = i % nu, c = ip / nu, mp = ip % nu;
  cplx v;
  if (direct) v = cu[(g * nkv + (r - c + 2 * hv)) * nku + (m - mp + 2 * hu)];
  else v = cu[((g * nv + r) * nv + c) * nku + (m - mp + 2 * hu)];
  conv[g * N * N + i + (long long)ip * N] = v;
}

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t assemble_workspace_bytes(int L, int ny, int nx, int hu, int hv) {
  const size_t nu = 2 * hu + 1, nv = 2 * hv + 1, N = nu * nv, nku = 4 * hu + 1, nkv = 4 * hv + 1;
  size_t b = 0;
  b += align256(sizeof(cplx) * L * 2 * nx * nkv);          // cv  (eps, 1/eps) column series
  b += align256(sizeof(cplx) * L * 2 * nv * nv * nx);      // inner inverses
  b += align256(sizeof(cplx) * L * 2 * nv * nv * nku);     // cu
  b += align256(sizeof(cplx) * L * nkv * nku);             // c2 (direct rule)
  b += align256(sizeof(cplx) * 2 * L * N * N);             // pre-inverse matrices
  b += align256(sizeof(int) * 2 * L * N);                  // pivots
  return b;
}

void assemble_li(cudaStream_t s, const cplx* eps, int L, int ny, int nx, int hu, int hv,
                 cplx* epx, cplx* epy, cplx* epz_i, void* ws, int32_t* status, const double* x_edges,
                 const double* y_edges) {
  const int nu = 2 * hu + 1, nv = 2 * hv + 1, N = nu * nv, nku = 4 * hu + 1, nkv = 4 * hv + 1;
  char* p = static_cast<char*>(ws);
  cplx* cv = reinterpret_cast<cplx*>(p); p += align256(sizeof(cplx) * L * 2 * nx * nkv);
  cplx* inner = reinterpret_cast<cplx*>(p); p += align256(sizeof(cplx) * L * 2 * nv * nv * nx);
  cplx* cu = reinterpret_cast<cplx*>(p); p += align256(sizeof(cplx) * L * 2 * nv * nv * nku);
  cplx* c2 = reinterpret_cast<cplx*>(p); p += align256(sizeof(cplx) * L * nkv * nku);
  cplx* pre = reinterpret_cast<cplx*>(p); p += align256(sizeof(cplx) * 2 * L * N * N);
  int* ipiv = reinterpret_cast<int*>(p);
  const long long plane = (long long)ny * nx;
  // 1. series along v of every column, for eps (groups 0..L-1) and 1/eps (groups L..2L-1);
  //    line = layer * nx + x
  for (int rec = 0; rec < 2; ++rec)
    launch_series(s, eps, (long long)L * nx, nx, plane, 1, nx, ny, hv, rec, y_edges, nx, L,
                  cv + (long long)rec * L * nx * nkv);
  // 2. inner Toeplitz inverses, groups (rec, layer): 2L groups of nx lines
  {
    size_t sm = sizeof(cplx) * nv * 2 * nv;
    // past the default 48 KB a block has to opt in (hv <= 42 keeps the tile within 227 KB)
    if (sm > 48 * 1024)
      cudaFuncSetAttribute(toeplitz_inverse_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    toeplitz_inverse_kernel<<<2 * L * nx, 128, sm, s>>>(cv, nx, hv, inner, status); note_launch();
  }
  // 3. series along u of every inner-inverse entry: 2L * nv^2 lines of nx points;
  //    line = ((rec * L + layer) * nv + r) * nv + c
  launch_series(s, inner, 2LL * L * nv * nv, 1, nx, 0, 1, nx, hu, 0, x_edges, (long long)nv * nv, L, cu);
  // 4. direct rule: series along u of the eps column series (lines (layer, kv), points x).
  //    cv for eps is laid out [(layer * nx + x) * nkv + kv]: line (layer, kv) has stride nkv per x
  launch_series(s, cv, (long long)L * nkv, nkv, (long long)nx * nkv, 1, nkv, nx, hu, 0, x_edges, nkv, L, c2);
  // 5. BTTB layouts: pre[0:L] = T_u([T_v(eps)]^-1), epy = T_u([T_v(1/eps)]^-1), pre[L:2L] = T_uv(eps)
  {
    long long th = (long long)L * N * N;
    unsigned blocks = (unsigned)((th + 255) / 256);
    bttb_scatter_kernel<<<blocks, 256, 0, s>>>(cu, L, hu, hv, 0, pre); note_launch();
    bttb_scatter_kernel<<<blocks, 256, 0, s>>>(cu + (long long)L * nv * nv * nku, L, hu, hv, 0, epy); note_launch();
    bttb_scatter_kernel<<<blocks, 256, 0, s>>>(c2, L, hu, hv, 1, pre + (long long)L * N * N); note_launch();
  }
  // 6. epx = inv(pre[0:L]), epz_i = inv(pre[L:2L])
  zgetrf(s, 2 * L, N, pre, N, (long long)N * N, ipiv, N, status, 1 << 30);
  zset_identity(s, L, N, epx, N, (long long)N * N);
  zset_identity(s, L, N, epz_i, N, (long long)N * N);
  zgetrs(s, L, N, pre, N, (long long)N * N, ipiv, N, epx, N, N, (long long)N * N, 0);
  zgetrs(s, L, N, pre + (long long)L * N * N, N, (long long)N * N, ipiv + (long long)L * N, N, epz_i, N, N,
         (long long)N * N, 0);
}

}  // namespace wb
