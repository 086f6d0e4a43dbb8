// Fourier orders of one line of a compressed raster: a profile that is constant on segments of
// the unit cell (the integrated coefficients). Host- and device-callable, so the same code is
// checked against the oracle on the CPU and run by segment_series_kernel on the GPU.
#pragma once
#include "wb_common.cuh"

namespace wb {

// Segment j of a line whose segments end at the right edges e_0 < ... < e_{n-1}:
//   right_j = e_j / e_{n-1},  left_j = right_{j-1} (0 for j = 0),  width_j = right_j - left_j
// (segment_bounds, rcwa/_engine/factorization.py:443-454).
WB_HD void segment_bounds(const double* edges, int npts, int j, double* left, double* width) {
  const double last = edges[npts - 1];
  const double right = edges[j] / last;
  *left = j ? edges[j - 1] / last : 0.0;
  *width = right - *left;
}

WB_HD cplx segment_value(const cplx* a, long long pt_stride, int j, int reciprocal) {
  const cplx v = a[j * pt_stride];
  return reciprocal ? cinv(v) : v;
}

// Order k of the line a_0..a_{n-1} (stride pt_stride; 1/a when `reciprocal`), in the jump form
// of the closed-form segment integrals (_segment_series, factorization.py:457-501):
//   c_0 = sum_j a_j width_j,
//   c_k = sum_j (a_j - a_{j-1}) exp(-2 pi i k left_j) / (2 pi i k),  a_{-1} = a_{n-1}.
WB_HD cplx segment_coefficient(const cplx* a, long long pt_stride, int npts, const double* edges, int k,
                               int reciprocal) {
  cplx acc = cmk(0.0, 0.0);
  if (k == 0) {
    for (int j = 0; j < npts; ++j) {
      double left, width;
      segment_bounds(edges, npts, j, &left, &width);
      const cplx v = segment_value(a, pt_stride, j, reciprocal);
      acc = cadd(acc, cscale(v, width));
    }
    return acc;
  }
  cplx prev = segment_value(a, pt_stride, npts - 1, reciprocal);
  for (int j = 0; j < npts; ++j) {
    double left, width;
    segment_bounds(edges, npts, j, &left, &width);
    const cplx cur = segment_value(a, pt_stride, j, reciprocal);
    double sn, cs;
    sincospi(-2.0 * ((double)k * left), &sn, &cs);
    acc = cfma(csub(cur, prev), cmk(cs, sn), acc);
    prev = cur;
  }
  // divide by 2 pi i k: (x + i y) / (i t) = (y - i x) / t
  const double t = 2.0 * 3.141592653589793 * (double)k;
  return cmk(acc.y / t, -acc.x / t);
}

// Element idx of one segment-series launch (thread idx of segment_series_kernel): line
// idx / (4h+1), order idx % (4h+1) - 2h. The line's points start at
// in[(line / lines_per_group) * group_stride + (line % lines_per_group) * line_stride], step
// pt_stride; its edges are row (line / lines_per_seg) % n_seg_rows of `edges` (npts each).
WB_HD void segment_series_at(long long idx, const cplx* in, int lines_per_group, long long group_stride,
                             long long line_stride, long long pt_stride, int npts, int h, int reciprocal,
                             const double* edges, long long lines_per_seg, int n_seg_rows, cplx* out) {
  const int nk = 4 * h + 1;
  const long long line = idx / nk;
  const int kk = (int)(idx % nk);
  const cplx* a = in + (line / lines_per_group) * group_stride + (line % lines_per_group) * line_stride;
  const double* e = edges + ((line / lines_per_seg) % n_seg_rows) * npts;
  out[line * nk + kk] = segment_coefficient(a, pt_stride, npts, e, kk - 2 * h, reciprocal);
}

}  // namespace wb
