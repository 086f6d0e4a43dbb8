// Shared device helpers for the RCWA raster-path kernels (sm_103a).
//
// Storage conventions used by every kernel in this library:
//   * complex numbers are interleaved (re, im) doubles, i.e. cuDoubleComplex / double2;
//   * matrices are column-major with a leading dimension: element (i, j) of a matrix at `a`
//     with leading dimension `ld` lives at a[i + j * ld];
//   * a batch of matrices is addressed by a base pointer plus a per-matrix stride (in elements).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define WB_HD __host__ __device__ __forceinline__
#define WB_D __device__ __forceinline__

typedef double2 cplx;

WB_HD cplx cmk(double re, double im) { cplx c; c.x = re; c.y = im; return c; }
WB_HD cplx cadd(cplx a, cplx b) { return cmk(a.x + b.x, a.y + b.y); }
WB_HD cplx csub(cplx a, cplx b) { return cmk(a.x - b.x, a.y - b.y); }
WB_HD cplx cmul(cplx a, cplx b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
WB_HD cplx cconj(cplx a) { return cmk(a.x, -a.y); }
WB_HD cplx cscale(cplx a, double s) { return cmk(a.x * s, a.y * s); }
WB_HD cplx cneg(cplx a) { return cmk(-a.x, -a.y); }
WB_HD double cabs1(cplx a) { return fabs(a.x) + fabs(a.y); }
WB_HD double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }
WB_HD double cabsv(cplx a) { return hypot(a.x, a.y); }
// c += a * b with four fused multiply-adds
WB_HD cplx cfma(cplx a, cplx b, cplx c) {
  c.x = fma(a.x, b.x, c.x); c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y); c.y = fma(a.y, b.x, c.y);
  return c;
}
// c += conj(a) * b
WB_HD cplx cfma_conj(cplx a, cplx b, cplx c) {
  c.x = fma(a.x, b.x, c.x); c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y); c.y = fma(-a.y, b.x, c.y);
  return c;
}
// a / b, scaled to avoid overflow (Smith's algorithm)
WB_HD cplx cdiv(cplx a, cplx b) {
  if (fabs(b.y) <= fabs(b.x)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return cmk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  double r = b.x / b.y, d = b.y + b.x * r;
  return cmk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
WB_HD cplx cinv(cplx b) { return cdiv(cmk(1.0, 0.0), b); }
// principal square root, Re >= 0 (branch cut on the negative real axis, sqrt(-a + 0i) = +i sqrt(a))
WB_HD cplx csqrt_p(cplx z) {
  double x = z.x, y = z.y;
  if (x == 0.0 && y == 0.0) return cmk(0.0, y);
  double t = sqrt(0.5 * (fabs(x) + hypot(x, y)));
  if (x >= 0.0) return cmk(t, y / (2.0 * t));
  return cmk(fabs(y) / (2.0 * t), copysign(t, y));
}
WB_HD cplx cexp_(cplx z) {
  double e = exp(z.x);
  double s, c;
  sincos(z.y, &s, &c);
  return cmk(e * c, e * s);
}

// Per-problem status bits written on the device (0 = ok); the same values as the public header.
#ifndef WB_ST_SINGULAR
#define WB_ST_SINGULAR 1     // an exact zero pivot in an LU factorisation
#define WB_ST_NOCONV 2       // the eigenvalue iteration hit its cap
#define WB_ST_NONFINITE 4    // a NaN/Inf reached an output
#define WB_ST_GRAZING 8      // min|w| < 1e-9 max|w| (the reference rebuilds such a layer)
#endif

__device__ __forceinline__ void wb_flag(int32_t* status, int code) {
  if (status) atomicOr(reinterpret_cast<int*>(status), code);
}
