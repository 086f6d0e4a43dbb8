// Scalar types the kernels are written for: IEEE double, IEEE float, and df64 — a double-float
// number (hi + lo, two FP32 values, ~48-bit significand) computed on the FP32 pipes.
//
// GB300 issues ~2 FP64 FMAs per clock per SM against 128 FP32 FMAs, so a df64 operation
// (8-20 FP32 instructions) still runs several times faster than native FP64 while keeping an
// FP64-class relative precision (~4e-15). The error-free transformations below are the
// classical ones: Knuth's two-sum, Dekker/Kahan's two-product through a fused multiply-add,
// and the double-word addition/multiplication of Hida, Li & Bailey (QD library paper, 2001)
// and Joldes, Muller & Popescu (ACM TOMS 44, 2017). The df64 exponent range is FP32's; the
// RCWA operators stay within 1e-30 .. 1e30 and tiny exponentials flush harmlessly to zero.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

#define WB_NHD __host__ __device__ __forceinline__
#define WB_ND __device__ __forceinline__

struct df64 {
  float hi, lo;
  df64() = default;
  WB_NHD constexpr df64(float h, float l) : hi(h), lo(l) {}
  WB_NHD df64(double d) {
    hi = (float)d;
    lo = (float)(d - (double)hi);
  }
  WB_NHD explicit operator double() const { return (double)hi + (double)lo; }
};

namespace wbn {
// s + e = a + b exactly
WB_ND void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly, |a| >= |b|
WB_ND void fast_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
}  // namespace wbn

WB_ND df64 operator+(df64 a, df64 b) {
  float s, e, t, f;
  wbn::two_sum(a.hi, b.hi, s, e);
  wbn::two_sum(a.lo, b.lo, t, f);
  e = __fadd_rn(e, t);
  wbn::fast_two_sum(s, e, s, e);
  e = __fadd_rn(e, f);
  wbn::fast_two_sum(s, e, s, e);
  return df64(s, e);
}
WB_ND df64 operator-(df64 a) { return df64(-a.hi, -a.lo); }
WB_ND df64 operator-(df64 a, df64 b) { return a + (-b); }
WB_ND df64 operator*(df64 a, df64 b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  float s, f;
  wbn::fast_two_sum(p, e, s, f);
  return df64(s, f);
}
WB_ND df64 operator/(df64 a, df64 b) {
  // one Newton correction of the FP32 quotient: q1 = a.hi/b.hi, r = a - q1 b, q2 = r.hi/b.hi
  float q1 = __fdiv_rn(a.hi, b.hi);
  df64 r = a - b * df64(q1, 0.f);
  float q2 = __fdiv_rn(r.hi, b.hi);
  df64 q = df64(q1, 0.f) + df64(q2, 0.f);
  r = a - b * q;
  float q3 = __fdiv_rn(r.hi, b.hi);
  return q + df64(q3, 0.f);
}
WB_ND df64& operator+=(df64& a, df64 b) { a = a + b; return a; }
WB_ND df64& operator-=(df64& a, df64 b) { a = a - b; return a; }
WB_ND df64& operator*=(df64& a, df64 b) { a = a * b; return a; }
WB_ND df64& operator/=(df64& a, df64 b) { a = a / b; return a; }
WB_NHD bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
WB_NHD bool operator>(df64 a, df64 b) { return b < a; }
WB_NHD bool operator<=(df64 a, df64 b) { return !(b < a); }
WB_NHD bool operator>=(df64 a, df64 b) { return !(a < b); }
WB_NHD bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
WB_NHD bool operator!=(df64 a, df64 b) { return !(a == b); }

// ------------------------------------------------------------ generic real helpers
template <class R> struct RealT;
template <> struct RealT<double> {
  WB_NHD static constexpr double eps() { return 2.220446049250313e-16; }
  WB_NHD static constexpr double tiny() { return 2.2250738585072014e-308; }
  WB_NHD static constexpr double big() { return 1e100; }     // rescaling bound, far below overflow
};
template <> struct RealT<float> {
  WB_NHD static constexpr float eps() { return 1.1920928955078125e-07f; }
  WB_NHD static constexpr float tiny() { return 1.1754943508222875e-38f; }
  WB_NHD static constexpr float big() { return 1e18f; }
};
template <> struct RealT<df64> {
  // unit roundoff of the double-word format ~ 2^-47; smallest safe value keeps hi normal
  static WB_ND df64 eps() { return df64(7.105427357601002e-15f, 0.f); }
  static WB_ND df64 tiny() { return df64(1.1754943508222875e-38f * 1024.f, 0.f); }
  static WB_ND df64 big() { return df64(1e18f, 0.f); }
};

WB_NHD double rabs(double a) { return fabs(a); }
WB_NHD float rabs(float a) { return fabsf(a); }
WB_ND df64 rabs(df64 a) { return a.hi < 0.f ? -a : a; }
WB_NHD double rsqrt_(double a) { return sqrt(a); }
WB_NHD float rsqrt_(float a) { return sqrtf(a); }
WB_ND df64 rsqrt_(df64 a) {
  if (a.hi <= 0.f) return df64(0.f, 0.f);
  float s = sqrtf(a.hi);
  df64 sd(s, 0.f);
  // one Newton step: s + (a - s^2) / (2 s)
  df64 r = a - sd * sd;
  float c = __fdiv_rn(r.hi, 2.f * s);
  return sd + df64(c, 0.f);
}
WB_NHD double rmax(double a, double b) { return fmax(a, b); }
WB_NHD float rmax(float a, float b) { return fmaxf(a, b); }
WB_ND df64 rmax(df64 a, df64 b) { return a < b ? b : a; }
WB_NHD double rmin(double a, double b) { return fmin(a, b); }
WB_NHD float rmin(float a, float b) { return fminf(a, b); }
WB_ND df64 rmin(df64 a, df64 b) { return a < b ? a : b; }
WB_NHD bool rfinite(double a) { return isfinite(a); }
WB_NHD bool rfinite(float a) { return isfinite(a); }
WB_NHD bool rfinite(df64 a) { return isfinite(a.hi) && isfinite(a.lo); }
WB_NHD double rfma(double a, double b, double c) { return fma(a, b, c); }
WB_NHD float rfma(float a, float b, float c) { return fmaf(a, b, c); }
WB_ND df64 rfma(df64 a, df64 b, df64 c) { return a * b + c; }
template <class R> WB_ND R rfrom(double d) { return R(d); }
WB_NHD double rto(double a) { return a; }
WB_NHD double rto(float a) { return (double)a; }
WB_NHD double rto(df64 a) { return (double)a; }

// ------------------------------------------------------------------- complex
template <class R> struct Cx {
  R x, y;
};

template <class R> WB_ND Cx<R> cxmk(R re, R im) { Cx<R> c; c.x = re; c.y = im; return c; }
template <class R> WB_ND Cx<R> cxzero() { return cxmk<R>(R(0.0), R(0.0)); }
template <class R> WB_ND Cx<R> cxone() { return cxmk<R>(R(1.0), R(0.0)); }
template <class R> WB_ND Cx<R> operator+(Cx<R> a, Cx<R> b) { return cxmk<R>(a.x + b.x, a.y + b.y); }
template <class R> WB_ND Cx<R> operator-(Cx<R> a, Cx<R> b) { return cxmk<R>(a.x - b.x, a.y - b.y); }
template <class R> WB_ND Cx<R> operator-(Cx<R> a) { return cxmk<R>(-a.x, -a.y); }
template <class R> WB_ND Cx<R> operator*(Cx<R> a, Cx<R> b) {
  return cxmk<R>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class R> WB_ND Cx<R> operator*(Cx<R> a, R s) { return cxmk<R>(a.x * s, a.y * s); }
template <class R> WB_ND Cx<R> cxconj(Cx<R> a) { return cxmk<R>(a.x, -a.y); }
// c + a b
template <class R> WB_ND Cx<R> cxfma(Cx<R> a, Cx<R> b, Cx<R> c) {
  c.x = rfma(a.x, b.x, c.x); c.x = rfma(-a.y, b.y, c.x);
  c.y = rfma(a.x, b.y, c.y); c.y = rfma(a.y, b.x, c.y);
  return c;
}
// c + conj(a) b
template <class R> WB_ND Cx<R> cxfma_conj(Cx<R> a, Cx<R> b, Cx<R> c) {
  c.x = rfma(a.x, b.x, c.x); c.x = rfma(a.y, b.y, c.x);
  c.y = rfma(a.x, b.y, c.y); c.y = rfma(-a.y, b.x, c.y);
  return c;
}
template <class R> WB_ND R cxabs1(Cx<R> a) { return rabs(a.x) + rabs(a.y); }
template <class R> WB_ND R cxabs2(Cx<R> a) { return a.x * a.x + a.y * a.y; }
template <class R> WB_ND R cxabs(Cx<R> a) {
  R ax = rabs(a.x), ay = rabs(a.y);
  R m = rmax(ax, ay);
  if (!(m > RealT<R>::tiny())) return m;     // zero or below the safe range: |a| ~ max part
  R s = R(1.0) / m;
  R u = ax * s, v = ay * s;
  return m * rsqrt_(u * u + v * v);
}
template <class R> WB_ND Cx<R> cxdiv(Cx<R> a, Cx<R> b) {
  if (rabs(b.y) <= rabs(b.x)) {
    R r = b.y / b.x, d = b.x + b.y * r;
    return cxmk<R>((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  R r = b.x / b.y, d = b.y + b.x * r;
  return cxmk<R>((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
template <class R> WB_ND Cx<R> cxinv(Cx<R> b) { return cxdiv(cxone<R>(), b); }
template <class R> WB_ND Cx<R> cxsqrt(Cx<R> z) {
  R x = z.x, y = z.y;
  if (x == R(0.0) && y == R(0.0)) return cxmk<R>(R(0.0), y);
  R t = rsqrt_(R(0.5) * (rabs(x) + cxabs(z)));
  if (!(t > R(0.0))) return cxmk<R>(R(0.0), R(0.0));       // below the representable range
  if (x >= R(0.0)) return cxmk<R>(t, y / (R(2.0) * t));
  R ay = rabs(y);
  return cxmk<R>(ay / (R(2.0) * t), y < R(0.0) ? -t : t);
}
template <class R> WB_ND bool cxfinite(Cx<R> a) { return rfinite(a.x) && rfinite(a.y); }

// conversion between the interleaved-double storage used at the ABI and Cx<R>
template <class R> WB_ND Cx<R> cxfrom(double2 d) { return cxmk<R>(R(d.x), R(d.y)); }
template <class R> WB_ND double2 cxto(Cx<R> c) { double2 d; d.x = rto(c.x); d.y = rto(c.y); return d; }
