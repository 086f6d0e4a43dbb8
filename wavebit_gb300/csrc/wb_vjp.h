// Reverse passes (vector-Jacobian products) of the RCWA raster path's three stages, as host
// drivers over a few batched primitives:
//
//   stage A  assemble_vjp      cotangents of (epx, epy, epz_i)          -> cotangent of the rasters
//   stage B  layer_modes_vjp   cotangents of (w, q, W, V) of each pair  -> cotangent of the slots
//   stage C  smm_vjp           cotangents of the per-order R, T         -> cotangents of W, V, q, d
//
// Reference: the reference differentiates the same path through its array backends:
// rcwa/_engine/modal_gradient.py:56-251 (eigen-solve generator, broadened reciprocal gaps),
// _common/backend.py:1724-1759 (_eig_grad), scattering.py:116-200 (gap waves, S-layer, star),
// :907-994 (efficiencies), factorization.py:289-671 (series, Li's nested rules).
//
// The drivers are templates over an Ops policy (below), so the same code runs on the GPU
// (wb_vjp.cu: the library's GEMM/LU kernels and one generic element-wise kernel) and, in the
// tests, over a plain C++ stand-in of the primitives that checks the index, stride and
// conjugation logic on the CPU. Everything here is FP64 complex (double2), column-major.
//
// Cotangent convention (torch's): for a real loss l and a complex variable z = x + i y the
// cotangent is dl/dx + i dl/dy; a real input's gradient is the real part of its cotangent.
//
// Ops policy:
//   template <class T> T* get(size_t count)          scratch, nullptr when exhausted (see bool ok())
//   void gemm(batch, m, n, k, alpha, A, a_rs, a_cs, a_bs, conjA, B, b_rs, b_cs, b_bs, conjB,
//             beta, C, c_rs, c_cs, c_bs)           C = alpha op(A) op(B) + beta C, element (r, c)
//                                                  of X at X + r * rs + c * cs + batch * bs
//   void getrf(batch, n, A, a_bs, piv, piv_bs, status, st_div)   LU with partial pivoting, lda n;
//                                                  a zero pivot flags status[batch / st_div]
//   void getrs(batch, n, LU, a_bs, piv, piv_bs, B, nrhs, b_bs, trans)  A X = B (0) or A^T X = B (1)
//   template <class F> void each(long long count, F f)           f(i) for every i in [0, count)
#pragma once
#include <cstddef>
#include <cstdint>
#include <cmath>
#include <vector_types.h>

#if defined(__CUDACC__)
#define WBV_HD __host__ __device__ __forceinline__
#define WBV_FN [=] __host__ __device__(long long i)
#else
#define WBV_HD inline
#define WBV_FN [=](long long i)
#endif

namespace wbv {

typedef double2 z;
typedef long long ll;

WBV_HD z mk(double a, double b) { z c; c.x = a; c.y = b; return c; }
WBV_HD z zero() { return mk(0.0, 0.0); }
WBV_HD z add(z a, z b) { return mk(a.x + b.x, a.y + b.y); }
WBV_HD z sub(z a, z b) { return mk(a.x - b.x, a.y - b.y); }
WBV_HD z mul(z a, z b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
WBV_HD z cj(z a) { return mk(a.x, -a.y); }
WBV_HD z sc(z a, double s) { return mk(a.x * s, a.y * s); }
WBV_HD double abs2(z a) { return a.x * a.x + a.y * a.y; }
WBV_HD z dv(z a, z b) {   // Smith's division
  if (fabs(b.y) <= fabs(b.x)) {
    double r = b.y / b.x, d = b.x + b.y * r;
    return mk((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  double r = b.x / b.y, d = b.y + b.x * r;
  return mk((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
WBV_HD z inv(z b) { return dv(mk(1.0, 0.0), b); }
WBV_HD z ex(z a) { double e = exp(a.x); return mk(e * cos(a.y), e * sin(a.y)); }
WBV_HD z delta(ll r, ll c) { return mk(r == c ? 1.0 : 0.0, 0.0); }

// 256-byte granular scratch sizes: the same rounding as the library's arena, so a counting pass
// over carve() gives the exact bytes a chunk needs.
struct Counter {
  size_t bytes = 0;
  template <class T> T* get(size_t count) {
    bytes += (count * sizeof(T) + 255) & ~(size_t)255;
    return nullptr;
  }
};

// Per-solve port vectors (the ports kernel's output): order wavevectors and s/p frame (B, N),
// half-space kz (B, N), gap W/V diagonals and the diagonal interface S blocks (B, 2N), indices (B).
struct Ports {
  const double *kx, *ky, *c, *s;
  const z *kz_top, *kz_bot;
  const z *wg, *vg, *r11, *r12, *r21, *r22, *t11, *t21;
  const z *nt, *nb;
};

// ===================================================================== stage B: layer_modes_vjp
//
// Forward (solve_2d.py:2377-2460, per pair; K = diag(k), real order wavevectors):
//   Omega^2 = [[Ky^2 + (Kx epz Kx - I) epx, Kx epz Ky epy - KxKy], [Ky epz Kx epx - KyKx, Kx^2 + (Ky epz Ky - I) epy]]
//   Omega_R = [[-KxKy, Kx^2 - epy], [epx - Ky^2, KyKx]]
//   w, W = eig(Omega^2);  q = mode_q(w) = +-sqrt(w);  V = Omega_R W diag(1/q)
// Reverse:
//   T = gV diag(conj(1/q));  gW' = gW + Omega_R^H T;  gOmega_R = T W^H (two N x N blocks needed)
//   gq' = gq + conj(-1/q^2) conj(q) colsum(conj(V) o gV);  gw' = gw + conj(1/(2q)) gq'
//   gOmega^2 = W^-H (diag(gw') + F o (W^H gW')) W^H,  F_ij = d_ij / (|d_ij|^2 + eps), d_ij = w_j - w_i,
//     eps = (n u max|w|)^2 (the Lorentzian-broadened reciprocal gap; F_ii = 0). Each mode's scale
//     is left free: the RCWA answers do not depend on it, so no normalisation term enters.
//   gepx = Kx epz^H (Kx G11 + Ky G21) - G11 + gOmega_R21
//   gepy = Ky epz^H (Kx G12 + Ky G22) - G22 - gOmega_R12
//   gepz = Kx (G11 epx^H) Kx + Kx (G12 epy^H) Ky + Ky (G21 epx^H) Kx + Ky (G22 epy^H) Ky
struct LmBufs {
  z *cv, *T, *gWp, *E, *Y, *LU, *U, *GR, *Zb, *Pm, *Q, *gcp, *gwp;
  int* piv;
  double* wmax;
  template <class A> bool carve(A& a, int P, int N) {
    const size_t n = 2 * (size_t)N, n2 = n * n, N2 = (size_t)N * N;
    cv = a.template get<z>(P * 3 * N2);
    T = a.template get<z>(P * n2);
    gWp = a.template get<z>(P * n2);
    E = a.template get<z>(P * n2);
    Y = a.template get<z>(P * n2);
    LU = a.template get<z>(P * n2);
    U = a.template get<z>(P * n2);
    GR = a.template get<z>(P * 2 * N2);
    Zb = a.template get<z>(P * 2 * N2);
    Pm = a.template get<z>(P * 2 * N2);
    Q = a.template get<z>(P * n2);
    gcp = a.template get<z>(P * 3 * N2);
    gwp = a.template get<z>(P * n);
    piv = a.template get<int>(P * n);
    wmax = a.template get<double>(P);
    return cv && T && gWp && E && Y && LU && U && GR && Zb && Pm && Q && gcp && gwp && piv && wmax;
  }
};

inline size_t layer_modes_vjp_bytes(int N, int P) {
  Counter c;
  LmBufs b;
  b.carve(c, P, N);
  return c.bytes;
}

// One chunk of P pairs. Every pointer addresses the chunk's first pair (conv and gconv: the whole
// slot table). gw, gq, gW, gV may be null (zero cotangents). Adds the chunk's slot cotangents to
// gconv (n_conv, 3, N, N).
template <class Ops>
void layer_modes_vjp(Ops& o, const LmBufs& b, int P, int N, int n_conv, const z* conv, const int* pl,
                     const double* kx, const double* ky, const z* w, const z* q, const z* W, const z* V,
                     const z* gw, const z* gq, const z* gW, const z* gV, z* gconv, int32_t* status) {
  const int n = 2 * N;
  const ll n2 = (ll)n * n, N2 = (ll)N * N, N3 = 3 * N2;
  const z one = mk(1, 0), nil = zero();
  z *cv = b.cv, *T = b.T, *gWp = b.gWp, *E = b.E, *Y = b.Y, *LU = b.LU, *U = b.U, *GR = b.GR, *Zb = b.Zb,
    *Pm = b.Pm, *Q = b.Q, *gcp = b.gcp, *gwp = b.gwp;
  double* wmax = b.wmax;
  // the pairs' slots
  o.each((ll)P * N3, WBV_FN { cv[i] = conv[(ll)pl[i / N3] * N3 + i % N3]; });
  // T = gV diag(conj(1/q)); gW' = gW
  o.each((ll)P * n2, WBV_FN {
    const ll p = i / n2, j = (i % n2) / n;
    T[i] = gV ? mul(gV[i], cj(inv(q[p * n + j]))) : nil;
    gWp[i] = gW ? gW[i] : nil;
  });
  // max |w| per pair; gw' per mode
  o.each((ll)P, WBV_FN {
    double m = 0.0;
    for (int j = 0; j < n; ++j) m = fmax(m, sqrt(abs2(w[i * n + j])));
    wmax[i] = fmax(m, 1e-300);
  });
  o.each((ll)P * n, WBV_FN {
    const ll p = i / n, j = i % n;
    const z qj = q[i];
    z giq = nil;
    if (gV)
      for (int r = 0; r < n; ++r) {
        const ll e = p * n2 + r + j * n;
        giq = add(giq, mul(cj(V[e]), gV[e]));
      }
    giq = mul(cj(qj), giq);
    const z iq = inv(qj);
    z gqt = add(gq ? gq[i] : nil, mul(cj(sc(mul(iq, iq), -1.0)), giq));
    gwp[i] = add(gw ? gw[i] : nil, mul(cj(sc(iq, 0.5)), gqt));
  });
  // Omega_R^H T: U1 = epx^H T2, U2 = epy^H T1 (each N x n)
  o.gemm(P, N, n, N, one, cv, N, 1, N3, true, T + N, 1, n, n2, false, nil, U, 1, N, n2);
  o.gemm(P, N, n, N, one, cv + N2, N, 1, N3, true, T, 1, n, n2, false, nil, U + (ll)N * n, 1, N, n2);
  o.each((ll)P * n2, WBV_FN {
    const ll p = i / n2, e = i % n2;
    const int r = (int)(e % n), c = (int)(e / n);
    const z* Tp = T + p * n2;
    const z* Up = U + p * n2;
    z v;
    if (r < N) {
      const double x = kx[p * N + r], y = ky[p * N + r];
      v = add(sub(sc(Tp[r + (ll)c * n], -x * y), sc(Tp[N + r + (ll)c * n], y * y)), Up[r + (ll)c * N]);
    } else {
      const int rr = r - N;
      const double x = kx[p * N + rr], y = ky[p * N + rr];
      v = sub(add(sc(Tp[rr + (ll)c * n], x * x), sc(Tp[r + (ll)c * n], x * y)), Up[(ll)N * n + rr + (ll)c * N]);
    }
    gWp[i] = add(gWp[i], v);
  });
  // gOmega_R21 = T2 W1^H, gOmega_R12 = T1 W2^H (N x N each)
  o.gemm(P, N, N, n, one, T + N, 1, n, n2, false, W, n, 1, n2, true, nil, GR, 1, N, 2 * N2);
  o.gemm(P, N, N, n, one, T, 1, n, n2, false, W + N, n, 1, n2, true, nil, GR + N2, 1, N, 2 * N2);
  // E = W^H gW'; then conj(M) = conj(diag(gw') + F o E) in place
  o.gemm(P, n, n, n, one, W, n, 1, n2, true, gWp, 1, n, n2, false, nil, E, 1, n, n2);
  o.each((ll)P * n2, WBV_FN {
    const ll p = i / n2, e = i % n2;
    const int r = (int)(e % n), c = (int)(e / n);
    if (r == c) {
      E[i] = cj(gwp[p * n + r]);
      return;
    }
    const z d = sub(w[p * n + c], w[p * n + r]);
    const double eb = (double)n * 2.220446049250313e-16 * wmax[p];
    const z F = sc(d, 1.0 / (abs2(d) + eb * eb));
    E[i] = cj(mul(F, E[i]));
  });
  // conj(M W^H) = conj(M) W^T; W^T X = conj(M W^H) gives X = conj(W^-H M W^H) = conj(gOmega^2)
  o.gemm(P, n, n, n, one, E, 1, n, n2, false, W, n, 1, n2, false, nil, Y, 1, n, n2);
  o.each((ll)P * n2, WBV_FN { LU[i] = W[i]; });
  o.getrf(P, n, LU, n2, b.piv, n, status, 1);
  o.getrs(P, n, LU, n2, b.piv, n, Y, n, n2, 1);
  o.each((ll)P * n2, WBV_FN { Y[i] = cj(Y[i]); });          // Y = G = gOmega^2
  // Zb = [Kx G11 + Ky G21, Kx G12 + Ky G22] (N x 2N); Pm = epz^H Zb
  o.each((ll)P * 2 * N2, WBV_FN {
    const ll p = i / (2 * N2), e = i % (2 * N2);
    const int r = (int)(e % N), c = (int)(e / N);
    const z* G = Y + p * n2;
    Zb[i] = add(sc(G[r + (ll)c * n], kx[p * N + r]), sc(G[N + r + (ll)c * n], ky[p * N + r]));
  });
  o.gemm(P, N, 2 * N, N, one, cv + 2 * N2, N, 1, N3, true, Zb, 1, N, 2 * N2, false, nil, Pm, 1, N, 2 * N2);
  // Q1 = [G11; G21] epx^H, Q2 = [G12; G22] epy^H (n x N each)
  o.gemm(P, n, N, N, one, Y, 1, n, n2, false, cv, N, 1, N3, true, nil, Q, 1, n, n2);
  o.gemm(P, n, N, N, one, Y + (ll)N * n, 1, n, n2, false, cv + N2, N, 1, N3, true, nil, Q + (ll)N * n, 1, n, n2);
  o.each((ll)P * N2, WBV_FN {
    const ll p = i / N2, e = i % N2;
    const int r = (int)(e % N), c = (int)(e / N);
    const z* G = Y + p * n2;
    const z* Pp = Pm + p * 2 * N2;
    const z* Gr = GR + p * 2 * N2;
    const z* Q1 = Q + p * n2;
    const z* Q2 = Q1 + (ll)N * n;
    const double xr = kx[p * N + r], yr = ky[p * N + r], xc = kx[p * N + c], yc = ky[p * N + c];
    z* out = gcp + p * N3;
    out[e] = add(sub(sc(Pp[e], xr), G[r + (ll)c * n]), Gr[e]);
    out[N2 + e] = sub(sub(sc(Pp[N2 + e], yr), G[N + r + (ll)(N + c) * n]), Gr[N2 + e]);
    const z top = add(sc(Q1[r + (ll)c * n], xc), sc(Q2[r + (ll)c * n], yc));
    const z bot = add(sc(Q1[N + r + (ll)c * n], xc), sc(Q2[N + r + (ll)c * n], yc));
    out[2 * N2 + e] = add(sc(top, xr), sc(bot, yr));
  });
  // every slot gathers the chunk's pairs that read it (a fixed order: deterministic sums)
  o.each((ll)n_conv * N3, WBV_FN {
    const ll c = i / N3, e = i % N3;
    z acc = nil;
    for (int p = 0; p < P; ++p)
      if (pl[p] == c) acc = add(acc, gcp[(ll)p * N3 + e]);
    gconv[i] = add(gconv[i], acc);
  });
}

// ===================================================================== stage C: smm_vjp
//
// Forward (the cascade of the stage-C kernels, scattering.py:116-200, with the efficiencies of
// :907-994), per solve, layers l = 0 (entry face) .. L-1, modes rotated to the s/p basis:
//   bW = [c W2 - s W1; c W1 + s W2], bV = [c V1 + s V2; c V2 - s V1],  X = exp(-k0 d q)
//   R_L = diag(t11); for l = L-1 .. 0:
//     P1 = bW^-1 diag(wg)(I + R_{l+1}), P2 = bV^-1 diag(vg)(I - R_{l+1}), M = P1 + P2,
//     rb = (P1 - P2) M^-1, rt = X rb X, X1 = (I - rt) bW^-1, X2 = (I + rt) bV^-1,
//     A = X1 diag(wg) + X2 diag(vg), R_l = A^-1 (X2 diag(vg) - X1 diag(wg))
//   g_0 = (I - diag(r22) R_0)^-1 diag(r21) C, cref = diag(r11) C + diag(r12) R_0 g_0
//   g_{l+1} = M_l^-1 X (bW^-1 diag(wg)(g_l + R_l g_l) + bV^-1 diag(vg)(g_l - R_l g_l)),  ctrn = diag(t21) g_L
//   R[col, i] = (|cref_i|^2 Re kz_top,i + |cref_N+i|^2 Re(kz_top,i / eps_top)) / den_col, T likewise
// The reverse walks the top-down pass backwards, then the reflection recursion top layer first.
struct SmmBufs {
  z *LW, *LV, *X, *P1, *P2, *Mk, *RB, *X1, *X2, *Ak, *Rk, *gM, *gR;   // per pair (Rk: L + 1 per solve)
  z *G0, *S1, *S2, *S3, *S4;                                          // per solve, n x n
  z *Cin, *gv, *hv, *b1, *b2, *cref, *ctrn, *GG, *GE, *GB, *GA1, *GA2, *GL, *GH, *gX;
  int *pivW, *pivV, *pivM, *pivA, *pivG;
  template <class A> bool carve(A& a, int Bc, int L, int N) {
    const size_t n = 2 * (size_t)N, n2 = n * n, P = (size_t)Bc * L, v3 = 3 * n;
    LW = a.template get<z>(P * n2); LV = a.template get<z>(P * n2);
    X = a.template get<z>(P * n);
    P1 = a.template get<z>(P * n2); P2 = a.template get<z>(P * n2);
    Mk = a.template get<z>(P * n2); RB = a.template get<z>(P * n2);
    X1 = a.template get<z>(P * n2); X2 = a.template get<z>(P * n2);
    Ak = a.template get<z>(P * n2);
    Rk = a.template get<z>((P + Bc) * n2);
    gM = a.template get<z>(P * n2); gR = a.template get<z>(P * n2);
    G0 = a.template get<z>(Bc * n2);
    S1 = a.template get<z>(Bc * n2); S2 = a.template get<z>(Bc * n2);
    S3 = a.template get<z>(Bc * n2); S4 = a.template get<z>(Bc * n2);
    Cin = a.template get<z>(Bc * v3);
    gv = a.template get<z>((P + Bc) * v3);
    hv = a.template get<z>(P * v3);
    b1 = a.template get<z>(P * v3); b2 = a.template get<z>(P * v3);
    cref = a.template get<z>(Bc * v3); ctrn = a.template get<z>(Bc * v3);
    GG = a.template get<z>(Bc * v3); GE = a.template get<z>(Bc * v3); GB = a.template get<z>(Bc * v3);
    GA1 = a.template get<z>(Bc * v3); GA2 = a.template get<z>(Bc * v3);
    GL = a.template get<z>(Bc * v3); GH = a.template get<z>(Bc * v3);
    gX = a.template get<z>(P * n);
    pivW = a.template get<int>(P * n); pivV = a.template get<int>(P * n);
    pivM = a.template get<int>(P * n); pivA = a.template get<int>(P * n);
    pivG = a.template get<int>(Bc * n);
    return LW && LV && X && P1 && P2 && Mk && RB && X1 && X2 && Ak && Rk && gM && gR && G0 && S1 && S2 && S3 &&
           S4 && Cin && gv && hv && b1 && b2 && cref && ctrn && GG && GE && GB && GA1 && GA2 && GL && GH && gX &&
           pivW && pivV && pivM && pivA && pivG;
  }
};

inline size_t smm_vjp_bytes(int N, int L, int Bc) {
  Counter c;
  SmmBufs b;
  b.carve(c, Bc, L, N);
  return c.bytes;
}

// One chunk of Bc solves (pairs p = b * L + l). Every per-solve / per-pair pointer addresses the
// chunk's first solve / pair; pv holds the chunk's port vectors. gR, gT (Bc, 3, N) may be null.
// Writes gW, gV (pairs, n, n) and gq (pairs, n) and g_thick (pairs) (overwritten).
template <class Ops>
void smm_vjp(Ops& o, const SmmBufs& b, int Bc, int L, int N, const Ports& pv, const z* W, const z* V, const z* q,
             const double* thick, const double* wavelength, const z* eps_top, const z* eps_bot, const z* pol,
             const double* gRin, const double* gTin, z* gW, z* gV, z* gq, double* g_thick, int32_t* status) {
  const int n = 2 * N, P = Bc * L;
  const ll n2 = (ll)n * n, v3 = 3 * (ll)n, Ln2 = (ll)L * n2, Ln = (ll)L * n, Rs = (ll)(L + 1) * n2;
  const ll gs = (ll)(L + 1) * v3, Lv3 = (ll)L * v3;
  const z one = mk(1, 0), mone = mk(-1, 0), nil = zero();
  z *LW = b.LW, *LV = b.LV, *X = b.X, *P1 = b.P1, *P2 = b.P2, *Mk = b.Mk, *RB = b.RB, *X1 = b.X1, *X2 = b.X2,
    *Ak = b.Ak, *Rk = b.Rk, *gM = b.gM, *gR = b.gR, *G0 = b.G0, *S1 = b.S1, *S2 = b.S2, *S3 = b.S3, *S4 = b.S4,
    *Cin = b.Cin, *gv = b.gv, *hv = b.hv, *b1 = b.b1, *b2 = b.b2, *cref = b.cref, *ctrn = b.ctrn, *gX = b.gX;
  const Ports P_ = pv;
  // ---- forward with its tape
  o.each((ll)P * N * n, WBV_FN {
    const ll p = i / ((ll)N * n), e = i % ((ll)N * n);
    const int r = (int)(e % N), c = (int)(e / N);
    const ll bs = p / L;
    const double cc = P_.c[bs * N + r], ss = P_.s[bs * N + r];
    const ll o1 = p * n2 + r + (ll)c * n, o2 = o1 + N;
    const z w1 = W[o1], w2 = W[o2], v1 = V[o1], v2 = V[o2];
    LW[o1] = sub(sc(w2, cc), sc(w1, ss)); LW[o2] = add(sc(w1, cc), sc(w2, ss));
    LV[o1] = add(sc(v1, cc), sc(v2, ss)); LV[o2] = sub(sc(v2, cc), sc(v1, ss));
  });
  o.each((ll)P * n, WBV_FN {
    const ll p = i / n;
    const double k0 = 2.0 * 3.141592653589793 / wavelength[p / L];
    X[i] = ex(sc(q[i], -k0 * thick[p]));
    gX[i] = zero();
  });
  o.getrf(P, n, LW, n2, b.pivW, n, status, L);
  o.getrf(P, n, LV, n2, b.pivV, n, status, L);
  o.each((ll)Bc * n2, WBV_FN {
    const ll bs = i / n2, e = i % n2;
    const int r = (int)(e % n), c = (int)(e / n);
    Rk[bs * Rs + (ll)L * n2 + e] = r == c ? P_.t11[bs * n + r] : zero();
  });
  for (int l = L - 1; l >= 0; --l) {
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const z Rb = Rk[bs * Rs + (ll)(l + 1) * n2 + e], d = delta(r, c);
      const ll p = bs * L + l;
      P1[p * n2 + e] = mul(P_.wg[bs * n + r], add(d, Rb));
      P2[p * n2 + e] = mul(P_.vg[bs * n + r], sub(d, Rb));
    });
    o.getrs(Bc, n, LW + l * n2, Ln2, b.pivW + l * n, Ln, P1 + l * n2, n, Ln2, 0);
    o.getrs(Bc, n, LV + l * n2, Ln2, b.pivV + l * n, Ln, P2 + l * n2, n, Ln2, 0);
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const ll p = bs * L + l;
      const z a = P1[p * n2 + e], d = P2[p * n2 + e];
      Mk[p * n2 + e] = add(a, d);
      S1[bs * n2 + c + (ll)r * n] = sub(a, d);                  // (P1 - P2)^T
    });
    o.getrf(Bc, n, Mk + l * n2, Ln2, b.pivM + l * n, Ln, status, 1);
    o.getrs(Bc, n, Mk + l * n2, Ln2, b.pivM + l * n, Ln, S1, n, n2, 1);     // rb^T = M^-T (P1 - P2)^T
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const ll p = bs * L + l;
      const z rbv = S1[bs * n2 + c + (ll)r * n];
      RB[p * n2 + e] = rbv;
      const z rt = mul(mul(X[p * n + r], rbv), X[p * n + c]), d = delta(r, c);
      S2[bs * n2 + c + (ll)r * n] = sub(d, rt);                 // (I - rt)^T
      S3[bs * n2 + c + (ll)r * n] = add(d, rt);                 // (I + rt)^T
    });
    o.getrs(Bc, n, LW + l * n2, Ln2, b.pivW + l * n, Ln, S2, n, n2, 1);     // X1^T
    o.getrs(Bc, n, LV + l * n2, Ln2, b.pivV + l * n, Ln, S3, n, n2, 1);     // X2^T
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const ll p = bs * L + l;
      const z x1 = S2[bs * n2 + c + (ll)r * n], x2 = S3[bs * n2 + c + (ll)r * n];
      X1[p * n2 + e] = x1; X2[p * n2 + e] = x2;
      const z a1 = mul(x1, P_.wg[bs * n + c]), a2 = mul(x2, P_.vg[bs * n + c]);
      Ak[p * n2 + e] = add(a1, a2);
      Rk[bs * Rs + (ll)l * n2 + e] = sub(a2, a1);
    });
    o.getrf(Bc, n, Ak + l * n2, Ln2, b.pivA + l * n, Ln, status, 1);
    o.getrs(Bc, n, Ak + l * n2, Ln2, b.pivA + l * n, Ln, Rk + l * n2, n, Rs, 0);
  }
  // top-down pass for the three incidence columns (given polarization, pure s, pure p)
  o.each((ll)Bc * n2, WBV_FN {
    const ll bs = i / n2, e = i % n2;
    const int r = (int)(e % n), c = (int)(e / n);
    G0[i] = sub(delta(r, c), mul(P_.r22[bs * n + r], Rk[bs * Rs + e]));
  });
  o.getrf(Bc, n, G0, n2, b.pivG, n, status, 1);
  o.each((ll)Bc * v3, WBV_FN {
    const ll bs = i / v3, e = i % v3;
    const int r = (int)(e % n), col = (int)(e / n), spec = N / 2;
    z as, ap;
    if (col == 0) { as = pol[2 * bs]; ap = pol[2 * bs + 1]; }
    else if (col == 1) { as = mk(1.0, 0.0); ap = mk(6.123233995736766e-17, 0.0); }
    else { as = zero(); ap = mk(1.0, 0.0); }
    z v = zero();
    if (r == spec) v = as;
    else if (r == N + spec) v = mul(mul(mk(0.0, -1.0), P_.nt[bs]), ap);
    Cin[i] = v;
    gv[bs * gs + e] = mul(P_.r21[bs * n + r], v);
  });
  o.getrs(Bc, n, G0, n2, b.pivG, n, gv, 3, gs, 0);                          // g_0
  for (int l = 0; l < L; ++l) {
    o.gemm(Bc, n, 3, n, one, Rk + l * n2, 1, n, Rs, false, gv + l * v3, 1, n, gs, false, nil, hv + l * v3, 1, n,
           Lv3);                                                            // h_l = R_l g_l
    if (l == 0)
      o.each((ll)Bc * v3, WBV_FN {
        const ll bs = i / v3, e = i % v3;
        const int r = (int)(e % n);
        cref[i] = add(mul(P_.r11[bs * n + r], Cin[i]), mul(P_.r12[bs * n + r], hv[bs * Lv3 + e]));
      });
    o.each((ll)Bc * v3, WBV_FN {
      const ll bs = i / v3, e = i % v3;
      const int r = (int)(e % n);
      const z g = gv[bs * gs + l * v3 + e], h = hv[bs * Lv3 + l * v3 + e];
      b1[bs * Lv3 + l * v3 + e] = mul(P_.wg[bs * n + r], add(g, h));
      b2[bs * Lv3 + l * v3 + e] = mul(P_.vg[bs * n + r], sub(g, h));
    });
    o.getrs(Bc, n, LW + l * n2, Ln2, b.pivW + l * n, Ln, b1 + l * v3, 3, Lv3, 0);
    o.getrs(Bc, n, LV + l * n2, Ln2, b.pivV + l * n, Ln, b2 + l * v3, 3, Lv3, 0);
    o.each((ll)Bc * v3, WBV_FN {
      const ll bs = i / v3, e = i % v3;
      const int r = (int)(e % n);
      const ll o3 = bs * Lv3 + l * v3 + e;
      gv[bs * gs + (l + 1) * v3 + e] = mul(X[(bs * L + l) * n + r], add(b1[o3], b2[o3]));
    });
    o.getrs(Bc, n, Mk + l * n2, Ln2, b.pivM + l * n, Ln, gv + (l + 1) * v3, 3, gs, 0);
  }
  // ---- efficiencies' cotangents -> gcref (GH), gctrn (GG)
  z *GG = b.GG, *GE = b.GE, *GB = b.GB, *GA1 = b.GA1, *GA2 = b.GA2, *GL = b.GL, *GH = b.GH;
  o.each((ll)Bc * v3, WBV_FN {
    const ll bs = i / v3, e = i % v3;
    const int r = (int)(e % n), col = (int)(e / n), half = r / N, ii = r % N;
    ctrn[i] = mul(P_.t21[bs * n + r], gv[bs * gs + (ll)L * v3 + e]);
    const z et = eps_top[bs], eb = eps_bot[bs];
    const z kzs = P_.kz_top[bs * N + N / 2];
    const double s_power = kzs.x, p_power = abs2(P_.nt[bs]) * dv(kzs, et).x;
    double den = col == 1 ? s_power : p_power;
    if (col == 0) den = abs2(pol[2 * bs]) * s_power + abs2(pol[2 * bs + 1]) * p_power;
    const z kzt = P_.kz_top[bs * N + ii], kzb = P_.kz_bot[bs * N + ii];
    const double wr = (half ? dv(kzt, et).x : kzt.x) / den;
    const double wt = (half ? dv(kzb, eb).x : kzb.x) / den;
    const double gr = gRin ? gRin[(bs * 3 + col) * N + ii] : 0.0;
    const double gt = gTin ? gTin[(bs * 3 + col) * N + ii] : 0.0;
    GH[i] = sc(cref[i], 2.0 * gr * wr);                          // gcref, kept for the end
    GG[i] = mul(cj(P_.t21[bs * n + r]), sc(ctrn[i], 2.0 * gt * wt));
  });
  // gW, gV accumulate the rotated modes' cotangents first
  o.each((ll)P * n2, WBV_FN { gW[i] = zero(); gV[i] = zero(); });
  // gcref is needed after the loop; move it to GB's slot at the end. Keep it in cref's buffer.
  o.each((ll)Bc * v3, WBV_FN { cref[i] = GH[i]; });
  // ---- reverse of the top-down pass
  for (int l = L - 1; l >= 0; --l) {
    // ge = M^-H gg  (M^H x = y  <=>  M^T conj(x) = conj(y))
    o.each((ll)Bc * v3, WBV_FN { GE[i] = cj(GG[i]); });
    o.getrs(Bc, n, Mk + l * n2, Ln2, b.pivM + l * n, Ln, GE, 3, v3, 1);
    o.each((ll)Bc * v3, WBV_FN { GE[i] = cj(GE[i]); });
    // gM_l = -ge g_{l+1}^H
    o.gemm(Bc, n, n, 3, mone, GE, 1, n, v3, false, gv + (l + 1) * v3, n, 1, gs, true, nil, gM + l * n2, 1, n, Ln2);
    // gX_l += sum_col conj(b1 + b2) o ge;  gb = conj(X) o ge
    o.each((ll)Bc * n, WBV_FN {
      const ll bs = i / n;
      const int r = (int)(i % n);
      z acc = zero();
      for (int col = 0; col < 3; ++col) {
        const ll o3 = bs * Lv3 + l * v3 + (ll)col * n + r;
        acc = add(acc, mul(cj(add(b1[o3], b2[o3])), GE[bs * v3 + (ll)col * n + r]));
      }
      const ll px = (bs * L + l) * n + r;
      gX[px] = add(gX[px], acc);
      for (int col = 0; col < 3; ++col) {
        const ll o3 = bs * v3 + (ll)col * n + r;
        GB[o3] = mul(cj(X[px]), GE[o3]);
        GA1[o3] = cj(GB[o3]);
        GA2[o3] = cj(GB[o3]);
      }
    });
    // ga1 = bW^-H gb, ga2 = bV^-H gb
    o.getrs(Bc, n, LW + l * n2, Ln2, b.pivW + l * n, Ln, GA1, 3, v3, 1);
    o.getrs(Bc, n, LV + l * n2, Ln2, b.pivV + l * n, Ln, GA2, 3, v3, 1);
    o.each((ll)Bc * v3, WBV_FN { GA1[i] = cj(GA1[i]); GA2[i] = cj(GA2[i]); });
    // gbW_l -= ga1 b1^H, gbV_l -= ga2 b2^H
    o.gemm(Bc, n, n, 3, mone, GA1, 1, n, v3, false, b1 + l * v3, n, 1, Lv3, true, one, gW + l * n2, 1, n, Ln2);
    o.gemm(Bc, n, n, 3, mone, GA2, 1, n, v3, false, b2 + l * v3, n, 1, Lv3, true, one, gV + l * n2, 1, n, Ln2);
    o.each((ll)Bc * v3, WBV_FN {
      const ll bs = i / v3;
      const int r = (int)((i % v3) % n);
      const z a = mul(cj(P_.wg[bs * n + r]), GA1[i]), c = mul(cj(P_.vg[bs * n + r]), GA2[i]);
      GL[i] = add(a, c);
      GH[i] = sub(a, c);
    });
    if (l > 0) {
      // h_l = R_l g_l: gR_l = gh g_l^H, gl += R_l^H gh
      o.gemm(Bc, n, n, 3, one, GH, 1, n, v3, false, gv + l * v3, n, 1, gs, true, nil, gR + l * n2, 1, n, Ln2);
      o.gemm(Bc, n, 3, n, one, Rk + l * n2, n, 1, Rs, true, GH, 1, n, v3, false, one, GL, 1, n, v3);
    }
    z* t = GG; GG = GL; GL = t;
  }
  // cref = r11 C + r12 h_0: gh_0 += conj(r12) gcref; gR_0 = gh_0 g_0^H; gg_0 = gg + R_0^H gh_0
  o.each((ll)Bc * v3, WBV_FN {
    const ll bs = i / v3;
    const int r = (int)((i % v3) % n);
    GH[i] = add(GH[i], mul(cj(P_.r12[bs * n + r]), cref[i]));
  });
  o.gemm(Bc, n, n, 3, one, GH, 1, n, v3, false, gv, n, 1, gs, true, nil, gR, 1, n, Ln2);
  o.gemm(Bc, n, 3, n, one, Rk, n, 1, Rs, true, GH, 1, n, v3, false, one, GG, 1, n, v3);
  // g_0 = G0^-1 r21 C: gk = G0^-H gg_0; gR_0 += conj(r22) o (gk g_0^H)
  o.each((ll)Bc * v3, WBV_FN { GE[i] = cj(GG[i]); });
  o.getrs(Bc, n, G0, n2, b.pivG, n, GE, 3, v3, 1);
  o.each((ll)Bc * v3, WBV_FN { GE[i] = cj(GE[i]); });
  o.gemm(Bc, n, n, 3, one, GE, 1, n, v3, false, gv, n, 1, gs, true, nil, S1, 1, n, n2);
  o.each((ll)Bc * n2, WBV_FN {
    const ll bs = i / n2, e = i % n2;
    const int r = (int)(e % n);
    gR[bs * Ln2 + e] = add(gR[bs * Ln2 + e], mul(cj(P_.r22[bs * n + r]), S1[i]));
  });
  // ---- reverse of the reflection recursion, top layer first
  for (int l = 0; l < L; ++l) {
    // gBt = A^-H gR_l (S1); gA = -gBt R_l^H (S2)
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      S1[i] = cj(gR[bs * Ln2 + l * n2 + e]);
    });
    o.getrs(Bc, n, Ak + l * n2, Ln2, b.pivA + l * n, Ln, S1, n, n2, 1);
    o.each((ll)Bc * n2, WBV_FN { S1[i] = cj(S1[i]); });
    o.gemm(Bc, n, n, n, mone, S1, 1, n, n2, false, Rk + l * n2, n, 1, Rs, true, nil, S2, 1, n, n2);
    // gX1 = (gA - gBt) diag(conj(wg)), gX2 = (gA + gBt) diag(conj(vg)); S3 = gX1^H, S4 = gX2^H
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const z gbt = S1[i], ga = S2[i];
      S3[bs * n2 + c + (ll)r * n] = mul(cj(sub(ga, gbt)), P_.wg[bs * n + c]);
      S4[bs * n2 + c + (ll)r * n] = mul(cj(add(ga, gbt)), P_.vg[bs * n + c]);
    });
    // K1 = gX1 bW^-H  <=>  K1^H = bW^-1 gX1^H  (likewise K2)
    o.getrs(Bc, n, LW + l * n2, Ln2, b.pivW + l * n, Ln, S3, n, n2, 0);
    o.getrs(Bc, n, LV + l * n2, Ln2, b.pivV + l * n, Ln, S4, n, n2, 0);
    // gbW_l -= X1^H K1, gbV_l -= X2^H K2
    o.gemm(Bc, n, n, n, mone, X1 + l * n2, n, 1, Ln2, true, S3, n, 1, n2, true, one, gW + l * n2, 1, n, Ln2);
    o.gemm(Bc, n, n, n, mone, X2 + l * n2, n, 1, Ln2, true, S4, n, 1, n2, true, one, gV + l * n2, 1, n, Ln2);
    // grt = K2 - K1 (S1); gX_l from rt = X rb X; grb = conj(X) grt conj(X) (S2)
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const ll t = bs * n2 + c + (ll)r * n;
      S1[i] = sub(cj(S4[t]), cj(S3[t]));
    });
    o.each((ll)Bc * n, WBV_FN {
      const ll bs = i / n;
      const int m = (int)(i % n);
      const ll p = bs * L + l;
      const z* rb = RB + p * n2;
      const z* Xp = X + p * n;
      const z* grt = S1 + bs * n2;
      z acc = zero();
      for (int j = 0; j < n; ++j) {
        acc = add(acc, mul(grt[m + (ll)j * n], cj(mul(rb[m + (ll)j * n], Xp[j]))));
        acc = add(acc, mul(grt[j + (ll)m * n], cj(mul(Xp[j], rb[j + (ll)m * n]))));
      }
      gX[p * n + m] = add(gX[p * n + m], acc);
    });
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const ll p = bs * L + l;
      S2[i] = mul(mul(cj(X[p * n + r]), S1[i]), cj(X[p * n + c]));
      S3[bs * n2 + c + (ll)r * n] = cj(S2[i]);                  // grb^H
    });
    // gNm = grb M^-H  <=>  gNm^H = M^-1 grb^H (S3); gM_l += -rb^H gNm
    o.getrs(Bc, n, Mk + l * n2, Ln2, b.pivM + l * n, Ln, S3, n, n2, 0);
    o.gemm(Bc, n, n, n, mone, RB + l * n2, n, 1, Ln2, true, S3, n, 1, n2, true, one, gM + l * n2, 1, n, Ln2);
    // gP1 = gM + gNm (S1), gP2 = gM - gNm (S2), as conjugates for the H-solves
    o.each((ll)Bc * n2, WBV_FN {
      const ll bs = i / n2, e = i % n2;
      const int r = (int)(e % n), c = (int)(e / n);
      const z gnm = cj(S3[bs * n2 + c + (ll)r * n]), gm = gM[bs * Ln2 + l * n2 + e];
      S1[i] = cj(add(gm, gnm));
      S2[i] = cj(sub(gm, gnm));
    });
    // gU1 = bW^-H gP1, gU2 = bV^-H gP2
    o.getrs(Bc, n, LW + l * n2, Ln2, b.pivW + l * n, Ln, S1, n, n2, 1);
    o.getrs(Bc, n, LV + l * n2, Ln2, b.pivV + l * n, Ln, S2, n, n2, 1);
    o.each((ll)Bc * n2, WBV_FN { S1[i] = cj(S1[i]); S2[i] = cj(S2[i]); });
    // gbW_l -= gU1 P1^H, gbV_l -= gU2 P2^H
    o.gemm(Bc, n, n, n, mone, S1, 1, n, n2, false, P1 + l * n2, n, 1, Ln2, true, one, gW + l * n2, 1, n, Ln2);
    o.gemm(Bc, n, n, n, mone, S2, 1, n, n2, false, P2 + l * n2, n, 1, Ln2, true, one, gV + l * n2, 1, n, Ln2);
    // U1 = wg (I + R_{l+1}), U2 = vg (I - R_{l+1}): gR_{l+1} += conj(wg) gU1 - conj(vg) gU2
    if (l + 1 < L)
      o.each((ll)Bc * n2, WBV_FN {
        const ll bs = i / n2, e = i % n2;
        const int r = (int)(e % n);
        const ll t = bs * Ln2 + (ll)(l + 1) * n2 + e;
        gR[t] = add(gR[t], sub(mul(cj(P_.wg[bs * n + r]), S1[i]), mul(cj(P_.vg[bs * n + r]), S2[i])));
      });
  }
  // ---- back to the Cartesian modes; q and d through X = exp(-k0 d q)
  o.each((ll)P * N * n, WBV_FN {
    const ll p = i / ((ll)N * n), e = i % ((ll)N * n);
    const int r = (int)(e % N), c = (int)(e / N);
    const ll bs = p / L;
    const double cc = P_.c[bs * N + r], ss = P_.s[bs * N + r];
    const ll o1 = p * n2 + r + (ll)c * n, o2 = o1 + N;
    const z gt = gW[o1], gb = gW[o2], vt = gV[o1], vb = gV[o2];
    gW[o1] = sub(sc(gb, cc), sc(gt, ss)); gW[o2] = add(sc(gt, cc), sc(gb, ss));
    gV[o1] = sub(sc(vt, cc), sc(vb, ss)); gV[o2] = add(sc(vt, ss), sc(vb, cc));
  });
  o.each((ll)P, WBV_FN {
    const double k0 = 2.0 * 3.141592653589793 / wavelength[i / L], d = thick[i];
    double acc = 0.0;
    for (int j = 0; j < n; ++j) {
      const ll t = i * n + j;
      gq[t] = mul(cj(sc(X[t], -k0 * d)), gX[t]);
      acc += mul(cj(sc(mul(q[t], X[t]), -k0)), gX[t]).x;
    }
    g_thick[i] = acc;
  });
}

// ===================================================================== stage A: assemble_vjp
//
// Forward (factorization.py:289-671, sampled coefficients, fixed nesting), per layer:
//   epx = inv(T_u([T_v(eps)]^-1)),  epy = T_u([T_v(1/eps)]^-1),  epz_i = inv(T_uv(eps))
// where T_v(a) is the (2hv+1)^2 Toeplitz matrix of the exact staircase series of one raster
// column (series S_v: (4hv+1) x ny, S[k, j] = sinc(k/m) e^{-i pi k/m} e^{-2 pi i k j/m} / m), the
// inverse is taken per column, and T_u applies the series along x to every entry and lays the
// result out as a block-Toeplitz N x N matrix (row r nu + m, column c nu + m').
// Reverse: an inverse Y gives -Y^H G Y^H; a Toeplitz layout gives the sums of G over its
// diagonals; a series S gives S^H; 1/eps gives conj(-1/eps^2).
struct AsmBufs {
  z *Su, *Sv, *rec, *cv, *Tv, *inner, *T1, *GP, *gcu, *gent, *gtmp, *gTv, *gcv, *gc2, *tm, *ginv;
  int* piv;
  template <class A> bool carve(A& a, int L, int ny, int nx, int hu, int hv) {
    const size_t nu = 2 * hu + 1, nv = 2 * hv + 1, N = nu * nv, nku = 4 * hu + 1, nkv = 4 * hv + 1;
    const size_t plane = (size_t)ny * nx, G = 2 * (size_t)L;
    Su = a.template get<z>(nku * nx);
    Sv = a.template get<z>(nkv * ny);
    rec = a.template get<z>(L * plane);
    cv = a.template get<z>(G * nkv * nx);
    Tv = a.template get<z>(G * nx * nv * nv);
    inner = a.template get<z>(G * nx * nv * nv);
    T1 = a.template get<z>(2 * L * N * N);
    GP = a.template get<z>(3 * L * N * N);
    gcu = a.template get<z>(G * nv * nv * nku);
    gent = a.template get<z>(G * nx * nv * nv);
    gtmp = a.template get<z>(G * nx * nv * nv);
    gTv = a.template get<z>(G * nx * nv * nv);
    gcv = a.template get<z>(G * nx * nkv);
    gc2 = a.template get<z>(L * nkv * nku);
    tm = a.template get<z>(L * nkv * nx);
    ginv = a.template get<z>(L * plane);
    piv = a.template get<int>(G * nx * nv);
    return Su && Sv && rec && cv && Tv && inner && T1 && GP && gcu && gent && gtmp && gTv && gcv && gc2 && tm &&
           ginv && piv;
  }
};

inline size_t assemble_vjp_bytes(int L, int ny, int nx, int hu, int hv) {
  Counter c;
  AsmBufs b;
  b.carve(c, L, ny, nx, hu, hv);
  return c.bytes;
}

// S[k + 2h, j] (column-major (4h+1) x m) of the staircase series of an m-point line
WBV_HD z series_entry(int kk, int j, int m, int h) {
  const int k = kk - 2 * h;
  const long long pm = (((long long)k * j) % m + m) % m;
  const double ang = -2.0 * 3.141592653589793 * (double)pm / (double)m;
  z v = mk(cos(ang) / m, sin(ang) / m);
  if (k != 0) {
    const double t = (double)k / (double)m;
    const double sinc = sin(3.141592653589793 * t) / (3.141592653589793 * t);
    v = mul(v, mk(sinc * cos(-3.141592653589793 * t), sinc * sin(-3.141592653589793 * t)));
  }
  return v;
}

// eps (L, ny, nx) row-major; epx, epz_i (L, N, N) the forward's outputs; g_* (L, N, N) cotangents
// (any may be null); g_eps (L, ny, nx) overwritten.
template <class Ops>
void assemble_vjp(Ops& o, const AsmBufs& b, int L, int ny, int nx, int hu, int hv, const z* eps, const z* epx,
                  const z* epz, const z* gepx, const z* gepy, const z* gepz, z* g_eps, int32_t* status) {
  const int nu = 2 * hu + 1, nv = 2 * hv + 1, N = nu * nv, nku = 4 * hu + 1, nkv = 4 * hv + 1;
  const ll N2 = (ll)N * N, plane = (ll)ny * nx, nv2 = (ll)nv * nv, G = 2 * (ll)L;
  const z one = mk(1, 0), mone = mk(-1, 0), nil = zero();
  z *Su = b.Su, *Sv = b.Sv, *rec = b.rec, *cv = b.cv, *Tv = b.Tv, *inner = b.inner, *T1 = b.T1, *GP = b.GP,
    *gcu = b.gcu, *gent = b.gent, *gtmp = b.gtmp, *gTv = b.gTv, *gcv = b.gcv, *gc2 = b.gc2, *tm = b.tm, *ginv = b.ginv;
  o.each((ll)nku * nx, WBV_FN { Su[i] = series_entry((int)(i % nku), (int)(i / nku), nx, hu); });
  o.each((ll)nkv * ny, WBV_FN { Sv[i] = series_entry((int)(i % nkv), (int)(i / nkv), ny, hv); });
  o.each((ll)L * plane, WBV_FN { rec[i] = inv(eps[i]); });
  // column series of eps (groups 0..L-1) and 1/eps (L..2L-1): cv[g] (nkv x nx) = Sv a_g
  o.gemm(L, nkv, nx, ny, one, Sv, 1, nkv, 0, false, eps, nx, 1, plane, false, nil, cv, 1, nkv, (ll)nkv * nx);
  o.gemm(L, nkv, nx, ny, one, Sv, 1, nkv, 0, false, rec, nx, 1, plane, false, nil, cv + (ll)L * nkv * nx, 1, nkv,
         (ll)nkv * nx);
  // the per-column Toeplitz matrices (column-major nv x nv) and their inverses
  o.each(G * nx * nv2, WBV_FN {
    const ll gx = i / nv2, e = i % nv2;
    const int r = (int)(e % nv), c = (int)(e / nv);
    const ll g = gx / nx, x = gx % nx;
    Tv[i] = cv[g * nkv * nx + x * nkv + (r - c + 2 * hv)];
    inner[i] = delta(r, c);
  });
  o.getrf((int)(G * nx), nv, Tv, nv2, b.piv, nv, status, (int)(G * nx));
  o.getrs((int)(G * nx), nv, Tv, nv2, b.piv, nv, inner, nv, nv2, 0);
  // outer inverses: GP_x = -epx^H gepx epx^H, GP_z = -epz^H gepz epz^H; GP_y = gepy
  o.each(3 * L * N2, WBV_FN { GP[i] = zero(); });
  if (gepx) {
    o.gemm(L, N, N, N, one, gepx, 1, N, N2, false, epx, N, 1, N2, true, nil, T1, 1, N, N2);
    o.gemm(L, N, N, N, mone, epx, N, 1, N2, true, T1, 1, N, N2, false, nil, GP, 1, N, N2);
  }
  if (gepy) o.each(L * N2, WBV_FN { GP[L * N2 + i] = gepy[i]; });
  if (gepz) {
    o.gemm(L, N, N, N, one, gepz, 1, N, N2, false, epz, N, 1, N2, true, nil, T1 + L * N2, 1, N, N2);
    o.gemm(L, N, N, N, mone, epz, N, 1, N2, true, T1 + L * N2, 1, N, N2, false, nil, GP + 2 * L * N2, 1, N, N2);
  }
  // nested slots: gcu[g, (c nv + r), d] = sum over m - m' + 2hu = d of G[(r nu + m), (c nu + m')]
  o.each(G * nv2 * nku, WBV_FN {
    const ll g = i / (nv2 * nku), e = i % (nv2 * nku);
    const int rc = (int)(e / nku), d = (int)(e % nku);
    const int c = rc / nv, r = rc % nv;
    const z* Gm = GP + g * N2;
    z acc = zero();
    for (int m = 0; m < nu; ++m) {
      const int mp = m - d + 2 * hu;
      if (mp < 0 || mp >= nu) continue;
      acc = add(acc, Gm[(ll)(r * nu + m) + (ll)(c * nu + mp) * N]);
    }
    gcu[i] = acc;
  });
  // gent[g] (column x: the nv x nv cotangent of inner_x) = gcu[g] conj(Su)
  o.gemm((int)G, (int)nv2, nx, nku, one, gcu, nku, 1, nv2 * nku, false, Su, 1, nku, 0, true, nil, gent, 1, nv2,
         (ll)nx * nv2);
  // gTv = -inner^H gent inner^H
  o.gemm((int)(G * nx), nv, nv, nv, one, gent, 1, nv, nv2, false, inner, nv, 1, nv2, true, nil, gtmp, 1, nv, nv2);
  o.gemm((int)(G * nx), nv, nv, nv, mone, inner, nv, 1, nv2, true, gtmp, 1, nv, nv2, false, nil, gTv, 1, nv, nv2);
  // gcv[g, x, e] = sum over r - c + 2hv = e of gTv_x[r, c]
  o.each(G * nx * nkv, WBV_FN {
    const ll gx = i / nkv;
    const int e = (int)(i % nkv);
    const z* T = gTv + gx * nv2;
    z acc = zero();
    for (int r = 0; r < nv; ++r) {
      const int c = r - e + 2 * hv;
      if (c < 0 || c >= nv) continue;
      acc = add(acc, T[r + (ll)c * nv]);
    }
    gcv[i] = acc;
  });
  // raster cotangents: Sv^H gcv[g]^T, the 1/eps group through conj(-1/eps^2)
  o.gemm(L, ny, nx, nkv, one, Sv, nkv, 1, 0, true, gcv, 1, nkv, (ll)nx * nkv, false, nil, g_eps, nx, 1, plane);
  o.gemm(L, ny, nx, nkv, one, Sv, nkv, 1, 0, true, gcv + (ll)L * nx * nkv, 1, nkv, (ll)nx * nkv, false, nil, ginv, nx,
         1, plane);
  o.each(L * plane, WBV_FN { g_eps[i] = add(g_eps[i], mul(cj(sc(mul(rec[i], rec[i]), -1.0)), ginv[i])); });
  // direct slot: gc2[l, e, d] = sum over r - c + 2hv = e, m - m' + 2hu = d of G_z; += Sv^H gc2 conj(Su)
  o.each((ll)L * nkv * nku, WBV_FN {
    const ll l = i / ((ll)nkv * nku), rem = i % ((ll)nkv * nku);
    const int e = (int)(rem / nku), d = (int)(rem % nku);
    const z* Gm = GP + (2 * L + l) * N2;
    z acc = zero();
    for (int r = 0; r < nv; ++r) {
      const int c = r - e + 2 * hv;
      if (c < 0 || c >= nv) continue;
      for (int m = 0; m < nu; ++m) {
        const int mp = m - d + 2 * hu;
        if (mp < 0 || mp >= nu) continue;
        acc = add(acc, Gm[(ll)(r * nu + m) + (ll)(c * nu + mp) * N]);
      }
    }
    gc2[i] = acc;
  });
  o.gemm(L, nkv, nx, nku, one, gc2, nku, 1, (ll)nkv * nku, false, Su, 1, nku, 0, true, nil, tm, 1, nkv, (ll)nkv * nx);
  o.gemm(L, ny, nx, nkv, one, Sv, nkv, 1, 0, true, tm, 1, nkv, (ll)nkv * nx, false, one, g_eps, nx, 1, plane);
}

}  // namespace wbv
