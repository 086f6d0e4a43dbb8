// A plain C++ stand-in for the batched device primitives of wb_vjp.h, so that the reverse-pass
// drivers (the same source the GPU library compiles) run on the CPU in the tests: GEMM with
// conjugated operands, LU with partial pivoting, triangular solves, and a loop for the
// element-wise steps. Test infrastructure only: nothing in the library links it.
#include <cstdlib>
#include <cstring>
#include <vector>
#include "wb_vjp.h"

using wbv::z;
using ll = long long;

namespace {

struct HostOps {
  std::vector<char> buf;
  size_t off = 0;
  bool failed = false;
  explicit HostOps(size_t bytes) : buf(bytes) {}
  template <class T> T* get(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
    if (failed || off + bytes > buf.size()) { failed = true; return nullptr; }
    T* p = reinterpret_cast<T*>(buf.data() + off);
    off += bytes;
    return p;
  }
  template <class F> void each(ll count, F f) {
    for (ll i = 0; i < count; ++i) f(i);
  }
  void gemm(int batch, int m, int n, int k, z alpha, const z* A, ll a_rs, ll a_cs, ll a_bs, bool ca, const z* B,
            ll b_rs, ll b_cs, ll b_bs, bool cb, z beta, z* C, ll c_rs, ll c_cs, ll c_bs) {
    std::vector<z> tmp((size_t)m * n);
    for (int e = 0; e < batch; ++e) {
      const z* a = A + e * a_bs;
      const z* b = B + e * b_bs;
      z* c = C + e * c_bs;
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
          z acc = wbv::zero();
          for (int t = 0; t < k; ++t) {
            z x = a[i * a_rs + t * a_cs], y = b[t * b_rs + j * b_cs];
            if (ca) x = wbv::cj(x);
            if (cb) y = wbv::cj(y);
            acc = wbv::add(acc, wbv::mul(x, y));
          }
          tmp[(size_t)i + (size_t)j * m] = acc;
        }
      const bool zb = beta.x == 0.0 && beta.y == 0.0;
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
          z v = wbv::mul(alpha, tmp[(size_t)i + (size_t)j * m]);
          if (!zb) v = wbv::add(v, wbv::mul(beta, c[i * c_rs + j * c_cs]));
          c[i * c_rs + j * c_cs] = v;
        }
    }
  }
  // LAPACK-style: piv[k] is the row exchanged with row k at step k
  void getrf(int batch, int n, z* A, ll a_bs, int* piv, ll piv_bs, int32_t* status, int st_div) {
    for (int e = 0; e < batch; ++e) {
      z* a = A + e * a_bs;
      int* p = piv + e * piv_bs;
      for (int k = 0; k < n; ++k) {
        int best = k;
        double bv = -1.0;
        for (int r = k; r < n; ++r) {
          double v = std::fabs(a[r + (ll)k * n].x) + std::fabs(a[r + (ll)k * n].y);
          if (v > bv) { bv = v; best = r; }
        }
        p[k] = best;
        if (best != k)
          for (int c = 0; c < n; ++c) std::swap(a[k + (ll)c * n], a[best + (ll)c * n]);
        const z d = a[k + (ll)k * n];
        if (d.x == 0.0 && d.y == 0.0) {
          if (status) status[e / (st_div < 1 ? 1 : st_div)] |= 1;
          continue;
        }
        const z id = wbv::inv(d);
        for (int r = k + 1; r < n; ++r) a[r + (ll)k * n] = wbv::mul(a[r + (ll)k * n], id);
        for (int c = k + 1; c < n; ++c) {
          const z f = a[k + (ll)c * n];
          for (int r = k + 1; r < n; ++r) a[r + (ll)c * n] = wbv::sub(a[r + (ll)c * n], wbv::mul(a[r + (ll)k * n], f));
        }
      }
    }
  }
  void getrs(int batch, int n, const z* LU, ll a_bs, const int* piv, ll piv_bs, z* B, int nrhs, ll b_bs, int trans) {
    for (int e = 0; e < batch; ++e) {
      const z* a = LU + e * a_bs;
      const int* p = piv + e * piv_bs;
      for (int j = 0; j < nrhs; ++j) {
        z* x = B + e * b_bs + (ll)j * n;
        if (trans == 0) {
          for (int k = 0; k < n; ++k) if (p[k] != k) std::swap(x[k], x[p[k]]);
          for (int r = 0; r < n; ++r)
            for (int c = 0; c < r; ++c) x[r] = wbv::sub(x[r], wbv::mul(a[r + (ll)c * n], x[c]));
          for (int r = n - 1; r >= 0; --r) {
            for (int c = r + 1; c < n; ++c) x[r] = wbv::sub(x[r], wbv::mul(a[r + (ll)c * n], x[c]));
            x[r] = wbv::dv(x[r], a[r + (ll)r * n]);
          }
        } else {
          // A^T = U^T L^T P: U^T y = x, L^T w = y, then undo the interchanges in reverse
          for (int r = 0; r < n; ++r) {
            for (int c = 0; c < r; ++c) x[r] = wbv::sub(x[r], wbv::mul(a[c + (ll)r * n], x[c]));
            x[r] = wbv::dv(x[r], a[r + (ll)r * n]);
          }
          for (int r = n - 1; r >= 0; --r)
            for (int c = r + 1; c < n; ++c) x[r] = wbv::sub(x[r], wbv::mul(a[c + (ll)r * n], x[c]));
          for (int k = n - 1; k >= 0; --k) if (p[k] != k) std::swap(x[k], x[p[k]]);
        }
      }
    }
  }
};

}  // namespace

extern "C" {

int host_layer_modes_vjp(int P, int N, int n_conv, const z* conv, const int* pl, const double* kx, const double* ky,
                         const z* w, const z* q, const z* W, const z* V, const z* gw, const z* gq, const z* gW,
                         const z* gV, z* gconv, int32_t* status) {
  HostOps o(wbv::layer_modes_vjp_bytes(N, P));
  wbv::LmBufs b;
  if (!b.carve(o, P, N)) return -1;
  for (ll i = 0; i < (ll)n_conv * 3 * N * N; ++i) gconv[i] = wbv::zero();
  wbv::layer_modes_vjp(o, b, P, N, n_conv, conv, pl, kx, ky, w, q, W, V, gw, gq, gW, gV, gconv, status);
  return 0;
}

int host_smm_vjp(int Bc, int L, int N, const double* kx, const double* ky, const double* c, const double* s,
                 const z* kz_top, const z* kz_bot, const z* wg, const z* vg, const z* r11, const z* r12, const z* r21,
                 const z* r22, const z* t11, const z* t21, const z* nt, const z* nb, const z* W, const z* V,
                 const z* q, const double* thick, const double* wavelength, const z* eps_top, const z* eps_bot,
                 const z* pol, const double* gR, const double* gT, z* gW, z* gV, z* gq, double* g_thick,
                 int32_t* status) {
  HostOps o(wbv::smm_vjp_bytes(N, L, Bc));
  wbv::SmmBufs b;
  if (!b.carve(o, Bc, L, N)) return -1;
  wbv::Ports pv{kx, ky, c, s, kz_top, kz_bot, wg, vg, r11, r12, r21, r22, t11, t21, nt, nb};
  wbv::smm_vjp(o, b, Bc, L, N, pv, W, V, q, thick, wavelength, eps_top, eps_bot, pol, gR, gT, gW, gV, gq, g_thick,
               status);
  return 0;
}

int host_assemble_vjp(int L, int ny, int nx, int hu, int hv, const z* eps, const z* epx, const z* epz,
                      const z* gepx, const z* gepy, const z* gepz, z* g_eps, int32_t* status) {
  HostOps o(wbv::assemble_vjp_bytes(L, ny, nx, hu, hv));
  wbv::AsmBufs b;
  if (!b.carve(o, L, ny, nx, hu, hv)) return -1;
  wbv::assemble_vjp(o, b, L, ny, nx, hu, hv, eps, epx, epz, gepx, gepy, gepz, g_eps, status);
  return 0;
}

}  // extern "C"
