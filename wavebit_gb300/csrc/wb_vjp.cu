// Reverse passes of stages A, B and C on the GPU: the drivers of wb_vjp.h over the library's
// batched FP64 kernels (GEMM with conjugated operands, LU, triangular solves) and one generic
// element-wise kernel that runs the drivers' per-element steps.
#include <algorithm>
#include "wb_common.cuh"
#include "wb_kernels.h"
#include "wb_internal.h"
#include "wb_vjp.h"
#include "wb_trace.h"

namespace wb {

// ports of a chunk of solves (wb_solve.cu)
void compute_ports(cudaStream_t s, const SolveDesc& d, int first, int Bc, const PortVectors& pv);

namespace {

template <class F>
__global__ void __launch_bounds__(256) each_kernel(long long count, F f) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < count) f(i);
}

// The largest batch one launch takes (the batched kernels put the batch on a grid dimension
// limited to 65535).
constexpr int kMaxBatch = 32768;

struct CudaOps {
  cudaStream_t s;
  Arena* ar;
  template <class T> T* get(size_t count) { return ar->get<T>(count); }
  template <class F> void each(long long count, F f) {
    if (count <= 0) return;
    each_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(count, f);
    note_launch();
  }
  void gemm(int batch, int m, int n, int k, cplx alpha, const cplx* A, long long a_rs, long long a_cs, long long a_bs,
            bool ca, const cplx* B, long long b_rs, long long b_cs, long long b_bs, bool cb, cplx beta, cplx* C,
            long long c_rs, long long c_cs, long long c_bs) {
    for (int b0 = 0; b0 < batch; b0 += kMaxBatch) {
      const int nb = std::min(kMaxBatch, batch - b0);
      zgemm_conj(s, nb, m, n, k, alpha, A + b0 * a_bs, a_rs, a_cs, a_bs, ca, B + b0 * b_bs, b_rs, b_cs, b_bs, cb,
                 beta, C + b0 * c_bs, c_rs, c_cs, c_bs);
    }
  }
  void getrf(int batch, int n, cplx* A, long long a_bs, int* piv, long long piv_bs, int32_t* status, int st_div) {
    if (st_div < 1) st_div = 1;
    if (batch <= kMaxBatch) { zgetrf(s, batch, n, A, n, a_bs, piv, piv_bs, status, st_div); return; }
    // chunks that start on a status boundary (or one status word for the whole batch)
    const int step = st_div >= batch ? kMaxBatch : std::max(st_div, (kMaxBatch / st_div) * st_div);
    for (int b0 = 0; b0 < batch; b0 += step) {
      const int nb = std::min(step, batch - b0);
      int32_t* st = status ? status + (st_div >= batch ? 0 : b0 / st_div) : nullptr;
      zgetrf(s, nb, n, A + b0 * a_bs, n, a_bs, piv + b0 * piv_bs, piv_bs, st, st_div >= batch ? (1 << 30) : st_div);
    }
  }
  void getrs(int batch, int n, const cplx* LU, long long a_bs, const int* piv, long long piv_bs, cplx* B, int nrhs,
             long long b_bs, int trans) {
    for (int b0 = 0; b0 < batch; b0 += kMaxBatch) {
      const int nb = std::min(kMaxBatch, batch - b0);
      zgetrs(s, nb, n, LU + b0 * a_bs, n, a_bs, piv + b0 * piv_bs, piv_bs, B + b0 * b_bs, nrhs, n, b_bs, trans);
    }
  }
};

// the largest chunk (from `want` down) whose scratch fits `budget` bytes
template <class Bytes>
int fit_chunk(int want, size_t budget, Bytes bytes) {
  int c = std::max(1, want);
  while (c > 1 && bytes(c) > budget) c = (c + 1) / 2;
  return c;
}

}  // namespace

size_t layer_modes_vjp_bytes(int N, int P) { return wbv::layer_modes_vjp_bytes(N, P); }
size_t smm_vjp_bytes(int N, int L, int Bc) {
  wbv::Counter c;
  const size_t n = 2 * (size_t)N;
  // port vectors: kx, ky, c, s (double), kz_top, kz_bot (N), wg .. t21 (n), nt, nb
  for (int k = 0; k < 4; ++k) c.get<double>((size_t)Bc * N);
  for (int k = 0; k < 2; ++k) c.get<cplx>((size_t)Bc * N);
  for (int k = 0; k < 8; ++k) c.get<cplx>((size_t)Bc * n);
  for (int k = 0; k < 2; ++k) c.get<cplx>((size_t)Bc);
  return c.bytes + wbv::smm_vjp_bytes(N, L, Bc);
}
size_t assemble_vjp_bytes(int L, int ny, int nx, int hu, int hv) {
  return wbv::assemble_vjp_bytes(L, ny, nx, hu, hv);
}

int layer_modes_vjp_run(cudaStream_t s, Arena& ar, size_t budget, int P, int N, int n_conv, const cplx* conv,
                        const int* pair_layer, const double* kx, const double* ky, const cplx* w, const cplx* q,
                        const cplx* W, const cplx* V, const cplx* gw, const cplx* gq, const cplx* gW, const cplx* gV,
                        cplx* gconv, int32_t* status) {
  TraceRange trace_("wb:layer_modes_vjp");
  const int n = 2 * N;
  const long long n2 = (long long)n * n;
  const int chunk = fit_chunk(P, budget, [&](int c) { return wbv::layer_modes_vjp_bytes(N, c); });
  CudaOps o{s, &ar};
  o.each((long long)n_conv * 3 * N * N, [=] __device__(long long i) { gconv[i] = cmk(0.0, 0.0); });
  for (int p0 = 0; p0 < P; p0 += chunk) {
    const int Pc = std::min(chunk, P - p0);
    ar.reset();
    wbv::LmBufs b;
    if (!b.carve(o, Pc, N) || !ar.ok()) return -1;
    wbv::layer_modes_vjp(o, b, Pc, N, n_conv, conv, pair_layer + p0, kx + (long long)p0 * N,
                         ky + (long long)p0 * N, w + (long long)p0 * n, q + (long long)p0 * n, W + p0 * n2,
                         V + p0 * n2, gw ? gw + (long long)p0 * n : nullptr, gq ? gq + (long long)p0 * n : nullptr,
                         gW ? gW + p0 * n2 : nullptr, gV ? gV + p0 * n2 : nullptr, gconv,
                         status ? status + p0 : nullptr);
  }
  return 0;
}

int layer_modes_vjp_chunk(int P, int N, size_t budget) {
  return fit_chunk(P, budget, [&](int c) { return wbv::layer_modes_vjp_bytes(N, c); });
}

int smm_vjp_chunk(int B, int N, int L, size_t budget) {
  return fit_chunk(B, budget, [&](int c) { return smm_vjp_bytes(N, L, c); });
}

int smm_vjp_run(cudaStream_t s, Arena& ar, size_t budget, const SolveDesc& d, const cplx* W, const cplx* V,
                const cplx* q, const double* gR, const double* gT, cplx* gW, cplx* gV, cplx* gq, double* g_thick,
                int32_t* status) {
  TraceRange trace_("wb:smm_solve_vjp");
  const int N = (2 * d.hu + 1) * (2 * d.hv + 1), n = 2 * N, L = d.n_layers, B = d.n_solves;
  const long long n2 = (long long)n * n;
  const int chunk = smm_vjp_chunk(B, N, L, budget);
  CudaOps o{s, &ar};
  for (int first = 0; first < B; first += chunk) {
    const int Bc = std::min(chunk, B - first);
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
    wbv::SmmBufs b;
    if (!ar.ok() || !b.carve(o, Bc, L, N) || !ar.ok()) return -1;
    compute_ports(s, d, first, Bc, pv);
    wbv::Ports P_{pv.kx, pv.ky, pv.c, pv.s, pv.kz_top, pv.kz_bot, pv.wg, pv.vg, pv.r11, pv.r12, pv.r21, pv.r22,
                  pv.t11, pv.t21, pv.nt, pv.nb};
    const long long off = (long long)first * L;
    wbv::smm_vjp(o, b, Bc, L, N, P_, W + off * n2, V + off * n2, q + off * n, d.thickness + off,
                 d.wavelength + first, d.eps_top + first, d.eps_bot + first, d.pol + 2 * first,
                 gR ? gR + (long long)first * 3 * N : nullptr, gT ? gT + (long long)first * 3 * N : nullptr,
                 gW + off * n2, gV + off * n2, gq + off * n, g_thick + off, status + first);
  }
  return 0;
}

int assemble_vjp_run(cudaStream_t s, Arena& ar, int L, int ny, int nx, int hu, int hv, const cplx* eps,
                     const cplx* epx, const cplx* epz, const cplx* gepx, const cplx* gepy, const cplx* gepz,
                     cplx* g_eps, int32_t* status) {
  TraceRange trace_("wb:assemble_li_vjp");
  CudaOps o{s, &ar};
  ar.reset();
  wbv::AsmBufs b;
  if (!b.carve(o, L, ny, nx, hu, hv) || !ar.ok()) return -1;
  wbv::assemble_vjp(o, b, L, ny, nx, hu, hv, eps, epx, epz, gepx, gepy, gepz, g_eps, status);
  return 0;
}

}  // namespace wb
