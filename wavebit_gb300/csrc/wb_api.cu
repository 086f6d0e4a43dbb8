// C ABI of libwbgpu.so (declared in include/wavebit_gb300.h): handles, the scratch arena,
// error reporting and the entry points that drive stages A, B and C.
#include <cstdio>
#include <cstring>
#include <cstdarg>
#include <string>
#include <vector>
#include <algorithm>
#include "../../include/wavebit_gb300.h"
#include "wb_common.cuh"
#include "wb_kernels.h"
#include "wb_internal.h"
#include "wb_trace.h"

struct wb_handle {
  int device = 0;
  size_t budget = 0;
  wb::Arena arena;
  void* buf = nullptr;
  size_t buf_bytes = 0;
  // device staging block of wb_solve_host (inputs, slots, outputs), kept between calls and grown
  // only when a call needs more; separate from the arena, which the solve itself uses
  void* io = nullptr;
  size_t io_bytes = 0;
};

namespace {
thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char msg[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  g_err = msg;
  return code;
}

int cuda_check(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(WB_E_CUDA, "%s: %s", where, cudaGetErrorString(e));
  return WB_OK;
}

// Grow the handle's arena to at least `bytes` (within the budget).
int reserve(wb_handle* h, size_t bytes) {
  if (bytes <= h->buf_bytes) { h->arena.base = (char*)h->buf; h->arena.cap = h->buf_bytes; return WB_OK; }
  if (bytes > h->budget)
    return fail(WB_E_NOMEM, "workspace of %zu bytes exceeds the handle budget of %zu bytes", bytes, h->budget);
  if (h->buf) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return fail(WB_E_CUDA, "synchronise before growing the arena: %s", cudaGetErrorString(e));
    cudaFree(h->buf);
    h->buf = nullptr; h->buf_bytes = 0;
  }
  cudaError_t e = cudaMalloc(&h->buf, bytes);
  if (e != cudaSuccess) {
    h->buf = nullptr;
    cudaGetLastError();
    return fail(WB_E_NOMEM, "cudaMalloc(%zu) for the arena: %s", bytes, cudaGetErrorString(e));
  }
  h->buf_bytes = bytes;
  h->arena.base = (char*)h->buf;
  h->arena.cap = bytes;
  h->arena.reset();
  return WB_OK;
}

bool valid_orders(int hu, int hv) { return wb::orders_fit(hu, hv); }
}  // namespace

namespace wb {
int noalloc_fail(const char* msg) { g_err = msg; return WB_E_INVALID; }
}

extern "C" {

int wb_version(void) { return 202; }

int wb_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return WB_E_INVALID;
  std::snprintf(buf, len, "%s", g_err.c_str());
  return WB_OK;
}

int wb_create(int device, size_t hbm_budget, wb_handle** out) {
  if (!out) return fail(WB_E_INVALID, "wb_create: out is NULL");
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(WB_E_CUDA, "wb_create: no CUDA device is visible");
  }
  if (device < 0 || device >= count) return fail(WB_E_INVALID, "wb_create: device %d of %d", device, count);
  if (cudaSetDevice(device) != cudaSuccess) return cuda_check("wb_create: cudaSetDevice");
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return cuda_check("wb_create: cudaMemGetInfo");
  wb_handle* h = new wb_handle();
  h->device = device;
  h->budget = hbm_budget ? hbm_budget : (size_t)(0.8 * (double)free_b);
  *out = h;
  return WB_OK;
}

int wb_destroy(wb_handle* h) {
  if (!h) return WB_OK;
  if (h->buf || h->io) {
    cudaSetDevice(h->device);
    cudaDeviceSynchronize();
    if (h->buf) cudaFree(h->buf);
    if (h->io) cudaFree(h->io);
  }
  delete h;
  return WB_OK;
}

int wb_reserve(wb_handle* h, size_t bytes) {
  if (!h) return fail(WB_E_INVALID, "wb_reserve: NULL handle");
  cudaSetDevice(h->device);
  return reserve(h, bytes);
}

int wb_build_indices(int hu, int hv, int32_t* labels_u, int32_t* labels_v, int32_t* toeplitz_u,
                     int32_t* toeplitz_v) {
  if (!valid_orders(hu, hv))
    return fail(WB_E_INVALID, "orders (%d, %d) out of range: 0 <= hv <= 42 and (2hu+1)(2hv+1) <= 3228", hu, hv);
  const int nu = 2 * hu + 1, nv = 2 * hv + 1;
  if (labels_u) for (int i = 0; i < nu; ++i) labels_u[i] = i - hu;
  if (labels_v) for (int i = 0; i < nv; ++i) labels_v[i] = i - hv;
  if (toeplitz_u) for (int r = 0; r < nu; ++r) for (int c = 0; c < nu; ++c) toeplitz_u[r * nu + c] = r - c + 2 * hu;
  if (toeplitz_v) for (int r = 0; r < nv; ++r) for (int c = 0; c < nv; ++c) toeplitz_v[r * nv + c] = r - c + 2 * hv;
  return WB_OK;
}

int wb_assemble_li(wb_handle* h, const wb_complex* eps, int L, int ny, int nx, int hu, int hv,
                   wb_complex* epx, wb_complex* epy, wb_complex* epz_i, int32_t* status, void* stream) {
  wb::TraceRange trace_("wb:assemble_li");
  if (!h || !eps || !epx || !epy || !epz_i) return fail(WB_E_INVALID, "wb_assemble_li: NULL argument");
  if (L <= 0 || ny <= 0 || nx <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_assemble_li: bad sizes L=%d ny=%d nx=%d orders=(%d,%d)", L, ny, nx, hu, hv);
  cudaSetDevice(h->device);
  size_t need = wb::assemble_workspace_bytes(L, ny, nx, hu, hv);
  int rc = reserve(h, need);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  wb::assemble_li(s, (const cplx*)eps, L, ny, nx, hu, hv, (cplx*)epx, (cplx*)epy, (cplx*)epz_i, h->buf, status);
  return cuda_check("wb_assemble_li");
}

int wb_assemble_li_vjp(wb_handle* h, const wb_complex* eps, int L, int ny, int nx, int hu, int hv,
                       const wb_complex* epx, const wb_complex* epz_i, const wb_complex* g_epx,
                       const wb_complex* g_epy, const wb_complex* g_epz_i, wb_complex* g_eps, int32_t* status,
                       void* stream) {
  wb::TraceRange trace_("wb:assemble_li_vjp");
  if (!h || !eps || !epx || !epz_i || !g_eps) return fail(WB_E_INVALID, "wb_assemble_li_vjp: NULL argument");
  if (L <= 0 || ny <= 0 || nx <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_assemble_li_vjp: bad sizes L=%d ny=%d nx=%d orders=(%d,%d)", L, ny, nx, hu, hv);
  cudaSetDevice(h->device);
  int rc = reserve(h, wb::assemble_vjp_bytes(L, ny, nx, hu, hv));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (status) cudaMemsetAsync(status, 0, sizeof(int32_t), s);
  if (wb::assemble_vjp_run(s, h->arena, L, ny, nx, hu, hv, (const cplx*)eps, (const cplx*)epx, (const cplx*)epz_i,
                           (const cplx*)g_epx, (const cplx*)g_epy, (const cplx*)g_epz_i, (cplx*)g_eps, status) != 0)
    return fail(WB_E_NOMEM, "wb_assemble_li_vjp: arena exhausted");
  return cuda_check("wb_assemble_li_vjp");
}

int wb_layer_modes_vjp(wb_handle* h, int n_pairs, int hu, int hv, int n_conv, const wb_complex* conv,
                       const int32_t* pair_layer, const double* kx, const double* ky, const wb_complex* w,
                       const wb_complex* q, const wb_complex* W, const wb_complex* V, const wb_complex* g_w,
                       const wb_complex* g_q, const wb_complex* g_W, const wb_complex* g_V, wb_complex* g_conv,
                       int32_t* status, void* stream) {
  wb::TraceRange trace_("wb:layer_modes_vjp");
  if (!h || !conv || !pair_layer || !kx || !ky || !w || !q || !W || !V || !g_conv)
    return fail(WB_E_INVALID, "wb_layer_modes_vjp: NULL argument");
  if (n_pairs <= 0 || n_conv <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_layer_modes_vjp: bad sizes n_pairs=%d n_conv=%d", n_pairs, n_conv);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  const int chunk = wb::layer_modes_vjp_chunk(n_pairs, N, h->budget);
  int rc = reserve(h, wb::layer_modes_vjp_bytes(N, chunk));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (status) cudaMemsetAsync(status, 0, sizeof(int32_t) * n_pairs, s);
  if (wb::layer_modes_vjp_run(s, h->arena, h->buf_bytes, n_pairs, N, n_conv, (const cplx*)conv,
                              (const int*)pair_layer, kx, ky, (const cplx*)w, (const cplx*)q, (const cplx*)W,
                              (const cplx*)V, (const cplx*)g_w, (const cplx*)g_q, (const cplx*)g_W, (const cplx*)g_V,
                              (cplx*)g_conv, status) != 0)
    return fail(WB_E_NOMEM, "wb_layer_modes_vjp: arena exhausted for a chunk of %d pairs", chunk);
  return cuda_check("wb_layer_modes_vjp");
}

int wb_smm_solve_vjp(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                     const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                     const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                     const wb_complex* pol, const double* g_R, const double* g_T, wb_complex* g_W, wb_complex* g_V,
                     wb_complex* g_q, double* g_thickness, int32_t* status, void* stream) {
  wb::TraceRange trace_("wb:smm_solve_vjp");
  if (!h || !W || !V || !q || !thickness || !wavelength || !period || !theta || !phi || !eps_top || !eps_bot ||
      !pol || !g_W || !g_V || !g_q || !g_thickness || !status)
    return fail(WB_E_INVALID, "wb_smm_solve_vjp: NULL argument");
  if (B <= 0 || L <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_smm_solve_vjp: bad sizes B=%d L=%d", B, L);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  const int chunk = wb::smm_vjp_chunk(B, N, L, h->budget);
  int rc = reserve(h, wb::smm_vjp_bytes(N, L, chunk));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int32_t) * B, s);
  wb::SolveDesc d{B, L, hu, hv, nullptr, nullptr, thickness, wavelength, period, theta, phi, (const cplx*)eps_top,
                  (const cplx*)eps_bot, (const cplx*)pol};
  if (wb::smm_vjp_run(s, h->arena, h->buf_bytes, d, (const cplx*)W, (const cplx*)V, (const cplx*)q, g_R, g_T,
                      (cplx*)g_W, (cplx*)g_V, (cplx*)g_q, g_thickness, status) != 0)
    return fail(WB_E_NOMEM, "wb_smm_solve_vjp: arena exhausted for a chunk of %d solves", chunk);
  return cuda_check("wb_smm_solve_vjp");
}

int wb_assemble_li_integrated(wb_handle* h, const wb_complex* eps, int L, int ny, int nx, const double* x_edges,
                              const double* y_edges, int hu, int hv, wb_complex* epx, wb_complex* epy,
                              wb_complex* epz_i, int32_t* status, void* stream) {
  wb::TraceRange trace_("wb:assemble_li_integrated");
  if (!h || !eps || !x_edges || !y_edges || !epx || !epy || !epz_i)
    return fail(WB_E_INVALID, "wb_assemble_li_integrated: NULL argument");
  if (L <= 0 || ny <= 0 || nx <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_assemble_li_integrated: bad sizes L=%d ny=%d nx=%d orders=(%d,%d)", L, ny, nx,
                hu, hv);
  cudaSetDevice(h->device);
  size_t need = wb::assemble_workspace_bytes(L, ny, nx, hu, hv);
  int rc = reserve(h, need);
  if (rc) return rc;
  wb::assemble_li((cudaStream_t)stream, (const cplx*)eps, L, ny, nx, hu, hv, (cplx*)epx, (cplx*)epy, (cplx*)epz_i,
                  h->buf, status, x_edges, y_edges);
  return cuda_check("wb_assemble_li_integrated");
}

size_t wb_solve_workspace_bytes(int hu, int hv, int L, int chunk) {
  if (!valid_orders(hu, hv) || L <= 0 || chunk <= 0) return 0;
  return wb::solve_chunk_bytes((2 * hu + 1) * (2 * hv + 1), L, chunk, WB_PRECISION_FP64);
}

size_t wb_workspace_bytes(int hu, int hv, int L, int chunk, int precision) {
  if (!valid_orders(hu, hv) || L <= 0 || chunk <= 0 || precision < WB_PRECISION_FP64 ||
      precision > WB_PRECISION_MIXED_DF64_EIG)
    return 0;
  return wb::solve_chunk_bytes((2 * hu + 1) * (2 * hv + 1), L, chunk, precision);
}

int wb_layer_modes(wb_handle* h, int n_pairs, int hu, int hv, const wb_complex* conv,
                   const int32_t* pair_layer, const double* kx, const double* ky, wb_complex* w,
                   wb_complex* q, wb_complex* W, wb_complex* V, int32_t* status, int precision,
                   void* stream) {
  wb::TraceRange trace_("wb:layer_modes");
  if (!h || !conv || !pair_layer || !kx || !ky || !w || !q || !W || !V)
    return fail(WB_E_INVALID, "wb_layer_modes: NULL argument");
  if (n_pairs <= 0 || !valid_orders(hu, hv)) return fail(WB_E_INVALID, "wb_layer_modes: bad sizes");
  if (precision < WB_PRECISION_FP64 || precision > WB_PRECISION_MIXED_DF64_EIG)
    return fail(WB_E_INVALID, "wb_layer_modes: precision %d", precision);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1), n = 2 * N;
  size_t need = wb::layer_modes_bytes(N, n_pairs, precision);
  int rc = reserve(h, need);
  if (rc) return rc;
  if (wb::layer_modes((cudaStream_t)stream, h->arena, n_pairs, N, (const cplx*)conv, (const int*)pair_layer, kx, ky,
                      (cplx*)w, (cplx*)q, (cplx*)W, (cplx*)V, status, precision) != 0)
    return fail(WB_E_NOMEM, "wb_layer_modes: arena exhausted for %d pairs", n_pairs);
  (void)n;
  return cuda_check("wb_layer_modes");
}

int wb_solve_batch(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* conv,
                   const int32_t* layer_index, const double* thickness, const double* wavelength,
                   const double* period, const double* theta, const double* phi,
                   const wb_complex* eps_top, const wb_complex* eps_bot, const wb_complex* pol,
                   double* R, double* T, wb_complex* amps, int32_t* status, int precision,
                   void* stream) {
  wb::TraceRange trace_("wb:solve_batch");
  if (!h || !conv || !layer_index || !thickness || !wavelength || !period || !theta || !phi || !eps_top ||
      !eps_bot || !pol || !R || !T || !status)
    return fail(WB_E_INVALID, "wb_solve_batch: NULL argument");
  if (B <= 0 || L <= 0 || !valid_orders(hu, hv)) return fail(WB_E_INVALID, "wb_solve_batch: bad sizes B=%d L=%d", B, L);
  if (precision < WB_PRECISION_FP64 || precision > WB_PRECISION_MIXED_DF64_EIG)
    return fail(WB_E_INVALID, "wb_solve_batch: precision %d", precision);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  // the largest chunk that fits the budget
  int chunk = B;
  while (chunk > 1 && wb::solve_chunk_bytes(N, L, chunk, precision) > h->budget) chunk = (chunk + 1) / 2;
  size_t need = wb::solve_chunk_bytes(N, L, chunk, precision);
  int rc = reserve(h, need);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int32_t) * B, s);
  wb::SolveDesc d{B, L, hu, hv, (const cplx*)conv, (const int*)layer_index, thickness, wavelength, period, theta,
                  phi, (const cplx*)eps_top, (const cplx*)eps_bot, (const cplx*)pol};
  wb::SolveOut o{R, T, (cplx*)amps, status};
  for (int first = 0; first < B; first += chunk) {
    int count = std::min(chunk, B - first);
    if (wb::solve_chunk(s, h->arena, d, first, count, o, precision) != 0)
      return fail(WB_E_NOMEM, "wb_solve_batch: arena exhausted for a chunk of %d", count);
  }
  return cuda_check("wb_solve_batch");
}

int wb_smm_solve(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                 const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                 const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                 const wb_complex* pol, double* R, double* T, wb_complex* amps, int32_t* status, int precision,
                 void* stream) {
  wb::TraceRange trace_("wb:smm_solve");
  if (!h || !W || !V || !q || !thickness || !wavelength || !period || !theta || !phi || !eps_top || !eps_bot ||
      !pol || !R || !T || !status)
    return fail(WB_E_INVALID, "wb_smm_solve: NULL argument");
  if (B <= 0 || L <= 0 || !valid_orders(hu, hv)) return fail(WB_E_INVALID, "wb_smm_solve: bad sizes B=%d L=%d", B, L);
  if (precision != WB_PRECISION_FP64 && precision != WB_PRECISION_MIXED)
    return fail(WB_E_INVALID, "wb_smm_solve: precision %d (FP64 or MIXED)", precision);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  int chunk = B;
  while (chunk > 1 && wb::smm_chunk_bytes(N, L, chunk, precision) > h->budget) chunk = (chunk + 1) / 2;
  int rc = reserve(h, wb::smm_chunk_bytes(N, L, chunk, precision));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int32_t) * B, s);
  wb::SolveDesc d{B, L, hu, hv, nullptr, nullptr, thickness, wavelength, period, theta, phi, (const cplx*)eps_top,
                  (const cplx*)eps_bot, (const cplx*)pol};
  wb::SolveOut o{R, T, (cplx*)amps, status};
  for (int first = 0; first < B; first += chunk) {
    int count = std::min(chunk, B - first);
    if (wb::smm_chunk(s, h->arena, d, (const cplx*)W, (const cplx*)V, (const cplx*)q, first, count, o, precision) != 0)
      return fail(WB_E_NOMEM, "wb_smm_solve: arena exhausted for a chunk of %d", count);
  }
  return cuda_check("wb_smm_solve");
}

int wb_etm_solve(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                 const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                 const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                 const wb_complex* pol, double* R, double* T, wb_complex* amps, int32_t* status, void* stream) {
  wb::TraceRange trace_("wb:etm_solve");
  if (!h || !W || !V || !q || !thickness || !wavelength || !period || !theta || !phi || !eps_top || !eps_bot ||
      !pol || !R || !T || !status)
    return fail(WB_E_INVALID, "wb_etm_solve: NULL argument");
  if (B <= 0 || L <= 0 || !valid_orders(hu, hv)) return fail(WB_E_INVALID, "wb_etm_solve: bad sizes B=%d L=%d", B, L);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  int chunk = B;
  while (chunk > 1 && wb::etm_chunk_bytes(N, L, chunk) > h->budget) chunk = (chunk + 1) / 2;
  int rc = reserve(h, wb::etm_chunk_bytes(N, L, chunk));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int32_t) * B, s);
  wb::SolveDesc d{B, L, hu, hv, nullptr, nullptr, thickness, wavelength, period, theta, phi, (const cplx*)eps_top,
                  (const cplx*)eps_bot, (const cplx*)pol};
  wb::SolveOut o{R, T, (cplx*)amps, status};
  for (int first = 0; first < B; first += chunk) {
    int count = std::min(chunk, B - first);
    if (wb::etm_chunk(s, h->arena, d, (const cplx*)W, (const cplx*)V, (const cplx*)q, first, count, o) != 0)
      return fail(WB_E_NOMEM, "wb_etm_solve: arena exhausted for a chunk of %d", count);
  }
  return cuda_check("wb_etm_solve");
}

int wb_layer_amplitudes(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                        const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                        const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                        const wb_complex* C, int k, wb_complex* plus, wb_complex* minus_top, wb_complex* minus_bottom,
                        wb_complex* cref, wb_complex* ctrn, int32_t* status, void* stream) {
  wb::TraceRange trace_("wb:layer_amplitudes");
  if (!h || !W || !V || !q || !thickness || !wavelength || !period || !theta || !phi || !eps_top || !eps_bot || !C ||
      !plus || !minus_top || !minus_bottom || !cref || !ctrn || !status)
    return fail(WB_E_INVALID, "wb_layer_amplitudes: NULL argument");
  if (B <= 0 || L <= 0 || k <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_layer_amplitudes: bad sizes B=%d L=%d k=%d", B, L, k);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  int chunk = B;
  while (chunk > 1 && wb::amplitudes_chunk_bytes(N, L, chunk, k) > h->budget) chunk = (chunk + 1) / 2;
  int rc = reserve(h, wb::amplitudes_chunk_bytes(N, L, chunk, k));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int32_t) * B, s);
  wb::SolveDesc d{B, L, hu, hv, nullptr, nullptr, thickness, wavelength, period, theta, phi, (const cplx*)eps_top,
                  (const cplx*)eps_bot, nullptr};
  for (int first = 0; first < B; first += chunk) {
    int count = std::min(chunk, B - first);
    if (wb::amplitudes_chunk(s, h->arena, d, (const cplx*)W, (const cplx*)V, (const cplx*)q, (const cplx*)C, k, first,
                             count, (cplx*)plus, (cplx*)minus_top, (cplx*)minus_bottom, (cplx*)cref, (cplx*)ctrn,
                             status) != 0)
      return fail(WB_E_NOMEM, "wb_layer_amplitudes: arena exhausted for a chunk of %d", count);
  }
  return cuda_check("wb_layer_amplitudes");
}

int wb_scattering_matrix(wb_handle* h, int B, int L, int hu, int hv, const wb_complex* W, const wb_complex* V,
                         const wb_complex* q, const double* thickness, const double* wavelength, const double* period,
                         const double* theta, const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                         wb_complex* S11, wb_complex* S12, wb_complex* S21, wb_complex* S22, int32_t* status,
                         void* stream) {
  wb::TraceRange trace_("wb:scattering_matrix");
  if (!h || !W || !V || !q || !thickness || !wavelength || !period || !theta || !phi || !eps_top || !eps_bot ||
      !S11 || !S12 || !S21 || !S22 || !status)
    return fail(WB_E_INVALID, "wb_scattering_matrix: NULL argument");
  if (B <= 0 || L <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_scattering_matrix: bad sizes B=%d L=%d", B, L);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  int chunk = B;
  while (chunk > 1 && wb::scattering_chunk_bytes(N, L, chunk) > h->budget) chunk = (chunk + 1) / 2;
  int rc = reserve(h, wb::scattering_chunk_bytes(N, L, chunk));
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int32_t) * B, s);
  wb::SolveDesc d{B, L, hu, hv, nullptr, nullptr, thickness, wavelength, period, theta, phi, (const cplx*)eps_top,
                  (const cplx*)eps_bot, nullptr};
  for (int first = 0; first < B; first += chunk) {
    int count = std::min(chunk, B - first);
    if (wb::scattering_chunk(s, h->arena, d, (const cplx*)W, (const cplx*)V, (const cplx*)q, first, count,
                             (cplx*)S11, (cplx*)S12, (cplx*)S21, (cplx*)S22, status) != 0)
      return fail(WB_E_NOMEM, "wb_scattering_matrix: arena exhausted for a chunk of %d", count);
  }
  return cuda_check("wb_scattering_matrix");
}

int wb_solve_host(wb_handle* h, int B, int L, int ny, int nx, int hu, int hv,
                  const wb_complex* eps, const int32_t* layer_index, const double* thickness,
                  const double* wavelength, const double* period, const double* theta,
                  const double* phi, const wb_complex* eps_top, const wb_complex* eps_bot,
                  const wb_complex* pol, double* R, double* T, int32_t* status, int precision) {
  wb::TraceRange trace_("wb:solve_host");
  if (!h || !eps || !layer_index || !thickness || !wavelength || !period || !theta || !phi || !eps_top ||
      !eps_bot || !pol || !R || !T || !status)
    return fail(WB_E_INVALID, "wb_solve_host: NULL argument");
  if (B <= 0 || L <= 0 || ny <= 0 || nx <= 0 || !valid_orders(hu, hv))
    return fail(WB_E_INVALID, "wb_solve_host: bad sizes");
  for (long long i = 0; i < (long long)B * L; ++i)
    if (layer_index[i] < 0 || layer_index[i] >= L)
      return fail(WB_E_INVALID, "wb_solve_host: layer_index[%lld] = %d outside [0, %d)", i, layer_index[i], L);
  cudaSetDevice(h->device);
  const int N = (2 * hu + 1) * (2 * hv + 1);
  const size_t NN = (size_t)N * N;
  // one device block for inputs, conv and outputs (separate from the arena)
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off += (b + 255) & ~(size_t)255; return o; };
  const size_t o_eps = take(sizeof(wb_complex) * L * ny * nx), o_conv = take(sizeof(wb_complex) * 3 * L * NN);
  const size_t o_li = take(sizeof(int32_t) * B * L), o_th = take(sizeof(double) * B * L);
  const size_t o_wl = take(sizeof(double) * B), o_per = take(sizeof(double) * 2 * B);
  const size_t o_th2 = take(sizeof(double) * B), o_ph = take(sizeof(double) * B);
  const size_t o_et = take(sizeof(wb_complex) * B), o_eb = take(sizeof(wb_complex) * B);
  const size_t o_pol = take(sizeof(wb_complex) * 2 * B);
  const size_t o_R = take(sizeof(double) * 3 * B * N), o_T = take(sizeof(double) * 3 * B * N);
  const size_t o_st = take(sizeof(int32_t) * B), o_ast = take(sizeof(int32_t));
  const size_t o_tmp = take(sizeof(wb_complex) * 3 * L * NN);   // slot planes before regrouping
  if (off > h->io_bytes) {
    if (h->io) {
      cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) return fail(WB_E_CUDA, "wb_solve_host: synchronise before growing: %s", cudaGetErrorString(e));
      cudaFree(h->io);
      h->io = nullptr; h->io_bytes = 0;
    }
    if (cudaMalloc(&h->io, off) != cudaSuccess) {
      cudaGetLastError();
      h->io = nullptr;
      return fail(WB_E_NOMEM, "wb_solve_host: cudaMalloc(%zu)", off);
    }
    h->io_bytes = off;
  }
  char* dev = (char*)h->io;
  cudaStream_t s = nullptr;
  auto H2D = [&](size_t o, const void* p, size_t b) { cudaMemcpyAsync(dev + o, p, b, cudaMemcpyHostToDevice, s); };
  H2D(o_eps, eps, sizeof(wb_complex) * L * ny * nx);
  H2D(o_li, layer_index, sizeof(int32_t) * B * L);
  H2D(o_th, thickness, sizeof(double) * B * L);
  H2D(o_wl, wavelength, sizeof(double) * B);
  H2D(o_per, period, sizeof(double) * 2 * B);
  H2D(o_th2, theta, sizeof(double) * B);
  H2D(o_ph, phi, sizeof(double) * B);
  H2D(o_et, eps_top, sizeof(wb_complex) * B);
  H2D(o_eb, eps_bot, sizeof(wb_complex) * B);
  H2D(o_pol, pol, sizeof(wb_complex) * 2 * B);
  cudaMemsetAsync(dev + o_ast, 0, sizeof(int32_t), s);
  // stage A into (L, 3, N, N): assemble into three (L, N, N) planes, then interleave per layer
  wb_complex* conv = (wb_complex*)(dev + o_conv);
  int rc = WB_OK;
  {
    // assemble each slot plane contiguously, then regroup to (L, 3, N, N)
    wb_complex* planes = (wb_complex*)(dev + o_tmp);
    wb_complex* ex = planes;
    wb_complex* ey = planes + (size_t)L * NN;
    wb_complex* ez = planes + (size_t)2 * L * NN;
    rc = wb_assemble_li(h, (const wb_complex*)(dev + o_eps), L, ny, nx, hu, hv, ex, ey, ez,
                        (int32_t*)(dev + o_ast), s);
    if (rc == WB_OK) {
      wb::regroup_slots(s, L, N, (const cplx*)planes, (cplx*)conv);
      rc = cuda_check("wb_solve_host: regroup");
    }
  }
  if (rc == WB_OK)
    rc = wb_solve_batch(h, B, L, hu, hv, conv, (const int32_t*)(dev + o_li), (const double*)(dev + o_th),
                        (const double*)(dev + o_wl), (const double*)(dev + o_per), (const double*)(dev + o_th2),
                        (const double*)(dev + o_ph), (const wb_complex*)(dev + o_et), (const wb_complex*)(dev + o_eb),
                        (const wb_complex*)(dev + o_pol), (double*)(dev + o_R), (double*)(dev + o_T), nullptr,
                        (int32_t*)(dev + o_st), precision, s);
  if (rc == WB_OK) {
    cudaMemcpyAsync(R, dev + o_R, sizeof(double) * 3 * B * N, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(T, dev + o_T, sizeof(double) * 3 * B * N, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(status, dev + o_st, sizeof(int32_t) * B, cudaMemcpyDeviceToHost, s);
    int32_t ast = 0;
    cudaMemcpyAsync(&ast, dev + o_ast, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) rc = fail(WB_E_CUDA, "wb_solve_host: %s", cudaGetErrorString(e));
    else if (ast) for (int b = 0; b < B; ++b) status[b] |= ast;
  } else {
    cudaStreamSynchronize(s);   // nothing queued may still read the caller's host buffers
    cudaGetLastError();
  }
  return rc;
}

long long wb_kernel_launches(wb_handle* h) { (void)h; return wb::launch_count(); }

static_assert(WB_TUNE_QR_THREADS == wb::kTuneQrThreads && WB_TUNE_HRD_THREADS == wb::kTuneHrdThreads &&
                  WB_TUNE_LU_THREADS == wb::kTuneLuThreads && WB_TUNE_TENSOR_CORES == wb::kTuneTensorCores &&
                  WB_TUNE_HRD_BLOCKED == wb::kTuneHrdBlocked && WB_TUNE_COUNT == wb::kTuneKeys,
              "public and internal tuning keys agree");

int wb_set_tuning(int key, int value) {
  if (key < 0 || key >= WB_TUNE_COUNT) return fail(WB_E_INVALID, "wb_set_tuning: key %d outside [0, %d)", key, WB_TUNE_COUNT);
  if (value < 0) return fail(WB_E_INVALID, "wb_set_tuning: value %d < 0", value);
  wb::set_tuning(key, value);
  return WB_OK;
}

int wb_get_tuning(int key) { return (key >= 0 && key < WB_TUNE_COUNT) ? wb::tuning(key) : -1; }

long long wb_tensor_core_errors(void) { return wb::tc_errors(); }

int wb_profile_qr(int enable) {
  wb::qr_profile(enable != 0);
  return cuda_check("wb_profile_qr");
}

int wb_profile_qr_read(int real_type, double* ms, long long* launches, double* bytes) {
  if (!ms || !launches || !bytes) return fail(WB_E_INVALID, "wb_profile_qr_read: NULL argument");
  const int rc = wb::qr_profile_read(real_type, ms, launches, bytes);
  if (rc == 1) return fail(WB_E_INVALID, "wb_profile_qr_read: real type %d outside 0..2", real_type);
  if (rc == 2) return cuda_check("wb_profile_qr_read");
  return WB_OK;
}

}  // extern "C"
