// wb_assemble_li_noalloc: stage-A assembly for callers that cannot allocate device memory.
//
// Some hosts of this library run where a cudaMalloc is not allowed or not safe: code that
// executes while another component is capturing a CUDA graph, inference servers and plugins
// whose host owns the whole device pool and forbids allocations from inside a request, and
// allocation-free real-time paths that must not hit the driver's allocator (which can
// synchronise the device). For them this entry point keeps its scratch in a fixed,
// file-scope device array instead of the handle's arena, and needs no handle at all. The
// caller still passes the raster and the three output slabs.
//
// The array is WB_NOALLOC_SCRATCH_BYTES (32 MiB) and every GPU that loads libwbgpu.so holds
// it until the process exits. Layers are assembled one at a time through it, so the limit is
// per layer: assemble_workspace_bytes(1, ny, nx, hu, hv) must fit (a 256x256 raster fits up to
// orders (14, 14), about 30 MiB; (15, 15) needs about 38 MiB). Larger requests are refused with
// WB_E_INVALID before any GPU work.
//
// All calls share the one array and each leaves its contents behind. Nothing in it has to start
// at zero: every scratch entry the assembly reads it has written earlier in the same call. Calls
// that overlap on the GPU (on different streams, or from different host threads) race on the
// array; the caller must order them.
#include <cstdio>
#include <mutex>
#include "../../include/wavebit_gb300.h"
#include "wb_common.cuh"
#include "wb_kernels.h"

namespace {
constexpr size_t WB_NOALLOC_SCRATCH_BYTES = size_t(32) << 20;
constexpr int WB_NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[WB_NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
void* g_scratch_ptr[WB_NOALLOC_MAX_DEVICES] = {nullptr};

// The array's name is only a host-side stand-in; the kernels need its device address, which
// the runtime gives once per device with that device current.
int scratch_for_current_device(void** out, char* msg, size_t len) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    snprintf(msg, len, "wb_assemble_li_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
    return WB_E_CUDA;
  }
  if (dev < 0 || dev >= WB_NOALLOC_MAX_DEVICES) {
    snprintf(msg, len, "wb_assemble_li_noalloc: device %d beyond the supported %d", dev, WB_NOALLOC_MAX_DEVICES);
    return WB_E_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      snprintf(msg, len, "wb_assemble_li_noalloc: cudaGetSymbolAddress on device %d: %s", dev,
               cudaGetErrorString(e));
      cudaGetLastError();
      return WB_E_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return WB_OK;
}
}  // namespace

namespace wb {
int noalloc_fail(const char* msg);   // wb_api.cu: records the thread's last error
}

extern "C" size_t wb_assemble_li_noalloc_limit(void) { return WB_NOALLOC_SCRATCH_BYTES; }

extern "C" int wb_assemble_li_noalloc(const wb_complex* eps, int L, int ny, int nx, int hu, int hv,
                                      wb_complex* epx, wb_complex* epy, wb_complex* epz_i, int32_t* status,
                                      void* stream) {
  char msg[256];
  if (!eps || !epx || !epy || !epz_i) return wb::noalloc_fail("wb_assemble_li_noalloc: NULL argument"), WB_E_INVALID;
  if (L <= 0 || ny <= 0 || nx <= 0 || !wb::orders_fit(hu, hv)) {
    snprintf(msg, sizeof(msg), "wb_assemble_li_noalloc: bad sizes L=%d ny=%d nx=%d orders=(%d,%d)", L, ny, nx, hu, hv);
    wb::noalloc_fail(msg);
    return WB_E_INVALID;
  }
  const size_t need = wb::assemble_workspace_bytes(1, ny, nx, hu, hv);
  if (need > WB_NOALLOC_SCRATCH_BYTES) {
    snprintf(msg, sizeof(msg),
             "wb_assemble_li_noalloc: one %dx%d layer at orders (%d,%d) needs %zu bytes of scratch; the fixed "
             "scratch holds %zu bytes (use wb_assemble_li with a handle)", ny, nx, hu, hv, need,
             WB_NOALLOC_SCRATCH_BYTES);
    wb::noalloc_fail(msg);
    return WB_E_INVALID;
  }
  void* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch, msg, sizeof(msg));
  if (rc != WB_OK) { wb::noalloc_fail(msg); return rc; }
  cudaStream_t s = (cudaStream_t)stream;
  const long long N = (long long)(2 * hu + 1) * (2 * hv + 1), NN = N * N, plane = (long long)ny * nx;
  for (int l = 0; l < L; ++l)
    wb::assemble_li(s, (const cplx*)eps + l * plane, 1, ny, nx, hu, hv, (cplx*)epx + l * NN, (cplx*)epy + l * NN,
                    (cplx*)epz_i + l * NN, scratch, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "wb_assemble_li_noalloc: %s", cudaGetErrorString(e));
    wb::noalloc_fail(msg);
    return WB_E_CUDA;
  }
  return WB_OK;
}
