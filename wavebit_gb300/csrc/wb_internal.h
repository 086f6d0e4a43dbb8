// Host-side internal types of libwbgpu.so: the workspace arena, the solve descriptor.
#pragma once
#include <cstddef>
#include "wb_common.cuh"

namespace wb {

// Bump allocator over one device buffer owned by the handle. get<T>(count) returns nullptr
// (and latches !ok()) when the buffer is exhausted; reset() rewinds it.
struct Arena {
  char* base = nullptr;
  size_t cap = 0, off = 0;
  bool failed = false;
  void reset() { off = 0; failed = false; }
  template <class T> T* get(size_t count) {
    size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
    if (failed || off + bytes > cap) { failed = true; return nullptr; }
    T* p = reinterpret_cast<T*>(base + off);
    off += bytes;
    return p;
  }
  bool ok() const { return !failed; }
};

// Per-solve vectors over the retained orders (N) or the s/p boundary basis (n = 2N).
struct PortVectors {
  double *kx, *ky, *c, *s;                 // (B, N)
  cplx *kz_top, *kz_bot;                   // (B, N)
  cplx *wg, *vg;                           // (B, n) gap W / V diagonals
  cplx *r11, *r12, *r21, *r22;             // (B, n) superstrate -> gap S blocks (diagonal)
  cplx *t11, *t21;                         // (B, n) gap -> substrate S blocks used
  cplx *nt, *nb;                           // (B) half-space indices
};

// Everything is a device pointer. Layers are listed entry face first (the superstrate side).
struct SolveDesc {
  int n_solves, n_layers, hu, hv;
  const cplx* conv;            // (n_conv, 3, N, N) column-major slots epx, epy, epz_i
  const int* layer_index;      // (B, L) index into conv
  const double* thickness;     // (B, L)
  const double* wavelength;    // (B)
  const double* period;        // (B, 2)
  const double* theta;         // (B)
  const double* phi;           // (B)
  const cplx* eps_top;         // (B)
  const cplx* eps_bot;         // (B)
  const cplx* pol;             // (B, 2) (a_s, a_p)
};

struct SolveOut {
  double* R;                   // (B, 3, N): given polarization, pure s, pure p
  double* T;                   // (B, 3, N)
  cplx* amps;                  // (B, 3, 4, N) r_s, r_p, t_s, t_p or nullptr
  int32_t* status;             // (B)
};

size_t solve_chunk_bytes(int N, int L, int chunk, int precision);
size_t layer_modes_bytes(int N, int n_pairs, int precision);
// precision 0: FP64 eigen-solve; 1: FP32 eigen-solve refined by Newton steps; others: double-float.
// Returns -1 when the arena cannot hold the scratch.
int layer_modes(cudaStream_t s, Arena& ar, int n_pairs, int N, const cplx* conv, const int* pair_layer,
                const double* kx, const double* ky, cplx* w, cplx* q, cplx* W, cplx* V, int32_t* status,
                int precision);
// (3 planes of L) (N, N) slots -> (L, 3, N, N)
void regroup_slots(cudaStream_t s, int L, int N, const cplx* planes, cplx* out);
int solve_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, int first, int count, const SolveOut& out,
                int precision);
// The stack's scattering matrix at the half-space ports from given modes (wb_scattering_matrix):
// S11..S22 (B, n, n) column-major, centre frame.
size_t scattering_chunk_bytes(int N, int L, int chunk);
int scattering_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* W, const cplx* V, const cplx* q,
                     int first, int count, cplx* S11, cplx* S12, cplx* S21, cplx* S22, int32_t* status);
// The ETM connecting algorithm from given modes (wb_etm_solve), FP64; outputs as solve_chunk.
size_t etm_chunk_bytes(int N, int L, int chunk);
int etm_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* W, const cplx* V, const cplx* q,
              int first, int count, const SolveOut& out);
// Every layer's mode amplitudes for k incidence columns (wb_layer_amplitudes), FP64: Cin (B, n, k);
// plus / minus_top / minus_bottom (B, L, n, k); cref / ctrn (B, n, k); all column-major per block.
size_t amplitudes_chunk_bytes(int N, int L, int chunk, int k);
int amplitudes_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* W, const cplx* V, const cplx* q,
                     const cplx* Cin, int k, int first, int count, cplx* plus, cplx* minus_top, cplx* minus_bottom,
                     cplx* cref, cplx* ctrn, int32_t* status);
// Reverse passes (wb_vjp.cu), FP64. Each returns -1 when the arena cannot hold one chunk.
// Stage B: P pairs; the slot cotangents gconv (n_conv, 3, N, N) are overwritten.
size_t layer_modes_vjp_bytes(int N, int P);
int layer_modes_vjp_chunk(int P, int N, size_t budget);
int layer_modes_vjp_run(cudaStream_t s, Arena& ar, size_t budget, int P, int N, int n_conv, const cplx* conv,
                        const int* pair_layer, const double* kx, const double* ky, const cplx* w, const cplx* q,
                        const cplx* W, const cplx* V, const cplx* gw, const cplx* gq, const cplx* gW, const cplx* gV,
                        cplx* gconv, int32_t* status);
// Stage C: the cotangents of W, V (B*L, n, n), q (B*L, n) and the thicknesses (B, L) from those
// of R and T (B, 3, N), through the FP64 cascade recomputed with its tape.
size_t smm_vjp_bytes(int N, int L, int Bc);
int smm_vjp_chunk(int B, int N, int L, size_t budget);
int smm_vjp_run(cudaStream_t s, Arena& ar, size_t budget, const SolveDesc& d, const cplx* W, const cplx* V,
                const cplx* q, const double* gR, const double* gT, cplx* gW, cplx* gV, cplx* gq, double* g_thick,
                int32_t* status);
// Stage A (sampled coefficients): the rasters' cotangents from those of the three slots.
size_t assemble_vjp_bytes(int L, int ny, int nx, int hu, int hv);
int assemble_vjp_run(cudaStream_t s, Arena& ar, int L, int ny, int nx, int hu, int hv, const cplx* eps,
                     const cplx* epx, const cplx* epz, const cplx* gepx, const cplx* gepy, const cplx* gepz,
                     cplx* g_eps, int32_t* status);
size_t smm_chunk_bytes(int N, int L, int chunk, int precision);
int smm_chunk(cudaStream_t s, Arena& ar, const SolveDesc& d, const cplx* W, const cplx* V, const cplx* q,
              int first, int count, const SolveOut& out, int precision);

}  // namespace wb
