// Internal launch wrappers shared by the translation units of libwbgpu.so (not the public ABI).
#pragma once
#include "wb_common.cuh"
#include "wb_num.cuh"

namespace wb {

// Kernel-launch accounting (every launch site in the library calls note_launch()).
void note_launch();
long long launch_count();

// Launch-shape tunables (process-wide; 0 = the library's own choice). Set through
// wb_set_tuning by the autotuner; read at every launch.
// (the same numbers as the public WB_TUNE_* keys)
enum TuneKey { kTuneQrThreads = 0, kTuneHrdThreads = 1, kTuneLuThreads = 2, kTuneTensorCores = 3, kTuneHrdBlocked = 4,
               kTuneKeys = 8 };
int tuning(int key);
void set_tuning(int key, int value);
// multiprocessor count of the current device (cached per device)
int sm_count();
// live timing of the QR-sweep launches (wb_eig.cu): on/off (clears), and per real type
// (0 double, 1 float, 2 df64) the summed event time, launches and algorithmic bytes
void qr_profile(bool on);
int qr_profile_read(int slot, double* ms, long long* launches, double* bytes);

// ---- dense linear algebra (wb_linalg.cu)
void zgemm(cudaStream_t s, int batch, int m, int n, int k, cplx alpha,
           const cplx* A, long long a_rs, long long a_cs, long long a_bs,
           const cplx* B, long long b_rs, long long b_cs, long long b_bs,
           cplx beta, cplx* C, long long c_rs, long long c_cs, long long c_bs);
// status (if non-null) of batch element e is status[e / st_div]
// zgemm with either operand conjugated on load (conj_a / conj_b); with transposed strides that is
// A^H or B^H without a copy
void zgemm_conj(cudaStream_t s, int batch, int m, int n, int k, cplx alpha, const cplx* A, long long a_rs,
                long long a_cs, long long a_bs, bool conj_a, const cplx* B, long long b_rs, long long b_cs,
                long long b_bs, bool conj_b, cplx beta, cplx* C, long long c_rs, long long c_cs, long long c_bs);
void zgetrf(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs, int* ipiv, long long piv_bs,
            int32_t* status, int st_div);
void zgetrs(cudaStream_t s, int batch, int n, const cplx* LU, int lda, long long a_bs,
            const int* ipiv, long long piv_bs, cplx* B, int nrhs, int ldb, long long b_bs, int trans);
void zset_identity(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs);
// C = alpha A B + beta C of FP64 operands with double-float accumulation on the FP32 pipes
// (about 2^-48 unit roundoff); A of batch entry z at A + (a_idx ? a_idx[z] : z) * a_bs
void zgemm_dd_idx(cudaStream_t s, int batch, int m, int n, int k, double2 alpha, const cplx* A, long long a_rs,
                  long long a_cs, long long a_bs, const int* a_idx, const cplx* B, long long b_rs, long long b_cs,
                  long long b_bs, double2 beta, cplx* C, long long c_rs, long long c_cs, long long c_bs);

// templated over R in {double, float, df64}; alpha/beta are passed as doubles
// complex FP32 products on the tensor cores (wb_tc.cu): false when not applicable (small
// shapes, switched off by WB_TUNE_TENSOR_CORES = 1); the count of CTAs that timed out
bool tc_cgemm(cudaStream_t s, int batch, int m, int n, int k, double2 alpha, const Cx<float>* A, long long a_rs,
              long long a_cs, long long a_bs, const Cx<float>* B, long long b_rs, long long b_cs, long long b_bs,
              double2 beta, Cx<float>* C, long long c_rs, long long c_cs, long long c_bs);
long long tc_errors();
template <class R>
void gemm(cudaStream_t s, int batch, int m, int n, int k, double2 alpha,
          const Cx<R>* A, long long a_rs, long long a_cs, long long a_bs,
          const Cx<R>* B, long long b_rs, long long b_cs, long long b_bs,
          double2 beta, Cx<R>* C, long long c_rs, long long c_cs, long long c_bs);
template <class R>
void gemm_idx(cudaStream_t s, int batch, int m, int n, int k, double2 alpha,
              const Cx<R>* A, long long a_rs, long long a_cs, long long a_bs, const int* a_idx,
              const Cx<R>* B, long long b_rs, long long b_cs, long long b_bs,
              double2 beta, Cx<R>* C, long long c_rs, long long c_cs, long long c_bs);
template <class R>
void getrf(cudaStream_t s, int batch, int n, Cx<R>* A, int lda, long long a_bs, int* ipiv, long long piv_bs,
           int32_t* status, int st_div);
template <class R>
void getrs(cudaStream_t s, int batch, int n, const Cx<R>* LU, int lda, long long a_bs, const int* ipiv,
           long long piv_bs, Cx<R>* B, int nrhs, int ldb, long long b_bs, int trans);
template <class R>
void set_identity(cudaStream_t s, int batch, int n, Cx<R>* A, int lda, long long a_bs);
template <class R1, class R2>
void convert(cudaStream_t s, const Cx<R1>* src, Cx<R2>* dst, long long count);

// ---- eigen-decomposition (wb_eig.cu)
void zgeev_schur(cudaStream_t s, int batch, int n, cplx* A, int lda, long long a_bs, cplx* Z, int ldz,
                 long long z_bs, cplx* w, cplx* tau, int32_t* status, int st_div);
void ztrevc(cudaStream_t s, int batch, int n, const cplx* T, int ldt, long long t_bs, cplx* X, int ldx,
            long long x_bs);
void znormalize_columns(cudaStream_t s, int batch, int n, cplx* W, int ldw, long long w_bs);

// ws (optional, batch stride ws_bs): scratch the FP32 form forms Q with in panels
template <class R>
void geev_schur(cudaStream_t s, int batch, int n, Cx<R>* A, int lda, long long a_bs, Cx<R>* Z, int ldz,
                long long z_bs, Cx<R>* w, Cx<R>* tau, int32_t* status, int st_div, Cx<R>* ws = nullptr,
                long long ws_bs = 0);
template <class R>
void trevc(cudaStream_t s, int batch, int n, const Cx<R>* T, int ldt, long long t_bs, Cx<R>* X, int ldx,
           long long x_bs);
template <class R>
void normalize_columns(cudaStream_t s, int batch, int n, Cx<R>* W, int ldw, long long w_bs);

// ---- order windows
// The largest windows the kernels hold on chip: stage A inverts an (2hv+1)^2 Toeplitz matrix
// beside its identity in one block's shared memory (32 (2hv+1)^2 bytes <= 227 KB: hv <= 42), and
// the eigen-solve keeps vectors of n = 2N complex values in shared memory (36 n bytes for the
// mixed form's group step: N <= 3228).
inline bool orders_fit(int hu, int hv) {
  return hu >= 0 && hv >= 0 && hv <= 42 && hu <= 1613 && (2LL * hu + 1) * (2LL * hv + 1) <= 3228;
}

// ---- stage A: convolution matrices (wb_assemble.cu)
// eps: (L, ny, nx) row-major raster; outputs (L, N, N) column-major; scratch from `ws`.
// x_edges (L, nx) and y_edges (L, ny), both NULL for sampled coefficients: the right edges of
// the column / row segments of compressed rasters, for integrated coefficients.
size_t assemble_workspace_bytes(int L, int ny, int nx, int hu, int hv);
void assemble_li(cudaStream_t s, const cplx* eps, int L, int ny, int nx, int hu, int hv,
                 cplx* epx, cplx* epy, cplx* epz_i, void* ws, int32_t* status,
                 const double* x_edges = nullptr, const double* y_edges = nullptr);

}  // namespace wb
