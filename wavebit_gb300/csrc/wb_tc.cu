// Host side of the tensor-core complex products (wb_tc.cuh): the dispatch that gemm<float> tries
// first, and the error counter of timed-out CTAs.
#include "wb_tc.cuh"
#include "wb_kernels.h"

namespace wb {

bool tc_cgemm(cudaStream_t s, int batch, int m, int n, int k, double2 alpha, const Cx<float>* A, long long a_rs,
              long long a_cs, long long a_bs, const Cx<float>* B, long long b_rs, long long b_cs, long long b_bs,
              double2 beta, Cx<float>* C, long long c_rs, long long c_cs, long long c_bs) {
  if (tuning(kTuneTensorCores) == 1) return false;          // switched off
  if (batch <= 0 || m < tc::kTileM || n < 64 || k < tc::kKb) return false;   // small: the SIMT kernel
  if (cudaFuncSetAttribute(tc::cgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kSmemBytes) !=
      cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  dim3 grid((m + tc::kTileM - 1) / tc::kTileM, (n + tc::kTileN - 1) / tc::kTileN, batch);
  tc::cgemm_kernel<<<grid, tc::kThreads, tc::kSmemBytes, s>>>(
      m, n, k, make_float2((float)alpha.x, (float)alpha.y), make_float2((float)beta.x, (float)beta.y), A, a_rs, a_cs,
      a_bs, B, b_rs, b_cs, b_bs, C, c_rs, c_cs, c_bs);
  note_launch();
  return true;
}

long long tc_errors() {
  unsigned int v = 0;
  if (cudaMemcpyFromSymbol(&v, tc::g_tc_error, sizeof(v)) != cudaSuccess) { cudaGetLastError(); return -1; }
  return (long long)v;
}

}  // namespace wb
