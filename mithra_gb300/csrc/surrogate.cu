// Learned surrogate of FEL runs: BF16 tensor-core GEMMs (tc_gemm.cuh) and the kernels of a small
// MLP trained on the device.  This file: the GEMM entry point.
#include <cuda_runtime.h>

#include "../../include/mithra_gpu.h"
#include "tc_gemm.cuh"

using namespace mithra;

extern "C" int mithra_tc_gemm(const void* A, const void* B, float* C, void* C_bf16, const float* bias, int M, int N,
                              int K, int act, void* stream, int* err_dev) {
  if (!A || !B || (!C && !C_bf16) || !err_dev || M <= 0 || N <= 0 || K <= 0) return MITHRA_ERR_ARG;
  if (M % tc::BM || N % tc::BN || K % tc::BK) return MITHRA_ERR_ARG;
  if (((uintptr_t)A | (uintptr_t)B) & 15) return MITHRA_ERR_ARG;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(tc::k_gemm_bf16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::kGemmSmem) !=
        cudaSuccess)
      return MITHRA_ERR_CUDA;
    attr = true;
  }
  dim3 grid(M / tc::BM, N / tc::BN);
  tc::k_gemm_bf16<<<grid, 128, tc::kGemmSmem, (cudaStream_t)stream>>>(
      (const __nv_bfloat16*)A, (const __nv_bfloat16*)B, C, (__nv_bfloat16*)C_bf16, bias, M, N, K, act, err_dev);
  return cudaGetLastError() == cudaSuccess ? MITHRA_OK : MITHRA_ERR_CUDA;
}
