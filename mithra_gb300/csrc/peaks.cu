// Device peak probe: the FP64 fused multiply-add rate of this GPU.
//
// The FP64 form of the time-marching loop is bound by the FP64 pipe on GB300 (its rate is a small
// fraction of the FP32 rate), so the bench places its dominant kernel against this measured
// rate rather than the nominal one.  Every thread runs kChains independent FMA chains (enough
// to cover the pipe's latency) for `iters` iterations; the result is written only when a
// runtime flag that is never set asks for it, so the chains are not removed by the compiler.
#include <cuda_runtime.h>

#include "../../include/mithra_gpu.h"

namespace {

constexpr int kChains = 8;
constexpr int kBlock = 256;

__global__ void __launch_bounds__(kBlock) k_dfma_probe(int iters, double seed, int write, double* out) {
  double a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) a[c] = seed + 1e-3 * (threadIdx.x + c);
  const double m = 1.0 - 1e-12, s = 1e-9;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = fma(a[c], m, s);
  }
  double t = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) t += a[c];
  if (write) out[blockIdx.x * kBlock + threadIdx.x] = t;
}

}  // namespace

extern "C" int mithra_probe_fp64_tflops(int device, double* tflops) {
  if (!tflops) return MITHRA_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return MITHRA_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MITHRA_ERR_CUDA;
  const int blocks = sms * 8, iters = 1 << 14;
  cudaStream_t st;
  cudaEvent_t e0, e1;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return MITHRA_ERR_CUDA;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma_probe<<<blocks, kBlock, 0, st>>>(iters, 1.0, 0, nullptr);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; rep++) {
    cudaEventRecord(e0, st);
    k_dfma_probe<<<blocks, kBlock, 0, st>>>(iters, 1.0 + rep, 0, nullptr);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  const cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  if (e != cudaSuccess) return MITHRA_ERR_CUDA;
  const double flop = 2.0 * kChains * (double)iters * blocks * kBlock;
  *tflops = flop / (best * 1e-3) / 1e12;
  return MITHRA_OK;
}
