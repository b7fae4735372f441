// Diagnostics: FP32 FMA throughput of the device, the denominator of the
// fused kernel's roofline (that kernel is bound by the FP32 pipe, not by HBM
// or the tensor cores).
#include <cuda_runtime.h>

#include "../../include/fnum.h"

namespace {

constexpr int CHAINS = 8;

__global__ void __launch_bounds__(256) fma_chains_kernel(float* out, int iters, float b, float c) {
  float a[CHAINS];
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) a[j] = threadIdx.x * 1e-3f + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int j = 0; j < CHAINS; ++j) a[j] = fmaf(a[j], b, c);
    }
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < CHAINS; ++j) s += a[j];
  if (s == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

extern "C" int fnum_diag_fp32_peak(int device, double* tflops) {
  if (!tflops) return FNUM_ERR_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_INVALID_DEVICE;
  }
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  const int blocks = nsm * 8, threads = 256, iters = 4096;
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_OUT_OF_MEMORY;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    fma_chains_kernel<<<blocks, threads>>>(out, iters, 0.9999f, 1e-4f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return FNUM_ERR_CUDA;
  const double flops = 2.0 * CHAINS * 4.0 * iters * (double)blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return FNUM_OK;
}
