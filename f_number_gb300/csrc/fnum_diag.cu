// Diagnostics: FP32 FMA throughput of the device, the denominator of the
// fused kernels' roofline (they are bound by FP32 issue, not by HBM), and the
// throughput of the warp-level mma.sync m16n8k16 (fp16 in, fp32 accumulate)
// that the tensor-core plane-wave kernel issues.
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

constexpr int MMA_CHAINS = 8;

__global__ void __launch_bounds__(256) mma_chains_kernel(float* out, int iters) {
  const unsigned a0 = 0x3c003c00u + (threadIdx.x & 7), a1 = 0x38003800u, a2 = 0x34003400u, a3 = 0x30003000u;
  const unsigned b0 = 0x1c001c00u, b1 = 0x18001800u;
  float d[MMA_CHAINS][4];
#pragma unroll
  for (int j = 0; j < MMA_CHAINS; ++j) d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.0f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < MMA_CHAINS; ++j)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                   "{%0,%1,%2,%3};\n"
                   : "+f"(d[j][0]), "+f"(d[j][1]), "+f"(d[j][2]), "+f"(d[j][3])
                   : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < MMA_CHAINS; ++j) s += d[j][0] + d[j][1] + d[j][2] + d[j][3];
  if (s == 123.456f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// best of four timed launches after one warm-up; returns ms or < 0 on error
template <typename L>
float time_best(L launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return cudaGetLastError() == cudaSuccess ? best : -1.0f;
}

}  // namespace

extern "C" int fnum_diag_mma_f16_peak(int device, double* tflops) {
  if (!tflops) return FNUM_ERR_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_INVALID_DEVICE;
  }
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
  const int blocks = nsm * 4, threads = 256, iters = 2048;
  float* out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_OUT_OF_MEMORY;
  }
  const float ms = time_best([&] { mma_chains_kernel<<<blocks, threads>>>(out, iters); });
  cudaFree(out);
  if (ms <= 0.0f) return FNUM_ERR_CUDA;
  const double flops = 2.0 * 16 * 8 * 16 * (double)MMA_CHAINS * iters * blocks * (threads / 32);
  *tflops = flops / (ms * 1e-3) / 1e12;
  return FNUM_OK;
}

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
