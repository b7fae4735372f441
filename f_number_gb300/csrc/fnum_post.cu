// Post-processing of beamformed images on the device: coherent compounding
// over angles and log compression to B-mode decibels.  The reference does
// both on the host after the beamformer (examples.m:78 sums the per-angle
// images; examples.m:88,96 display 20 log10(|I| / max |I|)).
#include <math.h>
#include <stdint.h>

#include "../../include/fnum.h"
#include "fnum_internal.h"

namespace {

constexpr int POST_THREADS = 256;

// |sum over images| per voxel -> mag, and the largest magnitude -> *max_bits
// (non-negative floats order like their bit patterns, so an integer atomicMax
// on the bits is a float max)
__global__ void __launch_bounds__(POST_THREADS)
compound_magnitude_kernel(const float2* __restrict__ img, long long n, int n_images, float* __restrict__ mag,
                          unsigned int* __restrict__ max_bits) {
  __shared__ float red[POST_THREADS / 32];
  float local = 0.0f;
  for (long long i = (long long)blockIdx.x * POST_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * POST_THREADS) {
    float re = 0.0f, im = 0.0f;
    for (int a = 0; a < n_images; ++a) {
      const float2 v = img[(size_t)a * n + i];
      re += v.x;
      im += v.y;
    }
    const float m = hypotf(re, im);
    mag[i] = m;
    local = fmaxf(local, m);
  }
  for (int o = 16; o > 0; o >>= 1) local = fmaxf(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.0f;
    for (int w = 0; w < POST_THREADS / 32; ++w) m = fmaxf(m, red[w]);
    atomicMax(max_bits, __float_as_uint(m));
  }
}

// mag -> 20 log10(mag / max), clamped below at floor_db (an all-zero image
// gives floor_db everywhere)
__global__ void __launch_bounds__(POST_THREADS)
log_compress_kernel(float* __restrict__ db, long long n, const unsigned int* __restrict__ max_bits, float floor_db) {
  const float mx = __uint_as_float(*max_bits);
  const float inv = (mx > 0.0f) ? 1.0f / mx : 0.0f;
  for (long long i = (long long)blockIdx.x * POST_THREADS + threadIdx.x; i < n;
       i += (long long)gridDim.x * POST_THREADS) {
    const float v = (mx > 0.0f) ? 20.0f * log10f(db[i] * inv) : floor_db;
    db[i] = fmaxf(v, floor_db);
  }
}

int grid_for(long long n) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n + POST_THREADS - 1) / POST_THREADS;
  const long long cap = (long long)(nsm > 0 ? nsm : 1) * 8;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

}  // namespace

extern "C" int fnum_bmode(const void* d_image, long long n_voxels, int n_images, float floor_db, float* d_db,
                          float* d_max_abs, void* stream) {
  if (!d_image || !d_db || !d_max_abs || n_voxels <= 0 || n_images <= 0) return FNUM_ERR_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  const int grid = grid_for(n_voxels);
  unsigned int* max_bits = reinterpret_cast<unsigned int*>(d_max_abs);
  cudaError_t e = cudaMemsetAsync(max_bits, 0, sizeof(unsigned int), st);
  if (e == cudaSuccess) {
    compound_magnitude_kernel<<<grid, POST_THREADS, 0, st>>>((const float2*)d_image, n_voxels, n_images, d_db,
                                                             max_bits);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    log_compress_kernel<<<grid, POST_THREADS, 0, st>>>(d_db, n_voxels, max_bits, floor_db);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_CUDA;
  }
  return FNUM_OK;
}
