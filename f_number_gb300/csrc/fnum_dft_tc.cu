// The band DFT on the Blackwell tensor cores (tcgen05 + TMA).
//
// Replaces the reference's cuFFT R2C of every RF line followed by the band
// selection (+cuda/gpu_bf_das_pw_rf.cu:917-925, +cuda/gpu_bf_saft_rf.cu:1031-1038):
// only the K band bins k_lb..k_ub of the order-N DFT are wanted, so the stage is
// the GEMM
//     S[signal][2k' + part] = sum_t x_signal(t) W[2k' + part][t],
//     W[2k'][t] + j W[2k'+1][t] = e^{-j 2 pi (k_lb + k') t / N},
// with the twiddle index (k t) mod N exact in integers and the twiddles of the
// FP64 table.  RF is first rounded to float (the reference's conversion,
// +cuda/gpu_bf_das_pw_rf.cu:787-793), then both operands are split into fp16
// hi + lo parts (RF scaled per line by a power of two into fp16 range) and the
// products hi.hi + hi.lo + lo.hi are accumulated in FP32 in tensor memory, which
// keeps about 22 bits of each operand: FP32-class spectra at tensor-core speed.
//
// Kernel: one CTA per 128 signals x 128 spectrum columns (64 bins), six warps.
// Warp 0 (one lane) streams 64-sample slices of the four operand tiles (A hi/lo,
// B hi/lo, 16 KB each, 128-byte swizzled) into a three-stage shared-memory ring
// with TMA; warp 1 (one lane) issues tcgen05.mma (M = 128, N = 128, K = 16, fp16
// in, fp32 accumulators in TMEM) and releases each stage with tcgen05.commit;
// warps 2-5 drain the accumulator.  The tensor cores' FP32 accumulation rounds
// toward zero, so a long chain of products into one accumulator drifts (4.1e-6 of
// the spectrum over 1024 samples, against 1.7e-7 for FP32 cuFFT); instead each
// stage's 12 products go into one of two TMEM accumulators, restarted from zero
// (the hi.lo and lo.hi products first, so that only the four hi.hi steps round a
// full-size sum), and the drain warps read it back
// with tcgen05.ld (warp w owns TMEM lanes 32 (w mod 4) .. +31, i.e. 32 signals)
// and add it to FP32 register sums, rounded to nearest, while the tensor cores
// fill the other accumulator.  The drain warps then write the spectra in the
// beamformers' layout.  Every wait on an mbarrier gives up after two seconds,
// records ERR_DFT_TIMEOUT in the error word and lets the CTA finish (free its
// TMEM) instead of spinning.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "fnum_internal.h"
#include "fnum_tc_ptx.cuh"

namespace fnum {

namespace {

constexpr int DT_BM = 128;                         // signals per tile = TMEM lanes
constexpr int DT_BN = 128;                         // spectrum columns per tile = TMEM columns
constexpr int DT_BK = 64;                          // samples per stage: one 128-byte fp16 row
constexpr int DT_STAGES = 3;
constexpr int DT_TILE_BYTES = DT_BM * DT_BK * 2;   // 16 KB (DT_BM == DT_BN)
constexpr int DT_STAGE_BYTES = 4 * DT_TILE_BYTES;  // A hi, A lo, B hi, B lo
constexpr int DT_SMEM = DT_STAGES * DT_STAGE_BYTES + 1024 + 128;   // + alignment slack + barriers
constexpr int DT_THREADS = 192;                    // producer, MMA issuer, four drain warps
constexpr int DT_TMEM_COLS = 2 * DT_BN;            // two accumulators

static_assert(DT_BM == DT_BN, "the four operand tiles share one size");

constexpr uint32_t DT_IDESC = tcx::idesc_f16(DT_BM, DT_BN);

using namespace tcx;

__device__ __forceinline__ void tc_mma_f16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate) {
  mma_f16(tmem_d, da, db, DT_IDESC, accumulate);
}

__device__ __forceinline__ void tc_commit(uint32_t bar) { mma_commit(bar); }

// ---------------------------------------------------------------------------
// operands
// ---------------------------------------------------------------------------
// One block per signal: x rounded to float, scaled by the power of two that brings
// max |x| below 2^14, split into fp16 hi and lo; samples nt..Kp-1 are zero.
template <typename T>
__global__ void __launch_bounds__(256) dft_tc_split_kernel(const T* __restrict__ rf, int nt, int Kp, size_t plane,
                                                           __half* __restrict__ a, float* __restrict__ inv_scale) {
  __shared__ float red[8];
  const int s = blockIdx.x;
  const T* x = rf + (size_t)s * nt;
  float m = 0.0f;
  for (int t = threadIdx.x; t < nt; t += blockDim.x) m = fmaxf(m, fabsf((float)x[t]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  m = red[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
  float sc = 1.0f;
  if (m > 0.0f && m < 3.0e38f) {
    int ex;
    frexpf(m, &ex);  // m < 2^ex
    sc = ldexpf(1.0f, min(max(14 - ex, -126), 126));
  }
  if (threadIdx.x == 0) inv_scale[s] = 1.0f / sc;
  __half2* hi = reinterpret_cast<__half2*>(a + (size_t)s * Kp);
  __half2* lo = reinterpret_cast<__half2*>(a + plane + (size_t)s * Kp);
  for (int p = threadIdx.x; p < Kp / 2; p += blockDim.x) {
    const int t = 2 * p;
    const float x0 = (t < nt) ? (float)x[t] * sc : 0.0f;
    const float x1 = (t + 1 < nt) ? (float)x[t + 1] * sc : 0.0f;
    const __half2 h = __floats2half2_rn(x0, x1);
    const float2 f = __half22float2(h);
    hi[p] = h;
    lo[p] = __floats2half2_rn(x0 - f.x, x1 - f.y);
  }
}

// B[n][t] (n = 2k' + part, part 0 the real, 1 the imaginary part of the twiddle
// e^{-j 2 pi (k_lb + k') t / N}) as fp16 hi and lo planes; zero for n >= 2K or t >= nt
__global__ void dft_tc_twiddle_kernel(const float2* __restrict__ tw, int N, int nt, int k_lb, int K, int Kp, int Np,
                                      __half* __restrict__ b) {
  const size_t plane = (size_t)Np * Kp;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < plane; i += (size_t)gridDim.x * blockDim.x) {
    const int n = (int)(i / Kp), t = (int)(i % Kp);
    float w = 0.0f;
    if (n < 2 * K && t < nt) {
      const float2 c = tw[((long long)(k_lb + n / 2) * t) % N];
      w = (n & 1) ? c.y : c.x;
    }
    const __half h = __float2half_rn(w);
    b[i] = h;
    b[plane + i] = __float2half_rn(w - __half2float(h));
  }
}

// ---------------------------------------------------------------------------
// the GEMM
// ---------------------------------------------------------------------------
struct DftOut {
  float2* X;
  const float* inv_scale;
  unsigned long long* err;
  int nsig, K, lo_n;
  long long s_hi, s_lo, s_k;   // X[(sig / lo_n) s_hi + (sig % lo_n) s_lo + k' s_k]
  int n_kb;                    // samples / DT_BK
};


__global__ void __launch_bounds__(DT_THREADS, 1)
dft_tc_gemm_kernel(const __grid_constant__ CUtensorMap tm_ahi, const __grid_constant__ CUtensorMap tm_alo,
                   const __grid_constant__ CUtensorMap tm_bhi, const __grid_constant__ CUtensorMap tm_blo,
                   const DftOut o) {
  extern __shared__ unsigned char dyn[];
  const uint32_t raw = smem_u32(dyn);
  const uint32_t base = (raw + 1023u) & ~1023u;                       // 128-byte swizzle wants 1024-B tiles
  unsigned char* gbase = dyn + (base - raw);
  uint64_t* bars = reinterpret_cast<uint64_t*>(gbase + DT_STAGES * DT_STAGE_BYTES);
  // bars: full[S], empty[S] (stage ring), accf[2], acce[2] (accumulators); then the TMEM
  // address and the abort flag
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * DT_STAGES + 4);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const uint32_t bar0 = smem_u32(bars);
  auto full = [&](int s) { return bar0 + 8u * (uint32_t)s; };
  auto empty = [&](int s) { return bar0 + 8u * (uint32_t)(DT_STAGES + s); };
  auto accf = [&](int j) { return bar0 + 8u * (uint32_t)(2 * DT_STAGES + j); };
  auto acce = [&](int j) { return bar0 + 8u * (uint32_t)(2 * DT_STAGES + 2 + j); };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * DT_BM, n0 = blockIdx.y * DT_BN;

  if (threadIdx.x == 0) {
    for (int s = 0; s < DT_STAGES; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int j = 0; j < 2; ++j) {
      mbar_init(accf(j), 1);
      mbar_init(acce(j), 128);   // every drain thread arrives
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(DT_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // producer: TMA into the stage ring
      for (int kb = 0; kb < o.n_kb; ++kb) {
        const int s = kb % DT_STAGES;
        const uint32_t ph = (uint32_t)(kb / DT_STAGES) & 1u;
        if (*abort_flag || !mbar_wait(empty(s), ph ^ 1u)) {
          *abort_flag = 1;
          break;
        }
        const uint32_t st = base + (uint32_t)s * DT_STAGE_BYTES;
        mbar_expect_tx(full(s), DT_STAGE_BYTES);
        tma_load_2d(st, &tm_ahi, kb * DT_BK, m0, full(s));
        tma_load_2d(st + DT_TILE_BYTES, &tm_alo, kb * DT_BK, m0, full(s));
        tma_load_2d(st + 2 * DT_TILE_BYTES, &tm_bhi, kb * DT_BK, n0, full(s));
        tma_load_2d(st + 3 * DT_TILE_BYTES, &tm_blo, kb * DT_BK, n0, full(s));
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer: per stage 4 k-steps x 3 products into accumulator kb mod 2, from zero
      for (int kb = 0; kb < o.n_kb; ++kb) {
        const int s = kb % DT_STAGES, j = kb & 1;
        const uint32_t ph = (uint32_t)(kb / DT_STAGES) & 1u;
        if (*abort_flag || !mbar_wait(full(s), ph) || !mbar_wait(acce(j), ((uint32_t)(kb >> 1) & 1u) ^ 1u)) {
          *abort_flag = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = base + (uint32_t)s * DT_STAGE_BYTES;
        const uint32_t acc = tmem + (uint32_t)(j * DT_BN);
        // descriptors once per stage; a k-step of 16 fp16 (32 bytes) adds 2 to the
        // start-address field
        const uint64_t dah = smem_desc(st), dal = smem_desc(st + DT_TILE_BYTES);
        const uint64_t dbh = smem_desc(st + 2 * DT_TILE_BYTES), dbl = smem_desc(st + 3 * DT_TILE_BYTES);
        // the small cross products first, so that only the four hi.hi steps round a
        // full-size accumulator
#pragma unroll
        for (int kk = 0; kk < DT_BK / 16; ++kk) {
          const uint64_t o = 2ull * (uint64_t)kk;
          tc_mma_f16(acc, dah + o, dbl + o, kk != 0);   // hi.lo
          tc_mma_f16(acc, dal + o, dbh + o, 1u);        // lo.hi
        }
#pragma unroll
        for (int kk = 0; kk < DT_BK / 16; ++kk) {
          const uint64_t o = 2ull * (uint64_t)kk;
          tc_mma_f16(acc, dah + o, dbh + o, 1u);        // hi.hi
        }
        tc_commit(empty(s));   // the stage is free once these products have read it
        tc_commit(accf(j));    // and the accumulator holds the stage's sums
      }
    }
  } else {
    // drain warps 2..5: TMEM lanes 32 (warp mod 4) .. +31 are their 32 signals
    const int q = warp & 3;
    const uint32_t lane_addr = (uint32_t)(32 * q) << 16;
    float sum[DT_BN];
#pragma unroll
    for (int c = 0; c < DT_BN; ++c) sum[c] = 0.0f;
    bool ok = true;
    for (int kb = 0; kb < o.n_kb; ++kb) {
      const int j = kb & 1;
      ok = __all_sync(0xffffffffu, !*abort_flag && mbar_wait(accf(j), (uint32_t)(kb >> 1) & 1u));
      if (!ok) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int c = 0; c < DT_BN / 32; ++c) {
        uint32_t v[32];
        tmem_ld32(tmem + lane_addr + (uint32_t)(j * DT_BN + 32 * c), v);
#pragma unroll
        for (int t = 0; t < 32; ++t) sum[32 * c + t] += __uint_as_float(v[t]);
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      mbar_arrive(acce(j));
    }
    if (!ok) {
      *abort_flag = 1;
      if (lane == 0) atomicOr(o.err, ERR_DFT_TIMEOUT);
    } else {
      const int sig = m0 + 32 * q + lane;
      if (sig < o.nsig) {
        const float isc = o.inv_scale[sig];
        float2* out = o.X + (long long)(sig / o.lo_n) * o.s_hi + (long long)(sig % o.lo_n) * o.s_lo;
#pragma unroll
        for (int t = 0; t < DT_BN / 2; ++t) {
          const int k = n0 / 2 + t;
          if (k < o.K) out[(long long)k * o.s_k] = make_float2(sum[2 * t] * isc, sum[2 * t + 1] * isc);
        }
      }
    }
  }
  __syncwarp();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DT_TMEM_COLS) : "memory");
  }
}

// 2-D fp16 map over rows x Kp (K-major), 64 x 128 boxes, 128-byte swizzle; rows
// beyond the matrix read as zero
bool encode_map(CUtensorMap* m, const void* base, int rows, int Kp) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  const cuuint32_t box[2] = {(cuuint32_t)DT_BK, (cuuint32_t)DT_BM};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

size_t dft_tc_bytes(int nsig, int nt, int K) {
  const size_t Kp = (size_t)((nt + DT_BK - 1) / DT_BK) * DT_BK;
  const size_t Np = (size_t)((2 * K + DT_BN - 1) / DT_BN) * DT_BN;
  return 2 * (size_t)nsig * Kp * 2 + 2 * Np * Kp * 2 + (size_t)nsig * sizeof(float);
}

cudaError_t dft_tc_setup(DftTc& d, int nsig, int nt, int N, int k_lb, int K, const float2* tw, void* a, void* b,
                         float* inv_scale, cudaStream_t s) {
  d.nsig = nsig;
  d.nt = nt;
  d.N = N;
  d.k_lb = k_lb;
  d.K = K;
  d.Kp = (nt + DT_BK - 1) / DT_BK * DT_BK;
  d.Np = (2 * K + DT_BN - 1) / DT_BN * DT_BN;
  d.a = a;
  d.b = b;
  d.inv_scale = inv_scale;
  const size_t aplane = (size_t)nsig * d.Kp, bplane = (size_t)d.Np * d.Kp;
  __half* ah = (__half*)a;
  __half* bh = (__half*)b;
  if (!encode_map(&d.tm[0], ah, nsig, d.Kp) || !encode_map(&d.tm[1], ah + aplane, nsig, d.Kp) ||
      !encode_map(&d.tm[2], bh, d.Np, d.Kp) || !encode_map(&d.tm[3], bh + bplane, d.Np, d.Kp))
    return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(dft_tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, DT_SMEM);
  if (e != cudaSuccess) return e;
  const size_t n = bplane;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 4096);
  dft_tc_twiddle_kernel<<<blocks, 256, 0, s>>>(tw, N, nt, k_lb, K, d.Kp, d.Np, bh);
  return cudaGetLastError();
}

cudaError_t dft_tc_run(const DftTc& d, const void* rf, int is_double, float2* X, int lo_n, long long s_hi,
                       long long s_lo, long long s_k, unsigned long long* err, cudaStream_t s) {
  const size_t aplane = (size_t)d.nsig * d.Kp;
  if (is_double)
    dft_tc_split_kernel<double><<<d.nsig, 256, 0, s>>>((const double*)rf, d.nt, d.Kp, aplane, (__half*)d.a,
                                                       d.inv_scale);
  else
    dft_tc_split_kernel<float><<<d.nsig, 256, 0, s>>>((const float*)rf, d.nt, d.Kp, aplane, (__half*)d.a,
                                                      d.inv_scale);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  DftOut o;
  o.X = X;
  o.inv_scale = d.inv_scale;
  o.err = err;
  o.nsig = d.nsig;
  o.K = d.K;
  o.lo_n = lo_n;
  o.s_hi = s_hi;
  o.s_lo = s_lo;
  o.s_k = s_k;
  o.n_kb = d.Kp / DT_BK;
  const dim3 grid((d.nsig + DT_BM - 1) / DT_BM, d.Np / DT_BN);
  dft_tc_gemm_kernel<<<grid, DT_THREADS, DT_SMEM, s>>>(d.tm[0], d.tm[1], d.tm[2], d.tm[3], o);
  return cudaGetLastError();
}

}  // namespace fnum
