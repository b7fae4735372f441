// GB300 (sm_103a) kernels of the Fourier-domain delay-and-sum beamformer.
//
// Stages (reference counterparts in the f_number project):
//   twiddles_kernel      table e^{-2 pi i m / N}, m < N (FP64 sincospi, rounded to float)
//   dft_band_kernel      RF -> band spectra, only bins k_lb..k_ub
//                        (replaces cufftPlan1d/cufftExecR2C, +cuda/gpu_bf_das_pw_rf.cu:917-925);
//                        float RF goes through one SGEMM against dft_matrix_kernel's
//                        twiddle matrix instead (host side)
//   pw_fused_kernel      one voxel per thread; replaces das_kernel_distances_pw,
//                        das_kernel_phase_shifts, the per-bin cublasCgemm and
//                        das_kernel_normalization (+cuda/gpu_bf_das_pw_rf.cu:965-1057)
//   pw_event_kernel      the same recurrence with the segment boundaries resolved ahead
//                        of the bin loop
//   pw_tc_kernel         the same image from per-bin [voxels x elements] . [elements x
//                        angles] products on the tensor cores (mma.sync, fp16 hi/lo)
//   sa_fused_kernel      the recurrence for synthetic-aperture data
//                        (+cuda/gpu_bf_saft_rf.cu:1144-1201, saft_kernel_phase_shifts.cu)
//   sa_event_kernel      the same for a boxcar receive window, boundaries resolved ahead
//   pw_plain_kernel / sa_plain_kernel
//                        one voxel per thread with the reference's FP32 arithmetic per term
//                        (__sincosf, float geometry): the plain drop-in baseline.
//
// Fused-kernel algorithm.  For a voxel v the image is
//   I(v) = (2/N) sum_k (1/W_k) sum_e a_{e,k} X_e(k) z_e^k,   z_e = e^{j 2 pi u_e},
// u_e = (d_tx + d_rx,e) f_s / (N c) + t0 / N in cycles per bin.  The apertures
// (and so a_{e,k} and W_k) change only at a few "segment" boundaries along k,
// computed once per voxel and kept in scratch.  Per element the sum over k is
// a Horner recurrence run from the top bin down:  A <- A z + X_k  (4 FMA per
// term).  At a boundary where the weight b = a/W changes from b_old to b_new
// the accumulator is rescaled by b_old / b_new; it is flushed (multiplied by
// b e^{j 2 pi k u} and added to the voxel) every flush_chunks * KCHUNK bins to
// bound the phase drift of the recurrence.  u_e is formed in double-float
// arithmetic and every exponential e^{j 2 pi k u} is reduced exactly to
// [-1/2, 1/2] cycles before sincospif, so FP32 only carries the final phasor.
// The plane-wave pre-pass sums each aperture's window in closed form (the
// elements are equally spaced), and the spectrum chunks are double-buffered
// in shared memory with cp.async so the next chunk loads during the current one.
#include "fnum_device.cuh"
#include "fnum_internal.h"

#include <cuda_fp16.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include <mutex>

namespace fnum {


// ---------------------------------------------------------------------------
// twiddles and the band DFT
// ---------------------------------------------------------------------------
__global__ void twiddles_kernel(float2* tw, int N) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < N) {
    double s, c;
    sincospi(2.0 * (double)m / (double)N, &s, &c);
    tw[m] = make_float2((float)c, (float)(-s));
  }
}

// One block per signal.  X[k] = sum_t x(t) e^{-j 2 pi k t / N} for k = k_lb..k_lb+K-1;
// the twiddle index (k t) mod N is carried exactly in integers.
constexpr int DFT_THREADS = 256;
constexpr int DFT_BINS = 4;

template <typename T>
__global__ void __launch_bounds__(DFT_THREADS)
dft_band_kernel(const T* __restrict__ rf, int nt, const float2* __restrict__ tw, int N, int k_lb, int K,
                float2* __restrict__ X, int out_stride_k, int out_stride_sig_hi, int out_stride_sig_lo,
                int sig_lo_count) {
  extern __shared__ float sig[];
  const int s = blockIdx.x;
  const T* x = rf + (size_t)s * nt;
  for (int t = threadIdx.x; t < nt; t += DFT_THREADS) sig[t] = (float)x[t];
  __syncthreads();
  const int s_hi = s / sig_lo_count, s_lo = s % sig_lo_count;
  float2* out = X + (size_t)s_hi * out_stride_sig_hi + (size_t)s_lo * out_stride_sig_lo;
  for (int kb = threadIdx.x * DFT_BINS; kb < K; kb += DFT_THREADS * DFT_BINS) {
    int kk[DFT_BINS], m[DFT_BINS];
    float re[DFT_BINS], im[DFT_BINS], re2[DFT_BINS], im2[DFT_BINS];
#pragma unroll
    for (int b = 0; b < DFT_BINS; ++b) {
      kk[b] = min(k_lb + kb + b, k_lb + K - 1);
      m[b] = 0;
      re[b] = im[b] = re2[b] = im2[b] = 0.0f;
    }
    int t = 0;
    for (; t + 1 < nt; t += 2) {
      const float x0 = sig[t], x1 = sig[t + 1];
#pragma unroll
      for (int b = 0; b < DFT_BINS; ++b) {
        const float2 w0 = __ldg(&tw[m[b]]);
        m[b] += kk[b];
        if (m[b] >= N) m[b] -= N;
        const float2 w1 = __ldg(&tw[m[b]]);
        m[b] += kk[b];
        if (m[b] >= N) m[b] -= N;
        re[b] = fmaf(x0, w0.x, re[b]);
        im[b] = fmaf(x0, w0.y, im[b]);
        re2[b] = fmaf(x1, w1.x, re2[b]);
        im2[b] = fmaf(x1, w1.y, im2[b]);
      }
    }
    if (t < nt) {
      const float x0 = sig[t];
#pragma unroll
      for (int b = 0; b < DFT_BINS; ++b) {
        const float2 w0 = __ldg(&tw[m[b]]);
        re[b] = fmaf(x0, w0.x, re[b]);
        im[b] = fmaf(x0, w0.y, im[b]);
      }
    }
#pragma unroll
    for (int b = 0; b < DFT_BINS; ++b) {
      if (kb + b < K) out[(size_t)(kb + b) * out_stride_k] = make_float2(re[b] + re2[b], im[b] + im2[b]);
    }
  }
}

cudaError_t launch_twiddles(float2* tw, int N, cudaStream_t s) {
  twiddles_kernel<<<(N + 255) / 256, 256, 0, s>>>(tw, N);
  return cudaGetLastError();
}

static cudaError_t dft_launch(const void* rf, int is_double, int nsig, int nt, const float2* tw, int N, int k_lb,
                              int K, float2* X, int sk, int shi, int slo, int nlo, cudaStream_t s) {
  const size_t smem = (size_t)nt * sizeof(float);
  if (smem > 48 * 1024) {
    cudaError_t e = is_double ? cudaFuncSetAttribute(dft_band_kernel<double>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                              : cudaFuncSetAttribute(dft_band_kernel<float>,
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  if (is_double)
    dft_band_kernel<double><<<nsig, DFT_THREADS, smem, s>>>((const double*)rf, nt, tw, N, k_lb, K, X, sk, shi,
                                                             slo, nlo);
  else
    dft_band_kernel<float><<<nsig, DFT_THREADS, smem, s>>>((const float*)rf, nt, tw, N, k_lb, K, X, sk, shi, slo,
                                                            nlo);
  return cudaGetLastError();
}

// PW: signal s = a * ne + e  ->  X[e][k][a]
cudaError_t launch_dft_pw(const void* rf, int is_double, int na, int ne, int nt, const float2* tw, int N, int k_lb,
                          int K, float2* X, cudaStream_t s) {
  return dft_launch(rf, is_double, na * ne, nt, tw, N, k_lb, K, X, /*k*/ na, /*hi=a*/ 1, /*lo=e*/ K * na, ne, s);
}
// SA: signal s = tx * ne + rx  ->  X[s][k]
cudaError_t launch_dft_sa(const void* rf, int is_double, int nsig, int nt, const float2* tw, int N, int k_lb, int K,
                          float2* X, cudaStream_t s) {
  return dft_launch(rf, is_double, nsig, nt, tw, N, k_lb, K, X, 1, 0, K, nsig, s);
}

// complex image -> separate real and imaginary planes (the MEX output layout)
__global__ void split_complex_kernel(const float2* __restrict__ in, size_t n, float* __restrict__ re,
                                     float* __restrict__ im) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float2 v = in[i];
    re[i] = v.x;
    im[i] = v.y;
  }
}
cudaError_t launch_split_complex(const float2* in, size_t n, float* re, float* im, cudaStream_t s) {
  split_complex_kernel<<<608, 256, 0, s>>>(in, n, re, im);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// fused plane-wave kernel
// ---------------------------------------------------------------------------
// aperture sum of one bin in closed form: left elements ilb .. emid-1 lie at
// x - c_e = l0 + j pitch (j counted from emid-1 outwards), right elements
// emid .. iub at c_e - x = l0 + j pitch (j counted from emid)
template <int WIN>
__device__ float aperture_sum_closed(const PWDev& d, float inv_par, dfl xm, int emid, int ilb, int iub,
                                     float invLl, float invLr) {
  float W = 0.0f;
  if (ilb < emid && invLl > 0.0f) {
    const dfl c = d.el_m[emid - 1];
    W += win_sum<WIN>((xm.x - c.x) + (xm.y - c.y), d.pitch_f, emid - ilb, invLl, d.window_par, inv_par);
  }
  if (iub >= emid && invLr > 0.0f) {
    const dfl c = d.el_m[emid];
    W += win_sum<WIN>((c.x - xm.x) + (c.y - xm.y), d.pitch_f, iub - emid + 1, invLr, d.window_par, inv_par);
  }
  return W;
}

// Segment pre-pass of one voxel: walks the band from the top bin down and
// writes one int4 per aperture change,
//   {k_start, i_lb | (i_ub+1) << 16, 1/W, (1/W of the previous segment) / (1/W)}.
// Also registers, per element, the highest bin at which it is active anywhere
// in the block (ktop) and the block's element range.
template <int WIN>
__device__ int pw_build_segments(const PWDev& d, float inv_par, int ic, int jc, bool valid, int4* seg, int* ktop,
                                 int* e_range, float& W_top, unsigned long long& n_active,
                                 unsigned long long& n_empty) {
  W_top = 0.0f;
  if (!valid) {
    seg[0] = make_int4(-1, seg_code(d.ne, -1), 0, 0);
    return 0;
  }
  const dfl xp = d.col_p[ic], zp = d.row_p[jc], xm = d.col_m[ic];
  const int emid = d.col_emid[ic];
  int nseg = 0, prev = -1, u_lo = d.ne, u_hi = -1, act = 0;
  float invW_prev = 0.0f;
  for (int kk = d.K - 1; kk >= 0; --kk) {
    int ilb, iub;
    aperture(xp, zp, d.g[kk], d.ne, ilb, iub);
    const int code = seg_code(ilb, iub);
    if (code != prev) {
      const float Ll = half_left(d.el_lb, xm, ilb, d.ne), Lr = half_right(d.el_ub, xm, iub);
      const float invLl = (Ll > 0.0f) ? 1.0f / Ll : 0.0f, invLr = (Lr > 0.0f) ? 1.0f / Lr : 0.0f;
      const float W = aperture_sum_closed<WIN>(d, inv_par, xm, emid, ilb, iub, invLl, invLr);
      const float invW = (W > 0.0f) ? (d.norm ? 1.0f / W : 1.0f) : 0.0f;
      const float wr = (invW > 0.0f) ? invW_prev / invW : 0.0f;
      if (nseg < d.seg_cap - 1)
        seg[nseg] = make_int4(kk + d.k_lb, code, __float_as_int(invW), __float_as_int(wr));
      else
        atomicOr(&d.counters[2], ERR_SEG_OVERFLOW);
      if (nseg == 0) W_top = W;
      ++nseg;
      prev = code;
      invW_prev = invW;
      const int lo = min(ilb, emid), hi = max(iub, emid - 1);
      act = (W > 0.0f) ? max(hi - lo + 1, 0) : 0;
      if (lo <= hi) {
        for (int e = lo; e <= hi && e < u_lo; ++e) atomicMax(&ktop[e], kk + d.k_lb);
        for (int e = max(u_hi + 1, lo); e <= hi; ++e) atomicMax(&ktop[e], kk + d.k_lb);
        u_lo = min(u_lo, lo);
        u_hi = max(u_hi, hi);
      }
    }
    if (act > 0) n_active += (unsigned long long)act; else n_empty += 1ull;
  }
  if (u_lo <= u_hi) {
    atomicMin(&e_range[0], u_lo);
    atomicMax(&e_range[1], u_hi);
  }
  // a sentinel after the last entry lets the recurrence prefetch entries
  // without testing the list length (its bin, -1, is never reached)
  nseg = min(nseg, d.seg_cap - 1);
  seg[nseg] = make_int4(-1, seg_code(d.ne, -1), 0, 0);
  return nseg;
}

// last segment whose k_start >= kt (entries sorted by k_start, descending)
__device__ __forceinline__ int seg_find1(const int4* seg, int nseg, int kt) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg[mid].x >= kt) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// asynchronous 8-byte global -> shared copy (completes at cp_async_wait_all)
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
// asynchronous 4-byte global -> shared copy
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Issues the copy of one spectrum chunk (bins kc_lo .. kc_lo + nk - 1 of
// elements e0 .. e0 + EPT - 1, angles a0 .. a0 + NA - 1) into a shared buffer
// laid out [bin][element][angle] with rows of ROW float2.
template <int EPT, int NA>
__device__ __forceinline__ void pw_stage_chunk(float2* dst, const PWDev& d, int e0, int a0, int kc_lo, int nk,
                                               int tid) {
  constexpr int CH = EPT * NA;
  constexpr int ROW = (CH + 1) & ~1;
  for (int t = tid; t < nk * CH; t += NTHREADS) {
    const int kk = t / CH, r = t - kk * CH, q = r / NA, a = r - q * NA;
    const int e = e0 + q, aa = a0 + a;
    float2* dp = &dst[kk * ROW + r];
    if (e < d.ne && aa < d.na)
      cp_async8(dp, &d.X[((size_t)e * d.K + (kc_lo - d.k_lb + kk)) * d.x_na + d.x_a0 + aa]);
    else
      *dp = make_float2(0.0f, 0.0f);
  }
  cp_async_commit();
}

constexpr int SEG_RING = 2;  // segment entries prefetched ahead of the recurrence

template <int EPT, int NA, int WIN>
__global__ void __launch_bounds__(NTHREADS, 4)
pw_fused_kernel(const PWDev d, float2* __restrict__ image, float* __restrict__ weights, int n_tiles_x,
                int n_tiles_z) {
  constexpr int CH = EPT * NA;
  constexpr int ROW = (CH + 1) & ~1;
  __shared__ __align__(16) float2 xs[2][KCHUNK * ROW];   // double-buffered spectrum chunks
  __shared__ dfl utx_s[NA][NTHREADS];     // transmit phase per angle, cycles per bin
  __shared__ int e_range[2];
  __shared__ int s_tile;
  extern __shared__ __align__(16) unsigned char dyn[];  // lb[ne], ub[ne] (dfl), ktop[ne]
  dfl* lb_s = (dfl*)dyn;
  dfl* ub_s = lb_s + d.ne;
  int* ktop = (int*)(ub_s + d.ne);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_tiles = n_tiles_x * n_tiles_z;
  int4* seg = d.seg + ((size_t)blockIdx.x * NTHREADS + tid) * (size_t)d.seg_cap * PW_SEG_INT4;
  const float inv_par = (d.window_par > 0.0f) ? 1.0f / d.window_par : 0.0f;
  unsigned long long n_active = 0, n_empty = 0, n_exec = 0;
  for (int e = tid; e < d.ne; e += NTHREADS) {
    lb_s[e] = d.el_lb[e];
    ub_s[e] = d.el_ub[e];
  }

  for (;;) {
    if (tid == 0) s_tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < d.ne; e += NTHREADS) ktop[e] = -1;
    if (tid == 0) {
      e_range[0] = d.ne;
      e_range[1] = -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    int tx, tz;
    tile_coords(tile, n_tiles_x, n_tiles_z, tx, tz);
    const int i = tx * TILE_X + warp;
    const int j = tz * TILE_Z + lane;
    const bool valid = (i < d.nx) && (j < d.nz);
    const int ic = min(i, d.nx - 1), jc = min(j, d.nz - 1);

    float W_top;
    const int nseg = pw_build_segments<WIN>(d, inv_par, ic, jc, valid, seg, ktop, e_range, W_top, n_active, n_empty);
    __syncthreads();
    const int E_lo = e_range[0], E_hi = e_range[1];

    const dfl xm = d.col_m[ic];
    const dfl xu = d.col_u[ic];
    const dfl zu2 = d.row_u2[jc];
    const int emid = d.col_emid[ic];
    float2 acc = make_float2(0.0f, 0.0f), comp = make_float2(0.0f, 0.0f);  // Kahan

    for (int a0 = 0; a0 < d.na; a0 += NA) {
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        const int aa = min(a0 + a, d.na - 1);
        utx_s[a][tid] = df_add(d.tx_ax[(size_t)aa * d.nx + ic], d.tx_az[(size_t)aa * d.nz + jc]);
      }
      for (int e0 = E_lo; e0 <= E_hi; e0 += EPT) {
        int kt = -1;
#pragma unroll
        for (int q = 0; q < EPT; ++q)
          if (e0 + q <= E_hi) kt = max(kt, ktop[e0 + q]);
        if (kt < d.k_lb) continue;
        if (tid == 0) n_exec += (unsigned long long)(kt - d.k_lb + 1) * CH * NTHREADS;

        float dxa[EPT], aw[EPT], b[EPT];
        dfl urx[EPT];
        float2 z[EPT][NA], A[EPT][NA];
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
          const int e = min(e0 + q, d.ne - 1);
          const dfl cm = d.el_m[e];
          dxa[q] = fabsf((cm.x - xm.x) + (cm.y - xm.y));
          urx[q] = df_sqrt(df_add(df_sqr(df_sub(d.el_u[e], xu)), zu2));
#pragma unroll
          for (int a = 0; a < NA; ++a) {
            z[q][a] = cis_ku(1, df_add(urx[q], utx_s[a][tid]));
            A[q][a] = make_float2(0.0f, 0.0f);
          }
        }
        // segment cursor at kt and the prefetch ring of the following entries
        int s = 0, code = seg_code(d.ne, -1);
        int4 ring[SEG_RING];
#pragma unroll
        for (int r = 0; r < SEG_RING; ++r) ring[r] = make_int4(-1, code, 0, 0);
        if (nseg > 0) {
          s = seg_find1(seg, nseg, kt);
          const int4 c0 = seg[s];
          code = c0.y;
          const int ilb = code_ilb(code), iub = code_iub(code);
          const int lo = min(ilb, emid), hi = max(iub, emid - 1);
          const float invW = __int_as_float(c0.z);
#pragma unroll
          for (int q = 0; q < EPT; ++q) {
            const int e = e0 + q;
            const bool left = e < emid;
            const bool act = (e >= lo) && (e <= hi) && (e <= E_hi);
            aw[q] = act ? win_t<WIN>(d.window_par, inv_par,
                                     dxa[q] * inv_half_width(lb_s, ub_s, xm, left, ilb, iub))
                        : 0.0f;
            b[q] = aw[q] * invW;
          }
#pragma unroll
          for (int r = 0; r < SEG_RING; ++r) ring[r] = seg[min(s + 1 + r, nseg)];
        } else {
#pragma unroll
          for (int q = 0; q < EPT; ++q) aw[q] = b[q] = 0.0f;
        }
        float2 part = make_float2(0.0f, 0.0f);

        // Chunks run from the one holding kt down to chunk 0.  The copy of the
        // next chunk is in flight while the current one is consumed.
        const int c_top = (kt - d.k_lb) / KCHUNK;
        __syncthreads();  // every thread is done with both buffers of the previous pass
        pw_stage_chunk<EPT, NA>(xs[0], d, e0, a0, d.k_lb + c_top * KCHUNK, kt - (d.k_lb + c_top * KCHUNK) + 1, tid);
        int buf = 0;
        for (int chunk = c_top; chunk >= 0; --chunk) {
          const int kc_lo = d.k_lb + chunk * KCHUNK;
          const int kc_hi = (chunk == c_top) ? kt : kc_lo + KCHUNK - 1;
          cp_async_wait_all();
          __syncthreads();  // the chunk is visible; the other buffer is free
          if (chunk > 0) pw_stage_chunk<EPT, NA>(xs[buf ^ 1], d, e0, a0, kc_lo - KCHUNK, KCHUNK, tid);
          const float2* xb = xs[buf];
          buf ^= 1;
          for (int k = kc_hi; k >= kc_lo; --k) {
            if (k == ring[0].x) {
              // enter the next segment at bin k
              const int pilb = code_ilb(code), piub = code_iub(code);
              code = ring[0].y;
              const float invW = __int_as_float(ring[0].z), wr = __int_as_float(ring[0].w);
#pragma unroll
              for (int r = 0; r + 1 < SEG_RING; ++r) ring[r] = ring[r + 1];
              ++s;
              ring[SEG_RING - 1] = seg[min(s + SEG_RING, nseg)];
              const int ilb = code_ilb(code), iub = code_iub(code);
              const int lo = min(ilb, emid), hi = max(iub, emid - 1);
#pragma unroll
              for (int q = 0; q < EPT; ++q) {
                const int e = e0 + q;
                const bool left = e < emid;
                const bool act = (e >= lo) && (e <= hi) && (e <= E_hi);
                const float bo = b[q];
                float r = wr;
                if (act) {
                  if ((left ? (ilb != pilb) : (iub != piub)) || bo == 0.0f) {
                    const float an = win_t<WIN>(d.window_par, inv_par,
                                              dxa[q] * inv_half_width(lb_s, ub_s, xm, left, ilb, iub));
                    r = __fdividef(aw[q], an) * wr;
                    aw[q] = an;
                  }
                } else {
                  aw[q] = 0.0f;
                }
                const float bn = aw[q] * invW;
                if (bn != 0.0f && bo != 0.0f) {
#pragma unroll
                  for (int a = 0; a < NA; ++a) {
                    A[q][a].x *= r;
                    A[q][a].y *= r;
                  }
                } else {
                  if (bo != 0.0f) {  // leaves the aperture below k+1: flush at k+1
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                      const float2 t = cmul(cis_ku(k + 1, df_add(urx[q], utx_s[a][tid])), A[q][a]);
                      part.x = fmaf(bo, t.x, part.x);
                      part.y = fmaf(bo, t.y, part.y);
                    }
                  }
#pragma unroll
                  for (int a = 0; a < NA; ++a) A[q][a] = make_float2(0.0f, 0.0f);
                }
                b[q] = bn;
              }
            }
            const float2* xr = &xb[(k - kc_lo) * ROW];
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
#pragma unroll
              for (int a = 0; a < NA; ++a) {
                const float2 x = xr[q * NA + a];
                const float2 Aq = A[q][a], zq = z[q][a];
                A[q][a].x = fmaf(Aq.x, zq.x, fmaf(-Aq.y, zq.y, x.x));
                A[q][a].y = fmaf(Aq.x, zq.y, fmaf(Aq.y, zq.x, x.y));
              }
            }
          }
          if (chunk % d.flush_chunks == 0) {
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
              if (b[q] != 0.0f) {
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                  const float2 t = cmul(cis_ku(kc_lo, df_add(urx[q], utx_s[a][tid])), A[q][a]);
                  part.x = fmaf(b[q], t.x, part.x);
                  part.y = fmaf(b[q], t.y, part.y);
                }
              }
#pragma unroll
              for (int a = 0; a < NA; ++a) A[q][a] = make_float2(0.0f, 0.0f);
            }
          }
        }
        // compensated accumulation of this element group's contribution
        {
          float y = part.x - comp.x, t = acc.x + y;
          comp.x = (t - acc.x) - y;
          acc.x = t;
          y = part.y - comp.y;
          t = acc.y + y;
          comp.y = (t - acc.y) - y;
          acc.y = t;
        }
      }
    }
    if (valid) {
      image[(size_t)ic * d.nz + jc] = make_float2(acc.x * d.scale, acc.y * d.scale);
      if (weights) weights[(size_t)ic * d.nz + jc] = W_top;
    }
    __syncthreads();
  }
  // terms are counted per angle
  n_active *= (unsigned long long)d.na;
  n_empty *= (unsigned long long)d.na;
  atomicAdd(&d.counters[0], n_active);
  atomicAdd(&d.counters[1], n_empty);
  if (tid == 0) atomicAdd(&d.counters[4], n_exec);
}

// Plane-wave recurrence with the segment boundaries resolved ahead of the bin
// loop.  Each lane walks its own boundaries of the next EVB bins and writes,
// per bin that carries one and per element of the pass, one value into a
// table in shared memory (a column per lane):
//   v > 0   the element stays in the aperture: rescale its accumulators by v
//   v == 0  it enters the aperture (or stays out): clear them
//   v < 0   it leaves the aperture: flush them with the weight -v, then clear
// plus a bit mask of the bins that carry a boundary.  The bin loop applies a
// table entry only where this lane has one, so a warp spends per bin of a
// boundary a load and a multiply instead of the window evaluation.  The
// arithmetic is that of pw_fused_kernel, which gives the same images.
template <int EPT, int NA, int WIN>
__global__ void __launch_bounds__(NTHREADS, 4)
pw_event_kernel(const PWDev d, float2* __restrict__ image, float* __restrict__ weights, int n_tiles_x,
                int n_tiles_z) {
  constexpr int CH = EPT * NA;
  constexpr int ROW = (CH + 1) & ~1;
  constexpr int EVB = (EPT <= 2) ? 32 : 16;   // bins per boundary table
  __shared__ __align__(16) float2 xs[2][KCHUNK * ROW];
  __shared__ dfl utx_s[NA][NTHREADS];
  __shared__ float ev[EVB][EPT][NTHREADS];
  __shared__ int e_range[2];
  __shared__ int s_tile;
  extern __shared__ __align__(16) unsigned char dyn[];  // lb[ne], ub[ne] (dfl), ktop[ne]
  dfl* lb_s = (dfl*)dyn;
  dfl* ub_s = lb_s + d.ne;
  int* ktop = (int*)(ub_s + d.ne);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_tiles = n_tiles_x * n_tiles_z;
  int4* seg = d.seg + ((size_t)blockIdx.x * NTHREADS + tid) * (size_t)d.seg_cap * PW_SEG_INT4;
  const float inv_par = (d.window_par > 0.0f) ? 1.0f / d.window_par : 0.0f;
  unsigned long long n_active = 0, n_empty = 0, n_exec = 0;
  for (int e = tid; e < d.ne; e += NTHREADS) {
    lb_s[e] = d.el_lb[e];
    ub_s[e] = d.el_ub[e];
  }

  for (;;) {
    if (tid == 0) s_tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < d.ne; e += NTHREADS) ktop[e] = -1;
    if (tid == 0) {
      e_range[0] = d.ne;
      e_range[1] = -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    int tx, tz;
    tile_coords(tile, n_tiles_x, n_tiles_z, tx, tz);
    const int i = tx * TILE_X + warp;
    const int j = tz * TILE_Z + lane;
    const bool valid = (i < d.nx) && (j < d.nz);
    const int ic = min(i, d.nx - 1), jc = min(j, d.nz - 1);

    float W_top;
    const int nseg = pw_build_segments<WIN>(d, inv_par, ic, jc, valid, seg, ktop, e_range, W_top, n_active, n_empty);
    __syncthreads();
    const int E_lo = e_range[0], E_hi = e_range[1];

    const dfl xm = d.col_m[ic];
    const dfl xu = d.col_u[ic];
    const dfl zu2 = d.row_u2[jc];
    const int emid = d.col_emid[ic];
    float2 acc = make_float2(0.0f, 0.0f), comp = make_float2(0.0f, 0.0f);  // Kahan

    for (int a0 = 0; a0 < d.na; a0 += NA) {
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        const int aa = min(a0 + a, d.na - 1);
        utx_s[a][tid] = df_add(d.tx_ax[(size_t)aa * d.nx + ic], d.tx_az[(size_t)aa * d.nz + jc]);
      }
      for (int e0 = E_lo; e0 <= E_hi; e0 += EPT) {
        int kt = -1;
#pragma unroll
        for (int q = 0; q < EPT; ++q)
          if (e0 + q <= E_hi) kt = max(kt, ktop[e0 + q]);
        if (kt < d.k_lb) continue;
        if (tid == 0) n_exec += (unsigned long long)(kt - d.k_lb + 1) * CH * NTHREADS;

        // pre-pass state: element distance, window value and weight b = a / W
        float dxa[EPT], aw[EPT], b[EPT];
        dfl urx[EPT];
        float2 z[EPT][NA], A[EPT][NA];
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
          const int e = min(e0 + q, d.ne - 1);
          const dfl cm = d.el_m[e];
          dxa[q] = fabsf((cm.x - xm.x) + (cm.y - xm.y));
          urx[q] = df_sqrt(df_add(df_sqr(df_sub(d.el_u[e], xu)), zu2));
#pragma unroll
          for (int a = 0; a < NA; ++a) {
            z[q][a] = cis_ku(1, df_add(urx[q], utx_s[a][tid]));
            A[q][a] = make_float2(0.0f, 0.0f);
          }
        }
        int s = 0, code = seg_code(d.ne, -1);
        int4 ring[SEG_RING];
#pragma unroll
        for (int r = 0; r < SEG_RING; ++r) ring[r] = make_int4(-1, code, 0, 0);
        if (nseg > 0) {
          s = seg_find1(seg, nseg, kt);
          const int4 c0 = seg[s];
          code = c0.y;
          const int ilb = code_ilb(code), iub = code_iub(code);
          const int lo = min(ilb, emid), hi = max(iub, emid - 1);
          const float invW = __int_as_float(c0.z);
#pragma unroll
          for (int q = 0; q < EPT; ++q) {
            const int e = e0 + q;
            const bool left = e < emid;
            const bool act = (e >= lo) && (e <= hi) && (e <= E_hi);
            aw[q] = act ? win_t<WIN>(d.window_par, inv_par,
                                     dxa[q] * inv_half_width(lb_s, ub_s, xm, left, ilb, iub))
                        : 0.0f;
            b[q] = aw[q] * invW;
          }
#pragma unroll
          for (int r = 0; r < SEG_RING; ++r) ring[r] = seg[min(s + 1 + r, nseg)];
        } else {
#pragma unroll
          for (int q = 0; q < EPT; ++q) aw[q] = b[q] = 0.0f;
        }
        float2 part = make_float2(0.0f, 0.0f);

        const int c_top = (kt - d.k_lb) / KCHUNK;
        __syncthreads();  // every thread is done with both buffers of the previous pass
        pw_stage_chunk<EPT, NA>(xs[0], d, e0, a0, d.k_lb + c_top * KCHUNK, kt - (d.k_lb + c_top * KCHUNK) + 1, tid);
        int buf = 0;
        for (int chunk = c_top; chunk >= 0; --chunk) {
          const int kc_lo = d.k_lb + chunk * KCHUNK;
          const int kc_hi = (chunk == c_top) ? kt : kc_lo + KCHUNK - 1;
          cp_async_wait_all();
          __syncthreads();  // the chunk is visible; the other buffer is free
          if (chunk > 0) pw_stage_chunk<EPT, NA>(xs[buf ^ 1], d, e0, a0, kc_lo - KCHUNK, KCHUNK, tid);
          const float2* xb = xs[buf];
          buf ^= 1;
          for (int ks_hi = kc_hi; ks_hi >= kc_lo; ks_hi -= EVB) {
            const int ks_lo = max(kc_lo, ks_hi - (EVB - 1));
            // this lane's boundaries in bins ks_lo .. ks_hi (the sentinel's bin -1 ends the walk)
            unsigned emask = 0u;
            while (ring[0].x >= ks_lo) {
              const int kb = ring[0].x;
              const int pilb = code_ilb(code), piub = code_iub(code);
              code = ring[0].y;
              const float invW = __int_as_float(ring[0].z), wr = __int_as_float(ring[0].w);
#pragma unroll
              for (int r = 0; r + 1 < SEG_RING; ++r) ring[r] = ring[r + 1];
              ++s;
              ring[SEG_RING - 1] = seg[min(s + SEG_RING, nseg)];
              const int ilb = code_ilb(code), iub = code_iub(code);
              const int lo = min(ilb, emid), hi = max(iub, emid - 1);
#pragma unroll
              for (int q = 0; q < EPT; ++q) {
                const int e = e0 + q;
                const bool left = e < emid;
                const bool act = (e >= lo) && (e <= hi) && (e <= E_hi);
                const float bo = b[q];
                float r = wr;
                if (act) {
                  if ((left ? (ilb != pilb) : (iub != piub)) || bo == 0.0f) {
                    const float an = win_t<WIN>(d.window_par, inv_par,
                                              dxa[q] * inv_half_width(lb_s, ub_s, xm, left, ilb, iub));
                    r = __fdividef(aw[q], an) * wr;
                    aw[q] = an;
                  }
                } else {
                  aw[q] = 0.0f;
                }
                const float bn = aw[q] * invW;
                ev[kb - ks_lo][q][tid] = (bn != 0.0f && bo != 0.0f) ? r : ((bo != 0.0f) ? -bo : 0.0f);
                b[q] = bn;
              }
              emask |= 1u << (kb - ks_lo);
            }
            int nev = emask ? ks_lo + 31 - __clz(emask) : -1;
            for (int k = ks_hi; k >= ks_lo; --k) {
              if (k == nev) {
#pragma unroll
                for (int q = 0; q < EPT; ++q) {
                  const float v = ev[k - ks_lo][q][tid];
                  if (v < 0.0f) {  // leaves the aperture below k+1: flush at k+1
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                      const float2 t = cmul(cis_ku(k + 1, df_add(urx[q], utx_s[a][tid])), A[q][a]);
                      part.x = fmaf(-v, t.x, part.x);
                      part.y = fmaf(-v, t.y, part.y);
                    }
                  }
                  const bool keep = v > 0.0f;
#pragma unroll
                  for (int a = 0; a < NA; ++a) {
                    A[q][a].x = keep ? A[q][a].x * v : 0.0f;
                    A[q][a].y = keep ? A[q][a].y * v : 0.0f;
                  }
                }
                emask &= ~(1u << (k - ks_lo));
                nev = emask ? ks_lo + 31 - __clz(emask) : -1;
              }
              const float2* xr = &xb[(k - kc_lo) * ROW];
#pragma unroll
              for (int q = 0; q < EPT; ++q) {
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                  const float2 x = xr[q * NA + a];
                  const float2 Aq = A[q][a], zq = z[q][a];
                  A[q][a].x = fmaf(Aq.x, zq.x, fmaf(-Aq.y, zq.y, x.x));
                  A[q][a].y = fmaf(Aq.x, zq.y, fmaf(Aq.y, zq.x, x.y));
                }
              }
            }
          }
          if (chunk % d.flush_chunks == 0) {
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
              if (b[q] != 0.0f) {
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                  const float2 t = cmul(cis_ku(kc_lo, df_add(urx[q], utx_s[a][tid])), A[q][a]);
                  part.x = fmaf(b[q], t.x, part.x);
                  part.y = fmaf(b[q], t.y, part.y);
                }
              }
#pragma unroll
              for (int a = 0; a < NA; ++a) A[q][a] = make_float2(0.0f, 0.0f);
            }
          }
        }
        {
          float y = part.x - comp.x, t = acc.x + y;
          comp.x = (t - acc.x) - y;
          acc.x = t;
          y = part.y - comp.y;
          t = acc.y + y;
          comp.y = (t - acc.y) - y;
          acc.y = t;
        }
      }
    }
    if (valid) {
      image[(size_t)ic * d.nz + jc] = make_float2(acc.x * d.scale, acc.y * d.scale);
      if (weights) weights[(size_t)ic * d.nz + jc] = W_top;
    }
    __syncthreads();
  }
  n_active *= (unsigned long long)d.na;
  n_empty *= (unsigned long long)d.na;
  atomicAdd(&d.counters[0], n_active);
  atomicAdd(&d.counters[1], n_empty);
  if (tid == 0) atomicAdd(&d.counters[4], n_exec);
}

// ---------------------------------------------------------------------------
// plane-wave kernel on the tensor cores
// ---------------------------------------------------------------------------
// Per bin k the compounded image gains
//   sum_a t_{v,a}^k G_k(v, a),   G_k(v, a) = sum_e R_k(v, e) X_k(e, a),
//   R_k(v, e) = b_{v,e,k} r_{v,e}^k,
// with r = e^{j 2 pi u_rx}, t = e^{j 2 pi u_tx} and b the apodization weight
// a / W.  G_k is a [voxels x elements] . [elements x angles] product per bin,
// run with warp-level mma.sync m16n8k16 (fp16 operands, fp32 accumulators) in
// real form,
//   [Rr Ri] . [[Xr Xi], [-Xi Xr]] = [Gr Gi],
// 16 voxels x 8 complex elements x 4 complex angles per instruction.  Each
// fp32 operand is split into fp16 hi + lo (the spectra scaled by a power of
// two into fp16 range) and hi.hi + hi.lo + lo.hi is accumulated, which keeps
// about 22 bits.  The transmit phases are applied by a Horner recurrence over
// bins per (voxel, angle) inside the accumulators, H <- H t + G_k, flushed with
// the exact phase at the end of every TC_TB bins, where the receive phasors
// r^k are also re-anchored exactly.  The weights b enter R bin by bin, so a
// segment boundary costs nothing in the recurrence: the per-(voxel, bin)
// aperture data (inverse half-widths, 1/W) come from the segment lists through a
// table in shared memory that lanes 0..15 of each warp fill ahead of the bins.
constexpr int TC_WARPS = NTHREADS / 32;
constexpr int TC_TB = 32;   // bins per flush and receive-phasor re-anchoring (at most; PWDev::tc_tb may pick 16)
constexpr int TC_TT = 16;   // bins per aperture table

__device__ __forceinline__ void tc_split(float x0, float x1, unsigned& hi, unsigned& lo) {
  const __half2 h = __floats2half2_rn(x0, x1);
  const float2 f = __half22float2(h);
  const __half2 l = __floats2half2_rn(x0 - f.x, x1 - f.y);
  hi = *reinterpret_cast<const unsigned*>(&h);
  lo = *reinterpret_cast<const unsigned*>(&l);
}

// the same split with the residual from sm_100's mixed-precision FMA: lo = x - hi
// in one instruction per value (fp16 source, fp32 result; x - hi is exact, so the
// halves are those of tc_split)
__device__ __forceinline__ void tc_split_mx(float x0, float x1, unsigned& hi, unsigned& lo) {
  asm("{\n\t.reg .b16 h0, h1, m;\n\t.reg .f32 l0, l1;\n\t"
      "cvt.rn.f16x2.f32 %0, %3, %2;\n\t"
      "mov.b32 {h0, h1}, %0;\n\t"
      "mov.b16 m, 0xBC00;\n\t"
      "fma.rn.f32.f16 l0, h0, m, %2;\n\t"
      "fma.rn.f32.f16 l1, h1, m, %3;\n\t"
      "cvt.rn.f16x2.f32 %1, l1, l0;\n\t}"
      : "=&r"(hi), "=r"(lo)
      : "f"(x0), "f"(x1));
}

// D += A B for one m16n8k16 tile (row-major A, column-major B, fp32 accumulators)
__device__ __forceinline__ void tc_mma(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// largest |component| of the band spectra of the launch's angles (float bits; >= 0 floats order as ints)
__global__ void __launch_bounds__(256) tc_absmax_kernel(const PWDev d, unsigned* out) {
  const size_t n = (size_t)d.ne * d.K * d.na;
  float m = 0.0f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t a = i % d.na, ek = i / d.na;
    const float2 x = d.X[ek * d.x_na + d.x_a0 + a];
    m = fmaxf(m, fmaxf(fabsf(x.x), fabsf(x.y)));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}


// B fragments of the spectra: for angle pass ap (nt n-tiles of 4 angles), bin kk, element
// group s (elements 8s .. 8s+7), n-tile j (angles ap*4nt + 4j .. +3) and lane (g = lane/4,
// q = lane%4):
//   b0 = {B[2q][g], B[2q+1][g]}, b1 = {B[2q+8][g], B[2q+9][g]} as fp16 hi, then lo,
// with rows 0..7 the Rr rows and 8..15 the Ri rows of the group's elements and
// column g = 2 (angle) + (0: Gr, 1: Gi).
__global__ void __launch_bounds__(256) tc_prep_kernel(const PWDev d, int n_ap, int nt) {
  const size_t n = (size_t)n_ap * d.K * d.tc_S * nt * 32;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float sigma = tc_scale(*d.tc_max);
  const int lane = (int)(i & 31);
  size_t r = i >> 5;
  const int j = (int)(r % nt);
  r /= nt;
  const int s = (int)(r % d.tc_S);
  r /= d.tc_S;
  const int kk = (int)(r % d.K);
  const int ap = (int)(r / d.K);
  const int g = lane >> 2, q = lane & 3;
  const int a = ap * 4 * nt + 4 * j + (g >> 1), part = g & 1;
  float rr[2], ri[2];
#pragma unroll
  for (int t = 0; t < 2; ++t) {
    const int e = 8 * s + 2 * q + t;
    float2 x = make_float2(0.0f, 0.0f);
    if (e < d.ne && a < d.na) x = d.X[((size_t)e * d.K + kk) * d.x_na + d.x_a0 + a];
    x.x *= sigma;
    x.y *= sigma;
    rr[t] = part ? x.y : x.x;
    ri[t] = part ? x.x : -x.y;
  }
  uint4 o;
  tc_split(rr[0], rr[1], o.x, o.z);
  tc_split(ri[0], ri[1], o.y, o.w);
  d.tc_B[i] = o;
}

// Shared memory of pw_tc_kernel's tile body.
struct TcShared {
  float4 apt[TC_WARPS][TC_TT][16];   // {segment index (int bits), 1/L_left, 1/L_right, 1/W} per bin, voxel
  int e_range[2];
  int s_nseg[TC_WARPS * 16];
  // table builders' state (entry in effect, next segment entry, its index) and the
  // threads' compensated sums per voxel, kept out of registers
  float4 b_ent[TC_WARPS * 16];
  int4 b_next[TC_WARPS * 16];
  int b_idx[TC_WARPS * 16];
  float4 s_acc[2][NTHREADS];   // {acc.x, acc.y, comp.x, comp.y} per voxel V
  // conj(r) of the thread's (voxel, element) pairs, packed over the two elements i of a
  // (voxel, k-step): {re, re, im, im}, and {-im, -im}
  float4 s_cr[2 * TC_KS][NTHREADS];
  float2 s_cin[2 * TC_KS][NTHREADS];
  float s_dx[4 * TC_KS][NTHREADS];    // |c_e - x| of the pairs, negative on the left side (e < emid)
  dfl s_ux[4 * TC_KS][NTHREADS];      // u_rx of the pairs (the receive re-anchors)
};

// Extra shared memory of the derivative variant: the pairs' receive delays and the
// compensated sums of dI/dc per voxel.
struct TcDerivShared {
  float s_urx[4 * TC_KS][NTHREADS];   // u_rx of the thread's (voxel, element) pairs
  float4 s_dacc[2][NTHREADS];
};

// One 64-voxel tile of frame d (2 columns x 32 rows): segment lists, then the bin loop
// on the tensor cores, then the image.  The caller has reset ktop[] and e_range and
// synchronised the block; the body ends with a block barrier.  lb_s / ub_s hold the
// frame's element edges.
//
// DERIV also writes the image's derivative with respect to the speed of sound, with
// the band, F table and apertures held fixed (fnum_pw_sharpness_grad, fnum_pw_adjoint).
// The phase of a term is 2 pi k u with u = U + t0/N and dU/dc = -U/c, U = u_rx + U_tx,
// so dI/dc = -(2 pi i / c) Draw with
//   Draw_v = s sum_k k sum_a t^k [U_tx(v,a) G_k(v,a) + G'_k(v,a)],
//   G'_k(v,a) = sum_e (R_k(v,e) u_rx(v,e)) X_k(e,a)
// (G' is a second product with the A operand scaled by u_rx).  sum_k k t^k Y_k comes from
// a second Horner chain beside each first one: going down the bins, Q <- (Q + P) t
// before P <- P t + Y, and a chunk ending at bin kc_lo contributes t^kc_lo (kc_lo P + Q).
// dimage receives Draw (scaled like the image).
//
// BATCH (the persistent batch kernel, whose descriptor lies in global memory) reads the
// descriptor fields used at every bin (k_lb, tc_S) once per tile; the per-frame kernels
// read their parameters' fields where they are used (constant-bank operands, no
// registers held).
template <int WIN, bool DERIV, bool BATCH = false, int NT = 3>
__device__ __forceinline__ void pw_tc_tile(const PWDev& d, int tile, int n_tiles_x, int n_tiles_z, TcShared& sh,
                                           const dfl* lb_s, const dfl* ub_s, int* ktop, float2* __restrict__ image,
                                           float* __restrict__ weights, unsigned long long& n_active,
                                           unsigned long long& n_empty, unsigned long long& n_exec,
                                           TcDerivShared* dsh = nullptr, float2* __restrict__ dimage = nullptr) {
  auto& apt = sh.apt;
  auto& e_range = sh.e_range;
  auto& s_nseg = sh.s_nseg;
  auto& b_ent = sh.b_ent;
  auto& b_next = sh.b_next;
  auto& b_idx = sh.b_idx;
  auto& s_acc = sh.s_acc;
  auto& s_cr = sh.s_cr;
  auto& s_cin = sh.s_cin;
  auto& s_dx = sh.s_dx;
  auto& s_ux = sh.s_ux;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, q = lane & 3;
  int4* seg_blk = d.seg + (size_t)blockIdx.x * NTHREADS * (size_t)d.seg_cap * PW_SEG_INT4;
  const float inv_par = (d.window_par > 0.0f) ? 1.0f / d.window_par : 0.0f;
  const float inv_sigma = 1.0f / tc_scale(*d.tc_max);
  const int b_k_lb = d.k_lb, b_tc_S = d.tc_S;
#define TC_D(field) (BATCH ? b_##field : d.field)
  const int tb = (d.tc_tb > 0 && d.tc_tb < TC_TB) ? d.tc_tb : TC_TB;   // bins per flush (a launch shape)
  constexpr int NA_P = 4 * NT;     // angles per pass
  constexpr int NB = 32 * NT;      // uint4 of B fragments per element group and bin
  {
    int tx, tz;
    tile_coords(tile, n_tiles_x, n_tiles_z, tx, tz);
    // block voxel vb (0..63): column vb / 32, row vb % 32; threads 0..63 build its segment list
    if (tid < TC_WARPS * 16) {
      const int i = tx * TC_TILE_X + (tid >> 5), j = tz * TILE_Z + (tid & 31);
      const bool valid = (i < d.nx) && (j < d.nz);
      const int ic = min(i, d.nx - 1), jc = min(j, d.nz - 1);
      float W_top;
      s_nseg[tid] = pw_build_segments<WIN>(d, inv_par, ic, jc, valid, seg_blk + (size_t)tid * d.seg_cap, ktop,
                                           e_range, W_top, n_active, n_empty);
      if (valid && weights) weights[(size_t)ic * d.nz + jc] = W_top;
    }
    __syncthreads();
    const int E_lo = e_range[0] & ~7, E_hi = e_range[1];

    // the thread's voxels: mma rows g and g + 8 of its warp
    int vic[2], vjc[2], emid[2];
    bool vvalid[2];
#pragma unroll
    for (int V = 0; V < 2; ++V) {
      const int vb = 16 * warp + g + 8 * V;
      const int i = tx * TC_TILE_X + (vb >> 5), j = tz * TILE_Z + (vb & 31);
      vvalid[V] = (i < d.nx) && (j < d.nz);
      vic[V] = min(i, d.nx - 1);
      vjc[V] = min(j, d.nz - 1);
      emid[V] = d.col_emid[vic[V]];
    }
    // table builder: lane l < 16 serves voxel 16 * warp + l
    const int bv = 16 * warp + (lane & 15);
    const int4* bseg = seg_blk + (size_t)bv * d.seg_cap;
    const int bnseg = s_nseg[bv];
    const dfl bxm = d.col_m[min(tx * TC_TILE_X + (bv >> 5), d.nx - 1)];
    auto entry_of = [&](int4 c) -> float4 {
      const int ilb = code_ilb(c.y), iub = code_iub(c.y);
      // An element is in the aperture exactly when its window argument u = d / L is
      // below 1: the nearest element outside lies (pitch - width/2) / L beyond it, the
      // outermost inside width/2 / L within (pitch > width is checked at plan creation;
      // the margin exceeds the FP32 rounding of u for any width above 1e-6 of L).  A side without aperture (no edge element,
      // or a half-width that is not positive) gets 1/L = 1e30, which sends its elements
      // to u >= 1 and keeps the other side's (distance 0 on this side) at u = d / L.
      float il = 1.0e30f, ir = 1.0e30f;
      if (ilb < d.ne) {
        const dfl l = lb_s[ilb];
        const float L = (bxm.x - l.x) + (bxm.y - l.y);
        if (L > 0.0f) il = __fdividef(1.0f, L);
      }
      if (iub >= 0) {
        const dfl u = ub_s[iub];
        const float L = (u.x - bxm.x) + (u.y - bxm.y);
        if (L > 0.0f) ir = __fdividef(1.0f, L);
      }
      return make_float4(0.0f, il, ir, __int_as_float(c.z));
    };
    s_acc[0][tid] = s_acc[1][tid] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if constexpr (DERIV) dsh->s_dacc[0][tid] = dsh->s_dacc[1][tid] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);

    for (int a0 = 0; a0 < d.na; a0 += NA_P) {
      float2 tph[2][NT];   // transmit phasor of (voxel V, angle a0 + 4j + q)
#pragma unroll
      for (int V = 0; V < 2; ++V)
#pragma unroll
        for (int j = 0; j < NT; ++j) {
          const int aa = min(a0 + 4 * j + q, d.na - 1);
          tph[V][j] = cis_ku(1, df_add(d.tx_ax[(size_t)aa * d.nx + vic[V]], d.tx_az[(size_t)aa * d.nz + vjc[V]]));
        }
      const uint4* Bp = d.tc_B + (size_t)(a0 / NA_P) * d.K * d.tc_S * NB;
      for (int e0 = E_lo; e0 <= E_hi; e0 += TC_EP) {
        int kt = -1;
        for (int e = max(e0, 0); e < min(e0 + TC_EP, E_hi + 1); ++e) kt = max(kt, ktop[e]);
        if (kt < TC_D(k_lb)) continue;
        if (tid == 0)
          n_exec += (unsigned long long)(kt - d.k_lb + 1) * TC_EP * min(NA_P, d.na - a0) * (TC_WARPS * 16);
        // the thread's (voxel, element) pairs: V, element e0 + 8s + 2q + i
        // receive phasors r^k packed over the two elements of a (voxel, k-step): {re, re}, {im, im}
        float2 pr[2][TC_KS], pim[2][TC_KS];
#pragma unroll
        for (int V = 0; V < 2; ++V) {
          const dfl xm = d.col_m[vic[V]], xu = d.col_u[vic[V]], zu2 = d.row_u2[vjc[V]];
#pragma unroll
          for (int s = 0; s < TC_KS; ++s)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
              const int e = min(e0 + 8 * s + 2 * q + i, d.ne - 1);
              const dfl cm = d.el_m[e];
              const float dx = fabsf((cm.x - xm.x) + (cm.y - xm.y));
              s_dx[2 * TC_KS * V + 2 * s + i][tid] = (e0 + 8 * s + 2 * q + i < emid[V]) ? -dx : dx;
              const dfl urx = df_sqrt(df_add(df_sqr(df_sub(d.el_u[e], xu)), zu2));
              s_ux[2 * TC_KS * V + 2 * s + i][tid] = urx;
              const float2 r = cis_ku(1, urx);
              if constexpr (DERIV) dsh->s_urx[2 * TC_KS * V + 2 * s + i][tid] = urx.x + urx.y;
              float* c = reinterpret_cast<float*>(&s_cr[TC_KS * V + s][tid]);
              c[i] = r.x;
              c[2 + i] = -r.y;
              reinterpret_cast<float*>(&s_cin[TC_KS * V + s][tid])[i] = r.y;
            }
        }
        float H[NT][4];
#pragma unroll
        for (int j = 0; j < NT; ++j) H[j][0] = H[j][1] = H[j][2] = H[j][3] = 0.0f;
        // derivative chains: HQ (second chain of H), HP (the u_rx-scaled product), HPQ
        float HQ[NT][4], HP[NT][4], HPQ[NT][4];
        if constexpr (DERIV) {
#pragma unroll
          for (int j = 0; j < NT; ++j)
#pragma unroll
            for (int c = 0; c < 4; ++c) HQ[j][c] = HP[j][c] = HPQ[j][c] = 0.0f;
        }
        // builder state: the segment in effect and the next entry
        if (lane < 16) {
          int bs = 0;
          float4 bent = make_float4(0.0f, 1.0e30f, 1.0e30f, 0.0f);  // empty aperture
          int4 bnext = make_int4(-1, 0, 0, 0);
          if (bnseg > 0) {
            bs = seg_find1(bseg, bnseg, kt);
            bent = entry_of(bseg[bs]);
            bent.x = __int_as_float(bs);
            bnext = bseg[min(bs + 1, bnseg)];
          }
          b_ent[bv] = bent;
          b_next[bv] = bnext;
          b_idx[bv] = bs;
        }
        const uint4* Bpe = Bp + (size_t)(e0 >> 3) * NB + lane;
        // the pairs' weights of the segment in effect, recomputed when a voxel enters a new segment
        float bw[2][TC_KS][2];
        int wid[2] = {-1, -1};
        for (int kc_hi = kt; kc_hi >= TC_D(k_lb); kc_hi -= tb) {
          const int kc_lo = max(TC_D(k_lb), kc_hi - (tb - 1));
          // receive phasors re-anchored exactly at the chunk's first bin
#pragma unroll
          for (int V = 0; V < 2; ++V) {
#pragma unroll
            for (int s = 0; s < TC_KS; ++s)
#pragma unroll
              for (int i = 0; i < 2; ++i) {
                const float2 c = cis_ku(kc_hi, s_ux[2 * TC_KS * V + 2 * s + i][tid]);
                if (i == 0) {
                  pr[V][s].x = c.x;
                  pim[V][s].x = c.y;
                } else {
                  pr[V][s].y = c.x;
                  pim[V][s].y = c.y;
                }
              }
          }
          for (int kt_hi = kc_hi; kt_hi >= kc_lo; kt_hi -= TC_TT) {
            const int kt_lo = max(kc_lo, kt_hi - (TC_TT - 1));
            __syncwarp();
            if (lane < 16) {
              int bs = b_idx[bv];
              float4 bent = b_ent[bv];
              int4 bnext = b_next[bv];
              for (int k = kt_hi; k >= kt_lo; --k) {
                if (k == bnext.x) {
                  bent = entry_of(bnext);
                  ++bs;
                  bent.x = __int_as_float(bs);
                  bnext = bseg[min(bs + 1, bnseg)];
                }
                apt[warp][kt_hi - k][lane] = bent;
              }
              b_ent[bv] = bent;
              b_next[bv] = bnext;
              b_idx[bv] = bs;
            }
            __syncwarp();
            for (int k = kt_hi; k >= kt_lo; --k) {
              float4 en[2];
              en[0] = apt[warp][kt_hi - k][g];
              en[1] = apt[warp][kt_hi - k][g + 8];
#pragma unroll
              for (int V = 0; V < 2; ++V) {
                const int sid = __float_as_int(en[V].x);
                if (sid != wid[V]) {
                  wid[V] = sid;
#pragma unroll
                  for (int s = 0; s < TC_KS; ++s)
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                      const float sd = s_dx[2 * TC_KS * V + 2 * s + i][tid];
                      const float u = fabsf(sd) * (sd < 0.0f ? en[V].y : en[V].z);
                      bw[V][s][i] = (u < 1.0f) ? win_t<WIN>(d.window_par, inv_par, u) * en[V].w : 0.0f;
                    }
                }
              }
              // H <- H t (derivative chains: Q <- (Q + P) t, P <- P t)
#pragma unroll
              for (int j = 0; j < NT; ++j)
#pragma unroll
                for (int V = 0; V < 2; ++V) {
                  const float hr = H[j][2 * V], hi = H[j][2 * V + 1];
                  const float2 t = tph[V][j];
                  if constexpr (DERIV) {
                    const float qr = HQ[j][2 * V] + hr, qi = HQ[j][2 * V + 1] + hi;
                    HQ[j][2 * V] = fmaf(qr, t.x, -qi * t.y);
                    HQ[j][2 * V + 1] = fmaf(qr, t.y, qi * t.x);
                    const float pr2 = HP[j][2 * V], pi2 = HP[j][2 * V + 1];
                    const float sr = HPQ[j][2 * V] + pr2, si = HPQ[j][2 * V + 1] + pi2;
                    HPQ[j][2 * V] = fmaf(sr, t.x, -si * t.y);
                    HPQ[j][2 * V + 1] = fmaf(sr, t.y, si * t.x);
                    HP[j][2 * V] = fmaf(pr2, t.x, -pi2 * t.y);
                    HP[j][2 * V + 1] = fmaf(pr2, t.y, pi2 * t.x);
                  }
                  H[j][2 * V] = fmaf(hr, t.x, -hi * t.y);
                  H[j][2 * V + 1] = fmaf(hr, t.y, hi * t.x);
                }
              const uint4* Bk = Bpe + (size_t)(k - TC_D(k_lb)) * TC_D(tc_S) * NB;
#pragma unroll
              for (int s = 0; s < TC_KS; ++s) {
                uint4 bf[NT];
#pragma unroll
                for (int j = 0; j < NT; ++j) bf[j] = __ldg(Bk + s * NB + j * 32);
                float2 rre[2], rim[2];
#pragma unroll
                for (int V = 0; V < 2; ++V) {
                  // R = b r^k and r^k <- r^k conj(r), two elements per packed FP32 instruction
                  const float2 bb = make_float2(bw[V][s][0], bw[V][s][1]);
                  const float2 Pr = pr[V][s], Pi = pim[V][s];
                  rre[V] = __fmul2_rn(bb, Pr);
                  rim[V] = __fmul2_rn(bb, Pi);
                  const float4 c4 = s_cr[TC_KS * V + s][tid];
                  const float2 cre = make_float2(c4.x, c4.y), cim = make_float2(c4.z, c4.w),
                               cimn = s_cin[TC_KS * V + s][tid];
                  pr[V][s] = __ffma2_rn(Pi, cimn, __fmul2_rn(Pr, cre));
                  pim[V][s] = __ffma2_rn(Pi, cre, __fmul2_rn(Pr, cim));
                }
                unsigned ah[4], al[4];
                tc_split_mx(rre[0].x, rre[0].y, ah[0], al[0]);
                tc_split_mx(rre[1].x, rre[1].y, ah[1], al[1]);
                tc_split_mx(rim[0].x, rim[0].y, ah[2], al[2]);
                tc_split_mx(rim[1].x, rim[1].y, ah[3], al[3]);
                // product-major order: consecutive mma.sync update different accumulators
#pragma unroll
                for (int j = 0; j < NT; ++j) tc_mma(H[j], ah, bf[j].x, bf[j].y);
#pragma unroll
                for (int j = 0; j < NT; ++j) tc_mma(H[j], ah, bf[j].z, bf[j].w);
#pragma unroll
                for (int j = 0; j < NT; ++j) tc_mma(H[j], al, bf[j].x, bf[j].y);
                if constexpr (DERIV) {
                  // the second product: A scaled by the pairs' receive delays
                  unsigned ah2[4], al2[4];
#pragma unroll
                  for (int V = 0; V < 2; ++V) {
                    const float2 uu = make_float2(dsh->s_urx[2 * TC_KS * V + 2 * s][tid],
                                                  dsh->s_urx[2 * TC_KS * V + 2 * s + 1][tid]);
                    const float2 r2 = __fmul2_rn(rre[V], uu), i2 = __fmul2_rn(rim[V], uu);
                    tc_split_mx(r2.x, r2.y, ah2[V], al2[V]);
                    tc_split_mx(i2.x, i2.y, ah2[2 + V], al2[2 + V]);
                  }
#pragma unroll
                  for (int j = 0; j < NT; ++j) tc_mma(HP[j], ah2, bf[j].x, bf[j].y);
#pragma unroll
                  for (int j = 0; j < NT; ++j) tc_mma(HP[j], ah2, bf[j].z, bf[j].w);
#pragma unroll
                  for (int j = 0; j < NT; ++j) tc_mma(HP[j], al2, bf[j].x, bf[j].y);
                }
              }
            }
          }
          // flush: the image gains t^{kc_lo} H with the exact phase
#pragma unroll
          for (int V = 0; V < 2; ++V) {
            float2 part = make_float2(0.0f, 0.0f), dpart = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int j = 0; j < NT; ++j) {
              const int a = a0 + 4 * j + q;
              if (a < d.na) {
                const dfl ut = df_add(d.tx_ax[(size_t)a * d.nx + vic[V]], d.tx_az[(size_t)a * d.nz + vjc[V]]);
                const float2 c = cis_ku(kc_lo, ut);
                const float2 t = cmul(c, make_float2(H[j][2 * V], H[j][2 * V + 1]));
                part.x += t.x;
                part.y += t.y;
                if constexpr (DERIV) {
                  // t^kc_lo [U_tx (kc_lo P + Q) + (kc_lo P' + Q')]
                  const float utx = (ut.x - d.t0N) + ut.y, kl = (float)kc_lo;
                  const float yr = utx * fmaf(kl, H[j][2 * V], HQ[j][2 * V]) + fmaf(kl, HP[j][2 * V], HPQ[j][2 * V]);
                  const float yi =
                      utx * fmaf(kl, H[j][2 * V + 1], HQ[j][2 * V + 1]) + fmaf(kl, HP[j][2 * V + 1], HPQ[j][2 * V + 1]);
                  const float2 dt = cmul(c, make_float2(yr, yi));
                  dpart.x += dt.x;
                  dpart.y += dt.y;
                }
              }
              H[j][2 * V] = H[j][2 * V + 1] = 0.0f;
              if constexpr (DERIV) {
                HQ[j][2 * V] = HQ[j][2 * V + 1] = HP[j][2 * V] = HP[j][2 * V + 1] = 0.0f;
                HPQ[j][2 * V] = HPQ[j][2 * V + 1] = 0.0f;
              }
            }
            if constexpr (DERIV) {
              float4 b4 = dsh->s_dacc[V][tid];
              float y = dpart.x - b4.z, t = b4.x + y;
              b4.z = (t - b4.x) - y;
              b4.x = t;
              y = dpart.y - b4.w;
              t = b4.y + y;
              b4.w = (t - b4.y) - y;
              b4.y = t;
              dsh->s_dacc[V][tid] = b4;
            }
            float4 a4 = s_acc[V][tid];
            float y = part.x - a4.z, t = a4.x + y;
            a4.z = (t - a4.x) - y;
            a4.x = t;
            y = part.y - a4.w;
            t = a4.y + y;
            a4.w = (t - a4.y) - y;
            a4.y = t;
            s_acc[V][tid] = a4;
          }
        }
      }
    }
    // the four lanes of a group hold the voxel's sums over their angles
#pragma unroll
    for (int V = 0; V < 2; ++V) {
      float x = s_acc[V][tid].x, y = s_acc[V][tid].y;
      x += __shfl_xor_sync(0xffffffffu, x, 1);
      y += __shfl_xor_sync(0xffffffffu, y, 1);
      x += __shfl_xor_sync(0xffffffffu, x, 2);
      y += __shfl_xor_sync(0xffffffffu, y, 2);
      if (q == 0 && vvalid[V])
        image[(size_t)vic[V] * d.nz + vjc[V]] = make_float2(x * d.scale * inv_sigma, y * d.scale * inv_sigma);
      if constexpr (DERIV) {
        float dx = dsh->s_dacc[V][tid].x, dy = dsh->s_dacc[V][tid].y;
        dx += __shfl_xor_sync(0xffffffffu, dx, 1);
        dy += __shfl_xor_sync(0xffffffffu, dy, 1);
        dx += __shfl_xor_sync(0xffffffffu, dx, 2);
        dy += __shfl_xor_sync(0xffffffffu, dy, 2);
        if (q == 0 && vvalid[V])
          dimage[(size_t)vic[V] * d.nz + vjc[V]] = make_float2(dx * d.scale * inv_sigma, dy * d.scale * inv_sigma);
      }
    }
    __syncthreads();
  }
}
#undef TC_D

// the per-frame statistics of pw_tc_tile, added to the frame's counters
__device__ __forceinline__ void pw_tc_flush_counts(const PWDev& d, unsigned long long& n_active,
                                                   unsigned long long& n_empty, unsigned long long& n_exec) {
  atomicAdd(&d.counters[0], n_active * (unsigned long long)d.na);
  atomicAdd(&d.counters[1], n_empty * (unsigned long long)d.na);
  if (threadIdx.x == 0) atomicAdd(&d.counters[4], n_exec);
  n_active = n_empty = n_exec = 0;
}

template <int WIN, int NT>
__global__ void __launch_bounds__(NTHREADS, 4)
pw_tc_kernel(const PWDev d, float2* __restrict__ image, float* __restrict__ weights, int n_tiles_x, int n_tiles_z) {
  __shared__ TcShared sh;
  __shared__ int s_tile;
  extern __shared__ __align__(16) unsigned char dyn[];  // lb[ne], ub[ne] (dfl), ktop[ne]
  dfl* lb_s = (dfl*)dyn;
  dfl* ub_s = lb_s + d.ne;
  int* ktop = (int*)(ub_s + d.ne);
  const int tid = threadIdx.x;
  const int n_tiles = n_tiles_x * n_tiles_z;
  unsigned long long n_active = 0, n_empty = 0, n_exec = 0;
  for (int e = tid; e < d.ne; e += NTHREADS) {
    lb_s[e] = d.el_lb[e];
    ub_s[e] = d.el_ub[e];
  }
  for (;;) {
    if (tid == 0) s_tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < d.ne; e += NTHREADS) ktop[e] = -1;
    if (tid == 0) {
      sh.e_range[0] = d.ne;
      sh.e_range[1] = -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    pw_tc_tile<WIN, false, false, NT>(d, tile, n_tiles_x, n_tiles_z, sh, lb_s, ub_s, ktop, image, weights, n_active,
                                      n_empty, n_exec);
  }
  pw_tc_flush_counts(d, n_active, n_empty, n_exec);
}

// One persistent launch over the tiles of many frames (a batch): each block draws
// global tile numbers from the batch's counter, in frame order (the host orders the
// frames largest first), finds the tile's frame, and runs pw_tc_tile on it.  The frames'
// descriptors stay in device memory (read through the cache; the host has set their
// segment scratch to the batch's), which measured faster than a copy in shared memory.
template <int WIN, int NT>
__global__ void __launch_bounds__(NTHREADS, 4) pw_tc_batch_kernel(const PWBatchDev B) {
  __shared__ TcShared sh;
  __shared__ int s_tile, s_frame;
  extern __shared__ __align__(16) unsigned char dyn[];  // lb[max_ne], ub[max_ne] (dfl), ktop[max_ne]
  dfl* lb_s = (dfl*)dyn;
  dfl* ub_s = lb_s + B.max_ne;
  int* ktop = (int*)(ub_s + B.max_ne);
  const int tid = threadIdx.x;
  unsigned long long n_active = 0, n_empty = 0, n_exec = 0;
  int cur = -1;
  for (;;) {
    if (tid == 0) {
      const int t = (int)atomicAdd(B.counter, 1ull);
      int f = -1;
      if (t < B.tile_start[B.n_frames]) {
        int lo = 0, hi = B.n_frames - 1;   // the frame whose tile range holds t
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (B.tile_start[mid] <= t) lo = mid; else hi = mid - 1;
        }
        f = lo;
        s_tile = t - B.tile_start[f];
      }
      s_frame = f;
    }
    __syncthreads();
    const int f = s_frame;
    if (f < 0) break;
    const PWDev& d = B.frames[f];
    if (f != cur) {
      if (cur >= 0) pw_tc_flush_counts(B.frames[cur], n_active, n_empty, n_exec);
      __syncthreads();   // every thread is done with the previous frame's element edges
      for (int e = tid; e < d.ne; e += NTHREADS) {
        lb_s[e] = d.el_lb[e];
        ub_s[e] = d.el_ub[e];
      }
      cur = f;
    }
    for (int e = tid; e < B.max_ne; e += NTHREADS) ktop[e] = -1;
    if (tid == 0) {
      sh.e_range[0] = d.ne;
      sh.e_range[1] = -1;
    }
    __syncthreads();
    const int ntx = (d.nx + TC_TILE_X - 1) / TC_TILE_X, ntz = (d.nz + TILE_Z - 1) / TILE_Z;
    pw_tc_tile<WIN, false, true, NT>(d, s_tile, ntx, ntz, sh, lb_s, ub_s, ktop, B.images[f], B.weights[f], n_active, n_empty,
                           n_exec);
  }
  if (cur >= 0) pw_tc_flush_counts(B.frames[cur], n_active, n_empty, n_exec);
}

// The image and its derivative with respect to the speed of sound (see pw_tc_tile).
template <int WIN>
__global__ void __launch_bounds__(NTHREADS, 3)
pw_tc_deriv_kernel(const PWDev d, float2* __restrict__ image, float2* __restrict__ dimage, int n_tiles_x,
                   int n_tiles_z) {
  __shared__ TcShared sh;
  __shared__ int s_tile;
  extern __shared__ __align__(16) unsigned char dyn[];  // TcDerivShared, lb[ne], ub[ne] (dfl), ktop[ne]
  TcDerivShared& dsh = *reinterpret_cast<TcDerivShared*>(dyn);
  dfl* lb_s = (dfl*)(dyn + sizeof(TcDerivShared));
  dfl* ub_s = lb_s + d.ne;
  int* ktop = (int*)(ub_s + d.ne);
  const int tid = threadIdx.x;
  const int n_tiles = n_tiles_x * n_tiles_z;
  unsigned long long n_active = 0, n_empty = 0, n_exec = 0;
  for (int e = tid; e < d.ne; e += NTHREADS) {
    lb_s[e] = d.el_lb[e];
    ub_s[e] = d.el_ub[e];
  }
  for (;;) {
    if (tid == 0) s_tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < d.ne; e += NTHREADS) ktop[e] = -1;
    if (tid == 0) {
      sh.e_range[0] = d.ne;
      sh.e_range[1] = -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    pw_tc_tile<WIN, true>(d, tile, n_tiles_x, n_tiles_z, sh, lb_s, ub_s, ktop, image, nullptr, n_active, n_empty,
                          n_exec, &dsh, dimage);
  }
  pw_tc_flush_counts(d, n_active, n_empty, n_exec);
}

typedef void (*pw_kernel_t)(const PWDev, float2*, float*, int, int);

template <int EPT, int NA>
static pw_kernel_t pw_pick_win(int window_id) {
  switch (window_id) {
    case 0: return pw_fused_kernel<EPT, NA, 0>;
    case 1: return pw_fused_kernel<EPT, NA, 1>;
    case 2: return pw_fused_kernel<EPT, NA, 2>;
    default: return pw_fused_kernel<EPT, NA, 4>;
  }
}
template <int EPT, int NA>
static pw_kernel_t pw_pick_event_win(int window_id) {
  switch (window_id) {
    case 0: return pw_event_kernel<EPT, NA, 0>;
    case 1: return pw_event_kernel<EPT, NA, 1>;
    case 2: return pw_event_kernel<EPT, NA, 2>;
    default: return pw_event_kernel<EPT, NA, 4>;
  }
}

// Kernel variants: how many elements (EPT) and angles (NA) one pass carries,
// and where the segment boundaries are resolved.
//   boundaries resolved ahead of the bin loop (pw_event_kernel):
//     1: EPT 1 x NA 11   2: EPT 2 x NA 4   3: EPT 2 x NA 2   4: EPT 4 x NA 1
//   boundaries resolved inside the bin loop (pw_fused_kernel):
//     5: EPT 1 x NA 11   6: EPT 2 x NA 4   7: EPT 2 x NA 2   8: EPT 4 x NA 1
//   9: tensor cores (pw_tc_kernel), 16 elements x 12 angles per pass, or 16
//      angles where that takes fewer passes (PWDev::tc_nt); needs the plan's
//      fragment scratch (PWDev::tc_B)
// Angles beyond NA run as further passes inside the launch.  PWDev::variant
// 0 picks by the angle count; a plan's autotuner may set another.
static pw_kernel_t pw_pick_tc_win(int window_id, int nt) {
  const bool n4 = nt == 4;
  switch (window_id) {
    case 0: return n4 ? pw_tc_kernel<0, 4> : pw_tc_kernel<0, 3>;
    case 1: return n4 ? pw_tc_kernel<1, 4> : pw_tc_kernel<1, 3>;
    case 2: return n4 ? pw_tc_kernel<2, 4> : pw_tc_kernel<2, 3>;
    default: return n4 ? pw_tc_kernel<4, 4> : pw_tc_kernel<4, 3>;
  }
}
// n-tiles per angle pass of frame d's tensor-core kernel (tc_ntiles_for, set at plan creation)
static int pw_tc_nt(const PWDev& d) { return d.tc_nt == 4 ? 4 : 3; }
static pw_kernel_t pw_variant_kernel(int v, const PWDev& d) {
  const int window_id = d.window_id;
  switch (v) {
    case TC_VARIANT: return pw_pick_tc_win(window_id, pw_tc_nt(d));
    case 1: return pw_pick_event_win<1, 11>(window_id);
    case 2: return pw_pick_event_win<2, 4>(window_id);
    case 3: return pw_pick_event_win<2, 2>(window_id);
    case 4: return pw_pick_event_win<4, 1>(window_id);
    case 5: return pw_pick_win<1, 11>(window_id);
    case 6: return pw_pick_win<2, 4>(window_id);
    case 7: return pw_pick_win<2, 2>(window_id);
    default: return pw_pick_win<4, 1>(window_id);
  }
}
// default pass shape by angle count; with the fragment scratch in place the
// tensor-core variant from 3 angles on (measured at 128 elements, 256 x 256)
static int pw_default_variant(const PWDev& d) {
  if (d.tc_B && d.na >= 3) return TC_VARIANT;
  if (d.na >= 11) return 1;
  if (d.na >= 4) return 2;
  if (d.na >= 2) return 3;
  return 4;
}
static pw_kernel_t pw_pick(const PWDev& d) {
  return pw_variant_kernel(d.variant > 0 ? d.variant : pw_default_variant(d), d);
}
int pw_variant_count() { return 9; }
int pw_variant_of(const PWDev& d) { return d.variant > 0 ? d.variant : pw_default_variant(d); }

static int pw_tiles_x(const PWDev& d) {
  const int tw = pw_variant_of(d) == TC_VARIANT ? TC_TILE_X : TILE_X;
  return (d.nx + tw - 1) / tw;
}

// The tensor-core tile kernels' static shared memory and their element tables (20
// bytes per element, dynamic) exceed the 48 KB a block may use without opting in:
// each of them is allowed the device's maximum once per device.
static cudaError_t pw_tc_smem_optin() {
  static std::mutex mu;
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (dev < 64 && done[dev]) return cudaSuccess;
  int optin = 0;
  if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
  const void* fns[] = {
      (const void*)pw_tc_kernel<0, 3>,       (const void*)pw_tc_kernel<1, 3>,
      (const void*)pw_tc_kernel<2, 3>,       (const void*)pw_tc_kernel<4, 3>,
      (const void*)pw_tc_kernel<0, 4>,       (const void*)pw_tc_kernel<1, 4>,
      (const void*)pw_tc_kernel<2, 4>,       (const void*)pw_tc_kernel<4, 4>,
      (const void*)pw_tc_batch_kernel<0, 3>, (const void*)pw_tc_batch_kernel<1, 3>,
      (const void*)pw_tc_batch_kernel<2, 3>, (const void*)pw_tc_batch_kernel<4, 3>,
      (const void*)pw_tc_batch_kernel<0, 4>, (const void*)pw_tc_batch_kernel<1, 4>,
      (const void*)pw_tc_batch_kernel<2, 4>, (const void*)pw_tc_batch_kernel<4, 4>,
      (const void*)pw_tc_deriv_kernel<0>,    (const void*)pw_tc_deriv_kernel<1>,
      (const void*)pw_tc_deriv_kernel<2>,    (const void*)pw_tc_deriv_kernel<4>};
  for (const void* f : fns) {
    cudaFuncAttributes a;
    if ((e = cudaFuncGetAttributes(&a, f)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)a.sharedSizeBytes)) != cudaSuccess)
      return e;
  }
  if (dev < 64) done[dev] = true;
  return cudaSuccess;
}

int pw_fused_grid(const PWDev& d, int* blocks_per_sm) {
  pw_kernel_t fn = pw_pick(d);
  int dev = 0, nsm = 0, bps = 0;
  (void)pw_tc_smem_optin();
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, NTHREADS, (size_t)d.ne * (sizeof(int) + 2 * sizeof(dfl)));
  if (bps < 1) bps = 1;
  if (d.blocks_per_sm > 0 && d.blocks_per_sm < bps) bps = d.blocks_per_sm;   // a launch shape of the autotuner
  if (blocks_per_sm) *blocks_per_sm = bps;
  const int tiles = pw_tiles_x(d) * ((d.nz + TILE_Z - 1) / TILE_Z);
  return tiles < nsm * bps ? tiles : nsm * bps;
}

int pw_fused_max_grid(const PWDev& d) {
  int g = 0;
  for (int v = 1; v <= pw_variant_count(); ++v) {
    PWDev t = d;
    t.variant = v;
    t.blocks_per_sm = 0;
    g = max(g, pw_fused_grid(t, nullptr));
  }
  return g;
}

cudaError_t launch_pw_fused(const PWDev& d, int grid, float2* image, float* weights, cudaStream_t s) {
  const int ntx = pw_tiles_x(d), ntz = (d.nz + TILE_Z - 1) / TILE_Z;
  const size_t smem = (size_t)d.ne * (sizeof(int) + 2 * sizeof(dfl));
  // each launch draws tiles from a fresh counter
  cudaError_t e = pw_tc_smem_optin();
  if (e == cudaSuccess) e = cudaMemsetAsync(d.counters + 3, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (pw_variant_of(d) == TC_VARIANT && (e = launch_pw_tc_prep(d, s)) != cudaSuccess) return e;
  pw_pick(d)<<<grid, NTHREADS, smem, s>>>(d, image, weights, ntx, ntz);
  return cudaGetLastError();
}

cudaError_t launch_pw_tc_prep(const PWDev& d, cudaStream_t s, int nt) {
  if (!d.tc_B || !d.tc_max) return cudaErrorInvalidValue;
  if (nt != 3 && nt != 4) nt = pw_tc_nt(d);
  // spectra -> fp16 B fragments, scaled by a power of two set by their largest component
  cudaError_t e = cudaMemsetAsync(d.tc_max, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  tc_absmax_kernel<<<304, 256, 0, s>>>(d, d.tc_max);
  const int n_ap = (d.na + 4 * nt - 1) / (4 * nt);
  const size_t n = (size_t)n_ap * d.K * d.tc_S * nt * 32;
  tc_prep_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(d, n_ap, nt);
  return cudaGetLastError();
}

typedef void (*pw_tc_deriv_t)(const PWDev, float2*, float2*, int, int);
static pw_tc_deriv_t pw_tc_deriv_pick(int window_id) {
  switch (window_id) {
    case 0: return pw_tc_deriv_kernel<0>;
    case 1: return pw_tc_deriv_kernel<1>;
    case 2: return pw_tc_deriv_kernel<2>;
    default: return pw_tc_deriv_kernel<4>;
  }
}

cudaError_t launch_pw_tc_deriv(const PWDev& d, float2* image, float2* dimage, cudaStream_t s) {
  if (!d.tc_B || !d.tc_max) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(d.counters, 0, 5 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = launch_pw_tc_prep(d, s, 3);   // the derivative kernel runs passes of 12 angles
  if (e != cudaSuccess) return e;
  const size_t smem = sizeof(TcDerivShared) + (size_t)d.ne * (sizeof(int) + 2 * sizeof(dfl));
  if ((e = pw_tc_smem_optin()) != cudaSuccess) return e;
  int dev = 0, nsm = 0, bps = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pw_tc_deriv_pick(d.window_id), NTHREADS, smem);
  if (bps < 1) bps = 1;
  const int ntx = (d.nx + TC_TILE_X - 1) / TC_TILE_X, ntz = (d.nz + TILE_Z - 1) / TILE_Z;
  // the plan's segment scratch holds pw_fused_max_grid blocks: at least this many
  const int grid = min(min(ntx * ntz, nsm * bps), pw_fused_max_grid(d));
  pw_tc_deriv_pick(d.window_id)<<<grid, NTHREADS, smem, s>>>(d, image, dimage, ntx, ntz);
  return cudaGetLastError();
}

int pw_tc_tiles(const PWDev& d) { return ((d.nx + TC_TILE_X - 1) / TC_TILE_X) * ((d.nz + TILE_Z - 1) / TILE_Z); }

typedef void (*pw_tc_batch_t)(const PWBatchDev);
static pw_tc_batch_t pw_tc_batch_pick(int window_id, int nt) {
  const bool n4 = nt == 4;
  switch (window_id) {
    case 0: return n4 ? pw_tc_batch_kernel<0, 4> : pw_tc_batch_kernel<0, 3>;
    case 1: return n4 ? pw_tc_batch_kernel<1, 4> : pw_tc_batch_kernel<1, 3>;
    case 2: return n4 ? pw_tc_batch_kernel<2, 4> : pw_tc_batch_kernel<2, 3>;
    default: return n4 ? pw_tc_batch_kernel<4, 4> : pw_tc_batch_kernel<4, 3>;
  }
}

int pw_tc_batch_grid(int max_ne, int window_id, int nt, int* blocks_per_sm) {
  int dev = 0, nsm = 0, bps = 0;
  (void)pw_tc_smem_optin();
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, pw_tc_batch_pick(window_id, nt), NTHREADS,
                                                (size_t)max_ne * (sizeof(int) + 2 * sizeof(dfl)));
  if (bps < 1) bps = 1;
  if (blocks_per_sm) *blocks_per_sm = bps;
  return nsm * bps;
}

cudaError_t launch_pw_tc_batch(const PWBatchDev& B, int window_id, int nt, int grid, cudaStream_t s) {
  cudaError_t e = pw_tc_smem_optin();
  if (e == cudaSuccess) e = cudaMemsetAsync(B.counter, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  const size_t smem = (size_t)B.max_ne * (sizeof(int) + 2 * sizeof(dfl));
  pw_tc_batch_pick(window_id, nt)<<<grid, NTHREADS, smem, s>>>(B);
  return cudaGetLastError();
}
// ---------------------------------------------------------------------------
// plain per-voxel plane-wave kernel (reference arithmetic per term)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ref_window(int id, float par, float l, float L) {
  // +cuda/gpu_bf_windows.cu with __cosf, as the reference
  if (fabsf(l) >= L) return 0.0f;
  switch (id) {
    case 0: return 1.0f;
    case 1: return (1.0f + __cosf(3.14159265358979f * l / L)) / 2.0f;
    case 2: {
      const float thr = 1.0f - par, ratio = fabsf(l) / L;
      if (ratio <= thr) return 1.0f;
      return (1.0f + __cosf(3.14159265358979f * (ratio - thr) / par)) / 2.0f;
    }
    case 4: return 1.0f - fabsf(l) / L;
    default: return 0.0f;
  }
}

// per-term apodization exactly as das_kernel_phase_shifts.cu:111-154 (float)
__device__ __forceinline__ float ref_apod(int id, float par, float F, float x, float z, float dx, const float* lb,
                                          const float* ub, int ne, float M, float pitch) {
  if (dx < 0.0f) {
    int ia = 0;
    if (F > FLT_EPSILON) ia = (int)fmaxf(ceilf(M + (x - z / (2.0f * F)) / pitch), 0.0f);
    return (ia < ne) ? ref_window(id, par, dx, x - lb[ia]) : 0.0f;
  }
  int ia = ne - 1;
  if (F > FLT_EPSILON) ia = (int)fminf(floorf(M + (x + z / (2.0f * F)) / pitch), (float)(ne - 1));
  return (ia >= 0) ? ref_window(id, par, dx, ub[ia] - x) : 0.0f;
}

__global__ void __launch_bounds__(NTHREADS) pw_plain_kernel(const PWDev d, float2* image, float* weights) {
  const int i = blockIdx.x * TILE_X + (threadIdx.x >> 5);
  const int j = blockIdx.y * TILE_Z + (threadIdx.x & 31);
  if (i >= d.nx || j >= d.nz) return;
  const float x = d.px_f[i], z = d.pz_f[j];
  float2 img = make_float2(0.0f, 0.0f);
  float Wlast = 0.0f;
  for (int a = 0; a < d.na; ++a) {
    const float4 t = d.tx_f[a];
    const float dtx = t.x * (x - t.z) + t.y * z;  // das_kernel_distances_pw.cu:27
    for (int kk = 0; kk < d.K; ++kk) {
      const int k = d.k_lb + kk;
      const float F = d.F_f[kk];
      float sr = 0.0f, si = 0.0f, W = 0.0f;
      for (int e = 0; e < d.ne; ++e) {
        const float dx = d.ctr_f[e] - x;
        const float drt = dtx + __fsqrt_rn(dx * dx + z * z);
        const float ap = ref_apod(d.window_id, d.window_par, F, x, z, dx, d.lb_f, d.ub_f, d.ne, d.M_f, d.pitch_f);
        float sn, cs;
        __sincosf((float)k * (d.coef_f * drt + d.add_f), &sn, &cs);
        const float2 X = d.X[((size_t)e * d.K + kk) * d.x_na + d.x_a0 + a];
        const float pr = ap * cs, pi = ap * sn;
        sr += pr * X.x - pi * X.y;
        si += pr * X.y + pi * X.x;
        W += ap;
      }
      if (d.norm) {
        if (W != 0.0f) {
          img.x += sr / W;
          img.y += si / W;
        }
      } else {
        img.x += sr;
        img.y += si;
      }
      Wlast = W;
    }
  }
  image[(size_t)i * d.nz + j] = make_float2(img.x * d.scale, img.y * d.scale);
  if (weights) weights[(size_t)i * d.nz + j] = Wlast;
}

cudaError_t launch_pw_plain(const PWDev& d, float2* image, float* weights, cudaStream_t s) {
  dim3 grid((d.nx + TILE_X - 1) / TILE_X, (d.nz + TILE_Z - 1) / TILE_Z);
  pw_plain_kernel<<<grid, NTHREADS, 0, s>>>(d, image, weights);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// fused synthetic-aperture kernel
// ---------------------------------------------------------------------------
// window value of element e for the aperture (ilb, iub) of a voxel at xm,
// 0 outside (edges from shared memory)
template <int WIN>
__device__ __forceinline__ float sa_apod(const dfl* lb_s, const dfl* ub_s, dfl xm, int e, int emid, int ilb, int iub,
                                         float dxa, float par, float inv_par) {
  const bool left = e < emid;
  if (left ? (e < ilb) : (e > iub)) return 0.0f;
  return win_t<WIN>(par, inv_par, dxa * inv_half_width(lb_s, ub_s, xm, left, ilb, iub));
}

// Issues the copy of one spectrum chunk (bins kc_lo .. kc_lo + nk - 1 of the
// receive elements r0 .. r0 + EPT - 1 of transmit t) into a shared buffer laid
// out [bin][receive] with rows of ROW float2; consecutive threads copy
// consecutive bins of one receive element.
template <int EPT>
__device__ __forceinline__ void sa_stage_chunk(float2* dst, const SADev& d, int t, int r0, int kc_lo, int nk, int tid,
                                               const float2* X) {
  constexpr int ROW = (EPT + 1) & ~1;
  for (int idx = tid; idx < KCHUNK * EPT; idx += NTHREADS) {
    const int kk = idx % KCHUNK, q = idx / KCHUNK;
    const int r = r0 + q;
    if (kk < nk && r < d.ne) cp_async8(&dst[kk * ROW + q], &X[((size_t)t * d.ne + r) * d.K + (kc_lo - d.k_lb + kk)]);
    else if (kk < nk) dst[kk * ROW + q] = make_float2(0.0f, 0.0f);
  }
  cp_async_commit();
}

template <int EPT, int WT, int WR>
__global__ void __launch_bounds__(NTHREADS, 4)
sa_fused_kernel(const SADev d, float2* __restrict__ image, float* __restrict__ wtx_out, float* __restrict__ wrx_out,
                int n_tiles_x, int n_tiles_z, int weights_only) {
  constexpr int ROW = (EPT + 1) & ~1;
  __shared__ __align__(16) float2 xs[2][KCHUNK * ROW];
  __shared__ int ranges[4];
  __shared__ int s_tile;
  __shared__ unsigned long long s_count[2];         // active terms, zero-weight bins
  __shared__ float dxq_s[EPT][NTHREADS];            // |c_r - x| of the pass's receive elements
  extern __shared__ __align__(16) unsigned char dyn[];  // lb[ne], ub[ne] (dfl), ktop_tx[ne], ktop_rx[ne]
  dfl* lb_s = (dfl*)dyn;
  dfl* ub_s = lb_s + d.ne;
  int* ktop_tx = (int*)(ub_s + d.ne);
  int* ktop_rx = ktop_tx + d.ne;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_tiles = n_tiles_x * n_tiles_z;
  int4* seg = d.seg + ((size_t)blockIdx.x * NTHREADS + tid) * (size_t)d.seg_cap * SA_SEG_INT4;
  const float ipt = (d.wtx_par > 0.0f) ? 1.0f / d.wtx_par : 0.0f;
  const float ipr = (d.wrx_par > 0.0f) ? 1.0f / d.wrx_par : 0.0f;
  const float2* Xsrc = d.Xs ? d.Xs : d.X;
  unsigned long long n_exec = 0;
  if (tid == 0) s_count[0] = s_count[1] = 0ull;
  for (int e = tid; e < d.ne; e += NTHREADS) {
    lb_s[e] = d.el_lb[e];
    ub_s[e] = d.el_ub[e];
  }

  for (;;) {
    if (tid == 0) s_tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < 2 * d.ne; e += NTHREADS) ktop_tx[e] = -1;
    if (tid == 0) {
      ranges[0] = ranges[2] = d.ne;
      ranges[1] = ranges[3] = -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    int tx_, tz_;
    tile_coords(tile, n_tiles_x, n_tiles_z, tx_, tz_);
    const int i = tx_ * TILE_X + warp;
    const int j = tz_ * TILE_Z + lane;
    const bool valid = (i < d.nx) && (j < d.nz);
    const int ic = min(i, d.nx - 1), jc = min(j, d.nz - 1);
    int nseg;
    {
      float Wtx_top, Wrx_top;
      unsigned long long n_active = 0, n_empty = 0;
      nseg = sa_build_segments(d, ic, jc, valid, seg, ktop_tx, ktop_rx, ranges, Wtx_top, Wrx_top, n_active, n_empty);
      atomicAdd(&s_count[0], n_active);
      atomicAdd(&s_count[1], n_empty);
      if (valid) {
        if (wtx_out) wtx_out[(size_t)ic * d.nz + jc] = Wtx_top;
        if (wrx_out) wrx_out[(size_t)ic * d.nz + jc] = Wrx_top;
      }
    }
    __syncthreads();
    const int T_lo = ranges[0], T_hi = weights_only ? -1 : ranges[1], R_lo = ranges[2], R_hi = ranges[3];

    const dfl xm = d.col_m[ic], xu = d.col_u[ic], zu2 = d.row_u2[jc];
    const int emid = d.col_emid[ic];
    float2 acc = make_float2(0.0f, 0.0f), comp = make_float2(0.0f, 0.0f);

    for (int t = T_lo; t <= T_hi; ++t) {
      const int kt_t = ktop_tx[t];
      if (kt_t < d.k_lb) continue;
      const dfl ctm = d.el_m[t];
      const float dxt = fabsf((ctm.x - xm.x) + (ctm.y - xm.y));
      // transmit delay plus the time offset t0 / N (the reference's argument_add)
      const dfl utx = df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[t], xu)), zu2)), d.t0N);
      for (int r0 = d.Xs ? max(R_lo, t) : R_lo; r0 <= R_hi; r0 += EPT) {
        int kt = -1;
#pragma unroll
        for (int q = 0; q < EPT; ++q)
          if (r0 + q <= R_hi) kt = max(kt, ktop_rx[r0 + q]);
        kt = min(kt, kt_t);
        if (kt < d.k_lb) continue;
        if (tid == 0) n_exec += (unsigned long long)(kt - d.k_lb + 1) * EPT * NTHREADS;
        // weight of chain q: f * ar[q], f = a_tx(t) / (W_tx W_rx) shared by the pass
        float ar[EPT];
        float2 z[EPT], A[EPT];
#pragma unroll
        for (int q = 0; q < EPT; ++q) {
          const int e = min(r0 + q, d.ne - 1);
          const dfl cm = d.el_m[e];
          dxq_s[q][tid] = fabsf((cm.x - xm.x) + (cm.y - xm.y));
          z[q] = cis_ku(1, df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[e], xu)), zu2)), utx));
          A[q] = make_float2(0.0f, 0.0f);
        }
        // segment in effect at kt and the prefetch ring of the following entries
        int s = 0;
        int4 cur = make_int4(-1, seg_code(d.ne, -1), seg_code(d.ne, -1), 0);
        int4 ring[SEG_RING];
        if (nseg > 0) {
          s = sa_seg_find(seg, nseg, kt);
          cur = seg[s];
        }
#pragma unroll
        for (int r = 0; r < SEG_RING; ++r) ring[r] = seg[min(s + 1 + r, nseg)];
        float at, f;
        {
          const int tlb = code_ilb(cur.y), tub = code_iub(cur.y), rlb = code_ilb(cur.z), rub = code_iub(cur.z);
          at = sa_apod<WT>(lb_s, ub_s, xm, t, emid, tlb, tub, dxt, d.wtx_par, ipt);
          f = at * __int_as_float(cur.w);
#pragma unroll
          for (int q = 0; q < EPT; ++q) {
            const int e = r0 + q;
            ar[q] = (e <= R_hi) ? sa_apod<WR>(lb_s, ub_s, xm, e, emid, rlb, rub, dxq_s[q][tid], d.wrx_par, ipr)
                                : 0.0f;
          }
        }
        float2 part = make_float2(0.0f, 0.0f);
        const int c_top = (kt - d.k_lb) / KCHUNK;
        __syncthreads();  // every thread is done with both buffers of the previous pass
        sa_stage_chunk<EPT>(xs[0], d, t, r0, d.k_lb + c_top * KCHUNK, kt - (d.k_lb + c_top * KCHUNK) + 1, tid, Xsrc);
        int buf = 0;
        for (int chunk = c_top; chunk >= 0; --chunk) {
          const int kc_lo = d.k_lb + chunk * KCHUNK;
          const int kc_hi = (chunk == c_top) ? kt : kc_lo + KCHUNK - 1;
          cp_async_wait_all();
          __syncthreads();
          if (chunk > 0) sa_stage_chunk<EPT>(xs[buf ^ 1], d, t, r0, kc_lo - KCHUNK, KCHUNK, tid, Xsrc);
          const float2* xb = xs[buf];
          buf ^= 1;
          for (int k = kc_hi; k >= kc_lo; --k) {
            if (k == ring[0].x) {
              // enter the next segment at bin k
              const int ptc = cur.y, prc = cur.z;
              const float fo = f;
              cur = ring[0];
#pragma unroll
              for (int r = 0; r + 1 < SEG_RING; ++r) ring[r] = ring[r + 1];
              ++s;
              ring[SEG_RING - 1] = seg[min(s + SEG_RING, nseg)];
              const int tlb = code_ilb(cur.y), tub = code_iub(cur.y), rlb = code_ilb(cur.z), rub = code_iub(cur.z);
              if (cur.y != ptc || at == 0.0f) at = sa_apod<WT>(lb_s, ub_s, xm, t, emid, tlb, tub, dxt, d.wtx_par, ipt);
              f = at * __int_as_float(cur.w);
              const bool rx_changed = cur.z != prc;
              const float rf = (fo != 0.0f && f != 0.0f) ? __fdividef(fo, f) : 0.0f;
#pragma unroll
              for (int q = 0; q < EPT; ++q) {
                const int e = r0 + q;
                const float ao = ar[q];
                float an = ao;
                if (rx_changed || ao == 0.0f)
                  an = (e <= R_hi) ? sa_apod<WR>(lb_s, ub_s, xm, e, emid, rlb, rub, dxq_s[q][tid], d.wrx_par, ipr) : 0.0f;
                const float bo = fo * ao, bn = f * an;
                if (bn != 0.0f && bo != 0.0f) {
                  const float r = (an == ao) ? rf : __fdividef(bo, bn);
                  A[q].x *= r;
                  A[q].y *= r;
                } else {
                  if (bo != 0.0f) {  // leaves the aperture below k+1: flush at k+1
                    const dfl u = df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[min(e, d.ne - 1)], xu)), zu2)), utx);
                    const float2 tt = cmul(cis_ku(k + 1, u), A[q]);
                    part.x = fmaf(bo, tt.x, part.x);
                    part.y = fmaf(bo, tt.y, part.y);
                  }
                  A[q] = make_float2(0.0f, 0.0f);
                }
                ar[q] = an;
              }
            }
            const float2* xr = &xb[(k - kc_lo) * ROW];
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
              const float2 x = xr[q];
              const float2 Aq = A[q], zq = z[q];
              A[q].x = fmaf(Aq.x, zq.x, fmaf(-Aq.y, zq.y, x.x));
              A[q].y = fmaf(Aq.x, zq.y, fmaf(Aq.y, zq.x, x.y));
            }
          }
          if (chunk % d.flush_chunks == 0) {
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
              const float bq = f * ar[q];
              if (bq != 0.0f) {
                const dfl u = df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[min(r0 + q, d.ne - 1)], xu)), zu2)), utx);
                const float2 tt = cmul(cis_ku(kc_lo, u), A[q]);
                part.x = fmaf(bq, tt.x, part.x);
                part.y = fmaf(bq, tt.y, part.y);
              }
              A[q] = make_float2(0.0f, 0.0f);
            }
          }
        }
        float y = part.x - comp.x, tt = acc.x + y;
        comp.x = (tt - acc.x) - y;
        acc.x = tt;
        y = part.y - comp.y;
        tt = acc.y + y;
        comp.y = (tt - acc.y) - y;
        acc.y = tt;
      }
    }
    if (valid) image[(size_t)ic * d.nz + jc] = make_float2(acc.x * d.scale, acc.y * d.scale);
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd(&d.counters[0], s_count[0]);
    atomicAdd(&d.counters[1], s_count[1]);
    atomicAdd(&d.counters[4], n_exec);
  }
}

// Synthetic-aperture recurrence for a boxcar receive window.  A receive
// element is then either out of the aperture or in it with the weight
// f = a_tx(t) / (W_tx W_rx) shared by the whole pass, so a segment boundary
// reduces to the new f and the mask of the pass's receive elements that are
// in.  Ahead of the recurrence each lane resolves its own boundaries of the
// next SA_EV_BINS bins into a table {f, mask} in shared memory (a column per
// lane) and a bit mask of the bins that carry one; the bin loop only applies
// them: one common rescale ratio for the elements that stay in, zero for the
// ones that enter, a flush for the ones that leave.  The boundary work is done
// per lane instead of per bin of the warp, and the arithmetic is that of
// sa_fused_kernel with a boxcar receive window.
constexpr int SA_EV_BINS = 32;

// Issues the copy of one spectrum chunk for sa_event_kernel: per bin, chains in pairs
// (2p, 2p+1) laid out {re_2p, re_2p+1, im_2p, im_2p+1}, so one 16-byte load feeds the
// packed recurrence of a pair.
template <int EPT>
__device__ __forceinline__ void sa_stage_chunk_pairs(float* dst, const SADev& d, int t, int r0, int kc_lo, int nk,
                                                     int tid, const float2* X) {
  constexpr int ROW = 2 * EPT;
  for (int idx = tid; idx < KCHUNK * EPT; idx += NTHREADS) {
    const int kk = idx % KCHUNK, q = idx / KCHUNK;
    const int r = r0 + q;
    if (kk >= nk) continue;
    float* o = &dst[kk * ROW + 4 * (q >> 1) + (q & 1)];
    if (r < d.ne) {
      const float* src = reinterpret_cast<const float*>(&X[((size_t)t * d.ne + r) * d.K + (kc_lo - d.k_lb + kk)]);
      cp_async4(o, src);
      cp_async4(o + 2, src + 1);
    } else {
      o[0] = 0.0f;
      o[2] = 0.0f;
    }
  }
  cp_async_commit();
}

template <int EPT, int WT>
__global__ void __launch_bounds__(NTHREADS, 4)
sa_event_kernel(const SADev d, float2* __restrict__ image, float* __restrict__ wtx_out, float* __restrict__ wrx_out,
                int n_tiles_x, int n_tiles_z, int weights_only) {
  static_assert(EPT <= 31 && EPT % 2 == 0, "receive mask, chain pairs");
  constexpr int NP = EPT / 2;     // chains are processed in pairs by packed FP32x2 instructions
  constexpr int ROW = 2 * EPT;    // floats per bin: per pair {re, re, im, im}
  __shared__ __align__(16) float xs[2][KCHUNK * ROW];
  __shared__ float2 ev[SA_EV_BINS][NTHREADS];        // {f from the bin on, receive mask}
  __shared__ int ranges[4];
  __shared__ int s_tile;
  __shared__ unsigned long long s_count[2];          // active terms, zero-weight bins
  extern __shared__ __align__(16) unsigned char dyn[];  // lb[ne], ub[ne] (dfl), ktop_tx[ne], ktop_rx[ne]
  dfl* lb_s = (dfl*)dyn;
  dfl* ub_s = lb_s + d.ne;
  int* ktop_tx = (int*)(ub_s + d.ne);
  int* ktop_rx = ktop_tx + d.ne;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_tiles = n_tiles_x * n_tiles_z;
  int4* seg = d.seg + ((size_t)blockIdx.x * NTHREADS + tid) * (size_t)d.seg_cap * SA_SEG_INT4;
  const float ipt = (d.wtx_par > 0.0f) ? 1.0f / d.wtx_par : 0.0f;
  const float2* Xsrc = d.Xs ? d.Xs : d.X;
  unsigned long long n_exec = 0;
  if (tid == 0) s_count[0] = s_count[1] = 0ull;
  for (int e = tid; e < d.ne; e += NTHREADS) {
    lb_s[e] = d.el_lb[e];
    ub_s[e] = d.el_ub[e];
  }

  for (;;) {
    if (tid == 0) s_tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < 2 * d.ne; e += NTHREADS) ktop_tx[e] = -1;
    if (tid == 0) {
      ranges[0] = ranges[2] = d.ne;
      ranges[1] = ranges[3] = -1;
    }
    __syncthreads();
    const int tile = s_tile;
    if (tile >= n_tiles) break;
    int tx_, tz_;
    tile_coords(tile, n_tiles_x, n_tiles_z, tx_, tz_);
    const int i = tx_ * TILE_X + warp;
    const int j = tz_ * TILE_Z + lane;
    const bool valid = (i < d.nx) && (j < d.nz);
    const int ic = min(i, d.nx - 1), jc = min(j, d.nz - 1);
    int nseg;
    {
      float Wtx_top, Wrx_top;
      unsigned long long n_active = 0, n_empty = 0;
      nseg = sa_build_segments(d, ic, jc, valid, seg, ktop_tx, ktop_rx, ranges, Wtx_top, Wrx_top, n_active, n_empty);
      atomicAdd(&s_count[0], n_active);
      atomicAdd(&s_count[1], n_empty);
      if (valid) {
        if (wtx_out) wtx_out[(size_t)ic * d.nz + jc] = Wtx_top;
        if (wrx_out) wrx_out[(size_t)ic * d.nz + jc] = Wrx_top;
      }
    }
    __syncthreads();
    const int T_lo = ranges[0], T_hi = weights_only ? -1 : ranges[1], R_lo = ranges[2], R_hi = ranges[3];

    const dfl xm = d.col_m[ic], xu = d.col_u[ic], zu2 = d.row_u2[jc];
    const int emid = d.col_emid[ic];
    float2 acc = make_float2(0.0f, 0.0f), comp = make_float2(0.0f, 0.0f);

    for (int t = T_lo; t <= T_hi; ++t) {
      const int kt_t = ktop_tx[t];
      if (kt_t < d.k_lb) continue;
      const dfl ctm = d.el_m[t];
      const float dxt = fabsf((ctm.x - xm.x) + (ctm.y - xm.y));
      // transmit delay plus the time offset t0 / N (the reference's argument_add)
      const dfl utx = df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[t], xu)), zu2)), d.t0N);
      for (int r0 = d.Xs ? max(R_lo, t) : R_lo; r0 <= R_hi; r0 += EPT) {
        int kt = -1;
#pragma unroll
        for (int q = 0; q < EPT; ++q)
          if (r0 + q <= R_hi) kt = max(kt, ktop_rx[r0 + q]);
        kt = min(kt, kt_t);
        if (kt < d.k_lb) continue;
        if (tid == 0) n_exec += (unsigned long long)(kt - d.k_lb + 1) * EPT * NTHREADS;
        // receive elements r0 + q in [m_lo, m_hi] form the mask of an aperture
        const int m_hi_cap = min(R_hi, r0 + EPT - 1);
        auto rx_mask = [&](int rcode) -> unsigned {
          const int lo = max(min(code_ilb(rcode), emid), r0);
          const int hi = min(max(code_iub(rcode), emid - 1), m_hi_cap);
          return (lo <= hi) ? ((2u << (hi - r0)) - (1u << (lo - r0))) : 0u;
        };
        // per pair of chains: accumulators {re, re}, {im, im} and steps {re, re}, {im, im}, {-im, -im}
        float2 AR[NP], AI[NP], ZR[NP], ZI[NP], NZI[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          const float2 z0 = cis_ku(1, df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[min(r0 + 2 * p, d.ne - 1)], xu)), zu2)), utx));
          const float2 z1 =
              cis_ku(1, df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[min(r0 + 2 * p + 1, d.ne - 1)], xu)), zu2)), utx));
          ZR[p] = make_float2(z0.x, z1.x);
          ZI[p] = make_float2(z0.y, z1.y);
          NZI[p] = make_float2(-z0.y, -z1.y);
          AR[p] = AI[p] = make_float2(0.0f, 0.0f);
        }
        auto getA = [&](int q) -> float2 {
          return (q & 1) ? make_float2(AR[q >> 1].y, AI[q >> 1].y) : make_float2(AR[q >> 1].x, AI[q >> 1].x);
        };
        auto setA = [&](int q, float2 v) {
          if (q & 1) {
            AR[q >> 1].y = v.x;
            AI[q >> 1].y = v.y;
          } else {
            AR[q >> 1].x = v.x;
            AI[q >> 1].x = v.y;
          }
        };
        // segment in effect at kt, and the state of the boundary pre-pass:
        // tx code and tx window value of the last resolved entry
        int s = 0;
        int4 cur = make_int4(-1, seg_code(d.ne, -1), seg_code(d.ne, -1), 0);
        if (nseg > 0) {
          s = sa_seg_find(seg, nseg, kt);
          cur = seg[s];
        }
        int4 ring[SEG_RING];
#pragma unroll
        for (int r = 0; r < SEG_RING; ++r) ring[r] = seg[min(s + 1 + r, nseg)];
        int p_ct = cur.y;
        float p_at = sa_apod<WT>(lb_s, ub_s, xm, t, emid, code_ilb(cur.y), code_iub(cur.y), dxt, d.wtx_par, ipt);
        float f = p_at * __int_as_float(cur.w);
        unsigned m = (f != 0.0f) ? rx_mask(cur.z) : 0u;

        float2 part = make_float2(0.0f, 0.0f);
        const int c_top = (kt - d.k_lb) / KCHUNK;
        __syncthreads();  // every thread is done with both buffers of the previous pass
        sa_stage_chunk_pairs<EPT>(xs[0], d, t, r0, d.k_lb + c_top * KCHUNK, kt - (d.k_lb + c_top * KCHUNK) + 1, tid,
                                  Xsrc);
        int buf = 0;
        for (int chunk = c_top; chunk >= 0; --chunk) {
          const int kc_lo = d.k_lb + chunk * KCHUNK;
          const int kc_hi = (chunk == c_top) ? kt : kc_lo + KCHUNK - 1;
          cp_async_wait_all();
          __syncthreads();
          if (chunk > 0) sa_stage_chunk_pairs<EPT>(xs[buf ^ 1], d, t, r0, kc_lo - KCHUNK, KCHUNK, tid, Xsrc);
          const float* xb = xs[buf];
          buf ^= 1;
          for (int ks_hi = kc_hi; ks_hi >= kc_lo; ks_hi -= SA_EV_BINS) {
            const int ks_lo = max(kc_lo, ks_hi - (SA_EV_BINS - 1));
            // this lane's boundaries in bins ks_lo .. ks_hi (entries sorted by
            // k_start, descending; the sentinel's bin -1 ends the walk)
            unsigned emask = 0u;
            while (ring[0].x >= ks_lo) {
              const int4 c = ring[0];
#pragma unroll
              for (int r = 0; r + 1 < SEG_RING; ++r) ring[r] = ring[r + 1];
              ++s;
              ring[SEG_RING - 1] = seg[min(s + SEG_RING, nseg)];
              if (c.y != p_ct || p_at == 0.0f)
                p_at = sa_apod<WT>(lb_s, ub_s, xm, t, emid, code_ilb(c.y), code_iub(c.y), dxt, d.wtx_par, ipt);
              p_ct = c.y;
              const float fn = p_at * __int_as_float(c.w);
              const unsigned mn = (fn != 0.0f) ? rx_mask(c.z) : 0u;
              ev[c.x - ks_lo][tid] = make_float2(fn, __uint_as_float(mn));
              emask |= 1u << (c.x - ks_lo);
            }
            int nev = emask ? ks_lo + 31 - __clz(emask) : -1;
            for (int k = ks_hi; k >= ks_lo; --k) {
              if (k == nev) {
                const float2 en = ev[k - ks_lo][tid];
                const float fn = en.x;
                const unsigned mn = __float_as_uint(en.y);
                const unsigned leave = m & ~mn, stay = m & mn;
                if (leave) {  // receive elements that leave the aperture below k+1: flush at k+1
#pragma unroll
                  for (int q = 0; q < EPT; ++q) {
                    if ((leave >> q) & 1u) {
                      const dfl u = df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[r0 + q], xu)), zu2)), utx);
                      const float2 tt = cmul(cis_ku(k + 1, u), getA(q));
                      part.x = fmaf(f, tt.x, part.x);
                      part.y = fmaf(f, tt.y, part.y);
                    }
                  }
                }
                const float r = stay ? __fdividef(f, fn) : 0.0f;
                if (stay == m && mn == m) {
                  const float2 rr = make_float2(r, r);
#pragma unroll
                  for (int p = 0; p < NP; ++p) {
                    AR[p] = __fmul2_rn(AR[p], rr);
                    AI[p] = __fmul2_rn(AI[p], rr);
                  }
                } else {
#pragma unroll
                  for (int q = 0; q < EPT; ++q) {
                    const bool st = (stay >> q) & 1u;
                    const float2 a = getA(q);
                    setA(q, make_float2(st ? a.x * r : 0.0f, st ? a.y * r : 0.0f));
                  }
                }
                f = fn;
                m = mn;
                emask &= ~(1u << (k - ks_lo));
                nev = emask ? ks_lo + 31 - __clz(emask) : -1;
              }
              const float4* xr = reinterpret_cast<const float4*>(&xb[(k - kc_lo) * ROW]);
              // A <- A z + x per chain, two chains per packed instruction (the same fused
              // operations as fmaf(Ax, zx, fmaf(-Ay, zy, xr)), fmaf(Ax, zy, fmaf(Ay, zx, xi)))
#pragma unroll
              for (int p = 0; p < NP; ++p) {
                const float4 xv = xr[p];
                const float2 ar = AR[p], ai = AI[p];
                AR[p] = __ffma2_rn(ar, ZR[p], __ffma2_rn(ai, NZI[p], make_float2(xv.x, xv.y)));
                AI[p] = __ffma2_rn(ar, ZI[p], __ffma2_rn(ai, ZR[p], make_float2(xv.z, xv.w)));
              }
            }
          }
          if (chunk % d.flush_chunks == 0) {
#pragma unroll
            for (int q = 0; q < EPT; ++q) {
              if ((m >> q) & 1u) {
                const dfl u = df_add(df_sqrt(df_add(df_sqr(df_sub(d.el_u[r0 + q], xu)), zu2)), utx);
                const float2 tt = cmul(cis_ku(kc_lo, u), getA(q));
                part.x = fmaf(f, tt.x, part.x);
                part.y = fmaf(f, tt.y, part.y);
              }
            }
#pragma unroll
            for (int p = 0; p < NP; ++p) AR[p] = AI[p] = make_float2(0.0f, 0.0f);
          }
        }
        float y = part.x - comp.x, tt = acc.x + y;
        comp.x = (tt - acc.x) - y;
        acc.x = tt;
        y = part.y - comp.y;
        tt = acc.y + y;
        comp.y = (tt - acc.y) - y;
        acc.y = tt;
      }
    }
    if (valid) image[(size_t)ic * d.nz + jc] = make_float2(acc.x * d.scale, acc.y * d.scale);
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd(&d.counters[0], s_count[0]);
    atomicAdd(&d.counters[1], s_count[1]);
    atomicAdd(&d.counters[4], n_exec);
  }
}

constexpr int SA_EPT = 8;      // receive chains per pass, boundaries resolved in the bin loop
constexpr int SA_EV_EPT = 12;  // receive chains per pass of sa_event_kernel
typedef void (*sa_kernel_t)(const SADev, float2*, float*, float*, int, int, int);

template <int WT>
static sa_kernel_t sa_pick_rx(int wr) {
  switch (wr) {
    case 0: return sa_event_kernel<SA_EV_EPT, WT>;   // boxcar receive window
    case 1: return sa_fused_kernel<SA_EPT, WT, 1>;
    case 2: return sa_fused_kernel<SA_EPT, WT, 2>;
    default: return sa_fused_kernel<SA_EPT, WT, 4>;
  }
}
static sa_kernel_t sa_pick(int wt, int wr) {
  switch (wt) {
    case 0: return sa_pick_rx<0>(wr);
    case 1: return sa_pick_rx<1>(wr);
    case 2: return sa_pick_rx<2>(wr);
    default: return sa_pick_rx<4>(wr);
  }
}
static size_t sa_smem(const SADev& d) { return (size_t)d.ne * (2 * sizeof(dfl) + 2 * sizeof(int)); }

int sa_fused_grid(const SADev& d, int* blocks_per_sm) {
  int dev = 0, nsm = 0, bps = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, sa_pick(d.wtx_id, d.wrx_id), NTHREADS, sa_smem(d));
  if (bps < 1) bps = 1;
  if (blocks_per_sm) *blocks_per_sm = bps;
  const int tiles = ((d.nx + TILE_X - 1) / TILE_X) * ((d.nz + TILE_Z - 1) / TILE_Z);
  return tiles < nsm * bps ? tiles : nsm * bps;
}

// Xs[t][r] = X[t][r] + X[r][t] for t < r and X[t][t] for t = r; the lower triangle is not read
__global__ void __launch_bounds__(256) sa_symmetrize_kernel(const SADev d) {
  const size_t n = (size_t)d.ne * d.ne * d.K;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(i % d.K);
    const size_t tr = i / d.K;
    const int r = (int)(tr % d.ne), t = (int)(tr / d.ne);
    if (r < t) continue;
    float2 x = d.X[i];
    if (r > t) {
      const float2 y = d.X[((size_t)r * d.ne + t) * d.K + k];
      x.x += y.x;
      x.y += y.y;
    }
    d.Xs[i] = x;
  }
}

cudaError_t launch_sa_fused(const SADev& d, int grid, float2* image, float* wtx, float* wrx, cudaStream_t s) {
  const int ntx = (d.nx + TILE_X - 1) / TILE_X, ntz = (d.nz + TILE_Z - 1) / TILE_Z;
  // each launch draws tiles from a fresh counter
  cudaError_t e = cudaMemsetAsync(d.counters + 3, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (d.Xs) sa_symmetrize_kernel<<<1216, 256, 0, s>>>(d);
  sa_pick(d.wtx_id, d.wrx_id)<<<grid, NTHREADS, sa_smem(d), s>>>(d, image, wtx, wrx, ntx, ntz,
                                                                  d.last_bin_only < 0 ? 1 : 0);
  return cudaGetLastError();
}

// plain per-voxel SAFT kernel: saft_kernel_phase_shifts.cu arithmetic per term
__global__ void __launch_bounds__(NTHREADS) sa_plain_kernel(const SADev d, float2* image, float* wtx_out,
                                                            float* wrx_out) {
  const int i = blockIdx.x * TILE_X + (threadIdx.x >> 5);
  const int j = blockIdx.y * TILE_Z + (threadIdx.x & 31);
  if (i >= d.nx || j >= d.nz) return;
  const float x = d.px_f[i], z = d.pz_f[j];
  float2 img = make_float2(0.0f, 0.0f);
  float Wt_last = 0.0f, Wr_last = 0.0f;
  for (int kk = 0; kk < d.K; ++kk) {
    const int k = d.k_lb + kk;
    const float Ft = d.Ftx_f[kk], Fr = d.Frx_f[kk];
    float sr = 0.0f, si = 0.0f, Wt = 0.0f, Wr = 0.0f;
    for (int t = 0; t < d.ne; ++t) {
      const float dxt = d.ctr_f[t] - x;  // das_kernel_distances_sw.cu:26-28 with z_tx = 0
      const float dtx = __fsqrt_rn(dxt * dxt + z * z);
      const float at = ref_apod(d.wtx_id, d.wtx_par, Ft, x, z, dxt, d.lb_f, d.ub_f, d.ne, d.M_f, d.pitch_f);
      Wt += at;
      for (int r = 0; r < d.ne; ++r) {
        const float dx = d.ctr_f[r] - x;
        const float drt = dtx + __fsqrt_rn(dx * dx + z * z);
        const float ar = ref_apod(d.wrx_id, d.wrx_par, Fr, x, z, dx, d.lb_f, d.ub_f, d.ne, d.M_f, d.pitch_f);
        if (t == 0) Wr += ar;
        float sn, cs;
        __sincosf((float)k * (d.coef_f * drt + d.add_f), &sn, &cs);
        const float2 X = d.X[((size_t)t * d.ne + r) * d.K + kk];
        const float pr = at * ar * cs, pi = at * ar * sn;
        sr += pr * X.x - pi * X.y;
        si += pr * X.y + pi * X.x;
      }
    }
    float den = 1.0f;
    if (d.norm_rx) den *= Wr;
    if (d.norm_tx) den *= Wt;
    if (d.last_bin_only > 0) {
      if (kk == d.K - 1) {
        img.x = sr;
        img.y = si;
      }
    } else if (den != 0.0f) {
      img.x += sr / den;
      img.y += si / den;
    }
    Wt_last = Wt;
    Wr_last = Wr;
  }
  if (d.last_bin_only < 0) img = make_float2(0.0f, 0.0f);
  image[(size_t)i * d.nz + j] = make_float2(img.x * d.scale, img.y * d.scale);
  if (wtx_out) wtx_out[(size_t)i * d.nz + j] = Wt_last;
  if (wrx_out) wrx_out[(size_t)i * d.nz + j] = Wr_last;
}

cudaError_t launch_sa_plain(const SADev& d, float2* image, float* wtx, float* wrx, cudaStream_t s) {
  dim3 grid((d.nx + TILE_X - 1) / TILE_X, (d.nz + TILE_Z - 1) / TILE_Z);
  sa_plain_kernel<<<grid, NTHREADS, 0, s>>>(d, image, wtx, wrx);
  return cudaGetLastError();
}

}  // namespace fnum

namespace fnum {

// ---------------------------------------------------------------------------
// Gradients of an image-sharpness loss of the compounded plane-wave image
//   L = -S4 / S2^2,  S2 = sum_v |I_v|^2,  S4 = sum_v |I_v|^4,
// with the DFT order, band, F table and apertures frozen (only the phases
// depend on the sound speed).  dL/dI_v* = G_v = -2 I_v (|I_v|^2/S2^2 - S4/S2^3).
//   dL/dX*_{e,k,a} = (2/N) sum_v G_v b_{v,e,k} e^{-j 2 pi k u_{v,e,a}}
//   dL/dc = 2 Re sum_{e,k,a} X (-j 2 pi k / c) (2/N) conj(H_{e,k,a}),
//   H_{e,k,a} = sum_v G_v b_{v,e,k} e^{-j 2 pi k u} U_{v,e,a},  U = u - t0/N,
// because u = f_s/(N c) (d_tx + d_rx) + t0/N gives du/dc = -U/c.
// No counterpart in the reference.
// ---------------------------------------------------------------------------

// 1/W (or 1, or 0 for an empty aperture) per voxel and band bin: [voxel][K]
template <int WIN>
__global__ void __launch_bounds__(NTHREADS) pw_invw_kernel(const PWDev d, float* __restrict__ invw) {
  const long long v = (long long)blockIdx.x * NTHREADS + threadIdx.x;
  if (v >= (long long)d.nx * d.nz) return;
  const int i = (int)(v / d.nz), j = (int)(v - (long long)i * d.nz);
  const dfl xp = d.col_p[i], zp = d.row_p[j], xm = d.col_m[i];
  const int emid = d.col_emid[i];
  const float inv_par = (d.window_par > 0.0f) ? 1.0f / d.window_par : 0.0f;
  int prev = -1;
  float iw = 0.0f;
  for (int kk = 0; kk < d.K; ++kk) {
    int ilb, iub;
    aperture(xp, zp, d.g[kk], d.ne, ilb, iub);
    const int code = seg_code(ilb, iub);
    if (code != prev) {
      const float Ll = half_left(d.el_lb, xm, ilb, d.ne), Lr = half_right(d.el_ub, xm, iub);
      const float W = aperture_sum_closed<WIN>(d, inv_par, xm, emid, ilb, iub, (Ll > 0.0f) ? 1.0f / Ll : 0.0f,
                                               (Lr > 0.0f) ? 1.0f / Lr : 0.0f);
      iw = (W > 0.0f) ? (d.norm ? 1.0f / W : 1.0f) : 0.0f;
      prev = code;
    }
    invw[(size_t)v * d.K + kk] = iw;
  }
}

// S2, S4 of an image (double accumulation)
__global__ void __launch_bounds__(256) pw_sharp_sums_kernel(const float2* __restrict__ img, long long n,
                                                            double* __restrict__ sums) {
  __shared__ double r2[8], r4[8];
  double s2 = 0.0, s4 = 0.0;
  for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const float2 v = img[i];
    const double m2 = (double)v.x * v.x + (double)v.y * v.y;
    s2 += m2;
    s4 += m2 * m2;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    s4 += __shfl_xor_sync(0xffffffffu, s4, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r2[threadIdx.x >> 5] = s2;
    r4[threadIdx.x >> 5] = s4;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < 8; ++w) {
      a += r2[w];
      b += r4[w];
    }
    atomicAdd(&sums[0], a);
    atomicAdd(&sums[1], b);
  }
}

// dL/dc = coef sum_v Im(conj(G_v) Draw_v), coef = 4 pi / c (dI/dc = -(2 pi i / c) Draw)
__global__ void __launch_bounds__(256) pw_dc_reduce_kernel(const float2* __restrict__ G, const float2* __restrict__ D,
                                                           long long n, double coef, double* __restrict__ out) {
  __shared__ double r[8];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const float2 g = G[i], dv = D[i];
    s += (double)g.x * dv.y - (double)g.y * dv.x;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) r[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < 8; ++w) a += r[w];
    atomicAdd(out, coef * a);
  }
}

cudaError_t launch_pw_invw(const PWDev& d, float* invw, cudaStream_t s) {
  const long long nv = (long long)d.nx * d.nz;
  const int grid = (int)((nv + NTHREADS - 1) / NTHREADS);
  switch (d.window_id) {
    case 0: pw_invw_kernel<0><<<grid, NTHREADS, 0, s>>>(d, invw); break;
    case 1: pw_invw_kernel<1><<<grid, NTHREADS, 0, s>>>(d, invw); break;
    case 2: pw_invw_kernel<2><<<grid, NTHREADS, 0, s>>>(d, invw); break;
    default: pw_invw_kernel<4><<<grid, NTHREADS, 0, s>>>(d, invw); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_pw_sharp_sums(const float2* img, long long n, double* sums, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(sums, 0, 2 * sizeof(double), s);
  if (e != cudaSuccess) return e;
  pw_sharp_sums_kernel<<<1216, 256, 0, s>>>(img, n, sums);
  return cudaGetLastError();
}

// cotangent of the sharpness loss L = -S4 / S2^2: dL/dI*_v = -2 I_v (|I_v|^2 / S2^2 - S4 / S2^3)
__global__ void __launch_bounds__(256) pw_sharp_cotangent_kernel(const float2* __restrict__ img, long long n, float gs2,
                                                                 float gs4, float2* __restrict__ G) {
  for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long long)gridDim.x * blockDim.x) {
    const float2 I = img[v];
    const float cg = -2.0f * ((I.x * I.x + I.y * I.y) * gs2 - gs4);
    G[v] = make_float2(cg * I.x, cg * I.y);
  }
}

cudaError_t launch_pw_sharp_cotangent(const float2* img, long long n, float gs2, float gs4, float2* G, cudaStream_t s) {
  pw_sharp_cotangent_kernel<<<1216, 256, 0, s>>>(img, n, gs2, gs4, G);
  return cudaGetLastError();
}

// fp16 scale of Q = conj(t^k) G / W: the power of two that brings max|G| max(1/W), a bound
// of |Q|, below 2^14 (gmax: float bits of max |G component| and of max 1/W)
__device__ __forceinline__ float adj_scale(const unsigned* gmax) {
  const float m = __uint_as_float(gmax[0]) * __uint_as_float(gmax[1]);
  if (!(m > 0.0f) || !(m < 3.0e38f)) return 1.0f;
  int ex;
  frexpf(m, &ex);
  return ldexpf(1.0f, min(max(14 - ex, -126), 126));
}

// largest |x| of n floats (float bits, >= 0 floats order as integers) into *out
__global__ void __launch_bounds__(256) absmax_f32_kernel(const float* __restrict__ x, size_t n, unsigned* out) {
  float m = 0.0f;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// FP64 sums {Xr, Xi} per (element, bin, angle) -> dL/dX* (scaled by 2/N, the fp16 scale undone)
__global__ void __launch_bounds__(256) pw_adjoint_finish_kernel(const double* __restrict__ acc, size_t n, double scale,
                                                                const unsigned* __restrict__ gmax,
                                                                float2* __restrict__ gX) {
  const double sc = scale / (double)adj_scale(gmax);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double* a = acc + 2 * i;
    gX[i] = make_float2((float)(sc * a[0]), (float)(sc * a[1]));
  }
}

// ---------------------------------------------------------------------------
// The adjoint on the tensor cores: per band bin k,
//   gX_k(e, a) = s sum_v conj(R_k(v, e)) Q_k(v, a),  R_k = b r^k,  Q_k = conj(t_va^k) G_v / W_vk,
// an [elements x voxels] . [voxels x angles] product reduced over the voxels (the
// forward's product transposed).  Block: 8 warps, warp w owns elements 16w..16w+15 of
// the block's element pass (mma rows); the voxels are the mma k dimension (8 complex per
// k-step, real form: columns 0..7 Re, 8..15 Im of conj(R)) and the angles the n dimension
// (3 tiles of 4).  A block takes one chunk of ADJ_TB bins and one slice of voxels; per
// group of 8 voxels it stages the aperture data and the B fragments of Q (fp16 hi and lo,
// scaled by a power of two) in shared memory, then each warp forms conj(R) for its 16
// elements x 8 voxels -- the receive phasor anchored exactly at the chunk's top bin and
// stepped down by r -- and accumulates the chunk's bins in registers (ADJ_TB x 12 floats).
// At the end of the slice the sums are added to FP64 accumulators.
constexpr int ADJ_TB = 6;           // bins per chunk (register accumulators per bin)
constexpr int ADJ_TC_SLICE = 8192;  // voxels per block
constexpr int ADJ_TC_WARPS = 8;

// e^{j 2 pi k u} with the exact reduction of cis_ku and the hardware sine and cosine of the
// reduced angle (absolute error below 4e-7): the adjoint's anchors
__device__ __forceinline__ float2 cis_ku_fast(int k, dfl u) {
  const float kf = (float)k;
  dfl p = two_prod(kf, u.x);
  const float n = rintf(p.x);
  const float rh = p.x - n;
  const float rl = fmaf(kf, u.y, p.y);
  const float r = rh + rl;
  float sn, cs;
  __sincosf(6.28318530717958647692f * r, &sn, &cs);
  return make_float2(cs, sn);
}

// the adjoint's receive table: u_rx in double-float and the step e^{2 pi i u_rx} of every
// (voxel, element) pair, formed as pw_adjoint_tc_kernel forms them without the table
__global__ void __launch_bounds__(256) pw_rx_table_kernel(const PWDev d) {
  const size_t n = (size_t)d.nx * d.nz * d.ne;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const size_t v = idx / d.ne;
    const int e = (int)(idx - v * d.ne);
    const int i = (int)(v / d.nz), j = (int)(v - (size_t)i * d.nz);
    const dfl urx = df_sqrt(df_add(df_sqr(df_sub(d.el_u[e], d.col_u[i])), d.row_u2[j]));
    const float2 st = cis_ku_fast(1, urx);
    d.rx_tab[idx] = make_float4(urx.x, urx.y, st.x, st.y);
  }
}

template <int WIN>
__global__ void __launch_bounds__(ADJ_TC_WARPS * 32, 2)
pw_adjoint_tc_kernel(const PWDev d, const float2* __restrict__ cot, const float* __restrict__ invw,
                     const unsigned* __restrict__ gmax, double* __restrict__ acc) {
  __shared__ float2 sQ[ADJ_TB][8][TC_NA];        // Q_k(v, a) sigma
  __shared__ uint4 sB[ADJ_TB][3][32];            // B fragments {b0 hi, b1 hi, b0 lo, b1 lo}
  __shared__ float2 sAp[ADJ_TB][8];              // {1/L_left, 1/L_right} per bin, voxel (1e30: no side)
  __shared__ int sVox[8][3];                     // column, row, first element right of x
  __shared__ int2 sRng[ADJ_TB][8];               // aperture element range {ilb, iub} per bin, voxel
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int kc_lo = d.k_lb + blockIdx.x * ADJ_TB, kc_hi = min(kc_lo + ADJ_TB, d.k_ub + 1) - 1;
  const int nb = kc_hi - kc_lo + 1;
  const long long nvox = (long long)d.nx * d.nz;
  const long long v_begin = (long long)blockIdx.y * ADJ_TC_SLICE;
  const long long v_end = min(nvox, v_begin + ADJ_TC_SLICE);
  const int e_pass = blockIdx.z * (ADJ_TC_WARPS * 16);
  const int eA = e_pass + 16 * warp + g, eB = eA + 8;   // the thread's elements (mma rows g, g + 8)
  const dfl cmA = d.el_m[min(eA, d.ne - 1)], cmB = d.el_m[min(eB, d.ne - 1)];
  const dfl cuA = d.el_u[min(eA, d.ne - 1)], cuB = d.el_u[min(eB, d.ne - 1)];
  const float inv_par = (d.window_par > 0.0f) ? 1.0f / d.window_par : 0.0f;
  const float sigma = adj_scale(gmax);
  float C[ADJ_TB][3][4];
#pragma unroll
  for (int b = 0; b < ADJ_TB; ++b)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[b][j][0] = C[b][j][1] = C[b][j][2] = C[b][j][3] = 0.0f;

  for (long long v0 = v_begin; v0 < v_end; v0 += 8) {
    const int nv = (int)min(8ll, v_end - v0);
    __syncthreads();   // the previous group's tables are consumed
    if (tid < 8) {
      const long long v = v0 + min(tid, nv - 1);
      const int i = (int)(v / d.nz), j = (int)(v - (long long)i * d.nz);
      sVox[tid][0] = i;
      sVox[tid][1] = j;
      sVox[tid][2] = d.col_emid[i];
    }
    __syncthreads();
    // Q (96 threads: voxel x angle) and the aperture data (ADJ_TB x 8 threads)
    if (tid < 8 * TC_NA) {
      const int vv = tid / TC_NA, a = tid - vv * TC_NA;
      float2 base = make_float2(0.0f, 0.0f), t = make_float2(1.0f, 0.0f);
      if (vv < nv && a < d.na) {
        const int i = sVox[vv][0], j = sVox[vv][1];
        const dfl ut = df_add(d.tx_ax[(size_t)a * d.nx + i], d.tx_az[(size_t)a * d.nz + j]);
        const float2 c = cis_ku_fast(kc_hi, ut);
        const float2 G = cot[v0 + vv];
        t = cis_ku_fast(1, ut);
        // conj(t^k) G sigma at the top bin; going down, conj(t^(k-1)) = conj(t^k) t
        base = make_float2(sigma * (G.x * c.x + G.y * c.y), sigma * (G.y * c.x - G.x * c.y));
      }
#pragma unroll
      for (int b = 0; b < ADJ_TB; ++b) {
        float2 qv = make_float2(0.0f, 0.0f);
        if (vv < nv && a < d.na && b < nb) {
          const float iw = invw[(size_t)(v0 + vv) * d.K + (kc_hi - b - d.k_lb)];
          qv = make_float2(base.x * iw, base.y * iw);
        }
        sQ[b][vv][a] = qv;
        base = cmul(base, t);
      }
    } else if (tid >= 128 && tid < 128 + ADJ_TB * 8) {
      const int b = (tid - 128) >> 3, vv = (tid - 128) & 7;
      float il = 1.0e30f, ir = 1.0e30f;
      int2 rng = make_int2(d.ne, -1);
      if (vv < nv && b < nb) {
        const int i = sVox[vv][0], j = sVox[vv][1];
        const dfl xm = d.col_m[i];
        int ilb, iub;
        aperture(d.col_p[i], d.row_p[j], d.g[kc_hi - b - d.k_lb], d.ne, ilb, iub);
        rng = make_int2(ilb, iub);
        if (ilb < d.ne) {
          const dfl l = d.el_lb[ilb];
          const float L = (xm.x - l.x) + (xm.y - l.y);
          if (L > 0.0f) il = __fdividef(1.0f, L);
        }
        if (iub >= 0) {
          const dfl u = d.el_ub[iub];
          const float L = (u.x - xm.x) + (u.y - xm.y);
          if (L > 0.0f) ir = __fdividef(1.0f, L);
        }
      }
      sAp[b][vv] = make_float2(il, ir);
      sRng[b][vv] = rng;
    }
    __syncthreads();
    // B fragments: lane (gg, qq) of n-tile j holds rows 2qq, 2qq+1 (voxels, Re block) and
    // 2qq+8, 2qq+9 (second block) of column gg = angle 4j + gg/2, part gg%2
    for (int f = tid; f < ADJ_TB * 3 * 32; f += ADJ_TC_WARPS * 32) {
      const int b = f / 96, j = (f / 32) % 3, ln = f & 31;
      const int gg = ln >> 2, qq = ln & 3, a = 4 * j + (gg >> 1), part = gg & 1;
      float r0[2], r1[2];
#pragma unroll
      for (int t2 = 0; t2 < 2; ++t2) {
        const float2 qv = sQ[b][2 * qq + t2][a];
        r0[t2] = part ? qv.y : qv.x;     // rows 0..7:  Re Q (column re) / Im Q (column im)
        r1[t2] = part ? qv.x : -qv.y;    // rows 8..15: -Im Q / Re Q
      }
      uint4 o;
      tc_split(r0[0], r0[1], o.x, o.z);
      tc_split(r1[0], r1[1], o.y, o.w);
      sB[b][j][ln] = o;
    }
    __syncthreads();
    // The bins in which one of the warp's 16 elements lies in the aperture range of one
    // of the 8 voxels: elements outside [ilb, iub] have window argument u >= 1 (weight
    // 0), so the other bins add nothing and are skipped, and with them the whole group
    // when none is left.  Lane p checks (bin p / 8, voxel p % 8) and p + 32.
    unsigned act = 0;
    {
      const int w_lo = e_pass + 16 * warp, w_hi = min(w_lo + 15, d.ne - 1);
      bool h0 = false, h1 = false;
      if (lane < ADJ_TB * 8) {
        const int2 r = sRng[lane >> 3][lane & 7];
        h0 = max(r.x, w_lo) <= min(r.y, w_hi);
      }
      if (lane + 32 < ADJ_TB * 8) {
        const int2 r = sRng[(lane + 32) >> 3][lane & 7];
        h1 = max(r.x, w_lo) <= min(r.y, w_hi);
      }
      const unsigned m0 = __ballot_sync(0xffffffffu, h0), m1 = __ballot_sync(0xffffffffu, h1);
#pragma unroll
      for (int b = 0; b < ADJ_TB; ++b) {
        const unsigned byte = (b < 4) ? (m0 >> (8 * b)) : (m1 >> (8 * (b - 4)));
        if (byte & 0xffu) act |= 1u << b;
      }
    }
    if (act == 0) continue;
    // conj(R) of elements (eA, eB) x voxels (2q, 2q+1)
    float2 P[2][2], st[2][2];   // [element][voxel]: conj(r^k) and the step r
    float dl[2][2], dr[2][2];   // distances to the voxel by aperture side
#pragma unroll
    for (int t2 = 0; t2 < 2; ++t2) {
      const int vv = 2 * q + t2;
      const int i = sVox[vv][0], j = sVox[vv][1];
      const dfl xm = d.col_m[i];
      const int emid = sVox[vv][2];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const dfl cm = m ? cmB : cmA;
        const int e = m ? eB : eA;
        dfl urx;
        if (d.rx_tab) {
          const float4 rx = d.rx_tab[(size_t)(v0 + min(vv, nv - 1)) * d.ne + min(e, d.ne - 1)];
          urx = make_float2(rx.x, rx.y);
          st[m][t2] = make_float2(rx.z, rx.w);
        } else {
          const dfl cu = m ? cuB : cuA;
          urx = df_sqrt(df_add(df_sqr(df_sub(cu, d.col_u[i])), d.row_u2[j]));
          st[m][t2] = cis_ku_fast(1, urx);
        }
        const float2 c = cis_ku_fast(kc_hi, urx);
        P[m][t2] = make_float2(c.x, -c.y);
        const float dx = fabsf((cm.x - xm.x) + (cm.y - xm.y));
        const bool ok = (vv < nv) && (e < d.ne);
        const bool left = e < emid;
        dl[m][t2] = ok ? (left ? dx : 0.0f) : 1.0e30f;   // an empty slot lies outside every aperture
        dr[m][t2] = ok ? (left ? 0.0f : dx) : 0.0f;
      }
    }
#pragma unroll
    for (int b = 0; b < ADJ_TB; ++b) {
      if (b < nb && !((act >> b) & 1u)) {
#pragma unroll
        for (int t2 = 0; t2 < 2; ++t2)
#pragma unroll
          for (int m = 0; m < 2; ++m) P[m][t2] = cmul(P[m][t2], st[m][t2]);
      } else if (b < nb) {
        float rr[2][2], ri[2][2];
#pragma unroll
        for (int t2 = 0; t2 < 2; ++t2) {
          const float2 ap = sAp[b][2 * q + t2];
#pragma unroll
          for (int m = 0; m < 2; ++m) {
            const float u = fmaf(dl[m][t2], ap.x, dr[m][t2] * ap.y);
            const float w = (u < 1.0f) ? win_t<WIN>(d.window_par, inv_par, u) : 0.0f;
            const float2 pc = P[m][t2];
            rr[m][t2] = w * pc.x;          // Re conj(R)
            ri[m][t2] = w * pc.y;          // Im conj(R)
            P[m][t2] = cmul(pc, st[m][t2]);
          }
        }
        unsigned ah[4], al[4];
        tc_split(rr[0][0], rr[0][1], ah[0], al[0]);   // row g:     columns 2q, 2q+1
        tc_split(rr[1][0], rr[1][1], ah[1], al[1]);   // row g + 8
        tc_split(ri[0][0], ri[0][1], ah[2], al[2]);   // row g:     columns 2q+8, 2q+9
        tc_split(ri[1][0], ri[1][1], ah[3], al[3]);   // row g + 8
        uint4 bf[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) bf[j] = sB[b][j][lane];
#pragma unroll
        for (int j = 0; j < 3; ++j) tc_mma(C[b][j], ah, bf[j].x, bf[j].y);
#pragma unroll
        for (int j = 0; j < 3; ++j) tc_mma(C[b][j], ah, bf[j].z, bf[j].w);
#pragma unroll
        for (int j = 0; j < 3; ++j) tc_mma(C[b][j], al, bf[j].x, bf[j].y);
      }
    }
  }
  // C[b][j]: rows g, g+8 (elements eA, eB), columns 2q, 2q+1 (angle 4j + q: re, im)
#pragma unroll
  for (int b = 0; b < ADJ_TB; ++b) {
    if (b >= nb) continue;
    const int kk = kc_hi - b - d.k_lb;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int a = 4 * j + q;
      if (a >= d.na) continue;
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        const int e = m ? eB : eA;
        if (e >= d.ne) continue;
        double* o = acc + 2 * (((size_t)e * d.K + kk) * d.na + a);
        atomicAdd(o, (double)C[b][j][2 * m]);
        atomicAdd(o + 1, (double)C[b][j][2 * m + 1]);
      }
    }
  }
}

cudaError_t launch_pw_adjoint(const PWDev& d, const float2* cot, const float* invw, unsigned* gmax, float2* gX,
                              double* acc, cudaStream_t s) {
  const size_t n = (size_t)d.ne * d.K * d.na;
  const long long nvox = (long long)d.nx * d.nz;
  // gmax[1] (max 1/W) is set once with the 1/W table; max |G| per call
  cudaError_t e = cudaMemsetAsync(acc, 0, 2 * n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(gmax, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  absmax_f32_kernel<<<608, 256, 0, s>>>(reinterpret_cast<const float*>(cot), 2 * (size_t)nvox, gmax);
  if (d.rx_tab) pw_rx_table_kernel<<<1216, 256, 0, s>>>(d);
  const dim3 grid((d.K + ADJ_TB - 1) / ADJ_TB, (unsigned)((nvox + ADJ_TC_SLICE - 1) / ADJ_TC_SLICE),
                  (d.ne + ADJ_TC_WARPS * 16 - 1) / (ADJ_TC_WARPS * 16));
  const int nt = ADJ_TC_WARPS * 32;
  switch (d.window_id) {
    case 0: pw_adjoint_tc_kernel<0><<<grid, nt, 0, s>>>(d, cot, invw, gmax, acc); break;
    case 1: pw_adjoint_tc_kernel<1><<<grid, nt, 0, s>>>(d, cot, invw, gmax, acc); break;
    case 2: pw_adjoint_tc_kernel<2><<<grid, nt, 0, s>>>(d, cot, invw, gmax, acc); break;
    default: pw_adjoint_tc_kernel<4><<<grid, nt, 0, s>>>(d, cot, invw, gmax, acc); break;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  pw_adjoint_finish_kernel<<<608, 256, 0, s>>>(acc, n, (double)d.scale, gmax, gX);
  return cudaGetLastError();
}

cudaError_t launch_absmax(const float* x, size_t n, unsigned* out, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  absmax_f32_kernel<<<608, 256, 0, s>>>(x, n, out);
  return cudaGetLastError();
}

cudaError_t launch_pw_dc_reduce(const float2* G, const float2* D, long long n, double coef, double* out,
                               cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(double), s);
  if (e != cudaSuccess) return e;
  pw_dc_reduce_kernel<<<608, 256, 0, s>>>(G, D, n, coef, out);
  return cudaGetLastError();
}

}  // namespace fnum

namespace fnum {

// ---------------------------------------------------------------------------
// das_pw.m semantics (the reference's CPU path, das_pw.m:310-481), per term:
//   N_dft padded with the first axial position; F = min(F(p/lambda), sqrt(f z /
//   (2.88 c))) per bin and depth (das_pw.m:371-377); 1-based aperture indices
//   from z / (2F) in double; boxcar on the ideal half-width z / (2F), other
//   windows on the element-edge half-widths over all elements without a cut-off
//   (das_pw.m:436-452, windows' compute_samples_scalar); normalisation by the
//   sum over elements, times the frequency window of normalizations.windowed
//   (windowed.m:69-87); bins with an empty index range skipped (das_pw.m:403);
//   spectra doubled (analytic signal) and no 2/N scaling (das_pw.m:384,467).
// Phases are exact per term (cis_ku of the delay in cycles per bin, formed in
// double).  One thread per voxel.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float win_m(int id, float par, float u) {
  u = fabsf(u);
  switch (id) {
    case 0: return (u < 1.0f) ? 1.0f : 0.0f;
    case 1: return 0.5f + 0.5f * cospif(u);
    case 2: {
      const float fr = 1.0f - par;
      if (!(u < 1.0f)) return 0.0f;
      return (u > fr) ? 0.5f * (1.0f + cospif((u - fr) / par)) : 1.0f;
    }
    case 4: return 1.0f - u;
    default: return 0.0f;
  }
}

struct MBin {
  bool valid;
  float inv_w;      // boxcar: 1 / (z / 2F)
  float inv_l, inv_r;
};

__device__ __forceinline__ MBin m_bin(const PWDev& d, int kk, double x, double z) {
  MBin b;
  const int k = d.k_lb + kk;
  const double f = d.m_fs * k / d.N_dft;
  const double F = fmin(d.m_F0[kk], sqrt(f * z / (2.88 * d.m_c)));
  const double w = z / (2.0 * F);
  const double ilb = fmax(ceil(d.m_M + (x - w) / d.m_pitch) + 1.0, 1.0);
  const double iub = fmin(floor(d.m_M + (x + w) / d.m_pitch) + 1.0, (double)d.ne);
  b.valid = ilb <= iub;
  b.inv_w = (float)(1.0 / w);
  if (b.valid) {
    const double lb = d.m_pitch * ((ilb - 1.0) - d.m_M) - d.m_width / 2.0;
    const double ub = d.m_pitch * ((iub - 1.0) - d.m_M) + d.m_width / 2.0;
    b.inv_l = (float)(1.0 / (x - lb));
    b.inv_r = (float)(1.0 / (ub - x));
  } else {
    b.inv_l = b.inv_r = 0.0f;
  }
  return b;
}

// window sample of element e (dl = c_e - x) in bin b
__device__ __forceinline__ float m_sample(const PWDev& d, const MBin& b, float dl) {
  if (d.window_id == 0) return win_m(0, 0.0f, dl * b.inv_w);
  return win_m(d.window_id, d.window_par, dl * ((dl < 0.0f) ? b.inv_l : b.inv_r));
}

__global__ void __launch_bounds__(NTHREADS) pw_m_kernel(const PWDev d, int compound, float2* __restrict__ image,
                                                        float* __restrict__ weights) {
  const int i = blockIdx.x * TILE_X + (threadIdx.x >> 5);
  const int j = blockIdx.y * TILE_Z + (threadIdx.x & 31);
  if (i >= d.nx || j >= d.nz) return;
  const double x = d.m_px[i], z = d.m_pz[j];
  dfl ue[M_MAXE];
  float dlf[M_MAXE];
  int cnt[M_MAXE];
  const bool last_col = (i == d.nx - 1) && d.m_sig;
  bool any_valid = false;
  float2 tot = make_float2(0.0f, 0.0f), tcomp = make_float2(0.0f, 0.0f);
  for (int e = 0; e < d.ne; ++e) dlf[e] = (float)(d.m_pitch * (e - d.m_M) - x);
  for (int a = 0; a < d.na; ++a) {
    const double ex = d.m_tx[3 * a], ez = d.m_tx[3 * a + 1], xref = d.m_tx[3 * a + 2];
    const double dtx = ex * (x - xref) + ez * z;
    for (int e = 0; e < d.ne; ++e) {
      const double dl = d.m_pitch * (e - d.m_M) - x;
      const double tof = dtx / d.m_c + d.m_t0 / d.m_fs + sqrt(dl * dl + z * z) / d.m_c;
      const double u = tof * d.m_fs / d.N_dft;  // cycles per bin
      const float hi = (float)u;
      ue[e] = make_float2(hi, (float)(u - (double)hi));
    }
    if (d.m_norm == 2) {  // windowed: bins at which each element's normalised sample is positive
      for (int e = 0; e < d.ne; ++e) cnt[e] = 0;
      for (int kk = 0; kk < d.K; ++kk) {
        const MBin b = m_bin(d, kk, x, z);
        if (!b.valid) continue;
        float W = 0.0f;
        for (int e = 0; e < d.ne; ++e) W += m_sample(d, b, dlf[e]);
        for (int e = 0; e < d.ne; ++e) cnt[e] += (m_sample(d, b, dlf[e]) / W > 0.0f) ? 1 : 0;
      }
    }
    float2 acc = make_float2(0.0f, 0.0f), comp = make_float2(0.0f, 0.0f);
    int idx = 0;
    for (int kk = 0; kk < d.K; ++kk) {
      const MBin b = m_bin(d, kk, x, z);
      if (!b.valid) {
        if (last_col) d.m_sig[(size_t)j * d.K + kk] = make_float2(0.0f, 0.0f);
        continue;
      }
      any_valid = true;
      const int k = d.k_lb + kk;
      float invW = 1.0f;
      if (d.m_norm != 0) {
        float W = 0.0f;
        for (int e = 0; e < d.ne; ++e) W += m_sample(d, b, dlf[e]);
        invW = 1.0f / W;
      }
      float2 S = make_float2(0.0f, 0.0f);
      for (int e = 0; e < d.ne; ++e) {
        float ws = m_sample(d, b, dlf[e]) * invW;
        if (d.m_norm == 2) {
          const float h = 0.5f * (float)cnt[e];
          ws *= win_m(d.m_nwin_id, d.m_nwin_par, ((float)idx - h) / h);
        }
        const float2 X = d.X[((size_t)e * d.K + kk) * d.x_na + d.x_a0 + a];
        const float2 ph = cis_ku(k, ue[e]);
        const float2 t = cmul(ph, X);
        S.x = fmaf(2.0f * ws, t.x, S.x);
        S.y = fmaf(2.0f * ws, t.y, S.y);
      }
      if (last_col) d.m_sig[(size_t)j * d.K + kk] = S;
      float y = S.x - comp.x, tt = acc.x + y;
      comp.x = (tt - acc.x) - y;
      acc.x = tt;
      y = S.y - comp.y;
      tt = acc.y + y;
      comp.y = (tt - acc.y) - y;
      acc.y = tt;
      ++idx;
    }
    if (compound) {
      float y = acc.x - tcomp.x, tt = tot.x + y;
      tcomp.x = (tt - tot.x) - y;
      tot.x = tt;
      y = acc.y - tcomp.y;
      tt = tot.y + y;
      tcomp.y = (tt - tot.y) - y;
      tot.y = tt;
    } else {
      image[((size_t)a * d.nx + i) * d.nz + j] = acc;
    }
  }
  if (compound) image[(size_t)i * d.nz + j] = tot;
  if (weights) weights[(size_t)i * d.nz + j] = 0.0f;
  if (last_col) d.m_sig_flag[j] = any_valid ? 1 : 0;
}

cudaError_t launch_pw_m(const PWDev& d, int compound, float2* image, float* weights, cudaStream_t s) {
  dim3 grid((d.nx + TILE_X - 1) / TILE_X, (d.nz + TILE_Z - 1) / TILE_Z);
  pw_m_kernel<<<grid, NTHREADS, 0, s>>>(d, compound, image, weights);
  return cudaGetLastError();
}

}  // namespace fnum
