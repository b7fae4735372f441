// The synthetic-aperture beamformer on the Blackwell tensor cores (tcgen05 + TMA).
//
// Replaces the reference's per-bin, per-transmit phase matrices and cublasCgemm
// calls (+cuda/gpu_bf_saft_rf.cu:1144-1201, +cuda/saft_kernel_phase_shifts.cu:8-199).
// For a voxel v and band bin k the image term is a bilinear form in the
// transmit and receive phasors:
//     I_k(v) = n_k(v) sum_t a_t Y_t,   Y_t = sum_r X'_k(t, r) b_r,
//     a_t = w_tx(v, t, k) e^{2 pi i k u_t(v)},   b_r = w_rx(v, r, k) e^{2 pi i k u_r(v)},
// with X'_k(t, r) = X_k(t, r) e^{2 pi i k t0 / N} (the time offset folded into the
// spectra), n_k = 1 / (W_tx W_rx) of the normalisations that are on, and
// u_e(v) = |v - c_e| f_s / (N c) the one-way delay in cycles per bin.
//
// Y is a GEMM per bin: for a tile of 128 voxels (4 columns x 32 rows),
//     D[v][2t + p] = sum_{r, q} A[v][2r + q] B[2t + p][2r + q]
// with A = (Re b_r, Im b_r) and B the real form of X'_k,
//     B[2t][2r] = Re X', B[2t][2r+1] = -Im X', B[2t+1][2r] = Im X', B[2t+1][2r+1] = Re X',
// so that D[v][2t] + i D[v][2t+1] = Y_t.  Both operands are split into fp16 hi +
// lo parts (the spectra scaled by a power of two into fp16 range) and the products
// hi.lo + lo.hi + hi.hi are accumulated in FP32 in tensor memory; the CUDA cores
// only form the phasors and the dot products with a (O(elements) work per voxel
// and bin, where the recurrence kernels do O(elements^2)).
//
// Kernel (persistent, one CTA per SM, tiles from a deepest-first counter), 16 warps.
// Warp w serves the TMEM lane quadrant w mod 4 (one tile column, 32 voxels, a voxel
// per lane) and the element slot w / 4 (elements 8s .. 8s+7 of every 32-element
// chunk, one mma k-step).  Per tile the elements span the union of its voxels'
// apertures; per bin only the chunks and k-steps that bin's apertures touch run
// (the per-bin ranges come from a warp reduction along each column's segment lists),
// with N = 16 ceil(transmit elements / 8).  Per bin and chunk the warps advance their
// phasors p = e^{2 pi i k u} by p <- p conj(rho) in packed FP32x2 (rho = e^{2 pi i u}
// kept in tensor memory, columns 256-511; exact re-anchoring every 32 bins and when a
// chunk comes back into range) and write their A rows (fp16 hi/lo, 128-byte swizzle)
// into a two-stage shared-memory ring.  The first warp through a stage issues the
// item's B tiles (TMA, a 3-D map over [bin][row][column]); the last one in issues its
// tcgen05.mma (M = 128, K = 16 per k-step: hi.lo and lo.hi first, then hi.hi) into
// the single D accumulator and commits the stage and, after the bin's last chunk, D.
// Once D is complete every thread reads its columns and adds n_k sum_t w_tx p_t Y_t
// to its voxel (compensated sum); the next bin's first products are only issued
// after every warp has passed that point, so D is free.  Waits sleep in the mbarrier
// and give up after two seconds: the CTA then records ERR_TC_TIMEOUT, gives its
// copies and products in flight time to land, frees its tensor memory and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "fnum_device.cuh"
#include "fnum_internal.h"
#include "fnum_tc_ptx.cuh"

namespace fnum {

namespace {

using namespace tcx;

constexpr int ST_M = 128;                            // voxels per tile = TMEM lanes = mma M
constexpr int ST_KC = 32;                            // elements per chunk (64 fp16 = one 128-byte row)
constexpr int ST_CMAX = 4;                           // chunks per bin: up to 128 elements
constexpr int ST_EPT = 8;                            // elements per thread and chunk
constexpr int ST_WARPS = 16;                         // 4 per TMEM lane quadrant
constexpr int ST_THREADS = ST_WARPS * 32;
constexpr int ST_STAGES = 2;
constexpr int ST_A_PLANE = ST_M * 128;               // 16 KB
constexpr int ST_B_PLANE = 2 * ST_KC * ST_CMAX * 128;   // up to 256 rows: 32 KB
constexpr int ST_STAGE = 2 * ST_A_PLANE + 2 * ST_B_PLANE;
constexpr int ST_SMEM = ST_STAGES * ST_STAGE + 1024;   // + alignment slack
constexpr int ST_BOX_ROWS = 2 * ST_KC;               // B rows per TMA box: 32 transmit elements
constexpr int ST_BOX_BYTES = ST_BOX_ROWS * 128;
constexpr int ST_TB = 32;                            // bins between exact re-anchorings
constexpr int ST_TMEM_COLS = 512;
constexpr int ST_RHO_COL = 256;

static_assert(ST_THREADS <= 1024, "block size");
static_assert(ST_WARPS == 4 * (ST_KC / ST_EPT), "four slots per lane quadrant");

// ---------------------------------------------------------------------------
// operands
// ---------------------------------------------------------------------------
// B planes [bin][n][kk] (n = 2t + p, kk = 2r + q, both < 2 nep) of X' scaled by the
// power of two sigma; zero for t or r >= ne.  One block per (t, 32 receive elements,
// 32 bins): the spectra are read along bins (coalesced) into shared memory and
// written along receive elements.
__global__ void __launch_bounds__(256) sa_tc_prep_kernel(const float2* __restrict__ X, int ne, int nep, int K,
                                                         const float2* __restrict__ rot,
                                                         const unsigned* __restrict__ maxbits,
                                                         __half2* __restrict__ bhi, __half2* __restrict__ blo) {
  __shared__ float2 tile[32][33];
  const int t = blockIdx.x, r0 = blockIdx.y * 32, k0 = blockIdx.z * 32;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int ri = w; ri < 32; ri += 8) {
    const int r = r0 + ri, k = k0 + lane;
    float2 x = make_float2(0.0f, 0.0f);
    if (t < ne && r < ne && k < K) x = X[((size_t)t * ne + r) * K + k];
    tile[ri][lane] = x;
  }
  __syncthreads();
  const float sigma = tc_scale(*maxbits);
  const size_t row = (size_t)nep;   // half2 per row: 2 nep fp16
  for (int ki = w; ki < 32; ki += 8) {
    const int k = k0 + ki, r = r0 + lane;
    if (k >= K || r >= nep) continue;
    float2 x = tile[lane][ki];
    const float2 c = rot[k];
    x = make_float2((x.x * c.x - x.y * c.y) * sigma, (x.x * c.y + x.y * c.x) * sigma);
    // row 2t: (Re, -Im); row 2t + 1: (Im, Re)
    const __half2 h0 = __floats2half2_rn(x.x, -x.y);
    const __half2 h1 = __floats2half2_rn(x.y, x.x);
    const float2 f0 = __half22float2(h0), f1 = __half22float2(h1);
    const __half2 l0 = __floats2half2_rn(x.x - f0.x, -x.y - f0.y);
    const __half2 l1 = __floats2half2_rn(x.y - f1.x, x.x - f1.y);
    const size_t i0 = ((size_t)k * 2 * nep + 2 * t) * row + r;
    bhi[i0] = h0;
    blo[i0] = l0;
    bhi[i0 + row] = h1;
    blo[i0 + row] = l1;
  }
}

// ---------------------------------------------------------------------------
// the beamformer
// ---------------------------------------------------------------------------
constexpr int ST_KMAX = 2048;       // bands up to this many bins get per-bin element ranges
constexpr int ST_NONE = 1 << 20;    // empty range marker

struct StShared {
  int ktop_tx[ST_M];
  int ktop_rx[ST_M];
  int nseg[ST_M];
  float2 red[ST_WARPS / 4][ST_M];   // per element slot: the voxel's sum over the slot's elements
  int ranges[4];
  int tile;
  int E_lo, E_hi, kt, nb;
  unsigned long long n_active, n_empty;
  uint32_t tmem;
  int abort_flag;
  int tma_cnt[2], mma_cnt[2];   // warps through each stage's item so far
  uint64_t bars[7];   // a_full[2], b_full[2], s_empty[2], d_full
  // per bin (relative to k_lb): the element range of the tile's apertures, tx and rx
  int lo[ST_KMAX];
  int hi[ST_KMAX];
};

// waits as long as no other thread has given up; records a timeout
__device__ __forceinline__ bool st_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                        unsigned long long* err) {
  if (mbar_test(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    // sleep in the barrier (up to 20 us per test) instead of spinning on issue slots
    if (mbar_test_sleep(bar, parity, 20000u)) return true;
    if (*abort_flag) return false;
    if (global_ns() - t0 > WAIT_NS) {
      *abort_flag = 1;
      atomicOr(err, ERR_TC_TIMEOUT);
      return false;
    }
  }
}

// window weight of element e of a voxel (0 outside its aperture).  The aperture's
// elements form the interval [a, b] = [min(i_lb, emid), max(i_ub, emid - 1)]: left of
// emid from i_lb, right of it up to i_ub.
template <int WIN>
__device__ __forceinline__ float st_weight(const SADev& d, int e, int emid, int a, int b, float iLl, float iLr,
                                           int ic, float par, float ipar) {
  const bool in = e >= a && e <= b;
  if (WIN == 0) return in ? 1.0f : 0.0f;
  if (!in) return 0.0f;
  const bool left = e < emid;
  const dfl c = d.el_m[e], xm = d.col_m[ic];
  const float dx = fabsf((c.x - xm.x) + (c.y - xm.y));
  return win_t<WIN>(par, ipar, dx * (left ? iLl : iLr));
}

__device__ __forceinline__ uint32_t h2u(__half2 h) { return *reinterpret_cast<uint32_t*>(&h); }

template <int WT, int WR>
__global__ void __launch_bounds__(ST_THREADS, 1)
sa_tc_kernel(const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo, const SADev d,
             const unsigned* __restrict__ maxbits, float2* __restrict__ image, float* __restrict__ wtx_out,
             float* __restrict__ wrx_out, int n_tiles_x, int n_tiles_z) {
  extern __shared__ unsigned char dyn[];
  __shared__ StShared sh;
  const uint32_t raw = smem_u32(dyn);
  const uint32_t base = (raw + 1023u) & ~1023u;   // the 128-byte swizzle wants 1024-byte tiles
  unsigned char* gbase = dyn + (base - raw);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n_tiles = n_tiles_x * n_tiles_z;
  volatile int* abort_flag = &sh.abort_flag;
  unsigned long long* err = &d.counters[2];
  const uint32_t bar0 = smem_u32(sh.bars);
  auto a_full = [&](int s) { return bar0 + 8u * (uint32_t)s; };
  auto b_full = [&](int s) { return bar0 + 8u * (uint32_t)(2 + s); };
  auto s_empty = [&](int s) { return bar0 + 8u * (uint32_t)(4 + s); };
  const uint32_t d_full = bar0 + 48u;
  const int per_bin = d.K <= ST_KMAX;
  const int n_bins_tab = per_bin ? d.K : 0;

  if (tid == 0) {
    for (int s = 0; s < ST_STAGES; ++s) {
      mbar_init(a_full(s), ST_WARPS);
      mbar_init(b_full(s), 1);
      mbar_init(s_empty(s), 1);
      sh.tma_cnt[s] = sh.mma_cnt[s] = 0;
    }
    mbar_init(d_full, 1);
    sh.abort_flag = 0;
    sh.n_active = sh.n_empty = 0ull;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async_smem();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh.tmem)),
                 "r"(ST_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = sh.tmem;

  const float sigma = tc_scale(*maxbits);
  const float ipt = (d.wtx_par > 0.0f) ? 1.0f / d.wtx_par : 0.0f;
  const float ipr = (d.wrx_par > 0.0f) ? 1.0f / d.wrx_par : 0.0f;
  // the warp's TMEM lane quadrant (tile column) and element slot
  const int q = warp & 3, slot = warp >> 2;
  const int vb = 32 * q + lane;
  const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
  const uint32_t row_off = (uint32_t)((vb >> 3) * 1024 + (vb & 7) * 128);
  const uint32_t ch0 = (uint32_t)(((2 * slot) ^ (vb & 7)) << 4), ch1 = (uint32_t)(((2 * slot + 1) ^ (vb & 7)) << 4);
  // running counts of (bin, chunk) items and of bins with products, the same in every warp
  uint32_t it = 0, bn = 0;
  unsigned long long n_exec = 0;

  for (;;) {
    if (tid == 0) sh.tile = (int)atomicAdd(&d.counters[3], 1ull);
    for (int e = tid; e < ST_M; e += ST_THREADS) sh.ktop_tx[e] = sh.ktop_rx[e] = -1;
    if (tid == 0) {
      sh.ranges[0] = sh.ranges[2] = d.ne;
      sh.ranges[1] = sh.ranges[3] = -1;
    }
    __syncthreads();
    const int tile = sh.tile;
    if (tile >= n_tiles || *abort_flag) break;
    int tx_, tz_;
    tile_coords(tile, n_tiles_x, n_tiles_z, tx_, tz_);
    const int i = tx_ * TILE_X + q, j = tz_ * TILE_Z + lane;
    const bool vvalid = (i < d.nx) && (j < d.nz);
    const int ic = min(i, d.nx - 1), jc = min(j, d.nz - 1);
    int4* seg = d.seg + ((size_t)blockIdx.x * ST_M + vb) * (size_t)d.seg_cap * SA_SEG_INT4;
    const int emid = d.col_emid[ic];
    for (int kk = tid; kk < n_bins_tab; kk += ST_THREADS) {
      sh.lo[kk] = ST_NONE;
      sh.hi[kk] = -1;
    }
    if (warp < 4) {
      float Wt, Wr;
      unsigned long long na = 0, nm = 0;
      sh.nseg[vb] = sa_build_segments(d, ic, jc, vvalid, seg, sh.ktop_tx, sh.ktop_rx, sh.ranges, Wt, Wr, na, nm);
      atomicAdd(&sh.n_active, na);
      atomicAdd(&sh.n_empty, nm);
      if (vvalid) {
        if (wtx_out) wtx_out[(size_t)ic * d.nz + jc] = Wt;
        if (wrx_out) wrx_out[(size_t)ic * d.nz + jc] = Wr;
      }
    }
    __syncthreads();
    if (tid == 0) {
      const int lo = min(sh.ranges[0], sh.ranges[2]), hi = max(sh.ranges[1], sh.ranges[3]);
      int kt = -1;
      if (lo <= hi)
        for (int e = lo; e <= min(hi, d.ne - 1); ++e) kt = max(kt, max(sh.ktop_tx[e], sh.ktop_rx[e]));
      sh.E_lo = lo;
      sh.E_hi = hi;
      sh.kt = kt;
      sh.nb = (lo <= hi && kt >= d.k_lb) ? kt - d.k_lb + 1 : 0;
    }
    __syncthreads();
    const int E_lo = sh.E_lo, E_hi = sh.E_hi, kt = sh.kt, nb = sh.nb;
    const int E0 = E_lo & ~7;   // the threads' elements: E0 + 32 c + 8 slot + i
    const int ns = sh.nseg[vb];
    // per bin, the element range of the tile's apertures: a reduction over each column's
    // voxels along their segment lists, then over the four columns
    if (per_bin && nb > 0 && warp < 4) {
      int sidx = (ns > 0) ? sa_seg_find(seg, ns, kt) : 0;
      int nxt = (ns > 0) ? seg[min(sidx + 1, ns)].x : -1;
      int a = ST_NONE, b = -1;
      auto rng = [&]() {
        a = ST_NONE;
        b = -1;
        if (ns == 0) return;
        const int4 cur = seg[sidx];
        if (cur.w == 0) return;   // an empty aperture: no term
        a = min(min(code_ilb(cur.y), code_ilb(cur.z)), emid);
        b = max(max(code_iub(cur.y), code_iub(cur.z)), emid - 1);
      };
      rng();
      for (int k = kt; k >= d.k_lb; --k) {
        if (k == nxt) {
          ++sidx;
          nxt = seg[min(sidx + 1, ns)].x;
          rng();
        }
        const int mn = __reduce_min_sync(0xffffffffu, a), mx = __reduce_max_sync(0xffffffffu, b);
        if (lane == 0 && mn <= mx) {
          atomicMin(&sh.lo[k - d.k_lb], mn);
          atomicMax(&sh.hi[k - d.k_lb], mx);
        }
      }
    }
    __syncthreads();
    float2 acc = make_float2(0.0f, 0.0f), comp = make_float2(0.0f, 0.0f);
    if (nb > 0) {
      auto u_of = [&](int e) {
        return df_sqrt(df_add(df_sqr(df_sub(d.el_u[min(e, d.ne - 1)], d.col_u[ic])), d.row_u2[jc]));
      };
      // rho = e^{2 pi i u} of the thread's elements into tensor memory, by element pairs
      // {Re rho_2j, Re rho_2j+1, Im rho_2j, Im rho_2j+1} (the packed recurrence's operands)
      for (int c = 0; c * ST_KC <= E_hi - E0; ++c) {
        float rv[16];
#pragma unroll
        for (int k2 = 0; k2 < ST_EPT; ++k2) {
          const float2 r = cis_ku(1, u_of(E0 + ST_KC * c + ST_EPT * slot + k2));
          rv[4 * (k2 >> 1) + (k2 & 1)] = r.x;
          rv[4 * (k2 >> 1) + 2 + (k2 & 1)] = r.y;
        }
        tmem_st16(tl + (uint32_t)(ST_RHO_COL + 2 * ST_KC * c + 2 * ST_EPT * slot), rv);
      }
      tmem_wait_st();
      // the segment in effect: its apertures, normaliser and (other windows) half-widths
      // (the next entry is loaded a boundary ahead, so its latency hides behind whole bins)
      int sidx = (ns > 0) ? sa_seg_find(seg, ns, kt) : 0;
      int4 nxt = (ns > 0) ? seg[min(sidx + 1, ns)] : make_int4(-1, 0, 0, 0);
      int ta = 0, tb = -1, ra = 0, rb = -1;
      float nrm = 0.0f, tLl = 0.0f, tLr = 0.0f, rLl = 0.0f, rLr = 0.0f;
      auto derive = [&](const int4 cur) {
        const int tlb = code_ilb(cur.y), tub = code_iub(cur.y), rlb = code_ilb(cur.z), rub = code_iub(cur.z);
        ta = min(tlb, emid);
        tb = max(tub, emid - 1);
        ra = min(rlb, emid);
        rb = max(rub, emid - 1);
        nrm = __int_as_float(cur.w);
        if (WT != 0 || WR != 0) {
          const dfl xm = d.col_m[ic];
          if (WT != 0) {
            tLl = (tlb < d.ne) ? inv_half_width(d.el_lb, d.el_ub, xm, true, tlb, tub) : 0.0f;
            tLr = (tub >= 0) ? inv_half_width(d.el_lb, d.el_ub, xm, false, tlb, tub) : 0.0f;
          }
          if (WR != 0) {
            rLl = (rlb < d.ne) ? inv_half_width(d.el_lb, d.el_ub, xm, true, rlb, rub) : 0.0f;
            rLr = (rub >= 0) ? inv_half_width(d.el_lb, d.el_ub, xm, false, rlb, rub) : 0.0f;
          }
        }
      };
      derive((ns > 0) ? seg[sidx] : make_int4(-1, seg_code(d.ne, -1), seg_code(d.ne, -1), 0));
      // phasors by element pairs: pr[c][j] = {Re p_2j, Re p_2j+1}, pm[c][j] = {Im p_2j, Im p_2j+1}
      float2 pr[ST_CMAX][ST_EPT / 2], pm[ST_CMAX][ST_EPT / 2];
#pragma unroll
      for (int c = 0; c < ST_CMAX; ++c)
#pragma unroll
        for (int j2 = 0; j2 < ST_EPT / 2; ++j2) pr[c][j2] = pm[c][j2] = make_float2(0.0f, 0.0f);
      // per chunk: p holds the phasors of the previous bin (else the next use re-anchors)
      unsigned live = 0u;
      bool ok = true;
      for (int b = 0; b < nb && ok; ++b) {
        const int k = kt - b;
        if (k == nxt.x) {
          const int4 cur = nxt;
          ++sidx;
          nxt = seg[min(sidx + 1, ns)];
          derive(cur);
        }
        int lo = E_lo, hi = E_hi;
        if (per_bin) {
          lo = sh.lo[k - d.k_lb];
          hi = sh.hi[k - d.k_lb];
        }
        if (lo > hi) {   // no aperture in the tile at this bin
          live = 0u;
          continue;
        }
        // this bin's chunks c_lo..c_hi; transmit rows from E0b (D column 2 (e - E0b))
        const int E0b = lo & ~7;
        const int c_lo = (lo - E0) >> 5, c_hi = (hi - E0) >> 5;
        const int nN = 16 * ((hi - E0b + 8) >> 3);
        const uint32_t idesc = idesc_f16(ST_M, nN);
        const int nbox = (nN + ST_BOX_ROWS - 1) / ST_BOX_ROWS;
        const uint32_t box_bytes = (uint32_t)(2 * nbox * ST_BOX_BYTES);
        const bool anchor = (b % ST_TB) == 0;
        unsigned nlive = 0u;
        int n_items = 0;
#pragma unroll
        for (int c = 0; c < ST_CMAX; ++c) {
          if (c >= c_lo && c <= c_hi) {
            const int g0 = E0 + ST_KC * c;
            const int s_lo = max(0, (lo - g0) >> 3), s_hi = min(ST_KC / ST_EPT - 1, (hi - g0) >> 3);
            const bool mine = slot >= s_lo && slot <= s_hi;
            const int eb = g0 + ST_EPT * slot;
            const bool exact = anchor || !(live & (1u << c));
            const int st = (int)(it & 1u);
            const uint32_t ph = (it >> 1) & 1u;
            unsigned char* ahi = gbase + st * ST_STAGE;
            unsigned char* alo = ahi + ST_A_PLANE;
            // two halves of 4 elements: phasors, A values, then (once the stage is free) the stores
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              uint32_t hq[4], lq[4];
              if (mine) {
                if (exact) {
#pragma unroll
                  for (int jj = 0; jj < 2; ++jj) {
                    const int j2 = 2 * h + jj;
                    const float2 z0 = cis_ku(k, u_of(eb + 2 * j2)), z1 = cis_ku(k, u_of(eb + 2 * j2 + 1));
                    pr[c][j2] = make_float2(z0.x, z1.x);
                    pm[c][j2] = make_float2(z0.y, z1.y);
                  }
                } else {
                  // p <- p conj(rho), two elements per packed FP32 instruction
                  float rv[8];
                  tmem_ld8_nowait(tl + (uint32_t)(ST_RHO_COL + 2 * ST_KC * c + 2 * ST_EPT * slot + 8 * h), rv);
                  tmem_wait_ld();
#pragma unroll
                  for (int jj = 0; jj < 2; ++jj) {
                    const int j2 = 2 * h + jj;
                    const float2 rr = make_float2(rv[4 * jj], rv[4 * jj + 1]);
                    const float2 ri = make_float2(rv[4 * jj + 2], rv[4 * jj + 3]);
                    const float2 a = pr[c][j2], m = pm[c][j2];
                    const float2 t = __fmul2_rn(a, ri);
                    pr[c][j2] = __ffma2_rn(m, ri, __fmul2_rn(a, rr));
                    pm[c][j2] = __ffma2_rn(m, rr, make_float2(-t.x, -t.y));
                  }
                }
#pragma unroll
                for (int kq = 0; kq < 4; ++kq) {
                  const int k2 = 4 * h + kq;
                  const float w = st_weight<WR>(d, eb + k2, emid, ra, rb, rLl, rLr, ic, d.wrx_par, ipr);
                  const float px = (k2 & 1) ? pr[c][k2 >> 1].y : pr[c][k2 >> 1].x;
                  const float py = (k2 & 1) ? pm[c][k2 >> 1].y : pm[c][k2 >> 1].x;
                  const float br = w * px, bi = w * py;
                  const __half2 hh = __floats2half2_rn(br, bi);
                  const float2 f = __half22float2(hh);
                  hq[kq] = h2u(hh);
                  lq[kq] = h2u(__floats2half2_rn(br - f.x, bi - f.y));
                }
              }
              if (h == 0) {
                // the stage is free once the products of the item two back have read it
                ok = __all_sync(0xffffffffu, st_wait(s_empty(st), ph ^ 1u, abort_flag, err));
                if (!ok) break;
                if (lane == 0) {
                  // the first warp through issues the item's B tiles, the last one resets the count
                  const int o = atomicAdd(&sh.tma_cnt[st], 1);
                  if (o == 0) {
                    const uint32_t bh = base + (uint32_t)(st * ST_STAGE + 2 * ST_A_PLANE);
                    const uint32_t bl = bh + ST_B_PLANE;
                    mbar_expect_tx(b_full(st), box_bytes);
                    const int x = 2 * g0, z = k - d.k_lb;
                    for (int jj = 0; jj < nbox; ++jj) {
                      const int y = 2 * E0b + ST_BOX_ROWS * jj;
                      tma_load_3d(bh + (uint32_t)(jj * ST_BOX_BYTES), &tm_hi, x, y, z, b_full(st));
                      tma_load_3d(bl + (uint32_t)(jj * ST_BOX_BYTES), &tm_lo, x, y, z, b_full(st));
                    }
                  } else if (o == ST_WARPS - 1) {
                    sh.tma_cnt[st] = 0;
                  }
                }
              }
              if (mine) {
                const uint32_t chh = h ? ch1 : ch0;
                *reinterpret_cast<uint4*>(ahi + row_off + chh) = make_uint4(hq[0], hq[1], hq[2], hq[3]);
                *reinterpret_cast<uint4*>(alo + row_off + chh) = make_uint4(lq[0], lq[1], lq[2], lq[3]);
              }
            }
            if (!ok) break;
            if (mine) {
              nlive |= 1u << c;
              fence_proxy_async_smem();
            }
            fence_before_sync();
            __syncwarp();
            if (lane == 0) {
              mbar_arrive(a_full(st));
              // the last warp in issues the item's products for the chunk's live k-steps (all A
              // rows are written, and for the bin's first chunk every warp has read the previous
              // bin's D)
              const int o = atomicAdd(&sh.mma_cnt[st], 1);
              if (o == ST_WARPS - 1) {
                sh.mma_cnt[st] = 0;
                if (st_wait(a_full(st), ph, abort_flag, err) && st_wait(b_full(st), ph, abort_flag, err)) {
                  fence_after_sync();
                  const uint32_t ah = base + (uint32_t)(st * ST_STAGE);
                  const uint32_t al = ah + ST_A_PLANE, bh = ah + 2 * ST_A_PLANE, bl = bh + ST_B_PLANE;
                  // the small cross products first, so that only the hi.hi steps round a full-size sum
                  for (int kk = s_lo; kk <= s_hi; ++kk) {
                    const uint32_t off = (uint32_t)kk * 32u;
                    mma_f16(tmem, smem_desc(ah + off), smem_desc(bl + off), idesc,
                            (c != c_lo || kk != s_lo) ? 1u : 0u);
                    mma_f16(tmem, smem_desc(al + off), smem_desc(bh + off), idesc, 1u);
                  }
                  for (int kk = s_lo; kk <= s_hi; ++kk) {
                    const uint32_t off = (uint32_t)kk * 32u;
                    mma_f16(tmem, smem_desc(ah + off), smem_desc(bh + off), idesc, 1u);
                  }
                  mma_commit(s_empty(st));
                  if (c == c_hi) mma_commit(d_full);
                }
                n_exec += (unsigned long long)ST_M * (ST_EPT * (s_hi - s_lo + 1)) * (nN / 2);
              }
            }
            __syncwarp();
            ++it;
            ++n_items;
          }
        }
        live = nlive;
        if (!ok) break;
        // the bin's Y: dot with the transmit phasors.  d_full is committed by the thread that
        // issued the bin's last products; the item before it (another issuer, other stage)
        // is complete when its stage is released (items on one stage complete in turn)
        ok = __all_sync(0xffffffffu, st_wait(d_full, bn & 1u, abort_flag, err) &&
                                         (n_items < 2 || st_wait(s_empty((int)(it & 1u)), ((it - 2) >> 1) & 1u,
                                                                 abort_flag, err)));
        if (!ok) break;
        fence_after_sync();
        float2 part = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int c = 0; c < ST_CMAX; ++c) {
          if (nlive & (1u << c)) {
            const int col = 2 * ST_KC * c + 2 * ST_EPT * slot - 2 * (E0b - E0);
            const int eb = E0 + ST_KC * c + ST_EPT * slot;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              float yv[8];
              tmem_ld8_nowait(tl + (uint32_t)(col + 8 * h), yv);
              tmem_wait_ld();
#pragma unroll
              for (int kq = 0; kq < 4; ++kq) {
                const int k2 = 4 * h + kq;
                const float w = st_weight<WT>(d, eb + k2, emid, ta, tb, tLl, tLr, ic, d.wtx_par, ipt);
                const float px = (k2 & 1) ? pr[c][k2 >> 1].y : pr[c][k2 >> 1].x;
                const float py = (k2 & 1) ? pm[c][k2 >> 1].y : pm[c][k2 >> 1].x;
                const float ar = w * px, ai = w * py;
                const float yr = yv[2 * kq], yi = yv[2 * kq + 1];
                part.x = fmaf(ar, yr, fmaf(-ai, yi, part.x));
                part.y = fmaf(ar, yi, fmaf(ai, yr, part.y));
              }
            }
          }
        }
        ++bn;
        // n_k Y into the voxel, compensated
        const float yx = nrm * part.x - comp.x, sx = acc.x + yx;
        comp.x = (sx - acc.x) - yx;
        acc.x = sx;
        const float yy = nrm * part.y - comp.y, sy = acc.y + yy;
        comp.y = (sy - acc.y) - yy;
        acc.y = sy;
      }
    }
    sh.red[slot][vb] = acc;
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (*abort_flag) break;
    if (warp < 4 && vvalid) {
      float sx = 0.0f, sy = 0.0f;
#pragma unroll
      for (int s = 0; s < ST_WARPS / 4; ++s) {
        sx += sh.red[s][vb].x;
        sy += sh.red[s][vb].y;
      }
      const float f = d.scale / sigma;
      image[(size_t)ic * d.nz + jc] = make_float2(sx * f, sy * f);
    }
  }
  atomicAdd(&d.counters[4], n_exec);
  if (tid == 0) {
    atomicAdd(&d.counters[0], sh.n_active);
    atomicAdd(&d.counters[1], sh.n_empty);
    // after a timeout, give the copies and products in flight time to land before the
    // tensor memory is freed (they take microseconds)
    if (*abort_flag) {
      const unsigned long long t0 = global_ns();
      while (global_ns() - t0 < 20000000ull) {
      }
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ST_TMEM_COLS) : "memory");
  }
}

typedef void (*st_kernel_t)(const CUtensorMap, const CUtensorMap, const SADev, const unsigned*, float2*, float*,
                            float*, int, int);

template <int WT>
st_kernel_t st_pick_rx(int wr) {
  switch (wr) {
    case 0: return sa_tc_kernel<WT, 0>;
    case 1: return sa_tc_kernel<WT, 1>;
    case 2: return sa_tc_kernel<WT, 2>;
    default: return sa_tc_kernel<WT, 4>;
  }
}
st_kernel_t st_pick(int wt, int wr) {
  switch (wt) {
    case 0: return st_pick_rx<0>(wr);
    case 1: return st_pick_rx<1>(wr);
    case 2: return st_pick_rx<2>(wr);
    default: return st_pick_rx<4>(wr);
  }
}

// 3-D fp16 map over [bins][2 nep rows][2 nep columns], 64 x 64 boxes, 128-byte swizzle;
// coordinates beyond the planes read as zero
bool st_encode(CUtensorMap* m, const void* base, int nep, int K) {
  EncodeTiled fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t n = (cuuint64_t)(2 * nep);
  const cuuint64_t dims[3] = {n, n, (cuuint64_t)K};
  const cuuint64_t strides[2] = {n * 2, n * n * 2};
  const cuuint32_t box[3] = {64, (cuuint32_t)ST_BOX_ROWS, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool sa_tc_supported(const SADev& d) { return d.ne >= 1 && d.ne <= ST_KC * ST_CMAX && d.last_bin_only == 0; }

size_t sa_tc_bytes(int ne, int K) {
  const size_t nep = (size_t)((ne + 3) / 4 * 4);
  return 2 * (size_t)K * (2 * nep) * (2 * nep) * sizeof(__half);
}

cudaError_t sa_tc_setup(SaTc& t, const SADev& d, void* planes, unsigned* maxbits, const float2* rot) {
  t.nep = (d.ne + 3) / 4 * 4;
  t.planes = planes;
  t.maxbits = maxbits;
  t.rot = rot;
  const size_t plane = (size_t)d.K * (2 * t.nep) * (2 * t.nep);
  const __half* b = (const __half*)planes;
  if (!st_encode(&t.tm[0], b, t.nep, d.K) || !st_encode(&t.tm[1], b + plane, t.nep, d.K))
    return cudaErrorInvalidValue;
  for (int wt : {0, 1, 2, 4})
    for (int wr : {0, 1, 2, 4}) {
      cudaError_t e = cudaFuncSetAttribute(st_pick(wt, wr), cudaFuncAttributeMaxDynamicSharedMemorySize, ST_SMEM);
      if (e != cudaSuccess) return e;
    }
  return cudaSuccess;
}

int sa_tc_grid(const SADev& d) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = ((d.nx + TILE_X - 1) / TILE_X) * ((d.nz + TILE_Z - 1) / TILE_Z);
  return std::max(1, std::min(tiles, nsm));
}

cudaError_t launch_sa_tc(const SADev& d, const SaTc& t, int grid, float2* image, float* wtx, float* wrx,
                         cudaStream_t s) {
  const int ntx = (d.nx + TILE_X - 1) / TILE_X, ntz = (d.nz + TILE_Z - 1) / TILE_Z;
  cudaError_t e = cudaMemsetAsync(d.counters + 3, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if ((e = launch_absmax((const float*)d.X, (size_t)d.ne * d.ne * d.K * 2, t.maxbits, s)) != cudaSuccess) return e;
  const size_t plane = (size_t)d.K * (2 * t.nep) * (2 * t.nep) / 2;   // half2 per plane
  __half2* bhi = (__half2*)t.planes;
  const dim3 pg(t.nep, (t.nep + 31) / 32, (d.K + 31) / 32);
  sa_tc_prep_kernel<<<pg, 256, 0, s>>>(d.X, d.ne, t.nep, d.K, t.rot, t.maxbits, bhi, bhi + plane);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  st_pick(d.wtx_id, d.wrx_id)<<<grid, ST_THREADS, ST_SMEM, s>>>(t.tm[0], t.tm[1], d, t.maxbits, image, wtx, wrx,
                                                                 ntx, ntz);
  return cudaGetLastError();
}

}  // namespace fnum
