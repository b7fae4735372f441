// Device helpers shared by the beamforming kernels (fnum_kernels.cu) and the
// tensor-core synthetic-aperture kernel (fnum_sa_tc.cu): double-float
// arithmetic, exact phasors, windows and their closed-form sums, apertures,
// tile order and the synthetic-aperture segment lists.
#pragma once
#include <cuda_fp16.h>
#include <float.h>
#include <math.h>
#include <stdint.h>

#include "fnum_internal.h"

namespace fnum {

// ---------------------------------------------------------------------------
// double-float arithmetic (Dekker / Knuth error-free transformations)
// ---------------------------------------------------------------------------
__device__ __forceinline__ dfl two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return make_float2(s, e);
}
__device__ __forceinline__ dfl fast_two_sum(float a, float b) {
  float s = a + b;
  float e = b - (s - a);
  return make_float2(s, e);
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b) {
  dfl s = two_sum(a.x, b.x);
  float t = s.y + (a.y + b.y);
  return fast_two_sum(s.x, t);
}
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ dfl two_prod(float a, float b) {
  float p = a * b;
  float e = fmaf(a, b, -p);
  return make_float2(p, e);
}
__device__ __forceinline__ dfl df_mul(dfl a, dfl b) {
  dfl p = two_prod(a.x, b.x);
  float t = fmaf(a.x, b.y, fmaf(a.y, b.x, p.y));
  return fast_two_sum(p.x, t);
}
__device__ __forceinline__ dfl df_sqr(dfl a) {
  dfl p = two_prod(a.x, a.x);
  float t = fmaf(2.0f * a.x, a.y, p.y);
  return fast_two_sum(p.x, t);
}
__device__ __forceinline__ dfl df_sqrt(dfl a) {
  if (!(a.x > 0.0f)) return make_float2(0.0f, 0.0f);
  float r = __fsqrt_rn(a.x);
  dfl r2 = two_prod(r, r);
  float d = ((a.x - r2.x) - r2.y) + a.y;  // a - r^2, a.x - r2.x exact (Sterbenz)
  float c = d * (0.5f / r);
  return fast_two_sum(r, c);
}
__device__ __forceinline__ float df_to_f(dfl a) { return a.x + a.y; }

// e^{j 2 pi k u}: k u reduced exactly to [-1/2, 1/2] cycles, sincospif on the
// leading part, first-order correction with the trailing part.
__device__ __forceinline__ float2 cis_ku(int k, dfl u) {
  const float kf = (float)k;
  dfl p = two_prod(kf, u.x);
  const float n = rintf(p.x);
  const float rh = p.x - n;                  // exact
  const float rl = fmaf(kf, u.y, p.y);
  dfl r = two_sum(rh, rl);
  float s, c;
  sincospif(2.0f * r.x, &s, &c);
  const float dphi = 6.28318530717958647692f * r.y;
  return make_float2(fmaf(-dphi, s, c), fmaf(dphi, c, s));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// ---------------------------------------------------------------------------
// windows (+cuda/gpu_bf_windows.cu:15-103; ids as gpu_bf_helper_functions.cu:56-97)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float win_apply(int id, float par, float l_abs, float L) {
  if (!(l_abs < L)) return 0.0f;
  const float u = l_abs / L;
  switch (id) {
    case 0: return 1.0f;
    case 1: return 0.5f * (1.0f + cospif(u));
    case 2: {
      const float thr = 1.0f - par;
      return (u <= thr) ? 1.0f : 0.5f * (1.0f + cospif((u - thr) / par));
    }
    case 4: return 1.0f - u;
    default: return 0.0f;
  }
}

// receive aperture bounds of one voxel at one bin (das_kernel_phase_shifts.cu:119-154):
//   left  i_lb = max(ceil(M + (x - z/(2F))/pitch), 0)      (ne = none)
//   right i_ub = min(floor(M + (x + z/(2F))/pitch), ne-1)  (-1 = none)
// with xp = M + x/pitch, zp = z/pitch, g = 1/(2F) in double-float.
__device__ __forceinline__ void aperture(dfl xp, dfl zp, dfl g, int ne, int& ilb, int& iub) {
  if (g.x < 0.0f) {  // F <= FLT_EPSILON: the whole array
    ilb = 0;
    iub = ne - 1;
    return;
  }
  const dfl w = df_mul(zp, g);
  const dfl tl = df_sub(xp, w);
  const dfl tr = df_add(xp, w);
  float cl = ceilf(tl.x);
  if (cl == tl.x && tl.y > 0.0f) cl += 1.0f;
  float fr = floorf(tr.x);
  if (fr == tr.x && tr.y < 0.0f) fr -= 1.0f;
  cl = fminf(fmaxf(cl, 0.0f), (float)ne);
  fr = fminf(fmaxf(fr, -1.0f), (float)(ne - 1));
  ilb = (int)cl;
  iub = (int)fr;
}

// half-widths of the left / right aperture
__device__ __forceinline__ float half_left(const dfl* el_lb, dfl xm, int ilb, int ne) {
  if (ilb >= ne) return 0.0f;
  const dfl l = el_lb[ilb];
  return (xm.x - l.x) + (xm.y - l.y);
}
__device__ __forceinline__ float half_right(const dfl* el_ub, dfl xm, int iub) {
  if (iub < 0) return 0.0f;
  const dfl u = el_ub[iub];
  return (u.x - xm.x) + (u.y - xm.y);
}

// apodization of element e (dx = c_e - x) for aperture (ilb, iub)
__device__ __forceinline__ float elem_apod(int id, float par, int e, int emid, int ilb, int iub, float dx,
                                           float Ll, float Lr) {
  if (e < emid) return (e >= ilb) ? win_apply(id, par, -dx, Ll) : 0.0f;
  return (e <= iub) ? win_apply(id, par, dx, Lr) : 0.0f;
}

// sum of the apodization over the aperture (the normaliser of one bin)
static __device__ float aperture_sum(int id, float par, const dfl* el_m, const dfl* el_lb, const dfl* el_ub, dfl xm,
                              int ne, int emid, int ilb, int iub) {
  float W = 0.0f;
  if (ilb < emid) {
    const float L = half_left(el_lb, xm, ilb, ne);
    for (int e = ilb; e < emid; ++e) {
      const dfl c = el_m[e];
      const float l = (xm.x - c.x) + (xm.y - c.y);
      W += win_apply(id, par, l, L);
    }
  }
  if (iub >= emid) {
    const float L = half_right(el_ub, xm, iub);
    for (int e = emid; e <= iub; ++e) {
      const dfl c = el_m[e];
      const float l = (c.x - xm.x) + (c.y - xm.y);
      W += win_apply(id, par, l, L);
    }
  }
  return W;
}

__device__ __forceinline__ int seg_code(int ilb, int iub) { return ilb | ((iub + 1) << 16); }
__device__ __forceinline__ int code_ilb(int c) { return c & 0xffff; }
__device__ __forceinline__ int code_iub(int c) { return (c >> 16) - 1; }

// Apodization of an element inside its aperture, u = |l| / L in [0, 1).
// Same windows as win_apply; the cosine is the hardware approximation
// (absolute error below 4e-7 on [0, pi]), which changes weights by < 1e-6.
__device__ __forceinline__ float win_fast(int id, float par, float inv_par, float u) {
  switch (id) {
    case 0: return 1.0f;
    case 1: return 0.5f + 0.5f * __cosf(3.14159265358979f * u);
    case 2: {
      const float thr = 1.0f - par;
      return (u <= thr) ? 1.0f : 0.5f + 0.5f * __cosf(3.14159265358979f * (u - thr) * inv_par);
    }
    case 4: return 1.0f - u;
    default: return 0.0f;
  }
}

// win_fast with the window id fixed at compile time (the recurrence kernels
// are instantiated per window, so the boundary handler carries no switch)
template <int WIN>
__device__ __forceinline__ float win_t(float par, float inv_par, float u) {
  if (WIN == 0) return 1.0f;
  if (WIN == 1) return 0.5f + 0.5f * __cosf(3.14159265358979f * u);
  if (WIN == 2) {
    const float thr = 1.0f - par;
    return (u <= thr) ? 1.0f : 0.5f + 0.5f * __cosf(3.14159265358979f * (u - thr) * inv_par);
  }
  if (WIN == 4) return 1.0f - u;
  return 0.0f;
}

// Sum of window values over n equally spaced elements at distances
// l_j = l0 + j p (j < n) from the voxel, all inside the half-width 1/invL:
//   boxcar      n
//   triangular  n - (n l0 + p n (n-1) / 2) invL
//   Hann        n/2 + 1/2 sum_j cos(theta0 + j delta)
//   Tukey       flat part (u <= 1 - par) counted, the taper summed like Hann
// with sum_{j<m} cos(t0 + j d) = sin(m d / 2) / sin(d / 2) cos(t0 + (m-1) d / 2).
__device__ __forceinline__ float cos_series(float t0, float dl, int m) {
  // angles in units of pi (sinpif / cospif need no large-argument reduction)
  if (m <= 0) return 0.0f;
  const float h = 0.5f * dl;
  const float sh = sinpif(h);
  const float c = cospif(t0 + (float)(m - 1) * h);
  return (fabsf(sh) > 1e-6f) ? sinpif((float)m * h) / sh * c : (float)m * c;
}
template <int WIN>
__device__ __forceinline__ float win_sum(float l0, float p, int n, float invL, float par, float inv_par) {
  if (n <= 0) return 0.0f;
  const float fn = (float)n;
  if (WIN == 0) return fn;
  if (WIN == 4) return fn - (fn * l0 + p * 0.5f * fn * (fn - 1.0f)) * invL;
  if (WIN == 1) return 0.5f * fn + 0.5f * cos_series(l0 * invL, p * invL, n);
  if (WIN == 2) {
    const float thr = 1.0f - par;
    // elements with u = l invL <= thr form the flat top
    int n1 = (int)floorf((thr / invL - l0) / p) + 1;
    n1 = min(max(n1, 0), n);
    const float t0 = ((l0 + (float)n1 * p) * invL - thr) * inv_par;
    return (float)n1 + 0.5f * (float)(n - n1) + 0.5f * cos_series(t0, p * invL * inv_par, n - n1);
  }
  return 0.0f;
}

// tiles are visited deepest rows first (they carry the widest apertures)
__device__ __forceinline__ void tile_coords(int tile, int n_tiles_x, int n_tiles_z, int& tx, int& tz) {
  tz = n_tiles_z - 1 - tile / n_tiles_x;
  tx = tile % n_tiles_x;
}

// 1 / half-width of the aperture side an element belongs to (edges from shared memory)
__device__ __forceinline__ float inv_half_width(const dfl* lb_s, const dfl* ub_s, dfl xm, bool left, int ilb, int iub) {
  float L;
  if (left) {
    const dfl l = lb_s[ilb];
    L = (xm.x - l.x) + (xm.y - l.y);
  } else {
    const dfl u = ub_s[iub];
    L = (u.x - xm.x) + (u.y - xm.y);
  }
  return __fdividef(1.0f, L);
}

// One segment entry per aperture change of a voxel (bins k_start down to the
// next entry's k_start + 1 share both apertures):
//   {k_start, tx code, rx code, 1/(W_tx W_rx)}
// with the sums of the normalisations that are on (1 for one that is off, 0
// for an empty aperture).  A sentinel entry (k_start = -1) ends every list.
// The weight of the pair (t, r) is a_tx(t) a_rx(r) / (W_tx W_rx).

// window sum of one aperture in closed form, window id known at run time
__device__ __forceinline__ float win_sum_rt(int id, float l0, float p, int n, float invL, float par, float inv_par) {
  switch (id) {
    case 0: return win_sum<0>(l0, p, n, invL, par, inv_par);
    case 1: return win_sum<1>(l0, p, n, invL, par, inv_par);
    case 2: return win_sum<2>(l0, p, n, invL, par, inv_par);
    case 4: return win_sum<4>(l0, p, n, invL, par, inv_par);
    default: return 0.0f;
  }
}
static __device__ float sa_aperture_sum(const SADev& d, int id, float par, dfl xm, int emid, int ilb, int iub) {
  const float inv_par = (par > 0.0f) ? 1.0f / par : 0.0f;
  float W = 0.0f;
  if (ilb < emid) {
    const float L = half_left(d.el_lb, xm, ilb, d.ne);
    if (L > 0.0f) {
      const dfl c = d.el_m[emid - 1];
      W += win_sum_rt(id, (xm.x - c.x) + (xm.y - c.y), d.pitch_f, emid - ilb, 1.0f / L, par, inv_par);
    }
  }
  if (iub >= emid) {
    const float L = half_right(d.el_ub, xm, iub);
    if (L > 0.0f) {
      const dfl c = d.el_m[emid];
      W += win_sum_rt(id, (c.x - xm.x) + (c.y - xm.y), d.pitch_f, iub - emid + 1, 1.0f / L, par, inv_par);
    }
  }
  return W;
}

static __device__ int sa_build_segments(const SADev& d, int ic, int jc, bool valid, int4* seg, int* ktop_tx, int* ktop_rx,
                                 int* ranges, float& Wtx_top, float& Wrx_top, unsigned long long& n_active,
                                 unsigned long long& n_empty) {
  const int4 sentinel = make_int4(-1, seg_code(d.ne, -1), seg_code(d.ne, -1), 0);
  Wtx_top = Wrx_top = 0.0f;
  if (!valid) {
    seg[0] = sentinel;
    return 0;
  }
  const dfl xp = d.col_p[ic], zp = d.row_p[jc], xm = d.col_m[ic];
  const int emid = d.col_emid[ic];
  int nseg = 0, prev_t = -1, prev_r = -1;
  int t_lo = d.ne, t_hi = -1, r_lo = d.ne, r_hi = -1;
  long long act = 0;
  for (int kk = d.K - 1; kk >= 0; --kk) {
    int tlb, tub, rlb, rub;
    aperture(xp, zp, d.gtx[kk], d.ne, tlb, tub);
    aperture(xp, zp, d.grx[kk], d.ne, rlb, rub);
    const int ct = seg_code(tlb, tub), cr = seg_code(rlb, rub);
    if (ct != prev_t || cr != prev_r) {
      const float Wt = sa_aperture_sum(d, d.wtx_id, d.wtx_par, xm, emid, tlb, tub);
      const float Wr = sa_aperture_sum(d, d.wrx_id, d.wrx_par, xm, emid, rlb, rub);
      const float it = (Wt > 0.0f) ? (d.norm_tx ? 1.0f / Wt : 1.0f) : 0.0f;
      const float ir = (Wr > 0.0f) ? (d.norm_rx ? 1.0f / Wr : 1.0f) : 0.0f;
      if (nseg < d.seg_cap - 1)
        seg[nseg] = make_int4(kk + d.k_lb, ct, cr, __float_as_int(it * ir));
      else
        atomicOr(&d.counters[2], ERR_SEG_OVERFLOW);
      if (nseg == 0) {
        Wtx_top = Wt;
        Wrx_top = Wr;
      }
      ++nseg;
      prev_t = ct;
      prev_r = cr;
      const int lo_t = min(tlb, emid), hi_t = max(tub, emid - 1);
      const int lo_r = min(rlb, emid), hi_r = max(rub, emid - 1);
      act = (Wt > 0.0f && Wr > 0.0f) ? (long long)max(hi_t - lo_t + 1, 0) * max(hi_r - lo_r + 1, 0) : 0;
      if (lo_t <= hi_t) {
        for (int e = lo_t; e <= hi_t && e < t_lo; ++e) atomicMax(&ktop_tx[e], kk + d.k_lb);
        for (int e = max(t_hi + 1, lo_t); e <= hi_t; ++e) atomicMax(&ktop_tx[e], kk + d.k_lb);
        t_lo = min(t_lo, lo_t);
        t_hi = max(t_hi, hi_t);
      }
      if (lo_r <= hi_r) {
        for (int e = lo_r; e <= hi_r && e < r_lo; ++e) atomicMax(&ktop_rx[e], kk + d.k_lb);
        for (int e = max(r_hi + 1, lo_r); e <= hi_r; ++e) atomicMax(&ktop_rx[e], kk + d.k_lb);
        r_lo = min(r_lo, lo_r);
        r_hi = max(r_hi, hi_r);
      }
    }
    if (act > 0) n_active += (unsigned long long)act; else n_empty += 1ull;
  }
  if (t_lo <= t_hi) {
    atomicMin(&ranges[0], t_lo);
    atomicMax(&ranges[1], t_hi);
  }
  if (r_lo <= r_hi) {
    atomicMin(&ranges[2], r_lo);
    atomicMax(&ranges[3], r_hi);
  }
  nseg = min(nseg, d.seg_cap - 1);
  seg[nseg] = sentinel;
  return nseg;
}

// last segment whose k_start >= kt (entries sorted by k_start, descending)
__device__ __forceinline__ int sa_seg_find(const int4* seg, int nseg, int kt) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (seg[mid].x >= kt) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// power-of-two scale that brings the spectra below 2^14 (exact in both directions)
__device__ __forceinline__ float tc_scale(unsigned maxbits) {
  const float m = __uint_as_float(maxbits);
  if (!(m > 0.0f) || !(m < 3.0e38f)) return 1.0f;
  int ex;
  frexpf(m, &ex);  // m < 2^ex
  return ldexpf(1.0f, min(max(14 - ex, -126), 126));
}

}  // namespace fnum
