/*
 * fnum_oracle.c -- FP64 C restatement of the f_number beamformer.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ as the checker at sizes the numpy
 * oracle cannot reach, and by bench.py as the timed CPU restatement of the
 * reference's CPU path (das_pw.m).  The product library never links it.
 *
 * Functions (file:line in the f_number project):
 *   oracle_pw_mex  cuda.gpu_bf_das_pw_rf per voxel: das_kernel_phase_shifts.cu:83-145,
 *                  cublasCgemm per bin (gpu_bf_das_pw_rf.cu:1034-1041),
 *                  das_kernel_normalization.cu:27-31, 2/N scaling (gpu_bf_das_pw_rf.cu:1118-1119)
 *   oracle_pw_m    das_pw.m:386-474 per voxel (CPU semantics)
 *   oracle_sa_mex  cuda.gpu_bf_saft_rf per voxel: saft_kernel_phase_shifts.cu:41-198,
 *                  gpu_bf_saft_rf.cu:1144-1201
 * Spectra X are inputs (band bins only, unnormalised e^{-j} DFT).
 * A bin whose apodization sum is zero contributes 0 and is counted (the MEX
 * produces NaN there).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FLT_EPS 1.1920928955078125e-07

/* +cuda/gpu_bf_windows.cu:15-103: 0 where |l| >= L */
static double win_mex(int id, double par, double l, double L) {
  if (!(fabs(l) < L)) return 0.0;
  const double u = fabs(l) / L;
  switch (id) {
    case 0: return 1.0;
    case 1: return (1.0 + cos(M_PI * u)) / 2.0;
    case 2: {
      const double thr = 1.0 - par;
      return (u <= thr) ? 1.0 : (1.0 + cos(M_PI * (u - thr) / par)) / 2.0;
    }
    case 4: return 1.0 - u;
    default: return 0.0;
  }
}

/* MATLAB compute_samples_scalar on |u|: +windows/boxcar.m:62, hann.m:62, tukey.m:101-105, triangular.m:62 */
static double win_m(int id, double par, double u) {
  u = fabs(u);
  switch (id) {
    case 0: return u < 1.0 ? 1.0 : 0.0;
    case 1: return (1.0 + cos(M_PI * u)) / 2.0;
    case 2: {
      const double fr = 1.0 - par;
      if (!(u < 1.0)) return 0.0;
      if (u > fr) return (1.0 + cos(M_PI * (u - fr) / par)) / 2.0;
      return 1.0;
    }
    case 4: return 1.0 - u;
    default: return 0.0;
  }
}

/* apodization of every element for one voxel and bin (das_kernel_phase_shifts.cu:111-154) */
static double apod_mex(int ne, double M, double pitch, const double* ctr, const double* lb, const double* ub,
                       int id, double par, double F, double x, double z, double* a) {
  double W = 0.0;
  int il = 0, ir = ne - 1;
  if (F > FLT_EPS) {
    const double w = z / (2.0 * F);
    double cl = ceil(M + (x - w) / pitch);
    double fr = floor(M + (x + w) / pitch);
    if (cl < 0) cl = 0;
    if (cl > ne) cl = ne;
    if (fr > ne - 1) fr = ne - 1;
    if (fr < -1) fr = -1;
    il = (int)cl;
    ir = (int)fr;
  }
  for (int e = 0; e < ne; ++e) {
    const double dx = ctr[e] - x;
    double v;
    if (dx < 0) v = (il < ne) ? win_mex(id, par, dx, x - lb[il]) : 0.0;
    else v = (ir >= 0) ? win_mex(id, par, dx, ub[ir] - x) : 0.0;
    a[e] = v;
    W += v;
  }
  return W;
}

/*
 * Plane wave, MEX semantics, compounded over na angles.
 * X: [na][ne][K] complex (re, im interleaved); F: [K].
 * voxels (ix[v], iz[v]); out: [nv] complex; wout: [nv] apodization sum of the last bin.
 */
int oracle_pw_mex(int ne, int K, int k_lb, int N, double pitch, double width, double fs, double c, double t0,
                  const double* px, const double* pz, int na, const double* angles, const double* X,
                  const double* F, int win_id, double win_par, int norm, int nv, const int* ix, const int* iz,
                  double* out, double* wout, long long* zero_bins, int nthreads) {
  const double M = (ne - 1.0) / 2.0;
  double* ctr = (double*)malloc(sizeof(double) * 3 * ne);
  double* lb = ctr + ne;
  double* ub = lb + ne;
  for (int e = 0; e < ne; ++e) {
    ctr[e] = pitch * (e - M);
    lb[e] = ctr[e] - width / 2.0;
    ub[e] = ctr[e] + width / 2.0;
  }
  const double coef = 2.0 * M_PI * fs / (N * c), add = 2.0 * M_PI * t0 / N;
  long long zb = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : zb)
#endif
  for (int v = 0; v < nv; ++v) {
    const double x = px[ix[v]], z = pz[iz[v]];
    double* a = (double*)malloc(sizeof(double) * ne * (1 + na));
    double* d = a + ne;
    for (int ai = 0; ai < na; ++ai) {
      const double ex = -sin(angles[ai]), ez = cos(angles[ai]);
      const double xref = (ex >= 0) ? -M * pitch : M * pitch;
      const double dtx = ex * (x - xref) + ez * z;
      for (int e = 0; e < ne; ++e) {
        const double dx = ctr[e] - x;
        d[ai * ne + e] = dtx + sqrt(dx * dx + z * z);
      }
    }
    double sr = 0.0, si = 0.0, Wl = 0.0;
    for (int kk = 0; kk < K; ++kk) {
      const int k = k_lb + kk;
      const double W = apod_mex(ne, M, pitch, ctr, lb, ub, win_id, win_par, F[kk], x, z, a);
      Wl = W;
      double br = 0.0, bi = 0.0;
      for (int ai = 0; ai < na; ++ai) {
        const double* Xa = X + 2 * ((size_t)ai * ne * K);
        for (int e = 0; e < ne; ++e) {
          if (a[e] == 0.0) continue;
          const double ph = k * (coef * d[ai * ne + e] + add);
          const double cs = cos(ph), sn = sin(ph);
          const double xr = Xa[2 * ((size_t)e * K + kk)], xi = Xa[2 * ((size_t)e * K + kk) + 1];
          br += a[e] * (cs * xr - sn * xi);
          bi += a[e] * (cs * xi + sn * xr);
        }
      }
      if (norm) {
        if (W == 0.0) {
          zb += na;
          continue;
        }
        br /= W;
        bi /= W;
      }
      sr += br;
      si += bi;
    }
    out[2 * v] = 2.0 * sr / N;
    out[2 * v + 1] = 2.0 * si / N;
    if (wout) wout[v] = Wl;
    free(a);
  }
  free(ctr);
  if (zero_bins) *zero_bins = zb;
  return 0;
}

/*
 * Plane wave, CPU semantics of das_pw.m (one angle per call, na angles summed).
 * ks: the K band bins (0-based), F0: F per bin before the depth cap.
 * norm: 0 off, 1 on, 2 windowed with (fwin_id, fwin_par).  No 2/N scaling.
 */
int oracle_pw_m(int ne, int K, const int* ks, int N, double pitch, double width, double fs, double c, double t0,
                const double* px, const double* pz, int na, const double* angles, const double* X, const double* F0,
                int win_id, double win_par, int norm, int fwin_id, double fwin_par, int nv, const int* ix,
                const int* iz, double* out, int nthreads) {
  const double M = (ne - 1.0) / 2.0;
  double* ctr = (double*)malloc(sizeof(double) * 3 * ne);
  double* lbs = ctr + ne;
  double* ubs = lbs + ne;
  for (int e = 0; e < ne; ++e) {
    ctr[e] = (-M + e) * pitch;
    lbs[e] = ctr[e] - width / 2.0;
    ubs[e] = ctr[e] + width / 2.0;
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int v = 0; v < nv; ++v) {
    const double x = px[ix[v]], z = pz[iz[v]];
    double* ws = (double*)malloc(sizeof(double) * (size_t)K * ne);
    int* kv = (int*)malloc(sizeof(int) * K);
    double* tof = (double*)malloc(sizeof(double) * ne);
    int nk = 0;
    /* valid bins and window samples (das_pw.m:399-457) */
    for (int kk = 0; kk < K; ++kk) {
      const double f = fs * ks[kk] / N;
      const double Fub = sqrt(f * z / (2.88 * c));
      const double F = F0[kk] < Fub ? F0[kk] : Fub;
      const double w = z / (2.0 * F);
      double il = ceil(M + (x - w) / pitch);
      double ir = floor(M + (x + w) / pitch);
      if (il < 0) il = 0;
      if (ir > ne - 1) ir = ne - 1;
      if (!(il <= ir)) continue;
      double* row = ws + (size_t)nk * ne;
      if (win_id == 0) {
        for (int e = 0; e < ne; ++e) row[e] = win_m(0, 0.0, (ctr[e] - x) / w);
      } else {
        const double wl = x - lbs[(int)il], wr = ubs[(int)ir] - x;
        for (int e = 0; e < ne; ++e) {
          const double dl = ctr[e] - x;
          row[e] = (dl < 0) ? win_m(win_id, win_par, dl / wl) : win_m(win_id, win_par, dl / wr);
        }
      }
      if (norm >= 1) {
        double s = 0.0;
        for (int e = 0; e < ne; ++e) s += row[e];
        for (int e = 0; e < ne; ++e) row[e] /= s;
      }
      kv[nk++] = kk;
    }
    if (norm == 2 && nk > 0) { /* +normalizations/windowed.m:81-86 */
      for (int e = 0; e < ne; ++e) {
        int cnt = 0;
        for (int r = 0; r < nk; ++r) cnt += ws[(size_t)r * ne + e] > 0;
        const double l2 = cnt / 2.0;
        for (int r = 0; r < nk; ++r) ws[(size_t)r * ne + e] *= win_m(fwin_id, fwin_par, (r - l2) / l2);
      }
    }
    double sr = 0.0, si = 0.0;
    for (int ai = 0; ai < na; ++ai) {
      const double ex = -sin(angles[ai]), ez = cos(angles[ai]);
      const double xref = (ex > 0 ? 1.0 : (ex < 0 ? -1.0 : 0.0)) * ctr[0];  /* sign(e_x) * x_1, das_pw.m:327 */
      const double tin = (ex * (x - xref) + ez * z) / c + t0 / fs;
      for (int e = 0; e < ne; ++e) {
        const double dl = ctr[e] - x;
        tof[e] = tin + sqrt((dl / c) * (dl / c) + (z / c) * (z / c));
      }
      const double* Xa = X + 2 * ((size_t)ai * ne * K);
      for (int r = 0; r < nk; ++r) {
        const int kk = kv[r];
        const double om = 2.0 * M_PI * fs * ks[kk] / N;
        const double* row = ws + (size_t)r * ne;
        for (int e = 0; e < ne; ++e) {
          const double ph = om * tof[e];
          const double cs = cos(ph), sn = sin(ph);
          const double xr = 2.0 * Xa[2 * ((size_t)e * K + kk)], xi = 2.0 * Xa[2 * ((size_t)e * K + kk) + 1];
          sr += row[e] * (cs * xr - sn * xi);
          si += row[e] * (cs * xi + sn * xr);
        }
      }
    }
    out[2 * v] = sr;
    out[2 * v + 1] = si;
    free(ws);
    free(kv);
    free(tof);
  }
  free(ctr);
  return 0;
}

/*
 * Synthetic aperture, MEX semantics.  X: [ne tx][ne rx][K] complex.
 * mode: 0 divide by the sums that are on (and accumulate); 1 keep only the
 * last bin unnormalised; -1 zero image.  norm_tx / norm_rx: sums on.
 */
int oracle_sa_mex(int ne, int K, int k_lb, int N, double pitch, double width, double fs, double c, double t0,
                  const double* px, const double* pz, const double* X, const double* Ftx, const double* Frx,
                  int wt_id, double wt_par, int wr_id, double wr_par, int norm_tx, int norm_rx, int mode, int nv,
                  const int* ix, const int* iz, double* out, double* wtx_out, double* wrx_out, long long* zero_bins,
                  int nthreads) {
  const double M = (ne - 1.0) / 2.0;
  double* ctr = (double*)malloc(sizeof(double) * 3 * ne);
  double* lb = ctr + ne;
  double* ub = lb + ne;
  for (int e = 0; e < ne; ++e) {
    ctr[e] = pitch * (e - M);
    lb[e] = ctr[e] - width / 2.0;
    ub[e] = ctr[e] + width / 2.0;
  }
  const double coef = 2.0 * M_PI * fs / (N * c), add = 2.0 * M_PI * t0 / N;
  long long zb = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : zb)
#endif
  for (int v = 0; v < nv; ++v) {
    const double x = px[ix[v]], z = pz[iz[v]];
    double* buf = (double*)malloc(sizeof(double) * ne * 7);
    double* at = buf;
    double* ar = at + ne;
    double* dist = ar + ne;
    double* pr = dist + ne;  /* phasor per element (re, im) = e^{j k coef d_e} */
    double* qr = pr + 2 * ne; /* e^{j k coef d_r} X, accumulated per tx */
    for (int e = 0; e < ne; ++e) {
      const double dx = ctr[e] - x;
      dist[e] = sqrt(dx * dx + z * z);
    }
    double sr = 0.0, si = 0.0, Wtl = 0.0, Wrl = 0.0;
    for (int kk = 0; kk < K; ++kk) {
      const int k = k_lb + kk;
      const double Wt = apod_mex(ne, M, pitch, ctr, lb, ub, wt_id, wt_par, Ftx[kk], x, z, at);
      const double Wr = apod_mex(ne, M, pitch, ctr, lb, ub, wr_id, wr_par, Frx[kk], x, z, ar);
      Wtl = Wt;
      Wrl = Wr;
      for (int e = 0; e < ne; ++e) {
        const double ph = k * coef * dist[e];
        pr[2 * e] = cos(ph);
        pr[2 * e + 1] = sin(ph);
      }
      const double ca = cos(k * add), sa = sin(k * add);
      double br = 0.0, bi = 0.0;
      for (int t = 0; t < ne; ++t) {
        if (at[t] == 0.0) continue;
        double tr = 0.0, ti = 0.0;
        for (int r = 0; r < ne; ++r) {
          if (ar[r] == 0.0) continue;
          const double* xp = X + 2 * (((size_t)t * ne + r) * K + kk);
          const double yr = pr[2 * r] * xp[0] - pr[2 * r + 1] * xp[1];
          const double yi = pr[2 * r] * xp[1] + pr[2 * r + 1] * xp[0];
          tr += ar[r] * yr;
          ti += ar[r] * yi;
        }
        const double ur = pr[2 * t] * tr - pr[2 * t + 1] * ti;
        const double ui = pr[2 * t] * ti + pr[2 * t + 1] * tr;
        br += at[t] * ur;
        bi += at[t] * ui;
      }
      { /* e^{j k add} */
        const double r_ = br * ca - bi * sa, i_ = br * sa + bi * ca;
        br = r_;
        bi = i_;
      }
      double den = 1.0;
      if (norm_rx) den *= Wr;
      if (norm_tx) den *= Wt;
      if (mode == 1) {
        if (kk == K - 1) {
          sr = br;
          si = bi;
        }
        continue;
      }
      if (den == 0.0) {
        zb += 1;
        continue;
      }
      sr += br / den;
      si += bi / den;
    }
    if (mode == -1) sr = si = 0.0;
    out[2 * v] = 2.0 * sr / N;
    out[2 * v + 1] = 2.0 * si / N;
    if (wtx_out) wtx_out[v] = Wtl;
    if (wrx_out) wrx_out[v] = Wrl;
    free(buf);
  }
  free(ctr);
  if (zero_bins) *zero_bins = zb;
  return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
