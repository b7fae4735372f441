// Host side of the C ABI declared in include/fnum.h: argument validation in
// the order and with the error identifiers of the reference's MEX gateways,
// the DFT order / band logic, the F-number classes, device-resident plans and
// the host-buffer entry points that stand in for the MEX calls.
#include "../../include/fnum.h"
#include "fnum_internal.h"
#include "fnum_host_tables.h"

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

using fnum::dfl;
using namespace fnum;

namespace fnum {

// ---------------------------------------------------------------------------
// status
// ---------------------------------------------------------------------------
struct StatusInfo {
  int code;
  const char* id;  // suffix of the MEX identifier
  const char* text;
};
const StatusInfo kStatus[] = {
    {FNUM_OK, "OK", "success"},
    {FNUM_ERR_NO_DEVICE, "NoCUDADevices", "Could not find any CUDA-enabled devices!"},
    {FNUM_ERR_INVALID_DEVICE, "InvalidCUDADevice", "Selected device does not exist!"},
    {FNUM_ERR_LATERAL_POSITIONS, "InvalidLateralPositions", "Lateral positions must be a real-valued finite vector!"},
    {FNUM_ERR_AXIAL_POSITIONS, "InvalidAxialPositions", "Axial positions must be a real-valued finite vector!"},
    {FNUM_ERR_RF_DATA, "InvalidRFData", "RF data must be a real-valued array of valid size!"},
    {FNUM_ERR_SAMPLING_RATE, "InvalidSamplingRate", "Sampling rate must be positive!"},
    {FNUM_ERR_STEERING_ANGLE, "InvalidSteeringAngle",
     "Steering angle must be larger than negative pi over two and smaller than pi over two!"},
    {FNUM_ERR_ELEMENT_WIDTH, "InvalidElementWidth", "Element width must be positive and finite!"},
    {FNUM_ERR_ELEMENT_PITCH, "InvalidElementPitch", "Element pitch must be finite and larger than element width!"},
    {FNUM_ERR_SOUND_SPEED, "InvalidSoundSpeed", "Average speed of sound must be positive and finite!"},
    {FNUM_ERR_FREQUENCY_BOUND, "InvalidFrequencyBound",
     "Frequency bounds must be positive, increasing and not exceed the Nyquist frequency!"},
    {FNUM_ERR_FREQUENCY_BOUNDS, "InvalidFrequencyBounds", "Frequency bounds lead to invalid indices!"},
    {FNUM_ERR_TIME_SHIFT, "InvalidTimeShift", "Time index must be nonnegative!"},
    {FNUM_ERR_WINDOW, "InvalidWindow", "Unknown window function or invalid window parameter!"},
    {FNUM_ERR_F_NUMBER, "InvalidFNumber", "Values of F-number must be nonnegative!"},
    {FNUM_ERR_NORMALIZATION, "InvalidNormalization", "Unknown normalization!"},
    {FNUM_ERR_VERBOSITY, "InvalidVerbosityLevel", "Selected verbosity level does not exist!"},
    {FNUM_ERR_ARGUMENT, "InvalidArgument", "Null pointer or size out of range!"},
    {FNUM_ERR_CUDA, "CUDAError", "CUDA error!"},
    {FNUM_ERR_OUT_OF_MEMORY, "CUDAError", "CUDA error: out of device memory!"},
    {FNUM_ERR_INTERNAL, "InternalError", "Device-side consistency check failed!"},
    {FNUM_ERR_TX_F_NUMBER, "InvalidTXFNumber", "Values of transmit F-number must be nonnegative!"},
    {FNUM_ERR_RX_F_NUMBER, "InvalidRXFNumber", "Values of receive F-number must be nonnegative!"},
    {FNUM_ERR_NOALLOC_TOO_LARGE, "NoAllocScratchTooSmall",
     "Problem exceeds the 64 MiB static scratch of fnum_das_pw_noalloc!"},
    {FNUM_ERR_M_ELEMENTS, "TooManyElements", "das_pw.m semantics support at most 256 array elements!"},
};

const StatusInfo* find_status(int s) {
  for (const auto& e : kStatus)
    if (e.code == s) return &e;
  return nullptr;
}

thread_local char g_id_buf[128];

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return FNUM_OK;
  if (e == cudaErrorMemoryAllocation) return FNUM_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return FNUM_ERR_NO_DEVICE;
  if (e == cudaErrorInvalidDevice) return FNUM_ERR_INVALID_DEVICE;
  return FNUM_ERR_CUDA;
}

#define FNUM_CUDA(call)                      \
  do {                                       \
    cudaError_t e_ = (call);                 \
    if (e_ != cudaSuccess) {                 \
      (void)cudaGetLastError();              \
      return cuda_status(e_);                \
    }                                        \
  } while (0)

// ---------------------------------------------------------------------------
// F-number classes (+f_numbers/**)
// ---------------------------------------------------------------------------
double deg2rad(double d) { return (M_PI / 180.0) * d; }

// +f_numbers/+distance/constant.m:90-120
void fn_distance_constant(double dist_deg, double F_ub, const double* p, int n, double* v) {
  const double rad = deg2rad(dist_deg);
  const double sin_d = sin(rad), opc = 1.0 + cos(rad);
  const double inv_sin = (sin_d != 0.0) ? 1.0 / sin_d : INFINITY;
  for (int i = 0; i < n; ++i) {
    const double pl = p[i];
    const bool lb = pl >= 1.0 / opc, ub = pl < inv_sin;
    double val = 0.0;
    if (!lb && pl >= 0.5) {
      const double t = 1.0 / pl - 1.0;
      val = sqrt(1.0 / (t * t) - 1.0) / 2.0;
    } else if (lb && ub) {
      const double t = pl * pl;
      val = (sqrt(2.0 * opc * t - 1.0) + opc * sin_d * t) / (2.0 - 2.0 * sin_d * sin_d * t);
      val = std::min(val, F_ub);
    }
    if (!ub) val = F_ub;
    v[i] = val;
  }
}

// +f_numbers/+grating/angle_lb.m:44-75 with the bounds of grating.m:72-75
void fn_angle_lb(double a_deg, double F_ub, double dist_deg, const double* p, int n, double* v) {
  const double thresh = sin(deg2rad(a_deg));
  const double lower = 1.0 / (1.0 + thresh);
  const double upper = 1.0 / (1.0 / sqrt(1.0 + (2.0 * F_ub) * (2.0 * F_ub)) + thresh);
  for (int i = 0; i < n; ++i) {
    const double pl = p[i];
    double val = 0.0;
    if (pl > lower && pl < upper) {
      const double t = 1.0 / pl - thresh;
      val = sqrt(1.0 / (t * t) - 1.0) / 2.0;
    } else if (pl >= upper) {
      val = F_ub;
    }
    v[i] = val;
  }
  if (dist_deg >= 0) {
    std::vector<double> aa(n);
    fn_distance_constant(dist_deg, INFINITY, p, n, aa.data());
    for (int i = 0; i < n; ++i) v[i] = std::max(v[i], aa[i]);
  }
}

// Brent's minimiser on [a, b] in the Forsythe-Malcolm-Moler "fmin" form
// (R. P. Brent, Algorithms for Minimization without Derivatives, 1973).
// Stands in for MATLAB fminbnd with TolX = 1e-4 (directivity.m:116).
template <typename F>
double fminbnd(F f, double ax, double bx, double tol) {
  const double c = 0.5 * (3.0 - sqrt(5.0));
  const double sqeps = sqrt(DBL_EPSILON);
  double a = ax, b = bx;
  double v = a + c * (b - a), w = v, x = v;
  double e = 0.0, d = 0.0;
  double fx = f(x), fv = fx, fw = fx;
  for (int it = 0; it < 500; ++it) {
    const double xm = 0.5 * (a + b);
    const double tol1 = sqeps * fabs(x) + tol / 3.0, tol2 = 2.0 * tol1;
    if (fabs(x - xm) <= tol2 - 0.5 * (b - a)) break;
    bool golden = true;
    if (fabs(e) > tol1) {
      double r = (x - w) * (fx - fv);
      double q = (x - v) * (fx - fw);
      double p = (x - v) * q - (x - w) * r;
      q = 2.0 * (q - r);
      if (q > 0.0) p = -p;
      q = fabs(q);
      r = e;
      e = d;
      if (fabs(p) < fabs(0.5 * q * r) && p > q * (a - x) && p < q * (b - x)) {
        d = p / q;
        const double u = x + d;
        if ((u - a) < tol2 || (b - u) < tol2) d = (xm - x) >= 0.0 ? tol1 : -tol1;
        golden = false;
      }
    }
    if (golden) {
      e = (x >= xm) ? (a - x) : (b - x);
      d = c * e;
    }
    const double u = (fabs(d) >= tol1) ? x + d : x + (d >= 0.0 ? tol1 : -tol1);
    const double fu = f(u);
    if (fu <= fx) {
      if (u >= x) a = x; else b = x;
      v = w; fv = fw;
      w = x; fw = fx;
      x = u; fx = fu;
    } else {
      if (u < x) a = u; else b = u;
      if (fu <= fw || w == x) {
        v = w; fv = fw;
        w = u; fw = fu;
      } else if (fu <= fv || v == x || v == w) {
        v = u; fv = fu;
      }
    }
  }
  return x;
}

double msinc(double x) {
  if (x == 0.0) return 1.0;
  const double y = M_PI * x;
  return sin(y) / y;
}

// +f_numbers/+directivity/directivity.m:91-120, obliquity rigid (1) or soft (cos)
void fn_directivity(double wop, int soft, double att_dB, const double* p, int n, double* v) {
  const double thresh = pow(10.0, -att_dB / 20.0);
  for (int i = 0; i < n; ++i) {
    const double wl = wop * p[i];
    auto f = [&](double th) {
      const double ob = soft ? cos(th) : 1.0;
      return fabs(ob * msinc(wl * sin(th)) - thresh);
    };
    const double alpha = fminbnd(f, 0.0, M_PI / 2.0, 1e-4);
    v[i] = 1.0 / (2.0 * tan(alpha));
  }
}

int f_number_values(const fnum_f_number* fn, const double* p, int n, double* v) {
  fnum_f_number def = {FNUM_F_ANGLE_LB, 0, {70.0, 1.5, 10.0}};  // gpu_bf_das_pw_rf.cu:360-365
  if (fn == nullptr || fn->kind == FNUM_F_DEFAULT) fn = &def;
  switch (fn->kind) {
    case FNUM_F_CONSTANT:
      if (!(fn->p[0] >= 0)) return FNUM_ERR_F_NUMBER;
      for (int i = 0; i < n; ++i) v[i] = fn->p[0];
      return FNUM_OK;
    case FNUM_F_ANGLE_LB:
      if (!(fn->p[0] >= 0 && fn->p[0] <= 90 && fn->p[1] >= 0 && fn->p[2] <= 90)) return FNUM_ERR_F_NUMBER;
      fn_angle_lb(fn->p[0], fn->p[1], fn->p[2], p, n, v);
      return FNUM_OK;
    case FNUM_F_DISTANCE_CONSTANT:
      if (!(fn->p[0] >= 0 && fn->p[0] <= 90 && fn->p[1] > 0)) return FNUM_ERR_F_NUMBER;
      fn_distance_constant(fn->p[0], fn->p[1], p, n, v);
      return FNUM_OK;
    case FNUM_F_DISTANCE_NONE:
      fn_distance_constant(0.0, INFINITY, p, n, v);
      return FNUM_OK;
    case FNUM_F_DIRECTIVITY:
      if (!(fn->p[0] >= 0 && fn->p[0] <= 1 && fn->p[1] > 0)) return FNUM_ERR_F_NUMBER;
      fn_directivity(fn->p[0], fn->obliquity == FNUM_OBLIQUITY_SOFT, fn->p[1], p, n, v);
      return FNUM_OK;
    case FNUM_F_SZABO:
      if (!(fn->p[0] >= 0 && fn->p[0] <= 1)) return FNUM_ERR_F_NUMBER;
      for (int i = 0; i < n; ++i) v[i] = fn->p[0] * p[i] / 1.2;  // szabo.m:86
      return FNUM_OK;
    default:
      return FNUM_ERR_F_NUMBER;
  }
}

// ---------------------------------------------------------------------------
// windows (host reference of +cuda/gpu_bf_windows.cu, double precision)
// ---------------------------------------------------------------------------
double window_value(fnum_window w, double l, double L) {
  if (!(fabs(l) < L)) return 0.0;
  const double u = fabs(l) / L;
  switch (w.id) {
    case FNUM_WINDOW_BOXCAR: return 1.0;
    case FNUM_WINDOW_HANN: return (1.0 + cos(M_PI * u)) / 2.0;
    case FNUM_WINDOW_TUKEY: {
      const double thr = 1.0 - w.parameter;
      return (u <= thr) ? 1.0 : (1.0 + cos(M_PI * (u - thr) / w.parameter)) / 2.0;
    }
    case FNUM_WINDOW_TRIANGULAR: return 1.0 - u;
    default: return 0.0;
  }
}

bool window_ok(fnum_window w) {
  if (!(w.parameter >= 0.0 && w.parameter <= 1.0)) return false;
  switch (w.id) {
    case FNUM_WINDOW_BOXCAR:
    case FNUM_WINDOW_HANN:
    case FNUM_WINDOW_TRIANGULAR: return true;
    case FNUM_WINDOW_TUKEY: return w.parameter > 0.0;
    default: return false;
  }
}

bool finite_vec(const double* v, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(v[i])) return false;
  return true;
}

// ---------------------------------------------------------------------------
// band (+cuda/gpu_bf_das_pw_rf.cu:494-556)
// ---------------------------------------------------------------------------
int compute_band(const double* pz, int nz, int nt, int ne, double fs, double width, double pitch, double c,
                 const double* fb, double t0, Band* b) {
  (void)width;
  const double M = (ne - 1.0) / 2.0;
  // the MEX pads with the second axial position (gpu_bf_das_pw_rf.cu:525); a
  // single axial position falls back to the first
  const double z1 = (nz >= 2) ? pz[1] : pz[0];
  // element centres in float, as the MEX (gpu_bf_das_pw_rf.cu:498-507)
  // (the aperture term is a float difference squared in float, gpu_bf_das_pw_rf.cu:525)
  const float c0 = (float)(pitch * (0 - M)), c1 = (float)(pitch * ((ne - 1) - M));
  const float apf = c1 - c0;
  const float ap2 = apf * apf;
  const int N_pad = (int)ceil((sqrt((double)ap2 + z1 * z1) - z1) * fs / c);
  const int N = nt + N_pad + 1 - ((nt + N_pad) % 2);
  const double f_lb = fb ? fb[0] : DBL_MIN, f_ub = fb ? fb[1] : fs / 2.0;
  const int k_lb = (int)ceil(f_lb * N / fs);
  const int k_ub = (int)floor(f_ub * N / fs);
  if (!(k_lb > 0 && k_lb <= k_ub && k_ub < N / 2 + 1)) return FNUM_ERR_FREQUENCY_BOUNDS;
  b->N = N;
  b->k_lb = k_lb;
  b->k_ub = k_ub;
  b->K = k_ub - k_lb + 1;
  b->coef = 2.0 * M_PI * fs / (N * c);
  b->add = 2.0 * M_PI * t0 / N;
  b->M = M;
  return FNUM_OK;
}

// DFT order and band of das_pw.m (das_pw.m:340-362): padding from the first axial
// position and the aperture in double; the same bin bounds
int compute_band_m(const double* pz, int nt, int ne, double fs, double pitch, double c, const double* fb, double t0,
                   Band* b) {
  const double M = (ne - 1.0) / 2.0;
  const double ap = pitch * ((ne - 1) - M) - pitch * (0 - M);
  const int N_pad = (int)ceil((sqrt(ap * ap + pz[0] * pz[0]) - pz[0]) * fs / c);
  const int N = nt + N_pad + 1 - ((nt + N_pad) % 2);
  const double f_lb = fb ? fb[0] : DBL_EPSILON, f_ub = fb ? fb[1] : fs / 2.0;
  const int k_lb = (int)ceil(f_lb * N / fs);
  const int k_ub = (int)floor(f_ub * N / fs);
  if (!(k_lb > 0 && k_lb <= k_ub && k_ub < N / 2 + 1)) return FNUM_ERR_FREQUENCY_BOUNDS;
  b->N = N;
  b->k_lb = k_lb;
  b->k_ub = k_ub;
  b->K = k_ub - k_lb + 1;
  b->coef = 2.0 * M_PI * fs / (N * c);
  b->add = 2.0 * M_PI * t0 / N;
  b->M = M;
  return FNUM_OK;
}

// geometry checks shared by both gateways (gpu_bf_das_pw_rf.cu:126-318)
int check_common(const double* px, int nx, const double* pz, int nz, int nt, int ne, double fs, double width,
                 double pitch, double c, const double* fb, double t0, int dev) {
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1) {
    (void)cudaGetLastError();
    return FNUM_ERR_NO_DEVICE;
  }
  if (!px || nx < 1 || !finite_vec(px, nx)) return FNUM_ERR_LATERAL_POSITIONS;
  if (!pz || nz < 1 || !finite_vec(pz, nz)) return FNUM_ERR_AXIAL_POSITIONS;
  if (nt < 2 || ne < 2 || ne > 4096) return FNUM_ERR_RF_DATA;
  if (!(fs > 0) || !std::isfinite(fs)) return FNUM_ERR_SAMPLING_RATE;
  (void)width;
  return FNUM_OK;
}

int check_array(double width, double pitch, double c) {
  if (!(width > 0 && std::isfinite(width))) return FNUM_ERR_ELEMENT_WIDTH;
  if (!(pitch > width && std::isfinite(pitch))) return FNUM_ERR_ELEMENT_PITCH;
  if (!(c > 0 && std::isfinite(c))) return FNUM_ERR_SOUND_SPEED;
  return FNUM_OK;
}

int check_band_args(double fs, const double* fb, double t0) {
  const double f_lb = fb ? fb[0] : DBL_MIN, f_ub = fb ? fb[1] : fs / 2.0;
  if (!(f_lb > 0)) return FNUM_ERR_FREQUENCY_BOUND;
  if (!(f_ub > f_lb)) return FNUM_ERR_FREQUENCY_BOUND;
  if (f_ub > fs / 2) return FNUM_ERR_FREQUENCY_BOUND;
  if (!(t0 >= 0 && std::isfinite(t0))) return FNUM_ERR_TIME_SHIFT;
  return FNUM_OK;
}

int check_device(int dev) {
  int n_dev = 0;
  if (cudaGetDeviceCount(&n_dev) != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_NO_DEVICE;
  }
  // the MEX test (index >= 0 || index < N) is always true (gpu_bf_das_pw_rf.cu:460); this is the intended one
  if (!(dev >= 0 && dev < n_dev)) return FNUM_ERR_INVALID_DEVICE;
  return FNUM_OK;
}

dfl to_df(double v) {
  const float hi = (float)v;
  const float lo = (float)(v - (double)hi);
  return make_float2(hi, lo);
}

// F table of the band; err = status to return for invalid values
int band_f_table(const fnum_f_number* fn, const double* values, int n_values, const Band& b, double pitch,
                 double fs, double c, int err, std::vector<double>& F) {
  F.assign(b.K, 0.0);
  if (values) {
    if (n_values == 1) {
      for (int i = 0; i < b.K; ++i) F[i] = values[0];
    } else if (n_values == b.K) {
      for (int i = 0; i < b.K; ++i) F[i] = values[i];
    } else {
      return err;
    }
  } else {
    std::vector<double> pl(b.K);
    for (int i = 0; i < b.K; ++i) pl[i] = pitch * (b.k_lb + i) * fs / ((double)b.N * c);  // gpu_bf_das_pw_rf.cu:571
    const int s = f_number_values(fn, pl.data(), b.K, F.data());
    if (s != FNUM_OK) return err;
  }
  for (int i = 0; i < b.K; ++i)
    if (!(F[i] >= 0 && F[i] <= DBL_MAX)) return err;  // gpu_bf_das_pw_rf.cu:578-587
  return FNUM_OK;
}

bool f_monotone(const std::vector<double>& F) {
  for (size_t i = 1; i < F.size(); ++i) {
    const double a = ((float)F[i - 1] > FLT_EPSILON) ? F[i - 1] : 0.0;
    const double b = ((float)F[i] > FLT_EPSILON) ? F[i] : 0.0;
    if (b < a) return false;
  }
  return true;
}

void g_table(const std::vector<double>& F, std::vector<dfl>& g) {
  g.resize(F.size());
  for (size_t i = 0; i < F.size(); ++i)
    g[i] = ((float)F[i] > FLT_EPSILON) ? to_df(1.0 / (2.0 * F[i])) : make_float2(-1.0f, 0.0f);
}

}  // namespace fnum

// ---------------------------------------------------------------------------
// plans
// ---------------------------------------------------------------------------
struct fnum_plan {
  int kind = 0;  // 0 = PW, 1 = SA
  int flags = 0;
  int device = 0;
  int n_out = 1;
  int grid = 0;
  int max_grid = 0;   // the segment scratch holds this many blocks
  Band band{};
  fnum::PWDev pw{};
  fnum::SADev sa{};
  std::vector<void*> allocs;
  float2* tw = nullptr;
  float2* X = nullptr;
  unsigned long long* counters = nullptr;
  std::vector<double> F, F2;
  fnum_plan_info info{};
  int nt = 0;
  // plane wave: what the phase tables are built from (fnum_pw_plan_set_sound_speed)
  std::vector<double> hx, hz, hang;
  double fs = 0.0, pitch = 0.0, width = 0.0, t0 = 0.0, c = 0.0;
  // sharpness-loss gradients (fnum_pw_sharpness_grad), allocated on first use
  float2* adj_img = nullptr;
  float2* adj_G = nullptr;     // cotangent dL/dI* of the sharpness loss
  float* adj_invw = nullptr;
  float2* adj_D = nullptr;     // Draw of the derivative forward (dI/dc = -(2 pi i / c) Draw)
  float2* adj_gX = nullptr;
  double* adj_sums = nullptr;
  double* adj_acc = nullptr;   // FP64 sums of the voxel slices, 2 per spectrum entry
  float4* adj_rx = nullptr;    // receive delays and steps of the adjoint (PWDev::rx_tab)
  bool adj_rx_tried = false;
  unsigned* adj_gmax = nullptr;  // fp16 scale inputs of the adjoint: max |G|, max 1/W
  bool adj_invw_ready = false;
  // band DFT on the tensor cores: fp16 hi/lo operand planes, per-line scales, TMA maps
  fnum::DftTc dft{};
  // synthetic aperture on the tensor cores: operand planes, TMA maps, scale word and
  // time-offset phasors (when the plan qualifies), and the chosen variant
  // (0: default = tensor cores when available, 1: recurrence kernels, 2: tensor cores)
  fnum::SaTc satc{};
  bool sa_tc_ok = false;
  int sa_variant = 0;
  // device buffers of the host-buffer entry points (fnum_das_pw / fnum_das_sa), kept for the
  // plan's life so that a cached plan runs without allocating
  double* h_rf = nullptr;
  float2* h_img = nullptr;
  float* h_planes = nullptr;   // real plane, then imaginary plane
  float* h_w = nullptr;
  float* h_w2 = nullptr;
  size_t h_rf_count = 0;

  template <typename T>
  int alloc(T** p, size_t count) {
    void* q = nullptr;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return cuda_status(e);
    }
    allocs.push_back(q);
    *p = (T*)q;
    return FNUM_OK;
  }
  template <typename T>
  int upload(T** p, const std::vector<T>& v) {
    int s = alloc(p, v.size());
    if (s) return s;
    FNUM_CUDA(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return FNUM_OK;
  }
  ~fnum_plan() {
    for (void* p : allocs) cudaFree(p);
  }
};

namespace fnum {

void build_geometry(const double* px, int nx, const double* pz, int nz, int ne, double width, double pitch,
                    double Ku, double M, GeomTables& g) {
  std::vector<double> ctr(ne);
  for (int e = 0; e < ne; ++e) ctr[e] = pitch * (e - M);
  g.col_u.resize(nx); g.col_p.resize(nx); g.col_m.resize(nx); g.col_emid.resize(nx);
  for (int i = 0; i < nx; ++i) {
    g.col_u[i] = to_df(Ku * px[i]);
    g.col_p[i] = to_df(M + px[i] / pitch);
    g.col_m[i] = to_df(px[i]);
    int em = ne;
    for (int e = 0; e < ne; ++e)
      if (ctr[e] >= px[i]) { em = e; break; }
    g.col_emid[i] = em;
  }
  g.row_u2.resize(nz); g.row_p.resize(nz);
  for (int j = 0; j < nz; ++j) {
    const double zu = Ku * pz[j];
    // (K_u z)^2 to double-float accuracy
    const double hi = zu * zu;
    const double lo = fma(zu, zu, -hi);
    const float h = (float)hi;
    g.row_u2[j] = make_float2(h, (float)((hi - (double)h) + lo));
    g.row_p[j] = to_df(pz[j] / pitch);
  }
  g.el_u.resize(ne); g.el_m.resize(ne); g.el_lb.resize(ne); g.el_ub.resize(ne);
  for (int e = 0; e < ne; ++e) {
    g.el_u[e] = to_df(Ku * ctr[e]);
    g.el_m[e] = to_df(ctr[e]);
    g.el_lb[e] = to_df(ctr[e] - width / 2.0);
    g.el_ub[e] = to_df(ctr[e] + width / 2.0);
  }
  // reference float geometry (gpu_bf_das_pw_rf.cu:495-507, 740-770)
  g.px_f.resize(nx); g.pz_f.resize(nz); g.ctr_f.resize(ne); g.lb_f.resize(ne); g.ub_f.resize(ne);
  for (int i = 0; i < nx; ++i) g.px_f[i] = (float)px[i];
  for (int j = 0; j < nz; ++j) g.pz_f[j] = (float)pz[j];
  for (int e = 0; e < ne; ++e) {
    g.ctr_f[e] = (float)(pitch * (e - M));
    g.lb_f[e] = (float)(g.ctr_f[e] - width / 2);
    g.ub_f[e] = (float)(g.ctr_f[e] + width / 2);
  }
}

void build_tx_tables(const double* px, int nx, const double* pz, int nz, const double* angles, int na, double Ku,
                     double M, double pitch, double t0, int N, std::vector<dfl>& ax, std::vector<dfl>& az) {
  ax.resize((size_t)na * nx);
  az.resize((size_t)na * nz);
  for (int a = 0; a < na; ++a) {
    const double ex = -sin(angles[a]), ez = cos(angles[a]);
    const double xref = (ex >= 0) ? -M * pitch : M * pitch;  // gpu_bf_das_pw_rf.cu:519
    for (int i = 0; i < nx; ++i) ax[(size_t)a * nx + i] = to_df(Ku * ex * (px[i] - xref) + t0 / N);
    for (int j = 0; j < nz; ++j) az[(size_t)a * nz + j] = to_df(Ku * ez * pz[j]);
  }
}

template <typename D>
int upload_geometry(fnum_plan* P, const GeomTables& g, D& d) {
  int s;
  dfl* p;
  int* ip;
  float* fp;
  if ((s = P->upload(&p, g.col_u))) return s; d.col_u = p;
  if ((s = P->upload(&p, g.col_p))) return s; d.col_p = p;
  if ((s = P->upload(&p, g.col_m))) return s; d.col_m = p;
  if ((s = P->upload(&ip, g.col_emid))) return s; d.col_emid = ip;
  if ((s = P->upload(&p, g.row_u2))) return s; d.row_u2 = p;
  if ((s = P->upload(&p, g.row_p))) return s; d.row_p = p;
  if ((s = P->upload(&p, g.el_u))) return s; d.el_u = p;
  if ((s = P->upload(&p, g.el_m))) return s; d.el_m = p;
  if ((s = P->upload(&p, g.el_lb))) return s; d.el_lb = p;
  if ((s = P->upload(&p, g.el_ub))) return s; d.el_ub = p;
  if ((s = P->upload(&fp, g.px_f))) return s; d.px_f = fp;
  if ((s = P->upload(&fp, g.pz_f))) return s; d.pz_f = fp;
  if ((s = P->upload(&fp, g.ctr_f))) return s; d.ctr_f = fp;
  if ((s = P->upload(&fp, g.lb_f))) return s; d.lb_f = fp;
  if ((s = P->upload(&fp, g.ub_f))) return s; d.ub_f = fp;
  return FNUM_OK;
}

int check_pw(const fnum_pw_desc* d, const double* angles, int na) {
  if (!d) return FNUM_ERR_ARGUMENT;
  int s = check_common(d->positions_x, d->n_x, d->positions_z, d->n_z, d->n_samples, d->n_elements, d->f_s,
                       d->element_width, d->element_pitch, d->c_0, d->f_bounds, d->index_t0, d->device);
  if (s) return s;
  if (!angles || na < 1) return FNUM_ERR_STEERING_ANGLE;
  for (int a = 0; a < na; ++a)
    if (!(angles[a] > -M_PI / 2 && angles[a] < M_PI / 2)) return FNUM_ERR_STEERING_ANGLE;
  if ((s = check_array(d->element_width, d->element_pitch, d->c_0))) return s;
  if ((s = check_band_args(d->f_s, d->f_bounds, d->index_t0))) return s;
  if (!window_ok(d->window)) return FNUM_ERR_WINDOW;
  if (d->normalization < 0 || d->normalization > 2) return FNUM_ERR_NORMALIZATION;
  return check_device(d->device);
}

int check_sa(const fnum_sa_desc* d) {
  if (!d) return FNUM_ERR_ARGUMENT;
  int s = check_common(d->positions_x, d->n_x, d->positions_z, d->n_z, d->n_samples, d->n_elements, d->f_s,
                       d->element_width, d->element_pitch, d->c_0, d->f_bounds, d->index_t0, d->device);
  if (s) return s;
  if ((s = check_array(d->element_width, d->element_pitch, d->c_0))) return s;
  if ((s = check_band_args(d->f_s, d->f_bounds, d->index_t0))) return s;
  if (!window_ok(d->window_tx) || !window_ok(d->window_rx)) return FNUM_ERR_WINDOW;
  if (d->normalization_tx < 0 || d->normalization_tx > 2 || d->normalization_rx < 0 || d->normalization_rx > 2)
    return FNUM_ERR_NORMALIZATION;
  return check_device(d->device);
}

// Band DFT on the tensor cores (fnum_dft_tc.cu): the operand planes for nsig RF
// lines and the twiddle planes, built once from the plan's FP64 twiddle table.
int setup_tc_dft(fnum_plan* P, int nsig, int k_lb, int K) {
  const size_t Kp = (size_t)(P->nt + 63) / 64 * 64, Np = (size_t)(2 * K + 127) / 128 * 128;
  __half_raw* a = nullptr;
  __half_raw* b = nullptr;
  float* sc = nullptr;
  int s;
  if ((s = P->alloc(&a, 2 * (size_t)nsig * Kp)) || (s = P->alloc(&b, 2 * Np * Kp)) || (s = P->alloc(&sc, nsig)))
    return s;
  P->info.scratch_bytes += (long long)fnum::dft_tc_bytes(nsig, P->nt, K);
  cudaError_t e = fnum::dft_tc_setup(P->dft, nsig, P->nt, P->band.N, k_lb, K, P->tw, a, b, sc, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e == cudaSuccess ? FNUM_OK : cuda_status(e);
}

int make_pw_plan(const fnum_pw_desc* d, const double* angles, int na, int flags, fnum_plan** out) {
  int s = check_pw(d, angles, na);
  if (s) return s;
  FNUM_CUDA(cudaSetDevice(d->device));
  const bool msem = (flags & FNUM_FLAG_M_SEMANTICS) != 0;
  if (msem && d->n_elements > fnum::M_MAXE) return FNUM_ERR_M_ELEMENTS;
  Band b;
  if (msem) {
    if ((s = compute_band_m(d->positions_z, d->n_samples, d->n_elements, d->f_s, d->element_pitch, d->c_0,
                            d->f_bounds, d->index_t0, &b)))
      return s;
  } else if ((s = compute_band(d->positions_z, d->n_z, d->n_samples, d->n_elements, d->f_s, d->element_width,
                               d->element_pitch, d->c_0, d->f_bounds, d->index_t0, &b))) {
    return s;
  }
  fnum_plan* P = new (std::nothrow) fnum_plan();
  if (!P) return FNUM_ERR_OUT_OF_MEMORY;
  P->kind = 0;
  P->flags = flags;
  P->device = d->device;
  P->band = b;
  P->nt = d->n_samples;
  if ((s = band_f_table(&d->f_number, d->f_number_values, d->n_f_number_values, b, d->element_pitch, d->f_s, d->c_0,
                        FNUM_ERR_F_NUMBER, P->F))) {
    delete P;
    return s;
  }
  const int nx = d->n_x, nz = d->n_z, ne = d->n_elements;
  const double Ku = d->f_s / ((double)b.N * d->c_0);
  GeomTables g;
  build_geometry(d->positions_x, nx, d->positions_z, nz, ne, d->element_width, d->element_pitch, Ku, b.M, g);
  fnum::PWDev& D = P->pw;
  D.nx = nx; D.nz = nz; D.ne = ne; D.na = na; D.K = b.K; D.k_lb = b.k_lb; D.k_ub = b.k_ub; D.N_dft = b.N;
  D.window_id = d->window.id; D.window_par = (float)d->window.parameter;
  D.norm = d->normalization != FNUM_NORMALIZATION_OFF;
  const bool mono = f_monotone(P->F);
  D.seg_cap = (mono ? std::min(b.K, 2 * ne + 16) : b.K) + 1;  // + the sentinel entry
  D.flush_chunks = 4;
  D.scale = (float)(2.0 / b.N);
  D.t0N = (float)(d->index_t0 / b.N);
  D.x_na = na;
  D.x_a0 = 0;
  std::vector<dfl> ax, az, gg;
  build_tx_tables(d->positions_x, nx, d->positions_z, nz, angles, na, Ku, b.M, d->element_pitch, d->index_t0, b.N, ax,
                  az);
  std::vector<float4> txf(na);
  for (int a = 0; a < na; ++a) {
    const double ex = -sin(angles[a]), ez = cos(angles[a]);
    const double xref = (ex >= 0) ? -b.M * d->element_pitch : b.M * d->element_pitch;  // gpu_bf_das_pw_rf.cu:519
    txf[a] = make_float4((float)ex, (float)ez, (float)xref, 0.0f);
  }
  g_table(P->F, gg);
  std::vector<float> Ff(b.K);
  for (int i = 0; i < b.K; ++i) Ff[i] = (float)P->F[i];
  dfl* p;
  float* fp;
  float4* f4;
  if ((s = upload_geometry(P, g, D)) || (s = P->upload(&p, ax))) goto fail;
  D.tx_ax = p;
  if ((s = P->upload(&p, az))) goto fail;
  D.tx_az = p;
  if ((s = P->upload(&p, gg))) goto fail;
  D.g = p;
  if ((s = P->upload(&fp, Ff))) goto fail;
  D.F_f = fp;
  if ((s = P->upload(&f4, txf))) goto fail;
  D.tx_f = f4;
  D.M_f = (float)b.M;
  D.pitch_f = (float)d->element_pitch;
  D.coef_f = (float)b.coef;
  D.add_f = (float)b.add;
  if ((s = P->alloc(&P->tw, b.N))) goto fail;
  if ((s = P->alloc(&P->X, (size_t)ne * b.K * na))) goto fail;
  D.X = P->X;
  if ((s = P->alloc(&P->counters, 8))) goto fail;
  D.counters = P->counters;
  if (cudaMemset(P->counters, 0, 8 * sizeof(unsigned long long)) != cudaSuccess) {
    s = FNUM_ERR_CUDA;
    goto fail;
  }
  if (msem) {
    // das_pw.m semantics: double geometry and tables of pw_m_kernel (no segment scratch)
    std::vector<double> mtx((size_t)3 * na), px(d->positions_x, d->positions_x + nx),
        pz(d->positions_z, d->positions_z + nz);
    for (int a = 0; a < na; ++a) {
      const double ex = -sin(angles[a]), ez = cos(angles[a]);
      const double c0 = d->element_pitch * (0 - b.M);
      mtx[3 * a] = ex;
      mtx[3 * a + 1] = ez;
      mtx[3 * a + 2] = (ex > 0 ? 1.0 : (ex < 0 ? -1.0 : 0.0)) * c0;  // x_ref = sign(e_x) c_1 (das_pw.m:327)
    }
    double* dp;
    if ((s = P->upload(&dp, px))) goto fail;
    D.m_px = dp;
    if ((s = P->upload(&dp, pz))) goto fail;
    D.m_pz = dp;
    if ((s = P->upload(&dp, mtx))) goto fail;
    D.m_tx = dp;
    if ((s = P->upload(&dp, P->F))) goto fail;
    D.m_F0 = dp;
    if ((s = P->alloc(&D.m_sig, (size_t)nz * b.K)) || (s = P->alloc(&D.m_sig_flag, (size_t)nz))) goto fail;
    D.m_sem = 1;
    D.m_norm = d->normalization == FNUM_NORMALIZATION_OFF ? 0 : (d->normalization == FNUM_NORMALIZATION_WINDOWED ? 2 : 1);
    D.m_nwin_id = d->normalization_window.id;
    D.m_nwin_par = (float)d->normalization_window.parameter;
    D.m_c = d->c_0;
    D.m_fs = d->f_s;
    D.m_t0 = d->index_t0;
    D.m_pitch = d->element_pitch;
    D.m_width = d->element_width;
    D.m_M = b.M;
    P->grid = 0;
    P->max_grid = 0;
  } else {
    int bps = 0;
    P->grid = fnum::pw_fused_grid(D, &bps);
    // scratch for the largest grid of any kernel variant, so the autotuner may switch
    P->max_grid = fnum::pw_fused_max_grid(D);
    int4* seg;
    if ((s = P->alloc(&seg, (size_t)P->max_grid * fnum::NTHREADS * D.seg_cap * fnum::PW_SEG_INT4))) goto fail;
    D.seg = seg;
    P->info.scratch_bytes =
        (long long)P->max_grid * fnum::NTHREADS * D.seg_cap * fnum::PW_SEG_INT4 * (long long)sizeof(int4);
    // tensor-core variant: spectra as mma fragments (32 uint4 per n-tile, bin and group of 8 elements)
    D.tc_S = (ne + 7) / 8 + fnum::TC_KS - 1;   // a pass may start in the last group of 8
    D.tc_nt = fnum::tc_ntiles_for(na);
    // the fragments in the layout of the plan's passes, or of 12-angle passes (the
    // derivative kernel's), whichever is larger
    size_t n_tc = 0;
    for (int nt : {3, D.tc_nt})
      n_tc = std::max(n_tc, (size_t)((na + 4 * nt - 1) / (4 * nt)) * D.K * D.tc_S * 32 * nt);
    if ((s = P->alloc(&D.tc_B, n_tc))) goto fail;
    if ((s = P->alloc(&D.tc_max, 1))) goto fail;
    P->info.scratch_bytes += (long long)(n_tc * sizeof(uint4) + sizeof(unsigned));
    // the default variant may now be the tensor-core one
    P->grid = std::min(fnum::pw_fused_grid(D, &bps), P->max_grid);
  }
  {
    cudaError_t e = fnum::launch_twiddles(P->tw, b.N, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      s = cuda_status(e);
      goto fail;
    }
  }
  if ((s = setup_tc_dft(P, na * ne, D.k_lb, D.K))) goto fail;
  P->n_out = (flags & FNUM_FLAG_COMPOUND) ? 1 : na;
  P->hx.assign(d->positions_x, d->positions_x + nx);
  P->hz.assign(d->positions_z, d->positions_z + nz);
  P->hang.assign(angles, angles + na);
  P->fs = d->f_s;
  P->pitch = d->element_pitch;
  P->width = d->element_width;
  P->t0 = d->index_t0;
  P->c = d->c_0;
  P->info.N_dft = b.N; P->info.k_lb = b.k_lb; P->info.k_ub = b.k_ub; P->info.n_bins = b.K;
  P->info.n_x = nx; P->info.n_z = nz; P->info.n_elements = ne; P->info.n_angles = na; P->info.n_samples = d->n_samples;
  P->info.f_monotone = mono;
  P->info.terms = (long long)nx * nz * ne * b.K * na;
  P->info.scale = 2.0 / b.N;
  *out = P;
  return FNUM_OK;
fail:
  delete P;
  return s;
}

int make_sa_plan(const fnum_sa_desc* d, int flags, fnum_plan** out) {
  int s = check_sa(d);
  if (s) return s;
  FNUM_CUDA(cudaSetDevice(d->device));
  Band b;
  if ((s = compute_band(d->positions_z, d->n_z, d->n_samples, d->n_elements, d->f_s, d->element_width,
                        d->element_pitch, d->c_0, d->f_bounds, d->index_t0, &b)))
    return s;
  fnum_plan* P = new (std::nothrow) fnum_plan();
  if (!P) return FNUM_ERR_OUT_OF_MEMORY;
  P->kind = 1;
  P->flags = flags;
  P->device = d->device;
  P->nt = d->n_samples;
  if ((s = band_f_table(&d->f_number_tx, d->f_number_tx_values, d->n_f_number_values, b, d->element_pitch, d->f_s,
                        d->c_0, FNUM_ERR_TX_F_NUMBER, P->F)) ||
      (s = band_f_table(&d->f_number_rx, d->f_number_rx_values, d->n_f_number_values, b, d->element_pitch, d->f_s,
                        d->c_0, FNUM_ERR_RX_F_NUMBER, P->F2))) {
    delete P;
    return s;
  }
  const bool on_tx = d->normalization_tx != FNUM_NORMALIZATION_OFF;
  const bool on_rx = d->normalization_rx != FNUM_NORMALIZATION_OFF;
  const bool intended = (flags & FNUM_FLAG_SAFT_INTENDED) != 0;
  int last_bin_only = 0;
  if (!intended && !on_tx && !on_rx) last_bin_only = 1;  // shared buffer cleared every bin (gpu_bf_saft_rf.cu:1128-1148)
  if (!intended && !on_tx && on_rx) last_bin_only = -1;  // never accumulated (gpu_bf_saft_rf.cu:1195-1199)
  // restrict the processed band to the single surviving bin
  Band bk = b;
  std::vector<double> Ftx = P->F, Frx = P->F2;
  if (last_bin_only == 1) {
    bk.k_lb = b.k_ub;
    bk.K = 1;
    Ftx.assign(1, P->F.back());
    Frx.assign(1, P->F2.back());
  }
  P->band = bk;
  const int nx = d->n_x, nz = d->n_z, ne = d->n_elements;
  const double Ku = d->f_s / ((double)b.N * d->c_0);
  GeomTables g;
  build_geometry(d->positions_x, nx, d->positions_z, nz, ne, d->element_width, d->element_pitch, Ku, b.M, g);
  fnum::SADev& D = P->sa;
  D.nx = nx; D.nz = nz; D.ne = ne; D.K = bk.K; D.k_lb = bk.k_lb; D.k_ub = bk.k_ub; D.N_dft = b.N;
  D.wtx_id = d->window_tx.id; D.wtx_par = (float)d->window_tx.parameter;
  D.wrx_id = d->window_rx.id; D.wrx_par = (float)d->window_rx.parameter;
  D.norm_tx = on_tx;
  D.norm_rx = on_rx;
  D.last_bin_only = last_bin_only;
  const bool mono = f_monotone(Ftx) && f_monotone(Frx);
  D.seg_cap = (mono ? std::min(bk.K, 4 * ne + 32) : bk.K) + 1;  // + the sentinel entry
  D.flush_chunks = 4;
  D.scale = (float)(2.0 / b.N);
  D.t0N = to_df(d->index_t0 / b.N);
  std::vector<dfl> gt, gr;
  g_table(Ftx, gt);
  g_table(Frx, gr);
  std::vector<float> Ftf(bk.K), Frf(bk.K);
  for (int i = 0; i < bk.K; ++i) {
    Ftf[i] = (float)Ftx[i];
    Frf[i] = (float)Frx[i];
  }
  dfl* p;
  float* fp;
  if ((s = upload_geometry(P, g, D)) || (s = P->upload(&p, gt))) goto fail;
  D.gtx = p;
  if ((s = P->upload(&p, gr))) goto fail;
  D.grx = p;
  if ((s = P->upload(&fp, Ftf))) goto fail;
  D.Ftx_f = fp;
  if ((s = P->upload(&fp, Frf))) goto fail;
  D.Frx_f = fp;
  D.M_f = (float)b.M;
  D.pitch_f = (float)d->element_pitch;
  D.coef_f = (float)b.coef;
  D.add_f = (float)b.add;
  if ((s = P->alloc(&P->tw, b.N))) goto fail;
  if ((s = P->alloc(&P->X, (size_t)ne * ne * bk.K))) goto fail;
  D.X = P->X;
  // transmit/receive symmetry: equal windows, F-number tables and normalisations make the
  // weight and phase of (t, r) and (r, t) equal
  D.Xs = nullptr;
  if (d->window_tx.id == d->window_rx.id && d->window_tx.parameter == d->window_rx.parameter && Ftx == Frx &&
      on_tx == on_rx && !(flags & FNUM_FLAG_PLAIN_KERNEL)) {
    if ((s = P->alloc(&D.Xs, (size_t)ne * ne * bk.K))) goto fail;
  }
  if ((s = P->alloc(&P->counters, 8))) goto fail;
  D.counters = P->counters;
  if (cudaMemset(P->counters, 0, 8 * sizeof(unsigned long long)) != cudaSuccess) {
    s = FNUM_ERR_CUDA;
    goto fail;
  }
  {
    int bps = 0;
    P->grid = fnum::sa_fused_grid(D, &bps);
    P->max_grid = P->grid;
    int4* seg;
    if ((s = P->alloc(&seg, (size_t)P->grid * fnum::NTHREADS * D.seg_cap * fnum::SA_SEG_INT4))) goto fail;
    D.seg = seg;
    P->info.scratch_bytes = (long long)P->grid * fnum::NTHREADS * D.seg_cap * fnum::SA_SEG_INT4 * (long long)sizeof(int4);
    if (D.Xs) P->info.scratch_bytes += (long long)ne * ne * bk.K * (long long)sizeof(float2);
  }
  if (!(flags & FNUM_FLAG_PLAIN_KERNEL) && fnum::sa_tc_supported(D)) {
    // operand planes of the tensor-core kernel and the phasors e^{2 pi i k t0 / N} of the band
    unsigned short* planes = nullptr;
    unsigned* mb = nullptr;
    float2* rot = nullptr;
    std::vector<float2> rv(bk.K);
    for (int i = 0; i < bk.K; ++i) {
      const double cyc = std::fmod((double)(bk.k_lb + i) * d->index_t0, (double)b.N) / (double)b.N;
      rv[i] = make_float2((float)std::cos(2.0 * M_PI * cyc), (float)std::sin(2.0 * M_PI * cyc));
    }
    const size_t nb = fnum::sa_tc_bytes(ne, bk.K);
    if ((s = P->alloc(&planes, nb / 2)) || (s = P->alloc(&mb, 1)) || (s = P->upload(&rot, rv))) goto fail;
    if (fnum::sa_tc_setup(P->satc, D, planes, mb, rot) == cudaSuccess) {
      P->sa_tc_ok = true;
      P->info.scratch_bytes += (long long)nb;
    } else {
      (void)cudaGetLastError();
    }
  }
  {
    cudaError_t e = fnum::launch_twiddles(P->tw, b.N, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      s = cuda_status(e);
      goto fail;
    }
  }
  if ((s = setup_tc_dft(P, ne * ne, D.k_lb, D.K))) goto fail;
  P->n_out = 1;
  P->info.N_dft = b.N; P->info.k_lb = bk.k_lb; P->info.k_ub = bk.k_ub; P->info.n_bins = bk.K;
  P->info.n_x = nx; P->info.n_z = nz; P->info.n_elements = ne; P->info.n_angles = 1; P->info.n_samples = d->n_samples;
  P->info.f_monotone = mono;
  P->info.terms = (long long)nx * nz * ne * ne * bk.K;
  P->info.scale = 2.0 / b.N;
  *out = P;
  return FNUM_OK;
fail:
  delete P;
  return s;
}

// the synthetic-aperture kernel a plan runs: 1 recurrence kernels, 2 tensor cores
int sa_variant_of(const fnum_plan* P) {
  if (P->sa_variant) return P->sa_variant;
  return P->sa_tc_ok ? 2 : 1;
}

// the band DFT of d_rf into the plan's spectra; counters[5] collects its error bits
int plan_dft(fnum_plan* P, const void* rf, int is_double, cudaStream_t st) {
  FNUM_CUDA(cudaMemsetAsync(P->counters + 5, 0, sizeof(unsigned long long), st));
  if (P->kind == 0) {
    // PW: signal s = a ne + e  ->  X[e][k][a]
    const fnum::PWDev& D = P->pw;
    return cuda_status(fnum::dft_tc_run(P->dft, rf, is_double, P->X, D.ne, 1, (long long)D.K * D.na, D.na,
                                        P->counters + 5, st));
  }
  // SA: signal s = tx ne + rx  ->  X[s][k]
  const fnum::SADev& D = P->sa;
  return cuda_status(fnum::dft_tc_run(P->dft, rf, is_double, P->X, D.ne * D.ne, 0, D.K, 1, P->counters + 5, st));
}

int plan_beamform(fnum_plan* P, void* image, float* w, float* w2, cudaStream_t st) {
  FNUM_CUDA(cudaMemsetAsync(P->counters, 0, 5 * sizeof(unsigned long long), st));   // [5] is the DFT's
  const bool plain = (P->flags & FNUM_FLAG_PLAIN_KERNEL) != 0;
  if (P->kind == 1) {
    cudaError_t e;
    if (plain) e = fnum::launch_sa_plain(P->sa, (float2*)image, w, w2, st);
    else if (sa_variant_of(P) == 2)
      e = fnum::launch_sa_tc(P->sa, P->satc, std::min(fnum::sa_tc_grid(P->sa), P->max_grid), (float2*)image, w, w2,
                             st);
    else e = fnum::launch_sa_fused(P->sa, P->grid, (float2*)image, w, w2, st);
    return cuda_status(e);
  }
  const fnum::PWDev& D = P->pw;
  if (D.m_sem) return cuda_status(fnum::launch_pw_m(D, P->n_out == 1, (float2*)image, w, st));
  if (P->n_out == 1) {
    cudaError_t e = plain ? fnum::launch_pw_plain(D, (float2*)image, w, st)
                          : fnum::launch_pw_fused(D, P->grid, (float2*)image, w, st);
    return cuda_status(e);
  }
  for (int a = 0; a < D.na; ++a) {
    fnum::PWDev Da = D;
    Da.na = 1;
    Da.x_a0 = a;
    Da.tx_ax = D.tx_ax + (size_t)a * D.nx;
    Da.tx_az = D.tx_az + (size_t)a * D.nz;
    Da.tx_f = D.tx_f + a;
    float2* img = (float2*)image + (size_t)a * D.nx * D.nz;
    float* wa = (a == 0) ? w : nullptr;
    cudaError_t e = plain ? fnum::launch_pw_plain(Da, img, wa, st) : fnum::launch_pw_fused(Da, P->grid, img, wa, st);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return FNUM_OK;
}

// device buffers of the host-buffer entry points, allocated once per plan
int host_buffers(fnum_plan* P, size_t rf_count) {
  const size_t nvox = (size_t)P->info.n_x * P->info.n_z;
  const size_t nimg = nvox * P->n_out;
  int s = FNUM_OK;
  if (!P->h_rf) {
    if ((s = P->alloc(&P->h_rf, rf_count)) ||
        (s = P->alloc(&P->h_img, nimg)) || (s = P->alloc(&P->h_planes, 2 * nimg)) ||
        (s = P->alloc(&P->h_w, nvox)) || (s = P->alloc(&P->h_w2, nvox)))
      return s;
    P->h_rf_count = rf_count;
  }
  return rf_count == P->h_rf_count ? FNUM_OK : FNUM_ERR_ARGUMENT;
}

// host-buffer execution shared by fnum_das_pw / fnum_das_sa
int run_host(fnum_plan* P, const double* rf, size_t rf_count, float* re, float* im, float* w, float* w2) {
  const size_t nvox = (size_t)P->info.n_x * P->info.n_z;
  const size_t nimg = nvox * P->n_out;
  int s = host_buffers(P, rf_count);
  if (s) return s;
  float* d_w = w ? P->h_w : nullptr;
  float* d_w2 = w2 ? P->h_w2 : nullptr;
  cudaError_t e = cudaMemcpy(P->h_rf, rf, rf_count * sizeof(double), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_status(e);
  // the band DFT rounds double RF to float first, as the reference does
  if ((s = plan_dft(P, P->h_rf, 1, 0))) return s;
  if ((s = plan_beamform(P, P->h_img, d_w, d_w2, 0))) return s;
  if ((e = fnum::launch_split_complex(P->h_img, nimg, P->h_planes, P->h_planes + nimg, 0)) != cudaSuccess)
    return cuda_status(e);
  e = cudaMemcpy(re, P->h_planes, nimg * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(im, P->h_planes + nimg, nimg * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && w) e = cudaMemcpy(w, d_w, nvox * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && w2) e = cudaMemcpy(w2, d_w2, nvox * sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  unsigned long long c[8];
  if ((e = cudaMemcpy(c, P->counters, sizeof(c), cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda_status(e);
  if ((c[2] & (fnum::ERR_SEG_OVERFLOW | fnum::ERR_TC_TIMEOUT)) || (c[5] & fnum::ERR_DFT_TIMEOUT)) return FNUM_ERR_INTERNAL;
  return FNUM_OK;
}

// Plans of the host-buffer gateways, kept across calls: repeated calls with the
// same arguments reuse the device tables and buffers (the reference allocates
// and frees everything per call).  The key holds the argument VALUES -- every
// scalar, position, bound, F value and angle that shapes a plan -- never the
// addresses of the caller's arrays, so equal geometry in fresh arrays (MATLAB
// temporaries) finds its plan.  A small least-recently-used list per gateway
// lets a caller alternate between a few geometries without rebuilding.
constexpr size_t kPlanCacheEntries = 4;

struct PlanCache {
  std::mutex mu;
  std::vector<std::pair<std::vector<unsigned char>, fnum_plan*>> lru;   // most recent last
  long long created = 0;
};
PlanCache g_pw_cache, g_sa_cache;

struct KeyWriter {
  std::vector<unsigned char> k;
  template <typename T>
  void put(T v) {
    const unsigned char* c = (const unsigned char*)&v;
    k.insert(k.end(), c, c + sizeof(T));
  }
  void put_array(const double* p, int n) {
    put(n);
    put((int)(p != nullptr));
    if (p && n > 0) {
      const unsigned char* c = (const unsigned char*)p;
      k.insert(k.end(), c, c + sizeof(double) * (size_t)n);
    }
  }
  void put_window(const fnum_window& w) {
    put(w.id);
    put(w.parameter);
  }
  void put_f_number(const fnum_f_number& f) {
    put(f.kind);
    put(f.obliquity);
    for (double v : f.p) put(v);
  }
};

// key of a plane-wave plan: the values of every input that shapes it
std::vector<unsigned char> pw_key(const fnum_pw_desc* desc, const double* steering_angles, int n_angles, int flags) {
  KeyWriter kw;
  kw.put_array(desc->positions_x, desc->n_x);
  kw.put_array(desc->positions_z, desc->n_z);
  kw.put(desc->n_samples);
  kw.put(desc->n_elements);
  kw.put(desc->f_s);
  kw.put(desc->element_width);
  kw.put(desc->element_pitch);
  kw.put(desc->c_0);
  kw.put_array(desc->f_bounds, 2);
  kw.put(desc->index_t0);
  kw.put_window(desc->window);
  kw.put_f_number(desc->f_number);
  kw.put_array(desc->f_number_values, desc->f_number_values ? desc->n_f_number_values : 0);
  kw.put(desc->normalization);
  kw.put(desc->device);
  kw.put_window(desc->normalization_window);
  kw.put_array(steering_angles, n_angles);
  kw.put(flags);
  return kw.k;
}

// the cached plan for `key`, or a new one from `make` (which may fail); the
// least recently used plan is destroyed when the list is full
template <typename Make>
int cached_plan(PlanCache& C, const std::vector<unsigned char>& key, Make make, fnum_plan** out) {
  for (size_t i = 0; i < C.lru.size(); ++i) {
    if (C.lru[i].first == key) {
      auto hit = C.lru[i];
      C.lru.erase(C.lru.begin() + (long)i);
      C.lru.push_back(hit);
      *out = hit.second;
      return FNUM_OK;
    }
  }
  fnum_plan* P = nullptr;
  const int s = make(&P);
  if (s) return s;
  ++C.created;
  if (C.lru.size() >= kPlanCacheEntries) {
    fnum_plan_destroy(C.lru.front().second);
    C.lru.erase(C.lru.begin());
  }
  C.lru.emplace_back(key, P);
  *out = P;
  return FNUM_OK;
}

}  // namespace fnum

// ---------------------------------------------------------------------------
// exported C ABI
// ---------------------------------------------------------------------------
extern "C" {

int fnum_abi_version(void) { return FNUM_ABI_VERSION; }

const char* fnum_status_string(int status) {
  const StatusInfo* e = find_status(status);
  return e ? e->text : "unknown status";
}

const char* fnum_status_id(int status, int saft) {
  const StatusInfo* e = find_status(status);
  const char* pre = (status == FNUM_ERR_CUDA || status == FNUM_ERR_OUT_OF_MEMORY)
                        ? "gpu_bf_error_handling"
                        : (saft ? "gpu_bf_saft_rf" : "gpu_bf_das_pw_rf");
  snprintf(g_id_buf, sizeof(g_id_buf), "%s:%s", pre, e ? e->id : "Unknown");
  return g_id_buf;
}

int fnum_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    (void)cudaGetLastError();
    return 0;
  }
  return n;
}

int fnum_band(const double* positions_z, int n_z, int n_samples, int n_elements, double f_s, double element_width,
              double element_pitch, double c_0, const double* f_bounds, double index_t0, int* N_dft, int* k_lb,
              int* k_ub) {
  if (!positions_z || n_z < 1 || n_samples < 2 || n_elements < 2 || !N_dft || !k_lb || !k_ub) return FNUM_ERR_ARGUMENT;
  if (!(f_s > 0)) return FNUM_ERR_SAMPLING_RATE;
  int s = check_array(element_width, element_pitch, c_0);
  if (s) return s;
  if ((s = check_band_args(f_s, f_bounds, index_t0))) return s;
  Band b;
  if ((s = compute_band(positions_z, n_z, n_samples, n_elements, f_s, element_width, element_pitch, c_0, f_bounds,
                        index_t0, &b)))
    return s;
  *N_dft = b.N;
  *k_lb = b.k_lb;
  *k_ub = b.k_ub;
  return FNUM_OK;
}

int fnum_f_number_values(const fnum_f_number* f_number, const double* pitch_over_lambda, int n, double* values) {
  if (!pitch_over_lambda || !values || n < 0) return FNUM_ERR_ARGUMENT;
  for (int i = 0; i < n; ++i)
    if (!(pitch_over_lambda[i] > 0)) return FNUM_ERR_ARGUMENT;  // f_number.m:99 mustBePositive
  return f_number_values(f_number, pitch_over_lambda, n, values);
}

double fnum_window_value(fnum_window window, double l, double L) { return window_value(window, l, L); }

int fnum_pw_plan_create(const fnum_pw_desc* desc, const double* steering_angles, int n_angles, int flags,
                        fnum_plan** plan) {
  if (!plan) return FNUM_ERR_ARGUMENT;
  *plan = nullptr;
  return make_pw_plan(desc, steering_angles, n_angles, flags, plan);
}

int fnum_sa_plan_create(const fnum_sa_desc* desc, int flags, fnum_plan** plan) {
  if (!plan) return FNUM_ERR_ARGUMENT;
  *plan = nullptr;
  return make_sa_plan(desc, flags, plan);
}

int fnum_plan_execute_dft(fnum_plan* plan, const void* d_rf, int rf_is_double, void* stream) {
  if (!plan || !d_rf) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  return plan_dft(plan, d_rf, rf_is_double, (cudaStream_t)stream);
}

int fnum_plan_execute_beamform(fnum_plan* plan, void* d_image, float* d_weights, float* d_weights_rx, void* stream) {
  if (!plan || !d_image) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  return plan_beamform(plan, d_image, d_weights, d_weights_rx, (cudaStream_t)stream);
}

int fnum_plan_execute(fnum_plan* plan, const void* d_rf, int rf_is_double, void* d_image, float* d_weights,
                      float* d_weights_rx, void* stream) {
  if (!plan || !d_rf || !d_image) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  int s = plan_dft(plan, d_rf, rf_is_double, (cudaStream_t)stream);
  if (s) return s;
  return plan_beamform(plan, d_image, d_weights, d_weights_rx, (cudaStream_t)stream);
}

int fnum_plan_spectra(const fnum_plan* plan, void* d_spectra, void* stream) {
  if (!plan || !d_spectra) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  const size_t n = plan->kind == 0 ? (size_t)plan->pw.ne * plan->pw.K * plan->pw.na
                                   : (size_t)plan->sa.ne * plan->sa.ne * plan->sa.K;
  FNUM_CUDA(cudaMemcpyAsync(d_spectra, plan->X, n * sizeof(float2), cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return FNUM_OK;
}

int fnum_plan_info_get(const fnum_plan* plan, fnum_plan_info* info) {
  if (!plan || !info) return FNUM_ERR_ARGUMENT;
  *info = plan->info;
  unsigned long long c[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  cudaError_t e = cudaSetDevice(plan->device);
  if (e == cudaSuccess) e = cudaMemcpy(c, plan->counters, sizeof(c), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return cuda_status(e);
  }
  info->active_terms = (long long)c[0];
  info->zero_weight_bins = (long long)c[1];
  info->executed_terms = (long long)c[4];
  info->kernel_variant = plan->kind == 0 ? fnum::pw_variant_of(plan->pw)
                        : ((plan->flags & FNUM_FLAG_PLAIN_KERNEL) ? 0 : fnum::sa_variant_of(plan));
  info->grid = plan->grid;
  info->blocks_per_sm = 0;
  info->bin_chunk = 0;
  if (plan->kind == 0 && !plan->pw.m_sem) {
    int bps = 0;
    (void)fnum::pw_fused_grid(plan->pw, &bps);
    info->blocks_per_sm = bps;
    info->bin_chunk = fnum::pw_variant_of(plan->pw) == fnum::TC_VARIANT
                          ? ((plan->pw.tc_tb > 0 && plan->pw.tc_tb < 32) ? plan->pw.tc_tb : 32)
                          : plan->pw.flush_chunks * fnum::KCHUNK;
  }
  if ((c[2] & (fnum::ERR_SEG_OVERFLOW | fnum::ERR_TC_TIMEOUT)) || (c[5] & fnum::ERR_DFT_TIMEOUT)) return FNUM_ERR_INTERNAL;
  return FNUM_OK;
}

int fnum_plan_f_numbers(const fnum_plan* plan, double* values) {
  if (!plan || !values) return FNUM_ERR_ARGUMENT;
  std::copy(plan->F.begin(), plan->F.end(), values);
  if (plan->kind == 1) std::copy(plan->F2.begin(), plan->F2.end(), values + plan->F.size());
  return FNUM_OK;
}

int fnum_plan_destroy(fnum_plan* plan) {
  if (!plan) return FNUM_OK;
  cudaSetDevice(plan->device);
  delete plan;
  (void)cudaGetLastError();
  return FNUM_OK;
}

int fnum_das_pw(const fnum_pw_desc* desc, const double* steering_angles, int n_angles, const double* data_rf,
                int flags, float* image_re, float* image_im, float* weights) {
  if (!desc || !data_rf || !image_re || !image_im) return FNUM_ERR_ARGUMENT;
  int s = check_pw(desc, steering_angles, n_angles);
  if (s) return s;
  // cache key: the values of every input that shapes the plan
  const std::vector<unsigned char> key = pw_key(desc, steering_angles, n_angles, flags);
  std::lock_guard<std::mutex> lock(g_pw_cache.mu);
  FNUM_CUDA(cudaSetDevice(desc->device));
  fnum_plan* P = nullptr;
  if ((s = cached_plan(g_pw_cache, key,
                       [&](fnum_plan** p) { return make_pw_plan(desc, steering_angles, n_angles, flags, p); }, &P)))
    return s;
  const size_t rf_count = (size_t)n_angles * desc->n_elements * desc->n_samples;
  return run_host(P, data_rf, rf_count, image_re, image_im, weights, nullptr);
}

int fnum_das_pw_sharpness_grad(const fnum_pw_desc* desc, const double* steering_angles, int n_angles,
                               const double* data_rf, double* loss, double* dloss_dc, float* grad_re,
                               float* grad_im) {
  if (!desc || !data_rf) return FNUM_ERR_ARGUMENT;
  int s = check_pw(desc, steering_angles, n_angles);
  if (s) return s;
  const std::vector<unsigned char> key = pw_key(desc, steering_angles, n_angles, FNUM_FLAG_COMPOUND);
  std::lock_guard<std::mutex> lock(g_pw_cache.mu);
  FNUM_CUDA(cudaSetDevice(desc->device));
  fnum_plan* P = nullptr;
  if ((s = cached_plan(g_pw_cache, key,
                       [&](fnum_plan** p) {
                         return make_pw_plan(desc, steering_angles, n_angles, FNUM_FLAG_COMPOUND, p);
                       },
                       &P)))
    return s;
  const size_t rf_count = (size_t)n_angles * desc->n_elements * desc->n_samples;
  if ((s = host_buffers(P, rf_count))) return s;
  FNUM_CUDA(cudaMemcpy(P->h_rf, data_rf, rf_count * sizeof(double), cudaMemcpyHostToDevice));
  if ((s = fnum_pw_sharpness_grad(P, P->h_rf, 1, loss, dloss_dc, nullptr, nullptr))) return s;
  if (grad_re || grad_im) {
    // plan layout [e][k][a] -> [a][e][k] (bins fastest, MATLAB's [N_bins x N_el x N_angles])
    const fnum::PWDev& D = P->pw;
    std::vector<float2> g((size_t)D.ne * D.K * D.na);
    FNUM_CUDA(cudaMemcpy(g.data(), P->adj_gX, g.size() * sizeof(float2), cudaMemcpyDeviceToHost));
    for (int a = 0; a < D.na; ++a)
      for (int e = 0; e < D.ne; ++e)
        for (int k = 0; k < D.K; ++k) {
          const float2 v = g[((size_t)e * D.K + k) * D.na + a];
          const size_t o = ((size_t)a * D.ne + e) * D.K + k;
          if (grad_re) grad_re[o] = v.x;
          if (grad_im) grad_im[o] = v.y;
        }
  }
  unsigned long long c[8];
  FNUM_CUDA(cudaMemcpy(c, P->counters, sizeof(c), cudaMemcpyDeviceToHost));
  if ((c[2] & (fnum::ERR_SEG_OVERFLOW | fnum::ERR_TC_TIMEOUT)) || (c[5] & fnum::ERR_DFT_TIMEOUT)) return FNUM_ERR_INTERNAL;
  return FNUM_OK;
}

int fnum_das_sa(const fnum_sa_desc* desc, const double* data_rf, int flags, float* image_re, float* image_im,
                float* weights_tx, float* weights_rx) {
  if (!desc || !data_rf || !image_re || !image_im) return FNUM_ERR_ARGUMENT;
  int s = check_sa(desc);
  if (s) return s;
  KeyWriter kw;
  kw.put_array(desc->positions_x, desc->n_x);
  kw.put_array(desc->positions_z, desc->n_z);
  kw.put(desc->n_samples);
  kw.put(desc->n_elements);
  kw.put(desc->f_s);
  kw.put(desc->element_width);
  kw.put(desc->element_pitch);
  kw.put(desc->c_0);
  kw.put_array(desc->f_bounds, 2);
  kw.put(desc->index_t0);
  kw.put_window(desc->window_tx);
  kw.put_window(desc->window_rx);
  kw.put_f_number(desc->f_number_tx);
  kw.put_f_number(desc->f_number_rx);
  const int nfv = desc->n_f_number_values;
  kw.put_array(desc->f_number_tx_values, desc->f_number_tx_values ? nfv : 0);
  kw.put_array(desc->f_number_rx_values, desc->f_number_rx_values ? nfv : 0);
  kw.put(desc->normalization_tx);
  kw.put(desc->normalization_rx);
  kw.put(desc->device);
  kw.put(flags);
  std::lock_guard<std::mutex> lock(g_sa_cache.mu);
  FNUM_CUDA(cudaSetDevice(desc->device));
  fnum_plan* P = nullptr;
  if ((s = cached_plan(g_sa_cache, kw.k, [&](fnum_plan** p) { return make_sa_plan(desc, flags, p); }, &P))) return s;
  const size_t rf_count = (size_t)desc->n_elements * desc->n_elements * desc->n_samples;
  return run_host(P, data_rf, rf_count, image_re, image_im, weights_tx, weights_rx);
}

int fnum_host_cache_info(int saft, long long* plans_created, int* plans_cached) {
  PlanCache& C = saft ? g_sa_cache : g_pw_cache;
  std::lock_guard<std::mutex> lock(C.mu);
  if (plans_created) *plans_created = C.created;
  if (plans_cached) *plans_cached = (int)C.lru.size();
  return FNUM_OK;
}

// ---------------------------------------------------------------------------
// autotuning and batches (no counterpart in the reference, which beamforms one
// angle per gateway call)
// ---------------------------------------------------------------------------
int fnum_plan_set_kernel_variant(fnum_plan* plan, int variant) {
  if (!plan) return FNUM_ERR_ARGUMENT;
  if (plan->kind != 0) {  // synthetic aperture: 1 recurrence kernels, 2 tensor cores
    if (variant < 0 || variant > 2 || (variant == 2 && !plan->sa_tc_ok)) return FNUM_ERR_ARGUMENT;
    if ((plan->flags & FNUM_FLAG_PLAIN_KERNEL) && variant != 0) return FNUM_ERR_ARGUMENT;
    plan->sa_variant = variant;
    return FNUM_OK;
  }
  if (variant < 0 || variant > fnum::pw_variant_count()) return FNUM_ERR_ARGUMENT;
  if (variant == fnum::TC_VARIANT && !plan->pw.tc_B) return FNUM_ERR_ARGUMENT;
  if (plan->pw.m_sem) return variant == 0 ? FNUM_OK : FNUM_ERR_ARGUMENT;     // one per-term kernel
  FNUM_CUDA(cudaSetDevice(plan->device));
  plan->pw.variant = variant;
  plan->grid = std::min(fnum::pw_fused_grid(plan->pw, nullptr), plan->max_grid);
  return FNUM_OK;
}

// synthetic aperture: times the recurrence kernels (1) and, when the plan has them, the
// tensor cores (2) on the plan's spectra and keeps the faster
int autotune_sa(fnum_plan* plan, const void* d_rf, int rf_is_double, int* variant, float* ms) {
  const int v0 = plan->sa_variant;
  if (plan->flags & FNUM_FLAG_PLAIN_KERNEL) {
    if (variant) *variant = 0;
    if (ms) *ms = 0.0f;
    return FNUM_OK;
  }
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float2* img = nullptr;
  float best = 3.0e38f;
  int best_v = 1, s = FNUM_OK;
  const size_t n_img = (size_t)plan->sa.nx * plan->sa.nz;
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMalloc(&img, n_img * sizeof(float2));
  if (e != cudaSuccess) s = cuda_status(e);
  if (!s) s = plan_dft(plan, d_rf, rf_is_double, st);
  for (int v = 1; v <= (plan->sa_tc_ok ? 2 : 1) && !s; ++v) {
    plan->sa_variant = v;
    if ((s = plan_beamform(plan, img, nullptr, nullptr, st))) break;
    float t = 0.0f;
    cudaError_t e2 = cudaEventRecord(e0, st);
    for (int r = 0; r < 2 && e2 == cudaSuccess && !s; ++r) s = plan_beamform(plan, img, nullptr, nullptr, st);
    if (s) break;
    if (e2 == cudaSuccess) e2 = cudaEventRecord(e1, st);
    if (e2 == cudaSuccess) e2 = cudaEventSynchronize(e1);
    if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&t, e0, e1);
    if (e2 != cudaSuccess) {
      s = cuda_status(e2);
      break;
    }
    if (t < best) {
      best = t;
      best_v = v;
    }
  }
  plan->sa_variant = s ? v0 : best_v;
  if (!s) {
    if (variant) *variant = best_v;
    if (ms) *ms = 0.5f * best;
  }
  if (img) cudaFree(img);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  (void)cudaGetLastError();
  return s;
}

int fnum_plan_autotune(fnum_plan* plan, const void* d_rf, int rf_is_double, int* variant, float* ms) {
  if (!plan || !d_rf) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  if (plan->kind != 0) return autotune_sa(plan, d_rf, rf_is_double, variant, ms);
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float2* img = nullptr;
  int s = FNUM_OK;
  const size_t n_img = (size_t)plan->n_out * plan->pw.nx * plan->pw.nz;
  const fnum::PWDev d0 = plan->pw;
  const int g0 = plan->grid;
  float best = 3.0e38f;
  fnum::PWDev best_d = plan->pw;
  int best_g = plan->grid;
  // times the plan's current variant and shape (a warm-up, then two beamforms)
  auto trial = [&]() -> int {
    plan->grid = std::min(fnum::pw_fused_grid(plan->pw, nullptr), plan->max_grid);
    int st2 = plan_beamform(plan, img, nullptr, nullptr, st);
    if (st2) return st2;
    float t = 0.0f;
    cudaError_t e2 = cudaEventRecord(e0, st);
    for (int r = 0; r < 2 && e2 == cudaSuccess && !st2; ++r) st2 = plan_beamform(plan, img, nullptr, nullptr, st);
    if (st2) return st2;
    if (e2 == cudaSuccess) e2 = cudaEventRecord(e1, st);
    if (e2 == cudaSuccess) e2 = cudaEventSynchronize(e1);
    if (e2 == cudaSuccess) e2 = cudaEventElapsedTime(&t, e0, e1);
    if (e2 != cudaSuccess) return cuda_status(e2);
    if (t < best) {
      best = t;
      best_d = plan->pw;
      best_g = plan->grid;
    }
    return FNUM_OK;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMalloc(&img, n_img * sizeof(float2));
  if (e != cudaSuccess) {
    s = cuda_status(e);
    goto done;
  }
  if ((s = plan_dft(plan, d_rf, rf_is_double, st))) goto done;
  // 1: the kernel variants (pass shapes) at the default launch shape
  for (int v = 1; v <= fnum::pw_variant_count() && !s; ++v) {
    plan->pw = d0;
    plan->pw.variant = v;
    plan->pw.blocks_per_sm = 0;
    plan->pw.tc_tb = 0;
    plan->pw.flush_chunks = 4;
    s = trial();
  }
  // 2: the launch shape of the best variant: resident blocks per SM (all, or one fewer,
  // which leaves each block more L1) and the bins between exact re-anchorings (tensor
  // cores: 32 or 16; FP32 kernels: 4 or 2 chunks of 64 bins).  Both alternatives
  // re-anchor at least as often, so none is less accurate than the default.
  if (!s) {
    const fnum::PWDev dv = best_d;
    int bps = 0;
    plan->pw = dv;
    (void)fnum::pw_fused_grid(plan->pw, &bps);
    for (int occ = 0; occ < 2 && !s; ++occ)
      for (int ch = 0; ch < 2 && !s; ++ch) {
        if (occ == 0 && ch == 0) continue;   // the default shape, timed above
        if (occ == 1 && bps <= 1) continue;
        plan->pw = dv;
        plan->pw.blocks_per_sm = occ ? bps - 1 : 0;
        if (fnum::pw_variant_of(dv) == fnum::TC_VARIANT) plan->pw.tc_tb = ch ? 16 : 0;
        else plan->pw.flush_chunks = ch ? 2 : 4;
        s = trial();
      }
  }
done:
  if (s) {
    plan->pw = d0;
    plan->grid = g0;
  } else {
    plan->pw = best_d;
    plan->grid = best_g;
    if (variant) *variant = fnum::pw_variant_of(best_d);
    if (ms) *ms = 0.5f * best;
  }
  if (img) cudaFree(img);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  (void)cudaGetLastError();
  return s;
}

int fnum_plan_set_shape(fnum_plan* plan, int blocks_per_sm, int bin_chunk) {
  if (!plan) return FNUM_ERR_ARGUMENT;
  if (plan->kind != 0 || plan->pw.m_sem)
    return (blocks_per_sm == 0 && bin_chunk == 0) ? FNUM_OK : FNUM_ERR_ARGUMENT;
  if (blocks_per_sm < 0 || bin_chunk < 0) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  fnum::PWDev& D = plan->pw;
  if (fnum::pw_variant_of(D) == fnum::TC_VARIANT) {
    if (bin_chunk != 0 && bin_chunk != 16 && bin_chunk != 32) return FNUM_ERR_ARGUMENT;
    D.tc_tb = bin_chunk;
  } else {
    if (bin_chunk != 0 && bin_chunk != 128 && bin_chunk != 256) return FNUM_ERR_ARGUMENT;
    D.flush_chunks = bin_chunk == 128 ? 2 : 4;
  }
  D.blocks_per_sm = blocks_per_sm;
  plan->grid = std::min(fnum::pw_fused_grid(D, nullptr), plan->max_grid);
  return FNUM_OK;
}

struct fnum_batch {
  int device = 0;
  int n = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> done;   // per frame, recorded when the frame's image is complete
  // persistent tensor-core launches, one per window and pass width of the compounded tensor-core frames
  struct TcGroup {
    int window_id = 0, grid = 0;
    int nt = 3;                     // n-tiles per angle pass of the group's frames
    std::vector<int> frames;        // batch frame indices, largest first
    fnum::PWBatchDev dev{};
  };
  std::vector<TcGroup> groups;
  std::vector<void*> allocs;
  int persistent_frames = 0;
  ~fnum_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (start) cudaEventDestroy(start);
    for (cudaEvent_t ev : done)
      if (ev) cudaEventDestroy(ev);
    for (void* p : allocs) cudaFree(p);
  }
};

extern "C++" {
namespace {

// a frame that the persistent tensor-core launch can take: a compounded plane-wave plan
// whose kernel variant is the tensor-core one
bool tc_persistent(const fnum_plan* P) {
  return P->kind == 0 && P->n_out == 1 && !P->pw.m_sem && !(P->flags & FNUM_FLAG_PLAIN_KERNEL) &&
         fnum::pw_variant_of(P->pw) == fnum::TC_VARIANT && P->pw.tc_B;
}

template <typename T>
int batch_upload(fnum_batch* B, T** dst, const std::vector<T>& v) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(v.size(), 1) * sizeof(T));
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return cuda_status(e);
  }
  B->allocs.push_back(q);
  *dst = (T*)q;
  if (!v.empty()) FNUM_CUDA(cudaMemcpy(q, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return FNUM_OK;
}

// descriptor arrays, tile prefix sums, counter and segment scratch of one persistent group
int build_tc_group(fnum_batch* B, fnum_batch::TcGroup& G, fnum_plan* const* plans, void* const* d_images,
                   float* const* d_weights) {
  std::vector<fnum::PWDev> frames;
  std::vector<float2*> images;
  std::vector<float*> weights;
  std::vector<int> tile_start(1, 0);
  int max_ne = 1, seg_cap = 1;
  for (int f : G.frames) {
    const fnum::PWDev& D = plans[f]->pw;
    frames.push_back(D);
    images.push_back((float2*)d_images[f]);
    weights.push_back(d_weights ? d_weights[f] : nullptr);
    tile_start.push_back(tile_start.back() + fnum::pw_tc_tiles(D));
    max_ne = std::max(max_ne, D.ne);
    seg_cap = std::max(seg_cap, D.seg_cap);
  }
  int s;
  fnum::PWBatchDev& dev = G.dev;
  dev.n_frames = (int)G.frames.size();
  dev.max_ne = max_ne;
  dev.seg_cap = seg_cap;
  G.grid = fnum::pw_tc_batch_grid(max_ne, G.window_id, G.nt, nullptr);
  fnum::PWDev* d_frames = nullptr;
  float2** d_img = nullptr;
  float** d_w = nullptr;
  int* d_ts = nullptr;
  std::vector<unsigned long long> zero(1, 0);
  unsigned long long* d_counter = nullptr;
  if ((s = batch_upload(B, &d_frames, frames)) || (s = batch_upload(B, &d_img, images)) ||
      (s = batch_upload(B, &d_w, weights)) || (s = batch_upload(B, &d_ts, tile_start)) ||
      (s = batch_upload(B, &d_counter, zero)))
    return s;
  void* seg = nullptr;
  cudaError_t e = cudaMalloc(&seg, (size_t)G.grid * fnum::NTHREADS * seg_cap * fnum::PW_SEG_INT4 * sizeof(int4));
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return cuda_status(e);
  }
  B->allocs.push_back(seg);
  // the descriptors the kernel reads carry the batch's segment scratch
  for (auto& D : frames) {
    D.seg = (int4*)seg;
    D.seg_cap = seg_cap;
  }
  FNUM_CUDA(cudaMemcpy(d_frames, frames.data(), frames.size() * sizeof(fnum::PWDev), cudaMemcpyHostToDevice));
  dev.frames = d_frames;
  dev.images = d_img;
  dev.weights = d_w;
  dev.tile_start = d_ts;
  dev.counter = d_counter;
  dev.seg = (int4*)seg;
  return FNUM_OK;
}

}  // namespace
}  // extern "C++"

int fnum_batch_create(fnum_plan* const* plans, int n, const void* const* d_rf, const int* rf_is_double,
                      void* const* d_images, float* const* d_weights, float* const* d_weights_rx, int n_streams,
                      fnum_batch** batch) {
  if (!plans || n <= 0 || !d_rf || !d_images || !batch) return FNUM_ERR_ARGUMENT;
  *batch = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!plans[i] || !d_rf[i] || !d_images[i]) return FNUM_ERR_ARGUMENT;
    if (plans[i]->device != plans[0]->device) return FNUM_ERR_ARGUMENT;
    for (int j = 0; j < i; ++j)
      if (plans[j] == plans[i]) return FNUM_ERR_ARGUMENT;  // a plan's buffers serve one frame at a time
  }
  FNUM_CUDA(cudaSetDevice(plans[0]->device));
  const int k = std::max(1, std::min(n_streams, n));
  // longest frames first, each to the branch with the least work so far
  std::vector<int> order(n), branch(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return plans[a]->info.terms > plans[b]->info.terms; });
  fnum_batch* B = new (std::nothrow) fnum_batch;
  if (!B) return FNUM_ERR_ARGUMENT;
  B->device = plans[0]->device;
  B->n = n;
  B->done.assign(n, nullptr);
  std::vector<cudaStream_t> st(k, nullptr);
  std::vector<cudaEvent_t> fj(k, nullptr);  // fork (0) and joins (1..k-1)
  int s = FNUM_OK;
  bool capturing = false;
  cudaError_t e = cudaEventCreate(&B->start);
  for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreate(&B->done[i]);
  for (int i = 0; i < k && e == cudaSuccess; ++i) e = cudaStreamCreateWithFlags(&st[i], cudaStreamNonBlocking);
  for (int i = 0; i < k && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&fj[i], cudaEventDisableTiming);
  // compounded tensor-core frames go to persistent launches (one per window and pass width), the others
  // keep a launch per frame on the branches
  std::vector<char> persistent(n, 0);
  for (int f : order) {
    if (!tc_persistent(plans[f])) continue;
    persistent[f] = 1;
    const int w = plans[f]->pw.window_id, nt = plans[f]->pw.tc_nt == 4 ? 4 : 3;
    size_t gi = 0;
    while (gi < B->groups.size() && (B->groups[gi].window_id != w || B->groups[gi].nt != nt)) ++gi;
    if (gi == B->groups.size()) {
      B->groups.emplace_back();
      B->groups.back().window_id = w;
      B->groups.back().nt = nt;
    }
    B->groups[gi].frames.push_back(f);   // `order` is largest first
    ++B->persistent_frames;
  }
  for (auto& G : B->groups)
    if ((s = build_tc_group(B, G, plans, d_images, d_weights))) break;
  // the other frames: each to the least-loaded branch (not branch 0, which runs the
  // persistent launches, when there are other branches)
  {
    const int b0 = (k > 1 && B->persistent_frames > 0) ? 1 : 0;
    std::vector<double> load(k, 0.0);
    for (int f : order) {
      if (persistent[f]) continue;
      const int b = (int)(std::min_element(load.begin() + b0, load.end()) - load.begin());
      branch[f] = b;
      load[b] += (double)plans[f]->info.terms;
    }
  }
  std::vector<cudaEvent_t> prep(k, nullptr);   // the persistent frames' DFTs done, per branch
  for (int i = 0; i < k && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&prep[i], cudaEventDisableTiming);
  if (e == cudaSuccess && !s) e = cudaStreamBeginCapture(st[0], cudaStreamCaptureModeThreadLocal);
  capturing = (e == cudaSuccess && !s);
  if (e == cudaSuccess && !s) e = cudaEventRecordWithFlags(B->start, st[0], cudaEventRecordExternal);
  if (e == cudaSuccess && !s) e = cudaEventRecord(fj[0], st[0]);
  for (int i = 1; i < k && e == cudaSuccess && !s; ++i) e = cudaStreamWaitEvent(st[i], fj[0], 0);
  if (e != cudaSuccess && !s) s = cuda_status(e);
  // the persistent frames' band DFTs, spectra fragments and counters, spread over the
  // branches; then branch 0 waits for them all and runs the persistent launches
  if (B->persistent_frames > 0) {
    int rr = 0;
    for (int f : order) {
      if (s || !persistent[f]) continue;
      cudaStream_t q = st[rr++ % k];
      if ((s = plan_dft(plans[f], d_rf[f], rf_is_double ? rf_is_double[f] : 0, q))) break;
      e = cudaMemsetAsync(plans[f]->counters, 0, 5 * sizeof(unsigned long long), q);
      if (e == cudaSuccess) e = fnum::launch_pw_tc_prep(plans[f]->pw, q);
      if (e != cudaSuccess) s = cuda_status(e);
    }
    for (int i = 1; i < k && !s; ++i) {
      e = cudaEventRecord(prep[i], st[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st[0], prep[i], 0);
      if (e != cudaSuccess) s = cuda_status(e);
    }
    for (auto& G : B->groups) {
      if (s) break;
      e = fnum::launch_pw_tc_batch(G.dev, G.window_id, G.nt, G.grid, st[0]);
      for (size_t j = 0; j < G.frames.size() && e == cudaSuccess; ++j)
        e = cudaEventRecordWithFlags(B->done[G.frames[j]], st[0], cudaEventRecordExternal);
      if (e != cudaSuccess) s = cuda_status(e);
    }
  }
  for (int f : order) {
    if (s) break;
    if (persistent[f]) continue;
    cudaStream_t q = st[branch[f]];
    if ((s = plan_dft(plans[f], d_rf[f], rf_is_double ? rf_is_double[f] : 0, q))) break;
    if ((s = plan_beamform(plans[f], d_images[f], d_weights ? d_weights[f] : nullptr,
                           d_weights_rx ? d_weights_rx[f] : nullptr, q)))
      break;
    e = cudaEventRecordWithFlags(B->done[f], q, cudaEventRecordExternal);
    if (e != cudaSuccess) s = cuda_status(e);
  }
  for (int i = 1; i < k && !s; ++i) {
    e = cudaEventRecord(fj[i], st[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st[0], fj[i], 0);
    if (e != cudaSuccess) s = cuda_status(e);
  }
  if (capturing) {
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(st[0], &g);
    if (!s && e != cudaSuccess) s = cuda_status(e);
    if (s) {
      if (g) cudaGraphDestroy(g);
    } else {
      B->graph = g;
      e = cudaGraphInstantiate(&B->exec, g, 0);
      if (e != cudaSuccess) s = cuda_status(e);
    }
  }
  for (int i = 0; i < k; ++i) {
    if (fj[i]) cudaEventDestroy(fj[i]);
    if (prep[i]) cudaEventDestroy(prep[i]);
    if (st[i]) cudaStreamDestroy(st[i]);
  }
  (void)cudaGetLastError();
  if (s) {
    delete B;
    return s;
  }
  *batch = B;
  return FNUM_OK;
}

int fnum_batch_execute(fnum_batch* batch, void* stream) {
  if (!batch || !batch->exec) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(batch->device));
  FNUM_CUDA(cudaGraphLaunch(batch->exec, (cudaStream_t)stream));
  return FNUM_OK;
}

int fnum_batch_frame_times(const fnum_batch* batch, float* ms) {
  if (!batch || !ms) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(batch->device));
  for (int i = 0; i < batch->n; ++i) {
    cudaError_t e = cudaEventElapsedTime(&ms[i], batch->start, batch->done[i]);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      return cuda_status(e);
    }
  }
  return FNUM_OK;
}

int fnum_batch_info(const fnum_batch* batch, int* persistent_frames, int* persistent_launches) {
  if (!batch) return FNUM_ERR_ARGUMENT;
  if (persistent_frames) *persistent_frames = batch->persistent_frames;
  if (persistent_launches) *persistent_launches = (int)batch->groups.size();
  return FNUM_OK;
}

int fnum_batch_destroy(fnum_batch* batch) {
  if (!batch) return FNUM_OK;
  cudaSetDevice(batch->device);
  delete batch;
  return FNUM_OK;
}

// ---------------------------------------------------------------------------
// sound speed and sharpness-loss gradients (no counterpart in the reference)
// ---------------------------------------------------------------------------
int fnum_pw_plan_set_sound_speed(fnum_plan* plan, double c_0) {
  if (!plan || plan->kind != 0 || !(c_0 > 0.0) || !std::isfinite(c_0)) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  fnum::PWDev& D = plan->pw;
  const Band& b = plan->band;
  const double Ku = plan->fs / ((double)b.N * c_0);
  GeomTables g;
  build_geometry(plan->hx.data(), D.nx, plan->hz.data(), D.nz, D.ne, plan->width, plan->pitch, Ku, b.M, g);
  std::vector<dfl> ax, az;
  build_tx_tables(plan->hx.data(), D.nx, plan->hz.data(), D.nz, plan->hang.data(), D.na, Ku, b.M, plan->pitch,
                  plan->t0, b.N, ax, az);
  FNUM_CUDA(cudaMemcpy((void*)D.col_u, g.col_u.data(), g.col_u.size() * sizeof(dfl), cudaMemcpyHostToDevice));
  FNUM_CUDA(cudaMemcpy((void*)D.row_u2, g.row_u2.data(), g.row_u2.size() * sizeof(dfl), cudaMemcpyHostToDevice));
  FNUM_CUDA(cudaMemcpy((void*)D.el_u, g.el_u.data(), g.el_u.size() * sizeof(dfl), cudaMemcpyHostToDevice));
  FNUM_CUDA(cudaMemcpy((void*)D.tx_ax, ax.data(), ax.size() * sizeof(dfl), cudaMemcpyHostToDevice));
  FNUM_CUDA(cudaMemcpy((void*)D.tx_az, az.data(), az.size() * sizeof(dfl), cudaMemcpyHostToDevice));
  D.coef_f = (float)(2.0 * M_PI * plan->fs / ((double)b.N * c_0));
  plan->c = c_0;
  return FNUM_OK;
}

namespace fnum {

// gradient buffers of a compounded plane-wave plan, allocated on first use; the 1/W
// table of the frozen apertures is built once
int adjoint_buffers(fnum_plan* plan, cudaStream_t st) {
  const fnum::PWDev& D = plan->pw;
  const long long nvox = (long long)D.nx * D.nz;
  const size_t nspec = (size_t)D.ne * D.K * D.na;
  int s = FNUM_OK;
  if (!plan->adj_img) {
    if ((s = plan->alloc(&plan->adj_img, (size_t)nvox)) || (s = plan->alloc(&plan->adj_G, (size_t)nvox)) ||
        (s = plan->alloc(&plan->adj_invw, (size_t)nvox * D.K)) || (s = plan->alloc(&plan->adj_D, (size_t)nvox)) ||
        (s = plan->alloc(&plan->adj_gX, nspec)) || (s = plan->alloc(&plan->adj_sums, 4)) ||
        (s = plan->alloc(&plan->adj_acc, 2 * nspec)) || (s = plan->alloc(&plan->adj_gmax, 2)))
      return s;
  }
  // the adjoint's per-(voxel, element) receive table (16 bytes a pair) is optional: without
  // the memory the kernel forms the same values itself
  if (!plan->adj_rx_tried) {
    plan->adj_rx_tried = true;
    if (plan->alloc(&plan->adj_rx, (size_t)nvox * D.ne) == FNUM_OK) plan->pw.rx_tab = plan->adj_rx;
  }
  if (!plan->adj_invw_ready) {
    FNUM_CUDA(fnum::launch_pw_invw(D, plan->adj_invw, st));
    FNUM_CUDA(fnum::launch_absmax(plan->adj_invw, (size_t)nvox * D.K, plan->adj_gmax + 1, st));
    plan->adj_invw_ready = true;
  }
  return FNUM_OK;
}

// dL/dX* into gX and (if dloss_dc) dL/dc for the cotangent G = dL/dI*, on the plan's
// spectra.  dL/dc needs the derivative image adj_D of those spectra: have_D says that the
// caller has just computed it (launch_pw_tc_deriv), else it is computed here.
int adjoint_core(fnum_plan* plan, const float2* G, float2* gX, double* dloss_dc, bool have_D, cudaStream_t st) {
  fnum::PWDev& D = plan->pw;
  const long long nvox = (long long)D.nx * D.nz;
  if (dloss_dc) {
    if (!have_D) FNUM_CUDA(fnum::launch_pw_tc_deriv(D, plan->adj_img, plan->adj_D, st));
    FNUM_CUDA(fnum::launch_pw_dc_reduce(G, plan->adj_D, nvox, 4.0 * M_PI / plan->c, plan->adj_sums + 2, st));
  }
  if (gX) FNUM_CUDA(fnum::launch_pw_adjoint(D, G, plan->adj_invw, plan->adj_gmax, gX, plan->adj_acc, st));
  if (dloss_dc) {
    double g = 0.0;
    FNUM_CUDA(cudaMemcpyAsync(&g, plan->adj_sums + 2, sizeof(double), cudaMemcpyDeviceToHost, st));
    FNUM_CUDA(cudaStreamSynchronize(st));
    *dloss_dc = g;
  } else {
    FNUM_CUDA(cudaStreamSynchronize(st));
  }
  return FNUM_OK;
}

}  // namespace fnum

int fnum_plan_set_spectra(fnum_plan* plan, const void* d_spectra, void* stream) {
  if (!plan || !d_spectra) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  const size_t n = plan->kind == 0 ? (size_t)plan->pw.ne * plan->pw.K * plan->pw.na
                                   : (size_t)plan->sa.ne * plan->sa.ne * plan->sa.K;
  FNUM_CUDA(cudaMemcpyAsync(plan->X, d_spectra, n * sizeof(float2), cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return FNUM_OK;
}

int fnum_pw_adjoint(fnum_plan* plan, const void* d_cotangent, void* d_grad_spectra, double* dloss_dc, void* stream) {
  if (!plan || !d_cotangent || plan->kind != 0 || plan->n_out != 1 || plan->pw.m_sem) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  cudaStream_t st = (cudaStream_t)stream;
  int s;
  if ((s = fnum::adjoint_buffers(plan, st))) return s;
  float2* gX = d_grad_spectra ? (float2*)d_grad_spectra : plan->adj_gX;
  return fnum::adjoint_core(plan, (const float2*)d_cotangent, gX, dloss_dc, false, st);
}

int fnum_pw_sharpness_grad(fnum_plan* plan, const void* d_rf, int rf_is_double, double* loss, double* dloss_dc,
                           void* d_grad_spectra, void* stream) {
  if (!plan || !d_rf || plan->kind != 0 || plan->n_out != 1 || plan->pw.m_sem) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  cudaStream_t st = (cudaStream_t)stream;
  fnum::PWDev& D = plan->pw;
  const long long nvox = (long long)D.nx * D.nz;
  const size_t nspec = (size_t)D.ne * D.K * D.na;
  int s = FNUM_OK;
  if ((s = fnum::adjoint_buffers(plan, st))) return s;
  if ((s = plan_dft(plan, d_rf, rf_is_double, st))) return s;
  // the image and its derivative in c in one pass of the tensor-core kernel
  FNUM_CUDA(fnum::launch_pw_tc_deriv(D, plan->adj_img, plan->adj_D, st));
  FNUM_CUDA(fnum::launch_pw_sharp_sums(plan->adj_img, nvox, plan->adj_sums, st));
  double S[2] = {0.0, 0.0};
  FNUM_CUDA(cudaMemcpyAsync(S, plan->adj_sums, sizeof(S), cudaMemcpyDeviceToHost, st));
  FNUM_CUDA(cudaStreamSynchronize(st));
  float2* gX = d_grad_spectra ? (float2*)d_grad_spectra : plan->adj_gX;
  if (!(S[0] > 0.0)) {  // an all-zero image: the loss is 0 and flat
    FNUM_CUDA(cudaMemsetAsync(gX, 0, nspec * sizeof(float2), st));
    FNUM_CUDA(cudaStreamSynchronize(st));
    if (loss) *loss = 0.0;
    if (dloss_dc) *dloss_dc = 0.0;
    return FNUM_OK;
  }
  const double gs2 = 1.0 / (S[0] * S[0]), gs4 = S[1] / (S[0] * S[0] * S[0]);
  FNUM_CUDA(fnum::launch_pw_sharp_cotangent(plan->adj_img, nvox, (float)gs2, (float)gs4, plan->adj_G, st));
  if ((s = fnum::adjoint_core(plan, plan->adj_G, gX, dloss_dc, true, st))) return s;
  if (loss) *loss = -S[1] / (S[0] * S[0]);
  return FNUM_OK;
}

int fnum_plan_m_signal(const fnum_plan* plan, double* spectrum_re_im, int* has_signal) {
  if (!plan || !spectrum_re_im || plan->kind != 0 || !plan->pw.m_sem) return FNUM_ERR_ARGUMENT;
  FNUM_CUDA(cudaSetDevice(plan->device));
  const fnum::PWDev& D = plan->pw;
  std::vector<int> flag(D.nz);
  FNUM_CUDA(cudaMemcpy(flag.data(), D.m_sig_flag, D.nz * sizeof(int), cudaMemcpyDeviceToHost));
  int j = D.nz - 1;
  while (j >= 0 && !flag[j]) --j;
  if (has_signal) *has_signal = j >= 0;
  std::vector<float2> sp(D.K, make_float2(0.0f, 0.0f));
  if (j >= 0)
    FNUM_CUDA(cudaMemcpy(sp.data(), D.m_sig + (size_t)j * D.K, D.K * sizeof(float2), cudaMemcpyDeviceToHost));
  for (int k = 0; k < D.K; ++k) {
    spectrum_re_im[2 * k] = sp[k].x;
    spectrum_re_im[2 * k + 1] = sp[k].y;
  }
  return FNUM_OK;
}

}  // extern "C"
