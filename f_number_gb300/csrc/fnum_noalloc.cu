// fnum_das_pw_noalloc: the plane-wave beamformer for callers that cannot
// allocate device memory.
//
// Some hosts must not call cudaMalloc while they run: real-time acquisition
// loops that may not block on the allocator, hosts that own a fixed device
// memory pool and forbid other allocations, or plug-ins loaded into a process
// whose device memory belongs to someone else.  For them this entry point
// runs the same band DFT and fused beamformer kernels as the plan path, with
// every piece of working memory (band and geometry tables, twiddles, band
// spectra, counters and the per-voxel aperture segments) carved out of one
// file-scope device array of FNUM_NOALLOC_SCRATCH_BYTES.  The caller passes
// the RF input and the image / weights outputs, already on the device.
//
// The array is created when the library's device code is loaded and is held
// by every GPU that loads the library until the process exits.  All calls
// share it and it keeps whatever the last call left there; everything that
// must start at zero is cleared on every call.  Calls whose GPU work overlaps
// (different streams, different host threads) race on the array.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/fnum.h"
#include "fnum_internal.h"
#include "fnum_host_tables.h"

namespace {

using fnum::dfl;

constexpr size_t kScratchBytes = (size_t)FNUM_NOALLOC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device: taken once per
// device, with that device current.  In host code the symbol itself is only a
// host-side stand-in; the kernels must be given this address.  The address is
// kept for the life of the process, so a host must not reset the device
// (cudaDeviceReset, MATLAB's reset(gpuDevice)) between calls: a reset reloads
// the library's device code and may move the array.
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return FNUM_ERR_INVALID_DEVICE;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      (void)cudaGetLastError();
      return FNUM_ERR_CUDA;
    }
    g_scratch_ptr[device] = p;
  }
  *out = (unsigned char*)g_scratch_ptr[device];
  return FNUM_OK;
}

// bump allocator over the scratch array (256-byte aligned pieces)
struct Carve {
  unsigned char* base;
  size_t used = 0;
  template <typename T>
  T* take(size_t count) {
    T* p = (T*)(base + used);
    used += (count * sizeof(T) + 255) & ~(size_t)255;
    return p;
  }
};

}  // namespace

extern "C" int fnum_das_pw_noalloc(const fnum_pw_desc* desc, const double* steering_angles, int n_angles,
                                   const float* d_rf, int flags, void* d_image, float* d_weights, void* stream) {
  if (!desc || !d_rf || !d_image) return FNUM_ERR_ARGUMENT;
  if (flags & ~FNUM_FLAG_COMPOUND) return FNUM_ERR_ARGUMENT;  // fused kernel, reference semantics only
  const cudaStream_t st = (cudaStream_t)stream;
  // the plan path's checks, in the gateway's order and with its identifiers
  int s = fnum::check_pw(desc, steering_angles, n_angles);
  if (s != FNUM_OK) return s;
  if (cudaSetDevice(desc->device) != cudaSuccess) {
    (void)cudaGetLastError();
    return FNUM_ERR_CUDA;
  }
  const int nx = desc->n_x, nz = desc->n_z, ne = desc->n_elements, na = n_angles, nt = desc->n_samples;
  const double fs = desc->f_s, pitch = desc->element_pitch, width = desc->element_width, c = desc->c_0;
  const int wid = desc->window.id;

  // band, F table and the kernels' tables: the plan path's definitions
  fnum::Band b;
  if ((s = fnum::compute_band(desc->positions_z, nz, nt, ne, fs, width, pitch, c, desc->f_bounds, desc->index_t0,
                              &b)) != FNUM_OK)
    return s;
  const int N = b.N, k_lb = b.k_lb, k_ub = b.k_ub, K = b.K;
  std::vector<double> F;
  if ((s = fnum::band_f_table(&desc->f_number, desc->f_number_values, desc->n_f_number_values, b, pitch, fs, c,
                              FNUM_ERR_F_NUMBER, F)) != FNUM_OK)
    return s;
  const bool mono = fnum::f_monotone(F);
  const double Ku = fs / ((double)N * c);
  fnum::GeomTables gt;
  fnum::build_geometry(desc->positions_x, nx, desc->positions_z, nz, ne, width, pitch, Ku, b.M, gt);
  std::vector<dfl> ax, az, g;
  fnum::build_tx_tables(desc->positions_x, nx, desc->positions_z, nz, steering_angles, na, Ku, b.M, pitch,
                        desc->index_t0, N, ax, az);
  fnum::g_table(F, g);
  const std::vector<dfl>&col_u = gt.col_u, &col_p = gt.col_p, &col_m = gt.col_m, &row_u2 = gt.row_u2,
                  &row_p = gt.row_p, &el_u = gt.el_u, &el_m = gt.el_m, &el_lb = gt.el_lb, &el_ub = gt.el_ub;
  const std::vector<int>& emid = gt.col_emid;

  // carve the scratch array
  unsigned char* base = nullptr;
  if ((s = scratch_address(desc->device, &base)) != FNUM_OK) return s;
  Carve cv{base};
  fnum::PWDev D;
  memset(&D, 0, sizeof(D));
  D.nx = nx; D.nz = nz; D.ne = ne; D.na = na; D.K = K; D.k_lb = k_lb; D.k_ub = k_ub; D.N_dft = N;
  D.window_id = wid; D.window_par = (float)desc->window.parameter;
  D.norm = desc->normalization != FNUM_NORMALIZATION_OFF;
  D.seg_cap = (mono ? std::min(K, 2 * ne + 16) : K) + 1;  // + the sentinel entry, as the plan path
  D.flush_chunks = 4;
  D.scale = (float)(2.0 / N);
  D.pitch_f = (float)pitch;  // element spacing of the closed-form aperture sums
  D.x_na = na;
  D.x_a0 = 0;
  unsigned long long* counters = cv.take<unsigned long long>(8);
  float2* tw = cv.take<float2>(N);
  dfl* p_col_u = cv.take<dfl>(nx); dfl* p_col_p = cv.take<dfl>(nx); dfl* p_col_m = cv.take<dfl>(nx);
  int* p_emid = cv.take<int>(nx);
  dfl* p_row_u2 = cv.take<dfl>(nz); dfl* p_row_p = cv.take<dfl>(nz);
  dfl* p_el_u = cv.take<dfl>(ne); dfl* p_el_m = cv.take<dfl>(ne); dfl* p_el_lb = cv.take<dfl>(ne);
  dfl* p_el_ub = cv.take<dfl>(ne);
  dfl* p_ax = cv.take<dfl>((size_t)na * nx); dfl* p_az = cv.take<dfl>((size_t)na * nz);
  dfl* p_g = cv.take<dfl>(K);
  float2* X = cv.take<float2>((size_t)ne * K * na);
  const size_t seg_per_cta = (size_t)fnum::NTHREADS * D.seg_cap * fnum::PW_SEG_INT4 * sizeof(int4);
  if (cv.used + seg_per_cta > kScratchBytes) return FNUM_ERR_NOALLOC_TOO_LARGE;
  int4* seg = cv.take<int4>(0);
  D.col_u = p_col_u; D.col_p = p_col_p; D.col_m = p_col_m; D.col_emid = p_emid;
  D.row_u2 = p_row_u2; D.row_p = p_row_p;
  D.el_u = p_el_u; D.el_m = p_el_m; D.el_lb = p_el_lb; D.el_ub = p_el_ub;
  D.tx_ax = p_ax; D.tx_az = p_az; D.g = p_g;
  D.X = X;
  D.seg = seg;
  D.counters = counters;
  int bps = 0;
  int grid = fnum::pw_fused_grid(D, &bps);
  const int fit = (int)((kScratchBytes - cv.used) / seg_per_cta);
  if (grid > fit) grid = fit;

  // stage the tables (pageable copies: the host vectors may go once the calls return)
  cudaError_t e = cudaSuccess;
#define FNUM_PUT(dst, v) \
  if (e == cudaSuccess) e = cudaMemcpyAsync((void*)(dst), (v).data(), (v).size() * sizeof((v)[0]), cudaMemcpyHostToDevice, st)
  FNUM_PUT(p_col_u, col_u); FNUM_PUT(p_col_p, col_p); FNUM_PUT(p_col_m, col_m); FNUM_PUT(p_emid, emid);
  FNUM_PUT(p_row_u2, row_u2); FNUM_PUT(p_row_p, row_p);
  FNUM_PUT(p_el_u, el_u); FNUM_PUT(p_el_m, el_m); FNUM_PUT(p_el_lb, el_lb); FNUM_PUT(p_el_ub, el_ub);
  FNUM_PUT(p_ax, ax); FNUM_PUT(p_az, az); FNUM_PUT(p_g, g);
#undef FNUM_PUT
  // counters (statistics, error bits, the tile counter) start at zero on every call
  if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 8 * sizeof(unsigned long long), st);
  if (e == cudaSuccess) e = fnum::launch_twiddles(tw, N, st);
  if (e == cudaSuccess) e = fnum::launch_dft_pw(d_rf, 0, na, ne, nt, tw, N, k_lb, K, X, st);
  if (e == cudaSuccess) {
    if (flags & FNUM_FLAG_COMPOUND) {
      e = fnum::launch_pw_fused(D, grid, (float2*)d_image, d_weights, st);
    } else {
      for (int a = 0; a < na && e == cudaSuccess; ++a) {
        fnum::PWDev Da = D;
        Da.na = 1;
        Da.x_a0 = a;
        Da.tx_ax = D.tx_ax + (size_t)a * nx;
        Da.tx_az = D.tx_az + (size_t)a * nz;
        e = fnum::launch_pw_fused(Da, grid, (float2*)d_image + (size_t)a * nx * nz, a == 0 ? d_weights : nullptr,
                                  st);
      }
    }
  }
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? FNUM_ERR_OUT_OF_MEMORY : FNUM_ERR_CUDA;
  }
  return FNUM_OK;
}
