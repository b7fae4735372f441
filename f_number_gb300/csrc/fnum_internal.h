// Internal plan layout shared by the host library (fnum_host.cpp) and the
// kernels (fnum_kernels.cu).  Not part of the public ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace fnum {

// double-float numbers are stored as float2 {hi, lo}, value = hi + lo
typedef float2 dfl;

// block shape of the fused kernels: TILE_X columns x TILE_Z rows of voxels,
// one voxel per thread, one column per warp
constexpr int TILE_X = 4;
constexpr int TILE_Z = 32;
constexpr int NTHREADS = TILE_X * TILE_Z;
// band bins per shared-memory spectrum chunk; flushes happen on chunk edges
constexpr int KCHUNK = 64;
// tensor-core plane-wave kernel: 4 warps of 16 voxels, TC_TILE_X columns x TILE_Z rows
constexpr int TC_TILE_X = 2;
constexpr int TC_NA = 12;   // angles per angle pass (3 mma n-tiles of 4 complex angles)
// A plane-wave plan's tensor-core kernel runs passes of 3 n-tiles (12 angles) or, when
// that takes fewer passes (13-16, 25-32, 37-64 angles, ...), of 4 (16 angles): each pass
// forms the same A operands, so fewer passes is less work.
inline int tc_ntiles_for(int na) { return ((na + 15) / 16 < (na + TC_NA - 1) / TC_NA) ? 4 : 3; }
constexpr int TC_EP = 16;   // elements per pass: TC_KS mma k-steps of 8 complex elements
constexpr int TC_KS = TC_EP / 8;
constexpr int TC_VARIANT = 9;

// one aperture segment of one voxel (bins k_start down to the next entry's
// k_start + 1 share the same apertures).  Plane wave: one int4
// {k_start, i_lb | (i_ub+1) << 16, 1/W, ratio of 1/W to the previous segment};
// SAFT: one int4 {k_start, tx code, rx code, 1/(W_tx W_rx)}.  Each list ends
// with a sentinel entry.  Kernels and the host's scratch allocation both size
// entries with these constants.
constexpr int PW_SEG_INT4 = 1;
constexpr int SA_SEG_INT4 = 1;

struct PWDev {
  int nx, nz, ne, na, K, k_lb, k_ub, N_dft;
  int window_id; float window_par;
  int norm;            // 1 = divide each bin by its apodization sum
  int seg_cap;         // segment entries per voxel
  int flush_chunks;    // flush Horner accumulators every flush_chunks * KCHUNK bins
  float scale;         // 2 / N_dft
  float t0N;           // index_t0 / N_dft, the part of tx_ax that does not scale with 1/c
  int variant;         // fused kernel variant, 0 = by angle count (launch_pw_fused)
  // launch shape picked by the autotuner (0 = default): resident blocks per SM, and the
  // bins between exact re-anchorings of the tensor-core kernel (32 or 16)
  int blocks_per_sm;
  int tc_tb;
  // per column [nx]
  const dfl* col_u;    // K_u x
  const dfl* col_p;    // M + x / pitch
  const dfl* col_m;    // x (m)
  const int* col_emid; // first element with centre >= x
  // per row [nz]
  const dfl* row_u2;   // (K_u z)^2
  const dfl* row_p;    // z / pitch
  // per element [ne]
  const dfl* el_u;     // K_u c_e
  const dfl* el_m;     // c_e (m)
  const dfl* el_lb;    // c_e - width/2 (m)
  const dfl* el_ub;    // c_e + width/2 (m)
  // per angle
  const dfl* tx_ax;    // [na][nx]  K_u e_x (x - x_ref) + t0 / N
  const dfl* tx_az;    // [na][nz]  K_u e_z z
  // per band bin [K]
  const dfl* g;        // 1 / (2 F); hi < 0 marks F <= FLT_EPSILON (full aperture)
  // band spectra [ne][K][x_na]; this launch uses angles x_a0 .. x_a0 + na - 1
  float2* X;
  int x_na, x_a0;
  // scratch: [grid][NTHREADS][seg_cap] int4
  int4* seg;
  // tensor-core variant: spectra as mma B fragments [angle pass][K][tc_S][3][32] (uint4),
  // and the largest |component| of the spectra (float bits) that sets their fp16 scale
  uint4* tc_B;
  unsigned* tc_max;
  int tc_S;            // element groups of 8 in tc_B (TC_KS - 1 zero groups of padding included)
  int tc_nt;           // mma n-tiles per angle pass of the tensor-core kernel (3 or 4; 0 reads as 3)
  unsigned long long* counters;   // [0] active terms, [1] zero-weight bins, [2] error bits,
                                  // [3] tile counter, [4] executed recurrence steps
  // the per-voxel FP32 kernel reads the reference's float geometry
  const float* px_f; const float* pz_f;
  const float* ctr_f; const float* lb_f; const float* ub_f;
  const float* F_f;    // [K]
  const float4* tx_f;  // [na] {e_x, e_z, x_ref, 0}
  float M_f, pitch_f, coef_f, add_f;
  // das_pw.m semantics (pw_m_kernel): double geometry, F before the depth cap
  int m_sem;            // 1 = das_pw.m semantics
  int m_norm;           // 0 off, 1 on, 2 windowed
  int m_nwin_id; float m_nwin_par;   // window of the windowed normalisation
  const double* m_px; const double* m_pz;
  const double* m_tx;   // [na][3] e_x, e_z, x_ref
  const double* m_F0;   // [K]
  double m_c, m_fs, m_t0, m_pitch, m_width, m_M;
  float2* m_sig;        // [nz][K] focused spectra of the last column (signal output)
  int* m_sig_flag;      // [nz] 1 where the voxel has an active bin
  // adjoint: {u_rx (double-float), e^{2 pi i u_rx}} per (voxel, element), voxel-major;
  // null when the table could not be allocated (the adjoint then forms them itself)
  float4* rx_tab;
};

struct SADev {
  int nx, nz, ne, K, k_lb, k_ub, N_dft;
  int wtx_id; float wtx_par; int wrx_id; float wrx_par;
  int norm_tx, norm_rx;   // divide by the tx / rx apodization sums
  int last_bin_only;      // reference: both normalisations off keep only bin k_ub
  int seg_cap;
  int flush_chunks;
  float scale;
  dfl t0N;                          // time offset index_t0 / N in cycles per bin
  const dfl* col_u; const dfl* col_p; const dfl* col_m; const int* col_emid;
  const dfl* row_u2; const dfl* row_p;
  const dfl* el_u; const dfl* el_m; const dfl* el_lb; const dfl* el_ub;
  const dfl* gtx; const dfl* grx;   // [K]
  float2* X;                        // [ntx][nrx][K]
  // transmit/receive symmetry (equal windows, F-numbers and normalisations): pairs
  // (t, r) and (r, t) share weight and phase, so Xs[t][r] = X[t][r] + X[r][t] for
  // t < r (Xs[t][t] = X[t][t]) and only r >= t is beamformed; nullptr = off
  float2* Xs;
  int4* seg;                        // [grid][NTHREADS][seg_cap]
  unsigned long long* counters;
  const float* px_f; const float* pz_f; const float* ctr_f; const float* lb_f; const float* ub_f;
  const float* Ftx_f; const float* Frx_f;
  float M_f, pitch_f, coef_f, add_f;
};

// One persistent launch of the tensor-core beamformer over the tiles of many
// compounded frames (fnum_batch_*): per-frame descriptors and outputs in device
// memory, the tiles numbered frame after frame (tile_start holds the prefix sums),
// one tile counter and one segment scratch for the launch.
struct PWBatchDev {
  const PWDev* frames;       // [n_frames]
  float2* const* images;     // [n_frames] image of each frame
  float* const* weights;     // [n_frames] weights of each frame (entries may be null)
  const int* tile_start;     // [n_frames + 1]
  int n_frames, max_ne, seg_cap;
  unsigned long long* counter;
  int4* seg;                 // [grid][NTHREADS][seg_cap]
};

// error bits in counters[2] (beamformers) and counters[5] (band DFT)
constexpr unsigned long long ERR_SEG_OVERFLOW = 1ull;
constexpr unsigned long long ERR_DFT_TIMEOUT = 2ull;   // a wait of the tensor-core DFT gave up
constexpr unsigned long long ERR_TC_TIMEOUT = 4ull;    // a wait of the tensor-core SAFT kernel gave up

// Band DFT on the tensor cores (fnum_dft_tc.cu): RF lines split into fp16 hi/lo
// planes a [2][nsig][Kp], twiddle planes b [2][Np][Kp], per-line scale; the TMA
// maps of the four planes are built once per plan.
struct DftTc {
  CUtensorMap tm[4];   // A hi, A lo, B hi, B lo (64-byte aligned)
  void* a;
  void* b;
  float* inv_scale;
  int nsig, nt, N, k_lb, K, Kp, Np;
};
// device bytes of a, b and inv_scale for nsig lines of nt samples and K bins
size_t dft_tc_bytes(int nsig, int nt, int K);
// binds the buffers (a: 2 nsig Kp halves, b: 2 Np Kp halves, inv_scale: nsig floats),
// builds the TMA maps and fills b from the twiddle table on stream s
cudaError_t dft_tc_setup(DftTc& d, int nsig, int nt, int N, int k_lb, int K, const float2* tw, void* a, void* b,
                         float* inv_scale, cudaStream_t s);
// rf [nsig][nt] (float or double) -> X[(sig / lo_n) s_hi + (sig % lo_n) s_lo + k' s_k];
// ERR_DFT_TIMEOUT is or-ed into *err if a wait gave up
cudaError_t dft_tc_run(const DftTc& d, const void* rf, int is_double, float2* X, int lo_n, long long s_hi,
                       long long s_lo, long long s_k, unsigned long long* err, cudaStream_t s);

// Synthetic-aperture beamformer on the tensor cores (fnum_sa_tc.cu): the spectra as
// fp16 hi/lo planes [bin][2 nep][2 nep] in real form, their TMA maps, the scale word
// and the time-offset phasors e^{2 pi i k t0 / N} of the band.
struct SaTc {
  CUtensorMap tm[2];   // hi, lo (64-byte aligned)
  void* planes;
  unsigned* maxbits;
  const float2* rot;
  int nep;             // elements rounded up to a multiple of 4
};
bool sa_tc_supported(const SADev& d);          // up to 128 elements, accumulating normalisations
size_t sa_tc_bytes(int ne, int K);             // bytes of the planes
cudaError_t sa_tc_setup(SaTc& t, const SADev& d, void* planes, unsigned* maxbits, const float2* rot);
int sa_tc_grid(const SADev& d);                // one block per SM (at most one per tile)
cudaError_t launch_sa_tc(const SADev& d, const SaTc& t, int grid, float2* image, float* wtx, float* wrx,
                         cudaStream_t s);

// --- launchers (fnum_kernels.cu) -------------------------------------------
cudaError_t launch_twiddles(float2* tw, int N, cudaStream_t s);
// rf [nsig][nt] (float or double) -> X[e][k][a] (pw: sig = a*ne + e) or X[sig][k] (sa)
cudaError_t launch_dft_pw(const void* rf, int is_double, int na, int ne, int nt, const float2* tw, int N,
                          int k_lb, int K, float2* X, cudaStream_t s);
cudaError_t launch_dft_sa(const void* rf, int is_double, int nsig, int nt, const float2* tw, int N, int k_lb,
                          int K, float2* X, cudaStream_t s);
cudaError_t launch_split_complex(const float2* in, size_t n, float* re, float* im, cudaStream_t s);
int pw_fused_grid(const PWDev& d, int* blocks_per_sm);   // grid of d's variant, all blocks resident
int pw_fused_max_grid(const PWDev& d);                     // largest of those over the variants
int pw_variant_count();
int pw_variant_of(const PWDev& d);
int sa_fused_grid(const SADev& d, int* blocks_per_sm);
cudaError_t launch_pw_fused(const PWDev& d, int grid, float2* image, float* weights, cudaStream_t s);
// the compounded image and, in dimage, Draw with dI/dc = -(2 pi i / c) Draw (tensor cores;
// prepares the fragments itself)
cudaError_t launch_pw_tc_deriv(const PWDev& d, float2* image, float2* dimage, cudaStream_t s);
// the tensor-core variant's spectra scale and B fragments for frame d (before a batch launch),
// laid out for passes of nt n-tiles (0: the plan's own, d.tc_nt)
cudaError_t launch_pw_tc_prep(const PWDev& d, cudaStream_t s, int nt = 0);
// tiles of a frame for the tensor-core kernel; grid of the batch kernel with all blocks resident
int pw_tc_tiles(const PWDev& d);
// nt: the n-tiles per angle pass of every frame of the launch (frames are grouped by it)
int pw_tc_batch_grid(int max_ne, int window_id, int nt, int* blocks_per_sm);
cudaError_t launch_pw_tc_batch(const PWBatchDev& B, int window_id, int nt, int grid, cudaStream_t s);
cudaError_t launch_pw_plain(const PWDev& d, float2* image, float* weights, cudaStream_t s);
constexpr int M_MAXE = 256;   // elements supported by the das_pw.m-semantics kernel
cudaError_t launch_pw_m(const PWDev& d, int compound, float2* image, float* weights, cudaStream_t s);
cudaError_t launch_sa_fused(const SADev& d, int grid, float2* image, float* wtx, float* wrx, cudaStream_t s);
cudaError_t launch_sa_plain(const SADev& d, float2* image, float* wtx, float* wrx, cudaStream_t s);
// sharpness-loss gradients of a compounded plane-wave plan (fnum_pw_sharpness_grad)
cudaError_t launch_pw_invw(const PWDev& d, float* invw, cudaStream_t s);
cudaError_t launch_pw_sharp_sums(const float2* img, long long n, double* sums, cudaStream_t s);
// G = dL/dI* of the sharpness loss from the image and its sums (gs2 = 1/S2^2, gs4 = S4/S2^3)
cudaError_t launch_pw_sharp_cotangent(const float2* img, long long n, float gs2, float gs4, float2* G, cudaStream_t s);
// adjoint of the compounded beamformer for a cotangent G = dL/dI* [nx][nz] on the tensor
// cores: gX = dL/dX*; acc: 2 doubles per spectrum entry
// gmax: two device words, [1] = max 1/W (launch_absmax over the 1/W table, once), [0] set here
cudaError_t launch_pw_adjoint(const PWDev& d, const float2* cot, const float* invw, unsigned* gmax, float2* gX,
                              double* acc, cudaStream_t s);
// float bits of max |x_i| of n floats into *out
cudaError_t launch_absmax(const float* x, size_t n, unsigned* out, cudaStream_t s);
// dL/dc = coef sum_v Im(conj(G_v) D_v) into *out (FP64)
cudaError_t launch_pw_dc_reduce(const float2* G, const float2* D, long long n, double coef, double* out,
                               cudaStream_t s);

}  // namespace fnum
