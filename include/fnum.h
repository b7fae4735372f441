/*
 * fnum.h -- C ABI of the GB300 Fourier-domain delay-and-sum beamformer.
 *
 * This is the boundary a MATLAB MEX gateway (or any other host) binds to in
 * place of the reference's CUDA MEX files.  Every entry point takes plain
 * pointers and sizes; no C++ or torch types appear here.
 *
 * Reference interfaces replaced (f_number project):
 *   fnum_das_pw   <- cuda.gpu_bf_das_pw_rf   (+cuda/gpu_bf_das_pw_rf.cu:110, called from das_pw.m:298)
 *   fnum_das_sa   <- cuda.gpu_bf_saft_rf     (+cuda/gpu_bf_saft_rf.cu:107, called from das_sa.m:285)
 *   fnum_band     <- DFT order / band logic  (+cuda/gpu_bf_das_pw_rf.cu:522-556)
 *   fnum_f_number_values <- f_numbers.f_number.compute_values (+f_numbers/f_number.m:50-114),
 *                     which the MEX reaches through mexCallMATLAB
 *                     (+cuda/gpu_bf_helper_functions.cu:35-51)
 *   fnum_window_value    <- windows (+cuda/gpu_bf_windows.cu:15-103)
 *   fnum_status_id       <- mexErrMsgIdAndTxt identifiers of both gateways
 *
 * Conventions (identical to the MEX gateways):
 *   positions_x [n_x], positions_z [n_z]           metres, double
 *   data_rf     PW : [n_elements][n_samples]        (MATLAB data_RF(t, e), time fastest)
 *               SA : [n_tx][n_rx][n_samples]        (MATLAB data_RF(t, rx, tx))
 *   images      [n_x][n_z]  (MATLAB N_z x N_x column-major), scaled by 2/N_dft,
 *               real and imaginary parts in separate planes (mxCOMPLEX single)
 *   weights     [n_x][n_z]  apodization sum of the highest band bin
 * Errors are returned as status codes; nothing exits, prints or resets the
 * device.  fnum_status_id() gives the reference's error identifier.
 */
#ifndef FNUM_H
#define FNUM_H

#ifdef __cplusplus
extern "C" {
#endif

#define FNUM_ABI_VERSION 4

typedef enum fnum_status {
  FNUM_OK = 0,
  FNUM_ERR_NO_DEVICE = 1,          /* gpu_bf_das_pw_rf:NoCUDADevices */
  FNUM_ERR_INVALID_DEVICE = 2,     /* :InvalidCUDADevice */
  FNUM_ERR_LATERAL_POSITIONS = 3,  /* :InvalidLateralPositions */
  FNUM_ERR_AXIAL_POSITIONS = 4,    /* :InvalidAxialPositions */
  FNUM_ERR_RF_DATA = 5,            /* :InvalidRFData */
  FNUM_ERR_SAMPLING_RATE = 6,      /* :InvalidSamplingRate */
  FNUM_ERR_STEERING_ANGLE = 7,     /* :InvalidSteeringAngle */
  FNUM_ERR_ELEMENT_WIDTH = 8,      /* :InvalidElementWidth */
  FNUM_ERR_ELEMENT_PITCH = 9,      /* :InvalidElementPitch */
  FNUM_ERR_SOUND_SPEED = 10,       /* :InvalidSoundSpeed */
  FNUM_ERR_FREQUENCY_BOUND = 11,   /* :InvalidFrequencyBound  (bounds themselves) */
  FNUM_ERR_FREQUENCY_BOUNDS = 12,  /* :InvalidFrequencyBounds (resulting bin indices) */
  FNUM_ERR_TIME_SHIFT = 13,        /* :InvalidTimeShift */
  FNUM_ERR_WINDOW = 14,            /* :InvalidWindow */
  FNUM_ERR_F_NUMBER = 15,          /* :InvalidFNumber */
  FNUM_ERR_NORMALIZATION = 16,     /* :InvalidNormalization */
  FNUM_ERR_VERBOSITY = 17,         /* :InvalidVerbosityLevel */
  FNUM_ERR_ARGUMENT = 18,          /* null pointer / size out of range */
  FNUM_ERR_CUDA = 19,              /* gpu_bf_error_handling:CUDAError */
  FNUM_ERR_OUT_OF_MEMORY = 20,     /* gpu_bf_error_handling:CUDAError (allocation) */
  FNUM_ERR_INTERNAL = 21,          /* device-side consistency check failed */
  FNUM_ERR_TX_F_NUMBER = 22,       /* gpu_bf_saft_rf:InvalidTXFNumber */
  FNUM_ERR_RX_F_NUMBER = 23,       /* gpu_bf_saft_rf:InvalidRXFNumber */
  FNUM_ERR_NOALLOC_TOO_LARGE = 24, /* fnum_das_pw_noalloc: problem exceeds FNUM_NOALLOC_SCRATCH_BYTES */
  FNUM_ERR_M_ELEMENTS = 25         /* FNUM_FLAG_M_SEMANTICS: more than 256 elements */
} fnum_status;

/* window ids follow the MEX mapping (+cuda/gpu_bf_helper_functions.cu:56-97) */
typedef enum fnum_window_id {
  FNUM_WINDOW_BOXCAR = 0,
  FNUM_WINDOW_HANN = 1,
  FNUM_WINDOW_TUKEY = 2,           /* parameter = fraction_cosine in (0, 1) */
  FNUM_WINDOW_TRIANGULAR = 4
} fnum_window_id;

typedef struct fnum_window {
  int id;
  double parameter;
} fnum_window;

typedef enum fnum_normalization {
  FNUM_NORMALIZATION_OFF = 0,      /* normalizations.off */
  FNUM_NORMALIZATION_ON = 1,       /* normalizations.on */
  FNUM_NORMALIZATION_WINDOWED = 2  /* normalizations.windowed: the MEX treats it as "on"
                                      (+cuda/gpu_bf_das_pw_rf.cu:421-427) */
} fnum_normalization;

/* F-number classes (+f_numbers/**).  p[] holds the constructor arguments. */
typedef enum fnum_f_number_kind {
  FNUM_F_DEFAULT = 0,              /* the MEX default angle_lb(70, 1.5, 10) */
  FNUM_F_CONSTANT = 1,             /* p[0] = value */
  FNUM_F_ANGLE_LB = 2,             /* grating.angle_lb: p[0] angle_lb_deg, p[1] F_number_ub, p[2] distance_deg */
  FNUM_F_DISTANCE_CONSTANT = 3,    /* distance.constant: p[0] distance_deg, p[1] F_number_ub (inf allowed) */
  FNUM_F_DISTANCE_NONE = 4,        /* distance.none */
  FNUM_F_DIRECTIVITY = 5,          /* directivity: p[0] width_over_pitch, p[1] attenuation_dB, obliquity */
  FNUM_F_SZABO = 6                 /* directivity.szabo: p[0] width_over_pitch */
} fnum_f_number_kind;

typedef enum fnum_obliquity { FNUM_OBLIQUITY_RIGID = 0, FNUM_OBLIQUITY_SOFT = 1 } fnum_obliquity;

typedef struct fnum_f_number {
  int kind;
  int obliquity;
  double p[3];
} fnum_f_number;

/* flags for fnum_das_pw / fnum_das_sa / plans */
#define FNUM_FLAG_COMPOUND        0x1  /* PW: sum the images of all angles into one image */
#define FNUM_FLAG_PLAIN_KERNEL    0x2  /* use the per-voxel FP32 kernel (reference arithmetic) */
#define FNUM_FLAG_SAFT_INTENDED   0x4  /* SA: divide by whichever sums are on, always accumulate */
/* PW: the semantics of the reference's CPU path (das_pw.m:310-481) instead of
   the MEX's: N_dft padded with positions_z[0]; F capped at sqrt(f z / (2.88 c))
   per bin and depth; boxcar on the ideal half-width; other windows over all
   elements without a cut-off; normalizations.windowed applied with
   normalization_window; image not scaled by 2/N_dft (spectra doubled).  Up to
   256 elements.  Weights outputs are written as 0. */
#define FNUM_FLAG_M_SEMANTICS     0x8

/* --- information ------------------------------------------------------ */
int fnum_abi_version(void);
const char* fnum_status_string(int status);
/* reference error identifier, e.g. "gpu_bf_das_pw_rf:InvalidFrequencyBounds";
   saft != 0 selects the gpu_bf_saft_rf prefix */
const char* fnum_status_id(int status, int saft);
int fnum_device_count(void);

/* --- band and parameter objects (host only, no GPU needed) -------------- */
/* DFT order and band bins exactly as +cuda/gpu_bf_das_pw_rf.cu:522-556.
   f_bounds may be NULL (default [DBL_MIN, f_s/2]). */
int fnum_band(const double* positions_z, int n_z, int n_samples, int n_elements, double f_s,
              double element_width, double element_pitch, double c_0, const double* f_bounds,
              double index_t0, int* N_dft, int* k_lb, int* k_ub);

/* F per normalised element pitch p/lambda (f_numbers.f_number.compute_values) */
int fnum_f_number_values(const fnum_f_number* f_number, const double* pitch_over_lambda, int n,
                         double* values);

/* window value at l relative to half-width L (0 where |l| >= L) */
double fnum_window_value(fnum_window window, double l, double L);

/* --- plane wave (das_pw) ------------------------------------------------ */
typedef struct fnum_pw_desc {
  const double* positions_x; int n_x;
  const double* positions_z; int n_z;
  int n_samples; int n_elements;
  double f_s;
  double element_width; double element_pitch;
  double c_0;
  const double* f_bounds;          /* [2] or NULL */
  double index_t0;
  fnum_window window;
  fnum_f_number f_number;
  const double* f_number_values;   /* optional: F per band bin (overrides f_number) */
  int n_f_number_values;
  int normalization;               /* fnum_normalization */
  int device;
  fnum_window normalization_window; /* frequency window of normalizations.windowed (FNUM_FLAG_M_SEMANTICS) */
} fnum_pw_desc;

/* One call = the reference's gpu_bf_das_pw_rf for each steering angle
   (n_angles >= 1; data_rf holds n_angles blocks of [n_elements][n_samples]).
   Outputs: image_re/image_im [n_out][n_x][n_z] with n_out = 1 under
   FNUM_FLAG_COMPOUND, else n_angles; weights [n_x][n_z] (may be NULL). */
int fnum_das_pw(const fnum_pw_desc* desc, const double* steering_angles, int n_angles,
                const double* data_rf, int flags, float* image_re, float* image_im, float* weights);

/* Sharpness-loss gradients from host buffers (no counterpart in the reference,
   which has no derivatives): the compounded image of all n_angles (data_rf as
   for fnum_das_pw), its loss L = -sum|I|^4 / (sum|I|^2)^2, dL/dc at desc->c_0
   (band, F table and apertures held at that speed) and, if grad_re / grad_im
   are not NULL, the Wirtinger gradient dL/dX* of the band spectra as separate
   real / imaginary planes [n_angles][n_elements][n_bins] (bins fastest:
   MATLAB's N_bins x N_el x N_angles).  Shares fnum_das_pw's plan cache.  The
   MATLAB binding is f_number_gb300/mex/gpu_bf_das_pw_sharpness_grad.cpp. */
int fnum_das_pw_sharpness_grad(const fnum_pw_desc* desc, const double* steering_angles, int n_angles,
                               const double* data_rf, double* loss, double* dloss_dc, float* grad_re,
                               float* grad_im);

/* --- synthetic aperture (das_sa) ---------------------------------------- */
typedef struct fnum_sa_desc {
  const double* positions_x; int n_x;
  const double* positions_z; int n_z;
  int n_samples; int n_elements;   /* n_tx == n_rx == n_elements */
  double f_s;
  double element_width; double element_pitch;
  double c_0;
  const double* f_bounds;
  double index_t0;
  fnum_window window_tx; fnum_window window_rx;
  fnum_f_number f_number_tx; fnum_f_number f_number_rx;
  const double* f_number_tx_values; const double* f_number_rx_values; int n_f_number_values;
  int normalization_tx; int normalization_rx;
  int device;
} fnum_sa_desc;

int fnum_das_sa(const fnum_sa_desc* desc, const double* data_rf, int flags, float* image_re,
                float* image_im, float* weights_tx, float* weights_rx);

/* --- device-resident plans (stream-ordered; inputs and outputs in HBM) --- */
typedef struct fnum_plan fnum_plan;

typedef struct fnum_plan_info {
  int N_dft; int k_lb; int k_ub; int n_bins;
  int n_x; int n_z; int n_elements; int n_angles; int n_samples;
  int f_monotone;                  /* F non-decreasing over the band */
  long long terms;                 /* voxel x element(-pair) x bin x angle terms of one execute */
  long long active_terms;          /* terms with nonzero apodization (counted on device, last execute) */
  long long zero_weight_bins;      /* (voxel, bin) pairs with zero apodization sum, last execute */
  long long scratch_bytes;         /* device scratch the plan owns */
  double scale;                    /* 2 / N_dft */
  long long executed_terms;        /* recurrence steps the fused kernel ran (>= active_terms), last execute */
  int kernel_variant;              /* PW: fused kernel variant (1..9, see fnum_plan_autotune); SA: 1 recurrence
                                      kernels, 2 tensor cores; 0 for FNUM_FLAG_PLAIN_KERNEL plans */
  int grid;                        /* blocks of the fused kernel's launch */
  int blocks_per_sm;               /* PW: resident blocks per SM of that launch (launch shape) */
  int bin_chunk;                   /* PW: bins between exact phase re-anchorings (tensor cores 32 or 16;
                                      FP32 kernels 256 or 128) */
} fnum_plan_info;

int fnum_pw_plan_create(const fnum_pw_desc* desc, const double* steering_angles, int n_angles,
                        int flags, fnum_plan** plan);
int fnum_sa_plan_create(const fnum_sa_desc* desc, int flags, fnum_plan** plan);
/* d_rf: device pointer, float (rf_is_double = 0) or double; layout as data_rf.
   d_image: float2 [n_out][n_x][n_z] (interleaved, scaled); d_weights / d_weights_rx
   may be NULL.  stream: a cudaStream_t (NULL = legacy default stream). */
int fnum_plan_execute(fnum_plan* plan, const void* d_rf, int rf_is_double, void* d_image,
                      float* d_weights, float* d_weights_rx, void* stream);
/* the band stage alone: d_rf -> d_spectra (plan-internal), for timing */
int fnum_plan_execute_dft(fnum_plan* plan, const void* d_rf, int rf_is_double, void* stream);
/* copies the band spectra of the last execute (or execute_dft) to d_spectra
   (device float2; plane wave [n_elements][n_bins][n_angles], synthetic aperture
   [n_tx][n_rx][n_bins]), stream-ordered.  No counterpart in the reference,
   whose spectra live only inside a gateway call. */
int fnum_plan_spectra(const fnum_plan* plan, void* d_spectra, void* stream);
/* the beamforming stage alone on the spectra of the last fnum_plan_execute_dft */
int fnum_plan_execute_beamform(fnum_plan* plan, void* d_image, float* d_weights, float* d_weights_rx,
                               void* stream);
int fnum_plan_info_get(const fnum_plan* plan, fnum_plan_info* info);

/* Plans of the two host-buffer entry points above are cached by the VALUES of
   their arguments (never the addresses of the caller's arrays), up to 4 per
   entry point, least recently used first out.  No counterpart in the reference
   (which allocates and frees per call).  plans_created counts the plans an
   entry point has built (saft = 0: fnum_das_pw, 1: fnum_das_sa); plans_cached
   is the number it holds now.  Either pointer may be NULL. */
int fnum_host_cache_info(int saft, long long* plans_created, int* plans_cached);

/* --- plane wave without device allocation ------------------------------- */
/* No counterpart in the reference (whose gateways allocate and free device
   memory on every call).  For callers that may not call cudaMalloc -- a
   real-time acquisition loop that must not block on the allocator, a host
   that owns a fixed device memory pool, a plug-in inside a process whose
   device memory belongs to someone else.  It runs the same band DFT and fused
   beamformer as fnum_plan_execute, but every piece of working memory (tables,
   twiddles, band spectra, counters, aperture segments) lives in one static
   device array of FNUM_NOALLOC_SCRATCH_BYTES that the library holds on every
   GPU that loads it, until the process exits.  Nothing is allocated on the
   device (host-side tables are built in ordinary host memory).
     d_rf      device float RF, [n_angles][n_elements][n_samples]
     d_image   device float2 image [n_out][n_x][n_z] (n_out = 1 with FNUM_FLAG_COMPOUND,
               else n_angles), scaled by 2 / N_dft; d_weights [n_x][n_z] or NULL
     flags     0 or FNUM_FLAG_COMPOUND
   The first call on a device looks up the array's device address (once per
   device, with that device current) and keeps it: do not reset the device
   (cudaDeviceReset, MATLAB's reset(gpuDevice)) between calls.  Arguments are
   checked as fnum_das_pw checks them, with the same status codes.  Problems whose tables, spectra and one block of aperture segments
   do not fit return FNUM_ERR_NOALLOC_TOO_LARGE; larger ones run with as many
   resident blocks as fit.  All calls share the array and it keeps the last
   call's contents; everything that must start at zero is cleared per call.
   Calls whose GPU work overlaps (other streams, other threads) race on it. */
#define FNUM_NOALLOC_SCRATCH_BYTES (64ull << 20)
int fnum_das_pw_noalloc(const fnum_pw_desc* desc, const double* steering_angles, int n_angles,
                        const float* d_rf, int flags, void* d_image, float* d_weights, void* stream);
/* --- autotuning and batches of frames ----------------------------------- */
/* No counterpart in the reference (one angle per gateway call, nothing kept).
   fnum_plan_autotune: runs the band DFT of d_rf, then times each fused-kernel
   variant of a plane-wave plan on it (1: 1 element x 11 angles per pass,
   2: 2 x 4, 3: 2 x 2, 4: 4 x 1, with the segment boundaries resolved ahead of
   the bin loop; 5..8: the same shapes resolving them inside the bin loop;
   9: tensor cores, 16 elements x 12 angles per pass -- 16 angles where that
   takes fewer passes -- the default from 3 angles on) at full occupancy, and
   keeps the fastest
   for the plan's later executes.  It allocates a temporary image and runs on
   a private stream (not capturable).  variant / ms (the chosen variant's
   beamform time) may be NULL.  A synthetic-aperture plan times its two
   variants (1: the per-pair recurrence kernels, 2: the tensor-core kernel, which
   needs up to 128 elements and a normalisation that accumulates, and is the
   default when available); a FNUM_FLAG_PLAIN_KERNEL plan returns variant 0. */
int fnum_plan_autotune(fnum_plan* plan, const void* d_rf, int rf_is_double, int* variant, float* ms);
/* fnum_plan_set_kernel_variant: pins the fused-kernel variant of a plane-wave
   plan (0 = by the angle count, 1..9 as above), e.g. one an earlier
   fnum_plan_autotune chose.  Every variant gives the same images up to the
   rounding of the per-pass sums.  A synthetic-aperture plan accepts 0 (default),
   1 and 2 (when available); a plan with FNUM_FLAG_M_SEMANTICS or
   FNUM_FLAG_PLAIN_KERNEL accepts only 0. */
int fnum_plan_set_kernel_variant(fnum_plan* plan, int variant);
/* fnum_plan_set_shape: pins the launch shape of a plane-wave plan's current
   variant: blocks_per_sm (0 = as many as fit) and bin_chunk, the bins between
   exact re-anchorings of the phase recurrences (0 = default; tensor cores 16 or
   32, FP32 kernels 128 or 256).  fnum_plan_autotune, after picking the variant,
   times these shapes (all or one fewer resident blocks, the default or the
   shorter bin chunk) and keeps the fastest.  A shorter chunk re-anchors more
   often, so no shape is less accurate than the default.  No counterpart in the
   reference. */
int fnum_plan_set_shape(fnum_plan* plan, int blocks_per_sm, int bin_chunk);

/* A batch binds n frames -- distinct plans with their device RF, image and
   weight buffers -- and captures their band DFTs and beamformers into one CUDA
   graph.  The frames are spread over n_streams concurrent branches (longest
   first, each to the least-loaded branch), so small frames share the GPU.
   Plans and buffers must outlive the batch; d_weights / d_weights_rx / their
   entries and rf_is_double may be NULL.  fnum_batch_execute launches the
   graph on `stream`; fnum_batch_frame_times gives, after it completed, each
   frame's completion time in ms from the batch's start (n values, in the
   order of `plans`). */
/* Compounded frames whose plans use the tensor-core kernel (variant 9) are not
   launched per frame: their band DFTs and spectra fragments run on the branches,
   then ONE persistent launch per window type and pass width (12 or 16 angles
   per pass) beamforms all of them -- each block
   draws tiles of all those frames from one counter, largest frames first, with
   each frame's descriptor read from device memory -- so no SM idles between
   frames.  The other frames keep a launch per frame on the other branches.
   fnum_batch_info reports how many frames the persistent launches carry and how
   many launches there are. */
typedef struct fnum_batch fnum_batch;
int fnum_batch_create(fnum_plan* const* plans, int n, const void* const* d_rf, const int* rf_is_double,
                      void* const* d_images, float* const* d_weights, float* const* d_weights_rx, int n_streams,
                      fnum_batch** batch);
int fnum_batch_execute(fnum_batch* batch, void* stream);
int fnum_batch_frame_times(const fnum_batch* batch, float* ms);
int fnum_batch_info(const fnum_batch* batch, int* persistent_frames, int* persistent_launches);
int fnum_batch_destroy(fnum_batch* batch);

/* After an execute of a plan with FNUM_FLAG_M_SEMANTICS: the focused spectrum of
   the last voxel das_pw.m processes (last column, deepest voxel with an active
   bin), complex interleaved per band bin (0 at bins without an active aperture);
   das_pw.m returns its inverse DFT as `signal` (das_pw.m:477-481).  *has_signal
   is 0 when no voxel of the last column has an active bin. */
int fnum_plan_m_signal(const fnum_plan* plan, double* spectrum_re_im, int* has_signal);

/* --- image-sharpness gradients (no counterpart in the reference) --------- */
/* Re-times a plane-wave plan's phase tables at sound speed c_0.  The DFT
   order, band, F table and apertures stay those of the speed the plan was
   created with, so images at nearby speeds differ only in their phases. */
int fnum_pw_plan_set_sound_speed(fnum_plan* plan, double c_0);
/* For a compounded plane-wave plan (FNUM_FLAG_COMPOUND): beamforms d_rf and
   returns the sharpness loss L = -sum|I|^4 / (sum|I|^2)^2 of the image,
   dL/dc at the plan's current sound speed (band, F table and apertures held
   fixed), and, if d_grad_spectra is not NULL, the Wirtinger gradient dL/dX*
   of the band spectra (device float2 [n_elements][n_bins][n_angles]; a change
   dX of the spectra changes L by 2 Re sum conj(dL/dX*) dX).  The first call
   allocates the plan's gradient buffers (a 1/W table of n_x n_z n_bins floats
   among them) and, if the memory is there, a receive table of 16 bytes per
   voxel and element (n_x n_z n_elements; 537 MB at 512 x 512 x 128) that
   speeds up dL/dX* -- without it the kernel forms the same values itself.
   Synchronises `stream`. */
int fnum_pw_sharpness_grad(fnum_plan* plan, const void* d_rf, int rf_is_double, double* loss, double* dloss_dc,
                           void* d_grad_spectra, void* stream);

/* The adjoint of a compounded plane-wave plan's beamformer, for any real loss L
   of its image I (no counterpart in the reference).  d_cotangent holds
   dL/dI* per voxel (device float2 [n_x][n_z], the image layout); the call
   returns, for the plan's current spectra X (those of the last execute, or of
   fnum_plan_set_spectra) and sound speed, the Wirtinger gradient dL/dX* (device
   float2 [n_elements][n_bins][n_angles]; NULL keeps it in the plan) and, if
   dloss_dc is not NULL, dL/dc = 2 Re sum_v conj(dL/dI*_v) dI_v/dc with the band,
   F table and apertures held fixed.  I is linear in X, so dL/dX* = A^H dL/dI*
   for the beamformer A.  Allocates the plan's gradient buffers on first use;
   synchronises `stream`. */
int fnum_pw_adjoint(fnum_plan* plan, const void* d_cotangent, void* d_grad_spectra, double* dloss_dc, void* stream);
/* loads band spectra (device float2, the layout of fnum_plan_spectra) into the
   plan, e.g. to beamform spectra a caller produced (fnum_plan_execute_beamform)
   or to take fnum_pw_adjoint at them.  No counterpart in the reference. */
int fnum_plan_set_spectra(fnum_plan* plan, const void* d_spectra, void* stream);

/* copies the plan's F table (n_bins values; two tables for SA: tx then rx) */
int fnum_plan_f_numbers(const fnum_plan* plan, double* values);
int fnum_plan_destroy(fnum_plan* plan);

/* --- post-processing on the device ---------------------------------------- */
/* B-mode image: d_db[i] = max(20 log10(|s_i| / max_j |s_j|), floor_db) with
   s_i = sum over the n_images images of d_image (float2 [n_images][n_voxels]),
   i.e. coherent compounding over angles and log compression in one call.
   Replaces the host-side steps of the reference's example script
   (examples.m:78 sums the per-angle images, examples.m:88,96 take
   20 log10(abs(image) / max(abs(image(:))))).  d_max_abs receives max_j |s_j|
   (one float on the device).  floor_db = -INFINITY keeps every value; an
   all-zero image gives floor_db everywhere (the script would give NaN). */
int fnum_bmode(const void* d_image, long long n_voxels, int n_images, float floor_db, float* d_db,
               float* d_max_abs, void* stream);

/* --- diagnostics (no counterpart in the reference) ---------------------- */
/* sustained FP32 FMA throughput of the device (TFLOP/s, 2 flops per FMA): the
   roofline denominator of the fused kernels, which are bound by the FP32 pipe */
int fnum_diag_fp32_peak(int device, double* tflops);
/* Throughput of warp-level mma.sync m16n8k16 (fp16 operands, fp32
   accumulators) on `device`, TFLOP/s (2 x 16 x 8 x 16 per instruction): the
   tensor-pipe denominator of the tensor-core plane-wave kernel (variant 9). */
int fnum_diag_mma_f16_peak(int device, double* tflops);

#ifdef __cplusplus
}
#endif
#endif /* FNUM_H */
