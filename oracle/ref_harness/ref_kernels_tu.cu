// Translation unit that compiles the reference's own CUDA kernels (f_number,
// +cuda/*.cu) into a device-only fatbin, from the files where they lie (the
// include path points at the reference's +cuda directory; nothing is copied).
// The block-size macros are the gateway's (+cuda/gpu_bf_das_pw_rf.cu:94-96).
//
// TEST INFRASTRUCTURE ONLY: loaded by oracle/ref_harness/ref_driver.cu to run
// the reference GPU algorithm as a parity pin and speed baseline.
#include <cuda.h>
#include <cufft.h>
#include <float.h>
#include <math.h>

#define N_THREADS_X 8
#define N_THREADS_Y 8
#define N_THREADS_PER_BLOCK 64

#include "gpu_bf_types.cuh"
#include "gpu_bf_windows.cu"
#include "das_kernel_distances_pw.cu"
#include "das_kernel_distances_sw.cu"
#include "das_kernel_f_number_constant.cu"
#include "das_kernel_phase_shifts.cu"
#include "das_kernel_normalization.cu"
#include "saft_kernel_phase_shifts.cu"
