// MEX gateway for MATLAB: cuda.gpu_bf_das_pw_sharpness_grad backed by libfnum
// (include/fnum.h, fnum_das_pw_sharpness_grad).  No counterpart in the
// reference, which has no derivatives; it takes cuda.gpu_bf_das_pw_rf's inputs
// (+cuda/gpu_bf_das_pw_rf.cu:110) with a vector of steering angles and RF
// stacked along a third dimension, and returns the image-sharpness loss of the
// compounded image and its gradients:
//
//   [L, dL_dc, dL_dX] = cuda.gpu_bf_das_pw_sharpness_grad(positions_x, positions_z,
//        data_RF /* N_t x N_el x N_angles */, f_s, steering_angles, element_width,
//        element_pitch, c_0, f_bounds, index_t0, window, F_number, normalization, index_gpu)
//
//   L      = -sum|I|^4 / (sum|I|^2)^2 of I = sum over angles of the MEX images
//   dL_dc  = dL/dc at c_0, with the DFT order, band, F table and apertures held
//            at c_0 (only the phases move)
//   dL_dX  = the Wirtinger gradient dL/dX* of the band spectra, single complex
//            N_bins x N_el x N_angles (a change dX changes L by 2 Re sum conj(dL_dX) dX)
//
// Inputs are read and checked as in gpu_bf_das_pw_rf.cpp (same identifiers,
// prefix gpu_bf_das_pw_rf).
//
// Build (MATLAB): mex -R2017b gpu_bf_das_pw_sharpness_grad.cpp -I<repo>/include -L<repo>/f_number_gb300 -lfnum
#include <math.h>
#include <string.h>

#include <vector>

#include "fnum.h"
#include "fnum_mex_objects.h"
#include "mex.h"

namespace {

const char* kId = "gpu_bf_das_pw_rf";

void fail(const char* suffix, const char* msg) {
  char id[128];
  snprintf(id, sizeof(id), "%s:%s", kId, suffix);
  mexErrMsgIdAndTxt(id, msg);
}

void fail_status(int s) { mexErrMsgIdAndTxt(fnum_status_id(s, 0), fnum_status_string(s)); }

bool real_double(const mxArray* a) { return mxIsDouble(a) && !mxIsComplex(a); }

bool isa(const mxArray* obj, const char* cls) {
  mxArray* lhs = nullptr;
  mxArray* rhs[2] = {mxDuplicateArray(obj), mxCreateString(cls)};
  mexCallMATLAB(1, &lhs, 2, rhs, "isa");
  const bool r = mxIsLogicalScalarTrue(lhs);
  mxDestroyArray(lhs);
  mxDestroyArray(rhs[0]);
  mxDestroyArray(rhs[1]);
  return r;
}

bool window_of(const mxArray* w, fnum_window* out) {
  if (mxIsClass(w, "windows.boxcar")) { *out = {FNUM_WINDOW_BOXCAR, 0.0}; return true; }
  if (mxIsClass(w, "windows.hann")) { *out = {FNUM_WINDOW_HANN, 0.0}; return true; }
  if (mxIsClass(w, "windows.triangular")) { *out = {FNUM_WINDOW_TRIANGULAR, 0.0}; return true; }
  if (mxIsClass(w, "windows.tukey")) {
    const mxArray* fc = mxGetProperty(w, 0, "fraction_cosine");
    if (!fc) return false;
    *out = {FNUM_WINDOW_TUKEY, mxGetScalar(fc)};
    return true;
  }
  return false;
}

double scalar(const mxArray* a, const char* suffix, const char* msg) {
  if (!(real_double(a) && mxIsScalar(a))) fail(suffix, msg);
  return mxGetScalar(a);
}

}  // namespace

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (fnum_device_count() < 1) fail("NoCUDADevices", "Could not find any CUDA-enabled devices!");
  if (nrhs < 8) fail("nrhs", "At least 8 inputs are required.");
  if (nrhs > 14) fail("nrhs", "At most 14 inputs are allowed.");
  if (nlhs > 3) fail("nlhs", "At most 3 outputs are allowed.");
  if (!(real_double(prhs[0]) && mxGetNumberOfDimensions(prhs[0]) == 2))
    fail("InvalidLateralPositions", "Lateral positions must be a real-valued matrix of type double!");
  if (!(real_double(prhs[1]) && mxGetNumberOfDimensions(prhs[1]) == 2))
    fail("InvalidAxialPositions", "Axial positions must be a real-valued matrix of type double!");
  const mwSize nd = mxGetNumberOfDimensions(prhs[2]);
  if (!(real_double(prhs[2]) && (nd == 2 || nd == 3)))
    fail("InvalidRFData", "RF data must be a real-valued array of type double with 2 or 3 dimensions!");
  const mwSize* dim = mxGetDimensions(prhs[2]);
  const int n_angles_rf = nd == 3 ? (int)dim[2] : 1;
  if (!(real_double(prhs[4]) && (int)mxGetNumberOfElements(prhs[4]) == n_angles_rf))
    fail("InvalidSteeringAngle", "Steering angles must be a real-valued vector of type double, one per RF block!");

  fnum_pw_desc d;
  memset(&d, 0, sizeof(d));
  d.positions_x = mxGetPr(prhs[0]);
  d.n_x = (int)mxGetN(prhs[0]);
  d.positions_z = mxGetPr(prhs[1]);
  d.n_z = (int)mxGetN(prhs[1]);
  d.n_samples = (int)dim[0];
  d.n_elements = (int)dim[1];
  d.f_s = scalar(prhs[3], "InvalidSamplingRate", "Sampling rate must be a real-valued scalar of type double!");
  d.element_width = scalar(prhs[5], "InvalidElementWidth", "Element width must be a real-valued scalar of type double!");
  d.element_pitch = scalar(prhs[6], "InvalidElementPitch", "Element pitch must be a real-valued scalar of type double!");
  d.c_0 = scalar(prhs[7], "InvalidSoundSpeed", "Speed of sound must be a real-valued scalar of type double!");
  double fb[2];
  if (nrhs >= 9 && !mxIsEmpty(prhs[8])) {
    if (!(real_double(prhs[8]) && mxGetNumberOfElements(prhs[8]) == 2))
      fail("InvalidFrequencyBounds", "Frequency bounds must be a real-valued vector with two entries of type double!");
    fb[0] = mxGetPr(prhs[8])[0];
    fb[1] = mxGetPr(prhs[8])[1];
    d.f_bounds = fb;
  }
  if (nrhs >= 10 && !mxIsEmpty(prhs[9]))
    d.index_t0 = scalar(prhs[9], "InvalidTimeShift", "Time index must be a real-valued scalar of type double!");
  d.window = {FNUM_WINDOW_BOXCAR, 0.0};
  if (nrhs >= 11 && !mxIsEmpty(prhs[10])) {
    if (!(isa(prhs[10], "windows.window") && mxIsScalar(prhs[10])))
      fail("InvalidWindow", "Receive window must be a single object of the class windows.window!");
    if (!window_of(prhs[10], &d.window)) fail("InvalidWindow", "Could not read window parameters!");
  }
  d.f_number.kind = FNUM_F_DEFAULT;
  std::vector<double> fvals;
  int N = 0, klb = 0, kub = 0;
  {
    const int s = fnum_band(d.positions_z, d.n_z, d.n_samples, d.n_elements, d.f_s, d.element_width,
                            d.element_pitch, d.c_0, d.f_bounds, d.index_t0, &N, &klb, &kub);
    if (s != FNUM_OK) fail_status(s);
  }
  if (nrhs >= 12 && !mxIsEmpty(prhs[11])) {
    if (!(isa(prhs[11], "f_numbers.f_number") && mxIsScalar(prhs[11])))
      fail("InvalidFNumber", "F-number must be a single object of the class f_numbers.f_number!");
    mxArray* pl = mxCreateDoubleMatrix(kub - klb + 1, 1, mxREAL);
    for (int k = klb; k <= kub; ++k) mxGetPr(pl)[k - klb] = d.element_pitch * k * d.f_s / (N * d.c_0);
    fnum_f_number nf;
    if (fnum_mex::native_f_number(prhs[11], &nf)) {
      fvals.resize(kub - klb + 1);
      const int st = fnum_f_number_values(&nf, mxGetPr(pl), kub - klb + 1, fvals.data());
      if (st != FNUM_OK) fail_status(st);
    } else {
      mxArray* lhs = nullptr;
      mxArray* rhs[2] = {mxDuplicateArray(prhs[11]), mxDuplicateArray(pl)};
      mexCallMATLAB(1, &lhs, 2, rhs, "compute_values");
      fvals.assign(mxGetPr(lhs), mxGetPr(lhs) + mxGetNumberOfElements(lhs));
      mxDestroyArray(lhs);
      mxDestroyArray(rhs[0]);
      mxDestroyArray(rhs[1]);
    }
    mxDestroyArray(pl);
    d.f_number_values = fvals.data();
    d.n_f_number_values = (int)fvals.size();
  }
  d.normalization = FNUM_NORMALIZATION_ON;
  if (nrhs >= 13 && !mxIsEmpty(prhs[12])) {
    if (!(isa(prhs[12], "normalizations.normalization") && mxIsScalar(prhs[12])))
      fail("InvalidNormalization", "Normalization must be a single object of the class normalizations.normalization!");
    if (mxIsClass(prhs[12], "normalizations.off")) d.normalization = FNUM_NORMALIZATION_OFF;
    if (mxIsClass(prhs[12], "normalizations.windowed")) d.normalization = FNUM_NORMALIZATION_WINDOWED;
  }
  if (nrhs >= 14 && !mxIsEmpty(prhs[13]))
    d.device = (int)scalar(prhs[13], "InvalidCUDADevice", "Device index must be a real-valued scalar of type double!");

  const int K = kub - klb + 1;
  const mwSize gdim[3] = {(mwSize)K, (mwSize)d.n_elements, (mwSize)n_angles_rf};
  mxArray* g = mxCreateNumericArray(3, gdim, mxSINGLE_CLASS, mxCOMPLEX);
  double L = 0.0, dc = 0.0;
  const int s = fnum_das_pw_sharpness_grad(&d, mxGetPr(prhs[4]), n_angles_rf, mxGetPr(prhs[2]), &L, &dc,
                                           (float*)mxGetData(g), (float*)mxGetImagData(g));
  if (s != FNUM_OK) {
    mxDestroyArray(g);
    fail_status(s);
  }
  plhs[0] = mxCreateDoubleMatrix(1, 1, mxREAL);
  mxGetPr(plhs[0])[0] = L;
  if (nlhs >= 2) {
    plhs[1] = mxCreateDoubleMatrix(1, 1, mxREAL);
    mxGetPr(plhs[1])[0] = dc;
  }
  if (nlhs >= 3) plhs[2] = g; else mxDestroyArray(g);
}
