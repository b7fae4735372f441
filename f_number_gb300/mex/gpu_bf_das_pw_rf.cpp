// MEX gateway for MATLAB: cuda.gpu_bf_das_pw_rf backed by libfnum (include/fnum.h).
//
// Drop-in for the reference's +cuda/gpu_bf_das_pw_rf.cu (mexFunction at line
// 110): same 8-15 inputs, same <= 2 outputs (single complex image, single
// weights), same error identifiers.  Parameter objects are read the way the
// reference reads them: windows by class (gpu_bf_helper_functions.cu:56-97).
// F-numbers of the built-in classes are tabulated by the library itself
// (fnum_mex_objects.h), so the call makes no MATLAB callback; other classes,
// such as user-defined subclasses, go through their MATLAB compute_values
// method on the band's normalised pitches, as in the reference
// (gpu_bf_helper_functions.cu:35-51).
//
// Build (MATLAB): mex -R2017b gpu_bf_das_pw_rf.cpp -I<repo>/include -L<repo>/f_number_gb300 -lfnum
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

// windows.* -> {id, parameter}
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
  if (nrhs > 15) fail("nrhs", "At most 15 inputs are allowed.");
  if (nlhs > 2) fail("nlhs", "At most 2 outputs are allowed.");
  if (!(real_double(prhs[0]) && mxGetNumberOfDimensions(prhs[0]) == 2))
    fail("InvalidLateralPositions", "Lateral positions must be a real-valued matrix of type double!");
  if (!(real_double(prhs[1]) && mxGetNumberOfDimensions(prhs[1]) == 2))
    fail("InvalidAxialPositions", "Axial positions must be a real-valued matrix of type double!");
  if (!(real_double(prhs[2]) && mxGetNumberOfDimensions(prhs[2]) == 2))
    fail("InvalidRFData", "RF data must be a real-valued matrix of type double!");

  fnum_pw_desc d;
  memset(&d, 0, sizeof(d));
  d.positions_x = mxGetPr(prhs[0]);
  d.n_x = (int)mxGetN(prhs[0]);
  d.positions_z = mxGetPr(prhs[1]);
  d.n_z = (int)mxGetN(prhs[1]);
  d.n_samples = (int)mxGetM(prhs[2]);
  d.n_elements = (int)mxGetN(prhs[2]);
  d.f_s = scalar(prhs[3], "InvalidSamplingRate", "Sampling rate must be a real-valued scalar of type double!");
  const double angle =
      scalar(prhs[4], "InvalidSteeringAngle", "Steering angle must be a real-valued scalar of type double!");
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
  // F-number table on the band: native for the built-in classes, else the object's compute_values
  d.f_number.kind = FNUM_F_DEFAULT;
  std::vector<double> fvals;
  if (nrhs >= 12 && !mxIsEmpty(prhs[11])) {
    if (!(isa(prhs[11], "f_numbers.f_number") && mxIsScalar(prhs[11])))
      fail("InvalidFNumber", "F-number must be a single object of the class f_numbers.f_number!");
    int N = 0, klb = 0, kub = 0;
    const int s = fnum_band(d.positions_z, d.n_z, d.n_samples, d.n_elements, d.f_s, d.element_width,
                            d.element_pitch, d.c_0, d.f_bounds, d.index_t0, &N, &klb, &kub);
    if (s != FNUM_OK) fail_status(s);
    mxArray* pl = mxCreateDoubleMatrix(kub - klb + 1, 1, mxREAL);
    for (int k = klb; k <= kub; ++k) mxGetPr(pl)[k - klb] = d.element_pitch * k * d.f_s / (N * d.c_0);
    fnum_f_number nf;
    if (fnum_mex::native_f_number(prhs[11], &nf)) {
      // built-in class: the library's own table, no MATLAB callback
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
  if (nrhs >= 15 && !mxIsEmpty(prhs[14])) {
    const double v = scalar(prhs[14], "InvalidVerbosityLevel", "Verbosity level must be a real-valued scalar of type double!");
    if (v < 0 || v >= 4) fail("InvalidVerbosityLevel", "Selected verbosity level does not exist!");
  }
  plhs[0] = mxCreateNumericMatrix(d.n_z, d.n_x, mxSINGLE_CLASS, mxCOMPLEX);
  mxArray* w = mxCreateNumericMatrix(d.n_z, d.n_x, mxSINGLE_CLASS, mxREAL);
  const int s = fnum_das_pw(&d, &angle, 1, mxGetPr(prhs[2]), 0, (float*)mxGetData(plhs[0]),
                            (float*)mxGetImagData(plhs[0]), (float*)mxGetData(w));
  if (s != FNUM_OK) {
    mxDestroyArray(w);
    fail_status(s);
  }
  if (nlhs >= 2) plhs[1] = w; else mxDestroyArray(w);
}
