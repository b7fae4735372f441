// MEX gateway for MATLAB: cuda.gpu_bf_saft_rf backed by libfnum (include/fnum.h).
//
// Drop-in for the reference's +cuda/gpu_bf_saft_rf.cu (mexFunction at line
// 107): 7-17 inputs (data_RF [N_t x N_rx x N_tx], N_rx == N_tx), <= 3 outputs
// (image, weights_tx, weights_rx), the reference's error identifiers and its
// normalisation behaviour (fnum flag FNUM_FLAG_SAFT_INTENDED is not set).
//
// Build (MATLAB): mex -R2017b gpu_bf_saft_rf.cpp -I<repo>/include -L<repo>/f_number_gb300 -lfnum
#include <string.h>

#include <vector>

#include "fnum.h"
#include "fnum_mex_objects.h"
#include "mex.h"

namespace {

const char* kId = "gpu_bf_saft_rf";

void fail(const char* suffix, const char* msg) {
  char id[128];
  snprintf(id, sizeof(id), "%s:%s", kId, suffix);
  mexErrMsgIdAndTxt(id, msg);
}

void fail_status(int s) { mexErrMsgIdAndTxt(fnum_status_id(s, 1), fnum_status_string(s)); }

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

void read_window(int nrhs, const mxArray* prhs[], int i, fnum_window* w, const char* which) {
  *w = {FNUM_WINDOW_BOXCAR, 0.0};
  if (nrhs > i && !mxIsEmpty(prhs[i])) {
    if (!(isa(prhs[i], "windows.window") && mxIsScalar(prhs[i])))
      fail("InvalidWindow", which);
    if (!window_of(prhs[i], w)) fail("InvalidWindow", "Could not read window parameters!");
  }
}

// F-number values on the band: native for the built-in classes (fnum_mex_objects.h),
// else through the object's MATLAB compute_values
void read_f_number(int nrhs, const mxArray* prhs[], int i, const fnum_sa_desc& d, std::vector<double>& v) {
  int N = 0, klb = 0, kub = 0;
  const int s = fnum_band(d.positions_z, d.n_z, d.n_samples, d.n_elements, d.f_s, d.element_width, d.element_pitch,
                          d.c_0, d.f_bounds, d.index_t0, &N, &klb, &kub);
  if (s != FNUM_OK) fail_status(s);
  mxArray* pl = mxCreateDoubleMatrix(kub - klb + 1, 1, mxREAL);
  for (int k = klb; k <= kub; ++k) mxGetPr(pl)[k - klb] = d.element_pitch * k * d.f_s / (N * d.c_0);
  if (nrhs > i && !mxIsEmpty(prhs[i])) {
    if (!(isa(prhs[i], "f_numbers.f_number") && mxIsScalar(prhs[i])))
      fail("InvalidFNumber", "F-number must be a single object of the class f_numbers.f_number!");
    fnum_f_number nf;
    if (fnum_mex::native_f_number(prhs[i], &nf)) {
      // built-in class: the library's own table, no MATLAB callback
      v.resize(kub - klb + 1);
      const int st = fnum_f_number_values(&nf, mxGetPr(pl), kub - klb + 1, v.data());
      if (st != FNUM_OK) fail_status(st);
    } else {
      mxArray* lhs = nullptr;
      mxArray* rhs[2] = {mxDuplicateArray(prhs[i]), mxDuplicateArray(pl)};
      mexCallMATLAB(1, &lhs, 2, rhs, "compute_values");
      v.assign(mxGetPr(lhs), mxGetPr(lhs) + mxGetNumberOfElements(lhs));
      mxDestroyArray(lhs);
      mxDestroyArray(rhs[0]);
      mxDestroyArray(rhs[1]);
    }
  } else {
    fnum_f_number def;
    memset(&def, 0, sizeof(def));
    v.resize(kub - klb + 1);
    const int st = fnum_f_number_values(&def, mxGetPr(pl), kub - klb + 1, v.data());
    if (st != FNUM_OK) fail_status(st);
  }
  mxDestroyArray(pl);
}

int read_normalization(int nrhs, const mxArray* prhs[], int i) {
  if (nrhs > i && !mxIsEmpty(prhs[i])) {
    if (!(isa(prhs[i], "normalizations.normalization") && mxIsScalar(prhs[i])))
      fail("InvalidNormalization", "Normalization must be a single object of the class normalizations.normalization!");
    if (mxIsClass(prhs[i], "normalizations.off")) return FNUM_NORMALIZATION_OFF;
    if (mxIsClass(prhs[i], "normalizations.windowed")) return FNUM_NORMALIZATION_WINDOWED;
  }
  return FNUM_NORMALIZATION_ON;
}

}  // namespace

void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (fnum_device_count() < 1) fail("NoCUDADevices", "Could not find any CUDA-enabled devices!");
  if (nrhs < 7) fail("nrhs", "At least 7 inputs are required.");
  if (nrhs > 17) fail("nrhs", "At most 17 inputs are allowed.");
  if (nlhs > 3) fail("nlhs", "At most 3 outputs are allowed.");
  if (!(real_double(prhs[0]) && mxGetNumberOfDimensions(prhs[0]) == 2))
    fail("InvalidLateralPositions", "Lateral positions must be a real-valued matrix of type double!");
  if (!(real_double(prhs[1]) && mxGetNumberOfDimensions(prhs[1]) == 2))
    fail("InvalidAxialPositions", "Axial positions must be a real-valued matrix of type double!");
  if (!(real_double(prhs[2]) && mxGetNumberOfDimensions(prhs[2]) == 3))
    fail("InvalidRFData", "RF data must be a real-valued array of type double with 3 dimensions!");
  const mwSize* dim = mxGetDimensions(prhs[2]);
  if (dim[1] != dim[2]) fail("InvalidRFData", "Size of RF data must be equal along 2nd and 3rd dimensions!");

  fnum_sa_desc d;
  memset(&d, 0, sizeof(d));
  d.positions_x = mxGetPr(prhs[0]);
  d.n_x = (int)mxGetN(prhs[0]);
  d.positions_z = mxGetPr(prhs[1]);
  d.n_z = (int)mxGetN(prhs[1]);
  d.n_samples = (int)dim[0];
  d.n_elements = (int)dim[1];
  d.f_s = scalar(prhs[3], "InvalidSamplingRate", "Sampling rate must be a real-valued scalar of type double!");
  d.element_width = scalar(prhs[4], "InvalidElementWidth", "Element width must be a real-valued scalar of type double!");
  d.element_pitch = scalar(prhs[5], "InvalidElementPitch", "Element pitch must be a real-valued scalar of type double!");
  d.c_0 = scalar(prhs[6], "InvalidSoundSpeed", "Speed of sound must be a real-valued scalar of type double!");
  double fb[2];
  if (nrhs >= 8 && !mxIsEmpty(prhs[7])) {
    if (!(real_double(prhs[7]) && mxGetNumberOfElements(prhs[7]) == 2))
      fail("InvalidFrequencyBounds", "Frequency bounds must be a real-valued vector with two entries of type double!");
    fb[0] = mxGetPr(prhs[7])[0];
    fb[1] = mxGetPr(prhs[7])[1];
    d.f_bounds = fb;
  }
  if (nrhs >= 9 && !mxIsEmpty(prhs[8]))
    d.index_t0 = scalar(prhs[8], "InvalidTimeShift", "Time index must be a real-valued scalar of type double!");
  read_window(nrhs, prhs, 9, &d.window_tx, "Transmit window must be a single object of the class windows.window!");
  read_window(nrhs, prhs, 10, &d.window_rx, "Receive window must be a single object of the class windows.window!");
  std::vector<double> ftx, frx;
  read_f_number(nrhs, prhs, 11, d, ftx);
  read_f_number(nrhs, prhs, 12, d, frx);
  d.f_number_tx_values = ftx.data();
  d.f_number_rx_values = frx.data();
  d.n_f_number_values = (int)ftx.size();
  d.normalization_tx = read_normalization(nrhs, prhs, 13);
  d.normalization_rx = read_normalization(nrhs, prhs, 14);
  if (nrhs >= 16 && !mxIsEmpty(prhs[15]))
    d.device = (int)scalar(prhs[15], "InvalidCUDADevice", "Device index must be a real-valued scalar of type double!");
  if (nrhs >= 17 && !mxIsEmpty(prhs[16])) {
    const double v = scalar(prhs[16], "InvalidVerbosityLevel", "Verbosity level must be a real-valued scalar of type double!");
    if (v < 0 || v >= 4) fail("InvalidVerbosityLevel", "Selected verbosity level does not exist!");
  }
  plhs[0] = mxCreateNumericMatrix(d.n_z, d.n_x, mxSINGLE_CLASS, mxCOMPLEX);
  mxArray* wt = mxCreateNumericMatrix(d.n_z, d.n_x, mxSINGLE_CLASS, mxREAL);
  mxArray* wr = mxCreateNumericMatrix(d.n_z, d.n_x, mxSINGLE_CLASS, mxREAL);
  const int s = fnum_das_sa(&d, mxGetPr(prhs[2]), 0, (float*)mxGetData(plhs[0]), (float*)mxGetImagData(plhs[0]),
                            (float*)mxGetData(wt), (float*)mxGetData(wr));
  if (s != FNUM_OK) {
    mxDestroyArray(wt);
    mxDestroyArray(wr);
    fail_status(s);
  }
  if (nlhs >= 2) plhs[1] = wt; else mxDestroyArray(wt);
  if (nlhs >= 3) plhs[2] = wr; else mxDestroyArray(wr);
}
