// Shared by the MEX gateways: reads a built-in f_numbers.* object into the C
// ABI's fnum_f_number, so that libfnum computes its table natively and the
// beamforming call makes no MATLAB callback.  The classes whose
// compute_values the library restates (+f_numbers/constant.m:61-74,
// +grating/angle_lb.m:44-75, +distance/constant.m:90-120, +distance/none.m,
// +directivity/directivity.m:91-120 with the rigid / soft obliquity,
// +directivity/szabo.m:71-87) are matched by their exact class name.  Any
// other class, such as a user-defined subclass, returns false, and the
// gateway then calls the object's own compute_values through MATLAB, as the
// reference does for every class (gpu_bf_helper_functions.cu:35-51).
#pragma once
#include <math.h>

#include "fnum.h"
#include "mex.h"

namespace fnum_mex {

inline bool prop(const mxArray* obj, const char* name, double* v) {
  const mxArray* p = mxGetProperty(obj, 0, name);
  if (!p || !mxIsDouble(p) || mxGetNumberOfElements(p) != 1) return false;
  *v = mxGetScalar(p);
  return true;
}

inline bool native_f_number(const mxArray* obj, fnum_f_number* out) {
  fnum_f_number f = {FNUM_F_DEFAULT, FNUM_OBLIQUITY_SOFT, {0.0, 0.0, 0.0}};
  if (mxIsClass(obj, "f_numbers.constant")) {
    f.kind = FNUM_F_CONSTANT;
    if (!prop(obj, "value", &f.p[0])) return false;
  } else if (mxIsClass(obj, "f_numbers.grating.angle_lb")) {
    f.kind = FNUM_F_ANGLE_LB;
    if (!prop(obj, "angle_lb_deg", &f.p[0]) || !prop(obj, "F_number_ub", &f.p[1]) ||
        !prop(obj, "distance_deg", &f.p[2]))
      return false;
  } else if (mxIsClass(obj, "f_numbers.distance.none")) {
    f.kind = FNUM_F_DISTANCE_NONE;
  } else if (mxIsClass(obj, "f_numbers.distance.constant")) {
    f.kind = FNUM_F_DISTANCE_CONSTANT;
    if (!prop(obj, "distance_deg", &f.p[0]) || !prop(obj, "F_number_ub", &f.p[1])) return false;
  } else if (mxIsClass(obj, "f_numbers.directivity.szabo")) {
    f.kind = FNUM_F_SZABO;
    if (!prop(obj, "width_over_pitch", &f.p[0])) return false;
  } else if (mxIsClass(obj, "f_numbers.directivity.directivity") || mxIsClass(obj, "f_numbers.directivity.rigid") ||
             mxIsClass(obj, "f_numbers.directivity.soft") || mxIsClass(obj, "f_numbers.directivity.perrot")) {
    f.kind = FNUM_F_DIRECTIVITY;
    if (!prop(obj, "width_over_pitch", &f.p[0]) || !prop(obj, "attenuation_dB", &f.p[1])) return false;
    const mxArray* o = mxGetProperty(obj, 0, "obliquity_factor");
    if (!o) return false;
    if (mxIsClass(o, "f_numbers.directivity.obliquity.rigid")) f.obliquity = FNUM_OBLIQUITY_RIGID;
    else if (mxIsClass(o, "f_numbers.directivity.obliquity.soft")) f.obliquity = FNUM_OBLIQUITY_SOFT;
    else return false;
  } else {
    return false;
  }
  *out = f;
  return true;
}

}  // namespace fnum_mex
