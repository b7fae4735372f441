// A minimal stand-in for MATLAB's MEX runtime, so that the gateways in
// f_number_gb300/mex run under the tests (MATLAB is not available here).
//
// TEST INFRASTRUCTURE ONLY.  It implements the mx / mex functions of mex.h on
// a small mxArray: numeric arrays (double, single; real or with a separate
// imaginary plane, any number of dimensions), logical scalars, strings, and
// objects with a class name, a list of superclasses (for isa) and named
// properties.  mexErrMsgIdAndTxt throws; shim_call catches and reports the
// identifier and message.  mexCallMATLAB serves "isa" itself and hands every
// other function (e.g. compute_values of a user-defined F-number class) to a
// callback the test registers.  Each gateway is linked with its own copy.
#include <stdarg.h>
#include <stdint.h>
#include <string.h>

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "mex.h"

struct mxArray_tag {
  mxClassID cls = mxDOUBLE_CLASS;
  std::string class_name;                 // objects: e.g. "windows.tukey"
  std::vector<std::string> supers;        // objects: classes isa() accepts besides class_name
  std::vector<mwSize> dims{0, 0};
  bool complex = false;
  std::vector<unsigned char> re, im;      // element bytes
  std::map<std::string, mxArray*> props;  // objects: owned
  ~mxArray_tag() {
    for (auto& p : props) delete p.second;
  }
};

namespace {

struct MexError {
  std::string id, msg;
};

typedef int (*Callback)(const char* name, int nlhs, mxArray** plhs, int nrhs, mxArray** prhs);
Callback g_callback = nullptr;

size_t elem_size(mxClassID c) {
  switch (c) {
    case mxDOUBLE_CLASS: return 8;
    case mxSINGLE_CLASS: return 4;
    case mxLOGICAL_CLASS: return 1;
    case mxCHAR_CLASS: return 2;
    default: return 0;
  }
}

size_t numel(const mxArray* a) {
  size_t n = 1;
  for (mwSize d : a->dims) n *= d;
  return n;
}

mxArray* make(mxClassID c, const std::vector<mwSize>& dims, bool complex) {
  mxArray* a = new mxArray_tag;
  a->cls = c;
  a->dims = dims;
  if (a->dims.size() < 2) a->dims.resize(2, 1);
  a->complex = complex;
  a->re.assign(numel(a) * elem_size(c), 0);
  if (complex) a->im.assign(numel(a) * elem_size(c), 0);
  return a;
}

mxArray* copy(const mxArray* a) {
  mxArray* b = new mxArray_tag;
  b->cls = a->cls;
  b->class_name = a->class_name;
  b->supers = a->supers;
  b->dims = a->dims;
  b->complex = a->complex;
  b->re = a->re;
  b->im = a->im;
  for (auto& p : a->props) b->props[p.first] = copy(p.second);
  return b;
}

double get(const std::vector<unsigned char>& v, mxClassID c, size_t i) {
  switch (c) {
    case mxDOUBLE_CLASS: return ((const double*)v.data())[i];
    case mxSINGLE_CLASS: return ((const float*)v.data())[i];
    case mxLOGICAL_CLASS: return v[i] ? 1.0 : 0.0;
    default: return 0.0;
  }
}

}  // namespace

extern "C" {

// ---- the MEX API ------------------------------------------------------------
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw MexError{id ? id : "", buf};
}

int mexCallMATLAB(int nlhs, mxArray* plhs[], int nrhs, mxArray* prhs[], const char* name) {
  if (strcmp(name, "isa") == 0 && nrhs == 2 && nlhs <= 1) {
    const mxArray* o = prhs[0];
    const std::string want((const char*)prhs[1]->re.data(), prhs[1]->re.size());
    bool r = o->class_name == want;
    for (const auto& s : o->supers) r = r || s == want;
    if (o->cls == mxDOUBLE_CLASS && want == "double") r = true;
    mxArray* out = make(mxLOGICAL_CLASS, {1, 1}, false);
    out->re[0] = r ? 1 : 0;
    plhs[0] = out;
    return 0;
  }
  if (g_callback && g_callback(name, nlhs, plhs, nrhs, prhs) == 0) return 0;
  mexErrMsgIdAndTxt("MATLAB:UndefinedFunction", "Undefined function '%s' in the MEX shim.", name);
  return 1;
}

bool mxIsDouble(const mxArray* a) { return a->cls == mxDOUBLE_CLASS; }
bool mxIsComplex(const mxArray* a) { return a->complex; }
bool mxIsScalar(const mxArray* a) { return numel(a) == 1; }
bool mxIsEmpty(const mxArray* a) { return numel(a) == 0; }
bool mxIsClass(const mxArray* a, const char* name) {
  if (a->cls == mxOBJECT_CLASS) return a->class_name == name;
  if (a->cls == mxDOUBLE_CLASS) return strcmp(name, "double") == 0;
  if (a->cls == mxSINGLE_CLASS) return strcmp(name, "single") == 0;
  if (a->cls == mxLOGICAL_CLASS) return strcmp(name, "logical") == 0;
  if (a->cls == mxCHAR_CLASS) return strcmp(name, "char") == 0;
  return false;
}
bool mxIsLogicalScalarTrue(const mxArray* a) { return a->cls == mxLOGICAL_CLASS && numel(a) == 1 && a->re[0]; }
mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->dims.size(); }
mwSize mxGetNumberOfElements(const mxArray* a) { return numel(a); }
const mwSize* mxGetDimensions(const mxArray* a) { return a->dims.data(); }
size_t mxGetM(const mxArray* a) { return a->dims[0]; }
size_t mxGetN(const mxArray* a) {
  size_t n = 1;
  for (size_t i = 1; i < a->dims.size(); ++i) n *= a->dims[i];
  return n;
}
double* mxGetPr(const mxArray* a) { return (double*)a->re.data(); }
void* mxGetData(const mxArray* a) { return (void*)a->re.data(); }
void* mxGetImagData(const mxArray* a) { return a->complex ? (void*)a->im.data() : nullptr; }
double mxGetScalar(const mxArray* a) { return numel(a) ? get(a->re, a->cls, 0) : 0.0; }
// MATLAB returns a copy the caller may destroy; the gateways only read it, so the
// shim returns the object's own value
mxArray* mxGetProperty(const mxArray* a, mwSize, const char* name) {
  auto it = a->props.find(name);
  return it == a->props.end() ? nullptr : it->second;
}
mxArray* mxDuplicateArray(const mxArray* a) { return copy(a); }
mxArray* mxCreateString(const char* s) {
  mxArray* a = make(mxCHAR_CLASS, {1, strlen(s)}, false);
  a->re.assign(s, s + strlen(s));   // kept as bytes (the shim's isa reads them back)
  return a;
}
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) { return make(mxDOUBLE_CLASS, {m, n}, c == mxCOMPLEX); }
mxArray* mxCreateNumericMatrix(mwSize m, mwSize n, mxClassID cls, mxComplexity c) {
  return make(cls, {m, n}, c == mxCOMPLEX);
}
mxArray* mxCreateNumericArray(mwSize nd, const mwSize* d, mxClassID cls, mxComplexity c) {
  return make(cls, std::vector<mwSize>(d, d + nd), c == mxCOMPLEX);
}
void mxDestroyArray(mxArray* a) { delete a; }

// ---- the tests' side ----------------------------------------------------------
mxArray* shim_numeric(int cls, int ndim, const size_t* dims, const double* re, const double* im) {
  mxArray* a = make((mxClassID)cls, std::vector<mwSize>(dims, dims + ndim), im != nullptr);
  const size_t n = numel(a);
  for (size_t i = 0; i < n; ++i) {
    if (a->cls == mxDOUBLE_CLASS) {
      ((double*)a->re.data())[i] = re[i];
      if (im) ((double*)a->im.data())[i] = im[i];
    } else if (a->cls == mxSINGLE_CLASS) {
      ((float*)a->re.data())[i] = (float)re[i];
      if (im) ((float*)a->im.data())[i] = (float)im[i];
    } else if (a->cls == mxLOGICAL_CLASS) {
      a->re[i] = re[i] != 0.0;
    }
  }
  return a;
}
// supers: comma-separated superclasses (e.g. "windows.window")
mxArray* shim_object(const char* class_name, const char* supers) {
  mxArray* a = new mxArray_tag;
  a->cls = mxOBJECT_CLASS;
  a->class_name = class_name;
  a->dims = {1, 1};
  std::string s(supers ? supers : "");
  size_t p = 0;
  while (p < s.size()) {
    size_t q = s.find(',', p);
    if (q == std::string::npos) q = s.size();
    if (q > p) a->supers.push_back(s.substr(p, q - p));
    p = q + 1;
  }
  return a;
}
void shim_set_property(mxArray* obj, const char* name, mxArray* value) {
  delete obj->props[name];
  obj->props[name] = value;
}
void shim_set_callback(Callback cb) { g_callback = cb; }
int shim_class(const mxArray* a) { return (int)a->cls; }
int shim_is_complex(const mxArray* a) { return a->complex ? 1 : 0; }
int shim_ndim(const mxArray* a) { return (int)a->dims.size(); }
void shim_dims(const mxArray* a, size_t* d) {
  for (size_t i = 0; i < a->dims.size(); ++i) d[i] = a->dims[i];
}
void shim_read(const mxArray* a, double* re, double* im) {
  const size_t n = numel(a);
  for (size_t i = 0; i < n; ++i) {
    re[i] = get(a->re, a->cls, i);
    if (im) im[i] = a->complex ? get(a->im, a->cls, i) : 0.0;
  }
}
void shim_free(mxArray* a) { delete a; }
// runs the gateway; 0 on success, 1 if it raised an error (identifier and message copied out)
int shim_call(int nlhs, mxArray** plhs, int nrhs, const mxArray** prhs, char* id, int id_len, char* msg, int msg_len) {
  try {
    for (int i = 0; i < nlhs; ++i) plhs[i] = nullptr;
    mexFunction(nlhs, plhs, nrhs, prhs);
    return 0;
  } catch (const MexError& e) {
    snprintf(id, (size_t)id_len, "%s", e.id.c_str());
    snprintf(msg, (size_t)msg_len, "%s", e.msg.c_str());
    return 1;
  }
}

}  // extern "C"
