/* The part of the MATLAB MEX C API (separate-complex, mxGetImagData) that the
   gateways in f_number_gb300/mex use.  MATLAB is not present here: these are
   implemented by tests/mexshim/mexshim.cpp, a minimal stand-in that lets the
   gateways run under the tests.  mexErrMsgIdAndTxt does not return (the shim
   throws, as MATLAB longjmps out of the gateway). */
#pragma once
#include <stddef.h>
#include <stdio.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
typedef enum {
  mxUNKNOWN_CLASS = 0,
  mxCHAR_CLASS = 4,
  mxLOGICAL_CLASS = 3,
  mxDOUBLE_CLASS = 6,
  mxSINGLE_CLASS = 7,
  mxOBJECT_CLASS = 18
} mxClassID;
#ifdef __cplusplus
extern "C" {
#endif
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexCallMATLAB(int nlhs, mxArray* plhs[], int nrhs, mxArray* prhs[], const char* name);
bool mxIsDouble(const mxArray*);
bool mxIsComplex(const mxArray*);
bool mxIsScalar(const mxArray*);
bool mxIsEmpty(const mxArray*);
bool mxIsClass(const mxArray*, const char*);
bool mxIsLogicalScalarTrue(const mxArray*);
mwSize mxGetNumberOfDimensions(const mxArray*);
mwSize mxGetNumberOfElements(const mxArray*);
const mwSize* mxGetDimensions(const mxArray*);
size_t mxGetM(const mxArray*);
size_t mxGetN(const mxArray*);
double* mxGetPr(const mxArray*);
void* mxGetData(const mxArray*);
void* mxGetImagData(const mxArray*);
double mxGetScalar(const mxArray*);
mxArray* mxGetProperty(const mxArray*, mwSize, const char*);
mxArray* mxDuplicateArray(const mxArray*);
mxArray* mxCreateString(const char*);
mxArray* mxCreateDoubleMatrix(mwSize, mwSize, mxComplexity);
mxArray* mxCreateNumericMatrix(mwSize, mwSize, mxClassID, mxComplexity);
mxArray* mxCreateNumericArray(mwSize, const mwSize*, mxClassID, mxComplexity);
void mxDestroyArray(mxArray*);
#ifdef __cplusplus
}
#endif
