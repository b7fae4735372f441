/* Declarations of the MATLAB MEX C API used by the gateways in
   f_number_gb300/mex (signature check only: the functions are provided by
   MATLAB at link time).  Separate-complex API (mxGetImagData). */
#pragma once
#include <stddef.h>
#include <stdio.h>
typedef struct mxArray_tag mxArray;
typedef size_t mwSize;
typedef enum { mxREAL, mxCOMPLEX } mxComplexity;
typedef enum { mxUNKNOWN_CLASS, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
#ifdef __cplusplus
extern "C" {
#endif
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
void mxDestroyArray(mxArray*);
#ifdef __cplusplus
}
#endif
