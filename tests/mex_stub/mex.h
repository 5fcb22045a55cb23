/* mex.h -- TEST DOUBLE of the MATLAB MEX C API, only what fd2d_mex.cpp uses.
 *
 * Declarations follow MathWorks' published MEX/Matrix API (R2018a interleaved
 * complex: mxGetDoubles, mxGetSingles, mxGetComplexDoubles).  The
 * implementations in mex_runtime.cpp keep arrays in plain heap buffers so that
 * the gateways can be compiled and exercised on a machine without MATLAB:
 * mexErrMsgIdAndTxt throws instead of returning to the MATLAB prompt, and
 * mexCallMATLAB answers only the three configuration getters the gateways
 * call.  Not part of the library. */
#pragma once

#include <cstddef>

typedef size_t mwSize;
typedef struct mxArray_tag mxArray;
typedef enum { mxUNKNOWN_CLASS = 0, mxCHAR_CLASS = 4, mxDOUBLE_CLASS = 6, mxSINGLE_CLASS = 7 } mxClassID;
typedef enum { mxREAL = 0, mxCOMPLEX = 1 } mxComplexity;
typedef struct {
  double real, imag;
} mxComplexDouble;

extern "C" {
mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity complexity);
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity complexity);
void mxDestroyArray(mxArray* a);
double* mxGetDoubles(const mxArray* a);
float* mxGetSingles(const mxArray* a);
mxComplexDouble* mxGetComplexDoubles(const mxArray* a);
size_t mxGetM(const mxArray* a);
size_t mxGetN(const mxArray* a);
mwSize mxGetNumberOfDimensions(const mxArray* a);
const mwSize* mxGetDimensions(const mxArray* a);
size_t mxGetNumberOfElements(const mxArray* a);
double mxGetScalar(const mxArray* a);
bool mxIsComplex(const mxArray* a);
bool mxIsDouble(const mxArray* a);
bool mxIsSingle(const mxArray* a);
bool mxIsEmpty(const mxArray* a);
int mexCallMATLAB(int nlhs, mxArray* plhs[], int nrhs, mxArray* prhs[], const char* name);
void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...);
int mexAtExit(void (*fn)(void));
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]);
}
