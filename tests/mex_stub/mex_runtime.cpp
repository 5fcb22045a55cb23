// mex_runtime.cpp -- TEST DOUBLE of the MATLAB MEX runtime (see mex.h), plus
// stub_* entry points through which the Python tests build arguments, call
// mexFunction and read the results.  Not part of the library.
#include "mex.h"

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

struct mxArray_tag {
  mxClassID cls = mxDOUBLE_CLASS;
  bool complex = false;
  std::vector<mwSize> dims;
  std::vector<unsigned char> data;  // column-major; complex doubles interleaved
  std::string text;                 // char arrays
};

namespace {

struct MexError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

size_t count(const std::vector<mwSize>& d) {
  size_t n = 1;
  for (mwSize v : d) n *= v;
  return n;
}

size_t elem_bytes(const mxArray* a) {
  return a->cls == mxSINGLE_CLASS ? 4 : (a->complex ? 16 : 8);
}

mxArray* make(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity c) {
  mxArray* a = new mxArray_tag;
  a->cls = cls;
  a->complex = c == mxCOMPLEX;
  a->dims.assign(dims, dims + ndim);
  while (a->dims.size() < 2) a->dims.push_back(1);
  while (a->dims.size() > 2 && a->dims.back() == 1) a->dims.pop_back();  // MATLAB drops trailing singletons
  a->data.assign(count(a->dims) * elem_bytes(a), 0);
  return a;
}

mxArray* scalar(double v) {
  const mwSize d[2] = {1, 1};
  mxArray* a = make(2, d, mxDOUBLE_CLASS, mxREAL);
  std::memcpy(a->data.data(), &v, 8);
  return a;
}

// configuration the three getters return
std::vector<double> g_ip(11, 0.0), g_f, g_ab(5, 0.0);
double g_fs = 5.0;
void (*g_exit)(void) = nullptr;

}  // namespace

extern "C" {

mxArray* mxCreateDoubleMatrix(mwSize m, mwSize n, mxComplexity c) {
  const mwSize d[2] = {m, n};
  return make(2, d, mxDOUBLE_CLASS, c);
}
mxArray* mxCreateNumericArray(mwSize ndim, const mwSize* dims, mxClassID cls, mxComplexity c) {
  return make(ndim, dims, cls, c);
}
void mxDestroyArray(mxArray* a) { delete a; }
double* mxGetDoubles(const mxArray* a) {
  return a->cls == mxDOUBLE_CLASS && !a->complex ? (double*)a->data.data() : nullptr;
}
float* mxGetSingles(const mxArray* a) { return a->cls == mxSINGLE_CLASS ? (float*)a->data.data() : nullptr; }
mxComplexDouble* mxGetComplexDoubles(const mxArray* a) {
  return a->cls == mxDOUBLE_CLASS && a->complex ? (mxComplexDouble*)a->data.data() : nullptr;
}
size_t mxGetM(const mxArray* a) { return a->dims[0]; }
size_t mxGetN(const mxArray* a) { return count(a->dims) / (a->dims[0] ? a->dims[0] : 1); }
mwSize mxGetNumberOfDimensions(const mxArray* a) { return a->dims.size(); }
const mwSize* mxGetDimensions(const mxArray* a) { return a->dims.data(); }
size_t mxGetNumberOfElements(const mxArray* a) { return count(a->dims); }
double mxGetScalar(const mxArray* a) {
  if (a->data.empty()) return 0.0;
  if (a->cls == mxSINGLE_CLASS) return *(const float*)a->data.data();
  return *(const double*)a->data.data();
}
bool mxIsComplex(const mxArray* a) { return a->complex; }
bool mxIsDouble(const mxArray* a) { return a->cls == mxDOUBLE_CLASS; }
bool mxIsSingle(const mxArray* a) { return a->cls == mxSINGLE_CLASS; }
bool mxIsEmpty(const mxArray* a) { return count(a->dims) == 0; }

int mexCallMATLAB(int nlhs, mxArray* plhs[], int, mxArray**, const char* name) {
  const std::string n(name);
  if (n == "input_parameters") {
    for (int i = 0; i < nlhs; ++i) {
      if (i == 8) {
        plhs[i] = make(0, nullptr, mxCHAR_CLASS, mxREAL);
        plhs[i]->text = "homogeneous";
      } else {
        plhs[i] = scalar(i < (int)g_ip.size() ? g_ip[i] : 0.0);
      }
    }
  } else if (n == "input_interferometry") {
    const mwSize d[2] = {1, g_f.size()};
    plhs[0] = make(2, d, mxDOUBLE_CLASS, mxREAL);
    std::memcpy(plhs[0]->data.data(), g_f.data(), g_f.size() * 8);
    for (int i = 1; i < nlhs; ++i) plhs[i] = scalar(i == 1 ? (double)g_f.size() : i == 4 ? g_fs : 0.0);
  } else if (n == "absorb_specs") {
    for (int i = 0; i < nlhs; ++i) plhs[i] = scalar(g_ab[i]);
  } else {
    throw MexError("mexCallMATLAB: unknown function " + n);
  }
  return 0;
}

void mexErrMsgIdAndTxt(const char* id, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  throw MexError(std::string(id) + "|" + buf);
}

int mexAtExit(void (*fn)(void)) {
  g_exit = fn;
  return 0;
}

// ---- test entry points ----------------------------------------------------------------
void stub_set_config(const double* ip11, const double* f, int K, double fs, const double* ab5) {
  g_ip.assign(ip11, ip11 + 11);
  g_f.assign(f, f + K);
  g_fs = fs;
  g_ab.assign(ab5, ab5 + 5);
}
mxArray* stub_array(int ndim, const size_t* dims, int cls, int complex) {
  return make((mwSize)ndim, dims, (mxClassID)cls, complex ? mxCOMPLEX : mxREAL);
}
void* stub_data(mxArray* a) { return a->data.data(); }
int stub_ndims(mxArray* a, size_t* dims) {
  for (size_t i = 0; i < a->dims.size(); ++i) dims[i] = a->dims[i];
  return (int)a->dims.size();
}
int stub_class(mxArray* a) { return (int)a->cls; }
int stub_is_complex(mxArray* a) { return a->complex ? 1 : 0; }
void stub_free(mxArray* a) { delete a; }
int stub_call(int nlhs, mxArray** plhs, int nrhs, mxArray** prhs, char* err, int errlen) {
  try {
    mexFunction(nlhs, plhs, nrhs, const_cast<const mxArray**>(prhs));
    return 0;
  } catch (const std::exception& e) {
    std::snprintf(err, (size_t)errlen, "%s", e.what());
    return 1;
  }
}
void stub_at_exit() {
  if (g_exit) g_exit();
  g_exit = nullptr;
}

}  // extern "C"
