// fd2d_mex.cpp -- MATLAB MEX gateways run_forward1_green_mex,
// run_forward2_correlation_mex and run_noise_adjoint_mex over libfd2d.
//
// The reference's callers reach the solvers under these names
// (code/calculate_data.m:195,198; inversion/optlib_callback_fct/
// eval_objective_and_gradient.m:49-104; eval_hessian_vector_product.m:58-170),
// normally the MATLAB-Coder MEX files built by code/mex_functions/compile_all.m.
// Built from this file instead, the same names run on the GPU:
//
//   mex -R2018a -DFD2D_MEX_FORWARD1    -output run_forward1_green_mex       fd2d_mex.cpp -I<repo>/include -L<lib> -lfd2d
//   mex -R2018a -DFD2D_MEX_CORRELATION -output run_forward2_correlation_mex fd2d_mex.cpp -I<repo>/include -L<lib> -lfd2d
//   mex -R2018a -DFD2D_MEX_ADJOINT     -output run_noise_adjoint_mex        fd2d_mex.cpp -I<repo>/include -L<lib> -lfd2d
//
// Argument lists, types and empties follow the codegen specification
// (code/mex_functions/compile_all.m:5-34): complex double 3-D (G_fft, stf),
// real double 2-D (mu, rho, spectrum, dmu), n-by-2 double (src, rec), scalar
// mode, real double 3-D (source_dist), single 3-D (G_in, C_in, u_fwd, u_in).
// The hidden configuration of the MATLAB solvers is read at every call from
// input_parameters(), input_interferometry() and absorb_specs() on the MATLAB
// path, so editing those files takes effect without recompiling.
// MATLAB's interleaved complex arrays are split into the library's real and
// imaginary planes and merged back.  Errors raise "fd2d:<status>" MATLAB errors.
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fd2d.h"
#include "mex.h"

namespace {

fd2d_ctx* g_ctx = nullptr;

void at_exit() {
  if (g_ctx) fd2d_ctx_destroy(g_ctx);
  g_ctx = nullptr;
}

void fail(fd2d_status s, const char* what) {
  const std::string id = "fd2d:" + std::to_string((int)s);
  mexErrMsgIdAndTxt(id.c_str(), "%s: %s", what, fd2d_last_error(g_ctx));
}

fd2d_ctx* context() {
  if (!g_ctx) {
    // The gateways stand in for the reference's FP64 solvers, so they compute
    // in FP64 unless the caller opts in to the FP32 form (relative L2 error
    // <= 1e-4 against FP64, about 80x the throughput): FD2D_PRECISION=fp32.
    const char* p = std::getenv("FD2D_PRECISION");
    const int prec = (p && std::strcmp(p, "fp32") == 0) ? FD2D_PREC_FP32 : FD2D_PREC_FP64;
    fd2d_status s = fd2d_ctx_create(0, prec, &g_ctx);
    if (s != FD2D_OK) fail(s, "fd2d_ctx_create");
    mexAtExit(at_exit);
  }
  return g_ctx;
}

double scalar_of(mxArray* a) {
  const double v = mxGetScalar(a);
  mxDestroyArray(a);
  return v;
}

// fd2d_config from the three MATLAB getters; `freqs` keeps f_sample alive.
fd2d_config config(std::vector<double>& freqs) {
  fd2d_config c{};
  mxArray* ip[11];
  mexCallMATLAB(11, ip, 0, nullptr, "input_parameters");
  c.Lx = scalar_of(ip[0]);
  c.Lz = scalar_of(ip[1]);
  c.nx = (int32_t)scalar_of(ip[2]);
  c.nz = (int32_t)scalar_of(ip[3]);
  c.dt = scalar_of(ip[4]);
  c.nt = (int32_t)scalar_of(ip[5]);
  c.order = (int32_t)scalar_of(ip[6]);
  mxDestroyArray(ip[7]);  // model_type
  mxDestroyArray(ip[8]);  // source_type
  c.n_basis_fct = (int32_t)scalar_of(ip[9]);
  c.fw_nth = (int32_t)scalar_of(ip[10]);
  mxArray* ii[5];
  mexCallMATLAB(5, ii, 0, nullptr, "input_interferometry");
  const double* f = mxGetDoubles(ii[0]);
  freqs.assign(f, f + mxGetNumberOfElements(ii[0]));
  c.n_sample = (int32_t)freqs.size();
  c.f_sample = freqs.data();
  c.freq_samp = (int32_t)mxGetScalar(ii[4]);
  for (mxArray* a : ii) mxDestroyArray(a);
  mxArray* ab[5];
  mexCallMATLAB(5, ab, 0, nullptr, "absorb_specs");
  c.absorb_width = scalar_of(ab[0]);
  c.absorb_left = (int32_t)scalar_of(ab[1]);
  c.absorb_right = (int32_t)scalar_of(ab[2]);
  c.absorb_top = (int32_t)scalar_of(ab[3]);
  c.absorb_bottom = (int32_t)scalar_of(ab[4]);
  return c;
}

bool empty(const mxArray* a) { return !a || mxIsEmpty(a); }

const double* dbl(const mxArray* a, const char* name) {
  if (empty(a)) return nullptr;
  if (!mxIsDouble(a) || mxIsComplex(a)) mexErrMsgIdAndTxt("fd2d:type", "%s must be real double", name);
  return mxGetDoubles(a);
}

const float* sgl(const mxArray* a, const char* name, int32_t* planes) {
  *planes = 0;
  if (empty(a)) return nullptr;
  if (!mxIsSingle(a) || mxIsComplex(a)) mexErrMsgIdAndTxt("fd2d:type", "%s must be real single", name);
  const mwSize nd = mxGetNumberOfDimensions(a);
  *planes = nd >= 3 ? (int32_t)mxGetDimensions(a)[2] : 1;
  return mxGetSingles(a);
}

// Rows of an n-by-2 position array.
int32_t rows2(const mxArray* a, const char* name) {
  if (empty(a)) return 0;
  if (mxGetN(a) != 2) mexErrMsgIdAndTxt("fd2d:shape", "%s must be n-by-2", name);
  return (int32_t)mxGetM(a);
}

// Complex (or real) double array -> split planes.
void split(const mxArray* a, std::vector<double>& re, std::vector<double>& im) {
  const size_t n = mxGetNumberOfElements(a);
  re.resize(n);
  im.assign(n, 0.0);
  if (mxIsComplex(a)) {
    const mxComplexDouble* z = mxGetComplexDoubles(a);
    for (size_t i = 0; i < n; ++i) {
      re[i] = z[i].real;
      im[i] = z[i].imag;
    }
  } else {
    std::memcpy(re.data(), mxGetDoubles(a), n * sizeof(double));
  }
}

mxArray* merge(const std::vector<double>& re, const std::vector<double>& im, mwSize nx, mwSize nz, mwSize K) {
  const mwSize dims[3] = {nx, nz, K};
  mxArray* a = mxCreateNumericArray(3, dims, mxDOUBLE_CLASS, mxCOMPLEX);
  mxComplexDouble* z = mxGetComplexDoubles(a);
  for (size_t i = 0; i < re.size(); ++i) {
    z[i].real = re[i];
    z[i].imag = im[i];
  }
  return a;
}

mxArray* singles(mwSize nx, mwSize nz, mwSize k) {
  const mwSize dims[3] = {nx, nz, k};
  return mxCreateNumericArray(3, dims, mxSINGLE_CLASS, mxREAL);
}

int32_t third(const mxArray* a) {
  if (empty(a)) return 0;
  return mxGetNumberOfDimensions(a) >= 3 ? (int32_t)mxGetDimensions(a)[2] : 1;
}

}  // namespace

#if defined(FD2D_MEX_FORWARD1)
// [G_fft, G_out, seismograms] = run_forward1_green_mex(mu, rho, src, rec, mode, dmu, G_in)
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 7) mexErrMsgIdAndTxt("fd2d:nargin", "run_forward1_green_mex takes 7 inputs");
  std::vector<double> freqs;
  const fd2d_config c = config(freqs);
  const int32_t ns = rows2(prhs[2], "src"), nr = rows2(prhs[3], "rec");
  fd2d_sizes z;
  fd2d_status s = fd2d_query_sizes(&c, nr, &z);
  if (s != FD2D_OK) fail(s, "configuration");
  int32_t n_G_in = 0;
  const float* G_in = sgl(prhs[6], "G_in", &n_G_in);
  const int mode = (int)mxGetScalar(prhs[4]);
  std::vector<double> re(z.G_fft), im(z.G_fft);
  mxArray* G_out = singles(c.nx, c.nz, mode ? z.n_fw_green : 0);
  mxArray* seis = mxCreateDoubleMatrix(nr, c.nt, mxREAL);
  s = fd2d_forward1_green(context(), &c, dbl(prhs[0], "mu"), dbl(prhs[1], "rho"), dbl(prhs[2], "src"), ns,
                          dbl(prhs[3], "rec"), nr, mode, dbl(prhs[5], "dmu"), G_in, n_G_in, re.data(), im.data(),
                          mode ? mxGetSingles(G_out) : nullptr, mxGetDoubles(seis));
  if (s != FD2D_OK) fail(s, "run_forward1_green");
  plhs[0] = merge(re, im, c.nx, c.nz, c.n_sample);
  if (nlhs > 1) plhs[1] = G_out; else mxDestroyArray(G_out);
  if (nlhs > 2) plhs[2] = seis; else mxDestroyArray(seis);
}
#elif defined(FD2D_MEX_CORRELATION)
// [seismograms, C_out] = run_forward2_correlation_mex(mu, rho, G_fft, spectrum, source_dist, rec, mode, dmu, C_in)
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 9) mexErrMsgIdAndTxt("fd2d:nargin", "run_forward2_correlation_mex takes 9 inputs");
  std::vector<double> freqs;
  const fd2d_config c = config(freqs);
  const int32_t nr = rows2(prhs[5], "rec");
  fd2d_sizes z;
  fd2d_status s = fd2d_query_sizes(&c, nr, &z);
  if (s != FD2D_OK) fail(s, "configuration");
  std::vector<double> gre, gim;
  split(prhs[2], gre, gim);
  int32_t n_C_in = 0;
  const float* C_in = sgl(prhs[8], "C_in", &n_C_in);
  const int mode = (int)mxGetScalar(prhs[6]);
  const int32_t n_src = empty(prhs[3]) ? 0 : (int32_t)mxGetN(prhs[3]);
  mxArray* seis = mxCreateDoubleMatrix(nr, z.ntc, mxREAL);
  mxArray* C_out = singles(c.nx, c.nz, mode ? z.n_fw_corr : 0);
  s = fd2d_forward2_correlation(context(), &c, dbl(prhs[0], "mu"), dbl(prhs[1], "rho"), gre.data(), gim.data(),
                                third(prhs[2]), dbl(prhs[3], "spectrum"), n_src, dbl(prhs[4], "source_dist"),
                                third(prhs[4]), dbl(prhs[5], "rec"), nr, mode, dbl(prhs[7], "dmu"), C_in, n_C_in,
                                mxGetDoubles(seis), mode ? mxGetSingles(C_out) : nullptr);
  if (s != FD2D_OK) fail(s, "run_forward2_correlation");
  plhs[0] = seis;
  if (nlhs > 1) plhs[1] = C_out; else mxDestroyArray(C_out);
}
#elif defined(FD2D_MEX_ADJOINT)
// [K, stf_fft, u_out, seismograms] = run_noise_adjoint_mex(mu, rho, u_fwd, stf, src, rec, spectrum,
//                                                          source_dist, G_fft, mode, dmu, u_in)
void mexFunction(int nlhs, mxArray* plhs[], int nrhs, const mxArray* prhs[]) {
  if (nrhs != 12) mexErrMsgIdAndTxt("fd2d:nargin", "run_noise_adjoint_mex takes 12 inputs");
  std::vector<double> freqs;
  const fd2d_config c = config(freqs);
  const int32_t ns = rows2(prhs[4], "src"), nr = rows2(prhs[5], "rec");
  fd2d_sizes z;
  fd2d_status s = fd2d_query_sizes(&c, nr, &z);
  if (s != FD2D_OK) fail(s, "configuration");
  int32_t n_u_fwd = 0, n_u_in = 0;
  const float* u_fwd = sgl(prhs[2], "u_fwd", &n_u_fwd);
  const float* u_in = sgl(prhs[11], "u_in", &n_u_in);
  std::vector<double> sre, sim, gre, gim;
  int64_t dims[3] = {0, 0, 0};
  if (!empty(prhs[3])) {
    split(prhs[3], sre, sim);
    const mwSize* d = mxGetDimensions(prhs[3]);
    const mwSize nd = mxGetNumberOfDimensions(prhs[3]);
    dims[0] = (int64_t)d[0];
    dims[1] = (int64_t)d[1];
    dims[2] = nd >= 3 ? (int64_t)d[2] : 1;
  }
  if (!empty(prhs[8])) split(prhs[8], gre, gim);
  const int mode = (int)mxGetScalar(prhs[9]);
  const int32_t n_src = empty(prhs[6]) ? 0 : (int32_t)mxGetN(prhs[6]);
  const mwSize kd[3] = {(mwSize)c.nx, (mwSize)c.nz, (mwSize)z.n_kernel_planes};
  mxArray* K = mxCreateNumericArray(3, kd, mxDOUBLE_CLASS, mxREAL);
  std::vector<double> fre(z.G_fft), fim(z.G_fft);
  const bool save_u = mode == 11 || mode == 13;
  mxArray* u_out = singles(c.nx, c.nz, save_u ? z.n_fw_corr : 0);
  mxArray* seis = mxCreateDoubleMatrix(nr, z.ntc, mxREAL);
  s = fd2d_noise_adjoint(context(), &c, dbl(prhs[0], "mu"), dbl(prhs[1], "rho"), u_fwd, n_u_fwd,
                         sre.empty() ? nullptr : sre.data(), sim.empty() ? nullptr : sim.data(), dims,
                         dbl(prhs[4], "src"), ns, dbl(prhs[5], "rec"), nr, dbl(prhs[6], "spectrum"), n_src,
                         dbl(prhs[7], "source_dist"), third(prhs[7]), gre.empty() ? nullptr : gre.data(),
                         gim.empty() ? nullptr : gim.data(), third(prhs[8]), mode, dbl(prhs[10], "dmu"), u_in,
                         n_u_in, mxGetDoubles(K), fre.data(), fim.data(), save_u ? mxGetSingles(u_out) : nullptr,
                         mxGetDoubles(seis));
  if (s != FD2D_OK) fail(s, "run_noise_adjoint");
  plhs[0] = K;
  if (nlhs > 1) plhs[1] = merge(fre, fim, c.nx, c.nz, c.n_sample);
  if (nlhs > 2) plhs[2] = u_out; else mxDestroyArray(u_out);
  if (nlhs > 3) plhs[3] = seis; else mxDestroyArray(seis);
}
#else
#error "define one of FD2D_MEX_FORWARD1, FD2D_MEX_CORRELATION, FD2D_MEX_ADJOINT"
#endif
