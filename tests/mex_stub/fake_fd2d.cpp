// fake_fd2d.cpp -- TEST DOUBLE of the six libfd2d entry points the MEX gateways
// call.  Each solver call records what it received (configuration, counts,
// which pointers are NULL, sums of the arrays) as one line of text that the
// Python tests read back with fake_last_call(), and fills its outputs with
// index patterns so the tests can check how the gateway hands them to MATLAB.
// fake_set_status() makes the next solver call fail.  Not part of the library.
#include <cstdio>
#include <cstring>
#include <string>

#include "fd2d.h"

namespace {

std::string g_last;
fd2d_status g_status = FD2D_OK;
std::string g_msg = "ok";
int g_ctx_dummy = 0;
int g_precision = -1;

double sum(const double* p, long n) {
  double s = 0.0;
  for (long i = 0; p && i < n; ++i) s += p[i];
  return s;
}
double sumf(const float* p, long n) {
  double s = 0.0;
  for (long i = 0; p && i < n; ++i) s += p[i];
  return s;
}

void add(std::string& s, const char* key, double v) {
  char b[96];
  std::snprintf(b, sizeof b, "%s=%.17g ", key, v);
  s += b;
}
void addp(std::string& s, const char* key, const void* p) { add(s, key, p ? 1.0 : 0.0); }

void cfg_fields(std::string& s, const fd2d_config* c) {
  add(s, "Lx", c->Lx); add(s, "Lz", c->Lz); add(s, "nx", c->nx); add(s, "nz", c->nz); add(s, "dt", c->dt);
  add(s, "nt", c->nt); add(s, "order", c->order); add(s, "nb", c->n_basis_fct); add(s, "fw", c->fw_nth);
  add(s, "K", c->n_sample); add(s, "f0", c->f_sample[0]); add(s, "fK", c->f_sample[c->n_sample - 1]);
  add(s, "fs", c->freq_samp); add(s, "width", c->absorb_width); add(s, "left", c->absorb_left);
  add(s, "right", c->absorb_right); add(s, "top", c->absorb_top); add(s, "bottom", c->absorb_bottom);
}

fd2d_status finish() {
  const fd2d_status s = g_status;
  g_status = FD2D_OK;
  return s;
}

}  // namespace

extern "C" {

fd2d_status fd2d_ctx_create(int32_t, int32_t precision, fd2d_ctx** out) {
  g_precision = precision;
  *out = reinterpret_cast<fd2d_ctx*>(&g_ctx_dummy);
  return FD2D_OK;
}
fd2d_status fd2d_ctx_destroy(fd2d_ctx*) { return FD2D_OK; }
const char* fd2d_last_error(const fd2d_ctx*) { return g_msg.c_str(); }

fd2d_status fd2d_query_sizes(const fd2d_config* c, int32_t nr, fd2d_sizes* z) {
  if (c->nx < 2 || c->nz < 2 || c->nt < 1 || c->n_sample < 1 || c->fw_nth < 1) {
    g_msg = "bad configuration";
    return FD2D_ERR_ARG;
  }
  std::memset(z, 0, sizeof *z);
  z->ntc = 2 * c->nt - 1;
  for (int n = c->nt; n <= 2 * c->nt - 1; ++n) z->n_fw_green += (n % c->fw_nth == 0);
  z->n_fw_corr = z->ntc / c->fw_nth;
  z->n_kernel_planes = c->n_basis_fct ? c->n_basis_fct + 1 : 2;
  z->npts = (int64_t)c->nx * c->nz;
  z->G_fft = z->npts * c->n_sample;
  z->seis_green = (int64_t)nr * c->nt;
  z->seis_corr = (int64_t)nr * z->ntc;
  return FD2D_OK;
}

fd2d_status fd2d_forward1_green(fd2d_ctx*, const fd2d_config* c, const double* mu, const double* rho,
                                const double* src, int32_t ns, const double* rec, int32_t nr, int32_t mode,
                                const double* dmu, const float* G_in, int32_t n_G_in, double* G_re, double* G_im,
                                float* G_out, double* seis) {
  const long np = (long)c->nx * c->nz;
  std::string s = "forward1 ";
  cfg_fields(s, c);
  add(s, "precision", g_precision);
  add(s, "mu", sum(mu, np)); add(s, "rho", sum(rho, np)); add(s, "src", sum(src, 2L * ns)); add(s, "ns", ns);
  add(s, "rec", sum(rec, 2L * nr)); add(s, "nr", nr); add(s, "mode", mode); addp(s, "dmu_set", dmu);
  addp(s, "G_in_set", G_in); add(s, "n_G_in", n_G_in); addp(s, "G_out_set", G_out);
  g_last = s;
  for (long i = 0; i < np * c->n_sample; ++i) {
    G_re[i] = (double)i;
    G_im[i] = -0.5 * (double)i;
  }
  for (long i = 0; i < (long)nr * c->nt; ++i) seis[i] = 0.25 * (double)i;
  if (G_out) {
    long n_fw = 0;
    for (int n = c->nt; n <= 2 * c->nt - 1; ++n) n_fw += (n % c->fw_nth == 0);
    for (long i = 0; i < np * n_fw; ++i) G_out[i] = (float)i;
  }
  return finish();
}

fd2d_status fd2d_forward2_correlation(fd2d_ctx*, const fd2d_config* c, const double* mu, const double* rho,
                                      const double* G_re, const double* G_im, int32_t n_G, const double* spectrum,
                                      int32_t n_src, const double* sd, int32_t n_dist, const double* rec,
                                      int32_t nr, int32_t mode, const double* dmu, const float* C_in,
                                      int32_t n_C_in, double* seis, float* C_out) {
  const long np = (long)c->nx * c->nz, ntc = 2L * c->nt - 1;
  std::string s = "correlation ";
  cfg_fields(s, c);
  add(s, "mu", sum(mu, np)); add(s, "rho", sum(rho, np)); add(s, "G_re", sum(G_re, np * n_G));
  add(s, "G_im", sum(G_im, np * n_G)); add(s, "n_G", n_G); add(s, "spectrum", sum(spectrum, (long)c->n_sample * n_src));
  add(s, "n_src", n_src); add(s, "sd", sum(sd, np * n_dist)); add(s, "n_dist", n_dist); add(s, "rec", sum(rec, 2L * nr));
  add(s, "nr", nr); add(s, "mode", mode); addp(s, "dmu_set", dmu); addp(s, "C_in_set", C_in);
  add(s, "n_C_in", n_C_in); add(s, "C_in", sumf(C_in, np * n_C_in)); addp(s, "C_out_set", C_out);
  g_last = s;
  for (long i = 0; i < nr * ntc; ++i) seis[i] = 2.0 * (double)i;
  if (C_out)
    for (long i = 0; i < np * (ntc / c->fw_nth); ++i) C_out[i] = -(float)i;
  return finish();
}

fd2d_status fd2d_noise_adjoint(fd2d_ctx*, const fd2d_config* c, const double* mu, const double* rho,
                               const float* u_fwd, int32_t n_u_fwd, const double* stf_re, const double* stf_im,
                               const int64_t stf_dims[3], const double* src, int32_t ns, const double* rec,
                               int32_t nr, const double* spectrum, int32_t n_src, const double* sd, int32_t n_dist,
                               const double* G_re, const double* G_im, int32_t n_G, int32_t mode, const double* dmu,
                               const float* u_in, int32_t n_u_in, double* K, double* sf_re, double* sf_im,
                               float* u_out, double* seis) {
  const long np = (long)c->nx * c->nz, ntc = 2L * c->nt - 1;
  const long nstf = (long)(stf_dims[0] * stf_dims[1] * stf_dims[2]);
  std::string s = "adjoint ";
  cfg_fields(s, c);
  add(s, "mu", sum(mu, np)); add(s, "u_fwd", sumf(u_fwd, np * n_u_fwd)); add(s, "n_u_fwd", n_u_fwd);
  add(s, "stf_re", sum(stf_re, nstf)); add(s, "stf_im", sum(stf_im, nstf)); add(s, "d0", (double)stf_dims[0]);
  add(s, "d1", (double)stf_dims[1]); add(s, "d2", (double)stf_dims[2]); add(s, "src", sum(src, 2L * ns));
  add(s, "ns", ns); add(s, "nr", nr); addp(s, "spectrum_set", spectrum); add(s, "n_src", n_src);
  addp(s, "sd_set", sd); add(s, "n_dist", n_dist); addp(s, "G_set", G_re); add(s, "G_re", sum(G_re, np * n_G));
  add(s, "n_G", n_G); add(s, "mode", mode); addp(s, "dmu_set", dmu); addp(s, "u_in_set", u_in);
  add(s, "n_u_in", n_u_in); addp(s, "u_out_set", u_out);
  g_last = s;
  const long kp = c->n_basis_fct ? c->n_basis_fct + 1 : 2;
  for (long i = 0; i < np * kp; ++i) K[i] = 3.0 * (double)i;
  for (long i = 0; i < np * c->n_sample; ++i) {
    sf_re[i] = (double)i;
    sf_im[i] = 1.0 + (double)i;
  }
  if (u_out)
    for (long i = 0; i < np * (ntc / c->fw_nth); ++i) u_out[i] = 0.5f * (float)i;
  for (long i = 0; i < nr * ntc; ++i) seis[i] = -(double)i;
  return finish();
}

// ---- test entry points ----------------------------------------------------------------
int fake_last_call(char* buf, int len) {
  std::snprintf(buf, (size_t)len, "%s", g_last.c_str());
  return (int)g_last.size();
}
void fake_set_status(int status, const char* msg) {
  g_status = (fd2d_status)status;
  g_msg = msg;
}

}  // extern "C"
