// fd2d_oracle.cpp -- TEST INFRASTRUCTURE, not part of the product.
//
// FP64 CPU restatement of the fd2d_noise wave-propagation solvers.  It is the
// correctness oracle of the CUDA library and the timed CPU baseline; only the
// tests, the smoke check and the benchmark's CPU leg load it.
//
// It follows the MATLAB sources statement by statement, keeping their loop
// order and their expression order (no FMA contraction: build with
// -ffp-contract=off), so the FP64 GPU path is compared against the same
// arithmetic:
//   code/run_forward1_green.m        -> oracle_forward1_green
//   code/run_forward2_correlation.m  -> oracle_forward2_correlation
//   code/run_noise_adjoint.m         -> oracle_noise_adjoint
//   code/propagation/{div_s,dx_v,dz_v,init_absbound,define_computational_domain,
//                     integration_limits}.m -> the helpers below
// One MATLAB rule matters for parity: dx_v/dz_v applied to a `single` snapshot
// stack (G_in, C_in, u_in, u_fwd) evaluate in single-precision arithmetic
// (mixed single/double operations are carried out in single), and the result
// is stored into the double array `out`.  dxv_single/dzv_single reproduce that.
//
// Orders 6 and 8 are an extension: the reference implements only 2 and 4
// (code/propagation/dx_v.m:20-32 returns zeros otherwise).  Their coefficients
// are derived here by solving the staggered-grid Taylor conditions.
//
// Pinning: tests/golden holds vectors made by running the reference's own .m
// files through a MATLAB-subset interpreter (tests/golden/make_golden.py); the
// oracle is checked against them in tests/test_oracle_golden.py.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "../include/fd2d.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

fd2d_status fail(fd2d_status s, const std::string& msg) {
  g_err = msg;
  return s;
}

const double kEps = 2.220446049250313e-16;  // MATLAB eps

// MATLAB a:d:b, following the published construction of the colon operator
// (symmetric about the midpoint, end point snapped to b within tolerance).
std::vector<double> colon(double a, double d, double b) {
  std::vector<double> out;
  if (d == 0 || (d > 0 && a > b) || (d < 0 && a < b)) return out;
  double tol = 2.0 * kEps * std::max(std::fabs(a), std::fabs(b));
  double sig = d > 0 ? 1.0 : -1.0;
  long n;
  if (a == std::floor(a) && d == 1) {
    n = (long)(std::floor(b) - a);
  } else if (a == std::floor(a) && d == std::floor(d)) {
    double q = std::floor(a / d);
    double r = a - q * d;
    n = (long)(std::floor((b - r) / d) - q);
  } else {
    n = (long)std::round((b - a) / d);
    if (sig * (a + n * d - b) > tol) n = n - 1;
  }
  if (n < 0) return out;
  double last = a + n * d;
  if (a == std::floor(a) && d == std::floor(d)) {
    last = std::floor(last);
  } else if (sig * (last - b) > -tol) {
    last = b;
  }
  out.assign(n + 1, 0.0);
  for (long k = 0; k <= n / 2; ++k) {
    out[k] = a + k * d;
    out[n - k] = last - k * d;
  }
  if (n % 2 == 0) out[n / 2] = (a + last) / 2;
  return out;
}

// min(find(min(abs(x-p)) == abs(x-p))): nearest node, ties to the lower index.
int nearest(const std::vector<double>& x, double p) {
  double best = INFINITY;
  int idx = 0;
  for (size_t i = 0; i < x.size(); ++i) {
    double d = std::fabs(x[i] - p);
    if (d < best) { best = d; idx = (int)i; }
  }
  return idx;
}

// Staggered-grid coefficients c_1..c_r of order 2r: sum_m c_m (2m-1)^(2p-1) = [p==1].
std::vector<double> stagger_coeffs(int r) {
  std::vector<double> A(r * r), b(r, 0.0);
  for (int p = 0; p < r; ++p)
    for (int m = 0; m < r; ++m) A[p * r + m] = std::pow(2.0 * (m + 1) - 1.0, 2.0 * (p + 1) - 1.0);
  b[0] = 1.0;
  // Gaussian elimination with partial pivoting (r <= 4).
  for (int c = 0; c < r; ++c) {
    int piv = c;
    for (int i = c + 1; i < r; ++i)
      if (std::fabs(A[i * r + c]) > std::fabs(A[piv * r + c])) piv = i;
    for (int j = 0; j < r; ++j) std::swap(A[c * r + j], A[piv * r + j]);
    std::swap(b[c], b[piv]);
    for (int i = c + 1; i < r; ++i) {
      double f = A[i * r + c] / A[c * r + c];
      for (int j = c; j < r; ++j) A[i * r + j] -= f * A[c * r + j];
      b[i] -= f * b[c];
    }
  }
  std::vector<double> x(r);
  for (int i = r - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < r; ++j) s -= A[i * r + j] * x[j];
    x[i] = s / A[i * r + i];
  }
  return x;
}

struct Setup {
  int nx, nz, nt, order, r, nb, fw, fs, K;
  double Lx, Lz, dt, dx, dz, dw;
  std::vector<double> x, z, w, absbound, c;
  std::vector<float> cf;  // coefficients in single, for the single-precision operators
};

fd2d_status make_setup(const fd2d_config* cfg, Setup& s) {
  if (!cfg) return fail(FD2D_ERR_ARG, "cfg is NULL");
  if (cfg->nx < 2 || cfg->nz < 2 || cfg->nt < 1 || cfg->freq_samp < 1 || cfg->fw_nth < 1)
    return fail(FD2D_ERR_ARG, "bad scalar in configuration");
  if (cfg->n_sample < 2 || !cfg->f_sample) return fail(FD2D_ERR_ARG, "need n_sample >= 2 frequencies");
  if (!(cfg->order == 2 || cfg->order == 4 || cfg->order == 6 || cfg->order == 8))
    return fail(FD2D_ERR_ORDER, "order must be 2, 4, 6 or 8");
  if (cfg->n_basis_fct < 0 || cfg->n_basis_fct == 1)
    return fail(FD2D_ERR_SHAPE, "n_basis_fct must be 0 or >= 2");
  s.nx = cfg->nx; s.nz = cfg->nz; s.nt = cfg->nt; s.order = cfg->order; s.r = cfg->order / 2;
  s.nb = cfg->n_basis_fct; s.fw = cfg->fw_nth; s.fs = cfg->freq_samp; s.K = cfg->n_sample;
  s.Lx = cfg->Lx; s.Lz = cfg->Lz; s.dt = cfg->dt;
  // define_computational_domain.m:18-22
  s.dx = s.Lx / (s.nx - 1);
  s.dz = s.Lz / (s.nz - 1);
  s.x = colon(0.0, s.dx, s.Lx);
  s.z = colon(0.0, s.dz, s.Lz);
  if ((int)s.x.size() != s.nx || (int)s.z.size() != s.nz)
    return fail(FD2D_ERR_SHAPE, "0:dx:Lx does not have nx points");
  // input_interferometry.m:18-20
  s.w.resize(s.K);
  for (int k = 0; k < s.K; ++k) s.w[k] = 2 * M_PI * cfg->f_sample[k];
  s.dw = s.w[1] - s.w[0];
  // init_absbound.m:8-31, X'(i,j) = x(i), Z'(i,j) = z(j)
  double width = cfg->absorb_width;
  s.absbound.assign((size_t)s.nx * s.nz, 1.0);
  for (int j = 0; j < s.nz; ++j)
    for (int i = 0; i < s.nx; ++i) {
      double X = s.x[i], Z = s.z[j], a = 1.0;
      if (cfg->absorb_left == 1)
        a = a * ((double)(X > width) + std::exp(-((X - width) * (X - width)) / ((2 * width) * (2 * width))) * (double)(X <= width));
      if (cfg->absorb_right == 1)
        a = a * ((double)(X < (s.Lx - width)) + std::exp(-((X - (s.Lx - width)) * (X - (s.Lx - width))) / ((2 * width) * (2 * width))) * (double)(X >= (s.Lx - width)));
      if (cfg->absorb_bottom == 1)
        a = a * ((double)(Z > width) + std::exp(-((Z - width) * (Z - width)) / ((2 * width) * (2 * width))) * (double)(Z <= width));
      if (cfg->absorb_top == 1)
        a = a * ((double)(Z < (s.Lz - width)) + std::exp(-((Z - (s.Lz - width)) * (Z - (s.Lz - width))) / ((2 * width) * (2 * width))) * (double)(Z >= (s.Lz - width)));
      s.absbound[i + (size_t)s.nx * j] = a;
    }
  s.c = stagger_coeffs(s.r);
  s.cf.resize(s.r);
  for (int m = 0; m < s.r; ++m) s.cf[m] = (float)s.c[m];
  return FD2D_OK;
}

// ---- FD operators (div_s.m, dx_v.m, dz_v.m), 0-based, column-major ---------
// sxy is (nx-1)-by-nz, szy is nx-by-(nz-1), v and out of div_s are nx-by-nz.

void div_s(const Setup& s, const double* sxy, const double* szy, double* out) {
  const int nx = s.nx, nz = s.nz, r = s.r;
  const double dx = s.dx, dz = s.dz;
  const int ldx = nx - 1;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nz; ++j) {
    for (int i = 0; i < nx; ++i) {
      double o = 0.0;
      // x part: MATLAB i = r+1..nx-r  ->  0-based i = r..nx-r-1; sxy(i) 1-based = sxy[i-1] 0-based
      if (i >= r && i <= nx - r - 1) {
        const double* S = sxy + (size_t)ldx * j;
        if (s.order == 2) {
          o = (S[i] - S[i - 1]) / dx;
        } else if (s.order == 4) {
          o = 9 * (S[i] - S[i - 1]) / (8 * dx) - (S[i + 1] - S[i - 2]) / (24 * dx);
        } else {
          double acc = 0.0;
          for (int m = 1; m <= r; ++m) acc = acc + s.c[m - 1] * (S[i + m - 1] - S[i - m]);
          o = acc / dx;
        }
      }
      if (j >= r && j <= nz - r - 1) {
        auto Z = [&](int jj) { return szy[i + (size_t)nx * jj]; };
        if (s.order == 2) {
          o = o + (Z(j) - Z(j - 1)) / dz;
        } else if (s.order == 4) {
          o = o + 9 * (Z(j) - Z(j - 1)) / (8 * dz) - (Z(j + 1) - Z(j - 2)) / (24 * dz);
        } else {
          double acc = 0.0;
          for (int m = 1; m <= r; ++m) acc = acc + s.c[m - 1] * (Z(j + m - 1) - Z(j - m));
          o = o + acc / dz;
        }
      }
      out[i + (size_t)nx * j] = o;
    }
  }
}

// dx_v.m: out (nx-1)-by-nz; MATLAB i = r..nx-r -> 0-based i = r-1..nx-r-1 uses v(i+1..)
template <typename T>
inline double dxv_point(const Setup& s, const T* V, int i) {
  // V points at column j of v; i is the 0-based row of out.
  if (s.order == 2) return (V[i + 1] - V[i]) / s.dx;
  if (s.order == 4) return 9 * (V[i + 1] - V[i]) / (8 * s.dx) - (V[i + 2] - V[i - 1]) / (24 * s.dx);
  double acc = 0.0;
  for (int m = 1; m <= s.r; ++m) acc = acc + s.c[m - 1] * (V[i + m] - V[i - m + 1]);
  return acc / s.dx;
}

void dx_v(const Setup& s, const double* v, double* out) {
  const int nx = s.nx, nz = s.nz, r = s.r, ld = nx - 1;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nz; ++j)
    for (int i = 0; i < ld; ++i)
      out[i + (size_t)ld * j] = (i >= r - 1 && i <= nx - r - 1) ? dxv_point(s, v + (size_t)nx * j, i) : 0.0;
}

void dz_v(const Setup& s, const double* v, double* out) {
  const int nx = s.nx, nz = s.nz, r = s.r;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nz - 1; ++j)
    for (int i = 0; i < nx; ++i) {
      double o = 0.0;
      if (j >= r - 1 && j <= nz - r - 1) {
        auto V = [&](int jj) { return v[i + (size_t)nx * jj]; };
        if (s.order == 2) o = (V(j + 1) - V(j)) / s.dz;
        else if (s.order == 4) o = 9 * (V(j + 1) - V(j)) / (8 * s.dz) - (V(j + 2) - V(j - 1)) / (24 * s.dz);
        else {
          double acc = 0.0;
          for (int m = 1; m <= r; ++m) acc = acc + s.c[m - 1] * (V(j + m) - V(j - m + 1));
          o = acc / s.dz;
        }
      }
      out[i + (size_t)nx * j] = o;
    }
}

// Single-precision evaluation of dx_v/dz_v on a `single` field (see header).
// a(i) returns the single value at offset i along the derivative direction.
template <typename F>
inline float dv_single(const Setup& s, F a, int i, double h) {
  if (s.order == 2) return (a(i + 1) - a(i)) / (float)h;
  if (s.order == 4) {
    float t1 = (9.0f * (a(i + 1) - a(i))) / (float)(8 * h);
    float t2 = (a(i + 2) - a(i - 1)) / (float)(24 * h);
    return t1 - t2;
  }
  float acc = 0.0f;
  for (int m = 1; m <= s.r; ++m) acc = acc + s.cf[m - 1] * (a(i + m) - a(i - m + 1));
  return acc / (float)h;
}

// out (nx-1)-by-nz double holding single results; f is an nx-by-nz single field.
void dxv_single(const Setup& s, const float* f, double* out) {
  const int nx = s.nx, nz = s.nz, r = s.r, ld = nx - 1;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nz; ++j) {
    const float* F = f + (size_t)nx * j;
    auto a = [&](int ii) { return F[ii]; };
    for (int i = 0; i < ld; ++i)
      out[i + (size_t)ld * j] = (i >= r - 1 && i <= nx - r - 1) ? (double)dv_single(s, a, i, s.dx) : 0.0;
  }
}

void dzv_single(const Setup& s, const float* f, double* out) {
  const int nx = s.nx, nz = s.nz, r = s.r;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < nz - 1; ++j)
    for (int i = 0; i < nx; ++i) {
      auto a = [&](int jj) { return f[i + (size_t)nx * jj]; };
      out[i + (size_t)nx * j] = (j >= r - 1 && j <= nz - r - 1) ? (double)dv_single(s, a, j, s.dz) : 0.0;
    }
}

// single(C_in(:,:,a) - C_in(:,:,b)) -- the difference is a single-precision operation.
void single_diff(const float* A, const float* B, float* out, size_t n) {
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)n; ++p) out[p] = A[p] - B[p];
}

// integration_limits.m:4-12 (1-based limits).
std::vector<int> integration_limits(int K, int nb) {
  std::vector<int> lim(2 * nb);
  double step = (double)K / nb;
  for (int i = 1; i <= nb; ++i) {
    lim[2 * (i - 1)] = (int)std::floor((i - 1) * step + 1);
    lim[2 * (i - 1) + 1] = (int)std::floor(i * step);
  }
  return lim;
}

// interpol_matrix of run_forward2_correlation.m:121-165 (K-by-max(nb,1), column-major).
fd2d_status interpol_matrix(int K, int nb, std::vector<double>& M) {
  int ncol = nb == 0 ? 1 : nb;
  M.assign((size_t)K * ncol, nb == 0 ? 1.0 : 0.0);
  if (nb == 0) return FD2D_OK;
  std::vector<int> lim = integration_limits(K, nb);
  for (int k = 1; k <= K; ++k) {
    int ib = 0;
    for (int b = 1; b <= nb; ++b)
      if (k >= lim[2 * (b - 1)] && k <= lim[2 * (b - 1) + 1]) { ib = b; break; }
    if (ib == 0) return fail(FD2D_ERR_INDEX, "frequency outside every band");
    int lo = lim[2 * (ib - 1)], hi = lim[2 * (ib - 1) + 1];
    int ni = hi - lo + 1;
    int below = -1, above = -1;
    if (ib == 1) { above = 2; }
    else if (ib == nb) { below = ib - 1; }
    else { below = ib - 1; above = ib + 1; }
    int i = k - lo + 1;
    double half = ni / 2.0;
    auto at = [&](int kk, int cc) -> double& { return M[(kk - 1) + (size_t)K * (cc - 1)]; };
    if (i < half) {
      at(k, ib) = 1 - (half - i) / ni;
      if (below > 0) at(k, below) = (half - i) / ni;
    } else if (i == half) {
      at(k, ib) = 1;
    } else {
      at(k, ib) = 1 - (i - half) / ni;
      if (above > 0) {
        if (above > nb) return fail(FD2D_ERR_INDEX, "interpol_matrix grows beyond n_basis_fct");
        at(k, above) = (i - half) / ni;
      }
    }
  }
  return FD2D_OK;
}

// distribution(ix,iz,:) = interpol_matrix * squeeze(source_distribution(ix,iz,:)).
void make_distribution(const Setup& s, const std::vector<double>& M, int ncol,
                       const double* sd, std::vector<double>& dist) {
  const size_t np = (size_t)s.nx * s.nz;
  dist.assign(np * s.K, 0.0);
#pragma omp parallel for schedule(static)
  for (long long p = 0; p < (long long)np; ++p)
    for (int k = 0; k < s.K; ++k) {
      double acc = 0.0;
      for (int b = 0; b < ncol; ++b) acc = acc + M[k + (size_t)s.K * b] * sd[p + np * b];
      dist[p + np * k] = acc;
    }
}

inline void coeff(double s_, double th, double scale, double& re, double& im) {
  // 1/sqrt(2*pi) * exp(1i*th) * scale, evaluated left to right.
  re = (s_ * std::cos(th)) * scale;
  im = (s_ * std::sin(th)) * scale;
}

}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// Staggered-grid coefficients derived from the Taylor conditions (for tests).
int oracle_stagger_coeffs(int order, double* out) {
  if (order < 2 || order > 8 || order % 2) return 1;
  std::vector<double> c = stagger_coeffs(order / 2);
  for (size_t i = 0; i < c.size(); ++i) out[i] = c[i];
  return 0;
}

// Grid coordinates and taper (for tests of the host-side setup).
int oracle_setup_arrays(const fd2d_config* cfg, double* x, double* z, double* absbound) {
  Setup s;
  if (make_setup(cfg, s) != FD2D_OK) return 1;
  std::memcpy(x, s.x.data(), sizeof(double) * s.nx);
  std::memcpy(z, s.z.data(), sizeof(double) * s.nz);
  std::memcpy(absbound, s.absbound.data(), sizeof(double) * s.nx * s.nz);
  return 0;
}

int oracle_nearest_indices(const fd2d_config* cfg, const double* pts, int n, int* ix, int* iz) {
  Setup s;
  if (make_setup(cfg, s) != FD2D_OK) return 1;
  for (int i = 0; i < n; ++i) {
    ix[i] = nearest(s.x, pts[i]);
    iz[i] = nearest(s.z, pts[n + i]);
  }
  return 0;
}

int oracle_interpol_matrix(int K, int nb, double* out) {
  std::vector<double> M;
  if (interpol_matrix(K, nb, M) != FD2D_OK) return 1;
  std::memcpy(out, M.data(), sizeof(double) * M.size());
  return 0;
}

// ---------------------------------------------------------------------------
// code/run_forward1_green.m
// ---------------------------------------------------------------------------
int oracle_forward1_green(const fd2d_config* cfg, const double* mu, const double* rho,
                          const double* src, int ns, const double* rec, int nr, int mode,
                          const double* dmu, const float* G_in, int n_G_in,
                          double* G_re, double* G_im, float* G_out, double* seis) {
  Setup s;
  fd2d_status st = make_setup(cfg, s);
  if (st != FD2D_OK) return st;
  const int nx = s.nx, nz = s.nz, nt = s.nt, K = s.K, fs = s.fs, fw = s.fw;
  const size_t np = (size_t)nx * nz;
  const double dt = s.dt;
  std::vector<double> t = colon(0.0, dt, (nt - 1) * dt);  // :41
  if ((int)t.size() != nt) return fail(FD2D_ERR_SHAPE, "time axis length");
  std::vector<int> sid(2 * ns), rid(2 * nr);               // :45-60
  for (int i = 0; i < ns; ++i) { sid[2 * i] = nearest(s.x, src[i]); sid[2 * i + 1] = nearest(s.z, src[ns + i]); }
  for (int i = 0; i < nr; ++i) { rid[2 * i] = nearest(s.x, rec[i]); rid[2 * i + 1] = nearest(s.z, rec[nr + i]); }
  const double stf = 1.0e9;                                // :64
  const double sq = 1 / std::sqrt(2 * M_PI);
  // :72-90 DFT coefficients for n = nt..2nt-1 with mod(n, freq_samp) == 0
  std::vector<double> cre, cim;
  for (int n = nt; n <= 2 * nt - 1; ++n)
    if (n % fs == 0)
      for (int k = 0; k < K; ++k) {
        double re, im;
        coeff(sq, -(s.w[k] * t[n - nt]), dt, re, im);
        cre.push_back(re); cim.push_back(im);
      }
  std::vector<double> v(np, 0.0), sxy((size_t)(nx - 1) * nz, 0.0), szy((size_t)nx * (nz - 1), 0.0);
  std::vector<double> DS(np), sdx(sxy.size()), sdz(szy.size()), bx(sxy.size()), bz(szy.size());
  int n_fw = 0;
  for (int n = nt; n <= 2 * nt - 1; ++n) if (n % fw == 0) ++n_fw;  // :98-103
  if (mode != 0 && n_fw > 0) std::memset(G_out, 0, sizeof(float) * np * n_fw);
  std::memset(seis, 0, sizeof(double) * (size_t)nr * nt);
  std::memset(G_re, 0, sizeof(double) * np * K);
  std::memset(G_im, 0, sizeof(double) * np * K);
  const bool born = dmu != nullptr;
  int i_ftc = 0, i_fw_out = 0, i_fw_in = 0;
  for (int n = 1; n <= nt; ++n) {                          // :130
    if (mode != 0 && (n + nt - 1) % fw == 0) {             // :133-137
      float* o = G_out + np * i_fw_out;
      for (size_t p = 0; p < np; ++p) o[p] = (float)v[p];
      ++i_fw_out;
    }
    if (born) {                                            // :140-144
      if (i_fw_in >= n_G_in) return fail(FD2D_ERR_INDEX, "G_in has fewer than nt snapshots");
      const float* g = G_in + np * i_fw_in;
      dxv_single(s, g, bx.data());
      dzv_single(s, g, bz.data());
      for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nx - 1; ++i) {
          size_t q = i + (size_t)(nx - 1) * j;
          sxy[q] = sxy[q] + (dt * dmu[i + (size_t)nx * j]) * bx[q];
        }
      for (size_t q = 0; q < szy.size(); ++q) szy[q] = szy[q] + (dt * dmu[q]) * bz[q];
      ++i_fw_in;
    }
    div_s(s, sxy.data(), szy.data(), DS.data());           // :148
    if (!born)                                             // :152-156
      for (int i = 0; i < ns; ++i) {
        size_t p = sid[2 * i] + (size_t)nx * sid[2 * i + 1];
        DS[p] = DS[p] + stf;
      }
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)np; ++p) {        // :160-164
      double vv = v[p] + (dt * DS[p]) / rho[p];
      v[p] = vv * s.absbound[p];
    }
    dx_v(s, v.data(), sdx.data());                         // :168-172
    dz_v(s, v.data(), sdz.data());
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nz; ++j)
      for (int i = 0; i < nx - 1; ++i) {
        size_t q = i + (size_t)(nx - 1) * j;
        sxy[q] = sxy[q] + (dt * mu[i + (size_t)nx * j]) * sdx[q];
      }
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)szy.size(); ++q) szy[q] = szy[q] + (dt * mu[q]) * sdz[q];
    if ((n + nt - 1) % fs == 0) {                          // :176-183
      const double* cr = cre.data() + (size_t)K * i_ftc;
      const double* ci = cim.data() + (size_t)K * i_ftc;
#pragma omp parallel for schedule(static)
      for (long long p = 0; p < (long long)np; ++p)
        for (int k = 0; k < K; ++k) {
          G_re[p + np * k] = G_re[p + np * k] + v[p] * cr[k];
          G_im[p + np * k] = G_im[p + np * k] + v[p] * ci[k];
        }
      ++i_ftc;
    }
    for (int ir = 0; ir < nr; ++ir)                        // :187-189
      seis[ir + (size_t)nr * (n - 1)] = v[rid[2 * ir] + (size_t)nx * rid[2 * ir + 1]];
  }
  for (size_t q = 0; q < np * K; ++q) G_im[q] = -G_im[q];  // :196-198 conj
  return FD2D_OK;
}

// ---------------------------------------------------------------------------
// code/run_forward2_correlation.m
// ---------------------------------------------------------------------------
int oracle_forward2_correlation(const fd2d_config* cfg, const double* mu, const double* rho,
                                const double* G_re, const double* G_im, int n_G,
                                const double* spectrum, int n_src,
                                const double* source_dist, int n_dist,
                                const double* rec, int nr, int mode,
                                const double* dmu, const float* C_in, int n_C_in,
                                double* seis, float* C_out) {
  Setup s;
  fd2d_status st = make_setup(cfg, s);
  if (st != FD2D_OK) return st;
  const int nx = s.nx, nz = s.nz, K = s.K, fs = s.fs, fw = s.fw, nb = s.nb;
  const size_t np = (size_t)nx * nz;
  const double dt = s.dt;
  if (n_G < K) return fail(FD2D_ERR_INDEX, "G_fft has fewer than n_sample planes");
  if (n_src < 1) return fail(FD2D_ERR_SHAPE, "spectrum needs at least one column");
  int ncol = nb == 0 ? 1 : nb;
  if (nb == 0 && n_src != 1) return fail(FD2D_ERR_SHAPE, "n_basis_fct == 0 needs one noise source");
  if (n_dist != (nb == 0 ? n_src : nb)) return fail(FD2D_ERR_SHAPE, "source_dist planes");
  std::vector<int> rid(2 * nr);
  for (int i = 0; i < nr; ++i) { rid[2 * i] = nearest(s.x, rec[i]); rid[2 * i + 1] = nearest(s.z, rec[nr + i]); }
  std::vector<double> t = colon(-(s.nt - 1) * dt, dt, (s.nt - 1) * dt);  // :68-69
  const int ntc = (int)t.size();
  const double sq = 1 / std::sqrt(2 * M_PI);
  const int n_ftc = ntc / fs;                               // :73-85
  std::vector<double> cre, cim;
  for (int n = 1; n <= ntc; ++n)
    if (n % fs == 0)
      for (int k = 0; k < K; ++k) {
        double re, im;
        coeff(sq, s.w[k] * t[n - 1], s.dw, re, im);
        cre.push_back(re); cim.push_back(im);
      }
  (void)n_ftc;
  std::vector<double> v(np, 0.0), u(np, 0.0), sxy((size_t)(nx - 1) * nz, 0.0), szy((size_t)nx * (nz - 1), 0.0);
  std::vector<double> DS(np), sdx(sxy.size()), sdz(szy.size()), bx(sxy.size()), bz(szy.size());
  std::vector<float> dC;
  const int n_fw = ntc / fw;
  if (mode != 0 && n_fw > 0) std::memset(C_out, 0, sizeof(float) * np * n_fw);
  std::memset(seis, 0, sizeof(double) * (size_t)nr * ntc);
  std::vector<double> M;
  st = interpol_matrix(K, nb, M);
  if (st != FD2D_OK) return st;
  std::vector<double> dist;
  make_distribution(s, M, ncol, source_dist, dist);          // :168-173
  const bool born = dmu != nullptr;
  if (born) {
    if (n_C_in < ntc) return fail(FD2D_ERR_INDEX, "C_in has fewer than 2*nt-1 snapshots");
    dC.resize(np);
  }
  int i_ftc = 0, i_fw_out = 0;
  std::vector<double> Sre(np), Sim(np);
  for (int n = 1; n <= ntc; ++n) {                          // :178
    if (mode != 0 && n % fw == 0) {                         // :182-186
      float* o = C_out + np * i_fw_out;
      for (size_t p = 0; p < np; ++p) o[p] = (float)u[p];
      ++i_fw_out;
    }
    div_s(s, sxy.data(), szy.data(), DS.data());            // :190
    if (n % fs == 0) {                                      // :195-216
      const double* cr = cre.data() + (size_t)K * i_ftc;
      const double* ci = cim.data() + (size_t)K * i_ftc;
      for (int is = 0; is < n_src; ++is) {
#pragma omp parallel for schedule(static)
        for (long long p = 0; p < (long long)np; ++p) {
          double sr = 0.0, si = 0.0;
          for (int k = 0; k < K; ++k) {
            double R = spectrum[k + (size_t)K * is] * dist[p + np * k];
            double a = R * G_re[p + np * k], b = R * G_im[p + np * k];
            sr = sr + (a * cr[k] - b * ci[k]);
            si = si + (a * ci[k] + b * cr[k]);
          }
          DS[p] = DS[p] + sr;
          Sim[p] = si;
        }
      }
      ++i_ftc;
    }
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)np; ++p) {         // :220-224
      double vv = v[p] + (dt * DS[p]) / rho[p];
      v[p] = vv * s.absbound[p];
    }
    dx_v(s, v.data(), sdx.data());                          // :228-229
    dz_v(s, v.data(), sdz.data());
    const bool born_now = born && n != ntc;                 // :232-238
    if (born_now) {
      single_diff(C_in + np * (n - 1), C_in + np * n, dC.data(), np);
      dxv_single(s, dC.data(), bx.data());
      dzv_single(s, dC.data(), bz.data());
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nz; ++j)
      for (int i = 0; i < nx - 1; ++i) {
        size_t q = i + (size_t)(nx - 1) * j;
        double val = sxy[q] + (dt * mu[i + (size_t)nx * j]) * sdx[q];
        if (born_now) val = val - dmu[i + (size_t)nx * j] * bx[q];
        sxy[q] = val;
      }
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)szy.size(); ++q) {
      double val = szy[q] + (dt * mu[q]) * sdz[q];
      if (born_now) val = val - dmu[q] * bz[q];
      szy[q] = val;
    }
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)np; ++p) u[p] = u[p] + v[p] * dt;  // :242
    for (int ir = 0; ir < nr; ++ir)                         // :246-248
      seis[ir + (size_t)nr * (n - 1)] = u[rid[2 * ir] + (size_t)nx * rid[2 * ir + 1]];
  }
  return FD2D_OK;
}

// ---------------------------------------------------------------------------
// code/run_noise_adjoint.m
// ---------------------------------------------------------------------------
int oracle_noise_adjoint(const fd2d_config* cfg, const double* mu, const double* rho,
                         const float* u_fwd, int n_u_fwd,
                         const double* stf_re, const double* stf_im, const int64_t* stf_dims,
                         const double* src, int ns, const double* rec, int nr,
                         const double* spectrum, int n_spec_src,
                         const double* source_dist, int n_dist,
                         const double* G_re, const double* G_im, int n_G,
                         int mode, const double* dmu, const float* u_in, int n_u_in,
                         double* Kout, double* sf_re, double* sf_im, float* u_out, double* seis) {
  Setup s;
  fd2d_status st = make_setup(cfg, s);
  if (st != FD2D_OK) return st;
  const int nx = s.nx, nz = s.nz, K = s.K, fs = s.fs, fw = s.fw, nb = s.nb;
  const size_t np = (size_t)nx * nz;
  const double dt = s.dt;
  std::vector<double> t = colon(-(s.nt - 1) * dt, dt, (s.nt - 1) * dt);  // :47-49
  const int n_zero = s.nt;
  const int ntc = (int)t.size();
  std::vector<int> sid(2 * ns), rid(2 * nr);                 // :57-73
  for (int i = 0; i < ns; ++i) { sid[2 * i] = nearest(s.x, src[i]); sid[2 * i + 1] = nearest(s.z, src[ns + i]); }
  for (int i = 0; i < nr; ++i) { rid[2 * i] = nearest(s.x, rec[i]); rid[2 * i + 1] = nearest(s.z, rec[nr + i]); }
  const double sq = 1 / std::sqrt(2 * M_PI);
  const int n_ftc = ntc / fs;                                // :77-91
  std::vector<double> fre, fim, ire, iim;
  for (int n = 1; n <= ntc; ++n)
    if (n % fs == 0)
      for (int k = 0; k < K; ++k) {
        double a, b;
        coeff(sq, -(s.w[k] * t[n - 1]), dt, a, b);
        fre.push_back(a); fim.push_back(b);
        coeff(sq, s.w[k] * t[n - 1], s.dw, a, b);
        ire.push_back(a); iim.push_back(b);
      }
  // ifft_coeff2(n,k) (:95-98) has the same value as the ifft coefficient of step n.
  const int64_t d0 = stf_dims ? stf_dims[0] : 0, d1 = stf_dims ? stf_dims[1] : 0, d2 = stf_dims ? stf_dims[2] : 0;
  const bool stf_empty = !stf_re || d0 * d1 * d2 == 0;
  const int64_t size3 = stf_empty ? 1 : d2;  // size(stf,3) of [] is 1
  const bool stf2d = !stf_empty && size3 == 1;
  const bool stf3d = !stf_empty && size3 != 1;
  if (stf2d && (d0 < ns)) return fail(FD2D_ERR_INDEX, "stf has fewer rows than adjoint sources");
  if (stf3d) {
    if (d0 != nx || d1 != nz) return fail(FD2D_ERR_SHAPE, "field stf must be nx-by-nz-by-K");
    if (d2 < K) return fail(FD2D_ERR_INDEX, "field stf has fewer than n_sample planes");
  }
  // :112-123
  int n_noise = 0;
  const bool have_dist = source_dist != nullptr && n_dist > 0;
  int ncol = nb == 0 ? 1 : nb;
  if (have_dist) {
    n_noise = n_spec_src;
    if (n_noise < 1 || !spectrum) return fail(FD2D_ERR_SHAPE, "source_dist needs a spectrum");
    if (nb == 0 && n_noise != 1) return fail(FD2D_ERR_SHAPE, "n_basis_fct == 0 needs one noise source");
    if (n_dist != (nb == 0 ? n_noise : nb)) return fail(FD2D_ERR_SHAPE, "source_dist planes");
  }
  std::vector<double> v(np, 0.0), u(np, 0.0), sxy((size_t)(nx - 1) * nz, 0.0), szy((size_t)nx * (nz - 1), 0.0);
  std::vector<double> DS(np), sdx(sxy.size()), sdz(szy.size()), sdxu(sxy.size()), sdzu(szy.size());
  std::vector<double> bx(sxy.size()), bz(szy.size());
  std::memset(sf_re, 0, sizeof(double) * np * K);
  std::memset(sf_im, 0, sizeof(double) * np * K);
  const int n_fw = ntc / fw;
  const bool save_u = (mode == 11 || mode == 13);
  if (save_u && n_fw > 0) std::memset(u_out, 0, sizeof(float) * np * n_fw);
  std::memset(seis, 0, sizeof(double) * (size_t)nr * ntc);
  std::vector<double> Kmu(np, 0.0), Ks(np * ncol, 0.0);
  int nt_loop = ntc;                                          // :165-167
  if ((mode == 0 || mode == 1) && size3 != 1) nt_loop = n_zero;
  std::vector<double> M;
  st = interpol_matrix(K, nb, M);
  if (st != FD2D_OK) return st;
  std::vector<double> dist;
  if (have_dist) make_distribution(s, M, ncol, source_dist, dist);  // :221-229
  const bool Gvalid = G_re != nullptr && n_G == K;            // :302
  if (Gvalid && (!spectrum || n_spec_src != 1))
    return fail(FD2D_ERR_SHAPE, "source kernel needs a one-column spectrum");
  const bool born = dmu != nullptr && n_u_in == ntc;          // :285
  const bool have_fwd = u_fwd != nullptr && n_u_fwd > 0;
  std::vector<float> dU;
  if (born) dU.resize(np);
  int i_ftc = 0, i_fw_in = 0, i_fw_out = 0;
  for (int n = 1; n <= nt_loop; ++n) {                        // :233
    if (save_u && n % fw == 0) {                              // :237-241
      float* o = u_out + np * i_fw_out;
      for (size_t p = 0; p < np; ++p) o[p] = (float)u[p];
      ++i_fw_out;
    }
    div_s(s, sxy.data(), szy.data(), DS.data());              // :245
    if (stf2d) {                                              // :249-253
      if (n > d1) return fail(FD2D_ERR_INDEX, "stf has fewer columns than time steps");
      for (int i = 0; i < ns; ++i) {
        size_t p = sid[2 * i] + (size_t)nx * sid[2 * i + 1];
        DS[p] = DS[p] + stf_re[i + (size_t)d0 * (n - 1)];
      }
    } else if (stf3d) {                                       // :255-268
      if (n % fs == 0) {
        if (i_ftc >= n_ftc) return fail(FD2D_ERR_INDEX, "ifft_coeff index exceeds its rows");
        const double* cr = ire.data() + (size_t)K * i_ftc;
        const double* ci = iim.data() + (size_t)K * i_ftc;
#pragma omp parallel for schedule(static)
        for (long long p = 0; p < (long long)np; ++p) {
          double tr = 0.0, ti = 0.0;
          for (int is = 0; is < n_noise; ++is)
            for (int k = 0; k < K; ++k) {
              double R = spectrum[k + (size_t)K * is] * dist[p + np * k];
              double a = R * stf_re[p + np * k];
              double b = R * (stf_im ? -stf_im[p + np * k] : -0.0);
              tr = tr + (a * cr[k] - b * ci[k]);
              ti = ti + (a * ci[k] + b * cr[k]);
            }
          DS[p] = DS[p] + tr;
        }
        ++i_ftc;
      }
    }
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)np; ++p) {           // :273-277
      double vv = v[p] + (dt * DS[p]) / rho[p];
      v[p] = vv * s.absbound[p];
    }
    dx_v(s, v.data(), sdx.data());                            // :281-282
    dz_v(s, v.data(), sdz.data());
    const bool born_now = born && n != ntc;                   // :285-291
    if (born_now) {
      single_diff(u_in + np * (n - 1), u_in + np * n, dU.data(), np);
      dxv_single(s, dU.data(), bx.data());
      dzv_single(s, dU.data(), bz.data());
    }
#pragma omp parallel for schedule(static)
    for (int j = 0; j < nz; ++j)
      for (int i = 0; i < nx - 1; ++i) {
        size_t q = i + (size_t)(nx - 1) * j;
        double val = sxy[q] + (dt * mu[i + (size_t)nx * j]) * sdx[q];
        if (born_now) val = val - dmu[i + (size_t)nx * j] * bx[q];
        sxy[q] = val;
      }
#pragma omp parallel for schedule(static)
    for (long long q = 0; q < (long long)szy.size(); ++q) {
      double val = szy[q] + (dt * mu[q]) * sdz[q];
      if (born_now) val = val - dmu[q] * bz[q];
      szy[q] = val;
    }
#pragma omp parallel for schedule(static)
    for (long long p = 0; p < (long long)np; ++p) u[p] = u[p] + v[p] * dt;  // :295
    dx_v(s, u.data(), sdxu.data());                           // :296-297
    dz_v(s, u.data(), sdzu.data());
    if (Gvalid && n % fs == 0) {                              // :302-320
      // ifft_coeff2(n,:) = 1/sqrt(2pi) exp(1i w t(n)) dw
      std::vector<double> c2r(K), c2i(K);
      for (int k = 0; k < K; ++k) coeff(sq, s.w[k] * t[n - 1], s.dw, c2r[k], c2i[k]);
#pragma omp parallel for schedule(static)
      for (long long p = 0; p < (long long)np; ++p) {
        for (int ib = 0; ib < ncol; ++ib) {
          double mr = 0.0, mi = 0.0;
          for (int k = 0; k < K; ++k) {
            double a = spectrum[k] * G_re[p + np * k];
            double b = spectrum[k] * (-G_im[p + np * k]);
            double er = a * c2r[k] - b * c2i[k];
            double ei = a * c2i[k] + b * c2r[k];
            double wgt = M[k + (size_t)K * ib];
            mr = mr + wgt * er;
            mi = mi + wgt * ei;
          }
          (void)mi;
          Ks[p + np * ib] = Ks[p + np * ib] + mr * u[p];
        }
      }
    }
    if (have_fwd && n_u_fwd >= i_fw_in + 1 && n % fw == 0) {  // :324-331
      const float* uf = u_fwd + np * (size_t)(n_u_fwd - 1 - i_fw_in);
      dxv_single(s, uf, bx.data());
      dzv_single(s, uf, bz.data());
#pragma omp parallel for schedule(static)
      for (int j = 0; j < nz; ++j)
        for (int i = 0; i < nx - 1; ++i) {
          size_t q = i + (size_t)(nx - 1) * j, p = i + (size_t)nx * j;
          Kmu[p] = Kmu[p] - (sdxu[q] * bx[q]) * fw;
        }
#pragma omp parallel for schedule(static)
      for (long long q = 0; q < (long long)szy.size(); ++q)
        Kmu[q] = Kmu[q] - (sdzu[q] * bz[q]) * fw;
      ++i_fw_in;
    }
    if (mode == 1 || mode == 12 || mode == 13) {              // :335-346
      if (n % fs == 0) {
        if (i_ftc >= n_ftc) return fail(FD2D_ERR_INDEX, "fft_coeff index exceeds its rows");
        const double* cr = fre.data() + (size_t)K * i_ftc;
        const double* ci = fim.data() + (size_t)K * i_ftc;
#pragma omp parallel for schedule(static)
        for (long long p = 0; p < (long long)np; ++p)
          for (int k = 0; k < K; ++k) {
            sf_re[p + np * k] = sf_re[p + np * k] + u[p] * cr[k];
            sf_im[p + np * k] = sf_im[p + np * k] + u[p] * ci[k];
          }
        ++i_ftc;
      }
    }
    for (int ir = 0; ir < nr; ++ir)                           // :350-352
      seis[ir + (size_t)nr * (n - 1)] = u[rid[2 * ir] + (size_t)nx * rid[2 * ir + 1]];
  }
  // :359-367
  std::memcpy(Kout, Ks.data(), sizeof(double) * np * ncol);
  if (nb == 0) std::memset(Kout + np, 0, sizeof(double) * np);  // K(:,:,2) of zeros(nx,nz,2) before K_mu overwrites it
  std::memcpy(Kout + np * ncol, Kmu.data(), sizeof(double) * np);
  return FD2D_OK;
}

}  // extern "C"
