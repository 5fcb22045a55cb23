// measure.cu -- misfits and adjoint source time functions of the correlations,
// FP64 on the device.
//
//   tools/measurement/make_adjoint_sources.m:31-175  (receiver loop, windows,
//                                                    velocity conversion)
//   tools/measurement/log_amp_ratio.m:23-93          (log amplitude ratio)
//   tools/measurement/waveform_difference.m:23-48    (waveform difference)
//   tools/measurement/cc_time_shift.m:21-61          (cross-correlation time shift)
//   tools/measurement/amp_diff.m:22-66               (relative amplitude difference)
//   tools/measurement/addons/cross_correlation_td.m  (xcorr over all lags)
//   tools/measurement/addons/get_window.m:1-35       (hann / cos_taper windows)
//
// The windows depend only on the time axis and are built on the host exactly
// as get_window does (MATLAB's symmetric Hann window 0.5*(1 - cos(2*pi*n/(N-1)))).
// One CTA per receiver evaluates the energies (trapezoidal rule with unit
// spacing times dt, as trapz(...)*dt) with FP64 block reductions and writes
// the time-reversed adjoint source.
#include "common.cuh"

#include <algorithm>
#include <cfloat>

namespace fd2d {
namespace {

constexpr int MT = 256;

struct MeasArgs {
  int nr, nt, kind, second, vel;
  double dt;
  const double *u, *u0, *du;  // nr-by-nt, column-major
  const double *wc, *wa;      // causal / acausal windows (wa unused for waveform_difference)
  double *misfit, *adstf;     // nr, nr-by-nt
  // time shift: the lag axis t_cc (2nt-1 values, MATLAB colon), the nonzero
  // span [s0, s1] of each window, scratch for the windowed traces (2nt per receiver)
  const double* tcc;
  int sc0, sc1, sa0, sa1;
  double* scratch;
};

__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = threadIdx.x < MT / 32 ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) sh[0] = s;
  }
  __syncthreads();
  s = sh[0];
  __syncthreads();
  return s;
}

// Seismogram value k of receiver n; the velocity form is diff(u)/dt with a zero
// last sample (make_adjoint_sources.m:44-56).
__device__ __forceinline__ double trace(const MeasArgs& a, const double* x, int n, int k) {
  if (!a.vel) return x[n + (int64_t)a.nr * k];
  if (k >= a.nt - 1) return 0.0;
  return (x[n + (int64_t)a.nr * (k + 1)] - x[n + (int64_t)a.nr * k]) / a.dt;
}

// The largest value and the first index holding it, over the block.
__device__ void block_argmax(double& v, int& i, double* sv, int* si) {
  for (int o = 16; o > 0; o >>= 1) {
    const double ov = __shfl_down_sync(0xffffffffu, v, o);
    const int oi = __shfl_down_sync(0xffffffffu, i, o);
    if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) { sv[w] = v; si[w] = i; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < MT / 32; ++q)
      if (sv[q] > sv[0] || (sv[q] == sv[0] && si[q] < si[0])) { sv[0] = sv[q]; si[0] = si[q]; }
  }
  __syncthreads();
  v = sv[0];
  i = si[0];
  __syncthreads();
}

// cc_time_shift.m for window w (span [s0, s1]) of receiver n: the misfit, and
// the adjoint source before its time reversal added into row.
__device__ double time_shift(const MeasArgs& a, int n, const double* w, int s0, int s1, bool u0_zero, double* row,
                             double* sh, double* sv, int* si) {
  const int nt = a.nt;
  double T = 1.0;
  if (!u0_zero) {
    // cc = xcorr(win.*u_0, win.*u): cc(m) = sum_j g(j+m) f(j), f = win.*u,
    // g = win.*u_0, lags m = -(nt-1) .. nt-1; only lags within the window's
    // span can be nonzero, and their sums run over the span in ascending j
    double* f = a.scratch + (int64_t)2 * nt * n;
    double* g = f + nt;
    for (int k = threadIdx.x; k < nt; k += MT) {
      f[k] = w[k] * trace(a, a.u, n, k);
      g[k] = w[k] * trace(a, a.u0, n, k);
    }
    __syncthreads();
    double best = -INFINITY;
    int ib = 2 * nt;
    const int L = s1 - s0;
    for (int m = -L + (int)threadIdx.x; m <= L && L >= 0; m += MT) {
      double acc = 0.0;
      const int j0 = max(s0, s0 - m), j1 = min(s1, s1 - m);
      for (int j = j0; j <= j1; ++j) acc = acc + g[j + m] * f[j];
      const int idx = m + nt - 1;
      if (acc > best || (acc == best && idx < ib)) { best = acc; ib = idx; }
    }
    block_argmax(best, ib, sv, si);
    // lags outside the span hold zeros; the first of them is lag -(nt-1)
    const bool outside = L < nt - 1;
    const int imax = (best > 0.0 || !outside) ? ib : 0;
    T = a.tcc[imax];
    if (fabs(T) > 3.5) T = 0.0;
  }
  // v = diff(u)/dt with a zero last sample; adstf = T*(win.^2.*v)/(sum((win.*v).^2)*dt)
  double den = 0.0;
  for (int k = threadIdx.x; k < nt; k += MT) {
    const double v = k < nt - 1 ? (trace(a, a.u, n, k + 1) - trace(a, a.u, n, k)) / a.dt : 0.0;
    den += (w[k] * v) * (w[k] * v);
  }
  den = block_sum(den, sh) * a.dt;
  for (int k = threadIdx.x; k < nt; k += MT) {
    const double v = k < nt - 1 ? (trace(a, a.u, n, k + 1) - trace(a, a.u, n, k)) / a.dt : 0.0;
    row[k] += T * ((w[k] * w[k]) * v) / den;
  }
  return T * T / 2.0;
}

// amp_diff.m for window w of receiver n: the misfit (first order), and the
// adjoint source before its time reversal added into row.
__device__ double amplitude(const MeasArgs& a, int n, const double* w, bool u0_zero, double* row, double* sh) {
  const int nt = a.nt;
  const double dt = a.dt;
  double s0 = 0, su = 0, suu = 0, sd = 0;
  for (int k = threadIdx.x; k < nt; k += MT) {
    const double u = trace(a, a.u, n, k), u0 = trace(a, a.u0, n, k);
    s0 += (w[k] * u0) * (w[k] * u0);
    su += (w[k] * u) * (w[k] * u);
    suu += u * u;
    if (a.second) sd += (w[k] * w[k]) * u * a.du[n + (int64_t)a.nr * k];
  }
  const double S0 = block_sum(s0, sh), e0 = S0 * dt, eu = block_sum(su, sh) * dt;
  const double Suu = block_sum(suu, sh), Sd = a.second ? block_sum(sd, sh) : 0.0;
  const double meas = (eu - e0) / (e0 + DBL_EPSILON);
  double misfit = 0.0;
  for (int k = threadIdx.x; k < nt; k += MT) {
    const double u = trace(a, a.u, n, k), w2 = w[k] * w[k];
    double r;
    if (!a.second) {
      // with zero observations the reference reverses u here and once more
      // at the end: the adjoint source is u itself, unreversed
      r = u0_zero ? 2.0 * trace(a, a.u, n, nt - 1 - k) / (Suu * dt) : 2.0 * meas * w2 * u / S0;
    } else {
      const double du = a.du[n + (int64_t)a.nr * k];
      r = 2.0 * meas * w2 * du / e0 * dt + 4.0 * w2 * u / (e0 * e0) * Sd * dt * dt;
    }
    row[k] += r;
  }
  if (!a.second) misfit = u0_zero ? 1.0 : meas * meas / 2.0;
  return misfit;
}

// trapz weight of sample k (unit spacing): 1/2 at both ends, 1 inside.
__device__ __forceinline__ double tw(int k, int nt) { return (k == 0 || k == nt - 1) ? 0.5 : 1.0; }

__global__ void k64_measure(MeasArgs a) {
  __shared__ double sh[MT / 32];
  __shared__ double sv[MT / 32];
  __shared__ int si[MT / 32];
  extern __shared__ double row[];  // nt: the adjoint source before reversal
  const int n = blockIdx.x, nt = a.nt;
  const double dt = a.dt;
  if (a.kind == FD2D_MEAS_CC_TIME_SHIFT || a.kind == FD2D_MEAS_AMPLITUDE_DIFFERENCE) {
    // make_adjoint_sources.m:118-151: the causal window and the acausal one
    // (bounds swapped and negated), their misfits and adjoint sources summed
    double nz0 = 0;
    for (int k = threadIdx.x; k < nt; k += MT) {
      nz0 += trace(a, a.u0, n, k) != 0.0 ? 1.0 : 0.0;
      row[k] = 0.0;
    }
    const bool u0_zero = block_sum(nz0, sh) == 0.0;  // (also orders the row clears)
    double m;
    if (a.kind == FD2D_MEAS_CC_TIME_SHIFT) {
      m = time_shift(a, n, a.wc, a.sc0, a.sc1, u0_zero, row, sh, sv, si);
      __syncthreads();
      m += time_shift(a, n, a.wa, a.sa0, a.sa1, u0_zero, row, sh, sv, si);
    } else {
      m = amplitude(a, n, a.wc, u0_zero, row, sh);
      __syncthreads();
      m += amplitude(a, n, a.wa, u0_zero, row, sh);
    }
    if (threadIdx.x == 0 && a.misfit) a.misfit[n] = a.second ? 0.0 : m;
  } else if (a.kind == FD2D_MEAS_WAVEFORM_DIFFERENCE) {
    double m = 0.0;
    for (int k = threadIdx.x; k < nt; k += MT) {
      const double w2 = a.wc[k] * a.wc[k];
      const double d = trace(a, a.u, n, k) - trace(a, a.u0, n, k);
      if (!a.second) m += w2 * (d * d);
      row[k] = a.second ? w2 * a.du[n + (int64_t)a.nr * k] * dt : w2 * d * dt;
    }
    m = block_sum(m, sh);
    if (threadIdx.x == 0 && a.misfit) a.misfit[n] = a.second ? 0.0 : 0.5 * m * dt;
  } else {
    // log amplitude ratio (log_amp_ratio.m:36-88)
    double ec = 0, ea = 0, e0c = 0, e0a = 0, dc = 0, da = 0, nz0 = 0;
    for (int k = threadIdx.x; k < nt; k += MT) {
      const double u = trace(a, a.u, n, k), u0 = trace(a, a.u0, n, k), w = tw(k, nt);
      const double wc = a.wc[k], wa = a.wa[k];
      ec += w * ((wc * u) * (wc * u));
      ea += w * ((wa * u) * (wa * u));
      e0c += w * ((wc * u0) * (wc * u0));
      e0a += w * ((wa * u0) * (wa * u0));
      nz0 += u0 != 0.0 ? 1.0 : 0.0;
      if (a.second) {
        const double du = a.du[n + (int64_t)a.nr * k];
        dc += w * (2 * (wc * wc) * u * du);
        da += w * (2 * (wa * wa) * u * du);
      }
    }
    const double e_c = block_sum(ec, sh) * dt, e_a = block_sum(ea, sh) * dt + DBL_EPSILON;
    const double e0_c = block_sum(e0c, sh) * dt, e0_a = block_sum(e0a, sh) * dt + DBL_EPSILON;
    const bool u0_zero = block_sum(nz0, sh) == 0.0;
    const double A = log(e_c / e_a), A0 = log(e0_c / e0_a);
    if (!a.second) {
      if (threadIdx.x == 0 && a.misfit) a.misfit[n] = 0.5 * (A - A0) * (A - A0);
      for (int k = threadIdx.x; k < nt; k += MT) {
        const double u = trace(a, a.u, n, k), wc = a.wc[k], wa = a.wa[k];
        const double g = (2 * (wc * wc) * u * dt) / e_c - (2 * (wa * wa) * u * dt) / e_a;
        row[k] = u0_zero ? g : (A - A0) * g;
      }
    } else {
      if (threadIdx.x == 0 && a.misfit) a.misfit[n] = 0.0;
      const double de_c = block_sum(dc, sh) * dt, de_a = block_sum(da, sh) * dt;
      for (int k = threadIdx.x; k < nt; k += MT) {
        const double u = trace(a, a.u, n, k), du = a.du[n + (int64_t)a.nr * k];
        const double wc2 = a.wc[k] * a.wc[k], wa2 = a.wa[k] * a.wa[k];
        row[k] = (A - A0) * (2 / e_c * wc2 - 2 / e_a * wa2) * du * dt +
                 (A - A0) * (-2 / (e_c * e_c) * wc2 * u * de_c + 2 / (e_a * e_a) * wa2 * u * de_a) * dt +
                 (2 / e_c * wc2 * u - 2 / e_a * wa2 * u) * (de_c / e_c - de_a / e_a) * dt;
      }
    }
  }
  __syncthreads();
  // adstf = fliplr(row); velocity form: adstf(1:nt-1) = -diff(adstf)/dt
  for (int k = threadIdx.x; k < nt; k += MT) {
    const double r = row[nt - 1 - k];
    double o = r;
    if (a.vel && k < nt - 1) o = -(row[nt - 2 - k] - r) / dt;
    a.adstf[n + (int64_t)a.nr * k] = o;
  }
}

// get_window(t, t_min, t_max, type) of tools/measurement/addons/get_window.m.
std::vector<double> get_window(const double* t, int nt, double t_min, double t_max, bool hann) {
  if (t_min > t_max) std::swap(t_min, t_max);
  std::vector<double> w(nt);
  for (int k = 0; k < nt; ++k) w[k] = (t[k] > t_min && t[k] < t_max) ? 1.0 : 0.0;
  if (hann) {
    int i1 = -1, i2 = -1;
    for (int k = 0; k < nt; ++k)
      if (w[k] != 0.0) {
        if (i1 < 0) i1 = k;
        i2 = k;
      }
    if (i1 >= 0) {
      const int L = i2 - i1 + 1;
      for (int q = 0; q < L; ++q) w[i1 + q] = L == 1 ? 1.0 : 0.5 * (1.0 - std::cos(2.0 * M_PI * q / (L - 1)));
    }
  } else {
    const double width = std::fabs(t_max - t_min) * 0.1;
    for (int k = 0; k < nt; ++k) {
      const double x = t[k];
      w[k] += (0.5 + 0.5 * std::cos(M_PI * (t_max - x) / width)) * ((x >= t_max && x < t_max + width) ? 1.0 : 0.0);
      w[k] += (0.5 + 0.5 * std::cos(M_PI * (t_min - x) / width)) * ((x > t_min - width && x <= t_min) ? 1.0 : 0.0);
    }
  }
  return w;
}

}  // namespace

// Windows of one measurement (host): causal wc and acausal wa.
fd2d_status measurement_windows(fd2d_ctx* ctx, int kind, const double* t, int nt, std::vector<double>& wc,
                                std::vector<double>& wa) {
  if (nt < 2) return set_error(ctx, FD2D_ERR_SHAPE, "time axis needs two samples");
  if (kind == FD2D_MEAS_WAVEFORM_DIFFERENCE) {
    wc = get_window(t, nt, t[0], t[nt - 1], false);
    wa.assign(nt, 0.0);
    return FD2D_OK;
  }
  if (kind != FD2D_MEAS_LOG_AMPLITUDE_RATIO && kind != FD2D_MEAS_CC_TIME_SHIFT &&
      kind != FD2D_MEAS_AMPLITUDE_DIFFERENCE)
    return set_error(ctx, FD2D_ERR_ARG, "unknown measurement");
  // make_adjoint_sources.m:87-103: the fixed 100-200 s window, clipped to the axis
  double left = 100.0, right = 200.0;
  if (left < 0) {
    int idx = -1;
    for (int k = 0; k < nt; ++k)
      if (t[k] == 0.0) { idx = k; break; }
    if (idx < 0 || idx + 1 >= nt) return set_error(ctx, FD2D_ERR_INDEX, "t == 0 not on the time axis");
    left = t[idx + 1];
  }
  if (right > t[nt - 1]) right = t[nt - 1];
  if (left > t[nt - 1]) return set_error(ctx, FD2D_ERR_SHAPE, "time series too short?");
  if (kind != FD2D_MEAS_LOG_AMPLITUDE_RATIO) {
    // cos_taper windows: [left, right] and, after [left, right] = swap(-left, -right),
    // [-right, -left]
    wc = get_window(t, nt, left, right, false);
    wa = get_window(t, nt, -right, -left, false);
    return FD2D_OK;
  }
  wc = get_window(t, nt, left, right, true);
  // log_amp_ratio.m:30-37: the causal window is the one whose maximum lies at t >= 0
  int imax = 0;
  for (int k = 1; k < nt; ++k)
    if (wc[k] > wc[imax]) imax = k;
  std::vector<double> flipped(wc.rbegin(), wc.rend());
  if (t[imax] < 0) {
    wa = wc;
    wc = flipped;
  } else {
    wa = flipped;
  }
  return FD2D_OK;
}

}  // namespace fd2d

using namespace fd2d;

extern "C" fd2d_status fd2d_make_adjoint_sources(fd2d_ctx* ctx, int32_t measurement, int32_t deriv_order,
                                                 int32_t velocity, const double* u, const double* u_0,
                                                 const double* du, int32_t n_rec, int32_t nt, const double* t,
                                                 double* misfit, double* adstf) {
  FD2D_TRY(check_ctx(ctx));
  if (n_rec < 0 || nt < 2 || !t || (n_rec > 0 && (!u || !u_0 || !adstf)) || (deriv_order != 1 && deriv_order != 2))
    return set_error(ctx, FD2D_ERR_ARG, "bad measurement arguments");
  if (deriv_order == 2 && n_rec > 0 && !du) return set_error(ctx, FD2D_ERR_ARG, "second order needs du");
  if (deriv_order == 2 && measurement == FD2D_MEAS_CC_TIME_SHIFT)
    return set_error(ctx, FD2D_ERR_ARG, "no Hessian vector products for traveltime measurements");
  if ((size_t)nt * 8 > 160 * 1024) return set_error(ctx, FD2D_ERR_SHAPE, "time series longer than 20480 samples");
  cudaSetDevice(ctx->device);
  std::vector<double> wc, wa;
  FD2D_TRY(measurement_windows(ctx, measurement, t, nt, wc, wa));
  if (n_rec == 0) return FD2D_OK;
  const size_t tr = (size_t)n_rec * nt * 8;
  const void *du_d = nullptr, *u_d, *u0_d;
  FD2D_TRY(stage_in(ctx, "meas.u", u, tr, &u_d));
  FD2D_TRY(stage_in(ctx, "meas.u0", u_0, tr, &u0_d));
  if (deriv_order == 2) FD2D_TRY(stage_in(ctx, "meas.du", du, tr, &du_d));
  double *wcd, *wad;
  FD2D_TRY(upload(ctx, "meas.wc", wc, &wcd));
  FD2D_TRY(upload(ctx, "meas.wa", wa, &wad));
  void *mis_d = nullptr, *ad_d = nullptr;
  FD2D_TRY(out_buffer(ctx, "meas.misfit", misfit, (size_t)n_rec * 8, &mis_d));
  FD2D_TRY(out_buffer(ctx, "meas.adstf", adstf, tr, &ad_d));
  MeasArgs a;
  a.nr = n_rec; a.nt = nt; a.kind = measurement; a.second = deriv_order == 2; a.vel = velocity != 0;
  a.dt = std::fabs(t[1] - t[0]);
  a.u = (const double*)u_d; a.u0 = (const double*)u0_d; a.du = (const double*)du_d;
  a.wc = wcd; a.wa = wad;
  a.misfit = (double*)mis_d; a.adstf = (double*)ad_d;
  a.tcc = nullptr;
  a.scratch = nullptr;
  a.sc0 = a.sa0 = 0;
  a.sc1 = a.sa1 = -1;
  if (measurement == FD2D_MEAS_CC_TIME_SHIFT) {
    // t_cc = -(n-1)*dt:dt:(n-1)*dt of cross_correlation_td.m (dt = t(2)-t(1))
    const double d = t[1] - t[0];
    std::vector<double> tcc = matlab_colon(-(nt - 1) * d, d, (nt - 1) * d);
    if ((int)tcc.size() != 2 * nt - 1) return set_error(ctx, FD2D_ERR_SHAPE, "lag axis of the time shift");
    double* tccd;
    FD2D_TRY(upload(ctx, "meas.tcc", tcc, &tccd));
    a.tcc = tccd;
    FD2D_TRY(workspace_t(ctx, "meas.scratch", (size_t)2 * nt * n_rec, &a.scratch));
    auto span = [&](const std::vector<double>& w, int& s0, int& s1) {
      s0 = 0;
      s1 = -1;
      for (int k = 0; k < nt; ++k)
        if (w[k] != 0.0) {
          if (s1 < 0) s0 = k;
          s1 = k;
        }
    };
    span(wc, a.sc0, a.sc1);
    span(wa, a.sa0, a.sa1);
  }
  const size_t smem = (size_t)nt * 8;
  if (smem > 48 * 1024)
    FD2D_CUDA(ctx, cudaFuncSetAttribute(k64_measure, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k64_measure<<<n_rec, MT, smem, ctx->stream>>>(a);
  FD2D_TRY(after_launch(ctx, "k64_measure"));
  FD2D_TRY(stage_out(ctx, misfit, mis_d, (size_t)n_rec * 8));
  FD2D_TRY(stage_out(ctx, adstf, ad_d, tr));
  return finish_call(ctx);
}
