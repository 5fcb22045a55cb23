// host_setup.cu -- host-side problem setup shared by both precisions.
//
//   grid            code/propagation/define_computational_domain.m:18-22
//   taper           code/propagation/init_absbound.m:8-31
//   node indices    code/run_forward1_green.m:45-60 (nearest node, ties low)
//   frequency bands code/propagation/integration_limits.m:4-12,
//                   code/run_forward2_correlation.m:121-165 (interpol_matrix)
//   FD coefficients code/propagation/dx_v.m:22-30 (orders 2, 4); orders 6, 8
//                   are the staggered-grid extension.
#include "common.cuh"

#include <algorithm>
#include <mutex>

namespace fd2d {

std::vector<double> matlab_colon(double a, double d, double b) {
  // MATLAB's colon operator: interval count rounded with tolerance
  // 2*eps*max(|a|,|b|), end point snapped to b, elements built from both ends.
  std::vector<double> out;
  if (d == 0 || (d > 0 && a > b) || (d < 0 && a < b)) return out;
  const double eps = 2.220446049250313e-16;
  const double tol = 2.0 * eps * std::max(std::fabs(a), std::fabs(b));
  const double sig = d > 0 ? 1.0 : -1.0;
  long n;
  const bool a_int = a == std::floor(a);
  if (a_int && d == 1) {
    n = (long)(std::floor(b) - a);
  } else if (a_int && d == std::floor(d)) {
    double q = std::floor(a / d);
    double rem = a - q * d;
    n = (long)(std::floor((b - rem) / d) - q);
  } else {
    n = (long)std::round((b - a) / d);
    if (sig * (a + n * d - b) > tol) --n;
  }
  if (n < 0) return out;
  double last = a + n * d;
  if (a_int && d == std::floor(d)) last = std::floor(last);
  else if (sig * (last - b) > -tol) last = b;
  out.resize(n + 1);
  for (long k = 0; k <= n / 2; ++k) {
    out[k] = a + k * d;
    out[n - k] = last - k * d;
  }
  if (n % 2 == 0) out[n / 2] = (a + last) / 2;
  return out;
}

int nearest_node(const std::vector<double>& x, double p) {
  int best = 0;
  double bd = INFINITY;
  for (size_t i = 0; i < x.size(); ++i) {
    const double d = std::fabs(x[i] - p);
    if (d < bd) {  // strict: the first minimum wins, as min(find(...)) does
      bd = d;
      best = (int)i;
    }
  }
  return best;
}

// Staggered first-derivative weights of order 2r, exact rationals from the
// Taylor conditions sum_m c_m (2m-1)^(2p-1) = [p == 1], p = 1..r.
static void stagger_weights(int r, double* c) {
  switch (r) {
    case 1: c[0] = 1.0; break;
    case 2: c[0] = 9.0 / 8.0; c[1] = -1.0 / 24.0; break;
    case 3: c[0] = 75.0 / 64.0; c[1] = -25.0 / 384.0; c[2] = 3.0 / 640.0; break;
    default:
      c[0] = 1225.0 / 1024.0; c[1] = -245.0 / 3072.0; c[2] = 49.0 / 5120.0; c[3] = -5.0 / 7168.0;
  }
}

static fd2d_status build_geometry(const fd2d_config* cfg, Geometry& g, std::string& err) {
  if (cfg->nx < 2 || cfg->nz < 2 || cfg->nt < 1 || cfg->freq_samp < 1 || cfg->fw_nth < 1 ||
      !(cfg->dt > 0) || !(cfg->Lx > 0) || !(cfg->Lz > 0)) {
    err = "configuration needs nx, nz >= 2, nt, freq_samp, fw_nth >= 1 and dt, Lx, Lz > 0";
    return FD2D_ERR_ARG;
  }
  if (cfg->n_sample < 2 || !cfg->f_sample) {
    err = "configuration needs at least two frequencies (dw = w(2) - w(1))";
    return FD2D_ERR_ARG;
  }
  if (!(cfg->order == 2 || cfg->order == 4 || cfg->order == 6 || cfg->order == 8)) {
    err = "order must be 2, 4, 6 or 8";
    return FD2D_ERR_ORDER;
  }
  if (cfg->n_basis_fct < 0 || cfg->n_basis_fct == 1) {
    err = "n_basis_fct must be 0 or >= 2 (one band makes interpol_matrix grow a column)";
    return FD2D_ERR_SHAPE;
  }
  if (cfg->nx < cfg->order || cfg->nz < cfg->order) {
    err = "grid smaller than the stencil";
    return FD2D_ERR_SHAPE;
  }
  g.nx = cfg->nx; g.nz = cfg->nz; g.nt = cfg->nt; g.ntc = 2 * cfg->nt - 1;
  g.order = cfg->order; g.r = cfg->order / 2; g.K = cfg->n_sample;
  g.fs = cfg->freq_samp; g.fw = cfg->fw_nth; g.nb = cfg->n_basis_fct;
  g.Lx = cfg->Lx; g.Lz = cfg->Lz; g.dt = cfg->dt;
  g.dx = g.Lx / (g.nx - 1);
  g.dz = g.Lz / (g.nz - 1);
  g.x = matlab_colon(0.0, g.dx, g.Lx);
  g.z = matlab_colon(0.0, g.dz, g.Lz);
  if ((int)g.x.size() != g.nx || (int)g.z.size() != g.nz) {
    err = "0:dx:Lx does not give nx points";
    return FD2D_ERR_SHAPE;
  }
  g.w.resize(g.K);
  for (int k = 0; k < g.K; ++k) g.w[k] = 2 * M_PI * cfg->f_sample[k];
  g.dw = g.w[1] - g.w[0];
  g.t_fwd = matlab_colon(0.0, g.dt, (g.nt - 1) * g.dt);
  g.t_corr = matlab_colon(-(g.nt - 1) * g.dt, g.dt, (g.nt - 1) * g.dt);
  if ((int)g.t_fwd.size() != g.nt || (int)g.t_corr.size() != g.ntc) {
    err = "time axis length differs from nt / 2nt-1";
    return FD2D_ERR_SHAPE;
  }
  // Cerjan taper, product over the enabled sides; exp(-(X-w)^2/(2w)^2) inside.
  const double wd = cfg->absorb_width;
  const double den = (2 * wd) * (2 * wd);
  auto ab = std::make_shared<std::vector<double>>((size_t)g.nx * g.nz, 1.0);
  for (int j = 0; j < g.nz; ++j) {
    const double Z = g.z[j];
    for (int i = 0; i < g.nx; ++i) {
      const double X = g.x[i];
      double a = 1.0;
      if (cfg->absorb_left == 1) {
        const double d = X - wd;
        a *= (X > wd ? 1.0 : 0.0) + std::exp(-(d * d) / den) * (X <= wd ? 1.0 : 0.0);
      }
      if (cfg->absorb_right == 1) {
        const double e = g.Lx - wd, d = X - e;
        a *= (X < e ? 1.0 : 0.0) + std::exp(-(d * d) / den) * (X >= e ? 1.0 : 0.0);
      }
      if (cfg->absorb_bottom == 1) {
        const double d = Z - wd;
        a *= (Z > wd ? 1.0 : 0.0) + std::exp(-(d * d) / den) * (Z <= wd ? 1.0 : 0.0);
      }
      if (cfg->absorb_top == 1) {
        const double e = g.Lz - wd, d = Z - e;
        a *= (Z < e ? 1.0 : 0.0) + std::exp(-(d * d) / den) * (Z >= e ? 1.0 : 0.0);
      }
      (*ab)[i + (size_t)g.nx * j] = a;
    }
  }
  g.absbound = ab;
  stagger_weights(g.r, g.c);
  return FD2D_OK;
}

uint64_t config_hash(const fd2d_config* c) {
  Sig s;
  s.add(c->Lx); s.add(c->Lz); s.add(c->nx); s.add(c->nz); s.add(c->dt); s.add(c->nt); s.add(c->order);
  s.add(c->n_basis_fct); s.add(c->fw_nth); s.add(c->n_sample); s.add(c->freq_samp); s.add(c->absorb_width);
  s.add(c->absorb_left); s.add(c->absorb_right); s.add(c->absorb_top); s.add(c->absorb_bottom);
  if (c->f_sample && c->n_sample > 0) s.bytes(c->f_sample, sizeof(double) * c->n_sample);
  return s.h | 1;
}

// Geometries of recently used configurations (grid, taper, time axes).
static std::mutex g_geo_mu;
static std::vector<std::pair<uint64_t, Geometry>> g_geo_cache;

fd2d_status make_geometry(const fd2d_config* cfg, Geometry& g, std::string& err) {
  if (!cfg) { err = "cfg is NULL"; return FD2D_ERR_ARG; }
  const uint64_t key = (cfg->f_sample || cfg->n_sample < 1) ? config_hash(cfg) : 0;
  if (key) {
    std::lock_guard<std::mutex> lk(g_geo_mu);
    for (auto& kv : g_geo_cache)
      if (kv.first == key) { g = kv.second; return FD2D_OK; }
  }
  fd2d_status s = build_geometry(cfg, g, err);
  g.key = key;
  if (s == FD2D_OK && key) {
    std::lock_guard<std::mutex> lk(g_geo_mu);
    if (g_geo_cache.size() >= 16) g_geo_cache.erase(g_geo_cache.begin());
    g_geo_cache.emplace_back(key, g);
  }
  return s;
}

fd2d_status make_interpol_matrix(int K, int nb, std::vector<double>& M, std::string& err) {
  const int ncol = nb == 0 ? 1 : nb;
  M.assign((size_t)K * ncol, nb == 0 ? 1.0 : 0.0);
  if (nb == 0) return FD2D_OK;
  const double step = (double)K / nb;
  std::vector<int> lo(nb), hi(nb);
  for (int b = 1; b <= nb; ++b) {
    lo[b - 1] = (int)std::floor((b - 1) * step + 1);
    hi[b - 1] = (int)std::floor(b * step);
  }
  for (int k = 1; k <= K; ++k) {
    int ib = 0;
    for (int b = 1; b <= nb && !ib; ++b)
      if (k >= lo[b - 1] && k <= hi[b - 1]) ib = b;
    if (!ib) { err = "frequency outside every band"; return FD2D_ERR_INDEX; }
    const int ni = hi[ib - 1] - lo[ib - 1] + 1;
    const int below = ib == 1 ? 0 : ib - 1;
    const int above = ib == nb ? 0 : ib + 1;
    const int i = k - lo[ib - 1] + 1;
    const double half = ni / 2.0;
    auto at = [&](int kk, int cc) -> double& { return M[(kk - 1) + (size_t)K * (cc - 1)]; };
    if (i < half) {
      at(k, ib) = 1 - (half - i) / ni;
      if (below) at(k, below) = (half - i) / ni;
    } else if (i == half) {
      at(k, ib) = 1;
    } else {
      at(k, ib) = 1 - (i - half) / ni;
      if (above) at(k, above) = (i - half) / ni;
    }
  }
  return FD2D_OK;
}

}  // namespace fd2d
