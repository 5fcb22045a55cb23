// solver_fp32.cu -- the FP32 form of the three solvers.
//
// Per time step ONE fused kernel (k32_step) advances a tile of the grid:
//   DS  = div_s(sxy, szy) (+ point sources) (+ injected correlation source)
//   v   = (v + DS * dt/rho) * absbound
//   sxy += dt*mu * dx_v(v),  szy += dt*mu * dz_v(v),  u += v*dt
// (code/run_forward1_green.m:148-172, code/run_forward2_correlation.m:190-242,
// code/run_noise_adjoint.m:245-297).  The tile stages sxy/szy with their halos
// in shared memory, recomputes the new v on the halo ring so the stress update
// needs no second pass, and writes v, sxy, szy, u once: 36 B (44 B with u) of
// HBM traffic per grid-point update.  Fields are ping-ponged between two
// buffers so neighbouring tiles never read a half-updated halo.
//
// The dense work leaves the time loop:
//  * the DFT of v (Green spectrum) / u (adjoint spectrum, source kernel) is a
//    contraction of stored snapshots with the DFT basis (contract.cuh), with
//    FP64 accumulation of the spectra;
//  * the correlation / adjoint field source real(sum_k P_k e^{i w_k t}) is a
//    contraction of P = spectrum*distribution*G planes with the time basis,
//    evaluated for all injection steps before the loop and read by the stencil
//    as one plane per injection step.
// The mu kernel accumulates in FP64 from FP32 strains; the source kernel is
// formed once from the adjoint spectrum (see fp32_adjoint).
#include "common.cuh"
#include "contract.cuh"

#include <algorithm>

namespace fd2d {
namespace {

constexpr int TX = 64, TZ = 16, NT = 256;
constexpr int MAX_BOX_SRC = 64;

struct Grid32 {
  int nx, nz;
  float c[4];
  float inv_dx, inv_dz, dt;
};

struct Fields32 {
  const float *b, *taper, *dtmu;
  float *v[2], *sxy[2], *szy[2], *u[2];
};

struct Step32 {
  int par;  // read buffers [par], write [1 - par]
  int has_u;
  const int* src_pt;
  int nsrc;
  const double* amp;  // per-source amplitude of this step, or nullptr -> amp_const
  float amp_const;
  const float* inj;     // injection plane of this step (npts) or nullptr
  float* snap_pre;      // single(old field), npts, or nullptr
  int snap_pre_u;
  float* snap_dft;      // new field (v or u) into the DFT snapshot plane, or nullptr
  const int* rec_pt;
  int nrec;
  double* seis_col;     // seismograms(:, n)
  int rec_u;
};

template <int R>
__global__ __launch_bounds__(NT) void k32_step(Grid32 G, Fields32 F, Step32 S) {
  constexpr int BW = TX + 2 * R - 1, BH = TZ + 2 * R - 1;
  constexpr int SXW = TX + 4 * R - 2, SZH = TZ + 4 * R - 2;
  __shared__ float s_sxy[BH * SXW];
  __shared__ float s_szy[SZH * BW];
  __shared__ float s_v[BH * BW];
  __shared__ int s_src[MAX_BOX_SRC];
  __shared__ float s_amp[MAX_BOX_SRC];
  __shared__ int s_nsrc;

  const int tid = threadIdx.x;
  const int nx = G.nx, nz = G.nz;
  const int x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ;
  const int bx0 = x0 - R + 1, bz0 = z0 - R + 1;
  const int sx0 = x0 - 2 * R + 1, sz0 = z0 - 2 * R + 1;
  const int par = S.par;
  const float* __restrict__ sxy = F.sxy[par];
  const float* __restrict__ szy = F.szy[par];
  const float* __restrict__ v = F.v[par];
  const float* __restrict__ u = F.u[par];

  if (tid == 0) s_nsrc = 0;
  for (int e = tid; e < BH * SXW; e += NT) {
    const int rr = e / SXW, cc = e - rr * SXW;
    const int gx = sx0 + cc, gz = bz0 + rr;
    s_sxy[e] = (gx >= 0 && gx < nx && gz >= 0 && gz < nz) ? sxy[gx + (int64_t)nx * gz] : 0.f;
  }
  for (int e = tid; e < SZH * BW; e += NT) {
    const int rr = e / BW, cc = e - rr * BW;
    const int gx = bx0 + cc, gz = sz0 + rr;
    s_szy[e] = (gx >= 0 && gx < nx && gz >= 0 && gz < nz) ? szy[gx + (int64_t)nx * gz] : 0.f;
  }
  __syncthreads();
  for (int k = tid; k < S.nsrc; k += NT) {
    const int p = S.src_pt[k];
    const int gx = p % nx, gz = p / nx;
    if (gx >= bx0 && gx < bx0 + BW && gz >= bz0 && gz < bz0 + BH) {
      const int slot = atomicAdd(&s_nsrc, 1);
      if (slot < MAX_BOX_SRC) {
        s_src[slot] = (gz - bz0) * BW + (gx - bx0);
        s_amp[slot] = S.amp ? (float)S.amp[k] : S.amp_const;
      }
    }
  }
  __syncthreads();
  const int nbs = s_nsrc;

  // new v on the tile plus its halo ring
  for (int e = tid; e < BH * BW; e += NT) {
    const int rr = e / BW, cc = e - rr * BW;
    const int gx = bx0 + cc, gz = bz0 + rr;
    float vn = 0.f;
    if (gx >= 0 && gx < nx && gz >= 0 && gz < nz) {
      const int64_t p = gx + (int64_t)nx * gz;
      float ds = 0.f;
      if (gx >= R && gx <= nx - R - 1) {
        const float* row = s_sxy + rr * SXW + cc + R;
        float acc = 0.f;
#pragma unroll
        for (int m = 1; m <= R; ++m) acc += G.c[m - 1] * (row[m - 1] - row[-m]);
        ds = acc * G.inv_dx;
      }
      if (gz >= R && gz <= nz - R - 1) {
        const float* col = s_szy + (rr + R) * BW + cc;
        float acc = 0.f;
#pragma unroll
        for (int m = 1; m <= R; ++m) acc += G.c[m - 1] * (col[(m - 1) * BW] - col[-m * BW]);
        ds += acc * G.inv_dz;
      }
      if (nbs) {
        if (nbs <= MAX_BOX_SRC) {
          for (int k = 0; k < nbs; ++k)
            if (s_src[k] == e) ds += s_amp[k];
        } else {
          for (int k = 0; k < S.nsrc; ++k)
            if (S.src_pt[k] == p) ds += S.amp ? (float)S.amp[k] : S.amp_const;
        }
      }
      if (S.inj) ds += S.inj[p];
      vn = (v[p] + ds * F.b[p]) * F.taper[p];
    }
    s_v[e] = vn;
  }
  __syncthreads();

  float* __restrict__ vo = F.v[1 - par];
  float* __restrict__ sxyo = F.sxy[1 - par];
  float* __restrict__ szyo = F.szy[1 - par];
  float* __restrict__ uo = F.u[1 - par];
#pragma unroll
  for (int k = 0; k < (TX * TZ) / NT; ++k) {
    const int e = tid + k * NT;
    const int tz = e / TX, tx = e - tz * TX;
    const int i = x0 + tx, j = z0 + tz;
    if (i >= nx || j >= nz) continue;
    const int64_t p = i + (int64_t)nx * j;
    const int cc = tx + R - 1, rr = tz + R - 1;
    const float vn = s_v[rr * BW + cc];
    if (S.snap_pre) S.snap_pre[p] = S.snap_pre_u ? u[p] : v[p];
    vo[p] = vn;
    const float dtmu = F.dtmu[p];
    if (i <= nx - 2) {
      float nw = s_sxy[rr * SXW + cc + R];
      if (i >= R - 1 && i <= nx - R - 1) {
        const float* row = s_v + rr * BW + cc;
        float acc = 0.f;
#pragma unroll
        for (int m = 1; m <= R; ++m) acc += G.c[m - 1] * (row[m] - row[1 - m]);
        nw += dtmu * (acc * G.inv_dx);
      }
      sxyo[p] = nw;
    }
    if (j <= nz - 2) {
      float nw = s_szy[(rr + R) * BW + cc];
      if (j >= R - 1 && j <= nz - R - 1) {
        const float* col = s_v + rr * BW + cc;
        float acc = 0.f;
#pragma unroll
        for (int m = 1; m <= R; ++m) acc += G.c[m - 1] * (col[m * BW] - col[(1 - m) * BW]);
        nw += dtmu * (acc * G.inv_dz);
      }
      szyo[p] = nw;
    }
    float x = vn;
    if (S.has_u) {
      x = u[p] + vn * G.dt;
      uo[p] = x;
    }
    if (S.snap_dft) S.snap_dft[p] = x;
  }
  if (S.nrec) {
    __syncthreads();
    for (int k = tid; k < S.nrec; k += NT) {
      const int p = S.rec_pt[k];
      const int gx = p % nx, gz = p / nx;
      if (gx >= x0 && gx < x0 + TX && gz >= z0 && gz < z0 + TZ)
        S.seis_col[k] = (double)(S.rec_u ? uo[p] : vo[p]);
    }
  }
}

// ---- point kernels ---------------------------------------------------------------
template <int R>
__device__ __forceinline__ float dx32(const Grid32& G, const float* f, const float* g, int i, int j) {
  if (i < R - 1 || i > G.nx - R - 1) return 0.f;
  const float* F = f + (int64_t)G.nx * j;
  const float* H = g ? g + (int64_t)G.nx * j : nullptr;
  float acc = 0.f;
#pragma unroll
  for (int m = 1; m <= R; ++m) {
    float a = H ? F[i + m] - H[i + m] : F[i + m];
    float b = H ? F[i - m + 1] - H[i - m + 1] : F[i - m + 1];
    acc += G.c[m - 1] * (a - b);
  }
  return acc * G.inv_dx;
}

template <int R>
__device__ __forceinline__ float dz32(const Grid32& G, const float* f, const float* g, int i, int j) {
  if (j < R - 1 || j > G.nz - R - 1) return 0.f;
  float acc = 0.f;
#pragma unroll
  for (int m = 1; m <= R; ++m) {
    const int64_t qa = i + (int64_t)G.nx * (j + m), qb = i + (int64_t)G.nx * (j - m + 1);
    float a = g ? f[qa] - g[qa] : f[qa];
    float b = g ? f[qb] - g[qb] : f[qb];
    acc += G.c[m - 1] * (a - b);
  }
  return acc * G.inv_dz;
}

// forward1 Born source before div_s: sxy += dt*dmu*dx_v(G_in(:,:,i))  (in place on the read buffers)
template <int R>
__global__ void k32_born_pre(Grid32 G, float* sxy, float* szy, const float* dtdmu, const float* Gs) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= G.nx || j >= G.nz) return;
  const int64_t p = i + (int64_t)G.nx * j;
  if (i <= G.nx - 2) sxy[p] += dtdmu[p] * dx32<R>(G, Gs, nullptr, i, j);
  if (j <= G.nz - 2) szy[p] += dtdmu[p] * dz32<R>(G, Gs, nullptr, i, j);
}

// correlation / adjoint Born term after the stress update: -= dmu*dx_v(C(n) - C(n+1))
template <int R>
__global__ void k32_born_post(Grid32 G, float* sxy, float* szy, const float* dmu, const float* Ca, const float* Cb) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= G.nx || j >= G.nz) return;
  const int64_t p = i + (int64_t)G.nx * j;
  if (i <= G.nx - 2) sxy[p] -= dmu[p] * dx32<R>(G, Ca, Cb, i, j);
  if (j <= G.nz - 2) szy[p] -= dmu[p] * dz32<R>(G, Ca, Cb, i, j);
}

// K_mu -= dx_v(u).*dx_v(u_fwd)*fw ; K_mu -= dz_v(u).*dz_v(u_fwd)*fw   (FP32 strains, FP64 sum)
template <int R>
__global__ void k32_kmu(Grid32 G, const float* u, const float* uf, double* Kmu, float fw) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= G.nx || j >= G.nz) return;
  const int64_t p = i + (int64_t)G.nx * j;
  double k = Kmu[p];
  if (i <= G.nx - 2) k -= (double)(dx32<R>(G, u, nullptr, i, j) * dx32<R>(G, uf, nullptr, i, j) * fw);
  if (j <= G.nz - 2) k -= (double)(dz32<R>(G, u, nullptr, i, j) * dz32<R>(G, uf, nullptr, i, j) * fw);
  Kmu[p] = k;
}

__global__ void k32_prep(const double* mu, const double* rho, const double* ab, double dt,
                         float* b, float* taper, float* dtmu, int64_t n) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= n) return;
  b[p] = (float)(dt / rho[p]);
  taper[p] = (float)ab[p];
  dtmu[p] = (float)(dt * mu[p]);
}

__global__ void k32_scale_f(const double* a, double s, float* out, int64_t n) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < n) out[p] = (float)(s * a[p]);
}

__global__ void k32_f_from_d(const double* a, float* out, int64_t n) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < n) out[p] = (float)a[p];
}

// P planes of the field source: P_k = spec(k) * (sum_b M(k,b) sd_b) * (Xre_k + i*sign*Xim_k)
// written as 2K float planes [Re P_0..Re P_{K-1}, Im P_0..Im P_{K-1}].
__global__ void k32_make_P(int K, int ncol, const double* M, const double* sd, const double* spec,
                           const double* Xre, const double* Xim, double sign, float* P, int64_t np) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  double sdv[16];
  for (int b = 0; b < ncol && b < 16; ++b) sdv[b] = sd[p + np * b];
  for (int k = 0; k < K; ++k) {
    double dist = 0.0;
    for (int b = 0; b < ncol; ++b) dist += M[k + (int64_t)K * b] * (b < 16 ? sdv[b] : sd[p + np * b]);
    const double R = spec[k] * dist;
    P[p + np * k] = (float)(R * Xre[p + np * k]);
    P[p + np * (K + k)] = (float)(R * sign * (Xim ? Xim[p + np * k] : 0.0));
  }
}

// K_s(:,:,b) = (dw/dt) sum_k M(k,b) spec(k) (G_re U_re - G_im U_im), U = sum_n u_n e^{-iwt}dt/sqrt(2pi)
__global__ void k32_source_kernel(int K, int ncol, const double* M, const double* spec,
                                  const double* Gre, const double* Gim, const double* Ure,
                                  const double* Uim, double scale, double* Ks, int64_t np) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  for (int b = 0; b < ncol; ++b) {
    double acc = 0.0;
    for (int k = 0; k < K; ++k) {
      const int64_t q = p + np * k;
      acc += M[k + (int64_t)K * b] * spec[k] * (Gre[q] * Ure[q] - Gim[q] * Uim[q]);
    }
    Ks[p + np * b] = scale * acc;
  }
}

// ---- host side ---------------------------------------------------------------------
struct Run {
  Grid32 G{};
  Fields32 F{};
  dim3 sgrid, pgrid, pblock{32, 8};
  int R = 2;
  int* rec_pt = nullptr;
  int* src_pt = nullptr;
  int64_t np = 0;
};

fd2d_status launch_step(fd2d_ctx* ctx, const Run& r, const Step32& s) {
  const int t0 = timer_begin(ctx, ctx->stream);
  switch (r.R) {
    case 1: k32_step<1><<<r.sgrid, NT, 0, ctx->stream>>>(r.G, r.F, s); break;
    case 2: k32_step<2><<<r.sgrid, NT, 0, ctx->stream>>>(r.G, r.F, s); break;
    case 3: k32_step<3><<<r.sgrid, NT, 0, ctx->stream>>>(r.G, r.F, s); break;
    default: k32_step<4><<<r.sgrid, NT, 0, ctx->stream>>>(r.G, r.F, s); break;
  }
  timer_end(ctx, ctx->stream, t0, s.has_u ? FD2D_TIMER_STEP_VU : FD2D_TIMER_STEP_V, r.np);
  return after_launch(ctx, "k32_step");
}

#define FD2D_DISPATCH_R(R_, KERNEL, ...)                                                 \
  switch (R_) {                                                                          \
    case 1: KERNEL<1><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;        \
    case 2: KERNEL<2><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;        \
    case 3: KERNEL<3><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;        \
    default: KERNEL<4><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;       \
  }

fd2d_status init_run(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a, bool with_u, Run& r) {
  const int64_t np = g.npts();
  r.np = np;
  r.R = g.r;
  r.G.nx = g.nx;
  r.G.nz = g.nz;
  for (int m = 0; m < 4; ++m) r.G.c[m] = (float)g.c[m];
  r.G.inv_dx = (float)(1.0 / g.dx);
  r.G.inv_dz = (float)(1.0 / g.dz);
  r.G.dt = (float)g.dt;
  float *b, *taper, *dtmu;
  FD2D_TRY(workspace_t(ctx, "f32.b", np, &b));
  FD2D_TRY(workspace_t(ctx, "f32.taper", np, &taper));
  FD2D_TRY(workspace_t(ctx, "f32.dtmu", np, &dtmu));
  double* ab;
  FD2D_TRY(upload(ctx, "f32.absbound64", g.absbound, &ab));
  k32_prep<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(a.mu, a.rho, ab, g.dt, b, taper, dtmu, np);
  FD2D_TRY(after_launch(ctx, "k32_prep"));
  r.F.b = b;
  r.F.taper = taper;
  r.F.dtmu = dtmu;
  static const char* names[2][4] = {{"f32.v0", "f32.sxy0", "f32.szy0", "f32.u0"},
                                    {"f32.v1", "f32.sxy1", "f32.szy1", "f32.u1"}};
  for (int q = 0; q < 2; ++q) {
    FD2D_TRY(workspace_t(ctx, names[q][0], np, &r.F.v[q]));
    FD2D_TRY(workspace_t(ctx, names[q][1], np, &r.F.sxy[q]));
    FD2D_TRY(workspace_t(ctx, names[q][2], np, &r.F.szy[q]));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.F.v[q], 0, np * 4, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.F.sxy[q], 0, np * 4, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.F.szy[q], 0, np * 4, ctx->stream));
    if (with_u) {
      FD2D_TRY(workspace_t(ctx, names[q][3], np, &r.F.u[q]));
      FD2D_CUDA(ctx, cudaMemsetAsync(r.F.u[q], 0, np * 4, ctx->stream));
    } else {
      r.F.u[q] = nullptr;
    }
  }
  std::vector<int> rec(a.rec_idx), src(a.src_idx);
  if (rec.empty()) rec.push_back(0);
  if (src.empty()) src.push_back(0);
  FD2D_TRY(upload(ctx, "f32.rec", rec, &r.rec_pt));
  FD2D_TRY(upload(ctx, "f32.src", src, &r.src_pt));
  r.sgrid = dim3((g.nx + TX - 1) / TX, (g.nz + TZ - 1) / TZ);
  r.pgrid = dim3((g.nx + 31) / 32, (g.nz + 7) / 8);
  return FD2D_OK;
}

// Frequency-band weights (interpol_matrix) on the device.
fd2d_status interp_dev(fd2d_ctx* ctx, const Geometry& g, double** M) {
  std::vector<double> h;
  std::string err;
  fd2d_status s = make_interpol_matrix(g.K, g.nb, h, err);
  if (s != FD2D_OK) return set_error(ctx, s, err);
  return upload(ctx, "f32.interp", h, M);
}

// Effective spectrum: sum over noise sources (they share one distribution).
fd2d_status spectrum_eff(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a, double** out) {
  std::vector<double> h((size_t)g.K * std::max(a.n_src, 1));
  FD2D_CUDA(ctx, cudaMemcpyAsync(h.data(), a.spectrum, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
  FD2D_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<double> e(g.K, 0.0);
  for (int s = 0; s < a.n_src; ++s)
    for (int k = 0; k < g.K; ++k) e[k] += h[k + (size_t)g.K * s];
  return upload(ctx, "f32.spec_eff", e, out);
}

// Injection planes for the listed coefficient rows (ifft rows, one per event).
// Builds P from X (G or conj(stf)) and evaluates inj[j] = Re sum_k P_k c_{row_j,k}.
struct Injection {
  std::vector<int> step_of_event;  // 1-based step n of event j
  std::vector<int> row_of_event;   // coefficient row used by event j
  float* planes = nullptr;         // [chunk][np]
  int chunk = 0, first = 0, count = 0;  // events [first, first+count) resident
  float* P = nullptr;
  float* B = nullptr;              // [2K][n_events] float
  int n_events = 0;
};

fd2d_status build_injection(fd2d_ctx* ctx, const Geometry& g, const double* Xre, const double* Xim,
                            double sign, const double* spec_eff, const double* M, const double* sd,
                            Injection& inj) {
  const int64_t np = g.npts();
  const int K = g.K, ncol = g.nb == 0 ? 1 : g.nb;
  inj.n_events = (int)inj.step_of_event.size();
  if (inj.n_events == 0) return FD2D_OK;
  FD2D_TRY(workspace_t(ctx, "f32.P", (size_t)np * 2 * K, &inj.P));
  k32_make_P<<<(unsigned)((np + 127) / 128), 128, 0, ctx->stream>>>(K, ncol, M, sd, spec_eff, Xre, Xim, sign, inj.P, np);
  FD2D_TRY(after_launch(ctx, "k32_make_P"));
  // B[k][j] = Re c(row_j, k); B[K+k][j] = -Im c(row_j, k)   (c = ifft_coeff, dw)
  std::vector<float> B((size_t)2 * K * inj.n_events);
  for (int j = 0; j < inj.n_events; ++j) {
    const int n = (inj.row_of_event[j] + 1) * g.fs;  // step whose time this row holds
    for (int k = 0; k < K; ++k) {
      double re, im;
      dft_coeff(g.w[k] * g.t_corr[n - 1], g.dw, re, im);
      B[(size_t)k * inj.n_events + j] = (float)re;
      B[(size_t)(K + k) * inj.n_events + j] = (float)(-im);
    }
  }
  FD2D_TRY(upload(ctx, "f32.injB", B, &inj.B));
  // resident chunk of injection planes (bounded to ~4 GiB)
  const size_t cap = (size_t)4 << 30;
  inj.chunk = (int)std::max<int64_t>(1, std::min<int64_t>(inj.n_events, (int64_t)(cap / (np * 4))));
  FD2D_TRY(workspace_t(ctx, "f32.inj", (size_t)np * inj.chunk, &inj.planes));
  inj.first = 0;
  inj.count = 0;
  return FD2D_OK;
}

// Plane of event j (evaluates the next chunk of planes when j is not resident).
fd2d_status injection_plane(fd2d_ctx* ctx, const Geometry& g, Injection& inj, int j, const float** out) {
  if (j < inj.first || j >= inj.first + inj.count) {
    inj.first = j;
    inj.count = std::min(inj.chunk, inj.n_events - j);
    ContractArgs c;
    c.A = inj.P;
    c.lda = g.npts();
    c.Kd = 2 * g.K;
    c.B = inj.B + j;
    c.ldb = inj.n_events;
    c.M = (int)g.npts();
    c.N = inj.count;
    c.out32 = inj.planes;
    c.ldo = g.npts();
    FD2D_TRY(contract(ctx, ctx->stream, c));
  }
  *out = inj.planes + (size_t)(j - inj.first) * g.npts();
  return FD2D_OK;
}

// DFT accumulation: snapshots of one field at listed steps, contracted in chunks.
struct Dft {
  int T = 0;          // chunk length
  int filled = 0;     // snapshots in the current chunk
  int done = 0;       // events already contracted
  float* snaps = nullptr;
  struct Target {
    float* B = nullptr;  // [n_events][2K] rows
    double *re = nullptr, *im = nullptr;
  };
  std::vector<Target> targets;
  int n_events = 0;
};

fd2d_status dft_init(fd2d_ctx* ctx, const Geometry& g, int n_events, Dft& d) {
  d.n_events = n_events;
  if (n_events == 0) return FD2D_OK;
  const int64_t np = g.npts();
  const size_t cap = (size_t)2 << 30;  // snapshot chunk <= 2 GiB
  d.T = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)n_events, (int64_t)1024, (int64_t)(cap / (np * 4))}));
  return workspace_t(ctx, "f32.dft_snaps", (size_t)np * d.T, &d.snaps);
}

// rows[e] = (re, im) coefficient pairs for event e, laid out [e][2K] as float.
fd2d_status dft_add_target(fd2d_ctx* ctx, const char* name, const std::vector<float>& rows, double* re,
                           double* im, Dft& d) {
  Dft::Target t;
  FD2D_TRY(upload(ctx, name, rows, &t.B));
  t.re = re;
  t.im = im;
  d.targets.push_back(t);
  return FD2D_OK;
}

float* dft_slot(const Geometry& g, Dft& d) { return d.snaps + (size_t)d.filled * g.npts(); }

fd2d_status dft_flush(fd2d_ctx* ctx, const Geometry& g, Dft& d) {
  if (d.filled == 0) return FD2D_OK;
  for (auto& t : d.targets) {
    ContractArgs c;
    c.A = d.snaps;
    c.lda = g.npts();
    c.Kd = d.filled;
    c.B = t.B + (size_t)d.done * 2 * g.K;
    c.ldb = 2 * g.K;
    c.M = (int)g.npts();
    c.N = 2 * g.K;
    c.acc0 = t.re;
    c.acc1 = t.im;
    c.nsplit = g.K;
    c.ldacc = g.npts();
    FD2D_TRY(contract(ctx, ctx->stream, c));
  }
  d.done += d.filled;
  d.filled = 0;
  return FD2D_OK;
}

fd2d_status dft_push(fd2d_ctx* ctx, const Geometry& g, Dft& d) {
  ++d.filled;
  if (d.filled == d.T || d.done + d.filled == d.n_events) return dft_flush(ctx, g, d);
  return FD2D_OK;
}

}  // namespace

// ---------------------------------------------------------------------------------
fd2d_status fp32_forward1(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Run r;
  FD2D_TRY(init_run(ctx, g, a, false, r));
  const int nt = g.nt, K = g.K;
  const int64_t np = r.np;
  // DFT events: steps n with mod(n+nt-1, freq_samp) == 0; coefficient of step n is
  // 1/sqrt(2pi) exp(-i w t(n)) dt with t(n) = (n-1) dt; conj(G_fft) is returned, so
  // the imaginary column carries -Im.
  std::vector<int> ev;
  for (int n = 1; n <= nt; ++n)
    if ((n + nt - 1) % g.fs == 0) ev.push_back(n);
  Dft d;
  FD2D_TRY(dft_init(ctx, g, (int)ev.size(), d));
  if (!ev.empty()) {
    std::vector<float> rows((size_t)ev.size() * 2 * K);
    for (size_t e = 0; e < ev.size(); ++e)
      for (int k = 0; k < K; ++k) {
        double re, im;
        dft_coeff(-(g.w[k] * g.t_fwd[ev[e] - 1]), g.dt, re, im);
        rows[e * 2 * K + k] = (float)re;
        rows[e * 2 * K + K + k] = (float)(-im);
      }
    FD2D_TRY(dft_add_target(ctx, "f32.dftB0", rows, a.G_re, a.G_im, d));
  }
  FD2D_CUDA(ctx, cudaMemsetAsync(a.G_re, 0, (size_t)np * K * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.G_im, 0, (size_t)np * K * 8, ctx->stream));
  float* dtdmu = nullptr;
  float* Gs = nullptr;
  const bool born = a.dmu != nullptr;
  if (born) {
    FD2D_TRY(workspace_t(ctx, "f32.dtdmu", np, &dtdmu));
    k32_scale_f<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(a.dmu, g.dt, dtdmu, np);
    FD2D_TRY(after_launch(ctx, "k32_scale_f"));
  }
  (void)Gs;
  const int nr = (int)a.rec_idx.size();
  int i_fw_out = 0, i_fw_in = 0, par = 0;
  for (int n = 1; n <= nt; ++n) {
    Step32 s{};
    s.par = par;
    if (a.mode != 0 && (n + nt - 1) % g.fw == 0) s.snap_pre = a.G_out + (size_t)np * (i_fw_out++);
    if (born) {
      FD2D_DISPATCH_R(r.R, k32_born_pre, r.G, r.F.sxy[par], r.F.szy[par], dtdmu, a.G_in + (size_t)np * (i_fw_in++));
      FD2D_TRY(after_launch(ctx, "k32_born_pre"));
    } else {
      s.src_pt = r.src_pt;
      s.nsrc = (int)a.src_idx.size();
      s.amp_const = 1.0e9f;
    }
    const bool is_dft = (n + nt - 1) % g.fs == 0;
    if (is_dft) s.snap_dft = dft_slot(g, d);
    s.rec_pt = r.rec_pt;
    s.nrec = nr;
    s.seis_col = a.seis + (size_t)nr * (n - 1);
    FD2D_TRY(launch_step(ctx, r, s));
    if (is_dft) FD2D_TRY(dft_push(ctx, g, d));
    par ^= 1;
  }
  return FD2D_OK;
}

fd2d_status fp32_correlation(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Run r;
  FD2D_TRY(init_run(ctx, g, a, true, r));
  const int ntc = g.ntc;
  const int64_t np = r.np;
  double *M, *spec;
  FD2D_TRY(interp_dev(ctx, g, &M));
  FD2D_TRY(spectrum_eff(ctx, g, a, &spec));
  Injection inj;
  for (int n = 1; n <= ntc; ++n)
    if (n % g.fs == 0) {
      inj.step_of_event.push_back(n);
      inj.row_of_event.push_back(n / g.fs - 1);
    }
  FD2D_TRY(build_injection(ctx, g, a.Gin_re, a.Gin_im, 1.0, spec, M, a.source_dist, inj));
  float* dmu32 = nullptr;
  const bool born = a.dmu != nullptr;
  if (born) {
    FD2D_TRY(workspace_t(ctx, "f32.dmu", np, &dmu32));
    k32_f_from_d<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(a.dmu, dmu32, np);
    FD2D_TRY(after_launch(ctx, "k32_f_from_d"));
  }
  const int nr = (int)a.rec_idx.size();
  int i_fw_out = 0, par = 0, ev = 0;
  for (int n = 1; n <= ntc; ++n) {
    Step32 s{};
    s.par = par;
    s.has_u = 1;
    if (a.mode != 0 && n % g.fw == 0) {
      s.snap_pre = a.C_out + (size_t)np * (i_fw_out++);
      s.snap_pre_u = 1;
    }
    if (n % g.fs == 0) FD2D_TRY(injection_plane(ctx, g, inj, ev++, &s.inj));
    s.rec_pt = r.rec_pt;
    s.nrec = nr;
    s.seis_col = a.seis + (size_t)nr * (n - 1);
    s.rec_u = 1;  // u does not depend on this step's Born stress correction
    FD2D_TRY(launch_step(ctx, r, s));
    par ^= 1;
    if (born && n != ntc) {
      FD2D_DISPATCH_R(r.R, k32_born_post, r.G, r.F.sxy[par], r.F.szy[par], dmu32,
                      a.C_in + (size_t)np * (n - 1), a.C_in + (size_t)np * n);
      FD2D_TRY(after_launch(ctx, "k32_born_post"));
    }
  }
  return FD2D_OK;
}

fd2d_status fp32_adjoint(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Run r;
  FD2D_TRY(init_run(ctx, g, a, true, r));
  const int ntc = g.ntc, K = g.K, mode = a.mode;
  const int64_t np = r.np;
  const int ncol = g.nb == 0 ? 1 : g.nb;
  const int64_t d0 = a.stf_dims[0], d1 = a.stf_dims[1], d2 = a.stf_dims[2];
  const bool stf_empty = !a.stf_re || d0 * d1 * d2 == 0;
  const int64_t size3 = stf_empty ? 1 : d2;
  const bool stf2d = !stf_empty && size3 == 1, stf3d = !stf_empty && size3 != 1;
  int nt_loop = ntc;
  if ((mode == 0 || mode == 1) && size3 != 1) nt_loop = g.nt;  // code/run_noise_adjoint.m:165-167
  const bool Gvalid = a.Gin_re != nullptr && a.n_G == K;
  const bool born = a.dmu != nullptr && a.n_C_in == ntc;
  const bool save_u = mode == 11 || mode == 13;
  const bool dft_u = mode == 1 || mode == 12 || mode == 13;
  const bool have_fwd = a.u_fwd != nullptr && a.n_u_fwd > 0;
  const int n_ftc = ntc / g.fs;
  // The reference shares one counter i_ftc between the field-source injection
  // and the stf_fft DFT (code/run_noise_adjoint.m:265,343); replay it.
  std::vector<int> inj_step, inj_row, dft_step, dft_row;
  {
    int i_ftc = 0;
    for (int n = 1; n <= nt_loop; ++n) {
      if (n % g.fs) continue;
      if (stf3d) { inj_step.push_back(n); inj_row.push_back(i_ftc++); }
      if (dft_u) { dft_step.push_back(n); dft_row.push_back(i_ftc++); }
    }
    if (i_ftc > n_ftc) return set_error(ctx, FD2D_ERR_INDEX, "fft_coeff row past the end");
  }
  double *M, *spec = nullptr;
  FD2D_TRY(interp_dev(ctx, g, &M));
  if (a.spectrum) FD2D_TRY(spectrum_eff(ctx, g, a, &spec));
  Injection inj;
  if (stf3d && a.source_dist) {
    inj.step_of_event = inj_step;
    inj.row_of_event = inj_row;
    const double* sim = a.stf_im;
    if (!sim) {
      double* z;
      FD2D_TRY(workspace_t(ctx, "f32.zero_im", (size_t)np * K, &z));
      FD2D_CUDA(ctx, cudaMemsetAsync(z, 0, (size_t)np * K * 8, ctx->stream));
      sim = z;
    }
    FD2D_TRY(build_injection(ctx, g, a.stf_re, sim, -1.0, spec, M, a.source_dist, inj));
  }
  // DFT of u at the fs steps: stf_fft with the rows the reference uses, and the
  // natural-row spectrum U that forms the source kernel.
  std::vector<int> ev;
  for (int n = 1; n <= nt_loop; ++n)
    if (n % g.fs == 0 && (dft_u || Gvalid)) ev.push_back(n);
  bool natural = true;
  for (size_t e = 0; e < dft_row.size(); ++e) natural &= dft_row[e] == dft_step[e] / g.fs - 1;
  FD2D_CUDA(ctx, cudaMemsetAsync(a.sf_re, 0, (size_t)np * K * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.sf_im, 0, (size_t)np * K * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.Kout, 0, (size_t)np * 8 * (ncol + 1), ctx->stream));
  Dft d;
  FD2D_TRY(dft_init(ctx, g, (int)ev.size(), d));
  double *Ure = nullptr, *Uim = nullptr;
  auto rows_for = [&](const std::vector<int>& rows_of_event) {
    std::vector<float> rows(ev.size() * 2 * K);
    for (size_t e = 0; e < ev.size(); ++e) {
      const int n = (rows_of_event[e] + 1) * g.fs;
      for (int k = 0; k < K; ++k) {
        double re, im;
        dft_coeff(-(g.w[k] * g.t_corr[n - 1]), g.dt, re, im);
        rows[e * 2 * K + k] = (float)re;
        rows[e * 2 * K + K + k] = (float)im;
      }
    }
    return rows;
  };
  if (!ev.empty()) {
    std::vector<int> nat(ev.size());
    for (size_t e = 0; e < ev.size(); ++e) nat[e] = ev[e] / g.fs - 1;
    if (dft_u) {
      FD2D_TRY(dft_add_target(ctx, "f32.dftB0", rows_for(dft_row), a.sf_re, a.sf_im, d));
      if (natural) { Ure = a.sf_re; Uim = a.sf_im; }
    }
    if (Gvalid && !Ure) {
      FD2D_TRY(workspace_t(ctx, "f32.Ure", (size_t)np * K, &Ure));
      FD2D_TRY(workspace_t(ctx, "f32.Uim", (size_t)np * K, &Uim));
      FD2D_CUDA(ctx, cudaMemsetAsync(Ure, 0, (size_t)np * K * 8, ctx->stream));
      FD2D_CUDA(ctx, cudaMemsetAsync(Uim, 0, (size_t)np * K * 8, ctx->stream));
      FD2D_TRY(dft_add_target(ctx, "f32.dftB1", rows_for(nat), Ure, Uim, d));
    }
  }
  float* dmu32 = nullptr;
  if (born) {
    FD2D_TRY(workspace_t(ctx, "f32.dmu", np, &dmu32));
    k32_f_from_d<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(a.dmu, dmu32, np);
    FD2D_TRY(after_launch(ctx, "k32_f_from_d"));
  }
  double* Kmu = a.Kout + (size_t)np * ncol;
  const int nr = (int)a.rec_idx.size();
  int i_fw_out = 0, i_fw_in = 0, par = 0, j_inj = 0;
  for (int n = 1; n <= nt_loop; ++n) {
    Step32 s{};
    s.par = par;
    s.has_u = 1;
    if (save_u && n % g.fw == 0) {
      s.snap_pre = a.C_out + (size_t)np * (i_fw_out++);
      s.snap_pre_u = 1;
    }
    if (stf2d) {
      s.src_pt = r.src_pt;
      s.nsrc = (int)a.src_idx.size();
      s.amp = a.stf_re + (size_t)d0 * (n - 1);
    } else if (!inj.step_of_event.empty() && j_inj < inj.n_events && inj.step_of_event[j_inj] == n) {
      FD2D_TRY(injection_plane(ctx, g, inj, j_inj++, &s.inj));
    }
    const bool is_dft = d.n_events && n % g.fs == 0;
    if (is_dft) s.snap_dft = dft_slot(g, d);
    s.rec_pt = r.rec_pt;
    s.nrec = nr;
    s.seis_col = a.seis + (size_t)nr * (n - 1);
    s.rec_u = 1;
    FD2D_TRY(launch_step(ctx, r, s));
    par ^= 1;
    if (born && n != ntc) {
      FD2D_DISPATCH_R(r.R, k32_born_post, r.G, r.F.sxy[par], r.F.szy[par], dmu32,
                      a.C_in + (size_t)np * (n - 1), a.C_in + (size_t)np * n);
      FD2D_TRY(after_launch(ctx, "k32_born_post"));
    }
    if (have_fwd && a.n_u_fwd >= i_fw_in + 1 && n % g.fw == 0) {
      const float* uf = a.u_fwd + (size_t)np * (a.n_u_fwd - 1 - i_fw_in);
      FD2D_DISPATCH_R(r.R, k32_kmu, r.G, r.F.u[par], uf, Kmu, (float)g.fw);
      FD2D_TRY(after_launch(ctx, "k32_kmu"));
      ++i_fw_in;
    }
    if (is_dft) FD2D_TRY(dft_push(ctx, g, d));
  }
  if (Gvalid) {
    k32_source_kernel<<<(unsigned)((np + 127) / 128), 128, 0, ctx->stream>>>(
        K, ncol, M, spec, a.Gin_re, a.Gin_im, Ure, Uim, g.dw / g.dt, a.Kout, np);
    FD2D_TRY(after_launch(ctx, "k32_source_kernel"));
  }
  if (nt_loop < ntc && nr > 0)
    FD2D_CUDA(ctx, cudaMemsetAsync(a.seis + (size_t)nr * nt_loop, 0, (size_t)nr * (ntc - nt_loop) * 8, ctx->stream));
  return FD2D_OK;
}

}  // namespace fd2d
