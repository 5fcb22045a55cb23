// solver_fp64.cu -- the plain FP64 GPU form of the three solvers.
//
// One solve at a time, FP64 throughout, one thread per grid point, and the
// reference's per-step structure: the DFT, the correlation-source injection
// and the source kernel are evaluated step by step as K-term sums per point,
// exactly as code/run_forward1_green.m:176-183, code/run_forward2_correlation.m:
// 195-216 and code/run_noise_adjoint.m:302-346 do.  It is the numerical twin of
// the CPU oracle (<= 1e-10 relative L2) and the denominator of the FP32 form's
// speed-up.  Divisions by dx, dz and rho are multiplications by reciprocals;
// the derivatives of `single` snapshots are evaluated in single precision with
// the reference's expression order (MATLAB evaluates mixed single/double
// arithmetic in single).
#include "common.cuh"

namespace fd2d {
namespace {

struct P64 {
  int nx, nz, r, order;
  int64_t np;
  double dt, inv_dx, inv_dz;
  double c[4];
  float hx, hx8, hx24, hz, hz8, hz24;  // (float)dx, (float)(8dx), (float)(24dx), same for z
  float cf[4];
  double *v, *sxy, *szy, *u;
  const double *mu, *inv_rho, *absbound, *dmu;
  const int *src_head, *src_next;  // point-source chains (src_head[p] = first source or -1)
};

constexpr int BX = 32, BY = 8;

// ---- FD operators at one point (code/propagation/div_s.m, dx_v.m, dz_v.m) --------
// sxy: (nx-1)-by-nz, szy: nx-by-(nz-1).  Rows/columns outside the reference's
// loop ranges are zero.
__device__ __forceinline__ double div_s_at(const P64& P, int i, int j) {
  const int nx = P.nx, nz = P.nz, r = P.r;
  double o = 0.0;
  if (i >= r && i <= nx - r - 1) {
    const double* S = P.sxy + (int64_t)(nx - 1) * j;
    double acc = 0.0;
#pragma unroll
    for (int m = 1; m <= 4; ++m)
      if (m <= r) acc += P.c[m - 1] * (S[i + m - 1] - S[i - m]);
    o = acc * P.inv_dx;
  }
  if (j >= r && j <= nz - r - 1) {
    double acc = 0.0;
#pragma unroll
    for (int m = 1; m <= 4; ++m)
      if (m <= r) acc += P.c[m - 1] * (P.szy[i + (int64_t)nx * (j + m - 1)] - P.szy[i + (int64_t)nx * (j - m)]);
    o = o + acc * P.inv_dz;
  }
  return o;
}

// dx_v at out-row i (0-based) of column j of an nx-by-nz double field f.
__device__ __forceinline__ double dxv_at(const P64& P, const double* f, int i, int j) {
  if (i < P.r - 1 || i > P.nx - P.r - 1) return 0.0;
  const double* F = f + (int64_t)P.nx * j;
  double acc = 0.0;
#pragma unroll
  for (int m = 1; m <= 4; ++m)
    if (m <= P.r) acc += P.c[m - 1] * (F[i + m] - F[i - m + 1]);
  return acc * P.inv_dx;
}

__device__ __forceinline__ double dzv_at(const P64& P, const double* f, int i, int j) {
  if (j < P.r - 1 || j > P.nz - P.r - 1) return 0.0;
  double acc = 0.0;
#pragma unroll
  for (int m = 1; m <= 4; ++m)
    if (m <= P.r) acc += P.c[m - 1] * (f[i + (int64_t)P.nx * (j + m)] - f[i + (int64_t)P.nx * (j - m + 1)]);
  return acc * P.inv_dz;
}

// Single-precision derivative of a `single` field, in MATLAB's evaluation order:
// order 2: (a(i+1)-a(i))/dx; order 4: 9*(a(i+1)-a(i))/(8dx) - (a(i+2)-a(i-1))/(24dx).
// A(k) returns the single value at offset k; `diff` selects A - B (Born terms).
template <typename F>
__device__ __forceinline__ float dv_single(const P64& P, F A, int i, float h, float h8, float h24) {
  if (P.order == 2) return __fdiv_rn(__fsub_rn(A(i + 1), A(i)), h);
  if (P.order == 4) {
    float t1 = __fdiv_rn(__fmul_rn(9.0f, __fsub_rn(A(i + 1), A(i))), h8);
    float t2 = __fdiv_rn(__fsub_rn(A(i + 2), A(i - 1)), h24);
    return __fsub_rn(t1, t2);
  }
  float acc = 0.0f;
  for (int m = 1; m <= P.r; ++m) acc = __fadd_rn(acc, __fmul_rn(P.cf[m - 1], __fsub_rn(A(i + m), A(i - m + 1))));
  return __fdiv_rn(acc, h);
}

// d/dx of single field (f or f - g) at out-row i, column j.
__device__ __forceinline__ double dxv_single_at(const P64& P, const float* f, const float* g, int i, int j) {
  if (i < P.r - 1 || i > P.nx - P.r - 1) return 0.0;
  const float* F = f + (int64_t)P.nx * j;
  const float* G = g ? g + (int64_t)P.nx * j : nullptr;
  auto A = [&](int k) { return G ? __fsub_rn(F[k], G[k]) : F[k]; };
  return (double)dv_single(P, A, i, P.hx, P.hx8, P.hx24);
}

__device__ __forceinline__ double dzv_single_at(const P64& P, const float* f, const float* g, int i, int j) {
  if (j < P.r - 1 || j > P.nz - P.r - 1) return 0.0;
  auto A = [&](int k) {
    int64_t q = i + (int64_t)P.nx * k;
    return g ? __fsub_rn(f[q], g[q]) : f[q];
  };
  return (double)dv_single(P, A, j, P.hz, P.hz8, P.hz24);
}

// ---- kernels -------------------------------------------------------------------
__global__ void k64_inv(const double* rho, double* inv_rho, int64_t n) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < n) inv_rho[p] = 1.0 / rho[p];
}

// forward1 Born term (code/run_forward1_green.m:140-144):
// sxy += dt*dmu(1:nx-1,:) .* dx_v(G_in(:,:,i)), szy likewise.
__global__ void k64_born_pre(P64 P, const float* Gs) {
  int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= P.nx || j >= P.nz) return;
  const double dm = P.dt * P.dmu[i + (int64_t)P.nx * j];
  if (i < P.nx - 1) {
    int64_t q = i + (int64_t)(P.nx - 1) * j;
    P.sxy[q] = P.sxy[q] + dm * dxv_single_at(P, Gs, nullptr, i, j);
  }
  if (j < P.nz - 1) {
    int64_t q = i + (int64_t)P.nx * j;
    P.szy[q] = P.szy[q] + dm * dzv_single_at(P, Gs, nullptr, i, j);
  }
}

struct StepV {
  float* snap;            // single(field) before the step, or nullptr
  int snap_u;             // 1: snapshot u, 0: snapshot v
  const double* amp;      // per-source amplitudes (stride 1), or nullptr for amp_const
  double amp_const;
  int use_src;            // point sources active
  // field injection: sum_k spectrum(k,is) * dist_k .* X_k * c_k, X = Xre + i*sign*Xim
  const double *cre, *cim;     // coefficient row (K), nullptr = no injection this step
  const double *Xre, *Xim;     // K planes
  double xsign;
  const double* spectrum;      // K x n_src
  const double* dist;          // K planes
  int K, n_src;
  int add_per_source;          // correlation adds real(S(:,:,ns)) per noise source
};

__global__ void k64_v(P64 P, StepV S) {
  extern __shared__ double sh[];
  const int K = S.K;
  if (S.cre) {
    for (int k = threadIdx.y * BX + threadIdx.x; k < K; k += BX * BY) {
      sh[k] = S.cre[k];
      sh[K + k] = S.cim[k];
    }
    __syncthreads();
  }
  int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= P.nx || j >= P.nz) return;
  const int64_t p = i + (int64_t)P.nx * j;
  const int64_t np = P.np;
  if (S.snap) S.snap[p] = (float)(S.snap_u ? P.u[p] : P.v[p]);
  double ds = div_s_at(P, i, j);
  if (S.use_src) {
    for (int s = P.src_head[p]; s >= 0; s = P.src_next[s]) ds = ds + (S.amp ? S.amp[s] : S.amp_const);
  }
  if (S.cre) {
    double tr = 0.0;
    for (int is = 0; is < S.n_src; ++is) {
      double sr = 0.0;
      for (int k = 0; k < K; ++k) {
        const double R = S.spectrum[k + (int64_t)K * is] * S.dist[p + np * k];
        const double a = R * S.Xre[p + np * k];
        const double b = R * (S.xsign * S.Xim[p + np * k]);
        sr = sr + (a * sh[k] - b * sh[K + k]);
      }
      if (S.add_per_source) ds = ds + sr;
      else tr = tr + sr;
    }
    if (!S.add_per_source) ds = ds + tr;
  }
  const double vv = P.v[p] + (P.dt * ds) * P.inv_rho[p];
  P.v[p] = vv * P.absbound[p];
}

struct StepS {
  const float *born_a, *born_b;  // -dmu * grad(single(born_a - born_b)), or nullptr
  int update_u;
  // DFT accumulation of x (v or u after the update): X_k += x * c_k
  const double *dcre, *dcim;
  double *Dre, *Dim;
  int dft_of_u;
  // source kernel (code/run_noise_adjoint.m:302-320)
  const double *kcre, *kcim;   // ifft_coeff2(n,:)
  const double *Gre, *Gim, *spec, *M;
  double* Ks;
  int ncol;
  int K;
};

__global__ void k64_stress(P64 P, StepS S) {
  extern __shared__ double sh[];
  const int K = S.K;
  const bool dft = S.dcre != nullptr, ks = S.kcre != nullptr;
  for (int k = threadIdx.y * BX + threadIdx.x; k < K; k += BX * BY) {
    if (dft) { sh[k] = S.dcre[k]; sh[K + k] = S.dcim[k]; }
    if (ks) { sh[2 * K + k] = S.kcre[k]; sh[3 * K + k] = S.kcim[k]; }
  }
  if (dft || ks) __syncthreads();
  int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= P.nx || j >= P.nz) return;
  const int64_t p = i + (int64_t)P.nx * j;
  const int64_t np = P.np;
  const double dtmu = P.dt * P.mu[p];
  if (i < P.nx - 1) {
    const int64_t q = i + (int64_t)(P.nx - 1) * j;
    double val = P.sxy[q] + dtmu * dxv_at(P, P.v, i, j);
    if (S.born_a) val = val - P.dmu[p] * dxv_single_at(P, S.born_a, S.born_b, i, j);
    P.sxy[q] = val;
  }
  if (j < P.nz - 1) {
    double val = P.szy[p] + dtmu * dzv_at(P, P.v, i, j);
    if (S.born_a) val = val - P.dmu[p] * dzv_single_at(P, S.born_a, S.born_b, i, j);
    P.szy[p] = val;
  }
  double x = P.v[p];
  if (S.update_u) {
    x = P.u[p] + x * P.dt;
    P.u[p] = x;
  }
  if (dft) {
    for (int k = 0; k < K; ++k) {
      S.Dre[p + np * k] = S.Dre[p + np * k] + x * sh[k];
      S.Dim[p + np * k] = S.Dim[p + np * k] + x * sh[K + k];
    }
  }
  if (ks) {
    for (int ib = 0; ib < S.ncol; ++ib) {
      double mr = 0.0;
      for (int k = 0; k < K; ++k) {
        const double a = S.spec[k] * S.Gre[p + np * k];
        const double b = S.spec[k] * (-S.Gim[p + np * k]);
        const double er = a * sh[2 * K + k] - b * sh[3 * K + k];
        mr = mr + S.M[k + (int64_t)K * ib] * er;
      }
      S.Ks[p + np * ib] = S.Ks[p + np * ib] + mr * x;
    }
  }
}

// K_mu -= dx_v(u) .* dx_v(u_fwd(:,:,slot)) * fw  (then the z term)
// code/run_noise_adjoint.m:324-331
__global__ void k64_kmu(P64 P, const float* uf, double* Kmu, double fw) {
  int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
  if (i >= P.nx || j >= P.nz) return;
  const int64_t p = i + (int64_t)P.nx * j;
  double k = Kmu[p];
  if (i < P.nx - 1) k = k - (dxv_at(P, P.u, i, j) * dxv_single_at(P, uf, nullptr, i, j)) * fw;
  if (j < P.nz - 1) k = k - (dzv_at(P, P.u, i, j) * dzv_single_at(P, uf, nullptr, i, j)) * fw;
  Kmu[p] = k;
}

__global__ void k64_record(const double* f, const int* rec, int nr, double* col) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nr) col[i] = f[rec[i]];
}

__global__ void k64_negate(double* a, int64_t n) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p < n) a[p] = -a[p];
}

// distribution(:,:,k) = sum_b interpol_matrix(k,b) * source_distribution(:,:,b)
__global__ void k64_distribution(const double* M, int K, int ncol, const double* sd, double* dist, int64_t np) {
  int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  for (int k = 0; k < K; ++k) {
    double acc = 0.0;
    for (int b = 0; b < ncol; ++b) acc = acc + M[k + (int64_t)K * b] * sd[p + np * b];
    dist[p + np * k] = acc;
  }
}

// ---- host helpers ------------------------------------------------------------------
struct Base {
  P64 P{};
  dim3 grid, block{BX, BY};
  int* rec_idx = nullptr;
};

fd2d_status init_base(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a, bool with_u, Base& B) {
  P64& P = B.P;
  P.nx = g.nx; P.nz = g.nz; P.r = g.r; P.order = g.order; P.np = g.npts();
  P.dt = g.dt; P.inv_dx = 1.0 / g.dx; P.inv_dz = 1.0 / g.dz;
  for (int m = 0; m < 4; ++m) { P.c[m] = g.c[m]; P.cf[m] = (float)g.c[m]; }
  P.hx = (float)g.dx; P.hx8 = (float)(8 * g.dx); P.hx24 = (float)(24 * g.dx);
  P.hz = (float)g.dz; P.hz8 = (float)(8 * g.dz); P.hz24 = (float)(24 * g.dz);
  const size_t np = (size_t)g.npts();
  FD2D_TRY(workspace_t(ctx, "f64.v", np, &P.v));
  FD2D_TRY(workspace_t(ctx, "f64.sxy", np, &P.sxy));
  FD2D_TRY(workspace_t(ctx, "f64.szy", np, &P.szy));
  FD2D_CUDA(ctx, cudaMemsetAsync(P.v, 0, np * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(P.sxy, 0, np * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(P.szy, 0, np * 8, ctx->stream));
  if (with_u) {
    FD2D_TRY(workspace_t(ctx, "f64.u", np, &P.u));
    FD2D_CUDA(ctx, cudaMemsetAsync(P.u, 0, np * 8, ctx->stream));
  }
  double* inv_rho;
  FD2D_TRY(workspace_t(ctx, "f64.inv_rho", np, &inv_rho));
  k64_inv<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(a.rho, inv_rho, (int64_t)np);
  FD2D_TRY(after_launch(ctx, "k64_inv"));
  P.inv_rho = inv_rho;
  double* ab;
  FD2D_TRY(upload(ctx, "f64.absbound", *g.absbound, &ab));
  P.absbound = ab;
  P.mu = a.mu;
  P.dmu = a.dmu;
  // point-source chains in source order
  std::vector<int> head(np, -1), next(a.src_idx.size() + 1, -1), tail(np, -1);
  for (size_t s = 0; s < a.src_idx.size(); ++s) {
    int p = a.src_idx[s];
    if (head[p] < 0) head[p] = (int)s;
    else next[tail[p]] = (int)s;
    tail[p] = (int)s;
  }
  int *dh, *dn;
  FD2D_TRY(upload(ctx, "f64.src_head", head, &dh));
  FD2D_TRY(upload(ctx, "f64.src_next", next, &dn));
  P.src_head = dh;
  P.src_next = dn;
  std::vector<int> rec(a.rec_idx);
  if (rec.empty()) rec.push_back(0);
  FD2D_TRY(upload(ctx, "f64.rec", rec, &B.rec_idx));
  B.grid = dim3((g.nx + BX - 1) / BX, (g.nz + BY - 1) / BY);
  return FD2D_OK;
}

fd2d_status record(fd2d_ctx* ctx, const Base& B, const double* f, int nr, double* col) {
  if (nr == 0) return FD2D_OK;
  k64_record<<<(nr + 127) / 128, 128, 0, ctx->stream>>>(f, B.rec_idx, nr, col);
  return after_launch(ctx, "k64_record");
}

fd2d_status make_dist(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a, double** dist, double** Mdev) {
  std::vector<double> M;
  std::string err;
  fd2d_status s = make_interpol_matrix(g.K, g.nb, M, err);
  if (s != FD2D_OK) return set_error(ctx, s, err);
  FD2D_TRY(upload(ctx, "f64.interp", M, Mdev));
  if (!a.source_dist) {
    *dist = nullptr;
    return FD2D_OK;
  }
  const int64_t np = g.npts();
  FD2D_TRY(workspace_t(ctx, "f64.dist", (size_t)np * g.K, dist));
  const int ncol = g.nb == 0 ? 1 : g.nb;
  k64_distribution<<<(unsigned)((np + 255) / 256), 256, 0, ctx->stream>>>(*Mdev, g.K, ncol, a.source_dist, *dist, np);
  return after_launch(ctx, "k64_distribution");
}

}  // namespace

// ---------------------------------------------------------------------------------
fd2d_status fp64_forward1(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Base B;
  FD2D_TRY(init_base(ctx, g, a, false, B));
  const int nt = g.nt, K = g.K;
  const size_t np = (size_t)g.npts();
  // fft_coeff rows for n' = nt..2nt-1 with mod(n', freq_samp) == 0 (code/run_forward1_green.m:72-90)
  std::vector<double> cre, cim;
  for (int n = nt; n <= 2 * nt - 1; ++n)
    if (n % g.fs == 0)
      for (int k = 0; k < K; ++k) {
        double re, im;
        dft_coeff(-(g.w[k] * g.t_fwd[n - nt]), g.dt, re, im);
        cre.push_back(re);
        cim.push_back(im);
      }
  double *dcre, *dcim;
  FD2D_TRY(upload(ctx, "f64.cre", cre, &dcre));
  FD2D_TRY(upload(ctx, "f64.cim", cim, &dcim));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.G_re, 0, np * K * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.G_im, 0, np * K * 8, ctx->stream));
  const int nr = (int)a.rec_idx.size();
  const bool born = a.dmu != nullptr;
  int i_ftc = 0, i_fw_out = 0, i_fw_in = 0;
  for (int n = 1; n <= nt; ++n) {
    StepV sv{};
    sv.K = K;
    if (a.mode != 0 && (n + nt - 1) % g.fw == 0) sv.snap = a.G_out + np * (size_t)(i_fw_out++);
    if (born) {
      k64_born_pre<<<B.grid, B.block, 0, ctx->stream>>>(B.P, a.G_in + np * (size_t)(i_fw_in++));
      FD2D_TRY(after_launch(ctx, "k64_born_pre"));
    } else {
      sv.use_src = !a.src_idx.empty();
      sv.amp_const = 1.0e9;  // stf = 1.0e9*ones(1,nt), code/run_forward1_green.m:64
    }
    k64_v<<<B.grid, B.block, 0, ctx->stream>>>(B.P, sv);
    FD2D_TRY(after_launch(ctx, "k64_v"));
    StepS ss{};
    ss.K = K;
    if ((n + nt - 1) % g.fs == 0) {
      ss.dcre = dcre + (size_t)K * i_ftc;
      ss.dcim = dcim + (size_t)K * i_ftc;
      ss.Dre = a.G_re;
      ss.Dim = a.G_im;
      ++i_ftc;
    }
    size_t shm = (ss.dcre ? 4 * K : 0) * sizeof(double);
    k64_stress<<<B.grid, B.block, shm, ctx->stream>>>(B.P, ss);
    FD2D_TRY(after_launch(ctx, "k64_stress"));
    FD2D_TRY(record(ctx, B, B.P.v, nr, a.seis + (size_t)nr * (n - 1)));
  }
  k64_negate<<<(unsigned)((np * K + 255) / 256), 256, 0, ctx->stream>>>(a.G_im, (int64_t)(np * K));
  return after_launch(ctx, "k64_negate");
}

fd2d_status fp64_correlation(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Base B;
  FD2D_TRY(init_base(ctx, g, a, true, B));
  const int ntc = g.ntc, K = g.K;
  const size_t np = (size_t)g.npts();
  std::vector<double> cre, cim;  // ifft_coeff, code/run_forward2_correlation.m:73-85
  for (int n = 1; n <= ntc; ++n)
    if (n % g.fs == 0)
      for (int k = 0; k < K; ++k) {
        double re, im;
        dft_coeff(g.w[k] * g.t_corr[n - 1], g.dw, re, im);
        cre.push_back(re);
        cim.push_back(im);
      }
  double *dcre, *dcim;
  FD2D_TRY(upload(ctx, "f64.cre", cre, &dcre));
  FD2D_TRY(upload(ctx, "f64.cim", cim, &dcim));
  double *dist, *M;
  FD2D_TRY(make_dist(ctx, g, a, &dist, &M));
  const int nr = (int)a.rec_idx.size();
  const bool born = a.dmu != nullptr;
  int i_ftc = 0, i_fw_out = 0;
  for (int n = 1; n <= ntc; ++n) {
    StepV sv{};
    sv.K = K;
    sv.snap_u = 1;
    if (a.mode != 0 && n % g.fw == 0) sv.snap = a.C_out + np * (size_t)(i_fw_out++);
    if (n % g.fs == 0) {
      sv.cre = dcre + (size_t)K * i_ftc;
      sv.cim = dcim + (size_t)K * i_ftc;
      ++i_ftc;
      sv.Xre = a.Gin_re;
      sv.Xim = a.Gin_im;
      sv.xsign = 1.0;
      sv.spectrum = a.spectrum;
      sv.dist = dist;
      sv.n_src = a.n_src;
      sv.add_per_source = 1;
    }
    k64_v<<<B.grid, B.block, (sv.cre ? 2 * K : 0) * sizeof(double), ctx->stream>>>(B.P, sv);
    FD2D_TRY(after_launch(ctx, "k64_v"));
    StepS ss{};
    ss.K = K;
    ss.update_u = 1;
    if (born && n != ntc) {
      ss.born_a = a.C_in + np * (size_t)(n - 1);
      ss.born_b = a.C_in + np * (size_t)n;
    }
    k64_stress<<<B.grid, B.block, 0, ctx->stream>>>(B.P, ss);
    FD2D_TRY(after_launch(ctx, "k64_stress"));
    FD2D_TRY(record(ctx, B, B.P.u, nr, a.seis + (size_t)nr * (n - 1)));
  }
  return FD2D_OK;
}

fd2d_status fp64_adjoint(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Base B;
  FD2D_TRY(init_base(ctx, g, a, true, B));
  const int ntc = g.ntc, K = g.K, mode = a.mode;
  const size_t np = (size_t)g.npts();
  // fft_coeff (dt) and ifft_coeff (dw) rows, code/run_noise_adjoint.m:77-91
  std::vector<double> fre, fim, ire, iim;
  for (int n = 1; n <= ntc; ++n)
    if (n % g.fs == 0)
      for (int k = 0; k < K; ++k) {
        double re, im;
        dft_coeff(-(g.w[k] * g.t_corr[n - 1]), g.dt, re, im);
        fre.push_back(re);
        fim.push_back(im);
        dft_coeff(g.w[k] * g.t_corr[n - 1], g.dw, re, im);
        ire.push_back(re);
        iim.push_back(im);
      }
  const int n_ftc = ntc / g.fs;
  double *dfre, *dfim, *dire, *diim;
  FD2D_TRY(upload(ctx, "f64.fre", fre, &dfre));
  FD2D_TRY(upload(ctx, "f64.fim", fim, &dfim));
  FD2D_TRY(upload(ctx, "f64.ire", ire, &dire));
  FD2D_TRY(upload(ctx, "f64.iim", iim, &diim));
  double *dist, *M;
  FD2D_TRY(make_dist(ctx, g, a, &dist, &M));
  const int ncol = g.nb == 0 ? 1 : g.nb;
  const int64_t d0 = a.stf_dims[0], d1 = a.stf_dims[1], d2 = a.stf_dims[2];
  const bool stf_empty = !a.stf_re || d0 * d1 * d2 == 0;
  const int64_t size3 = stf_empty ? 1 : d2;
  const bool stf2d = !stf_empty && size3 == 1, stf3d = !stf_empty && size3 != 1;
  int nt_loop = ntc;
  if ((mode == 0 || mode == 1) && size3 != 1) nt_loop = g.nt;  // :165-167
  const bool Gvalid = a.Gin_re != nullptr && a.n_G == K;
  const bool born = a.dmu != nullptr && a.n_C_in == ntc;
  const bool save_u = mode == 11 || mode == 13;
  const bool dft_u = mode == 1 || mode == 12 || mode == 13;
  const bool have_fwd = a.u_fwd != nullptr && a.n_u_fwd > 0;
  // stf with a zero imaginary part: pass a zero plane
  const double* stf_im = a.stf_im;
  if (stf3d && !stf_im) {
    double* z;
    FD2D_TRY(workspace_t(ctx, "f64.zero_im", (size_t)np * K, &z));
    FD2D_CUDA(ctx, cudaMemsetAsync(z, 0, np * K * 8, ctx->stream));
    stf_im = z;
  }
  FD2D_CUDA(ctx, cudaMemsetAsync(a.Kout, 0, np * 8 * (ncol + 1), ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.sf_re, 0, np * 8 * K, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.sf_im, 0, np * 8 * K, ctx->stream));
  double* Kmu = a.Kout + np * ncol;
  const int nr = (int)a.rec_idx.size();
  int i_ftc = 0, i_fw_in = 0, i_fw_out = 0;
  for (int n = 1; n <= nt_loop; ++n) {
    StepV sv{};
    sv.K = K;
    sv.snap_u = 1;
    if (save_u && n % g.fw == 0) sv.snap = a.C_out + np * (size_t)(i_fw_out++);
    if (stf2d) {
      sv.use_src = !a.src_idx.empty();
      sv.amp = a.stf_re + (size_t)d0 * (n - 1);
    } else if (stf3d && n % g.fs == 0) {
      if (i_ftc >= n_ftc) return set_error(ctx, FD2D_ERR_INDEX, "ifft_coeff row past the end");
      sv.cre = dire + (size_t)K * i_ftc;
      sv.cim = diim + (size_t)K * i_ftc;
      ++i_ftc;
      sv.Xre = a.stf_re;
      sv.Xim = stf_im;
      sv.xsign = -1.0;  // conj(stf)
      sv.spectrum = a.spectrum;
      sv.dist = dist;
      sv.n_src = dist ? a.n_src : 0;
      sv.add_per_source = 0;
    }
    k64_v<<<B.grid, B.block, (sv.cre ? 2 * K : 0) * sizeof(double), ctx->stream>>>(B.P, sv);
    FD2D_TRY(after_launch(ctx, "k64_v"));
    StepS ss{};
    ss.K = K;
    ss.update_u = 1;
    if (born && n != ntc) {
      ss.born_a = a.C_in + np * (size_t)(n - 1);
      ss.born_b = a.C_in + np * (size_t)n;
    }
    if (Gvalid && n % g.fs == 0) {
      const int row = n / g.fs - 1;  // ifft_coeff2(n,:) equals ifft_coeff of step n
      ss.kcre = dire + (size_t)K * row;
      ss.kcim = diim + (size_t)K * row;
      ss.Gre = a.Gin_re;
      ss.Gim = a.Gin_im;
      ss.spec = a.spectrum;
      ss.M = M;
      ss.Ks = a.Kout;
      ss.ncol = ncol;
    }
    if (dft_u && n % g.fs == 0) {
      if (i_ftc >= n_ftc) return set_error(ctx, FD2D_ERR_INDEX, "fft_coeff row past the end");
      ss.dcre = dfre + (size_t)K * i_ftc;
      ss.dcim = dfim + (size_t)K * i_ftc;
      ss.Dre = a.sf_re;
      ss.Dim = a.sf_im;
      ss.dft_of_u = 1;
      ++i_ftc;
    }
    size_t shm = ((ss.dcre || ss.kcre) ? 4 * K : 0) * sizeof(double);
    k64_stress<<<B.grid, B.block, shm, ctx->stream>>>(B.P, ss);
    FD2D_TRY(after_launch(ctx, "k64_stress"));
    if (have_fwd && a.n_u_fwd >= i_fw_in + 1 && n % g.fw == 0) {
      const float* uf = a.u_fwd + np * (size_t)(a.n_u_fwd - 1 - i_fw_in);
      k64_kmu<<<B.grid, B.block, 0, ctx->stream>>>(B.P, uf, Kmu, (double)g.fw);
      FD2D_TRY(after_launch(ctx, "k64_kmu"));
      ++i_fw_in;
    }
    FD2D_TRY(record(ctx, B, B.P.u, nr, a.seis + (size_t)nr * (n - 1)));
  }
  if (nt_loop < ntc && nr > 0)
    FD2D_CUDA(ctx, cudaMemsetAsync(a.seis + (size_t)nr * nt_loop, 0, (size_t)nr * (ntc - nt_loop) * 8, ctx->stream));
  return FD2D_OK;
}

}  // namespace fd2d
