// gaussblur.cu -- separable Gaussian smoothing of model and gradient maps, FP64.
//
// tools/addons/gaussblur2d.m:2-38: GY = (W1 * Y * W2') ./ (w1' * w2) with
// W(i,j) = exp(-(|x(i)-x(j)|/sigma)^2/2) for |x(i)-x(j)| < sqrt(14)*sigma and 0
// beyond, and w(j) = sum_i W(i,j) (the normalisation).  Used on every gradient
// by inversion/optlib_callback_fct/map_gradparameters_to_gradm.m:40-50 and on
// the model by map_m_to_parameters.m:37-49.
//
// The weights of each axis are formed once (n^2 exponentials); each pass then
// gives every output element to one thread, which sums its in-range terms with
// j ascending -- the reference's summation order.
//
// The 'ring' parameterisation (map_m_to_parameters.m:22-29,
// map_gradparameters_to_gradm.m:27-35) smooths the structure plane with
// imfilter(Y, h, 'circular') of MATLAB's Image Processing Toolbox instead:
// correlation with h, output the size of Y, Y extended periodically, the centre
// of h at floor((size(h)+1)/2).  k_imfilter_circular gives each output element
// to one thread, adding the terms v-major, u-minor.
#include "common.cuh"

namespace fd2d {
namespace {

// W[i*n + j] (0 outside the cut-off) and wsum[j] = sum over i ascending of W(i,j).
__global__ void k_gb_weights(const double* x, int n, double sigma, double* W) {
  const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const double dist = fabs(x[i] - x[j]);
  double w = 0.0;
  if (dist < sqrt(14.0) * sigma) {
    const double r = dist / sigma;
    w = exp(-__dmul_rn(r, r) / 2.0);
  }
  W[(int64_t)i * n + j] = w;
}

__global__ void k_gb_wsum(const double* W, int n, double* wsum) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    const double w = W[(int64_t)i * n + j];
    if (w > 0.0) s = s + w;
  }
  wsum[j] = s;
}

// Along the first axis: M(i, c) = sum_j W1(i,j) Y(j, c)   (Y column-major, n1 x n2)
__global__ void k_gb_pass1(const double* W1, const double* Y, int n1, int n2, double* M) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (i >= n1 || c >= n2) return;
  const double* w = W1 + (int64_t)i * n1;
  const double* y = Y + (int64_t)n1 * c;
  double acc = 0.0;
  for (int j = 0; j < n1; ++j)
    if (w[j] > 0.0) acc = __dadd_rn(acc, __dmul_rn(w[j], y[j]));  // no FMA: the reference's rounding
  M[i + (int64_t)n1 * c] = acc;
}

// Along the second axis and normalised: GY(r, i) = (sum_j W2(i,j) M(r, j)) / (w1(r) w2(i))
__global__ void k_gb_pass2(const double* W2, const double* M, const double* w1, const double* w2, int n1, int n2,
                           double* GY) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
  if (r >= n1 || i >= n2) return;
  const double* w = W2 + (int64_t)i * n2;
  double acc = 0.0;
  for (int j = 0; j < n2; ++j)
    if (w[j] > 0.0) acc = __dadd_rn(acc, __dmul_rn(w[j], M[r + (int64_t)n1 * j]));
  GY[r + (int64_t)n1 * i] = acc / __dmul_rn(w1[r], w2[i]);
}

__device__ __forceinline__ int wrap_index(int k, int n) {
  k %= n;
  return k < 0 ? k + n : k;
}

// B(i, j) = sum_{v, u} h(u, v) Y((i + u - c1) mod n1, (j + v - c2) mod n2), all column-major.
__global__ void k_imfilter_circular(const double* Y, int n1, int n2, const double* h, int m1, int m2,
                                    double* B) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= n1 || j >= n2) return;
  const int c1 = (m1 + 1) / 2 - 1, c2 = (m2 + 1) / 2 - 1;
  double acc = 0.0;
  for (int v = 0; v < m2; ++v) {
    const double* col = Y + (int64_t)n1 * wrap_index(j + v - c2, n2);
    for (int u = 0; u < m1; ++u)
      acc = __dadd_rn(acc, __dmul_rn(h[u + (int64_t)m1 * v], col[wrap_index(i + u - c1, n1)]));
  }
  B[i + (int64_t)n1 * j] = acc;
}

}  // namespace
}  // namespace fd2d

using namespace fd2d;

extern "C" fd2d_status fd2d_gaussblur2d(fd2d_ctx* ctx, const double* Y, int32_t n1, int32_t n2, const double* x1,
                                        const double* x2, double sigma1, double sigma2, double* GY) {
  FD2D_TRY(check_ctx(ctx));
  if (n1 < 1 || n2 < 1 || !Y || !x1 || !x2 || !GY || !(sigma1 > 0) || !(sigma2 > 0))
    return set_error(ctx, FD2D_ERR_ARG, "gaussblur2d needs n1, n2 >= 1, arrays and positive sigmas");
  const size_t nm = (size_t)n1 * n2;
  const void *y, *a1, *a2;
  FD2D_TRY(stage_in(ctx, "gb.Y", Y, nm * 8, &y));
  FD2D_TRY(stage_in(ctx, "gb.x1", x1, (size_t)n1 * 8, &a1));
  FD2D_TRY(stage_in(ctx, "gb.x2", x2, (size_t)n2 * 8, &a2));
  double *W1, *W2, *w1, *w2, *M;
  FD2D_TRY(workspace_t(ctx, "gb.W1", (size_t)n1 * n1, &W1));
  FD2D_TRY(workspace_t(ctx, "gb.W2", (size_t)n2 * n2, &W2));
  FD2D_TRY(workspace_t(ctx, "gb.w1", (size_t)n1, &w1));
  FD2D_TRY(workspace_t(ctx, "gb.w2", (size_t)n2, &w2));
  FD2D_TRY(workspace_t(ctx, "gb.M", nm, &M));
  void* out;
  FD2D_TRY(out_buffer(ctx, "gb.GY", GY, nm * 8, &out));
  cudaStream_t s = ctx->stream;
  const int B = 128;
  k_gb_weights<<<dim3((n1 + B - 1) / B, n1), B, 0, s>>>((const double*)a1, n1, sigma1, W1);
  FD2D_TRY(after_launch(ctx, "k_gb_weights"));
  k_gb_weights<<<dim3((n2 + B - 1) / B, n2), B, 0, s>>>((const double*)a2, n2, sigma2, W2);
  FD2D_TRY(after_launch(ctx, "k_gb_weights"));
  k_gb_wsum<<<(n1 + B - 1) / B, B, 0, s>>>(W1, n1, w1);
  FD2D_TRY(after_launch(ctx, "k_gb_wsum"));
  k_gb_wsum<<<(n2 + B - 1) / B, B, 0, s>>>(W2, n2, w2);
  FD2D_TRY(after_launch(ctx, "k_gb_wsum"));
  k_gb_pass1<<<dim3((n1 + B - 1) / B, n2), B, 0, s>>>(W1, (const double*)y, n1, n2, M);
  FD2D_TRY(after_launch(ctx, "k_gb_pass1"));
  k_gb_pass2<<<dim3((n1 + B - 1) / B, n2), B, 0, s>>>(W2, M, w1, w2, n1, n2, (double*)out);
  FD2D_TRY(after_launch(ctx, "k_gb_pass2"));
  FD2D_TRY(stage_out(ctx, GY, out, nm * 8));
  return finish_call(ctx);
}

extern "C" fd2d_status fd2d_imfilter_circular(fd2d_ctx* ctx, const double* Y, int32_t n1, int32_t n2,
                                              const double* h, int32_t m1, int32_t m2, double* B) {
  FD2D_TRY(check_ctx(ctx));
  if (n1 < 1 || n2 < 1 || m1 < 1 || m2 < 1 || !Y || !h || !B)
    return set_error(ctx, FD2D_ERR_ARG, "imfilter_circular needs n1, n2, m1, m2 >= 1 and arrays");
  const size_t nm = (size_t)n1 * n2, hm = (size_t)m1 * m2;
  const void *y, *hh;
  FD2D_TRY(stage_in(ctx, "imf.Y", Y, nm * 8, &y));
  FD2D_TRY(stage_in(ctx, "imf.h", h, hm * 8, &hh));
  void* out;
  FD2D_TRY(out_buffer(ctx, "imf.B", B, nm * 8, &out));
  const int T = 128;
  k_imfilter_circular<<<dim3((n1 + T - 1) / T, n2), T, 0, ctx->stream>>>((const double*)y, n1, n2,
                                                                          (const double*)hh, m1, m2, (double*)out);
  FD2D_TRY(after_launch(ctx, "k_imfilter_circular"));
  FD2D_TRY(stage_out(ctx, B, out, nm * 8));
  return finish_call(ctx);
}
