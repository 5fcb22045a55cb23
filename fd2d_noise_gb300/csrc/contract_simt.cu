// contract_simt.cu -- FP32 CUDA-core implementation of the dense contraction
// R[n][m] = sum_k A[k][m] B[k][n] (see contract.cuh).
#include "contract.cuh"

namespace fd2d {
namespace {

constexpr int BM = 128, BN = 64, BK = 16, NT = 256;

__global__ __launch_bounds__(NT) void k_contract_simt(ContractArgs a) {
  __shared__ float As[BK][BM];
  __shared__ float Bs[BK][BN + 4];
  const int tid = threadIdx.x;
  const int tm = tid & 31, tn = tid >> 5;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  float acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < a.Kd; k0 += BK) {
#pragma unroll
    for (int e = 0; e < (BK * BM) / NT; ++e) {
      const int idx = tid + e * NT;
      const int kk = idx / BM, mm = idx % BM;
      const int k = k0 + kk, m = m0 + mm;
      As[kk][mm] = (k < a.Kd && m < a.M) ? a.A[(int64_t)k * a.lda + m] : 0.f;
    }
#pragma unroll
    for (int e = 0; e < (BK * BN) / NT; ++e) {
      const int idx = tid + e * NT;
      const int kk = idx / BN, nn = idx % BN;
      const int k = k0 + kk, n = n0 + nn;
      Bs[kk][nn] = (k < a.Kd && n < a.N) ? a.B[(int64_t)k * a.ldb + n] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float av[4], bv[8];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][tm + 32 * i];
#pragma unroll
      for (int j = 0; j < 8; ++j) bv[j] = Bs[kk][tn * 8 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int n = n0 + tn * 8 + j;
    if (n >= a.N) continue;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int m = m0 + tm + 32 * i;
      if (m >= a.M) continue;
      if (a.out32) a.out32[(int64_t)n * a.ldo + m] = acc[i][j];
      if (a.acc0) {
        double* p = n < a.nsplit ? a.acc0 + (int64_t)n * a.ldacc + m
                                 : a.acc1 + (int64_t)(n - a.nsplit) * a.ldacc + m;
        *p += (double)acc[i][j];
      }
    }
  }
}

}  // namespace

fd2d_status contract(fd2d_ctx* ctx, cudaStream_t stream, const ContractArgs& a) {
  if (a.M <= 0 || a.N <= 0 || a.Kd <= 0) return FD2D_OK;
  dim3 grid((a.M + BM - 1) / BM, (a.N + BN - 1) / BN);
  const int t0 = timer_begin(ctx, stream);
  k_contract_simt<<<grid, NT, 0, stream>>>(a);
  timer_end(ctx, stream, t0, FD2D_TIMER_CONTRACT, (int64_t)a.M * a.N * a.Kd);
  return after_launch(ctx, "k_contract_simt");
}

}  // namespace fd2d
