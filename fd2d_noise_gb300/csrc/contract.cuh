// contract.cuh -- the dense contractions of the FP32 path.
//
// Both the on-the-fly DFT of the wavefield (code/run_forward1_green.m:176-183,
// code/run_noise_adjoint.m:335-346) and the correlation-source injection
// (code/run_forward2_correlation.m:195-216, code/run_noise_adjoint.m:255-268)
// are the same product over grid points m:
//
//     R[n][m] = sum_k A[k][m] * B[k][n]
//
//   DFT:       A = wavefield snapshots (k = time), B = [Re c | Im c] (n = 2K)
//   injection: A = [Re P ; Im P] planes (k = 2K), B = time coefficients (n = steps)
//
// A is plane-major (points contiguous), as the stencil writes it; B is small.
// The result either accumulates into FP64 planes (spectra) or is stored as
// FP32 planes (injection sources).
#pragma once

#include "common.cuh"

namespace fd2d {

// Column tile and K block of the tensor-core contraction.
constexpr int CONTRACT_BN = 128, CONTRACT_BK = 32;

struct ContractArgs {
  int M = 0, N = 0, Kd = 0;
  // A: Kd planes of M points, FP32, plane k at a32 + k*lda (lda a multiple of
  // 4, a32 16-byte aligned); split into TF32 halves inside the contraction
  const float* a32 = nullptr;
  int64_t lda = 0;
  // B as its split image (contract_image): column n of this call is column
  // img_nt0*CONTRACT_BN + n of the imaged table, K row k is its row
  // img_kb0*CONTRACT_BK + k; img_nkb = K blocks of the imaged table.
  const float* bimg = nullptr;
  int img_nt0 = 0, img_kb0 = 0, img_nkb = 0;
  // FP64 accumulation: column n < nsplit -> acc0[n*ldacc + m], else acc1[(n-nsplit)*ldacc + m]
  double* acc0 = nullptr;
  double* acc1 = nullptr;
  int nsplit = 0;
  int64_t ldacc = 0;
  int overwrite = 0;  // FP64 planes: 1 = store the result, 0 = add it to them
  // When remap_pitch > 0 the points m are a pitched grid (m = i + remap_pitch*j)
  // and the FP64 planes are MATLAB-layout nx-by-nz: m -> i + remap_nx*j, and
  // points outside the grid are dropped.
  int remap_pitch = 0, remap_nx = 0, remap_nz = 0;
  // Lanes: when lane_m > 0 the points are lane_m-long runs of independent
  // solves, m = l*lane_m + (pitched point), and lane l's FP64 planes start
  // l*acc_lane elements after acc0 / acc1.
  int64_t lane_m = 0, acc_lane = 0;
  // FP32 store: out32[n*ldo + m]
  float* out32 = nullptr;
  int64_t ldo = 0;
  // 2: the K blocks are summed in two halves, each in its own FP32 tensor-memory
  // accumulator, and the halves added once in the epilogue (a long DFT loses
  // less to FP32 rounding of small late terms against a large running sum);
  // 1: one accumulator.
  int k_partials = 1;
};

fd2d_status contract(fd2d_ctx* ctx, cudaStream_t stream, const ContractArgs& a);
// Split image of a K-by-X matrix (Kd rows of X values, row stride ld): floats
// needed, and the kernel that writes it (queued on `stream`).
size_t contract_image_floats(int X, int Kd);
fd2d_status contract_image(fd2d_ctx* ctx, cudaStream_t stream, const float* src, int64_t ld, int X, int Kd,
                           float* img);
// One-time kernel attributes; call before any stream capture that contracts.
fd2d_status contract_prepare(fd2d_ctx* ctx);

}  // namespace fd2d
