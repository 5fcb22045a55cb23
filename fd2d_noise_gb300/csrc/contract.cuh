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

struct ContractArgs {
  const float* A = nullptr;  // Kd planes, plane stride lda (>= M)
  int64_t lda = 0;
  const float* B = nullptr;  // Kd rows of N values, row stride ldb
  int64_t ldb = 0;
  int M = 0, N = 0, Kd = 0;
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
};

fd2d_status contract(fd2d_ctx* ctx, cudaStream_t stream, const ContractArgs& a);
// One-time kernel attributes; call before any stream capture that contracts.
fd2d_status contract_prepare(fd2d_ctx* ctx);

}  // namespace fd2d
