// solver_fp32.cu -- placeholder until the FP32 path lands.
#include "common.cuh"
namespace fd2d {
fd2d_status fp32_forward1(fd2d_ctx* ctx, const Geometry&, const SolveArgs&) { return set_error(ctx, FD2D_ERR_UNSUPPORTED, "fp32 not built"); }
fd2d_status fp32_correlation(fd2d_ctx* ctx, const Geometry&, const SolveArgs&) { return set_error(ctx, FD2D_ERR_UNSUPPORTED, "fp32 not built"); }
fd2d_status fp32_adjoint(fd2d_ctx* ctx, const Geometry&, const SolveArgs&) { return set_error(ctx, FD2D_ERR_UNSUPPORTED, "fp32 not built"); }
}
