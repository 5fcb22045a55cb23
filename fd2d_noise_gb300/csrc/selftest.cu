// selftest.cu -- a check that device-side waits end.
//
// Every kernel of the library that waits on an mbarrier (the stencil's tile
// loads, the contraction's pipeline) bounds the wait by %globaltimer, sets the
// context's error flag when it gives up, lets its own copies land and
// returns; the host turns the flag into FD2D_ERR_TIMEOUT and the context stays
// usable.  fd2d_check_bounded_wait runs that path on purpose, on a barrier
// nothing ever completes (no copy, no other thread), with a short limit.
#include "common.cuh"
#include "tma.cuh"

namespace fd2d {
namespace {

__global__ void k_wait_probe(uint64_t limit_ns, int* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  // no thread arrives and no copy is issued: the wait can only give up
  if (!mbar_wait_bounded(&bar, 0, limit_ns)) set_error_flag(err, 3);
}

}  // namespace
}  // namespace fd2d

using namespace fd2d;

extern "C" fd2d_status fd2d_check_bounded_wait(fd2d_ctx* ctx, int64_t limit_us) {
  FD2D_TRY(check_ctx(ctx));
  if (limit_us < 1 || limit_us > 2000000)
    return set_error(ctx, FD2D_ERR_ARG, "limit_us must be in [1, 2000000]");
  k_wait_probe<<<1, 32, 0, ctx->stream>>>((uint64_t)limit_us * 1000ull, ctx->d_err);
  FD2D_TRY(after_launch(ctx, "k_wait_probe"));
  return fd2d_ctx_synchronize(ctx);
}
