// tma_host.cu -- host-side encoding of TMA tensor maps (see tma.cuh).
#include <cudaTypedefs.h>

#include <mutex>

#include "tma.cuh"

namespace fd2d {

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::mutex g_encode_mu;

fd2d_status make_tmap_f32(fd2d_ctx* ctx, CUtensorMap* map, const float* base, int w, int h,
                          int64_t pitch_elems, int bw, int bh, int d, int64_t plane_elems) {
  {
    std::lock_guard<std::mutex> lk(g_encode_mu);
    if (!g_encode) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
      if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return set_error(ctx, FD2D_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
      }
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
  }
  if ((reinterpret_cast<uintptr_t>(base) & 15) || (pitch_elems * 4) % 16 || bw % 4 || bw > 256 || bh > 256)
    return set_error(ctx, FD2D_ERR_ARG, "tensor map needs 16-byte aligned base, pitch and box width");
  const cuuint32_t rank = (d > 1 || plane_elems > 0) ? 3 : 2;
  cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)d};
  cuuint64_t strides[2] = {(cuuint64_t)pitch_elems * 4, (cuuint64_t)plane_elems * 4};
  cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank, const_cast<float*>(base), dims, strides,
                        box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    return set_error(ctx, FD2D_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
  return FD2D_OK;
}

}  // namespace fd2d
