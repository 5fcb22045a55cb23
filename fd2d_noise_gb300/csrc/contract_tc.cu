// contract_tc.cu -- tensor-core (tcgen05) implementation of the dense
// contraction R[n][m] = sum_k A[k][m] B[k][n] (contract.cuh) in split TF32.
//
// Split precision: every FP32 operand x is written as hi + lo with hi = x with
// its 13 low mantissa bits cleared (exactly representable in TF32) and
// lo = x - hi; the product keeps hi*hi + hi*lo + lo*hi ("3xTF32"), dropping
// lo*lo (~2^-22 relative), and accumulates in FP32 in tensor memory.  Spectra
// are then accumulated across snapshot chunks in FP64.
//
// CTA tile: 128 points (M) x 256 columns (N), K blocks of 32.
//   warps 0-7 : producers -- read A (points contiguous) and B (columns
//               contiguous) from global memory, split them, and store them
//               transposed into K-major, 128-byte-swizzled shared memory;
//   warp 8    : allocates TMEM, one lane issues tcgen05.mma (M=128, N=256,
//               K=8 per instruction, 12 per K block) and commits to mbarriers;
//   warps 0-3 : epilogue -- tcgen05.ld of their 32 TMEM lanes, FP64
//               accumulation (optionally remapped from the pitched grid to
//               MATLAB layout) or FP32 store.
// Every mbarrier wait is bounded in time; a wait that gives up sets the
// context's error flag and the CTA drains and frees its TMEM.
#include "contract.cuh"
#include "tma.cuh"

namespace fd2d {
namespace {

constexpr int BM = 128, BN = 256, BK = 32, STAGES = 2;
constexpr int NPROD = 256;                  // producer threads (warps 0-7)
constexpr int NTHREADS = NPROD + 32;        // + MMA warp
constexpr int A_BYTES = BM * BK * 4;        // 16 KB per split half
constexpr int B_BYTES = BN * BK * 4;        // 32 KB per split half
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;  // + 1024-byte alignment slack
constexpr uint32_t TMEM_COLS = 256;

// Instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
// The N field (bits 17-22) is set per launch: the N tile is the smallest
// multiple of 16 that covers N in ceil(N/256) tiles.
constexpr uint32_t IDESC_BASE = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BM >> 4) << 24);

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Byte offset of element (row r, k) in a K-major SW128 tile of 32 TF32 per row.
__device__ __forceinline__ uint32_t sw128(int r, int chunk) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((chunk ^ (r & 7)) << 4));
}

__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  lo = x - hi;
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, float a, float b, float c, float d) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d)
               : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
      "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__global__ __launch_bounds__(NTHREADS, 1) void k_contract_tc(ContractArgs a, int bn, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * bn;
  const uint32_t idesc = IDESC_BASE | ((uint32_t)(bn >> 3) << 17);
  const int nkb = (a.Kd + BK - 1) / BK;
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const uint32_t sbase = smem_u32(smem);
  auto a_hi = [&](int s) { return sbase + s * STAGE_BYTES; };
  auto a_lo = [&](int s) { return sbase + s * STAGE_BYTES + A_BYTES; };
  auto b_hi = [&](int s) { return sbase + s * STAGE_BYTES + 2 * A_BYTES; };
  auto b_lo = [&](int s) { return sbase + s * STAGE_BYTES + 2 * A_BYTES + B_BYTES; };

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], NPROD / 32);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
    fail = 0;
    fence_mbar_init();
  }
  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp < 8) {
    // ---------------- producers ----------------
    const int r = tid;  // B row (column n0 + r); A row m0 + r for r < 128
    const int n = n0 + r;
    const int m = m0 + r;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % STAGES;
      const uint32_t ph = (kb / STAGES) & 1;
      if (!mbar_wait_bounded(&empty_bar[s], ph ^ 1)) {
        atomicExch(&fail, 1);
        break;
      }
      const int k0 = kb * BK;
      // all global loads of the K block first (column n of B, row m of A) ...
      float xb[BK], xa[BK];
#pragma unroll
      for (int k = 0; k < BK; ++k)
        xb[k] = (r < bn && n < a.N && k0 + k < a.Kd) ? __ldg(a.B + (int64_t)(k0 + k) * a.ldb + n) : 0.f;
      if (r < BM) {
#pragma unroll
        for (int k = 0; k < BK; ++k)
          xa[k] = (m < a.M && k0 + k < a.Kd) ? a.A[(int64_t)(k0 + k) * a.lda + m] : 0.f;
      }
      // ... then split and store the transposed, swizzled rows
#pragma unroll
      for (int c = 0; c < BK / 4; ++c) {
        float h[4], l[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) split_tf32(xb[c * 4 + q], h[q], l[q]);
        st_shared_v4(b_hi(s) + sw128(r, c), h[0], h[1], h[2], h[3]);
        st_shared_v4(b_lo(s) + sw128(r, c), l[0], l[1], l[2], l[3]);
      }
      if (r < BM) {
#pragma unroll
        for (int c = 0; c < BK / 4; ++c) {
          float h[4], l[4];
#pragma unroll
          for (int q = 0; q < 4; ++q) split_tf32(xa[c * 4 + q], h[q], l[q]);
          st_shared_v4(a_hi(s) + sw128(r, c), h[0], h[1], h[2], h[3]);
          st_shared_v4(a_lo(s) + sw128(r, c), l[0], l[1], l[2], l[3]);
        }
      }
      // generic-proxy smem writes -> visible to the tensor core (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&full_bar[s]);
    }
  } else {
    // ---------------- MMA issuer (warp 8) ----------------
    if (lane == 0) {
      bool ok = true;
      for (int kb = 0; kb < nkb && ok; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!mbar_wait_bounded(&full_bar[s], ph)) {
          atomicExch(&fail, 1);
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int kk = 0; kk < BK / 8; ++kk) {
          const uint64_t ah = smem_desc(a_hi(s) + kk * 32), al = smem_desc(a_lo(s) + kk * 32);
          const uint64_t bh = smem_desc(b_hi(s) + kk * 32), bl = smem_desc(b_lo(s) + kk * 32);
          mma_tf32(tmem, ah, bh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
          mma_tf32(tmem, ah, bl, idesc, 1u);
          mma_tf32(tmem, al, bh, idesc, 1u);
        }
        mma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
      }
      mma_commit(&done_bar);  // all issued MMAs complete -> accumulator ready
    }
    __syncwarp();
  }

  // ---------------- epilogue (warps 0-3: TMEM lanes 32*warp .. +31) ----------------
  if (warp < 4) {
    const bool ok = mbar_wait_bounded(&done_bar, 0);
    if (!ok) atomicExch(&fail, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = warp * 32 + lane;
    const int m = m0 + row;
    int64_t q = m;
    bool valid = ok && m < a.M;
    if (valid && a.remap_pitch) {
      int64_t mm = m, lane_off = 0;
      if (a.lane_m) {
        const int64_t l = mm / a.lane_m;
        mm -= l * a.lane_m;
        lane_off = l * a.acc_lane;
      }
      const int ii = (int)(mm % a.remap_pitch), jj = (int)(mm / a.remap_pitch);
      valid = ii < a.remap_nx && jj < a.remap_nz;
      q = lane_off + ii + (int64_t)a.remap_nx * jj;
    }
    for (int c0 = 0; c0 < bn; c0 += 32) {
      float v[32];
      // all lanes of the warp take part in tcgen05.ld (sync.aligned)
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (!valid) continue;
      if (a.out32) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int n = n0 + c0 + j;
          if (n < a.N && c0 + j < bn) a.out32[(int64_t)n * a.ldo + m] = v[j];
        }
      }
      if (a.acc0) {
        // Column n of the tile goes to plane n (acc0) or n - nsplit (acc1).
        // Overwrite: plain stores.  Accumulate: 8 loads in flight per group.
#pragma unroll
        for (int g = 0; g < 32; g += 8) {
          double* p[8];
          double old[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int n = n0 + c0 + g + j;
            const bool in = n < a.N && c0 + g + j < bn;
            p[j] = !in ? nullptr
                       : (n < a.nsplit ? a.acc0 + (int64_t)n * a.ldacc + q
                                       : a.acc1 + (int64_t)(n - a.nsplit) * a.ldacc + q);
            old[j] = (p[j] && !a.overwrite) ? *p[j] : 0.0;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j)
            if (p[j]) *p[j] = old[j] + (double)v[g + j];
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 8) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
  if (tid == 0 && fail) set_error_flag(err, 2);
}

}  // namespace

fd2d_status contract_prepare(fd2d_ctx* ctx) {
  static bool attr = false;
  if (!attr) {
    FD2D_CUDA(ctx, cudaFuncSetAttribute(k_contract_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    attr = true;
  }
  return FD2D_OK;
}

fd2d_status contract(fd2d_ctx* ctx, cudaStream_t stream, const ContractArgs& a) {
  if (a.M <= 0 || a.N <= 0 || a.Kd <= 0) return FD2D_OK;
  const int ntiles = (a.N + BN - 1) / BN;
  const int bn = ((a.N + ntiles - 1) / ntiles + 15) / 16 * 16;
  dim3 grid((a.M + BM - 1) / BM, ntiles);
  const int t0 = timer_begin(ctx, stream);
  k_contract_tc<<<grid, NTHREADS, SMEM_BYTES, stream>>>(a, bn, ctx->d_err);
  timer_end(ctx, stream, t0, FD2D_TIMER_CONTRACT, (int64_t)a.M * a.N * a.Kd);
  return after_launch(ctx, "k_contract_tc");
}

}  // namespace fd2d

extern "C" fd2d_status fd2d_contract_f32(fd2d_ctx* ctx, const float* A, int64_t lda, const float* B,
                                         int64_t ldb, int32_t M, int32_t N, int32_t Kd, float* R,
                                         int64_t ldr) {
  using namespace fd2d;
  if (!ctx) return set_error(nullptr, FD2D_ERR_ARG, "ctx is NULL");
  if (!A || !B || !R || M < 0 || N < 0 || Kd < 0 || lda < M || ldb < N || ldr < M)
    return set_error(ctx, FD2D_ERR_ARG, "bad contraction arguments");
  cudaSetDevice(ctx->device);
  FD2D_TRY(contract_prepare(ctx));
  ContractArgs c;
  c.A = A; c.lda = lda; c.B = B; c.ldb = ldb; c.M = M; c.N = N; c.Kd = Kd; c.out32 = R; c.ldo = ldr;
  return contract(ctx, ctx->stream, c);
}
