// contract_tc.cu -- tensor-core (tcgen05) implementation of the dense
// contraction R[n][m] = sum_k A[k][m] B[k][n] (contract.cuh) in split TF32.
//
// Split precision: every FP32 operand x is written as hi + lo with hi = x with
// its 13 low mantissa bits cleared (exactly representable in TF32) and
// lo = x - hi; the product keeps hi*hi + hi*lo + lo*hi ("3xTF32"), dropping
// lo*lo (~2^-22 relative), and accumulates in FP32 in tensor memory.  Spectra
// are then accumulated across snapshot chunks in FP64.
//
// B (the DFT / inverse-DFT basis, one table shared by every CTA) is split
// once into an "image" (k_image): for each 128-row tile and 32-deep K block,
// its hi and lo halves already in the K-major, 128-byte-swizzled layout the
// tensor core reads.  A (the wavefield snapshot chunk or the injection P
// planes, points contiguous, as the stencil writes them) is read as FP32 by
// TMA, one 128-point by 32-deep block at a time, and split into the same
// layout by converter warps in shared memory (the raw block lands in the lo
// slot of its stage and is split in place), so it crosses HBM once, at 4
// bytes per element.
//
// k_contract_tc is persistent (one CTA per SM) over 128 x 128 output tiles,
// with a 3-stage ring of 64 KB stages (A and B blocks, hi and lo) and two
// TMEM accumulators, so the epilogue of one tile overlaps the main loop of
// the next.
// Each accumulator has two halves (all 512 TMEM columns): with k_partials = 2
// the first half of the K blocks sums into one and the rest into the other,
// and the epilogue adds the two FP32 partial sums.
// Every mbarrier wait is bounded in time; a wait that gives up sets the
// context's error flag, the CTA lets its own copies land (bounded) and frees
// its TMEM.
#include "contract.cuh"
#include "fp_bits.cuh"
#include "tma.cuh"

#include <algorithm>

namespace fd2d {
namespace {

constexpr int BM = 128, BN = CONTRACT_BN, BK = CONTRACT_BK, STAGES = 3;
constexpr int A_BYTES = BM * BK * 4;        // 16 KB per split half
constexpr int B_BYTES = BN * BK * 4;        // 16 KB per split half
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
// A arrives as FP32 (points contiguous, one 32-deep K block of 128 points per
// copy) in the stage's lo slot, and the converter warps split it into the
// stage's hi / lo blocks in place
constexpr int RAW_BYTES = BM * BK * 4;
static_assert(RAW_BYTES == A_BYTES, "the raw A block fills the lo slot of its stage");
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;  // + 1024-byte alignment slack
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory of the contraction");
constexpr uint32_t TMEM_COLS = BN;          // one partial accumulator
constexpr uint32_t TMEM_ALLOC = 4 * TMEM_COLS;  // 2 accumulators x 2 partials = 512 columns

// Instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Byte offset of the 16-byte chunk `chunk` (4 TF32) of row r in a K-major SW128
// tile of 32 TF32 per row.
__host__ __device__ __forceinline__ uint32_t sw128(int r, int chunk) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((chunk ^ (r & 7)) << 4));
}

__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  lo = x - hi;
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
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

// Image of a K-by-X matrix src (row k at src + k*ld, X values contiguous): for
// each 128-row tile of X and 32-deep K block, the hi and lo halves in the
// K-major SW128 layout of sw128() (rows x, 32 TF32 per row), block (xt, kb) at
// ((xt * nkb) + kb) * 2 * TILE_BYTES.  Entries outside the matrix are zero.
// One CTA per block: a coalesced load of the 32 x 128 tile into shared memory
// (row stride 129: conflict-free column reads), then coalesced 16-byte stores.
constexpr int TILE_BYTES = 128 * BK * 4;  // 16 KB: one split half of one block
static_assert(TILE_BYTES == A_BYTES && TILE_BYTES == B_BYTES, "A and B tiles share the image format");

__global__ __launch_bounds__(256) void k_image(const float* __restrict__ src, int64_t ld, int X, int Kd, int nkb,
                                               float* __restrict__ img) {
  __shared__ float tile[BK][129];
  const int xt = blockIdx.x, kb = blockIdx.y, tid = threadIdx.x;
  for (int e = tid; e < BK * 128; e += 256) {
    const int k = e >> 7, x = e & 127;
    const int gk = kb * BK + k, gx = xt * 128 + x;
    tile[k][x] = (gk < Kd && gx < X) ? src[(int64_t)gk * ld + gx] : 0.f;
  }
  __syncthreads();
  unsigned char* blk = reinterpret_cast<unsigned char*>(img) + ((size_t)xt * nkb + kb) * 2 * TILE_BYTES;
  for (int q = tid; q < 2 * 128 * (BK / 4); q += 256) {
    const int half = q >> 10, r = (q >> 3) & 127, c = q & 7;
    float v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float hi, lo;
      split_tf32(tile[c * 4 + j][r], hi, lo);
      v[j] = half ? lo : hi;
    }
    *reinterpret_cast<float4*>(blk + half * TILE_BYTES + sw128(r, c)) = make_float4(v[0], v[1], v[2], v[3]);
  }
}

// Persistent contraction over output tiles (m_tile, n_tile), column tile
// fastest, tile = blockIdx.x, blockIdx.x + gridDim.x, ...
//   warp 0    : one lane issues the copies of each stage (STAGES-deep ring):
//               B's image block by bulk copy, A's FP32 block by TMA into the
//               stage's A lo slot;
//   warp 1    : allocates TMEM (two 128-column accumulators); one lane issues
//               the MMAs (12 per K block) and commits stages and accumulators;
//   warps 2-5 : split each raw A block into its hi / lo halves, written in
//               the K-major 128-byte-swizzled layout the MMAs read (every
//               converter reads its row first, then all write);
//   warps 6-13: epilogue, TMEM lanes 32*(warp%4) .. +31 of the accumulator the
//               MMAs are not writing, columns 64*((warp-6)/4) .. +63 -- it
//               overlaps the next tile's main loop.  Two warps per TMEM lane
//               quarter keep enough stores in flight for the FP64 spectra.
constexpr int EPI_WARPS = 8;
constexpr int CONV_WARPS = 4;
constexpr int EPI_WARP0 = 2 + CONV_WARPS;
constexpr int NTHREADS_P = 32 * EPI_WARP0 + 32 * EPI_WARPS;
static_assert(32 * CONV_WARPS == BM, "one converter thread per row of A's block");
static_assert(EPI_WARPS % 4 == 0 && BN % (32 * (EPI_WARPS / 4)) == 0, "epilogue warps split the columns in 32s");

__global__ __launch_bounds__(NTHREADS_P, 1) void k_contract_tc(ContractArgs a, int ntn, int n_tiles, int* err,
                                                              const __grid_constant__ CUtensorMap amap) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[STAGES];   // B's blocks and the raw A block landed (tx)
  __shared__ __align__(8) uint64_t afull_bar[STAGES];  // A's split blocks of the stage written (converters)
  __shared__ __align__(8) uint64_t empty_bar[STAGES];  // MMAs done reading the stage
  __shared__ __align__(8) uint64_t accf_bar[2];        // accumulator complete
  __shared__ __align__(8) uint64_t acce_bar[2];        // accumulator read out (every epilogue warp)
  __shared__ uint32_t tmem_base;
  __shared__ int fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nkb = (a.Kd + BK - 1) / BK;
  // K blocks [0, kb_half) go to partial 0, [kb_half, nkb) to partial 1
  const bool two = a.k_partials == 2 && nkb > 1;
  const int kb_half = two ? (nkb + 1) / 2 : nkb;
  unsigned char* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t sbase = smem_u32(smem);
  auto a_hi = [&](int s) { return sbase + s * STAGE_BYTES; };
  auto a_lo = [&](int s) { return sbase + s * STAGE_BYTES + A_BYTES; };
  auto b_hi = [&](int s) { return sbase + s * STAGE_BYTES + 2 * A_BYTES; };
  auto b_lo = [&](int s) { return sbase + s * STAGE_BYTES + 2 * A_BYTES + B_BYTES; };

  if (tid == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&afull_bar[s], CONV_WARPS);
      mbar_init(&empty_bar[s], 1);
    }

    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf_bar[b], 1);
      mbar_init(&acce_bar[b], EPI_WARPS);
    }
    fail = 0;
    fence_mbar_init();
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TMEM_ALLOC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 0) {
    // ---------------- bulk copies ----------------
    if (lane == 0) {
      const unsigned char* bi = reinterpret_cast<const unsigned char*>(a.bimg);
      int g = 0;  // stage uses so far
      bool bad = false;
      for (int t = blockIdx.x; t < n_tiles && !bad; t += gridDim.x) {
        const int mt = t / ntn, nt = a.img_nt0 + (t - mt * ntn);
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int s = g % STAGES;
          if (!mbar_wait_bounded_sleep(&empty_bar[s], ((g / STAGES) & 1) ^ 1) || fail) {
            atomicExch(&fail, 1);
            bad = true;
            break;
          }
          mbar_expect_tx(&full_bar[s], 2 * B_BYTES + RAW_BYTES);
          bulk_copy(b_hi(s), bi + ((size_t)nt * a.img_nkb + a.img_kb0 + kb) * 2 * B_BYTES, 2 * B_BYTES,
                    &full_bar[s]);
          // into the lo slot; rows past Kd and points past M arrive as zeros
          tma_load_2d(smem + s * STAGE_BYTES + A_BYTES, &amap, mt * BM, kb * BK, &full_bar[s]);
        }
      }
      if (bad) {
        // let this CTA's copies land before it exits (bounded)
        for (int h = (g > STAGES ? g - STAGES : 0); h < g; ++h)
          mbar_wait_bounded_sleep(&full_bar[h % STAGES], (h / STAGES) & 1, 100000000ull);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      int g = 0, i = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < n_tiles && ok; t += gridDim.x, ++i) {
        const int acc = i & 1;
        const uint32_t d0 = tmem + (uint32_t)(2 * acc * TMEM_COLS);
        if (!mbar_wait_bounded(&acce_bar[acc], ((i >> 1) & 1) ^ 1)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int s = g % STAGES;
          if (!mbar_wait_bounded(&full_bar[s], (g / STAGES) & 1) || !mbar_wait_bounded(&afull_bar[s], (g / STAGES) & 1)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const bool second = kb >= kb_half;
          const uint32_t d = second ? d0 + TMEM_COLS : d0;
          const int kb_first = second ? kb_half : 0;  // first K block of this partial
#pragma unroll
          for (int kk = 0; kk < BK / 8; ++kk) {
            const uint64_t ah = smem_desc(a_hi(s) + kk * 32), al = smem_desc(a_lo(s) + kk * 32);
            const uint64_t bh = smem_desc(b_hi(s) + kk * 32), bl = smem_desc(b_lo(s) + kk * 32);
            mma_tf32(d, ah, bh, (kb > kb_first || kk > 0) ? 1u : 0u);
            mma_tf32(d, ah, bl, 1u);
            mma_tf32(d, al, bh, 1u);
          }
          mma_commit(&empty_bar[s]);  // frees the stage once these MMAs have read it
        }
        if (ok) mma_commit(&accf_bar[acc]);  // accumulator ready for the epilogue
      }
      if (!ok) atomicExch(&fail, 1);
    }
    __syncwarp();
  } else if (warp < EPI_WARP0) {
    // ---------------- converters: warps 2-5 ----------------
    // Thread c splits row c of the block: its 32 K values are read down the
    // raw block's columns (consecutive lanes: consecutive banks) into
    // registers; once every converter has read (named barrier 1), the 8 hi
    // and 8 lo 16-byte chunks of the swizzled row overwrite the stage's A slots.
    const int c = tid - 64;
    int g = 0;
    bool done = false;
    for (int t = blockIdx.x; t < n_tiles && !done; t += gridDim.x) {
      for (int kb = 0; kb < nkb; ++kb, ++g) {
        const int s = g % STAGES;
        const bool ok = mbar_wait_bounded_sleep(&full_bar[s], (g / STAGES) & 1);
        unsigned char* hi = smem + s * STAGE_BYTES;
        unsigned char* lo = hi + A_BYTES;
        const float* rb = reinterpret_cast<const float*>(lo);
        float x[BK];
#pragma unroll
        for (int k = 0; k < BK; ++k) x[k] = rb[k * BM + c];
        // every converter has read the raw block (and agrees on a failure)
        int any_bad;
        asm volatile(
            "{\n .reg .pred p, q;\n setp.ne.s32 q, %1, 0;\n bar.red.or.pred p, 1, %2, q;\n"
            " selp.s32 %0, 1, 0, p;\n}\n"
            : "=r"(any_bad)
            : "r"((int)(!ok || fail)), "n"(32 * CONV_WARPS)
            : "memory");
        if (any_bad) {
          if (c == 0) atomicExch(&fail, 1);
          done = true;
          break;
        }
#pragma unroll
        for (int q = 0; q < BK / 4; ++q) {
          float h4[4], l4[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) split_tf32(x[4 * q + j], h4[j], l4[j]);
          *reinterpret_cast<float4*>(hi + sw128(c, q)) = make_float4(h4[0], h4[1], h4[2], h4[3]);
          *reinterpret_cast<float4*>(lo + sw128(c, q)) = make_float4(l4[0], l4[1], l4[2], l4[3]);
        }
        // the tensor core reads these blocks through the async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&afull_bar[s]);
      }
    }
  } else {
    // ---------------- epilogue: warps 4-11 ----------------
    const int quarter = warp & 3;  // TMEM lanes 32*quarter .. +31
    constexpr int CW = BN / (EPI_WARPS / 4);   // columns per warp
    const int cbeg = CW * ((warp - EPI_WARP0) / 4);  // this warp's first column
    int i = 0;
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, ++i) {
      const int acc = i & 1;
      const bool ok = mbar_wait_bounded_sleep(&accf_bar[acc], (i >> 1) & 1);
      // warp-uniform decision: tcgen05.ld below needs every lane
      if (__any_sync(0xffffffffu, !ok || fail)) {
        if (lane == 0) atomicExch(&fail, 1);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const int mt = t / ntn, n0 = (t - mt * ntn) * BN;
      const int m = mt * BM + quarter * 32 + lane;
      int64_t q = m;
      bool valid = m < a.M;
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
      for (int c0 = cbeg; c0 < cbeg + CW; c0 += 32) {
        float v[32];
        // all lanes of the warp take part in tcgen05.ld (sync.aligned)
        const uint32_t ta = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(2 * acc * TMEM_COLS + c0);
        tmem_ld32(ta, v);
        if (two) {
          float w[32];
          tmem_ld32(ta + TMEM_COLS, w);
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = __fadd_rn(v[j], w[j]);
        }
        if (c0 + 32 == cbeg + CW) {
          // the accumulator is in registers: hand it back to the MMAs
          asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
          __syncwarp();
          if (lane == 0) mbar_arrive(&acce_bar[acc]);
        }
        if (!valid) continue;
        if (a.out32) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c0 + j;
            if (n < a.N) a.out32[(int64_t)n * a.ldo + m] = v[j];
          }
        }
        if (a.acc0) {
          // Column n of the tile goes to plane n (acc0) or n - nsplit (acc1).
          const int nb = n0 + c0;
          if (a.overwrite && nb + 32 <= a.N && (nb + 32 <= a.nsplit || nb >= a.nsplit)) {
            // the 32 columns are whole and on one side of the split: plain
            // stores along one plane stride (warp-uniform branch)
            double* p = nb < a.nsplit ? a.acc0 + (int64_t)nb * a.ldacc + q
                                      : a.acc1 + (int64_t)(nb - a.nsplit) * a.ldacc + q;
#pragma unroll
            for (int j = 0; j < 32; ++j, p += a.ldacc) *p = widen_exact(v[j]);
            continue;
          }
          if (!a.overwrite) {
            // Accumulate: FP64 reductions performed in L2.  Each element has
            // one writer per pass, so this is the same IEEE addition as a
            // load, add and store, without the load's round trip.
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const int n = nb + j;
              if (n < a.N)
                atomicAdd(n < a.nsplit ? a.acc0 + (int64_t)n * a.ldacc + q
                                       : a.acc1 + (int64_t)(n - a.nsplit) * a.ldacc + q,
                          widen_exact(v[j]));
            }
            continue;
          }
          // Overwrite with a partial or split group of columns: plain stores.
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = nb + j;
            if (n < a.N)
              *(n < a.nsplit ? a.acc0 + (int64_t)n * a.ldacc + q
                             : a.acc1 + (int64_t)(n - a.nsplit) * a.ldacc + q) = widen_exact(v[j]);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_ALLOC)
                 : "memory");
  }
  if (tid == 0 && fail) set_error_flag(err, 2);
}

}  // namespace

size_t contract_image_floats(int X, int Kd) {
  const size_t nxt = (size_t)(X + 127) / 128, nkb = (size_t)(Kd + BK - 1) / BK;
  return std::max<size_t>(1, nxt * nkb) * 2 * 128 * BK;
}

fd2d_status contract_image(fd2d_ctx* ctx, cudaStream_t stream, const float* src, int64_t ld, int X, int Kd,
                           float* img) {
  if (X <= 0 || Kd <= 0) return FD2D_OK;
  dim3 grid((X + 127) / 128, (Kd + BK - 1) / BK);
  // timed with the contractions it feeds (inside a time loop it is not stencil time)
  const int t0 = timer_begin(ctx, stream);
  k_image<<<grid, 256, 0, stream>>>(src, ld, X, Kd, (Kd + BK - 1) / BK, img);
  timer_end(ctx, stream, t0, FD2D_TIMER_CONTRACT, 0);
  return after_launch(ctx, "k_image");
}

PerDeviceOnce g_contract_attributes;
fd2d_status contract_prepare(fd2d_ctx* ctx) {
  return g_contract_attributes.run(ctx, [ctx]() -> fd2d_status {
    FD2D_CUDA(ctx, cudaFuncSetAttribute(k_contract_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
    return FD2D_OK;
  });
}

fd2d_status contract(fd2d_ctx* ctx, cudaStream_t stream, const ContractArgs& a) {
  if (a.M <= 0 || a.N <= 0 || a.Kd <= 0) return FD2D_OK;
  const int nkb = (a.Kd + BK - 1) / BK;
  if (!a.a32 || !a.bimg || a.img_nkb < nkb + a.img_kb0 || a.lda < a.M || a.lda % 4 ||
      (reinterpret_cast<uintptr_t>(a.a32) & 15))
    return set_error(ctx, FD2D_ERR_ARG, "contraction without an aligned A or a B image covering its K blocks");
  // A in FP32, one 128-point by 32-deep block per copy (zeros past M and Kd)
  CUtensorMap amap;
  FD2D_TRY(make_tmap_f32(ctx, &amap, a.a32, a.M, a.Kd, a.lda, BM, BK));
  const int ntn = (a.N + BN - 1) / BN;
  const int64_t tiles = (int64_t)((a.M + BM - 1) / BM) * ntn;
  if (tiles > 0x7fffffff) return set_error(ctx, FD2D_ERR_SHAPE, "contraction too large for one launch");
  const int grid = (int)std::min<int64_t>(tiles, std::max(ctx->sm_count, 1));
  const int t0 = timer_begin(ctx, stream);
  // Highest scheduling priority: the persistent grid needs a whole SM per CTA,
  // and beside other solves' step kernels (parallel branches of a batch) an SM
  // only frees up if its CTAs are preferred when slots drain.
  int prio_least = 0, prio_greatest = 0;
  cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(NTHREADS_P);
  cfg.dynamicSmemBytes = SMEM_BYTES;
  cfg.stream = stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio_greatest;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_contract_tc, a, ntn, (int)tiles, ctx->d_err, amap);
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
  if (M == 0 || N == 0 || Kd == 0) return FD2D_OK;
  // A is read by the tensor-memory copies: a 16-byte aligned copy with a row
  // stride of a multiple of 4 floats when the caller's is not
  const float* a32 = A;
  int64_t la = lda;
  if ((reinterpret_cast<uintptr_t>(A) & 15) || lda % 4) {
    la = (M + 3) / 4 * 4;
    float* ac = nullptr;
    FD2D_TRY(workspace_t(ctx, "contract.a", (size_t)la * Kd, &ac));
    FD2D_CUDA(ctx, cudaMemcpy2DAsync(ac, la * 4, A, lda * 4, (size_t)M * 4, Kd, cudaMemcpyDeviceToDevice,
                                     ctx->stream));
    a32 = ac;
  }
  float* bimg = nullptr;
  FD2D_TRY(workspace_t(ctx, "contract.bimg", contract_image_floats(N, Kd), &bimg));
  FD2D_TRY(contract_image(ctx, ctx->stream, B, ldb, N, Kd, bimg));
  ContractArgs c;
  c.M = M; c.N = N; c.Kd = Kd; c.out32 = R; c.ldo = ldr;
  c.a32 = a32; c.lda = la;
  c.bimg = bimg; c.img_nkb = (Kd + CONTRACT_BK - 1) / CONTRACT_BK;
  return contract(ctx, ctx->stream, c);
}
