// solver_fp32.cu -- the FP32 form of the three solvers.
//
// Per time step ONE fused kernel (k32_step) advances a 32x32 tile of the grid:
//   DS  = div_s(sxy, szy) (+ point sources) (+ injected correlation source)
//   v   = (v + DS * dt/rho) * absbound
//   sxy += dt*mu * dx_v(v),  szy += dt*mu * dz_v(v),  u += v*dt
// (code/run_forward1_green.m:148-172, code/run_forward2_correlation.m:190-242,
// code/run_noise_adjoint.m:245-297).  One elected thread stages the tile's
// halo boxes (sxy, szy, v, dt/rho, taper, injection plane, dt*mu, u) into
// shared memory with TMA tensor loads -- the hardware zero-fills everything
// outside the grid -- while the other threads read their point sources.  The
// CTA then recomputes the new v on the halo ring, so the stress update needs no
// second pass, and writes v, sxy, szy, u once: 36 B (44 B with u) of HBM
// traffic per grid-point update.  Fields are ping-ponged between two buffers
// so neighbouring tiles never read a half-updated halo.
//
// Internal FP32 arrays are pitched (row pitch P = nx rounded up to 32 floats,
// a multiple of 16 bytes as TMA requires); user arrays keep MATLAB layout.
//
// The dense work leaves the time loop:
//  * the DFT of v (Green spectrum) / u (adjoint spectrum, source kernel) is a
//    contraction of stored snapshots with the DFT basis (contract.cuh), with
//    FP64 accumulation of the spectra;
//  * the correlation / adjoint field source real(sum_k P_k e^{i w_k t}) is a
//    contraction of P = spectrum*distribution*G planes with the time basis,
//    evaluated for all injection steps before the loop and read by the stencil
//    as one plane per injection step.
// The mu kernel accumulates in FP64 from FP32 strains; the source kernel is
// formed once from the adjoint spectrum (see fp32_adjoint).  Time loops run as
// cached CUDA graphs (run_captured).
#include "common.cuh"
#include "contract.cuh"
#include "fp_bits.cuh"
#include "tma.cuh"

#include <algorithm>
#include <cstdlib>
#include <type_traits>

namespace fd2d {
namespace {

// Tiles are TX = 32 points wide and TZ rows high; TZ is 16, 30, 32 or 40
// (chosen per grid and lane count by tune_tile_rows), with TX/4 * TZ threads
// per CTA.
constexpr int TX = 32;
constexpr int N_TILE_ROWS = 4;
constexpr int TILE_ROWS[N_TILE_ROWS] = {16, 30, 32, 40};
constexpr int MAX_BOX_SRC = 64;
constexpr int MAX_TILE_REC = 32;  // receivers of one tile kept in shared memory

struct Grid32 {
  int nx, nz, P;  // P: row pitch of internal arrays (floats)
  int S;          // lanes: solves of this grid advanced by one launch
  int ntx, ntz;   // step tiles per lane along x and z
  int64_t ps;     // plane stride of the pitched arrays; lane l's plane starts at l*ps
  float c[4];
  float inv_dx, inv_dz, dt;
  int* err;       // device error flag (bounded waits)
  // tiles blockIdx.x in [t1x0, t1x1], blockIdx.y in [t1z0, t1z1] have taper == 1
  // exactly on their whole halo box: they skip its load and the multiply
  int t1x0, t1x1, t1z0, t1z1;
};

// tile (tx, tz) in the all-ones taper rectangle of G
__device__ __forceinline__ bool taper_is_one(const Grid32& G, int tx, int tz) {
  return tx >= G.t1x0 && tx <= G.t1x1 && tz >= G.t1z0 && tz <= G.t1z1;
}

// Rows of the first part of a tile's field loads: the box rows the first
// round of phase-1 items covers (NT items of `quads` per row), rounded up to a
// multiple of 4 so that the second part starts 128-byte aligned in shared
// memory (rows are 160 or 192 bytes); and the szy rows those box rows read.
__host__ __device__ constexpr int split_top_rows(int nt, int quads, int bh) {
  return ((nt + quads - 1) / quads + 3) / 4 * 4 < bh ? ((nt + quads - 1) / quads + 3) / 4 * 4 : bh - 1;
}
__host__ __device__ constexpr int split_top_szy(int h1, int r, int szh) {
  return (h1 + 2 * r - 1 + 3) / 4 * 4 < szh ? (h1 + 2 * r - 1 + 3) / 4 * 4 : szh;
}

// Shared-memory layout of one tile (floats, regions 128-byte aligned); the
// displacement (HU) and injection (HI) regions exist only in the variants
// that load them.  The new v is written over the old one in place.  Tiles of
// 30 rows or more read the injection plane straight from L2 (it is only
// needed point-wise), which keeps five (30, 32 rows) or four (40 rows) of them
// resident per SM.
template <int R, bool HU = true, bool HI = true, int TZ_ = 32>
struct Tile {
  static constexpr int TZ = TZ_;
  // one 4-wide row segment per thread in phase 2, at most 256 threads
  static constexpr int NT = (TX / 4) * TZ < 256 ? (TX / 4) * TZ : 256;
  static constexpr bool INJ_SMEM = HI && TZ < 30;
  // otherwise interior tiles (taper all ones) load the injection box into the
  // taper region, and edge tiles read it from L2
  static constexpr bool INJ_IN_T = HI && !INJ_SMEM;
  static constexpr int BWc = TX + 2 * R - 1;  // computed v box width (x from x0-R+1)
  static constexpr int BH = TZ + 2 * R - 1;   // box rows (z from z0-R+1)
  static constexpr int SZH = TZ + 4 * R - 2;  // szy rows (z from z0-2R+1)
  static constexpr int BWa = TX + 8;          // loaded box width (x from x0-4)
  static constexpr int SXWa = TX + 16;        // sxy region width (x from x0-8)
  static constexpr int al(int n) { return (n + 31) / 32 * 32; }
  static constexpr int O_SXY = 0;
  static constexpr int O_SZY = O_SXY + al(BH * SXWa);
  static constexpr int O_V = O_SZY + al(SZH * BWa);
  static constexpr int O_B = O_V + al(BH * BWa);
  static constexpr int O_T = O_B + al(BH * BWa);
  static constexpr int O_I = O_T + al(BH * BWa);
  static constexpr int O_MU = O_I + (INJ_SMEM ? al(BH * BWa) : 0);
  static constexpr int O_U = O_MU + al(TZ * TX);
  static constexpr int TOTAL = O_U + (HU ? al(TZ * TX) : 0);
  static_assert(BH + 2 * R - 1 <= SZH, "the z sum of the last box row stays inside the szy rows");
  // The field boxes arrive in two parts with a barrier each: rows [0, H1) of
  // sxy and v and rows [0, H1Z) of szy (everything the first round of
  // phase-1 items reads), then the rest and u, so the first round computes
  // while the second part is still in flight.
  static constexpr int H1 = split_top_rows(NT, BWa / 4, BH);
  static constexpr int H1Z = split_top_szy(H1, R, SZH);
  static_assert(H1 > 0 && H1 < BH && H1Z > 0 && H1Z <= SZH, "two-part field loads");
  static constexpr int BYTES = TOTAL * 4 + 128;      // + alignment slack
  // resident CTAs per SM the shared memory allows (228 KB per SM, 1 KB per CTA
  // reserved, ~1 KB of static shared variables), at most 8
  static constexpr int CTAS = (228 * 1024) / (BYTES + 2048) < 8 ? (228 * 1024) / (BYTES + 2048) : 8;
  // CTAs per SM to ask of the register allocator: the shared-memory limit, but
  // no fewer than 64 registers per thread (4 CTAs of 256 threads at order 8)
  // -- except for 30- and 32-row tiles, which run five CTAs per SM within 48
  // registers without spilling: two 600x600 lanes are 760 tiles of 32x30,
  // exactly five on each of the 152 SMs (722 tiles of 32x32 leave 38 SMs with
  // four while the step waits for the SMs with five)
  static constexpr int MINB_64 = CTAS < 65536 / (NT * 64) ? CTAS : 65536 / (NT * 64);
  static constexpr int MINB = (TZ == 30 || TZ == 32) ? (CTAS < 5 ? CTAS : 5) : MINB_64;
};

// Field maps come in pairs: the top part (rows [0, H1) of the box, [0, H1Z)
// of szy) and the bottom part of the tile's boxes.
struct alignas(64) StepMaps {
  CUtensorMap sxy_t, sxy_b, szy_t, szy_b, v_t, v_b, u, b, taper, dtmu, inj;
};

// Per-step arguments.  Arrays marked "per lane" hold lane l's part at the
// stated offset (lanes are the solves of one launch, blockIdx.z).
struct Step32 {
  float *vo, *sxyo, *szyo, *uo;  // fields written this step (buffer 1 - par); per lane + l*ps
  int has_u;
  int inj_plane;                 // plane of the injection map (lane l reads plane inj_plane*S + l), or -1
  const int2* src_xy;            // per lane + l*nsrc
  int nsrc;
  const double* amp;             // per-source amplitude of this step (per lane + l*nsrc), or nullptr -> amp_const
  float amp_const;
  float* snap_pre;               // single(old field) in MATLAB layout, or nullptr (one lane only)
  int snap_pre_u;
  const float* inj_base;         // injection planes ([plane][lane] of stride ps), read when not staged
  float* snap_dft;               // new field (v or u) into the DFT snapshot plane (pitched); per lane + l*ps
  const int2* rec_xy;            // per lane + l*nrec
  int nrec;
  const int2* tile_rec;          // per (lane, tile): {first entry, count} of its receivers
  const int2* rec_ent;           // receiver entries {k, (z - z0)*TX + (x - x0)}
  double* seis_col;              // seismograms(:, n); per lane + l*seis_lane
  int64_t seis_lane;
  int rec_u;
};

// Where a CTA's tile lies.  One-geometry launches: blockIdx = (tile column,
// tile row, lane); multi-geometry launches: one solve's rows of the stacked
// field arrays (k32_step_multi).
struct TileLoc {
  int tx, tz;      // tile column and row in the solve
  int x0, z0;      // first point of the tile
  int lane;        // lane (third tensor-map coordinate)
  int t;           // tile number in the solve's receiver tables
  int ty0;         // first row of the solve in the field arrays (tensor-map y offset)
  int64_t lo;      // element offset of the solve's plane in the field arrays (row pitch G.P)
  int64_t slo;     // offset of the tile's lane in the DFT snapshot planes
  int sp;          // row pitch of the DFT snapshot and injection planes
};

template <int R, bool HU, bool HI, int TZ, bool MULTI>
__device__ __forceinline__ void issue_tile(const Grid32& G, const StepMaps& M, const Step32& S, float* buf,
                                           uint64_t* bar, const TileLoc& L, bool coeffs, bool fields) {
  using T = Tile<R, HU, HI, TZ>;
  static_assert(!(MULTI && T::INJ_SMEM), "multi-geometry launches read the injection planes from L2");
  const int x0 = L.x0, z0 = L.ty0 + L.z0, lane = L.lane;
  const int bz0 = z0 - R + 1, zz0 = z0 - 2 * R + 1;
  if (coeffs) {
    // Coefficient planes and the injection plane are not written by the time
    // loop, so they load before the wait for the previous step.  Tiles whose
    // taper is all ones do not load it; the injection box takes its place.
    const bool t1 = taper_is_one(G, L.tx, L.tz);
    const bool inj_t = T::INJ_IN_T && !MULTI && t1;
    uint32_t b0 = 4u * (T::BH * T::BWa + TZ * TX + T::H1 * T::SXWa + T::H1Z * T::BWa + T::H1 * T::BWa);
    if (!t1) b0 += 4u * T::BH * T::BWa;
    if (T::INJ_SMEM || inj_t) b0 += 4u * T::BH * T::BWa;
    uint32_t b1 = 4u * ((T::BH - T::H1) * (T::SXWa + T::BWa) + (T::SZH - T::H1Z) * T::BWa);
    if (HU) b1 += 4u * TZ * TX;
    mbar_expect_tx(&bar[0], b0);
    mbar_expect_tx(&bar[1], b1);
    tma_load_3d(buf + T::O_B, &M.b, x0 - 4, bz0, lane, &bar[0]);
    if (!t1) tma_load_3d(buf + T::O_T, &M.taper, x0 - 4, bz0, lane, &bar[0]);
    tma_load_3d(buf + T::O_MU, &M.dtmu, x0, z0, lane, &bar[0]);
    if (T::INJ_SMEM) tma_load_3d(buf + T::O_I, &M.inj, x0 - 4, bz0, S.inj_plane * G.S + lane, &bar[0]);
    else if (inj_t) tma_load_3d(buf + T::O_T, &M.inj, x0 - 4, bz0, S.inj_plane * G.S + lane, &bar[0]);
  }
  if (fields) {
    tma_load_3d(buf + T::O_SXY, &M.sxy_t, x0 - 8, bz0, lane, &bar[0]);
    tma_load_3d(buf + T::O_SZY, &M.szy_t, x0 - 4, zz0, lane, &bar[0]);
    tma_load_3d(buf + T::O_V, &M.v_t, x0 - 4, bz0, lane, &bar[0]);
    tma_load_3d(buf + T::O_SXY + T::H1 * T::SXWa, &M.sxy_b, x0 - 8, bz0 + T::H1, lane, &bar[1]);
    if (T::SZH > T::H1Z) tma_load_3d(buf + T::O_SZY + T::H1Z * T::BWa, &M.szy_b, x0 - 4, zz0 + T::H1Z, lane, &bar[1]);
    tma_load_3d(buf + T::O_V + T::H1 * T::BWa, &M.v_b, x0 - 4, bz0 + T::H1, lane, &bar[1]);
    if (HU) tma_load_3d(buf + T::O_U, &M.u, x0, z0, lane, &bar[1]);
  }
}

// The step of one tile: everything a CTA of k32_step or k32_step_multi does.
// G, S and L are the kernel's parameters (one-geometry launches) or shared
// copies resolved per CTA (multi-geometry launches); cf are the FD weights.
template <int R, bool HU, bool HI, int TZ, bool MULTI>
__device__ __forceinline__ void step_tile(const Grid32& G, const StepMaps& M, const Step32& S, const TileLoc& L,
                                          const float* cf) {
  using T = Tile<R, HU, HI, TZ>;
  constexpr int NT = T::NT;
  extern __shared__ __align__(128) unsigned char sm_raw[];
  // TMA destinations: 128-byte aligned regardless of the static smem in front
  // (offset arithmetic on the shared array keeps the pointer in the shared
  // address space, so the float4 accesses below compile to shared loads)
  float* sm = reinterpret_cast<float*>(sm_raw + ((128u - (smem_u32(sm_raw) & 127u)) & 127u));
#define inv_dx G.inv_dx
#define inv_dz G.inv_dz
#define gdt G.dt
  __shared__ __align__(8) uint64_t bar[2];  // top part (+ coefficients), bottom part (+ u)
  __shared__ int s_src[MAX_BOX_SRC];
  __shared__ float s_amp[MAX_BOX_SRC];
  __shared__ int s_nsrc;
  __shared__ int2 s_rec[MAX_TILE_REC];
  __shared__ int s_nrec;

  const int tid = threadIdx.x;
  const int nx = G.nx, nz = G.nz, P = G.P;
  constexpr int W = T::BWa;  // 40: row stride of the box regions
  float* s_vn = sm + T::O_V;  // new v, written over the old v of the same point
  constexpr bool inj = HI;
  const int t = L.t;  // tile number in the receiver tables
  if (tid == 0) {
    s_nsrc = 0;
    s_nrec = 0;
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    // coefficient planes are not written by the time loop: their loads may
    // overlap the end of the previous step (programmatic dependent launch)
    issue_tile<R, HU, HI, TZ, MULTI>(G, M, S, sm, bar, L, true, false);
    // The fields are what the previous launch wrote (or will write what it
    // read: ping-pong buffers): wait for it to complete, then load them.  The
    // other threads touch those buffers only after this tile's loads land, so
    // this thread's wait orders the whole CTA after the previous step.
    asm volatile("griddepcontrol.wait;" ::: "memory");
    issue_tile<R, HU, HI, TZ, MULTI>(G, M, S, sm, bar, L, false, true);
  }
  {
    const float* buf = sm;
    const int x0 = L.x0, z0 = L.z0, lane = L.lane;
    const int bz0 = z0 - R + 1, vx0 = x0 - 4;
    const int64_t lo = L.lo;
    const int2* src_xy = S.src_xy + (int64_t)lane * S.nsrc;
    const double* amp = S.amp ? S.amp + (int64_t)lane * S.nsrc : nullptr;
    __syncthreads();  // barrier initialised, lists cleared
    // receivers and point sources of this tile (static tables), read while
    // the tile's loads are in flight
    if (S.nrec && tid < 32) {
      if (S.tile_rec) {
        const int2 se = S.tile_rec[t];
        if (tid == 0) s_nrec = se.y <= MAX_TILE_REC ? se.y : -1;
        for (int q = tid; q < se.y && q < MAX_TILE_REC; q += 32) s_rec[q] = S.rec_ent[se.x + q];
      } else if (tid == 0) {
        s_nrec = -1;  // no tables: search the receiver list after the update
      }
    }
    // point sources in the box, listed by warp 0 in source order (the
    // reference's order of addition, so the sums are reproducible)
    if (tid < 32 && S.nsrc) {
      int base = 0;
      for (int k0 = 0; k0 < S.nsrc; k0 += 32) {
        const int k = k0 + tid;
        int2 q = make_int2(0, 0);
        bool in = false;
        if (k < S.nsrc) {
          q = src_xy[k];
          in = q.x >= vx0 && q.x < vx0 + W && q.y >= bz0 && q.y < bz0 + T::BH;
        }
        const unsigned m = __ballot_sync(0xffffffffu, in);
        const int slot = base + __popc(m & ((1u << tid) - 1u));
        if (in && slot < MAX_BOX_SRC) {
          s_src[slot] = (q.y - bz0) * W + (q.x - vx0);
          s_amp[slot] = amp ? (float)amp[k] : S.amp_const;
        }
        base += __popc(m);
      }
      if (tid == 0) s_nsrc = base;
    }
    // one warp waits for the top part of the tile (suspending); the others
    // wait at the barrier
    bool ok = true;
    if (tid < 32) ok = mbar_wait_bounded_sleep(&bar[0], 0);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        set_error_flag(G.err, 1);
        // let started copies land (bounded)
        mbar_wait_bounded_sleep(&bar[0], 0, 100000000ull);
        mbar_wait_bounded_sleep(&bar[1], 0, 100000000ull);
      }
      return;
    }
    // the bottom part: waited for by every thread with a second-round
    // phase-1 item before it, and by warp 0 before phase 2
    bool ok1 = true, waited1 = false, bad = false;
    // the tile is in shared memory: the next step may launch and run its
    // prologue (its own wait orders it after this grid's stores)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int nbs = s_nsrc;
    const float* s_sxy = buf + T::O_SXY;
    const float* s_szy = buf + T::O_SZY;
    const float* s_v = buf + T::O_V;
    const float* s_b = buf + T::O_B;
    const float* s_t = buf + T::O_T;
    const bool t1 = taper_is_one(G, L.tx, L.tz);
    const float* s_i = buf + T::O_I;
    const float* s_mu = buf + T::O_MU;
    const float* s_u = buf + T::O_U;

    // Interior tiles (the halo box inside the operator's range on every side)
    // skip the edge selects and partial stores: one uniform branch per CTA.
    const bool edge = !(x0 >= R + 4 && x0 + TX + 4 + R <= nx && z0 >= 2 * R - 1 && z0 + TZ + 2 * R <= nz);
    auto compute = [&](auto edge_tag) {
      constexpr bool EDGE = decltype(edge_tag)::value;
    // Every rounding below is spelled out (__fmaf_rn / __fmul_rn / __fadd_rn), so
    // the result of a point does not depend on which kernel instantiation (tile
    // shape, edge or interior path) computes it.
    // ---- new v on the box: 4-wide blocks of rows ---------------------------------------
    // DS = div_s(sxy, szy) (+ sources) (+ injection); v = (v + DS*dt/rho)*taper.
    // Sums are formed in the same order as the scalar form (m = 1..R).
    {
      // work item: a 4-wide block of NB1 rows; NB1 = 1 keeps the kernel within
      // 64 registers (4 resident CTAs per SM) without spills
      constexpr int NB1 = 1;
      constexpr int NQ = W / 4, NRB = (T::BH + NB1 - 1) / NB1;
      for (int item = tid; item < NQ * NRB; item += NT) {
        if (item >= NT && !waited1) {
          ok1 = mbar_wait_bounded_sleep(&bar[1], 0);
          waited1 = true;
        }
        if (!ok1) break;
        const int q = item % NQ, r0 = NB1 * (item / NQ);
        const int c0 = 4 * q;  // box column of element 0; global x = vx0 + c0 + e
        float zs[2 * R + NB1 - 1][4];
#pragma unroll
        for (int k = 0; k < 2 * R + NB1 - 1; ++k) {
          // szy row r0 + k holds szy(gz0 + k - R) for gz0 = global z of row r0
          // (one-row items never reach past the last szy row: no clamp)
          const int rr = NB1 == 1 ? r0 + k : min(r0 + k, T::SZH - 1);
          const float4 f = *reinterpret_cast<const float4*>(s_szy + rr * W + c0);
          zs[k][0] = f.x; zs[k][1] = f.y; zs[k][2] = f.z; zs[k][3] = f.w;
        }
#pragma unroll
        for (int k = 0; k < NB1; ++k) {
          const int rr = r0 + k;
          if (NB1 > 1 && rr >= T::BH) break;
          const int gz = bz0 + rr;
          const bool zin = gz >= R && gz <= nz - R - 1;
          float xs[12];  // sxy columns c0 .. c0+11 (x from x0-8 = box column - 4)
          {
            const float4* rowp = reinterpret_cast<const float4*>(s_sxy + rr * T::SXWa + c0);
#pragma unroll
            for (int h = 0; h < 3; ++h) {
              const float4 f = rowp[h];
              xs[4 * h] = f.x; xs[4 * h + 1] = f.y; xs[4 * h + 2] = f.z; xs[4 * h + 3] = f.w;
            }
          }
          float dsv[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int gx = vx0 + c0 + e;
            // both sums are formed everywhere and selected (no divergent branches)
            // sxy(gx + m - 1) is xs[e + 3 + m], sxy(gx - m) is xs[e + 4 - m]
            float ax = 0.f;
#pragma unroll
            for (int m = 1; m <= R; ++m) ax = __fmaf_rn(cf[m - 1], __fsub_rn(xs[e + 3 + m], xs[e + 4 - m]), ax);
            // szy(gz + m - 1) is zs[k + R + m - 1], szy(gz - m) is zs[k + R - m]
            float az = 0.f;
#pragma unroll
            for (int m = 1; m <= R; ++m) az = __fmaf_rn(cf[m - 1], __fsub_rn(zs[k + R + m - 1][e], zs[k + R - m][e]), az);
            float ds = (!EDGE || (gx >= R && gx <= nx - R - 1)) ? __fmul_rn(ax, inv_dx) : 0.f;
            ds = (!EDGE || zin) ? __fmaf_rn(az, inv_dz, ds) : ds;
            dsv[e] = ds;
          }
          if (nbs) {
            // point sources in this block (only tiles that hold one), added in
            // list order after the stencil sums
            const int idx0 = rr * W + c0;
            if (nbs <= MAX_BOX_SRC) {
              for (int qq = 0; qq < nbs; ++qq) {
                const int d = s_src[qq] - idx0;
#pragma unroll
                for (int e = 0; e < 4; ++e)
                  if (d == e) dsv[e] = __fadd_rn(dsv[e], s_amp[qq]);
              }
            } else {
              for (int qq = 0; qq < S.nsrc; ++qq) {
                const int2 w = src_xy[qq];
                const int d = w.x - (vx0 + c0);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                  if (w.y == gz && d == e) dsv[e] = __fadd_rn(dsv[e], amp ? (float)amp[qq] : S.amp_const);
              }
            }
          }
          // the point-wise operands are read once the stencil sums are formed
          // (fewer live registers)
          const float4 v4 = *reinterpret_cast<const float4*>(s_v + rr * W + c0);
          const float4 b4 = *reinterpret_cast<const float4*>(s_b + rr * W + c0);
          const float4 t4 = t1 ? make_float4(1.f, 1.f, 1.f, 1.f)
                               : *reinterpret_cast<const float4*>(s_t + rr * W + c0);
          float4 i4 = make_float4(0.f, 0.f, 0.f, 0.f);
          if (T::INJ_SMEM) {
            i4 = *reinterpret_cast<const float4*>(s_i + rr * W + c0);
          } else if (inj && t1 && !MULTI) {
            i4 = *reinterpret_cast<const float4*>(s_t + rr * W + c0);  // the injection box (issue_tile)
          } else if (inj) {
            // from L2; outside the grid the plane is zero (as the TMA fill)
            const int gx0 = vx0 + c0;
            if (gx0 >= 0 && gx0 < L.sp && gz >= 0 && gz < nz)
              i4 = __ldg(reinterpret_cast<const float4*>(S.inj_base + ((int64_t)S.inj_plane * G.S + lane) * G.ps +
                                                         (int64_t)L.sp * gz + gx0));
          }
          if (S.snap_pre && !S.snap_pre_u && rr >= R - 1 && rr < R - 1 + TZ && c0 >= 4 && c0 < 4 + TX) {
            // single(v) before the update at the tile's own points, taken here
            // because the new v replaces the old one in shared memory
            const int gx0 = vx0 + c0;
            const float vo[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (!EDGE || (gx0 + e < nx && gz < nz)) S.snap_pre[gx0 + e + (int64_t)nx * gz] = vo[e];
          }
          const float vv[4] = {v4.x, v4.y, v4.z, v4.w}, bb[4] = {b4.x, b4.y, b4.z, b4.w};
          const float tt[4] = {t4.x, t4.y, t4.z, t4.w}, ii[4] = {i4.x, i4.y, i4.z, i4.w};
          float out[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float ds = inj ? __fadd_rn(dsv[e], ii[e]) : dsv[e];
            // (a taper of exactly 1 leaves the product unchanged: skipped)
            out[e] = t1 ? __fmaf_rn(ds, bb[e], vv[e]) : __fmul_rn(__fmaf_rn(ds, bb[e], vv[e]), tt[e]);
          }
          *reinterpret_cast<float4*>(s_vn + rr * W + c0) = make_float4(out[0], out[1], out[2], out[3]);
        }
      }
    }
    if (tid < 32 && !waited1) ok1 = mbar_wait_bounded_sleep(&bar[1], 0);
    if (__syncthreads_or(!ok1)) {
      if (tid == 0) {
        set_error_flag(G.err, 1);
        mbar_wait_bounded_sleep(&bar[1], 0, 100000000ull);  // let started copies land (bounded)
      }
      bad = true;
      return;
    }

    // ---- stress, displacement and outputs: each thread 4-wide row segments -----------
    constexpr int NQ2 = TX / 4;  // 8 quads per row
    for (int it = tid; it < NQ2 * TZ; it += NT) {
      const int q = it % NQ2, tz = it / NQ2;
      const int j = z0 + tz;
      const int i0 = x0 + 4 * q;
      if (tz < TZ && (!EDGE || (j < nz && i0 < nx))) {
        const int rr = tz + R - 1;  // box row of output row j
        const int cv = 4 + 4 * q;   // box column of element 0
        // vx = box columns cv-4 .. cv+7: v(i) is vx[e + 4], v(i + m) is vx[e + m + 4],
        // v(i - m + 1) is vx[e - m + 5]
        float vx[12];
        {
          const float4* rowp = reinterpret_cast<const float4*>(s_vn + rr * W + cv - 4);
#pragma unroll
          for (int h = 0; h < 3; ++h) {
            const float4 f = rowp[h];
            vx[4 * h] = f.x; vx[4 * h + 1] = f.y; vx[4 * h + 2] = f.z; vx[4 * h + 3] = f.w;
          }
        }
        float vz[2 * R][4];  // box rows rr - R + 1 .. rr + R; row rr is vx[4..7]
#pragma unroll
        for (int k = 0; k < 2 * R; ++k) {
          if (k == R - 1) {
            vz[k][0] = vx[4]; vz[k][1] = vx[5]; vz[k][2] = vx[6]; vz[k][3] = vx[7];
            continue;
          }
          const float4 f = *reinterpret_cast<const float4*>(s_vn + (rr - R + 1 + k) * W + cv);
          vz[k][0] = f.x; vz[k][1] = f.y; vz[k][2] = f.z; vz[k][3] = f.w;
        }
        const float4 mu4 = *reinterpret_cast<const float4*>(s_mu + tz * TX + 4 * q);
        const float4 sx4 = *reinterpret_cast<const float4*>(s_sxy + rr * T::SXWa + 8 + 4 * q);
        const float4 sz4 = *reinterpret_cast<const float4*>(s_szy + (tz + 2 * R - 1) * W + 4 + 4 * q);
        float4 u4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (HU) u4 = *reinterpret_cast<const float4*>(s_u + tz * TX + 4 * q);
        const float mu[4] = {mu4.x, mu4.y, mu4.z, mu4.w}, sxo[4] = {sx4.x, sx4.y, sx4.z, sx4.w};
        const float szo[4] = {sz4.x, sz4.y, sz4.z, sz4.w}, uo[4] = {u4.x, u4.y, u4.z, u4.w};
        const bool zin = j >= R - 1 && j <= nz - R - 1;
        float nsx[4], nsz[4], nu[4], vn[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int i = i0 + e;
          vn[e] = vx[e + 4];
          float ax = 0.f, az = 0.f;
#pragma unroll
          for (int m = 1; m <= R; ++m) ax = __fmaf_rn(cf[m - 1], __fsub_rn(vx[e + m + 4], vx[e - m + 5]), ax);
#pragma unroll
          for (int m = 1; m <= R; ++m) az = __fmaf_rn(cf[m - 1], __fsub_rn(vz[R - 1 + m][e], vz[R - m][e]), az);
          nsx[e] = (!EDGE || (i >= R - 1 && i <= nx - R - 1)) ? __fmaf_rn(mu[e], __fmul_rn(ax, inv_dx), sxo[e])
                                                              : sxo[e];
          nsz[e] = (!EDGE || zin) ? __fmaf_rn(mu[e], __fmul_rn(az, inv_dz), szo[e]) : szo[e];
          nu[e] = HU ? __fmaf_rn(vn[e], gdt, uo[e]) : vn[e];
        }
        const int64_t p = lo + i0 + (int64_t)P * j;
        const int64_t ps_ = L.slo + i0 + (int64_t)L.sp * j;  // in the DFT snapshot plane
        if (!EDGE || i0 + 3 < nx) {
          // whole quad inside the grid: vector stores
          *reinterpret_cast<float4*>(S.vo + p) = make_float4(vn[0], vn[1], vn[2], vn[3]);
          if (!EDGE || i0 + 3 <= nx - 2) {
            *reinterpret_cast<float4*>(S.sxyo + p) = make_float4(nsx[0], nsx[1], nsx[2], nsx[3]);
          } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (i0 + e <= nx - 2) S.sxyo[p + e] = nsx[e];
          }
          if (!EDGE || j <= nz - 2) *reinterpret_cast<float4*>(S.szyo + p) = make_float4(nsz[0], nsz[1], nsz[2], nsz[3]);
          if (HU) *reinterpret_cast<float4*>(S.uo + p) = make_float4(nu[0], nu[1], nu[2], nu[3]);
          if (S.snap_dft) *reinterpret_cast<float4*>(S.snap_dft + ps_) = make_float4(nu[0], nu[1], nu[2], nu[3]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            if (i0 + e >= nx) break;
            S.vo[p + e] = vn[e];
            if (i0 + e <= nx - 2) S.sxyo[p + e] = nsx[e];
            if (j <= nz - 2) S.szyo[p + e] = nsz[e];
            if (HU) S.uo[p + e] = nu[e];
            if (S.snap_dft) S.snap_dft[ps_ + e] = nu[e];
          }
        }
        if (S.nrec && s_nrec > 0) {
          // receivers in this quad take the new value straight from registers
          double* seis = S.seis_col + lane * S.seis_lane;
          const int l0 = tz * TX + 4 * q;
          for (int r = 0; r < s_nrec; ++r) {
            const int2 e = s_rec[r];
            const int d = e.y - l0;
            if (d >= 0 && d < 4) {
              const float xu = d == 0 ? nu[0] : d == 1 ? nu[1] : d == 2 ? nu[2] : nu[3];
              const float xv = d == 0 ? vn[0] : d == 1 ? vn[1] : d == 2 ? vn[2] : vn[3];
              seis[e.x] = (double)(S.rec_u ? xu : xv);
            }
          }
        }
        if (HU && S.snap_pre && S.snap_pre_u) {
          const float* old = s_u + tz * TX + 4 * q;
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (!EDGE || i0 + e < nx) S.snap_pre[i0 + e + (int64_t)nx * j] = old[e];
        }
      }
    }
    };
    if (edge)
      compute(std::true_type{});
    else
      compute(std::false_type{});
    if (bad) return;
    if (S.nrec && s_nrec < 0) {
      // more receivers in this tile than the shared list holds: read them back
      __syncthreads();
      const int2* rec_xy = S.rec_xy + (int64_t)lane * S.nrec;
      double* seis = S.seis_col + lane * S.seis_lane;
      for (int k = tid; k < S.nrec; k += NT) {
        const int2 q = rec_xy[k];
        if (q.x >= x0 && q.x < x0 + TX && q.y >= z0 && q.y < z0 + TZ) {
          const int64_t p = lo + q.x + P * q.y;
          seis[k] = (double)(S.rec_u ? S.uo[p] : S.vo[p]);
        }
      }
    }
  }
}
#undef inv_dx
#undef inv_dz
#undef gdt

// One-geometry step: one CTA per tile, blockIdx = (tile column, tile row, lane).
template <int R, bool HU, bool HI, int TZ>
__global__ __launch_bounds__(Tile<R, HU, HI, TZ>::NT, Tile<R, HU, HI, TZ>::MINB) void k32_step(
    Grid32 G, const __grid_constant__ StepMaps M, Step32 S) {
  TileLoc L;
  L.tx = blockIdx.x;
  L.tz = blockIdx.y;
  L.lane = blockIdx.z;
  L.x0 = L.tx * TX;
  L.z0 = L.tz * TZ;
  L.t = L.tx + G.ntx * (L.tz + G.ntz * L.lane);
  L.ty0 = 0;
  L.lo = (int64_t)L.lane * G.ps;
  L.slo = L.lo;
  L.sp = G.P;
  // coefficients stay in the parameter bank (FFMA constant operands, no registers)
  step_tile<R, HU, HI, TZ, false>(G, M, S, L, G.c);
}

// ---- two time steps per launch (time blocking, orders 2 and 4) ---------------------
// One CTA advances its 32 x TZ tile by two time steps.  It loads one box of
// every array -- x from x0-8 (56 points), z from z0-6 (TZ+12 rows), the same
// origin for all -- and recomputes the first step on a ring wide enough for
// the second:
//   A  v1 on x in [x0-4, x0+39], z in [z0-4, z0+TZ+4]   (needs stresses to x0-6 .. x0+40)
//   B  s1 on x in [x0-4, x0+35], z in [z0-3, z0+TZ+2]   (step-1 outputs on the tile)
//   C  v2 on x in [x0-4, x0+35], z in [z0-1, z0+TZ+1]
//   D  s2, v2, u2 on the tile, stored
// For R <= 2 the values each phase needs lie inside what the previous phase
// computed (at R = 2, s2 on the tile needs v2 on [x0-1, x0+33], which needs s1
// on [x0-3, x0+34], which needs v1 on [x0-4, x0+36]; in z likewise); points
// computed beyond that are never read.
// Every point is updated by the same rounded operations as in step_tile, and
// points outside the grid come out zero (all their inputs are the tensor
// maps' zero fill), so fields, seismograms and snapshots are bit for bit those
// of two launches of k32_step.
constexpr int TB_W = 56;  // box width (floats)
constexpr int TB_X = 8;   // box starts at x0 - TB_X
constexpr int TB_Z = 6;   // and z0 - TB_Z

template <int TZ_, bool HU, bool HI>
struct Tile2 {
  static constexpr int TZ = TZ_;
  static constexpr int H = TZ + 2 * TB_Z;
  static constexpr int NT = (TX / 4) * TZ < 256 ? (TX / 4) * TZ : 256;
  static constexpr int A = (TB_W * H + 31) / 32 * 32;  // floats per box array (128-byte multiples)
  static constexpr int O_SXY = 0, O_SZY = A, O_V = 2 * A, O_B = 3 * A, O_T = 4 * A, O_MU = 5 * A;
  static constexpr int O_I = 6 * A;  // injection planes of step 1 and step 2
  static constexpr int O_U = O_I + (HI ? 2 * A : 0);
  static constexpr int TOTAL = O_U + (HU ? TX * TZ : 0);
  static constexpr int BYTES = TOTAL * 4 + 128;
  // phase ranges (box quads of 4 points, box rows)
  static constexpr int QA0 = 1, QA1 = 11, RA0 = 2, RA1 = TZ + 10;
  static constexpr int QB0 = 1, QB1 = 10, RB0 = 3, RB1 = TZ + 8;
  static constexpr int QC0 = 1, QC1 = 10, RC0 = 5, RC1 = TZ + 7;
};

struct alignas(64) StepMaps2 {
  CUtensorMap sxy, szy, v, b, taper, dtmu, inj, u;
};

struct Step2 {
  Step32 s[2];  // steps n and n+1; outputs (vo, sxyo, szyo, uo) of s[1]
};

// v = (v + DS*b) * taper on one 4-wide item of box row r, box column c0 (R <= 2).
template <int R, bool EDGE>
__device__ __forceinline__ void tb_v_item(const Grid32& G, const float* cf, float* s_v, const float* s_sxy,
                                          const float* s_szy, const float* s_b, const float* s_t, const float* s_i,
                                          int r, int c0, int bx, int bz, const int* s_src, const float* s_amp,
                                          int nbs, float* snap_v, int tz) {
  constexpr int W = TB_W;
  const int gz = bz + r;
  const bool zin = gz >= R && gz <= G.nz - R - 1;
  float xs[12];
  {
    const float4* rowp = reinterpret_cast<const float4*>(s_sxy + r * W + c0 - 4);
#pragma unroll
    for (int h = 0; h < 3; ++h) {
      const float4 f = rowp[h];
      xs[4 * h] = f.x; xs[4 * h + 1] = f.y; xs[4 * h + 2] = f.z; xs[4 * h + 3] = f.w;
    }
  }
  float zs[2 * R][4];
#pragma unroll
  for (int k = 0; k < 2 * R; ++k) {
    // zs[k] holds szy(gz + k - R)
    const float4 f = *reinterpret_cast<const float4*>(s_szy + (r - R + k) * W + c0);
    zs[k][0] = f.x; zs[k][1] = f.y; zs[k][2] = f.z; zs[k][3] = f.w;
  }
  float dsv[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int gx = bx + c0 + e;
    float ax = 0.f;
#pragma unroll
    for (int m = 1; m <= R; ++m) ax = __fmaf_rn(cf[m - 1], __fsub_rn(xs[e + 3 + m], xs[e + 4 - m]), ax);
    float az = 0.f;
#pragma unroll
    for (int m = 1; m <= R; ++m) az = __fmaf_rn(cf[m - 1], __fsub_rn(zs[R + m - 1][e], zs[R - m][e]), az);
    float ds = (!EDGE || (gx >= R && gx <= G.nx - R - 1)) ? __fmul_rn(ax, G.inv_dx) : 0.f;
    ds = (!EDGE || zin) ? __fmaf_rn(az, G.inv_dz, ds) : ds;
    dsv[e] = ds;
  }
  const int idx0 = r * W + c0;
  for (int qq = 0; qq < nbs; ++qq) {
    const int d = s_src[qq] - idx0;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (d == e) dsv[e] = __fadd_rn(dsv[e], s_amp[qq]);
  }
  const float4 v4 = *reinterpret_cast<const float4*>(s_v + idx0);
  const float4 b4 = *reinterpret_cast<const float4*>(s_b + idx0);
  const float4 t4 = *reinterpret_cast<const float4*>(s_t + idx0);
  float4 i4 = make_float4(0.f, 0.f, 0.f, 0.f);
  if (s_i) i4 = *reinterpret_cast<const float4*>(s_i + idx0);
  const float vv[4] = {v4.x, v4.y, v4.z, v4.w}, bb[4] = {b4.x, b4.y, b4.z, b4.w};
  const float tt[4] = {t4.x, t4.y, t4.z, t4.w}, ii[4] = {i4.x, i4.y, i4.z, i4.w};
  if (snap_v && r >= TB_Z && r < TB_Z + tz && c0 >= TB_X && c0 < TB_X + TX) {
    // single(v) before the update at the tile's own points (mode != 0 snapshots)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int gx = bx + c0 + e;
      if (!EDGE || (gx < G.nx && gz < G.nz)) snap_v[gx + (int64_t)G.nx * gz] = vv[e];
    }
  }
  float out[4];
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float ds = s_i ? __fadd_rn(dsv[e], ii[e]) : dsv[e];
    // a taper of exactly 1 leaves the product unchanged, as step_tile's skip of it
    out[e] = __fmul_rn(__fmaf_rn(ds, bb[e], vv[e]), tt[e]);
  }
  *reinterpret_cast<float4*>(s_v + idx0) = make_float4(out[0], out[1], out[2], out[3]);
}

// sxy += mu*dx_v(v), szy += mu*dz_v(v) on one 4-wide item (stresses out of the
// operator's range keep their value); returns the item's v in vn.
template <int R, bool EDGE>
__device__ __forceinline__ void tb_s_item(const Grid32& G, const float* cf, const float* s_v, const float* s_sxy,
                                          const float* s_szy, const float* s_mu, int r, int c0, int bx, int bz,
                                          float nsx[4], float nsz[4], float vn[4]) {
  constexpr int W = TB_W;
  const int j = bz + r;
  float vx[12];
  {
    const float4* rowp = reinterpret_cast<const float4*>(s_v + r * W + c0 - 4);
#pragma unroll
    for (int h = 0; h < 3; ++h) {
      const float4 f = rowp[h];
      vx[4 * h] = f.x; vx[4 * h + 1] = f.y; vx[4 * h + 2] = f.z; vx[4 * h + 3] = f.w;
    }
  }
  float vz[2 * R][4];  // box rows r - R + 1 .. r + R
#pragma unroll
  for (int k = 0; k < 2 * R; ++k) {
    const float4 f = *reinterpret_cast<const float4*>(s_v + (r - R + 1 + k) * W + c0);
    vz[k][0] = f.x; vz[k][1] = f.y; vz[k][2] = f.z; vz[k][3] = f.w;
  }
  const float4 mu4 = *reinterpret_cast<const float4*>(s_mu + r * W + c0);
  const float4 sx4 = *reinterpret_cast<const float4*>(s_sxy + r * W + c0);
  const float4 sz4 = *reinterpret_cast<const float4*>(s_szy + r * W + c0);
  const float mu[4] = {mu4.x, mu4.y, mu4.z, mu4.w}, sxo[4] = {sx4.x, sx4.y, sx4.z, sx4.w};
  const float szo[4] = {sz4.x, sz4.y, sz4.z, sz4.w};
  const bool zin = j >= R - 1 && j <= G.nz - R - 1;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int i = bx + c0 + e;
    vn[e] = vx[e + 4];
    float ax = 0.f, az = 0.f;
#pragma unroll
    for (int m = 1; m <= R; ++m) ax = __fmaf_rn(cf[m - 1], __fsub_rn(vx[e + m + 4], vx[e - m + 5]), ax);
#pragma unroll
    for (int m = 1; m <= R; ++m) az = __fmaf_rn(cf[m - 1], __fsub_rn(vz[R - 1 + m][e], vz[R - m][e]), az);
    nsx[e] = (!EDGE || (i >= R - 1 && i <= G.nx - R - 1)) ? __fmaf_rn(mu[e], __fmul_rn(ax, G.inv_dx), sxo[e]) : sxo[e];
    nsz[e] = (!EDGE || zin) ? __fmaf_rn(mu[e], __fmul_rn(az, G.inv_dz), szo[e]) : szo[e];
  }
}

// Outputs of one step at a tile item: DFT snapshot and receivers of the new
// field (u with displacement, else v).
__device__ __forceinline__ void tb_outputs(const Grid32& G, const Step32& S, bool edge, int lane, int64_t lo,
                                           int i0, int j, int l0, const float nu[4], const float vn[4],
                                           const int2* s_rec, int nrec) {
  if (S.snap_dft && (!edge || j < G.nz)) {
    const int64_t ps_ = lo + i0 + (int64_t)G.P * j;
    if (!edge || i0 + 3 < G.nx) {
      *reinterpret_cast<float4*>(S.snap_dft + ps_) = make_float4(nu[0], nu[1], nu[2], nu[3]);
    } else {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        if (i0 + e < G.nx) S.snap_dft[ps_ + e] = nu[e];
    }
  }
  if (S.nrec) {
    double* seis = S.seis_col + lane * S.seis_lane;
    for (int q = 0; q < nrec; ++q) {
      const int2 e = s_rec[q];
      const int d = e.y - l0;
      if (d >= 0 && d < 4) {
        const float xu = d == 0 ? nu[0] : d == 1 ? nu[1] : d == 2 ? nu[2] : nu[3];
        const float xv = d == 0 ? vn[0] : d == 1 ? vn[1] : d == 2 ? vn[2] : vn[3];
        seis[e.x] = (double)(S.rec_u ? xu : xv);
      }
    }
  }
}

template <int R, bool HU, bool HI, int TZ>
__global__ __launch_bounds__(Tile2<TZ, HU, HI>::NT) void k32_step2(Grid32 G, const __grid_constant__ StepMaps2 M,
                                                                    Step2 Q) {
  using T = Tile2<TZ, HU, HI>;
  constexpr int NT = T::NT, W = TB_W;
  static_assert(R <= 2, "two steps per launch need R <= 2 (orders 2 and 4)");
  extern __shared__ __align__(128) unsigned char sm_raw[];
  float* sm = reinterpret_cast<float*>(sm_raw + ((128u - (smem_u32(sm_raw) & 127u)) & 127u));
  __shared__ __align__(8) uint64_t bar[1];
  __shared__ int s_src[MAX_BOX_SRC];
  __shared__ float s_amp0[MAX_BOX_SRC], s_amp1[MAX_BOX_SRC];  // amplitudes of steps 1 and 2
  __shared__ int s_nsrc;
  __shared__ int2 s_rec[MAX_TILE_REC];
  __shared__ int s_nrec;
  const Step32& S0 = Q.s[0];
  const Step32& S1 = Q.s[1];
  const int tid = threadIdx.x;
  const int lane = blockIdx.z, x0 = blockIdx.x * TX, z0 = blockIdx.y * TZ;
  const int bx = x0 - TB_X, bz = z0 - TB_Z;
  const int64_t lo = (int64_t)lane * G.ps;
  const int t = blockIdx.x + G.ntx * (blockIdx.y + G.ntz * lane);
  const float* cf = G.c;
  const bool inj0 = HI && S0.inj_plane >= 0, inj1 = HI && S1.inj_plane >= 0;
  if (tid == 0) {
    s_nsrc = 0;
    s_nrec = 0;
    mbar_init(&bar[0], 1);
    fence_mbar_init();
    const uint32_t box = 4u * W * T::H;
    uint32_t bytes = 6u * box + (inj0 ? box : 0u) + (inj1 ? box : 0u) + (HU ? 4u * TX * TZ : 0u);
    mbar_expect_tx(&bar[0], bytes);
    // coefficients and injection planes are not written by the time loop
    tma_load_3d(sm + T::O_B, &M.b, bx, bz, lane, &bar[0]);
    tma_load_3d(sm + T::O_T, &M.taper, bx, bz, lane, &bar[0]);
    tma_load_3d(sm + T::O_MU, &M.dtmu, bx, bz, lane, &bar[0]);
    if (inj0) tma_load_3d(sm + T::O_I, &M.inj, bx, bz, S0.inj_plane * G.S + lane, &bar[0]);
    if (inj1) tma_load_3d(sm + T::O_I + T::A, &M.inj, bx, bz, S1.inj_plane * G.S + lane, &bar[0]);
    asm volatile("griddepcontrol.wait;" ::: "memory");
    tma_load_3d(sm + T::O_SXY, &M.sxy, bx, bz, lane, &bar[0]);
    tma_load_3d(sm + T::O_SZY, &M.szy, bx, bz, lane, &bar[0]);
    tma_load_3d(sm + T::O_V, &M.v, bx, bz, lane, &bar[0]);
    if (HU) tma_load_3d(sm + T::O_U, &M.u, x0, z0, lane, &bar[0]);
  }
  __syncthreads();
  if (S0.nrec && tid < 32 && S0.tile_rec) {
    const int2 se = S0.tile_rec[t];
    if (tid == 0) {
      s_nrec = se.y <= MAX_TILE_REC ? se.y : MAX_TILE_REC;
      if (se.y > MAX_TILE_REC) set_error_flag(G.err, 1);  // the host pairs steps only below this
    }
    for (int q = tid; q < se.y && q < MAX_TILE_REC; q += 32) s_rec[q] = S0.rec_ent[se.x + q];
  }
  if (tid < 32 && S0.nsrc) {
    // point sources in the box, in source order (as step_tile)
    const int2* src_xy = S0.src_xy + (int64_t)lane * S0.nsrc;
    int base = 0;
    for (int k0 = 0; k0 < S0.nsrc; k0 += 32) {
      const int k = k0 + tid;
      int2 q = make_int2(0, 0);
      bool in = false;
      if (k < S0.nsrc) {
        q = src_xy[k];
        in = q.x >= bx && q.x < bx + W && q.y >= bz && q.y < bz + T::H;
      }
      const unsigned m = __ballot_sync(0xffffffffu, in);
      const int slot = base + __popc(m & ((1u << tid) - 1u));
      if (in && slot < MAX_BOX_SRC) {
        s_src[slot] = (q.y - bz) * W + (q.x - bx);
        s_amp0[slot] = S0.amp ? (float)S0.amp[(int64_t)lane * S0.nsrc + k] : S0.amp_const;
        s_amp1[slot] = S1.amp ? (float)S1.amp[(int64_t)lane * S1.nsrc + k] : S1.amp_const;
      }
      base += __popc(m);
    }
    if (tid == 0) {
      s_nsrc = base;
      if (base > MAX_BOX_SRC) set_error_flag(G.err, 1);  // the host pairs steps only below this
    }
  }
  bool ok = true;
  if (tid < 32) ok = mbar_wait_bounded_sleep(&bar[0], 0);
  if (__syncthreads_or(!ok)) {
    if (tid == 0) {
      set_error_flag(G.err, 1);
      mbar_wait_bounded_sleep(&bar[0], 0, 100000000ull);  // let started copies land (bounded)
    }
    return;
  }
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int nbs = min(s_nsrc, MAX_BOX_SRC), nrec = s_nrec;
  float* s_sxy = sm + T::O_SXY;
  float* s_szy = sm + T::O_SZY;
  float* s_v = sm + T::O_V;
  const float* s_b = sm + T::O_B;
  const float* s_t = sm + T::O_T;
  const float* s_mu = sm + T::O_MU;
  float* s_u = sm + T::O_U;
  const float* s_i0 = inj0 ? sm + T::O_I : nullptr;
  const float* s_i1 = inj1 ? sm + T::O_I + T::A : nullptr;
  // every computed point (phase A reaches furthest) inside the operators' ranges
  const bool edge = !(x0 - 4 >= R && x0 + 40 + R <= G.nx && z0 - 4 >= R && z0 + TZ + 5 + R <= G.nz);
  auto run = [&](auto edge_tag) {
    constexpr bool EDGE = decltype(edge_tag)::value;
    constexpr int NQA = T::QA1 - T::QA0 + 1, NQB = T::QB1 - T::QB0 + 1, NQC = T::QC1 - T::QC0 + 1;
    // A: v1
    for (int it = tid; it < NQA * (T::RA1 - T::RA0 + 1); it += NT)
      tb_v_item<R, EDGE>(G, cf, s_v, s_sxy, s_szy, s_b, s_t, s_i0, T::RA0 + it / NQA, 4 * (T::QA0 + it % NQA), bx,
                         bz, s_src, s_amp0, nbs, S0.snap_pre_u ? nullptr : S0.snap_pre, TZ);
    __syncthreads();
    // B: s1 (in place: an item reads its own old stresses only); step-1 outputs on the tile
    for (int it = tid; it < NQB * (T::RB1 - T::RB0 + 1); it += NT) {
      const int r = T::RB0 + it / NQB, c0 = 4 * (T::QB0 + it % NQB);
      float nsx[4], nsz[4], vn[4];
      tb_s_item<R, EDGE>(G, cf, s_v, s_sxy, s_szy, s_mu, r, c0, bx, bz, nsx, nsz, vn);
      *reinterpret_cast<float4*>(s_sxy + r * W + c0) = make_float4(nsx[0], nsx[1], nsx[2], nsx[3]);
      *reinterpret_cast<float4*>(s_szy + r * W + c0) = make_float4(nsz[0], nsz[1], nsz[2], nsz[3]);
      const int tr = r - TB_Z, tq = c0 / 4 - TB_X / 4;  // tile row and quad
      if (tr >= 0 && tr < TZ && tq >= 0 && tq < TX / 4) {
        const int j = z0 + tr, i0 = x0 + 4 * tq;
        float nu[4];
        if (HU) {
          float* up = s_u + tr * TX + 4 * tq;
          if (S0.snap_pre && S0.snap_pre_u) {
            // single(u) before step 1 (mode != 0 snapshots)
#pragma unroll
            for (int e = 0; e < 4; ++e)
              if (!EDGE || (i0 + e < G.nx && j < G.nz)) S0.snap_pre[i0 + e + (int64_t)G.nx * j] = up[e];
          }
#pragma unroll
          for (int e = 0; e < 4; ++e) nu[e] = __fmaf_rn(vn[e], G.dt, up[e]);
          *reinterpret_cast<float4*>(up) = make_float4(nu[0], nu[1], nu[2], nu[3]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e) nu[e] = vn[e];
        }
        if (!EDGE || (j < G.nz && i0 < G.nx))
          tb_outputs(G, S0, EDGE, lane, lo, i0, j, tr * TX + 4 * tq, nu, vn, s_rec, nrec);
      }
    }
    __syncthreads();
    // C: v2
    for (int it = tid; it < NQC * (T::RC1 - T::RC0 + 1); it += NT)
      tb_v_item<R, EDGE>(G, cf, s_v, s_sxy, s_szy, s_b, s_t, s_i1, T::RC0 + it / NQC, 4 * (T::QC0 + it % NQC), bx,
                         bz, s_src, s_amp1, nbs, S1.snap_pre_u ? nullptr : S1.snap_pre, TZ);
    __syncthreads();
    // D: s2, u2 and the stores of the tile
    for (int it = tid; it < (TX / 4) * TZ; it += NT) {
      const int tq = it % (TX / 4), tr = it / (TX / 4);
      const int j = z0 + tr, i0 = x0 + 4 * tq;
      if (EDGE && (j >= G.nz || i0 >= G.nx)) continue;
      const int r = tr + TB_Z, c0 = 4 * tq + TB_X;
      float nsx[4], nsz[4], vn[4], nu[4];
      tb_s_item<R, EDGE>(G, cf, s_v, s_sxy, s_szy, s_mu, r, c0, bx, bz, nsx, nsz, vn);
      if (HU) {
        const float* up = s_u + tr * TX + 4 * tq;
        if (S1.snap_pre && S1.snap_pre_u) {
          // single(u) before step 2
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (!EDGE || i0 + e < G.nx) S1.snap_pre[i0 + e + (int64_t)G.nx * j] = up[e];
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) nu[e] = __fmaf_rn(vn[e], G.dt, up[e]);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) nu[e] = vn[e];
      }
      const int64_t p = lo + i0 + (int64_t)G.P * j;
      if (!EDGE || i0 + 3 < G.nx) {
        *reinterpret_cast<float4*>(S1.vo + p) = make_float4(vn[0], vn[1], vn[2], vn[3]);
        if (!EDGE || i0 + 3 <= G.nx - 2) {
          *reinterpret_cast<float4*>(S1.sxyo + p) = make_float4(nsx[0], nsx[1], nsx[2], nsx[3]);
        } else {
#pragma unroll
          for (int e = 0; e < 4; ++e)
            if (i0 + e <= G.nx - 2) S1.sxyo[p + e] = nsx[e];
        }
        if (!EDGE || j <= G.nz - 2) *reinterpret_cast<float4*>(S1.szyo + p) = make_float4(nsz[0], nsz[1], nsz[2], nsz[3]);
        if (HU) *reinterpret_cast<float4*>(S1.uo + p) = make_float4(nu[0], nu[1], nu[2], nu[3]);
      } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          if (i0 + e >= G.nx) break;
          S1.vo[p + e] = vn[e];
          if (i0 + e <= G.nx - 2) S1.sxyo[p + e] = nsx[e];
          if (j <= G.nz - 2) S1.szyo[p + e] = nsz[e];
          if (HU) S1.uo[p + e] = nu[e];
        }
      }
      tb_outputs(G, S1, EDGE, lane, lo, i0, j, tr * TX + 4 * tq, nu, vn, s_rec, nrec);
    }
  };
  if (edge)
    run(std::true_type{});
  else
    run(std::false_type{});
}

// ---- multi-geometry step -----------------------------------------------------------
// Solves on grids of different sizes (the reference stations of a batch, one
// configuration each) advance together, one launch per time step.  Their
// fields are stacked in tall arrays of a common row pitch: solve i occupies
// rows [row0, row0 + nz) with rows of zeros above and below it and zeros past
// its nx columns, so one set of tensor maps serves every solve and a halo box
// reads zeros outside each grid, as the tensor-map fill does for one grid.
// DFT snapshots and injection planes stay compact per solve (pitch P).
struct Seg {
  int nx, nz, P, ntx, ntz;  // grid, compact row pitch, tiles
  int row0;                 // first row in the stacked field arrays
  int tile0;                // first CTA of the solve in a launch
  int nt;                   // forward steps (DFT schedule of the Green run)
  int dft_T;                // snapshots per DFT chunk
  int inj_chunk;            // injection planes per chunk
  int nsrc, nrec;
  int t1[4];                // all-ones taper tile rectangle
  float inv_dx, inv_dz, dt;
  int64_t ps;               // compact plane stride
  float* snaps;             // DFT snapshot chunk
  const float* inj;         // resident injection planes
  const int2 *src_xy, *rec_xy, *tile_rec, *rec_ent;
  double* seis;             // nrec-by-steps seismograms
};

constexpr int MULTI_MAX_SEG = 64;  // solves of one multi-geometry loop

struct MultiStep {
  int n;         // time step (1-based)
  int n_seg;     // solves active at this step (a prefix of the table)
  int tile0[MULTI_MAX_SEG];  // first CTA of each solve (the parameter bank serves the search)
  int fs;        // DFT / injection decimation
  int green;     // 1: Green run (point force, DFT of v), 0: correlation run
  int Pf;        // row pitch of the stacked field arrays
  float c[4];    // FD weights
  const Seg* segs;
  float *vo, *sxyo, *szyo, *uo;  // stacked fields written this step
  int* err;
};

template <int R, bool HU, bool HI, int TZ>
__global__ __launch_bounds__(Tile<R, HU, HI, TZ>::NT, Tile<R, HU, HI, TZ>::MINB) void k32_step_multi(
    MultiStep Q, const __grid_constant__ StepMaps M) {
  __shared__ Grid32 s_G;
  __shared__ Step32 s_S;
  __shared__ TileLoc s_L;
  if (threadIdx.x == 0) {
    // the solve of this CTA: the last one whose first CTA is at or before it
    const int b = blockIdx.x;
    int lo = 0, hi = Q.n_seg - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if (Q.tile0[mid] <= b) lo = mid;
      else hi = mid - 1;
    }
    const Seg& g = Q.segs[lo];
    Grid32 G{};
    G.nx = g.nx; G.nz = g.nz; G.P = Q.Pf; G.S = 1; G.ntx = g.ntx; G.ntz = g.ntz; G.ps = g.ps;
    for (int m = 0; m < 4; ++m) G.c[m] = Q.c[m];
    G.inv_dx = g.inv_dx; G.inv_dz = g.inv_dz; G.dt = g.dt; G.err = Q.err;
    G.t1x0 = g.t1[0]; G.t1x1 = g.t1[1]; G.t1z0 = g.t1[2]; G.t1z1 = g.t1[3];
    Step32 S{};
    S.vo = Q.vo; S.sxyo = Q.sxyo; S.szyo = Q.szyo; S.uo = Q.uo;
    S.has_u = HU;
    S.inj_plane = -1;
    const int n = Q.n;
    if (Q.green) {
      S.src_xy = g.src_xy;
      S.nsrc = g.nsrc;
      S.amp_const = 1.0e9f;  // stf = 1.0e9*ones(1,nt), code/run_forward1_green.m:64
      if ((n + g.nt - 1) % Q.fs == 0) {
        // DFT events so far, this one included: the snapshot slot of the chunk
        const int e = (n + g.nt - 1) / Q.fs - (g.nt - 1) / Q.fs;
        S.snap_dft = g.snaps + (int64_t)((e - 1) % g.dft_T) * g.ps;
      }
    } else {
      S.src_xy = g.src_xy;
      S.rec_u = 1;
      if (HI) S.inj_plane = (n / Q.fs - 1) % g.inj_chunk;
    }
    S.inj_base = g.inj;
    S.rec_xy = g.rec_xy;
    S.nrec = g.nrec;
    S.tile_rec = g.tile_rec;
    S.rec_ent = g.rec_ent;
    S.seis_col = g.seis + (int64_t)g.nrec * (n - 1);
    TileLoc L;
    L.t = b - g.tile0;
    L.tx = L.t % g.ntx;
    L.tz = L.t / g.ntx;
    L.x0 = L.tx * TX;
    L.z0 = L.tz * TZ;
    L.lane = 0;
    L.ty0 = g.row0;
    L.lo = (int64_t)g.row0 * Q.Pf;
    L.slo = 0;
    L.sp = g.P;
    s_G = G;
    s_S = S;
    s_L = L;
  }
  __syncthreads();
  // the FD weights from the parameter bank; the per-solve values from shared memory
  step_tile<R, HU, HI, TZ, true>(s_G, M, s_S, s_L, Q.c);
}

// ---- point kernels ---------------------------------------------------------------
// FP32 staggered derivatives of a field with row pitch `ld` (f, or f - g).
template <int R>
__device__ __forceinline__ float dx32(const Grid32& G, const float* f, const float* g, int ld, int i, int j) {
  if (i < R - 1 || i > G.nx - R - 1) return 0.f;
  const float* F = f + (int64_t)ld * j;
  const float* H = g ? g + (int64_t)ld * j : nullptr;
  float acc = 0.f;
#pragma unroll
  for (int m = 1; m <= R; ++m) {
    const float a = H ? F[i + m] - H[i + m] : F[i + m];
    const float b = H ? F[i - m + 1] - H[i - m + 1] : F[i - m + 1];
    acc += G.c[m - 1] * (a - b);
  }
  return acc * G.inv_dx;
}

template <int R>
__device__ __forceinline__ float dz32(const Grid32& G, const float* f, const float* g, int ld, int i, int j) {
  if (j < R - 1 || j > G.nz - R - 1) return 0.f;
  float acc = 0.f;
#pragma unroll
  for (int m = 1; m <= R; ++m) {
    const int64_t qa = i + (int64_t)ld * (j + m), qb = i + (int64_t)ld * (j - m + 1);
    const float a = g ? f[qa] - g[qa] : f[qa];
    const float b = g ? f[qb] - g[qb] : f[qb];
    acc += G.c[m - 1] * (a - b);
  }
  return acc * G.inv_dz;
}

// forward1 Born source before div_s: sxy += dt*dmu*dx_v(G_in(:,:,i)), on the read buffers
template <int R>
__global__ void k32_born_pre(Grid32 G, float* sxy, float* szy, const float* dtdmu, const float* Gs) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= G.nx || j >= G.nz) return;
  const int64_t p = i + (int64_t)G.P * j;
  const float dm = dtdmu[p];
  if (i <= G.nx - 2) sxy[p] += dm * dx32<R>(G, Gs, nullptr, G.nx, i, j);
  if (j <= G.nz - 2) szy[p] += dm * dz32<R>(G, Gs, nullptr, G.nx, i, j);
}

// correlation / adjoint Born term after the stress update: -= dmu*dx_v(C(n) - C(n+1))
template <int R>
__global__ void k32_born_post(Grid32 G, float* sxy, float* szy, const float* dmu, const float* Ca, const float* Cb) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= G.nx || j >= G.nz) return;
  const int64_t p = i + (int64_t)G.P * j;
  if (i <= G.nx - 2) sxy[p] -= dmu[p] * dx32<R>(G, Ca, Cb, G.nx, i, j);
  if (j <= G.nz - 2) szy[p] -= dmu[p] * dz32<R>(G, Ca, Cb, G.nx, i, j);
}

// K_mu -= dx_v(u).*dx_v(u_fwd)*fw ; K_mu -= dz_v(u).*dz_v(u_fwd)*fw   (FP32 strains, FP64 sum)
template <int R>
__global__ void k32_kmu(Grid32 G, const float* u, const float* uf, double* Kmu, float fw) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= G.nx || j >= G.nz) return;
  const int64_t p = i + (int64_t)G.nx * j;
  double k = Kmu[p];
  if (i <= G.nx - 2) k -= (double)(dx32<R>(G, u, nullptr, G.P, i, j) * dx32<R>(G, uf, nullptr, G.nx, i, j) * fw);
  if (j <= G.nz - 2) k -= (double)(dz32<R>(G, u, nullptr, G.P, i, j) * dz32<R>(G, uf, nullptr, G.nx, i, j) * fw);
  Kmu[p] = k;
}

// dt/rho, taper, dt*mu into pitched FP32 arrays (zero in the pitch padding).
__global__ void k32_prep(const double* mu, const double* rho, const double* ab, double dt, int nx, int nz, int P,
                         float* b, float* taper, float* dtmu) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= P || j >= nz) return;
  const int64_t q = i + (int64_t)P * j;
  if (i >= nx) {
    b[q] = taper[q] = dtmu[q] = 0.f;
    return;
  }
  const int64_t p = i + (int64_t)nx * j;
  b[q] = (float)(dt / rho[p]);
  taper[q] = (float)ab[p];
  dtmu[q] = (float)(dt * mu[p]);
}

// FP32 copy of an FP64 MATLAB-layout array into a pitched array, scaled.
__global__ void k32_pitched(const double* a, double s, int nx, int nz, int P, float* out) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= P || j >= nz) return;
  out[i + (int64_t)P * j] = i < nx ? (float)(s * a[i + (int64_t)nx * j]) : 0.f;
}

// Band weights of the field source: W(k,b) = spec(k) * M(k,b), FP32 (K x ncol).
__global__ void k32_band_weights(int K, int ncol, const double* M, const double* spec, float* W) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K * ncol) return;
  const int k = e % K;
  W[e] = narrow_rn(spec[k] * M[e]);
}

// P planes of the field source: P_k = (sum_b W(k,b) sd_b) * (Xre_k + i*sign*Xim_k)
// as 2K pitched float planes [Re P_0..Re P_{K-1}, Im P_0..Im P_{K-1}], plane
// stride ps.  FP32 arithmetic on narrowed inputs (the planes are FP32 anyway):
// the FP64 pipe of this part would otherwise bound the kernel.
__global__ void k32_make_P(int K, int ncol, const float* __restrict__ W, const double* __restrict__ sd,
                           const double* __restrict__ Xre, const double* __restrict__ Xim, float sign, int nx,
                           int nz, int P, int64_t ps, float* __restrict__ Pl) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= P || j >= nz) return;
  const int64_t q = i + (int64_t)P * j;
  if (i >= nx) {
    for (int k = 0; k < 2 * K; ++k) Pl[q + ps * k] = 0.f;
    return;
  }
  const int64_t np = (int64_t)nx * nz, p = i + (int64_t)nx * j;
  float sdv[8];
  for (int b = 0; b < ncol && b < 8; ++b) sdv[b] = narrow_rn(sd[p + np * b]);
  // groups of 4 frequencies: all 8 spectrum loads are issued before any store
  constexpr int G = 4;
  for (int k0 = 0; k0 < K; k0 += G) {
    double xr[G], xi[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int k = k0 + g;
      xr[g] = k < K ? Xre[p + np * k] : 0.0;
      xi[g] = (k < K && Xim) ? Xim[p + np * k] : 0.0;
    }
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int k = k0 + g;
      if (k >= K) break;
      float dist = 0.f;
      for (int b = 0; b < ncol; ++b)
        dist += W[k + (int64_t)K * b] * (b < 8 ? sdv[b] : narrow_rn(sd[p + np * b]));
      Pl[q + ps * k] = dist * narrow_rn(xr[g]);
      Pl[q + ps * (K + k)] = dist * (sign * narrow_rn(xi[g]));
    }
  }
}

// K_s(:,:,b) = (dw/dt) sum_k M(k,b) spec(k) (G_re U_re - G_im U_im), U = sum_n u_n e^{-iwt}dt/sqrt(2pi)
__global__ void k32_source_kernel(int K, int ncol, const double* M, const double* spec,
                                  const double* Gre, const double* Gim, const double* Ure,
                                  const double* Uim, double scale, double* Ks, int64_t np) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= np) return;
  for (int b = 0; b < ncol; ++b) {
    double acc = 0.0;
    for (int k = 0; k < K; ++k) {
      const int64_t q = p + np * k;
      acc += M[k + (int64_t)K * b] * spec[k] * (Gre[q] * Ure[q] - Gim[q] * Uim[q]);
    }
    Ks[p + np * b] = scale * acc;
  }
}

// ---- host side ---------------------------------------------------------------------
struct Run {
  Grid32 G{};
  float *b = nullptr, *taper = nullptr, *dtmu = nullptr;
  float *v[2] = {}, *sxy[2] = {}, *szy[2] = {}, *u[2] = {};
  StepMaps maps[2];  // read buffers 0 / 1
  dim3 sgrid, pgrid, pblock{32, 8};
  int R = 2;
  int tz = 32;  // tile rows of the step kernel (TILE_ROWS)
  // Programmatic dependent launch of the steps: on when the solve has the GPU
  // to itself.  Beside other work (lane groups of a batch in parallel graph
  // branches, serving slots) an early-launched step would park CTAs that wait
  // for their predecessor in SM slots the other solves could use.
  bool pdl = true;
  int t1[N_TILE_ROWS][4] = {};  // per tile shape: all-ones taper tile range (Grid32::t1x0..)
  const float* inj_planes = nullptr;  // injection planes (set_inj_map)
  int inj_n_planes = 0;
  int2* rec_xy = nullptr;
  int2* src_xy = nullptr;
  int2* tile_rec = nullptr;  // per (lane, tile): {first entry, count}
  int2* rec_ent = nullptr;   // {receiver k, offset in the tile}
  int64_t np = 0;   // nx*nz
  int64_t ps = 0;   // pitched plane size P*nz rounded up to 128
  int S = 1;        // lanes; every internal array holds S planes (lane l at l*ps)
  int64_t lanes_ps() const { return (int64_t)S * ps; }
  // two steps per launch (k32_step2): chosen by tune_time_depth; maps2 valid when depth == 2
  int depth = 1;
  int max_tile_rec = 0;  // most receivers of one (lane, tile)
  StepMaps2 maps2[2];
};

// Step launches carry the programmatic-stream-serialization attribute: a step
// may be scheduled while the previous one drains; k32_step waits for it with
// griddepcontrol.wait before touching the fields.
template <int R, bool HU, bool HI, int TZ>
void launch_step_t(fd2d_ctx* ctx, const Run& r, int par, const Step32& s) {
  using T = Tile<R, HU, HI, TZ>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = r.sgrid;
  cfg.blockDim = dim3(T::NT);
  cfg.dynamicSmemBytes = T::BYTES;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = r.pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k32_step<R, HU, HI, TZ>, r.G, r.maps[par], s);
}

template <int R, bool HU, bool HI>
void launch_step_v(fd2d_ctx* ctx, const Run& r, int par, const Step32& s) {
  if (r.tz == 16) launch_step_t<R, HU, HI, 16>(ctx, r, par, s);
  else if (r.tz == 30) launch_step_t<R, HU, HI, 30>(ctx, r, par, s);
  else if (r.tz == 40) launch_step_t<R, HU, HI, 40>(ctx, r, par, s);
  else launch_step_t<R, HU, HI, 32>(ctx, r, par, s);
}

template <int R>
void launch_step_r(fd2d_ctx* ctx, const Run& r, int par, const Step32& s) {
  const bool hi = s.inj_plane >= 0;
  if (s.has_u) {
    if (hi) launch_step_v<R, true, true>(ctx, r, par, s);
    else launch_step_v<R, true, false>(ctx, r, par, s);
  } else {
    if (hi) launch_step_v<R, false, true>(ctx, r, par, s);
    else launch_step_v<R, false, false>(ctx, r, par, s);
  }
}

template <int R, int TZ>
fd2d_status step_attributes_t(fd2d_ctx* ctx) {
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step<R, false, false, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, false, false, TZ>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step<R, false, true, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, false, true, TZ>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step<R, true, false, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, true, false, TZ>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step<R, true, true, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, true, true, TZ>::BYTES));
  return FD2D_OK;
}

template <int R>
fd2d_status step_attributes_r(fd2d_ctx* ctx) {
  FD2D_TRY((step_attributes_t<R, 16>(ctx)));
  FD2D_TRY((step_attributes_t<R, 30>(ctx)));
  FD2D_TRY((step_attributes_t<R, 40>(ctx)));
  return step_attributes_t<R, 32>(ctx);
}

template <int R, int TZ>
fd2d_status step2_attributes_t(fd2d_ctx* ctx) {
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step2<R, false, false, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile2<TZ, false, false>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step2<R, false, true, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile2<TZ, false, true>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step2<R, true, false, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile2<TZ, true, false>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step2<R, true, true, TZ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile2<TZ, true, true>::BYTES));
  return FD2D_OK;
}

template <int R>
fd2d_status step2_attributes_r(fd2d_ctx* ctx) {
  FD2D_TRY((step2_attributes_t<R, 16>(ctx)));
  FD2D_TRY((step2_attributes_t<R, 30>(ctx)));
  FD2D_TRY((step2_attributes_t<R, 40>(ctx)));
  return step2_attributes_t<R, 32>(ctx);
}

// Opt the step kernels in to their dynamic shared memory (once per device,
// before any capture on it).
PerDeviceOnce g_step_attributes;
fd2d_status step_attributes(fd2d_ctx* ctx) {
  return g_step_attributes.run(ctx, [ctx]() -> fd2d_status {
    FD2D_TRY(step_attributes_r<1>(ctx));
    FD2D_TRY(step_attributes_r<2>(ctx));
    FD2D_TRY(step_attributes_r<3>(ctx));
    FD2D_TRY(step_attributes_r<4>(ctx));
    FD2D_TRY(step2_attributes_r<1>(ctx));
    return step2_attributes_r<2>(ctx);
  });
}

fd2d_status launch_step(fd2d_ctx* ctx, const Run& r, int par, Step32 s) {
  s.inj_base = r.inj_planes;
  s.tile_rec = r.tile_rec;
  s.rec_ent = r.rec_ent;
  s.vo = r.v[1 - par];
  s.sxyo = r.sxy[1 - par];
  s.szyo = r.szy[1 - par];
  s.uo = r.u[1 - par];
  switch (r.R) {
    case 1: launch_step_r<1>(ctx, r, par, s); break;
    case 2: launch_step_r<2>(ctx, r, par, s); break;
    case 3: launch_step_r<3>(ctx, r, par, s); break;
    default: launch_step_r<4>(ctx, r, par, s); break;
  }
  return after_launch(ctx, "k32_step");
}

template <int R, bool HU, bool HI, int TZ>
void launch_step2_t(fd2d_ctx* ctx, const Run& r, int par, const Step2& q) {
  using T = Tile2<TZ, HU, HI>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = r.sgrid;
  cfg.blockDim = dim3(T::NT);
  cfg.dynamicSmemBytes = T::BYTES;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = r.pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k32_step2<R, HU, HI, TZ>, r.G, r.maps2[par], q);
}

template <int R, bool HU, bool HI>
void launch_step2_v(fd2d_ctx* ctx, const Run& r, int par, const Step2& q) {
  if (r.tz == 16) launch_step2_t<R, HU, HI, 16>(ctx, r, par, q);
  else if (r.tz == 30) launch_step2_t<R, HU, HI, 30>(ctx, r, par, q);
  else if (r.tz == 40) launch_step2_t<R, HU, HI, 40>(ctx, r, par, q);
  else launch_step2_t<R, HU, HI, 32>(ctx, r, par, q);
}

template <int R>
void launch_step2_r(fd2d_ctx* ctx, const Run& r, int par, const Step2& q) {
  const bool hi = q.s[0].inj_plane >= 0 || q.s[1].inj_plane >= 0;
  if (q.s[0].has_u) {
    if (hi) launch_step2_v<R, true, true>(ctx, r, par, q);
    else launch_step2_v<R, true, false>(ctx, r, par, q);
  } else {
    if (hi) launch_step2_v<R, false, true>(ctx, r, par, q);
    else launch_step2_v<R, false, false>(ctx, r, par, q);
  }
}

// Steps n and n+1 (s0, s1) in one launch: the fields of read buffer `par` are
// advanced twice and written to buffer 1 - par.
fd2d_status launch_step2(fd2d_ctx* ctx, const Run& r, int par, Step32 s0, Step32 s1) {
  if (r.R > 2 || r.depth != 2 || s0.nsrc != s1.nsrc || s0.src_xy != s1.src_xy ||
      (s0.snap_pre && s0.snap_pre_u != s0.has_u) || (s1.snap_pre && s1.snap_pre_u != s1.has_u))
    return set_error(ctx, FD2D_ERR_UNSUPPORTED, "two-step launch of an unsupported step");
  Step2 q;
  for (int k = 0; k < 2; ++k) {
    Step32& s = k ? s1 : s0;
    s.inj_base = r.inj_planes;
    s.tile_rec = r.tile_rec;
    s.rec_ent = r.rec_ent;
    s.vo = r.v[1 - par];
    s.sxyo = r.sxy[1 - par];
    s.szyo = r.szy[1 - par];
    s.uo = r.u[1 - par];
    q.s[k] = s;
  }
  if (r.R == 1) launch_step2_r<1>(ctx, r, par, q);
  else launch_step2_r<2>(ctx, r, par, q);
  return after_launch(ctx, "k32_step2");
}

#define FD2D_DISPATCH_R(R_, KERNEL, ...)                                                 \
  switch (R_) {                                                                          \
    case 1: KERNEL<1><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;        \
    case 2: KERNEL<2><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;        \
    case 3: KERNEL<3><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;        \
    default: KERNEL<4><<<r.pgrid, r.pblock, 0, ctx->stream>>>(__VA_ARGS__); break;       \
  }

fd2d_status make_maps(fd2d_ctx* ctx, Run& r) {
  const int nx = r.G.nx, nz = r.G.nz, P = r.G.P, R = r.R, TZ = r.tz;
  const int BH = TZ + 2 * R - 1, SZH = TZ + 4 * R - 2, BWa = TX + 8, SXWa = TX + 16;
  // the two parts of the field boxes (Tile::H1, Tile::H1Z)
  const int NT = std::min(TX / 4 * TZ, 256);
  const int H1 = split_top_rows(NT, BWa / 4, BH), H1Z = split_top_szy(H1, R, SZH);
  for (int q = 0; q < 2; ++q) {
    StepMaps& m = r.maps[q];
    // lanes are the third dimension (plane stride ps)
    const int S = r.S;
    const int64_t ps = r.ps;
    FD2D_TRY(make_tmap_f32(ctx, &m.sxy_t, r.sxy[q], nx, nz, P, SXWa, H1, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.sxy_b, r.sxy[q], nx, nz, P, SXWa, BH - H1, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.szy_t, r.szy[q], nx, nz, P, BWa, H1Z, S, ps));
    // (no bottom szy part when the top part holds every row; the map is then unused)
    FD2D_TRY(make_tmap_f32(ctx, &m.szy_b, r.szy[q], nx, nz, P, BWa, std::max(SZH - H1Z, 1), S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.v_t, r.v[q], nx, nz, P, BWa, H1, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.v_b, r.v[q], nx, nz, P, BWa, BH - H1, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.u, r.u[q] ? r.u[q] : r.v[q], nx, nz, P, TX, TZ, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.b, r.b, nx, nz, P, BWa, BH, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.taper, r.taper, nx, nz, P, BWa, BH, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.dtmu, r.dtmu, nx, nz, P, TX, TZ, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.inj, r.b, nx, nz, P, BWa, BH));  // replaced when planes exist
  }
  return FD2D_OK;
}

// Injection planes are [event][lane] planes of stride ps: lane l of event j is plane j*S + l.
// Tensor maps of the two-step kernel: one box (TB_W x TZ+12) for every array, u
// by tile.
fd2d_status make_maps2(fd2d_ctx* ctx, Run& r) {
  const int nx = r.G.nx, nz = r.G.nz, P = r.G.P, H = r.tz + 2 * TB_Z, S = r.S;
  const int64_t ps = r.ps;
  for (int q = 0; q < 2; ++q) {
    StepMaps2& m = r.maps2[q];
    FD2D_TRY(make_tmap_f32(ctx, &m.sxy, r.sxy[q], nx, nz, P, TB_W, H, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.szy, r.szy[q], nx, nz, P, TB_W, H, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.v, r.v[q], nx, nz, P, TB_W, H, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.u, r.u[q] ? r.u[q] : r.v[q], nx, nz, P, TX, r.tz, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.b, r.b, nx, nz, P, TB_W, H, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.taper, r.taper, nx, nz, P, TB_W, H, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.dtmu, r.dtmu, nx, nz, P, TB_W, H, S, ps));
    FD2D_TRY(make_tmap_f32(ctx, &m.inj, r.inj_planes ? r.inj_planes : r.b, nx, nz, P, TB_W, H,
                           r.inj_planes ? r.inj_n_planes : S, ps));
  }
  return FD2D_OK;
}

fd2d_status set_inj_map(fd2d_ctx* ctx, Run& r, const float* planes, int n_planes) {
  const int BH = r.tz + 2 * r.R - 1, BWa = TX + 8;
  r.inj_planes = planes;
  r.inj_n_planes = n_planes;
  for (int q = 0; q < 2; ++q)
    FD2D_TRY(make_tmap_f32(ctx, &r.maps[q].inj, planes, r.G.nx, r.G.nz, r.G.P, BWa, BH, n_planes, r.ps));
  if (r.depth == 2)
    for (int q = 0; q < 2; ++q)
      FD2D_TRY(make_tmap_f32(ctx, &r.maps2[q].inj, planes, r.G.nx, r.G.nz, r.G.P, TB_W, r.tz + 2 * TB_Z, n_planes,
                             r.ps));
  return FD2D_OK;
}

// CSR of receivers by (lane, tile) of the step grid: table[(l*ntz + tz)*ntx + tx]
// = {first, count} into ent = {k, (z - tz*TZ)*TX + (x - tx*TX)}; TZ = tile rows.
void build_tile_receivers_idx(int nx, int nz, int TZ, const std::vector<const std::vector<int>*>& lanes,
                              std::vector<int2>& table, std::vector<int2>& ent) {
  const int ntx = (nx + TX - 1) / TX, ntz = (nz + TZ - 1) / TZ;
  const int S = (int)lanes.size();
  table.assign((size_t)S * ntx * ntz, make_int2(0, 0));
  std::vector<std::vector<int2>> per(table.size());
  for (int l = 0; l < S; ++l) {
    const std::vector<int>& rec = *lanes[l];
    for (int k = 0; k < (int)rec.size(); ++k) {
      const int x = rec[k] % nx, z = rec[k] / nx;
      const int tx = x / TX, tz = z / TZ;
      per[((size_t)l * ntz + tz) * ntx + tx].push_back(make_int2(k, (z - tz * TZ) * TX + (x - tx * TX)));
    }
  }
  ent.clear();
  for (size_t t = 0; t < per.size(); ++t) {
    table[t] = make_int2((int)ent.size(), (int)per[t].size());
    ent.insert(ent.end(), per[t].begin(), per[t].end());
  }
  if (ent.empty()) ent.push_back(make_int2(0, 0));
}

void build_tile_receivers(int nx, int nz, int TZ, const SolveArgs* a, int S, std::vector<int2>& table,
                          std::vector<int2>& ent) {
  std::vector<const std::vector<int>*> lanes;
  for (int l = 0; l < S; ++l) lanes.push_back(&a[l].rec_idx);
  build_tile_receivers_idx(nx, nz, TZ, lanes, table, ent);
}

// Per tile shape, the range of tiles whose halo box (the 40-wide, BH-row box
// of the dt/rho and taper loads) lies inside the grid with an FP32 taper of
// exactly 1; the taper is separable, so these tiles form a rectangle (an empty
// range if not).
void taper_ones(const std::vector<double>& ab, int nx, int nz, int R, int out[N_TILE_ROWS][4]) {
  const size_t W = (size_t)nx + 1;
  std::vector<int> pre(W * (nz + 1), 0);  // prefix counts of taper != 1
  for (int j = 0; j < nz; ++j)
    for (int i = 0; i < nx; ++i)
      pre[(j + 1) * W + i + 1] = ((float)ab[i + (size_t)nx * j] != 1.0f) + pre[j * W + i + 1] +
                                 pre[(j + 1) * W + i] - pre[j * W + i];
  auto bad = [&](int x0, int x1, int z0, int z1) {  // inclusive ranges
    return pre[(z1 + 1) * W + x1 + 1] - pre[z0 * W + x1 + 1] - pre[(z1 + 1) * W + x0] + pre[z0 * W + x0];
  };
  for (int c = 0; c < N_TILE_ROWS; ++c) {
    const int tz = TILE_ROWS[c], BH = tz + 2 * R - 1;
    const int ntx = (nx + TX - 1) / TX, ntz = (nz + tz - 1) / tz;
    std::vector<char> one((size_t)ntx * ntz, 0);
    int bx0 = ntx, bx1 = -1, bz0 = ntz, bz1 = -1;
    for (int b = 0; b < ntz; ++b)
      for (int a = 0; a < ntx; ++a) {
        const int x0 = a * TX - 4, x1 = a * TX + TX + 3, z0 = b * tz - R + 1, z1 = z0 + BH - 1;
        if (x0 < 0 || x1 > nx - 1 || z0 < 0 || z1 > nz - 1 || bad(x0, x1, z0, z1)) continue;
        one[(size_t)b * ntx + a] = 1;
        bx0 = std::min(bx0, a); bx1 = std::max(bx1, a);
        bz0 = std::min(bz0, b); bz1 = std::max(bz1, b);
      }
    bool rect = bx1 >= bx0;
    for (int b = bz0; rect && b <= bz1; ++b)
      for (int a = bx0; rect && a <= bx1; ++a) rect = one[(size_t)b * ntx + a];
    const int e[4] = {1, 0, 1, 0};
    const int f[4] = {bx0, bx1, bz0, bz1};
    for (int k = 0; k < 4; ++k) out[c][k] = rect ? f[k] : e[k];
  }
}

// Step grid and tensor maps of the run's tile rows r.tz.
fd2d_status set_tiling(fd2d_ctx* ctx, Run& r) {
  r.G.ntx = (r.G.nx + TX - 1) / TX;
  r.G.ntz = (r.G.nz + r.tz - 1) / r.tz;
  r.sgrid = dim3(r.G.ntx, r.G.ntz, r.S);
  for (int c = 0; c < N_TILE_ROWS; ++c)
    if (TILE_ROWS[c] == r.tz) {
      r.G.t1x0 = r.t1[c][0]; r.G.t1x1 = r.t1[c][1]; r.G.t1z0 = r.t1[c][2]; r.G.t1z1 = r.t1[c][3];
    }
  return make_maps(ctx, r);
}

// Resident CTAs per SM of the (largest, displacement) step kernel with TZ rows.
template <int R, int TZ>
int step_ctas_t() {
  using T = Tile<R, true, false, TZ>;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k32_step<R, true, false, TZ>, T::NT, T::BYTES) != cudaSuccess) {
    cudaGetLastError();
    n = 1;
  }
  return std::max(n, 1);
}

template <int R>
int step_ctas_r(int tz) {
  return tz == 16 ? step_ctas_t<R, 16>() : tz == 30 ? step_ctas_t<R, 30>()
                  : tz == 40 ? step_ctas_t<R, 40>() : step_ctas_t<R, 32>();
}

int step_ctas(int R, int tz) {
  switch (R) {
    case 1: return step_ctas_r<1>(tz);
    case 2: return step_ctas_r<2>(tz);
    case 3: return step_ctas_r<3>(tz);
    default: return step_ctas_r<4>(tz);
  }
}

// Tile rows of the step kernel for this grid and lane count (TILE_ROWS).
// Forced by fd2d_ctx_set_tile_rows (or FD2D_TILE_ROWS).  Otherwise, when the
// context's stream is idle and no other lane group of a batch runs beside this
// one, every shape is timed once per context on this run's freshly zeroed
// fields -- 24 steps of the run's kind (with or without the displacement u)
// with no sources, receivers or snapshots, in three rounds of which the
// fastest counts -- and the fastest shape is kept for later runs of the same
// grid, order, lane count and kind if it beats the size rule's shape by more
// than 3 % (plain timed steps differ from real loops, with sources,
// receivers, snapshots and kernel terms, by about that much).  When timing
// would stall queued or concurrent work, or during a stream capture, the size
// rule decides: the fewest waves of CTAs (tiles over resident CTAs per SM x
// SMs), the shortest tiles among equals.  The step time is set by the waves: on
// GB300 a 600x600 Green step takes ~5.5 us for any tile count up to one wave
// and ~7.7 us just past it.
fd2d_status tune_tile_rows(fd2d_ctx* ctx, Run& r) {
  int forced = ctx->tile_rows;
  if (forced == FD2D_TILE_ROWS_AUTO) {
    const char* e = std::getenv("FD2D_TILE_ROWS");
    if (e) forced = std::atoi(e);
  }
  for (int tz : TILE_ROWS)
    if (forced == tz) {
      r.tz = forced;
      return FD2D_OK;
    }
  const bool with_u = r.u[0] != nullptr;
  Sig key;
  key.add(r.G.nx); key.add(r.G.nz); key.add(r.R); key.add(r.S); key.add((int)with_u);
  auto it = ctx->tile_choice.find(key.h);
  if (it != ctx->tile_choice.end()) {
    r.tz = it->second;
    return FD2D_OK;
  }
  int rule = TILE_ROWS[0];
  int64_t rule_waves = -1;
  for (int tz : TILE_ROWS) {
    const int64_t tiles = (int64_t)((r.G.nx + TX - 1) / TX) * ((r.G.nz + tz - 1) / tz) * r.S;
    const int64_t slots = (int64_t)step_ctas(r.R, tz) * std::max(ctx->sm_count, 1);
    const int64_t waves = (tiles + slots - 1) / slots;
    if (rule_waves < 0 || waves < rule_waves) {
      rule = tz;
      rule_waves = waves;
    }
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FD2D_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cs));
  bool idle = cs == cudaStreamCaptureStatusNone && ctx->concurrent_groups <= 1 && !ctx->shared_gpu &&
              forced != FD2D_TILE_ROWS_RULE;
  if (idle) {
    idle = cudaStreamQuery(ctx->stream) == cudaSuccess;
    cudaGetLastError();  // a busy stream answers cudaErrorNotReady
  }
  if (!idle) {
    r.tz = rule;
    return FD2D_OK;
  }
  // ROUNDS rounds over the shapes, the fastest round of each shape counts
  // (timings of a few microseconds per step vary from round to round)
  constexpr int WARM = 3, TIMED = 24, ROUNDS = 3;
  cudaEvent_t e0, e1;
  FD2D_CUDA(ctx, cudaEventCreate(&e0));
  FD2D_CUDA(ctx, cudaEventCreate(&e1));
  float ms_of[N_TILE_ROWS] = {};
  fd2d_status st = FD2D_OK;
  for (int round = 0; round < ROUNDS && st == FD2D_OK; ++round)
    for (int c = 0; c < N_TILE_ROWS; ++c) {
      r.tz = TILE_ROWS[c];
      if ((st = set_tiling(ctx, r)) != FD2D_OK) break;
      Step32 s{};
      s.inj_plane = -1;
      s.has_u = with_u;
      s.src_xy = r.src_xy;
      s.rec_xy = r.rec_xy;
      for (int n = 0; n < WARM && st == FD2D_OK; ++n) st = launch_step(ctx, r, n & 1, s);
      cudaEventRecord(e0, ctx->stream);
      for (int n = 0; n < TIMED && st == FD2D_OK; ++n) st = launch_step(ctx, r, n & 1, s);
      cudaEventRecord(e1, ctx->stream);
      if (st != FD2D_OK) break;
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        st = set_error(ctx, FD2D_ERR_CUDA, "tile-row timing failed");
        break;
      }
      ms_of[c] = round == 0 ? ms : std::min(ms_of[c], ms);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != FD2D_OK) return st;
  // the timed steps ran on the zeroed fields: zero them again
  const size_t bytes = (size_t)r.lanes_ps() * 4;
  for (int q = 0; q < 2; ++q) {
    FD2D_CUDA(ctx, cudaMemsetAsync(r.v[q], 0, bytes, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.sxy[q], 0, bytes, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.szy[q], 0, bytes, ctx->stream));
    if (with_u) FD2D_CUDA(ctx, cudaMemsetAsync(r.u[q], 0, bytes, ctx->stream));
  }
  int best = 0, ri = 0;
  for (int c = 0; c < N_TILE_ROWS; ++c) {
    if (ms_of[c] < ms_of[best]) best = c;
    if (TILE_ROWS[c] == rule) ri = c;
  }
  r.tz = ms_of[best] < 0.97f * ms_of[ri] ? TILE_ROWS[best] : rule;
  ctx->tile_choice[key.h] = r.tz;
  return FD2D_OK;
}

// Buffers, coefficient planes and tensor maps of S lanes a[0..S-1] (solves of
// one geometry with the same numbers of sources and receivers).
fd2d_status tune_time_depth(fd2d_ctx* ctx, Run& r, int nsrc, const int* crowded);

// two_step: the loop may advance two steps per launch (tune_time_depth decides)
fd2d_status init_run(fd2d_ctx* ctx, const Geometry& g, const SolveArgs* a, int S, bool with_u, Run& r,
                     bool two_step = false) {
  const int nx = g.nx, nz = g.nz;
  const int P = (nx + 31) / 32 * 32;
  for (int l = 1; l < S; ++l)
    if (a[l].src_idx.size() != a[0].src_idx.size() || a[l].rec_idx.size() != a[0].rec_idx.size())
      return set_error(ctx, FD2D_ERR_SHAPE, "lanes of one launch need equal source and receiver counts");
  r.S = S;
  r.np = g.npts();
  r.ps = ((int64_t)P * nz + 127) / 128 * 128;
  r.R = g.r;
  r.G.nx = nx;
  r.G.nz = nz;
  r.G.P = P;
  r.G.S = S;
  r.G.ps = r.ps;
  for (int m = 0; m < 4; ++m) r.G.c[m] = (float)g.c[m];
  r.G.inv_dx = (float)(1.0 / g.dx);
  r.G.inv_dz = (float)(1.0 / g.dz);
  r.G.dt = (float)g.dt;
  r.G.err = ctx->d_err;
  r.pblock = dim3(32, 8);
  const size_t ps = (size_t)r.ps, sps = (size_t)r.lanes_ps();
  FD2D_TRY(workspace_t(ctx, "f32.b", sps, &r.b));
  FD2D_TRY(workspace_t(ctx, "f32.taper", sps, &r.taper));
  FD2D_TRY(workspace_t(ctx, "f32.dtmu", sps, &r.dtmu));
  double* ab;
  FD2D_TRY(upload_tagged<double>(ctx, "f32.absbound64", g.key, g.absbound->size(),
                                  [&](std::vector<double>& h) { h = *g.absbound; }, &ab));
  dim3 pg((P + 31) / 32, (nz + 7) / 8);
  for (int l = 0; l < S; ++l) {
    k32_prep<<<pg, r.pblock, 0, ctx->stream>>>(a[l].mu, a[l].rho, ab, g.dt, nx, nz, P, r.b + l * ps,
                                               r.taper + l * ps, r.dtmu + l * ps);
    FD2D_TRY(after_launch(ctx, "k32_prep"));
  }
  static const char* names[2][4] = {{"f32.v0", "f32.sxy0", "f32.szy0", "f32.u0"},
                                    {"f32.v1", "f32.sxy1", "f32.szy1", "f32.u1"}};
  for (int q = 0; q < 2; ++q) {
    FD2D_TRY(workspace_t(ctx, names[q][0], sps, &r.v[q]));
    FD2D_TRY(workspace_t(ctx, names[q][1], sps, &r.sxy[q]));
    FD2D_TRY(workspace_t(ctx, names[q][2], sps, &r.szy[q]));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.v[q], 0, sps * 4, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.sxy[q], 0, sps * 4, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.szy[q], 0, sps * 4, ctx->stream));
    if (with_u) {
      FD2D_TRY(workspace_t(ctx, names[q][3], sps, &r.u[q]));
      FD2D_CUDA(ctx, cudaMemsetAsync(r.u[q], 0, sps * 4, ctx->stream));
    }
  }
  // node lists of all lanes, lane after lane
  auto xy = [&](bool rec) {
    std::vector<int2> out;
    for (int l = 0; l < S; ++l)
      for (int p : rec ? a[l].rec_idx : a[l].src_idx) out.push_back(make_int2(p % nx, p / nx));
    if (out.empty()) out.push_back(make_int2(-1 << 30, -1 << 30));
    return out;
  };
  FD2D_TRY(upload(ctx, "f32.rec", xy(true), &r.rec_xy));
  FD2D_TRY(upload(ctx, "f32.src", xy(false), &r.src_xy));
  r.pgrid = dim3((nx + 31) / 32, (nz + 7) / 8);
  r.pdl = ctx->concurrent_groups <= 1 && !ctx->shared_gpu;
  taper_ones(*g.absbound, nx, nz, r.R, r.t1);
  FD2D_TRY(step_attributes(ctx));
  FD2D_TRY(contract_prepare(ctx));
  FD2D_TRY(tune_tile_rows(ctx, r));
  r.depth = 1;
  if (two_step) {
    // receivers per tile for every shape: two steps per launch keep at most
    // MAX_TILE_REC of them per tile
    int crowded[N_TILE_ROWS];
    for (int c = 0; c < N_TILE_ROWS; ++c) {
      std::vector<int2> table, ent;
      build_tile_receivers(nx, nz, TILE_ROWS[c], a, S, table, ent);
      int m = 0;
      for (const int2& e : table) m = std::max(m, e.y);
      crowded[c] = m > MAX_TILE_REC;
    }
    FD2D_TRY(tune_time_depth(ctx, r, (int)a[0].src_idx.size(), crowded));
  }
  ctx->last_tile_rows = r.tz;
  ctx->last_time_depth = r.depth;
  {
    // receivers grouped by step tile, so each CTA finds its own in one read
    std::vector<int2> table, ent;
    build_tile_receivers(nx, nz, r.tz, a, S, table, ent);
    r.max_tile_rec = 0;
    for (const int2& e : table) r.max_tile_rec = std::max(r.max_tile_rec, e.y);
    FD2D_TRY(upload(ctx, "f32.tile_rec", table, &r.tile_rec));
    FD2D_TRY(upload(ctx, "f32.rec_ent", ent, &r.rec_ent));
  }
  FD2D_TRY(set_tiling(ctx, r));
  return r.depth == 2 ? make_maps2(ctx, r) : FD2D_OK;
}

// Time steps per launch of this run, 1 or 2 (k32_step2), and with them the tile
// shape.  Two steps per launch need FD order 2 or 4, at most MAX_BOX_SRC point
// sources and at most MAX_TILE_REC receivers per tile (crowded[c]: shape c has
// more).  Forced by fd2d_ctx_set_time_depth (or FD2D_TIME_DEPTH), with the
// tile shape tune_tile_rows chose.  Otherwise, on an idle stream with the GPU to
// itself, 24 steps are timed one per launch on that shape and two per launch
// on every shape (on the run's zeroed fields, zeroed again after; the fastest
// of three rounds counts); two steps per launch are kept if they beat one step
// per launch by more than 1 %, on another shape only if by 3 % more,
// remembered per grid, order, lane count and kind.  A forced tile shape is
// kept.  One step per launch otherwise.  The tile tables and tensor maps of
// the result are set up by the caller.
fd2d_status tune_time_depth(fd2d_ctx* ctx, Run& r, int nsrc, const int* crowded) {
  r.depth = 1;
  int forced = ctx->time_depth;
  if (forced == 0) {
    const char* e = std::getenv("FD2D_TIME_DEPTH");
    if (e) forced = std::atoi(e);
  }
  int ci = 0;
  for (int c = 0; c < N_TILE_ROWS; ++c)
    if (TILE_ROWS[c] == r.tz) ci = c;
  if (r.R > 2 || nsrc > MAX_BOX_SRC || forced == 1) return FD2D_OK;
  if (forced == 2) {
    r.depth = crowded[ci] ? 1 : 2;
    return FD2D_OK;
  }
  int forced_rows = ctx->tile_rows;
  if (forced_rows == FD2D_TILE_ROWS_AUTO) {
    const char* e = std::getenv("FD2D_TILE_ROWS");
    if (e) forced_rows = std::atoi(e);
  }
  const bool rows_fixed = forced_rows != FD2D_TILE_ROWS_AUTO;
  const bool with_u = r.u[0] != nullptr;
  Sig key;
  key.add(r.G.nx); key.add(r.G.nz); key.add(r.R); key.add(r.S); key.add((int)with_u); key.add(r.tz);
  key.add((int)rows_fixed); key.bytes(crowded, sizeof(int) * N_TILE_ROWS);
  auto it = ctx->depth_choice.find(key.h);
  if (it != ctx->depth_choice.end()) {
    r.depth = it->second / 100;
    r.tz = it->second % 100;
    return FD2D_OK;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  FD2D_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cs));
  bool idle = cs == cudaStreamCaptureStatusNone && ctx->concurrent_groups <= 1 && !ctx->shared_gpu;
  if (idle) {
    idle = cudaStreamQuery(ctx->stream) == cudaSuccess;
    cudaGetLastError();  // a busy stream answers cudaErrorNotReady
  }
  if (!idle) return FD2D_OK;
  constexpr int WARM = 4, TIMED = 24, ROUNDS = 3;
  const int tz1 = r.tz;
  cudaEvent_t e0, e1;
  FD2D_CUDA(ctx, cudaEventCreate(&e0));
  FD2D_CUDA(ctx, cudaEventCreate(&e1));
  fd2d_status st = FD2D_OK;
  Step32 s{};
  s.inj_plane = -1;
  s.has_u = with_u;
  s.src_xy = r.src_xy;
  s.rec_xy = r.rec_xy;
  // candidates: (depth 1, the chosen shape), then depth 2 on each eligible
  // shape; ROUNDS rounds, the fastest round of each candidate counts
  float ms_of[N_TILE_ROWS + 1] = {};
  for (int round = 0; round < ROUNDS && st == FD2D_OK; ++round)
    for (int c = -1; c < N_TILE_ROWS && st == FD2D_OK; ++c) {
      const int d = c < 0 ? 1 : 2;
      if (d == 2 && (crowded[c] || (rows_fixed && TILE_ROWS[c] != tz1))) continue;
      r.tz = c < 0 ? tz1 : TILE_ROWS[c];
      r.depth = d;
      if ((st = set_tiling(ctx, r)) != FD2D_OK) break;
      if (d == 2 && (st = make_maps2(ctx, r)) != FD2D_OK) break;
      auto steps = [&](int n) {
        for (int k = 0; k < n && st == FD2D_OK; k += d)
          st = d == 1 ? launch_step(ctx, r, (k / d) & 1, s) : launch_step2(ctx, r, (k / d) & 1, s, s);
      };
      steps(WARM);
      cudaEventRecord(e0, ctx->stream);
      steps(TIMED);
      cudaEventRecord(e1, ctx->stream);
      if (st != FD2D_OK) break;
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        st = set_error(ctx, FD2D_ERR_CUDA, "time-depth timing failed");
        break;
      }
      ms_of[c + 1] = round == 0 ? ms : std::min(ms_of[c + 1], ms);
    }
  // two steps per launch on the tile tuner's shape if faster by 1 %; another
  // shape only if faster still by 3 % (plain timed steps favour large tiles a
  // little more than loops with sources, receivers and K_mu terms do)
  float best_ms = ms_of[0];
  int best_d = 1, best_tz = tz1;
  int c1 = -1;
  for (int c = 0; c < N_TILE_ROWS; ++c)
    if (TILE_ROWS[c] == tz1) c1 = c;
  if (c1 >= 0 && ms_of[c1 + 1] > 0.f && ms_of[c1 + 1] < 0.99f * best_ms) {
    best_ms = ms_of[c1 + 1];
    best_d = 2;
  }
  for (int c = 0; c < N_TILE_ROWS; ++c)
    if (c != c1 && ms_of[c + 1] > 0.f && ms_of[c + 1] < (best_d == 2 ? 0.97f : 0.99f) * best_ms) {
      best_ms = ms_of[c + 1];
      best_d = 2;
      best_tz = TILE_ROWS[c];
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != FD2D_OK) return st;
  const size_t bytes = (size_t)r.lanes_ps() * 4;
  for (int q = 0; q < 2; ++q) {
    FD2D_CUDA(ctx, cudaMemsetAsync(r.v[q], 0, bytes, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.sxy[q], 0, bytes, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(r.szy[q], 0, bytes, ctx->stream));
    if (with_u) FD2D_CUDA(ctx, cudaMemsetAsync(r.u[q], 0, bytes, ctx->stream));
  }
  r.depth = best_d;
  r.tz = best_tz;
  ctx->depth_choice[key.h] = best_d * 100 + best_tz;
  return FD2D_OK;
}

// Frequency-band weights (interpol_matrix) on the device.
fd2d_status interp_dev(fd2d_ctx* ctx, const Geometry& g, double** M) {
  std::vector<double> h;
  std::string err;
  fd2d_status s = make_interpol_matrix(g.K, g.nb, h, err);
  if (s != FD2D_OK) return set_error(ctx, s, err);
  return upload_tagged<double>(ctx, "f32.interp", g.key, h.size(), [&](std::vector<double>& o) { o = h; }, M);
}

// e[k] = sum_s spectrum(k, s), summed in source order.
__global__ void k32_spectrum_eff(const double* spec, int K, int n_src, double* e) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  double acc = 0.0;
  for (int s = 0; s < n_src; ++s) acc += spec[k + (int64_t)K * s];
  e[k] = acc;
}

// Effective spectrum: sum over noise sources (they share one distribution);
// lane l's K values at out + l*K.
fd2d_status spectrum_eff(fd2d_ctx* ctx, const Geometry& g, const SolveArgs* a, int S, double** out) {
  FD2D_TRY(workspace_t(ctx, "f32.spec_eff", (size_t)g.K * S, out));
  for (int l = 0; l < S; ++l) {
    k32_spectrum_eff<<<(g.K + 127) / 128, 128, 0, ctx->stream>>>(a[l].spectrum, g.K, a[l].n_src, *out + l * g.K);
    FD2D_TRY(after_launch(ctx, "k32_spectrum_eff"));
  }
  return FD2D_OK;
}

// Tag of a coefficient table: configuration, table kind and the rows it holds.
uint64_t table_tag(const Geometry& g, int kind, const std::vector<int>& rows) {
  Sig s;
  s.add(g.key); s.add(kind); s.add_vec(rows);
  return g.key ? (s.h | 1) : 0;
}

// Injection planes for the listed coefficient rows (ifft rows, one per event).
struct Injection {
  std::vector<int> step_of_event;  // 1-based step n of event j
  std::vector<int> row_of_event;   // coefficient row used by event j
  float* planes = nullptr;         // [chunk][ps]
  int chunk = 0, first = 0, count = 0;  // events [first, first+count) resident
  float* P = nullptr;              // 2K planes of S lanes: [k][lane][ps]
  float* B = nullptr;              // [2K][n_events] float
  float* bimg = nullptr;           // split image of B for the tensor cores
  int n_events = 0;
};

// Per lane l: X = (Xre[l], Xim[l]) spectra, source distribution sd[l], and
// effective spectrum spec_eff + l*K.
fd2d_status build_injection(fd2d_ctx* ctx, const Geometry& g, Run& r, const double* const* Xre,
                            const double* const* Xim, double sign, const double* spec_eff, const double* M,
                            const double* const* sd, Injection& inj) {
  const int K = g.K, ncol = g.nb == 0 ? 1 : g.nb;
  inj.n_events = (int)inj.step_of_event.size();
  if (inj.n_events == 0) return FD2D_OK;
  const int64_t sps = r.lanes_ps();
  FD2D_TRY(workspace_t(ctx, "f32.P", (size_t)sps * 2 * K, &inj.P));
  dim3 pg((r.G.P + 31) / 32, (g.nz + 7) / 8);
  float* W;
  FD2D_TRY(workspace_t(ctx, "f32.band_w", (size_t)K * ncol * r.S, &W));
  for (int l = 0; l < r.S; ++l) {
    float* Wl = W + (size_t)l * K * ncol;
    k32_band_weights<<<(K * ncol + 127) / 128, 128, 0, ctx->stream>>>(K, ncol, M, spec_eff + l * K, Wl);
    FD2D_TRY(after_launch(ctx, "k32_band_weights"));
    k32_make_P<<<pg, r.pblock, 0, ctx->stream>>>(K, ncol, Wl, sd[l], Xre[l], Xim[l], (float)sign, g.nx, g.nz,
                                                 r.G.P, sps, inj.P + l * r.ps);
    FD2D_TRY(after_launch(ctx, "k32_make_P"));
  }
  // B[k][j] = Re c(row_j, k); B[K+k][j] = -Im c(row_j, k)   (c = ifft_coeff, dw)
  auto fill = [&](std::vector<float>& B) {
    for (int j = 0; j < inj.n_events; ++j) {
      const int n = (inj.row_of_event[j] + 1) * g.fs;  // step whose time this row holds
      for (int k = 0; k < K; ++k) {
        double re, im;
        dft_coeff(g.w[k] * g.t_corr[n - 1], g.dw, re, im);
        B[(size_t)k * inj.n_events + j] = (float)re;
        B[(size_t)(K + k) * inj.n_events + j] = (float)(-im);
      }
    }
  };
  FD2D_TRY(upload_tagged<float>(ctx, "f32.injB", table_tag(g, 2, inj.row_of_event),
                                (size_t)2 * K * inj.n_events, fill, &inj.B));
  FD2D_TRY(workspace_t(ctx, "f32.inj_bimg", contract_image_floats(inj.n_events, 2 * K), &inj.bimg));
  FD2D_TRY(contract_image(ctx, ctx->stream, inj.B, inj.n_events, inj.n_events, 2 * K, inj.bimg));
  const size_t cap = (size_t)4 << 30;  // resident injection planes <= 4 GiB
  inj.chunk = (int)std::max<int64_t>(1, std::min<int64_t>(inj.n_events, (int64_t)(cap / (sps * 4))));
  if (ctx->max_inj_chunk > 0) inj.chunk = std::min(inj.chunk, (int)ctx->max_inj_chunk);
  // chunks start on column tiles of the image
  if (inj.chunk < inj.n_events) inj.chunk = std::max(CONTRACT_BN, inj.chunk / CONTRACT_BN * CONTRACT_BN);
  FD2D_TRY(workspace_t(ctx, "f32.inj", (size_t)sps * inj.chunk, &inj.planes));
  inj.first = 0;
  inj.count = 0;
  return set_inj_map(ctx, r, inj.planes, inj.chunk * r.S);
}

// Plane index of event j in the resident chunk (evaluates the next chunk when needed).
fd2d_status injection_plane(fd2d_ctx* ctx, const Run& r, const Geometry& g, Injection& inj, int j, int* plane) {
  if (j < inj.first || j >= inj.first + inj.count) {
    inj.first = j;
    inj.count = std::min(inj.chunk, inj.n_events - j);
    ContractArgs c;
    c.a32 = inj.P;
    c.lda = r.lanes_ps();
    c.Kd = 2 * g.K;
    c.bimg = inj.bimg;
    c.img_nt0 = j / CONTRACT_BN;
    c.img_nkb = (2 * g.K + CONTRACT_BK - 1) / CONTRACT_BK;
    c.M = (int)r.lanes_ps();
    c.N = inj.count;
    c.out32 = inj.planes;
    c.ldo = r.lanes_ps();
    FD2D_TRY(contract(ctx, ctx->stream, c));
  }
  *plane = j - inj.first;
  return FD2D_OK;
}

// DFT accumulation: snapshots of one field at listed steps, contracted in chunks.
struct Dft {
  int T = 0;          // chunk length
  int filled = 0;     // snapshots in the current chunk
  int done = 0;       // events already contracted
  float* snaps = nullptr;
  struct Target {
    float* B = nullptr;     // [n_events][2K] rows
    float* bimg = nullptr;  // their split image
    double *re = nullptr, *im = nullptr;  // lane 0's spectra; lane l's start l*lane_stride later
    int64_t lane_stride = 0;
  };
  std::vector<Target> targets;
  int n_events = 0;
};

fd2d_status dft_init(fd2d_ctx* ctx, const Run& r, int n_events, Dft& d) {
  d.n_events = n_events;
  if (n_events == 0) return FD2D_OK;
  const size_t cap = (size_t)2 << 30;  // snapshot chunk <= 2 GiB
  const int64_t sps = r.lanes_ps();
  const int64_t lim = ctx->max_dft_chunk > 0 ? ctx->max_dft_chunk : DFT_CHUNK_DEFAULT;
  d.T = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)n_events, lim, (int64_t)(cap / (sps * 4))}));
  // chunks start on K blocks of the coefficient image
  if (d.T < n_events) d.T = std::max(CONTRACT_BK, d.T / CONTRACT_BK * CONTRACT_BK);
  FD2D_TRY(workspace_t(ctx, "f32.dft_snaps", (size_t)sps * d.T, &d.snaps));
  // the pitch padding of the snapshot planes is never written by the stencil
  FD2D_CUDA(ctx, cudaMemsetAsync(d.snaps, 0, (size_t)sps * d.T * 4, ctx->stream));
  return FD2D_OK;
}

// rows[e] = (re, im) coefficient pairs for event e, laid out [e][2K] as float;
// `fill` generates them when the buffer does not already hold table `tag`.
template <typename F>
fd2d_status dft_add_target(fd2d_ctx* ctx, const char* name, uint64_t tag, size_t count, F&& fill, double* re,
                           double* im, int64_t lane_stride, Dft& d) {
  Dft::Target t;
  FD2D_TRY(upload_tagged<float>(ctx, name, tag, count, fill, &t.B));
  const int K2 = (int)(count / std::max(d.n_events, 1));  // 2K columns
  FD2D_TRY(workspace_t(ctx, (std::string(name) + ".img").c_str(), contract_image_floats(K2, d.n_events), &t.bimg));
  FD2D_TRY(contract_image(ctx, ctx->stream, t.B, K2, K2, d.n_events, t.bimg));
  t.re = re;
  t.im = im;
  t.lane_stride = lane_stride;
  d.targets.push_back(t);
  return FD2D_OK;
}

float* dft_slot(const Run& r, Dft& d) { return d.snaps + (size_t)d.filled * r.lanes_ps(); }

fd2d_status dft_flush(fd2d_ctx* ctx, const Run& r, const Geometry& g, Dft& d) {
  if (d.filled == 0) return FD2D_OK;
  for (auto& t : d.targets) {
    ContractArgs c;
    c.a32 = d.snaps;
    c.lda = r.lanes_ps();
    c.Kd = d.filled;
    c.bimg = t.bimg;
    c.img_kb0 = d.done / CONTRACT_BK;
    c.img_nkb = (d.n_events + CONTRACT_BK - 1) / CONTRACT_BK;
    c.M = (int)r.lanes_ps();
    if (r.S > 1) {
      c.lane_m = r.ps;
      c.acc_lane = t.lane_stride;
    }
    c.N = 2 * g.K;
    c.acc0 = t.re;
    c.acc1 = t.im;
    c.nsplit = g.K;
    c.ldacc = g.npts();
    c.remap_pitch = r.G.P;
    c.remap_nx = g.nx;
    c.remap_nz = g.nz;
    c.overwrite = d.done == 0;  // the first chunk defines the spectra
    c.k_partials = 2;
    FD2D_TRY(contract(ctx, ctx->stream, c));
  }
  d.done += d.filled;
  d.filled = 0;
  return FD2D_OK;
}

// whether the next dft_push ends a chunk (and contracts it)
bool dft_would_flush(const Dft& d) { return d.filled + 1 == d.T || d.done + d.filled + 1 == d.n_events; }

fd2d_status dft_push(fd2d_ctx* ctx, const Run& r, const Geometry& g, Dft& d) {
  ++d.filled;
  if (d.filled == d.T || d.done + d.filled == d.n_events) return dft_flush(ctx, r, g, d);
  return FD2D_OK;
}

// Everything of a Run the captured loop depends on.
void sig_run(Sig& sg, const Run& r) {
  sg.add(r.G);
  sg.add(r.b); sg.add(r.taper); sg.add(r.dtmu);
  for (int q = 0; q < 2; ++q) { sg.add(r.v[q]); sg.add(r.sxy[q]); sg.add(r.szy[q]); sg.add(r.u[q]); }
  sg.bytes(r.maps, sizeof(r.maps));
  sg.add(r.sgrid.x); sg.add(r.sgrid.y); sg.add(r.sgrid.z); sg.add(r.pgrid.x); sg.add(r.pgrid.y);
  sg.add(r.R); sg.add(r.tz); sg.add((int)r.pdl); sg.add(r.inj_planes); sg.add(r.rec_xy); sg.add(r.src_xy); sg.add(r.np); sg.add(r.ps);
  sg.add(r.depth);
  if (r.depth == 2) sg.bytes(r.maps2, sizeof(r.maps2));
}

void sig_args(Sig& sg, const Geometry& g, const SolveArgs& a) {
  sg.add(g.nx); sg.add(g.nz); sg.add(g.nt); sg.add(g.fs); sg.add(g.fw); sg.add(g.K); sg.add(g.nb);
  sg.add(a.mode); sg.add(a.src_idx.size()); sg.add(a.rec_idx.size());
  sg.add(a.G_out); sg.add(a.G_in); sg.add(a.n_G_in); sg.add(a.G_re); sg.add(a.G_im);
  sg.add(a.dmu); sg.add(a.C_in); sg.add(a.n_C_in); sg.add(a.C_out); sg.add(a.u_fwd); sg.add(a.n_u_fwd);
  sg.add(a.stf_re); sg.add(a.stf_dims[0]); sg.add(a.stf_dims[1]); sg.add(a.stf_dims[2]);
  sg.add(a.Kout); sg.add(a.sf_re); sg.add(a.sf_im); sg.add(a.seis);
}

void sig_dft(Sig& sg, const Dft& d) {
  sg.add(d.T); sg.add(d.n_events); sg.add(d.snaps); sg.add(d.targets.size());
  for (const auto& t : d.targets) { sg.add(t.B); sg.add(t.bimg); sg.add(t.re); sg.add(t.im); sg.add(t.lane_stride); }
}

void sig_inj(Sig& sg, const Injection& j) {
  sg.add(j.n_events); sg.add(j.chunk); sg.add(j.planes); sg.add(j.P); sg.add(j.B); sg.add(j.bimg);
  sg.add_vec(j.step_of_event);
}

fd2d_status f32_copy_pitched(fd2d_ctx* ctx, const Run& r, const double* a, double scale, const char* name,
                             float** out) {
  FD2D_TRY(workspace_t(ctx, name, (size_t)r.ps, out));
  dim3 pg((r.G.P + 31) / 32, (r.G.nz + 7) / 8);
  k32_pitched<<<pg, r.pblock, 0, ctx->stream>>>(a, scale, r.G.nx, r.G.nz, r.G.P, *out);
  return after_launch(ctx, "k32_pitched");
}

}  // namespace

// ---------------------------------------------------------------------------------
// forward1 / correlation are split into an eager prepare step (buffers, uploads,
// P planes) and a capturable time loop, so that a batch can run the loops of
// many solves as parallel branches of one CUDA graph.
// Lanes a[0..S-1]: solves of one geometry advanced together (S > 1: mode 0,
// no Born term, outputs at constant strides from lane 0's).
template <typename T>
static fd2d_status lane_stride_of(fd2d_ctx* ctx, int S, T* const* p, int64_t* out) {
  *out = 0;
  if (S < 2) return FD2D_OK;
  *out = p[1] - p[0];
  for (int l = 2; l < S; ++l)
    if (p[l] - p[l - 1] != *out) return set_error(ctx, FD2D_ERR_ARG, "lane outputs are not equally spaced");
  return FD2D_OK;
}

static fd2d_status check_lanes(fd2d_ctx* ctx, const SolveArgs* a, int S) {
  if (S < 1) return set_error(ctx, FD2D_ERR_ARG, "no lanes");
  for (int l = 0; l < S && S > 1; ++l)
    if (a[l].mode != 0 || a[l].dmu)
      return set_error(ctx, FD2D_ERR_UNSUPPORTED, "lanes advance mode-0 solves without Born terms only");
  return FD2D_OK;
}

fd2d_status fp32_forward1_plan(fd2d_ctx* ctx, const Geometry& g, const SolveArgs* al, int S, LoopPlan& plan) {
  FD2D_TRY(check_lanes(ctx, al, S));
  const SolveArgs& a = al[0];
  std::vector<double*> gre(S), gim(S), seis(S);
  for (int l = 0; l < S; ++l) { gre[l] = al[l].G_re; gim[l] = al[l].G_im; seis[l] = al[l].seis; }
  int64_t g_lane = 0, gi_lane = 0, seis_lane = 0;
  FD2D_TRY(lane_stride_of(ctx, S, gre.data(), &g_lane));
  FD2D_TRY(lane_stride_of(ctx, S, gim.data(), &gi_lane));
  FD2D_TRY(lane_stride_of(ctx, S, seis.data(), &seis_lane));
  if (g_lane != gi_lane) return set_error(ctx, FD2D_ERR_ARG, "lane spectra strides differ");
  Run r;
  FD2D_TRY(init_run(ctx, g, al, S, false, r, a.dmu == nullptr));
  const int nt = g.nt, K = g.K;
  const int64_t np = r.np;
  // DFT events: steps n with mod(n+nt-1, freq_samp) == 0; coefficient of step n is
  // 1/sqrt(2pi) exp(-i w t(n)) dt with t(n) = (n-1) dt; conj(G_fft) is returned, so
  // the imaginary column carries -Im.
  std::vector<int> ev;
  for (int n = 1; n <= nt; ++n)
    if ((n + nt - 1) % g.fs == 0) ev.push_back(n);
  Dft d;
  FD2D_TRY(dft_init(ctx, r, (int)ev.size(), d));
  if (!ev.empty()) {
    auto fill = [&](std::vector<float>& rows) {
      for (size_t e = 0; e < ev.size(); ++e)
        for (int k = 0; k < K; ++k) {
          double re, im;
          dft_coeff(-(g.w[k] * g.t_fwd[ev[e] - 1]), g.dt, re, im);
          rows[e * 2 * K + k] = (float)re;
          rows[e * 2 * K + K + k] = (float)(-im);
        }
    };
    FD2D_TRY(dft_add_target(ctx, "f32.dftB0", table_tag(g, 0, ev), ev.size() * 2 * K, fill, a.G_re, a.G_im,
                            g_lane, d));
  } else {
    // no DFT step: the spectra are zero (otherwise the first flush overwrites them)
    for (int l = 0; l < S; ++l) {
      FD2D_CUDA(ctx, cudaMemsetAsync(al[l].G_re, 0, (size_t)np * K * 8, ctx->stream));
      FD2D_CUDA(ctx, cudaMemsetAsync(al[l].G_im, 0, (size_t)np * K * 8, ctx->stream));
    }
  }
  float* dtdmu = nullptr;
  const bool born = a.dmu != nullptr;
  if (born) FD2D_TRY(f32_copy_pitched(ctx, r, a.dmu, g.dt, "f32.dtdmu", &dtdmu));
  Sig sg;
  sig_run(sg, r); sig_args(sg, g, a); sig_dft(sg, d); sg.add(dtdmu); sg.add(S); sg.add(seis_lane);
  plan.name = "fp32_forward1";
  plan.key = sg.h;
  plan.loop = [ctx, g, a, r, d, dtdmu, born, seis_lane]() -> fd2d_status {
    Dft dd = d;  // the loop's own chunk bookkeeping
    const int nt = g.nt, nr = (int)a.rec_idx.size();
    const int64_t np = r.np;
    int i_fw_out = 0, i_fw_in = 0, par = 0;
    const int tl = timer_begin(ctx, ctx->stream);  // whole loop; contractions are timed inside it
    auto pre = [&](int n) { return a.mode != 0 && (n + nt - 1) % g.fw == 0; };
    auto is_dft_step = [&](int n) { return (n + nt - 1) % g.fs == 0; };
    for (int n = 1; n <= nt; ++n) {
      // two steps in one launch when nothing has to happen between them (no DFT
      // contraction after the first); snapshots before either step are taken in it
      if (r.depth == 2 && !born && n < nt && !(is_dft_step(n) && dft_would_flush(dd))) {
        Step32 s2[2] = {};
        for (int k = 0; k < 2; ++k) {
          Step32& s = s2[k];
          s.inj_plane = -1;
          if (pre(n + k)) s.snap_pre = a.G_out + (size_t)np * (i_fw_out++);
          s.src_xy = r.src_xy;
          s.nsrc = (int)a.src_idx.size();
          s.amp_const = 1.0e9f;
          s.rec_xy = r.rec_xy;
          s.nrec = nr;
          s.seis_col = a.seis + (size_t)nr * (n + k - 1);
          s.seis_lane = seis_lane;
        }
        const bool d0 = is_dft_step(n), d1 = is_dft_step(n + 1);
        if (d0) s2[0].snap_dft = dft_slot(r, dd);
        if (d1) s2[1].snap_dft = dd.snaps + (size_t)(dd.filled + (d0 ? 1 : 0)) * r.lanes_ps();
        FD2D_TRY(launch_step2(ctx, r, par, s2[0], s2[1]));
        if (d0) FD2D_TRY(dft_push(ctx, r, g, dd));
        if (d1) FD2D_TRY(dft_push(ctx, r, g, dd));
        par ^= 1;
        ++n;
        continue;
      }
      Step32 s{};
      s.inj_plane = -1;
      if (pre(n)) s.snap_pre = a.G_out + (size_t)np * (i_fw_out++);
      if (born) {
        FD2D_DISPATCH_R(r.R, k32_born_pre, r.G, r.sxy[par], r.szy[par], dtdmu, a.G_in + (size_t)np * (i_fw_in++));
        FD2D_TRY(after_launch(ctx, "k32_born_pre"));
      } else {
        s.src_xy = r.src_xy;
        s.nsrc = (int)a.src_idx.size();
        s.amp_const = 1.0e9f;  // stf = 1.0e9*ones(1,nt), code/run_forward1_green.m:64
      }
      const bool is_dft = is_dft_step(n);
      if (is_dft) s.snap_dft = dft_slot(r, dd);
      s.rec_xy = r.rec_xy;
      s.nrec = nr;
      s.seis_col = a.seis + (size_t)nr * (n - 1);
      s.seis_lane = seis_lane;
      FD2D_TRY(launch_step(ctx, r, par, s));
      if (is_dft) FD2D_TRY(dft_push(ctx, r, g, dd));
      par ^= 1;
    }
    timer_end(ctx, ctx->stream, tl, FD2D_TIMER_STEP_V, np * nt * r.S, nt);
    return FD2D_OK;
  };
  return FD2D_OK;
}

fd2d_status fp32_correlation_plan(fd2d_ctx* ctx, const Geometry& g, const SolveArgs* al, int S, LoopPlan& plan) {
  FD2D_TRY(check_lanes(ctx, al, S));
  const SolveArgs& a = al[0];
  std::vector<double*> seis(S);
  std::vector<const double*> xre(S), xim(S), sd(S);
  for (int l = 0; l < S; ++l) {
    seis[l] = al[l].seis;
    xre[l] = al[l].Gin_re;
    xim[l] = al[l].Gin_im;
    sd[l] = al[l].source_dist;
  }
  int64_t seis_lane = 0;
  FD2D_TRY(lane_stride_of(ctx, S, seis.data(), &seis_lane));
  Run r;
  FD2D_TRY(init_run(ctx, g, al, S, true, r, a.dmu == nullptr));
  const int ntc = g.ntc;
  double *M, *spec;
  FD2D_TRY(interp_dev(ctx, g, &M));
  FD2D_TRY(spectrum_eff(ctx, g, al, S, &spec));
  Injection inj;
  for (int n = 1; n <= ntc; ++n)
    if (n % g.fs == 0) {
      inj.step_of_event.push_back(n);
      inj.row_of_event.push_back(n / g.fs - 1);
    }
  FD2D_TRY(build_injection(ctx, g, r, xre.data(), xim.data(), 1.0, spec, M, sd.data(), inj));
  float* dmu32 = nullptr;
  const bool born = a.dmu != nullptr;
  if (born) FD2D_TRY(f32_copy_pitched(ctx, r, a.dmu, 1.0, "f32.dmu", &dmu32));
  Sig sg;
  sig_run(sg, r); sig_args(sg, g, a); sig_inj(sg, inj); sg.add(dmu32); sg.add(S); sg.add(seis_lane);
  plan.name = "fp32_correlation";
  plan.key = sg.h;
  plan.loop = [ctx, g, a, r, inj, dmu32, born, seis_lane]() -> fd2d_status {
    Injection ij = inj;  // the loop's own chunk bookkeeping
    const int ntc = g.ntc, nr = (int)a.rec_idx.size();
    const int64_t np = r.np;
    int i_fw_out = 0, par = 0, ev = 0;
    const int tl = timer_begin(ctx, ctx->stream);
    auto pre = [&](int n) { return a.mode != 0 && n % g.fw == 0; };
    for (int n = 1; n <= ntc; ++n) {
      Step32 s{};
      s.inj_plane = -1;
      s.has_u = 1;
      if (pre(n)) {
        s.snap_pre = a.C_out + (size_t)np * (i_fw_out++);
        s.snap_pre_u = 1;
      }
      if (n % g.fs == 0) FD2D_TRY(injection_plane(ctx, r, g, ij, ev++, &s.inj_plane));
      s.rec_xy = r.rec_xy;
      s.nrec = nr;
      s.seis_col = a.seis + (size_t)nr * (n - 1);
      s.seis_lane = seis_lane;
      s.rec_u = 1;  // u does not depend on this step's Born stress correction
      // two steps in one launch when the next step's injection plane (if any) is
      // already resident; snapshots before either step are taken in it
      if (r.depth == 2 && !born && n < ntc &&
          ((n + 1) % g.fs != 0 || (ev >= ij.first && ev < ij.first + ij.count))) {
        Step32 s1 = s;
        s1.inj_plane = -1;
        if ((n + 1) % g.fs == 0) s1.inj_plane = ev++ - ij.first;
        s1.snap_pre = pre(n + 1) ? a.C_out + (size_t)np * (i_fw_out++) : nullptr;
        s1.snap_pre_u = 1;
        s1.seis_col = a.seis + (size_t)nr * n;
        FD2D_TRY(launch_step2(ctx, r, par, s, s1));
        par ^= 1;
        ++n;
        continue;
      }
      FD2D_TRY(launch_step(ctx, r, par, s));
      par ^= 1;
      if (born && n != ntc) {
        FD2D_DISPATCH_R(r.R, k32_born_post, r.G, r.sxy[par], r.szy[par], dmu32,
                        a.C_in + (size_t)np * (n - 1), a.C_in + (size_t)np * n);
        FD2D_TRY(after_launch(ctx, "k32_born_post"));
      }
    }
    timer_end(ctx, ctx->stream, tl, FD2D_TIMER_STEP_VU, np * ntc * r.S, ntc);
    return FD2D_OK;
  };
  return FD2D_OK;
}

fd2d_status fp32_forward1(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  LoopPlan p;
  FD2D_TRY(fp32_forward1_plan(ctx, g, &a, 1, p));
  return run_captured(ctx, p.name.c_str(), p.key, p.loop);
}

fd2d_status fp32_correlation(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  LoopPlan p;
  FD2D_TRY(fp32_correlation_plan(ctx, g, &a, 1, p));
  return run_captured(ctx, p.name.c_str(), p.key, p.loop);
}

fd2d_status fp32_adjoint(fd2d_ctx* ctx, const Geometry& g, const SolveArgs& a) {
  Run r;
  FD2D_TRY(init_run(ctx, g, &a, 1, true, r, !(a.dmu != nullptr && a.n_C_in == g.ntc)));
  const int ntc = g.ntc, K = g.K, mode = a.mode;
  const int64_t np = r.np;
  const int ncol = g.nb == 0 ? 1 : g.nb;
  const int64_t d0 = a.stf_dims[0], d1 = a.stf_dims[1], d2 = a.stf_dims[2];
  const bool stf_empty = !a.stf_re || d0 * d1 * d2 == 0;
  const int64_t size3 = stf_empty ? 1 : d2;
  const bool stf2d = !stf_empty && size3 == 1, stf3d = !stf_empty && size3 != 1;
  int nt_loop = ntc;
  if ((mode == 0 || mode == 1) && size3 != 1) nt_loop = g.nt;  // code/run_noise_adjoint.m:165-167
  const bool Gvalid = a.Gin_re != nullptr && a.n_G == K;
  const bool born = a.dmu != nullptr && a.n_C_in == ntc;
  const bool save_u = mode == 11 || mode == 13;
  const bool dft_u = mode == 1 || mode == 12 || mode == 13;
  const bool have_fwd = a.u_fwd != nullptr && a.n_u_fwd > 0;
  const int n_ftc = ntc / g.fs;
  // The reference shares one counter i_ftc between the field-source injection
  // and the stf_fft DFT (code/run_noise_adjoint.m:265,343); replay it.
  std::vector<int> inj_step, inj_row, dft_step, dft_row;
  {
    int i_ftc = 0;
    for (int n = 1; n <= nt_loop; ++n) {
      if (n % g.fs) continue;
      if (stf3d) { inj_step.push_back(n); inj_row.push_back(i_ftc++); }
      if (dft_u) { dft_step.push_back(n); dft_row.push_back(i_ftc++); }
    }
    if (i_ftc > n_ftc) return set_error(ctx, FD2D_ERR_INDEX, "fft_coeff row past the end");
  }
  double *M, *spec = nullptr;
  FD2D_TRY(interp_dev(ctx, g, &M));
  if (a.spectrum) FD2D_TRY(spectrum_eff(ctx, g, &a, 1, &spec));
  Injection inj;
  if (stf3d && a.source_dist) {
    inj.step_of_event = inj_step;
    inj.row_of_event = inj_row;
    const double* sim = a.stf_im;
    if (!sim) {
      double* z;
      FD2D_TRY(workspace_t(ctx, "f32.zero_im", (size_t)np * K, &z));
      FD2D_CUDA(ctx, cudaMemsetAsync(z, 0, (size_t)np * K * 8, ctx->stream));
      sim = z;
    }
    FD2D_TRY(build_injection(ctx, g, r, &a.stf_re, &sim, -1.0, spec, M, &a.source_dist, inj));
  }
  // DFT of u at the fs steps: stf_fft with the rows the reference uses, and the
  // natural-row spectrum U that forms the source kernel.
  std::vector<int> ev;
  for (int n = 1; n <= nt_loop; ++n)
    if (n % g.fs == 0 && (dft_u || Gvalid)) ev.push_back(n);
  bool natural = true;
  for (size_t e = 0; e < dft_row.size(); ++e) natural &= dft_row[e] == dft_step[e] / g.fs - 1;
  FD2D_CUDA(ctx, cudaMemsetAsync(a.sf_re, 0, (size_t)np * K * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.sf_im, 0, (size_t)np * K * 8, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(a.Kout, 0, (size_t)np * 8 * (ncol + 1), ctx->stream));
  Dft d;
  FD2D_TRY(dft_init(ctx, r, (int)ev.size(), d));
  double *Ure = nullptr, *Uim = nullptr;
  auto rows_for = [&](const std::vector<int>& rows_of_event) {
    return [&g, &ev, &rows_of_event, K](std::vector<float>& rows) {
      for (size_t e = 0; e < ev.size(); ++e) {
        const int n = (rows_of_event[e] + 1) * g.fs;
        for (int k = 0; k < K; ++k) {
          double re, im;
          dft_coeff(-(g.w[k] * g.t_corr[n - 1]), g.dt, re, im);
          rows[e * 2 * K + k] = (float)re;
          rows[e * 2 * K + K + k] = (float)im;
        }
      }
    };
  };
  const size_t nrows = ev.size() * 2 * K;
  if (!ev.empty()) {
    std::vector<int> nat(ev.size());
    for (size_t e = 0; e < ev.size(); ++e) nat[e] = ev[e] / g.fs - 1;
    if (dft_u) {
      FD2D_TRY(dft_add_target(ctx, "f32.dftB0", table_tag(g, 1, dft_row), nrows, rows_for(dft_row), a.sf_re,
                              a.sf_im, 0, d));
      if (natural) { Ure = a.sf_re; Uim = a.sf_im; }
    }
    if (Gvalid && !Ure) {
      FD2D_TRY(workspace_t(ctx, "f32.Ure", (size_t)np * K, &Ure));
      FD2D_TRY(workspace_t(ctx, "f32.Uim", (size_t)np * K, &Uim));
      FD2D_CUDA(ctx, cudaMemsetAsync(Ure, 0, (size_t)np * K * 8, ctx->stream));
      FD2D_CUDA(ctx, cudaMemsetAsync(Uim, 0, (size_t)np * K * 8, ctx->stream));
      FD2D_TRY(dft_add_target(ctx, "f32.dftB1", table_tag(g, 1, nat), nrows, rows_for(nat), Ure, Uim, 0, d));
    }
  }
  float* dmu32 = nullptr;
  if (born) FD2D_TRY(f32_copy_pitched(ctx, r, a.dmu, 1.0, "f32.dmu", &dmu32));
  double* Kmu = a.Kout + (size_t)np * ncol;
  const int nr = (int)a.rec_idx.size();
  Sig sg;
  sig_run(sg, r); sig_args(sg, g, a); sig_dft(sg, d); sig_inj(sg, inj);
  sg.add(dmu32); sg.add(Ure); sg.add(Uim); sg.add(nt_loop);
  FD2D_TRY(run_captured(ctx, "fp32_adjoint", sg.h, [&]() -> fd2d_status {
    int i_fw_out = 0, i_fw_in = 0, par = 0, j_inj = 0;
    const int tl = timer_begin(ctx, ctx->stream);
    for (int n = 1; n <= nt_loop; ++n) {
      Step32 s{};
      s.inj_plane = -1;
      s.has_u = 1;
      if (save_u && n % g.fw == 0) {
        s.snap_pre = a.C_out + (size_t)np * (i_fw_out++);
        s.snap_pre_u = 1;
      }
      if (stf2d) {
        s.src_xy = r.src_xy;
        s.nsrc = (int)a.src_idx.size();
        s.amp = a.stf_re + (size_t)d0 * (n - 1);
      } else if (inj.n_events && j_inj < inj.n_events && inj.step_of_event[j_inj] == n) {
        FD2D_TRY(injection_plane(ctx, r, g, inj, j_inj++, &s.inj_plane));
      }
      const bool is_dft = d.n_events && n % g.fs == 0;
      if (is_dft) s.snap_dft = dft_slot(r, d);
      s.rec_xy = r.rec_xy;
      s.nrec = nr;
      s.seis_col = a.seis + (size_t)nr * (n - 1);
      s.rec_u = 1;
      // two steps in one launch when nothing has to happen between them: no
      // K_mu term and no DFT contraction after the first, and the second step's
      // injection plane (if any) resident; stored u before either step is
      // taken in it
      if (r.depth == 2 && !born && n < nt_loop && !(have_fwd && a.n_u_fwd >= i_fw_in + 1 && n % g.fw == 0) &&
          !(is_dft && dft_would_flush(d))) {
        Step32 s1 = s;
        s1.inj_plane = -1;
        bool can = true;
        if (stf2d) {
          s1.amp = a.stf_re + (size_t)d0 * n;
        } else if (inj.n_events && j_inj < inj.n_events && inj.step_of_event[j_inj] == n + 1) {
          can = j_inj >= inj.first && j_inj < inj.first + inj.count;
          if (can) s1.inj_plane = j_inj++ - inj.first;
        }
        if (can) {
          s1.snap_pre = (save_u && (n + 1) % g.fw == 0) ? a.C_out + (size_t)np * (i_fw_out++) : nullptr;
          s1.snap_pre_u = 1;
          const bool is_dft1 = d.n_events && (n + 1) % g.fs == 0;
          s1.snap_dft = is_dft1 ? d.snaps + (size_t)(d.filled + (is_dft ? 1 : 0)) * r.lanes_ps() : nullptr;
          s1.seis_col = a.seis + (size_t)nr * n;
          FD2D_TRY(launch_step2(ctx, r, par, s, s1));
          par ^= 1;
          if (is_dft) FD2D_TRY(dft_push(ctx, r, g, d));
          if (have_fwd && a.n_u_fwd >= i_fw_in + 1 && (n + 1) % g.fw == 0) {
            const float* uf = a.u_fwd + (size_t)np * (a.n_u_fwd - 1 - i_fw_in);
            FD2D_DISPATCH_R(r.R, k32_kmu, r.G, r.u[par], uf, Kmu, (float)g.fw);
            FD2D_TRY(after_launch(ctx, "k32_kmu"));
            ++i_fw_in;
          }
          if (is_dft1) FD2D_TRY(dft_push(ctx, r, g, d));
          ++n;
          continue;
        }
      }
      FD2D_TRY(launch_step(ctx, r, par, s));
      par ^= 1;
      if (born && n != ntc) {
        FD2D_DISPATCH_R(r.R, k32_born_post, r.G, r.sxy[par], r.szy[par], dmu32,
                        a.C_in + (size_t)np * (n - 1), a.C_in + (size_t)np * n);
        FD2D_TRY(after_launch(ctx, "k32_born_post"));
      }
      if (have_fwd && a.n_u_fwd >= i_fw_in + 1 && n % g.fw == 0) {
        const float* uf = a.u_fwd + (size_t)np * (a.n_u_fwd - 1 - i_fw_in);
        FD2D_DISPATCH_R(r.R, k32_kmu, r.G, r.u[par], uf, Kmu, (float)g.fw);
        FD2D_TRY(after_launch(ctx, "k32_kmu"));
        ++i_fw_in;
      }
      if (is_dft) FD2D_TRY(dft_push(ctx, r, g, d));
    }
    timer_end(ctx, ctx->stream, tl, FD2D_TIMER_STEP_VU, np * nt_loop, nt_loop);
    return FD2D_OK;
  }));
  if (Gvalid) {
    k32_source_kernel<<<(unsigned)((np + 127) / 128), 128, 0, ctx->stream>>>(
        K, ncol, M, spec, a.Gin_re, a.Gin_im, Ure, Uim, g.dw / g.dt, a.Kout, np);
    FD2D_TRY(after_launch(ctx, "k32_source_kernel"));
  }
  if (nt_loop < ntc && nr > 0)
    FD2D_CUDA(ctx, cudaMemsetAsync(a.seis + (size_t)nr * nt_loop, 0, (size_t)nr * (ntc - nt_loop) * 8, ctx->stream));
  return FD2D_OK;
}


// ---------------------------------------------------------------------------------
// Multi-geometry loops: the reference stations of a batch whose grids differ
// (the parfor over stations of code/calculate_data.m:189-202) advance in one
// k32_step_multi launch per time step, each solve for its own nt / ntc steps;
// the DFT and injection contractions stay per solve.
namespace {

constexpr int MULTI_TZ = 32;  // tile rows of the multi-geometry step

template <int R, bool HU, bool HI>
void launch_multi_t(fd2d_ctx* ctx, const MultiStep& q, const StepMaps& m, int n_tiles, bool pdl) {
  using T = Tile<R, HU, HI, MULTI_TZ>;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(n_tiles);
  cfg.blockDim = dim3(T::NT);
  cfg.dynamicSmemBytes = T::BYTES;
  cfg.stream = ctx->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k32_step_multi<R, HU, HI, MULTI_TZ>, q, m);
}

template <int R>
void launch_multi_r(fd2d_ctx* ctx, bool hu, bool hi, const MultiStep& q, const StepMaps& m, int n_tiles, bool pdl) {
  if (!hu) launch_multi_t<R, false, false>(ctx, q, m, n_tiles, pdl);
  else if (hi) launch_multi_t<R, true, true>(ctx, q, m, n_tiles, pdl);
  else launch_multi_t<R, true, false>(ctx, q, m, n_tiles, pdl);
}

fd2d_status launch_multi(fd2d_ctx* ctx, int R, bool hu, bool hi, const MultiStep& q, const StepMaps& m,
                         int n_tiles, bool pdl) {
  switch (R) {
    case 1: launch_multi_r<1>(ctx, hu, hi, q, m, n_tiles, pdl); break;
    case 2: launch_multi_r<2>(ctx, hu, hi, q, m, n_tiles, pdl); break;
    case 3: launch_multi_r<3>(ctx, hu, hi, q, m, n_tiles, pdl); break;
    default: launch_multi_r<4>(ctx, hu, hi, q, m, n_tiles, pdl); break;
  }
  return after_launch(ctx, "k32_step_multi");
}

template <int R>
fd2d_status multi_attributes_r(fd2d_ctx* ctx) {
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step_multi<R, false, false, MULTI_TZ>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, false, false, MULTI_TZ>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step_multi<R, true, false, MULTI_TZ>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, true, false, MULTI_TZ>::BYTES));
  FD2D_CUDA(ctx, cudaFuncSetAttribute(k32_step_multi<R, true, true, MULTI_TZ>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      Tile<R, true, true, MULTI_TZ>::BYTES));
  return FD2D_OK;
}

PerDeviceOnce g_multi_attributes;
fd2d_status multi_attributes(fd2d_ctx* ctx) {
  return g_multi_attributes.run(ctx, [ctx]() -> fd2d_status {
    FD2D_TRY(multi_attributes_r<1>(ctx));
    FD2D_TRY(multi_attributes_r<2>(ctx));
    FD2D_TRY(multi_attributes_r<3>(ctx));
    return multi_attributes_r<4>(ctx);
  });
}

// Host state of one solve of a multi-geometry loop.
struct MultiSolve {
  Geometry g;
  SolveArgs a;
  Run r;          // one-lane compact layout of the solve's DFT snapshots and injection planes
  Dft d;
  Injection inj;
  Seg seg{};
  int nsteps = 0;
};

// The stacked field arrays and the device table of the solves.
struct MultiLayout {
  int R = 2, Pf = 32, rows = 0, fs = 1;
  float *v[2] = {}, *sxy[2] = {}, *szy[2] = {}, *u[2] = {};
  float *b = nullptr, *taper = nullptr, *dtmu = nullptr;
  StepMaps maps[2];
  Seg* segs = nullptr;
  std::vector<int> tiles;  // tiles[k]: CTAs of the first k solves
  float c[4] = {0, 0, 0, 0};
  bool pdl = true;
};

// Solves sorted by steps (longest first, so the solves still running at a
// step are a prefix), stacked fields, coefficient planes, node tables and
// tensor maps.  The DFT / injection parts are added by the callers.
fd2d_status multi_layout(fd2d_ctx* ctx, std::vector<MultiSolve>& ms, bool with_u, MultiLayout& L) {
  if (ms.empty() || ms.size() > (size_t)MULTI_MAX_SEG)
    return set_error(ctx, FD2D_ERR_ARG, "a multi-geometry loop takes 1 to 64 solves");
  std::stable_sort(ms.begin(), ms.end(), [](const MultiSolve& x, const MultiSolve& y) { return x.nsteps > y.nsteps; });
  L.R = ms[0].g.r;
  L.fs = ms[0].g.fs;
  for (int m = 0; m < 4; ++m) L.c[m] = (float)ms[0].g.c[m];
  const int R = L.R, TZ = MULTI_TZ, MZ = 2 * R;  // zero rows above and below every solve
  L.Pf = 32;
  int rows = 0, tiles = 0;
  L.tiles.assign(1, 0);
  for (auto& s : ms) {
    const Geometry& g = s.g;
    Seg& q = s.seg;
    q.nx = g.nx;
    q.nz = g.nz;
    q.P = (g.nx + 31) / 32 * 32;
    q.ps = ((int64_t)q.P * g.nz + 127) / 128 * 128;
    q.ntx = (g.nx + TX - 1) / TX;
    q.ntz = (g.nz + TZ - 1) / TZ;
    q.row0 = rows + MZ;
    rows += MZ + q.ntz * TZ + MZ;
    q.tile0 = tiles;
    tiles += q.ntx * q.ntz;
    L.tiles.push_back(tiles);
    q.nt = g.nt;
    q.inv_dx = (float)(1.0 / g.dx);
    q.inv_dz = (float)(1.0 / g.dz);
    q.dt = (float)g.dt;
    L.Pf = std::max(L.Pf, q.P);
  }
  L.rows = rows;
  const size_t n = (size_t)L.Pf * rows;
  static const char* names[2][4] = {{"m.v0", "m.sxy0", "m.szy0", "m.u0"}, {"m.v1", "m.sxy1", "m.szy1", "m.u1"}};
  for (int q = 0; q < 2; ++q) {
    FD2D_TRY(workspace_t(ctx, names[q][0], n, &L.v[q]));
    FD2D_TRY(workspace_t(ctx, names[q][1], n, &L.sxy[q]));
    FD2D_TRY(workspace_t(ctx, names[q][2], n, &L.szy[q]));
    FD2D_CUDA(ctx, cudaMemsetAsync(L.v[q], 0, n * 4, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(L.sxy[q], 0, n * 4, ctx->stream));
    FD2D_CUDA(ctx, cudaMemsetAsync(L.szy[q], 0, n * 4, ctx->stream));
    if (with_u) {
      FD2D_TRY(workspace_t(ctx, names[q][3], n, &L.u[q]));
      FD2D_CUDA(ctx, cudaMemsetAsync(L.u[q], 0, n * 4, ctx->stream));
    }
  }
  FD2D_TRY(workspace_t(ctx, "m.b", n, &L.b));
  FD2D_TRY(workspace_t(ctx, "m.taper", n, &L.taper));
  FD2D_TRY(workspace_t(ctx, "m.dtmu", n, &L.dtmu));
  FD2D_CUDA(ctx, cudaMemsetAsync(L.b, 0, n * 4, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(L.taper, 0, n * 4, ctx->stream));
  FD2D_CUDA(ctx, cudaMemsetAsync(L.dtmu, 0, n * 4, ctx->stream));
  int ti = 0;
  for (int c = 0; c < N_TILE_ROWS; ++c)
    if (TILE_ROWS[c] == TZ) ti = c;
  for (size_t i = 0; i < ms.size(); ++i) {
    MultiSolve& s = ms[i];
    const Geometry& g = s.g;
    Seg& q = s.seg;
    ctx->ws_prefix = "m" + std::to_string(i) + ":";
    double* ab;
    FD2D_TRY(upload_tagged<double>(ctx, "f32.absbound64", g.key, g.absbound->size(),
                                    [&](std::vector<double>& h) { h = *g.absbound; }, &ab));
    const size_t off = (size_t)q.row0 * L.Pf;
    dim3 pg((L.Pf + 31) / 32, (g.nz + 7) / 8);
    k32_prep<<<pg, dim3(32, 8), 0, ctx->stream>>>(s.a.mu, s.a.rho, ab, g.dt, g.nx, g.nz, L.Pf, L.b + off,
                                                  L.taper + off, L.dtmu + off);
    FD2D_TRY(after_launch(ctx, "k32_prep"));
    int t1[N_TILE_ROWS][4];
    taper_ones(*g.absbound, g.nx, g.nz, R, t1);
    for (int k = 0; k < 4; ++k) q.t1[k] = t1[ti][k];
    std::vector<int2> rxy, sxy, table, ent;
    for (int p : s.a.rec_idx) rxy.push_back(make_int2(p % g.nx, p / g.nx));
    for (int p : s.a.src_idx) sxy.push_back(make_int2(p % g.nx, p / g.nx));
    if (rxy.empty()) rxy.push_back(make_int2(-1 << 30, -1 << 30));
    if (sxy.empty()) sxy.push_back(make_int2(-1 << 30, -1 << 30));
    std::vector<const std::vector<int>*> lanes{&s.a.rec_idx};
    build_tile_receivers_idx(g.nx, g.nz, TZ, lanes, table, ent);
    int2 *d_rxy, *d_sxy, *d_tab, *d_ent;
    FD2D_TRY(upload(ctx, "m.rec", rxy, &d_rxy));
    FD2D_TRY(upload(ctx, "m.src", sxy, &d_sxy));
    FD2D_TRY(upload(ctx, "m.tile_rec", table, &d_tab));
    FD2D_TRY(upload(ctx, "m.rec_ent", ent, &d_ent));
    q.rec_xy = d_rxy;
    q.src_xy = d_sxy;
    q.tile_rec = d_tab;
    q.rec_ent = d_ent;
    q.nrec = (int)s.a.rec_idx.size();
    q.nsrc = (int)s.a.src_idx.size();
    q.seis = s.a.seis;
    // the solve's compact one-lane layout for its DFT and injection
    Run& r = s.r;
    r.S = 1;
    r.np = g.npts();
    r.ps = q.ps;
    r.R = R;
    r.tz = TZ;
    r.G.nx = g.nx;
    r.G.nz = g.nz;
    r.G.P = q.P;
    r.G.S = 1;
    r.G.ps = q.ps;
    r.G.err = ctx->d_err;
  }
  ctx->ws_prefix.clear();
  // tensor maps over the stacked arrays (2-D arrays as 3-D maps of depth 1)
  const int BH = TZ + 2 * R - 1, SZH = TZ + 4 * R - 2, BWa = TX + 8, SXWa = TX + 16;
  const int NT = std::min(TX / 4 * TZ, 256);
  const int H1 = split_top_rows(NT, BWa / 4, BH), H1Z = split_top_szy(H1, R, SZH);
  const int W = L.Pf, Hh = rows;
  const int64_t pl = (int64_t)L.Pf * rows;
  for (int q = 0; q < 2; ++q) {
    StepMaps& m = L.maps[q];
    FD2D_TRY(make_tmap_f32(ctx, &m.sxy_t, L.sxy[q], W, Hh, L.Pf, SXWa, H1, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.sxy_b, L.sxy[q], W, Hh, L.Pf, SXWa, BH - H1, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.szy_t, L.szy[q], W, Hh, L.Pf, BWa, H1Z, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.szy_b, L.szy[q], W, Hh, L.Pf, BWa, std::max(SZH - H1Z, 1), 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.v_t, L.v[q], W, Hh, L.Pf, BWa, H1, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.v_b, L.v[q], W, Hh, L.Pf, BWa, BH - H1, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.u, L.u[q] ? L.u[q] : L.v[q], W, Hh, L.Pf, TX, TZ, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.b, L.b, W, Hh, L.Pf, BWa, BH, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.taper, L.taper, W, Hh, L.Pf, BWa, BH, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.dtmu, L.dtmu, W, Hh, L.Pf, TX, TZ, 1, pl));
    FD2D_TRY(make_tmap_f32(ctx, &m.inj, L.b, W, Hh, L.Pf, BWa, BH, 1, pl));  // unused: planes come from L2
  }
  L.pdl = ctx->concurrent_groups <= 1 && !ctx->shared_gpu;
  FD2D_TRY(step_attributes(ctx));
  FD2D_TRY(multi_attributes(ctx));
  return contract_prepare(ctx);
}

fd2d_status multi_upload_segs(fd2d_ctx* ctx, const std::vector<MultiSolve>& ms, MultiLayout& L) {
  std::vector<Seg> h(ms.size());
  for (size_t i = 0; i < ms.size(); ++i) h[i] = ms[i].seg;
  return upload(ctx, "m.segs", h, &L.segs);
}

void sig_multi(Sig& sg, const std::vector<MultiSolve>& ms, const MultiLayout& L) {
  sg.add(L.R); sg.add(L.Pf); sg.add(L.rows); sg.add(L.fs); sg.add(L.segs); sg.add((int)L.pdl);
  sg.bytes(L.maps, sizeof(L.maps));
  for (const auto& s : ms) {
    sg.bytes(&s.seg, sizeof(Seg));
    sig_args(sg, s.g, s.a);
    sig_dft(sg, s.d);
    sig_inj(sg, s.inj);
    sg.add(s.nsteps);
  }
}

}  // namespace

fd2d_status fp32_multi_forward1_plan(fd2d_ctx* ctx, const std::vector<const Geometry*>& gs,
                                     const std::vector<const SolveArgs*>& as, LoopPlan& plan) {
  std::vector<MultiSolve> ms(gs.size());
  for (size_t i = 0; i < gs.size(); ++i) {
    ms[i].g = *gs[i];
    ms[i].a = *as[i];
    ms[i].nsteps = gs[i]->nt;
  }
  MultiLayout L;
  FD2D_TRY(multi_layout(ctx, ms, false, L));
  for (size_t i = 0; i < ms.size(); ++i) {
    MultiSolve& s = ms[i];
    const Geometry& g = s.g;
    const int nt = g.nt, K = g.K;
    ctx->ws_prefix = "m" + std::to_string(i) + ":";
    // DFT events and coefficients as in fp32_forward1_plan
    std::vector<int> ev;
    for (int n = 1; n <= nt; ++n)
      if ((n + nt - 1) % g.fs == 0) ev.push_back(n);
    FD2D_TRY(dft_init(ctx, s.r, (int)ev.size(), s.d));
    if (!ev.empty()) {
      auto fill = [&](std::vector<float>& rows) {
        for (size_t e = 0; e < ev.size(); ++e)
          for (int k = 0; k < K; ++k) {
            double re, im;
            dft_coeff(-(g.w[k] * g.t_fwd[ev[e] - 1]), g.dt, re, im);
            rows[e * 2 * K + k] = (float)re;
            rows[e * 2 * K + K + k] = (float)(-im);
          }
      };
      FD2D_TRY(dft_add_target(ctx, "f32.dftB0", table_tag(g, 0, ev), ev.size() * 2 * K, fill, s.a.G_re,
                              s.a.G_im, 0, s.d));
    } else {
      FD2D_CUDA(ctx, cudaMemsetAsync(s.a.G_re, 0, (size_t)g.npts() * K * 8, ctx->stream));
      FD2D_CUDA(ctx, cudaMemsetAsync(s.a.G_im, 0, (size_t)g.npts() * K * 8, ctx->stream));
    }
    s.seg.dft_T = std::max(s.d.T, 1);
    s.seg.snaps = s.d.snaps;
  }
  ctx->ws_prefix.clear();
  FD2D_TRY(multi_upload_segs(ctx, ms, L));
  Sig sg;
  sg.add(1);
  sig_multi(sg, ms, L);
  plan.name = "fp32_multi_forward1";
  plan.key = sg.h;
  plan.loop = [ctx, ms, L]() -> fd2d_status {
    std::vector<Dft> dd(ms.size());
    for (size_t i = 0; i < ms.size(); ++i) dd[i] = ms[i].d;  // the loop's own chunk bookkeeping
    const int nmax = ms[0].nsteps;
    int64_t units = 0;
    for (const auto& s : ms) units += s.g.npts() * s.g.nt;
    const int tl = timer_begin(ctx, ctx->stream);
    int n_seg = (int)ms.size(), par = 0;
    for (int n = 1; n <= nmax; ++n) {
      while (n_seg > 0 && ms[n_seg - 1].nsteps < n) --n_seg;
      MultiStep q{};
      q.n = n;
      q.n_seg = n_seg;
      for (int i = 0; i < n_seg; ++i) q.tile0[i] = ms[i].seg.tile0;
      q.fs = L.fs;
      q.green = 1;
      q.Pf = L.Pf;
      for (int m = 0; m < 4; ++m) q.c[m] = L.c[m];
      q.segs = L.segs;
      q.vo = L.v[1 - par];
      q.sxyo = L.sxy[1 - par];
      q.szyo = L.szy[1 - par];
      q.uo = nullptr;
      q.err = ctx->d_err;
      FD2D_TRY(launch_multi(ctx, L.R, false, false, q, L.maps[par], L.tiles[n_seg], L.pdl));
      for (int i = 0; i < n_seg; ++i) {
        const MultiSolve& s = ms[i];
        if (dd[i].n_events && (n + s.g.nt - 1) % s.g.fs == 0) FD2D_TRY(dft_push(ctx, s.r, s.g, dd[i]));
      }
      par ^= 1;
    }
    timer_end(ctx, ctx->stream, tl, FD2D_TIMER_STEP_V, units, nmax);
    return FD2D_OK;
  };
  return FD2D_OK;
}

fd2d_status fp32_multi_correlation_plan(fd2d_ctx* ctx, const std::vector<const Geometry*>& gs,
                                        const std::vector<const SolveArgs*>& as, LoopPlan& plan) {
  std::vector<MultiSolve> ms(gs.size());
  for (size_t i = 0; i < gs.size(); ++i) {
    ms[i].g = *gs[i];
    ms[i].a = *as[i];
    ms[i].nsteps = gs[i]->ntc;
  }
  MultiLayout L;
  FD2D_TRY(multi_layout(ctx, ms, true, L));
  for (size_t i = 0; i < ms.size(); ++i) {
    MultiSolve& s = ms[i];
    const Geometry& g = s.g;
    ctx->ws_prefix = "m" + std::to_string(i) + ":";
    double *M, *spec;
    FD2D_TRY(interp_dev(ctx, g, &M));
    FD2D_TRY(spectrum_eff(ctx, g, &s.a, 1, &spec));
    for (int n = 1; n <= g.ntc; ++n)
      if (n % g.fs == 0) {
        s.inj.step_of_event.push_back(n);
        s.inj.row_of_event.push_back(n / g.fs - 1);
      }
    const double* xre = s.a.Gin_re;
    const double* xim = s.a.Gin_im;
    const double* sd = s.a.source_dist;
    FD2D_TRY(build_injection(ctx, g, s.r, &xre, &xim, 1.0, spec, M, &sd, s.inj));
    s.seg.inj = s.inj.planes;
    s.seg.inj_chunk = std::max(s.inj.chunk, 1);
    s.seg.nsrc = 0;
  }
  ctx->ws_prefix.clear();
  FD2D_TRY(multi_upload_segs(ctx, ms, L));
  Sig sg;
  sg.add(2);
  sig_multi(sg, ms, L);
  plan.name = "fp32_multi_correlation";
  plan.key = sg.h;
  plan.loop = [ctx, ms, L]() -> fd2d_status {
    std::vector<Injection> ij(ms.size());
    for (size_t i = 0; i < ms.size(); ++i) ij[i] = ms[i].inj;  // the loop's own chunk bookkeeping
    const int nmax = ms[0].nsteps;
    int64_t units = 0;
    for (const auto& s : ms) units += s.g.npts() * s.g.ntc;
    const int tl = timer_begin(ctx, ctx->stream);
    int n_seg = (int)ms.size(), par = 0;
    for (int n = 1; n <= nmax; ++n) {
      while (n_seg > 0 && ms[n_seg - 1].nsteps < n) --n_seg;
      const bool hi = n % L.fs == 0;
      if (hi)
        for (int i = 0; i < n_seg; ++i) {
          int plane = 0;  // the kernel derives it; this makes the event's chunk resident
          if (ij[i].n_events) FD2D_TRY(injection_plane(ctx, ms[i].r, ms[i].g, ij[i], n / L.fs - 1, &plane));
        }
      MultiStep q{};
      q.n = n;
      q.n_seg = n_seg;
      for (int i = 0; i < n_seg; ++i) q.tile0[i] = ms[i].seg.tile0;
      q.fs = L.fs;
      q.green = 0;
      q.Pf = L.Pf;
      for (int m = 0; m < 4; ++m) q.c[m] = L.c[m];
      q.segs = L.segs;
      q.vo = L.v[1 - par];
      q.sxyo = L.sxy[1 - par];
      q.szyo = L.szy[1 - par];
      q.uo = L.u[1 - par];
      q.err = ctx->d_err;
      FD2D_TRY(launch_multi(ctx, L.R, true, hi, q, L.maps[par], L.tiles[n_seg], L.pdl));
      par ^= 1;
    }
    timer_end(ctx, ctx->stream, tl, FD2D_TIMER_STEP_VU, units, nmax);
    return FD2D_OK;
  };
  return FD2D_OK;
}

}  // namespace fd2d

// ---------------------------------------------------------------------------------
// Allocation-free entry point (include/fd2d.h: fd2d_forward1_seismograms_noalloc).
// For callers that must not allocate GPU memory: all working memory of the
// Green-function time loop lives in the statically sized device array below.
// ---------------------------------------------------------------------------------
#include <mutex>

namespace fd2d {
namespace {

// The scratch array.  In host code this name is only a host-side stand-in for
// the device symbol -- never an address to hand to a kernel; its device
// address is looked up with cudaGetSymbolAddress once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[FD2D_NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void* g_noalloc_dev_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up on the
// first call for that device, with the device current).
fd2d_status noalloc_scratch(int dev, unsigned char** out) {
  if (dev < 0 || dev >= kMaxDevices) return set_error(nullptr, FD2D_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_dev_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return set_error(nullptr, FD2D_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    }
    g_noalloc_dev_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_noalloc_dev_ptr[dev]);
  return FD2D_OK;
}

// dt/rho and dt*mu into pitched planes (taper comes from the host).
__global__ void k32_prep_coeffs(const double* mu, const double* rho, double dt, int nx, int nz, int P, float* b,
                                float* dtmu) {
  const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
  if (i >= P || j >= nz) return;
  const int64_t q = i + (int64_t)P * j;
  if (i >= nx) {
    b[q] = dtmu[q] = 0.f;
    return;
  }
  const int64_t p = i + (int64_t)nx * j;
  b[q] = (float)(dt / rho[p]);
  dtmu[q] = (float)(dt * mu[p]);
}

}  // namespace
}  // namespace fd2d

extern "C" fd2d_status fd2d_forward1_seismograms_noalloc(const fd2d_config* cfg, const double* mu,
                                                         const double* rho, const double* src, int32_t ns,
                                                         const double* rec, int32_t nr, double* seismograms,
                                                         void* stream_ptr) {
  using namespace fd2d;
  Geometry g;
  std::string err;
  fd2d_status st = make_geometry(cfg, g, err);
  if (st != FD2D_OK) return set_error(nullptr, st, err);
  if (!mu || !rho) return set_error(nullptr, FD2D_ERR_ARG, "mu and rho are required");
  if (ns < 0 || nr < 0 || (ns && !src) || (nr && !rec) || (nr && !seismograms))
    return set_error(nullptr, FD2D_ERR_ARG, "bad source / receiver arguments");
  const int nx = g.nx, nz = g.nz, P = (nx + 31) / 32 * 32;
  const int64_t ps = ((int64_t)P * nz + 127) / 128 * 128;
  const size_t plane = (size_t)ps * 4;
  const size_t head = 256 + ((((size_t)ns + (size_t)nr) * sizeof(int2) + 255) / 256) * 256;
  const size_t need = head + 9 * plane;
  if (need > FD2D_NOALLOC_SCRATCH_BYTES)
    return set_error(nullptr, FD2D_ERR_SHAPE,
                     "grid needs " + std::to_string(need) + " bytes of scratch; the allocation-free entry point has " +
                         std::to_string((size_t)FD2D_NOALLOC_SCRATCH_BYTES));
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) return set_error(nullptr, FD2D_ERR_NO_DEVICE, cudaGetErrorString(ce));
  unsigned char* base = nullptr;
  FD2D_TRY(noalloc_scratch(dev, &base));
  cudaStream_t stream = static_cast<cudaStream_t>(stream_ptr);
  // carve the scratch: error flag | sources, receivers | 9 planes
  int* d_err = reinterpret_cast<int*>(base);
  int2* src_xy = reinterpret_cast<int2*>(base + 256);
  int2* rec_xy = src_xy + ns;
  float* planes = reinterpret_cast<float*>(base + head);
  Run r;
  r.np = g.npts();
  r.ps = ps;
  r.R = g.r;
  r.G.nx = nx; r.G.nz = nz; r.G.P = P;
  r.G.S = 1; r.G.ps = ps;
  for (int m = 0; m < 4; ++m) r.G.c[m] = (float)g.c[m];
  r.G.inv_dx = (float)(1.0 / g.dx);
  r.G.inv_dz = (float)(1.0 / g.dz);
  r.G.dt = (float)g.dt;
  r.G.err = d_err;
  r.b = planes;
  r.taper = planes + ps;
  r.dtmu = planes + 2 * ps;
  for (int q = 0; q < 2; ++q) {
    r.v[q] = planes + (3 + q) * ps;
    r.sxy[q] = planes + (5 + q) * ps;
    r.szy[q] = planes + (7 + q) * ps;
    r.u[q] = nullptr;
  }
  r.tz = 32;  // no timing here: the allocation-free path keeps one shape
  r.G.t1x0 = 1; r.G.t1x1 = 0; r.G.t1z0 = 1; r.G.t1z1 = 0;  // taper loaded on every tile
  r.G.ntx = (nx + TX - 1) / TX;
  r.G.ntz = (nz + r.tz - 1) / r.tz;
  r.sgrid = dim3(r.G.ntx, r.G.ntz, 1);
  r.pgrid = dim3((P + 31) / 32, (nz + 7) / 8);
  // The array keeps the previous call's contents: clear what must start at zero.
  FD2D_CUDA(nullptr, cudaMemsetAsync(d_err, 0, sizeof(int), stream));
  FD2D_CUDA(nullptr, cudaMemsetAsync(r.v[0], 0, 6 * plane, stream));  // v, sxy, szy of both buffers
  // host-side inputs: taper (pitched FP32), source / receiver nodes
  std::vector<float> taper((size_t)ps, 0.f);
  for (int j = 0; j < nz; ++j)
    for (int i = 0; i < nx; ++i) taper[i + (size_t)P * j] = (float)(*g.absbound)[i + (size_t)nx * j];
  std::vector<int2> xy;
  for (int k = 0; k < ns; ++k) xy.push_back(make_int2(nearest_node(g.x, src[k]), nearest_node(g.z, src[ns + k])));
  for (int k = 0; k < nr; ++k) xy.push_back(make_int2(nearest_node(g.x, rec[k]), nearest_node(g.z, rec[nr + k])));
  FD2D_CUDA(nullptr, cudaMemcpyAsync(r.taper, taper.data(), plane, cudaMemcpyHostToDevice, stream));
  if (!xy.empty())
    FD2D_CUDA(nullptr, cudaMemcpyAsync(src_xy, xy.data(), xy.size() * sizeof(int2), cudaMemcpyHostToDevice, stream));
  k32_prep_coeffs<<<r.pgrid, r.pblock, 0, stream>>>(mu, rho, g.dt, nx, nz, P, r.b, r.dtmu);
  FD2D_CUDA(nullptr, cudaGetLastError());
  FD2D_TRY(step_attributes(nullptr));
  FD2D_TRY(make_maps(nullptr, r));
  for (int n = 1, par = 0; n <= g.nt; ++n, par ^= 1) {
    Step32 s{};
    s.inj_plane = -1;
    s.src_xy = src_xy;
    s.nsrc = ns;
    s.amp_const = 1.0e9f;  // stf = 1.0e9*ones(1,nt), code/run_forward1_green.m:64
    s.rec_xy = rec_xy;
    s.nrec = nr;
    s.seis_col = seismograms + (size_t)nr * (n - 1);
    s.vo = r.v[1 - par];
    s.sxyo = r.sxy[1 - par];
    s.szyo = r.szy[1 - par];
    s.uo = nullptr;
#define FD2D_NOALLOC_STEP(R_)                                                                            \
  k32_step<R_, false, false, 32><<<r.sgrid, Tile<R_, false, false, 32>::NT, Tile<R_, false, false, 32>::BYTES, \
                                   stream>>>(r.G, r.maps[par], s)
    switch (r.R) {
      case 1: FD2D_NOALLOC_STEP(1); break;
      case 2: FD2D_NOALLOC_STEP(2); break;
      case 3: FD2D_NOALLOC_STEP(3); break;
      default: FD2D_NOALLOC_STEP(4); break;
    }
#undef FD2D_NOALLOC_STEP
    FD2D_CUDA(nullptr, cudaGetLastError());
  }
  int herr = 0;
  FD2D_CUDA(nullptr, cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, stream));
  FD2D_CUDA(nullptr, cudaStreamSynchronize(stream));
  if (herr) return set_error(nullptr, FD2D_ERR_TIMEOUT, "a bounded device-side wait gave up");
  return FD2D_OK;
}
