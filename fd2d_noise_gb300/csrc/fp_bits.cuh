// fp_bits.cuh -- FP32 <-> FP64 conversions with integer operations.
//
// On this part the FP64 pipe is narrow (a few operations per clock per SM), and
// the hardware conversion instructions run on it.  Kernels that convert every
// element (the FP64 spectra written by the DFT, the FP32 injection planes made
// from FP64 spectra) use these bit-level versions instead: exact widening and
// round-to-nearest-even narrowing of normal numbers (zeros, subnormals,
// infinities, NaNs and out-of-range values fall back to the hardware
// conversion there; the widening handles every class with integers).  Host-compilable so the rounding can be checked on the CPU.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define FD2D_HD __host__ __device__ __forceinline__
#else
#define FD2D_HD inline
#endif

namespace fd2d {

FD2D_HD uint32_t f32_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}

FD2D_HD float f32_from(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}

FD2D_HD uint64_t f64_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

FD2D_HD double f64_from(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

FD2D_HD int clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return __clz((int)v);
#else
  return v ? __builtin_clz(v) : 32;
#endif
}

// Exact FP32 -> FP64, integer operations only (every class: signed zeros,
// subnormals normalised, infinities, NaNs quietened with their payload).
FD2D_HD double widen_exact(float x) {
  const uint32_t u = f32_bits(x);
  const uint32_t e = (u >> 23) & 0xFFu;
  uint32_t m = u & 0x7FFFFFu;
  uint64_t eb;
  if (e == 0xFFu) {
    eb = 0x7FFu;
    if (m) m |= 0x400000u;  // quiet NaN
  } else if (e != 0) {
    eb = e + 896u;          // rebias 127 -> 1023
  } else if (m == 0) {
    eb = 0;                 // signed zero
  } else {
    // subnormal m * 2^-149 with its leading one at bit p: exponent p - 149
    const int p = 31 - clz32(m);
    eb = (uint64_t)(p + 874);
    m = (m << (23 - p)) & 0x7FFFFFu;
  }
  return f64_from(((uint64_t)(u & 0x80000000u) << 32) | (eb << 52) | ((uint64_t)m << 29));
}

// FP64 -> FP32, round to nearest, ties to even (the C conversion).
FD2D_HD float narrow_rn(double x) {
  const uint64_t u = f64_bits(x);
  const int e = (int)((u >> 52) & 0x7FFu) - 1023 + 127;  // FP32 biased exponent
  if (e <= 0 || e >= 0xFF) return (float)x;               // zero, subnormal, inf, nan, out of range
  const uint64_t m = u & 0xFFFFFFFFFFFFFull;              // 52 mantissa bits
  uint32_t keep = (uint32_t)(m >> 29);                    // 23 bits
  const uint64_t rem = m & 0x1FFFFFFFull;                 // 29 dropped bits
  const uint64_t half = 0x10000000ull;
  uint32_t ef = (uint32_t)e;
  if (rem > half || (rem == half && (keep & 1u))) {
    if (++keep == 0x800000u) {  // mantissa overflow: next binade
      keep = 0;
      if (++ef == 0xFFu) return (float)x;
    }
  }
  return f32_from(((uint32_t)(u >> 32) & 0x80000000u) | (ef << 23) | keep);
}

}  // namespace fd2d
