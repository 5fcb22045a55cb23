// Checks the bit-level conversions of fd2d_noise_gb300/csrc/fp_bits.cuh against
// the C conversions on random and hand-picked values (ties, binade edges).
#include <cmath>
#include <cstdio>
#include <limits>
#include <random>

#include "fp_bits.cuh"

int main() {
  using namespace fd2d;
  std::mt19937_64 rng(12345);
  long bad = 0, n = 0;
  auto check_d = [&](double x) {
    ++n;
    const float a = narrow_rn(x), b = (float)x;
    if (f32_bits(a) != f32_bits(b) && !(std::isnan(a) && std::isnan(b))) {
      if (bad < 5) std::printf("narrow %.17g: %a vs %a\n", x, a, b);
      ++bad;
    }
  };
  auto check_f = [&](float x) {
    ++n;
    const double a = widen_exact(x), b = (double)x;
    if (f64_bits(a) != f64_bits(b) && !(std::isnan(a) && std::isnan(b))) {
      if (bad < 5) std::printf("widen %a\n", x);
      ++bad;
    }
  };
  for (int i = 0; i < 4000000; ++i) {
    const uint64_t r = rng();
    double x;
    std::memcpy(&x, &r, 8);
    check_d(x);
    const uint32_t s = (uint32_t)(r >> 11);
    float f;
    std::memcpy(&f, &s, 4);
    check_f(f);
    // values near FP32 ties: a float plus exactly half an FP32 ulp, +- 1 ulp of FP64
    const float g = (float)std::ldexp((double)(r % 1000003) + 1.0, (int)(r % 200) - 100);
    const double ulp = std::nextafter((double)g, 1e300) - (double)g;
    const double tie = (double)g + std::ldexp(1.0, std::ilogb(g) - 24);
    check_d(tie);
    check_d(tie + ulp);
    check_d(tie - ulp);
    check_d(-tie);
  }
  const double special[] = {0.0, -0.0, 1e-45, 1e-40, 3.4028234663852886e38, 3.4028235677973366e38, 1e300,
                            -1e300, std::numeric_limits<double>::infinity(), std::nan(""), 1.17549435e-38,
                            1.1754942e-38, 0.999999999, 1.0, 16777217.0, 16777219.0};
  for (double x : special) check_d(x);
  const float fspecial[] = {0.0f, -0.0f, 1e-45f, -1e-45f, 1e-40f, 5.8774718e-39f, 1.1754942e-38f, 1.17549435e-38f,
                            3.4028235e38f, std::numeric_limits<float>::infinity(),
                            -std::numeric_limits<float>::infinity(), std::nanf("")};
  for (float x : fspecial) check_f(x);
  for (uint32_t m = 1; m < 0x800000u; m += 997) {  // subnormals across every leading-one position
    float f;
    std::memcpy(&f, &m, 4);
    check_f(f);
    check_f(-f);
  }
  std::printf("%s %ld of %ld\n", bad ? "FAIL" : "ok", bad, n);
  return bad ? 1 : 0;
}
