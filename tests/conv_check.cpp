// Host check of numrs_gb300/csrc/conv.cuh against the compiler's conversions.
// Built and run by tests/test_conv.py; prints "ok" or the first mismatch.
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cmath>
#include "conv.cuh"

using namespace gbfft::conv;

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t next() {  // splitmix64
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int main(int argc, char** argv) {
  long n = argc > 1 ? atol(argv[1]) : 2000000;
  for (long i = 0; i < n; ++i) {
    // random doubles: random bits (all exponents) and random scaled normals
    double x = (i & 1) ? bitsd(next()) : ldexp((double)(int64_t)next() / 9.2e18, (int)(next() % 300) - 150);
    // every other draw: a double near or below the float subnormal range
    if ((i & 3) == 2) x = ldexp((double)(int64_t)next() / 9.2e18, -120 - (int)(next() % 40));
    // NaNs included: both conversions make them quiet and keep the top
    // payload bits, as the host's IEEE conversions do
    float a = d2f(x), b = (float)x;
    if (fbits(a) != fbits(b)) {
      printf("d2f mismatch %a -> %a vs %a\n", x, a, b);
      return 1;
    }
    // random float bits, every fourth one a subnormal, zero or non-finite
    uint32_t fb = (uint32_t)next();
    if ((i & 3) == 1) fb &= 0x807FFFFFu;
    if ((i & 7) == 3) fb |= 0x7F800000u;
    float f = bitsf(fb);
    {
      double c = f2d(f), e = (double)f;
      if (dbits(c) != dbits(e)) {
        printf("f2d mismatch %a -> %a vs %a\n", f, c, e);
        return 1;
      }
    }
    if (std::isfinite(x) && std::fabs(x) < 1e38 && std::fabs(x) > 1e-30) {
      float hi, lo;
      d2df(x, hi, lo);
      double back = (double)hi + (double)lo;
      if (std::fabs(back - x) > std::ldexp(std::fabs(x), -47)) {
        printf("d2df error %a -> %a + %a\n", x, hi, lo);
        return 1;
      }
      // renormalise like the double-float arithmetic does, then convert back
      float s2 = hi + lo, e2 = lo - (s2 - hi);
      double d = df2d(s2, e2), want = (double)s2 + (double)e2;
      if (std::fabs(d - want) > std::ldexp(std::fabs(want), -51)) {
        printf("df2d error (%a, %a) -> %a vs %a\n", s2, e2, d, want);
        return 1;
      }
      // opposite-sign and power-of-two corner cases
      float p2 = std::ldexp(1.0f, (int)(next() % 200) - 100);
      float t = -std::ldexp(p2, -30) * (float)(next() % 1000) / 1000.0f;
      double d3 = df2d(p2, t), w3 = (double)p2 + (double)t;
      if (std::fabs(d3 - w3) > std::ldexp(std::fabs(w3), -51)) {
        printf("df2d corner (%a, %a) -> %a vs %a\n", p2, t, d3, w3);
        return 1;
      }
    }
  }
  // exact corner values: zeros, infinities, the float range limits and the
  // halfway points around them
  const double corners[] = {0.0, -0.0, HUGE_VAL, -HUGE_VAL, 3.4028234663852886e38,
                            3.4028235677973366e38, 3.4028235677973362e38, 1.1754943508222875e-38,
                            1.1754942807573643e-38, 1.401298464324817e-45, 7.006492321624085e-46,
                            7.006492321624087e-46, 2.1019476964872256e-45, 4.9406564584124654e-324};
  for (double c : corners) {
    for (int sgn = 0; sgn < 2; ++sgn) {
      const double x = sgn ? -c : c;
      if (fbits(d2f(x)) != fbits((float)x)) {
        printf("d2f corner mismatch %a\n", x);
        return 1;
      }
    }
  }
  printf("ok\n");
  return 0;
}
