// conv.cuh -- float <-> double conversions without the FP64 pipe.
//
// On GB300 the FP64 pipe executes at 2 lanes per SM per cycle, and the
// hardware F2F conversions between float and double run on it.  The FP32 and
// double-float forms convert every element they read from or write to the
// caller's f64 arrays, so those conversions are done here with integer and
// FP32 operations on the IEEE bit patterns instead.  d2f and f2d are integer
// restatements of IEEE round-to-nearest-even for every input: with a hardware
// conversion kept for the rare cases, the FP64-pipe counters still showed one
// instruction per converted element (the rare path was evaluated on the
// common one).  The
// double-float split and join below keep a hardware path for values outside
// their bit paths' ranges.
//
// The same source compiles for the host (g++) so that tests/test_conv.py can
// check every path against the compiler's own conversions.
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

#if defined(__CUDACC__)
#define GBFFT_HD __host__ __device__ __forceinline__
#else
#define GBFFT_HD inline
#endif

namespace gbfft {
namespace conv {

GBFFT_HD uint64_t dbits(double x) {
  uint64_t b;
  memcpy(&b, &x, 8);
  return b;
}
GBFFT_HD double bitsd(uint64_t b) {
  double x;
  memcpy(&x, &b, 8);
  return x;
}
GBFFT_HD uint32_t fbits(float x) {
  uint32_t b;
  memcpy(&b, &x, 4);
  return b;
}
GBFFT_HD float bitsf(uint32_t b) {
  float x;
  memcpy(&x, &b, 4);
  return x;
}

GBFFT_HD uint32_t clz32(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__clz((int)v);
#else
  return v ? (uint32_t)__builtin_clz(v) : 32u;
#endif
}

// d2f for the biased exponents outside 897..1150 (infinities, NaNs,
// overflow, subnormal and zero results); returns the float's bits without
// the sign.  Integer operations only, so that no conversion instruction can be
// hoisted out of the rare branch into the common path.
GBFFT_HD uint32_t d2f_rare(uint32_t hw, uint32_t lw, uint32_t ex) {
  if (ex == 0x7FFu) {
    // infinity, or a NaN made quiet with its top fraction bits kept
    const uint32_t frac = ((hw & 0xFFFFFu) << 3) | (lw >> 29);
    return (((hw & 0xFFFFFu) | lw) != 0u) ? (0x7FC00000u | frac) : 0x7F800000u;
  }
  if (ex > 1150u) return 0x7F800000u;  // rounds to infinity
  // The value is S * 2^(ex - 1075) with S = 2^52 + fraction; in units of the
  // smallest subnormal float 2^-149 it is S / 2^(926 - ex), below one half
  // for ex < 873 (double subnormals and zero included).
  if (ex < 873u) return 0u;
  const uint64_t S = ((uint64_t)((hw & 0xFFFFFu) | 0x100000u) << 32) | lw;
  const uint32_t sh = 926u - ex;  // 30..53
  const uint64_t q = S >> sh;
  const uint64_t rem = S & ((1ull << sh) - 1ull);
  const uint64_t half = 1ull << (sh - 1u);
  const uint32_t up = (uint32_t)(rem > half) | ((uint32_t)(rem == half) & (uint32_t)(q & 1u));
  // q + up = 2^23 is the smallest normal float, as IEEE rounding gives
  return (uint32_t)q + up;
}

// double -> float, round to nearest even, for every input.  The common case
// (a normal float result, biased double exponent 897..1150 before rounding)
// is a handful of integer operations.
GBFFT_HD float d2f(double x) {
  const uint64_t b = dbits(x);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const uint32_t ex = (hw >> 20) & 0x7FFu;
  uint32_t r;
  if (ex - 897u <= 253u) {
    const uint32_t mant = ((hw & 0xFFFFFu) << 3) | (lw >> 29);  // top 23 fraction bits
    const uint32_t rest = lw & 0x1FFFFFFFu;                       // 29 dropped bits
    const uint32_t up = (rest > 0x10000000u) | ((rest == 0x10000000u) & (mant & 1u));
    // a carry out of the fraction bumps the exponent, as IEEE rounding does;
    // 1150 + carry gives 0x7F800000 (infinity), also as IEEE rounding does
    r = ((ex - 896u) << 23) + mant + up;
  } else {
    r = d2f_rare(hw, lw, ex);
  }
  return bitsf((hw & 0x80000000u) | r);
}

// f2d for zeros, subnormals, infinities and NaNs (NaNs made quiet); writes
// the double's high and low words without the sign.
GBFFT_HD void f2d_rare(uint32_t e8, uint32_t frac, uint32_t& hw, uint32_t& lw) {
  if (e8 == 0xFFu) {
    hw = 0x7FF00000u | (frac >> 3) | (frac ? 0x80000u : 0u);
    lw = frac << 29;
    return;
  }
  if (frac == 0u) {
    hw = 0u;
    lw = 0u;
    return;
  }
  // subnormal: frac * 2^-149 with its leading one at bit p
  const uint32_t p = 31u - clz32(frac);  // 0..22
  const uint32_t m = frac << (23u - p);  // leading one at bit 23
  hw = ((p + 874u) << 20) | ((m & 0x7FFFFFu) >> 3);
  lw = m << 29;
}

// float -> double, exact, for every input.
GBFFT_HD double f2d(float x) {
  const uint32_t f = fbits(x);
  const uint32_t e8 = (f >> 23) & 0xFFu;
  const uint32_t frac = f & 0x7FFFFFu;
  uint32_t hw, lw;
  if (e8 - 1u < 254u) {
    hw = ((e8 + 896u) << 20) | (frac >> 3);
    lw = frac << 29;
  } else {
    f2d_rare(e8, frac, hw, lw);
  }
  return bitsd(((uint64_t)((f & 0x80000000u) | hw) << 32) | lw);
}

// Exact value of a 29-bit unsigned integer r, rounded to float (two magic-number
// conversions of 23-bit halves and one FMA).
GBFFT_HD float u29_to_f(uint32_t r) {
  const float lo = bitsf(0x4B000000u | (r & 0x7FFFFFu)) - 8388608.0f;  // exact
  const float hi = bitsf(0x4B000000u | (r >> 23)) - 8388608.0f;        // exact
  return fmaf(hi, 8388608.0f, lo);
}

// double -> (hi, lo) floats with hi + lo = x to about 48 bits: hi keeps the
// top 24 significand bits (truncated), lo the remaining 29 rounded to a float.
// Bit path for biased exponents 949..1150, where hi is a normal float and lo's
// scale 2^(ex-1075) is a normal float too.
GBFFT_HD void d2df(double x, float& hi, float& lo) {
  const uint64_t b = dbits(x);
  const uint32_t hw = (uint32_t)(b >> 32), lw = (uint32_t)b;
  const uint32_t ex = (hw >> 20) & 0x7FFu;
  if (ex < 949u || ex > 1150u) {
    hi = (float)x;
    lo = (float)(x - (double)hi);
    return;
  }
  const uint32_t sign = hw & 0x80000000u;
  hi = bitsf(sign | ((((hw & 0x7FFFFFFFu) - (896u << 20)) << 3) | (lw >> 29)));
  const float scale = bitsf((ex - 948u) << 23);  // 2^(ex - 1075)
  const float l = u29_to_f(lw & 0x1FFFFFFFu) * scale;
  lo = sign ? -l : l;
}

// (hi, lo) -> nearest-ish double of hi + lo (error below 2^-53 |hi| plus the
// rounding of lo's offset, i.e. well inside the pair's own ~2^-48 precision).
// Bit path: hi a normal float with a non-zero fraction or lo of the same sign
// (so the sum stays in hi's binade), and |lo| small against hi.
GBFFT_HD double df2d(float hi, float lo) {
  const uint32_t h = fbits(hi), l = fbits(lo);
  const uint32_t eh = (h >> 23) & 0xFFu;
  const uint32_t el = (l >> 23) & 0xFFu;
  const bool same = ((h ^ l) & 0x80000000u) == 0u;
  if (eh < 53u || eh == 0xFFu || el == 0xFFu || ((h & 0x7FFFFFu) == 0u && !same) ||
      (el != 0u && el + 24u > eh)) {
    return (double)hi + (double)lo;
  }
  // double bits of hi
  const uint64_t hb = ((uint64_t)((h & 0x80000000u) | ((eh + 896u) << 20) | ((h & 0x7FFFFFu) >> 3))
                       << 32) | ((uint64_t)(h & 7u) << 29);
  if (el == 0u) return bitsd(hb);  // lo is zero (or a subnormal far below hi's ulp)
  // lo in units of hi's double ulp 2^(eh-179): an exact power-of-two scaling,
  // 0 <= kf < 2^29 because lo sits at least 24 binades below hi
  const float kf = fabsf(lo) * bitsf((306u - eh) << 23);
  // kf to an integer k: nearest below 2^22 (the 1.5*2^23 magic number);
  // above, from its bits (toward zero, an error under one double ulp of hi)
  uint32_t k;
  if (kf < 4194304.0f) {
    k = fbits(kf + 12582912.0f) - 0x4B400000u;
  } else {
    const uint32_t kb = fbits(kf);
    const int sh = (int)((kb >> 23) & 0xFFu) - 150;
    const uint32_t m = (kb & 0x7FFFFFu) | 0x800000u;
    k = sh >= 0 ? (m << sh) : (m >> (-sh));
  }
  // hb's low 29 bits are zero and k < 2^29: no carry or borrow leaves them
  // except the borrow of hb - k, which stays inside hi's binade because hi's
  // fraction is non-zero on that path
  return bitsd(same ? hb + k : hb - k);
}

}  // namespace conv
}  // namespace gbfft
