// arith.cuh -- complex arithmetic for the three CUDA-core precision forms.
//
//   F64   IEEE double throughout (the reference's arithmetic type).
//   F32   IEEE float, inputs and outputs converted at the boundary.
//   DF64  "double-float": each real is an unevaluated sum hi+lo of two floats
//         (about 48 significand bits).  On GB300 the FP64 pipe runs at about
//         1/61 of the FP32 rate, so compensated FP32 pairs reach FP64-class
//         accuracy (relative L2 ~1e-14 on FFTs) at several times the FP64
//         throughput.  The algorithms are the classic error-free
//         transformations: TwoSum (Knuth), FastTwoSum (Dekker) and TwoProd via
//         a fused multiply-add.
//
// Every form exposes the same static interface so one kernel template serves
// all of them:
//   C            register complex type
//   S            shared-memory element (16 or 8 bytes)
//   TW           twiddle-table element
//   add/sub/mul/mulc/mul_j/scale, to_s/from_s, ld_tw
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "conv.cuh"

namespace gbfft {

struct alignas(16) d2 { double x, y; };
struct alignas(8) f2 { float x, y; };
struct alignas(16) f4 { float x, y, z, w; };  // (re.hi, re.lo, im.hi, im.lo)

// ---------------------------------------------------------------------------
// F64
// ---------------------------------------------------------------------------
struct F64 {
  static constexpr int kind = 0;
  static constexpr bool kTensor = false;
  using real = double;
  struct C { double x, y; };
  using S = d2;
  using TW = d2;
  static constexpr int kPadShift = 4;  // one pad slot per 16 elements of 16 B
  __device__ __forceinline__ static C make(double a, double b) { return {a, b}; }
  __device__ __forceinline__ static C add(C a, C b) { return {a.x + b.x, a.y + b.y}; }
  __device__ __forceinline__ static C sub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
  // a * w
  __device__ __forceinline__ static C mul(C a, C w) {
    return {fma(a.x, w.x, -a.y * w.y), fma(a.x, w.y, a.y * w.x)};
  }
  // a * (c + i s) for constants c, s
  __device__ __forceinline__ static C mulcs(C a, double c, double s) {
    return {fma(a.x, c, -a.y * s), fma(a.x, s, a.y * c)};
  }
  // a * (c + i*c)*sgn-style: (a.x - sg*a.y)*h, (a.y + sg*a.x)*h -- the 45-degree rotations
  __device__ __forceinline__ static C rot45(C a, double h, int sg) {
    return sg > 0 ? C{(a.x - a.y) * h, (a.y + a.x) * h} : C{(a.x + a.y) * h, (a.y - a.x) * h};
  }
  // a * (sg * i)
  __device__ __forceinline__ static C mul_j(C a, int sg) {
    return sg > 0 ? C{-a.y, a.x} : C{a.y, -a.x};
  }
  __device__ __forceinline__ static C scale(C a, double s) { return {a.x * s, a.y * s}; }
  __device__ __forceinline__ static C conj(C a) { return {a.x, -a.y}; }
  __device__ __forceinline__ static S to_s(C a) { return {a.x, a.y}; }
  __device__ __forceinline__ static C from_s(S s) { return {s.x, s.y}; }
  __device__ __forceinline__ static C from_d(double a, double b) { return {a, b}; }
  __device__ __forceinline__ static void to_d(C a, double& x, double& y) { x = a.x; y = a.y; }
  __device__ __forceinline__ static C ld_tw(const TW* p, int sg) {
    d2 t = *p;
    return {t.x, sg > 0 ? t.y : -t.y};
  }
  __device__ __forceinline__ static double re(C a) { return a.x; }
  __device__ __forceinline__ static double im(C a) { return a.y; }
  __device__ __forceinline__ static real rmake(double v) { return v; }
};

// ---------------------------------------------------------------------------
// F32
// ---------------------------------------------------------------------------
struct F32 {
  static constexpr int kind = 1;
  static constexpr bool kTensor = false;
  using real = float;
  struct C { float x, y; };
  using S = f2;
  using TW = f2;
  static constexpr int kPadShift = 5;
  __device__ __forceinline__ static C add(C a, C b) { return {a.x + b.x, a.y + b.y}; }
  __device__ __forceinline__ static C sub(C a, C b) { return {a.x - b.x, a.y - b.y}; }
  __device__ __forceinline__ static C mul(C a, C w) {
    return {fmaf(a.x, w.x, -a.y * w.y), fmaf(a.x, w.y, a.y * w.x)};
  }
  __device__ __forceinline__ static C mulcs(C a, double c, double s) {
    const float cf = (float)c, sf = (float)s;
    return {fmaf(a.x, cf, -a.y * sf), fmaf(a.x, sf, a.y * cf)};
  }
  __device__ __forceinline__ static C rot45(C a, double h, int sg) {
    const float hf = (float)h;
    return sg > 0 ? C{(a.x - a.y) * hf, (a.y + a.x) * hf} : C{(a.x + a.y) * hf, (a.y - a.x) * hf};
  }
  __device__ __forceinline__ static C mul_j(C a, int sg) {
    return sg > 0 ? C{-a.y, a.x} : C{a.y, -a.x};
  }
  __device__ __forceinline__ static C scale(C a, double s) {
    const float sf = (float)s;
    return {a.x * sf, a.y * sf};
  }
  __device__ __forceinline__ static C conj(C a) { return {a.x, -a.y}; }
  __device__ __forceinline__ static S to_s(C a) { return {a.x, a.y}; }
  __device__ __forceinline__ static C from_s(S s) { return {s.x, s.y}; }
  // conversions on the integer/FP32 pipes (conv.cuh), not GB300's FP64 pipe
  __device__ __forceinline__ static C from_d(double a, double b) {
    return {conv::d2f(a), conv::d2f(b)};
  }
  __device__ __forceinline__ static void to_d(C a, double& x, double& y) {
    x = conv::f2d(a.x);
    y = conv::f2d(a.y);
  }
  __device__ __forceinline__ static C ld_tw(const TW* p, int sg) {
    f2 t = *p;
    return {t.x, sg > 0 ? t.y : -t.y};
  }
  __device__ __forceinline__ static float re(C a) { return a.x; }
  __device__ __forceinline__ static float im(C a) { return a.y; }
};

// ---------------------------------------------------------------------------
// DF64: double-float pairs
// ---------------------------------------------------------------------------
struct df { float hi, lo; };

// Error-free transformations (round-to-nearest intrinsics are never contracted).
__device__ __forceinline__ df two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}
// Sum of two double-floats.  The normwise error bound (relative to |a|+|b|) is
// what FFT accuracy needs, so the cheaper "sloppy" form is used: one TwoSum on
// the high parts, the low parts added in, one renormalisation.
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
// a*b with TwoProd through FMA; the cross terms are accumulated with FMAs.
__device__ __forceinline__ df df_mul(df a, df b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
// a*b - c*d evaluated as one compensated dot product (used by complex multiply).
__device__ __forceinline__ df df_mul_sub(df a, df b, df c, df d) {
  float p1 = __fmul_rn(a.hi, b.hi);
  float e1 = __fmaf_rn(a.hi, b.hi, -p1);
  float p2 = __fmul_rn(c.hi, d.hi);
  float e2 = __fmaf_rn(c.hi, d.hi, -p2);
  df s = two_sum(p1, -p2);
  float e = __fsub_rn(e1, e2);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  e = __fmaf_rn(-c.hi, d.lo, e);
  e = __fmaf_rn(-c.lo, d.hi, e);
  e = __fadd_rn(e, s.lo);
  return fast_two_sum(s.hi, e);
}
__device__ __forceinline__ df df_mul_add(df a, df b, df c, df d) {
  return df_mul_sub(a, b, df_neg(c), d);
}
__device__ __forceinline__ df df_scale_f(df a, float s) {  // s exact float constant
  float p = __fmul_rn(a.hi, s);
  float e = __fmaf_rn(a.hi, s, -p);
  e = __fmaf_rn(a.lo, s, e);
  return fast_two_sum(p, e);
}
// conversions on the integer/FP32 pipes (conv.cuh), not GB300's FP64 pipe
__device__ __forceinline__ df df_from_double(double v) {
  df r;
  conv::d2df(v, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ double df_to_double(df a) { return conv::df2d(a.hi, a.lo); }

struct DF64 {
  static constexpr int kind = 2;
  static constexpr bool kTensor = false;
  using real = df;
  struct C { df x, y; };
  using S = f4;
  using TW = f4;
  static constexpr int kPadShift = 4;
  __device__ __forceinline__ static C add(C a, C b) { return {df_add(a.x, b.x), df_add(a.y, b.y)}; }
  __device__ __forceinline__ static C sub(C a, C b) { return {df_sub(a.x, b.x), df_sub(a.y, b.y)}; }
  __device__ __forceinline__ static C mul(C a, C w) {
    return {df_mul_sub(a.x, w.x, a.y, w.y), df_mul_add(a.x, w.y, a.y, w.x)};
  }
  // constants c, s are split into double-float at compile time by the caller
  __device__ __forceinline__ static C mulcs(C a, double c, double s) {
    df cd = {(float)c, (float)(c - (double)(float)c)};
    df sd = {(float)s, (float)(s - (double)(float)s)};
    return {df_mul_sub(a.x, cd, a.y, sd), df_mul_add(a.x, sd, a.y, cd)};
  }
  __device__ __forceinline__ static C rot45(C a, double h, int sg) {
    df hd = {(float)h, (float)(h - (double)(float)h)};
    if (sg > 0) return {df_mul(df_sub(a.x, a.y), hd), df_mul(df_add(a.y, a.x), hd)};
    return {df_mul(df_add(a.x, a.y), hd), df_mul(df_sub(a.y, a.x), hd)};
  }
  __device__ __forceinline__ static C mul_j(C a, int sg) {
    return sg > 0 ? C{df_neg(a.y), a.x} : C{a.y, df_neg(a.x)};
  }
  __device__ __forceinline__ static C scale(C a, double s) {
    // only exact powers of two or small exact floats are passed here
    float sf = (float)s;
    return {df_scale_f(a.x, sf), df_scale_f(a.y, sf)};
  }
  __device__ __forceinline__ static C conj(C a) { return {a.x, df_neg(a.y)}; }
  __device__ __forceinline__ static S to_s(C a) { return {a.x.hi, a.x.lo, a.y.hi, a.y.lo}; }
  __device__ __forceinline__ static C from_s(S s) { return {{s.x, s.y}, {s.z, s.w}}; }
  __device__ __forceinline__ static C from_d(double a, double b) {
    return {df_from_double(a), df_from_double(b)};
  }
  __device__ __forceinline__ static void to_d(C a, double& x, double& y) {
    x = df_to_double(a.x);
    y = df_to_double(a.y);
  }
  __device__ __forceinline__ static C ld_tw(const TW* p, int sg) {
    f4 t = *p;
    C w = {{t.x, t.y}, {t.z, t.w}};
    if (sg < 0) w.y = df_neg(w.y);
    return w;
  }
};

// ---------------------------------------------------------------------------
// TC32: FP32 storage and CUDA-core arithmetic, with every radix-16 sub-pass
// done on the tensor cores as a 3xTF32 DFT-matrix product (tc16.cuh).
// ---------------------------------------------------------------------------
struct TC32 : F32 {
  static constexpr bool kTensor = true;
};

}  // namespace gbfft
