// tc16.cuh -- radix-16 Stockham sub-pass on the tensor cores.
//
// A radix-16 sub-pass applies the 16-point DFT to many columns at once, i.e.
// it is the product of the 16x16 complex DFT matrix F with a 16 x NB matrix X
// of butterfly inputs.  In real arithmetic
//
//     [Yr]   [Fr  -Fi] [Xr]          Fr[k][t] = cos(2 pi k t / 16)
//     [Yi] = [Fi   Fr] [Xi],         Fi[k][t] = SG sin(2 pi k t / 16)
//
// which is computed as Yr = Fr Xr + Fi (-Xi) and Yi = Fi Xr + Fr Xi with
// warp-level mma.sync m16n8k8 TF32 products accumulated in FP32.  TF32 keeps
// 11 significand bits, so every operand is split as hi + lo (both TF32) and
// each product is the three-term sum hi*hi + hi*lo + lo*hi ("3xTF32"), which
// recovers about 22 bits -- close to FP32 accuracy.  Twiddles between
// sub-passes stay on the CUDA cores in FP32.
//
// Fragment layouts of m16n8k8 .tf32 (PTX ISA): with g = lane / 4 and
// q = lane % 4,
//   A (16x8, row): a0 (g, q)  a1 (g+8, q)  a2 (g, q+4)  a3 (g+8, q+4)
//   B (8x8, col):  b0 (q, g)  b1 (q+4, g)
//   C (16x8):      c0 (g, 2q) c1 (g, 2q+1) c2 (g+8, 2q) c3 (g+8, 2q+1)
#pragma once
#include "arith.cuh"
#include "gbfft_internal.h"

namespace gbfft {

__device__ __forceinline__ uint32_t tf32_of(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_of(x);
  lo = tf32_of(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4],
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// The A fragments of Fr and Fi for the two k-blocks (t in [0,8) and [8,16)),
// hi and lo parts, built from the FP32 twiddle table (level 16).
struct Dft16Frags {
  uint32_t fr_hi[2][4], fr_lo[2][4], fi_hi[2][4], fi_lo[2][4];
};

template <int SG>
__device__ __forceinline__ void dft16_frags(const f2* tw_dense, Dft16Frags& fr) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, q = lane & 3;
#pragma unroll
  for (int kb = 0; kb < 2; ++kb) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int row = g + ((r & 1) ? 8 : 0);
      const int col = 8 * kb + q + ((r & 2) ? 4 : 0);
      const f2 w = tw_dense[16 + ((row * col) & 15)];
      split_tf32(w.x, fr.fr_hi[kb][r], fr.fr_lo[kb][r]);
      split_tf32(SG > 0 ? w.y : -w.y, fr.fi_hi[kb][r], fr.fi_lo[kb][r]);
    }
  }
}

// Y += A * B with the three-term split product.
__device__ __forceinline__ void mma3(float (&d)[4], const uint32_t (&ahi)[4],
                                     const uint32_t (&alo)[4], uint32_t bh0, uint32_t bh1,
                                     uint32_t bl0, uint32_t bl1) {
  mma_tf32(d, alo, bh0, bh1);
  mma_tf32(d, ahi, bl0, bl1);
  mma_tf32(d, ahi, bh0, bh1);
}

// The 16-point DFTs of 8 butterflies: lane (g, q) supplies inputs t = q + 4i
// (i < 4) of butterfly g as xr/xi and receives outputs k = g, g + 8 of
// butterflies 2q, 2q + 1 in dr/di (the C fragment layout).  Each output is the
// FP32 (round-to-nearest) sum of four product chains, one per matrix (Fr, Fi)
// and k-block, each accumulated on the tensor cores from zero.  The tensor
// cores' accumulation rounding, which is not round-to-nearest, then compounds
// over 3 products per chain instead of 12: measured, this cuts the form's
// error about 3x.
__device__ __forceinline__ void dft16_tc_products(const Dft16Frags& A, const float (&xr)[4],
                                                  const float (&xi)[4], float (&dr)[4],
                                                  float (&di)[4]) {
  // B fragments: k-block 0 holds t = q, q+4 (b0, b1); k-block 1 t = q+8, q+12
  uint32_t rh[4], rl[4], ih[4], il[4], nh[4], nl[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    split_tf32(xr[i], rh[i], rl[i]);
    split_tf32(xi[i], ih[i], il[i]);
    // round-to-nearest-away is symmetric: the split of -x is the negated split of x
    nh[i] = ih[i] ^ 0x80000000u;
    nl[i] = il[i] ^ 0x80000000u;
  }
  float c[8][4];
#pragma unroll
  for (int k = 0; k < 8; ++k)
#pragma unroll
    for (int r = 0; r < 4; ++r) c[k][r] = 0.f;
  // Yr = Fr Xr + Fi (-Xi);  Yi = Fi Xr + Fr Xi; one chain per matrix and k-block
  mma3(c[0], A.fr_hi[0], A.fr_lo[0], rh[0], rh[1], rl[0], rl[1]);
  mma3(c[1], A.fr_hi[1], A.fr_lo[1], rh[2], rh[3], rl[2], rl[3]);
  mma3(c[2], A.fi_hi[0], A.fi_lo[0], nh[0], nh[1], nl[0], nl[1]);
  mma3(c[3], A.fi_hi[1], A.fi_lo[1], nh[2], nh[3], nl[2], nl[3]);
  mma3(c[4], A.fi_hi[0], A.fi_lo[0], rh[0], rh[1], rl[0], rl[1]);
  mma3(c[5], A.fi_hi[1], A.fi_lo[1], rh[2], rh[3], rl[2], rl[3]);
  mma3(c[6], A.fr_hi[0], A.fr_lo[0], ih[0], ih[1], il[0], il[1]);
  mma3(c[7], A.fr_hi[1], A.fr_lo[1], ih[2], ih[3], il[2], il[3]);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    dr[r] = (c[0][r] + c[1][r]) + (c[2][r] + c[3][r]);
    di[r] = (c[4][r] + c[5][r]) + (c[6][r] + c[7][r]);
  }
}

// One radix-16 Stockham sub-pass over C columns of R points in shared memory
// (layout and index rules as subpass<F, SG, 16> in fft_core.cuh).  Each warp
// takes 32 consecutive butterflies in four chunks of 8 (the mma N dimension).
template <int SG>
__device__ __forceinline__ void subpass16_tc(f2* sm, int logR, int cs, int logNs,
                                             const Twiddles& tw, const Dft16Frags& A, int tid) {
  constexpr int sh = 5;  // FP32 shared-memory padding (F32::kPadShift)
  const int lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int logRQ = logR - 4;
  const int RQ = 1 << logRQ;
  const int Ns = 1 << logNs;
  const f2* twd = reinterpret_cast<const f2*>(tw.dense);
  // outputs held across the barrier: 4 chunks x (k = g, g+8) x (cols 2q, 2q+1)
  float yr[4][4], yi[4][4];
  int ocol[4][2], orow[4][2];
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    // this thread's inputs: butterfly g of the chunk, elements t = q + 4i
    const int b = warp * 32 + ch * 8 + g;
    const int c = b >> logRQ;
    const int j = b & (RQ - 1);
    const int cb = c * cs;
    const int jm = j & (Ns - 1);
    float xr[4], xi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int t = q + 4 * i;
      f2 v = sm[cb + pidx(j + t * RQ, sh)];
      if (logNs > 0 && jm != 0 && t != 0) {
        const f2 w = twd[(1 << (logNs + 4)) + ((jm * t) & ((Ns << 4) - 1))];
        const float wy = SG > 0 ? w.y : -w.y;
        const float re = fmaf(v.x, w.x, -v.y * wy);
        const float im = fmaf(v.x, wy, v.y * w.x);
        v.x = re;
        v.y = im;
      }
      xr[i] = v.x;
      xi[i] = v.y;
    }
    float dr[4], di[4];
    dft16_tc_products(A, xr, xi, dr, di);
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      yr[ch][r] = dr[r];
      yi[ch][r] = di[r];
    }
    // output base of the two butterflies whose results this thread holds
#pragma unroll
    for (int cc = 0; cc < 2; ++cc) {
      const int bo = warp * 32 + ch * 8 + 2 * q + cc;
      const int co = bo >> logRQ;
      const int jo = bo & (RQ - 1);
      ocol[ch][cc] = co * cs;
      orow[ch][cc] = ((jo >> logNs) << (logNs + 4)) + (jo & (Ns - 1));
    }
  }
  __syncthreads();
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    // c0 (k=g, col 2q) c1 (k=g, col 2q+1) c2 (k=g+8, col 2q) c3 (k=g+8, col 2q+1)
    sm[ocol[ch][0] + pidx(orow[ch][0] + g * Ns, sh)] = f2{yr[ch][0], yi[ch][0]};
    sm[ocol[ch][1] + pidx(orow[ch][1] + g * Ns, sh)] = f2{yr[ch][1], yi[ch][1]};
    sm[ocol[ch][0] + pidx(orow[ch][0] + (g + 8) * Ns, sh)] = f2{yr[ch][2], yi[ch][2]};
    sm[ocol[ch][1] + pidx(orow[ch][1] + (g + 8) * Ns, sh)] = f2{yr[ch][3], yi[ch][3]};
  }
  __syncthreads();
}

}  // namespace gbfft
