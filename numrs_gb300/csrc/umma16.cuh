// umma16.cuh -- radix-16 Stockham sub-pass on the 5th-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), for the tensor-core form.
//
// A radix-16 sub-pass over a tile of 4096 complex points is 256 butterflies
// of 16 points.  In real arithmetic it is one matrix product
//
//     D[b][n] = sum_k X[b][k] W[n][k]      (256 x 32) = (256 x 32)(32 x 32)^T
//
// with X[b] = (Re x_0 .. Re x_15, Im x_0 .. Im x_15), the twiddled inputs of
// butterfly b, and W the real form of the 16-point DFT matrix:
//     W[n][t] = cos(2 pi n t/16)      W[n][16+t]    = -SG sin(2 pi n t/16)
//     W[16+n][t] = SG sin(2 pi n t/16)  W[16+n][16+t] = cos(2 pi n t/16)
// so that D[b][n] = Re y_n and D[b][16+n] = Im y_n.  The products run as
// tcgen05.mma kind::tf32 with M = 128 butterflies, N = 32, K = 8 per
// instruction, issued by one thread, operands in shared memory and the
// accumulators in tensor memory (TMEM).  TF32 keeps 11 significand bits, so X
// and W are split as hi + lo (both TF32) and D = Xhi Whi + Xlo Whi + Xhi Wlo
// ("3xTF32").  Each of the three products accumulates in its own TMEM region
// from zero, and the three are summed in FP32 round-to-nearest when read
// back: the tensor cores' accumulation is not round-to-nearest, so short
// chains keep the form's error near FP32's.
//
// Operand layout: K-major without swizzle -- core matrices of 8 rows x 16
// bytes (4 TF32 values), K-adjacent core matrices 128 B apart (the leading
// byte offset), 8-row groups 1024 B apart (the stride byte offset).  X takes
// two 16 KB blocks of 128 rows (hi and lo each), W 4 KB (hi and lo each).
// TMEM: per 128-row block three 32-column regions (hh, lh, hl); 192 of the
// 256 columns a CTA allocates.
#pragma once
#include <cstdint>

#include "arith.cuh"
#include "gbfft_internal.h"
#include "tma.cuh"

namespace gbfft {

constexpr uint32_t kUmmaXBlock = 16384;      // 128 rows x 32 TF32
constexpr uint32_t kUmmaXBytes = 2 * kUmmaXBlock;  // 256 butterflies
constexpr uint32_t kUmmaWBytes = 4096;       // 32 rows x 32 TF32
constexpr uint32_t kUmmaTmemCols = 256;
constexpr uint32_t kUmmaWaitLimit = 1u << 22;  // polls of one MMA completion wait

// Shared-memory descriptor of a K-major operand without swizzle (the sm_100
// descriptor layout: start address, leading and stride byte offsets in 16-byte
// units, version 1 in bits 46-47, base offset 0, layout type 0).
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)(128u >> 4) << 16;   // K-adjacent core matrices
  d |= (uint64_t)(1024u >> 4) << 32;  // 8-row groups
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor: D F32, A and B TF32, both K-major, N = 32, M = 128.
constexpr uint32_t kUmmaIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((32u >> 3) << 17) |
                                ((128u >> 4) << 24);

// Byte offset of element (row, k) of a K-major operand.
__device__ __forceinline__ uint32_t umma_off(int row, int k) {
  return (uint32_t)((row & 7) * 16 + (row >> 3) * 1024 + (k >> 2) * 128 + (k & 3) * 4);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(kUmmaIdesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Warp-wide: 32 lanes x 32 consecutive FP32 columns of TMEM from taddr.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Per-CTA state of the tensor-core sub-passes.
struct UmmaCtx {
  unsigned char* xhi;  // X operands (generic pointers for the writes)
  unsigned char* xlo;
  uint32_t xhi_s, xlo_s, whi_s, wlo_s;  // shared addresses for the descriptors
  uint32_t tmem;
  uint64_t* bar;
  uint32_t phase;
};

__device__ __forceinline__ uint32_t tf32_bits(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// W hi and lo (direction SG) from the FP32 twiddle table (level 16), all
// threads of the CTA.
template <int SG>
__device__ __forceinline__ void umma_build_w(unsigned char* whi, unsigned char* wlo,
                                             const f2* twd, int tid, int nthreads) {
  for (int i = tid; i < 32 * 32; i += nthreads) {
    const int n = i >> 5, k = i & 31;
    const f2 w = twd[16 + (((n & 15) * (k & 15)) & 15)];
    const float cr = w.x, ci = SG > 0 ? w.y : -w.y;
    const float val = (n < 16) ? (k < 16 ? cr : -ci) : (k < 16 ? ci : cr);
    const uint32_t hi = tf32_bits(val);
    const uint32_t lo = tf32_bits(val - __uint_as_float(hi));
    *reinterpret_cast<uint32_t*>(whi + umma_off(n, k)) = hi;
    *reinterpret_cast<uint32_t*>(wlo + umma_off(n, k)) = lo;
  }
}

// One radix-16 Stockham sub-pass of a 4096-point tile (256 threads, one
// butterfly each; layout and index rules as subpass<F, SG, 16>).  SRC = 0 takes
// the inputs from the shared tile (sub-pass twiddles of level 16 Ns); SRC = 1
// is a pass's first sub-pass and loads them straight from global memory with
// the pass's inter-pass twiddles.  DST = 0 writes the outputs into the tile;
// DST = 1 is a pass's last sub-pass and stores them straight from TMEM to
// global memory.  Butterfly b of the X rows is (column, row) =
// butterfly_cj(b) with the global side's contiguity when a side is global, so
// that lanes of a warp stay coalesced.  Starts after a barrier that made the
// tile visible, ends with one.  Returns false when the wait for the products
// ran out (the outputs are then not written).
template <int SG, int SRC, int DST, int IN, int OUT, bool L2_ONLY>
__device__ __forceinline__ bool subpass16_umma(const PassParams& p, long long line0, long long j0,
                                               f2* sm, int cs, int logNs, UmmaCtx& u, int tid) {
  using IE = typename IOElem<IN>::T;
  using OE = typename IOElem<OUT>::T;
  constexpr int sh = 5;  // FP32 shared-memory padding (F32::kPadShift)
  const int logR = p.logR;
  const int logRQ = logR - 4, RQ = 1 << logRQ, Ns = 1 << logNs;
  const f2* twd = reinterpret_cast<const f2*>(p.tw.dense);
  const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
  // the butterfly of X row b
  auto cj = [&](int b, int& c, int& j) {
    if (SRC == 1) butterfly_cj(b, p.in_rcontig, logRQ, p.logC, c, j);
    else if (DST == 1) butterfly_cj(b, p.out_rcontig, logRQ, p.logC, c, j);
    else { c = b >> logRQ; j = b & (RQ - 1); }
  };
  {
    const int b = tid;
    int c, j;
    cj(b, c, j);
    float xr[16], xi[16];
    if (SRC == 1) {
      // inputs from global memory; inter-pass twiddles w^(jm (j + t R/16))
      const long long rs = (p.L >> logR) * p.s;
      const long long step = rs << logRQ;
      IE raw[16];
      if (c < rem) {
        const IE* src = col_src<IN>(p, line0, j0, c) + j * rs;
#pragma unroll
        for (int t = 0; t < 16; ++t) load_elem<IE, L2_ONLY>(src + t * step, raw[t]);
      } else {
#pragma unroll
        for (int t = 0; t < 16; ++t) memset(&raw[t], 0, sizeof(IE));
      }
      const long long jg = (p.mode == 0) ? j0 + c : j0;
      const unsigned jm = (unsigned)(jg & (p.Ns - 1));
      const int logS = p.logNs + logR;
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        F32::C v = gload<F32, IN>(&raw[t], 0);
        const unsigned r = (unsigned)(j + (t << logRQ));
        if (p.logNs > 0 && jm != 0 && r != 0) v = F32::mul(v, twiddle<F32>(p.tw, logS, jm * r, SG));
        xr[t] = v.x;
        xi[t] = v.y;
      }
    } else {
      const int cb = c * cs, jm = j & (Ns - 1);
#pragma unroll
      for (int t = 0; t < 16; ++t) {
        f2 v = sm[cb + pidx(j + t * RQ, sh)];
        if (logNs > 0 && jm != 0 && t != 0) {
          const f2 w = twd[(1 << (logNs + 4)) + ((jm * t) & ((Ns << 4) - 1))];
          const float wy = SG > 0 ? w.y : -w.y;
          const float re = fmaf(v.x, w.x, -v.y * wy);
          const float im = fmaf(v.x, wy, v.y * w.x);
          v.x = re;
          v.y = im;
        }
        xr[t] = v.x;
        xi[t] = v.y;
      }
    }
    // hi/lo split into row b of X
    const uint32_t row = (uint32_t)(b >> 7) * kUmmaXBlock + umma_off(b & 127, 0);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t h[4], l[4], hh[4], ll[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        h[i] = tf32_bits(xr[4 * q + i]);
        l[i] = tf32_bits(xr[4 * q + i] - __uint_as_float(h[i]));
        hh[i] = tf32_bits(xi[4 * q + i]);
        ll[i] = tf32_bits(xi[4 * q + i] - __uint_as_float(hh[i]));
      }
      *reinterpret_cast<uint4*>(u.xhi + row + q * 128) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4*>(u.xlo + row + q * 128) = make_uint4(l[0], l[1], l[2], l[3]);
      *reinterpret_cast<uint4*>(u.xhi + row + (q + 4) * 128) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
      *reinterpret_cast<uint4*>(u.xlo + row + (q + 4) * 128) = make_uint4(ll[0], ll[1], ll[2], ll[3]);
    }
  }
  // the operands' generic-proxy writes before the tensor cores read them
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  if (tid == 0) {
    tc_fence_after();
#pragma unroll
    for (int blk = 0; blk < 2; ++blk) {
      const uint32_t col = u.tmem + blk * 96;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const uint64_t ahi = umma_desc(u.xhi_s + blk * kUmmaXBlock + ks * 256);
        const uint64_t alo = umma_desc(u.xlo_s + blk * kUmmaXBlock + ks * 256);
        const uint64_t bhi = umma_desc(u.whi_s + ks * 256);
        const uint64_t blo = umma_desc(u.wlo_s + ks * 256);
        const uint32_t acc = ks > 0 ? 1u : 0u;
        umma_tf32(col, ahi, bhi, acc);
        umma_tf32(col + 32, alo, bhi, acc);
        umma_tf32(col + 64, ahi, blo, acc);
      }
    }
    umma_commit(u.bar);
  }
  const bool ok = mbar_wait_bounded(u.bar, u.phase, kUmmaWaitLimit);
  u.phase ^= 1u;
  tc_fence_after();
  if (ok) {
    // warp w reads block w/4, TMEM lanes 32 (w % 4) ..: one butterfly per lane
    const int warp = tid >> 5, lane = tid & 31;
    const uint32_t ta = u.tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(warp >> 2) * 96;
    float y[32], t[32];
    tmem_ld32(ta, y);
    tmem_ld32(ta + 32, t);
    float s2[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) s2[i] = t[i];
    tmem_ld32(ta + 64, t);
#pragma unroll
    for (int i = 0; i < 32; ++i) y[i] = y[i] + (s2[i] + t[i]);
    const int b2 = (warp >> 2) * 128 + (warp & 3) * 32 + lane;
    int c2, j2;
    cj(b2, c2, j2);
    if (DST == 1) {
      // last sub-pass (Ns = R/16): outputs k at rows j + k R/16 of the column
      if (c2 < rem) {
        const long long rs = p.Ns * p.s;
        const long long step = rs << logRQ;
        OE* dst = col_dst<OUT>(p, line0, j0, c2) + j2 * rs;
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          F32::C w = {y[k], y[16 + k]};
          if (p.do_scale) w = apply_scale<F32>(w, p);
          gstore<F32, OUT>(dst, k * step, w);
        }
      }
    } else {
      const int ob = c2 * cs;
      const int orow = ((j2 >> logNs) << (logNs + 4)) + (j2 & (Ns - 1));
#pragma unroll
      for (int k = 0; k < 16; ++k) sm[ob + pidx(orow + k * Ns, sh)] = f2{y[k], y[16 + k]};
    }
  }
  tc_fence_before();
  __syncthreads();
  return ok;
}

}  // namespace gbfft
