// fft_core.cuh -- the Stockham pass kernel shared by every precision form.
//
// One launch performs one radix-R pass of a Stockham autosort FFT along an
// axis (R <= 4096).  Each CTA owns a tile of C columns x R rows, multiplies by
// the inter-pass twiddles, and runs the R-point DFT of every column as a short
// sequence of radix-2/4/8/16 register sub-passes (themselves Stockham steps)
// with shared memory between them.  Two tile schedules:
//   staged  load the tile into shared memory, run the sub-passes there, store
//           the tile (FP64, double-float)
//   fused   the first sub-pass loads its butterfly inputs straight from global
//           memory and the last one stores straight to global memory (FP32,
//           TC32; every CUDA-core form in the persistent batch kernel)
// Global accesses are coalesced along whichever index is contiguous.  Axes of
// at most 4096 points take one launch; longer axes take 2-3 launches that
// ping-pong through scratch, the last one writing the caller's array.
#pragma once
#include <atomic>

#include "arith.cuh"
#include "gbfft_internal.h"

namespace gbfft {

constexpr int kEPT = kTileEPT;  // complex elements per thread per tile

// Devices on which a one-time per-kernel setting has been made.  Function
// attributes belong to a device's context, so a process that launches on
// several GPUs sets them on each one.  The bits are atomic: two host threads
// whose first launches race both set the same attribute value, which is
// harmless.  Devices 64 and above are set up on every launch.
struct DeviceOnce {
  std::atomic<unsigned long long> bits{0};
};

// Raise a kernel's dynamic shared memory limit to `smem` bytes on the current
// device, once per device.
template <class K>
inline cudaError_t smem_opt_in(K kernel, size_t smem, DeviceOnce& once) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (once.bits.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (bit) once.bits.fetch_or(bit, std::memory_order_acq_rel);
  return cudaSuccess;
}

// Shared-memory tile layout: column c, row r at c*cs + pidx(r).  The row
// padding (one element per 2^sh) spreads strided accesses within a column
// over the banks; one extra element per column (columns of 16 rows or more)
// does the same for accesses whose lanes step across columns.
__device__ __forceinline__ int pidx(int i, int sh) { return i + (i >> sh); }
__host__ __device__ __forceinline__ int col_stride(int logR, int sh) {
  const int R = 1 << logR;
  return R + (R >> sh) + (logR >= 4 ? 1 : 0);
}

}  // namespace gbfft
#include "tc16.cuh"
namespace gbfft {

// ---------------------------------------------------------------------------
// Twiddle lookup: w_S^e with sign, S = 2^logS and 0 <= e < S <= 2^29, so
// that every index fits 32-bit arithmetic.
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ typename F::C twiddle(const Twiddles& tw, int logS, unsigned int e,
                                                 int sg) {
  using TW = typename F::TW;
  const TW* dense = reinterpret_cast<const TW*>(tw.dense);
  if (logS <= tw.dense_log) return F::ld_tw(dense + ((1u << logS) + e), sg);
  if (logS == tw.top_log) return F::ld_tw(reinterpret_cast<const TW*>(tw.top) + e, sg);
  const TW* part = reinterpret_cast<const TW*>(tw.partial);
  typename F::C hi = F::ld_tw(dense + ((1u << (logS - kPartialLog)) + (e >> kPartialLog)), sg);
  typename F::C lo = F::ld_tw(part + ((unsigned)(logS - tw.dense_log - 1) * kPartial +
                                      (e & (kPartial - 1))), sg);
  return F::mul(hi, lo);
}

// ---------------------------------------------------------------------------
// Small DFTs in registers, X_k = sum_t v_t exp(+SG 2 pi i t k / Q), in place.
// ---------------------------------------------------------------------------
template <class F, int SG>
__device__ __forceinline__ void dft2(typename F::C& a, typename F::C& b) {
  typename F::C t = F::sub(a, b);
  a = F::add(a, b);
  b = t;
}

template <class F, int SG>
__device__ __forceinline__ void dft4(typename F::C& a0, typename F::C& a1, typename F::C& a2,
                                     typename F::C& a3) {
  using C = typename F::C;
  C t0 = F::add(a0, a2), t1 = F::sub(a0, a2);
  C t2 = F::add(a1, a3), t3 = F::mul_j(F::sub(a1, a3), SG);
  a0 = F::add(t0, t2);
  a2 = F::sub(t0, t2);
  a1 = F::add(t1, t3);
  a3 = F::sub(t1, t3);
}

constexpr double kH = 0.70710678118654752440084436210484903928;   // cos(pi/4)
constexpr double kC1 = 0.92387953251128675612818318939678828682;  // cos(pi/8)
constexpr double kS1 = 0.38268343236508977172845998403039886676;  // sin(pi/8)

template <class F, int SG>
__device__ __forceinline__ void dft8(typename F::C* v) {
  using C = typename F::C;
  // decimation in time: even and odd 4-point DFTs, then twiddles w8^k
  C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<F, SG>(e0, e1, e2, e3);
  dft4<F, SG>(o0, o1, o2, o3);
  o1 = F::rot45(o1, kH, SG);
  o2 = F::mul_j(o2, SG);
  o3 = F::mul_j(F::rot45(o3, kH, SG), SG);
  v[0] = F::add(e0, o0); v[4] = F::sub(e0, o0);
  v[1] = F::add(e1, o1); v[5] = F::sub(e1, o1);
  v[2] = F::add(e2, o2); v[6] = F::sub(e2, o2);
  v[3] = F::add(e3, o3); v[7] = F::sub(e3, o3);
}

template <class F, int SG>
__device__ __forceinline__ void dft16(typename F::C* v) {
  using C = typename F::C;
  // 4 x 4: X_{k1+4k2} = sum_{n2} w4^{n2 k2} w16^{n2 k1} sum_{n1} v_{n2+4n1} w4^{n1 k1}
  C a[4][4];
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) {
    a[n2][0] = v[n2]; a[n2][1] = v[n2 + 4]; a[n2][2] = v[n2 + 8]; a[n2][3] = v[n2 + 12];
    dft4<F, SG>(a[n2][0], a[n2][1], a[n2][2], a[n2][3]);
  }
  // twiddles w16^{n2 k1}
  a[1][1] = F::mulcs(a[1][1], kC1, SG * kS1);       // w^1
  a[1][2] = F::rot45(a[1][2], kH, SG);              // w^2
  a[1][3] = F::mulcs(a[1][3], kS1, SG * kC1);       // w^3
  a[2][1] = F::rot45(a[2][1], kH, SG);              // w^2
  a[2][2] = F::mul_j(a[2][2], SG);                  // w^4
  a[2][3] = F::mul_j(F::rot45(a[2][3], kH, SG), SG);  // w^6
  a[3][1] = F::mulcs(a[3][1], kS1, SG * kC1);       // w^3
  a[3][2] = F::mul_j(F::rot45(a[3][2], kH, SG), SG);  // w^6
  a[3][3] = F::mulcs(a[3][3], -kC1, -SG * kS1);     // w^9
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    C b0 = a[0][k1], b1 = a[1][k1], b2 = a[2][k1], b3 = a[3][k1];
    dft4<F, SG>(b0, b1, b2, b3);
    v[k1] = b0; v[k1 + 4] = b1; v[k1 + 8] = b2; v[k1 + 12] = b3;
  }
}

template <class F, int SG, int Q>
__device__ __forceinline__ void dftq(typename F::C* v) {
  if constexpr (Q == 2) dft2<F, SG>(v[0], v[1]);
  else if constexpr (Q == 4) dft4<F, SG>(v[0], v[1], v[2], v[3]);
  else if constexpr (Q == 8) dft8<F, SG>(v);
  else dft16<F, SG>(v);
}

// ---------------------------------------------------------------------------
// One in-CTA Stockham sub-pass of radix Q over C columns of R points held in
// shared memory (column c at c*R, padded).  Every thread owns 16/Q butterflies.
// ---------------------------------------------------------------------------
template <class F, int SG, int Q, int EPT = kEPT>
__device__ __forceinline__ void subpass(typename F::S* sm, int logR, int cs, int logNs,
                                        const Twiddles& tw, int tid, int T) {
  using C = typename F::C;
  constexpr int B = EPT / Q;
  constexpr int LQ = (Q == 2) ? 1 : (Q == 4) ? 2 : (Q == 8) ? 3 : 4;
  constexpr int sh = F::kPadShift;
  const int logRQ = logR - LQ;
  const int RQ = 1 << logRQ;
  const int Ns = 1 << logNs;
  C v[B][Q];
  int ob[B], oc[B];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int b = tid + i * T;
    const int c = b >> logRQ;
    const int j = b & (RQ - 1);
    const int cb = c * cs;
#pragma unroll
    for (int t = 0; t < Q; ++t) v[i][t] = F::from_s(sm[cb + pidx(j + t * RQ, sh)]);
    const int jm = j & (Ns - 1);
    if (logNs > 0 && jm != 0) {
#pragma unroll
      for (int t = 1; t < Q; ++t)
        v[i][t] = F::mul(v[i][t], twiddle<F>(tw, logNs + LQ, (unsigned)(jm * t), SG));
    }
    dftq<F, SG, Q>(v[i]);
    oc[i] = cb;
    ob[i] = ((j >> logNs) << (logNs + LQ)) + jm;
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < B; ++i) {
#pragma unroll
    for (int t = 0; t < Q; ++t) sm[oc[i] + pidx(ob[i] + t * Ns, sh)] = F::to_s(v[i][t]);
  }
  __syncthreads();
}

// Output scaling: the FP32-pipe forms use the float copy of the scale.
template <class F>
__device__ __forceinline__ typename F::C apply_scale(typename F::C w, const PassParams& p) {
  if constexpr (F::kind == 1) return {w.x * p.fscale, w.y * p.fscale};
  else if constexpr (F::kind == 2) return {df_scale_f(w.x, p.fscale), df_scale_f(w.y, p.fscale)};
  else return F::scale(w, p.scale);
}

// Spectrum epilogue of a transform's last pass (magnitude_spectrum and
// power_spectrum, src/FFT_1.rs:206-228, fused into the store): spec[i] =
// |X|^2 or its square root, in double, for the output element of index i.
template <class F>
__device__ __forceinline__ void spec_store(const PassParams& p, long long i,
                                           const typename F::C& v) {
  double x, y;
  F::to_d(v, x, y);
  const double pw = x * x + y * y;
  p.spec[i] = p.spec_kind == 1 ? sqrt(pw) : pw;
}

// ---------------------------------------------------------------------------
// Global element access with format conversion.
// ---------------------------------------------------------------------------
template <class F, int IO>
__device__ __forceinline__ typename F::C gload(const void* p, long long i) {
  if constexpr (IO == IO_D2) {
    d2 v = reinterpret_cast<const d2*>(p)[i];
    return F::from_d(v.x, v.y);
  } else if constexpr (IO == IO_F2) {
    f2 v = reinterpret_cast<const f2*>(p)[i];
    if constexpr (F::kind == 1) {
      return F::from_s(v);
    } else {
      return F::from_d((double)v.x, (double)v.y);
    }
  } else {
    f4 v = reinterpret_cast<const f4*>(p)[i];
    if constexpr (F::kind == 2) {
      return F::from_s(v);
    } else {
      return F::from_d((double)v.x + (double)v.y, (double)v.z + (double)v.w);
    }
  }
}

template <class F, int IO>
__device__ __forceinline__ void gstore(void* p, long long i, typename F::C a) {
  if constexpr (IO == IO_D2) {
    double x, y;
    F::to_d(a, x, y);
    reinterpret_cast<d2*>(p)[i] = d2{x, y};
  } else if constexpr (IO == IO_F2) {
    if constexpr (F::kind == 1) {
      reinterpret_cast<f2*>(p)[i] = F::to_s(a);
    } else {
      double x, y;
      F::to_d(a, x, y);
      reinterpret_cast<f2*>(p)[i] = f2{(float)x, (float)y};
    }
  } else {
    if constexpr (F::kind == 2) {
      reinterpret_cast<f4*>(p)[i] = F::to_s(a);
    } else {
      double x, y;
      F::to_d(a, x, y);
      float xh = (float)x, yh = (float)y;
      reinterpret_cast<f4*>(p)[i] = f4{xh, (float)(x - xh), yh, (float)(y - yh)};
    }
  }
}

// ---------------------------------------------------------------------------
// One tile of one pass (T threads, 16*T complex elements).  Used by the
// per-pass kernel (one tile per CTA) and by the persistent batch kernel.
// L2_ONLY loads bypass L1 (data written by other CTAs of the same launch).
// ---------------------------------------------------------------------------
template <int IO>
struct IOElem;
template <> struct IOElem<IO_D2> { using T = d2; };
template <> struct IOElem<IO_F2> { using T = f2; };
template <> struct IOElem<IO_F4> { using T = f4; };

// tile index -> first line and first column j of the tile
__device__ __forceinline__ void tile_origin(const PassParams& p, long long tile, long long& line0,
                                            long long& j0) {
  const int logLR = p.logL - p.logR;
  if (p.mode == 0) {
    const int logTpl = logLR - p.logC;  // tiles per line
    line0 = tile >> logTpl;
    j0 = (tile & ((1ll << logTpl) - 1)) << p.logC;
  } else {
    // j0 fastest: L/R is a power of two, so no division (an integer division
    // is a software sequence, partly on the FP64 pipe)
    j0 = tile & ((1ll << logLR) - 1);
    line0 = (tile >> logLR) << p.logC;
  }
}

// (column, row) of tile element e in the load order: contiguous along r when
// the tile's columns are contiguous runs in memory, along c otherwise.
__device__ __forceinline__ void elem_cr(int e, int rcontig, int logR, int logC, int& c, int& r) {
  if (rcontig) { r = e & ((1 << logR) - 1); c = e >> logR; }
  else { c = e & ((1 << logC) - 1); r = e >> logC; }
}

// Element e of the tile (raw value from global memory or a staging buffer):
// convert, apply the inter-pass twiddle, store into the padded tile.
template <class F, int SG, int IN>
__device__ __forceinline__ void stage_elem(const PassParams& p, long long line0, long long j0,
                                           int e, const typename IOElem<IN>::T& rawv,
                                           typename F::S* sm) {
  using C = typename F::C;
  int c, r;
  elem_cr(e, p.in_rcontig, p.logR, p.logC, c, r);
  const long long line = (p.mode == 0) ? line0 : line0 + c;
  C v = (line < p.nlines) ? gload<F, IN>(&rawv, 0) : F::from_d(0.0, 0.0);
  if (p.logNs > 0) {
    const long long j = (p.mode == 0) ? j0 + c : j0;
    const unsigned jm = (unsigned)(j & (p.Ns - 1));
    // jm * r < Ns * R <= L
    if (jm != 0 && r != 0) v = F::mul(v, twiddle<F>(p.tw, p.logNs + p.logR, jm * (unsigned)r, SG));
  }
  sm[c * col_stride(p.logR, F::kPadShift) + pidx(r, F::kPadShift)] = F::to_s(v);
}

// Global index of a line's first element.
__device__ __forceinline__ long long line_base(const PassParams& p, long long line) {
  return (line >> p.lq_log) * p.lstride + (line & ((1ll << p.lq_log) - 1));
}

// Linear layouts (no per-line pointer table): the global index of slot k of
// thread tid is thread_base_in/out + in_off/out_off[k].  ct receives the
// thread's part of the slot's column, used for the column bound of mode 1.
__device__ __forceinline__ long long thread_base_in(const PassParams& p, long long line0,
                                                    long long j0, int tid, long long& ct) {
  long long c, r;
  tile_cr(tid, p.in_rcontig, p.logR, p.logC, c, r);
  ct = c;
  return line_base(p, line0) + j0 * p.s + col_off_in(p, c) + r * ((p.L >> p.logR) * p.s);
}
__device__ __forceinline__ long long thread_base_out(const PassParams& p, long long line0,
                                                     long long j0, int tid, long long& ct) {
  long long c, r;
  tile_cr(tid, p.out_rcontig, p.logR, p.logC, c, r);
  ct = c;
  const long long jd0 = ((j0 >> p.logNs) << (p.logNs + p.logR)) + (j0 & (p.Ns - 1));
  return line_base(p, line0) + jd0 * p.s + col_off_out(p, c) + r * (p.Ns * p.s);
}

// The R-point DFTs of the tile's columns in shared memory: the pass's
// sub-passes in order.  Starts after a barrier that made the tile visible and
// ends with one.  EPT elements per thread allow sub-passes of radix <= EPT
// (the planner splits accordingly).
template <class F, int SG, int T, int EPT = kEPT>
__device__ __forceinline__ void run_subpasses(const PassParams& p, typename F::S* sm, int cs,
                                              int tid) {
  const int logR = p.logR;
  int logNsub = 0;
  for (int k = 0; k < p.nq; ++k) {
    const int lq = p.q[k];
    switch (lq) {
      case 4:
        if constexpr (EPT >= 16) {
          if constexpr (F::kTensor) {
            Dft16Frags A;
            dft16_frags<SG>(reinterpret_cast<const f2*>(p.tw.dense), A);
            subpass16_tc<SG>(reinterpret_cast<f2*>(sm), logR, cs, logNsub, p.tw, A, tid);
          } else {
            subpass<F, SG, 16, EPT>(sm, logR, cs, logNsub, p.tw, tid, T);
          }
        }
        break;
      case 3:
        if constexpr (EPT >= 8) subpass<F, SG, 8, EPT>(sm, logR, cs, logNsub, p.tw, tid, T);
        break;
      case 2: subpass<F, SG, 4, EPT>(sm, logR, cs, logNsub, p.tw, tid, T); break;
      default: subpass<F, SG, 2, EPT>(sm, logR, cs, logNsub, p.tw, tid, T); break;
    }
    logNsub += lq;
  }
}

// The store of a transformed tile at the autosorted positions (after the
// barrier that ends the last sub-pass).
template <class F, int SG, int OUT, int T, int EPT = kEPT>
__device__ __forceinline__ void store_tile(const PassParams& p, long long line0, long long j0,
                                           const typename F::S* sm, int tid) {
  using C = typename F::C;
  using OE = typename IOElem<OUT>::T;
  constexpr int sh = F::kPadShift;
  const int logR = p.logR, logC = p.logC;
  const int cs = col_stride(logR, sh);
  if (p.out_ptrs == nullptr) {
    // linear layout: per-thread base plus the slot offsets out_off[k]
    long long ct;
    const long long tb = thread_base_out(p, line0, j0, tid, ct);
    OE* dst = reinterpret_cast<OE*>(p.out) + tb;
    const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
#pragma unroll 4
    for (int k = 0; k < EPT; ++k) {
      const int e = tid + k * T;
      int c, r;
      elem_cr(e, p.out_rcontig, logR, logC, c, r);
      long long ck, rk;
      tile_cr((long long)k * T, p.out_rcontig, logR, logC, ck, rk);
      if (ct + ck >= rem) continue;
      C v = F::from_s(sm[c * cs + pidx(r, sh)]);
      if (p.do_scale) v = apply_scale<F>(v, p);
      gstore<F, OUT>(dst, p.out_off[k], v);
      if (p.spec_kind) spec_store<F>(p, tb + p.out_off[k], v);
    }
    return;
  }
#pragma unroll 4
  for (int k = 0; k < EPT; ++k) {
    const int e = tid + k * T;
    int c, r;
    elem_cr(e, p.out_rcontig, logR, logC, c, r);
    long long line = line0, j = j0;
    if (p.mode == 0) j += c; else line += c;
    if (line >= p.nlines) continue;
    C v = F::from_s(sm[c * cs + pidx(r, sh)]);
    if (p.do_scale) v = apply_scale<F>(v, p);
    OE* base = reinterpret_cast<OE*>(p.out_ptrs[line]);
    const long long jd = ((j >> p.logNs) << (p.logNs + logR)) + (j & (p.Ns - 1));
    gstore<F, OUT>(base, (jd + ((long long)r << p.logNs)) * p.s, v);
  }
}

// The R-point DFTs of the tile's columns, then the store at the autosorted
// positions.  Starts after a barrier that made the staged tile visible.
template <class F, int SG, int OUT, int T, int EPT = kEPT>
__device__ __forceinline__ void tile_compute_store(const PassParams& p, long long line0,
                                                   long long j0, typename F::S* sm, int tid) {
  run_subpasses<F, SG, T, EPT>(p, sm, col_stride(p.logR, F::kPadShift), tid);
  store_tile<F, SG, OUT, T, EPT>(p, line0, j0, sm, tid);
}

// Address of tile element e in global memory, input side, for tiles whose
// lines come from a per-line pointer table.
template <int IN>
__device__ __forceinline__ const typename IOElem<IN>::T* elem_src(const PassParams& p,
                                                                  long long line0, long long j0,
                                                                  int e, bool& valid) {
  using IE = typename IOElem<IN>::T;
  int c, r;
  elem_cr(e, p.in_rcontig, p.logR, p.logC, c, r);
  long long line = line0, j = j0;
  if (p.mode == 0) j += c; else line += c;
  valid = line < p.nlines;
  if (!valid) return nullptr;
  const IE* base = reinterpret_cast<const IE*>(p.in_ptrs[line]);
  return base + (j + ((long long)r << (p.logL - p.logR))) * p.s;
}

template <class IE, bool L2_ONLY>
__device__ __forceinline__ void load_elem(const IE* src, IE& dst) {
  if constexpr (L2_ONLY) {
    if constexpr (sizeof(IE) == 8) {
      float2 t = __ldcg(reinterpret_cast<const float2*>(src));
      memcpy(&dst, &t, 8);
    } else {
      float4 t = __ldcg(reinterpret_cast<const float4*>(src));
      memcpy(&dst, &t, 16);
    }
  } else {
    dst = *src;
  }
}

// The sixteen raw elements of thread tid's slots (zero outside the lines).
// All loads are issued before any is used, so that each SM keeps enough
// bytes in flight to cover the memory latency.
template <class IE, int IN, int T, bool L2_ONLY, int EPT = kEPT>
__device__ __forceinline__ void load_tile_raw(const PassParams& p, long long line0, long long j0,
                                              int tid, IE (&raw)[EPT]) {
  if (p.in_ptrs == nullptr) {
    // linear layout: per-thread base plus the slot offsets in_off[k]
    long long ct;
    const IE* src = reinterpret_cast<const IE*>(p.in) + thread_base_in(p, line0, j0, tid, ct);
    const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
      long long ck, rk;
      tile_cr((long long)k * T, p.in_rcontig, p.logR, p.logC, ck, rk);
      if (ct + ck < rem) load_elem<IE, L2_ONLY>(src + p.in_off[k], raw[k]);
      else memset(&raw[k], 0, sizeof(IE));
    }
  } else {
#pragma unroll
    for (int k = 0; k < EPT; ++k) {
      bool valid;
      const IE* src = elem_src<IN>(p, line0, j0, tid + k * T, valid);
      if (valid) load_elem<IE, L2_ONLY>(src, raw[k]);
      else memset(&raw[k], 0, sizeof(IE));
    }
  }
}

// One full tile from global memory.  L2_ONLY loads bypass L1 (data written by
// other CTAs of the same launch).
// Stage a thread's EPT raw elements into the tile with their inter-pass
// twiddles.  The twiddles are gathered in groups of eight, all loads of a
// group issued before any is used, so that a thread waits on one table
// round trip per group instead of one per element; the exponent-0 entries
// (j mod Ns = 0 or r = 0) read the table's exact 1 + 0i.
template <class F, int SG, int IN, int T, int EPT>
__device__ __forceinline__ void stage_tile(const PassParams& p, long long line0, long long j0,
                                           int tid, const typename IOElem<IN>::T (&raw)[EPT],
                                           typename F::S* sm) {
  using C = typename F::C;
  constexpr int G = EPT >= 8 ? 8 : EPT;
  constexpr int sh = F::kPadShift;
  const int cs = col_stride(p.logR, sh);
  const bool tw_on = p.logNs > 0;
  const int logS = p.logNs + p.logR;
#pragma unroll
  for (int g0 = 0; g0 < EPT; g0 += G) {
    C w[G];
    if (tw_on) {
#pragma unroll
      for (int i = 0; i < G; ++i) {
        int c, r;
        elem_cr(tid + (g0 + i) * T, p.in_rcontig, p.logR, p.logC, c, r);
        const long long j = (p.mode == 0) ? j0 + c : j0;
        const unsigned jm = (unsigned)(j & (p.Ns - 1));
        w[i] = twiddle<F>(p.tw, logS, jm * (unsigned)r, SG);  // jm * r < Ns * R <= L
      }
    }
#pragma unroll
    for (int i = 0; i < G; ++i) {
      int c, r;
      elem_cr(tid + (g0 + i) * T, p.in_rcontig, p.logR, p.logC, c, r);
      const long long line = (p.mode == 0) ? line0 : line0 + c;
      C v = (line < p.nlines) ? gload<F, IN>(&raw[g0 + i], 0) : F::from_d(0.0, 0.0);
      if (tw_on) v = F::mul(v, w[i]);
      sm[c * cs + pidx(r, sh)] = F::to_s(v);
    }
  }
}

template <class F, int SG, int IN, int OUT, int T, bool L2_ONLY, int EPT = kEPT>
__device__ __forceinline__ void pass_tile(const PassParams& p, long long tile,
                                          typename F::S* sm, int tid) {
  using IE = typename IOElem<IN>::T;
  long long line0, j0;
  tile_origin(p, tile, line0, j0);
  IE raw[EPT];
  load_tile_raw<IE, IN, T, L2_ONLY, EPT>(p, line0, j0, tid, raw);
  stage_tile<F, SG, IN, T, EPT>(p, line0, j0, tid, raw, sm);
  __syncthreads();
  tile_compute_store<F, SG, OUT, T, EPT>(p, line0, j0, sm, tid);
}

// ---------------------------------------------------------------------------
// Fused form of a tile (passes of two or more in-CTA sub-passes, CUDA-core
// forms): the first sub-pass takes its butterfly inputs straight from global
// memory and the last one writes its outputs straight to global memory, so
// that the tile crosses shared memory once per inner sub-pass boundary only.
//
// Butterfly b of a sub-pass of radix Q covers rows j + t*R/Q (t < Q) of column
// c.  For global accesses, consecutive lanes take consecutive rows (j fastest)
// when the tile's columns are contiguous runs of rows in memory, and
// consecutive columns (c fastest) otherwise, so that both loads and stores stay
// coalesced.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void butterfly_cj(int b, int rcontig, int logRQ, int logC, int& c,
                                             int& j) {
  if (rcontig) { j = b & ((1 << logRQ) - 1); c = b >> logRQ; }
  else { c = b & ((1 << logC) - 1); j = b >> logC; }
}

// Global index (elements of the IO type) of row 0 of tile column c, and the
// index step of one row; input side.
template <int IN>
__device__ __forceinline__ const typename IOElem<IN>::T* col_src(const PassParams& p,
                                                                 long long line0, long long j0,
                                                                 int c) {
  using IE = typename IOElem<IN>::T;
  if (p.in_ptrs == nullptr)
    return reinterpret_cast<const IE*>(p.in) + (line_base(p, line0) + j0 * p.s + col_off_in(p, c));
  const long long line = (p.mode == 0) ? line0 : line0 + c;
  const long long j = (p.mode == 0) ? j0 + c : j0;
  return reinterpret_cast<const IE*>(p.in_ptrs[line]) + j * p.s;
}

// Linear-layout index (IO elements from p.out) of row 0 of output column c.
__device__ __forceinline__ long long col_index_out(const PassParams& p, long long line0,
                                                   long long j0, int c) {
  const long long jd0 = ((j0 >> p.logNs) << (p.logNs + p.logR)) + (j0 & (p.Ns - 1));
  return line_base(p, line0) + jd0 * p.s + col_off_out(p, c);
}

template <int OUT>
__device__ __forceinline__ typename IOElem<OUT>::T* col_dst(const PassParams& p, long long line0,
                                                           long long j0, int c) {
  using OE = typename IOElem<OUT>::T;
  const long long jd0 = ((j0 >> p.logNs) << (p.logNs + p.logR)) + (j0 & (p.Ns - 1));
  if (p.out_ptrs == nullptr)
    return reinterpret_cast<OE*>(p.out) + (line_base(p, line0) + jd0 * p.s + col_off_out(p, c));
  const long long line = (p.mode == 0) ? line0 : line0 + c;
  const long long j = (p.mode == 0) ? j0 + c : j0;
  const long long jd = ((j >> p.logNs) << (p.logNs + p.logR)) + (j & (p.Ns - 1));
  return reinterpret_cast<OE*>(p.out_ptrs[line]) + jd * p.s;
}

// First sub-pass (radix Q, no intra-tile twiddles) from global memory: load
// every input of the thread's 16/Q butterflies, apply the inter-pass
// twiddles, transform, write the outputs into the shared tile.  The caller
// synchronises before the next sub-pass reads the tile.
template <class F, int SG, int IN, int Q, int T, bool L2_ONLY>
__device__ __forceinline__ void first_subpass(const PassParams& p, long long line0, long long j0,
                                              typename F::S* sm, int cs, int tid) {
  using C = typename F::C;
  using IE = typename IOElem<IN>::T;
  constexpr int B = kEPT / Q;
  constexpr int LQ = (Q == 2) ? 1 : (Q == 4) ? 2 : (Q == 8) ? 3 : 4;
  constexpr int sh = F::kPadShift;
  const int logR = p.logR;
  const int logRQ = logR - LQ;
  const long long rs = (p.L >> logR) * p.s;  // index step of one row
  const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
  IE raw[B][Q];
  int cc[B], jj[B];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    butterfly_cj(tid + i * T, p.in_rcontig, logRQ, p.logC, cc[i], jj[i]);
    if (cc[i] < rem) {
      const IE* src = col_src<IN>(p, line0, j0, cc[i]) + jj[i] * rs;
      const long long step = rs << logRQ;
#pragma unroll
      for (int t = 0; t < Q; ++t) load_elem<IE, L2_ONLY>(src + t * step, raw[i][t]);
    } else {
#pragma unroll
      for (int t = 0; t < Q; ++t) memset(&raw[i][t], 0, sizeof(IE));
    }
  }
  const int logS = p.logNs + logR;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int c = cc[i], j = jj[i];
    const long long jg = (p.mode == 0) ? j0 + c : j0;
    const unsigned jm = (unsigned)(jg & (p.Ns - 1));
    C v[Q];
#pragma unroll
    for (int t = 0; t < Q; ++t) v[t] = gload<F, IN>(&raw[i][t], 0);
    if constexpr (F::kind == 1 && Q >= 4) {
      // FP32: the twiddles w^(jm (j + t R/Q)), t = 4a + b, are products
      // w^(jm (j + 4a R/Q)) * w^(jm b R/Q) of two correctly rounded table
      // entries (one more rounding): Q/4 + 3 gathered table loads instead of Q.
      // Every exponent is below jm * R <= Ns * R = 2^logS.
      if (p.logNs > 0 && jm != 0) {
        const unsigned base = jm * (unsigned)j, step = jm << logRQ;
        C sb[4];
        sb[0] = F::from_s(typename F::S{1.f, 0.f});
#pragma unroll
        for (int b = 1; b < 4; ++b) sb[b] = twiddle<F>(p.tw, logS, step * (unsigned)b, SG);
#pragma unroll
        for (int a = 0; a < Q / 4; ++a) {
          const C la = twiddle<F>(p.tw, logS, base + step * (unsigned)(4 * a), SG);
          v[4 * a] = F::mul(v[4 * a], la);
#pragma unroll
          for (int b = 1; b < 4; ++b) v[4 * a + b] = F::mul(v[4 * a + b], F::mul(la, sb[b]));
        }
      }
    } else {
#pragma unroll
      for (int t = 0; t < Q; ++t) {
        const unsigned r = (unsigned)(j + (t << logRQ));
        // jm * r < Ns * R <= L
        if (p.logNs > 0 && jm != 0 && r != 0) v[t] = F::mul(v[t], twiddle<F>(p.tw, logS, jm * r, SG));
      }
    }
    dftq<F, SG, Q>(v);
    const int cb = c * cs;
#pragma unroll
    for (int t = 0; t < Q; ++t) sm[cb + pidx(j * Q + t, sh)] = F::to_s(v[t]);
  }
}

// Last sub-pass (radix Q, Ns = R/Q) from the shared tile to global memory:
// twiddle, transform, scale, store at the autosorted global positions.
template <class F, int SG, int OUT, int Q, int T>
__device__ __forceinline__ void last_subpass(const PassParams& p, long long line0, long long j0,
                                             const typename F::S* sm, int cs, int tid) {
  using C = typename F::C;
  using OE = typename IOElem<OUT>::T;
  constexpr int B = kEPT / Q;
  constexpr int LQ = (Q == 2) ? 1 : (Q == 4) ? 2 : (Q == 8) ? 3 : 4;
  constexpr int sh = F::kPadShift;
  const int logR = p.logR;
  const int logRQ = logR - LQ;  // = log2 of the sub-pass's Ns
  const long long rs = p.Ns * p.s;  // index step of one output row
  const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    int c, j;
    butterfly_cj(tid + i * T, p.out_rcontig, logRQ, p.logC, c, j);
    const int cb = c * cs;
    C v[Q];
#pragma unroll
    for (int t = 0; t < Q; ++t) v[t] = F::from_s(sm[cb + pidx(j + (t << logRQ), sh)]);
    if (j != 0) {
#pragma unroll
      for (int t = 1; t < Q; ++t) v[t] = F::mul(v[t], twiddle<F>(p.tw, logR, (unsigned)(j * t), SG));
    }
    dftq<F, SG, Q>(v);
    if (c >= rem) continue;
    OE* dst = col_dst<OUT>(p, line0, j0, c) + j * rs;
    const long long step = rs << logRQ;
#pragma unroll
    for (int t = 0; t < Q; ++t) {
      C w = v[t];
      if (p.do_scale) w = apply_scale<F>(w, p);
      gstore<F, OUT>(dst, t * step, w);
    }
    if (p.spec_kind) {
      const long long i0 = col_index_out(p, line0, j0, c) + j * rs;
#pragma unroll
      for (int t = 0; t < Q; ++t) {
        C w = v[t];
        if (p.do_scale) w = apply_scale<F>(w, p);
        spec_store<F>(p, i0 + t * step, w);
      }
    }
  }
}

// A pass of one sub-pass (R = Q <= 16, single-pass transforms, whose load and
// store layouts agree): every thread transforms 16/Q columns from global
// memory to global memory without touching shared memory.
template <class F, int SG, int IN, int OUT, int Q, int T, bool L2_ONLY>
__device__ __forceinline__ void only_subpass(const PassParams& p, long long line0, long long j0,
                                             int tid) {
  using C = typename F::C;
  using IE = typename IOElem<IN>::T;
  using OE = typename IOElem<OUT>::T;
  constexpr int B = kEPT / Q;
  const long long rs_in = (p.L >> p.logR) * p.s;
  const long long rs_out = p.Ns * p.s;
  const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
  IE raw[B][Q];
  int cc[B];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    cc[i] = tid + i * T;  // one butterfly per column
    if (cc[i] < rem) {
      const IE* src = col_src<IN>(p, line0, j0, cc[i]);
#pragma unroll
      for (int t = 0; t < Q; ++t) load_elem<IE, L2_ONLY>(src + t * rs_in, raw[i][t]);
    } else {
#pragma unroll
      for (int t = 0; t < Q; ++t) memset(&raw[i][t], 0, sizeof(IE));
    }
  }
  const int logS = p.logNs + p.logR;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int c = cc[i];
    if (c >= rem) continue;
    const long long jg = (p.mode == 0) ? j0 + c : j0;
    const unsigned jm = (unsigned)(jg & (p.Ns - 1));
    C v[Q];
#pragma unroll
    for (int t = 0; t < Q; ++t) {
      v[t] = gload<F, IN>(&raw[i][t], 0);
      if (p.logNs > 0 && jm != 0 && t != 0) v[t] = F::mul(v[t], twiddle<F>(p.tw, logS, jm * t, SG));
    }
    dftq<F, SG, Q>(v);
    OE* dst = col_dst<OUT>(p, line0, j0, c);
#pragma unroll
    for (int t = 0; t < Q; ++t) {
      C w = v[t];
      if (p.do_scale) w = apply_scale<F>(w, p);
      gstore<F, OUT>(dst, t * rs_out, w);
      if (p.spec_kind) spec_store<F>(p, col_index_out(p, line0, j0, c) + t * rs_out, w);
    }
  }
}

template <class F, int SG, int IN, int T, bool L2_ONLY>
__device__ __forceinline__ void first_subpass_q(int lq, const PassParams& p, long long line0,
                                                long long j0, typename F::S* sm, int cs, int tid) {
  switch (lq) {
    case 4: first_subpass<F, SG, IN, 16, T, L2_ONLY>(p, line0, j0, sm, cs, tid); break;
    case 3: first_subpass<F, SG, IN, 8, T, L2_ONLY>(p, line0, j0, sm, cs, tid); break;
    case 2: first_subpass<F, SG, IN, 4, T, L2_ONLY>(p, line0, j0, sm, cs, tid); break;
    default: first_subpass<F, SG, IN, 2, T, L2_ONLY>(p, line0, j0, sm, cs, tid); break;
  }
}

template <class F, int SG, int OUT, int T>
__device__ __forceinline__ void last_subpass_q(int lq, const PassParams& p, long long line0,
                                               long long j0, const typename F::S* sm, int cs,
                                               int tid) {
  switch (lq) {
    case 4: last_subpass<F, SG, OUT, 16, T>(p, line0, j0, sm, cs, tid); break;
    case 3: last_subpass<F, SG, OUT, 8, T>(p, line0, j0, sm, cs, tid); break;
    case 2: last_subpass<F, SG, OUT, 4, T>(p, line0, j0, sm, cs, tid); break;
    default: last_subpass<F, SG, OUT, 2, T>(p, line0, j0, sm, cs, tid); break;
  }
}

// ---------------------------------------------------------------------------
// Fused radix-16 sub-passes on the tensor cores (TC32 form).  Fragment layout,
// splitting and products as subpass16_tc (tc16.cuh): a warp takes 32
// butterflies in four chunks of 8; lane (g, q) holds inputs t = q + 4i of
// butterfly g of a chunk and, after the products, outputs k = g and g + 8 of
// butterflies 2q and 2q + 1.
// ---------------------------------------------------------------------------
// First radix-16 sub-pass from global memory (inter-pass twiddles applied on
// the way in) to the shared tile.
template <int SG, int IN, bool L2_ONLY>
__device__ __forceinline__ void first_subpass16_tc(const PassParams& p, long long line0,
                                                   long long j0, f2* sm, int cs,
                                                   const Dft16Frags& A, int tid) {
  using IE = typename IOElem<IN>::T;
  constexpr int sh = F32::kPadShift;
  const int lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int logR = p.logR, logRQ = logR - 4;
  const long long rs = (p.L >> logR) * p.s;
  const long long step = rs << logRQ;
  const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
  const int logS = p.logNs + logR;
  IE raw[4][4];
  int cc[4], jj[4];
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    butterfly_cj(warp * 32 + ch * 8 + g, p.in_rcontig, logRQ, p.logC, cc[ch], jj[ch]);
    if (cc[ch] < rem) {
      const IE* src = col_src<IN>(p, line0, j0, cc[ch]) + jj[ch] * rs;
#pragma unroll
      for (int i = 0; i < 4; ++i) load_elem<IE, L2_ONLY>(src + (q + 4 * i) * step, raw[ch][i]);
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) memset(&raw[ch][i], 0, sizeof(IE));
    }
  }
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    const long long jg = (p.mode == 0) ? j0 + cc[ch] : j0;
    const unsigned jm = (unsigned)(jg & (p.Ns - 1));
    float xr[4], xi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      F32::C v = gload<F32, IN>(&raw[ch][i], 0);
      const unsigned r = (unsigned)(jj[ch] + ((q + 4 * i) << logRQ));
      // jm * r < Ns * R <= L
      if (p.logNs > 0 && jm != 0 && r != 0) v = F32::mul(v, twiddle<F32>(p.tw, logS, jm * r, SG));
      xr[i] = v.x;
      xi[i] = v.y;
    }
    float dr[4], di[4];
    dft16_tc_products(A, xr, xi, dr, di);
    // outputs k = g, g + 8 of butterflies 2q, 2q + 1 at rows 16 j + k (Ns = 1)
#pragma unroll
    for (int c2 = 0; c2 < 2; ++c2) {
      int co, jo;
      butterfly_cj(warp * 32 + ch * 8 + 2 * q + c2, p.in_rcontig, logRQ, p.logC, co, jo);
      const int cb = co * cs;
      sm[cb + pidx(jo * 16 + g, sh)] = f2{dr[c2], di[c2]};
      sm[cb + pidx(jo * 16 + g + 8, sh)] = f2{dr[2 + c2], di[2 + c2]};
    }
  }
}

// Last radix-16 sub-pass (Ns = R/16) from the shared tile to global memory.
template <int SG, int OUT>
__device__ __forceinline__ void last_subpass16_tc(const PassParams& p, long long line0,
                                                  long long j0, const f2* sm, int cs,
                                                  const Dft16Frags& A, int tid) {
  using OE = typename IOElem<OUT>::T;
  constexpr int sh = F32::kPadShift;
  const int lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, q = lane & 3;
  const int logR = p.logR, logRQ = logR - 4;
  const f2* twd = reinterpret_cast<const f2*>(p.tw.dense);
  const long long rs = p.Ns * p.s;
  const long long step = rs << logRQ;
  const long long rem = (p.mode == 0) ? (1ll << 62) : p.nlines - line0;
#pragma unroll
  for (int ch = 0; ch < 4; ++ch) {
    int c, j;
    butterfly_cj(warp * 32 + ch * 8 + g, p.out_rcontig, logRQ, p.logC, c, j);
    const int cb = c * cs;
    float xr[4], xi[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int t = q + 4 * i;
      f2 v = sm[cb + pidx(j + (t << logRQ), sh)];
      if (j != 0 && t != 0) {
        // w_R^(j t), j < R/16
        const f2 w = twd[(1 << logR) + ((j * t) & ((1 << logR) - 1))];
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
    // outputs k = g, g + 8 of butterflies 2q, 2q + 1 at rows j + k R/16
#pragma unroll
    for (int c2 = 0; c2 < 2; ++c2) {
      int co, jo;
      butterfly_cj(warp * 32 + ch * 8 + 2 * q + c2, p.out_rcontig, logRQ, p.logC, co, jo);
      if (co >= rem) continue;
      OE* dst = col_dst<OUT>(p, line0, j0, co) + jo * rs;
      F32::C y0 = {dr[c2], di[c2]}, y1 = {dr[2 + c2], di[2 + c2]};
      if (p.do_scale) {
        y0 = apply_scale<F32>(y0, p);
        y1 = apply_scale<F32>(y1, p);
      }
      gstore<F32, OUT>(dst, g * step, y0);
      gstore<F32, OUT>(dst, (g + 8) * step, y1);
      if (p.spec_kind) {
        const long long i0 = col_index_out(p, line0, j0, co) + jo * rs;
        spec_store<F32>(p, i0 + g * step, y0);
        spec_store<F32>(p, i0 + (g + 8) * step, y1);
      }
    }
  }
}

// Fused tile of the TC32 form: radix-16 first and last sub-passes on the
// tensor cores straight from and to global memory; other radices on the CUDA
// cores (the form's arithmetic is FP32).
template <int SG, int IN, int OUT, int T, bool L2_ONLY>
__device__ __forceinline__ void pass_tile_fused_tc(const PassParams& p, long long tile, f2* sm,
                                                   int tid) {
  long long line0, j0;
  tile_origin(p, tile, line0, j0);
  if (p.nq == 1) {
    switch (p.q[0]) {
      case 4: only_subpass<TC32, SG, IN, OUT, 16, T, L2_ONLY>(p, line0, j0, tid); break;
      case 3: only_subpass<TC32, SG, IN, OUT, 8, T, L2_ONLY>(p, line0, j0, tid); break;
      case 2: only_subpass<TC32, SG, IN, OUT, 4, T, L2_ONLY>(p, line0, j0, tid); break;
      default: only_subpass<TC32, SG, IN, OUT, 2, T, L2_ONLY>(p, line0, j0, tid); break;
    }
    return;
  }
  const int cs = col_stride(p.logR, F32::kPadShift);
  Dft16Frags A;
  dft16_frags<SG>(reinterpret_cast<const f2*>(p.tw.dense), A);
  if (p.q[0] == 4) first_subpass16_tc<SG, IN, L2_ONLY>(p, line0, j0, sm, cs, A, tid);
  else first_subpass_q<TC32, SG, IN, T, L2_ONLY>(p.q[0], p, line0, j0, sm, cs, tid);
  __syncthreads();
  int logNsub = p.q[0];
  for (int k = 1; k + 1 < p.nq; ++k) {
    switch (p.q[k]) {
      case 4: subpass16_tc<SG>(sm, p.logR, cs, logNsub, p.tw, A, tid); break;
      case 3: subpass<TC32, SG, 8>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
      case 2: subpass<TC32, SG, 4>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
      default: subpass<TC32, SG, 2>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
    }
    logNsub += p.q[k];
  }
  const int lq = p.q[p.nq - 1];
  if (lq == 4) last_subpass16_tc<SG, OUT>(p, line0, j0, sm, cs, A, tid);
  else last_subpass_q<TC32, SG, OUT, T>(lq, p, line0, j0, sm, cs, tid);
}

template <class F, int SG, int IN, int OUT, int T, bool L2_ONLY>
__device__ __forceinline__ void pass_tile_fused(const PassParams& p, long long tile,
                                                typename F::S* sm, int tid) {
  long long line0, j0;
  tile_origin(p, tile, line0, j0);
  if (p.nq == 1) {
    switch (p.q[0]) {
      case 4: only_subpass<F, SG, IN, OUT, 16, T, L2_ONLY>(p, line0, j0, tid); break;
      case 3: only_subpass<F, SG, IN, OUT, 8, T, L2_ONLY>(p, line0, j0, tid); break;
      case 2: only_subpass<F, SG, IN, OUT, 4, T, L2_ONLY>(p, line0, j0, tid); break;
      default: only_subpass<F, SG, IN, OUT, 2, T, L2_ONLY>(p, line0, j0, tid); break;
    }
    return;
  }
  const int cs = col_stride(p.logR, F::kPadShift);
  first_subpass_q<F, SG, IN, T, L2_ONLY>(p.q[0], p, line0, j0, sm, cs, tid);
  __syncthreads();
  int logNsub = p.q[0];
  for (int k = 1; k + 1 < p.nq; ++k) {
    switch (p.q[k]) {
      case 4: subpass<F, SG, 16>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
      case 3: subpass<F, SG, 8>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
      case 2: subpass<F, SG, 4>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
      default: subpass<F, SG, 2>(sm, p.logR, cs, logNsub, p.tw, tid, T); break;
    }
    logNsub += p.q[k];
  }
  last_subpass_q<F, SG, OUT, T>(p.q[p.nq - 1], p, line0, j0, sm, cs, tid);
}

// One tile, fused (FUSE) or staged.
template <class F, int SG, int IN, int OUT, int T, bool L2_ONLY, bool FUSE>
__device__ __forceinline__ void run_tile(const PassParams& p, long long tile, typename F::S* sm,
                                         int tid) {
  if constexpr (FUSE && !F::kTensor) {
    pass_tile_fused<F, SG, IN, OUT, T, L2_ONLY>(p, tile, sm, tid);
  } else if constexpr (FUSE) {
    pass_tile_fused_tc<SG, IN, OUT, T, L2_ONLY>(p, tile, reinterpret_cast<f2*>(sm), tid);
  } else {
    pass_tile<F, SG, IN, OUT, T, L2_ONLY>(p, tile, sm, tid);
  }
}

// Whether the per-pass kernel fuses its first and last sub-passes with the
// global loads and stores.  Measured on four1 N=2^24: FP32 passes run 13 %
// faster fused, while the FP64-pipe bound FP64 and double-float passes run
// 11-14 % slower (their FP64-pipe time per pass grows), so those stay staged.
template <class F>
constexpr bool pass_fused() {
  return F::kind == 1;
}

// Resident 256-thread CTAs per SM that a pass kernel is compiled for.  The
// FP64 and double-float forms keep two (128 registers, 2 x 74 KB of shared
// memory), which covers the FP64 pipe's latency and holds their working set
// without spills.  The FP32 form is memory-latency bound, so it trades
// registers for resident warps: four CTAs (64 registers) when the input is
// FP32 scratch, three (80 registers) when it is the caller's f64 data, whose
// sixteen in-flight loads per thread need twice the registers.  TC32 keeps two:
// its DFT-matrix fragments alone take 32 registers.
template <class F, int IN>
constexpr int pass_min_blocks() {
  if constexpr (F::kind == 1 && !F::kTensor) return IN == IO_D2 ? 3 : 4;
  else return 2;  // FP64, double-float, and TC32 (its fragments need the registers)
}

// One CTA per tile.
template <class F, int SG, int IN, int OUT, int T>
__global__ void __launch_bounds__(T, (T == 256 ? pass_min_blocks<F, IN>() : 1))
    k_pass(PassParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the FP32-pipe forms read their tiles through L2 only (ld.global.cg): each
  // element is read once; same-GPU A/B, four1 2^28 FP32 4.73 -> 4.68 ms,
  // fourn 256 x 256 x 512 1.63 -> 1.62 ms
  run_tile<F, SG, IN, OUT, T, F::kind == 1, pass_fused<F>()>(
      p, blockIdx.x, reinterpret_cast<typename F::S*>(smem_raw), threadIdx.x);
}

template <class F>
inline size_t pass_smem_bytes(int T) {
  // rows padded as pidx, plus one element for each column of 16 rows or more
  const int E = kEPT * T;
  return sizeof(typename F::S) * (size_t)(E + (E >> F::kPadShift) + E / 16);
}

// Launch one k_pass instantiation; its dynamic shared memory limit is raised
// once per instantiation and device (the record lives in this function
// template).
template <class F, int SG, int IN, int OUT, int T>
inline cudaError_t launch_pass_one(const PassParams& p, cudaStream_t st) {
  static DeviceOnce attr_done;
  const size_t smem = pass_smem_bytes<F>(T);
  cudaError_t e = smem_opt_in(k_pass<F, SG, IN, OUT, T>, smem, attr_done);
  if (e != cudaSuccess) return e;
  if (p.tiles <= 0 || p.tiles > 0x7FFFFFFFll) return cudaErrorInvalidValue;  // grid.x limit
  PassParams q = p;
  set_slot_offsets(q, T);
  k_pass<F, SG, IN, OUT, T><<<dim3((unsigned)q.tiles), T, smem, st>>>(q);
  return cudaGetLastError();
}

template <class F, int SG, int IN, int OUT>
cudaError_t launch_pass_t(const PassParams& p, int threads, cudaStream_t st) {
  switch (threads) {
    case 256: return launch_pass_one<F, SG, IN, OUT, 256>(p, st);
    case 128: return launch_pass_one<F, SG, IN, OUT, 128>(p, st);
    case 64: return launch_pass_one<F, SG, IN, OUT, 64>(p, st);
    default: return launch_pass_one<F, SG, IN, OUT, 32>(p, st);
  }
}

// ---------------------------------------------------------------------------
// Latency kernel for the latency-mode plans (lone transforms of 2^10..2^14
// points, two passes of radix <= 2^7).  GB300 issues FP64 at 2 lanes per SM, so the FP64 time
// of a pass is set by how many SMs share its arithmetic: 16-point-per-thread
// tiles of 512 points put a 4096-point pass on 8 one-warp CTAs (8 SMs).
// These tiles hold 128 points, four per thread of one warp, with radix-2/4
// sub-passes, so the same pass runs on 32 SMs.  Staged tiles for every form;
// the radix <= 4 sub-passes run on the CUDA cores in the tensor-core form too.
// ---------------------------------------------------------------------------
constexpr int kLatThreads = 32;

template <class F, int SG, int IN, int OUT>
__global__ void __launch_bounds__(kLatThreads) k_pass_lat(PassParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pass_tile<F, SG, IN, OUT, kLatThreads, false, kLatencyEPT>(
      p, blockIdx.x, reinterpret_cast<typename F::S*>(smem_raw), threadIdx.x);
}

template <class F, int SG, int IN, int OUT>
inline cudaError_t launch_lat_one(const PassParams& p, cudaStream_t st) {
  constexpr int E = kLatencyEPT * kLatThreads;
  const size_t smem = sizeof(typename F::S) * (size_t)(E + (E >> F::kPadShift) + E / 16);
  if (p.tiles <= 0 || p.tiles > 0x7FFFFFFFll) return cudaErrorInvalidValue;
  if ((1 << (p.logR + p.logC)) != E || p.logR < 4) return cudaErrorInvalidValue;
  for (int k = 0; k < p.nq; ++k)
    if (p.q[k] < 1 || p.q[k] > 2) return cudaErrorInvalidValue;
  PassParams q = p;
  set_slot_offsets(q, kLatThreads);
  k_pass_lat<F, SG, IN, OUT><<<dim3((unsigned)q.tiles), kLatThreads, smem, st>>>(q);
  return cudaGetLastError();
}

template <class F, int SG>
cudaError_t dispatch_lat(IOType in, IOType out, const PassParams& p, cudaStream_t st) {
  constexpr int S = (F::kind == 2) ? IO_F4 : IO_F2;
  if (in == IO_D2 && out == IO_D2) return launch_lat_one<F, SG, IO_D2, IO_D2>(p, st);
  if constexpr (F::kind != 0) {
    if (in == IO_D2 && out == S) return launch_lat_one<F, SG, IO_D2, S>(p, st);
    if (in == S && out == IO_D2) return launch_lat_one<F, SG, S, IO_D2>(p, st);
    if (in == S && out == S) return launch_lat_one<F, SG, S, S>(p, st);
  }
  return cudaErrorInvalidValue;
}

// All IO combinations of one form and direction (FP64 uses double I/O only).
// Each (form, direction) is instantiated in its own translation unit so that
// the library builds in parallel.
template <class F, int SG>
cudaError_t dispatch_io(IOType in, IOType out, const PassParams& p, int threads,
                        cudaStream_t st) {
  constexpr int S = (F::kind == 2) ? IO_F4 : IO_F2;
  if (in == IO_D2 && out == IO_D2) return launch_pass_t<F, SG, IO_D2, IO_D2>(p, threads, st);
  if constexpr (F::kind != 0) {
    if (in == IO_D2 && out == S) return launch_pass_t<F, SG, IO_D2, S>(p, threads, st);
    if (in == S && out == IO_D2) return launch_pass_t<F, SG, S, IO_D2>(p, threads, st);
    if (in == S && out == S) return launch_pass_t<F, SG, S, S>(p, threads, st);
  }
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// realft twist fused into a pass (src/Real_FT.rs:24-46 forward, :120-142
// inverse, restated 0-based; the same arithmetic as k_realft_twist): the
// forward twist is applied by the last pass of the n/2-point forward FFT as it
// stores, the inverse twist by the first pass of the inverse FFT after it
// loads.  Output k of a line of L = n/2 points combines Z_k with Z_{L-k}, so a
// tile holds both: in a multi-pass schedule a "mirror tile" owns columns j and
// NC - j (NC = L/R columns per line); single-pass tiles hold whole lines.
// The input and output element types are dispatched at run time, so one
// kernel per form, direction and thread count serves every IO combination.
// ---------------------------------------------------------------------------
// Column of tile column c of mirror tile tl (tiles of C = 2^logC columns):
// the first C/2 columns are tl*C/2 + c, the second C/2 their mirrors NC - j
// in ascending order, with column NC/2 (its own mirror) standing in for the
// mirror of column 0.  Over the NC/C tiles every column appears once.
__device__ __forceinline__ long long mirror_col(long long tl, int c, int logC, long long NC) {
  const int half = 1 << (logC - 1);
  if (c < half) return tl * half + c;
  const long long j = NC - (tl + 1) * half + 1 + (c - half);
  return j == NC ? (NC >> 1) : j;
}

// Tile position (c2, r2) of the element paired with (c, r): index
// k = j + r NC of the line pairs with L - k = (NC - j) + (R - 1 - r) NC.
__device__ __forceinline__ void mirror_partner(long long tl, int c, int r, int logC, int logR,
                                               int& c2, int& r2) {
  const int Cn = 1 << logC, R = 1 << logR;
  if (tl == 0 && c == 0) { c2 = 0; r2 = (R - r) & (R - 1); }        // column 0
  else if (tl == 0 && c == Cn - 1) { c2 = Cn - 1; r2 = R - 1 - r; }  // column NC/2
  else { c2 = Cn - 1 - c; r2 = R - 1 - r; }
}

// Twisted value of slot k (0 < k < L) from Z_k (own) and Z_{L-k} (part):
// h1 = (Z_k + conj Z_{L-k})/2, h2 = -IS i (Z_k - conj Z_{L-k})/2, result
// h1 + w^k h2 with w = exp(IS 2 pi i / n), 2^logn = n.  Slot 0 packs DC and
// Nyquist: (h + v, h - v) forward, half that inverse.  Slot L/2 pairs with
// itself and comes out unchanged.
template <class F, int IS>
__device__ __forceinline__ typename F::C twist_elem(typename F::C own, typename F::C part,
                                                    long long k, int logn, const Twiddles& tw) {
  using C = typename F::C;
  if (k == 0) {
    const C s = F::add(C{own.x, own.x}, F::conj(C{own.y, own.y}));
    return IS > 0 ? s : F::scale(s, 0.5);
  }
  const C cp = F::conj(part);
  const C h1 = F::scale(F::add(own, cp), 0.5);
  const C h2 = F::scale(F::mul_j(F::sub(own, cp), -IS), 0.5);
  return F::add(h1, F::mul(h2, twiddle<F>(tw, logn, (unsigned)k, IS)));
}

// rlft3 form: h1 + w h2 for a twiddle w that is 1 at k = 0 (no DC packing;
// the k3 = 0 plane pairs with speq).  mate, when given, receives the value of
// the partner slot, conj(h1 - w h2).
template <class F, int IS>
__device__ __forceinline__ typename F::C twist_gen(typename F::C own, typename F::C part,
                                                   long long k, int logn, const Twiddles& tw,
                                                   typename F::C* mate = nullptr) {
  using C = typename F::C;
  const C cp = F::conj(part);
  const C h1 = F::scale(F::add(own, cp), 0.5);
  const C h2 = F::scale(F::mul_j(F::sub(own, cp), -IS), 0.5);
  const C t = (k == 0) ? h2 : F::mul(h2, twiddle<F>(tw, logn, (unsigned)k, IS));
  if (mate) *mate = F::conj(F::sub(h1, t));
  return F::add(h1, t);
}

// rlft3 mirror-line tiling of a pass whose lines form a U x V grid (line
// (u, v) = u V + v; U = 2^logU, V = 2^logV).  A line pairs with
// ((U - u) mod U, (V - v) mod V).  Rows u = 0 and U/2 pair with themselves
// and are tiled as a 1-D mirror tiling (mirror_col); the other rows go in
// pairs (u, U - u): a tile takes C/2 consecutive lines of row u and their
// C/2 mirrors in row U - u.  Tiles run [row 0][row U/2][row pairs].  Returns
// the line of tile column c, its (u, v), and in c2 the tile column of its
// mirror line.
__device__ __forceinline__ long long mirror_line(long long tile, int c, int logC, int logU,
                                                 int logV, int& c2, long long& v_out,
                                                 long long& u_out) {
  const long long U = 1ll << logU, V = 1ll << logV;
  const int Cn = 1 << logC, half = Cn >> 1;
  const long long tpr = V >> logC;  // tiles of a self-paired row
  long long u0, u1, tl;
  bool self;
  if (tile < tpr) { u0 = u1 = 0; tl = tile; self = true; }
  else if (U > 1 && tile < 2 * tpr) { u0 = u1 = U >> 1; tl = tile - tpr; self = true; }
  else {
    const long long t2 = tile - 2 * tpr;
    const int logper = logV - logC + 1;  // 2V/C tiles per row pair
    u0 = 1 + (t2 >> logper);
    u1 = U - u0;
    tl = t2 & ((1ll << logper) - 1);
    self = false;
  }
  long long u, v;
  if (c < half) {
    u = u0;
    v = tl * half + c;
  } else {
    u = u1;
    v = V - (tl + 1) * half + 1 + (c - half);
    if (v == V) v = self ? (V >> 1) : 0;
  }
  if (self && tl == 0 && c == 0) c2 = 0;
  else if (self && tl == 0 && c == Cn - 1) c2 = Cn - 1;
  else c2 = Cn - 1 - c;
  u_out = u;
  v_out = v;
  return u * V + v;
}

template <class F>
__device__ __forceinline__ typename F::C gload_rt(int io, const void* p, long long i) {
  if (io == IO_D2) return gload<F, IO_D2>(p, i);
  if (io == IO_F2) return gload<F, IO_F2>(p, i);
  return gload<F, IO_F4>(p, i);
}
template <class F>
__device__ __forceinline__ void gstore_rt(int io, void* p, long long i, typename F::C v) {
  if (io == IO_D2) gstore<F, IO_D2>(p, i, v);
  else if (io == IO_F2) gstore<F, IO_F2>(p, i, v);
  else gstore<F, IO_F4>(p, i, v);
}

// One tile per CTA, staged.  SG > 0: the forward FFT's last pass with the
// forward twist on its stores; SG < 0: the inverse FFT's first pass with the
// inverse twist on its loaded tile.  Lines are linear (no pointer tables).
template <class F, int SG, int T>
__global__ void __launch_bounds__(T) k_twist_pass(PassParams p, int in_io, int out_io) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using C = typename F::C;
  typename F::S* sm = reinterpret_cast<typename F::S*>(smem_raw);
  constexpr int sh = F::kPadShift;
  const int tid = threadIdx.x;
  const int logR = p.logR, logC = p.logC;
  const int R = 1 << logR, Cn = 1 << logC;
  const int cs = col_stride(logR, sh);
  const int logn = p.logL + 1;  // n = 2L reals
  long long line0, j0;
  tile_origin(p, blockIdx.x, line0, j0);
  const bool r3 = p.twist == 2 || p.twist == -2;  // rlft3: mirror lines
  const bool mir = !r3 && p.mode == 0;           // realft multi-pass: mirror columns
  const long long NC = p.L >> logR;
  const long long tl = mir ? (j0 >> logC) : 0;
  // line of tile column c (whole-line tiles)
  auto line_of = [&](int c) -> long long {
    if (!r3) return line0 + c;
    int c2;
    long long u, v;
    return mirror_line(blockIdx.x, c, logC, p.mirror_logU, p.mirror_logV, c2, v, u);
  };
  // 1. load the tile (all loads first), inter-pass twiddles, stage
  {
    C v[kEPT];
#pragma unroll
    for (int k = 0; k < kEPT; ++k) {
      int c, r;
      elem_cr(tid + k * T, p.in_rcontig, logR, logC, c, r);
      const long long line = mir ? line0 : line_of(c);
      const long long j = mir ? mirror_col(tl, c, logC, NC) : j0;
      v[k] = (line < p.nlines)
                 ? gload_rt<F>(in_io, p.in, line_base(p, line) + (j + (long long)r * NC) * p.s)
                 : F::from_d(0.0, 0.0);
    }
#pragma unroll
    for (int k = 0; k < kEPT; ++k) {
      int c, r;
      elem_cr(tid + k * T, p.in_rcontig, logR, logC, c, r);
      if (p.logNs > 0) {
        const long long j = mir ? mirror_col(tl, c, logC, NC) : j0;
        const unsigned jm = (unsigned)(j & (p.Ns - 1));
        if (jm != 0 && r != 0)
          v[k] = F::mul(v[k], twiddle<F>(p.tw, p.logNs + logR, jm * (unsigned)r, SG));
      }
      sm[c * cs + pidx(r, sh)] = F::to_s(v[k]);
    }
  }
  __syncthreads();
  // 2. inverse twist of the loaded tile (first pass of the inverse FFT)
  if constexpr (SG < 0) {
    C tv[kEPT];
#pragma unroll
    for (int k = 0; k < kEPT; ++k) {
      const int e = tid + k * T;
      const int c = e & (Cn - 1), r = e >> logC;
      int c2 = c, r2 = (R - r) & (R - 1);
      if (r3) {
        // rows are i3 (R = nn3/2 points); row 0 pairs with speq at the
        // mirrored (i1, i2), the others with row R - r of the mirror line
        long long u, vv;
        mirror_line(blockIdx.x, c, logC, p.mirror_logU, p.mirror_logV, c2, vv, u);
        C part;
        if (r == 0) {
          const long long U = 1ll << p.mirror_logU, V = 1ll << p.mirror_logV;
          const d2 sq =
              reinterpret_cast<const d2*>(p.aux)[((U - u) & (U - 1)) * V + ((V - vv) & (V - 1))];
          part = F::from_d(sq.x, sq.y);
        } else {
          part = F::from_s(sm[c2 * cs + pidx(r2, sh)]);
        }
        tv[k] = twist_gen<F, -1>(F::from_s(sm[c * cs + pidx(r, sh)]), part, r, logR + 1, p.tw);
        continue;
      }
      if (mir) mirror_partner(tl, c, r, logC, logR, c2, r2);
      const long long kk = mir ? mirror_col(tl, c, logC, NC) + (long long)r * NC : r;
      tv[k] = twist_elem<F, -1>(F::from_s(sm[c * cs + pidx(r, sh)]),
                                F::from_s(sm[c2 * cs + pidx(r2, sh)]), kk, logn, p.tw);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kEPT; ++k) {
      const int e = tid + k * T;
      sm[(e & (Cn - 1)) * cs + pidx(e >> logC, sh)] = F::to_s(tv[k]);
    }
    __syncthreads();
  }
  // 3. the R-point DFTs of the columns
  run_subpasses<F, SG, T>(p, sm, cs, tid);
  // 4. store at the autosorted positions (forward twist in the last pass)
#pragma unroll 4
  for (int k = 0; k < kEPT; ++k) {
    int c, r;
    elem_cr(tid + k * T, p.out_rcontig, logR, logC, c, r);
    int c3 = c;
    long long u3 = 0, v3 = 0;
    const long long line =
        mir ? line0
            : (r3 ? mirror_line(blockIdx.x, c, logC, p.mirror_logU, p.mirror_logV, c3, v3, u3)
                  : line0 + c);
    if (line >= p.nlines) continue;
    const long long j = mir ? mirror_col(tl, c, logC, NC) : j0;
    const long long jd = ((j >> p.logNs) << (p.logNs + logR)) + (j & (p.Ns - 1));
    C v = F::from_s(sm[c * cs + pidx(r, sh)]);
    if constexpr (SG > 0) {
      int c2 = c, r2 = (R - r) & (R - 1);
      if (r3) {
        // rows are i1 (the axis-0 pass); the twist runs along i3 = v3 of the
        // line; the i3 = 0 lines also write speq at the mirrored (i1, i2)
        C mate;
        v = twist_gen<F, 1>(v, F::from_s(sm[c3 * cs + pidx(r2, sh)]), v3, p.mirror_logV + 1,
                            p.tw, &mate);
        if (v3 == 0) {
          const long long U = 1ll << p.mirror_logU;
          double mx, my;
          F::to_d(mate, mx, my);
          reinterpret_cast<d2*>(p.aux)[(long long)((R - r) & (R - 1)) * U + ((U - u3) & (U - 1))] =
              d2{mx, my};
        }
      } else {
        if (mir) mirror_partner(tl, c, r, logC, logR, c2, r2);
        v = twist_elem<F, 1>(v, F::from_s(sm[c2 * cs + pidx(r2, sh)]), jd + (long long)r * p.Ns,
                             logn, p.tw);
      }
    }
    if (p.do_scale) v = apply_scale<F>(v, p);
    gstore_rt<F>(out_io, p.out, line_base(p, line) + (jd + (long long)r * p.Ns) * p.s, v);
  }
}

template <class F, int SG, int T>
inline cudaError_t launch_twist_one(IOType in, IOType out, const PassParams& p, cudaStream_t st) {
  static DeviceOnce attr_done;
  const size_t smem = pass_smem_bytes<F>(T);
  cudaError_t e = smem_opt_in(k_twist_pass<F, SG, T>, smem, attr_done);
  if (e != cudaSuccess) return e;
  if (p.tiles <= 0 || p.tiles > 0x7FFFFFFFll) return cudaErrorInvalidValue;
  k_twist_pass<F, SG, T><<<dim3((unsigned)p.tiles), T, smem, st>>>(p, (int)in, (int)out);
  return cudaGetLastError();
}

template <class F, int SG>
cudaError_t dispatch_twist(IOType in, IOType out, const PassParams& p, int threads,
                           cudaStream_t st) {
  switch (threads) {
    case 256: return launch_twist_one<F, SG, 256>(in, out, p, st);
    case 128: return launch_twist_one<F, SG, 128>(in, out, p, st);
    case 64: return launch_twist_one<F, SG, 64>(in, out, p, st);
    default: return launch_twist_one<F, SG, 32>(in, out, p, st);
  }
}

#define GBFFT_DECLARE_DISPATCH(FORM)                                                          \
  extern template cudaError_t dispatch_io<FORM, 1>(IOType, IOType, const PassParams&, int,    \
                                                   cudaStream_t);                             \
  extern template cudaError_t dispatch_io<FORM, -1>(IOType, IOType, const PassParams&, int,   \
                                                    cudaStream_t);                            \
  extern template cudaError_t dispatch_twist<FORM, 1>(IOType, IOType, const PassParams&, int, \
                                                      cudaStream_t);                          \
  extern template cudaError_t dispatch_twist<FORM, -1>(IOType, IOType, const PassParams&, int, \
                                                       cudaStream_t);

}  // namespace gbfft
