// gbfft_internal.h -- declarations shared by the kernel translation units and
// the host runtime.  Nothing here is part of the public C ABI (include/gbfft.h).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>

namespace gbfft {

enum Form : int { FORM_F64 = 0, FORM_F32 = 1, FORM_DF64 = 2, FORM_TC32 = 3 };
constexpr int kForms = 4;

// Element types a pass reads or writes in global memory.
//   IO_D2  interleaved double complex (the caller's layout)
//   IO_F2  float complex (FP32 intermediate)
//   IO_F4  double-float complex (re.hi, re.lo, im.hi, im.lo) (DF64 intermediate)
enum IOType : int { IO_D2 = 0, IO_F2 = 1, IO_F4 = 2 };

inline size_t io_bytes(IOType t) { return t == IO_F2 ? 8 : 16; }

// Twiddle tables of one form.  dense holds levels S = 2^1 .. 2^dense_log
// back to back, entry S+e = exp(+2 pi i e / S).  partial holds, for each
// level S = 2^(dense_log+1) .. 2^kMaxLog, the first kPartial entries of that
// level; a twiddle of a larger level is the product of one dense entry of
// level S/kPartial and one partial entry (two loads and one complex product
// instead of one load).  The library's tables are dense up to 2^kDenseLog
// (2^20: every twiddle of an axis of up to 2^20 points is one load); the
// no-allocation entry point keeps its fixed tables at the smaller
// kDenseLogMin.
constexpr int kDenseLog = 20;
constexpr int kDenseLogMin = 16;
constexpr int kPartialLog = 12;
constexpr int kPartial = 1 << kPartialLog;
constexpr int kMaxLog = kDenseLogMin + kPartialLog;  // 2^28 points per axis
__host__ __device__ constexpr size_t dense_entries(int dense_log) { return size_t(2) << dense_log; }
__host__ __device__ constexpr size_t partial_entries(int dense_log) {
  return size_t(kMaxLog - dense_log) * kPartial;
}

constexpr int kTileEPT = 16;  // complex elements per thread per tile
constexpr int kLatencyEPT = 4;  // elements per thread in the latency kernel's tiles

struct Twiddles {
  const void* dense = nullptr;
  const void* partial = nullptr;
  int dense_log = kDenseLog;  // largest level held densely
  // optional dense copy of one level above dense_log (the last pass of a
  // long FP64 or double-float axis): entry e = w_{2^top_log}^e; 0 = none
  const void* top = nullptr;
  int top_log = 0;
};

// One Stockham pass over an axis.  The axis has length L and stride s
// (complex elements).  Lines are the independent 1-D sequences along the
// axis; line l starts at (l >> lq_log) * lstride + (l & ((1<<lq_log)-1)).
// The pass applies, to every column j in [0, L/R), the twiddles
// w_{Ns R}^{(j mod Ns) r} and an R-point DFT, reading element r at
// j + r L/R and writing it at expand(j) + r Ns (Stockham autosort).
// A CTA works on a tile of C = 2^logC columns:
//   mode 0  the columns are C consecutive j of one line (s == 1, L/R >= C)
//   mode 1  the columns are C consecutive lines at one j
struct PassParams {
  const void* in;
  void* out;
  // optional per-line base pointers (complex elements of the IO type); when
  // set they replace in/out + the line offset (lines are separate arrays)
  const void* const* in_ptrs;
  void* const* out_ptrs;
  Twiddles tw;
  long long L;
  long long s;
  long long lstride;
  long long nlines;
  long long Ns;
  int lq_log;
  int logL;
  int logR;
  int logC;
  int logNs;
  int mode;
  int in_rcontig;   // 1: tile elements are contiguous along r in global memory
  int out_rcontig;
  int nq;
  int q[4];         // log2 of the in-CTA sub-pass radices (sum = logR)
  int do_scale;
  double scale;
  float fscale;     // scale as a float for the FP32-pipe forms (set at launch)
  long long tiles;  // grid size
  // Spectrum epilogue (last pass of a transform, linear layouts only): beside
  // the complex output element i, spec[i] = |X| (spec_kind 1) or |X|^2
  // (spec_kind 2); 0 = off.
  double* spec;
  int spec_kind;
  // Real-transform twist fused into this pass (the pass runs as k_twist_pass):
  //   +1 / -1  realft (src/Real_FT.rs:24-46,120-142): forward twist after the
  //            last pass of the forward FFT / inverse twist before the first
  //            pass of the inverse FFT; lines have L = n/2 points
  //   +2 / -2  rlft3 (src/Real_FT3.rs:58-127): the forward twist in the last
  //            (axis-0) pass of the forward 3-D FFT, the inverse twist in the
  //            first (last-axis) pass of the inverse; the pass's lines form a
  //            grid of 2^mirror_logU x 2^mirror_logV lines, and aux is speq
  //   0        none
  int twist;
  int mirror_logU;
  int mirror_logV;
  double* aux;
  // 1: the pass runs on a four-CTA cluster (k_pass_cl, FP32 two-pass plans):
  // tiles of four columns, logC = 2, one cluster per tile
  int cluster;
  // 1: a latency-mode pass (k_pass_lat): one-warp tiles of 128 points, four
  // per thread, radix-2/4 sub-passes
  int lat;
  // Per-slot parts of the global element indices of a tile, for layouts
  // without per-line pointer tables: slot k of thread tid holds tile element
  // e = tid + k*T, and its index is a per-thread base plus in_off[k] (load
  // order) or out_off[k] (store order).  Filled for the launch's thread count
  // T by set_slot_offsets.
  long long in_off[kTileEPT];
  long long out_off[kTileEPT];
};

// (column, row) of tile element e: e splits at bit b = logR when the tile's
// columns are contiguous runs of rows in memory (rcontig), at b = logC
// otherwise.  For e = tid + k*T with T a power of two, the thread's part and
// the slot's part of e occupy disjoint bits, so the column and row of e are
// the sums of those of tid and of k*T.
__host__ __device__ inline void tile_cr(long long e, int rcontig, int logR, int logC, long long& c,
                                        long long& r) {
  if (rcontig) { r = e & ((1ll << logR) - 1); c = e >> logR; }
  else { c = e & ((1ll << logC) - 1); r = e >> logC; }
}

// Index offset of tile column c from column 0, input and output side.  Both
// are linear in the bit fields of c (mode 0: columns are consecutive j of one
// line; mode 1: consecutive lines of the line grouping), so the offset of a
// sum of disjoint-bit columns is the sum of their offsets.
__host__ __device__ inline long long col_off_in(const PassParams& p, long long c) {
  if (p.mode == 0) return c * p.s;
  return (c >> p.lq_log) * p.lstride + (c & ((1ll << p.lq_log) - 1));
}
__host__ __device__ inline long long col_off_out(const PassParams& p, long long c) {
  if (p.mode == 0) return (((c >> p.logNs) << (p.logNs + p.logR)) + (c & (p.Ns - 1))) * p.s;
  return (c >> p.lq_log) * p.lstride + (c & ((1ll << p.lq_log) - 1));
}

inline void set_slot_offsets(PassParams& p, int T) {
  // the float copy of the output scale, converted once on the host so that no
  // kernel converts it per element (a double->float conversion runs on the
  // FP64 pipe)
  p.fscale = (float)p.scale;
  const long long rs_in = (p.L >> p.logR) * p.s;
  const long long rs_out = p.Ns * p.s;
  for (int k = 0; k < kTileEPT; ++k) {
    long long c, r;
    tile_cr((long long)k * T, p.in_rcontig, p.logR, p.logC, c, r);
    p.in_off[k] = col_off_in(p, c) + r * rs_in;
    tile_cr((long long)k * T, p.out_rcontig, p.logR, p.logC, c, r);
    p.out_off[k] = col_off_out(p, c) + r * rs_out;
  }
}

// kernel launchers (one per form, defined in fft_<form>.cu)
cudaError_t launch_pass_f64(int sign, IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st);
cudaError_t launch_pass_f32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st);
cudaError_t launch_pass_df64(int sign, IOType in, IOType out, const PassParams& p, int threads,
                             cudaStream_t st);
cudaError_t launch_pass_tc32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                             cudaStream_t st);
// latency-mode pass of any form (fft_lat.cu)
cudaError_t launch_pass_lat(Form f, int sign, IOType in, IOType out, const PassParams& p,
                            cudaStream_t st);
// FP32 pass of a two-pass plan on a four-CTA cluster (fft_f32_cl_*.cu)
cudaError_t launch_pass_cl_f32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                               cudaStream_t st);
cudaError_t launch_twiddles(Form f, void* dense, void* partial, int dense_log, cudaStream_t st);
cudaError_t launch_twiddle_level(Form f, void* level, int logS, cudaStream_t st);

// spectral / real-transform kernels (spectral.cu)
struct SpecArgs {
  Twiddles tw;
  int form;
};
// realft twist on `batch` packed real transforms of n reals each (data viewed
// as n/2 complex), lines `dist` doubles apart.  isign=+1: after the forward
// n/2-point FFT; isign=-1: before the inverse FFT.
cudaError_t launch_realft_twist(Form f, int isign, double* data, long long n, long long batch,
                                long long dist, Twiddles tw, cudaStream_t st);
// Fused convlv/correl spectral step on two raw n/2-point spectra A (data) and
// B (response / data2), each n/2 complex: forward twists, product (kind 0:
// convolve, 1: deconvolve, 2: correlate), scale 1/(n/2), inverse twist.
// Writes the packed input of the inverse n/2-point FFT to out (may alias a).
cudaError_t launch_spectral_product(Form f, int kind, const double* a, const double* b,
                                    double* out, long long n, Twiddles tw, cudaStream_t st);
// The same step on `lines` lines whose a, b, out are sa, sb, so doubles apart
// (sb = 0: one shared response spectrum).
cudaError_t launch_spectral_lines(Form f, int kind, const double* a, long long sa,
                                  const double* b, long long sb, double* out, long long so,
                                  long long lines, long long n, Twiddles tw, cudaStream_t st);
// Numerical Recipes wrap-around expansion of an m-tap response into n reals;
// also copies `data` (n reals) to dst_data when non-null.
cudaError_t launch_expand_response(const double* respns, long long m, double* dst, long long n,
                                   const double* data, double* dst_data, cudaStream_t st);
// Direct linear correlation for n <= 32 (the reference's small-n branch).
cudaError_t launch_correl_direct(const double* a, const double* b, double* out, long long n,
                                 cudaStream_t st);
// twofft split (Numerical Recipes contract): fft1 holds the n-point FFT of
// data1 + i data2; writes the two spectra into fft1 / fft2.
cudaError_t launch_twofft_pack(const double* d1, const double* d2, double* fft1, long long n,
                               cudaStream_t st);
cudaError_t launch_twofft_split(double* fft1, double* fft2, long long n, cudaStream_t st);
// twofft-packed convlv/correl: z = a + i s b (m > 0: b is an m-tap response,
// expanded in wrap-around order; s a power of two near |a|/|b| computed on the
// device into sums[0..1], or 1 when sums is null), then after the n-point FFT
// the fused split, product (undoing s) and inverse twist in place (kind as
// launch_spectral_product; the same sums).
cudaError_t launch_pack_pair(const double* a, const double* b, long long m, double* z, long long n,
                             double* sums, cudaStream_t st);
cudaError_t launch_spectral_two(Form f, int kind, double* z, long long n, Twiddles tw,
                                const double* sums, cudaStream_t st);
// rlft3 steps: speq gather (forward) and the twist along the last axis.
cudaError_t launch_rlft3_speq(const double* data, double* speq, long long nn1, long long nn2,
                              long long nn3, cudaStream_t st);
cudaError_t launch_rlft3_twist(Form f, int isign, double* data, double* speq, long long nn1,
                               long long nn2, long long nn3, Twiddles tw, cudaStream_t st);
// sine / cosine transform pre- and post-passes around realft.
cudaError_t launch_sinft_pre(double* y, long long n, Twiddles tw, cudaStream_t st);
cudaError_t launch_cosft1_pre(double* y, long long n, double* partial, Twiddles tw,
                              cudaStream_t st);
cudaError_t launch_cosft2_pre(int isign, double* y, long long n, Twiddles tw, cudaStream_t st);
cudaError_t launch_cosft2_rot(int isign, double* y, long long n, Twiddles tw, cudaStream_t st);
cudaError_t launch_cosft2_inv_pre(const double* y, double* w, long long n, Twiddles tw,
                                  cudaStream_t st);
cudaError_t launch_cosft2_inv_post(const double* w, double* y, long long n, Twiddles tw,
                                   cudaStream_t st);
// Ordered prefix sums on the odd/even slots after realft (sinft/cosft1/cosft2).
cudaError_t launch_trig_scan(int kind, double* y, long long n, double* partial, double* work,
                             cudaStream_t st);
cudaError_t launch_scale(double* data, long long count, double s, cudaStream_t st);
cudaError_t launch_set_lines(const void** dst, const void* a, const void* b, cudaStream_t st);
// Normalised correlation helpers (src/Correlation.rs:189-270).
cudaError_t launch_correl_direct_centered(const double* a, const double* b, double* out,
                                          long long n, double ma, double mb, double norm,
                                          cudaStream_t st);
cudaError_t launch_moment(const double* x, long long n, double shift, int p, double* partial,
                          double* out, cudaStream_t st);
cudaError_t launch_standardize(const double* x, long long n, double mean, double stdv,
                               double* out, cudaStream_t st);
cudaError_t launch_twiddle_lines(double* data, long long lines, int loglen, long long line0,
                                 int logn, int isign, const Twiddles& tw, cudaStream_t st);
cudaError_t launch_spectrum(int kind, const double* c, double* out, long long nn,
                            cudaStream_t st);

}  // namespace gbfft
