/*
 * gbfft.h -- C ABI of the GB300 FFT library (libgbfft.so).
 *
 * Drop-in boundary for the FFT family of the numrs crate.  Each entry point
 * replaces one Rust function of the crate; the crate's conventions are kept:
 *
 *   - data are interleaved f64 (re, im, re, im, ...) and transformed in place
 *   - isign = +1 computes X_k = sum_j x_j exp(+2 pi i jk/N), isign = -1 the
 *     conjugate sum; transforms are unnormalised
 *   - realft packs Re X_{n/2} into data[1]; rlft3 returns the Nyquist plane in
 *     speq; convlv takes its response in wrap-around order and scales by 2/n
 *
 * Arrays are 0-based.  Routines whose Rust versions take 1-based slices
 * (cosft1, cosft2) take the 0-based array that starts at the crate's index 1.
 *
 * Every function returns a gbfft_status.  Pointers are host memory unless
 * opts->device_ptrs is set.  Calls are synchronous for host pointers; for
 * device pointers they are ordered on opts->stream (NULL = the default
 * stream) and synchronous unless opts->async is set.  Device arrays that a
 * transform works on in place must start on a 16-byte boundary (cudaMalloc
 * memory always does); an unaligned one is rejected with GBFFT_INVALID_ARG
 * before any launch.  Host arrays may start on any 8-byte boundary.  Calls
 * share the library's work buffers: an asynchronous call on one stream is
 * ordered (by an event) before any later call on another stream.  The
 * library is thread-safe (one internal lock).  No entry point changes any GPU
 * setting.
 */
#ifndef GBFFT_H
#define GBFFT_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GBFFT_OK = 0,
  GBFFT_INVALID_ARG = 1,       /* bad isign, null pointer, length mismatch ...   */
  GBFFT_UNSUPPORTED_SIZE = 2,  /* size is not a power of two or exceeds limits   */
  GBFFT_CUDA_ERROR = 3,        /* a CUDA call failed; see gbfft_last_error()     */
  GBFFT_TIMEOUT = 4,           /* a bounded device wait gave up                  */
  GBFFT_OOM = 5,               /* device allocation failed                       */
  /* convlv / correl error enums of the crate (Convolve.rs:226-238,
   * Correlation.rs:389-399) */
  GBFFT_EMPTY_INPUT = 10,
  GBFFT_RESPONSE_TOO_LONG = 11,
  GBFFT_INVALID_ISIGN = 12,
  GBFFT_LENGTH_MISMATCH = 13,
  GBFFT_ZERO_STD_DEV = 14
} gbfft_status;

/* Arithmetic form of a call. */
typedef enum {
  GBFFT_FORM_FP64 = 0,  /* IEEE double throughout (the crate's arithmetic)      */
  GBFFT_FORM_FP32 = 1,  /* IEEE float arithmetic, f64 in and out               */
  GBFFT_FORM_DF64 = 2,  /* double-float (compensated FP32 pairs), f64 in/out    */
  GBFFT_FORM_TC32 = 3   /* FP32, radix-16 stages as 3xTF32 tensor-core products */
} gbfft_form;

typedef struct {
  int form;          /* gbfft_form; 0 = FP64                                   */
  int device_ptrs;   /* 1: all array arguments are device pointers             */
  void* stream;      /* cudaStream_t of device-pointer calls, NULL = default   */
  int async;         /* device-pointer calls only: 1 = do not synchronise      */
} gbfft_opts;

/* Library control ------------------------------------------------------- */
/* Optional: binds the library to `device`.  Without it (or with -1) the first
 * call binds it to the device current on the calling thread.  Every later
 * call runs on that device and leaves the caller's current device as it was.
 * Naming another device once bound is GBFFT_INVALID_ARG. */
int gbfft_init(int device);
const char* gbfft_last_error(void);      /* message of the last failure      */
int gbfft_version(void);                 /* 10000*major + 100*minor + patch  */
/* Device scratch currently held by the library, in bytes. */
size_t gbfft_scratch_bytes(void);
/* Free cached plans, graphs, scratch and the dense copies of large twiddle
 * levels (the base twiddle tables are kept). */
int gbfft_release(void);
/* Autotuner (no counterpart in the crate): when enabled, the first plan of
 * each axis shape and form times candidate tile sizes on a scratch array and
 * keeps the fastest, and the first batch of each signature (form, direction,
 * multiset of sizes) times candidate schedules of the persistent launch --
 * the first-pass radix of every bin above 4096 points and the resident CTAs
 * per SM -- on a zeroed device copy of the batch (also GBFFT_AUTOTUNE=1;
 * GBFFT_TUNE_CACHE=<file> keeps the choices across processes).  Tuning
 * synchronises the device once per shape or signature. */
int gbfft_set_autotune(int enable);
/* Forward transforms of gbfft_convlv / gbfft_correl (no counterpart switch in
 * the crate; the batched forms always use path 0, which transforms a shared
 * response once):
 *   0  the two real inputs as two n/2-point realft lines in one batched
 *      launch sequence (the default)
 *   1  the two real inputs packed as the real and imaginary parts of one
 *      n-point complex FFT, as twofft does (src/FFT_2.rs:3-17), then one
 *      kernel splits the two spectra, multiplies them and applies the
 *      inverse realft twist
 * Both give the same results within the parity bars. */
int gbfft_set_spectral_path(int path);
/* Instrumentation (no counterpart in the crate).  Kernel launches issued
 * since the last reset; optional event timing of every launch on its stream,
 * summed per kind: 0 = FFT passes, 1 = realft twists, 2 = spectral products,
 * 3 = other.  bytes = algorithmic bytes moved by those launches, flops =
 * nominal 5 N log2 R of each radix-R pass over N points. */
long long gbfft_launch_count(int reset);
/* Failure injection for tests (no counterpart in the crate).  Keys:
 *   GBFFT_DEBUG_FAIL_ALLOC_AT     the value-th device allocation from now on
 *                                 fails as if the device were out of memory
 *                                 (the call returns GBFFT_OOM); 0 = never
 *   GBFFT_DEBUG_BATCH_SPIN_LIMIT  polls before a wait of the persistent batch
 *                                 kernel gives up (0 = the default, 2^24)
 *   GBFFT_DEBUG_BATCH_NEED_EXTRA  added to the tile count a pass-2 tile waits
 *                                 for, so that its wait cannot be met and
 *                                 must run out (the call returns
 *                                 GBFFT_TIMEOUT); 0 = off
 *   GBFFT_DEBUG_BATCH_FIRST_RADIX_DELTA  shifts the first-pass radix of the
 *                                 batch launch's two-pass bins away from
 *                                 half the length (the splits the autotuner
 *                                 tries), so tests can check each one
 *   GBFFT_DEBUG_FUSED_TWIST       0: realft runs its twist as a kernel of its
 *                                 own instead of on a pass (1, the default)
 *   GBFFT_DEBUG_TC_UMMA           1: the tensor-core batch form on tcgen05
 *                                 (the default), 0: on mma.sync (also
 *                                 GBFFT_TC_UMMA=0 at start-up)
 *   GBFFT_DEBUG_CLUSTER_PASS      1: FP32 axes of 2^22..2^28 points run as
 *                                 two passes on four-CTA clusters (also
 *                                 GBFFT_CLUSTER_PASS=1 at start-up), 0: as
 *                                 three per-CTA passes (the default, faster)
 *   GBFFT_DEBUG_TOP_TWIDDLES      1: the last pass of a long FP64 axis
 *                                 reads its twiddles from a dense copy of
 *                                 their level (the default), 0: as products
 *                                 of two table entries (also
 *                                 GBFFT_TOP_TWIDDLES=0 at start-up)
 * The batch settings drop the cached batch plan.  Nothing here hangs or
 * faults a GPU: every device wait stays bounded. */
enum {
  GBFFT_DEBUG_FAIL_ALLOC_AT = 1,
  GBFFT_DEBUG_BATCH_SPIN_LIMIT = 2,
  GBFFT_DEBUG_BATCH_NEED_EXTRA = 3,
  GBFFT_DEBUG_BATCH_FIRST_RADIX_DELTA = 4,
  GBFFT_DEBUG_FUSED_TWIST = 5,
  GBFFT_DEBUG_TC_UMMA = 6,
  GBFFT_DEBUG_CLUSTER_PASS = 7,
  GBFFT_DEBUG_TOP_TWIDDLES = 8
};
int gbfft_debug_set(int key, long long value);
int gbfft_profile(int enable);  /* also clears the records */
int gbfft_profile_read(int kind, double* ms, long long* launches, double* bytes,
                       double* flops);

/* Complex FFT ----------------------------------------------------------- */
/* four1: src/FFT_1.rs:5 `pub fn four1(data: &mut [f64], nn: usize, isign: i32)`.
 * data holds 2*nn doubles; nn a power of two <= 2^28. */
int gbfft_four1(double* data, size_t nn, int isign, const gbfft_opts* opts);

/* FFTProcessor::fft_batch: src/FFT_1.rs:185
 * `pub fn fft_batch(&self, batches: &mut [&mut [f64]], isign: i32)`.
 * count transforms, ptrs[t] holds 2*nn[t] doubles; sizes may differ. */
int gbfft_four1_batch(double* const* ptrs, const size_t* nn, size_t count, int isign,
                      const gbfft_opts* opts);

/* four1 that allocates nothing.  No counterpart in the crate: it serves
 * callers that cannot call cudaMalloc when they need a transform (hosts that
 * fix their GPU memory budget up front, such as real-time or embedded
 * systems, and plugins inside another framework's memory pool that may not
 * allocate behind its back).  Same transform as gbfft_four1 in FP64, in place
 * on DEVICE memory `data` (16-byte aligned), ordered on `stream`
 * (NULL = default).
 * Its scratch and twiddle tables are fixed arrays in the library image (about
 * 19 MiB held by every GPU that loads the library, until exit), so nn is
 * limited to 2^20 (GBFFT_UNSUPPORTED_SIZE above).  The first call on a device
 * sets it up and waits for that; make it before any stream capture (a first
 * call on a capturing stream is refused with GBFFT_CUDA_ERROR).  Calls share
 * the scratch array, which keeps the last call's contents: calls that overlap
 * on the GPU race and must be ordered by the caller. */
int gbfft_four1_noalloc(double* data, size_t nn, int isign, void* stream);

/* FFTProcessor::fft followed by magnitude_spectrum (kind 0) or power_spectrum
 * (kind 1): src/FFT_1.rs:166,206,218.  data (2*nn doubles) is transformed in
 * place as gbfft_four1 does, and the transform's last pass also writes
 * spec[k] = |X_k| or |X_k|^2 (k < nn) from the values it stores, so the
 * spectrum costs no pass of its own over the data. */
int gbfft_four1_spectrum(double* data, size_t nn, int isign, int kind, double* spec,
                         const gbfft_opts* opts);

/* Uniform batch: `count` transforms of nn points, `dist` doubles apart
 * (dist >= 2*nn). */
int gbfft_four1_many(double* data, size_t nn, size_t count, size_t dist, int isign,
                     const gbfft_opts* opts);

/* twofft: src/FFT_2.rs:3
 * `pub fn twofft(data1: &[f64], data2: &[f64], fft1: &mut [f64], fft2: &mut [f64])`.
 * data1, data2: n reals; fft1, fft2: 2n+2 doubles (the n-point spectra fill
 * [0, 2n); the last two doubles are left as they are). */
int gbfft_twofft(const double* data1, const double* data2, double* fft1, double* fft2,
                 size_t n, const gbfft_opts* opts);

/* Real FFT -------------------------------------------------------------- */
/* realft: src/Real_FT.rs:4 `pub fn realft(data: &mut [f64], n: usize, isign: i32)`.
 * n reals (power of two >= 2).  Forward output: data[0] = X_0,
 * data[1] = X_{n/2}, data[2k], data[2k+1] = Re, Im X_k.  Inverse returns
 * (n/2) x. */
int gbfft_realft(double* data, size_t n, int isign, const gbfft_opts* opts);

/* fourn: src/Fourn.rs:278 `fourn_simd(data: &mut [f64], nn: &[usize], ndim, isign)`
 * with validate_inputs (src/Fourn.rs:367-378): ndim in 1..=nn_len, isign +-1,
 * every nn[d] > 1.  Row-major, nn[ndim-1] contiguous. */
int gbfft_fourn(double* data, const size_t* nn, size_t nn_len, size_t ndim, int isign,
                const gbfft_opts* opts);

/* FourFS::fourfs: src/Four_FS.rs:55 `fourfs(&mut self, nn: &[usize], ndim, isign)`,
 * the out-of-core N-D FFT (validate_inputs, src/Four_FS.rs:328-339, as fourn).
 * data is HOST memory (it may be larger than the GPU's memory), row-major,
 * interleaved complex, transformed in place; every pass reads and writes host
 * memory directly over the CPU-GPU link, and the GPU holds only its twiddle
 * tables.  work: host scratch of 16 bytes per complex element, or NULL for one
 * allocated (pageable) for the call.  data and work start on 16-byte
 * boundaries.  Needs a GPU that reaches pageable host memory through the host
 * page tables (Grace-Blackwell); elsewhere GBFFT_UNSUPPORTED_SIZE. */
int gbfft_fourfs(double* data, const size_t* nn, size_t nn_len, size_t ndim, int isign,
                 double* work, const gbfft_opts* opts);

/* rlft3: src/Real_FT3.rs:8 / rlft3_optimized :145
 * `(data: &mut [f64], speq: &mut [f64], nn1, nn2, nn3, isign)`.
 * data nn1*nn2*nn3 reals, speq nn1*2*nn2 doubles.  Inverse returns
 * (nn1 nn2 nn3 / 2) x. */
int gbfft_rlft3(double* data, double* speq, size_t nn1, size_t nn2, size_t nn3, int isign,
                const gbfft_opts* opts);

/* Sine and cosine transforms --------------------------------------------- */
/* sinft (README.md:72, Numerical Recipes contract): y[0..n), y[0] taken as 0. */
int gbfft_sinft(double* y, size_t n, const gbfft_opts* opts);
/* cosft1: src/Cos_FT.rs:7 `cosft1(y: &mut [f64], n)`; y[0..n] (n+1 values). */
int gbfft_cosft1(double* y, size_t n, const gbfft_opts* opts);
/* cosft2: src/Cos_FT2.rs:7 `cosft2(y: &mut [f64], n, isign)`; y[0..n). */
int gbfft_cosft2(double* y, size_t n, int isign, const gbfft_opts* opts);

/* Spectral routines ------------------------------------------------------ */
/* convlv: src/Convolve.rs:8
 * `convlv(data: &[f64], respns: &[f64], isign: i32) -> Result<Array1<f64>, ConvlvError>`.
 * data n reals, respns m <= n taps in wrap-around order, ans n reals.
 * Errors: GBFFT_EMPTY_INPUT, GBFFT_RESPONSE_TOO_LONG, GBFFT_INVALID_ISIGN
 * (checked in that order, Convolve.rs:13-21); n must be a power of two. */
int gbfft_convlv(const double* data, size_t n, const double* respns, size_t m, int isign,
                 double* ans, const gbfft_opts* opts);

/* correl: src/Correlation.rs:8
 * `correl(data1: &[f64], data2: &[f64]) -> Result<Array1<f64>, CorrelError>`.
 * n <= 32 uses the reference's direct linear sum; larger n must be a power of
 * two and gives the circular correlation. */
int gbfft_correl(const double* data1, size_t n1, const double* data2, size_t n2, double* ans,
                 const gbfft_opts* opts);

/* convlv_batch: src/Convolve.rs:241
 * `convlv_batch(data_batch: &[&[f64]], respns: &[f64], isign: i32)
 *   -> Result<Vec<Array1<f64>>, ConvlvError>` (also ConvlvProcessor::process_batch,
 * Convolve.rs:333).  `count` arrays data[i] of n[i] reals share one response of
 * m taps; ans[i] receives n[i] reals.  convlv's checks run item by item in
 * index order and the first failure is returned before any work.  Items of
 * equal length are transformed together and share one response spectrum. */
int gbfft_convlv_batch(const double* const* data, const size_t* n, size_t count,
                       const double* respns, size_t m, int isign, double* const* ans,
                       const gbfft_opts* opts);

/* correl_batch: src/Correlation.rs:273
 * `correl_batch(data_pairs: &[(&[f64], &[f64])]) -> Result<Vec<Array1<f64>>, CorrelError>`.
 * Pair i is (data1[i], n1[i]), (data2[i], n2[i]); ans[i] receives n1[i]
 * values.  correl's checks run item by item in index order. */
int gbfft_correl_batch(const double* const* data1, const size_t* n1, const double* const* data2,
                       const size_t* n2, size_t count, double* const* ans,
                       const gbfft_opts* opts);

/* correl_normalized: src/Correlation.rs:189 (fast = 0: two-pass statistics) and
 * correl_normalized_fast: :226 (fast = 1: one-pass sums; n <= 32 direct).
 * Inputs are standardised with their mean and population standard deviation,
 * then correlated as correl does.  Errors: GBFFT_EMPTY_INPUT,
 * GBFFT_LENGTH_MISMATCH, GBFFT_ZERO_STD_DEV. */
int gbfft_correl_normalized(const double* data1, size_t n1, const double* data2, size_t n2,
                            double* ans, int fast, const gbfft_opts* opts);

/* fourn (src/Fourn.rs:278 contract: row-major, nn[ndim-1] fastest) along the
 * axes whose bits are set in `axes` (bit i = axis i) only: the local steps of
 * an N-D transform split across ranks (the Python mirror's
 * numrs_gb300.dist.fourn_sharded).  Every nn[i] a power of two >= 1. */
int gbfft_fourn_axes(double* data, const size_t* nn, size_t ndim, unsigned long long axes,
                     int isign, const gbfft_opts* opts);

/* Four-step twiddle of a four1 of n points split across ranks (one GPU each;
 * the Python mirror's numrs_gb300.dist runs column transforms, this twiddle,
 * one all-to-all and row transforms).  data: `lines` lines of `len` complex
 * values in DEVICE memory (opts->device_ptrs set); element k of line c is
 * multiplied by exp(isign 2 pi i ((line0 + c) k mod n) / n).  n and len are
 * powers of two, len <= n <= 2^28.  No crate counterpart: the crate's four1
 * (src/FFT_1.rs:5-107) runs on one host. */
int gbfft_twiddle_lines(double* data, size_t lines, size_t len, size_t line0, size_t n, int isign,
                        const gbfft_opts* opts);

/* magnitude_spectrum / power_spectrum: src/FFT_1.rs:206,218.  c holds nn
 * interleaved complex values; out[nn].  The crate maps chunks(2) of its slice,
 * so for an odd-length slice it appends one 0.0 for the trailing half chunk:
 * the binding passes nn = len / 2 and appends that entry. */
int gbfft_magnitude_spectrum(const double* c, size_t nn, double* out, const gbfft_opts* opts);
int gbfft_power_spectrum(const double* c, size_t nn, double* out, const gbfft_opts* opts);

#ifdef __cplusplus
}
#endif

#endif /* GBFFT_H */
