// spectral.cu -- the real-data and spectral kernels around the complex passes:
// twiddle tables, the realft twist, the fused convlv/correl spectral step,
// the response expansion, the small-n direct correlation, twofft, rlft3 and
// the sine/cosine transform pre/post passes.
//
// Index conventions are 0-based restatements of the Numerical Recipes
// routines the reference crate follows (file:line at each kernel).
#include "arith.cuh"
#include "fft_core.cuh"
#include "gbfft_internal.h"

namespace gbfft {

// ---------------------------------------------------------------------------
// Twiddle tables: exp(+2 pi i e / S) from sincospi in double, stored in the
// form's twiddle element.
// ---------------------------------------------------------------------------
template <class F>
__device__ __forceinline__ void put_tw(typename F::TW* t, size_t i, double c, double s) {
  if constexpr (F::kind == 0) {
    t[i] = d2{c, s};
  } else if constexpr (F::kind == 1) {
    t[i] = f2{(float)c, (float)s};
  } else {
    float ch = (float)c, sh = (float)s;
    t[i] = f4{ch, (float)(c - (double)ch), sh, (float)(s - (double)sh)};
  }
}

template <class F>
__global__ void k_twiddles(typename F::TW* dense, typename F::TW* partial, int dense_log) {
  const size_t nd = dense_entries(dense_log);
  const size_t total = nd + partial_entries(dense_log);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    double c, s;
    if (i < nd) {
      // entry S + e of level S: S = highest power of two <= i
      if (i < 2) {
        c = 1.0; s = 0.0;
      } else {
        int logS = 63 - __clzll((long long)i);
        long long S = 1ll << logS;
        long long e = (long long)i - S;
        sincospi(2.0 * (double)e / (double)S, &s, &c);
      }
      put_tw<F>(dense, i, c, s);
    } else {
      size_t j = i - nd;
      int lvl = (int)(j >> kPartialLog) + dense_log + 1;
      long long e = (long long)(j & (kPartial - 1));
      sincospi(2.0 * (double)e / (double)(1ll << lvl), &s, &c);
      put_tw<F>(partial, j, c, s);
    }
  }
}

// One dense level: entry e = exp(+2 pi i e / 2^logS), e < 2^logS.
template <class F>
__global__ void k_twiddle_level(typename F::TW* level, int logS) {
  const size_t n = (size_t)1 << logS;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n;
       e += (size_t)gridDim.x * blockDim.x) {
    double c, s;
    if (e == 0) {
      c = 1.0; s = 0.0;
    } else {
      sincospi(2.0 * (double)e / (double)n, &s, &c);
    }
    put_tw<F>(level, e, c, s);
  }
}

cudaError_t launch_twiddle_level(Form f, void* level, int logS, cudaStream_t st) {
  dim3 g(152 * 16), b(256);
  if (f == FORM_F64) k_twiddle_level<F64><<<g, b, 0, st>>>((d2*)level, logS);
  else if (f == FORM_DF64) k_twiddle_level<DF64><<<g, b, 0, st>>>((f4*)level, logS);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_twiddles(Form f, void* dense, void* partial, int dense_log, cudaStream_t st) {
  dim3 g(1024), b(256);
  if (f == FORM_F64) k_twiddles<F64><<<g, b, 0, st>>>((d2*)dense, (d2*)partial, dense_log);
  else if (f == FORM_F32) k_twiddles<F32><<<g, b, 0, st>>>((f2*)dense, (f2*)partial, dense_log);
  else k_twiddles<DF64><<<g, b, 0, st>>>((f4*)dense, (f4*)partial, dense_log);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// realft twist (src/Real_FT.rs:24-213 restated 0-based).  For the pair of
// complex slots k and m = n/2 - k of the n/2-point spectrum Z:
//   h1 = (Z_k + conj Z_m)/2,  h2 = -isign * i (Z_k - conj Z_m)/2,
//   t = w^k h2 with w = exp(isign 2 pi i / n),
//   Z_k <- h1 + t,  Z_m <- conj(h1 - t).
// Slot 0 packs DC and Nyquist; slot n/4 is left unchanged (the reference
// loop stops at n/4 - 1 as well).
// ---------------------------------------------------------------------------
template <class F, int IS>
__device__ __forceinline__ void twist_pair(typename F::C& zk, typename F::C& zm,
                                           typename F::C w) {
  using C = typename F::C;
  C czm = F::conj(zm);
  C h1 = F::scale(F::add(zk, czm), 0.5);
  C h2 = F::scale(F::mul_j(F::sub(zk, czm), -IS), 0.5);
  C t = F::mul(h2, w);
  zk = F::add(h1, t);
  zm = F::conj(F::sub(h1, t));
}

// The same twist without its two factors of 1/2: returns 2 Z_k and 2 Z_m.
// The fused spectral kernel folds those factors into its one product scale.
template <class F, int IS>
__device__ __forceinline__ void twist2_pair(typename F::C& zk, typename F::C& zm,
                                            typename F::C w) {
  using C = typename F::C;
  C czm = F::conj(zm);
  C h1 = F::add(zk, czm);
  C h2 = F::mul_j(F::sub(zk, czm), -IS);
  C t = F::mul(h2, w);
  zk = F::add(h1, t);
  zm = F::conj(F::sub(h1, t));
}

template <class F>
__device__ __forceinline__ typename F::C ldc(const double* p, long long k) {
  d2 v = reinterpret_cast<const d2*>(p)[k];
  return F::from_d(v.x, v.y);
}
template <class F>
__device__ __forceinline__ void stc(double* p, long long k, typename F::C a) {
  double x, y;
  F::to_d(a, x, y);
  reinterpret_cast<d2*>(p)[k] = d2{x, y};
}

template <class F, int IS>
__global__ void k_realft_twist(double* data, long long n, long long batch, long long dist,
                               Twiddles tw) {
  const long long nq = n / 4;  // pairs k = 1..nq-1, plus slot 0
  const long long per = nq > 0 ? nq : 1;
  const int logn = 63 - __clzll(n);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < per * batch;
       g += (long long)gridDim.x * blockDim.x) {
    const long long bidx = g / per;
    const long long k = g - bidx * per;
    double* d = data + bidx * dist;
    if (k == 0) {
      if (IS > 0) {
        double h = d[0], v = d[1];
        d[0] = h + v;
        d[1] = h - v;
      } else {
        double h = d[0], v = d[1];
        d[0] = 0.5 * (h + v);
        d[1] = 0.5 * (h - v);
      }
      continue;
    }
    const long long m = n / 2 - k;
    typename F::C zk = ldc<F>(d, k), zm = ldc<F>(d, m);
    typename F::C w = twiddle<F>(tw, logn, k, IS);
    twist_pair<F, IS>(zk, zm, w);
    stc<F>(d, k, zk);
    stc<F>(d, m, zm);
  }
}

cudaError_t launch_realft_twist(Form f, int isign, double* data, long long n, long long batch,
                                long long dist, Twiddles tw, cudaStream_t st) {
  long long work = (n / 4 > 0 ? n / 4 : 1) * batch;
  int blocks = (int)((work + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
#define TW_LAUNCH(FT)                                                                    \
  (isign > 0 ? (k_realft_twist<FT, 1><<<blocks, 256, 0, st>>>(data, n, batch, dist, tw)) \
             : (k_realft_twist<FT, -1><<<blocks, 256, 0, st>>>(data, n, batch, dist, tw)))
  if (f == FORM_F64) TW_LAUNCH(F64);
  else if (f == FORM_F32 || f == FORM_TC32) TW_LAUNCH(F32);
  else TW_LAUNCH(DF64);
#undef TW_LAUNCH
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Fused convlv / correl spectral step (src/Convolve.rs:90-138,
// src/Correlation.rs:68-110; products at Convolve.rs:112-128 and
// Correlation.rs:90-96).  a and b hold the raw n/2-point complex FFTs of the
// two real inputs (forward, isign=+1).  Per pair (k, n/2-k): forward twist of
// both, product scaled by 1/(n/2), inverse twist -- the packed input of the
// inverse n/2-point FFT, written to out (which may alias a).
// ---------------------------------------------------------------------------
// x, y are `pre` times the true spectra (pre = 1 or 2; exact powers of two
// keep every comparison and quotient identical).
template <class F, int KIND>
__device__ __forceinline__ typename F::C spec_prod(typename F::C x, typename F::C y, double inv_no2,
                                                   double pre = 1.0) {
  using C = typename F::C;
  if constexpr (KIND == 0) {
    return F::scale(F::mul(x, y), inv_no2);
  } else if constexpr (KIND == 2) {
    return F::scale(F::mul(x, F::conj(y)), inv_no2);
  } else {
    // deconvolution in double: zero where |y|^2 < 1e-12 (src/Convolve.rs:118-122)
    double xr, xi, yr, yi;
    F::to_d(x, xr, xi);
    F::to_d(y, yr, yi);
    double mag2 = yr * yr + yi * yi;
    double o_r = 0.0, o_i = 0.0;
    if (!(mag2 < 1e-12 * pre * pre)) {
      o_r = (xr * yr + xi * yi) / mag2 * inv_no2;
      o_i = (xi * yr - xr * yi) / mag2 * inv_no2;
    }
    return F::from_d(o_r, o_i);
  }
}

template <class F, int KIND>
__device__ __forceinline__ double spec_prod_real(double x, double y, double inv_no2) {
  if constexpr (KIND == 1) {
    double mag2 = y * y;
    return (mag2 < 1e-12) ? 0.0 : (x * y) / mag2 * inv_no2;
  } else {
    return x * y * inv_no2;
  }
}

// One line per blockIdx.y: lines of a, b and out are sa, sb, so doubles apart
// (sb = 0 shares one response spectrum among all lines).
template <class F, int KIND>
__global__ void k_spectral(const double* a, const double* b, double* out, long long n,
                           Twiddles tw, long long sa, long long sb, long long so) {
  using C = typename F::C;
  a += (long long)blockIdx.y * sa;
  b += (long long)blockIdx.y * sb;
  out += (long long)blockIdx.y * so;
  const long long nq = n / 4;
  const long long per = nq > 0 ? nq : 1;
  const double inv_no2 = 2.0 / (double)n;
  const int logn = 63 - __clzll(n);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= per;
       k += (long long)gridDim.x * blockDim.x) {
    if (k == 0) {
      // DC in slot 0 real part, Nyquist in slot 0 imaginary part after the twist
      double a0 = a[0], a1 = a[1], b0 = b[0], b1 = b[1];
      double ad = a0 + a1, an = a0 - a1, bd = b0 + b1, bn = b0 - b1;
      if (n == 2) {  // the n/2 = 1 point "FFT" holds (x0 + x1) + i 0
        ad = a0 + a1; an = a0 - a1;
      }
      double pd = spec_prod_real<F, KIND>(ad, bd, inv_no2);
      double pn = spec_prod_real<F, KIND>(an, bn, inv_no2);
      out[0] = 0.5 * (pd + pn);
      out[1] = 0.5 * (pd - pn);
      continue;
    }
    if (k > nq) continue;
    if (k == nq) {
      // middle slot n/4: both twists are the identity
      C x = ldc<F>(a, k), y = ldc<F>(b, k);
      stc<F>(out, k, spec_prod<F, KIND>(x, y, inv_no2));
      continue;
    }
    const long long m = n / 2 - k;
    C ak = ldc<F>(a, k), am = ldc<F>(a, m), bk = ldc<F>(b, k), bm = ldc<F>(b, m);
    C w = twiddle<F>(tw, logn, k, 1);
    // unscaled twists give 2A and 2B; the unscaled inverse twist doubles again
    twist2_pair<F, 1>(ak, am, w);
    twist2_pair<F, 1>(bk, bm, w);
    const double sc = (KIND == 1) ? 0.5 * inv_no2 : 0.125 * inv_no2;
    C pk = spec_prod<F, KIND>(ak, bk, sc, 2.0);
    C pm = spec_prod<F, KIND>(am, bm, sc, 2.0);
    twist2_pair<F, -1>(pk, pm, F::conj(w));
    stc<F>(out, k, pk);
    stc<F>(out, m, pm);
  }
}

cudaError_t launch_spectral_lines(Form f, int kind, const double* a, long long sa,
                                  const double* b, long long sb, double* out, long long so,
                                  long long lines, long long n, Twiddles tw, cudaStream_t st) {
  long long work = n / 4 + 1;
  int blocks = (int)((work + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  for (long long l0 = 0; l0 < lines; l0 += 65535) {
    const unsigned ny = (unsigned)(lines - l0 < 65535 ? lines - l0 : 65535);
    const dim3 grid((unsigned)blocks, ny);
    const double* al = a + l0 * sa;
    const double* bl = b + l0 * sb;
    double* ol = out + l0 * so;
#define SP_LAUNCH(FT)                                                                           \
  switch (kind) {                                                                               \
    case 0: k_spectral<FT, 0><<<grid, 256, 0, st>>>(al, bl, ol, n, tw, sa, sb, so); break;      \
    case 1: k_spectral<FT, 1><<<grid, 256, 0, st>>>(al, bl, ol, n, tw, sa, sb, so); break;      \
    default: k_spectral<FT, 2><<<grid, 256, 0, st>>>(al, bl, ol, n, tw, sa, sb, so); break;     \
  }
    if (f == FORM_F64) { SP_LAUNCH(F64) }
    else if (f == FORM_F32 || f == FORM_TC32) { SP_LAUNCH(F32) }
    else { SP_LAUNCH(DF64) }
#undef SP_LAUNCH
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_spectral_product(Form f, int kind, const double* a, const double* b,
                                    double* out, long long n, Twiddles tw, cudaStream_t st) {
  return launch_spectral_lines(f, kind, a, 0, b, 0, out, 0, 1, n, tw, st);
}

// ---------------------------------------------------------------------------
// Response expansion (Numerical Recipes convlv contract): r[0..m) = respns,
// r[n-k] = respns[m-k] for k = 1..(m-1)/2, zeros in [(m+1)/2, n-(m-1)/2).
// ---------------------------------------------------------------------------
__global__ void k_expand(const double* respns, long long m, double* dst, long long n,
                         const double* data, double* dst_data) {
  const long long half = (m - 1) / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double v;
    if (half > 0 && i >= n - half) v = respns[m - (n - i)];
    else if (i < (m + 1) / 2) v = respns[i];
    else v = 0.0;
    dst[i] = v;
    if (dst_data) dst_data[i] = data[i];
  }
}

cudaError_t launch_expand_response(const double* respns, long long m, double* dst, long long n,
                                   const double* data, double* dst_data, cudaStream_t st) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_expand<<<blocks, 256, 0, st>>>(respns, m, dst, n, data, dst_data);
  return cudaGetLastError();
}

// Direct linear correlation, the reference's n <= 32 branch
// (src/Correlation.rs:37-50): out[lag] = sum_{i < n-lag} a[i+lag] b[i].
__global__ void k_correl_direct(const double* a, const double* b, double* out, long long n) {
  long long lag = threadIdx.x;
  if (lag >= n) return;
  double sum = 0.0;
  for (long long i = 0; i < n - lag; ++i) sum += a[i + lag] * b[i];
  out[lag] = sum;
}

cudaError_t launch_correl_direct(const double* a, const double* b, double* out, long long n,
                                 cudaStream_t st) {
  k_correl_direct<<<1, 32, 0, st>>>(a, b, out, n);
  return cudaGetLastError();
}

// Centered direct linear correlation for correl_normalized_fast's n <= 32
// branch (src/Correlation.rs:251-263): out[lag] = norm * sum (a-ma)(b-mb).
__global__ void k_correl_direct_centered(const double* a, const double* b, double* out,
                                         long long n, double ma, double mb, double norm) {
  long long lag = threadIdx.x;
  if (lag >= n) return;
  double sum = 0.0;
  for (long long i = 0; i < n - lag; ++i) sum += (a[i + lag] - ma) * (b[i] - mb);
  out[lag] = sum * norm;
}

cudaError_t launch_correl_direct_centered(const double* a, const double* b, double* out,
                                          long long n, double ma, double mb, double norm,
                                          cudaStream_t st) {
  k_correl_direct_centered<<<1, 32, 0, st>>>(a, b, out, n, ma, mb, norm);
  return cudaGetLastError();
}

// Per-block partial sums of (x - shift)^p, p = 1 or 2, for the normalised
// correlation's statistics; 256 blocks, summed in a fixed order afterwards.
__global__ void k_block_moment(const double* x, long long n, double shift, int p,
                               double* partial) {
  __shared__ double red[256];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double d = x[i] - shift;
    acc += (p == 2) ? d * d : d;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s2 = blockDim.x / 2; s2 > 0; s2 >>= 1) {
    if ((int)threadIdx.x < s2) red[threadIdx.x] += red[threadIdx.x + s2];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void k_sum256(const double* partial, double* out) {
  __shared__ double red[256];
  red[threadIdx.x] = partial[threadIdx.x];
  __syncthreads();
  for (int s2 = 128; s2 > 0; s2 >>= 1) {
    if ((int)threadIdx.x < s2) red[threadIdx.x] += red[threadIdx.x + s2];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// out = sum over the array of (x - shift)^p; partial holds 256 doubles.
cudaError_t launch_moment(const double* x, long long n, double shift, int p, double* partial,
                          double* out, cudaStream_t st) {
  k_block_moment<<<256, 256, 0, st>>>(x, n, shift, p, partial);
  k_sum256<<<1, 256, 0, st>>>(partial, out);
  return cudaGetLastError();
}

__global__ void k_standardize(const double* x, long long n, double mean, double stdv,
                              double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (x[i] - mean) / stdv;
}

cudaError_t launch_standardize(const double* x, long long n, double mean, double stdv,
                               double* out, cudaStream_t st) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_standardize<<<blocks, 256, 0, st>>>(x, n, mean, stdv, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// twofft (src/FFT_2.rs:3-132, Numerical Recipes contract): pack data1 + i
// data2, and after the n-point FFT split the spectrum into the two real
// inputs' spectra; the mirror of slot k is n-k.
// ---------------------------------------------------------------------------
__global__ void k_twofft_pack(const double* d1, const double* d2v, double* fft1, long long n) {
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    reinterpret_cast<d2*>(fft1)[j] = d2{d1[j], d2v[j]};
  }
}

__global__ void k_twofft_split(double* fft1, double* fft2, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= n / 2;
       k += (long long)gridDim.x * blockDim.x) {
    if (k == 0) {
      fft2[0] = fft1[1];
      fft1[1] = 0.0;
      fft2[1] = 0.0;
      continue;
    }
    const long long j = 2 * k, jr = 2 * n - 2 * k;
    double rep = 0.5 * (fft1[j] + fft1[jr]);
    double rem = 0.5 * (fft1[j] - fft1[jr]);
    double aip = 0.5 * (fft1[j + 1] + fft1[jr + 1]);
    double aim = 0.5 * (fft1[j + 1] - fft1[jr + 1]);
    fft1[j] = rep;
    fft1[j + 1] = aim;
    fft1[jr] = rep;
    fft1[jr + 1] = -aim;
    fft2[j] = aip;
    fft2[j + 1] = -rem;
    fft2[jr] = aip;
    fft2[jr + 1] = rem;
  }
}

cudaError_t launch_twofft_pack(const double* d1, const double* d2v, double* fft1, long long n,
                               cudaStream_t st) {
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_twofft_pack<<<blocks, 256, 0, st>>>(d1, d2v, fft1, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// twofft-packed convlv / correl (the fast path of src/FFT_2.rs:3-17 applied to
// the two forward transforms of src/Convolve.rs:66-77 and
// src/Correlation.rs:53-55): the two real inputs travel as the real and
// imaginary parts of one n-point complex FFT.
// ---------------------------------------------------------------------------
// The two inputs' sums of squares (b: its nb stored values), one block, a
// fixed reduction order: sums[0] = |a|^2, sums[1] = |b|^2.
__global__ void k_sumsq_pair(const double* a, long long na, const double* b, long long nb,
                             double* sums) {
  __shared__ double red[2][256];
  double sa = 0.0, sb = 0.0;
  for (long long i = threadIdx.x; i < na; i += blockDim.x) sa += a[i] * a[i];
  for (long long i = threadIdx.x; i < nb; i += blockDim.x) sb += b[i] * b[i];
  red[0][threadIdx.x] = sa;
  red[1][threadIdx.x] = sb;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    sums[0] = red[0][0];
    sums[1] = red[1][0];
  }
}

// Power of two s near |a| / |b|: the packed imaginary part s b then has the
// real part's magnitude, so that the rounding of the shared transform (relative
// to the larger input) does not swamp the smaller input's spectrum.  Exact in
// every form; 1 when either input is zero.
__device__ __forceinline__ double pack_scale(const double* sums) {
  if (!sums || !(sums[0] > 0.0) || !(sums[1] > 0.0)) return 1.0;
  int e = (int)rint(0.5 * log2(sums[0] / sums[1]));
  e = e > 600 ? 600 : (e < -600 ? -600 : e);
  return ldexp(1.0, e);
}

// z_j = a_j + i s b_j.  With m > 0, b is an m-tap response in wrap-around
// order (Numerical Recipes convlv contract) expanded on the fly to n values.
__global__ void k_pack_pair(const double* a, const double* b, long long m, double* z, long long n,
                            const double* sums) {
  const long long half = (m - 1) / 2;
  const double sc = pack_scale(sums);
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n;
       j += (long long)gridDim.x * blockDim.x) {
    double v;
    if (m == 0) v = b[j];
    else if (half > 0 && j >= n - half) v = b[m - (n - j)];
    else if (j < (m + 1) / 2) v = b[j];
    else v = 0.0;
    reinterpret_cast<d2*>(z)[j] = d2{a[j], sc * v};
  }
}

cudaError_t launch_pack_pair(const double* a, const double* b, long long m, double* z, long long n,
                             double* sums, cudaStream_t st) {
  if (sums) k_sumsq_pair<<<1, 256, 0, st>>>(a, n, b, m > 0 ? m : n, sums);
  int blocks = (int)((n + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_pack_pair<<<blocks, 256, 0, st>>>(a, b, m, z, n, sums);
  return cudaGetLastError();
}

// Z is the n-point FFT (isign = +1) of a + i b.  The spectra of a and b are
// A_k = (Z_k + conj Z_{n-k})/2 and B_k = -i (Z_k - conj Z_{n-k})/2.  For each
// pair (k, n/2 - k) of the packed half spectrum: both products (scaled by
// 2/n as k_spectral's), then the inverse realft twist -- the input of the
// inverse n/2-point FFT, written over the first n/2 slots of Z.  Every slot
// of Z is read by one thread only, the one that writes it, so the step runs
// in place.
template <class F, int KIND>
__global__ void k_spectral_two(double* z, long long n, Twiddles tw, const double* sums) {
  using C = typename F::C;
  const long long nh = n / 2, nq = n / 4;
  // B was packed as s b: the products take 1/s (deconvolution is packed
  // unscaled, sums = nullptr, so that its |B|^2 threshold keeps its meaning)
  const double inv_no2 = (2.0 / (double)n) / pack_scale(sums);
  const int logn = 63 - __clzll(n);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k <= nq;
       k += (long long)gridDim.x * blockDim.x) {
    if (k == 0) {
      // DC and Nyquist bins of A and B are real: Re/Im of Z_0 and Z_{n/2}
      const double ad = z[0], bd = z[1];
      const double an = (n > 1) ? z[2 * nh] : 0.0, bn = (n > 1) ? z[2 * nh + 1] : 0.0;
      const double pd = spec_prod_real<F, KIND>(ad, bd, inv_no2);
      const double pn = spec_prod_real<F, KIND>(an, bn, inv_no2);
      z[0] = 0.5 * (pd + pn);
      z[1] = 0.5 * (pd - pn);
      continue;
    }
    if (k == nq) {
      // middle slot n/4: the twists are the identity
      const C zk = ldc<F>(z, k), zr = F::conj(ldc<F>(z, n - k));
      const C a2 = F::add(zk, zr), b2 = F::mul_j(F::sub(zk, zr), -1);  // 2A, 2B
      stc<F>(z, k, spec_prod<F, KIND>(a2, b2, (KIND == 1) ? inv_no2 : 0.25 * inv_no2, 2.0));
      continue;
    }
    const long long m = nh - k;
    const C zk = ldc<F>(z, k), zkr = F::conj(ldc<F>(z, n - k));
    const C zm = ldc<F>(z, m), zmr = F::conj(ldc<F>(z, n - m));
    const C ak = F::add(zk, zkr), bk = F::mul_j(F::sub(zk, zkr), -1);  // 2A_k, 2B_k
    const C am = F::add(zm, zmr), bm = F::mul_j(F::sub(zm, zmr), -1);
    const double sc = (KIND == 1) ? 0.5 * inv_no2 : 0.125 * inv_no2;
    C pk = spec_prod<F, KIND>(ak, bk, sc, 2.0);
    C pm = spec_prod<F, KIND>(am, bm, sc, 2.0);
    twist2_pair<F, -1>(pk, pm, F::conj(twiddle<F>(tw, logn, k, 1)));
    stc<F>(z, k, pk);
    stc<F>(z, m, pm);
  }
}

cudaError_t launch_spectral_two(Form f, int kind, double* z, long long n, Twiddles tw,
                                const double* sums, cudaStream_t st) {
  long long work = n / 4 + 1;
  int blocks = (int)((work + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
#define SP2_LAUNCH(FT)                                                              \
  switch (kind) {                                                                   \
    case 0: k_spectral_two<FT, 0><<<blocks, 256, 0, st>>>(z, n, tw, sums); break;   \
    case 1: k_spectral_two<FT, 1><<<blocks, 256, 0, st>>>(z, n, tw, sums); break;   \
    default: k_spectral_two<FT, 2><<<blocks, 256, 0, st>>>(z, n, tw, sums); break;  \
  }
  if (f == FORM_F64) { SP2_LAUNCH(F64) }
  else if (f == FORM_F32 || f == FORM_TC32) { SP2_LAUNCH(F32) }
  else { SP2_LAUNCH(DF64) }
#undef SP2_LAUNCH
  return cudaGetLastError();
}

cudaError_t launch_twofft_split(double* fft1, double* fft2, long long n, cudaStream_t st) {
  long long work = n / 2 + 1;
  int blocks = (int)((work + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_twofft_split<<<blocks, 256, 0, st>>>(fft1, fft2, n);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// rlft3 (src/Real_FT3.rs:8-141, Numerical Recipes contract).  data is
// nn1 x nn2 x nn3 reals = nn1 x nn2 x nh complex (nh = nn3/2); speq is
// nn1 x nn2 complex.  After the forward 3-D FFT, speq takes the k3 = 0 plane.
// ---------------------------------------------------------------------------
__global__ void k_rlft3_speq(const double* data, double* speq, long long nn1, long long nn2,
                             long long nn3) {
  const long long total = nn1 * nn2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    reinterpret_cast<d2*>(speq)[g] = reinterpret_cast<const d2*>(data)[g * (nn3 / 2)];
  }
}

cudaError_t launch_rlft3_speq(const double* data, double* speq, long long nn1, long long nn2,
                              long long nn3, cudaStream_t st) {
  long long total = nn1 * nn2;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_rlft3_speq<<<blocks, 256, 0, st>>>(data, speq, nn1, nn2, nn3);
  return cudaGetLastError();
}

// The twist pairs element (i1, i2, i3) with (j1, j2, nh - i3), j = mirrored
// indices; i3 = 0 pairs with the speq entry (j1, j2).  Each unordered pair is
// handled by exactly one thread: i3 in 1..nh/2-1 own their pair outright; at
// i3 = 0 and i3 = nh/2 the pair partner lies in the same plane, so the thread
// with the lexicographically smaller (i1, i2) owns it.
// Forward (isign=+1) and inverse share the formulas of the reference loop
// (src/Real_FT3.rs:60-127) with c2 = -isign/2 and w = exp(isign 2 pi i i3/nn3).
template <class F, int IS>
__global__ void k_rlft3_twist(double* data, double* speq, long long nn1, long long nn2,
                              long long nn3, Twiddles tw) {
  using C = typename F::C;
  const long long nh = nn3 / 2;
  // planes i3 = 0 .. nh/2-1; the middle plane i3 = nh/2 maps onto itself and
  // the twist there is the identity (w = isign*i makes h1 + w h2 = Z_k).
  const long long planes = nh >= 2 ? nh / 2 : 1;
  const long long total = nn1 * nn2 * planes;
  const int logn3 = 63 - __clzll(nn3);
  d2* sp = reinterpret_cast<d2*>(speq);
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
       g += (long long)gridDim.x * blockDim.x) {
    const long long i3 = g % planes;
    const long long i12 = g / planes;
    const long long i2 = i12 % nn2, i1 = i12 / nn2;
    const long long j1 = i1 ? nn1 - i1 : 0, j2 = i2 ? nn2 - i2 : 0;
    const long long self = i1 * nn2 + i2, mate = j1 * nn2 + j2;
    if (i3 == 0) {
      // data(i1,i2,0) pairs with speq(j1,j2) and data(j1,j2,0) with
      // speq(i1,i2); the thread with the smaller line index does both.
      if (mate < self) continue;
      const C one = F::from_d(1.0, 0.0);
      C zk = ldc<F>(data, self * nh);
      C zs = F::from_d(sp[mate].x, sp[mate].y);
      C zk2 = zk, zs2 = zs;
      if (mate != self) {
        zk2 = ldc<F>(data, mate * nh);
        zs2 = F::from_d(sp[self].x, sp[self].y);
      }
      twist_pair<F, IS>(zk, zs, one);
      double x, y;
      if (mate != self) {
        twist_pair<F, IS>(zk2, zs2, one);
        stc<F>(data, mate * nh, zk2);
        F::to_d(zs2, x, y);
        sp[self] = d2{x, y};
      }
      stc<F>(data, self * nh, zk);
      F::to_d(zs, x, y);
      sp[mate] = d2{x, y};
      continue;
    }
    const long long i3m = nh - i3;
    C w = twiddle<F>(tw, logn3, i3, IS);
    C zk = ldc<F>(data, self * nh + i3);
    C zm = ldc<F>(data, mate * nh + i3m);
    twist_pair<F, IS>(zk, zm, w);
    stc<F>(data, self * nh + i3, zk);
    stc<F>(data, mate * nh + i3m, zm);
  }
}

cudaError_t launch_rlft3_twist(Form f, int isign, double* data, double* speq, long long nn1,
                               long long nn2, long long nn3, Twiddles tw, cudaStream_t st) {
  long long total = nn1 * nn2 * (nn3 / 4 > 0 ? nn3 / 4 : 1);
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
#define R3_LAUNCH(FT)                                                                       \
  (isign > 0 ? (k_rlft3_twist<FT, 1><<<blocks, 256, 0, st>>>(data, speq, nn1, nn2, nn3, tw)) \
             : (k_rlft3_twist<FT, -1><<<blocks, 256, 0, st>>>(data, speq, nn1, nn2, nn3, tw)))
  if (f == FORM_F64) R3_LAUNCH(F64);
  else if (f == FORM_F32 || f == FORM_TC32) R3_LAUNCH(F32);
  else R3_LAUNCH(DF64);
#undef R3_LAUNCH
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Element-wise helpers.
// ---------------------------------------------------------------------------
__global__ void k_scale(double* d, long long count, double s) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    d[i] *= s;
}

// Writes two line pointers into device memory in stream order (a copy from
// pageable host memory would first wait for the stream to drain).
__global__ void k_set_lines(const void** dst, const void* a, const void* b) {
  dst[0] = a;
  dst[1] = b;
}

cudaError_t launch_set_lines(const void** dst, const void* a, const void* b, cudaStream_t st) {
  k_set_lines<<<1, 1, 0, st>>>(dst, a, b);
  return cudaGetLastError();
}

cudaError_t launch_scale(double* data, long long count, double s, cudaStream_t st) {
  int blocks = (int)((count + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_scale<<<blocks, 256, 0, st>>>(data, count, s);
  return cudaGetLastError();
}

// Four-step twiddle of a transform of n = 2^logn points sharded over ranks:
// element k of line c, data[c len + k], times w_n^((line0 + c) k) with
// w_n = exp(isign 2 pi i / n).  The exponent is reduced mod n in 64-bit
// integers and looked up in the FP64 twiddle tables.
__global__ void k_twiddle_lines(double* data, long long lines, int loglen, long long line0,
                                int logn, int isign, Twiddles tw) {
  const long long total = lines << loglen;
  const unsigned long long mask = (1ull << logn) - 1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long c = (unsigned long long)(i >> loglen);
    const unsigned long long k = (unsigned long long)(i & ((1ll << loglen) - 1));
    const unsigned long long e = ((unsigned long long)line0 + c) * k & mask;
    if (e == 0) continue;
    d2* q = reinterpret_cast<d2*>(data) + i;
    const d2 v = *q;
    const F64::C w = twiddle<F64>(tw, logn, (unsigned)e, isign);
    *q = d2{v.x * w.x - v.y * w.y, v.x * w.y + v.y * w.x};
  }
}

cudaError_t launch_twiddle_lines(double* data, long long lines, int loglen, long long line0,
                                 int logn, int isign, const Twiddles& tw, cudaStream_t st) {
  const long long total = lines << loglen;
  long long blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_twiddle_lines<<<(int)blocks, 256, 0, st>>>(data, lines, loglen, line0, logn, isign, tw);
  return cudaGetLastError();
}

// magnitude_spectrum / power_spectrum (src/FFT_1.rs:206-228)
__global__ void k_spectrum(int kind, const double* c, double* out, long long nn) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nn;
       i += (long long)gridDim.x * blockDim.x) {
    d2 v = reinterpret_cast<const d2*>(c)[i];
    double p = v.x * v.x + v.y * v.y;
    out[i] = kind == 0 ? sqrt(p) : p;
  }
}

cudaError_t launch_spectrum(int kind, const double* c, double* out, long long nn,
                            cudaStream_t st) {
  int blocks = (int)((nn + 255) / 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_spectrum<<<blocks, 256, 0, st>>>(kind, c, out, nn);
  return cudaGetLastError();
}

}  // namespace gbfft
