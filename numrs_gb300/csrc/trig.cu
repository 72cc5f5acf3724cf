// trig.cu -- sine and cosine transforms (sinft, cosft1, cosft2) as
// pre/post passes around realft, and the device-wide ordered scans their
// recurrences need.
//
//   sinft   Numerical Recipes contract (README.md:72 lists Sin_FT)
//   cosft1  src/Cos_FT.rs:7-68
//   cosft2  src/Cos_FT2.rs:7-173
//
// All routines run in FP64; twiddles come from the FP64 tables
// (w_S^e = exp(2 pi i e / S), so sin(pi j / n) = Im w_{2n}^j).
#include "arith.cuh"
#include "fft_core.cuh"
#include "gbfft_internal.h"

namespace gbfft {

namespace {

__device__ __forceinline__ d2 tw64(const Twiddles& tw, int logS, long long e) {
  F64::C w = twiddle<F64>(tw, logS, e, 1);
  return d2{w.x, w.y};
}

inline int blocks_for(long long work, int per_block, int cap = 152 * 16) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (int)b;
}

}  // namespace

// ---------------------------------------------------------------------------
// Pre-passes (pairs j, n-j are independent: one thread per pair).
// ---------------------------------------------------------------------------

// sinft: y1 = sin(pi j/n)(y_j + y_{n-j}), y2 = (y_j - y_{n-j})/2, j = 1..n/2.
__global__ void k_sinft_pre(double* y, long long n, Twiddles tw) {
  const int logS = 63 - __clzll(2 * n);
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j <= n / 2;
       j += (long long)gridDim.x * blockDim.x) {
    if (j == 0) {
      y[0] = 0.0;
      continue;
    }
    const double wi = tw64(tw, logS, j).y;
    const double a = y[j], b = y[n - j];
    const double y1 = wi * (a + b), y2 = 0.5 * (a - b);
    y[j] = y1 + y2;
    y[n - j] = y1 - y2;  // j = n/2 writes the same slot with the same value
  }
}

// cosft1: y1 = (y_j + y_{n-j})/2, y2 = y_j - y_{n-j}; y_j = y1 - sin y2,
// y_{n-j} = y1 + sin y2, and the running sum of cos(pi j/n) y2 (reduced per
// block into partial[blockIdx]).  Thread 0 also folds (y_0 - y_n)/2 into the
// sum and sets y_0 = (y_0 + y_n)/2.
__global__ void k_cosft1_pre(double* y, long long n, double* partial, Twiddles tw) {
  __shared__ double red[256];
  const int logS = 63 - __clzll(2 * n);
  double acc = 0.0;
  for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n / 2;
       j += (long long)gridDim.x * blockDim.x) {
    if (j == 0) {
      const double a = y[0], b = y[n];
      acc += 0.5 * (a - b);
      y[0] = 0.5 * (a + b);
      continue;
    }
    const d2 w = tw64(tw, logS, j);
    const double a = y[j], b = y[n - j];
    const double y1 = 0.5 * (a + b), y2 = a - b;
    y[j] = y1 - w.y * y2;
    y[n - j] = y1 + w.y * y2;
    acc += w.x * y2;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Sum of the per-block partials in a fixed order (one block).
__global__ void k_sum_partials(const double* partial, int count, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) acc += partial[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// cosft2 forward pre-pass: pairs (i, n-1-i), weight sin(pi (i + 1/2)/n).
__global__ void k_cosft2_pre(double* y, long long n, Twiddles tw) {
  const int logS = 63 - __clzll(4 * n);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n / 2;
       i += (long long)gridDim.x * blockDim.x) {
    const double s = tw64(tw, logS, 2 * i + 1).y;
    const double a = y[i], b = y[n - 1 - i];
    const double y1 = 0.5 * (a + b), y2 = s * (a - b);
    y[i] = y1 + y2;
    y[n - 1 - i] = y1 - y2;
  }
}

// cosft2 forward rotation of bins k = 1..n/2-1 by exp(+i pi k/n).
__global__ void k_cosft2_rot(double* y, long long n, Twiddles tw) {
  const int logS = 63 - __clzll(2 * n);
  for (long long k = 1 + blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n / 2;
       k += (long long)gridDim.x * blockDim.x) {
    const d2 w = tw64(tw, logS, k);
    const double a = y[2 * k], b = y[2 * k + 1];
    y[2 * k] = a * w.x - b * w.y;
    y[2 * k + 1] = b * w.x + a * w.y;
  }
}

// cosft2 inverse pre-pass, out of place: differences of the odd outputs,
// Nyquist slot, then rotation by exp(-i pi k/n) (src/Cos_FT2.rs:96-131 restated).
__global__ void k_cosft2_inv_pre(const double* y, double* w, long long n, Twiddles tw) {
  const int logS = 63 - __clzll(2 * n);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n / 2;
       k += (long long)gridDim.x * blockDim.x) {
    if (k == 0) {
      w[0] = y[0];
      w[1] = 2.0 * y[n - 1];
      continue;
    }
    const d2 t = tw64(tw, logS, k);
    const double re = y[2 * k];
    const double im = y[2 * k - 1] - y[2 * k + 1];
    w[2 * k] = re * t.x + im * t.y;
    w[2 * k + 1] = im * t.x - re * t.y;
  }
}

// cosft2 inverse post-pass, out of place: undo the pre-pass pairing.
__global__ void k_cosft2_inv_post(const double* w, double* y, long long n, Twiddles tw) {
  const int logS = 63 - __clzll(4 * n);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n / 2;
       i += (long long)gridDim.x * blockDim.x) {
    const double s = tw64(tw, logS, 2 * i + 1).y;
    const double a = w[i], b = w[n - 1 - i];
    const double y1 = a + b, y2 = (0.5 / s) * (a - b);
    y[i] = 0.5 * (y1 + y2);
    y[n - 1 - i] = 0.5 * (y1 - y2);
  }
}

// ---------------------------------------------------------------------------
// Ordered scans over M = n/2 slots (three phases: block scans, scan of block
// totals, add offsets).  kind selects the recurrence:
//   0 sinft   v_t = y[2t] (t=0: y[0]/2); y[2t+1] <- inclusive prefix,
//             y[2t] <- old y[2t+1] (t=0: 0)
//   1 cosft1  v_0 = sum0, v_t = y[2t+1]; y[2t+1] <- inclusive prefix;
//             y[n] <- old y[1] (done by phase 1)
//   2 cosft2  v_t = y[n-1-2t]; y[n-1-2t] <- y[1]/2 + exclusive prefix
// ---------------------------------------------------------------------------
constexpr int kScanT = 256;
constexpr int kScanPer = 8;
constexpr int kScanChunk = kScanT * kScanPer;

__device__ __forceinline__ double scan_load(int kind, const double* y, long long n, long long t,
                                            const double* sum0) {
  if (kind == 0) return t == 0 ? 0.5 * y[0] : y[2 * t];
  if (kind == 1) return t == 0 ? *sum0 : y[2 * t + 1];
  return y[n - 1 - 2 * t];
}

// Phase 1: per-chunk inclusive scan into work[t]; chunk totals into totals[b].
__global__ void k_scan_chunks(int kind, double* y, long long n, const double* sum0, double* work,
                              double* totals, double* half_y1) {
  __shared__ double sh[kScanT];
  const long long M = n / 2;
  const long long base = (long long)blockIdx.x * kScanChunk;
  const int tid = threadIdx.x;
  if (blockIdx.x == 0 && tid == 0) {
    if (kind == 1) y[n] = y[1];
    if (kind == 2) *half_y1 = 0.5 * y[1];
  }
  double v[kScanPer];
  double run = 0.0;
#pragma unroll
  for (int i = 0; i < kScanPer; ++i) {
    long long t = base + (long long)tid * kScanPer + i;
    double x = (t < M) ? scan_load(kind, y, n, t, sum0) : 0.0;
    run += x;
    v[i] = run;
  }
  sh[tid] = run;
  __syncthreads();
  // Hillis-Steele over the thread totals
  for (int off = 1; off < kScanT; off <<= 1) {
    double add = (tid >= off) ? sh[tid - off] : 0.0;
    __syncthreads();
    sh[tid] += add;
    __syncthreads();
  }
  const double before = (tid > 0) ? sh[tid - 1] : 0.0;
#pragma unroll
  for (int i = 0; i < kScanPer; ++i) {
    long long t = base + (long long)tid * kScanPer + i;
    if (t < M) work[t] = before + v[i];
  }
  if (tid == kScanT - 1) totals[blockIdx.x] = sh[kScanT - 1];
}

// Phase 2: exclusive scan of the chunk totals in place (one block).
__global__ void k_scan_totals(double* totals, long long count) {
  __shared__ double sh[1024];
  const int tid = threadIdx.x;
  const long long per = (count + 1023) / 1024;
  const long long b0 = tid * per;
  double s = 0.0;
  for (long long i = 0; i < per; ++i)
    if (b0 + i < count) s += totals[b0 + i];
  sh[tid] = s;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    double add = (tid >= off) ? sh[tid - off] : 0.0;
    __syncthreads();
    sh[tid] += add;
    __syncthreads();
  }
  double run = (tid > 0) ? sh[tid - 1] : 0.0;
  for (long long i = 0; i < per; ++i) {
    if (b0 + i < count) {
      double x = totals[b0 + i];
      totals[b0 + i] = run;
      run += x;
    }
  }
}

// Phase 3: add the chunk offset and write the recurrence outputs.
__global__ void k_scan_apply(int kind, double* y, long long n, const double* work,
                             const double* totals, const double* half_y1) {
  const long long M = n / 2;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < M;
       t += (long long)gridDim.x * blockDim.x) {
    const double incl = work[t] + totals[t / kScanChunk];
    if (kind == 0) {
      const double odd = (t == 0) ? 0.0 : y[2 * t + 1];
      y[2 * t] = odd;
      y[2 * t + 1] = incl;
    } else if (kind == 1) {
      y[2 * t + 1] = incl;
    } else {
      const long long i = n - 1 - 2 * t;
      const double excl = incl - y[i];
      y[i] = *half_y1 + excl;
    }
  }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_sinft_pre(double* y, long long n, Twiddles tw, cudaStream_t st) {
  k_sinft_pre<<<blocks_for(n / 2 + 1, 256), 256, 0, st>>>(y, n, tw);
  return cudaGetLastError();
}

// partial must hold at least 152*16 + 1 doubles; the sum lands in partial[152*16].
cudaError_t launch_cosft1_pre(double* y, long long n, double* partial, Twiddles tw,
                              cudaStream_t st) {
  int b = blocks_for(n / 2, 256);
  k_cosft1_pre<<<b, 256, 0, st>>>(y, n, partial, tw);
  k_sum_partials<<<1, 256, 0, st>>>(partial, b, partial + 152 * 16);
  return cudaGetLastError();
}

cudaError_t launch_cosft2_pre(int isign, double* y, long long n, Twiddles tw, cudaStream_t st) {
  (void)isign;
  k_cosft2_pre<<<blocks_for(n / 2, 256), 256, 0, st>>>(y, n, tw);
  return cudaGetLastError();
}

cudaError_t launch_cosft2_rot(int isign, double* y, long long n, Twiddles tw, cudaStream_t st) {
  (void)isign;
  k_cosft2_rot<<<blocks_for(n / 2, 256), 256, 0, st>>>(y, n, tw);
  return cudaGetLastError();
}

cudaError_t launch_cosft2_inv_pre(const double* y, double* w, long long n, Twiddles tw,
                                  cudaStream_t st) {
  k_cosft2_inv_pre<<<blocks_for(n / 2, 256), 256, 0, st>>>(y, w, n, tw);
  return cudaGetLastError();
}

cudaError_t launch_cosft2_inv_post(const double* w, double* y, long long n, Twiddles tw,
                                   cudaStream_t st) {
  k_cosft2_inv_post<<<blocks_for(n / 2, 256), 256, 0, st>>>(w, y, n, tw);
  return cudaGetLastError();
}

// work: n/2 + chunks + 2 doubles.  sum0 (cosft1) is read from partial.
cudaError_t launch_trig_scan(int kind, double* y, long long n, double* partial, double* work,
                             cudaStream_t st) {
  const long long M = n / 2;
  const long long chunks = (M + kScanChunk - 1) / kScanChunk;
  double* totals = work + M;
  double* half_y1 = totals + chunks;
  const double* sum0 = partial ? partial + 152 * 16 : nullptr;
  k_scan_chunks<<<(unsigned)chunks, kScanT, 0, st>>>(kind, y, n, sum0, work, totals, half_y1);
  k_scan_totals<<<1, 1024, 0, st>>>(totals, chunks);
  k_scan_apply<<<blocks_for(M, 256), 256, 0, st>>>(kind, y, n, work, totals, half_y1);
  return cudaGetLastError();
}

}  // namespace gbfft
