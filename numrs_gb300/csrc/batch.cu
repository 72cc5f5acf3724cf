// batch.cu -- persistent batched FFT over thousands of transforms of uneven
// power-of-two sizes in one launch (FFTProcessor::fft_batch,
// src/FFT_1.rs:185-190, which runs one rayon task per transform).
//
// The host sorts the transforms into size bins and lays the work out as a
// queue of tiles:
//
//   [pass 1 of every two-pass bin] [single-pass bins, largest first]
//   [pass 2 of every two-pass bin]
//
// Resident CTAs take tiles from the queue with one atomicAdd each.  A pass-2
// tile needs every pass-1 tile of its transform: pass-1 tiles bump a
// per-transform counter after a fence, and a pass-2 tile polls that counter.
// The poll is bounded (spin_limit iterations with __nanosleep); if it runs out
// the CTA records an error flag, skips the tile and goes on, and the host
// reports GBFFT_TIMEOUT.  A pass-2 tile only ever waits on tiles that were
// handed out before it, so the wait always ends unless a CTA died.
#include "fft_core.cuh"
#include "batch.h"

namespace gbfft {

template <class F, int SG, int SIO>
__global__ void __launch_bounds__(256, 2) k_batch(BatchParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  typename F::S* sm = reinterpret_cast<typename F::S*>(smem_raw);
  __shared__ long long s_item;
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_item = (long long)atomicAdd(P.head, 1ull);
    __syncthreads();
    const long long item = s_item;
    __syncthreads();
    if (item >= P.total) break;
    int ri = 0;
    while (ri + 1 < P.nranges && item >= P.ranges[ri + 1].item0) ++ri;
    const BatchRange& R = P.ranges[ri];
    const PassParams& p = R.p;
    const long long tile = item - R.item0;
    // mode-0 tiles of the two-pass bins cover one transform each
    const long long line0 = (R.kind != 0) ? (tile >> ((p.logL - p.logR) - p.logC)) : 0;
    if (R.kind == 2) {
      if (tid == 0) {
        volatile unsigned int* cnt = P.done + R.first + line0;
        unsigned int it = 0;
        int ok = 1;
        while (*cnt < R.need) {
          if (++it > P.spin_limit) {
            atomicExch(P.err, 1);
            ok = 0;
            break;
          }
          __nanosleep(128);
        }
        __threadfence();
        s_ok = ok;
      }
      __syncthreads();
      if (!s_ok) continue;
      pass_tile<F, SG, SIO, IO_D2, 256, true>(p, tile, sm, tid);
    } else if (R.kind == 1) {
      pass_tile<F, SG, IO_D2, SIO, 256, false>(p, tile, sm, tid);
      __threadfence();
      __syncthreads();
      if (tid == 0) atomicAdd(P.done + R.first + line0, 1u);
    } else {
      pass_tile<F, SG, IO_D2, IO_D2, 256, false>(p, tile, sm, tid);
    }
    __syncthreads();
  }
}

// Raise the dynamic shared memory limit of one instantiation (idempotent;
// called before any stream capture).
template <class F, int SG, int SIO>
static cudaError_t prepare_t() {
  static bool done = false;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_batch<F, SG, SIO>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)pass_smem_bytes<F>(256));
  if (e == cudaSuccess) done = true;
  return e;
}

template <class F, int SG, int SIO>
static cudaError_t launch_batch_t(const BatchParams& P, int grid, cudaStream_t st) {
  cudaError_t e = prepare_t<F, SG, SIO>();
  if (e != cudaSuccess) return e;
  k_batch<F, SG, SIO><<<grid, 256, pass_smem_bytes<F>(256), st>>>(P);
  return cudaGetLastError();
}

template <class F, int SG, int SIO>
static int occupancy_t() {
  int n = 0;
  if (prepare_t<F, SG, SIO>() != cudaSuccess) return 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch<F, SG, SIO>, 256,
                                                pass_smem_bytes<F>(256));
  return n;
}

cudaError_t launch_batch(Form f, int sign, const BatchParams& P, int grid, cudaStream_t st) {
  if (f == FORM_F64)
    return sign > 0 ? launch_batch_t<F64, 1, IO_D2>(P, grid, st)
                    : launch_batch_t<F64, -1, IO_D2>(P, grid, st);
  if (f == FORM_F32)
    return sign > 0 ? launch_batch_t<F32, 1, IO_F2>(P, grid, st)
                    : launch_batch_t<F32, -1, IO_F2>(P, grid, st);
  if (f == FORM_TC32)
    return sign > 0 ? launch_batch_t<TC32, 1, IO_F2>(P, grid, st)
                    : launch_batch_t<TC32, -1, IO_F2>(P, grid, st);
  return sign > 0 ? launch_batch_t<DF64, 1, IO_F4>(P, grid, st)
                  : launch_batch_t<DF64, -1, IO_F4>(P, grid, st);
}

int batch_blocks_per_sm(Form f, int sign) {
  if (f == FORM_F64)
    return sign > 0 ? occupancy_t<F64, 1, IO_D2>() : occupancy_t<F64, -1, IO_D2>();
  if (f == FORM_F32)
    return sign > 0 ? occupancy_t<F32, 1, IO_F2>() : occupancy_t<F32, -1, IO_F2>();
  if (f == FORM_TC32)
    return sign > 0 ? occupancy_t<TC32, 1, IO_F2>() : occupancy_t<TC32, -1, IO_F2>();
  return sign > 0 ? occupancy_t<DF64, 1, IO_F4>() : occupancy_t<DF64, -1, IO_F4>();
}

}  // namespace gbfft
