// batch_kernels.cuh -- persistent batched FFT over thousands of transforms of
// uneven power-of-two sizes in one launch (FFTProcessor::fft_batch,
// src/FFT_1.rs:185-190, which runs one rayon task per transform).  The
// kernels are instantiated one form per translation unit (batch_<form>.cu) so
// that the library builds in parallel; batch.cu dispatches on the form.
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
#pragma once
#include <cstdio>
#include <cstdlib>
#include "fft_core.cuh"
#include "batch.h"
#include "tma.cuh"
#include "umma16.cuh"

namespace gbfft {

template <class F, int SG, int SIO>
__global__ void __launch_bounds__(256, (F::kind == 1 && !F::kTensor ? 3 : 2))
    k_batch(BatchParams P) {
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
      run_tile<F, SG, SIO, IO_D2, 256, true, true>(p, tile, sm, tid);
    } else if (R.kind == 1) {
      run_tile<F, SG, IO_D2, SIO, 256, false, true>(p, tile, sm, tid);
      __threadfence();
      __syncthreads();
      if (tid == 0) atomicAdd(P.done + R.first + line0, 1u);
    } else {
      run_tile<F, SG, IO_D2, IO_D2, 256, false, true>(p, tile, sm, tid);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Tensor-core form on tcgen05 (umma16.cuh): the same queue, pass-1 counters and
// bounded waits as k_batch; tiles are staged in shared memory, radix-16
// sub-passes run as tcgen05.mma products with TMEM accumulators, the other
// radices on the CUDA cores in FP32.  Each persistent CTA allocates its TMEM
// columns once and builds the DFT matrix once.
// Shared memory: [padded tile][X hi][X lo][W hi][W lo].
// ---------------------------------------------------------------------------
constexpr size_t kUmmaTileBytes = 36864;  // >= pass_smem_bytes<F32>(256), 1 KB multiple

inline size_t umma_smem_bytes() { return kUmmaTileBytes + 2 * kUmmaXBytes + 2 * kUmmaWBytes; }

// One tile, fused as the mma.sync kernel's tiles are: the first sub-pass reads
// global memory and the last one writes it; radix-16 sub-passes run as
// tcgen05 products, the other radices on the CUDA cores in FP32.  A pass of a
// single sub-pass runs on the CUDA cores from global to global.
template <int SG, int IN, int OUT, bool L2_ONLY>
__device__ __forceinline__ bool umma_tile(const PassParams& p, long long tile, f2* sm, UmmaCtx& u,
                                          int tid) {
  long long line0, j0;
  tile_origin(p, tile, line0, j0);
  if (p.nq == 1) {
    switch (p.q[0]) {
      case 4: only_subpass<TC32, SG, IN, OUT, 16, 256, L2_ONLY>(p, line0, j0, tid); break;
      case 3: only_subpass<TC32, SG, IN, OUT, 8, 256, L2_ONLY>(p, line0, j0, tid); break;
      case 2: only_subpass<TC32, SG, IN, OUT, 4, 256, L2_ONLY>(p, line0, j0, tid); break;
      default: only_subpass<TC32, SG, IN, OUT, 2, 256, L2_ONLY>(p, line0, j0, tid); break;
    }
    return true;
  }
  const int cs = col_stride(p.logR, F32::kPadShift);
  bool ok = true;
  if (p.q[0] == 4) {
    ok = subpass16_umma<SG, 1, 0, IN, OUT, L2_ONLY>(p, line0, j0, sm, cs, 0, u, tid);
  } else {
    first_subpass_q<TC32, SG, IN, 256, L2_ONLY>(p.q[0], p, line0, j0, sm, cs, tid);
    __syncthreads();
  }
  int logNsub = p.q[0];
  for (int k = 1; k + 1 < p.nq; ++k) {
    switch (p.q[k]) {
      case 4:
        ok = subpass16_umma<SG, 0, 0, IN, OUT, L2_ONLY>(p, line0, j0, sm, cs, logNsub, u, tid) && ok;
        break;
      case 3: subpass<F32, SG, 8>(sm, p.logR, cs, logNsub, p.tw, tid, 256); break;
      case 2: subpass<F32, SG, 4>(sm, p.logR, cs, logNsub, p.tw, tid, 256); break;
      default: subpass<F32, SG, 2>(sm, p.logR, cs, logNsub, p.tw, tid, 256); break;
    }
    logNsub += p.q[k];
  }
  if (p.q[p.nq - 1] == 4)
    ok = subpass16_umma<SG, 0, 1, IN, OUT, L2_ONLY>(p, line0, j0, sm, cs, logNsub, u, tid) && ok;
  else
    last_subpass_q<TC32, SG, OUT, 256>(p.q[p.nq - 1], p, line0, j0, sm, cs, tid);
  return ok;
}

template <int SG, int SIO>
__global__ void __launch_bounds__(256, 2) k_batch_umma(BatchParams P) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  f2* sm = reinterpret_cast<f2*>(smem_raw);
  unsigned char* xhi = smem_raw + kUmmaTileBytes;
  unsigned char* whi = xhi + 2 * kUmmaXBytes;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ long long s_item;
  __shared__ int s_ok, s_fail;
  const int tid = threadIdx.x;
  if (tid < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&tslot)),
                 "r"(kUmmaTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    s_fail = 0;
  }
  umma_build_w<SG>(whi, whi + kUmmaWBytes, reinterpret_cast<const f2*>(P.ranges[0].p.tw.dense),
                   tid, 256);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  UmmaCtx u;
  u.xhi = xhi;
  u.xlo = xhi + kUmmaXBytes;
  u.xhi_s = smem_addr(u.xhi);
  u.xlo_s = smem_addr(u.xlo);
  u.whi_s = smem_addr(whi);
  u.wlo_s = smem_addr(whi + kUmmaWBytes);
  u.tmem = tslot;
  u.bar = &bar;
  u.phase = 0;
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
    const long long line0 = (R.kind != 0) ? (tile >> ((p.logL - p.logR) - p.logC)) : 0;
    bool ok;
    if (R.kind == 2) {
      if (tid == 0) {
        volatile unsigned int* cnt = P.done + R.first + line0;
        unsigned int it = 0;
        int okw = 1;
        while (*cnt < R.need) {
          if (++it > P.spin_limit) {
            atomicExch(P.err, 1);
            okw = 0;
            break;
          }
          __nanosleep(128);
        }
        __threadfence();
        s_ok = okw;
      }
      __syncthreads();
      if (!s_ok) continue;
      ok = umma_tile<SG, SIO, IO_D2, true>(p, tile, sm, u, tid);
    } else if (R.kind == 1) {
      ok = umma_tile<SG, IO_D2, SIO, false>(p, tile, sm, u, tid);
      __threadfence();
      __syncthreads();
      if (tid == 0 && ok) atomicAdd(P.done + R.first + line0, 1u);
    } else {
      ok = umma_tile<SG, IO_D2, IO_D2, false>(p, tile, sm, u, tid);
    }
    if (!ok) {
      // a wait for the tensor cores ran out: report, stop taking tiles
      if (tid == 0) {
        atomicExch(P.err, 1);
        s_fail = 1;
      }
    }
    __syncthreads();
    if (s_fail) break;
  }
  // the products of a wait that ran out may still be in flight: wait for
  // them (bounded) before the TMEM is freed
  if (s_fail) mbar_wait_bounded(&bar, u.phase ^ 1u, kUmmaWaitLimit);
  tc_fence_before();
  __syncthreads();
  if (tid < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(u.tmem),
                 "r"(kUmmaTmemCols)
                 : "memory");
}

template <int SG, int SIO>
static cudaError_t prepare_umma_t() {
  static DeviceOnce done;
  static DeviceOnce carveout;
  cudaError_t e = smem_opt_in(k_batch_umma<SG, SIO>, umma_smem_bytes(), done);
  if (e != cudaSuccess) return e;
  // two CTAs of 108 KB need the largest shared-memory configuration of the
  // SM; without the preference the occupancy (and the launch) assume one
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (carveout.bits.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(k_batch_umma<SG, SIO>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           (int)cudaSharedmemCarveoutMaxShared);
  if (e == cudaSuccess && bit) carveout.bits.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

template <int SG, int SIO>
static cudaError_t launch_batch_umma_t(const BatchParams& P, int grid, cudaStream_t st) {
  cudaError_t e = prepare_umma_t<SG, SIO>();
  if (e != cudaSuccess) return e;
  k_batch_umma<SG, SIO><<<grid, 256, umma_smem_bytes(), st>>>(P);
  return cudaGetLastError();
}

template <int SG, int SIO>
static int occupancy_umma_t() {
  int n = 0;
  cudaError_t e = prepare_umma_t<SG, SIO>();
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_umma<SG, SIO>, 256,
                                                      umma_smem_bytes());
  // The occupancy query has been seen to report one CTA where the launch
  // fits two (registers and shared memory both allow two, by the kernel's
  // attributes and by the hardware's own occupancy limits).  Count from the
  // attributes as well and take the larger figure when both resources fit.
  int fit = 0;
  if (e == cudaSuccess) {
    cudaFuncAttributes fa;
    cudaDeviceProp dp;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaFuncGetAttributes(&fa, k_batch_umma<SG, SIO>) == cudaSuccess &&
        cudaGetDeviceProperties(&dp, dev) == cudaSuccess) {
      const size_t per_cta = umma_smem_bytes() + fa.sharedSizeBytes + dp.reservedSharedMemPerBlock;
      const int by_smem = (int)(dp.sharedMemPerMultiprocessor / per_cta);
      const int by_regs = fa.numRegs > 0 ? dp.regsPerMultiprocessor / (fa.numRegs * 256) : 0;
      fit = by_smem < by_regs ? by_smem : by_regs;
    }
    cudaGetLastError();
  }
  if (getenv("GBFFT_TUNE_VERBOSE"))
    fprintf(stderr,
            "gbfft k_batch_umma: %d CTAs per SM by the occupancy query (%s), %d by the kernel's "
            "attributes, %zu B dynamic shared memory\n",
            n, cudaGetErrorString(e), fit, umma_smem_bytes());
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  if (fit > n) n = fit;
  // each CTA holds kUmmaTmemCols of the SM's 512 TMEM columns
  return n < (int)(512 / kUmmaTmemCols) ? n : (int)(512 / kUmmaTmemCols);
}

// ---------------------------------------------------------------------------
// Prefetching variant (FP32, tensor-core and double-float forms, all caller
// arrays 16-byte aligned).  While a CTA computes one tile, warp 0 has the
// bulk-copy engine (cp.async.bulk, completed on an mbarrier) bring the raw
// elements of the CTA's next tile into a staging buffer, so the load latency
// of one tile hides behind the arithmetic of the previous one.  Pass-2 tiles
// of two-pass bins are not prefetched: they must first see their transform's
// pass-1 counter, so they load as in k_batch.
// Shared memory: [staging: 4096 x 16 B][padded tile][mbarrier]
// ---------------------------------------------------------------------------
constexpr size_t kStagingBytes = size_t(kEPT) * 256 * 16;
// try_wait calls before a bulk-copy wait gives up (each may suspend the
// thread for a short hardware-defined time)
constexpr uint32_t kCopyWaitLimit = 1u << 20;

// Warp 0: start the bulk copies of `item` into staging.  Returns 1 when copies
// were issued (the mbarrier will complete a phase), 0 when nothing was (end
// of queue or a pass-2 tile).
__device__ __forceinline__ int prefetch_item(const BatchParams& P, long long item, d2* staging,
                                             uint64_t* bar, int lane) {
  if (item >= P.total) return 0;
  int ri = 0;
  while (ri + 1 < P.nranges && item >= P.ranges[ri + 1].item0) ++ri;
  const BatchRange& R = P.ranges[ri];
  if (R.kind == 2) return 0;
  const PassParams& p = R.p;
  long long line0, j0;
  tile_origin(p, item - R.item0, line0, j0);
  const int Rn = 1 << p.logR, Cn = 1 << p.logC;
  int ncopies;
  uint32_t bytes_each;
  if (p.in_rcontig) {
    // single-pass bin: one contiguous transform per column
    long long valid = p.nlines - line0;
    ncopies = (int)(valid < Cn ? valid : Cn);
    bytes_each = (uint32_t)Rn * 16u;
  } else {
    // pass 1 of a two-pass bin: one run of C elements per row
    ncopies = Rn;
    bytes_each = (uint32_t)Cn * 16u;
  }
  if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)ncopies * bytes_each);
  __syncwarp();
  for (int i = lane; i < ncopies; i += 32) {
    const d2* src;
    d2* dst;
    if (p.in_rcontig) {
      src = reinterpret_cast<const d2*>(p.in_ptrs[line0 + i]);
      dst = staging + (size_t)i * Rn;
    } else {
      src = reinterpret_cast<const d2*>(p.in_ptrs[line0]) + j0 +
            ((long long)i << (p.logL - p.logR));
      dst = staging + (size_t)i * Cn;
    }
    bulk_copy_g2s(dst, src, bytes_each, bar);
  }
  return 1;
}

template <class F, int SG, int SIO>
__global__ void __launch_bounds__(256, (F::kind == 2 ? 1 : 2)) k_batch_pf(BatchParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  d2* staging = reinterpret_cast<d2*>(smem_raw);
  typename F::S* sm = reinterpret_cast<typename F::S*>(smem_raw + kStagingBytes);
  __shared__ __align__(8) uint64_t bar;
  __shared__ long long s_item, s_next;
  __shared__ int s_pref, s_pref_next, s_ok, s_fail;
  const int tid = threadIdx.x, lane = tid & 31;
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    s_fail = 0;
  }
  __syncthreads();
  if (tid < 32) {
    long long it = 0;
    if (lane == 0) it = (long long)atomicAdd(P.head, 1ull);
    it = __shfl_sync(0xffffffffu, it, 0);
    const int pf = prefetch_item(P, it, staging, &bar, lane);
    if (lane == 0) {
      s_item = it;
      s_pref = pf;
    }
  }
  __syncthreads();
  uint32_t parity = 0;
  for (;;) {
    const long long item = s_item;
    const int pref = s_pref;
    if (item >= P.total) break;
    int ri = 0;
    while (ri + 1 < P.nranges && item >= P.ranges[ri + 1].item0) ++ri;
    const BatchRange& R = P.ranges[ri];
    const PassParams& p = R.p;
    const long long tile = item - R.item0;
    long long line0, j0;
    tile_origin(p, tile, line0, j0);
    if (pref) {
      // every thread waits for the bulk copies (bounded), then stages its
      // sixteen elements from the staging buffer into the padded tile
      if (!mbar_wait_bounded(&bar, parity, kCopyWaitLimit)) atomicOr(&s_fail, 1);
      parity ^= 1u;
      __syncthreads();
      if (s_fail) {
        if (tid == 0) atomicExch(P.err, 1);
        break;
      }
#pragma unroll
      for (int k = 0; k < kEPT; ++k) {
        const int e = tid + k * 256;
        stage_elem<F, SG, IO_D2>(p, line0, j0, e, staging[e], sm);
      }
    } else {
      // pass-2 tile: wait for the transform's pass-1 tiles, then load
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
      if (!s_ok) break;  // error already recorded; the host reports GBFFT_TIMEOUT
      using IE = typename IOElem<SIO>::T;
      IE raw[kEPT];
      load_tile_raw<IE, SIO, 256, true>(p, line0, j0, tid, raw);
#pragma unroll
      for (int k = 0; k < kEPT; ++k) stage_elem<F, SG, SIO>(p, line0, j0, tid + k * 256, raw[k], sm);
    }
    __syncthreads();  // tile staged; the staging buffer is free again
    if (tid < 32) {
      fence_proxy_async_smem();
      long long nx = 0;
      if (lane == 0) nx = (long long)atomicAdd(P.head, 1ull);
      nx = __shfl_sync(0xffffffffu, nx, 0);
      const int pf = prefetch_item(P, nx, staging, &bar, lane);
      if (lane == 0) {
        s_next = nx;
        s_pref_next = pf;
      }
    }
    if (R.kind == 1) {
      tile_compute_store<F, SG, SIO, 256>(p, line0, j0, sm, tid);
      __threadfence();
      __syncthreads();
      if (tid == 0) atomicAdd(P.done + R.first + line0, 1u);
    } else {
      tile_compute_store<F, SG, IO_D2, 256>(p, line0, j0, sm, tid);
    }
    __syncthreads();
    if (tid == 0) {
      s_item = s_next;
      s_pref = s_pref_next;
    }
    __syncthreads();
  }
  // a copy still in flight (only after a failed wait) must land before exit
  if (s_pref && s_item < P.total) mbar_wait_bounded(&bar, parity, kCopyWaitLimit);
}

template <class F>
inline size_t pf_smem_bytes() {
  return kStagingBytes + pass_smem_bytes<F>(256);
}

template <class F, int SG, int SIO>
static cudaError_t prepare_pf_t() {
  static DeviceOnce done;
  return smem_opt_in(k_batch_pf<F, SG, SIO>, pf_smem_bytes<F>(), done);
}

template <class F, int SG, int SIO>
static cudaError_t launch_batch_pf_t(const BatchParams& P, int grid, cudaStream_t st) {
  cudaError_t e = prepare_pf_t<F, SG, SIO>();
  if (e != cudaSuccess) return e;
  k_batch_pf<F, SG, SIO><<<grid, 256, pf_smem_bytes<F>(), st>>>(P);
  return cudaGetLastError();
}

template <class F, int SG, int SIO>
static int occupancy_pf_t() {
  int n = 0;
  if (prepare_pf_t<F, SG, SIO>() != cudaSuccess) return 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_pf<F, SG, SIO>, 256,
                                                pf_smem_bytes<F>());
  return n;
}

// Raise the dynamic shared memory limit of one instantiation on the current
// device (once per device; called before any stream capture).
template <class F, int SG, int SIO>
static cudaError_t prepare_t() {
  static DeviceOnce done;
  return smem_opt_in(k_batch<F, SG, SIO>, pass_smem_bytes<F>(256), done);
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

}  // namespace gbfft
