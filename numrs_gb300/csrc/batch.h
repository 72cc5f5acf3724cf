// batch.h -- descriptors of the persistent batched FFT launch (batch.cu).
#pragma once
#include "gbfft_internal.h"

namespace gbfft {

// One pass of one size bin: a contiguous run of queue items.
//   kind 0  single-pass bin: caller arrays -> caller arrays
//   kind 1  pass 1 of a two-pass bin: caller arrays -> bin scratch; each tile
//           bumps done[first + line] when its stores are visible
//   kind 2  pass 2: bin scratch -> caller arrays; each tile first waits until
//           done[first + line] == need
struct BatchRange {
  PassParams p;
  long long item0;
  long long first;
  unsigned int need;
  int kind;
};

// Bins of 2^1..2^12 points take one range each, bins of 2^13..2^20 two.
constexpr int kMaxBatchRanges = 32;

// Passed by value, so the range table lives in the kernel's parameter space:
// reads of it go through the constant cache and the compiler may keep them
// in registers across the tile's barriers and stores (a table in global
// memory has to be re-read after each of them).
struct BatchParams {
  BatchRange ranges[kMaxBatchRanges];  // sorted by item0
  int nranges;
  long long total;           // queue length
  unsigned long long* head;  // next queue item (zeroed before the launch)
  unsigned int* done;        // per-transform pass-1 tile counters (zeroed)
  int* err;                  // set to 1 when a bounded wait gives up (zeroed)
  unsigned int spin_limit;
};
static_assert(sizeof(BatchParams) <= 32000, "kernel parameters are limited to 32764 bytes");

cudaError_t launch_batch(Form f, int sign, const BatchParams& P, int grid, cudaStream_t st);
// Resident CTAs per SM; also raises the kernel's shared memory limit, so it
// is called before the launch is captured.
int batch_blocks_per_sm(Form f, int sign);
// Prefetching variant (FP32, TC32, DF64 forms; every caller array 16-byte
// aligned): bulk copies of the next tile overlap the current tile's compute.
cudaError_t launch_batch_pf(Form f, int sign, const BatchParams& P, int grid, cudaStream_t st);
int batch_pf_blocks_per_sm(Form f, int sign);

// The tensor-core form on tcgen05 (batch_umma.cu): radix-16 sub-passes as
// tcgen05.mma products with TMEM accumulators.
cudaError_t launch_batch_umma(int sign, const BatchParams& P, int grid, cudaStream_t st);
int batch_blocks_per_sm_umma(int sign);

// per-form launchers (batch_<form>.cu), behind the dispatchers above
cudaError_t launch_batch_f64(int sign, const BatchParams& P, int grid, cudaStream_t st);
cudaError_t launch_batch_f32(int sign, const BatchParams& P, int grid, cudaStream_t st);
cudaError_t launch_batch_tc32(int sign, const BatchParams& P, int grid, cudaStream_t st);
cudaError_t launch_batch_df64(int sign, const BatchParams& P, int grid, cudaStream_t st);
int batch_blocks_per_sm_f64(int sign);
int batch_blocks_per_sm_f32(int sign);
int batch_blocks_per_sm_tc32(int sign);
int batch_blocks_per_sm_df64(int sign);
cudaError_t launch_batch_pf_f32(int sign, const BatchParams& P, int grid, cudaStream_t st);
cudaError_t launch_batch_pf_tc32(int sign, const BatchParams& P, int grid, cudaStream_t st);
cudaError_t launch_batch_pf_df64(int sign, const BatchParams& P, int grid, cudaStream_t st);
int batch_pf_blocks_per_sm_f32(int sign);
int batch_pf_blocks_per_sm_tc32(int sign);
int batch_pf_blocks_per_sm_df64(int sign);

}  // namespace gbfft
