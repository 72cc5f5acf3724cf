// noalloc.cu -- gbfft_four1_noalloc: the complex FFT of gbfft_four1 for
// callers that must not allocate GPU memory.
//
// Some callers cannot call cudaMalloc at the moment they need an FFT: hosts
// that fix their GPU memory budget before the first frame (real-time and
// embedded systems, whose allocator may not be entered later), and plugins
// that live inside another framework's memory pool and may not allocate
// behind its back.  gbfft_four1 takes its ping-pong scratch and its twiddle
// tables from the library's allocator; this entry point takes them from
// arrays of fixed size that are part of the library image (file-scope
// __device__ arrays below).  Every GPU that loads the library holds them
// (about 19 MiB) until the process exits.
//
// Limits and rules:
//   - nn is a power of two with nn <= 2^20; larger sizes are rejected with
//     GBFFT_UNSUPPORTED_SIZE (they would need more scratch than the array has)
//   - data is device memory on a 16-byte boundary; the transform is in place,
//     FP64, on `stream`
//   - the first call on a device sets that device up (looks up the arrays'
//     device addresses and fills the twiddle table, then waits for the fill);
//     make that first call before any stream capture.  A first call made on a
//     capturing stream is refused with GBFFT_CUDA_ERROR before anything is
//     launched.
//   - all calls share the one scratch array, which keeps what the last call
//     left in it: calls that overlap on the GPU (other streams, or a second
//     host thread) race on it and must be ordered by the caller.  Every call
//     writes the scratch fully before it reads it, so nothing needs clearing
//     between calls.
#include <mutex>

#include "../../include/gbfft.h"
#include "arith.cuh"
#include "gbfft_internal.h"

namespace gbfft {

constexpr int kNoAllocMaxLog = 20;

// The arrays.  In host code these names are host-side stand-ins, not device
// addresses; host code only ever passes the addresses that
// cudaGetSymbolAddress returns for them.
static __device__ __align__(256) d2 g_noalloc_scratch[size_t(1) << kNoAllocMaxLog];
static __device__ __align__(256) d2 g_noalloc_tw_dense[dense_entries(kDenseLogMin)];
static __device__ __align__(256) d2 g_noalloc_tw_partial[partial_entries(kDenseLogMin)];

namespace {

constexpr int kMaxDevices = 64;

struct NoAllocDevice {
  bool ready = false;
  d2* scratch = nullptr;
  d2* dense = nullptr;
  d2* partial = nullptr;
};

NoAllocDevice g_noalloc_dev[kMaxDevices];
std::mutex g_noalloc_mu;

// exp(+2 pi i e / S) for every dense and partial entry (the layout of the
// library's FP64 tables, dense up to 2^kDenseLogMin only so that the fixed
// arrays stay small).
__global__ void k_noalloc_twiddles(d2* dense, d2* partial) {
  constexpr size_t nd = dense_entries(kDenseLogMin);
  const size_t total = nd + partial_entries(kDenseLogMin);
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    double c = 1.0, s = 0.0;
    if (i < nd) {
      if (i >= 2) {
        const int logS = 63 - __clzll((long long)i);
        const long long S = 1ll << logS;
        sincospi(2.0 * (double)((long long)i - S) / (double)S, &s, &c);
      }
      dense[i] = d2{c, s};
    } else {
      const size_t j = i - nd;
      const int lvl = (int)(j >> kPartialLog) + kDenseLogMin + 1;
      sincospi(2.0 * (double)(j & (kPartial - 1)) / (double)(1ll << lvl), &s, &c);
      partial[j] = d2{c, s};
    }
  }
}

// Set up device `dev` (the current device) on its first call.  Returns a
// message on failure, nullptr on success.
const char* setup_device(int dev, cudaStream_t st, NoAllocDevice** out) {
  if (dev < 0 || dev >= kMaxDevices) return "four1_noalloc: device index beyond 63";
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  NoAllocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    // The set-up launches a fill kernel and waits for it, which a stream
    // under capture cannot do: refuse before launching anything.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
      cudaGetLastError();
      return "four1_noalloc: cannot query the stream's capture state";
    }
    if (cs != cudaStreamCaptureStatusNone)
      return "four1_noalloc: the first call on a device must not be made under stream capture";
    if (cudaGetSymbolAddress((void**)&d.scratch, g_noalloc_scratch) != cudaSuccess ||
        cudaGetSymbolAddress((void**)&d.dense, g_noalloc_tw_dense) != cudaSuccess ||
        cudaGetSymbolAddress((void**)&d.partial, g_noalloc_tw_partial) != cudaSuccess) {
      cudaGetLastError();
      return "four1_noalloc: cudaGetSymbolAddress failed";
    }
    k_noalloc_twiddles<<<256, 256, 0, st>>>(d.dense, d.partial);
    if (cudaGetLastError() != cudaSuccess) return "four1_noalloc: twiddle fill launch failed";
    if (cudaStreamSynchronize(st) != cudaSuccess) return "four1_noalloc: twiddle fill failed";
    d.ready = true;
  }
  *out = &d;
  return nullptr;
}

// One pass of the Stockham schedule of a single line of L points (the same
// rules as the library's axis planner for s = 1, one line).
void plan_pass(PassParams& p, long long L, int logL, int logR, int logNs) {
  p = PassParams{};
  p.L = L;
  p.s = 1;
  p.lstride = L;
  p.nlines = 1;
  p.lq_log = 0;
  p.logL = logL;
  p.logR = logR;
  p.logNs = logNs;
  p.Ns = 1ll << logNs;
  const long long LR = L >> logR;
  int logC;
  if (LR > 1) {
    p.mode = 0;
    int lr = 63 - __builtin_clzll((unsigned long long)LR);
    logC = (12 - logR) < lr ? (12 - logR) : lr;
    p.in_rcontig = 0;
    p.out_rcontig = (logNs == 0) ? 1 : 0;
  } else {
    p.mode = 1;
    logC = 0;
    p.in_rcontig = 1;
    p.out_rcontig = 1;
  }
  if (logR + logC < 9) logC = 9 - logR;
  p.logC = logC;
  const int nsub = (logR + 3) / 4 > 0 ? (logR + 3) / 4 : 1;
  const int base = logR / nsub, extra = logR % nsub;
  p.nq = nsub;
  for (int i = 0; i < nsub; ++i) p.q[i] = base + (i < extra ? 1 : 0);
  p.tiles = (p.mode == 0) ? (LR >> logC) : 1;
  p.do_scale = 0;
  p.scale = 1.0;
}

}  // namespace

// Records the last error of the library (defined with the rest of the
// runtime); only called on failure.
void record_error(int code, const char* msg);

}  // namespace gbfft

extern "C" int gbfft_four1_noalloc(double* data, size_t nn, int isign, void* stream) {
  using namespace gbfft;
  if (!data) {
    record_error(GBFFT_INVALID_ARG, "four1_noalloc: null data");
    return GBFFT_INVALID_ARG;
  }
  if (isign != 1 && isign != -1) {
    record_error(GBFFT_INVALID_ARG, "four1_noalloc: isign must be 1 or -1");
    return GBFFT_INVALID_ARG;
  }
  if (((uintptr_t)data) & 15u) {
    // the passes move complex values as 16-byte vectors
    record_error(GBFFT_INVALID_ARG, "four1_noalloc: device arrays must start on a 16-byte boundary");
    return GBFFT_INVALID_ARG;
  }
  if (nn == 0 || (nn & (nn - 1)) || nn > (size_t(1) << kNoAllocMaxLog)) {
    record_error(GBFFT_UNSUPPORTED_SIZE,
                 "four1_noalloc: nn must be a power of two <= 2^20 (the size of its static "
                 "scratch array)");
    return GBFFT_UNSUPPORTED_SIZE;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    record_error(GBFFT_CUDA_ERROR, "four1_noalloc: no current device");
    return GBFFT_CUDA_ERROR;
  }
  NoAllocDevice* d = nullptr;
  if (const char* msg = setup_device(dev, st, &d)) {
    record_error(GBFFT_CUDA_ERROR, msg);
    return GBFFT_CUDA_ERROR;
  }
  if (nn == 1) return GBFFT_OK;
  const int logL = 63 - __builtin_clzll((unsigned long long)nn);
  const long long L = (long long)nn;
  // one pass up to 4096 points; otherwise two passes through the scratch
  int radix[2] = {logL, 0};
  int P = 1;
  if (logL > 12) {
    P = 2;
    radix[0] = (logL + 1) / 2;
    radix[1] = logL / 2;
  }
  Twiddles tw;
  tw.dense = d->dense;
  tw.partial = d->partial;
  tw.dense_log = kDenseLogMin;
  int logNs = 0;
  for (int i = 0; i < P; ++i) {
    PassParams p;
    plan_pass(p, L, logL, radix[i], logNs);
    p.tw = tw;
    p.in_ptrs = nullptr;
    p.out_ptrs = nullptr;
    p.in = (i == 0) ? (const void*)data : (const void*)d->scratch;
    p.out = (i == P - 1) ? (void*)data : (void*)d->scratch;
    const int threads = (1 << (p.logR + p.logC)) / 16;
    if (launch_pass_f64(isign, IO_D2, IO_D2, p, threads, st) != cudaSuccess) {
      record_error(GBFFT_CUDA_ERROR, "four1_noalloc: pass launch failed");
      return GBFFT_CUDA_ERROR;
    }
    logNs += radix[i];
  }
  return GBFFT_OK;
}
