// host.cu -- runtime behind the C ABI: device context, twiddle tables,
// axis plans (Stockham pass schedules), scratch management and the entry
// points declared in include/gbfft.h.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gbfft.h"
#include "batch.h"
#include "gbfft_internal.h"

namespace gbfft {

namespace {

constexpr int kMaxPassLog = 10;  // radix of a pass in a multi-pass schedule
constexpr int kMaxAxisLog = kMaxLog;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

struct ProfRec {
  int kind;
  cudaEvent_t a, b;
  double bytes;
  double flops;
};

struct Ctx {
  bool inited = false;
  int device = -1;  // bound at the first call (-1: not yet)
  cudaStream_t stream = nullptr;  // library stream
  cudaStream_t cur = nullptr;     // stream of the call in progress
  // Calls share the library's work buffers.  An asynchronous device call
  // records order_ev on its stream; a later call on another stream waits for
  // it, so that calls never overlap on those buffers.
  cudaEvent_t order_ev = nullptr;
  cudaStream_t order_stream = nullptr;
  bool order_pending = false;
  void* tw_dense[kForms] = {nullptr, nullptr, nullptr, nullptr};
  void* tw_part[kForms] = {nullptr, nullptr, nullptr, nullptr};
  std::map<int, void*> tw_top[kForms];  // dense copies of levels above kDenseLog
  bool top_tables = true;               // GBFFT_TOP_TWIDDLES=0 or the debug key: off
  DevBuf scratch;   // Stockham ping-pong buffer
  DevBuf work;      // spectral working set (two n-real lines)
  DevBuf stage_a;   // device copies of host arguments
  DevBuf stage_b;
  DevBuf stage_c;
  DevBuf ptrtab;
  std::vector<char> host_pack;
  std::string err;
  long long launches = 0;
  bool host_direct = false;  // kernels may read/write the caller's host arrays
  bool autotune = false;     // time candidate tile sizes on a plan's first use
  bool tune_verbose = false;
  std::string tune_cache;    // file of tuned tile sizes (GBFFT_TUNE_CACHE)
  bool profiling = false;
  std::vector<ProfRec> prof;
  std::vector<cudaEvent_t> evpool;
  // Failure injection (gbfft_debug_set): fail the k-th device allocation
  // counted from the setting (0 = never); the persistent batch kernel's poll
  // limit (0 = the default) and an addition to its pass-2 wait targets.
  long long fail_alloc_at = 0;
  long long alloc_calls = 0;
  unsigned int dbg_spin_limit = 0;
  unsigned int dbg_need_extra = 0;
  int dbg_first_radix_delta = 0;  // shifts the default two-pass batch split
  // tensor-core batch form on tcgen05 (the default) or on the warp-level
  // mma.sync kernel (GBFFT_TC_UMMA=0); the tcgen05 kernel measured 5 % faster
  // on the 20,000-transform batch
  bool tc_umma = true;
  bool fused_twist = true;  // realft twist on a pass (off: its own kernel)
  // FP32 axes of 2^22..2^28 points in two cluster passes (k_pass_cl) instead
  // of three per-CTA passes (GBFFT_CLUSTER_PASS=1 or the debug key).  Off by
  // default: the exchange over distributed shared memory costs more than the
  // HBM pass it saves (four1 2^28: 8.36 against 4.63 ms)
  bool cluster_pass = false;
  // convlv/correl forward transforms: 0 = the two inputs as two n/2-point
  // realft lines, 1 = packed as one n-point complex FFT (twofft)
  int spectral_path = 0;
};

Ctx g;
std::mutex g_mu;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g.err = buf;
  return code;
}

#define CK(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail(e_ == cudaErrorMemoryAllocation ? GBFFT_OOM : GBFFT_CUDA_ERROR,          \
                  "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__);    \
  } while (0)

#define TRY(expr)            \
  do {                       \
    int s_ = (expr);         \
    if (s_ != GBFFT_OK) return s_; \
  } while (0)

bool is_pow2(unsigned long long x) { return x && !(x & (x - 1)); }
int ilog2(unsigned long long x) { return 63 - __builtin_clzll(x); }
unsigned long long npow2(unsigned long long x) {
  unsigned long long p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Every device allocation of the library goes through here, so that a test
// can make the k-th one fail (gbfft_debug_set) and check that the call
// reports GBFFT_OOM and that the library works afterwards.
cudaError_t dev_alloc(void** p, size_t bytes) {
  if (g.fail_alloc_at > 0 && ++g.alloc_calls == g.fail_alloc_at) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();  // clear the (non-sticky) allocation error
  }
  return e;
}

int ensure(DevBuf& b, size_t bytes) {
  if (b.bytes >= bytes) return GBFFT_OK;
  if (b.p) {
    cudaDeviceSynchronize();
    cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  size_t want = std::max(bytes, (size_t)1 << 20);
  cudaError_t e = dev_alloc(&b.p, want);
  if (e != cudaSuccess)
    return fail(GBFFT_OOM, "cudaMalloc(%zu) failed: %s", want, cudaGetErrorString(e));
  b.bytes = want;
  return GBFFT_OK;
}

// The library binds to one device: `device` when gbfft_init names one (>= 0),
// else the device current on the calling thread at its first call (one
// process per GPU: each rank selects its device before its first call).
// Later calls run their work on that device whatever the calling thread's
// current device is (StreamScope), and leave the caller's current device as
// they found it.
int init_locked(int device) {
  if (g.inited) return GBFFT_OK;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    return fail(GBFFT_CUDA_ERROR, "no CUDA device: %s", cudaGetErrorString(e));
  int cur = 0;
  CK(cudaGetDevice(&cur));
  if (device < 0) device = cur;
  if (device >= n) return fail(GBFFT_INVALID_ARG, "init: device %d of %d", device, n);
  struct Restore {
    int dev;
    bool on;
    ~Restore() { if (on) cudaSetDevice(dev); }
  } restore{cur, device != cur};
  if (device != cur) CK(cudaSetDevice(device));
  CK(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&g.order_ev, cudaEventDisableTiming));
  g.cur = g.stream;
  g.device = device;
  // On systems where the GPU reaches pageable host memory through the host's
  // page tables (Grace + GB300 over NVLink-C2C), host-pointer calls let the
  // first pass read the caller's arrays and the last pass write them, so the
  // link transfers overlap the compute instead of preceding and following it.
  int pma = 0;
  cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
  const char* env = getenv("GBFFT_HOST_DIRECT");
  g.host_direct = pma != 0 && !(env && env[0] == '0');
  const char* at = getenv("GBFFT_AUTOTUNE");
  g.autotune = at && at[0] == '1';
  const char* tv = getenv("GBFFT_TUNE_VERBOSE");
  g.tune_verbose = tv && tv[0] == '1';
  const char* tc = getenv("GBFFT_TUNE_CACHE");
  if (tc) g.tune_cache = tc;
  const char* um = getenv("GBFFT_TC_UMMA");
  g.tc_umma = !(um && um[0] == '0');
  const char* tt = getenv("GBFFT_TOP_TWIDDLES");
  g.top_tables = !(tt && tt[0] == '0');
  const char* cp = getenv("GBFFT_CLUSTER_PASS");
  g.cluster_pass = cp && cp[0] == '1';
  g.inited = true;
  return GBFFT_OK;
}

int tables(Form f, Twiddles& tw) {
  if (f == FORM_TC32) f = FORM_F32;  // the tensor-core form uses the FP32 tables
  if (!g.tw_dense[f] || !g.tw_part[f]) {
    // both tables or neither: a failed allocation leaves none behind
    size_t esz = (f == FORM_F32) ? 8 : 16;
    void* dense = nullptr;
    void* part = nullptr;
    cudaError_t e = dev_alloc(&dense, dense_entries(kDenseLog) * esz);
    if (e == cudaSuccess) e = dev_alloc(&part, partial_entries(kDenseLog) * esz);
    if (e != cudaSuccess) {
      if (dense) cudaFree(dense);
      return fail(e == cudaErrorMemoryAllocation ? GBFFT_OOM : GBFFT_CUDA_ERROR,
                  "twiddle tables: cudaMalloc failed: %s", cudaGetErrorString(e));
    }
    CK(launch_twiddles(f, dense, part, kDenseLog, g.cur));
    g.launches++;
    g.tw_dense[f] = dense;
    g.tw_part[f] = part;
  }
  tw.dense = g.tw_dense[f];
  tw.partial = g.tw_part[f];
  tw.dense_log = kDenseLog;
  return GBFFT_OK;
}

// A dense copy of twiddle level logS (above the dense tables) for the FP64
// form, built on first use and kept: the last pass of a long axis (2^21..2^28
// points) then reads one table entry per twiddle instead of multiplying two,
// 4 FP64-pipe instructions per point less (four1 2^24 2.91 -> 2.80 ms, 2^28
// 52.65 -> 51.50 ms, same GPU).  The level takes 16 B per entry, as much as
// the transform's data.  The double-float form keeps the product: it runs on
// the FP32 pipe, cheaper than gathering 16-byte entries from a table of that
// size (four1 2^24 1.15 -> 1.31 ms with the table).  Skipped, and the product
// kept, when the level would take more than a quarter of the free device
// memory, when the allocation fails, or while the stream captures a graph.
void top_table(Form f, int logS, Twiddles& tw) {
  if (f != FORM_F64 || !g.top_tables) return;
  if (logS <= tw.dense_log || logS > kMaxLog) return;
  auto& m = g.tw_top[f];
  auto it = m.find(logS);
  void* p = nullptr;
  if (it != m.end()) {
    p = it->second;
  } else {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(g.cur, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
      cudaGetLastError();
      return;
    }
    const size_t bytes = ((size_t)1 << logS) * 16;
    size_t freeb = 0, totalb = 0;
    if (cudaMemGetInfo(&freeb, &totalb) != cudaSuccess || bytes > freeb / 4) {
      cudaGetLastError();
      return;
    }
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    if (launch_twiddle_level(f, p, logS, g.cur) != cudaSuccess) {
      cudaFree(p);
      cudaGetLastError();
      return;
    }
    g.launches++;
    m[logS] = p;
  }
  tw.top = p;
  tw.top_log = logS;
}

// ---------------------------------------------------------------------------
// Optional per-kernel timing: events around every launch on the launching
// stream, summed per kernel kind on request.
// ---------------------------------------------------------------------------
enum ProfKind { PK_PASS = 0, PK_TWIST = 1, PK_SPECTRAL = 2, PK_OTHER = 3, PK_COUNT = 4 };

cudaEvent_t pool_event() {
  if (!g.evpool.empty()) {
    cudaEvent_t e = g.evpool.back();
    g.evpool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

struct ProfScope {
  bool on;
  ProfRec r;
  ProfScope(int kind, double bytes, double flops = 0.0) : on(g.profiling) {
    if (!on) return;
    r.kind = kind;
    r.bytes = bytes;
    r.flops = flops;
    r.a = pool_event();
    r.b = pool_event();
    cudaEventRecord(r.a, g.cur);
  }
  ~ProfScope() {
    if (!on) return;
    cudaEventRecord(r.b, g.cur);
    g.prof.push_back(r);
  }
};

IOType scratch_io(Form f) {
  return f == FORM_F64 ? IO_D2 : (f == FORM_DF64 ? IO_F4 : IO_F2);
}

// ---------------------------------------------------------------------------
// Axis plan: the Stockham pass schedule for `nlines` lines of length L along
// an axis of stride s.  Line l starts at (l >> lq_log) * lstride + (l & mask).
// ---------------------------------------------------------------------------
struct Pass {
  PassParams p;
  int threads;
  int in_user;   // 1: reads the caller buffer, 0: the scratch buffer
  int out_user;
};

struct AxisPlan {
  std::vector<Pass> passes;
  size_t scratch_elems = 0;
};

// The largest twiddle level of a plan's passes.
int plan_top_log(const AxisPlan& ap) {
  int m = 0;
  for (const Pass& ps : ap.passes) m = std::max(m, ps.p.logNs + ps.p.logR);
  return m;
}

// Sub-passes of radix <= 4 (latency tiles hold four points per thread).
void split_subpasses_r4(int logR, PassParams& p) {
  p.nq = (logR + 1) / 2;
  for (int i = 0; i < 4; ++i) p.q[i] = 0;
  for (int i = 0; i < p.nq; ++i) p.q[i] = (i < logR / 2) ? 2 : 1;
}

void split_subpasses(int logR, PassParams& p) {
  int nsub = (logR + 3) / 4;
  if (nsub < 1) nsub = 1;
  int base = logR / nsub, extra = logR % nsub;
  p.nq = nsub;
  for (int i = 0; i < 4; ++i) p.q[i] = 0;
  for (int i = 0; i < nsub; ++i) p.q[i] = base + (i < extra ? 1 : 0);
}

// Latency mode: one or two small transforms (2^10..2^14 points, at most 16384
// points in all) would run on 1-4 SMs in 4096-point tiles, and an FP64
// transform of 4096 points then takes ~40 us on one SM (GB300 issues FP64 at 2
// lanes per SM).  Two passes of 128-point one-warp tiles (k_pass_lat, four
// points per thread, radix <= 2^7 per pass) spread the same work over 16-128
// SMs.
constexpr long long kLatencyMaxWork = 16384;
constexpr int kLatencyTileLog = 7;  // kLatencyEPT points x 32 threads

// tileLog: log2 of the complex elements per CTA tile (10..12); multi-pass
// radices are kept 4 columns below it so that strided rows stay >= 64 bytes.
// radices: an explicit pass schedule (log2 radix of each pass, summing to
// log2 L, each at most tileLog) instead of the default one.
AxisPlan make_axis_plan(long long L, long long s, long long nlines, int lq_log,
                        long long lstride, bool full_tile = false, int tileLog = 12,
                        const std::vector<int>* radices = nullptr) {
  AxisPlan ap;
  const int logL = ilog2((unsigned long long)L);
  const int maxPassLog = std::min(kMaxPassLog, tileLog - 2);
  std::vector<int> radix;
  const bool latency = !full_tile && s == 1 && logL >= 10 && logL <= 2 * kLatencyTileLog &&
                       L * nlines <= kLatencyMaxWork;
  if (radices) {
    radix = *radices;
  } else if (latency) {
    radix.push_back((logL + 1) / 2);
    radix.push_back(logL / 2);
  } else if (logL <= tileLog) {
    radix.push_back(logL);
  } else {
    int P = (logL + maxPassLog - 1) / maxPassLog;
    int base = logL / P, extra = logL % P;
    for (int i = 0; i < P; ++i) radix.push_back(base + (i < extra ? 1 : 0));
  }
  int logNs = 0;
  const int P = (int)radix.size();
  for (int i = 0; i < P; ++i) {
    Pass ps;
    PassParams& p = ps.p;
    std::memset(&p, 0, sizeof p);
    const int logR = radix[i];
    p.in_ptrs = nullptr;
    p.out_ptrs = nullptr;
    p.L = L;
    p.s = s;
    p.lstride = lstride;
    p.nlines = nlines;
    p.lq_log = lq_log;
    p.logL = logL;
    p.logR = logR;
    p.logNs = logNs;
    p.Ns = 1ll << logNs;
    const long long LR = L >> logR;
    int logC;
    if (s == 1 && LR > 1) {
      p.mode = 0;
      const int tl = latency ? kLatencyTileLog : tileLog;
      logC = std::min(tl - logR, ilog2((unsigned long long)LR));
      p.in_rcontig = 0;
      p.out_rcontig = (logNs == 0) ? 1 : 0;
    } else {
      p.mode = 1;
      int want = tileLog - logR;
      int have = ilog2(npow2((unsigned long long)nlines));
      logC = full_tile ? want : std::min(want, have);
      p.in_rcontig = (s == 1) ? 1 : 0;
      p.out_rcontig = (s == 1) ? 1 : 0;
    }
    // at least one full warp: 16 * 32 = 512 elements per tile (latency tiles:
    // 4 * 32 = 128)
    const int minTile = latency ? kLatencyTileLog : 9;
    if (logR + logC < minTile) logC = minTile - logR;
    p.logC = logC;
    ps.threads = (1 << (logR + logC)) / (latency ? kLatencyEPT : kTileEPT);
    if (latency) split_subpasses_r4(logR, p);
    else split_subpasses(logR, p);
    p.lat = latency ? 1 : 0;
    if (p.mode == 0) p.tiles = nlines * (LR >> logC);
    else p.tiles = LR * ((nlines + (1ll << logC) - 1) >> logC);
    p.do_scale = 0;
    p.scale = 1.0;
    ap.passes.push_back(ps);
    logNs += logR;
  }
  // buffers: ping-pong through scratch, last pass into the caller buffer
  bool in_user = true;
  for (int i = 0; i < P; ++i) {
    Pass& ps = ap.passes[i];
    ps.in_user = in_user ? 1 : 0;
    if (i == P - 1) ps.out_user = 1;
    else ps.out_user = in_user ? 0 : 1;
    in_user = ps.out_user;
  }
  if (P > 1) {
    // the scratch mirrors the caller layout
    if (s == 1) ap.scratch_elems = (size_t)((nlines - 1) * lstride + L);
    else ap.scratch_elems = (size_t)(nlines * L);
  }
  return ap;
}

int launch_pass(Form f, int sign, IOType in, IOType out, const PassParams& p, int threads) {
  cudaError_t e;
  const double pts = (double)p.L * (double)p.nlines;
  ProfScope ps(PK_PASS, pts * (double)(io_bytes(in) + io_bytes(out)), 5.0 * pts * p.logR);
  if (p.cluster) e = launch_pass_cl_f32(sign, in, out, p, threads, g.cur);
  else if (p.lat) e = launch_pass_lat(f, sign, in, out, p, g.cur);
  else if (f == FORM_F64) e = launch_pass_f64(sign, in, out, p, threads, g.cur);
  else if (f == FORM_F32) e = launch_pass_f32(sign, in, out, p, threads, g.cur);
  else if (f == FORM_TC32) e = launch_pass_tc32(sign, in, out, p, threads, g.cur);
  else e = launch_pass_df64(sign, in, out, p, threads, g.cur);
  g.launches++;
  if (e != cudaSuccess)
    return fail(GBFFT_CUDA_ERROR, "pass launch (L=%lld R=2^%d): %s", p.L, p.logR,
                cudaGetErrorString(e));
  return GBFFT_OK;
}

// Run an axis plan on `data` (interleaved double complex, device memory).
// spec/spec_kind: optional spectrum epilogue of the last pass (see PassParams).
// Work riding on an axis plan's first or last pass.
struct AxisExtras {
  double* spec = nullptr;  // spectrum epilogue of the last pass (PassParams)
  int spec_kind = 0;
  int twist = 0;           // real-transform twist (PassParams::twist): > 0 on
                           // the last pass, < 0 on the first
  int logU = 0, logV = 0;  // rlft3: the pass's line grid
  double* aux = nullptr;   // rlft3: speq
};

// twist: realft twist fused into the last (+1) or first (-1) pass.
// ext_scratch: scratch supplied by the caller (at least 16 bytes per complex
// element of the axis' span) instead of the library's device scratch.
// ex: the extras as one record (replaces spec, spec_kind and twist).
int run_axis(Form f, int sign, const AxisPlan& ap, void* data, double scale = 1.0,
             double* spec = nullptr, int spec_kind = 0, int twist = 0,
             void* ext_scratch = nullptr, const AxisExtras* ex = nullptr) {
  AxisExtras local;
  if (!ex) {
    local.spec = spec;
    local.spec_kind = spec_kind;
    local.twist = twist;
    ex = &local;
  }
  Twiddles tw;
  TRY(tables(f, tw));
  top_table(f, plan_top_log(ap), tw);
  const IOType sio = scratch_io(f);
  const size_t P = ap.passes.size();
  // With FP32 scratch (half the size of the caller's f64 data) a plan of three
  // or more passes ping-pongs between two scratch halves, so that only the
  // first pass reads and only the last pass writes the caller's array.
  const bool two = sio == IO_F2 && P >= 3;
  const size_t half = ap.scratch_elems * io_bytes(sio);
  void* sb = ext_scratch;
  if (!sb) {
    if (ap.scratch_elems) TRY(ensure(g.scratch, half * (two ? 2 : 1)));
    sb = g.scratch.p;
  }
  void* sbuf[2] = {sb, two ? (void*)((char*)sb + half) : sb};
  for (size_t i = 0; i < P; ++i) {
    const Pass& ps = ap.passes[i];
    const bool first = i == 0, last = i + 1 == P;
    PassParams p = ps.p;
    p.tw = tw;
    IOType in_t, out_t;
    if (two) {
      p.in = first ? data : sbuf[(i - 1) & 1];
      p.out = last ? data : sbuf[i & 1];
      in_t = first ? IO_D2 : sio;
      out_t = last ? IO_D2 : sio;
    } else {
      p.in = ps.in_user ? data : sb;
      p.out = ps.out_user ? data : sb;
      in_t = ps.in_user ? IO_D2 : sio;
      out_t = ps.out_user ? IO_D2 : sio;
    }
    if (last && scale != 1.0) {
      p.do_scale = 1;
      p.scale = scale;
    }
    if (last && ex->spec_kind) {
      p.spec = ex->spec;
      p.spec_kind = ex->spec_kind;
    }
    if ((ex->twist > 0 && last) || (ex->twist < 0 && first)) {
      p.twist = ex->twist;
      p.mirror_logU = ex->logU;
      p.mirror_logV = ex->logV;
      p.aux = ex->aux;
    }
    TRY(launch_pass(f, sign, in_t, out_t, p, ps.threads));
  }
  return GBFFT_OK;
}

// Whether the realft twist can ride on the plan's last (twist > 0) or first
// (twist < 0) pass: a multi-pass plan's mirror tiles need at least two
// columns; a single-pass plan's tiles hold whole lines.
bool twist_fits(const AxisPlan& ap, int twist) {
  if (ap.passes.empty()) return false;
  const PassParams& p = (twist > 0 ? ap.passes.back() : ap.passes.front()).p;
  if (p.s != 1 || p.cluster || p.lat) return false;
  if (p.mode == 0) return p.logC >= 1 && (p.L >> p.logR) >= (1ll << p.logC);
  return ap.passes.size() == 1;
}

// Out-of-place run of a plan: the first pass reads `in` (or the per-line
// pointers `in_lines`, a device array), the last pass writes `out`; the passes
// between ping-pong through device scratch (two halves for three or more
// passes).  `in` and `out` may be host memory when g.host_direct is set: the
// link traffic then overlaps the first and last passes' arithmetic instead of
// preceding and following the transform as staging copies.
int run_axis_io(Form f, int sign, const AxisPlan& ap, const void* in,
                const void* const* in_lines, void* out, double* spec = nullptr,
                int spec_kind = 0) {
  Twiddles tw;
  TRY(tables(f, tw));
  top_table(f, plan_top_log(ap), tw);
  const IOType sio = scratch_io(f);
  const size_t P = ap.passes.size();
  const size_t half = ap.scratch_elems * io_bytes(sio);
  if (P >= 2) TRY(ensure(g.scratch, half * (P >= 3 ? 2 : 1)));
  void* sbuf[2] = {g.scratch.p, P >= 3 ? (void*)((char*)g.scratch.p + half) : g.scratch.p};
  for (size_t i = 0; i < P; ++i) {
    PassParams p = ap.passes[i].p;
    p.tw = tw;
    const bool first = i == 0, last = i + 1 == P;
    p.in = first ? in : sbuf[(i - 1) & 1];
    p.in_ptrs = first ? in_lines : nullptr;
    p.out = last ? out : sbuf[i & 1];
    if (last && spec_kind) {
      p.spec = spec;
      p.spec_kind = spec_kind;
    }
    TRY(launch_pass(f, sign, first ? IO_D2 : sio, last ? IO_D2 : sio, p, ap.passes[i].threads));
  }
  return GBFFT_OK;
}

// Plan cache keyed by (L, s, nlines, lq_log, lstride, tile size).
std::map<std::tuple<long long, long long, long long, int, long long, int>, AxisPlan> g_plans;

// Autotuner: the tile size of each (axis shape, form), chosen by timing the
// candidates 2^12, 2^11 and 2^10 elements per CTA on a zeroed scratch array
// the first time the shape is planned.  Results can be kept in a file
// (GBFFT_TUNE_CACHE), one line "L s nlines lq_log lstride form tileLog".
using TuneKey = std::tuple<long long, long long, long long, int, long long, int>;
std::map<TuneKey, int> g_tuned;
bool g_tune_loaded = false;

void tune_load() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  if (g.tune_cache.empty()) return;
  FILE* fp = fopen(g.tune_cache.c_str(), "r");
  if (!fp) return;
  long long L, s, nl, ls;
  int lq, f, tl;
  char line[8192];
  while (fgets(line, sizeof line, fp)) {
    // tile lines; the batch tuner's lines start with "batch"
    if (sscanf(line, "%lld %lld %lld %d %lld %d %d", &L, &s, &nl, &lq, &ls, &f, &tl) == 7)
      g_tuned[std::make_tuple(L, s, nl, lq, ls, f)] = tl;
  }
  fclose(fp);
}

int tune_tile(Form f, long long L, long long s, long long nlines, int lq_log, long long lstride) {
  const size_t span = (s == 1) ? (size_t)((nlines - 1) * lstride + L) : (size_t)(nlines * L);
  if (span * 16 > (size_t(512) << 20) || L <= 64) return 12;
  void* tmp = nullptr;
  if (dev_alloc(&tmp, span * 16) != cudaSuccess) return 12;
  cudaMemsetAsync(tmp, 0, span * 16, g.cur);
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  int best_tl = 12;
  const bool prof = g.profiling;
  g.profiling = false;
  for (int tl = 12; tl >= 10; --tl) {
    AxisPlan ap = make_axis_plan(L, s, nlines, lq_log, lstride, false, tl);
    if (run_axis(f, 1, ap, tmp, 1.0) != GBFFT_OK) continue;
    cudaEventRecord(a, g.cur);
    for (int r = 0; r < 3; ++r) run_axis(f, 1, ap, tmp, 1.0);
    cudaEventRecord(b, g.cur);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (g.tune_verbose)
      fprintf(stderr, "gbfft tune L=%lld s=%lld lines=%lld form=%d tile=2^%d: %.4f ms\n", L, s,
              nlines, (int)f, tl, ms / 3);
    if (ms < best * 0.97f) {  // prefer the larger tile unless clearly slower
      best = ms;
      best_tl = tl;
    }
  }
  g.profiling = prof;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(tmp);
  cudaGetLastError();
  return best_tl;
}

// FP32 two-pass schedule of a long unit-stride axis: radices 2^ceil(logL/2)
// and 2^floor(logL/2), each pass on four-CTA clusters of four columns
// (k_pass_cl).  FP32 scratch between the passes mirrors the caller layout.
constexpr int kClusterMinLog = 22;  // radix >= 2^11: at least 128 threads per CTA
constexpr int kClusterTile = 99;    // plan-cache key of these plans
bool cluster_fits(Form f, long long L, long long s, int lq_log) {
  if (!g.cluster_pass || f != FORM_F32 || s != 1 || lq_log != 0) return false;
  const int logL = ilog2((unsigned long long)L);
  return logL >= kClusterMinLog && logL <= 2 * 14;
}

AxisPlan make_cluster_plan(long long L, long long nlines, long long lstride) {
  AxisPlan ap;
  const int logL = ilog2((unsigned long long)L);
  const int radix[2] = {(logL + 1) / 2, logL / 2};
  int logNs = 0;
  for (int i = 0; i < 2; ++i) {
    Pass ps;
    PassParams& p = ps.p;
    std::memset(&p, 0, sizeof p);
    const int logR = radix[i];
    p.L = L;
    p.s = 1;
    p.lstride = lstride;
    p.nlines = nlines;
    p.lq_log = 0;
    p.logL = logL;
    p.logR = logR;
    p.logNs = logNs;
    p.Ns = 1ll << logNs;
    p.mode = 0;
    p.logC = 2;
    p.in_rcontig = 0;
    p.out_rcontig = (logNs == 0) ? 1 : 0;
    split_subpasses(logR - 2, p);  // the M = R/4-point DFTs of each CTA
    p.tiles = nlines * ((L >> logR) >> 2);
    p.scale = 1.0;
    p.cluster = 1;
    ps.threads = (1 << logR) / 16;
    ps.in_user = (i == 0) ? 1 : 0;
    ps.out_user = (i == 1) ? 1 : 0;
    ap.passes.push_back(ps);
    logNs += logR;
  }
  ap.scratch_elems = (size_t)((nlines - 1) * lstride + L);
  return ap;
}

const AxisPlan& axis_plan(long long L, long long s, long long nlines, int lq_log,
                          long long lstride, Form f = FORM_F64) {
  if (cluster_fits(f, L, s, lq_log)) {
    auto key = std::make_tuple(L, s, nlines, lq_log, lstride, kClusterTile);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) return it->second;
    return g_plans.emplace(key, make_cluster_plan(L, nlines, lstride)).first->second;
  }
  int tl = 12;
  if (g.autotune) {
    tune_load();
    const TuneKey tk = std::make_tuple(L, s, nlines, lq_log, lstride, (int)f);
    auto t = g_tuned.find(tk);
    if (t != g_tuned.end()) {
      tl = t->second;
    } else {
      tl = tune_tile(f, L, s, nlines, lq_log, lstride);
      g_tuned[tk] = tl;
      if (!g.tune_cache.empty()) {
        FILE* fp = fopen(g.tune_cache.c_str(), "a");
        if (fp) {
          fprintf(fp, "%lld %lld %lld %d %lld %d %d\n", L, s, nlines, lq_log, lstride, (int)f, tl);
          fclose(fp);
        }
      }
    }
  }
  auto key = std::make_tuple(L, s, nlines, lq_log, lstride, tl);
  auto it = g_plans.find(key);
  if (it != g_plans.end()) return it->second;
  return g_plans.emplace(key, make_axis_plan(L, s, nlines, lq_log, lstride, false, tl))
      .first->second;
}

// Contiguous batch of 1-D complex transforms: nlines lines `dist` complex apart.
int fft_lines(Form f, int sign, void* data, long long L, long long nlines, long long dist,
              double scale = 1.0) {
  if (L == 1) {
    if (scale != 1.0) {
      // scaling of a 1-point transform: every line holds one complex value
      for (long long l = 0; l < nlines; ++l) {
        CK(launch_scale((double*)data + 2 * l * dist, 2, scale, g.cur));
        g.launches++;
      }
    }
    return GBFFT_OK;
  }
  return run_axis(f, sign, axis_plan(L, 1, nlines, 0, dist, f), data, scale);
}

struct Call {
  const gbfft_opts* o;
  gbfft_opts def;
  explicit Call(const gbfft_opts* opts) {
    std::memset(&def, 0, sizeof def);
    o = opts ? opts : &def;
  }
  Form form() const { return (Form)o->form; }
  bool dev() const { return o->device_ptrs != 0; }
};

int check_form(const Call& c) {
  if (c.o->form < 0 || c.o->form >= kForms) return fail(GBFFT_INVALID_ARG, "unknown form %d", c.o->form);
  return GBFFT_OK;
}

// Stream handling: a device-pointer call runs on the caller's stream (NULL is
// the default stream, so the call is ordered after earlier default-stream
// work); host-pointer calls run on the library stream.
// Calls on a stream that is capturing a CUDA graph neither wait on nor record
// the ordering event: an event recorded outside a capture cannot be waited on
// inside it, and the graph itself orders what it captures.
// Makes the library's device current for the duration of a call and puts the
// caller's back afterwards.
struct DeviceGuard {
  int prev = -1;
  DeviceGuard() {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != g.device) cudaSetDevice(g.device);
  }
  ~DeviceGuard() {
    if (prev >= 0 && prev != g.device) cudaSetDevice(prev);
  }
};

struct StreamScope {
  DeviceGuard dg;
  bool capturing = false;
  explicit StreamScope(const Call& c) {
    g.cur = c.dev() ? (cudaStream_t)c.o->stream : g.stream;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (c.dev() && cudaStreamIsCapturing(g.cur, &cs) == cudaSuccess)
      capturing = cs != cudaStreamCaptureStatusNone;
    if (!capturing && g.order_pending && g.order_stream != g.cur)
      cudaStreamWaitEvent(g.cur, g.order_ev, 0);
  }
  int finish(const Call& c) {
    if (capturing) {
      CK(cudaGetLastError());
      g.cur = g.stream;
      return GBFFT_OK;
    }
    if (!c.dev() || !c.o->async) {
      CK(cudaStreamSynchronize(g.cur));
      g.order_pending = false;
    } else {
      CK(cudaEventRecord(g.order_ev, g.cur));
      g.order_stream = g.cur;
      g.order_pending = true;
    }
    CK(cudaGetLastError());
    g.cur = g.stream;
    return GBFFT_OK;
  }
};

int h2d(void* dst, const void* src, size_t bytes) {
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g.cur));
  return GBFFT_OK;
}
int d2h(void* dst, const void* src, size_t bytes) {
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g.cur));
  return GBFFT_OK;
}
int d2d(void* dst, const void* src, size_t bytes) {
  if (dst == src || bytes == 0) return GBFFT_OK;
  CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, g.cur));
  return GBFFT_OK;
}

// Device view of an in/out array: the caller's pointer, or a staged copy.
int stage_inout(const Call& c, DevBuf& buf, double* user, size_t doubles, double** dptr,
                bool copy_in = true) {
  if (c.dev()) {
    *dptr = user;
    return GBFFT_OK;
  }
  TRY(ensure(buf, doubles * sizeof(double)));
  *dptr = (double*)buf.p;
  if (copy_in) TRY(h2d(buf.p, user, doubles * sizeof(double)));
  return GBFFT_OK;
}
int unstage(const Call& c, double* user, const double* dptr, size_t doubles) {
  if (c.dev()) return GBFFT_OK;
  return d2h(user, dptr, doubles * sizeof(double));
}

int check_isign(int isign) {
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "isign must be 1 or -1, got %d", isign);
  return GBFFT_OK;
}

// The kernels move complex values as 16-byte vectors, so every array they
// touch in place must start on a 16-byte boundary.  Host arrays are staged
// through aligned device buffers when they are not (the direct host path is
// taken only for aligned arrays); device arrays must be aligned by the caller
// (cudaMalloc and torch allocations always are), and an unaligned one is
// rejected before any launch.
inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int dev_aligned(const Call& c, const char* fn, std::initializer_list<const void*> ptrs) {
  if (!c.dev()) return GBFFT_OK;
  for (const void* q : ptrs)
    if (q && !al16(q))
      return fail(GBFFT_INVALID_ARG, "%s: device arrays must start on a 16-byte boundary", fn);
  return GBFFT_OK;
}

// ---------------------------------------------------------------------------
// realft on device data (n reals, power of two >= 2), `batch` lines `dist`
// doubles apart.
// ---------------------------------------------------------------------------
int realft_dev(Form f, double* d, long long n, int isign, long long batch = 1,
               long long dist = 0) {
  if (dist == 0) dist = n;
  Twiddles tw;
  TRY(tables(f, tw));
  const long long nh = n / 2;
  if (nh >= 2 && g.fused_twist) {
    // the twist rides on the last pass of the forward FFT or the first pass
    // of the inverse one: no pass of its own over the data
    const AxisPlan& ap = axis_plan(nh, 1, batch, 0, dist / 2, f);
    if (twist_fits(ap, isign)) return run_axis(f, isign, ap, d, 1.0, nullptr, 0, isign);
  }
  if (isign == 1) {
    TRY(fft_lines(f, 1, d, nh, batch, dist / 2));
    {
      ProfScope ps(PK_TWIST, 2.0 * n * batch * 8);
      CK(launch_realft_twist(f, 1, d, n, batch, dist, tw, g.cur));
    }
    g.launches++;
  } else {
    {
      ProfScope ps(PK_TWIST, 2.0 * n * batch * 8);
      CK(launch_realft_twist(f, -1, d, n, batch, dist, tw, g.cur));
    }
    g.launches++;
    TRY(fft_lines(f, -1, d, nh, batch, dist / 2));
  }
  return GBFFT_OK;
}

// The plan of axis dd of an N-D array of dims nn (row-major, last axis
// contiguous).
const AxisPlan& nd_axis_plan(Form f, const long long* nn, int ndim, int dd) {
  long long total = 1, s = 1;
  for (int i = 0; i < ndim; ++i) total *= nn[i];
  for (int i = ndim - 1; i > dd; --i) s *= nn[i];
  const long long L = nn[dd], nl = total / L;
  if (s == 1) return axis_plan(L, 1, nl, 0, L, f);
  return axis_plan(L, s, nl, ilog2((unsigned long long)s), L * s, f);
}

// The plan for the rlft3 twist riding on a single-pass plan whose lines form
// a 2^logU x 2^logV grid: tiles of whole lines, C >= 2 columns and at most
// one grid row of them (the mirror-line tiling), at least one warp per tile.
// Returns false when the plan does not qualify.
bool rlft3_twist_plan(const AxisPlan& base, int logU, int logV, AxisPlan& out) {
  if (base.passes.size() != 1) return false;
  const PassParams& b = base.passes[0].p;
  if (b.mode != 1 || logU < 1 || b.nlines != (1ll << (logU + logV))) return false;
  const int logC = std::min(b.logC, logV);
  if (logC < 1 || b.logR + logC < 9) return false;
  out = base;
  Pass& ps = out.passes[0];
  ps.p.logC = logC;
  ps.threads = (1 << (b.logR + logC)) / 16;
  ps.p.tiles = (b.L >> b.logR) * (b.nlines >> logC);
  return true;
}

// fourn on device data.  ex (3-D only): the rlft3 twist on the last axis
// processed (axis 0, forward) or the first (the last axis, inverse), whose
// plan is twist_plan.
// axes: bit dd set = transform axis dd (default: every axis).
int fourn_dev(Form f, double* d, const long long* nn, int ndim, int isign,
              const AxisExtras* ex = nullptr, const AxisPlan* twist_plan = nullptr,
              unsigned long long axes = ~0ull) {
  for (int dd = ndim - 1; dd >= 0; --dd) {
    if (nn[dd] <= 1 || !((axes >> dd) & 1ull)) continue;
    const bool with = ex && ((ex->twist > 0 && dd == 0) || (ex->twist < 0 && dd == ndim - 1));
    TRY(run_axis(f, isign, with ? *twist_plan : nd_axis_plan(f, nn, ndim, dd), d, 1.0, nullptr, 0,
                 0, nullptr, with ? ex : nullptr));
  }
  return GBFFT_OK;
}

// Two real lines of n in `w` (2n doubles): forward FFT both, fused spectral
// step into line 0, inverse FFT of line 0.
int spectral_dev(Form f, int kind, double* w, long long n) {
  Twiddles tw;
  TRY(tables(f, tw));
  const long long nh = n / 2;
  TRY(fft_lines(f, 1, w, nh, 2, nh));
  {
    ProfScope ps(PK_SPECTRAL, 3.0 * n * 8);
    CK(launch_spectral_product(f, kind, w, w + n, w, n, tw, g.cur));
  }
  g.launches++;
  TRY(fft_lines(f, -1, w, nh, 1, nh));
  return GBFFT_OK;
}

// ---------------------------------------------------------------------------
// Persistent batched FFT (uneven sizes).  The plan of the most recent call is
// kept with an instantiated CUDA graph of [reset counters, persistent launch];
// an identical call (same sizes, pointers, form, direction) replays it.
// ---------------------------------------------------------------------------
constexpr int kBatchMaxLog = 20;   // two passes at most in the persistent queue

struct BatchPlan {
  std::vector<size_t> nn;
  std::vector<const void*> ptrs;
  int form = -1, sign = 0;
  DevBuf ptrtab, done, flags, scratch;
  BatchParams P;
  int grid = 0;
  bool prefetch = false;  // bulk-copy prefetching kernel
  bool umma = false;      // tensor-core form on tcgen05 (k_batch_umma)
  bool host = false;      // the arrays are host memory, accessed directly
  cudaGraphExec_t exec = nullptr;
  long long launches_per_call = 0;
  bool valid = false;
};
BatchPlan g_batch;

void batch_plan_free(BatchPlan& b) {
  if (b.exec || b.done.p) cudaDeviceSynchronize();  // an earlier replay may be in flight
  if (b.exec) cudaGraphExecDestroy(b.exec);
  b.exec = nullptr;
  for (DevBuf* d : {&b.ptrtab, &b.done, &b.flags, &b.scratch}) {
    if (d->p) cudaFree(d->p);
    d->p = nullptr;
    d->bytes = 0;
  }
  b.valid = false;
}

// Pass schedule of the persistent batch launch, chosen by the autotuner: per
// bin length above 4096 points, the log2 radix of the first of its two passes
// (absent: half the length, rounded up), and the resident CTAs per SM (0: the
// occupancy maximum).
struct BatchTune {
  std::map<long long, int> first_radix;
  int per = 0;
};

// The passes of a bin of length L under a tune record (nullptr: default).
std::vector<int> batch_radices(long long L, const BatchTune* tune) {
  const int logL = ilog2((unsigned long long)L);
  int first = -1;
  if (tune) {
    auto it = tune->first_radix.find(L);
    if (it != tune->first_radix.end()) first = it->second;
  }
  if (logL <= 12) return {logL};
  if (first < 0) first = std::min(12, std::max(logL - 12, (logL + 1) / 2 + g.dbg_first_radix_delta));
  return {first, logL - first};
}

int build_batch_plan(BatchPlan& b, Form f, int sign, double* const* dptrs, const size_t* nn,
                     size_t count, bool host_ptrs, const BatchTune* tune = nullptr) {
  batch_plan_free(b);
  b.nn.assign(nn, nn + count);
  b.ptrs.assign((const void* const*)dptrs, (const void* const*)dptrs + count);
  b.form = f;
  b.sign = sign;
  b.host = host_ptrs;
  std::vector<size_t> order(count);
  for (size_t i = 0; i < count; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t c) { return nn[a] > nn[c]; });
  std::vector<const void*> table(count);
  for (size_t i = 0; i < count; ++i) table[i] = dptrs[order[i]];
  TRY(ensure(b.ptrtab, count * sizeof(void*)));
  CK(cudaMemcpy(b.ptrtab.p, table.data(), count * sizeof(void*), cudaMemcpyHostToDevice));
  const void* const* dtab = (const void* const*)b.ptrtab.p;
  // bins
  struct Bin { long long L, count, first; };
  std::vector<Bin> bins;
  for (size_t i = 0; i < count;) {
    size_t j = i;
    while (j < count && nn[order[j]] == nn[order[i]]) ++j;
    bins.push_back({(long long)nn[order[i]], (long long)(j - i), (long long)i});
    i = j;
  }
  const IOType sio = scratch_io(f);
  size_t scratch_elems = 0;
  for (auto& bn : bins)
    if (bn.L > 1 && batch_radices(bn.L, tune).size() == 2) scratch_elems += (size_t)(bn.L * bn.count);
  if (scratch_elems) TRY(ensure(b.scratch, scratch_elems * io_bytes(sio)));
  Twiddles tw;
  TRY(tables(f, tw));
  std::vector<BatchRange> first_pass, single, second_pass;
  size_t soff = 0;
  for (auto& bn : bins) {
    if (bn.L == 1) continue;  // 1-point transforms are the identity
    const std::vector<int> rad = batch_radices(bn.L, tune);
    AxisPlan ap = make_axis_plan(bn.L, 1, bn.count, 0, bn.L, true, 12, &rad);
    if (ap.passes.size() == 1) {
      BatchRange r;
      std::memset(&r, 0, sizeof r);
      r.p = ap.passes[0].p;
      r.p.tw = tw;
      r.p.in_ptrs = (const void* const*)(dtab + bn.first);
      r.p.out_ptrs = (void* const*)(dtab + bn.first);
      r.kind = 0;
      r.first = bn.first;
      single.push_back(r);
    } else {
      char* sbase = (char*)b.scratch.p + soff * io_bytes(sio);
      soff += (size_t)(bn.L * bn.count);
      BatchRange r1, r2;
      std::memset(&r1, 0, sizeof r1);
      std::memset(&r2, 0, sizeof r2);
      r1.p = ap.passes[0].p;
      r1.p.tw = tw;
      r1.p.in_ptrs = (const void* const*)(dtab + bn.first);
      r1.p.out = sbase;
      r1.kind = 1;
      r1.first = bn.first;
      r2.p = ap.passes[1].p;
      r2.p.tw = tw;
      r2.p.in = sbase;
      r2.p.out_ptrs = (void* const*)(dtab + bn.first);
      r2.kind = 2;
      r2.first = bn.first;
      r2.need = (unsigned int)(r1.p.tiles / bn.count) + g.dbg_need_extra;
      first_pass.push_back(r1);
      second_pass.push_back(r2);
    }
  }
  std::vector<BatchRange> all;
  for (auto* v : {&first_pass, &single, &second_pass})
    for (auto& r : *v) all.push_back(r);
  // the persistent kernels run full 4096-element tiles on 256 threads
  for (auto& r : all) set_slot_offsets(r.p, 256);
  long long item = 0;
  for (auto& r : all) {
    r.item0 = item;
    item += r.p.tiles;
  }
  if (item > 0x7FFFFFFFll)
    return fail(GBFFT_UNSUPPORTED_SIZE, "batch: %lld tiles (at most 2^31 - 1)", item);
  if (all.size() > (size_t)kMaxBatchRanges)
    return fail(GBFFT_UNSUPPORTED_SIZE, "batch: %zu size ranges (at most %d)", all.size(),
                kMaxBatchRanges);
  TRY(ensure(b.done, std::max<size_t>(count, 1) * sizeof(unsigned int)));
  TRY(ensure(b.flags, 64));
  std::memset(&b.P, 0, sizeof b.P);
  for (size_t i = 0; i < all.size(); ++i) b.P.ranges[i] = all[i];
  b.P.nranges = (int)all.size();
  b.P.total = item;
  b.P.head = (unsigned long long*)b.flags.p;
  b.P.err = (int*)((char*)b.flags.p + 8);
  b.P.done = (unsigned int*)b.done.p;
  b.P.spin_limit = g.dbg_spin_limit ? g.dbg_spin_limit : (1u << 24);
  int dev_sms = 0;
  CK(cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, g.device));
  // The prefetching kernel (opt-in: GBFFT_BATCH_PREFETCH=1) needs 16-byte
  // aligned caller arrays for its bulk copies.  Measured on the 20,000-transform
  // batch it is slower than k_batch in every form (FP32 1.75 vs 1.37 ms): its
  // staging buffer costs a resident CTA per SM and the copies wait at barriers.
  bool aligned = true;
  for (size_t i = 0; i < count; ++i)
    if (((uintptr_t)dptrs[i]) & 15u) aligned = false;
  const char* pfenv = getenv("GBFFT_BATCH_PREFETCH");
  // (bulk copies are not used on host memory)
  b.prefetch = f != FORM_F64 && aligned && !host_ptrs && pfenv && pfenv[0] == '1';
  // the tensor-core form runs its radix-16 sub-passes on tcgen05 unless
  // GBFFT_TC_UMMA=0 selects the warp-level mma.sync kernel
  b.umma = f == FORM_TC32 && !b.prefetch && g.tc_umma;
  int per = b.prefetch ? batch_pf_blocks_per_sm(f, sign)
                       : (b.umma ? batch_blocks_per_sm_umma(sign) : batch_blocks_per_sm(f, sign));
  if (tune && tune->per > 0 && tune->per < per) per = tune->per;
  if (per < 1) per = 1;
  b.grid = (int)std::min<long long>((long long)dev_sms * per, std::max<long long>(item, 1));
  // capture [reset counters, persistent launch] on the library stream
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(g.stream, cudaStreamCaptureModeThreadLocal));
  cudaMemsetAsync(b.flags.p, 0, 16, g.stream);
  cudaMemsetAsync(b.done.p, 0, std::max<size_t>(count, 1) * sizeof(unsigned int), g.stream);
  cudaError_t le = cudaSuccess;
  if (item > 0)
    le = b.prefetch ? launch_batch_pf(f, sign, b.P, b.grid, g.stream)
                    : (b.umma ? launch_batch_umma(sign, b.P, b.grid, g.stream)
                              : launch_batch(f, sign, b.P, b.grid, g.stream));
  cudaError_t ce = cudaStreamEndCapture(g.stream, &graph);
  if (le != cudaSuccess || ce != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail(GBFFT_CUDA_ERROR, "batch graph capture: %s / %s", cudaGetErrorString(le),
                cudaGetErrorString(ce));
  }
  CK(cudaGraphInstantiate(&b.exec, graph, 0));
  cudaGraphDestroy(graph);
  b.launches_per_call = item > 0 ? 1 : 0;
  b.valid = true;
  return GBFFT_OK;
}

bool batch_plan_matches(const BatchPlan& b, Form f, int sign, double* const* dptrs,
                        const size_t* nn, size_t count, bool host_ptrs) {
  if (!b.valid || b.form != (int)f || b.sign != sign || b.nn.size() != count ||
      b.host != host_ptrs)
    return false;
  for (size_t i = 0; i < count; ++i)
    if (b.nn[i] != nn[i] || b.ptrs[i] != (const void*)dptrs[i]) return false;
  return true;
}

// ---------------------------------------------------------------------------
// Autotuner of the persistent batch launch (on when autotuning is: the
// GBFFT_AUTOTUNE=1 switch or gbfft_set_autotune).  For a batch signature (form,
// direction, the multiset of sizes) it times candidate schedules -- per size
// bin one pass or two passes with the first radix around half the length,
// and the resident CTAs per SM -- on a zeroed device copy of the batch (the
// caller's arrays are never touched), by coordinate descent from the default
// schedule: bins in decreasing order of work, then the grid.  Each candidate is
// one CUDA-graph replay timed with events (best of three after one warm-up).
// Results live for the process and, with GBFFT_TUNE_CACHE, in that file.
// ---------------------------------------------------------------------------
std::map<std::string, BatchTune> g_batch_tuned;
bool g_batch_tune_loaded = false;

std::string batch_signature(Form f, int sign, const size_t* nn, size_t count) {
  std::map<size_t, size_t> bins;
  for (size_t i = 0; i < count; ++i) bins[nn[i]]++;
  std::string k = std::to_string((int)f) + "," + std::to_string(sign);
  for (auto& b : bins) k += ";" + std::to_string(b.first) + "x" + std::to_string(b.second);
  return k;
}

std::string tune_str(const BatchTune& t) {
  std::string s = std::to_string(t.per);
  for (auto& fr : t.first_radix) s += " " + std::to_string(fr.first) + ":" + std::to_string(fr.second);
  return s;
}

void batch_tune_load() {
  if (g_batch_tune_loaded) return;
  g_batch_tune_loaded = true;
  if (g.tune_cache.empty()) return;
  FILE* fp = fopen(g.tune_cache.c_str(), "r");
  if (!fp) return;
  char line[8192];
  while (fgets(line, sizeof line, fp)) {
    // "batch <signature> <per> <L>:<first> ..."
    if (strncmp(line, "batch ", 6) != 0) continue;
    char sig[4096];
    int per = 0, n = 0;
    if (sscanf(line + 6, "%4095s %d%n", sig, &per, &n) != 2) continue;
    BatchTune t;
    t.per = per;
    const char* q = line + 6 + n;
    long long L;
    int fr, m;
    while (sscanf(q, " %lld:%d%n", &L, &fr, &m) == 2) {
      t.first_radix[L] = fr;
      q += m;
    }
    g_batch_tuned[sig] = t;
  }
  fclose(fp);
}

// Time one candidate schedule on the scratch arrays: best of three replays.
float time_batch(Form f, int sign, double* const* tp, const size_t* nn, size_t count,
                 const BatchTune& t, cudaEvent_t a, cudaEvent_t b) {
  BatchPlan bp;
  float best = 1e30f;
  if (build_batch_plan(bp, f, sign, tp, nn, count, false, &t) == GBFFT_OK) {
    cudaGraphLaunch(bp.exec, g.cur);
    for (int r = 0; r < 3; ++r) {
      cudaEventRecord(a, g.cur);
      cudaGraphLaunch(bp.exec, g.cur);
      cudaEventRecord(b, g.cur);
      cudaEventSynchronize(b);
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess && ms < best) best = ms;
    }
  }
  batch_plan_free(bp);
  cudaGetLastError();
  return best;
}

BatchTune tune_batch(Form f, int sign, const size_t* nn, size_t count) {
  BatchTune best;
  size_t total = 0;
  for (size_t i = 0; i < count; ++i) total += 2 * nn[i];
  void* buf = nullptr;
  if (total * sizeof(double) > (size_t(8) << 30) || dev_alloc(&buf, total * sizeof(double)) != cudaSuccess)
    return best;  // too large to copy for tuning: keep the default schedule
  cudaMemsetAsync(buf, 0, total * sizeof(double), g.cur);
  std::vector<double*> tp(count);
  size_t off = 0;
  for (size_t i = 0; i < count; ++i) {
    tp[i] = (double*)buf + off;
    off += 2 * nn[i];
  }
  const bool prof = g.profiling;
  g.profiling = false;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  // bins in decreasing order of work
  std::map<size_t, size_t> bins;
  for (size_t i = 0; i < count; ++i) bins[nn[i]]++;
  std::vector<std::pair<double, long long>> order;
  for (auto& bn : bins)
    if (bn.first > 1)
      order.push_back({-(double)bn.first * bn.second * ilog2(bn.first), (long long)bn.first});
  std::sort(order.begin(), order.end());
  float cur = time_batch(f, sign, tp.data(), nn, count, best, a, b);
  for (auto& o : order) {
    const long long L = o.second;
    const int logL = ilog2((unsigned long long)L);
    const int def = (logL + 1) / 2;
    // the persistent kernel's tiles are 4096 elements of one transform, so
    // bins of up to 4096 points take one pass; longer ones choose the split
    std::vector<int> cands;
    if (logL > 12)
      for (int r = (logL + 1) / 2 - 2; r <= (logL + 1) / 2 + 2; ++r)
        if (r >= logL - 12 && r <= 12) cands.push_back(r);
    if (cands.empty()) continue;
    int keep = def;
    for (int r : cands) {
      if (r == def) continue;
      BatchTune t = best;
      t.first_radix[L] = r;
      const float ms = time_batch(f, sign, tp.data(), nn, count, t, a, b);
      if (g.tune_verbose)
        fprintf(stderr, "gbfft batch tune L=%lld first=%d: %.4f ms (best %.4f)\n", L, r, ms, cur);
      if (ms < cur * 0.98f) {
        cur = ms;
        keep = r;
      }
    }
    best.first_radix[L] = keep;
  }
  const int occ = (f == FORM_TC32 && g.tc_umma) ? batch_blocks_per_sm_umma(sign)
                                                 : batch_blocks_per_sm(f, sign);
  for (int per = occ - 1; per >= 1 && per >= occ - 2; --per) {
    BatchTune t = best;
    t.per = per;
    const float ms = time_batch(f, sign, tp.data(), nn, count, t, a, b);
    if (g.tune_verbose)
      fprintf(stderr, "gbfft batch tune per=%d: %.4f ms (best %.4f)\n", per, ms, cur);
    if (ms < cur * 0.98f) {
      cur = ms;
      best.per = per;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  g.profiling = prof;
  cudaStreamSynchronize(g.cur);
  cudaFree(buf);
  cudaGetLastError();
  return best;
}

// The tune record of a batch signature when autotuning is on (tuning it on
// first sight), else nullptr.
const BatchTune* batch_tune_for(Form f, int sign, const size_t* nn, size_t count) {
  if (!g.autotune) return nullptr;
  batch_tune_load();
  const std::string sig = batch_signature(f, sign, nn, count);
  auto it = g_batch_tuned.find(sig);
  if (it != g_batch_tuned.end()) return &it->second;
  BatchTune t = tune_batch(f, sign, nn, count);
  auto ins = g_batch_tuned.emplace(sig, t).first;
  if (!g.tune_cache.empty()) {
    FILE* fp = fopen(g.tune_cache.c_str(), "a");
    if (fp) {
      fprintf(fp, "batch %s %s\n", sig.c_str(), tune_str(t).c_str());
      fclose(fp);
    }
  }
  return &ins->second;
}

// Transforms of at most 2^20 points go through the persistent launch; larger
// ones (rare in a batch) run their own pass schedule.
int run_batch_dev(Form f, int sign, double* const* dptrs, const size_t* nn, size_t count,
                  bool check_err, bool host_ptrs = false) {
  std::vector<double*> small_p, big_p;
  std::vector<size_t> small_n, big_n;
  for (size_t i = 0; i < count; ++i) {
    if (ilog2(nn[i]) <= kBatchMaxLog) { small_p.push_back(dptrs[i]); small_n.push_back(nn[i]); }
    else { big_p.push_back(dptrs[i]); big_n.push_back(nn[i]); }
  }
  if (!small_p.empty()) {
    if (!batch_plan_matches(g_batch, f, sign, small_p.data(), small_n.data(), small_p.size(),
                            host_ptrs)) {
      const BatchTune* tune = batch_tune_for(f, sign, small_n.data(), small_n.size());
      TRY(build_batch_plan(g_batch, f, sign, small_p.data(), small_n.data(), small_p.size(),
                           host_ptrs, tune));
    }
    {
      ProfScope ps(PK_PASS, 0.0);
      CK(cudaGraphLaunch(g_batch.exec, g.cur));
    }
    g.launches += g_batch.launches_per_call;
    if (check_err) {
      int err = 0;
      CK(cudaMemcpyAsync(&err, g_batch.P.err, sizeof(int), cudaMemcpyDeviceToHost, g.cur));
      CK(cudaStreamSynchronize(g.cur));
      if (err) return fail(GBFFT_TIMEOUT, "four1_batch: a bounded device wait gave up");
    }
  }
  for (size_t i = 0; i < big_p.size(); ++i)
    TRY(fft_lines(f, sign, big_p[i], (long long)big_n[i], 1, (long long)big_n[i]));
  return GBFFT_OK;
}

// convlv / correl with the caller's host arrays read and written by the
// kernels themselves (g.host_direct; n >= 4): the first forward pass reads data
// (and, for correl, data2) from the host, the last inverse pass writes ans.
int spectral_direct(Form f, int kind, const double* a, const double* b, long long n, long long m,
                    double* ans) {
  Twiddles tw;
  TRY(tables(f, tw));
  const long long nh = n / 2;
  TRY(ensure(g.work, 2 * (size_t)n * sizeof(double)));
  double* w = (double*)g.work.p;
  const void* lines[2];
  lines[0] = a;
  if (kind == 2) {
    lines[1] = b;
  } else {
    CK(launch_expand_response(b, m, w + n, n, nullptr, nullptr, g.cur));
    g.launches++;
    lines[1] = w + n;
  }
  TRY(ensure(g.ptrtab, 64));
  CK(launch_set_lines((const void**)g.ptrtab.p, lines[0], lines[1], g.cur));
  g.launches++;
  TRY(run_axis_io(f, 1, axis_plan(nh, 1, 2, 0, nh, f), nullptr, (const void* const*)g.ptrtab.p, w));
  {
    ProfScope ps(PK_SPECTRAL, 3.0 * n * 8);
    CK(launch_spectral_product(f, kind, w, w + n, w, n, tw, g.cur));
  }
  g.launches++;
  TRY(run_axis_io(f, -1, axis_plan(nh, 1, 1, 0, nh, f), w, nullptr, ans));
  return GBFFT_OK;
}

// Whether run_axis_io takes the plan of `nlines` lines of L points, with the
// first pass reading through a per-line pointer table (pass counts of one or
// two; the pointer-table layouts are used only by the convolution paths).
bool io_fits(long long L, long long nlines, Form f) {
  return L <= (1ll << kBatchMaxLog) && axis_plan(L, 1, nlines, 0, L, f).passes.size() <= 2;
}
// Whether a linear host array of `nlines` lines of L points can be read and
// written by the plan's first and last passes directly (any pass count).
bool direct_fits(long long L, long long nlines, Form f) {
  (void)L;
  (void)nlines;
  (void)f;
  return g.host_direct;
}

}  // namespace

void record_error(int code, const char* msg) {
  std::lock_guard<std::mutex> lk(g_mu);
  fail(code, "%s", msg);
}

}  // namespace gbfft

using namespace gbfft;

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int gbfft_init(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g.inited && device >= 0 && device != g.device)
    return fail(GBFFT_INVALID_ARG, "init: the library is bound to device %d already", g.device);
  return init_locked(device);
}

const char* gbfft_last_error(void) { return g.err.c_str(); }

int gbfft_version(void) { return 100; }

size_t gbfft_scratch_bytes(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g.scratch.bytes + g.work.bytes + g.stage_a.bytes + g.stage_b.bytes + g.stage_c.bytes;
}

int gbfft_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g.inited) return GBFFT_OK;
  DeviceGuard dg;
  cudaDeviceSynchronize();
  g.order_pending = false;
  for (DevBuf* b : {&g.scratch, &g.work, &g.stage_a, &g.stage_b, &g.stage_c, &g.ptrtab}) {
    if (b->p) cudaFree(b->p);
    b->p = nullptr;
    b->bytes = 0;
  }
  g_plans.clear();
  batch_plan_free(g_batch);
  // the dense copies of large twiddle levels are as large as the data they
  // served; they are rebuilt on the next transform that needs one
  for (auto& m : g.tw_top) {
    for (auto& kv : m) cudaFree(kv.second);
    m.clear();
  }
  return GBFFT_OK;
}

int gbfft_set_autotune(int enable) {
  std::lock_guard<std::mutex> lk(g_mu);
  TRY(init_locked(g.device));
  g.autotune = enable != 0;
  return GBFFT_OK;
}

int gbfft_profile(int enable) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g.inited) cudaDeviceSynchronize();
  for (auto& r : g.prof) {
    g.evpool.push_back(r.a);
    g.evpool.push_back(r.b);
  }
  g.prof.clear();
  g.profiling = enable != 0;
  return GBFFT_OK;
}

int gbfft_profile_read(int kind, double* ms, long long* launches, double* bytes,
                       double* flops) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (kind < 0 || kind >= PK_COUNT) return fail(GBFFT_INVALID_ARG, "profile kind %d", kind);
  double t = 0.0, by = 0.0, fl = 0.0;
  long long n = 0;
  for (auto& r : g.prof) {
    if (r.kind != kind) continue;
    CK(cudaEventSynchronize(r.b));
    float x = 0.f;
    CK(cudaEventElapsedTime(&x, r.a, r.b));
    t += x;
    by += r.bytes;
    fl += r.flops;
    ++n;
  }
  if (ms) *ms = t;
  if (launches) *launches = n;
  if (bytes) *bytes = by;
  if (flops) *flops = fl;
  return GBFFT_OK;
}

int gbfft_set_spectral_path(int path) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (path != 0 && path != 1) return fail(GBFFT_INVALID_ARG, "spectral path must be 0 or 1");
  g.spectral_path = path;
  return GBFFT_OK;
}

int gbfft_debug_set(int key, long long value) {
  std::lock_guard<std::mutex> lk(g_mu);
  switch (key) {
    case GBFFT_DEBUG_FAIL_ALLOC_AT:
      if (value < 0) return fail(GBFFT_INVALID_ARG, "debug_set: negative allocation index");
      g.fail_alloc_at = value;
      g.alloc_calls = 0;
      return GBFFT_OK;
    case GBFFT_DEBUG_FUSED_TWIST:
      g.fused_twist = value != 0;
      return GBFFT_OK;
    case GBFFT_DEBUG_TC_UMMA:
      g.tc_umma = value != 0;
      batch_plan_free(g_batch);
      return GBFFT_OK;
    case GBFFT_DEBUG_CLUSTER_PASS:
      g.cluster_pass = value != 0;
      return GBFFT_OK;
    case GBFFT_DEBUG_TOP_TWIDDLES:
      g.top_tables = value != 0;
      return GBFFT_OK;
    case GBFFT_DEBUG_BATCH_FIRST_RADIX_DELTA:
      if (value < -12 || value > 12) return fail(GBFFT_INVALID_ARG, "debug_set: value out of range");
      g.dbg_first_radix_delta = (int)value;
      batch_plan_free(g_batch);
      return GBFFT_OK;
    case GBFFT_DEBUG_BATCH_SPIN_LIMIT:
    case GBFFT_DEBUG_BATCH_NEED_EXTRA:
      if (value < 0 || value > 0xFFFFFFFFll) return fail(GBFFT_INVALID_ARG, "debug_set: value out of range");
      if (key == GBFFT_DEBUG_BATCH_SPIN_LIMIT) g.dbg_spin_limit = (unsigned int)value;
      else g.dbg_need_extra = (unsigned int)value;
      // the cached batch plan (and its graph) holds the old values
      batch_plan_free(g_batch);
      return GBFFT_OK;
    default:
      return fail(GBFFT_INVALID_ARG, "debug_set: unknown key %d", key);
  }
}

long long gbfft_launch_count(int reset) {
  std::lock_guard<std::mutex> lk(g_mu);
  long long v = g.launches;
  if (reset) g.launches = 0;
  return v;
}

int gbfft_four1(double* data, size_t nn, int isign, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!data) return fail(GBFFT_INVALID_ARG, "four1: null data");
  TRY(dev_aligned(c, "four1", {data}));
  TRY(check_isign(isign));
  if (!is_pow2(nn) || ilog2(nn) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "four1: nn=%zu must be a power of two <= 2^%d", nn, kMaxAxisLog);
  TRY(init_locked(g.device));
  StreamScope ss(c);
  if (!c.dev() && nn > 1 && al16(data) && direct_fits((long long)nn, 1, c.form())) {
    // the first pass reads the caller's array, the last pass writes it back
    TRY(run_axis_io(c.form(), isign, axis_plan((long long)nn, 1, 1, 0, (long long)nn, c.form()), data,
                    nullptr, data));
    return ss.finish(c);
  }
  double* d;
  TRY(stage_inout(c, g.stage_a, data, 2 * nn, &d));
  TRY(fft_lines(c.form(), isign, d, (long long)nn, 1, (long long)nn));
  TRY(unstage(c, data, d, 2 * nn));
  return ss.finish(c);
}

// FFTProcessor::fft followed by magnitude_spectrum / power_spectrum
// (src/FFT_1.rs:166,206,218) with the spectrum written by the transform's
// last pass, from the values it stores: no separate pass over the spectrum.
int gbfft_four1_spectrum(double* data, size_t nn, int isign, int kind, double* spec,
                         const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!data || !spec) return fail(GBFFT_INVALID_ARG, "four1_spectrum: null pointer");
  TRY(dev_aligned(c, "four1_spectrum", {data}));
  TRY(check_isign(isign));
  if (kind != 0 && kind != 1)
    return fail(GBFFT_INVALID_ARG, "four1_spectrum: kind must be 0 (magnitude) or 1 (power)");
  if (!is_pow2(nn) || ilog2(nn) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "four1_spectrum: nn=%zu must be a power of two <= 2^%d",
                nn, kMaxAxisLog);
  TRY(init_locked(g.device));
  StreamScope ss(c);
  const int sk = kind == 0 ? 1 : 2;
  const Form f = c.form();
  if (!c.dev() && nn > 1 && al16(data) && direct_fits((long long)nn, 1, f)) {
    // the first pass reads the caller's array, the last pass writes it and
    // the spectrum straight into host memory
    TRY(run_axis_io(f, isign, axis_plan((long long)nn, 1, 1, 0, (long long)nn, f), data, nullptr,
                    data, spec, sk));
    return ss.finish(c);
  }
  double* d;
  TRY(stage_inout(c, g.stage_a, data, 2 * nn, &d));
  double* sp = spec;
  if (!c.dev()) {
    TRY(ensure(g.stage_b, nn * sizeof(double)));
    sp = (double*)g.stage_b.p;
  }
  if (nn == 1) {
    // the 1-point transform is the identity
    CK(launch_spectrum(kind, d, sp, 1, g.cur));
    g.launches++;
  } else {
    TRY(run_axis(f, isign, axis_plan((long long)nn, 1, 1, 0, (long long)nn, f), d, 1.0, sp, sk));
  }
  TRY(unstage(c, data, d, 2 * nn));
  if (!c.dev()) TRY(d2h(spec, sp, nn * sizeof(double)));
  return ss.finish(c);
}

int gbfft_four1_many(double* data, size_t nn, size_t count, size_t dist, int isign,
                     const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!data && count) return fail(GBFFT_INVALID_ARG, "four1_many: null data");
  TRY(dev_aligned(c, "four1_many", {data}));
  TRY(check_isign(isign));
  if (!is_pow2(nn) || ilog2(nn) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "four1_many: nn=%zu must be a power of two", nn);
  if (dist < 2 * nn || (dist & 1)) return fail(GBFFT_INVALID_ARG, "four1_many: dist=%zu < 2*nn or odd", dist);
  if (count == 0) return GBFFT_OK;
  TRY(init_locked(g.device));
  StreamScope ss(c);
  double* d;
  size_t span = (count - 1) * dist + 2 * nn;
  TRY(stage_inout(c, g.stage_a, data, span, &d));
  TRY(fft_lines(c.form(), isign, d, (long long)nn, (long long)count, (long long)(dist / 2)));
  TRY(unstage(c, data, d, span));
  return ss.finish(c);
}

int gbfft_four1_batch(double* const* ptrs, const size_t* nn, size_t count, int isign,
                      const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  TRY(check_isign(isign));
  if (count == 0) return GBFFT_OK;
  if (!ptrs || !nn) return fail(GBFFT_INVALID_ARG, "four1_batch: null arrays");
  for (size_t t = 0; t < count; ++t) {
    if (!ptrs[t]) return fail(GBFFT_INVALID_ARG, "four1_batch: null pointer at %zu", t);
    TRY(dev_aligned(c, "four1_batch", {ptrs[t]}));
    if (!is_pow2(nn[t]) || ilog2(nn[t]) > kMaxAxisLog)
      return fail(GBFFT_UNSUPPORTED_SIZE, "four1_batch: nn[%zu]=%zu", t, nn[t]);
  }
  TRY(init_locked(g.device));
  StreamScope ss(c);
  const bool check = !c.dev() || !c.o->async;
  if (c.dev()) {
    TRY(run_batch_dev(c.form(), isign, ptrs, nn, count, check));
    return ss.finish(c);
  }
  // Host arrays.  When the GPU reaches pageable host memory directly and every
  // array is 16-byte aligned (and fits the persistent launch), the batched
  // kernel reads and writes the caller's arrays in place: no staging copies.
  bool direct = g.host_direct;
  for (size_t t = 0; direct && t < count; ++t)
    if (!al16(ptrs[t]) || ilog2(nn[t]) > kBatchMaxLog) direct = false;
  if (direct) {
    TRY(run_batch_dev(c.form(), isign, ptrs, nn, count, true, true));
    return ss.finish(c);
  }
  // otherwise: pack into one staging buffer (one copy each way)
  size_t total = 0;
  for (size_t t = 0; t < count; ++t) total += 2 * nn[t];
  TRY(ensure(g.stage_b, total * sizeof(double)));
  double* packed = (double*)g.stage_b.p;
  g.host_pack.resize(total * sizeof(double));
  double* hp = (double*)g.host_pack.data();
  std::vector<double*> dp(count);
  size_t off = 0;
  for (size_t t = 0; t < count; ++t) {
    std::memcpy(hp + off, ptrs[t], 2 * nn[t] * sizeof(double));
    dp[t] = packed + off;
    off += 2 * nn[t];
  }
  TRY(h2d(packed, hp, total * sizeof(double)));
  TRY(run_batch_dev(c.form(), isign, dp.data(), nn, count, check));
  TRY(d2h(hp, packed, total * sizeof(double)));
  CK(cudaStreamSynchronize(g.cur));
  off = 0;
  for (size_t t = 0; t < count; ++t) {
    std::memcpy(ptrs[t], hp + off, 2 * nn[t] * sizeof(double));
    off += 2 * nn[t];
  }
  return ss.finish(c);
}

int gbfft_twofft(const double* data1, const double* data2, double* fft1, double* fft2,
                 size_t n, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!data1 || !data2 || !fft1 || !fft2) return fail(GBFFT_INVALID_ARG, "twofft: null pointer");
  TRY(dev_aligned(c, "twofft", {fft1, fft2}));
  if (!is_pow2(n) || ilog2(n) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "twofft: n=%zu must be a power of two", n);
  TRY(init_locked(g.device));
  StreamScope ss(c);
  const double *d1 = data1, *d2p = data2;
  double *f1, *f2;
  if (!c.dev()) {
    TRY(ensure(g.stage_a, 2 * n * sizeof(double)));
    TRY(ensure(g.stage_b, 2 * n * sizeof(double)));
    TRY(ensure(g.stage_c, 2 * n * sizeof(double)));
    double* in = (double*)g.stage_c.p;
    TRY(h2d(in, data1, n * sizeof(double)));
    TRY(h2d(in + n, data2, n * sizeof(double)));
    d1 = in;
    d2p = in + n;
    f1 = (double*)g.stage_a.p;
    f2 = (double*)g.stage_b.p;
  } else {
    f1 = fft1;
    f2 = fft2;
  }
  CK(launch_twofft_pack(d1, d2p, f1, (long long)n, g.cur));
  g.launches++;
  TRY(fft_lines(c.form(), 1, f1, (long long)n, 1, (long long)n));
  CK(launch_twofft_split(f1, f2, (long long)n, g.cur));
  g.launches++;
  if (!c.dev()) {
    TRY(d2h(fft1, f1, 2 * n * sizeof(double)));
    TRY(d2h(fft2, f2, 2 * n * sizeof(double)));
  }
  return ss.finish(c);
}

int gbfft_realft(double* data, size_t n, int isign, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!data) return fail(GBFFT_INVALID_ARG, "realft: null data");
  TRY(dev_aligned(c, "realft", {data}));
  TRY(check_isign(isign));
  if (n < 2 || !is_pow2(n) || ilog2(n) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "realft: n=%zu must be a power of two >= 2", n);
  TRY(init_locked(g.device));
  StreamScope ss(c);
  double* d;
  TRY(stage_inout(c, g.stage_a, data, n, &d));
  TRY(realft_dev(c.form(), d, (long long)n, isign));
  TRY(unstage(c, data, d, n));
  return ss.finish(c);
}

int gbfft_fourn(double* data, const size_t* nn, size_t nn_len, size_t ndim, int isign,
                const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  // validate_inputs, src/Fourn.rs:367-378
  if (!nn || ndim == 0 || ndim > nn_len) return fail(GBFFT_INVALID_ARG, "fourn: invalid dimensions");
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "fourn: isign must be 1 or -1");
  for (size_t i = 0; i < ndim; ++i)
    if (nn[i] <= 1) return fail(GBFFT_INVALID_ARG, "fourn: invalid dimension size");
  if (!data) return fail(GBFFT_INVALID_ARG, "fourn: null data");
  TRY(dev_aligned(c, "fourn", {data}));
  long long dims[16];
  if (ndim > 16) return fail(GBFFT_UNSUPPORTED_SIZE, "fourn: ndim > 16");
  size_t total = 1;
  for (size_t i = 0; i < ndim; ++i) {
    if (!is_pow2(nn[i]) || ilog2(nn[i]) > kMaxAxisLog)
      return fail(GBFFT_UNSUPPORTED_SIZE, "fourn: nn[%zu]=%zu must be a power of two", i, nn[i]);
    dims[i] = (long long)nn[i];
    total *= nn[i];
  }
  TRY(init_locked(g.device));
  StreamScope ss(c);
  double* d;
  TRY(stage_inout(c, g.stage_a, data, 2 * total, &d));
  TRY(fourn_dev(c.form(), d, dims, (int)ndim, isign));
  TRY(unstage(c, data, d, 2 * total));
  return ss.finish(c);
}

// fourn along a subset of the axes: the local steps of an N-D transform split
// across ranks (slabs of axis 0 transform the other axes, exchange, then axis
// 0).  Every dimension a power of two >= 1; `axes` a non-empty bit set of
// axes below ndim.
int gbfft_fourn_axes(double* data, const size_t* nn, size_t ndim, unsigned long long axes,
                     int isign, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!nn || ndim == 0 || ndim > 16) return fail(GBFFT_INVALID_ARG, "fourn_axes: invalid dimensions");
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "fourn_axes: isign must be 1 or -1");
  if (axes == 0 || (ndim < 64 && (axes >> ndim) != 0))
    return fail(GBFFT_INVALID_ARG, "fourn_axes: axes must name axes below ndim");
  if (!data) return fail(GBFFT_INVALID_ARG, "fourn_axes: null data");
  TRY(dev_aligned(c, "fourn_axes", {data}));
  long long dims[16];
  size_t total = 1;
  for (size_t i = 0; i < ndim; ++i) {
    if (!is_pow2(nn[i]) || ilog2(nn[i]) > kMaxAxisLog)
      return fail(GBFFT_UNSUPPORTED_SIZE, "fourn_axes: nn[%zu]=%zu must be a power of two", i, nn[i]);
    dims[i] = (long long)nn[i];
    total *= nn[i];
  }
  TRY(init_locked(g.device));
  StreamScope ss(c);
  double* d;
  TRY(stage_inout(c, g.stage_a, data, 2 * total, &d));
  TRY(fourn_dev(c.form(), d, dims, (int)ndim, isign, nullptr, nullptr, axes));
  TRY(unstage(c, data, d, 2 * total));
  return ss.finish(c);
}

// FourFS::fourfs (src/Four_FS.rs:55-73), the crate's out-of-core N-D FFT,
// restated for a GPU that reaches host memory: the data stay in host memory
// (they may exceed the GPU's memory), and every pass of every axis reads and
// writes host memory directly over the CPU-GPU link, ping-ponging through a
// host work array; the GPU holds only its twiddle tables.
int gbfft_fourfs(double* data, const size_t* nn, size_t nn_len, size_t ndim, int isign,
                 double* work, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  // validate_inputs, src/Four_FS.rs:328-339
  if (!nn || ndim == 0 || ndim > nn_len) return fail(GBFFT_INVALID_ARG, "fourfs: invalid dimensions");
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "fourfs: isign must be 1 or -1");
  for (size_t i = 0; i < ndim; ++i)
    if (nn[i] <= 1) return fail(GBFFT_INVALID_ARG, "fourfs: invalid dimension size");
  if (!data) return fail(GBFFT_INVALID_ARG, "fourfs: null data");
  if (c.dev())
    return fail(GBFFT_INVALID_ARG, "fourfs: data must be host memory (gbfft_fourn takes device data)");
  if (!al16(data) || (work && !al16(work)))
    return fail(GBFFT_INVALID_ARG, "fourfs: data and work must start on a 16-byte boundary");
  long long dims[16];
  if (ndim > 16) return fail(GBFFT_UNSUPPORTED_SIZE, "fourfs: ndim > 16");
  size_t total = 1;
  for (size_t i = 0; i < ndim; ++i) {
    if (!is_pow2(nn[i]) || ilog2(nn[i]) > kMaxAxisLog)
      return fail(GBFFT_UNSUPPORTED_SIZE, "fourfs: nn[%zu]=%zu must be a power of two", i, nn[i]);
    dims[i] = (long long)nn[i];
    total *= nn[i];
  }
  TRY(init_locked(g.device));
  if (!g.host_direct)
    return fail(GBFFT_UNSUPPORTED_SIZE,
                "fourfs: this GPU does not reach pageable host memory directly (GBFFT_HOST_DIRECT=0 "
                "or no host page-table access)");
  StreamScope ss(c);
  // the host work array: the caller's, or one allocated for this call
  struct HostWork {
    void* p = nullptr;
    ~HostWork() {
      if (p) {
        cudaStreamSynchronize(g.cur);  // no pass may still read or write it
        std::free(p);
      }
    }
  } own;
  void* ws = work;
  if (!ws) {
    const size_t bytes = ((total * 16 + 4095) / 4096) * 4096;
    own.p = std::aligned_alloc(4096, bytes);
    if (!own.p) return fail(GBFFT_OOM, "fourfs: host work allocation (%zu bytes) failed", bytes);
    ws = own.p;
  }
  long long s = 1;
  for (int dd = (int)ndim - 1; dd >= 0; --dd) {
    const long long L = dims[dd];
    const long long nl = (long long)total / L;
    if (s == 1) TRY(run_axis(c.form(), isign, axis_plan(L, 1, nl, 0, L, c.form()), data, 1.0,
                             nullptr, 0, 0, ws));
    else TRY(run_axis(c.form(), isign, axis_plan(L, s, nl, ilog2((unsigned long long)s), L * s, c.form()),
                      data, 1.0, nullptr, 0, 0, ws));
    s *= L;
  }
  return ss.finish(c);
}

int gbfft_rlft3(double* data, double* speq, size_t nn1, size_t nn2, size_t nn3, int isign,
                const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (!data || !speq) return fail(GBFFT_INVALID_ARG, "rlft3: null pointer");
  TRY(dev_aligned(c, "rlft3", {data, speq}));
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "rlft3: isign must be 1 or -1");
  if (!is_pow2(nn1) || !is_pow2(nn2) || !is_pow2(nn3) || nn3 < 2 ||
      ilog2(nn1) > kMaxAxisLog || ilog2(nn2) > kMaxAxisLog || ilog2(nn3) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "rlft3: dims must be powers of two, nn3 >= 2");
  TRY(init_locked(g.device));
  StreamScope ss(c);
  Twiddles tw;
  TRY(tables(c.form(), tw));
  const size_t total = nn1 * nn2 * nn3;
  double *d, *sp;
  TRY(stage_inout(c, g.stage_a, data, total, &d));
  TRY(stage_inout(c, g.stage_b, speq, 2 * nn1 * nn2, &sp, isign == -1));
  long long dims[3] = {(long long)nn1, (long long)nn2, (long long)(nn3 / 2)};
  // The twist rides on the forward FFT's last pass (axis 0, whose lines form
  // the nn2 x nn3/2 grid) or the inverse FFT's first pass (the last axis,
  // lines on the nn1 x nn2 grid) when those are single passes; otherwise it
  // runs as its own kernels.
  AxisExtras ex;
  ex.twist = 2 * isign;
  ex.aux = sp;
  bool fused = nn1 >= 2 && nn2 >= 2 && nn3 >= 4;
  AxisPlan tplan;
  if (fused) {
    if (isign == 1) {
      ex.logU = ilog2(nn2);
      ex.logV = ilog2(nn3 / 2);
      fused = rlft3_twist_plan(nd_axis_plan(c.form(), dims, 3, 0), ex.logU, ex.logV, tplan);
    } else {
      ex.logU = ilog2(nn1);
      ex.logV = ilog2(nn2);
      fused = rlft3_twist_plan(nd_axis_plan(c.form(), dims, 3, 2), ex.logU, ex.logV, tplan);
    }
  }
  if (isign == 1) {
    if (fused) {
      TRY(fourn_dev(c.form(), d, dims, 3, 1, &ex, &tplan));
    } else {
      TRY(fourn_dev(c.form(), d, dims, 3, 1));
      CK(launch_rlft3_speq(d, sp, nn1, nn2, nn3, g.cur));
      g.launches++;
      CK(launch_rlft3_twist(c.form(), 1, d, sp, nn1, nn2, nn3, tw, g.cur));
      g.launches++;
    }
  } else {
    if (fused) {
      TRY(fourn_dev(c.form(), d, dims, 3, -1, &ex, &tplan));
    } else {
      CK(launch_rlft3_twist(c.form(), -1, d, sp, nn1, nn2, nn3, tw, g.cur));
      g.launches++;
      TRY(fourn_dev(c.form(), d, dims, 3, -1));
    }
  }
  TRY(unstage(c, data, d, total));
  TRY(unstage(c, speq, sp, 2 * nn1 * nn2));
  return ss.finish(c);
}

static int load_one(const Call& c, double* dst, const double* src, size_t doubles) {
  return c.dev() ? d2d(dst, src, doubles * sizeof(double)) : h2d(dst, src, doubles * sizeof(double));
}

// The twofft-packed form of convlv/correl (n >= 4): the inputs become the
// real and imaginary parts of one n-point complex FFT (the pack kernel reads
// the caller's arrays and expands the response), one kernel splits the two
// spectra, multiplies them and applies the inverse realft twist in place, and
// the inverse n/2-point FFT writes the answer.
static int spectral_twofft(const Call& c, int kind, const double* a, const double* b, size_t n,
                           size_t m, double* ans) {
  const Form f = c.form();
  Twiddles tw;
  TRY(tables(f, tw));
  TRY(ensure(g.work, 2 * n * sizeof(double)));
  double* z = (double*)g.work.p;
  const double *da = a, *db = b;
  const size_t mb = (kind == 2) ? n : m;  // doubles of the second input
  if (!c.dev() && !g.host_direct) {
    TRY(ensure(g.stage_c, (n + mb) * sizeof(double)));
    double* in = (double*)g.stage_c.p;
    TRY(h2d(in, a, n * sizeof(double)));
    TRY(h2d(in + n, b, mb * sizeof(double)));
    da = in;
    db = in + n;
  }
  // the packed imaginary part is scaled to the real part's magnitude (not for
  // deconvolution, whose |R|^2 threshold is absolute)
  double* sums = nullptr;
  if (kind != 1) {
    TRY(ensure(g.ptrtab, 64));
    sums = (double*)g.ptrtab.p;
  }
  CK(launch_pack_pair(da, db, kind == 2 ? 0 : (long long)m, z, (long long)n, sums, g.cur));
  g.launches += sums ? 2 : 1;
  TRY(run_axis(f, 1, axis_plan((long long)n, 1, 1, 0, (long long)n, f), z));
  {
    ProfScope ps(PK_SPECTRAL, 3.0 * n * 8);
    CK(launch_spectral_two(f, kind, z, (long long)n, tw, sums, g.cur));
  }
  g.launches++;
  const long long nh = (long long)n / 2;
  if (al16(ans) && (c.dev() || g.host_direct) && io_fits(nh, 1, f)) {
    TRY(run_axis_io(f, -1, axis_plan(nh, 1, 1, 0, nh, f), z, nullptr, ans));
    return GBFFT_OK;
  }
  TRY(run_axis(f, -1, axis_plan(nh, 1, 1, 0, nh, f), z));
  if (c.dev()) TRY(d2d(ans, z, n * sizeof(double)));
  else TRY(d2h(ans, z, n * sizeof(double)));
  return GBFFT_OK;
}

static int spectral_call(const Call& c, int kind, const double* a, const double* b, size_t n,
                         size_t m, double* ans) {
  TRY(init_locked(g.device));
  StreamScope ss(c);
  if (g.spectral_path == 1 && n >= 4 && !(kind == 2 && a == b)) {
    TRY(spectral_twofft(c, kind, a, b, n, m, ans));
    return ss.finish(c);
  }
  if (kind == 2 && a == b) {
    // autocorrelation (src/Correlation.rs:281-286): one forward transform, its
    // spectrum used as both operands of the conjugate product
    Twiddles tw;
    TRY(tables(c.form(), tw));
    TRY(ensure(g.work, n * sizeof(double)));
    double* w = (double*)g.work.p;
    TRY(load_one(c, w, a, n));
    const long long nh = (long long)n / 2;
    TRY(fft_lines(c.form(), 1, w, nh, 1, nh));
    {
      ProfScope ps(PK_SPECTRAL, 2.0 * n * 8);
      CK(launch_spectral_product(c.form(), 2, w, w, w, (long long)n, tw, g.cur));
    }
    g.launches++;
    TRY(fft_lines(c.form(), -1, w, nh, 1, nh));
    if (c.dev()) TRY(d2d(ans, w, n * sizeof(double)));
    else TRY(d2h(ans, w, n * sizeof(double)));
    return ss.finish(c);
  }
  // Direct path: the first forward pass reads the caller's inputs through a
  // pointer table and the last inverse pass writes the answer, with no copies
  // (host arrays when the GPU reaches host memory, device arrays always).  It
  // moves 16-byte vectors, so it needs aligned arrays.
  if (n >= 4 && al16(a) && al16(ans) && (kind != 2 || al16(b)) &&
      (c.dev() || g.host_direct) && io_fits((long long)n / 2, 2, c.form()) &&
      io_fits((long long)n / 2, 1, c.form())) {
    TRY(spectral_direct(c.form(), kind, a, b, (long long)n, (long long)m, ans));
    return ss.finish(c);
  }
  TRY(ensure(g.work, 2 * n * sizeof(double)));
  double* w = (double*)g.work.p;
  const double *da = a, *db = b;
  if (!c.dev()) {
    TRY(ensure(g.stage_c, (n + m) * sizeof(double)));
    double* in = (double*)g.stage_c.p;
    TRY(h2d(in, a, n * sizeof(double)));
    TRY(h2d(in + n, b, m * sizeof(double)));
    da = in;
    db = in + n;
  }
  if (kind == 2) {
    TRY(d2d(w, da, n * sizeof(double)));
    TRY(d2d(w + n, db, n * sizeof(double)));
  } else {
    CK(launch_expand_response(db, (long long)m, w + n, (long long)n, da, w, g.cur));
    g.launches++;
  }
  TRY(spectral_dev(c.form(), kind, w, (long long)n));
  if (c.dev()) TRY(d2d(ans, w, n * sizeof(double)));
  else TRY(d2h(ans, w, n * sizeof(double)));
  return ss.finish(c);
}

int gbfft_convlv(const double* data, size_t n, const double* respns, size_t m, int isign,
                 double* ans, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  // order of checks as src/Convolve.rs:13-21
  if (n == 0 || m == 0) return fail(GBFFT_EMPTY_INPUT, "convlv: input arrays cannot be empty");
  if (m > n) return fail(GBFFT_RESPONSE_TOO_LONG, "convlv: response function longer than data");
  if (isign != 1 && isign != -1)
    return fail(GBFFT_INVALID_ISIGN, "convlv: isign must be 1 (convolution) or -1 (deconvolution)");
  if (!data || !respns || !ans) return fail(GBFFT_INVALID_ARG, "convlv: null pointer");
  if (n < 2 || !is_pow2(n) || ilog2(n) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "convlv: n=%zu must be a power of two >= 2", n);
  return spectral_call(c, isign == 1 ? 0 : 1, data, respns, n, m, ans);
}

// The reference's direct linear branch for n <= 32 (src/Correlation.rs:19,37-50).
static int correl_small(const Call& c, const double* data1, const double* data2, size_t n,
                        double* ans) {
  const double *a = data1, *b = data2;
  double* out = ans;
  if (!c.dev()) {
    TRY(ensure(g.stage_c, 3 * n * sizeof(double)));
    double* in = (double*)g.stage_c.p;
    TRY(h2d(in, data1, n * sizeof(double)));
    TRY(h2d(in + n, data2, n * sizeof(double)));
    a = in;
    b = in + n;
    out = in + 2 * n;
  }
  CK(launch_correl_direct(a, b, out, (long long)n, g.cur));
  g.launches++;
  if (!c.dev()) TRY(d2h(ans, out, n * sizeof(double)));
  return GBFFT_OK;
}

int gbfft_correl(const double* data1, size_t n1, const double* data2, size_t n2, double* ans,
                 const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (n1 == 0) return fail(GBFFT_EMPTY_INPUT, "correl: input arrays cannot be empty");
  if (n2 != n1) return fail(GBFFT_LENGTH_MISMATCH, "correl: input arrays must have the same length");
  if (!data1 || !data2 || !ans) return fail(GBFFT_INVALID_ARG, "correl: null pointer");
  const size_t n = n1;
  if (n <= 32) {
    TRY(init_locked(g.device));
    StreamScope ss(c);
    TRY(correl_small(c, data1, data2, n, ans));
    return ss.finish(c);
  }
  if (!is_pow2(n) || ilog2(n) > kMaxAxisLog)
    return fail(GBFFT_UNSUPPORTED_SIZE, "correl: n=%zu must be a power of two when > 32", n);
  return spectral_call(c, 2, data1, data2, n, n, ans);
}

// ---------------------------------------------------------------------------
// Batched convolution and correlation (src/Convolve.rs:241 convlv_batch and
// ConvlvProcessor::process_batch :333; src/Correlation.rs:273 correl_batch).
// Items of equal length are transformed together: one batched forward FFT of
// all their lines, one spectral launch over all lines, one batched inverse
// FFT.  For convlv the response spectrum is computed once per length and
// shared by every item.
// ---------------------------------------------------------------------------
namespace {

int load_line(const Call& c, double* dst, const double* src, size_t doubles) {
  return c.dev() ? d2d(dst, src, doubles * sizeof(double)) : h2d(dst, src, doubles * sizeof(double));
}
int store_line(const Call& c, double* dst, const double* src, size_t doubles) {
  return c.dev() ? d2d(dst, src, doubles * sizeof(double)) : d2h(dst, src, doubles * sizeof(double));
}

// item indices grouped by length, groups in increasing length, items in order
std::map<size_t, std::vector<size_t>> by_length(const size_t* n, size_t count) {
  std::map<size_t, std::vector<size_t>> groups;
  for (size_t i = 0; i < count; ++i) groups[n[i]].push_back(i);
  return groups;
}

// lines per chunk of one group: at most 2^27 doubles (1 GiB) of work space
size_t lines_per_chunk(size_t n, size_t reserved_lines) {
  const size_t cap = ((size_t)1 << 27) / n;
  return cap > reserved_lines + 1 ? cap - reserved_lines : 1;
}

int convlv_group(const Call& c, const std::vector<size_t>& items, const double* const* data,
                 size_t n, const double* rdev, size_t m, int kind, double* const* ans) {
  const Form f = c.form();
  Twiddles tw;
  TRY(tables(f, tw));
  const long long nh = (long long)n / 2;
  const size_t per = lines_per_chunk(n, 1);
  for (size_t i0 = 0; i0 < items.size(); i0 += per) {
    const size_t cnt = std::min(per, items.size() - i0);
    TRY(ensure(g.work, (cnt + 1) * n * sizeof(double)));
    double* w = (double*)g.work.p;  // [response | data 0 | data 1 | ...]
    CK(launch_expand_response(rdev, (long long)m, w, (long long)n, nullptr, nullptr, g.cur));
    g.launches++;
    for (size_t j = 0; j < cnt; ++j) TRY(load_line(c, w + (j + 1) * n, data[items[i0 + j]], n));
    TRY(fft_lines(f, 1, w, nh, (long long)cnt + 1, nh));
    {
      ProfScope ps(PK_SPECTRAL, 3.0 * (double)n * 8 * (double)cnt);
      CK(launch_spectral_lines(f, kind, w + n, (long long)n, w, 0, w + n, (long long)n,
                               (long long)cnt, (long long)n, tw, g.cur));
    }
    g.launches++;
    TRY(fft_lines(f, -1, w + n, nh, (long long)cnt, nh));
    for (size_t j = 0; j < cnt; ++j) TRY(store_line(c, ans[items[i0 + j]], w + (j + 1) * n, n));
  }
  return GBFFT_OK;
}

int correl_group(const Call& c, const std::vector<size_t>& items, const double* const* data1,
                 const double* const* data2, size_t n, double* const* ans) {
  const Form f = c.form();
  Twiddles tw;
  TRY(tables(f, tw));
  const long long nh = (long long)n / 2;
  const size_t per = std::max<size_t>(1, lines_per_chunk(n, 0) / 2);
  for (size_t i0 = 0; i0 < items.size(); i0 += per) {
    const size_t cnt = std::min(per, items.size() - i0);
    TRY(ensure(g.work, 2 * cnt * n * sizeof(double)));
    double* w = (double*)g.work.p;  // [data1 lines | data2 lines]
    double* wb = w + cnt * n;
    for (size_t j = 0; j < cnt; ++j) {
      TRY(load_line(c, w + j * n, data1[items[i0 + j]], n));
      TRY(load_line(c, wb + j * n, data2[items[i0 + j]], n));
    }
    TRY(fft_lines(f, 1, w, nh, 2 * (long long)cnt, nh));
    {
      ProfScope ps(PK_SPECTRAL, 3.0 * (double)n * 8 * (double)cnt);
      CK(launch_spectral_lines(f, 2, w, (long long)n, wb, (long long)n, w, (long long)n,
                               (long long)cnt, (long long)n, tw, g.cur));
    }
    g.launches++;
    TRY(fft_lines(f, -1, w, nh, (long long)cnt, nh));
    for (size_t j = 0; j < cnt; ++j) TRY(store_line(c, ans[items[i0 + j]], w + j * n, n));
  }
  return GBFFT_OK;
}

}  // namespace

int gbfft_convlv_batch(const double* const* data, const size_t* n, size_t count,
                       const double* respns, size_t m, int isign, double* const* ans,
                       const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (count == 0) return GBFFT_OK;
  if (!data || !n || !ans) return fail(GBFFT_INVALID_ARG, "convlv_batch: null arrays");
  // convlv's checks (src/Convolve.rs:13-21), item by item in index order
  for (size_t i = 0; i < count; ++i) {
    if (n[i] == 0 || m == 0)
      return fail(GBFFT_EMPTY_INPUT, "convlv_batch: item %zu: input arrays cannot be empty", i);
    if (m > n[i])
      return fail(GBFFT_RESPONSE_TOO_LONG, "convlv_batch: item %zu: response function longer than data", i);
    if (isign != 1 && isign != -1)
      return fail(GBFFT_INVALID_ISIGN, "convlv_batch: isign must be 1 (convolution) or -1 (deconvolution)");
    if (!data[i] || !ans[i] || !respns)
      return fail(GBFFT_INVALID_ARG, "convlv_batch: item %zu: null pointer", i);
    if (n[i] < 2 || !is_pow2(n[i]) || ilog2(n[i]) > kMaxAxisLog)
      return fail(GBFFT_UNSUPPORTED_SIZE, "convlv_batch: item %zu: n=%zu must be a power of two >= 2", i, n[i]);
  }
  TRY(init_locked(g.device));
  StreamScope ss(c);
  const double* rdev = respns;
  if (!c.dev()) {
    TRY(ensure(g.stage_c, m * sizeof(double)));
    TRY(h2d(g.stage_c.p, respns, m * sizeof(double)));
    rdev = (const double*)g.stage_c.p;
  }
  for (auto& grp : by_length(n, count))
    TRY(convlv_group(c, grp.second, data, grp.first, rdev, m, isign == 1 ? 0 : 1, ans));
  return ss.finish(c);
}

int gbfft_correl_batch(const double* const* data1, const size_t* n1, const double* const* data2,
                       const size_t* n2, size_t count, double* const* ans,
                       const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (count == 0) return GBFFT_OK;
  if (!data1 || !n1 || !data2 || !n2 || !ans)
    return fail(GBFFT_INVALID_ARG, "correl_batch: null arrays");
  // correl's checks (src/Correlation.rs:10-16), item by item in index order
  for (size_t i = 0; i < count; ++i) {
    if (n1[i] == 0) return fail(GBFFT_EMPTY_INPUT, "correl_batch: item %zu: input arrays cannot be empty", i);
    if (n2[i] != n1[i])
      return fail(GBFFT_LENGTH_MISMATCH, "correl_batch: item %zu: input arrays must have the same length", i);
    if (!data1[i] || !data2[i] || !ans[i])
      return fail(GBFFT_INVALID_ARG, "correl_batch: item %zu: null pointer", i);
    if (n1[i] > 32 && (!is_pow2(n1[i]) || ilog2(n1[i]) > kMaxAxisLog))
      return fail(GBFFT_UNSUPPORTED_SIZE, "correl_batch: item %zu: n=%zu must be a power of two when > 32", i, n1[i]);
  }
  TRY(init_locked(g.device));
  StreamScope ss(c);
  for (auto& grp : by_length(n1, count)) {
    if (grp.first <= 32) {
      for (size_t i : grp.second) TRY(correl_small(c, data1[i], data2[i], grp.first, ans[i]));
    } else {
      TRY(correl_group(c, grp.second, data1, data2, grp.first, ans));
    }
  }
  return ss.finish(c);
}

// correl_normalized (fast = 0, src/Correlation.rs:189-223) and
// correl_normalized_fast (fast = 1, :226-270).  The statistics are computed on
// the GPU; the host reads the four scalars back to decide ZeroStdDev.
int gbfft_correl_normalized(const double* data1, size_t n1, const double* data2, size_t n2,
                            double* ans, int fast, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(check_form(c));
  if (n1 == 0) return fail(GBFFT_EMPTY_INPUT, "correl_normalized: input arrays cannot be empty");
  if (n2 != n1) return fail(GBFFT_LENGTH_MISMATCH, "correl_normalized: input arrays must have the same length");
  if (!data1 || !data2 || !ans) return fail(GBFFT_INVALID_ARG, "correl_normalized: null pointer");
  const size_t n = n1;
  if (n > 32 && (!is_pow2(n) || ilog2(n) > kMaxAxisLog))
    return fail(GBFFT_UNSUPPORTED_SIZE, "correl_normalized: n=%zu must be a power of two when > 32", n);
  TRY(init_locked(g.device));
  StreamScope ss(c);
  // device copies: inputs (staged for host pointers) and z-scores
  const size_t need = 4 * n + 256 + 8;
  TRY(ensure(g.stage_c, need * sizeof(double)));
  double* base = (double*)g.stage_c.p;
  const double *a = data1, *b = data2;
  if (!c.dev()) {
    TRY(h2d(base, data1, n * sizeof(double)));
    TRY(h2d(base + n, data2, n * sizeof(double)));
    a = base;
    b = base + n;
  }
  double* za = base + 2 * n;
  double* zb = base + 3 * n;
  double* partial = base + 4 * n;
  double* scal = partial + 256;  // sum1, sum2, m2_1, m2_2
  const double nd = (double)n;
  double h[4] = {0, 0, 0, 0};
  CK(launch_moment(a, (long long)n, 0.0, 1, partial, scal, g.cur));
  CK(launch_moment(b, (long long)n, 0.0, 1, partial, scal + 1, g.cur));
  if (fast) {
    CK(launch_moment(a, (long long)n, 0.0, 2, partial, scal + 2, g.cur));
    CK(launch_moment(b, (long long)n, 0.0, 2, partial, scal + 3, g.cur));
    g.launches += 8;
    TRY(d2h(h, scal, 4 * sizeof(double)));
    CK(cudaStreamSynchronize(g.cur));
  } else {
    g.launches += 4;
    TRY(d2h(h, scal, 2 * sizeof(double)));
    CK(cudaStreamSynchronize(g.cur));
    CK(launch_moment(a, (long long)n, h[0] / nd, 2, partial, scal + 2, g.cur));
    CK(launch_moment(b, (long long)n, h[1] / nd, 2, partial, scal + 3, g.cur));
    g.launches += 4;
    TRY(d2h(h + 2, scal + 2, 2 * sizeof(double)));
    CK(cudaStreamSynchronize(g.cur));
  }
  const double m1 = h[0] / nd, m2 = h[1] / nd;
  const double s1 = fast ? std::sqrt(h[2] / nd - m1 * m1) : std::sqrt(h[2] / nd);
  const double s2 = fast ? std::sqrt(h[3] / nd - m2 * m2) : std::sqrt(h[3] / nd);
  if (s1 == 0.0 || s2 == 0.0 || std::isnan(s1) || std::isnan(s2))
    return fail(GBFFT_ZERO_STD_DEV, "Normalization error: standard deviation is zero");
  if (fast && n <= 32) {
    double* o = c.dev() ? ans : zb;
    CK(launch_correl_direct_centered(a, b, o, (long long)n, m1, m2, 1.0 / (s1 * s2 * nd), g.cur));
    g.launches++;
    if (!c.dev()) TRY(d2h(ans, zb, n * sizeof(double)));
    return ss.finish(c);
  }
  CK(launch_standardize(a, (long long)n, m1, s1, za, g.cur));
  CK(launch_standardize(b, (long long)n, m2, s2, zb, g.cur));
  g.launches += 2;
  if (n <= 32) {
    double* o = c.dev() ? ans : partial;
    CK(launch_correl_direct(za, zb, o, (long long)n, g.cur));
    g.launches++;
    if (!c.dev()) TRY(d2h(ans, o, n * sizeof(double)));
    return ss.finish(c);
  }
  TRY(ensure(g.work, 2 * n * sizeof(double)));
  double* w = (double*)g.work.p;
  TRY(d2d(w, za, n * sizeof(double)));
  TRY(d2d(w + n, zb, n * sizeof(double)));
  TRY(spectral_dev(c.form(), 2, w, (long long)n));
  if (c.dev()) TRY(d2d(ans, w, n * sizeof(double)));
  else TRY(d2h(ans, w, n * sizeof(double)));
  return ss.finish(c);
}

static int spectrum_call(int kind, const double* cdata, size_t nn, double* out,
                         const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  if (!cdata || !out) return fail(GBFFT_INVALID_ARG, "spectrum: null pointer");
  TRY(dev_aligned(c, "spectrum", {cdata}));
  if (nn == 0) return GBFFT_OK;
  TRY(init_locked(g.device));
  StreamScope ss(c);
  const double* in = cdata;
  double* o = out;
  if (!c.dev()) {
    TRY(ensure(g.stage_c, 3 * nn * sizeof(double)));
    double* s = (double*)g.stage_c.p;
    TRY(h2d(s, cdata, 2 * nn * sizeof(double)));
    in = s;
    o = s + 2 * nn;
  }
  CK(launch_spectrum(kind, in, o, (long long)nn, g.cur));
  g.launches++;
  if (!c.dev()) TRY(d2h(out, o, nn * sizeof(double)));
  return ss.finish(c);
}

int gbfft_twiddle_lines(double* data, size_t lines, size_t len, size_t line0, size_t n, int isign,
                        const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  if (!data) return fail(GBFFT_INVALID_ARG, "twiddle_lines: null data");
  if (!c.dev()) return fail(GBFFT_INVALID_ARG, "twiddle_lines: device data only");
  TRY(dev_aligned(c, "twiddle_lines", {data}));
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "twiddle_lines: isign must be +-1");
  if (!is_pow2(n) || !is_pow2(len) || len > n || ilog2(n) > kMaxLog)
    return fail(GBFFT_UNSUPPORTED_SIZE,
                "twiddle_lines: n=%zu and len=%zu must be powers of two, len <= n <= 2^%d", n, len,
                kMaxLog);
  if (lines == 0 || n == 1) return GBFFT_OK;
  TRY(init_locked(g.device));
  StreamScope ss(c);
  Twiddles tw;
  TRY(tables(FORM_F64, tw));
  CK(launch_twiddle_lines(data, (long long)lines, ilog2(len), (long long)line0, ilog2(n), isign,
                          tw, g.cur));
  g.launches++;
  return ss.finish(c);
}

int gbfft_magnitude_spectrum(const double* c, size_t nn, double* out, const gbfft_opts* opts) {
  return spectrum_call(0, c, nn, out, opts);
}
int gbfft_power_spectrum(const double* c, size_t nn, double* out, const gbfft_opts* opts) {
  return spectrum_call(1, c, nn, out, opts);
}

// The sine/cosine transforms turn realft outputs into running sums over n/2
// terms, which multiplies the FFT's rounding error by up to ~200 at 2^20
// points.  Double-float arithmetic (about 48 significand bits) would then miss
// the FP64 bar, so the DF64 form runs their realft in FP64.
static Form trig_form(Form f) { return f == FORM_DF64 ? FORM_F64 : f; }

static int trig_check(const Call& c, double* y, size_t n, const char* what) {
  TRY(check_form(c));
  if (!y) return fail(GBFFT_INVALID_ARG, "%s: null data", what);
  TRY(dev_aligned(c, what, {y}));
  if (n < 2 || !is_pow2(n) || ilog2(n) > kMaxAxisLog - 2)
    return fail(GBFFT_UNSUPPORTED_SIZE, "%s: n=%zu must be a power of two >= 2", what, n);
  return GBFFT_OK;
}

// work area for the trig scans: n/2 values, chunk totals, a few scalars, and
// the per-block partial sums of cosft1
static int trig_work(size_t n, double** work, double** partial) {
  const size_t M = n / 2;
  const size_t chunks = (M + 2047) / 2048;
  const size_t np = 152 * 16 + 1;
  TRY(ensure(g.work, (M + chunks + 2 + np + 8) * sizeof(double)));
  *work = (double*)g.work.p;
  *partial = *work + M + chunks + 4;
  return GBFFT_OK;
}

int gbfft_sinft(double* y, size_t n, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(trig_check(c, y, n, "sinft"));
  TRY(init_locked(g.device));
  StreamScope ss(c);
  Twiddles tw;
  TRY(tables(FORM_F64, tw));
  double* d;
  TRY(stage_inout(c, g.stage_a, y, n, &d));
  double *work, *partial;
  TRY(trig_work(n, &work, &partial));
  CK(launch_sinft_pre(d, (long long)n, tw, g.cur));
  g.launches++;
  TRY(realft_dev(trig_form(c.form()), d, (long long)n, 1));
  CK(launch_trig_scan(0, d, (long long)n, nullptr, work, g.cur));
  g.launches += 3;
  TRY(unstage(c, y, d, n));
  return ss.finish(c);
}

int gbfft_cosft1(double* y, size_t n, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(trig_check(c, y, n, "cosft1"));
  TRY(init_locked(g.device));
  StreamScope ss(c);
  Twiddles tw;
  TRY(tables(FORM_F64, tw));
  double* d;
  TRY(stage_inout(c, g.stage_a, y, n + 1, &d));
  double *work, *partial;
  TRY(trig_work(n, &work, &partial));
  CK(launch_cosft1_pre(d, (long long)n, partial, tw, g.cur));
  g.launches += 2;
  TRY(realft_dev(trig_form(c.form()), d, (long long)n, 1));
  CK(launch_trig_scan(1, d, (long long)n, partial, work, g.cur));
  g.launches += 3;
  TRY(unstage(c, y, d, n + 1));
  return ss.finish(c);
}

int gbfft_cosft2(double* y, size_t n, int isign, const gbfft_opts* opts) {
  std::lock_guard<std::mutex> lk(g_mu);
  Call c(opts);
  TRY(trig_check(c, y, n, "cosft2"));
  // src/Cos_FT2.rs:8-12 panics on any other isign
  if (isign != 1 && isign != -1) return fail(GBFFT_INVALID_ARG, "Invalid isign value: %d. Must be 1 or -1", isign);
  TRY(init_locked(g.device));
  StreamScope ss(c);
  Twiddles tw;
  TRY(tables(FORM_F64, tw));
  double* d;
  TRY(stage_inout(c, g.stage_a, y, n, &d));
  double *work, *partial;
  TRY(trig_work(n, &work, &partial));
  if (isign == 1) {
    CK(launch_cosft2_pre(1, d, (long long)n, tw, g.cur));
    g.launches++;
    TRY(realft_dev(trig_form(c.form()), d, (long long)n, 1));
    CK(launch_cosft2_rot(1, d, (long long)n, tw, g.cur));
    g.launches++;
    CK(launch_trig_scan(2, d, (long long)n, nullptr, work, g.cur));
    g.launches += 3;
  } else {
    TRY(ensure(g.stage_c, n * sizeof(double)));
    double* w = (double*)g.stage_c.p;
    CK(launch_cosft2_inv_pre(d, w, (long long)n, tw, g.cur));
    g.launches++;
    TRY(realft_dev(trig_form(c.form()), w, (long long)n, -1));
    CK(launch_cosft2_inv_post(w, d, (long long)n, tw, g.cur));
    g.launches++;
  }
  TRY(unstage(c, y, d, n));
  return ss.finish(c);
}

}  // extern "C"
