// cluster_pass.cuh -- a Stockham pass of radix R = 2^11..2^14 on a cluster of
// four CTAs (FP32 form), so that a transform of up to 2^28 points takes two
// passes over HBM instead of three.
//
// A cluster owns four consecutive columns j0..j0+3 of one line.  Column j's
// pass computes X_k = sum_r x_r w_R^(rk), x_r = in[j + r L/R] times the
// inter-pass twiddle w_(Ns R)^((j mod Ns) r) (the same pass as k_pass).  With
// R = 4M and r = 4m + q it splits as
//   X_(k' + M s) = sum_q w_4^(q s) (w_R^(q k') Y_q[k']),
//   Y_q[k'] = sum_m x_(4m+q) w_M^(m k')         (k' < M, s < 4)
// CTA q loads the decimated rows r = q mod 4 of the four columns (4M points),
// computes their M-point DFTs Y_q in its shared memory with the radix-2..16
// sub-passes of the per-pass kernel, and after a cluster barrier CTA s reads
// Y_0..Y_3[k'] over distributed shared memory and writes the outputs
// k = k' + M s: one exchange of three quarters of the tile per pass.
// Global rows of the four columns are runs of four elements (32 B of FP32
// scratch, 64 B of f64) in both directions.
#pragma once
#include "fft_core.cuh"

namespace gbfft {

constexpr int kClRanks = 4;  // CTAs per cluster
constexpr int kClLogC = 2;   // columns per cluster tile

__device__ __forceinline__ unsigned cl_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Barrier over every thread of the cluster; shared-memory writes before it
// are visible to the cluster's loads after it.
__device__ __forceinline__ void cl_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared::cluster address, in CTA `rank`, of the shared variable at `p`.
__device__ __forceinline__ unsigned cl_map(const void* p, unsigned rank) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  unsigned r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}

__device__ __forceinline__ F32::C cl_ld(unsigned addr) {
  F32::C v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
  return v;
}

template <int IO>
__device__ __forceinline__ const typename IOElem<IO>::T* cl_line_in(const PassParams& p,
                                                                    long long line) {
  using E = typename IOElem<IO>::T;
  if (p.in_ptrs) return reinterpret_cast<const E*>(p.in_ptrs[line]);
  return reinterpret_cast<const E*>(p.in) + line_base(p, line);
}
template <int IO>
__device__ __forceinline__ typename IOElem<IO>::T* cl_line_out(const PassParams& p,
                                                              long long line) {
  using E = typename IOElem<IO>::T;
  if (p.out_ptrs) return reinterpret_cast<E*>(p.out_ptrs[line]);
  return reinterpret_cast<E*>(p.out) + line_base(p, line);
}

// First sub-pass (radix Q) of CTA q's M-point DFTs, from global memory:
// butterfly (c, b) of column j0 + c reads the local rows b + t M/Q, i.e. the
// global rows r = 4 b + q + t R/Q, applies the inter-pass twiddles and writes
// its outputs to local rows b Q + t of the shared tile.
template <int SG, int IN, int Q, int T>
__device__ __forceinline__ void cl_first(const PassParams& p, long long line, long long j0,
                                         unsigned q, int logM, f2* sm, int cs, int tid) {
  using C = F32::C;
  using IE = typename IOElem<IN>::T;
  constexpr int B = kEPT / Q;
  constexpr int LQ = (Q == 2) ? 1 : (Q == 4) ? 2 : (Q == 8) ? 3 : 4;
  constexpr int sh = F32::kPadShift;
  const int logR = p.logR;
  const long long LR = p.L >> logR;
  const IE* base = cl_line_in<IN>(p, line) + j0;
  const long long rstep = LR << (logR - LQ);  // global index step between a butterfly's inputs
  // The f64 inputs are loaded in two halves of Q/2, each converted to FP32
  // as it arrives, so that 1024-thread CTAs fit their 64 registers; eight
  // 16-byte loads in flight per thread still keep 128 KB in flight per SM.
  constexpr int H = (sizeof(IE) == 16 && Q >= 8) ? 2 : 1;
  C v[B][Q];
  int cc[B], bb[B];
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int e = tid + i * T;
    cc[i] = e & 3;
    bb[i] = e >> 2;
  }
#pragma unroll
  for (int h = 0; h < H; ++h) {
    IE raw[B][Q / H];
#pragma unroll
    for (int i = 0; i < B; ++i) {
      const IE* src = base + cc[i] + LR * (long long)(4 * bb[i] + (int)q);
#pragma unroll
      for (int t = 0; t < Q / H; ++t) raw[i][t] = src[(h * (Q / H) + t) * rstep];
    }
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int t = 0; t < Q / H; ++t) v[i][h * (Q / H) + t] = gload<F32, IN>(&raw[i][t], 0);
  }
  const int logS = p.logNs + logR;
#pragma unroll
  for (int i = 0; i < B; ++i) {
    const int c = cc[i], b = bb[i];
    const unsigned jm = (unsigned)((j0 + c) & (p.Ns - 1));
    C* w = v[i];
    if (p.logNs > 0 && jm != 0) {
      // w^(jm (r0 + t R/Q)), t = 4a + u, as w^(jm (r0 + 4a R/Q)) * w^(jm u R/Q):
      // every exponent is below jm R <= Ns R = 2^logS
      const unsigned r0 = 4u * (unsigned)b + q;
      const unsigned step = jm << (logR - LQ);
      if constexpr (Q >= 4) {
        C su[4];
        su[0] = C{1.f, 0.f};
#pragma unroll
        for (int u = 1; u < 4; ++u) su[u] = twiddle<F32>(p.tw, logS, step * (unsigned)u, SG);
#pragma unroll
        for (int a = 0; a < Q / 4; ++a) {
          const C la = twiddle<F32>(p.tw, logS, jm * r0 + step * (unsigned)(4 * a), SG);
          w[4 * a] = F32::mul(w[4 * a], la);
#pragma unroll
          for (int u = 1; u < 4; ++u) w[4 * a + u] = F32::mul(w[4 * a + u], F32::mul(la, su[u]));
        }
      } else {
#pragma unroll
        for (int t = 0; t < Q; ++t)
          w[t] = F32::mul(w[t], twiddle<F32>(p.tw, logS, jm * r0 + step * (unsigned)t, SG));
      }
    }
    dftq<F32, SG, Q>(w);
    const int cb = c * cs;
#pragma unroll
    for (int t = 0; t < Q; ++t) sm[cb + pidx(b * Q + t, sh)] = F32::to_s(w[t]);
  }
}

template <int SG, int IN, int T>
__device__ __forceinline__ void cl_first_q(int lq, const PassParams& p, long long line,
                                           long long j0, unsigned q, int logM, f2* sm, int cs,
                                           int tid) {
  // the M-point DFTs (M = 2^9..2^12) split into radix-8 and radix-16
  // sub-passes only (checked at launch)
  if (lq == 4) cl_first<SG, IN, 16, T>(p, line, j0, q, logM, sm, cs, tid);
  else cl_first<SG, IN, 8, T>(p, line, j0, q, logM, sm, cs, tid);
}

// Output k = k' + M s of column c: sum_q w_4^(q s) w_R^(q k') Y_q[k'].
template <int SG>
__device__ __forceinline__ F32::C cl_combine(const unsigned (&peer)[kClRanks], int off, int kp,
                                             int logR, unsigned s, const Twiddles& tw) {
  using C = F32::C;
  C z[kClRanks];
#pragma unroll
  for (int u = 0; u < kClRanks; ++u) z[u] = cl_ld(peer[u] + (unsigned)off * 8u);
  if (kp != 0) {
#pragma unroll
    for (int u = 1; u < kClRanks; ++u)
      z[u] = F32::mul(z[u], twiddle<F32>(tw, logR, (unsigned)(u * kp), SG));
  }
  // w_4 = exp(SG 2 pi i / 4) = SG i
  const C a = F32::add(z[0], z[2]), b = F32::sub(z[0], z[2]);
  const C c = F32::add(z[1], z[3]), d = F32::mul_j(F32::sub(z[1], z[3]), SG);
  switch (s) {
    case 0: return F32::add(a, c);
    case 1: return F32::add(b, d);
    case 2: return F32::sub(a, c);
    default: return F32::sub(b, d);
  }
}

// 1024 resident threads per SM for every thread count (64 registers each)
template <int SG, int IN, int OUT, int T>
__global__ void __cluster_dims__(kClRanks, 1, 1) __launch_bounds__(T, 1024 / T)
    k_pass_cl(PassParams p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  f2* sm = reinterpret_cast<f2*>(smem_raw);
  using C = F32::C;
  constexpr int sh = F32::kPadShift;
  const int tid = threadIdx.x;
  const unsigned q = cl_rank();
  const long long tile = (long long)(blockIdx.x / kClRanks);
  long long line, j0;
  tile_origin(p, tile, line, j0);  // mode 0 tiles of four columns
  const int logR = p.logR, logM = logR - 2;
  const int cs = col_stride(logM, sh);

  // M-point DFTs of this CTA's decimated rows, in shared memory
  cl_first_q<SG, IN, T>(p.q[0], p, line, j0, q, logM, sm, cs, tid);
  __syncthreads();
  int logNsub = p.q[0];
  for (int k = 1; k < p.nq; ++k) {
    if (p.q[k] == 4) subpass<F32, SG, 16>(sm, logM, cs, logNsub, p.tw, tid, T);
    else subpass<F32, SG, 8>(sm, logM, cs, logNsub, p.tw, tid, T);
    logNsub += p.q[k];
  }

  // exchange: every CTA's Y_q visible to the cluster
  cl_sync();
  unsigned peer[kClRanks];
#pragma unroll
  for (int u = 0; u < kClRanks; ++u) peer[u] = cl_map(sm, (unsigned)u);
  using OE = typename IOElem<OUT>::T;
  OE* dst = cl_line_out<OUT>(p, line);
  const long long lb = line_base(p, line);
  const long long M = 1ll << logM;
  const long long Ns = p.Ns;
#pragma unroll 4
  for (int i = 0; i < kEPT; ++i) {
    const int e = tid + i * T;
    int c, kp;
    if (p.out_rcontig) { kp = e & (int)(M - 1); c = e >> logM; }
    else { c = e & 3; kp = e >> 2; }
    C v = cl_combine<SG>(peer, c * cs + pidx(kp, sh), kp, logR, q, p.tw);
    if (p.do_scale) v = apply_scale<F32>(v, p);
    const long long j = j0 + c;
    const long long jd = ((j >> p.logNs) << (p.logNs + logR)) + (j & (Ns - 1));
    const long long k = (long long)kp + M * (long long)q;
    const long long idx = jd + k * Ns;
    gstore<F32, OUT>(dst, idx, v);
    if (p.spec_kind) spec_store<F32>(p, lb + idx, v);
  }
  // no CTA leaves (its shared memory) while a peer may still read it
  cl_sync();
}

inline size_t cl_smem_bytes(int logR) {
  return sizeof(f2) * (size_t)(1 << kClLogC) * (size_t)col_stride(logR - 2, F32::kPadShift);
}

template <int SG, int IN, int OUT, int T>
inline cudaError_t launch_cl_one(const PassParams& p, cudaStream_t st) {
  static DeviceOnce attr_done;
  // T threads hold R = 16 T points: four columns of R / 4 rows
  if (p.logR < 4 || (1 << p.logR) != 16 * T || p.q[0] < 3 || p.q[0] > 4) return cudaErrorInvalidValue;
  for (int k = 1; k < p.nq; ++k)
    if (p.q[k] < 3 || p.q[k] > 4) return cudaErrorInvalidValue;
  const size_t smem = cl_smem_bytes(p.logR);
  cudaError_t e = smem_opt_in(k_pass_cl<SG, IN, OUT, T>, smem, attr_done);
  if (e != cudaSuccess) return e;
  const long long grid = p.tiles * kClRanks;
  if (p.tiles <= 0 || grid > 0x7FFFFFFFll) return cudaErrorInvalidValue;
  PassParams q = p;
  q.fscale = (float)q.scale;
  k_pass_cl<SG, IN, OUT, T><<<dim3((unsigned)grid), T, smem, st>>>(q);
  return cudaGetLastError();
}

template <int SG, int IN, int OUT>
cudaError_t launch_cl_t(const PassParams& p, int threads, cudaStream_t st) {
  switch (threads) {
    case 1024: return launch_cl_one<SG, IN, OUT, 1024>(p, st);
    case 512: return launch_cl_one<SG, IN, OUT, 512>(p, st);
    case 256: return launch_cl_one<SG, IN, OUT, 256>(p, st);
    case 128: return launch_cl_one<SG, IN, OUT, 128>(p, st);
    default: return cudaErrorInvalidValue;
  }
}

// A two-pass plan reads the caller's f64 array into FP32 scratch and back.
template <int SG>
cudaError_t dispatch_cl(IOType in, IOType out, const PassParams& p, int threads,
                        cudaStream_t st) {
  if (in == IO_D2 && out == IO_F2) return launch_cl_t<SG, IO_D2, IO_F2>(p, threads, st);
  if (in == IO_F2 && out == IO_D2) return launch_cl_t<SG, IO_F2, IO_D2>(p, threads, st);
  return cudaErrorInvalidValue;
}

}  // namespace gbfft
