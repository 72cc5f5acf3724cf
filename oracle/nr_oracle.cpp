// nr_oracle.cpp -- CPU oracle for the numrs FFT family.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity checker and the timed CPU
// baseline; the shipped library never links or calls it.
//
// It restates, in plain C++ with IEEE double arithmetic and no FMA contraction
// (built with -ffp-contract=off so every product is rounded like Rust's f64
// arithmetic), the algorithms of the numrs crate:
//
//   four1            src/FFT_1.rs:5-107   (hybrid: recurrence for mmax<1024,
//                                          per-stage cos/sin table above)
//   four1_optimized  src/FFT_1.rs:110-140 (recurrence for every stage)
//   four1_nr         src/Real_FT.rs:430-476, src/FFT_2.rs:310-358 (the private
//                                          1-based copies used by realft/twofft)
//   fft_batch        src/FFT_1.rs:166-190 (FFTProcessor::fft dispatch)
//   realft           src/Real_FT.rs:4-213
//   twofft           src/FFT_2.rs:3-132
//   fourn            N-D contract of src/Fourn.rs:278 (fourn_simd signature) and
//                    the call sites src/Real_FT3.rs:35,168
//   rlft3            src/Real_FT3.rs:8-141
//   cosft1           src/Cos_FT.rs:7-68
//   cosft2           src/Cos_FT2.rs:7-173
//   sinft            (listed in README.md:72, no file) -- Numerical Recipes
//                    sine-transform contract
//   convlv           src/Convolve.rs:8-138
//   correl           src/Correlation.rs:8-110,174-186 (n<=32 direct branch kept)
//
// Where a reference routine is numerically wrong (index shifted by one slot,
// wrong mirror index, constant instead of running twiddle) the restatement
// follows the Numerical Recipes contract the routine was written against; each
// correction is named at the function.  All arrays are 0-based.
//
// Sign convention (as the reference): isign=+1 computes
//   X_k = sum_j x_j exp(+2 pi i jk/N); transforms are unnormalised.

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>
#include <thread>
#include <mutex>
#include <condition_variable>
#include <functional>
#include <atomic>
#include <algorithm>

namespace {

const double PI = 3.14159265358979323846264338327950288;

// ---------------------------------------------------------------------------
// A tiny fork-join pool standing in for rayon (par_chunks / par_iter / join).
// ---------------------------------------------------------------------------
class Pool {
 public:
  explicit Pool(int n) : nthreads_(n < 1 ? 1 : n) {
    for (int t = 1; t < nthreads_; ++t) workers_.emplace_back([this, t] { loop(t); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& w : workers_) w.join();
  }
  int size() const { return nthreads_; }
  // Run fn(i) for i in [0, count), spread over the pool; returns when all done.
  // A call made from inside a pool task runs serially in that task.
  void parallel_for(size_t count, const std::function<void(size_t)>& fn) {
    if (nthreads_ == 1 || count < 2 || t_in_task) {
      for (size_t i = 0; i < count; ++i) fn(i);
      return;
    }
    std::unique_lock<std::mutex> lk(m_);
    job_ = &fn;
    count_ = count;
    next_.store(0);
    pending_ = nthreads_ - 1;
    ++gen_;
    lk.unlock();
    cv_.notify_all();
    work();
    lk.lock();
    done_cv_.wait(lk, [this] { return pending_ == 0; });
    job_ = nullptr;
  }

 private:
  void work() {
    t_in_task = true;
    for (;;) {
      size_t i = next_.fetch_add(1);
      if (i >= count_) break;
      (*job_)(i);
    }
    t_in_task = false;
  }
  static thread_local bool t_in_task;
  void loop(int) {
    uint64_t seen = 0;
    for (;;) {
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return gen_ != seen; });
      seen = gen_;
      if (stop_) return;
      lk.unlock();
      work();
      lk.lock();
      if (--pending_ == 0) done_cv_.notify_one();
    }
  }
  int nthreads_;
  std::vector<std::thread> workers_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t)>* job_ = nullptr;
  size_t count_ = 0;
  std::atomic<size_t> next_{0};
  int pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

thread_local bool Pool::t_in_task = false;

Pool* g_pool = nullptr;
Pool& pool() {
  if (!g_pool) g_pool = new Pool(1);
  return *g_pool;
}

// ---------------------------------------------------------------------------
// four1 family
// ---------------------------------------------------------------------------

// Bit-reversal permutation, src/FFT_1.rs:9-22 (1-based j and i as written there).
void bitrev(double* data, size_t nn) {
  size_t n = nn * 2;
  size_t j = 1;
  for (size_t i = 1; i < n; i += 2) {
    if (j > i) {
      std::swap(data[j - 1], data[i - 1]);
      std::swap(data[j], data[i]);
    }
    size_t m = nn;
    while (m >= 2 && j > m) {
      j -= m;
      m >>= 1;
    }
    j += m;
  }
}

// src/FFT_1.rs:47-72.  Loops are bounded by the slice length `len`, as there.
void butterflies_sequential(double* data, size_t len, size_t mmax, size_t istep, double wpr,
                            double wpi) {
  double wr = 1.0, wi = 0.0;
  for (size_t m = 0; m < mmax; m += 2) {
    for (size_t i = m; i < len; i += istep) {
      size_t j = i + mmax;
      if (j >= len) continue;
      double tempr = wr * data[j] - wi * data[j + 1];
      double tempi = wr * data[j + 1] + wi * data[j];
      data[j] = data[i] - tempr;
      data[j + 1] = data[i + 1] - tempi;
      data[i] += tempr;
      data[i + 1] += tempi;
    }
    double wtemp = wr;
    wr = wtemp * wpr - wi * wpi + wr;
    wi = wi * wpr + wtemp * wpi + wi;
  }
}

// src/FFT_1.rs:75-107: a per-stage cos/sin table, butterfly groups (chunks of
// istep doubles) processed in parallel.  Each chunk is independent, so the
// result does not depend on the thread count.
void butterflies_parallel(double* data, size_t len, size_t mmax, size_t istep, int isign) {
  std::vector<double> wr(mmax / 2), wi(mmax / 2);
  for (size_t m = 0; m < mmax / 2; ++m) {
    double angle = (double)isign * 2.0 * PI * (double)m / (double)mmax;
    wr[m] = std::cos(angle);
    wi[m] = std::sin(angle);
  }
  size_t nchunks = len / istep;  // par_chunks_mut: a short tail chunk returns early
  pool().parallel_for(nchunks, [&](size_t c) {
    double* chunk = data + c * istep;
    size_t clen = istep;
    for (size_t m = 0; m < mmax / 2; ++m) {
      for (size_t i = m * 2; i < clen - mmax; i += istep) {
        size_t j = i + mmax;
        double tempr = wr[m] * chunk[j] - wi[m] * chunk[j + 1];
        double tempi = wr[m] * chunk[j + 1] + wi[m] * chunk[j];
        chunk[j] = chunk[i] - tempr;
        chunk[j + 1] = chunk[i + 1] - tempi;
        chunk[i] += tempr;
        chunk[i + 1] += tempi;
      }
    }
  });
}

// src/FFT_1.rs:5-44 (hybrid = true) and :110-140 (hybrid = false).
void four1_impl(double* data, size_t len, size_t nn, int isign, bool hybrid) {
  size_t n = nn * 2;
  bitrev(data, nn);
  size_t mmax = 2;
  while (n > mmax) {
    size_t istep = mmax << 1;
    double theta = (double)isign * (2.0 * PI / (double)mmax);
    double wtemp = std::sin(0.5 * theta);
    double wpr = -2.0 * wtemp * wtemp;
    double wpi = std::sin(theta);
    if (hybrid && mmax >= 1024)
      butterflies_parallel(data, len, mmax, istep, isign);
    else
      butterflies_sequential(data, len, mmax, istep, wpr, wpi);
    mmax = istep;
  }
}

// The private 1-based copy, src/Real_FT.rs:430-476 (identical to
// src/FFT_2.rs:310-358): recurrence twiddles, theta = isign*2*PI/mmax.
void four1_nr(double* data, size_t nn, int isign) {
  size_t n = nn * 2;
  bitrev(data, nn);
  size_t mmax = 2;
  while (n > mmax) {
    size_t istep = mmax << 1;
    double theta = (double)isign * 2.0 * PI / (double)mmax;
    double wtemp = std::sin(theta / 2.0);
    double wpr = -2.0 * wtemp * wtemp;
    double wpi = std::sin(theta);
    double wr = 1.0, wi = 0.0;
    for (size_t m = 1; m < mmax; m += 2) {
      for (size_t i = m; i <= n; i += istep) {
        size_t j = i + mmax;
        double tempr = wr * data[j - 1] - wi * data[j];
        double tempi = wr * data[j] + wi * data[j - 1];
        data[j - 1] = data[i - 1] - tempr;
        data[j] = data[i] - tempi;
        data[i - 1] += tempr;
        data[i] += tempi;
      }
      double wt = wr;
      wr = wt * wpr - wi * wpi + wr;
      wi = wi * wpr + wt * wpi + wi;
    }
    mmax = istep;
  }
}

// ---------------------------------------------------------------------------
// realft  (src/Real_FT.rs:4-213)
//
// Correction: the reference applies the 1-based Numerical Recipes indices
// i1=2i-1.. directly to a 0-based slice (src/Real_FT.rs:61-64), shifting every
// access by one double.  Here k = i-1 is the 0-based complex index, and the
// mirror of k is n/2-k.  The table branch (n >= 1024) uses angle (i-2)*theta
// (src/Real_FT.rs:93,189); the recurrence branch uses (i-1)*theta
// (src/Real_FT.rs:30-31); the correct twiddle is w^k = exp(i*k*theta), k=i-1.
// ---------------------------------------------------------------------------
inline void twist_pair(double* data, size_t k, size_t n, double c1, double c2, double wr,
                       double wi) {
  size_t i1 = 2 * k, i2 = i1 + 1;
  size_t i3 = n - 2 * k, i4 = i3 + 1;  // complex slot n/2-k
  double h1r = c1 * (data[i1] + data[i3]);
  double h1i = c1 * (data[i2] - data[i4]);
  double h2r = -c2 * (data[i2] + data[i4]);
  double h2i = c2 * (data[i1] - data[i3]);
  data[i1] = h1r + wr * h2r - wi * h2i;
  data[i2] = h1i + wr * h2i + wi * h2r;
  data[i3] = h1r - wr * h2r + wi * h2i;
  data[i4] = -h1i + wr * h2i + wi * h2r;
}

void realft_twist(double* data, size_t n, double c2, double theta) {
  const double c1 = 0.5;
  if (n >= 1024) {
    // table branch, src/Real_FT.rs:83-117 / :179-213
    for (size_t k = 1; k < n / 4; ++k) {
      double angle = (double)k * theta;
      twist_pair(data, k, n, c1, c2, std::cos(angle), std::sin(angle));
    }
  } else {
    // recurrence branch, src/Real_FT.rs:49-80 / :145-176
    double wtemp = std::sin(0.5 * theta);
    double wpr = -2.0 * wtemp * wtemp;
    double wpi = std::sin(theta);
    double wr = 1.0 + wpr, wi = wpi;
    for (size_t k = 1; k < n / 4; ++k) {
      twist_pair(data, k, n, c1, c2, wr, wi);
      double wt = wr;
      wr = wt * wpr - wi * wpi + wr;
      wi = wi * wpr + wt * wpi + wi;
    }
  }
}

void realft(double* data, size_t n, int isign) {
  size_t half_n = n / 2;
  if (isign == 1) {
    four1_nr(data, half_n, 1);
    realft_twist(data, n, -0.5, PI / (double)half_n);
    double h1r = data[0];
    data[0] = h1r + data[1];
    data[1] = h1r - data[1];
  } else {
    const double c1 = 0.5;
    double h1r = data[0];
    data[0] = c1 * (h1r + data[1]);
    data[1] = c1 * (h1r - data[1]);
    realft_twist(data, n, 0.5, -PI / (double)half_n);
    four1_nr(data, half_n, -1);
  }
}

}  // namespace

extern "C" {

// Thread count for the parallel stages (rayon pool size stand-in).
void orc_set_threads(int n) {
  delete g_pool;
  g_pool = new Pool(n);
}
int orc_get_threads() { return pool().size(); }

void orc_four1(double* data, size_t len, size_t nn, int isign) {
  four1_impl(data, len, nn, isign, true);
}
void orc_four1_optimized(double* data, size_t len, size_t nn, int isign) {
  four1_impl(data, len, nn, isign, false);
}
void orc_four1_nr(double* data, size_t nn, int isign) { four1_nr(data, nn, isign); }

// FFTProcessor::fft (src/FFT_1.rs:166-182) with use_optimized = true.
static void processor_fft(double* data, size_t len, int isign) {
  size_t nn = len / 2;
  if (nn >= 512)
    four1_impl(data, len, nn, isign, false);
  else
    four1_impl(data, len, nn, isign, true);
}

// FFTProcessor::fft_batch (src/FFT_1.rs:185-190): one transform per pool task.
void orc_fft_batch(double** ptrs, const size_t* lens, size_t count, int isign) {
  pool().parallel_for(count, [&](size_t t) {
    // nested parallel stages run serially inside a batch task (nn<512 never
    // reaches them; four1_optimized has none)
    processor_fft(ptrs[t], lens[t], isign);
  });
}

void orc_realft(double* data, size_t n, int isign) { realft(data, n, isign); }

// twofft (src/FFT_2.rs:3-132).  fft1/fft2 have length 2n+2 (src/FFT_2.rs:6-7);
// the n-point spectra occupy [0, 2n).  Correction: the mirror of complex slot k
// is n-k (doubles 2n-2k), not 2n+2-2k as at src/FFT_2.rs:74,111; the split
// covers k = 1..n/2 including the Nyquist slot.
void orc_twofft(const double* data1, const double* data2, double* fft1, double* fft2,
                size_t n) {
  for (size_t j = 0; j < n; ++j) {
    fft1[2 * j] = data1[j];
    fft1[2 * j + 1] = data2[j];
  }
  four1_nr(fft1, n, 1);
  fft2[0] = fft1[1];
  fft1[1] = 0.0;
  fft2[1] = 0.0;
  for (size_t k = 1; k <= n / 2; ++k) {
    size_t j = 2 * k, jr = 2 * n - 2 * k;
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

// fourn: in-memory N-D complex FFT, row-major, nn[ndim-1] contiguous,
// interleaved complex.  The reference has no working in-memory body
// (src/Fourn.rs:56-87 are stubs); the contract is the fourn_simd signature
// (src/Fourn.rs:278) and validate_inputs (src/Fourn.rs:367-378).  Each axis is
// transformed with four1 (src/FFT_1.rs:5) on a gathered line.  Returns 0 or -1
// (invalid input, the io::ErrorKind::InvalidInput of validate_inputs).
static void fourn_impl(double* data, const size_t* nn, size_t ndim, int isign);

int orc_fourn(double* data, const size_t* nn, size_t nn_len, size_t ndim, int isign) {
  if (ndim == 0 || ndim > nn_len) return -1;
  if (isign != 1 && isign != -1) return -1;
  for (size_t d = 0; d < ndim; ++d)
    if (nn[d] <= 1) return -1;
  fourn_impl(data, nn, ndim, isign);
  return 0;
}

// The transform itself; axes of length 1 are the identity.
static void fourn_impl(double* data, const size_t* nn, size_t ndim, int isign) {
  size_t total = 1;
  for (size_t d = 0; d < ndim; ++d) total *= nn[d];
  size_t stride = 1;  // in complex elements
  for (size_t dd = ndim; dd-- > 0;) {
    size_t len = nn[dd];
    if (len == 1) continue;
    const size_t outer = total / (len * stride);
    // Lines are independent, so they are spread over the pool (in groups of
    // consecutive lines); each line's arithmetic is the same whatever the
    // thread count.
    const size_t lines = outer * stride;
    const size_t group = std::max<size_t>(1, std::min<size_t>(64, lines / 256));
    pool().parallel_for((lines + group - 1) / group, [&](size_t gi) {
      std::vector<double> line(2 * len);
      for (size_t li = gi * group; li < std::min(lines, (gi + 1) * group); ++li) {
        const size_t o = li / stride, s = li % stride;
        double* base = data + 2 * (o * len * stride + s);
        for (size_t l = 0; l < len; ++l) {
          line[2 * l] = base[2 * l * stride];
          line[2 * l + 1] = base[2 * l * stride + 1];
        }
        four1_impl(line.data(), 2 * len, len, isign, true);
        for (size_t l = 0; l < len; ++l) {
          base[2 * l * stride] = line[2 * l];
          base[2 * l * stride + 1] = line[2 * l + 1];
        }
      }
    });
    stride *= len;
  }
}

// rlft3 (src/Real_FT3.rs:8-141 and the flat form :145-258).  data is
// nn1 x nn2 x nn3 reals (row-major), viewed after the transform as
// nn1 x nn2 x nn3/2 complex; speq is nn1 x 2*nn2.  Forward: data holds
// H[k1,k2,k3] for k3 < nn3/2, speq[k1][2k2..2k2+1] holds H[k1,k2,nn3/2].
// Inverse returns (nn1*nn2*nn3/2) * the real array.
// Correction: the forward speq store is in natural k2 order (the reference
// mirrors it at src/Real_FT3.rs:47,173); the twist then reads speq at the
// mirrored (j1, j2) exactly as the Numerical Recipes routine does.
void orc_rlft3(double* data, double* speq, size_t nn1, size_t nn2, size_t nn3, int isign) {
  const double c1 = 0.5;
  const double c2 = -0.5 * (double)isign;
  const double theta = (double)isign * (2.0 * PI / (double)nn3);
  double wtemp = std::sin(0.5 * theta);
  const double wpr = -2.0 * wtemp * wtemp;
  const double wpi = std::sin(theta);
  const size_t nh = nn3 >> 1;
  size_t nn[3] = {nn1, nn2, nh};
  auto D = [&](size_t i1, size_t i2, size_t e) -> double& {
    return data[(i1 * nn2 + i2) * nn3 + e];
  };
  auto S = [&](size_t i1, size_t e) -> double& { return speq[i1 * 2 * nn2 + e]; };
  if (isign == 1) {
    fourn_impl(data, nn, 3, 1);
    for (size_t i1 = 0; i1 < nn1; ++i1)
      for (size_t i2 = 0; i2 < nn2; ++i2) {
        S(i1, 2 * i2) = D(i1, i2, 0);
        S(i1, 2 * i2 + 1) = D(i1, i2, 1);
      }
  }
  for (size_t i1 = 0; i1 < nn1; ++i1) {
    size_t j1 = i1 ? nn1 - i1 : 0;
    double wr = 1.0, wi = 0.0;
    for (size_t i3 = 0; i3 <= (nn3 >> 2); ++i3) {
      size_t ii3 = 2 * i3;
      for (size_t i2 = 0; i2 < nn2; ++i2) {
        if (i3 == 0) {
          size_t j2 = i2 ? 2 * (nn2 - i2) : 0;
          double h1r = c1 * (D(i1, i2, 0) + S(j1, j2));
          double h1i = c1 * (D(i1, i2, 1) - S(j1, j2 + 1));
          double h2i = c2 * (D(i1, i2, 0) - S(j1, j2));
          double h2r = -c2 * (D(i1, i2, 1) + S(j1, j2 + 1));
          D(i1, i2, 0) = h1r + h2r;
          D(i1, i2, 1) = h1i + h2i;
          S(j1, j2) = h1r - h2r;
          S(j1, j2 + 1) = h2i - h1i;
        } else {
          size_t j2 = i2 ? nn2 - i2 : 0;
          size_t j3 = nn3 - 2 * i3;
          double h1r = c1 * (D(i1, i2, ii3) + D(j1, j2, j3));
          double h1i = c1 * (D(i1, i2, ii3 + 1) - D(j1, j2, j3 + 1));
          double h2i = c2 * (D(i1, i2, ii3) - D(j1, j2, j3));
          double h2r = -c2 * (D(i1, i2, ii3 + 1) + D(j1, j2, j3 + 1));
          D(i1, i2, ii3) = h1r + wr * h2r - wi * h2i;
          D(i1, i2, ii3 + 1) = h1i + wr * h2i + wi * h2r;
          D(j1, j2, j3) = h1r - wr * h2r + wi * h2i;
          D(j1, j2, j3 + 1) = -h1i + wr * h2i + wi * h2r;
        }
      }
      double wt = wr;
      wr = wt * wpr - wi * wpi + wr;
      wi = wi * wpr + wt * wpi + wi;
    }
  }
  if (isign == -1) fourn_impl(data, nn, 3, -1);
}

// sinft: y[0..n), y[0] is taken as 0.  Output y[k] = sum_{j=1}^{n-1}
// y_j sin(pi jk/n) (y[0] = 0).  Self-inverse up to 2/n.  Numerical Recipes
// contract (no reference file exists; README.md:72 lists Sin_FT).
void orc_sinft(double* y, size_t n) {
  double theta = PI / (double)n;
  double wtemp = std::sin(0.5 * theta);
  double wpr = -2.0 * wtemp * wtemp;
  double wpi = std::sin(theta);
  double wr = 1.0, wi = 0.0;
  y[0] = 0.0;
  for (size_t j = 1; j <= n / 2; ++j) {
    double wt = wr;
    wr = wt * wpr - wi * wpi + wr;
    wi = wi * wpr + wt * wpi + wi;
    double y1 = wi * (y[j] + y[n - j]);
    double y2 = 0.5 * (y[j] - y[n - j]);
    y[j] = y1 + y2;
    y[n - j] = y1 - y2;
  }
  realft(y, n, 1);
  y[0] *= 0.5;
  double sum = 0.0;
  y[1] = 0.0;
  for (size_t j = 0; j + 1 < n; j += 2) {
    sum += y[j];
    y[j] = y[j + 1];
    y[j + 1] = sum;
  }
}

// cosft1 (src/Cos_FT.rs:7-68): y[0..n] holds n+1 samples (the reference uses
// the 1-based slice y[1..=n+1]).  Output Y_k = (y_0 + (-1)^k y_n)/2 +
// sum_{j=1}^{n-1} y_j cos(pi jk/n), k = 0..n.  Self-inverse up to 2/n.
// Correction: the reference drops the store of the running sum into slot 1
// after realft (src/Cos_FT.rs:60-67).
void orc_cosft1(double* y, size_t n) {
  double theta = PI / (double)n;
  double wtemp = std::sin(0.5 * theta);
  double wpr = -2.0 * wtemp * wtemp;
  double wpi = std::sin(theta);
  double wr = 1.0, wi = 0.0;
  double sum = 0.5 * (y[0] - y[n]);
  y[0] = 0.5 * (y[0] + y[n]);
  for (size_t j = 1; j < n / 2; ++j) {
    double wt = wr;
    wr = wt * wpr - wi * wpi + wr;
    wi = wi * wpr + wt * wpi + wi;
    double y1 = 0.5 * (y[j] + y[n - j]);
    double y2 = (y[j] - y[n - j]);
    y[j] = y1 - wi * y2;
    y[n - j] = y1 + wi * y2;
    sum += wr * y2;
  }
  realft(y, n, 1);
  y[n] = y[1];
  y[1] = sum;
  for (size_t j = 3; j < n; j += 2) {
    sum += y[j];
    y[j] = sum;
  }
}

// cosft2 (src/Cos_FT2.rs:7-173): y[0..n).  isign=+1: Y_k = sum_j y_j
// cos(pi k (j+1/2)/n) (DCT-II).  isign=-1: the inverse times n/2, i.e.
// y_j = Y_0/2 + sum_{k>=1} Y_k cos(pi k (j+1/2)/n) (DCT-III).  Returns -1 for
// any other isign (the reference panics, src/Cos_FT2.rs:11).
// Corrections: the pre-pass twiddle advances with j (the reference holds wi1
// constant, src/Cos_FT2.rs:26-36); the post-rotation recurrence adds its own
// state (src/Cos_FT2.rs:58-59,112-113 add wr1/wi1); the inverse rotation is
// the conjugate of the forward one (src/Cos_FT2.rs:126-127 swap terms).
int orc_cosft2(double* y, size_t n, int isign) {
  if (isign != 1 && isign != -1) return -1;
  const double theta = 0.5 * PI / (double)n;
  double wr1 = std::cos(theta), wi1 = std::sin(theta);
  const double wpr = -2.0 * wi1 * wi1;
  const double wpi = std::sin(2.0 * theta);
  double wr = 1.0, wi = 0.0;
  if (isign == 1) {
    for (size_t i = 0; i < n / 2; ++i) {
      double y1 = 0.5 * (y[i] + y[n - 1 - i]);
      double y2 = wi1 * (y[i] - y[n - 1 - i]);
      y[i] = y1 + y2;
      y[n - 1 - i] = y1 - y2;
      double wt = wr1;
      wr1 = wt * wpr - wi1 * wpi + wr1;
      wi1 = wi1 * wpr + wt * wpi + wi1;
    }
    realft(y, n, 1);
    for (size_t i = 2; i < n; i += 2) {
      double wt = wr;
      wr = wt * wpr - wi * wpi + wr;
      wi = wi * wpr + wt * wpi + wi;
      double y1 = y[i] * wr - y[i + 1] * wi;
      double y2 = y[i + 1] * wr + y[i] * wi;
      y[i] = y1;
      y[i + 1] = y2;
    }
    double sum = 0.5 * y[1];
    for (size_t i = n - 1; i >= 1; i -= 2) {
      double sum1 = sum;
      sum += y[i];
      y[i] = sum1;
      if (i < 2) break;
    }
  } else {
    double ytemp = y[n - 1];
    for (size_t i = n - 1; i >= 3; i -= 2) y[i] = y[i - 2] - y[i];
    y[1] = 2.0 * ytemp;
    for (size_t i = 2; i < n; i += 2) {
      double wt = wr;
      wr = wt * wpr - wi * wpi + wr;
      wi = wi * wpr + wt * wpi + wi;
      double y1 = y[i] * wr + y[i + 1] * wi;
      double y2 = y[i + 1] * wr - y[i] * wi;
      y[i] = y1;
      y[i + 1] = y2;
    }
    realft(y, n, -1);
    for (size_t i = 0; i < n / 2; ++i) {
      double y1 = y[i] + y[n - 1 - i];
      double y2 = (0.5 / wi1) * (y[i] - y[n - 1 - i]);
      y[i] = 0.5 * (y1 + y2);
      y[n - 1 - i] = 0.5 * (y1 - y2);
      double wt = wr1;
      wr1 = wt * wpr - wi1 * wpi + wr1;
      wi1 = wi1 * wpr + wt * wpi + wi1;
    }
  }
  return 0;
}

// convlv (src/Convolve.rs:8-138).  data: n reals; respns: m taps in
// wrap-around order (respns[0]=h_0, respns[k]=h_{+k} for k<=(m-1)/2,
// respns[m-k]=h_{-k}).  ans: n reals.  isign=+1 convolves, isign=-1
// deconvolves; bins with |R|^2 < 1e-12 give 0 (src/Convolve.rs:118-122).
// Return codes follow ConvlvError (src/Convolve.rs:226-238):
//   0 ok, 1 EmptyInput, 2 ResponseTooLong, 3 InvalidIsign, 4 unsupported n.
// Corrections: the response is expanded into a length-n buffer the
// Numerical Recipes way (negative lags at the end, zeros between) instead of
// src/Convolve.rs:41-63; the product covers the n/2+1 packed bins of the two
// realft spectra instead of slots 1..n of a 2n buffer (src/Convolve.rs:106).
int orc_convlv(const double* data, size_t n, const double* respns, size_t m, int isign,
               double* ans) {
  if (n == 0 || m == 0) return 1;
  if (m > n) return 2;
  if (isign != 1 && isign != -1) return 3;
  if (n < 2 || (n & (n - 1))) return 4;
  std::vector<double> r(n, 0.0);
  // Numerical Recipes expansion: r[0..m) = respns; r[n-k] = respns[m-k] for
  // k = 1..(m-1)/2; r[(m+1)/2 .. n-(m-1)/2) = 0.
  for (size_t i = 0; i < m; ++i) r[i] = respns[i];
  size_t half = (m - 1) / 2;
  for (size_t k = 1; k <= half; ++k) r[n - k] = respns[m - k];
  for (size_t i = (m + 1) / 2; i < n - half; ++i) r[i] = 0.0;
  std::vector<double> d(data, data + n);
  // compute_parallel_ffts: the two forward transforms run concurrently
  // (rayon::join, src/Convolve.rs:71) -- here two pool tasks.
  pool().parallel_for(2, [&](size_t t) { realft(t == 0 ? d.data() : r.data(), n, 1); });
  const double no2 = (double)(n >> 1);
  for (size_t k = 0; k <= n / 2; ++k) {
    // bin k: (re, im); k = 0 and k = n/2 are real and live in slots 0 and 1
    double dr, di, rr, ri;
    if (k == 0) { dr = d[0]; di = 0.0; rr = r[0]; ri = 0.0; }
    else if (k == n / 2) { dr = d[1]; di = 0.0; rr = r[1]; ri = 0.0; }
    else { dr = d[2 * k]; di = d[2 * k + 1]; rr = r[2 * k]; ri = r[2 * k + 1]; }
    double outr, outi;
    if (isign == 1) {
      outr = (dr * rr - di * ri) / no2;
      outi = (dr * ri + di * rr) / no2;
    } else {
      double mag2 = rr * rr + ri * ri;
      if (mag2 < 1e-12) {
        outr = 0.0;
        outi = 0.0;
      } else {
        outr = (dr * rr + di * ri) / mag2 / no2;
        outi = (di * rr - dr * ri) / mag2 / no2;
      }
    }
    if (k == 0) ans[0] = outr;
    else if (k == n / 2) ans[1] = outr;
    else { ans[2 * k] = outr; ans[2 * k + 1] = outi; }
  }
  realft(ans, n, -1);
  return 0;
}

// Expanded-response convolution: resp is already a length-n wrap-around
// buffer (negative lags at the end).  Same arithmetic as orc_convlv.
int orc_convlv_expanded(const double* data, size_t n, const double* resp, int isign,
                        double* ans) {
  return orc_convlv(data, n, resp, n, isign, ans);
}

// correl (src/Correlation.rs:8-110).  ans[k] = sum_j data1[(j+k) mod n] *
// data2[j] for n > 32 (negative lags at ans[n-k]); for n <= 32 the reference's
// direct linear sum (src/Correlation.rs:37-50) is kept so its known answers
// hold.  Return codes follow CorrelError (src/Correlation.rs:389-399):
//   0 ok, 1 EmptyInput, 2 LengthMismatch, 4 unsupported n.
// Corrections: the spectra come from realft (not the O(n^2) placeholder DFT
// at src/Correlation.rs:326-386), the Nyquist bin is packed into slot 1
// before the inverse, and the result is read from the real output directly
// (src/Correlation.rs:174-186 reads every other slot).
int orc_correl(const double* data1, size_t n1, const double* data2, size_t n2, double* ans) {
  if (n1 == 0) return 1;
  if (n2 != n1) return 2;
  size_t n = n1;
  if (n <= 32) {
    for (size_t lag = 0; lag < n; ++lag) {
      double sum = 0.0;
      for (size_t i = 0; i < n - lag; ++i) sum += data1[i + lag] * data2[i];
      ans[lag] = sum;
    }
    return 0;
  }
  if (n & (n - 1)) return 4;
  std::vector<double> f1(data1, data1 + n), f2(data2, data2 + n);
  pool().parallel_for(2, [&](size_t t) { realft(t == 0 ? f1.data() : f2.data(), n, 1); });
  const double no2 = (double)(n >> 1);
  for (size_t k = 0; k <= n / 2; ++k) {
    double ar, ai, br, bi;
    if (k == 0) { ar = f1[0]; ai = 0.0; br = f2[0]; bi = 0.0; }
    else if (k == n / 2) { ar = f1[1]; ai = 0.0; br = f2[1]; bi = 0.0; }
    else { ar = f1[2 * k]; ai = f1[2 * k + 1]; br = f2[2 * k]; bi = f2[2 * k + 1]; }
    // fft1 * conj(fft2), src/Correlation.rs:90-96
    double outr = (ar * br + ai * bi) / no2;
    double outi = (ai * br - ar * bi) / no2;
    if (k == 0) ans[0] = outr;
    else if (k == n / 2) ans[1] = outr;
    else { ans[2 * k] = outr; ans[2 * k + 1] = outi; }
  }
  realft(ans, n, -1);
  return 0;
}

// correl_normalized (fast = 0, src/Correlation.rs:189-223) and
// correl_normalized_fast (fast = 1, :226-270).  Return codes as orc_correl,
// plus 5 for ZeroStdDev.
int orc_correl_normalized(const double* d1, size_t n1, const double* d2, size_t n2, double* ans,
                          int fast) {
  if (n1 == 0) return 1;
  if (n2 != n1) return 2;
  const size_t n = n1;
  const double nd = (double)n;
  double mean1, mean2, std1, std2;
  if (!fast) {
    double s1 = 0, s2 = 0;
    for (size_t i = 0; i < n; ++i) { s1 += d1[i]; s2 += d2[i]; }
    mean1 = s1 / nd;
    mean2 = s2 / nd;
    double v1 = 0, v2 = 0;
    for (size_t i = 0; i < n; ++i) {
      v1 += (d1[i] - mean1) * (d1[i] - mean1);
      v2 += (d2[i] - mean2) * (d2[i] - mean2);
    }
    std1 = std::sqrt(v1 / nd);
    std2 = std::sqrt(v2 / nd);
  } else {
    double s1 = 0, s2 = 0, q1 = 0, q2 = 0;
    for (size_t i = 0; i < n; ++i) {
      s1 += d1[i]; s2 += d2[i]; q1 += d1[i] * d1[i]; q2 += d2[i] * d2[i];
    }
    mean1 = s1 / nd;
    mean2 = s2 / nd;
    std1 = std::sqrt(q1 / nd - mean1 * mean1);
    std2 = std::sqrt(q2 / nd - mean2 * mean2);
  }
  if (std1 == 0.0 || std2 == 0.0 || std::isnan(std1) || std::isnan(std2)) return 5;
  if (fast && n <= 32) {
    const double norm = 1.0 / (std1 * std2 * nd);
    for (size_t lag = 0; lag < n; ++lag) {
      double sum = 0.0;
      for (size_t i = 0; i < n - lag; ++i) sum += (d1[i + lag] - mean1) * (d2[i] - mean2);
      ans[lag] = sum * norm;
    }
    return 0;
  }
  std::vector<double> z1(n), z2(n);
  for (size_t i = 0; i < n; ++i) {
    z1[i] = (d1[i] - mean1) / std1;
    z2[i] = (d2[i] - mean2) / std2;
  }
  return orc_correl(z1.data(), n, z2.data(), n, ans);
}

// magnitude_spectrum / power_spectrum (src/FFT_1.rs:206-228).
void orc_magnitude_spectrum(const double* c, size_t nn, double* out) {
  for (size_t k = 0; k < nn; ++k) out[k] = std::sqrt(c[2 * k] * c[2 * k] + c[2 * k + 1] * c[2 * k + 1]);
}
void orc_power_spectrum(const double* c, size_t nn, double* out) {
  for (size_t k = 0; k < nn; ++k) out[k] = c[2 * k] * c[2 * k] + c[2 * k + 1] * c[2 * k + 1];
}

// ---------------------------------------------------------------------------
// Exact-arithmetic spot checks at full size: selected bins X_k of a direct
// DFT, X_k = sum_j x_j exp(+2 pi i isign jk/nn), evaluated with compensated
// (twice-working-precision) dot products, so that each bin is accurate to
// about one rounding of its magnitude whatever nn is.  Independent of every
// FFT in this file and in the library.
// ---------------------------------------------------------------------------
// exp(2 pi i m / nn), 0 <= m < nn, nn a power of two, with the angle reduced
// to [0, pi/4] before cos/sin so that each value is within about one ulp.
static void unit_root(size_t m, size_t nn, double& c, double& s) {
  bool neg_s = false, neg_c = false, swap = false;
  if (m > nn / 2) { m = nn - m; neg_s = true; }   // exp(i(2 pi - a)) = conj exp(ia)
  if (m > nn / 4) { m = nn / 2 - m; neg_c = true; }  // exp(i(pi - a)) = -cos a + i sin a
  if (m > nn / 8) { m = nn / 4 - m; swap = true; }   // cos(pi/2 - a) = sin a
  const double a = 2.0 * PI * (double)m / (double)nn;
  double cc = std::cos(a), ss = std::sin(a);
  if (swap) std::swap(cc, ss);
  c = neg_c ? -cc : cc;
  s = neg_s ? -ss : ss;
}

// Error-free transformations: a + b = s + e exactly (Knuth's TwoSum) and
// a * b = p + e exactly (through a fused multiply-add).
static inline void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
static inline void two_prod(double a, double b, double& p, double& e) {
  p = a * b;
  e = std::fma(a, b, -p);
}

// Compensated complex accumulator: (sr + cr) + i (si + ci).
struct CAcc {
  double sr = 0, cr = 0, si = 0, ci = 0;
  inline void add_prod(double ar, double ai, double br, double bi) {
    double p, e, t, f;
    two_prod(ar, br, p, e); two_sum(sr, p, t, f); sr = t; cr += e + f;
    two_prod(-ai, bi, p, e); two_sum(sr, p, t, f); sr = t; cr += e + f;
    two_prod(ar, bi, p, e); two_sum(si, p, t, f); si = t; ci += e + f;
    two_prod(ai, br, p, e); two_sum(si, p, t, f); si = t; ci += e + f;
  }
};

void orc_dft_bins(const double* in, size_t nn, int isign, const size_t* bins, size_t nb,
                  double* out) {
  // j = j1 + N1 j2: exp(2 pi i jk/nn) = A[j1] B[j2] with A[j1] = w^(j1 k),
  // B[j2] = w^(N1 j2 k).  Inner sums over j1 and the outer sum over j2 are
  // both compensated.
  int lg = 0;
  while ((size_t(1) << lg) < nn) ++lg;
  const size_t N1 = size_t(1) << ((lg + 1) / 2), N2 = nn / N1;
  const double sg = isign > 0 ? 1.0 : -1.0;
  pool().parallel_for(nb, [&](size_t b) {
    const size_t k = bins[b] % nn;
    std::vector<double> ar(N1), ai(N1);
    for (size_t j1 = 0; j1 < N1; ++j1) {
      unit_root((j1 * k) % nn, nn, ar[j1], ai[j1]);
      ai[j1] *= sg;
    }
    CAcc outer;
    for (size_t j2 = 0; j2 < N2; ++j2) {
      CAcc inner;
      const double* x = in + 2 * j2 * N1;
      for (size_t j1 = 0; j1 < N1; ++j1) inner.add_prod(x[2 * j1], x[2 * j1 + 1], ar[j1], ai[j1]);
      double br, bi;
      unit_root((N1 * ((j2 * k) % nn)) % nn, nn, br, bi);
      bi *= sg;
      // (s + c) * B: the rounded inner sum and its correction, each times B
      outer.add_prod(inner.sr, inner.si, br, bi);
      outer.add_prod(inner.cr, inner.ci, br, bi);
    }
    out[2 * b] = outer.sr + outer.cr;
    out[2 * b + 1] = outer.si + outer.ci;
  });
}

// Long-double direct DFT for small spot checks: X_k = sum_j x_j exp(+2 pi i isign jk/n).
void orc_dft_ld(const double* in, size_t nn, int isign, double* out) {
  const long double tau = 6.283185307179586476925286766559005768L;
  for (size_t k = 0; k < nn; ++k) {
    long double sr = 0, si = 0;
    for (size_t j = 0; j < nn; ++j) {
      size_t e = (j * k) % nn;
      long double a = tau * (long double)isign * (long double)e / (long double)nn;
      long double c = cosl(a), s = sinl(a);
      sr += (long double)in[2 * j] * c - (long double)in[2 * j + 1] * s;
      si += (long double)in[2 * j] * s + (long double)in[2 * j + 1] * c;
    }
    out[2 * k] = (double)sr;
    out[2 * k + 1] = (double)si;
  }
}

}  // extern "C"
