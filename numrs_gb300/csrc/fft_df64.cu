// fft_df64.cu -- Stockham pass kernels in double-float (compensated FP32
// pairs).  Intermediate passes of long axes keep the full hi/lo pairs.
#include "fft_core.cuh"

namespace gbfft {

template <int SG>
static cudaError_t dispatch(IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st) {
  if (in == IO_D2 && out == IO_D2) return launch_pass_t<DF64, SG, IO_D2, IO_D2>(p, threads, st);
  if (in == IO_D2 && out == IO_F4) return launch_pass_t<DF64, SG, IO_D2, IO_F4>(p, threads, st);
  if (in == IO_F4 && out == IO_D2) return launch_pass_t<DF64, SG, IO_F4, IO_D2>(p, threads, st);
  if (in == IO_F4 && out == IO_F4) return launch_pass_t<DF64, SG, IO_F4, IO_F4>(p, threads, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_pass_df64(int sign, IOType in, IOType out, const PassParams& p, int threads,
                             cudaStream_t st) {
  return sign > 0 ? dispatch<1>(in, out, p, threads, st) : dispatch<-1>(in, out, p, threads, st);
}

}  // namespace gbfft
