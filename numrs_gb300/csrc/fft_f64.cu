// fft_f64.cu -- Stockham pass kernels in IEEE double (the plain FP64 form).
#include "fft_core.cuh"

namespace gbfft {

cudaError_t launch_pass_f64(int sign, IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st) {
  if (in != IO_D2 || out != IO_D2) return cudaErrorInvalidValue;
  return sign > 0 ? launch_pass_t<F64, 1, IO_D2, IO_D2>(p, threads, st)
                  : launch_pass_t<F64, -1, IO_D2, IO_D2>(p, threads, st);
}

}  // namespace gbfft
