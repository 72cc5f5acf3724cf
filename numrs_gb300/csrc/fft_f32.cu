// fft_f32.cu -- Stockham pass kernels in IEEE float.  The caller's data stay
// interleaved double; intermediate passes of long axes keep float complex.
#include "fft_core.cuh"

namespace gbfft {

template <int SG>
static cudaError_t dispatch(IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st) {
  if (in == IO_D2 && out == IO_D2) return launch_pass_t<F32, SG, IO_D2, IO_D2>(p, threads, st);
  if (in == IO_D2 && out == IO_F2) return launch_pass_t<F32, SG, IO_D2, IO_F2>(p, threads, st);
  if (in == IO_F2 && out == IO_D2) return launch_pass_t<F32, SG, IO_F2, IO_D2>(p, threads, st);
  if (in == IO_F2 && out == IO_F2) return launch_pass_t<F32, SG, IO_F2, IO_F2>(p, threads, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_pass_f32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st) {
  return sign > 0 ? dispatch<1>(in, out, p, threads, st) : dispatch<-1>(in, out, p, threads, st);
}

}  // namespace gbfft
