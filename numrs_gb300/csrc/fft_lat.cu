// fft_lat.cu -- the latency-mode pass kernels of every form (one-warp tiles
// of 128 points) and the launcher the runtime calls.
#include "fft_core.cuh"

namespace gbfft {

cudaError_t launch_pass_lat(Form f, int sign, IOType in, IOType out, const PassParams& p,
                            cudaStream_t st) {
  if (f == FORM_F64)
    return sign > 0 ? dispatch_lat<F64, 1>(in, out, p, st) : dispatch_lat<F64, -1>(in, out, p, st);
  if (f == FORM_DF64)
    return sign > 0 ? dispatch_lat<DF64, 1>(in, out, p, st) : dispatch_lat<DF64, -1>(in, out, p, st);
  // FP32 and the tensor-core form (its twiddle tables are FP32 ones; radix
  // <= 4 sub-passes have no tensor-core stage)
  return sign > 0 ? dispatch_lat<F32, 1>(in, out, p, st) : dispatch_lat<F32, -1>(in, out, p, st);
}

}  // namespace gbfft
