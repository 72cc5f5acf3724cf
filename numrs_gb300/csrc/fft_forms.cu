// fft_forms.cu -- the per-form pass launchers the runtime calls; the kernels
// themselves are instantiated in fft_<form>_<direction>.cu.
#include "fft_core.cuh"

namespace gbfft {

GBFFT_DECLARE_DISPATCH(F64)
GBFFT_DECLARE_DISPATCH(F32)
GBFFT_DECLARE_DISPATCH(DF64)
GBFFT_DECLARE_DISPATCH(TC32)

cudaError_t launch_pass_f64(int sign, IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st) {
  if (p.twist)
    return sign > 0 ? dispatch_twist<F64, 1>(in, out, p, threads, st)
                    : dispatch_twist<F64, -1>(in, out, p, threads, st);
  return sign > 0 ? dispatch_io<F64, 1>(in, out, p, threads, st)
                  : dispatch_io<F64, -1>(in, out, p, threads, st);
}
cudaError_t launch_pass_f32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                            cudaStream_t st) {
  if (p.twist)
    return sign > 0 ? dispatch_twist<F32, 1>(in, out, p, threads, st)
                    : dispatch_twist<F32, -1>(in, out, p, threads, st);
  return sign > 0 ? dispatch_io<F32, 1>(in, out, p, threads, st)
                  : dispatch_io<F32, -1>(in, out, p, threads, st);
}
cudaError_t launch_pass_df64(int sign, IOType in, IOType out, const PassParams& p, int threads,
                             cudaStream_t st) {
  if (p.twist)
    return sign > 0 ? dispatch_twist<DF64, 1>(in, out, p, threads, st)
                    : dispatch_twist<DF64, -1>(in, out, p, threads, st);
  return sign > 0 ? dispatch_io<DF64, 1>(in, out, p, threads, st)
                  : dispatch_io<DF64, -1>(in, out, p, threads, st);
}
cudaError_t launch_pass_tc32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                             cudaStream_t st) {
  if (p.twist)
    return sign > 0 ? dispatch_twist<TC32, 1>(in, out, p, threads, st)
                    : dispatch_twist<TC32, -1>(in, out, p, threads, st);
  return sign > 0 ? dispatch_io<TC32, 1>(in, out, p, threads, st)
                  : dispatch_io<TC32, -1>(in, out, p, threads, st);
}

}  // namespace gbfft
