// fft_f32_cl_m.cu -- cluster pass kernels in IEEE float, inverse (isign = -1),
// and the launcher the runtime calls.
#include "cluster_pass.cuh"

namespace gbfft {
template cudaError_t dispatch_cl<-1>(IOType, IOType, const PassParams&, int, cudaStream_t);
extern template cudaError_t dispatch_cl<1>(IOType, IOType, const PassParams&, int, cudaStream_t);

cudaError_t launch_pass_cl_f32(int sign, IOType in, IOType out, const PassParams& p, int threads,
                               cudaStream_t st) {
  return sign > 0 ? dispatch_cl<1>(in, out, p, threads, st) : dispatch_cl<-1>(in, out, p, threads, st);
}
}  // namespace gbfft
