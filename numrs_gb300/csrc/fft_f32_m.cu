// fft_f32_m.cu -- Stockham pass kernels in IEEE float, inverse (isign = -1).
#include "fft_core.cuh"

namespace gbfft {
template cudaError_t dispatch_io<F32, -1>(IOType, IOType, const PassParams&, int,
                                          cudaStream_t);
template cudaError_t dispatch_twist<F32, -1>(IOType, IOType, const PassParams&, int,
                                            cudaStream_t);
}  // namespace gbfft
