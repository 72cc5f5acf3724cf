// fft_tc32_p.cu -- Stockham pass kernels of the tensor-core form (FP32 data, 3xTF32 radix-16 stages), forward (isign = +1).
#include "fft_core.cuh"

namespace gbfft {
template cudaError_t dispatch_io<TC32, 1>(IOType, IOType, const PassParams&, int,
                                          cudaStream_t);
template cudaError_t dispatch_twist<TC32, 1>(IOType, IOType, const PassParams&, int,
                                            cudaStream_t);
}  // namespace gbfft
