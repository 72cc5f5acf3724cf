// fft_df64_p.cu -- Stockham pass kernels in double-float (compensated FP32 pairs), forward (isign = +1).
#include "fft_core.cuh"

namespace gbfft {
template cudaError_t dispatch_io<DF64, 1>(IOType, IOType, const PassParams&, int,
                                          cudaStream_t);
template cudaError_t dispatch_twist<DF64, 1>(IOType, IOType, const PassParams&, int,
                                            cudaStream_t);
}  // namespace gbfft
