// fft_f64.cu -- Stockham pass kernels in IEEE double (the plain FP64 form),
// both directions.
#include "fft_core.cuh"

namespace gbfft {
template cudaError_t dispatch_io<F64, 1>(IOType, IOType, const PassParams&, int, cudaStream_t);
template cudaError_t dispatch_io<F64, -1>(IOType, IOType, const PassParams&, int, cudaStream_t);
template cudaError_t dispatch_twist<F64, 1>(IOType, IOType, const PassParams&, int,
                                            cudaStream_t);
template cudaError_t dispatch_twist<F64, -1>(IOType, IOType, const PassParams&, int,
                                            cudaStream_t);
}  // namespace gbfft
