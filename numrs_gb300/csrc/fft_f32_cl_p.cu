// fft_f32_cl_p.cu -- cluster pass kernels in IEEE float, forward (isign = +1).
#include "cluster_pass.cuh"

namespace gbfft {
template cudaError_t dispatch_cl<1>(IOType, IOType, const PassParams&, int, cudaStream_t);
}  // namespace gbfft
