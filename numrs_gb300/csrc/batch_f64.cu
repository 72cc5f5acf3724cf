// batch_f64.cu -- the persistent batched-FFT kernels of the F64 form (both
// directions); see batch_kernels.cuh.
#include "batch_kernels.cuh"

namespace gbfft {

cudaError_t launch_batch_f64(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_t<F64, 1, IO_D2>(P, grid, st)
                  : launch_batch_t<F64, -1, IO_D2>(P, grid, st);
}

int batch_blocks_per_sm_f64(int sign) {
  return sign > 0 ? occupancy_t<F64, 1, IO_D2>() : occupancy_t<F64, -1, IO_D2>();
}

}  // namespace gbfft
