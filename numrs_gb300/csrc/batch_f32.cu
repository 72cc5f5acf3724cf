// batch_f32.cu -- the persistent batched-FFT kernels of the F32 form (both
// directions); see batch_kernels.cuh.
#include "batch_kernels.cuh"

namespace gbfft {

cudaError_t launch_batch_f32(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_t<F32, 1, IO_F2>(P, grid, st)
                  : launch_batch_t<F32, -1, IO_F2>(P, grid, st);
}

int batch_blocks_per_sm_f32(int sign) {
  return sign > 0 ? occupancy_t<F32, 1, IO_F2>() : occupancy_t<F32, -1, IO_F2>();
}

cudaError_t launch_batch_pf_f32(int sign, const BatchParams& P, int grid, cudaStream_t st) {
  return sign > 0 ? launch_batch_pf_t<F32, 1, IO_F2>(P, grid, st)
                  : launch_batch_pf_t<F32, -1, IO_F2>(P, grid, st);
}

int batch_pf_blocks_per_sm_f32(int sign) {
  return sign > 0 ? occupancy_pf_t<F32, 1, IO_F2>() : occupancy_pf_t<F32, -1, IO_F2>();
}

}  // namespace gbfft
